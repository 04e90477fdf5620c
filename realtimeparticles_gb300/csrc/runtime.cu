// runtime.cu - model handles, step pipelines, CUDA-graph executor and the C ABI.
//
// Replaces the OpenCL runtime role of CL::Context (physics/ocl/Context.cpp: buffer
// registry, runKernel, profiling) and the host update() sequences of the three models.
// One handle = one model on one CUDA stream.  A step is recorded once into a CUDA graph
// and replayed; the graph is re-recorded whenever a parameter, the particle count or the
// boundary changes.  When profiling is on, every kernel of the graph is bracketed by
// captured event-record nodes, so per-kernel device times come from the replays
// themselves (Context::runKernel's event profiling, Context.cpp:692-705).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "boids.cuh"
#include "clouds.cuh"
#include "fluids.cuh"
#include "rtp_internal.hpp"
#include "side.cuh"
#include "target.hpp"
#include "warmstart.cuh"

namespace rtp {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return RTP_ERR_NO_DEVICE;
  if (e == cudaErrorMemoryAllocation) return RTP_ERR_OUT_OF_MEMORY;
  return RTP_ERR_CUDA;
}

void ensure_dynamic_smem(const void* k, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = done[{k, dev}];
  if (have >= bytes) return;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess) have = bytes;
}

constexpr float PI_F = 3.1415927f;  // utils/Math.hpp:69

// Utils::FloatToStr (utils/Utils.cpp:24-28) + the OpenCL compiler's parse of the literal.
static float round_trip(float v) {
  char buf[128];
  std::snprintf(buf, sizeof buf, "%.10f", (double)v);
  return std::strtof(buf, nullptr);
}

static int derive_constants(int model, const rtp_model_params* p, rtp_grid_constants* c) {
  if (!p || !c) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  std::memset(c, 0, sizeof *c);
  for (int a = 0; a < 3; ++a) {
    if (p->gridRes[a] == 0 || !(p->boxSize[a] > 0.0f)) return fail(RTP_ERR_INVALID_ARGUMENT, "empty box or grid");
    c->gridRes[a] = p->gridRes[a];
    c->absWall[a] = round_trip(p->boxSize[a] / 2.0f);  // Fluids.cpp:108-110
  }
  const float bx = p->boxSize[0];
  const float rx = (float)p->gridRes[0];
  c->cellSize = round_trip(bx / rx);  // Fluids.cpp:114
  const uint64_t nc = (uint64_t)p->gridRes[0] * p->gridRes[1] * p->gridRes[2];
  if (nc > (1ull << 30)) return fail(RTP_ERR_INVALID_ARGUMENT, "grid too large");
  c->numCells = (uint32_t)nc;
  const float effectRadius = bx / rx;  // Fluids.cpp:104
  c->effectRadius = round_trip(effectRadius);
  c->effectRadiusSquared = round_trip(1.0f * bx * bx / (float)(p->gridRes[0] * p->gridRes[0]));  // Boids.cpp:104
  c->poly6Coeff = round_trip(315.0f / (64.0f * PI_F * std::pow(effectRadius, 9.f)));             // Fluids.cpp:117
  c->spikyCoeff = round_trip(15.0f / (PI_F * std::pow(effectRadius, 6.f)));                      // Fluids.cpp:118
  c->maxVel = round_trip(30.0f);                                                                 // Fluids.cpp:119
  uint32_t cap = p->maxNbPartsInCell;
  if (cap == 0) cap = (model == RTP_MODEL_BOIDS) ? 3000u : 100u;  // Boids.cpp:78, Fluids.cpp:79
  c->maxPartsInCell = cap;
  // Largest key: every axis at +W (index == GRID_RES aliases, grid.cl:33-35).
  uint32_t top[3];
  for (int a = 0; a < 3; ++a) {
    const float q = std::fmin(std::fmax(c->absWall[a], -c->absWall[a]), c->absWall[a]) + c->absWall[a];
    top[a] = (uint32_t)std::floor(q / c->cellSize);
  }
  const uint64_t kb = (uint64_t)top[0] * c->gridRes[2] * c->gridRes[1] + (uint64_t)top[1] * c->gridRes[2] + top[2] + 1;
  if (kb > 0xFFFFFFFFull) return fail(RTP_ERR_INVALID_ARGUMENT, "key range exceeds 32 bits");
  c->keyBound = (uint32_t)kb;
  uint32_t bits = 0;
  while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)c->keyBound) ++bits;
  c->keyBits = bits;
  return RTP_OK;
}

FluidK make_fluidk(const rtp_grid_constants& c, const rtp_fluid_params& p) {
  FluidK k;
  k.rho0 = p.restDensity;
  k.invRho0 = 1.0f / p.restDensity;
  k.invRho0Sq = 1.0f / (p.restDensity * p.restDensity);
  k.relaxCFM = p.relaxCFM;
  k.dt = p.timeStep;
  k.lo = make_float4(-c.absWall[0] + 0.01f, -c.absWall[1] + 0.01f, -c.absWall[2] + 0.01f, 0.0f);
  k.hi = make_float4(c.absWall[0] - 0.1f, c.absWall[1] - 0.1f, c.absWall[2] - 0.1f, 0.0f);
  k.artPressure = p.isArtPressureEnabled ? 1 : 0;
  k.apCoeff = p.artPressureCoeff;
  // poly6L(artPressureRadius * h, h), sph.cl:16-19.
  const float h = c.effectRadius;
  const float L = p.artPressureRadius * h;
  const float q = h * h - L * L;
  const float wq = (L < h ? 1.0f : 0.0f) * c.poly6Coeff * (q * q * q);
  k.apInvWq = wq != 0.0f ? 1.0f / wq : 0.0f;
  k.apExp = p.artPressureExp;
  k.vorticity = p.isVorticityConfEnabled ? 1 : 0;
  k.vortCoeff = p.vorticityConfCoeff;
  k.xsph = p.xsphViscosityCoeff;
  return k;
}

// ---------------------------------------------------------------------------------------
struct TimedSlot {
  std::string name;
  int ev;  // index of the start event; end = ev + 1
};

struct KernelStat {
  uint64_t launches = 0;
  double ms = 0.0;
};

struct Handle {
  int model = 0;
  rtp_model_params mp{};
  rtp_grid_constants gc{};
  GridK g{};
  rtp_fluid_params fp{};
  uint32_t iters = 2;
  rtp_boids_params bp{};
  float boidsDt = 0.1f;
  rtp_cloud_params cp{};
  rtp_cloud_env env{};
  float* ground = nullptr;
  int boundary = RTP_BOUNDARY_BOUNCING_WALL;
  bool paused = false;
  uint64_t maxN = 0, curN = 0;
  int device = 0;
  cudaStream_t stream = nullptr;

  // Canonical state (the Model's buffers) and the sorted working copies.
  float4 *pos = nullptr, *vel = nullptr, *posS = nullptr, *velS = nullptr;
  float4 *predTmp = nullptr, *predA = nullptr, *predB = nullptr, *predFinal = nullptr;
  float4 *vort = nullptr, *acc = nullptr, *totCorr = nullptr, *totCorrS = nullptr;
  float *lambda = nullptr, *density = nullptr;
  float4* predLam = nullptr;  // (x, y, z, lambda) in each Jacobi iteration, then (x, y, z, |omega|)
  float *temp = nullptr, *vapor = nullptr, *cloud = nullptr, *buoy = nullptr;
  float *tempS = nullptr, *vaporS = nullptr, *cloudS = nullptr, *buoyS = nullptr;
  float *lapT = nullptr, *lamT = nullptr;
  uint32_t *ids = nullptr, *idsS = nullptr, *cellId = nullptr;
  uint2* table = nullptr;
  uint2* tableRef = nullptr;
  void* sortMem = nullptr;
  SortScratch ss{};
  double* mAcc = nullptr;
  uint32_t* mHist = nullptr;
  PairList pairs{};
  std::vector<void*> allocs;
  // Sort fault word in mapped pinned memory: the sort passes raise it (never in a correct
  // run); the calls that synchronise with the stream read it and report it.
  uint32_t* faultHost = nullptr;
  uint32_t* faultDev = nullptr;

  // Graph executor.
  cudaGraphExec_t graph = nullptr;
  bool graphValid = false;
  bool graphProfiled = false;
  // A fluids or boids step over host-resident state (rtp_update_host with pinned buffers): the
  // same step captured with the host pointers it reads and writes (io, set while capturing).
  // A few captures are kept (least recently used replaced), so alternating buffer pairs do
  // not recapture on every call.
  HostIO io{};
  struct HostGraph {
    HostIO io{};
    cudaGraphExec_t exec = nullptr;
    bool valid = false;
    uint64_t used = 0;
  };
  HostGraph hostGraphs[4];
  uint64_t hostGraphClock = 0;

  // Profiling.
  bool profiling = false;
  std::vector<cudaEvent_t> events;
  std::vector<TimedSlot> slots;
  std::map<std::string, KernelStat> stats;

  // Timing.
  void* flush = nullptr;
  size_t flushBytes = 0;
  cudaEvent_t t0 = nullptr, t1 = nullptr;

  bool hasStep = false;  // a step ran since the last upload (cell table / keys valid)

  // Learned warm start (fluids).
  bool wsOn = false;
  uint32_t wsExtra = 0;
  bool wsRelaxAll = false;     // the network's omega relaxes every iteration, not the first only
  float* wsOmega = nullptr;    // per-particle omega of the step (relaxAll)
  float wsTol = 0.0f;
  bool statsOn = false;        // solver statistics in plain steps
  void* mlpBlock = nullptr;    // packed network
  float* mlpTmp = nullptr;     // upload staging for the packer
  float* lamTot = nullptr;     // lambda summed over the last warm-started / recording step
  // Training through the solve (allocated on first use): features and network outputs of
  // every particle, dL/dy, dL/dx', the plain lambda, the corrected positions and their
  // densities, per-block loss sums, and the trainer.
  float* trFeats = nullptr;
  float* trY = nullptr;
  float* trDy = nullptr;
  float4* trG = nullptr;
  float* trLam = nullptr;
  float4* trXp = nullptr;
  float* trRho = nullptr;
  float* trLoss = nullptr;
  WsTrainer* trainer = nullptr;
  float* errPartial = nullptr; // per-block density-error sums
  SolverStatsDev* solverStats = nullptr;
  PairList pairsRec{};         // pairs at the predicted positions while recording samples
  cudaStream_t stream2 = nullptr;  // captures the guard's rerun body

  // Tuning (fluids): lanes per particle of the list sweeps; batch cell size = cellFactor * h.
  uint32_t lanes = 4;
  uint32_t tiles = 0;  // brick-tiled lambda sweep (rtp_tuning.tiledSweeps)
  float cellFactor = 1.0f;

  // Batched scenes (fluids): scene s owns slots [sceneOff[s], sceneOff[s] + desc[s].nbParticles).
  bool isBatch = false;
  float batchH = 0.0f;
  std::vector<rtp_batch_scene> sceneDesc;
  std::vector<uint64_t> sceneOff;
  std::vector<SceneK> hScenes;
  std::vector<rtp_grid_constants> sceneConst;  // each scene's own grid (keys without the base)
  SceneK* dScenes = nullptr;
  uint16_t* dSceneOf = nullptr;
  // Side outputs (allocated on first use).
  float4* col = nullptr;
  uint32_t *camDist = nullptr, *camSorted = nullptr, *drawOrder = nullptr;
  float* gridDet = nullptr;
  void* camSortMem = nullptr;
  SortScratch camSS{};
  uint32_t tableCells = 0;  // cells the table was allocated for
  uint32_t sortKeyBits = 0; // key bits the sort scratch was allocated for
  // Boids target attractor: parameters, the host trajectory, and the device track of the
  // target positions of up to kTargetChunk steps (slot 0: step counter), filled from
  // pinned staging ahead of the graph launches that read it.
  rtp_target_params tp{};
  bool targetVisible = false;
  TargetTrajectory traj{0.0f};
  float4* targetTrack = nullptr;
  float4* targetHost = nullptr;
  cudaEvent_t targetUp = nullptr;  // the last upload has read targetHost
  bool targetUpPending = false;
};

constexpr uint32_t kTargetChunk = 1024;
static bool target_on(const Handle* h) { return h->model == RTP_MODEL_BOIDS && h->tp.enabled; }

// The fluids parameters a step's kernels get: shared values, tuning and the batch tables.
static FluidK fluidk_of(const Handle* h) {
  FluidK k = make_fluidk(h->gc, h->fp);
  k.lanes = (int)h->lanes;
  k.tiles = (int)h->tiles;
  k.sortedKeys = h->cellId;
  if (h->isBatch) {
    k.bt.scenes = h->dScenes;
    k.bt.sceneOf = h->dSceneOf;
  }
  return k;
}

int Launcher::begin(const char* name) {
  if (!profiling || !owner) return RTP_OK;
  Handle* h = (Handle*)owner;
  const int ev = (int)h->slots.size() * 2;
  while ((int)h->events.size() < ev + 2) {
    cudaEvent_t e;
    RTP_CUDA(cudaEventCreate(&e));
    h->events.push_back(e);
  }
  h->slots.push_back({name, ev});
  // External record nodes: inside a capture a plain record only orders work.
  RTP_CUDA(cudaEventRecordWithFlags(h->events[ev], stream, cudaEventRecordExternal));
  return RTP_OK;
}

int Launcher::end(const char* name) {
  (void)name;
  if (!profiling || !owner) return RTP_OK;
  Handle* h = (Handle*)owner;
  RTP_CUDA(cudaEventRecordWithFlags(h->events[h->slots.back().ev + 1], stream, cudaEventRecordExternal));
  return RTP_OK;
}

template <class T>
static int dalloc(Handle* h, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  RTP_CUDA(cudaMalloc((void**)p, sizeof(T) * count));
  RTP_CUDA(cudaMemset(*p, 0, sizeof(T) * count));
  h->allocs.push_back((void*)*p);
  return RTP_OK;
}

#define RTP_TRY(x)           \
  do {                       \
    int _rc = (x);           \
    if (_rc) return _rc;     \
  } while (0)

static int alloc_buffers(Handle* h) {
  const size_t M = h->maxN;
  RTP_TRY(dalloc(h, &h->pos, M));
  RTP_TRY(dalloc(h, &h->vel, M));
  RTP_TRY(dalloc(h, &h->posS, M));
  RTP_TRY(dalloc(h, &h->velS, M));
  RTP_TRY(dalloc(h, &h->ids, M));
  RTP_TRY(dalloc(h, &h->idsS, M));
  RTP_TRY(dalloc(h, &h->cellId, M));
  RTP_TRY(dalloc(h, &h->table, h->gc.numCells));
  RTP_TRY(dalloc(h, &h->tableRef, h->gc.numCells));
  RTP_TRY(dalloc(h, &h->mAcc, 4));
  RTP_TRY(dalloc(h, &h->mHist, 80));
  RTP_CUDA(cudaHostAlloc((void**)&h->faultHost, sizeof(uint32_t), cudaHostAllocMapped));
  *h->faultHost = 0;
  RTP_CUDA(cudaHostGetDevicePointer((void**)&h->faultDev, h->faultHost, 0));
  if (h->model == RTP_MODEL_BOIDS) {
    RTP_TRY(dalloc(h, &h->acc, M));
  } else {
    RTP_TRY(dalloc(h, &h->predTmp, M));
    RTP_TRY(dalloc(h, &h->predA, M));
    RTP_TRY(dalloc(h, &h->predB, M));
    RTP_TRY(dalloc(h, &h->vort, M));
    RTP_TRY(dalloc(h, &h->lambda, M));
    RTP_TRY(dalloc(h, &h->predLam, M));
    RTP_TRY(dalloc(h, &h->density, M));
    h->predFinal = h->predA;
    RTP_TRY(dalloc(h, &h->pairs.idx, (size_t)kPairListK * M));
    RTP_TRY(dalloc(h, &h->pairs.count, M));
    h->pairs.stride = (uint32_t)M;
    h->pairs.K = kPairListK;
  }
  if (h->model == RTP_MODEL_FLUIDS) RTP_TRY(dalloc(h, &h->lamTot, M));
  if (h->model == RTP_MODEL_CLOUDS) {
    RTP_TRY(dalloc(h, &h->totCorr, M));
    RTP_TRY(dalloc(h, &h->totCorrS, M));
    RTP_TRY(dalloc(h, &h->temp, M));
    RTP_TRY(dalloc(h, &h->vapor, M));
    RTP_TRY(dalloc(h, &h->cloud, M));
    RTP_TRY(dalloc(h, &h->buoy, M));
    RTP_TRY(dalloc(h, &h->tempS, M));
    RTP_TRY(dalloc(h, &h->vaporS, M));
    RTP_TRY(dalloc(h, &h->cloudS, M));
    RTP_TRY(dalloc(h, &h->buoyS, M));
    RTP_TRY(dalloc(h, &h->lapT, M));
    RTP_TRY(dalloc(h, &h->lamT, M));
  }
  h->tableCells = h->gc.numCells;
  h->sortKeyBits = h->gc.keyBits;
  const SortPlan full = make_sort_plan((uint32_t)M, h->gc.keyBits);
  const size_t sb = sort_scratch_bytes(full);
  RTP_CUDA(cudaMalloc(&h->sortMem, sb));
  h->allocs.push_back(h->sortMem);
  sort_scratch_carve(full, h->sortMem, h->ss);
  // Identity ids.
  std::vector<uint32_t> id(M);
  for (size_t i = 0; i < M; ++i) id[i] = (uint32_t)i;
  RTP_CUDA(cudaMemcpy(h->ids, id.data(), sizeof(uint32_t) * M, cudaMemcpyHostToDevice));
  return RTP_OK;
}

static void free_handle(Handle* h) {
  if (!h) return;
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (auto& hg : h->hostGraphs)
    if (hg.exec) cudaGraphExecDestroy(hg.exec);
  for (void* p : h->allocs) cudaFree(p);
  if (h->ground) cudaFree(h->ground);
  if (h->flush) cudaFree(h->flush);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  if (h->t0) cudaEventDestroy(h->t0);
  if (h->t1) cudaEventDestroy(h->t1);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->stream2) cudaStreamDestroy(h->stream2);
  if (h->targetHost) cudaFreeHost(h->targetHost);
  if (h->faultHost) cudaFreeHost(h->faultHost);
  if (h->trainer) ws_trainer_destroy(h->trainer);
  if (h->targetUp) cudaEventDestroy(h->targetUp);
  delete h;
}

// Buffers of the warm start and of the solver statistics (allocated on first use).
static int ws_alloc(Handle* h) {
  if (h->errPartial) return RTP_OK;
  const size_t M = h->maxN;
  RTP_TRY(dalloc(h, &h->errPartial, ws_error_blocks((uint32_t)M)));
  RTP_TRY(dalloc(h, &h->wsOmega, M));
  RTP_TRY(dalloc(h, &h->solverStats, 1));
  char* blk = nullptr;
  RTP_TRY(dalloc(h, &blk, MlpLayout::bytes));
  h->mlpBlock = blk;
  RTP_TRY(dalloc(h, &h->mlpTmp, mlp_upload_tmp_floats()));
  if (!h->stream2) RTP_CUDA(cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking));
  return RTP_OK;
}

static int ws_alloc_rec(Handle* h) {
  RTP_TRY(ws_alloc(h));
  if (h->pairsRec.idx) return RTP_OK;
  const size_t M = h->maxN;
  RTP_TRY(dalloc(h, &h->pairsRec.idx, (size_t)kPairListK * M));
  RTP_TRY(dalloc(h, &h->pairsRec.count, M));
  h->pairsRec.stride = (uint32_t)M;
  h->pairsRec.K = kPairListK;
  return RTP_OK;
}

static int ws_alloc_train(Handle* h) {
  RTP_TRY(ws_alloc_rec(h));
  if (h->trainer) return RTP_OK;
  const size_t M = h->maxN;
  RTP_TRY(dalloc(h, &h->trFeats, (size_t)kMlpIn * M));
  RTP_TRY(dalloc(h, &h->trY, (size_t)kMlpOut * M));
  RTP_TRY(dalloc(h, &h->trDy, (size_t)kMlpOut * M));
  RTP_TRY(dalloc(h, &h->trG, M));
  RTP_TRY(dalloc(h, &h->trLam, M));
  RTP_TRY(dalloc(h, &h->trXp, M));
  RTP_TRY(dalloc(h, &h->trRho, M));
  RTP_TRY(dalloc(h, &h->trLoss, ws_loss_blocks((uint32_t)M)));
  return ws_trainer_create((uint32_t)M, &h->trainer);
}

// A new state has no lambda totals yet.
static int ws_forget(Handle* h) {
  if (h->lamTot) RTP_CUDA(cudaMemsetAsync(h->lamTot, 0, sizeof(float) * h->maxN, h->stream));
  return RTP_OK;
}

static void invalidate(Handle* h) {
  h->graphValid = false;
  for (auto& hg : h->hostGraphs) hg.valid = false;
}

// ---- one model step (the update() sequences) ------------------------------------------
// Fluids.cpp:412-424: predict, cell ids, sort {pos, vel, predPos} (+ ids), cell table.
// clampOut: store the clamped prediction (a Jacobi iteration or correction consumes it).
static int fluids_presort(Handle* h, Launcher& L, const FluidK& fk, bool clampOut) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const SortPlan plan = make_sort_plan(n, h->gc.keyBits);
  const ZeroJob zero = step_zero_job(plan, h->ss, h->table, h->gc.numCells);
  RTP_TRY(fluid_presort(g, fk, h->pos, h->vel, n, h->predTmp, h->ss.keysA, plan, h->ss.hist, clampOut, L, zero, h->io));
  GatherList gl;
  gl.fault = h->faultDev;
  gl.src4[0] = h->pos;
  gl.dst4[0] = h->posS;
  gl.src4[1] = h->vel;
  gl.dst4[1] = h->velS;
  gl.src4[2] = h->predTmp;
  gl.dst4[2] = h->predA;
  gl.n4 = 3;
  gl.src1[0] = h->ids;
  gl.dst1[0] = h->idsS;
  gl.n1 = 1;
  RTP_TRY(launch_sort_passes(plan, h->ss.keysA, h->cellId, h->ss, gl, L));
  return launch_cell_table(g, h->cellId, n, h->table, L, h->isBatch ? h->dSceneOf : nullptr, true);
}

// `count` plain Jacobi iterations from `in`; the outputs alternate between dest and spare
// so that the last lands in dest.  With trackTot the total lambda is accumulated (started
// by the first iteration unless firstAdds).
// With omega the lambdas of every iteration are relaxed by it (the warm start's relaxation kept
// for the plain iterations after the first).
static int plain_iterations(Handle* h, Launcher& L, const FluidK& fk, const float4* in, uint32_t count, float4* dest,
                            float4* spare, bool trackTot, bool firstAdds, const float* omega = nullptr) {
  const uint32_t n = (uint32_t)h->curN;
  const float4* cur = in;
  for (uint32_t it = 0; it < count; ++it) {
    float4* out = ((count - it) % 2 == 1) ? dest : spare;
    const int mode = !trackTot ? kTotNone : ((it == 0 && !firstAdds) ? kTotWrite : kTotAdd);
    RTP_TRY(fluid_iteration(h->g, fk, cur, out, h->table, n, h->lambda, h->density, it + 1 == count, h->posS, h->velS,
                            h->pairs, L, h->lamTot, mode, h->predLam, omega));
    cur = out;
  }
  return RTP_OK;
}

// Solver-output density error into errPartial: fused into the vorticity sweep when that
// runs (returns true), else a separate sweep.
static int solver_error(Handle* h, Launcher& L, const FluidK& fk, const float4* x, bool* vortDone) {
  const uint32_t n = (uint32_t)h->curN;
  if (fk.vorticity) {
    RTP_TRY(fluid_vorticity(h->g, fk, x, h->velS, h->vort, h->table, n, h->pairs, h->errPartial, L, h->predLam));
    *vortDone = true;
    return RTP_OK;
  }
  *vortDone = false;
  return ws_density_error(h->g, fk, x, h->table, n, h->errPartial, L);
}

static int record_fluids_ws_step(Handle* h, Launcher& L);

// The warm-started first iteration from predA (the network `block` relaxes the plain lambda)
// and E iterations after it, plain or (relaxAll) relaxed by the same per-particle omega; the
// solver output lands in predB.
static int ws_first_iteration(Handle* h, Launcher& L, const FluidK& fk, const void* block, uint32_t E, bool relaxAll) {
  const uint32_t n = (uint32_t)h->curN;
  RTP_TRY(ws_lambda_infer(h->g, fk, h->predA, h->velS, h->table, n, h->lambda, h->density, h->lamTot, h->pairs, block,
                          h->predLam, relaxAll ? h->wsOmega : nullptr, L));
  float4* warmOut = (E % 2 == 0) ? h->predB : h->predTmp;
  RTP_TRY(fluid_deltap(h->g, fk, h->predA, warmOut, h->lambda, h->table, n, E == 0, h->posS, h->velS, h->pairs, nullptr,
                       L, h->predLam));
  return plain_iterations(h, L, fk, warmOut, E, h->predB, h->predTmp, true, true, relaxAll ? h->wsOmega : nullptr);
}

// Training through the solve, after the presort of a step (x* = predA): features and plain
// lambda at x* (pairs P* in h->pairs), y = network(features) (the trainer's weights), the
// correction x' = clamp(x* + dp(omega(y) lambda)), the density at x' (pairs P' in
// h->pairsRec), then dL/dx' and dL/dy of L = 1/n sum C(x')^2 into trDy; per-block sums of
// C(x')^2 in trLoss.  With skipFeatures the features of this presort are in trFeats already.
static int ws_train_pass(Handle* h, Launcher& L, bool skipFeatures) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  if (!skipFeatures)
    RTP_TRY(ws_lambda_record(g, fk, h->predA, h->velS, h->table, n, h->trLam, h->density, h->lamTot, h->pairs, 1, 0,
                             h->trFeats, n, L));
  RTP_TRY(ws_trainer_forward(h->trainer, h->trFeats, n, h->trY, L.stream));
  RTP_TRY(ws_apply_omega(h->predA, h->trLam, h->trY, n, h->lambda, h->predLam, L));
  RTP_TRY(fluid_deltap(g, fk, h->predA, h->trXp, h->lambda, h->table, n, false, h->posS, h->velS, h->pairs, nullptr, L,
                       h->predLam));
  RTP_TRY(fluid_lambda_sweep(g, fk, h->trXp, h->table, n, h->lamTot, h->trRho, h->pairsRec, L));
  RTP_TRY(ws_loss_grad_x(g, fk, h->trXp, h->trRho, h->table, n, h->pairsRec, h->trG, h->trLoss, L));
  return ws_grad_y(g, fk, h->predA, h->trLam, h->trY, h->trG, h->table, n, h->pairs, h->trDy, L);
}

// Mean of C(x')^2 from the per-block sums (synchronises the stream).
static int ws_train_loss(Handle* h, double* loss) {
  const uint32_t n = (uint32_t)h->curN;
  std::vector<float> part(ws_loss_blocks(n));
  RTP_CUDA(cudaMemcpyAsync(part.data(), h->trLoss, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  double a = 0.0;
  for (float v : part) a += (double)v;
  *loss = n ? a / (double)n : 0.0;
  return RTP_OK;
}

static int record_fluids_step(Handle* h, Launcher& L) {
  const uint32_t n = (uint32_t)h->curN;
  if (n == 0) return RTP_OK;
  if (h->wsOn) return record_fluids_ws_step(h, L);
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  RTP_TRY(fluids_presort(h, L, fk, h->iters > 0));
  // Fluids.cpp:427-442.
  float4* cur = h->predA;
  float4* nxt = h->predB;
  for (uint32_t it = 0; it < h->iters; ++it) {
    RTP_TRY(fluid_iteration(g, fk, cur, nxt, h->table, n, h->lambda, h->density, it + 1 == h->iters, h->posS, h->velS,
                            h->pairs, L, nullptr, kTotNone, h->predLam));
    std::swap(cur, nxt);
  }
  if (h->iters == 0) RTP_TRY(fluid_update_vel(g, fk, cur, h->posS, n, h->velS, L));
  h->predFinal = cur;
  bool vortDone = false;
  if (h->statsOn) {
    RTP_TRY(solver_error(h, L, fk, cur, &vortDone));
    RTP_TRY(ws_guard(h->errPartial, n, 0.0f, h->solverStats, 0, false, false, L));
  }
  // Fluids.cpp:444-457.
  return fluid_post(g, fk, cur, h->velS, h->vort, h->table, n, h->idsS, h->pos, h->vel, h->ids, h->pairs, L, vortDone,
                    h->io, h->predLam);
}

// The warm-start guard's conditional graph node, in three parts around ws_guard: a handle in
// the step graph being captured on L.stream; then an if-node on it, whose body is captured on
// stream2 (conditional bodies take kernels, memsets and copies only: no profiling events);
// then the end of that capture.
static int guard_handle(Launcher& L, cudaGraphConditionalHandle* hnd) {
  cudaStreamCaptureStatus st;
  cudaGraph_t capGraph = nullptr;
  RTP_CUDA(cudaStreamGetCaptureInfo(L.stream, &st, nullptr, &capGraph, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive) return fail(RTP_ERR_STATE, "warm-start guard needs a captured step");
  RTP_CUDA(cudaGraphConditionalHandleCreate(hnd, capGraph, 0, cudaGraphCondAssignDefault));
  return RTP_OK;
}

static int guard_body_begin(Handle* h, Launcher& L, cudaGraphConditionalHandle hnd) {
  cudaStreamCaptureStatus st;
  cudaGraph_t capGraph = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  RTP_CUDA(cudaStreamGetCaptureInfo(L.stream, &st, nullptr, &capGraph, &deps, &edges, &nd));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = hnd;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  RTP_CUDA(cudaGraphAddNode(&node, capGraph, deps, edges, nd, &np));
  RTP_CUDA(cudaStreamUpdateCaptureDependencies(L.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  RTP_CUDA(cudaStreamBeginCaptureToGraph(h->stream2, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  return RTP_OK;
}

static int guard_body_end(Handle* h, int rc) {
  cudaGraph_t bodyOut = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(h->stream2, &bodyOut);
  if (rc) return rc;
  if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture(guard body)");
  return RTP_OK;
}

// Warm-started substep: the network's lambda and residual give the first correction, then
// wsExtra plain iterations; the guard reruns the solve with the plain iteration count from
// the same predicted positions (predA) inside a conditional graph node.  The solver output
// always ends in predB (predTmp, free after the sort, is the third buffer).
static int record_fluids_ws_step(Handle* h, Launcher& L) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  RTP_TRY(fluids_presort(h, L, fk, true));
  RTP_TRY(ws_first_iteration(h, L, fk, h->mlpBlock, h->wsExtra, h->wsRelaxAll));
  h->predFinal = h->predB;
  bool vortDone = false;
  RTP_TRY(solver_error(h, L, fk, h->predB, &vortDone));
  const bool guard = h->wsTol > 0.0f;
  cudaGraphConditionalHandle hnd = 0;
  if (guard) RTP_TRY(guard_handle(L, &hnd));
  RTP_TRY(ws_guard(h->errPartial, n, h->wsTol, h->solverStats, hnd, guard, false, L));
  if (guard) {
    RTP_TRY(guard_body_begin(h, L, hnd));
    Launcher L2;
    L2.stream = h->stream2;
    int rc = RTP_OK;
    if (h->iters > 0) {
      rc = plain_iterations(h, L2, fk, h->predA, h->iters, h->predB, h->predTmp, true, false);
    } else {
      const cudaError_t ce =
          cudaMemcpyAsync(h->predB, h->predA, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream2);
      rc = ce == cudaSuccess ? RTP_OK : cuda_fail(ce, "cudaMemcpyAsync");
      if (!rc) rc = fluid_update_vel(g, fk, h->predB, h->posS, n, h->velS, L2);
      if (!rc) rc = cudaMemsetAsync(h->lamTot, 0, sizeof(float) * n, h->stream2) == cudaSuccess
                        ? RTP_OK
                        : fail(RTP_ERR_CUDA, "cudaMemsetAsync");
    }
    bool vd2 = false;
    if (!rc) rc = solver_error(h, L2, fk, h->predB, &vd2);
    if (!rc) rc = ws_guard(h->errPartial, n, 0.0f, h->solverStats, 0, false, true, L2);
    RTP_TRY(guard_body_end(h, rc));
  }
  return fluid_post(g, fk, h->predB, h->velS, h->vort, h->table, n, h->idsS, h->pos, h->vel, h->ids, h->pairs, L,
                    vortDone, h->io, h->predLam);
}

// One plain step with `iters` iterations that also writes training samples.
static int record_sample_step(Handle* h, uint32_t iters, uint32_t stride, uint32_t phase, float* feats, float* targets,
                              uint32_t count) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(fluids_presort(h, L, fk, true));
  RTP_TRY(ws_lambda_record(g, fk, h->predA, h->velS, h->table, n, h->lambda, h->density, h->lamTot,
                           h->pairsRec, stride, phase, feats, count, L));
  float4* out0 = (iters % 2 == 1) ? h->predB : h->predTmp;
  RTP_TRY(fluid_deltap(g, fk, h->predA, out0, h->lambda, h->table, n, iters == 1, h->posS, h->velS, h->pairsRec,
                       nullptr, L));
  RTP_TRY(plain_iterations(h, L, fk, out0, iters - 1, h->predB, h->predTmp, true, true));
  RTP_TRY(ws_record_targets(g, fk, h->predA, h->lamTot, h->table, n, h->predB, h->pairsRec, stride, phase, count,
                            targets, L));
  h->predFinal = h->predB;
  return fluid_post(g, fk, h->predB, h->velS, h->vort, h->table, n, h->idsS, h->pos, h->vel, h->ids, h->pairs, L,
                    false, HostIO{}, h->predLam);
}

static int record_boids_step(Handle* h, Launcher& L) {
  const uint32_t n = (uint32_t)h->curN;
  if (n == 0) return RTP_OK;
  const GridK& g = h->g;
  const SortPlan plan = make_sort_plan(n, h->gc.keyBits);
  const ZeroJob zero = step_zero_job(plan, h->ss, h->table, h->gc.numCells);
  // Boids.cpp:335-344.
  TargetK tk;
  if (target_on(h)) {
    tk.track = h->targetTrack;
    tk.cap = kTargetChunk;
    tk.radius = h->tp.radiusEffect;
    tk.sign = (float)h->tp.signEffect;
  }
  RTP_TRY(boids_presort(g, h->pos, h->vel, n, h->ss.keysA, plan, h->ss.hist, L, zero, tk, h->io));
  GatherList gl;
  gl.fault = h->faultDev;
  gl.src4[0] = h->pos;
  gl.dst4[0] = h->posS;
  gl.src4[1] = h->vel;
  gl.dst4[1] = h->velS;
  gl.n4 = 2;
  gl.src1[0] = h->ids;
  gl.dst1[0] = h->idsS;
  gl.n1 = 1;
  RTP_TRY(launch_sort_passes(plan, h->ss.keysA, h->cellId, h->ss, gl, L));
  RTP_TRY(launch_cell_table(g, h->cellId, n, h->table, L, nullptr, true));
  // Boids.cpp:346-373 (the target rule, :351-358, inside the rules kernel).
  BoidsK bk;
  bk.velocityScale = h->bp.velocityScale;
  bk.alignmentScale = h->bp.alignmentScale;
  bk.separationScale = h->bp.separationScale;
  bk.cohesionScale = h->bp.cohesionScale;
  bk.dt = h->boidsDt;
  bk.maxVelocity = h->bp.velocityScale;
  // Boids.cpp:346-349: the 2D rules kernel for a 2D model.
  return boids_rules_update(g, bk, h->boundary == RTP_BOUNDARY_CYCLIC_WALL, h->mp.dimension == 2, h->posS, h->velS,
                            h->table, n, h->idsS,
                            h->pos, h->vel, h->acc, h->ids, L, tk, h->io);
}

static CloudK make_cloudk(const Handle* h) {
  CloudK c;
  c.dim = h->cp.dim;
  c.dt = h->cp.timeStep;
  c.cloudRho0 = h->cp.restDensity;
  c.cloudRelax = h->cp.relaxCFM;
  c.groundHeat = h->cp.groundHeatCoeff;
  c.buoyancy = h->cp.buoyancyCoeff;
  c.gravCoeff = h->cp.gravCoeff;
  c.adiabatic = h->cp.adiabaticLapseRate;
  c.phaseRate = h->cp.phaseTransitionRate;
  c.latent = h->cp.latentHeatCoeff;
  c.initVapor = h->cp.initVaporDensityCoeff;
  c.wind = h->cp.windCoeff;
  c.smoothing = h->cp.isTempSmoothingEnabled ? 1 : 0;
  c.T0 = h->env.groundTemp0;
  c.lapse = h->env.lapseRate;
  c.heatDecay = h->env.heatDecay;
  c.windX = h->env.windDecayX;
  c.windZ = h->env.windDecayZ;
  c.ground = h->ground;
  c.nx = h->ground ? h->env.groundNx : 0u;
  c.nz = h->ground ? h->env.groundNz : 0u;
  return c;
}

// Clouds.cpp:516-567: thermodynamics, predict, mixed boundary, cell ids, the sort, the cell
// table and the temperature smoothing.
static int clouds_presort(Handle* h, Launcher& L) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const CloudK ck = make_cloudk(h);
  const SortPlan plan = make_sort_plan(n, h->gc.keyBits);
  const ZeroJob zero = step_zero_job(plan, h->ss, h->table, h->gc.numCells);
  // Clouds.cpp:516-541: thermodynamics, predict, mixed boundary, cell ids.
  RTP_TRY(cloud_presort(g, ck, h->pos, h->vel, n, h->temp, h->vapor, h->cloud, h->buoy, h->predTmp, h->totCorr,
                        h->ss.keysA, plan, h->ss.hist, L, zero));
  // Clouds.cpp:543.
  GatherList gl;
  gl.fault = h->faultDev;
  gl.src4[0] = h->pos;
  gl.dst4[0] = h->posS;
  gl.src4[1] = h->vel;
  gl.dst4[1] = h->velS;
  gl.src4[2] = h->predTmp;
  gl.dst4[2] = h->predA;
  gl.src4[3] = h->totCorr;
  gl.dst4[3] = h->totCorrS;
  gl.n4 = 4;
  gl.src1[0] = reinterpret_cast<const uint32_t*>(h->temp);
  gl.dst1[0] = reinterpret_cast<uint32_t*>(h->tempS);
  gl.src1[1] = reinterpret_cast<const uint32_t*>(h->buoy);
  gl.dst1[1] = reinterpret_cast<uint32_t*>(h->buoyS);
  gl.src1[2] = reinterpret_cast<const uint32_t*>(h->vapor);
  gl.dst1[2] = reinterpret_cast<uint32_t*>(h->vaporS);
  gl.src1[3] = reinterpret_cast<const uint32_t*>(h->cloud);
  gl.dst1[3] = reinterpret_cast<uint32_t*>(h->cloudS);
  gl.src1[4] = h->ids;
  gl.dst1[4] = h->idsS;
  gl.n1 = 5;
  RTP_TRY(launch_sort_passes(plan, h->ss.keysA, h->cellId, h->ss, gl, L));
  RTP_TRY(launch_cell_table(g, h->cellId, n, h->table, L, nullptr, true));
  // Clouds.cpp:554-567.
  if (ck.smoothing)
    RTP_TRY(cloud_temperature(g, ck, h->posS, h->tempS, h->lamT, h->table, n, h->pairs, L, h->predLam));
  return RTP_OK;
}

// Clouds.cpp:570-587 from predA: `count` plain iterations, the last landing in dest (spare is
// the other buffer) and updating the velocities; with no iteration the velocities come from
// the step's total correction alone and dest is not written (returns the output buffer).
static int cloud_plain_iterations(Handle* h, Launcher& L, const FluidK& fk, const float4* in, uint32_t count,
                                  float4* dest, float4* spare) {
  const uint32_t n = (uint32_t)h->curN;
  const float4* cur = in;
  for (uint32_t it = 0; it < count; ++it) {
    float4* out = ((count - it) % 2 == 1) ? dest : spare;
    RTP_TRY(cloud_iteration(h->g, fk, cur, out, h->totCorrS, h->table, n, h->lambda, h->density, it + 1 == count,
                            h->velS, h->pairs, L, h->predLam));
    cur = out;
  }
  return RTP_OK;
}

// Clouds.cpp:570-590 from predA: the plain Jacobi loop, or with `block` the warm-started first
// iteration (the network relaxes the plain lambda) and E plain iterations; the solver output
// ends in predB (predA with no iteration at all).  With `guarded` and a guard tolerance the
// step's solver-output density error decides, inside a conditional graph node, whether the
// solve reruns plain (the handle's iteration count) from predA with the step's total
// correction restored.  Then (statistics) the solver output's density error, then
// Clouds.cpp:592-605.
static int clouds_solve_post(Handle* h, Launcher& L, const void* block, uint32_t E, bool guarded) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  const CloudK ck = make_cloudk(h);
  const bool guard = guarded && block && h->wsTol > 0.0f;
  float4* out = h->predB;
  if (block) {
    // The total correction at the start of the solve, for a rerun (vort is free until the post).
    if (guard)
      RTP_CUDA(cudaMemcpyAsync(h->vort, h->totCorrS, sizeof(float4) * n, cudaMemcpyDeviceToDevice, L.stream));
    float4* warmOut = (E % 2 == 0) ? h->predB : h->predTmp;
    RTP_TRY(cloud_ws_lambda(g, fk, ck, h->predA, h->velS, h->tempS, h->buoyS, h->table, n, h->lambda, h->density,
                            h->pairs, h->predLam, nullptr, block, L));
    RTP_TRY(cloud_deltap(g, fk, h->predA, warmOut, h->totCorrS, h->lambda, h->table, n, E == 0, h->velS, h->pairs, L,
                         h->predLam));
    RTP_TRY(cloud_plain_iterations(h, L, fk, warmOut, E, h->predB, h->predTmp));
  } else if (h->iters > 0) {
    RTP_TRY(cloud_plain_iterations(h, L, fk, h->predA, h->iters, h->predB, h->predTmp));
  } else {
    RTP_TRY(cloud_update_vel(g, fk, h->totCorrS, n, h->velS, L));
    out = h->predA;
  }
  h->predFinal = out;
  if (h->statsOn || guard) {
    RTP_TRY(cloud_density_error(g, fk, out, h->table, n, h->errPartial, L));
    cudaGraphConditionalHandle hnd = 0;
    if (guard) RTP_TRY(guard_handle(L, &hnd));
    RTP_TRY(ws_guard(h->errPartial, n, guard ? h->wsTol : 0.0f, h->solverStats, hnd, guard, false, L));
    if (guard) {
      RTP_TRY(guard_body_begin(h, L, hnd));
      Launcher L2;
      L2.stream = h->stream2;
      int rc = cudaMemcpyAsync(h->totCorrS, h->vort, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream2) ==
                       cudaSuccess
                   ? RTP_OK
                   : fail(RTP_ERR_CUDA, "cudaMemcpyAsync(guard)");
      if (!rc && h->iters > 0) {
        rc = cloud_plain_iterations(h, L2, fk, h->predA, h->iters, h->predB, h->predTmp);
      } else if (!rc) {
        rc = cudaMemcpyAsync(h->predB, h->predA, sizeof(float4) * n, cudaMemcpyDeviceToDevice, h->stream2) ==
                     cudaSuccess
                 ? RTP_OK
                 : fail(RTP_ERR_CUDA, "cudaMemcpyAsync(guard)");
        if (!rc) rc = cloud_update_vel(g, fk, h->totCorrS, n, h->velS, L2);
      }
      if (!rc) rc = cloud_density_error(g, fk, h->predB, h->table, n, h->errPartial, L2);
      if (!rc) rc = ws_guard(h->errPartial, n, 0.0f, h->solverStats, 0, false, true, L2);
      RTP_TRY(guard_body_end(h, rc));
    }
  }
  // Clouds.cpp:592-605.
  CloudState s;
  s.pos = h->pos;
  s.vel = h->vel;
  s.temp = h->temp;
  s.vapor = h->vapor;
  s.cloud = h->cloud;
  s.buoy = h->buoy;
  s.tempS = h->tempS;
  s.vaporS = h->vaporS;
  s.cloudS = h->cloudS;
  s.buoyS = h->buoyS;
  s.ids = h->ids;
  s.idsS = h->idsS;
  return cloud_post(g, fk, ck, out, h->velS, h->vort, h->table, n, s, h->pairs, L, h->predLam);
}

// clouds_presort for rtp_warm_start_loss_grad: the thermodynamics it runs change temp, vapor,
// cloud and buoyancy in place, so they are saved first and put back after (the sorted copies
// the training pass reads are kept).
static int clouds_presort_keep_state(Handle* h, Launcher& L) {
  const size_t b = sizeof(float) * h->curN;
  float* save[4] = {h->temp, h->vapor, h->cloud, h->buoy};
  // Scratch: the network-output rows (4 floats a particle), written only after the restore.
  for (int k = 0; k < 4; ++k)
    RTP_CUDA(cudaMemcpyAsync(h->trY + (size_t)k * h->curN, save[k], b, cudaMemcpyDeviceToDevice, L.stream));
  RTP_TRY(clouds_presort(h, L));
  for (int k = 0; k < 4; ++k)
    RTP_CUDA(cudaMemcpyAsync(save[k], h->trY + (size_t)k * h->curN, b, cudaMemcpyDeviceToDevice, L.stream));
  return RTP_OK;
}

// Clouds::update (Clouds.cpp:503-610).
int record_clouds_step(Handle* h, Launcher& L) {
  if (h->curN == 0) return RTP_OK;
  RTP_TRY(clouds_presort(h, L));
  return clouds_solve_post(h, L, h->wsOn ? h->mlpBlock : nullptr, h->wsExtra, true);
}

// Training through the clouds solve after clouds_presort (x* = predA): as ws_train_pass, with
// the clouds sweeps (periodic images in x and z, the mixed boundary) and the step's total
// correction left untouched (the correction is applied to a copy of it).
static int cloud_train_pass(Handle* h, Launcher& L, bool skipFeatures) {
  const uint32_t n = (uint32_t)h->curN;
  const GridK& g = h->g;
  const FluidK fk = fluidk_of(h);
  const CloudK ck = make_cloudk(h);
  if (!skipFeatures)
    RTP_TRY(cloud_ws_lambda(g, fk, ck, h->predA, h->velS, h->tempS, h->buoyS, h->table, n, h->trLam, h->density,
                            h->pairs, h->predLam, h->trFeats, nullptr, L));
  RTP_TRY(ws_trainer_forward(h->trainer, h->trFeats, n, h->trY, L.stream));
  RTP_TRY(ws_apply_omega(h->predA, h->trLam, h->trY, n, h->lambda, h->predLam, L));
  RTP_CUDA(cudaMemcpyAsync(h->vort, h->totCorrS, sizeof(float4) * n, cudaMemcpyDeviceToDevice, L.stream));
  RTP_TRY(cloud_deltap(g, fk, h->predA, h->trXp, h->vort, h->lambda, h->table, n, false, h->velS, h->pairs, L,
                       h->predLam));
  RTP_TRY(cloud_density(g, fk, h->trXp, h->table, n, h->lamT, h->trRho, h->pairsRec, h->predLam, L));
  RTP_TRY(cloud_ws_loss_grad_x(g, fk, h->trXp, h->trRho, h->table, n, h->pairsRec, h->trG, h->trLoss, L));
  return cloud_ws_grad_y(g, fk, h->predA, h->trLam, h->trY, h->trG, h->table, n, h->pairs, h->trDy, L);
}

// ---- Model::reset: reference defaults + the case's initial particles ------------------
struct V3 {
  float x, y, z;
};

// Geometry::GenerateBoxGrid, uniform (utils/Geometry.cpp:190-219).
static void box_grid(std::vector<V3>& out, const int res[3], V3 s, V3 e) {
  const V3 sp = {(e.x - s.x) / res[0], (e.y - s.y) / res[1], (e.z - s.z) / res[2]};
  for (int ix = 0; ix < res[0]; ++ix)
    for (int iy = 0; iy < res[1]; ++iy)
      for (int iz = 0; iz < res[2]; ++iz) out.push_back({s.x + ix * sp.x, s.y + iy * sp.y, s.z + iz * sp.z});
}

// Geometry::GenerateBoxGrid, random (utils/Geometry.cpp:220-230), seeded instead of rand().
static void box_random(std::vector<V3>& out, int count, V3 s, V3 e, uint64_t seed) {
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (float)((st >> 40) & 0xFFFFFF) / (float)0xFFFFFF;
  };
  const V3 v = {e.x - s.x, e.y - s.y, e.z - s.z};
  for (int i = 0; i < count; ++i) {
    const float a = next(), b = next(), c = next();
    out.push_back({a * v.x + s.x, b * v.y + s.y, c * v.z + s.z});
  }
}

// Geometry::GenerateSphereGrid (utils/Geometry.cpp:236-263).
static void sphere_grid(std::vector<V3>& out, const int res[3], V3 s, V3 e) {
  const V3 v = {e.x - s.x, e.y - s.y, e.z - s.z};
  const V3 c = {s.x + v.x / 2.0f, s.y + v.y / 2.0f, s.z + v.z / 2.0f};
  const float radius = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z) / 2.0f;
  const float dphi = PI_F / res[0], dth = 2.0f * PI_F / res[1], dr = radius / res[2];
  for (int ip = 0; ip < res[0]; ++ip)
    for (int it = 0; it < res[1]; ++it)
      for (int ir = 0; ir < res[2]; ++ir) {
        const float r = (ir + 1) * dr;
        out.push_back({c.x + r * std::cos(it * dth) * std::sin(ip * dphi), c.y + r * std::sin(it * dth) * std::sin(ip * dphi),
                       c.z + r * std::cos(ip * dphi)});
      }
}

// Geometry::GenerateRectangularGrid in the YZ plane, uniform (utils/Geometry.cpp:70-126):
// res2 = (count along y, count along z), spacing (0, dy / res2[0], dz / res2[1]).
static void rect_grid_yz(std::vector<V3>& out, const int res2[2], V3 s, V3 e) {
  const V3 sp = {0.0f, (e.y - s.y) / res2[0], (e.z - s.z) / res2[1]};
  for (int iy = 0; iy < res2[0]; ++iy)
    for (int iz = 0; iz < res2[1]; ++iz) out.push_back({s.x + 0 * sp.x, s.y + iy * sp.y, s.z + iz * sp.z});
}

// Geometry::GenerateCircularGrid in the YZ plane (utils/Geometry.cpp:128-185): res2 =
// (angles, radii); radius = |end - start| / 2 around the midpoint.
static void circle_grid_yz(std::vector<V3>& out, const int res2[2], V3 s, V3 e) {
  const V3 v = {e.x - s.x, e.y - s.y, e.z - s.z};
  const V3 c = {s.x + v.x / 2.0f, s.y + v.y / 2.0f, s.z + v.z / 2.0f};
  const float radius = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z) / 2.0f;
  const float da = 2.0f * PI_F / res2[0], dr = radius / res2[1];
  for (int io = 0; io < res2[0]; ++io)
    for (int ir = 0; ir < res2[1]; ++ir)
      out.push_back({c.x, c.y + ((ir + 1) * dr) * std::cos(io * da), c.z + ((ir + 1) * dr) * std::sin(io * da)});
}

// Utils::ALL_NB_PARTICLES subdiv2D (utils/Parameters.hpp:89-98).
static bool subdiv2(uint64_t n, int out[2]) {
  static const struct {
    uint64_t n;
    int s[2];
  } T[] = {{512, {32, 16}},    {1024, {32, 32}},   {4096, {64, 64}},   {8192, {128, 64}},
           {16384, {128, 128}}, {32768, {128, 256}}, {65536, {256, 256}}, {131072, {256, 512}}};
  for (const auto& e : T)
    if (e.n == n) {
      out[0] = e.s[0];
      out[1] = e.s[1];
      return true;
    }
  return false;
}

// The 2D cases (particles in the x = 0 plane): Fluids.cpp:287-333, Boids.cpp:291-299,
// Clouds.cpp:417-446.
static int case_2d(const Handle* h, std::vector<V3>& verts, uint64_t& n) {
  const float by = h->mp.boxSize[1], bz = h->mp.boxSize[2];
  const int pc = h->mp.pCase;
  int res2[2];
  if (h->model == RTP_MODEL_FLUIDS) {
    if (pc == RTP_CASE_FLUIDS_DAM) {
      n = 4096;
      subdiv2(n, res2);
      rect_grid_yz(verts, res2, {0.0f, by / -2.0f, bz / -2.0f}, {0.0f, 0.0f, 0.0f});
    } else if (pc == RTP_CASE_FLUIDS_BOMB) {
      n = 4096;
      subdiv2(n, res2);
      rect_grid_yz(verts, res2, {0.0f, by / -6.0f, bz / -6.0f}, {0.0f, by / 6.0f, bz / 6.0f});
    } else if (pc == RTP_CASE_FLUIDS_DROP) {
      n = 512;
      subdiv2(n, res2);
      rect_grid_yz(verts, res2, {0.0f, 2.0f * by / 10.0f, bz / -10.0f}, {0.0f, 4.0f * by / 10.0f, bz / 10.0f});
      const int bottom[2] = {64, 128};
      rect_grid_yz(verts, bottom, {0.0f, by / -2.0f, bz / -2.0f}, {0.0f, 0.0f, bz / 2.0f});
      n += 4096;
    } else {
      return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a fluids case");
    }
  } else if (h->model == RTP_MODEL_BOIDS) {
    if (pc == RTP_CASE_BOIDS_SMALL) n = 512;
    else if (pc == RTP_CASE_BOIDS_MEDIUM) n = 16384;
    else if (pc == RTP_CASE_BOIDS_LARGE) n = 65536;
    else if (pc == RTP_CASE_BOIDS_XLARGE) n = 131072;
    else return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a boids case");
    subdiv2(n, res2);
    circle_grid_yz(verts, res2, {0.0f, by / -6.0f, bz / -6.0f}, {0.0f, by / 6.0f, bz / 6.0f});
  } else {
    n = 8192;
    subdiv2(n, res2);
    const int count = res2[0] * res2[1];
    if (pc == RTP_CASE_CLOUDS_CUMULUS)
      box_random(verts, count, {0.0f, by / -2.0f, bz / -2.0f}, {0.0f, 0.0f, bz / 2.0f}, 1);
    else if (pc == RTP_CASE_CLOUDS_HOMOGENEOUS)
      box_random(verts, count, {0.0f, by / -2.0f, bz / -2.0f}, {0.0f, by / 2.0f, bz / 2.0f}, 1);
    else
      return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a clouds case");
  }
  return RTP_OK;
}

// Utils::ALL_NB_PARTICLES subdiv3D (utils/Parameters.hpp:89-98).
static bool subdiv3(uint64_t n, int out[3]) {
  static const struct {
    uint64_t n;
    int s[3];
  } T[] = {{512, {8, 8, 8}},       {1024, {16, 8, 8}},     {4096, {16, 16, 16}}, {8192, {32, 16, 16}},
           {16384, {32, 32, 16}},  {32768, {32, 32, 32}}, {65536, {64, 32, 32}}, {131072, {64, 64, 32}}};
  for (const auto& e : T)
    if (e.n == n) {
      out[0] = e.s[0];
      out[1] = e.s[1];
      out[2] = e.s[2];
      return true;
    }
  return false;
}

static int init_case(Handle* h) {
  {  // Fluids.cpp:214, Boids.cpp:271, Clouds.cpp:397: resetCellIDs over maxNb slots.
    Launcher L;
    L.stream = h->stream;
    RTP_TRY(launch_reset_cell_ids(h->cellId, (uint32_t)h->maxN, h->gc.numCells, L));
  }
  const float bx = h->mp.boxSize[0], by = h->mp.boxSize[1], bz = h->mp.boxSize[2];
  std::vector<V3> verts;
  int res[3];
  uint64_t n = 0;
  const int pc = h->mp.pCase;
  if (h->mp.dimension == 2) {
    RTP_TRY(case_2d(h, verts, n));
  } else if (h->model == RTP_MODEL_FLUIDS) {
    if (pc == RTP_CASE_FLUIDS_DAM) {  // Fluids.cpp:341-346
      n = 131072;
      subdiv3(n, res);
      box_grid(verts, res, {bx / -2.0f, by / -2.0f, bz / -2.0f}, {bx / 2.0f, 0.0f, 0.0f});
    } else if (pc == RTP_CASE_FLUIDS_BOMB) {  // :347-352
      n = 65536;
      subdiv3(n, res);
      sphere_grid(verts, res, {bx / -6.0f, by / -6.0f, bz / -6.0f}, {bx / 6.0f, by / 6.0f, bz / 6.0f});
    } else if (pc == RTP_CASE_FLUIDS_DROP) {  // :353-380
      n = 4096;
      subdiv3(n, res);
      box_grid(verts, res, {bx / -10.0f, 2.0f * by / 10.0f, bz / -10.0f}, {bx / 10.0f, 4.0f * by / 10.0f, bz / 10.0f});
      const int bottom[3] = {64, 16, 64};
      box_grid(verts, bottom, {bx / -2.0f, by / -2.0f, bz / -2.0f}, {bx / 2.0f, by / -2.55f, bz / 2.0f});
      n += 65536;
    } else {
      return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a fluids case");
    }
  } else if (h->model == RTP_MODEL_BOIDS) {  // Boids.cpp:235-257, 300-308
    if (pc == RTP_CASE_BOIDS_SMALL) n = 512;
    else if (pc == RTP_CASE_BOIDS_MEDIUM) n = 16384;
    else if (pc == RTP_CASE_BOIDS_LARGE) n = 65536;
    else if (pc == RTP_CASE_BOIDS_XLARGE) n = 131072;
    else return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a boids case");
    subdiv3(n, res);
    sphere_grid(verts, res, {bx / -6.0f, by / -6.0f, bz / -6.0f}, {bx / 6.0f, by / 6.0f, bz / 6.0f});
  } else {  // Clouds.cpp:451-471
    n = 65536;
    if (pc == RTP_CASE_CLOUDS_CUMULUS)
      box_random(verts, (int)n, {bx / -2.0f, by / -2.0f, bz / -2.0f}, {bx / 2.0f, by / -4.0f, bz / 2.0f}, 1);
    else if (pc == RTP_CASE_CLOUDS_HOMOGENEOUS)
      box_random(verts, (int)n, {bx / -2.0f, by / -2.0f, bz / -2.0f}, {bx / 2.0f, by / 2.0f, bz / 2.0f}, 1);
    else
      return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: not a clouds case");
  }
  if (n > h->maxN) return fail(RTP_ERR_CAPACITY, "rtp_reset: the case needs more than maxNbParticles");
  const float inf = INFINITY;
  std::vector<float4> pos(h->maxN, make_float4(inf, inf, inf, 0.0f)), vel(h->maxN, make_float4(0.f, 0.f, 0.f, 0.f));
  // Every generated vertex is written, as the reference's std::transform over gridVerts does
  // (Fluids.cpp:383-386): the 2D Drop case generates 512 + 64 x 128 vertices but counts
  // 512 + 4096 particles, so its buffer holds finite positions past the particle count.
  for (size_t i = 0; i < verts.size() && i < h->maxN; ++i)
    pos[i] = make_float4(verts[i].x, verts[i].y, verts[i].z, 0.0f);
  if (h->model == RTP_MODEL_BOIDS) vel = pos;  // Boids.cpp:317-318: vel initialised from the position buffer
  std::vector<uint32_t> id(h->maxN);
  for (size_t i = 0; i < id.size(); ++i) id[i] = (uint32_t)i;
  RTP_CUDA(cudaMemcpyAsync(h->pos, pos.data(), sizeof(float4) * h->maxN, cudaMemcpyHostToDevice, h->stream));
  RTP_CUDA(cudaMemcpyAsync(h->vel, vel.data(), sizeof(float4) * h->maxN, cudaMemcpyHostToDevice, h->stream));
  RTP_CUDA(cudaMemcpyAsync(h->ids, id.data(), sizeof(uint32_t) * h->maxN, cudaMemcpyHostToDevice, h->stream));
  h->curN = n;
  RTP_TRY(ws_forget(h));
  if (h->model == RTP_MODEL_CLOUDS) {
    Launcher L;
    L.stream = h->stream;
    RTP_TRY(cloud_init(h->g, make_cloudk(h), h->pos, (uint32_t)h->maxN, h->temp, h->vapor, h->cloud, h->buoy, L));
  }
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  h->hasStep = false;
  return RTP_OK;
}

// ---- batched scenes ----------------------------------------------------------------------
// Scene grids for cell size cellFactor * h: R_a = ceil(box_a / cell) (at least 3, so the 27
// cells around a particle are distinct), keys as getCell1DIndexFromPos (grid.cl:29-38) offset
// by base_s = sum of the key bounds of the scenes before s (the +W alias keys stay inside a
// scene's own range).  Fills h->hScenes, h->sceneConst and the handle's global constants.
static int batch_grids(Handle* h, float cellFactor) {
  const float H = h->batchH;
  const float cell = round_trip(H * cellFactor);
  rtp_grid_constants base{};
  {
    rtp_model_params mp{};
    mp.currNbParticles = mp.maxNbParticles = 1;
    for (int a = 0; a < 3; ++a) {
      mp.boxSize[a] = H * 4.0f;
      mp.gridRes[a] = 4;
    }
    mp.dimension = 3;
    mp.maxNbPartsInCell = h->mp.maxNbPartsInCell;
    RTP_TRY(derive_constants(RTP_MODEL_FLUIDS, &mp, &base));  // h-derived constants (poly6, spiky, ...)
  }
  uint64_t keyBase = 0;
  h->hScenes.assign(h->sceneDesc.size(), SceneK{});
  h->sceneConst.assign(h->sceneDesc.size(), rtp_grid_constants{});
  for (size_t s = 0; s < h->sceneDesc.size(); ++s) {
    rtp_grid_constants c = base;
    for (int a = 0; a < 3; ++a) {
      const float L = h->sceneDesc[s].boxSize[a];
      c.absWall[a] = round_trip(L / 2.0f);
      const double r = std::ceil((double)L / (double)cell - 1e-6);
      c.gridRes[a] = (uint32_t)std::max(3.0, r);
    }
    c.cellSize = cell;
    c.effectRadius = base.effectRadius;
    const uint64_t nc = (uint64_t)c.gridRes[0] * c.gridRes[1] * c.gridRes[2];
    uint32_t top[3];
    for (int a = 0; a < 3; ++a) {
      const float q = std::fmin(std::fmax(c.absWall[a], -c.absWall[a]), c.absWall[a]) + c.absWall[a];
      top[a] = (uint32_t)std::floor(q / c.cellSize);
    }
    const uint64_t kb = (uint64_t)top[0] * c.gridRes[2] * c.gridRes[1] + (uint64_t)top[1] * c.gridRes[2] + top[2] + 1;
    if (nc > (1ull << 30) || kb > (1ull << 30)) return fail(RTP_ERR_INVALID_ARGUMENT, "batch scene grid too large");
    c.numCells = (uint32_t)nc;
    c.keyBound = (uint32_t)kb;
    uint32_t bits = 0;
    while (bits < 32 && ((uint64_t)1 << bits) < kb) ++bits;
    c.keyBits = bits;
    h->sceneConst[s] = c;
    SceneK& sk = h->hScenes[s];
    sk.g = make_gridk(c);
    sk.g.base = (uint32_t)keyBase;
    sk.lo = make_float4(-c.absWall[0] + 0.01f, -c.absWall[1] + 0.01f, -c.absWall[2] + 0.01f, 0.0f);
    sk.hi = make_float4(c.absWall[0] - 0.1f, c.absWall[1] - 0.1f, c.absWall[2] - 0.1f, 0.0f);
    keyBase += kb;
    if (keyBase > (1ull << 31)) return fail(RTP_ERR_INVALID_ARGUMENT, "batch: too many cells");
  }
  rtp_grid_constants g = base;
  g.absWall[0] = g.absWall[1] = g.absWall[2] = 0.0f;
  g.gridRes[0] = g.gridRes[1] = g.gridRes[2] = 0;
  g.cellSize = cell;
  g.numCells = (uint32_t)keyBase;  // the global table: every scene's key range
  g.keyBound = (uint32_t)keyBase;
  uint32_t bits = 0;
  while (bits < 32 && ((uint64_t)1 << bits) < keyBase) ++bits;
  g.keyBits = bits;
  h->gc = g;
  h->g = make_gridk(g);
  h->cellFactor = cellFactor;
  return RTP_OK;
}

static int batch_upload_scenes(Handle* h) {
  RTP_CUDA(cudaMemcpyAsync(h->dScenes, h->hScenes.data(), sizeof(SceneK) * h->hScenes.size(), cudaMemcpyHostToDevice,
                           h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
}

static int record_step(Handle* h, Launcher& L) {
  switch (h->model) {
    case RTP_MODEL_FLUIDS:
      return record_fluids_step(h, L);
    case RTP_MODEL_BOIDS:
      return record_boids_step(h, L);
    case RTP_MODEL_CLOUDS:
      return record_clouds_step(h, L);
  }
  return fail(RTP_ERR_STATE, "unknown model");
}

static int build_graph(Handle* h) {
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  h->slots.clear();
  Launcher L;
  L.stream = h->stream;
  L.profiling = h->profiling;
  L.owner = h;
  RTP_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = record_step(h, L);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(h->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
  const cudaError_t ei = cudaGraphInstantiate(&h->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return cuda_fail(ei, "cudaGraphInstantiate");
  h->graphValid = true;
  h->graphProfiled = h->profiling;
  return RTP_OK;
}

static bool same_io(const HostIO& a, const HostIO& b) {
  return a.inPos == b.inPos && a.inVel == b.inVel && a.outPos == b.outPos && a.outVel == b.outVel;
}

// The step capturing host I/O `io` (no profiling events): a kept capture, or a new one in the
// least recently used slot.
static int host_graph(Handle* h, const HostIO& io, cudaGraphExec_t* out) {
  Handle::HostGraph* slot = nullptr;
  for (auto& hg : h->hostGraphs)
    if (hg.valid && same_io(hg.io, io)) slot = &hg;
  if (!slot) {
    slot = &h->hostGraphs[0];
    for (auto& hg : h->hostGraphs) {
      if (!hg.valid) {
        slot = &hg;
        break;
      }
      if (hg.used < slot->used) slot = &hg;
    }
    if (slot->exec) {
      cudaGraphExecDestroy(slot->exec);
      slot->exec = nullptr;
    }
    slot->valid = false;
    Launcher L;
    L.stream = h->stream;
    h->io = io;
    RTP_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = record_step(h, L);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &graph);
    h->io = HostIO{};
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaStreamEndCapture");
    const cudaError_t ei = cudaGraphInstantiate(&slot->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) return cuda_fail(ei, "cudaGraphInstantiate");
    slot->io = io;
    slot->valid = true;
  }
  slot->used = ++h->hostGraphClock;
  *out = slot->exec;
  return RTP_OK;
}

// The device-visible address of pinned host memory p (nullptr in, nullptr out); false when p
// is not pinned (pageable memory goes through cudaMemcpyAsync instead).
static bool pinned_device_ptr(const void* p, void** out) {
  *out = nullptr;
  if (!p) return true;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
  *out = a.devicePointer;
  return true;
}

static int collect_profile(Handle* h) {
  if (!h->graphProfiled || h->slots.empty()) return RTP_OK;
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  for (const TimedSlot& s : h->slots) {
    float ms = 0.0f;
    RTP_CUDA(cudaEventElapsedTime(&ms, h->events[s.ev], h->events[s.ev + 1]));
    KernelStat& k = h->stats[s.name];
    k.launches += 1;
    k.ms += ms;
  }
  return RTP_OK;
}

// Target::updatePos for the next k <= kTargetChunk steps (Boids.cpp:351-356), uploaded with
// the step counter reset ahead of the graph launches that read them.
static int feed_target(Handle* h, uint32_t k) {
  if (h->targetUpPending) RTP_CUDA(cudaEventSynchronize(h->targetUp));
  h->targetUpPending = false;
  const uint32_t before = 0xffffffffu;
  std::memcpy(&h->targetHost[0], &before, sizeof before);
  for (uint32_t s = 0; s < k; ++s) {
    h->traj.advance(h->mp.dimension != 2, h->bp.velocityScale);
    const float* p = h->traj.pos();
    h->targetHost[1 + s] = make_float4(p[0], p[1], p[2], 0.0f);
  }
  RTP_CUDA(cudaMemcpyAsync(h->targetTrack, h->targetHost, sizeof(float4) * (1 + (size_t)k), cudaMemcpyHostToDevice,
                           h->stream));
  RTP_CUDA(cudaEventRecord(h->targetUp, h->stream));
  h->targetUpPending = true;
  return RTP_OK;
}

static inline uint32_t target_feed_size(const Handle* h, uint32_t s, uint32_t nsteps) {
  if (!target_on(h) || s % kTargetChunk != 0) return 0;
  return std::min(kTargetChunk, nsteps - s);
}

static int run_steps(Handle* h, uint32_t nsteps) {
  if (h->paused || nsteps == 0) return RTP_OK;
  if (h->curN == 0) {
    // No particles: the step launches nothing, the target still moves (Boids.cpp:351-353).
    if (target_on(h))
      for (uint32_t s = 0; s < nsteps; ++s) h->traj.advance(h->mp.dimension != 2, h->bp.velocityScale);
    return RTP_OK;
  }
  if (!h->graphValid || h->graphProfiled != h->profiling) RTP_TRY(build_graph(h));
  for (uint32_t s = 0; s < nsteps; ++s) {
    if (const uint32_t k = target_feed_size(h, s, nsteps)) RTP_TRY(feed_target(h, k));
    RTP_CUDA(cudaGraphLaunch(h->graph, h->stream));
    if (h->graphProfiled) RTP_TRY(collect_profile(h));
  }
  h->hasStep = true;
  return RTP_OK;
}

static Handle* H(void* p) { return reinterpret_cast<Handle*>(p); }

// After a synchronisation with the handle's stream: a raised sort fault word becomes an error
// (and is cleared).  No correct run raises it; it stands for state the sort could not write.
static int check_fault(Handle* h) {
  if (!h->faultHost) return RTP_OK;
  volatile uint32_t* f = h->faultHost;
  if (*f == 0) return RTP_OK;
  *f = 0;
  return fail(RTP_ERR_CUDA,
              "radix sort: digit offsets inconsistent with the keys placed elements outside the sorted range; they "
              "were not written and the model state is not valid");
}

}  // namespace rtp

using namespace rtp;

#define RTP_GUARD_BEGIN try {
#define RTP_GUARD_END                                              \
  }                                                                \
  catch (const std::bad_alloc&) {                                  \
    return fail(RTP_ERR_OUT_OF_MEMORY, "host allocation failed");  \
  }                                                                \
  catch (...) {                                                    \
    return fail(RTP_ERR_STATE, "unexpected C++ exception");        \
  }

extern "C" {

const char* rtp_last_error(void) { return g_last_error.c_str(); }
int rtp_abi_version(void) { return RTP_ABI_VERSION; }

int rtp_get_constants(int model, const rtp_model_params* params, rtp_grid_constants* out) {
  RTP_GUARD_BEGIN
  if (model < RTP_MODEL_BOIDS || model > RTP_MODEL_CLOUDS) return fail(RTP_ERR_INVALID_ARGUMENT, "unknown model");
  return derive_constants(model, params, out);
  RTP_GUARD_END
}

// JSON defaults: Fluids.cpp:52-74.
int rtp_fluid_params_default(rtp_fluid_params* p) {
  if (!p) return fail(RTP_ERR_INVALID_ARGUMENT, "null");
  p->restDensity = 450.0f;
  p->relaxCFM = 600.0f;
  p->timeStep = 0.010f;
  p->dim = 3;
  p->isArtPressureEnabled = 1;
  p->artPressureRadius = 0.006f;
  p->artPressureCoeff = 0.001f;
  p->artPressureExp = 4;
  p->isVorticityConfEnabled = 1;
  p->vorticityConfCoeff = 0.0004f;
  p->xsphViscosityCoeff = 0.0001f;
  return RTP_OK;
}

// JSON defaults: Boids.cpp:41-73 (all rules enabled).
int rtp_boids_params_default(rtp_boids_params* p) {
  if (!p) return fail(RTP_ERR_INVALID_ARGUMENT, "null");
  p->velocityScale = 0.5f;
  p->alignmentScale = 1.6f;
  p->separationScale = 1.6f;
  p->cohesionScale = 1.45f;
  return RTP_OK;
}

// JSON defaults: Clouds.cpp:67-102 (shared fluid values copied as in :307-311).
int rtp_cloud_params_default(rtp_cloud_params* p) {
  if (!p) return fail(RTP_ERR_INVALID_ARGUMENT, "null");
  p->dim = 3;
  p->timeStep = 0.010f;
  p->restDensity = 450.0f;
  p->groundHeatCoeff = 10.0f;
  p->buoyancyCoeff = 0.10f;
  p->gravCoeff = 0.0005f;
  p->adiabaticLapseRate = 5.0f;
  p->phaseTransitionRate = 0.3485f;
  p->latentHeatCoeff = 0.07f;
  p->isTempSmoothingEnabled = 1;
  p->relaxCFM = 600.0f;
  p->initVaporDensityCoeff = 0.75f;
  p->windCoeff = 1.0f;
  return RTP_OK;
}

// Constants of clouds.cl:72-89 and :951-952.
int rtp_cloud_env_reference(rtp_cloud_env* e) {
  if (!e) return fail(RTP_ERR_INVALID_ARGUMENT, "null");
  e->groundTemp0 = 293.0f;
  e->lapseRate = 3.5f;
  e->heatDecay = 3.0f;
  e->windDecayX = 0.2f;
  e->windDecayZ = 0.3f;
  e->groundNx = 0;
  e->groundNz = 0;
  return RTP_OK;
}

int rtp_create(int model, const rtp_model_params* params, void** out_handle) {
  RTP_GUARD_BEGIN
  if (!params || !out_handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create: null argument");
  *out_handle = nullptr;
  if (model < RTP_MODEL_BOIDS || model > RTP_MODEL_CLOUDS) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create: unknown model");
  if (params->maxNbParticles == 0 || params->maxNbParticles > (1ull << 28))
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create: maxNbParticles must be in [1, 2^28]");
  if (params->currNbParticles > params->maxNbParticles)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create: currNbParticles > maxNbParticles");
  if (params->dimension != 3 && params->dimension != 2)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create: dimension must be 2 or 3");
  int ndev = 0;
  const cudaError_t de = cudaGetDeviceCount(&ndev);
  if (de != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(RTP_ERR_NO_DEVICE, "rtp_create: no CUDA device");
  }
  Handle* h = new Handle();
  h->model = model;
  h->mp = *params;
  h->maxN = params->maxNbParticles;
  h->curN = params->currNbParticles;
  int rc = derive_constants(model, params, &h->gc);
  if (rc) {
    delete h;
    return rc;
  }
  h->g = make_gridk(h->gc);
  rtp_fluid_params_default(&h->fp);
  rtp_boids_params_default(&h->bp);
  rtp_cloud_params_default(&h->cp);
  rtp_cloud_env_reference(&h->env);
  rtp_target_params_default(&h->tp);
  h->traj = TargetTrajectory(params->boxSize[0]);  // Boids.cpp:80
  h->iters = (model == RTP_MODEL_CLOUDS) ? 1u : 2u;  // Clouds.cpp:111, Fluids.cpp:81
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  rc = alloc_buffers(h);
  if (!rc) {
    Launcher L;
    L.stream = h->stream;
    rc = launch_reset_cell_ids(h->cellId, (uint32_t)h->maxN, h->gc.numCells, L);
  }
  if (!rc) {
    e = cudaEventCreate(&h->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->t1);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  }
  if (rc) {
    free_handle(h);
    return rc;
  }
  *out_handle = h;
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_destroy(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return RTP_OK;
  Handle* h = H(handle);
  cudaStreamSynchronize(h->stream);
  free_handle(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_update(void* handle, uint32_t nsteps) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_update: null handle");
  return run_steps(H(handle), nsteps);
  RTP_GUARD_END
}

int rtp_reset(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_reset: null handle");
  Handle* h = H(handle);
  if (h->isBatch) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_reset: a batch has no preset cases (upload positions)");
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  rtp_fluid_params_default(&h->fp);
  rtp_boids_params_default(&h->bp);
  rtp_cloud_params_default(&h->cp);
  // FluidKernelInputs.dim / CloudKernelInputs.dim follow the model (Fluids.cpp:234, Clouds.cpp:289).
  h->fp.dim = h->cp.dim = h->mp.dimension == 2 ? 2u : 3u;
  h->iters = (h->model == RTP_MODEL_CLOUDS) ? 1u : 2u;
  h->boidsDt = 0.1f;
  // The JSON defaults switch the target off (Boids.cpp:233); its trajectory keeps going.
  rtp_target_params_default(&h->tp);
  h->targetVisible = false;
  invalidate(h);
  return init_case(h);
  RTP_GUARD_END
}

int rtp_clouds_init(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_clouds_init: null handle");
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_CLOUDS) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_clouds_init: not a clouds model");
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(cloud_init(h->g, make_cloudk(h), h->pos, (uint32_t)h->curN, h->temp, h->vapor, h->cloud, h->buoy, L));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_set_fluid_params(void* handle, const rtp_fluid_params* p) {
  if (!handle || !p) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_fluid_params: null argument");
  if (!(p->restDensity > 0.0f) || !(p->timeStep > 0.0f))
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_fluid_params: restDensity and timeStep must be > 0");
  H(handle)->fp = *p;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_get_fluid_params(void* handle, rtp_fluid_params* p) {
  if (!handle || !p) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_get_fluid_params: null argument");
  *p = H(handle)->fp;
  return RTP_OK;
}

int rtp_set_jacobi_iterations(void* handle, uint32_t iters) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  if (iters > 64) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_jacobi_iterations: at most 64");
  H(handle)->iters = iters;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_set_boids_params(void* handle, const rtp_boids_params* p) {
  if (!handle || !p) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_boids_params: null argument");
  H(handle)->bp = *p;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_set_boids_time_step(void* handle, float dt) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  H(handle)->boidsDt = dt;
  invalidate(H(handle));
  return RTP_OK;
}

// Target group defaults, Boids.cpp:45-51.
int rtp_target_params_default(rtp_target_params* p) {
  if (!p) return fail(RTP_ERR_INVALID_ARGUMENT, "null");
  p->enabled = 0;
  p->visible = 1;
  p->radiusEffect = 2.0f;
  p->signEffect = 1;
  return RTP_OK;
}

// Boids::transferJsonInputsToModel, target part (Boids.cpp:193-202).
int rtp_set_target(void* handle, const rtp_target_params* p) {
  RTP_GUARD_BEGIN
  if (!handle || !p) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_target: null argument");
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_BOIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_target: boids only");
  if (std::isnan(p->radiusEffect)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_target: radiusEffect is NaN");
  if (p->enabled && !h->targetTrack) {
    RTP_TRY(dalloc(h, &h->targetTrack, 1 + (size_t)kTargetChunk));
    RTP_CUDA(cudaMallocHost((void**)&h->targetHost, sizeof(float4) * (1 + (size_t)kTargetChunk)));
    RTP_CUDA(cudaEventCreateWithFlags(&h->targetUp, cudaEventDisableTiming));
  }
  h->tp = *p;
  h->tp.enabled = p->enabled ? 1 : 0;
  h->targetVisible = h->tp.enabled && p->visible;  // Target::show after activate (Target.hpp:25)
  invalidate(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_get_target(void* handle, float pos[3], int* activated, int* visible) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_get_target: null handle");
  const Handle* h = H(handle);
  const bool boids = h->model == RTP_MODEL_BOIDS;
  if (pos)
    for (int k = 0; k < 3; ++k) pos[k] = boids ? h->traj.pos()[k] : 0.0f;
  if (activated) *activated = boids && h->tp.enabled;
  if (visible) *visible = boids && h->targetVisible;
  return RTP_OK;
}

int rtp_set_cloud_params(void* handle, const rtp_cloud_params* p) {
  if (!handle || !p) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_cloud_params: null argument");
  H(handle)->cp = *p;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_set_cloud_environment(void* handle, const rtp_cloud_env* env, const float* groundTemp) {
  RTP_GUARD_BEGIN
  if (!handle || !env) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_cloud_environment: null argument");
  Handle* h = H(handle);
  const bool field = groundTemp && env->groundNx >= 2 && env->groundNz >= 2;
  if (h->ground) {
    RTP_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(h->ground);
    h->ground = nullptr;
  }
  h->env = *env;
  if (field) {
    const size_t cnt = (size_t)env->groundNx * env->groundNz;
    RTP_CUDA(cudaMalloc((void**)&h->ground, sizeof(float) * cnt));
    RTP_CUDA(cudaMemcpy(h->ground, groundTemp, sizeof(float) * cnt, cudaMemcpyHostToDevice));
  } else {
    h->env.groundNx = h->env.groundNz = 0;
  }
  invalidate(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_set_nb_particles(void* handle, uint64_t n) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  if (H(handle)->isBatch) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_nb_particles: scene sizes of a batch are fixed");
  if (n > H(handle)->maxN) return fail(RTP_ERR_CAPACITY, "rtp_set_nb_particles: n > maxNbParticles");
  H(handle)->curN = n;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_get_nb_particles(void* handle, uint64_t* n) {
  if (!handle || !n) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  *n = H(handle)->curN;
  return RTP_OK;
}

int rtp_set_boundary(void* handle, int boundary) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  if (boundary != RTP_BOUNDARY_BOUNCING_WALL && boundary != RTP_BOUNDARY_CYCLIC_WALL)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_boundary: unknown boundary");
  H(handle)->boundary = boundary;
  invalidate(H(handle));
  return RTP_OK;
}

int rtp_set_dimension(void* handle, uint32_t dim) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  if (dim != 2 && dim != 3) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_dimension: dimension must be 2 or 3");
  if (H(handle)->isBatch) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_dimension: batches are 3D");
  // Model::setDimension (Model.hpp:109-113): store, then reset.
  H(handle)->mp.dimension = dim;
  return rtp_reset(handle);
}

int rtp_set_case(void* handle, int pcase) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  H(handle)->mp.pCase = pcase;
  return RTP_OK;
}

int rtp_pause(void* handle, int pause) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  H(handle)->paused = pause != 0;
  return RTP_OK;
}

static int buffer_info(Handle* h, int buf, void** dptr, size_t* elem, uint64_t* cap) {
  *cap = h->maxN;
  switch (buf) {
    case RTP_BUF_POS: *dptr = h->pos; *elem = 16; break;
    case RTP_BUF_VEL: *dptr = h->vel; *elem = 16; break;
    case RTP_BUF_PRED_POS: *dptr = h->predFinal; *elem = 16; break;
    case RTP_BUF_DENSITY: *dptr = h->density; *elem = 4; break;
    case RTP_BUF_LAMBDA: *dptr = h->lambda; *elem = 4; break;
    case RTP_BUF_TEMP: *dptr = h->temp; *elem = 4; break;
    case RTP_BUF_VAPOR: *dptr = h->vapor; *elem = 4; break;
    case RTP_BUF_CLOUD: *dptr = h->cloud; *elem = 4; break;
    case RTP_BUF_BUOYANCY: *dptr = h->buoy; *elem = 4; break;
    case RTP_BUF_ID: *dptr = h->ids; *elem = 4; break;
    case RTP_BUF_CELL_ID: *dptr = h->cellId; *elem = 4; break;
    case RTP_BUF_CELL_TABLE: *dptr = h->tableRef; *elem = 8; *cap = h->gc.numCells; break;
    case RTP_BUF_VORTICITY: *dptr = h->vort; *elem = 16; break;
    case RTP_BUF_ACC: *dptr = h->acc; *elem = 16; break;
    case RTP_BUF_LAMBDA_TOTAL: *dptr = h->lamTot; *elem = 4; break;
    case RTP_BUF_COLOR: *dptr = h->col; *elem = 16; break;
    case RTP_BUF_CAMERA_DIST: *dptr = h->camDist; *elem = 4; break;
    case RTP_BUF_DRAW_ORDER: *dptr = h->drawOrder; *elem = 4; break;
    case RTP_BUF_GRID_DETECTOR: *dptr = h->gridDet; *elem = 32; *cap = h->gc.numCells; break;
    default: return fail(RTP_ERR_INVALID_ARGUMENT, "unknown buffer");
  }
  if (!*dptr) return fail(RTP_ERR_INVALID_ARGUMENT, "buffer not used by this model");
  return RTP_OK;
}

int rtp_upload(void* handle, int buffer, const void* host, uint64_t count) {
  RTP_GUARD_BEGIN
  if (!handle || (count && !host)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_upload: null argument");
  Handle* h = H(handle);
  void* d;
  size_t elem;
  uint64_t cap;
  RTP_TRY(buffer_info(h, buffer, &d, &elem, &cap));
  if (buffer == RTP_BUF_CELL_TABLE || buffer == RTP_BUF_CELL_ID)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_upload: derived buffer is read-only");
  if (count > cap) return fail(RTP_ERR_CAPACITY, "rtp_upload: count exceeds capacity");
  RTP_CUDA(cudaMemcpyAsync(d, host, elem * count, cudaMemcpyHostToDevice, h->stream));
  if (buffer == RTP_BUF_POS) RTP_TRY(ws_forget(h));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_download(void* handle, int buffer, void* host, uint64_t count) {
  RTP_GUARD_BEGIN
  if (!handle || (count && !host)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_download: null argument");
  Handle* h = H(handle);
  void* d;
  size_t elem;
  uint64_t cap;
  RTP_TRY(buffer_info(h, buffer, &d, &elem, &cap));
  if (count > cap) return fail(RTP_ERR_CAPACITY, "rtp_download: count exceeds capacity");
  if (buffer == RTP_BUF_CELL_TABLE) {
    Launcher L;
    L.stream = h->stream;
    RTP_TRY(launch_cell_table_to_reference(h->g, h->table, h->tableRef, L));
  }
  RTP_CUDA(cudaMemcpyAsync(host, d, elem * count, cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return check_fault(h);
  RTP_GUARD_END
}

int rtp_device_ptr(void* handle, int buffer, void** dptr) {
  if (!handle || !dptr) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_device_ptr: null argument");
  size_t elem;
  uint64_t cap;
  return buffer_info(H(handle), buffer, dptr, &elem, &cap);
}

int rtp_stream(void* handle, void** stream) {
  if (!handle || !stream) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  *stream = (void*)H(handle)->stream;
  return RTP_OK;
}

int rtp_update_host(void* handle, const void* posIn, const void* velIn, uint64_t count, uint32_t nsteps, void* posOut,
                    void* velOut) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_update_host: null handle");
  Handle* h = H(handle);
  if (count != h->curN) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_update_host: count must equal the particle count");
  const size_t bytes = sizeof(float4) * (size_t)count;
  // One fluids or boids step on pinned buffers: its first kernel reads them and its last
  // writes them (no separate copies); other cases copy with cudaMemcpyAsync around rtp_update.
  const bool direct = h->model == RTP_MODEL_FLUIDS || h->model == RTP_MODEL_BOIDS;
  if (direct && nsteps == 1 && count > 0 && !h->paused && !h->profiling) {
    void *ip, *iv, *op, *ov;
    if (pinned_device_ptr(posIn, &ip) && pinned_device_ptr(velIn, &iv) && pinned_device_ptr(posOut, &op) &&
        pinned_device_ptr(velOut, &ov)) {
      HostIO io;
      io.inPos = (const float4*)ip;
      io.inVel = (const float4*)iv;
      io.outPos = (float4*)op;
      io.outVel = (float4*)ov;
      cudaGraphExec_t exec = nullptr;
      RTP_TRY(host_graph(h, io, &exec));
      if (posIn) RTP_TRY(ws_forget(h));
      if (target_on(h)) RTP_TRY(feed_target(h, 1));
      RTP_CUDA(cudaGraphLaunch(exec, h->stream));
      h->hasStep = true;
      RTP_CUDA(cudaStreamSynchronize(h->stream));
      return check_fault(h);
    }
  }
  if (posIn && bytes) {
    RTP_CUDA(cudaMemcpyAsync(h->pos, posIn, bytes, cudaMemcpyHostToDevice, h->stream));
    RTP_TRY(ws_forget(h));
  }
  if (velIn && bytes) RTP_CUDA(cudaMemcpyAsync(h->vel, velIn, bytes, cudaMemcpyHostToDevice, h->stream));
  RTP_TRY(run_steps(h, nsteps));
  if (posOut && bytes) RTP_CUDA(cudaMemcpyAsync(posOut, h->pos, bytes, cudaMemcpyDeviceToHost, h->stream));
  if (velOut && bytes) RTP_CUDA(cudaMemcpyAsync(velOut, h->vel, bytes, cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return check_fault(h);
  RTP_GUARD_END
}

int rtp_synchronize(void* handle) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  RTP_CUDA(cudaStreamSynchronize(H(handle)->stream));
  return check_fault(H(handle));
}

int rtp_enable_profiling(void* handle, int enable) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  H(handle)->profiling = enable != 0;
  return RTP_OK;
}

int rtp_is_profiling_enabled(void* handle, int* enabled) {
  if (!handle || !enabled) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  *enabled = H(handle)->profiling ? 1 : 0;
  return RTP_OK;
}

int rtp_get_kernel_times(void* handle, rtp_kernel_time* out, uint32_t capacity, uint32_t* count) {
  RTP_GUARD_BEGIN
  if (!handle || !count) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  uint32_t i = 0;
  for (const auto& kv : h->stats) {
    if (out && i < capacity) {
      std::memset(out[i].name, 0, sizeof out[i].name);
      std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
      out[i].launches = kv.second.launches;
      out[i].total_ms = kv.second.ms;
    }
    ++i;
  }
  *count = i;
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_reset_kernel_times(void* handle) {
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  H(handle)->stats.clear();
  return RTP_OK;
}

int rtp_time_steps(void* handle, uint32_t nsteps, uint64_t flush_bytes, double* total_ms) {
  RTP_GUARD_BEGIN
  if (!handle || !total_ms) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  *total_ms = 0.0;
  if (h->curN == 0 || nsteps == 0) return RTP_OK;
  if (flush_bytes && flush_bytes != h->flushBytes) {
    if (h->flush) cudaFree(h->flush);
    h->flush = nullptr;
    h->flushBytes = 0;
    RTP_CUDA(cudaMalloc(&h->flush, flush_bytes));
    h->flushBytes = flush_bytes;
  }
  if (!h->graphValid || h->graphProfiled != h->profiling) RTP_TRY(build_graph(h));
  for (uint32_t s = 0; s < nsteps; ++s) {
    if (const uint32_t k = target_feed_size(h, s, nsteps)) RTP_TRY(feed_target(h, k));
    if (flush_bytes) RTP_CUDA(cudaMemsetAsync(h->flush, (int)(s & 0xff), flush_bytes, h->stream));
    RTP_CUDA(cudaEventRecord(h->t0, h->stream));
    RTP_CUDA(cudaGraphLaunch(h->graph, h->stream));
    RTP_CUDA(cudaEventRecord(h->t1, h->stream));
    RTP_CUDA(cudaEventSynchronize(h->t1));
    float ms = 0.0f;
    RTP_CUDA(cudaEventElapsedTime(&ms, h->t0, h->t1));
    *total_ms += ms;
    if (h->graphProfiled) RTP_TRY(collect_profile(h));
  }
  h->hasStep = true;
  return check_fault(h);
  RTP_GUARD_END
}

int rtp_get_metrics(void* handle, rtp_metrics* out) {
  RTP_GUARD_BEGIN
  if (!handle || !out) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  std::memset(out, 0, sizeof *out);
  if (h->model == RTP_MODEL_BOIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_get_metrics: fluids and clouds only");
  const uint32_t n = (uint32_t)h->curN;
  if (n == 0) return RTP_OK;  // no particles: all zero
  if (!h->hasStep) return fail(RTP_ERR_STATE, "rtp_get_metrics: run a step first (the cell table is built by update)");
  RTP_CUDA(cudaMemsetAsync(h->mAcc, 0, sizeof(double) * 4, h->stream));
  RTP_CUDA(cudaMemsetAsync(h->mHist, 0, sizeof(uint32_t) * 80, h->stream));
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(fluid_metrics(h->g, fluidk_of(h), h->predFinal, h->vel, h->table, n, h->mAcc, h->mHist, L));
  if (h->pairs.count) RTP_TRY(pair_list_stats(h->pairs, n, h->mHist + 70, L));
  double acc[4];
  uint32_t hist[80];
  RTP_CUDA(cudaMemcpyAsync(acc, h->mAcc, sizeof acc, cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaMemcpyAsync(hist, h->mHist, sizeof hist, cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  out->meanDensityError = acc[0] / n;
  float mx;
  std::memcpy(&mx, &hist[64], sizeof mx);
  out->maxDensityError = mx;
  out->kineticEnergy = acc[1];
  out->meanNeighbours = acc[2] / n;
  out->meanCompression = acc[3] / n;
  for (int i = 0; i < 64; ++i) out->neighbourHist[i] = hist[i];
  out->pairListOverflows = hist[70];
  out->pairListMax = hist[71];
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_set_warm_start(void* handle, const rtp_mlp* net, const rtp_warm_start_config* cfg) {
  RTP_GUARD_BEGIN
  if (!handle || !cfg) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_warm_start: null argument");
  Handle* h = H(handle);
  if (h->model == RTP_MODEL_BOIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_warm_start: fluids and clouds only");
  if (h->model == RTP_MODEL_CLOUDS && cfg->enabled && cfg->relaxAllIterations)
    return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_warm_start: clouds take no relaxation of every iteration");
  if (!cfg->enabled) {
    h->wsOn = false;
    invalidate(h);
    return RTP_OK;
  }
  if (!net) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_warm_start: null network");
  if (cfg->extraIterations > 64) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_warm_start: at most 64 extra iterations");
  for (int k = 0; k < RTP_MLP_IN; ++k)
    if (!std::isfinite(net->inMean[k]) || !std::isfinite(net->inScale[k]))
      return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_warm_start: non-finite normalisation");
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  RTP_TRY(ws_alloc(h));
  RTP_TRY(mlp_upload_packed(*net, h->mlpTmp, h->mlpBlock, h->stream));
  h->wsOn = true;
  h->wsExtra = cfg->extraIterations;
  h->wsRelaxAll = cfg->relaxAllIterations != 0;
  h->wsTol = cfg->guardTolerance;
  invalidate(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_enable_solver_stats(void* handle, int enable) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  Handle* h = H(handle);
  if (h->model == RTP_MODEL_BOIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_enable_solver_stats: fluids and clouds only");
  if (enable) RTP_TRY(ws_alloc(h));
  h->statsOn = enable != 0;
  invalidate(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_get_solver_stats(void* handle, rtp_solver_stats* out) {
  RTP_GUARD_BEGIN
  if (!handle || !out) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  std::memset(out, 0, sizeof *out);
  if (!h->solverStats) return RTP_OK;
  SolverStatsDev d;
  RTP_CUDA(cudaMemcpyAsync(&d, h->solverStats, sizeof d, cudaMemcpyDeviceToHost, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  out->steps = d.steps;
  out->reruns = d.reruns;
  out->sumDensityError = d.sumErr;
  out->maxDensityError = d.maxErr;
  out->sumFirstError = d.sumFirst;
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_reset_solver_stats(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  Handle* h = H(handle);
  if (!h->solverStats) return RTP_OK;
  RTP_CUDA(cudaMemsetAsync(h->solverStats, 0, sizeof(SolverStatsDev), h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_record_warm_start_samples(void* handle, uint32_t referenceIterations, uint32_t stride, uint32_t phase,
                                  float* d_features, float* d_targets, uint64_t capacity, uint64_t* written) {
  RTP_GUARD_BEGIN
  if (!handle || !written) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_record_warm_start_samples: null argument");
  *written = 0;
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_FLUIDS || h->isBatch)
    return fail(RTP_ERR_NOT_SUPPORTED, "rtp_record_warm_start_samples: single fluids scenes only");
  if (referenceIterations == 0 || referenceIterations > 64)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_record_warm_start_samples: referenceIterations must be in [1, 64]");
  if (stride == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_record_warm_start_samples: stride must be > 0");
  const uint32_t n = (uint32_t)h->curN;
  const uint64_t avail = phase < n ? (uint64_t)(n - phase + stride - 1) / stride : 0;
  const uint32_t count = (uint32_t)std::min<uint64_t>(avail, capacity);
  if (count && (!d_features || !d_targets))
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_record_warm_start_samples: null sample arrays");
  if (n == 0 || h->paused) return RTP_OK;
  RTP_TRY(ws_alloc_rec(h));
  RTP_TRY(record_sample_step(h, referenceIterations, stride, phase, d_features, d_targets, count));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  h->hasStep = true;
  *written = count;
  return RTP_OK;
  RTP_GUARD_END
}

static int check_trainable(Handle* h, const char* who) {
  if (h->model == RTP_MODEL_BOIDS || h->isBatch)
    return fail(RTP_ERR_NOT_SUPPORTED, std::string(who) + ": single fluids or clouds scenes only");
  if (h->curN == 0) return fail(RTP_ERR_STATE, std::string(who) + ": no particles");
  if (h->paused) return fail(RTP_ERR_STATE, std::string(who) + ": the model is paused");
  return RTP_OK;
}

int rtp_warm_start_loss_grad(void* handle, const rtp_mlp* net, float* d_dy, double* loss) {
  RTP_GUARD_BEGIN
  if (!handle || !net || !loss) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_warm_start_loss_grad: null argument");
  Handle* h = H(handle);
  RTP_TRY(check_trainable(h, "rtp_warm_start_loss_grad"));
  const uint32_t n = (uint32_t)h->curN;
  RTP_TRY(ws_alloc_train(h));
  RTP_TRY(ws_trainer_set_net(h->trainer, *net, h->stream));
  Launcher L;
  L.stream = h->stream;
  const bool clouds = h->model == RTP_MODEL_CLOUDS;
  if (clouds) {
    // The clouds presort advances the thermodynamic state: run it on a copy of it.
    RTP_TRY(clouds_presort_keep_state(h, L));
    RTP_TRY(cloud_train_pass(h, L, false));
  } else {
    RTP_TRY(fluids_presort(h, L, fluidk_of(h), true));
    RTP_TRY(ws_train_pass(h, L, false));
  }
  if (d_dy) RTP_TRY(ws_scatter_by_id(h->idsS, h->trDy, kMlpOut, n, d_dy, L));
  RTP_TRY(ws_train_loss(h, loss));
  return check_fault(h);
  RTP_GUARD_END
}

int rtp_train_warm_start_rollout(void* handle, const rtp_train_config* cfg, uint32_t steps, uint32_t extraIterations,
                                 int init, rtp_mlp* net, float* loss_history) {
  RTP_GUARD_BEGIN
  if (!handle || !cfg || !net) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_train_warm_start_rollout: null argument");
  Handle* h = H(handle);
  RTP_TRY(check_trainable(h, "rtp_train_warm_start_rollout"));
  if (extraIterations > 64) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_train_warm_start_rollout: extraIterations > 64");
  const uint32_t n = (uint32_t)h->curN;
  RTP_TRY(ws_alloc_train(h));
  Launcher L;
  L.stream = h->stream;
  const FluidK fk = fluidk_of(h);
  const bool clouds = h->model == RTP_MODEL_CLOUDS;
  for (uint32_t s = 0; s < steps; ++s) {
    if (clouds) RTP_TRY(clouds_presort(h, L));
    else RTP_TRY(fluids_presort(h, L, fk, true));
    bool haveFeatures = false;
    if (s == 0) {
      if (init) {
        if (clouds)
          RTP_TRY(cloud_ws_lambda(h->g, fk, make_cloudk(h), h->predA, h->velS, h->tempS, h->buoyS, h->table, n,
                                  h->trLam, h->density, h->pairs, h->predLam, h->trFeats, nullptr, L));
        else
          RTP_TRY(ws_lambda_record(h->g, fk, h->predA, h->velS, h->table, n, h->trLam, h->density, h->lamTot, h->pairs,
                                   1, 0, h->trFeats, n, L));
        RTP_TRY(ws_init_net(h->trFeats, n, cfg->seed, *net, h->stream));
        haveFeatures = true;
      }
      RTP_TRY(ws_trainer_set_net(h->trainer, *net, h->stream));
    }
    if (clouds) RTP_TRY(cloud_train_pass(h, L, haveFeatures));
    else RTP_TRY(ws_train_pass(h, L, haveFeatures));
    double loss = 0.0;
    RTP_TRY(ws_train_loss(h, &loss));
    if (loss_history) loss_history[s] = (float)loss;
    const double frac = steps > 1 ? (double)s / (double)(steps - 1) : 0.0;
    const double lrScale = cfg->finalLrFraction + (1.0 - cfg->finalLrFraction) * 0.5 * (1.0 + std::cos(M_PI * frac));
    RTP_TRY(ws_trainer_adam_step(h->trainer, h->trFeats, h->trDy, n, *cfg, lrScale, h->stream));
    // The simulation advances with the updated network (the states it trains on are the ones
    // the warm-started solver itself produces).
    if (clouds) {
      RTP_TRY(clouds_solve_post(h, L, ws_trainer_block(h->trainer), extraIterations, false));
    } else {
      RTP_TRY(ws_first_iteration(h, L, fk, ws_trainer_block(h->trainer), extraIterations, false));
      h->predFinal = h->predB;
      RTP_TRY(fluid_post(h->g, fk, h->predB, h->velS, h->vort, h->table, n, h->idsS, h->pos, h->vel, h->ids, h->pairs,
                         L, false, HostIO{}, h->predLam));
    }
    h->hasStep = true;
  }
  RTP_TRY(ws_trainer_get_net(h->trainer, *net, h->stream));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return check_fault(h);
  RTP_GUARD_END
}

int rtp_fill_fluid_color(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_FLUIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_fill_fluid_color: fluids only");
  if (!h->hasStep) return fail(RTP_ERR_STATE, "rtp_fill_fluid_color: run a step first (density)");
  if (!h->col) RTP_TRY(dalloc(h, &h->col, h->maxN));
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(side_fluid_color(h->density, (uint32_t)h->curN, h->fp.restDensity, h->col, L));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_fill_color_float(void* handle, int buffer, float minVal, float maxVal) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  Handle* h = H(handle);
  if (buffer != RTP_BUF_DENSITY && buffer != RTP_BUF_LAMBDA && buffer != RTP_BUF_TEMP && buffer != RTP_BUF_VAPOR &&
      buffer != RTP_BUF_CLOUD && buffer != RTP_BUF_BUOYANCY && buffer != RTP_BUF_LAMBDA_TOTAL)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_fill_color_float: not a per-particle float buffer");
  void* q;
  size_t elem;
  uint64_t cap;
  RTP_TRY(buffer_info(h, buffer, &q, &elem, &cap));
  if (!h->col) RTP_TRY(dalloc(h, &h->col, h->maxN));
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(side_color_float((const float*)q, (uint32_t)h->curN, minVal, maxVal, h->col, L));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_fill_camera_order(void* handle, const float cameraPos[3]) {
  RTP_GUARD_BEGIN
  if (!handle || !cameraPos) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  const uint32_t M = (uint32_t)h->maxN;
  if (!h->camDist) {
    RTP_TRY(dalloc(h, &h->camDist, M));
    RTP_TRY(dalloc(h, &h->camSorted, M));
    RTP_TRY(dalloc(h, &h->drawOrder, M));
    const SortPlan plan = make_sort_plan(M, 20);  // keys <= FAR_DIST < 2^20
    RTP_CUDA(cudaMalloc(&h->camSortMem, sort_scratch_bytes(plan)));
    h->allocs.push_back(h->camSortMem);
    sort_scratch_carve(plan, h->camSortMem, h->camSS);
  }
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(side_camera_dist(h->pos, (uint32_t)h->curN, M, cameraPos, h->camDist, L));
  const SortPlan plan = make_sort_plan(M, 20);
  RTP_TRY(launch_sort_clear(plan, h->camSS, L));
  RTP_TRY(launch_sort_histogram(plan, h->camDist, h->camSS, L));
  GatherList gl;
  gl.fault = h->faultDev;
  gl.perm = h->drawOrder;
  RTP_TRY(launch_sort_passes(plan, h->camDist, h->camSorted, h->camSS, gl, L));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_fill_grid_detector(void* handle) {
  RTP_GUARD_BEGIN
  if (!handle) return fail(RTP_ERR_INVALID_ARGUMENT, "null handle");
  Handle* h = H(handle);
  if (h->isBatch) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_fill_grid_detector: one grid per scene in a batch");
  if (!h->gridDet) RTP_TRY(dalloc(h, &h->gridDet, (size_t)h->gc.numCells * 8));
  Launcher L;
  L.stream = h->stream;
  RTP_TRY(side_grid_detector(h->g, h->pos, (uint32_t)h->curN, h->gridDet, L));
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_create_batch(uint32_t nscenes, const rtp_batch_scene* scenes, float effectRadius, uint32_t maxNbPartsInCell,
                     void** out_handle) {
  RTP_GUARD_BEGIN
  if (!scenes || !out_handle) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: null argument");
  *out_handle = nullptr;
  if (nscenes == 0 || nscenes > 65535) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: 1 to 65535 scenes");
  if (!(effectRadius > 0.0f)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: effectRadius must be > 0");
  uint64_t total = 0;
  for (uint32_t s = 0; s < nscenes; ++s) {
    if (scenes[s].nbParticles == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: empty scene");
    for (int a = 0; a < 3; ++a)
      if (!(scenes[s].boxSize[a] > 0.0f)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: empty box");
    total += scenes[s].nbParticles;
  }
  if (total > (1ull << 28)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_create_batch: more than 2^28 particles");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(RTP_ERR_NO_DEVICE, "rtp_create_batch: no CUDA device");
  }
  Handle* h = new Handle();
  h->model = RTP_MODEL_FLUIDS;
  h->isBatch = true;
  h->batchH = effectRadius;
  h->sceneDesc.assign(scenes, scenes + nscenes);
  h->sceneOff.resize(nscenes);
  uint64_t off = 0;
  for (uint32_t s = 0; s < nscenes; ++s) {
    h->sceneOff[s] = off;
    off += scenes[s].nbParticles;
  }
  h->mp.currNbParticles = h->mp.maxNbParticles = total;
  for (int a = 0; a < 3; ++a) h->mp.boxSize[a] = scenes[0].boxSize[a];
  h->mp.dimension = 3;
  h->mp.pCase = RTP_CASE_INVALID;
  h->mp.maxNbPartsInCell = maxNbPartsInCell;
  h->maxN = h->curN = total;
  int rc = batch_grids(h, 1.0f);
  if (rc) {
    delete h;
    return rc;
  }
  rtp_fluid_params_default(&h->fp);
  rtp_boids_params_default(&h->bp);
  rtp_cloud_params_default(&h->cp);
  rtp_cloud_env_reference(&h->env);
  h->iters = 2u;
  cudaGetDevice(&h->device);
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  rc = alloc_buffers(h);
  if (!rc) rc = dalloc(h, &h->dScenes, nscenes);
  if (!rc) rc = dalloc(h, &h->dSceneOf, total);
  if (!rc) {
    std::vector<uint16_t> so(total);
    for (uint32_t s = 0; s < nscenes; ++s)
      std::fill(so.begin() + h->sceneOff[s], so.begin() + h->sceneOff[s] + scenes[s].nbParticles, (uint16_t)s);
    e = cudaMemcpy(h->dSceneOf, so.data(), sizeof(uint16_t) * total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy(sceneOf)");
  }
  if (!rc) rc = batch_upload_scenes(h);
  if (!rc) {
    e = cudaEventCreate(&h->t0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->t1);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate");
  }
  if (rc) {
    free_handle(h);
    return rc;
  }
  *out_handle = h;
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_batch_scene_range(void* handle, uint32_t scene, uint64_t* offset, uint64_t* count) {
  if (!handle || !offset || !count) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  if (!h->isBatch) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_batch_scene_range: not a batch");
  if (scene >= h->sceneDesc.size()) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_batch_scene_range: no such scene");
  *offset = h->sceneOff[scene];
  *count = h->sceneDesc[scene].nbParticles;
  return RTP_OK;
}

int rtp_batch_scene_constants(void* handle, uint32_t scene, rtp_grid_constants* out) {
  if (!handle || !out) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  if (!h->isBatch) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_batch_scene_constants: not a batch");
  if (scene >= h->sceneDesc.size()) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_batch_scene_constants: no such scene");
  *out = h->sceneConst[scene];
  return RTP_OK;
}

int rtp_batch_scene_key_base(void* handle, uint32_t scene, uint32_t* base) {
  if (!handle || !base) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  if (!h->isBatch || scene >= h->hScenes.size()) return fail(RTP_ERR_INVALID_ARGUMENT, "no such batch scene");
  *base = h->hScenes[scene].g.base;
  return RTP_OK;
}

int rtp_set_tuning(void* handle, const rtp_tuning* t) {
  RTP_GUARD_BEGIN
  if (!handle || !t) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_FLUIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_set_tuning: fluids only");
  if (t->lanes != 2 && t->lanes != 4 && t->lanes != 8) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_tuning: lanes 2, 4 or 8");
  if (!h->isBatch && t->cellFactor != 1.0f)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_tuning: a single scene keeps the reference's grid (cellFactor 1)");
  if (!(t->cellFactor >= 1.0f && t->cellFactor <= 4.0f))
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_tuning: cellFactor in [1, 4]");
  if (t->tiledSweeps > 1) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_set_tuning: tiledSweeps 0 or 1");
  RTP_CUDA(cudaStreamSynchronize(h->stream));
  if (h->isBatch && t->cellFactor != h->cellFactor) {
    const float old = h->cellFactor;
    int rc = batch_grids(h, t->cellFactor);
    if (!rc && (h->gc.numCells > h->tableCells || h->gc.keyBits > h->sortKeyBits))
      rc = fail(RTP_ERR_CAPACITY, "rtp_set_tuning: grid larger than allocated");
    if (rc) {
      batch_grids(h, old);
      return rc;
    }
    RTP_TRY(batch_upload_scenes(h));
    h->hasStep = false;
  }
  h->lanes = t->lanes;
  h->tiles = t->tiledSweeps;
  invalidate(h);
  return RTP_OK;
  RTP_GUARD_END
}

int rtp_get_tuning(void* handle, rtp_tuning* t) {
  if (!handle || !t) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  t->lanes = H(handle)->lanes;
  t->cellFactor = H(handle)->cellFactor;
  t->tiledSweeps = H(handle)->tiles;
  return RTP_OK;
}

int rtp_autotune(void* handle, uint32_t steps, rtp_tune_result* out) {
  RTP_GUARD_BEGIN
  if (!handle || !out) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  Handle* h = H(handle);
  if (h->model != RTP_MODEL_FLUIDS) return fail(RTP_ERR_NOT_SUPPORTED, "rtp_autotune: fluids only");
  if (steps == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_autotune: steps must be > 0");
  std::memset(out, 0, sizeof *out);
  const uint32_t lanes[3] = {2, 4, 8};
  const float factors[4] = {1.0f, 1.25f, 1.5f, 2.0f};
  const int nf = h->isBatch ? 4 : 1;
  const uint32_t nt = h->isBatch ? 1u : 2u;  // tiled sweeps: single scenes only
  double best = 1e300;
  rtp_tuning bestT{4, 1.0f, 0u};
  for (int f = 0; f < nf; ++f)
    for (uint32_t tl = 0; tl < nt; ++tl)
      for (int l = 0; l < 3; ++l) {
        rtp_tuning t{lanes[l], factors[f], tl};
        if (rtp_set_tuning(handle, &t) != RTP_OK) continue;
        RTP_TRY(run_steps(h, 2));
        double ms = 0.0;
        RTP_TRY(rtp_time_steps(handle, steps, 256ull << 20, &ms));
        ms /= steps;
        if (out->tried < RTP_TUNE_MAX_CANDIDATES) {
          out->candidates[out->tried] = t;
          out->msPerStep[out->tried] = ms;
          out->tried += 1;
        }
        if (ms < best) {
          best = ms;
          bestT = t;
        }
      }
  RTP_TRY(rtp_set_tuning(handle, &bestT));
  out->best = bestT;
  out->bestMsPerStep = best;
  return RTP_OK;
  RTP_GUARD_END
}

}  // extern "C"
