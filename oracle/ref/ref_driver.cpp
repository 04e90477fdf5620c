// ref_driver.cpp - runs the reference's own step kernels (generated into oracle/_ref/ by
// build_ref.py from physics/ocl/kernels/*.cl) on the CPU, in the order of the reference's
// update() functions, behind the same C entry points as the oracle (prefix ref_).
//
// TEST INFRASTRUCTURE ONLY: used to check the oracle and to produce golden fixtures.
// Kernels are called once per work-item in an OpenMP loop; get_global_id() reads the
// thread-local index set before each call.  The only step not taken from the reference's
// kernels is the radix sort, replaced by its contract (a stable sort by cell key and a
// gather of the payloads, RadixSort.cpp:122-189).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "../oracle.h"
#include "clshim.hpp"

rtp_grid_constants ref_consts;

namespace clshim {
thread_local uint g_global_id = 0;
thread_local uint g_global_size = 0;
}  // namespace clshim

#include "ref_boids.cpp"
#include "ref_clouds.cpp"
#include "ref_fluids.cpp"

// Physics::PerlinNoise (physics/utils/PerlinNoise.cpp, copied by build_ref.py with the
// utils/Math.hpp it includes); Target.cpp itself needs spdlog and nlohmann/json, absent here.
#if __has_include("perlin/PerlinNoise.cpp")
#include "perlin/PerlinNoise.cpp"
#define REF_HAS_PERLIN 1
#endif

namespace {

using clshim::float4;
using clshim::uint2;

template <class K>
void run(uint32_t n, K&& kernel) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    clshim::g_global_id = (uint32_t)i;
    clshim::g_global_size = n;
    kernel();
  }
}

inline float4* F4(float* p) { return reinterpret_cast<float4*>(p); }

// The stable-sort contract of RadixSort::sort plus the payload gathers.
struct Sorted {
  std::vector<uint32_t> perm;
};

void sort_keys(uint32_t n, std::vector<uint32_t>& keys, std::vector<uint32_t>& perm) {
  perm.resize(n);
  std::iota(perm.begin(), perm.end(), 0u);
  std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  std::vector<uint32_t> sk(n);
  for (uint32_t i = 0; i < n; ++i) sk[i] = keys[perm[i]];
  std::copy(sk.begin(), sk.end(), keys.begin());
}

void gather4(float* a, const std::vector<uint32_t>& perm, uint32_t n) {
  if (!a) return;
  std::vector<float> t(a, a + 4 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) std::memcpy(a + 4 * (size_t)i, t.data() + 4 * (size_t)perm[i], 16);
}
template <class T>
void gather1(T* a, const std::vector<uint32_t>& perm, uint32_t n) {
  if (!a) return;
  std::vector<T> t(a, a + n);
  for (uint32_t i = 0; i < n; ++i) a[i] = t[perm[i]];
}

// Sorting and the start/end table with the reference's grid.cl kernels.  keys has n + 1
// entries: entry n is the inactive sentinel that fillEndCell reads past the active range
// (resetCellIDs gives slot n the key 2 * GRID_NUM_CELLS + n).
template <class Prog>
void cell_table(uint32_t n, std::vector<uint32_t>& keys, std::vector<uint32_t>& table, Prog) {
  const uint32_t nc = ref_consts.numCells;
  keys[n] = 2 * nc + n;
  uint2* t = reinterpret_cast<uint2*>(table.data());
  run(nc, [&] { Prog::resetStartEndCell(t); });
  run(n, [&] { Prog::fillStartCell(keys.data(), t); });
  run(n, [&] { Prog::fillEndCell(keys.data(), t); });
  run(nc, [&] { Prog::adjustEndCell(t); });
}

struct FluidsProg {
  static void resetStartEndCell(uint2* t) { ref_fluids::resetStartEndCell(t); }
  static void fillStartCell(const uint32_t* k, uint2* t) { ref_fluids::fillStartCell(k, t); }
  static void fillEndCell(const uint32_t* k, uint2* t) { ref_fluids::fillEndCell(k, t); }
  static void adjustEndCell(uint2* t) { ref_fluids::adjustEndCell(t); }
};
struct BoidsProg {
  static void resetStartEndCell(uint2* t) { ref_boids::resetStartEndCell(t); }
  static void fillStartCell(const uint32_t* k, uint2* t) { ref_boids::fillStartCell(k, t); }
  static void fillEndCell(const uint32_t* k, uint2* t) { ref_boids::fillEndCell(k, t); }
  static void adjustEndCell(uint2* t) { ref_boids::adjustEndCell(t); }
};
struct CloudsProg {
  static void resetStartEndCell(uint2* t) { ref_clouds::resetStartEndCell(t); }
  static void fillStartCell(const uint32_t* k, uint2* t) { ref_clouds::fillStartCell(k, t); }
  static void fillEndCell(const uint32_t* k, uint2* t) { ref_clouds::fillEndCell(k, t); }
  static void adjustEndCell(uint2* t) { ref_clouds::adjustEndCell(t); }
};

template <class P, class S>
P as(const S& s) {
  static_assert(sizeof(P) == sizeof(S), "parameter struct layout");
  P p;
  std::memcpy(&p, &s, sizeof p);
  return p;
}

}  // namespace

extern "C" {

void ref_fill_cell_ids(const rtp_grid_constants* c, const float* pos4, uint32_t n, uint32_t* keys) {
  ref_consts = *c;
  const float4* p = reinterpret_cast<const float4*>(pos4);
  run(n, [&] { ref_fluids::fillCellIDs(p, keys); });
}

void ref_cell_table(const rtp_grid_constants* c, const uint32_t* sorted_keys, uint32_t n, uint32_t* table2) {
  ref_consts = *c;
  std::vector<uint32_t> keys(sorted_keys, sorted_keys + n);
  keys.push_back(0);
  std::vector<uint32_t> table(2 * (size_t)c->numCells);
  cell_table(n, keys, table, FluidsProg());
  std::memcpy(table2, table.data(), sizeof(uint32_t) * table.size());
}

// Fluids::update (Fluids.cpp:412-457).
int ref_fluids_step(const rtp_grid_constants* c, const rtp_fluid_params* fp, uint32_t iters, uint32_t n, or_state* s) {
  ref_consts = *c;
  const ref_fluids::FluidParams P = as<ref_fluids::FluidParams>(*fp);
  float4 *pos = F4(s->pos), *vel = F4(s->vel), *pred = F4(s->predPos);
  run(n, [&] { ref_fluids::fld_predictPosition(pos, vel, P, pred); });
  std::vector<uint32_t> keys(n + 1), perm;
  run(n, [&] { ref_fluids::fillCellIDs(pred, keys.data()); });
  sort_keys(n, keys, perm);
  gather4(s->pos, perm, n);
  gather4(s->vel, perm, n);
  gather4(s->predPos, perm, n);
  gather1(s->id, perm, n);
  if (s->cellId) std::memcpy(s->cellId, keys.data(), sizeof(uint32_t) * n);
  std::vector<uint32_t> table(2 * (size_t)c->numCells);
  cell_table(n, keys, table, FluidsProg());
  const uint2* T = reinterpret_cast<const uint2*>(table.data());
  std::vector<float> density(n), lambda(n), corr(4 * (size_t)n);
  float4* corrP = F4(corr.data());
  for (uint32_t it = 0; it < iters; ++it) {
    run(n, [&] { ref_fluids::fld_applyBoundaryCondition(pred); });
    run(n, [&] { ref_fluids::fld_computeDensity(pred, T, P, density.data()); });
    run(n, [&] { ref_fluids::fld_computeConstraintFactor(pred, density.data(), T, P, lambda.data()); });
    run(n, [&] { ref_fluids::fld_computeConstraintCorrection(lambda.data(), T, pred, P, corrP); });
    run(n, [&] { ref_fluids::fld_correctPosition(corrP, pred); });
  }
  if (s->density) std::memcpy(s->density, density.data(), sizeof(float) * n);
  if (s->lambda) std::memcpy(s->lambda, lambda.data(), sizeof(float) * n);
  run(n, [&] { ref_fluids::fld_updateVel(pred, pos, P, vel); });
  if (fp->isVorticityConfEnabled) {
    std::vector<float> vort(4 * (size_t)n), velIn(4 * (size_t)n);
    float4 *W = F4(vort.data()), *VI = F4(velIn.data());
    run(n, [&] { ref_fluids::fld_computeVorticity(pred, T, vel, P, W); });
    run(n, [&] { ref_fluids::fld_applyVorticityConfinement(pred, T, W, P, vel); });
    std::memcpy(velIn.data(), s->vel, sizeof(float) * 4 * n);
    run(n, [&] { ref_fluids::fld_applyXsphViscosityCorrection(pred, T, VI, P, vel); });
    if (s->vort) std::memcpy(s->vort, vort.data(), sizeof(float) * 4 * n);
  }
  run(n, [&] { ref_fluids::fld_updatePosition(pred, pos); });
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());
  return RTP_OK;
}

// Boids::update (Boids.cpp:335-373), dt a parameter; the target rule (:351-358) runs when
// target is not NULL, with the target's position of this step.
int ref_boids_step_target(const rtp_grid_constants* c, const rtp_boids_params* bp, float dt, int boundary, int dim,
                          const float* target, float targetRadius, int targetSign, uint32_t n, or_state* s) {
  ref_consts = *c;
  const ref_boids::BoidsRuleParams P = as<ref_boids::BoidsRuleParams>(*bp);
  float4 *pos = F4(s->pos), *vel = F4(s->vel);
  std::vector<uint32_t> keys(n + 1), perm;
  run(n, [&] { ref_boids::fillCellIDs(pos, keys.data()); });
  sort_keys(n, keys, perm);
  gather4(s->pos, perm, n);
  gather4(s->vel, perm, n);
  gather1(s->id, perm, n);
  if (s->cellId) std::memcpy(s->cellId, keys.data(), sizeof(uint32_t) * n);
  std::vector<uint32_t> table(2 * (size_t)c->numCells);
  cell_table(n, keys, table, BoidsProg());
  const uint2* T = reinterpret_cast<const uint2*>(table.data());
  std::vector<float> acc(4 * (size_t)n);
  float4* A = F4(acc.data());
  if (dim == 2)  // Boids.cpp:346-349
    run(n, [&] { ref_boids::bd_applyBoidsRulesWithGrid2D(pos, vel, T, P, A); });
  else
    run(n, [&] { ref_boids::bd_applyBoidsRulesWithGrid3D(pos, vel, T, P, A); });
  if (target) {
    const float4 tp = clshim::make_float4(target[0], target[1], target[2], 0.0f);
    ref_boids::TargetParams TP;
    TP.targetRadiusEffect = targetRadius;
    TP.targetSignEffect = targetSign;
    run(n, [&] { ref_boids::bd_addTargetRule(pos, tp, TP, A); });
  }
  const float vmax = bp->velocityScale;
  run(n, [&] { ref_boids::bd_updateVel(A, dt, vmax, vel); });
  if (boundary == RTP_BOUNDARY_CYCLIC_WALL)
    run(n, [&] { ref_boids::bd_updatePosAndApplyPeriodicBC(vel, dt, pos); });
  else
    run(n, [&] { ref_boids::bd_updatePosAndApplyWallBC(vel, dt, pos); });
  if (s->acc) std::memcpy(s->acc, acc.data(), sizeof(float) * 4 * n);
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());
  return RTP_OK;
}

// Clouds::update (Clouds.cpp:516-605) with the reference's built-in environment.
int ref_clouds_step(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp, uint32_t iters,
                    uint32_t n, or_state* s) {
  ref_consts = *c;
  const ref_clouds::FluidParams F = as<ref_clouds::FluidParams>(*fp);
  const ref_clouds::CloudParams C = as<ref_clouds::CloudParams>(*cp);
  float4 *pos = F4(s->pos), *vel = F4(s->vel), *pred = F4(s->predPos), *tot = F4(s->totCorrPos);
  std::vector<float> tempIn(n), vaporIn(n), cloudIn(n), gen(n);
  std::memcpy(tempIn.data(), s->temp, sizeof(float) * n);
  run(n, [&] { ref_clouds::cld_heatFromGround(tempIn.data(), pos, C, s->temp); });
  run(n, [&] { ref_clouds::cld_computeBuoyancy(s->temp, pos, s->cloud, C, s->buoyancy); });
  run(n, [&] { ref_clouds::cld_applyAdiabaticCooling(s->temp, vel, C, tempIn.data()); });
  run(n, [&] { ref_clouds::cld_generateCloud(tempIn.data(), s->vapor, s->cloud, C, gen.data()); });
  std::memcpy(vaporIn.data(), s->vapor, sizeof(float) * n);
  std::memcpy(cloudIn.data(), s->cloud, sizeof(float) * n);
  run(n, [&] { ref_clouds::cld_applyPhaseTransition(vaporIn.data(), cloudIn.data(), gen.data(), C, s->vapor, s->cloud); });
  run(n, [&] { ref_clouds::cld_applyLatentHeat(tempIn.data(), gen.data(), C, s->temp); });
  run(n, [&] { ref_clouds::cld_predictPosition(pos, vel, s->buoyancy, C, pred, tot); });
  run(n, [&] { ref_clouds::cld_applyMixedBoundaryConditions(pred); });
  std::vector<uint32_t> keys(n + 1), perm;
  run(n, [&] { ref_clouds::fillCellIDs(pred, keys.data()); });
  sort_keys(n, keys, perm);
  gather4(s->pos, perm, n);
  gather4(s->vel, perm, n);
  gather4(s->predPos, perm, n);
  gather4(s->totCorrPos, perm, n);
  gather1(s->temp, perm, n);
  gather1(s->buoyancy, perm, n);
  gather1(s->vapor, perm, n);
  gather1(s->cloud, perm, n);
  gather1(s->id, perm, n);
  if (s->cellId) std::memcpy(s->cellId, keys.data(), sizeof(uint32_t) * n);
  std::vector<uint32_t> table(2 * (size_t)c->numCells);
  cell_table(n, keys, table, CloudsProg());
  const uint2* T = reinterpret_cast<const uint2*>(table.data());
  if (cp->isTempSmoothingEnabled) {
    std::vector<float> lap(n), lamT(n), corrT(n);
    run(n, [&] { ref_clouds::cld_computeLaplacianTemp(pos, s->temp, T, C, lap.data()); });
    run(n, [&] { ref_clouds::cld_computeConstraintFactorTemp(pos, lap.data(), T, C, lamT.data()); });
    run(n, [&] { ref_clouds::cld_computeConstraintCorrectionTemp(lamT.data(), T, pos, C, corrT.data()); });
    run(n, [&] { ref_clouds::cld_correctTemperature(corrT.data(), s->temp); });
  }
  std::vector<float> density(n), lambda(n), corr(4 * (size_t)n);
  float4* corrP = F4(corr.data());
  for (uint32_t it = 0; it < iters; ++it) {
    run(n, [&] { ref_clouds::cld_computeDensity(pred, T, F, density.data()); });
    run(n, [&] { ref_clouds::cld_computeConstraintFactor(pred, density.data(), T, F, lambda.data()); });
    run(n, [&] { ref_clouds::cld_computeConstraintCorrection(lambda.data(), T, pred, F, corrP); });
    run(n, [&] { ref_clouds::cld_correctPosition(corrP, pred); });
    run(n, [&] { ref_clouds::cld_correctPosition(corrP, tot); });
    run(n, [&] { ref_clouds::cld_applyMixedBoundaryConditions(pred); });
  }
  if (s->density) std::memcpy(s->density, density.data(), sizeof(float) * n);
  if (s->lambda) std::memcpy(s->lambda, lambda.data(), sizeof(float) * n);
  run(n, [&] { ref_clouds::cld_updateVel(tot, F, vel); });
  if (fp->isVorticityConfEnabled) {
    std::vector<float> vort(4 * (size_t)n), velIn(4 * (size_t)n);
    float4 *W = F4(vort.data()), *VI = F4(velIn.data());
    run(n, [&] { ref_clouds::cld_computeVorticity(pred, T, vel, F, W); });
    run(n, [&] { ref_clouds::cld_applyVorticityConfinement(pred, T, W, F, vel); });
    std::memcpy(velIn.data(), s->vel, sizeof(float) * 4 * n);
    run(n, [&] { ref_clouds::cld_applyXsphViscosityCorrection(pred, T, VI, F, vel); });
    if (s->vort) std::memcpy(s->vort, vort.data(), sizeof(float) * 4 * n);
  }
  run(n, [&] { ref_clouds::cld_updatePosition(pred, C, pos); });
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());
  return RTP_OK;
}

// cld_initTemperature + cld_initVaporDensity (Clouds.cpp:495-498).
void ref_clouds_init(const rtp_grid_constants* c, const rtp_cloud_params* cp, uint32_t n, or_state* s) {
  ref_consts = *c;
  const ref_clouds::CloudParams C = as<ref_clouds::CloudParams>(*cp);
  const float4* pos = F4(s->pos);
  run(n, [&] { ref_clouds::cld_initTemperature(pos, s->temp); });
  run(n, [&] { ref_clouds::cld_initVaporDensity(C, s->temp, s->vapor); });
  for (uint32_t i = 0; i < n; ++i) s->cloud[i] = 0.0f;
}

}  // extern "C"

extern "C" {

// Side outputs through the reference's own kernels.
void ref_fill_fluid_color(const rtp_grid_constants* c, const rtp_fluid_params* fp, const float* density, uint32_t n,
                          float* col) {
  ref_consts = *c;
  const ref_fluids::FluidParams P = as<ref_fluids::FluidParams>(*fp);
  run(n, [&] { ref_fluids::fld_fillFluidColor(density, P, F4(col)); });
}

void ref_fill_color_float(const rtp_grid_constants* c, const float* q, uint32_t n, float minVal, float maxVal,
                          float* col) {
  ref_consts = *c;
  run(n, [&] { ref_clouds::fillColorFloat(q, minVal, maxVal, F4(col)); });
}

void ref_fill_camera_dist(const rtp_grid_constants* c, const float* pos, uint32_t n, uint32_t maxN, const float cam[3],
                          uint32_t* dist) {
  ref_consts = *c;
  clshim::float3 cp{cam[0], cam[1], cam[2]};
  run(maxN, [&] { ref_fluids::resetCameraDist(dist); });
  run(n, [&] { ref_fluids::fillCameraDist(F4(const_cast<float*>(pos)), &cp, dist); });
}

void ref_fill_grid_detector(const rtp_grid_constants* c, const float* pos, uint32_t n, float* det) {
  ref_consts = *c;
  clshim::float8* d = reinterpret_cast<clshim::float8*>(det);
  run(c->numCells, [&] { ref_fluids::resetGridDetector(d); });
  run(n, [&] { ref_fluids::fillGridDetector(F4(const_cast<float*>(pos)), d); });
}

int ref_boids_step(const rtp_grid_constants* c, const rtp_boids_params* bp, float dt, int boundary, int dim, uint32_t n,
                   or_state* s) {
  return ref_boids_step_target(c, bp, dt, boundary, dim, nullptr, 0.0f, 0, n, s);
}

// PerlinNoise(seed).computeNoiseValue({x, y, z}); -1 when the copy of PerlinNoise.cpp is absent.
float ref_perlin_noise(int seed, float x, float y, float z) {
#ifdef REF_HAS_PERLIN
  Physics::PerlinNoise noise(seed);
  return noise.computeNoiseValue(Math::float3(x, y, z));
#else
  (void)seed, (void)x, (void)y, (void)z;
  return -1.0f;
#endif
}

}  // extern "C"
