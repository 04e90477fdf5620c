/*
 * rtp.h - C ABI of the GB300 (sm_103a) RealTimeParticles simulation step.
 *
 * This library replaces the OpenCL compute path that sits behind the reference's
 * `Physics::Model` interface (physics/Model.hpp:81-216, created by
 * `Physics::CreateModel`, physics/Model.cpp:10-24).  Every entry point below names the
 * reference interface it replaces.  The ABI is plain C: POD structs, plain pointers and
 * sizes, `int` status codes (`rtp_status`), no exceptions and no C++ or torch types.
 *
 * Threading: one handle per host thread.  All work of a handle is ordered on the
 * handle's own CUDA stream; `rtp_download` and `rtp_synchronize` wait for it.
 * Errors: every function returns RTP_OK or an error code; `rtp_last_error()` returns a
 * thread-local message describing the last failure on the calling thread.
 *
 * There is no CPU fallback and no multi-backend dispatch: without a CUDA device every
 * compute call fails with RTP_ERR_NO_DEVICE.
 */
#ifndef RTP_H
#define RTP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: rtp_tuning gained tiledSweeps (12 bytes; version 1 had 8). */
#define RTP_ABI_VERSION 2

/* Status codes.  The reference reports errors as `bool` + log lines and throws
 * std::runtime_error on bad JSON paths (physics/ocl/Fluids.cpp:245-250); across a C ABI
 * they become return codes. */
typedef enum rtp_status {
  RTP_OK = 0,
  RTP_ERR_INVALID_ARGUMENT = 1,
  RTP_ERR_OUT_OF_MEMORY = 2,
  RTP_ERR_CUDA = 3,
  RTP_ERR_NOT_SUPPORTED = 4,
  RTP_ERR_STATE = 5,
  RTP_ERR_NO_DEVICE = 6,
  RTP_ERR_CAPACITY = 7
} rtp_status;

/* Physics::ModelType, physics/Model.hpp:16-21 (same values). */
typedef enum rtp_model_type {
  RTP_MODEL_BOIDS = 0,
  RTP_MODEL_FLUIDS = 1,
  RTP_MODEL_CLOUDS = 2
} rtp_model_type;

/* Physics::Boundary, physics/Model.hpp:38-44 (same order). */
typedef enum rtp_boundary {
  RTP_BOUNDARY_BOUNCING_WALL = 0,
  RTP_BOUNDARY_CYCLIC_WALL = 1
} rtp_boundary;

/* Utils::PhysicsCase, utils/Parameters.hpp:17-39 (same values). */
typedef enum rtp_case {
  RTP_CASE_BOIDS_SMALL = 1,
  RTP_CASE_BOIDS_MEDIUM = 2,
  RTP_CASE_BOIDS_LARGE = 3,
  RTP_CASE_BOIDS_XLARGE = 4,
  RTP_CASE_FLUIDS_DAM = 7,
  RTP_CASE_FLUIDS_BOMB = 8,
  RTP_CASE_FLUIDS_DROP = 9,
  RTP_CASE_CLOUDS_CUMULUS = 12,
  RTP_CASE_CLOUDS_HOMOGENEOUS = 13,
  RTP_CASE_INVALID = -1
} rtp_case;

/* Physics::ModelParams, physics/Model.hpp:60-73.  The four GL VBO ids are replaced by
 * headless device buffers owned by the handle (see rtp_device_ptr).  Box extents are
 * float (the reference's Geometry::BoxSize3D is size_t, utils/Geometry.hpp:42-47), so
 * non-integer boxes are expressible.  `maxNbPartsInCell` is the constructor constant
 * m_maxNbPartsInCell (Fluids.cpp:79, Boids.cpp:78, Clouds.cpp:107); 0 selects the
 * reference value for the model. */
typedef struct rtp_model_params {
  uint64_t currNbParticles;
  uint64_t maxNbParticles;
  float boxSize[3];
  uint32_t gridRes[3];
  float velocity;
  uint32_t dimension; /* 2 or 3 */
  int32_t pCase;      /* rtp_case */
  uint32_t maxNbPartsInCell;
} rtp_model_params;

/* FluidKernelInputs, physics/ocl/Fluids.hpp:17-32 == FluidParams, kernels/define.cl:13-25.
 * Same field order and types (44 bytes). */
typedef struct rtp_fluid_params {
  float restDensity;
  float relaxCFM;
  float timeStep;
  uint32_t dim;
  uint32_t isArtPressureEnabled;
  float artPressureRadius;
  float artPressureCoeff;
  uint32_t artPressureExp;
  uint32_t isVorticityConfEnabled;
  float vorticityConfCoeff;
  float xsphViscosityCoeff;
} rtp_fluid_params;

/* BoidsRuleKernelInputs, physics/ocl/Boids.hpp:14-20 == BoidsRuleParams, boids.cl:12-17. */
typedef struct rtp_boids_params {
  float velocityScale;
  float alignmentScale;
  float separationScale;
  float cohesionScale;
} rtp_boids_params;

/* CloudKernelInputs, physics/ocl/Clouds.hpp:15-45 == CloudParams, clouds.cl:19-33
 * (same field order, 52 bytes). */
typedef struct rtp_cloud_params {
  uint32_t dim;
  float timeStep;
  float restDensity;
  float groundHeatCoeff;
  float buoyancyCoeff;
  float gravCoeff;
  float adiabaticLapseRate;
  float phaseTransitionRate;
  float latentHeatCoeff;
  uint32_t isTempSmoothingEnabled;
  float relaxCFM;
  float initVaporDensityCoeff;
  float windCoeff;
} rtp_cloud_params;

/* Environment of the clouds model.  The reference hard-codes it in clouds.cl:72-89 and
 * clouds.cl:951-952 for a 10x20x10 box: T_env(y) = 293 - 3.5 (y + W_y), ground heat
 * source exp(-(y + W_y) / 3), wind profiles 1 - exp(-0.2 (y + W_y)) and
 * 1 - exp(-0.3 (y + W_y)).  rtp_cloud_env_reference() returns exactly those values.
 * `groundTemp` (optional, groundNx x groundNz floats, row-major in z) replaces the
 * constant ground temperature by a field over (x, z), bilinearly sampled over
 * [-W_x, W_x] x [-W_z, W_z]. */
typedef struct rtp_cloud_env {
  float groundTemp0;  /* 293 K: ground temperature when no field is given */
  float lapseRate;    /* 3.5 K per box unit */
  float heatDecay;    /* 3.0 box units */
  float windDecayX;   /* 0.2 per box unit */
  float windDecayZ;   /* 0.3 per box unit */
  uint32_t groundNx;
  uint32_t groundNz;
} rtp_cloud_env;

/* The -D constants the reference bakes into its JIT program (Fluids.cpp:104-119,
 * Boids.cpp:103-113, Clouds.cpp:134-147), each round-tripped through the reference's
 * 10-decimal FloatToStr (utils/Utils.cpp:24-28) exactly as the OpenCL compiler sees it. */
typedef struct rtp_grid_constants {
  float absWall[3];          /* ABS_WALL_X/Y/Z */
  uint32_t gridRes[3];       /* GRID_RES_X/Y/Z */
  float cellSize;            /* GRID_CELL_SIZE_XYZ */
  uint32_t numCells;         /* GRID_NUM_CELLS */
  uint32_t maxPartsInCell;   /* NUM_MAX_PARTS_IN_CELL */
  float effectRadius;        /* EFFECT_RADIUS (fluids, clouds) */
  float effectRadiusSquared; /* EFFECT_RADIUS_SQUARED (boids) */
  float poly6Coeff;          /* POLY6_COEFF */
  float spikyCoeff;          /* SPIKY_COEFF */
  float maxVel;              /* MAX_VEL */
  uint32_t keyBound;         /* 1 + largest cell key fillCellIDs can emit (grid.cl:33-35) */
  uint32_t keyBits;          /* bits needed to sort keys < keyBound */
} rtp_grid_constants;

/* Buffers of a handle (headless replacement of the VBOs and named CL buffers,
 * physics/ocl/Fluids.cpp:128-150).  float4 buffers hold xyzw with w = 0. */
typedef enum rtp_buffer {
  RTP_BUF_POS = 0,        /* float4 p_pos */
  RTP_BUF_VEL = 1,        /* float4 p_vel */
  RTP_BUF_PRED_POS = 2,   /* float4 p_predPos (after the last step) */
  RTP_BUF_DENSITY = 3,    /* float  p_density (last Jacobi iteration) */
  RTP_BUF_LAMBDA = 4,     /* float  p_constFactor (last Jacobi iteration) */
  RTP_BUF_TEMP = 5,       /* float  p_temp (clouds) */
  RTP_BUF_VAPOR = 6,      /* float  p_vaporDens (clouds) */
  RTP_BUF_CLOUD = 7,      /* float  p_cloudDens (clouds) */
  RTP_BUF_BUOYANCY = 8,   /* float  p_buoyancy (clouds) */
  RTP_BUF_ID = 9,         /* uint   particle id carried through every sort (p_partID) */
  RTP_BUF_CELL_ID = 10,   /* uint   p_cellID: sorted cell keys of the last step */
  RTP_BUF_CELL_TABLE = 11,/* uint2  c_startEndPartID in the reference's inclusive format */
  RTP_BUF_VORTICITY = 12, /* float4 p_vort */
  RTP_BUF_ACC = 13,       /* float4 p_acc (boids) */
  RTP_BUF_LAMBDA_TOTAL = 14, /* float: lambda summed over the iterations of the last warm-started
                                or sample-recording step (fluids; the warm start's multiplier
                                plus the extra iterations' lambdas).  Cleared by uploading POS. */
  RTP_BUF_COLOR = 15,         /* float4 p_col (rtp_fill_fluid_color / rtp_fill_color_float) */
  RTP_BUF_CAMERA_DIST = 16,   /* uint   p_cameraDist of every slot (rtp_fill_camera_order) */
  RTP_BUF_DRAW_ORDER = 17,    /* uint   slots in the order the reference draws them */
  RTP_BUF_GRID_DETECTOR = 18  /* float8 per cell: 1 where a particle is (rtp_fill_grid_detector) */
} rtp_buffer;

/* Per-kernel device time, collected when profiling is enabled (the reference's
 * Context::runKernel profiling, physics/ocl/Context.cpp:692-705). */
typedef struct rtp_kernel_time {
  char name[48];
  uint64_t launches;
  double total_ms;
} rtp_kernel_time;

/* Step metrics (new: the reference has no physics metrics).  Filled by rtp_get_metrics
 * from the current state on the device. */
typedef struct rtp_metrics {
  double meanDensityError;  /* mean |rho_i / rho0 - 1| over active particles */
  double maxDensityError;
  double kineticEnergy;     /* 0.5 * sum |v|^2 (unit mass) */
  double meanNeighbours;    /* mean neighbours within the effect radius */
  uint32_t neighbourHist[64];
  double meanCompression;     /* mean max(rho_i / rho0 - 1, 0): compression only */
  uint32_t pairListOverflows; /* particles whose last recorded pair list overflowed */
  uint32_t pairListMax;       /* longest recorded pair list of the last step */
} rtp_metrics;

/* Library. */
const char* rtp_last_error(void);
int rtp_abi_version(void);
/* Host-only: derives the JIT constants of a model from its parameters
 * (Fluids::createProgram, Fluids.cpp:97-126; Boids.cpp:96-120; Clouds.cpp:127-160). */
int rtp_get_constants(int model, const rtp_model_params* params, rtp_grid_constants* out);
/* Host-only: the reference's default parameters (JSON defaults Fluids.cpp:52-74,
 * Boids.cpp:41-73, Clouds.cpp:67-102). */
int rtp_fluid_params_default(rtp_fluid_params* out);
int rtp_boids_params_default(rtp_boids_params* out);
int rtp_cloud_params_default(rtp_cloud_params* out);
int rtp_cloud_env_reference(rtp_cloud_env* out);

/* Model lifecycle: Physics::CreateModel (Model.cpp:10-24), ~Model, Model::reset
 * (Fluids.cpp:196-216, Boids.cpp:228-275, Clouds.cpp:379-399), Model::update
 * (Fluids.cpp:400-471, Boids.cpp:323-384, Clouds.cpp:503-627) called nsteps times. */
int rtp_create(int model, const rtp_model_params* params, void** out_handle);
int rtp_destroy(void* handle);
int rtp_reset(void* handle);
int rtp_update(void* handle, uint32_t nsteps);

/* Parameter setters: OclModel::updateModelWithInputJson -> transferKernelInputsToGPU
 * (OclModel.hpp:48-57; Fluids.cpp:218-271; Boids.cpp:177-226; Clouds.cpp:279-377). */
int rtp_set_fluid_params(void* handle, const rtp_fluid_params* p);
int rtp_get_fluid_params(void* handle, rtp_fluid_params* p);
int rtp_set_jacobi_iterations(void* handle, uint32_t iters); /* "Nb Jacobi Iterations" */
int rtp_set_boids_params(void* handle, const rtp_boids_params* p);
int rtp_set_boids_time_step(void* handle, float dt);  /* Boids.cpp:334 hard-codes 0.1 */
/* Boids target attractor: the JSON "Target" group (Boids.cpp:45-51, transferred at
 * :193-202) with TargetKernelInputs (Boids.hpp:22-26).  While enabled, every step moves
 * the target along its Perlin-noise trajectory (Target::updatePos, Target.cpp:27-50, with
 * the velocity scale of the rules) and adds bd_addTargetRule (boids.cl:226-241) to the
 * rules' acceleration before the velocity update (Boids.cpp:351-358).  The trajectory is
 * a host state of the model: reset does not restart it, disabling pauses it. */
typedef struct rtp_target_params {
  int32_t enabled;    /* "Enable##Target" (default 0) */
  int32_t visible;    /* "Show" (default 1); reported visible only while enabled (Target.hpp:25) */
  float radiusEffect; /* "Radius"[0] (default 2.0) */
  int32_t signEffect; /* (int)"Attract": 1 (default); Attract = false gives 0, no effect */
} rtp_target_params;
int rtp_target_params_default(rtp_target_params* out);
int rtp_set_target(void* handle, const rtp_target_params* p);         /* boids only */
/* Model::targetPos / isTargetActivated / isTargetVisible (physics/Model.hpp:130-132): the
 * position after the last step taken (0, 0, 0 before the first). Other models: 0 and false. */
int rtp_get_target(void* handle, float pos[3], int* activated, int* visible);
int rtp_set_cloud_params(void* handle, const rtp_cloud_params* p);
int rtp_set_cloud_environment(void* handle, const rtp_cloud_env* env, const float* groundTemp);
/* cld_initTemperature + cld_initVaporDensity over the current positions, cloud = 0
 * (Clouds.cpp:495-498, clouds.cl:116-135); call after uploading positions. */
int rtp_clouds_init(void* handle);

/* Model setters (physics/Model.hpp:106-128). */
int rtp_set_nb_particles(void* handle, uint64_t n);
int rtp_get_nb_particles(void* handle, uint64_t* n);
int rtp_set_boundary(void* handle, int boundary);
/* Model::setDimension (Model.hpp:109-113): stores the dimension and resets.  A 2D model keeps
 * its particles in the x = 0 plane (the reference's YZ cases, Fluids.cpp:287-333,
 * Boids.cpp:291-299, Clouds.cpp:417-446); boids use the 9-cell 2D rules (boids.cl:137-221),
 * fluids and clouds the same kernels as in 3D with dim = 2 in their parameters. */
int rtp_set_dimension(void* handle, uint32_t dim);
int rtp_set_case(void* handle, int pcase);
int rtp_pause(void* handle, int pause);

/* Buffers (replaces the CL-GL VBO sharing, physics/ocl/Context.cpp:710-750 and
 * loadBufferFromHost).  `count` is in elements of the buffer's type (float4, float,
 * uint or uint2) and must be <= maxNbParticles (or numCells for the cell table). */
int rtp_upload(void* handle, int buffer, const void* host, uint64_t count);
int rtp_download(void* handle, int buffer, void* host, uint64_t count);
int rtp_device_ptr(void* handle, int buffer, void** dptr);
int rtp_stream(void* handle, void** stream);
int rtp_synchronize(void* handle);
/* A step over host-resident state in one call (new: the reference keeps its state in GL
 * buffers): copies `count` float4 positions and velocities from host memory into the model,
 * runs nsteps updates (rtp_update) and copies them back, all ordered on the handle's stream
 * with a single synchronisation at the end; it returns once posOut / velOut hold the result.
 * count must equal the current particle count.  A NULL input skips that upload, a NULL output
 * that download; in and out may be the same buffer.  For one fluids or boids step on pinned
 * host memory (cudaHostAlloc, cudaHostRegister) the step's first kernel reads the inputs and
 * its last kernel writes the outputs over the host link directly (no separate copies);
 * otherwise the buffers are copied with cudaMemcpyAsync. */
int rtp_update_host(void* handle, const void* posIn, const void* velIn, uint64_t count, uint32_t nsteps, void* posOut,
                    void* velOut);

/* Profiling (OclModel::isProfilingEnabled/enableProfiling, OclModel.hpp:28-38). */
int rtp_enable_profiling(void* handle, int enable);
int rtp_is_profiling_enabled(void* handle, int* enabled);
int rtp_get_kernel_times(void* handle, rtp_kernel_time* out, uint32_t capacity, uint32_t* count);
int rtp_reset_kernel_times(void* handle);
/* Device-timed steps: runs `nsteps` updates, each bracketed by CUDA events on the
 * handle's stream; when `flush_bytes` > 0 a buffer of that size is overwritten
 * before every step (outside the timed interval) so every step starts with a cold L2. */
int rtp_time_steps(void* handle, uint32_t nsteps, uint64_t flush_bytes, double* total_ms);

/* Metrics (new). */
int rtp_get_metrics(void* handle, rtp_metrics* out);

/* Grid / sort operators on caller-owned device memory, ordered on `stream`
 * (a cudaStream_t, NULL = legacy default stream).  They are the stand-alone forms of
 * fillCellIDs (grid.cl:76-86), RadixSort::sort (physics/utils/RadixSort.cpp:122-189)
 * and resetStartEndCell/fillStartCell/fillEndCell/adjustEndCell (grid.cl:91-152). */
int rtp_fill_cell_ids(const rtp_grid_constants* c, const float* d_pos4, uint32_t n,
                      uint32_t* d_keys, void* stream);
/* Stable sort of n keys < 2^keyBits: keys_out = keys in ascending order, equal keys in
 * input order; perm_out[i] = input index of keys_out[i].  `d_scratch` must hold
 * rtp_radix_sort_scratch_bytes(n, keyBits) bytes. */
int rtp_radix_sort_scratch_bytes(uint32_t n, uint32_t keyBits, size_t* bytes);
int rtp_radix_sort(const uint32_t* d_keys_in, uint32_t n, uint32_t keyBits,
                   uint32_t* d_keys_out, uint32_t* d_perm_out,
                   void* d_scratch, size_t scratch_bytes, void* stream);
/* One stable scatter pass of the LSD radix sort with caller-supplied digit offsets (the pass
 * RadixSort::sort runs per digit, radixSort.cl:147-168 `reorder`, with the histogram and scan of
 * radixSort.cl:19-141 done by the caller).  Keys are split in tiles of RTP_SORT_TILE; digit
 * d = (key >> shift) & (2^bits - 1), bits 1..9.  d_tile_offsets[t * RTP_SORT_BINS + d] = number of
 * keys with digit d in tiles < t; d_digit_totals[d] = number of keys with digit d.  Keys go to
 * keys_out in digit order, stable, perm_out (optional) receives their input indices.  Offsets
 * inconsistent with the keys would place an element outside [0, n): such an element is not
 * written and 1 is ORed into *d_fault (device memory).  Inside a model step the same guard raises
 * the handle's fault word, which rtp_synchronize, rtp_download, rtp_update_host and
 * rtp_time_steps report as RTP_ERR_CUDA. */
#define RTP_SORT_TILE 2048u
#define RTP_SORT_BINS 512u
int rtp_radix_sort_pass(const uint32_t* d_keys_in, uint32_t n, uint32_t shift, uint32_t bits,
                        const uint32_t* d_tile_offsets, const uint32_t* d_digit_totals, uint32_t* d_keys_out,
                        uint32_t* d_perm_out, uint32_t* d_fault, void* stream);
/* Cell table from n sorted keys, in the reference's format: uint2 per cell,
 * (start, end) inclusive, empty = (1, 0), capped at maxPartsInCell. */
int rtp_build_cell_table(const rtp_grid_constants* c, const uint32_t* d_sorted_keys,
                         uint32_t n, uint32_t* d_table2, void* stream);

/* Radix sort that allocates nothing.  No counterpart in the reference (RadixSort owns
 * its buffers, physics/utils/RadixSort.cpp:78-96).  For callers that cannot allocate device
 * memory where they sort: a plugin whose host application owns the GPU heap, a frame loop
 * that must not stall on cudaMalloc's implicit synchronisation, code that must not fail
 * with out-of-memory after start-up.  Same result as rtp_radix_sort (stable, keys < 2^keyBits,
 * perm_out optional), using a fixed scratch array inside the library instead of caller
 * memory:
 *  - at most RTP_NOALLOC_SORT_MAX_KEYS keys; more returns RTP_ERR_CAPACITY, nothing runs;
 *  - the array (RTP_NOALLOC_SORT_SCRATCH_BYTES) is held by every GPU that loads the library
 *    until the process exits;
 *  - the first call in each CUDA context (per device; again after cudaDeviceReset re-creates
 *    the primary context, or from another context on the same device) looks up the array's
 *    address in that context: make that call before any stream capture;
 *  - every call shares the array, so calls that overlap on the GPU race: order them on one
 *    stream or synchronise between them. */
#define RTP_NOALLOC_SORT_MAX_KEYS 262144u
#define RTP_NOALLOC_SORT_SCRATCH_BYTES 5253120u
int rtp_radix_sort_noalloc(const uint32_t* d_keys_in, uint32_t n, uint32_t keyBits, uint32_t* d_keys_out,
                           uint32_t* d_perm_out, void* stream);

/* ---- Headless side outputs (render-only in the reference) -------------------------------
 * Computed on demand from the current state into device buffers (rtp_device_ptr /
 * rtp_download); nothing here changes the simulation state.  The first call allocates the
 * buffer. */
/* fld_fillFluidColor (fluids.cl:458-478, Fluids.cpp:459-463) from the last step's density. */
int rtp_fill_fluid_color(void* handle);
/* fillColorFloat (utils.cl, Clouds.cpp:612-619): a float buffer (RTP_BUF_DENSITY, _LAMBDA,
 * _TEMP, _VAPOR, _CLOUD, _BUOYANCY, _LAMBDA_TOTAL) mapped to [0, 1] between minVal and maxVal,
 * 0 outside, as grey levels. */
int rtp_fill_color_float(void* handle, int buffer, float minVal, float maxVal);
/* resetCameraDist + fillCameraDist (utils.cl) for a camera at cameraPos, then the stable
 * ascending order of those keys (the reference sorts the whole state by them before drawing,
 * Fluids.cpp:466-468; here the state stays and RTP_BUF_DRAW_ORDER holds the slot order). */
#define RTP_FAR_DIST 1000000.0f
int rtp_fill_camera_order(void* handle, const float cameraPos[3]);
/* resetGridDetector + fillGridDetector (grid.cl:43-60) over the current positions. */
int rtp_fill_grid_detector(void* handle);

/* ---- Learned warm start of the fluids' constraint solve (new: no counterpart in the
 * reference, whose Jacobi loop starts every substep from a zero correction,
 * physics/ocl/Fluids.cpp:427-442).
 *
 * A per-particle MLP, RTP_MLP_IN features -> 64 GELU -> 64 GELU -> RTP_MLP_OUT, evaluated
 * with BF16 tensor-core MMAs (FP32 accumulate) inside the first density/lambda sweep of each
 * substep, at the predicted positions.  Features, in order, with h the effect radius,
 * rho0 the rest density, dt the time step and sums over neighbours j != i within h:
 *   0 neighbour count             1 rho_i / rho0 - 1
 *   2-4 h/rho0 * sum grad W_ij    5 (h/rho0)^2 * sum |grad W_ij|^2
 *   6 dt/rho0 * sum (v_j - v_i) . grad W_ij   (v = the step's input velocities)
 *   7-9 wall proximity per axis: clamp(2 - (x - lo)/h, 0, 2) - clamp(2 - (hi - x)/h, 0, 2)
 *       with lo, hi the fld_applyBoundaryCondition bounds
 *   10 lambda_i of the plain first iteration
 *   11 |v_i| dt / h
 * Output: the network's value y_i (output 0 times outScale[0]; outputs 1-3 are not used by the
 * solve) sets a relaxation of the plain first-iteration lambda (feature 10):
 *   omega_i = 1 + tanh(y_i) * (2 if y_i > 0 else 1), in (0, 3);  lambda_i <- omega_i lambda_i.
 * y = 0 gives omega = 1 exactly, so a network whose output layer is zero is the plain solver bit
 * for bit.  The first correction is x_i += dp_i(omega lambda) (fld_computeConstraintCorrection
 * with the relaxed lambdas, Fluids.cpp:433-434), then `extraIterations` Jacobi iterations, plain
 * or (relaxAllIterations) relaxed by the same omega.
 * Guard: the solver output's mean |rho_i/rho0 - 1| is measured in the vorticity sweep; a
 * step above `guardTolerance` reruns from the same predicted positions with the plain
 * iteration count (rtp_set_jacobi_iterations) before vorticity confinement and XSPH.
 *
 * Clouds handles (the clouds Jacobi loop, Clouds.cpp:570-587) take the same network in the
 * first cld_computeDensity / cld_computeConstraintFactor sweep, with neighbours over the
 * periodic x and z images and the y walls (clouds.cl:305-436), and features 7 and 9 (the x
 * and z wall proximities, always 0 under the periodic boundary) replaced by
 *   7 b_i dt^2 / h      (the step's buoyancy, cld_computeBuoyancy, as a displacement)
 *   9 (T_i - T_env(x_i)) / 10   (the smoothed temperature above the environment, K / 10)
 * feature 8 being the y-wall proximity with the box walls +-W_y.  The relaxed first
 * correction is cld_computeConstraintCorrection + the mixed boundary; then `extraIterations`
 * plain iterations.  The guard works as for fluids (a rerun restores the step's total
 * correction, clouds' cld_updateVel input); there is no relaxation of every iteration. */
#define RTP_MLP_IN 12
#define RTP_MLP_HIDDEN 64
#define RTP_MLP_OUT 4
typedef struct rtp_mlp {
  float inMean[RTP_MLP_IN]; /* network input = (feature - inMean) * inScale */
  float inScale[RTP_MLP_IN];
  float w1[RTP_MLP_HIDDEN][RTP_MLP_IN];
  float b1[RTP_MLP_HIDDEN];
  float w2[RTP_MLP_HIDDEN][RTP_MLP_HIDDEN];
  float b2[RTP_MLP_HIDDEN];
  float w3[RTP_MLP_OUT][RTP_MLP_HIDDEN];
  float b3[RTP_MLP_OUT];
  float outScale[RTP_MLP_OUT]; /* output o = network value o * outScale[o] */
} rtp_mlp;

typedef struct rtp_warm_start_config {
  uint32_t enabled;         /* 0: plain solver */
  uint32_t extraIterations; /* plain Jacobi iterations after the warm-started one */
  float guardTolerance;     /* mean |rho/rho0 - 1| that triggers a plain rerun; <= 0: no guard */
  uint32_t relaxAllIterations; /* != 0: the extra iterations' lambdas are relaxed by the same
                                  per-particle omega (set once per step by the network) */
} rtp_warm_start_config;

typedef struct rtp_solver_stats {
  uint64_t steps;            /* warm-started steps since the last reset */
  uint64_t reruns;           /* steps the guard sent back to the plain solver */
  double sumDensityError;    /* sum over steps of the accepted solver output's mean |rho/rho0 - 1| */
  double maxDensityError;    /* largest of those means */
  double sumFirstError;      /* sum over steps of the warm-started output's mean (before reruns) */
} rtp_solver_stats;

/* Installs (or with cfg->enabled == 0 removes) the warm start on a fluids or clouds handle
 * (clouds: relaxAllIterations gives RTP_ERR_NOT_SUPPORTED). */
int rtp_set_warm_start(void* handle, const rtp_mlp* net, const rtp_warm_start_config* cfg);
/* Also measure the plain solver's output error per step (fluids: warm-started steps always
 * do; clouds: only while enabled).  Fluids and clouds handles. */
int rtp_enable_solver_stats(void* handle, int enable);
int rtp_get_solver_stats(void* handle, rtp_solver_stats* out);
int rtp_reset_solver_stats(void* handle);

/* Regression data: runs one plain step with `referenceIterations` Jacobi iterations (the
 * simulation advances) and writes one sample for each cell-sorted particle index
 * phase, phase + stride, ... < n: its RTP_MLP_IN raw features (as above) into
 * d_features[k][RTP_MLP_IN] and its targets into d_targets[k][RTP_MLP_OUT]: the sum of
 * lambda over the iterations, then x_final - x_0 - dp(lambda sum) evaluated at x_0 (3).
 * At most `capacity` samples are written; *written receives the count. */
int rtp_record_warm_start_samples(void* handle, uint32_t referenceIterations, uint32_t stride, uint32_t phase,
                                  float* d_features, float* d_targets, uint64_t capacity, uint64_t* written);

typedef struct rtp_train_config {
  uint32_t epochs;
  uint32_t batch;          /* samples per Adam step */
  float learningRate;      /* cosine-decayed to learningRate * finalLrFraction */
  float finalLrFraction;
  float beta1, beta2, eps; /* Adam */
  float weightDecay;       /* decoupled (AdamW) */
  float lossWeights[RTP_MLP_OUT];
  uint64_t seed;           /* initialisation and shuffling */
} rtp_train_config;

/* Trains `net` on n samples in device memory: sets the input and output normalisation from
 * the data (mean / standard deviation of each feature, root mean square of each target),
 * initialises the weights from cfg->seed, then runs cfg->epochs of shuffled minibatch AdamW
 * with the library's BF16 tensor-core forward / backward kernels.  loss_history (host,
 * cfg->epochs floats, may be NULL) receives each epoch's mean loss. */
int rtp_train_warm_start(const float* d_features, const float* d_targets, uint64_t n, const rtp_train_config* cfg,
                         rtp_mlp* net, float* loss_history, void* stream);
/* Training through the solve.  The loss of a state is the mean squared density constraint after
 * the warm-started correction:
 *   x* = the step's predicted positions, clamped (fld_predictPosition, fld_applyBoundaryCondition),
 *   x' = clamp(x* + dp(omega(y) lambda)) with y = network(features at x*),
 *   L  = 1/n sum_i (rho_i(x') / rho0 - 1)^2, rho(x') over the 27 cells of the step's table.
 * Clouds: x* = the predicted positions after the step's thermodynamics and temperature
 * smoothing, x' = the mixed boundary of x* + dp(omega(y) lambda), rho over the periodic images;
 * the thermodynamic state (temperature, vapour, cloud, buoyancy) is restored afterwards.
 * rtp_warm_start_loss_grad evaluates L and dL/dy for the handle's current state (it runs the next
 * step's predict, sort and cell table; the model's positions and velocities are not changed):
 * d_dy (device, optional) receives dL/dy_i at index = particle id (RTP_BUF_ID), n floats. */
int rtp_warm_start_loss_grad(void* handle, const rtp_mlp* net, float* d_dy, double* loss);
/* Trains `net` on the handle's own rollout: each of `steps` steps computes L and its gradient at
 * that step's predicted positions (the backward sweeps dL/dx', dL/dy, then the network's backward
 * kernels) and takes one AdamW step (cfg: learningRate cosine-decayed to learningRate *
 * finalLrFraction over the steps, beta1, beta2, eps, weightDecay, seed; epochs, batch and
 * lossWeights are not used), then advances the simulation one step with the updated network and
 * `extraIterations` plain iterations, so it trains on the states the warm-started solver visits.
 * init != 0 starts a new network: input normalisation from the first step's features,
 * Xavier-uniform hidden layers (cfg->seed), a zero output layer (omega = 1) and unit output
 * scales; init == 0 continues from *net.  loss_history (host, `steps` floats, may be NULL)
 * receives each step's L before its update.  Single fluids or clouds scenes (not batches). */
int rtp_train_warm_start_rollout(void* handle, const rtp_train_config* cfg, uint32_t steps, uint32_t extraIterations,
                                 int init, rtp_mlp* net, float* loss_history);
/* Loss and gradient of `net` over n samples (forward and backward kernels of the trainer):
 *   loss = 1/n sum_s sum_o lossWeights[o] * (y_so - t_so / outScale[o])^2,
 * y the network value.  grad gets d loss / d (w1, b1, w2, b2, w3, b3); its normalisation
 * fields are zero. */
int rtp_mlp_loss_grad(const rtp_mlp* net, const float* lossWeights, const float* d_features, const float* d_targets,
                      uint64_t n, double* loss, rtp_mlp* grad, void* stream);
/* Backward kernels of the trainer with a given output gradient: grad = d/d(w1, b1, w2, b2, w3, b3)
 * of sum_s sum_o d_dy[s][o] * y_so (y in network units, rows of RTP_MLP_OUT). */
int rtp_mlp_backward(const rtp_mlp* net, const float* d_features, const float* d_dy, uint64_t n, rtp_mlp* grad,
                     void* stream);
/* Inference kernel of the warm start on stand-alone features: d_out[s][o] = y_so * outScale[o]. */
int rtp_mlp_forward(const rtp_mlp* net, const float* d_features, uint64_t n, float* d_out, void* stream);

/* ---- Batched scenes and tuning (new: no counterpart in the reference) --------------------
 * Many independent fluids scenes of uneven sizes stepped together.  Their particles share one
 * set of device buffers (scene s occupies slots [offset_s, offset_s + nbParticles_s) of every
 * buffer; rtp_batch_scene_range) and every stage of the step is a single launch over all scenes.
 * Each scene has its own box (float extents, any aspect) and grid of cells cellFactor * h wide
 * (rtp_tuning); all share the effect radius h, the fluid parameters, the Jacobi iteration count
 * and the warm start.  Every scene evolves as the same scene on its own handle would: the
 * stable sort keeps each scene in its slot range, and each scene's first sorted particle is
 * left out of its cell as the reference's fillStartCell does.  On a batch handle rtp_reset,
 * rtp_set_nb_particles and sample recording return RTP_ERR_NOT_SUPPORTED; everything else,
 * including rtp_upload / rtp_download of whole buffers, works as on a fluids handle. */
typedef struct rtp_batch_scene {
  uint64_t nbParticles;
  float boxSize[3];
} rtp_batch_scene;

int rtp_create_batch(uint32_t nscenes, const rtp_batch_scene* scenes, float effectRadius,
                     uint32_t maxNbPartsInCell, void** out_handle);
int rtp_batch_scene_range(void* handle, uint32_t scene, uint64_t* offset, uint64_t* count);
/* The scene's own grid constants (cell keys counted from 0 within the scene) and the offset
 * of its keys in the batch's cell-key space (RTP_BUF_CELL_ID, RTP_BUF_CELL_TABLE). */
int rtp_batch_scene_constants(void* handle, uint32_t scene, rtp_grid_constants* out);
int rtp_batch_scene_key_base(void* handle, uint32_t scene, uint32_t* base);

/* Launch shape of a fluids handle: lanes per particle in the sweeps that walk recorded pair
 * lists (2, 4 or 8; default 4); for a batch, the cell size as a multiple of h (>= 1;
 * default 1; a single scene keeps the reference's grid); and tiledSweeps (0 or 1): the
 * lambda sweep of a single scene of more than 49,152 particles on a grid of at least 6 cells
 * per axis runs tiled by bricks of 4 x 4 x 4 cells, each brick's particles and one-cell halo
 * staged in shared memory (same pairs, same order, same results bit for bit; no effect on a
 * batch).  rtp_autotune times every candidate (lanes x tiledSweeps {0, 1} for a single scene,
 * lanes x {1, 1.25, 1.5, 2} cell factors for a batch) over `steps` steps, L2 flushed before
 * each, and keeps the fastest; the simulation advances meanwhile. */
typedef struct rtp_tuning {
  uint32_t lanes;
  float cellFactor;
  uint32_t tiledSweeps;
} rtp_tuning;
#define RTP_TUNE_MAX_CANDIDATES 32
typedef struct rtp_tune_result {
  rtp_tuning best;
  double bestMsPerStep;
  uint32_t tried;
  rtp_tuning candidates[RTP_TUNE_MAX_CANDIDATES];
  double msPerStep[RTP_TUNE_MAX_CANDIDATES];
} rtp_tune_result;
int rtp_set_tuning(void* handle, const rtp_tuning* t);
int rtp_get_tuning(void* handle, rtp_tuning* t);
int rtp_autotune(void* handle, uint32_t steps, rtp_tune_result* out);

#ifdef __cplusplus
}
#endif

#endif /* RTP_H */
