/*
 * oracle.h - CPU restatement of the RealTimeParticles simulation step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA library is compared with: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs load it.
 * The product (realtimeparticles_gb300) never links, loads or calls anything here.
 *
 * Every function restates one reference kernel (or host sequence) in the same operation
 * order, citing the file:line it follows (paths relative to the reference project).
 * It is compiled with -ffp-contract=off so the float arithmetic is the same on x86-64
 * and aarch64.  Parity is pinned by comparing it bit-for-bit with the reference's own
 * kernel sources compiled for the CPU (oracle/ref/, outputs in oracle/_ref/), and by the
 * golden fixtures under tests/golden/ that were produced from those reference kernels.
 */
#ifndef RTP_ORACLE_H
#define RTP_ORACLE_H

#include <stdint.h>

#include "../include/rtp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Number of OpenMP threads used by the oracle (0 = all). */
void or_set_threads(int n);
int or_get_threads(void);

/* JIT constants, Fluids.cpp:104-119 / Boids.cpp:103-113 / Clouds.cpp:134-147. */
int or_derive_constants(int model, const rtp_model_params* p, rtp_grid_constants* c);

/* grid.cl:76-86 (fillCellIDs) over n float4 positions. */
void or_fill_cell_ids(const rtp_grid_constants* c, const float* pos4, uint32_t n, uint32_t* keys);
/* The contract of RadixSort::sort (RadixSort.cpp:122-189): stable ascending sort. */
void or_stable_sort(const uint32_t* keys, uint32_t n, uint32_t* keys_out, uint32_t* perm);
/* grid.cl:91-152: resetStartEndCell, fillStartCell, fillEndCell, adjustEndCell. */
void or_cell_table(const rtp_grid_constants* c, const uint32_t* sorted_keys, uint32_t n, uint32_t* table2);

/* State arrays of one model, all of length n (float4 arrays hold 4*n floats).
 * Unused members may be NULL. */
typedef struct or_state {
  float* pos;
  float* vel;
  float* predPos;
  float* totCorrPos;
  float* acc;
  float* vort;
  float* density;
  float* lambda;
  float* temp;
  float* vapor;
  float* cloud;
  float* buoyancy;
  uint32_t* id;
  uint32_t* cellId;   /* sorted keys of the step */
  uint32_t* table;    /* 2 * numCells */
} or_state;

/* One Fluids::update (Fluids.cpp:400-457 without the render-only lines 459-468). */
int or_fluids_step(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t iters,
                   uint32_t n, or_state* s);
/* One Boids::update (Boids.cpp:323-377, target rule off, dt a parameter). */
int or_boids_step(const rtp_grid_constants* c, const rtp_boids_params* p, float dt,
                  int boundary, uint32_t n, or_state* s);
/* The same for a 2D (dim = 2) or 3D model. */
int or_boids_step_dim(const rtp_grid_constants* c, const rtp_boids_params* p, float dt,
                      int boundary, int dim, uint32_t n, or_state* s);
/* The same with the target rule (bd_addTargetRule, boids.cl:226-241) for a target at
 * target[0..2] this step, or without it when target is NULL. */
int or_boids_step_target(const rtp_grid_constants* c, const rtp_boids_params* p, float dt,
                         int boundary, int dim, const float* target, float targetRadius,
                         int targetSign, uint32_t n, or_state* s);
/* Physics::PerlinNoise(seed).computeNoiseValue(x, y, z) (PerlinNoise.cpp:10-85). */
float or_perlin_noise(int seed, float x, float y, float z);
/* Target::updatePos (Target.cpp:27-50) nsteps times from a new Target of box width
 * boxWidth: out[3 * step + k]. */
void or_target_trajectory(float boxWidth, int dim, float particlesVel, uint32_t nsteps, float* out);
/* One Clouds::update (Clouds.cpp:503-610). `ground` may be NULL (constant groundTemp0). */
int or_clouds_step(const rtp_grid_constants* c, const rtp_fluid_params* fp,
                   const rtp_cloud_params* cp, const rtp_cloud_env* env, const float* ground,
                   uint32_t iters, uint32_t n, or_state* s);
/* The clouds warm-start features at sorted positions x0 (rows of 12: the neighbour count,
 * C, h/rho0 sum gradW (3), (h/rho0)^2 sum |gradW|^2, dt/rho0 sum (v_j - v_i).gradW,
 * b dt^2 / h, the y-wall proximity, (T - T_env) / 10, the plain lambda, |v| dt / h). */
void or_clouds_ws_features(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_env* env,
                           const float* ground, const float* x0, const float* vel, const float* temp,
                           const float* buoy, const uint32_t* table, uint32_t n, float* feats);
/* One warm-started Clouds::update: the network relaxes the first iteration's lambda by
 * omega(y) (BF16 operand rounding as on the GPU), then extraIters plain iterations.
 * featsOut (12 n) and omegaOut (n), rows by sorted index, may be NULL. */
int or_clouds_ws_step(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                      const rtp_cloud_env* env, const float* ground, const rtp_mlp* net, uint32_t extraIters,
                      uint32_t n, or_state* s, float* featsOut, float* omegaOut);
/* The clouds warm start's training loss: after the step's presort (s advances through it),
 * mean (rho(x')/rho0 - 1)^2 at the relaxed first correction x' (emulate = the GPU's BF16
 * operand rounding in the network).  featsOut (12 n, sorted rows) may be NULL. */
int or_clouds_ws_loss(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                      const rtp_cloud_env* env, const float* ground, const rtp_mlp* net, int emulate, uint32_t n,
                      or_state* s, double* loss, float* featsOut);
/* cld_initTemperature + cld_initVaporDensity (clouds.cl:116-135), cloud = 0. */
void or_clouds_init(const rtp_grid_constants* c, const rtp_cloud_params* cp,
                    const rtp_cloud_env* env, const float* ground, uint32_t n, or_state* s);

/* Single kernels on a sorted state with a built table, for per-kernel parity. */
void or_fld_density(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* predPos,
                    const uint32_t* table, uint32_t n, float* density);
void or_fld_lambda(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* predPos,
                   const float* density, const uint32_t* table, uint32_t n, float* lambda);
void or_fld_correction(const rtp_grid_constants* c, const rtp_fluid_params* p,
                       const float* predPos, const float* lambda, const uint32_t* table,
                       uint32_t n, float* corr);
/* Mean |rho/rho0 - 1|, max, kinetic energy and neighbour statistics of a fluid state
 * (uses the sorted state and its table, like the sweeps). */
void or_fluid_metrics(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* predPos,
                      const float* vel, const uint32_t* table, uint32_t n, rtp_metrics* m);

/* Side outputs (render-only in the reference): fld_fillFluidColor (fluids.cl:458-478),
 * fillColorFloat and resetCameraDist + fillCameraDist (utils.cl), resetGridDetector +
 * fillGridDetector (grid.cl:43-60; 8 floats per cell). */
void or_fill_fluid_color(const float* density, uint32_t n, float restDensity, float* col);
void or_fill_color_float(const float* q, uint32_t n, float minVal, float maxVal, float* col);
void or_fill_camera_dist(const float* pos, uint32_t n, uint32_t maxN, const float cam[3], uint32_t* dist);
void or_fill_grid_detector(const rtp_grid_constants* c, const float* pos, uint32_t n, float* det);

/* ---- learned warm start (new; restates the GPU method, not a reference kernel) ---------- */
/* Raw features (rtp.h, RTP_MLP_IN per particle) at the clamped predicted positions x0 of a
 * sorted state: vel = the step's input velocities. */
void or_ws_features(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* x0, const float* vel,
                    const uint32_t* table, uint32_t n, float* feats);
/* Network outputs in target units, double arithmetic; emulate = round the operands to BF16
 * where the GPU's tensor-core GEMMs do. */
void or_mlp_forward(const rtp_mlp* net, const float* feats, uint64_t n, int emulate, float* out);
/* Loss and gradient (w1, b1, w2, b2, w3, b3 as 5252 doubles), as rtp_mlp_loss_grad. */
void or_mlp_loss_grad(const rtp_mlp* net, const float* lossW, const float* feats, const float* targets, uint64_t n,
                      int emulate, double* loss, double* grad);
/* One warm-started Fluids step; lamTot receives the multiplier totals (sorted order). */
// Backward of the network with a given output gradient dy (rows of 4): 5252 doubles (w1, b1,
// w2, b2, w3, b3) of d/dparams sum_s sum_o dy_so y_so.
void or_mlp_backward(const rtp_mlp* net, const float* feats, const float* dy, uint64_t n, int emulate, double* grad);
// Loss of the warm start through the solve (mean squared density constraint after the
// omega-relaxed first correction) and dL/dy per particle id; see oracle.cpp.
int or_ws_loss_grad(const rtp_grid_constants* c, const rtp_fluid_params* p, const rtp_mlp* net, int emulate,
                    uint32_t n, or_state* s, double* loss, double* dyById, double* omegaById);
int or_ws_step(const rtp_grid_constants* c, const rtp_fluid_params* p, const rtp_mlp* net, uint32_t extraIters,
               float guardTol, uint32_t plainIters, uint32_t n, or_state* s, float* lamTot, double* solverErr,
               int* rerun, int relaxAll);
/* One plain step with `iters` iterations (lamTot receives the lambda sums) that also returns
 * the samples of particles
 * phase, phase + stride, ... (features and targets as rtp_record_warm_start_samples). */
int or_ws_record_step(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t iters, uint32_t stride,
                      uint32_t phase, uint32_t n, or_state* s, float* lamTot, float* feats, float* targets,
                      uint32_t* count);

#ifdef __cplusplus
}
#endif

#endif
