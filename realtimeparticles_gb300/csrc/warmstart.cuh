// warmstart.cuh - learned warm start of the PBF constraint solve: launchers (warmstart.cu,
// mlp_train.cu) shared with the runtime.
#pragma once

#include "fluids.cuh"
#include "mlp.cuh"

namespace rtp {

// Device-side solver statistics (rtp_solver_stats).
struct SolverStatsDev {
  unsigned long long steps;
  unsigned long long reruns;
  double sumErr;
  double maxErr;
  double sumFirst;
};

// Feature sweep of the first Jacobi iteration at the predicted positions `pred`.
//   record: plain lambda (and total lambda = lambda); raw features of the sampled particles
//           (phase, phase + stride, ...) to feats[k][12].
//   infer:  the network's lambda (also the total lambda) and residual displacement res.
// Both record the pairs within h into pl.
int ws_lambda_record(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                     uint32_t stride, uint32_t phase, float* feats, uint32_t capacity, Launcher& L);
int ws_lambda_infer(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                    const void* mlpBlock, float4* res, Launcher& L);
// Targets of the sampled particles: total lambda, then xFinal - x0 - dp(total lambda) at x0
// over the pairs pl0 recorded at x0.
int ws_record_targets(const GridK& g, const FluidK& p, const float4* x0, const float* lamTot, const uint2* table,
                      uint32_t n, const float4* xFinal, const PairList& pl0, uint32_t stride, uint32_t phase,
                      uint32_t count, float* targets, Launcher& L);
// Per-block sums of |rho_i / rho0 - 1| at `pos` by a 27-cell search (when no vorticity sweep runs).
int ws_density_error(const GridK& g, const FluidK& p, const float4* pos, const uint2* table, uint32_t n,
                     float* errPartial, Launcher& L);
// Guard: mean error from the partials; updates the statistics; with a conditional handle
// sets it to 1 when the step must rerun with the plain solver.  accept = the rerun's error.
int ws_guard(const float* errPartial, uint32_t n, float tol, SolverStatsDev* st, cudaGraphConditionalHandle hnd,
             bool hasCond, bool accept, Launcher& L);
inline uint32_t ws_error_blocks(uint32_t n) { return (n + kSweepThreads - 1) / kSweepThreads; }

// ---- network (mlp_train.cu) -------------------------------------------------------------
// FP32 master parameters (MlpParamOffsets order) + normalisation -> packed BF16 block.
int mlp_pack(const float* master, const float* inMean, const float* inScale, const float* outScale, void* block,
             cudaStream_t s);
// Host rtp_mlp -> packed block (uploads the master parameters through `tmp`, which holds
// mlp_upload_tmp_floats() floats of device memory); returns after the stream is idle.
int mlp_upload_packed(const rtp_mlp& net, float* tmp, void* block, cudaStream_t s);
size_t mlp_upload_tmp_floats();

}  // namespace rtp
