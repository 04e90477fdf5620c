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
//   infer:  omega(network) x the plain lambda (also the total lambda), and (x, y, z, that
//           lambda) into packed for the correction sweep; omega itself into omegaOut (if set).
// Both record the pairs within h into pl.
int ws_lambda_record(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                     uint32_t stride, uint32_t phase, float* feats, uint32_t capacity, Launcher& L);
int ws_lambda_infer(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                    const void* mlpBlock, float4* packed, float* omegaOut, Launcher& L);
// ---- training through the solve ---------------------------------------------------------
// lamOut = omega(y) lam, packed = (xs, lamOut); y: the network's outputs, rows of RTP_MLP_OUT.
int ws_apply_omega(const float4* xs, const float* lam, const float* y, uint32_t n, float* lamOut, float4* packed,
                   Launcher& L);
// dL/dx' of L = 1/n sum C'^2 (C' from rho2 at xp, pairs pl2), clamp-masked; per-block sums of
// C'^2 into lossPart (ws_loss_blocks(n) entries).
uint32_t ws_loss_blocks(uint32_t n);
int ws_loss_grad_x(const GridK& g, const FluidK& p, const float4* xp, const float* rho2, const uint2* table, uint32_t n,
                   const PairList& pl2, float4* gOut, float* lossPart, Launcher& L);
// dL/dy per particle through the correction at xs with the plain lambda lam (pairs pl), as
// rows of RTP_MLP_OUT (output 0; the others 0).
int ws_grad_y(const GridK& g, const FluidK& p, const float4* xs, const float* lam, const float* y, const float4* gIn,
              const uint2* table, uint32_t n, const PairList& pl, float* dy, Launcher& L);
// dst[ids[i]] = src[i * stride].
int ws_scatter_by_id(const uint32_t* ids, const float* src, uint32_t stride, uint32_t n, float* dst, Launcher& L);
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

// The network's trainer, for training through the solve (mlp_train.cu).
struct WsTrainer;
int ws_trainer_create(uint32_t cap, WsTrainer** out);
void ws_trainer_destroy(WsTrainer* t);
const void* ws_trainer_block(const WsTrainer* t);  // packed BF16 block of the current weights
// A new start: the weights of `net`, zero Adam moments.
int ws_trainer_set_net(WsTrainer* t, const rtp_mlp& net, cudaStream_t s);
int ws_trainer_get_net(WsTrainer* t, rtp_mlp& net, cudaStream_t s);
// y = network(feats) for n rows (rows of RTP_MLP_OUT, times outScale).
int ws_trainer_forward(WsTrainer* t, const float* feats, uint32_t n, float* y, cudaStream_t s);
// One AdamW step with the output gradient dy (rows of RTP_MLP_OUT) over n rows; learning rate
// cfg.learningRate * lrScale.
int ws_trainer_adam_step(WsTrainer* t, const float* feats, const float* dy, uint32_t n, const rtp_train_config& cfg,
                         double lrScale, cudaStream_t s);
// A new network for n feature rows: input normalisation from the rows, Xavier-uniform hidden
// layers from seed, zero output layer, unit output scales.
int ws_init_net(const float* feats, uint64_t n, uint64_t seed, rtp_mlp& net, cudaStream_t s);

}  // namespace rtp
