// mlp_train.cu - the warm-start network's own training kernels (BF16 tensor cores, FP32
// accumulate) and the stand-alone inference kernel.
//
// One Adam step over a minibatch of B samples:
//   k_train_fwd_bwd  one warp per 16-sample tile: gathers and normalises the features, runs
//                    the three layers (mma.m16n8k16), the loss and the per-sample backward
//                    pass (dH2 = dY W3, dH1 = dZ2 W2, times GELU'), and stores the BF16
//                    operands of the weight gradients transposed ([feature][sample])
//   k_train_wgrad    split-K weight gradients dW = dZ^T H over sample chunks, one partial
//                    per block (48 16x8 output tiles over 8 warps) + bias row sums
//   k_train_adam     partials summed in block order (deterministic), AdamW on the FP32
//                    master copy
//   k_mlp_pack       master copy -> the packed BF16 fragment block used by every forward
// The normalisation (feature mean / std, target RMS) comes from k_norm_partial.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "warmstart.cuh"

namespace rtp {

constexpr int kParams = MlpParamOffsets::count;

// ---- packing -------------------------------------------------------------------------------
__device__ __forceinline__ float wget(const float* w, int rows, int cols, int r, int c) {
  return (r < rows && c < cols) ? w[r * cols + c] : 0.0f;
}

// Forward fragment (B[k][n] = W[n][k]) of n-tile nt, k-step ks for `lane`.
__device__ __forceinline__ uint2 frag_fwd(const float* w, int rows, int cols, int nt, int ks, int lane) {
  const int n = nt * 8 + (lane >> 2), k0 = ks * 16 + 2 * (lane & 3);
  return make_uint2(pack_bf16(wget(w, rows, cols, n, k0), wget(w, rows, cols, n, k0 + 1)),
                    pack_bf16(wget(w, rows, cols, n, k0 + 8), wget(w, rows, cols, n, k0 + 9)));
}
// Backward fragment (B[k][n] = W[k][n]: k = output, n = input).
__device__ __forceinline__ uint2 frag_bwd(const float* w, int rows, int cols, int nt, int ks, int lane) {
  const int n = nt * 8 + (lane >> 2), k0 = ks * 16 + 2 * (lane & 3);
  return make_uint2(pack_bf16(wget(w, rows, cols, k0, n), wget(w, rows, cols, k0 + 1, n)),
                    pack_bf16(wget(w, rows, cols, k0 + 8, n), wget(w, rows, cols, k0 + 9, n)));
}

__global__ void k_mlp_pack(const float* __restrict__ mp, const float* __restrict__ inMean,
                           const float* __restrict__ inScale, const float* __restrict__ outScale, char* __restrict__ blk) {
  using O = MlpParamOffsets;
  using B = MlpLayout;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // Fragments: w1f 8x1, w2f 8x4, w3f 1x4, w2b 8x4, w3b 8x1 (x 32 lanes).
  int f = t;
  if (f < 8 * 32) {
    ((uint2*)(blk + B::w1f))[f] = frag_fwd(mp + O::w1, kMlpHidden, kMlpIn, f / 32, 0, f % 32);
    return;
  }
  f -= 8 * 32;
  if (f < 8 * 4 * 32) {
    const int tile = f / 32;
    ((uint2*)(blk + B::w2f))[f] = frag_fwd(mp + O::w2, kMlpHidden, kMlpHidden, tile / 4, tile % 4, f % 32);
    return;
  }
  f -= 8 * 4 * 32;
  if (f < 4 * 32) {
    ((uint2*)(blk + B::w3f))[f] = frag_fwd(mp + O::w3, kMlpOut, kMlpHidden, 0, f / 32, f % 32);
    return;
  }
  f -= 4 * 32;
  if (f < 8 * 4 * 32) {
    const int tile = f / 32;
    ((uint2*)(blk + B::w2b))[f] = frag_bwd(mp + O::w2, kMlpHidden, kMlpHidden, tile / 4, tile % 4, f % 32);
    return;
  }
  f -= 8 * 4 * 32;
  if (f < 8 * 32) {
    ((uint2*)(blk + B::w3b))[f] = frag_bwd(mp + O::w3, kMlpOut, kMlpHidden, f / 32, 0, f % 32);
    return;
  }
  f -= 8 * 32;
  if (f < kMlpHidden) {
    ((float*)(blk + B::b1))[f] = mp[O::b1 + f];
    ((float*)(blk + B::b2))[f] = mp[O::b2 + f];
    return;
  }
  f -= kMlpHidden;
  if (f < 16) {
    if (f < 8) ((float*)(blk + B::b3))[f] = f < kMlpOut ? mp[O::b3 + f] : 0.0f;
    ((float*)(blk + B::inMean))[f] = f < kMlpIn ? inMean[f] : 0.0f;
    ((float*)(blk + B::inScale))[f] = f < kMlpIn ? inScale[f] : 0.0f;
    if (f < 8) ((float*)(blk + B::outScale))[f] = f < kMlpOut ? outScale[f] : 0.0f;
  }
}
constexpr int kPackItems = 8 * 32 + 8 * 4 * 32 + 4 * 32 + 8 * 4 * 32 + 8 * 32 + kMlpHidden + 16;

// ---- inference on stand-alone rows ----------------------------------------------------------
__global__ void __launch_bounds__(128) k_mlp_forward_rows(MlpDev m, const float* __restrict__ feats, uint64_t n,
                                                          float* __restrict__ out) {
  __shared__ uint32_t s_stage[4][32 * 9];
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = r < n;
  float x[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k)
    x[k] = active ? (feats[r * kMlpIn + k] - __ldg(m.inMean + k)) * __ldg(m.inScale + k) : 0.0f;
  float y[kMlpOut];
  mlp_warp_forward(m, x, y, s_stage[threadIdx.x >> 5]);
  if (!active) return;
#pragma unroll
  for (int o = 0; o < kMlpOut; ++o) out[r * kMlpOut + o] = y[o] * __ldg(m.outScale + o);
}

// ---- training -------------------------------------------------------------------------------
// Transposed BF16 operands of one minibatch: rows x ld (ld = padded sample count).
struct TrainAct {
  __nv_bfloat16* xT;    // 16 rows (inputs, 12..15 zero)
  __nv_bfloat16* h1T;   // 64
  __nv_bfloat16* h2T;   // 64
  __nv_bfloat16* dz1T;  // 64
  __nv_bfloat16* dz2T;  // 64
  __nv_bfloat16* dyT;   // 16 (outputs, 4..15 zero)
  uint32_t ld;
};
constexpr int kActRows = 16 + 64 + 64 + 64 + 64 + 16;

struct LossW {
  float w[kMlpOut];
};

__device__ __forceinline__ void st_bf16(__nv_bfloat16* T, uint32_t ld, uint32_t row, uint32_t col, uint32_t packed) {
  const uint16_t lo = (uint16_t)(packed & 0xFFFFu), hi = (uint16_t)(packed >> 16);
  reinterpret_cast<uint16_t*>(T)[(size_t)row * ld + col] = lo;
  reinterpret_cast<uint16_t*>(T)[(size_t)(row + 1) * ld + col] = hi;
}

// Stores the 4 k-step A fragments of a 16 x 64 activation tile (rows = samples s0..s0+15)
// transposed into T[64][ld].
__device__ __forceinline__ void store_a_frags_T(__nv_bfloat16* T, uint32_t ld, uint32_t s0, const uint32_t (&a)[4][4],
                                                uint32_t lane) {
  const uint32_t g = lane >> 2, c = lane & 3;
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint32_t k0 = ks * 16 + 2 * c;
    st_bf16(T, ld, k0, s0 + g, a[ks][0]);
    st_bf16(T, ld, k0, s0 + g + 8, a[ks][1]);
    st_bf16(T, ld, k0 + 8, s0 + g, a[ks][2]);
    st_bf16(T, ld, k0 + 8, s0 + g + 8, a[ks][3]);
  }
}

__device__ __forceinline__ void d_to_a(const float (&z)[kMlpH8][4], uint32_t (&a)[kMlpH16][4]) {
#pragma unroll
  for (int ks = 0; ks < kMlpH16; ++ks) {
    a[ks][0] = pack_bf16(z[2 * ks][0], z[2 * ks][1]);
    a[ks][1] = pack_bf16(z[2 * ks][2], z[2 * ks][3]);
    a[ks][2] = pack_bf16(z[2 * ks + 1][0], z[2 * ks + 1][1]);
    a[ks][3] = pack_bf16(z[2 * ks + 1][2], z[2 * ks + 1][3]);
  }
}

// Minibatch rows [0, B) are samples perm[base + r] (or base + r without perm).  dY carries
// the factor invTotal (1 / samples of the loss).  lossPart[tile] = sum of w_o (y - t)^2.
// With dyIn (rows of kMlpOut) the output gradient is given instead of the regression loss's:
// dY = dyIn, no loss.
__global__ void __launch_bounds__(128) k_train_fwd_bwd(MlpDev m, const float* __restrict__ feats,
                                                       const float* __restrict__ targets,
                                                       const uint32_t* __restrict__ perm, uint64_t base, uint32_t B,
                                                       LossW lw, float invTotal, TrainAct act,
                                                       float* __restrict__ lossPart, const float* __restrict__ dyIn) {
  const uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
  const uint32_t s0 = tile * 16;
  if (s0 >= B) return;  // uniform per warp
  const uint32_t rA = s0 + g, rB = s0 + g + 8;
  const bool vA = rA < B, vB = rB < B;
  const uint64_t iA = vA ? (perm ? (uint64_t)perm[base + rA] : base + rA) : 0;
  const uint64_t iB = vB ? (perm ? (uint64_t)perm[base + rB] : base + rB) : 0;
  // Inputs: columns 2c, 2c+1, 2c+8, 2c+9 of rows rA, rB.
  float xa[4], xb[4];
  const int cols[4] = {(int)(2 * c), (int)(2 * c + 1), (int)(2 * c + 8), (int)(2 * c + 9)};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int col = cols[j];
    const bool cv = col < kMlpIn;
    const float mu = cv ? __ldg(m.inMean + col) : 0.0f, sc = cv ? __ldg(m.inScale + col) : 0.0f;
    xa[j] = (vA && cv) ? (feats[iA * kMlpIn + col] - mu) * sc : 0.0f;
    xb[j] = (vB && cv) ? (feats[iB * kMlpIn + col] - mu) * sc : 0.0f;
  }
  uint32_t a0[4] = {pack_bf16(xa[0], xa[1]), pack_bf16(xb[0], xb[1]), pack_bf16(xa[2], xa[3]),
                    pack_bf16(xb[2], xb[3])};
  st_bf16(act.xT, act.ld, 2 * c, rA, a0[0]);
  st_bf16(act.xT, act.ld, 2 * c, rB, a0[1]);
  st_bf16(act.xT, act.ld, 2 * c + 8, rA, a0[2]);
  st_bf16(act.xT, act.ld, 2 * c + 8, rB, a0[3]);

  // Forward.
  float z1[kMlpH8][4], z2[kMlpH8][4];
  uint32_t h1[kMlpH16][4], h2[kMlpH16][4];
  mlp_layer1(m, a0, z1, lane);
  gelu_to_a(z1, h1);
  mlp_layer2<kMlpH8>(m, h1, 0, z2, lane);
  gelu_to_a(z2, h2);
  float y[4];
  {
    const float2 b3 = c < 2 ? __ldg(reinterpret_cast<const float2*>(m.b3 + 2 * c)) : make_float2(0.f, 0.f);
    y[0] = b3.x;
    y[1] = b3.y;
    y[2] = b3.x;
    y[3] = b3.y;
#pragma unroll
    for (int ks = 0; ks < kMlpH16; ++ks) mma_bf16(y, h2[ks], __ldg(m.w3f + ks * 32 + lane));
  }
  // Loss and dY (columns 2c, 2c+1 of rows rA, rB; outputs live in lanes c < 2).
  float dy[4] = {0.f, 0.f, 0.f, 0.f};
  float loss = 0.0f;
  if (c < 2) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int o = 2 * c + (j & 1);
      const bool rowA = j < 2;
      if ((rowA ? vA : vB) && dyIn) {
        dy[j] = dyIn[(rowA ? iA : iB) * kMlpOut + o];
      } else if (rowA ? vA : vB) {
        const uint64_t idx = rowA ? iA : iB;
        const float t = targets[idx * kMlpOut + o] / __ldg(m.outScale + o);
        const float d = y[j] - t;
        loss += lw.w[o] * d * d;
        dy[j] = 2.0f * lw.w[o] * d * invTotal;
      }
    }
  }
  const uint32_t ady[4] = {pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], dy[3]), 0u, 0u};
  if (c < 2) {
    st_bf16(act.dyT, act.ld, 2 * c, rA, ady[0]);
    st_bf16(act.dyT, act.ld, 2 * c, rB, ady[1]);
  }
  // Backward through layer 3 and GELU: dZ2 = (dY W3) * gelu'(Z2).
  float dz[kMlpH8][4];
#pragma unroll
  for (int nt = 0; nt < kMlpH8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma_bf16(d, ady, __ldg(m.w3b + nt * 32 + lane));
#pragma unroll
    for (int j = 0; j < 4; ++j) dz[nt][j] = d[j] * gelu_grad(z2[nt][j]);
  }
  uint32_t adz2[kMlpH16][4];
  d_to_a(dz, adz2);
  // dZ1 = (dZ2 W2) * gelu'(Z1).
#pragma unroll
  for (int nt = 0; nt < kMlpH8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < kMlpH16; ++ks) mma_bf16(d, adz2[ks], __ldg(m.w2b + (nt * kMlpH16 + ks) * 32 + lane));
#pragma unroll
    for (int j = 0; j < 4; ++j) dz[nt][j] = d[j] * gelu_grad(z1[nt][j]);
  }
  uint32_t adz1[kMlpH16][4];
  d_to_a(dz, adz1);
  store_a_frags_T(act.h1T, act.ld, s0, h1, lane);
  store_a_frags_T(act.h2T, act.ld, s0, h2, lane);
  store_a_frags_T(act.dz2T, act.ld, s0, adz2, lane);
  store_a_frags_T(act.dz1T, act.ld, s0, adz1, lane);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
  if (lane == 0) lossPart[tile] = loss;
}

// Split-K weight gradients over samples [blk * chunk, min(+chunk, Bpad)).
constexpr int kWgradThreads = 256;
__global__ void __launch_bounds__(kWgradThreads) k_train_wgrad(TrainAct act, uint32_t chunk, uint32_t Bpad,
                                                               float* __restrict__ partials) {
  using O = MlpParamOffsets;
  const uint32_t sb = blockIdx.x * chunk, se = min(sb + chunk, Bpad);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, c = lane & 3;
  float* out = partials + (size_t)blockIdx.x * kParams;
  const uint32_t ld = act.ld;
  for (uint32_t tile = warp; tile < 48; tile += kWgradThreads / 32) {
    const __nv_bfloat16 *A, *Bm;
    uint32_t mt, nt, mReal, nReal, woff, ncols;
    if (tile < 32) {
      A = act.dz2T, Bm = act.h1T, mt = tile / 8, nt = tile % 8, mReal = 64, nReal = 64, woff = O::w2, ncols = 64;
    } else if (tile < 40) {
      const uint32_t t = tile - 32;
      A = act.dz1T, Bm = act.xT, mt = t / 2, nt = t % 2, mReal = 64, nReal = kMlpIn, woff = O::w1, ncols = kMlpIn;
    } else {
      A = act.dyT, Bm = act.h2T, mt = 0, nt = tile - 40, mReal = kMlpOut, nReal = 64, woff = O::w3, ncols = 64;
    }
    const uint32_t* Aw = reinterpret_cast<const uint32_t*>(A);
    const uint32_t* Bw = reinterpret_cast<const uint32_t*>(Bm);
    const uint32_t m0 = mt * 16, n0 = nt * 8;
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t k0 = sb; k0 < se; k0 += 16) {
      uint32_t a[4];
      a[0] = __ldg(Aw + ((size_t)(m0 + g) * ld + k0 + 2 * c) / 2);
      a[1] = __ldg(Aw + ((size_t)(m0 + g + 8) * ld + k0 + 2 * c) / 2);
      a[2] = __ldg(Aw + ((size_t)(m0 + g) * ld + k0 + 2 * c + 8) / 2);
      a[3] = __ldg(Aw + ((size_t)(m0 + g + 8) * ld + k0 + 2 * c + 8) / 2);
      uint2 b;
      b.x = __ldg(Bw + ((size_t)(n0 + g) * ld + k0 + 2 * c) / 2);
      b.y = __ldg(Bw + ((size_t)(n0 + g) * ld + k0 + 2 * c + 8) / 2);
      mma_bf16(d, a, b);
    }
    const uint32_t r0 = m0 + g, r1 = m0 + g + 8, c0 = n0 + 2 * c, c1 = c0 + 1;
    if (r0 < mReal && c0 < nReal) out[woff + r0 * ncols + c0] = d[0];
    if (r0 < mReal && c1 < nReal) out[woff + r0 * ncols + c1] = d[1];
    if (r1 < mReal && c0 < nReal) out[woff + r1 * ncols + c0] = d[2];
    if (r1 < mReal && c1 < nReal) out[woff + r1 * ncols + c1] = d[3];
  }
  // Bias gradients: row sums of dZ1^T, dZ2^T, dY^T over the chunk.
  for (uint32_t r = threadIdx.x; r < 64 + 64 + kMlpOut; r += kWgradThreads) {
    const __nv_bfloat16* row;
    uint32_t dst;
    if (r < 64) row = act.dz1T + (size_t)r * ld, dst = O::b1 + r;
    else if (r < 128) row = act.dz2T + (size_t)(r - 64) * ld, dst = O::b2 + (r - 64);
    else row = act.dyT + (size_t)(r - 128) * ld, dst = O::b3 + (r - 128);
    float s = 0.0f;
    for (uint32_t k = sb; k < se; ++k) s += __bfloat162float(row[k]);
    out[dst] = s;
  }
}

struct AdamStep {
  float lr, beta1, beta2, eps, wd, bc1, bc2;
};

// Sums the partials in block order; with grad != nullptr writes the gradient, else AdamW.
__global__ void k_train_adam(const float* __restrict__ partials, uint32_t nblk, float* __restrict__ master,
                             float* __restrict__ mom, float* __restrict__ var, AdamStep st, float* __restrict__ grad) {
  using O = MlpParamOffsets;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  float gs = 0.0f;
  for (uint32_t b = 0; b < nblk; ++b) gs += partials[(size_t)b * kParams + p];
  if (grad) {
    grad[p] = gs;
    return;
  }
  const float mm = st.beta1 * mom[p] + (1.0f - st.beta1) * gs;
  const float vv = st.beta2 * var[p] + (1.0f - st.beta2) * gs * gs;
  mom[p] = mm;
  var[p] = vv;
  const bool isWeight = p < O::b1 || (p >= O::w2 && p < O::b2) || (p >= O::w3 && p < O::b3);
  const float w = master[p];
  const float upd = (mm / st.bc1) / (sqrtf(vv / st.bc2) + st.eps) + (isWeight ? st.wd * w : 0.0f);
  master[p] = w - st.lr * upd;
}

// acc += sum of v[0..n) (one block, fixed order).
__global__ void __launch_bounds__(256) k_sum_into(const float* __restrict__ v, uint32_t n, double* acc) {
  __shared__ double s[256];
  double a = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += 256) a += (double)v[i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *acc += s[0];
}

// Normalisation statistics: per block sums over a contiguous sample range.
// out[blk][0..11] = sum f, [12..23] = sum f^2, [24..27] = sum t^2.
constexpr int kNormStats = 2 * kMlpIn + kMlpOut;
__global__ void __launch_bounds__(256) k_norm_partial(const float* __restrict__ feats, const float* __restrict__ targets,
                                                      uint64_t n, uint64_t per, double* __restrict__ out) {
  __shared__ double s[256];
  const uint64_t b0 = (uint64_t)blockIdx.x * per, b1 = min(b0 + per, n);
  for (int q = 0; q < kNormStats; ++q) {
    double a = 0.0;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += 256) {
      double v;
      if (q < kMlpIn) v = feats[i * kMlpIn + q];
      else if (q < 2 * kMlpIn) {
        v = feats[i * kMlpIn + (q - kMlpIn)];
        v *= v;
      } else {
        v = targets[i * kMlpOut + (q - 2 * kMlpIn)];
        v *= v;
      }
      a += v;
    }
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * kNormStats + q] = s[0];
    __syncthreads();
  }
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}

int mlp_pack(const float* master, const float* inMean, const float* inScale, const float* outScale, void* block,
             cudaStream_t s) {
  k_mlp_pack<<<(kPackItems + 255) / 256, 256, 0, s>>>(master, inMean, inScale, outScale, (char*)block);
  return check("k_mlp_pack");
}

// Host rtp_mlp <-> flat arrays.
static void net_to_master(const rtp_mlp& net, float* mp) {
  using O = MlpParamOffsets;
  std::memcpy(mp + O::w1, net.w1, sizeof(net.w1));
  std::memcpy(mp + O::b1, net.b1, sizeof(net.b1));
  std::memcpy(mp + O::w2, net.w2, sizeof(net.w2));
  std::memcpy(mp + O::b2, net.b2, sizeof(net.b2));
  std::memcpy(mp + O::w3, net.w3, sizeof(net.w3));
  std::memcpy(mp + O::b3, net.b3, sizeof(net.b3));
}
static void master_to_net(const float* mp, rtp_mlp& net) {
  using O = MlpParamOffsets;
  std::memcpy(net.w1, mp + O::w1, sizeof(net.w1));
  std::memcpy(net.b1, mp + O::b1, sizeof(net.b1));
  std::memcpy(net.w2, mp + O::w2, sizeof(net.w2));
  std::memcpy(net.b2, mp + O::b2, sizeof(net.b2));
  std::memcpy(net.w3, mp + O::w3, sizeof(net.w3));
  std::memcpy(net.b3, mp + O::b3, sizeof(net.b3));
}

// tmp: kParams + 32 floats of device memory.
constexpr int kNormFloats = 16 + 16 + 8;
int mlp_upload_packed(const rtp_mlp& net, float* tmp, void* block, cudaStream_t s) {
  std::vector<float> h(kParams + kNormFloats, 0.0f);
  net_to_master(net, h.data());
  std::memcpy(h.data() + kParams, net.inMean, sizeof(net.inMean));
  std::memcpy(h.data() + kParams + 16, net.inScale, sizeof(net.inScale));
  std::memcpy(h.data() + kParams + 32, net.outScale, sizeof(net.outScale));
  RTP_CUDA(cudaMemcpyAsync(tmp, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  const int rc = mlp_pack(tmp, tmp + kParams, tmp + kParams + 16, tmp + kParams + 32, block, s);
  if (rc) return rc;
  RTP_CUDA(cudaStreamSynchronize(s));  // h goes out of scope
  return RTP_OK;
}
size_t mlp_upload_tmp_floats() { return kParams + kNormFloats; }

// ---- scoped device allocations for the host entry points -------------------------------------
struct DevArena {
  std::vector<void*> ptrs;
  ~DevArena() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  int alloc(T** p, size_t count, bool zero = true) {
    *p = nullptr;
    if (count == 0) count = 1;
    RTP_CUDA(cudaMalloc((void**)p, count * sizeof(T)));
    ptrs.push_back((void*)*p);
    if (zero) RTP_CUDA(cudaMemset(*p, 0, count * sizeof(T)));
    return RTP_OK;
  }
};

#define RTP_TRY2(x)          \
  do {                       \
    int _rc = (x);           \
    if (_rc) return _rc;     \
  } while (0)

constexpr uint32_t kWgradChunk = 512;

struct Trainer {
  DevArena A;
  float *master = nullptr, *mom = nullptr, *var = nullptr, *partials = nullptr, *lossPart = nullptr, *norm = nullptr;
  void* block = nullptr;
  TrainAct act{};
  uint32_t cap = 0;  // padded minibatch capacity
  double* lossAcc = nullptr;

  int init(uint32_t batchCap) {
    cap = (batchCap + 15) / 16 * 16;
    const uint32_t nblk = (cap + kWgradChunk - 1) / kWgradChunk;
    RTP_TRY2(A.alloc(&master, kParams));
    RTP_TRY2(A.alloc(&mom, kParams));
    RTP_TRY2(A.alloc(&var, kParams));
    RTP_TRY2(A.alloc(&partials, (size_t)nblk * kParams));
    RTP_TRY2(A.alloc(&lossPart, cap / 16));
    RTP_TRY2(A.alloc(&norm, kNormFloats));
    RTP_TRY2(A.alloc(&lossAcc, 1));
    char* blk = nullptr;
    RTP_TRY2(A.alloc(&blk, MlpLayout::bytes));
    block = blk;
    __nv_bfloat16* base = nullptr;
    RTP_TRY2(A.alloc(&base, (size_t)kActRows * cap));
    act.ld = cap;
    act.xT = base;
    act.h1T = act.xT + (size_t)16 * cap;
    act.h2T = act.h1T + (size_t)64 * cap;
    act.dz1T = act.h2T + (size_t)64 * cap;
    act.dz2T = act.dz1T + (size_t)64 * cap;
    act.dyT = act.dz2T + (size_t)64 * cap;
    return RTP_OK;
  }

  int set_net(const rtp_mlp& net, cudaStream_t s) {
    std::vector<float> h(kParams);
    net_to_master(net, h.data());
    RTP_CUDA(cudaMemcpyAsync(master, h.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, s));
    std::vector<float> nm(kNormFloats, 0.0f);
    std::memcpy(nm.data(), net.inMean, sizeof(net.inMean));
    std::memcpy(nm.data() + 16, net.inScale, sizeof(net.inScale));
    std::memcpy(nm.data() + 32, net.outScale, sizeof(net.outScale));
    RTP_CUDA(cudaMemcpyAsync(norm, nm.data(), kNormFloats * sizeof(float), cudaMemcpyHostToDevice, s));
    RTP_TRY2(repack(s));
    RTP_CUDA(cudaStreamSynchronize(s));
    return RTP_OK;
  }

  int repack(cudaStream_t s) { return mlp_pack(master, norm, norm + 16, norm + 32, block, s); }

  // Forward + backward + weight gradients of rows [base, base + B) (through perm); with dyIn
  // the output gradient is given (rows of kMlpOut) and targets are not read.
  int grads(const float* feats, const float* targets, const uint32_t* perm, uint64_t base, uint32_t B,
            const LossW& lw, float invTotal, cudaStream_t s, uint32_t* nblkOut, const float* dyIn = nullptr) {
    const uint32_t tiles = (B + 15) / 16;
    const uint32_t Bpad = tiles * 16;
    k_train_fwd_bwd<<<(tiles + 3) / 4, 128, 0, s>>>(mlp_dev(block), feats, targets, perm, base, B, lw, invTotal, act,
                                                    lossPart, dyIn);
    RTP_TRY2(check("k_train_fwd_bwd"));
    const uint32_t nblk = (Bpad + kWgradChunk - 1) / kWgradChunk;
    k_train_wgrad<<<nblk, kWgradThreads, 0, s>>>(act, kWgradChunk, Bpad, partials);
    RTP_TRY2(check("k_train_wgrad"));
    k_sum_into<<<1, 256, 0, s>>>(lossPart, tiles, lossAcc);
    RTP_TRY2(check("k_sum_into"));
    *nblkOut = nblk;
    return RTP_OK;
  }
};

static uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double uniform01(uint64_t& x) { return (double)(splitmix64(x) >> 11) * (1.0 / 9007199254740992.0); }

// ---- trainer for the runtime (training through the solve) ----------------------------------
struct WsTrainer {
  Trainer T;
  uint64_t steps = 0;
};

int ws_trainer_create(uint32_t cap, WsTrainer** out) {
  *out = nullptr;
  WsTrainer* t = new WsTrainer();
  const int rc = t->T.init(cap);
  if (rc) {
    delete t;
    return rc;
  }
  *out = t;
  return RTP_OK;
}
void ws_trainer_destroy(WsTrainer* t) { delete t; }
const void* ws_trainer_block(const WsTrainer* t) { return t->T.block; }

int ws_trainer_set_net(WsTrainer* t, const rtp_mlp& net, cudaStream_t s) {
  RTP_CUDA(cudaMemsetAsync(t->T.mom, 0, kParams * sizeof(float), s));
  RTP_CUDA(cudaMemsetAsync(t->T.var, 0, kParams * sizeof(float), s));
  t->steps = 0;
  return t->T.set_net(net, s);
}

int ws_trainer_get_net(WsTrainer* t, rtp_mlp& net, cudaStream_t s) {
  std::vector<float> h(kParams);
  RTP_CUDA(cudaMemcpyAsync(h.data(), t->T.master, kParams * sizeof(float), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaStreamSynchronize(s));
  master_to_net(h.data(), net);
  return RTP_OK;
}

int ws_trainer_forward(WsTrainer* t, const float* feats, uint32_t n, float* y, cudaStream_t s) {
  if (n == 0) return RTP_OK;
  k_mlp_forward_rows<<<(n + 127) / 128, 128, 0, s>>>(mlp_dev(t->T.block), feats, n, y);
  return check("k_mlp_forward_rows");
}

int ws_trainer_adam_step(WsTrainer* t, const float* feats, const float* dy, uint32_t n, const rtp_train_config& cfg,
                         double lrScale, cudaStream_t s) {
  if (n == 0) return RTP_OK;
  LossW lw{};
  uint32_t nblk = 0;
  RTP_TRY2(t->T.grads(feats, nullptr, nullptr, 0, n, lw, 1.0f, s, &nblk, dy));
  ++t->steps;
  AdamStep st;
  st.lr = (float)(cfg.learningRate * lrScale);
  st.beta1 = cfg.beta1;
  st.beta2 = cfg.beta2;
  st.eps = cfg.eps;
  st.wd = cfg.weightDecay;
  st.bc1 = (float)(1.0 - std::pow((double)cfg.beta1, (double)t->steps));
  st.bc2 = (float)(1.0 - std::pow((double)cfg.beta2, (double)t->steps));
  k_train_adam<<<(kParams + 255) / 256, 256, 0, s>>>(t->T.partials, nblk, t->T.master, t->T.mom, t->T.var, st, nullptr);
  RTP_TRY2(check("k_train_adam"));
  return t->T.repack(s);
}

int ws_init_net(const float* feats, uint64_t n, uint64_t seed, rtp_mlp& net, cudaStream_t s) {
  if (n == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "no feature rows");
  DevArena A;
  const uint64_t per = 65536;
  const uint32_t nb = (uint32_t)((n + per - 1) / per);
  double* part = nullptr;
  float* tz = nullptr;
  RTP_TRY2(A.alloc(&part, (size_t)nb * kNormStats));
  RTP_TRY2(A.alloc(&tz, (size_t)n * kMlpOut));
  k_norm_partial<<<nb, 256, 0, s>>>(feats, tz, n, per, part);
  RTP_TRY2(check("k_norm_partial"));
  std::vector<double> h((size_t)nb * kNormStats);
  RTP_CUDA(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaStreamSynchronize(s));
  double sum[kNormStats] = {0};
  for (uint32_t b = 0; b < nb; ++b)
    for (int q = 0; q < kNormStats; ++q) sum[q] += h[(size_t)b * kNormStats + q];
  std::memset(&net, 0, sizeof(net));
  for (int k = 0; k < kMlpIn; ++k) {
    const double mu = sum[k] / (double)n;
    const double sd = std::sqrt(std::max(0.0, sum[kMlpIn + k] / (double)n - mu * mu));
    net.inMean[k] = (float)mu;
    net.inScale[k] = sd > 1e-30 * (std::fabs(mu) + 1e-30) && sd > 0.0 ? (float)(1.0 / sd) : 1.0f;
  }
  for (int o = 0; o < kMlpOut; ++o) net.outScale[o] = 1.0f;
  uint64_t rs = seed ^ 0x5DEECE66Dull;
  auto fill = [&](float* w, int rows, int cols) {
    const double a = std::sqrt(6.0 / (double)(rows + cols));
    for (int i = 0; i < rows * cols; ++i) w[i] = (float)((2.0 * uniform01(rs) - 1.0) * a);
  };
  fill(&net.w1[0][0], kMlpHidden, kMlpIn);
  fill(&net.w2[0][0], kMlpHidden, kMlpHidden);
  return RTP_OK;
}

}  // namespace rtp

using namespace rtp;

extern "C" {

int rtp_mlp_backward(const rtp_mlp* net, const float* d_features, const float* d_dy, uint64_t n, rtp_mlp* grad,
                     void* stream) {
  if (!net || !d_features || !d_dy || !grad) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0 || n > (1u << 24)) return fail(RTP_ERR_INVALID_ARGUMENT, "sample count must be in [1, 2^24]");
  cudaStream_t s = (cudaStream_t)stream;
  Trainer T;
  RTP_TRY2(T.init((uint32_t)n));
  RTP_TRY2(T.set_net(*net, s));
  LossW lw{};
  uint32_t nblk = 0;
  RTP_TRY2(T.grads(d_features, nullptr, nullptr, 0, (uint32_t)n, lw, 1.0f, s, &nblk, d_dy));
  float* g = nullptr;
  RTP_TRY2(T.A.alloc(&g, kParams));
  AdamStep st{};
  k_train_adam<<<(kParams + 255) / 256, 256, 0, s>>>(T.partials, nblk, T.master, T.mom, T.var, st, g);
  RTP_TRY2(check("k_train_adam(grad)"));
  std::vector<float> h(kParams);
  RTP_CUDA(cudaMemcpyAsync(h.data(), g, kParams * sizeof(float), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaStreamSynchronize(s));
  std::memset(grad, 0, sizeof(*grad));
  master_to_net(h.data(), *grad);
  return RTP_OK;
}

int rtp_mlp_forward(const rtp_mlp* net, const float* d_features, uint64_t n, float* d_out, void* stream) {
  if (!net || (!d_features && n) || (!d_out && n)) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return RTP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  DevArena A;
  float* tmp = nullptr;
  char* blk = nullptr;
  RTP_TRY2(A.alloc(&tmp, mlp_upload_tmp_floats()));
  RTP_TRY2(A.alloc(&blk, MlpLayout::bytes));
  RTP_TRY2(mlp_upload_packed(*net, tmp, blk, s));
  k_mlp_forward_rows<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(mlp_dev(blk), d_features, n, d_out);
  RTP_TRY2(check("k_mlp_forward_rows"));
  RTP_CUDA(cudaStreamSynchronize(s));
  return RTP_OK;
}

int rtp_mlp_loss_grad(const rtp_mlp* net, const float* lossWeights, const float* d_features, const float* d_targets,
                      uint64_t n, double* loss, rtp_mlp* grad, void* stream) {
  if (!net || !lossWeights || !loss || !grad || !d_features || !d_targets)
    return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0 || n > (1u << 24)) return fail(RTP_ERR_INVALID_ARGUMENT, "sample count must be in [1, 2^24]");
  cudaStream_t s = (cudaStream_t)stream;
  Trainer T;
  RTP_TRY2(T.init((uint32_t)n));
  RTP_TRY2(T.set_net(*net, s));
  LossW lw;
  for (int o = 0; o < kMlpOut; ++o) lw.w[o] = lossWeights[o];
  uint32_t nblk = 0;
  RTP_TRY2(T.grads(d_features, d_targets, nullptr, 0, (uint32_t)n, lw, (float)(1.0 / (double)n), s, &nblk));
  float* g = nullptr;
  RTP_TRY2(T.A.alloc(&g, kParams));
  AdamStep st{};
  k_train_adam<<<(kParams + 255) / 256, 256, 0, s>>>(T.partials, nblk, T.master, T.mom, T.var, st, g);
  RTP_TRY2(check("k_train_adam(grad)"));
  std::vector<float> h(kParams);
  double acc = 0.0;
  RTP_CUDA(cudaMemcpyAsync(h.data(), g, kParams * sizeof(float), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaMemcpyAsync(&acc, T.lossAcc, sizeof(double), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaStreamSynchronize(s));
  std::memset(grad, 0, sizeof(*grad));
  master_to_net(h.data(), *grad);
  *loss = acc / (double)n;
  return RTP_OK;
}

int rtp_train_warm_start(const float* d_features, const float* d_targets, uint64_t n, const rtp_train_config* cfg,
                         rtp_mlp* net, float* loss_history, void* stream) {
  if (!d_features || !d_targets || !cfg || !net) return fail(RTP_ERR_INVALID_ARGUMENT, "null argument");
  if (n < 16 || n > (1ull << 31)) return fail(RTP_ERR_INVALID_ARGUMENT, "sample count must be in [16, 2^31]");
  if (cfg->batch < 16 || cfg->epochs == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "batch >= 16 and epochs >= 1 required");
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t B = (uint32_t)std::min<uint64_t>(cfg->batch, n);
  Trainer T;
  RTP_TRY2(T.init(B));

  // Normalisation from the data.
  {
    const uint64_t per = 65536;
    const uint32_t nb = (uint32_t)((n + per - 1) / per);
    double* part = nullptr;
    RTP_TRY2(T.A.alloc(&part, (size_t)nb * kNormStats));
    k_norm_partial<<<nb, 256, 0, s>>>(d_features, d_targets, n, per, part);
    RTP_TRY2(check("k_norm_partial"));
    std::vector<double> h((size_t)nb * kNormStats);
    RTP_CUDA(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    RTP_CUDA(cudaStreamSynchronize(s));
    double sum[kNormStats] = {0};
    for (uint32_t b = 0; b < nb; ++b)
      for (int q = 0; q < kNormStats; ++q) sum[q] += h[(size_t)b * kNormStats + q];
    for (int k = 0; k < kMlpIn; ++k) {
      const double mu = sum[k] / (double)n;
      const double var = std::max(0.0, sum[kMlpIn + k] / (double)n - mu * mu);
      const double sd = std::sqrt(var);
      net->inMean[k] = (float)mu;
      net->inScale[k] = sd > 1e-30 * (std::fabs(mu) + 1e-30) && sd > 0.0 ? (float)(1.0 / sd) : 1.0f;
    }
    for (int o = 0; o < kMlpOut; ++o) {
      const double rms = std::sqrt(sum[2 * kMlpIn + o] / (double)n);
      net->outScale[o] = rms > 0.0 ? (float)rms : 1.0f;
    }
  }
  // Xavier-uniform weights, zero biases.
  {
    uint64_t rs = cfg->seed ^ 0x5DEECE66Dull;
    auto fill = [&](float* w, int rows, int cols) {
      const double a = std::sqrt(6.0 / (double)(rows + cols));
      for (int i = 0; i < rows * cols; ++i) w[i] = (float)((2.0 * uniform01(rs) - 1.0) * a);
    };
    fill(&net->w1[0][0], kMlpHidden, kMlpIn);
    fill(&net->w2[0][0], kMlpHidden, kMlpHidden);
    fill(&net->w3[0][0], kMlpOut, kMlpHidden);
    std::memset(net->b1, 0, sizeof(net->b1));
    std::memset(net->b2, 0, sizeof(net->b2));
    std::memset(net->b3, 0, sizeof(net->b3));
  }
  RTP_TRY2(T.set_net(*net, s));

  uint32_t* perm = nullptr;
  RTP_TRY2(T.A.alloc(&perm, n, false));
  std::vector<uint32_t> hp(n);
  for (uint64_t i = 0; i < n; ++i) hp[i] = (uint32_t)i;
  uint64_t shuffleState = cfg->seed * 0x2545F4914F6CDD1Dull + 1;
  LossW lw;
  for (int o = 0; o < kMlpOut; ++o) lw.w[o] = cfg->lossWeights[o];
  const uint64_t stepsPerEpoch = (n + B - 1) / B;
  const double totalSteps = (double)stepsPerEpoch * cfg->epochs;
  uint64_t step = 0;
  for (uint32_t e = 0; e < cfg->epochs; ++e) {
    for (uint64_t i = n - 1; i > 0; --i) {  // Fisher-Yates
      const uint64_t j = splitmix64(shuffleState) % (i + 1);
      std::swap(hp[i], hp[j]);
    }
    RTP_CUDA(cudaMemcpyAsync(perm, hp.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    RTP_CUDA(cudaMemsetAsync(T.lossAcc, 0, sizeof(double), s));
    for (uint64_t b0 = 0; b0 < n; b0 += B) {
      const uint32_t bs = (uint32_t)std::min<uint64_t>(B, n - b0);
      uint32_t nblk = 0;
      RTP_TRY2(T.grads(d_features, d_targets, perm, b0, bs, lw, 1.0f / (float)bs, s, &nblk));
      ++step;
      const double frac = (double)(step - 1) / std::max(1.0, totalSteps - 1.0);
      const double lrScale = cfg->finalLrFraction + (1.0 - cfg->finalLrFraction) * 0.5 * (1.0 + std::cos(M_PI * frac));
      AdamStep st;
      st.lr = (float)(cfg->learningRate * lrScale);
      st.beta1 = cfg->beta1;
      st.beta2 = cfg->beta2;
      st.eps = cfg->eps;
      st.wd = cfg->weightDecay;
      st.bc1 = (float)(1.0 - std::pow((double)cfg->beta1, (double)step));
      st.bc2 = (float)(1.0 - std::pow((double)cfg->beta2, (double)step));
      k_train_adam<<<(kParams + 255) / 256, 256, 0, s>>>(T.partials, nblk, T.master, T.mom, T.var, st, nullptr);
      RTP_TRY2(check("k_train_adam"));
      RTP_TRY2(T.repack(s));
    }
    double acc = 0.0;
    RTP_CUDA(cudaMemcpyAsync(&acc, T.lossAcc, sizeof(double), cudaMemcpyDeviceToHost, s));
    RTP_CUDA(cudaStreamSynchronize(s));
    if (loss_history) loss_history[e] = (float)(acc / (double)n);
  }
  std::vector<float> h(kParams);
  RTP_CUDA(cudaMemcpyAsync(h.data(), T.master, kParams * sizeof(float), cudaMemcpyDeviceToHost, s));
  RTP_CUDA(cudaStreamSynchronize(s));
  master_to_net(h.data(), *net);
  return RTP_OK;
}

}  // extern "C"
