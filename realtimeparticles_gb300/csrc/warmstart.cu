// warmstart.cu - learned warm start of the PBF constraint solve (new: the reference's Jacobi
// loop, physics/ocl/Fluids.cpp:427-442, always starts from a zero correction).
//
// Per substep with the warm start on:
//   k_ws_lambda<kInfer>   the first density / lambda sweep (fld_computeDensity +
//                         fld_computeConstraintFactor at the predicted positions) also sums
//                         the network's features, then each warp evaluates the MLP for its 32
//                         particles on the tensor cores.  The network's output y sets a
//                         per-particle relaxation omega(y) in (0, 3) of the plain lambda:
//                         lambda_i <- omega_i lambda_i (omega = 1 exactly at y = 0, so a
//                         network whose last layer is zero is the plain solver)
//   k_fluid_deltap        x_i += dp_i(omega lambda), then the extra plain iterations
//   vorticity sweep       also sums |rho_i / rho0 - 1| per block at the solver output
//   k_ws_guard            mean error -> statistics; sets the graph's conditional to rerun the
//                         step's solve with the plain iteration count when above tolerance
// Training through the solve (rtp_train_warm_start_rollout): the loss is the mean squared
// density constraint after the warm-started correction, L = 1/N sum_i C_i(x')^2 with
// x' = clamp(x* + dp(omega lambda)); k_ws_loss_grad_x and k_ws_grad_y are its backward
// sweeps (dL/dx', then dL/dy), and the trainer's kernels take dL/dy through the network.
// Regression samples (features, converged lambda) come from plain steps:
// k_ws_lambda<kRecord> writes the features of the sampled particles, k_ws_record_targets
// their targets once the plain solve has finished.
#include "warmstart.cuh"

namespace rtp {

constexpr int kRecord = 0, kInfer = 1;

// Neighbour sums of the feature sweep.
struct WsSums {
  float rho = 0.0f, sgx = 0.0f, sgy = 0.0f, sgz = 0.0f, ssq = 0.0f, div = 0.0f;
  uint32_t cnt = 0;
};

// fld_computeDensity + fld_computeConstraintFactor at xi (as k_fluid_lambda: filter pass into
// the pair list, then the list in order) plus the feature sums.
__device__ __forceinline__ void ws_sweep(const GridK& g, const uint2* __restrict__ table,
                                         const float4* __restrict__ pred, const float4* __restrict__ velS, uint32_t i,
                                         float4 xi, float4 vi, const PairList& pl, WsSums& S) {
  const Sph k(g);
  uint32_t cnt = 0;
  uint32_t* lst = pl.idx + i;
  filter_fluid_neighbours_to(g, table, xi, k.h2, [&](uint32_t j) { return ld4(pred + j); }, [&](uint32_t j) {
    if (cnt < pl.K) lst[(size_t)cnt * pl.stride] = j;
    ++cnt;
  });
  auto ld = [&](uint32_t j) { return Pair44{ld4(pred + j), ld4(velS + j)}; };
  auto body = [&](uint32_t j, Pair44 a) {
    const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      S.rho += k.w(r2);
      float r;
      const float s = k.gs(r2, r);
      const float gxx = vx * s, gyy = vy * s, gzz = vz * s;
      S.sgx += gxx;
      S.sgy += gyy;
      S.sgz += gzz;
      S.ssq += gxx * gxx + gyy * gyy + gzz * gzz;
      if (j != i) {
        ++S.cnt;
        S.div += (a.v.x - vi.x) * gxx + (a.v.y - vi.y) * gyy + (a.v.z - vi.z) * gzz;
      }
    }
  };
  if (cnt <= pl.K)
    visit_list_x4(0, cnt, 1, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ld, body);
  else
    for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { body(j, ld(j)); });
  pl.count[i] = cnt <= pl.K ? cnt : kListOverflow;
}

// The network's relaxation of the plain first-iteration lambda: omega = 1 + tanh(y) * (2 for
// y > 0, 1 for y <= 0), in (0, 3); omega(0) = 1 exactly.
__device__ __forceinline__ float ws_omega(float y) { return 1.0f + tanhf(y) * (y > 0.0f ? 2.0f : 1.0f); }
__device__ __forceinline__ float ws_omega_grad(float y) {
  const float t = tanhf(y);
  return (1.0f - t * t) * (y > 0.0f ? 2.0f : 1.0f);
}

// Wall proximity along one axis: positive within 2h of the low wall, negative within 2h of
// the high wall, 0 in between.
__device__ __forceinline__ float wall_proximity(float x, float lo, float hi, float invH) {
  return fminf(fmaxf(2.0f - (x - lo) * invH, 0.0f), 2.0f) - fminf(fmaxf(2.0f - (hi - x) * invH, 0.0f), 2.0f);
}

// Inference holds the network's fragments after the sweep: 14 blocks of 64 threads per SM
// (73 registers) still keep 131,072 particles in one wave on 152 SMs.
// kInfer also writes (x, y, z, omega lambda) to `packed` for the correction sweep, and omega to
// omegaOut when given.
template <int MODE, bool BATCH>
__global__ void __launch_bounds__(kSweepThreads, MODE == 0 ? 16 : 14)
    k_ws_lambda(GridK g, FluidK p, const float4* __restrict__ pred, const float4* __restrict__ velS,
                const uint2* __restrict__ table, uint32_t n,
                float* __restrict__ lambda, float* __restrict__ density, float* __restrict__ lamTot, PairList pl,
                uint32_t stride, uint32_t phase, float* __restrict__ feats, uint32_t capacity, MlpDev m,
                float4* __restrict__ packed, float* __restrict__ omegaOut) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  float f[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) f[k] = 0.0f;
  float lam = 0.0f;
  float4 xi = f4(0.0f, 0.0f, 0.0f, 0.0f);
  if (active) {
    scene_of<BATCH>(i, g, p);
    xi = ld4(pred + i);
    const float4 vi = ld4(velS + i);
    WsSums S;
    ws_sweep(g, table, pred, velS, i, xi, vi, pl, S);
    // fld_computeConstraintFactor, same operations as k_fluid_lambda.
    const float C = S.rho / p.rho0 - 1.0f;
    const float ssqAll = (S.ssq + (S.sgx * S.sgx + S.sgy * S.sgy + S.sgz * S.sgz)) * p.invRho0Sq;
    lam = -C / (ssqAll + p.relaxCFM);
    density[i] = S.rho;
    const float hr = g.h * p.invRho0, invH = 1.0f / g.h;
    f[0] = (float)S.cnt;
    f[1] = C;
    f[2] = S.sgx * hr;
    f[3] = S.sgy * hr;
    f[4] = S.sgz * hr;
    f[5] = S.ssq * hr * hr;
    f[6] = S.div * (p.dt * p.invRho0);
    f[7] = wall_proximity(xi.x, p.lo.x, p.hi.x, invH);
    f[8] = wall_proximity(xi.y, p.lo.y, p.hi.y, invH);
    f[9] = wall_proximity(xi.z, p.lo.z, p.hi.z, invH);
    f[10] = lam;
    f[11] = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * p.dt * invH;
  }
  if constexpr (MODE == kRecord) {
    if (!active) return;
    lambda[i] = lam;
    lamTot[i] = lam;
    if (i >= phase && (i - phase) % stride == 0) {
      const uint32_t s = (i - phase) / stride;
      if (s < capacity) {
        float* o = feats + (size_t)s * kMlpIn;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) o[k] = f[k];
      }
    }
  } else {
    // Inference: every lane of the warp takes part (inactive lanes with zero inputs).
    __shared__ uint32_t s_stage[kSweepThreads / 32][32 * 9];
    float x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = active ? (f[k] - __ldg(m.inMean + k)) * __ldg(m.inScale + k) : 0.0f;
    __syncwarp();
    float y[kMlpOut];
    mlp_warp_forward(m, x, y, s_stage[threadIdx.x >> 5]);
    if (!active) return;
    const float om = ws_omega(y[0] * __ldg(m.outScale + 0));
    const float lw = om * lam;
    if (omegaOut) omegaOut[i] = om;
    lambda[i] = lw;
    lamTot[i] = lw;
    packed[i] = f4(xi.x, xi.y, xi.z, lw);
  }
}

// Training: lambda_i <- omega(y_i) lambda_i, with y the network's output 0 per particle
// (rows of 4) and (x, y, z, omega lambda) into packed for the correction sweep.
__global__ void k_ws_apply_omega(const float4* __restrict__ xs, const float* __restrict__ lam,
                                 const float* __restrict__ y, uint32_t n, float* __restrict__ lamOut,
                                 float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = ld4(xs + i);
  const float lw = ws_omega(__ldg(y + (size_t)i * kMlpOut)) * __ldg(lam + i);
  lamOut[i] = lw;
  packed[i] = f4(x.x, x.y, x.z, lw);
}

// Backward of the loss L = invN sum_m C'_m^2 to the corrected positions x' (the density sweep
// at x' recorded its pairs in pl2 and rho' in rho2):
//   g_m = 2 invN / rho0 sum_{j in P'(m)} (C'_m + C'_j) gradW_poly6(x'_m - x'_j),
// with gradW_poly6(v) = -6 POLY6 (h^2 - r^2)^2 v, zeroed on a coordinate the clamp held (x'
// on a bound of fld_applyBoundaryCondition).  lossPart[block] = sum of C'^2 over its particles.
__global__ void __launch_bounds__(128) k_ws_loss_grad_x(GridK g, FluidK p, const float4* __restrict__ xp,
                                                        const float* __restrict__ rho2, const uint2* __restrict__ table,
                                                        uint32_t n, PairList pl2, float invN,
                                                        float4* __restrict__ gOut, float* __restrict__ lossPart) {
  pdl_enter();
  __shared__ float s_loss[128 / kQuad];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;
  const Sph k(g);
  const float4 xi = ld4(xp + ii);
  const float ci = __ldg(rho2 + ii) * p.invRho0 - 1.0f;
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
  if (active) {
    auto ld = [&](uint32_t j) { return Pair4{ld4(xp + j), __ldg(rho2 + j)}; };
    quad_pairs(g, table, pl2, i, q, xi, ld, [&](uint32_t, Pair4 a) {
      const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        const float d = k.h2 - r2;
        const float f = (ci + (a.s * p.invRho0 - 1.0f)) * (-6.0f * k.poly6 * d * d);
        gx += vx * f;
        gy += vy * f;
        gz += vz * f;
      }
    });
  }
  gx = quad_sum(gx);
  gy = quad_sum(gy);
  gz = quad_sum(gz);
  const float sc = 2.0f * invN * p.invRho0;
  if (q == 0) s_loss[threadIdx.x / kQuad] = active ? ci * ci : 0.0f;
  if (active && q == 0)
    gOut[i] = f4((xi.x == p.lo.x || xi.x == p.hi.x) ? 0.0f : gx * sc, (xi.y == p.lo.y || xi.y == p.hi.y) ? 0.0f : gy * sc,
                 (xi.z == p.lo.z || xi.z == p.hi.z) ? 0.0f : gz * sc, 0.0f);
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.0f;
    for (int u = 0; u < 128 / kQuad; ++u) a += s_loss[u];
    lossPart[blockIdx.x] = a;
  }
}

// dL/dy_k = omega'(y_k) lambda_k / rho0 sum_{j in P*(k)} (g_k - g_j) . gradSpiky(x*_k - x*_j)
// over the pairs recorded at the predicted positions x* (the correction's own pairs).
__global__ void __launch_bounds__(128) k_ws_grad_y(GridK g, FluidK p, const float4* __restrict__ xs,
                                                   const float* __restrict__ lam, const float* __restrict__ y,
                                                   const float4* __restrict__ gIn, const uint2* __restrict__ table,
                                                   uint32_t n, PairList pl, float* __restrict__ dy) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;
  const Sph k(g);
  const float4 xi = ld4(xs + ii), gi = ld4(gIn + ii);
  float acc = 0.0f;
  if (active) {
    auto ld = [&](uint32_t j) { return Pair44{ld4(xs + j), ld4(gIn + j)}; };
    quad_pairs(g, table, pl, i, q, xi, ld, [&](uint32_t, Pair44 a) {
      const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        acc += ((gi.x - a.v.x) * vx + (gi.y - a.v.y) * vy + (gi.z - a.v.z) * vz) * s;
      }
    });
  }
  acc = quad_sum(acc);
  if (!active || q != 0) return;
  // Rows of kMlpOut: the gradient of output 0; outputs 1..3 are not used by the solve.
  *reinterpret_cast<float4*>(dy + (size_t)i * kMlpOut) =
      f4(ws_omega_grad(__ldg(y + (size_t)i * kMlpOut)) * __ldg(lam + i) * p.invRho0 * acc, 0.0f, 0.0f, 0.0f);
}

// dst[ids[i]] = src[i * stride]: sorted order -> particle ids.
__global__ void k_scatter_by_id(const uint32_t* __restrict__ ids, const float* __restrict__ src, uint32_t stride,
                                uint32_t n, float* __restrict__ dst) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[__ldg(ids + i)] = __ldg(src + (size_t)i * stride);
}

// Targets of sample s (particle i = phase + s * stride): (Lambda_i, xFinal_i - x0_i -
// dp_i(Lambda)), dp as fld_computeConstraintCorrection over the pairs recorded at x0.
__global__ void __launch_bounds__(128) k_ws_record_targets(GridK g, FluidK p, const float4* __restrict__ x0,
                                                           const float* __restrict__ lamTot,
                                                           const uint2* __restrict__ table, uint32_t n,
                                                           const float4* __restrict__ xFinal, PairList pl0,
                                                           uint32_t stride, uint32_t phase, uint32_t count,
                                                           float* __restrict__ targets) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t s = t / kQuad, q = t % kQuad;
  const uint32_t i = phase + s * stride;
  const bool active = s < count && i < n;
  float cx = 0.0f, cy = 0.0f, cz = 0.0f;
  float4 xi = f4(0.f, 0.f, 0.f, 0.f);
  float li = 0.0f;
  if (active) {
    const Sph k(g);
    xi = ld4(x0 + i);
    li = __ldg(lamTot + i);
    auto ld = [&](uint32_t j) { return Pair4{ld4(x0 + j), __ldg(lamTot + j)}; };
    quad_pairs(g, table, pl0, i, q, xi, ld, [&](uint32_t, Pair4 a) {
      const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float sg = k.gs(r2, r);
        float sc = 0.0f;
        if (p.artPressure) sc = -p.apCoeff * powi(k.w(r2) * p.apInvWq, p.apExp);
        const float f = (li + a.s + sc) * sg;
        cx += vx * f;
        cy += vy * f;
        cz += vz * f;
      }
    });
  }
  cx = quad_sum(cx);
  cy = quad_sum(cy);
  cz = quad_sum(cz);
  if (!active || q != 0) return;
  const float4 xf = ld4(xFinal + i);
  float* o = targets + (size_t)s * kMlpOut;
  o[0] = li;
  o[1] = xf.x - (xi.x + cx * p.invRho0);
  o[2] = xf.y - (xi.y + cy * p.invRho0);
  o[3] = xf.z - (xi.z + cz * p.invRho0);
}

template <bool BATCH>
__global__ void __launch_bounds__(kSweepThreads) k_ws_density_error(GridK g, FluidK p, const float4* __restrict__ pos,
                                                                    const uint2* __restrict__ table, uint32_t n,
                                                                    float* __restrict__ errPartial) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float err = 0.0f;
  if (i < n) {
    scene_of<BATCH>(i, g, p);
    const Sph k(g);
    const float4 xi = ld4(pos + i);
    float rho = 0.0f;
    for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) {
      const float4 xj = ld4(pos + j);
      const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) rho += k.w(r2);
    });
    err = fabsf(rho / p.rho0 - 1.0f);
  }
  block_error_partial(err, errPartial);
}

// One block: the partial sums in a fixed order (deterministic), then the decision.
constexpr int kGuardThreads = 256;
__global__ void __launch_bounds__(kGuardThreads) k_ws_guard(const float* __restrict__ part, uint32_t nblk, uint32_t n,
                                                           float tol, SolverStatsDev* st,
                                                           cudaGraphConditionalHandle hnd, int hasCond, int accept) {
  pdl_enter();
  __shared__ double s_sum[kGuardThreads];
  double v = 0.0;
  for (uint32_t b = threadIdx.x; b < nblk; b += kGuardThreads) v += (double)part[b];
  s_sum[threadIdx.x] = v;
  __syncthreads();
  for (int w = kGuardThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s_sum[threadIdx.x] += s_sum[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double mean = n ? s_sum[0] / (double)n : 0.0;
  if (accept) {
    st->sumErr += mean;
    st->maxErr = fmax(st->maxErr, mean);
    return;
  }
  st->steps += 1;
  st->sumFirst += mean;
  const bool rerun = hasCond && tol > 0.0f && mean > (double)tol;
  if (rerun) {
    st->reruns += 1;
  } else {
    st->sumErr += mean;
    st->maxErr = fmax(st->maxErr, mean);
  }
  if (hasCond) cudaGraphSetConditional(hnd, rerun ? 1u : 0u);
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}

static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

int ws_lambda_record(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                     uint32_t stride, uint32_t phase, float* feats, uint32_t capacity, Launcher& L) {
  if (stride == 0) return fail(RTP_ERR_INVALID_ARGUMENT, "sample stride must be > 0");
  MlpDev m{};
  L.begin("ws_lambda_record");
  if (p.bt.scenes) return fail(RTP_ERR_NOT_SUPPORTED, "sample recording runs on single scenes");
  launch(L, k_ws_lambda<kRecord, false>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads),
      g, p, pred, velS, table, n, lambda, density, lamTot, pl, stride, phase, feats, capacity, m, nullptr, nullptr);
  L.end("ws_lambda_record");
  return check("k_ws_lambda<record>");
}

int ws_lambda_infer(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, const uint2* table, uint32_t n, float* lambda, float* density, float* lamTot, const PairList& pl,
                    const void* mlpBlock, float4* packed, float* omegaOut, Launcher& L) {
  const MlpDev m = mlp_dev(mlpBlock);
  L.begin("ws_lambda_mlp");
  if (p.bt.scenes)
    launch(L, k_ws_lambda<kInfer, true>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads),
        g, p, pred, velS, table, n, lambda, density, lamTot, pl, 1, 0, nullptr, 0, m, packed, omegaOut);
  else
    launch(L, k_ws_lambda<kInfer, false>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads),
        g, p, pred, velS, table, n, lambda, density, lamTot, pl, 1, 0, nullptr, 0, m, packed, omegaOut);
  L.end("ws_lambda_mlp");
  return check("k_ws_lambda<infer>");
}

int ws_apply_omega(const float4* xs, const float* lam, const float* y, uint32_t n, float* lamOut, float4* packed,
                   Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_ws_apply_omega, dim3(blocks(n, 256)), dim3(256), xs, lam, y, n, lamOut, packed);
  return check("k_ws_apply_omega");
}

uint32_t ws_loss_blocks(uint32_t n) { return blocks(n * kQuad, 128); }

int ws_loss_grad_x(const GridK& g, const FluidK& p, const float4* xp, const float* rho2, const uint2* table, uint32_t n,
                   const PairList& pl2, float4* gOut, float* lossPart, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_ws_loss_grad_x, dim3(ws_loss_blocks(n)), dim3(128), g, p, xp, rho2, table, n, pl2,
         (float)(1.0 / (double)n), gOut, lossPart);
  return check("k_ws_loss_grad_x");
}

int ws_grad_y(const GridK& g, const FluidK& p, const float4* xs, const float* lam, const float* y, const float4* gIn,
              const uint2* table, uint32_t n, const PairList& pl, float* dy, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_ws_grad_y, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, xs, lam, y, gIn, table, n, pl, dy);
  return check("k_ws_grad_y");
}

int ws_scatter_by_id(const uint32_t* ids, const float* src, uint32_t stride, uint32_t n, float* dst, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_scatter_by_id, dim3(blocks(n, 256)), dim3(256), ids, src, stride, n, dst);
  return check("k_scatter_by_id");
}

int ws_record_targets(const GridK& g, const FluidK& p, const float4* x0, const float* lamTot, const uint2* table,
                      uint32_t n, const float4* xFinal, const PairList& pl0, uint32_t stride, uint32_t phase,
                      uint32_t count, float* targets, Launcher& L) {
  if (count == 0) return RTP_OK;
  L.begin("ws_record_targets");
  launch(L, k_ws_record_targets, dim3(blocks(count * kQuad, 128)), dim3(128), g, p, x0, lamTot, table, n, xFinal, pl0, stride,
                                                                         phase, count, targets);
  L.end("ws_record_targets");
  return check("k_ws_record_targets");
}

int ws_density_error(const GridK& g, const FluidK& p, const float4* pos, const uint2* table, uint32_t n,
                     float* errPartial, Launcher& L) {
  L.begin("ws_density_error");
  if (p.bt.scenes)
    launch(L, k_ws_density_error<true>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, pos, table, n, errPartial);
  else
    launch(L, k_ws_density_error<false>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, pos, table, n, errPartial);
  L.end("ws_density_error");
  return check("k_ws_density_error");
}

int ws_guard(const float* errPartial, uint32_t n, float tol, SolverStatsDev* st, cudaGraphConditionalHandle hnd,
             bool hasCond, bool accept, Launcher& L) {
  L.begin(accept ? "ws_accept" : "ws_guard");
  launch(L, k_ws_guard, dim3(1), dim3(kGuardThreads), errPartial, ws_error_blocks(n), n, tol, st, hnd, hasCond ? 1 : 0,
                                                accept ? 1 : 0);
  L.end(accept ? "ws_accept" : "ws_guard");
  return check("k_ws_guard");
}

}  // namespace rtp
