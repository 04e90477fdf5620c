// clouds.cu - clouds step: PBF with mixed boundaries + thermodynamics (GB300, sm_103a).
//
// Replaces kernels/clouds.cl driven by Clouds::update (physics/ocl/Clouds.cpp:503-610):
//   k_cloud_thermo_predict  cld_heatFromGround, cld_computeBuoyancy, cld_applyAdiabaticCooling,
//                           cld_generateCloud, cld_applyPhaseTransition, cld_applyLatentHeat
//                           (the reference's 6 kernels + 3 buffer copies), cld_predictPosition,
//                           cld_applyMixedBoundaryConditions, fillCellIDs, sort histogram
//   sort passes             {pos, vel, predPos, totCorrPos} + {temp, buoyancy, vapor, cloud, id}
//   k_cloud_temp_lambda     cld_computeLaplacianTemp + cld_computeConstraintFactorTemp (one sweep)
//   k_cloud_temp_correct    cld_computeConstraintCorrectionTemp + cld_correctTemperature
//   I x k_cloud_lambda      cld_computeDensity + cld_computeConstraintFactor
//   I x k_cloud_deltap      cld_computeConstraintCorrection + cld_correctPosition (predPos and
//                           totCorrPos) + the mixed boundary; the last adds cld_updateVel
//   vorticity, confinement, XSPH + cld_updatePosition (wind drift), state written back.
// Neighbour sweeps follow clouds.cl:326-356: x and z periodic with image shifts of
// 2W * sign, y walls.  As in fluids.cu, the first sweep at given positions records the pairs
// within h (entry = particle index | image code << 28) for the sweeps that follow at the
// same positions, which give 4 lanes to each particle.
#include "clouds.cuh"
#include "mlp.cuh"

namespace rtp {

template <class F>
__device__ __forceinline__ void for_each_cloud_neighbour(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                         F&& f) {
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  for (int dx = -1; dx <= 1; ++dx) {
    const int ux = cx + dx;
    const int nx = (ux + g.R[0]) % g.R[0];
    const float shx = ux >= g.R[0] ? 2.0f * g.W[0] : (ux < 0 ? -2.0f * g.W[0] : 0.0f);
    for (int dy = -1; dy <= 1; ++dy) {
      const int ny = cy + dy;
      if (ny >= g.R[1] || ny < 0) continue;
      const uint32_t row = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2];
      for (int dz = -1; dz <= 1; ++dz) {
        const int uz = cz + dz;
        const int nz = (uz + g.R[2]) % g.R[2];
        const float shz = uz >= g.R[2] ? 2.0f * g.W[2] : (uz < 0 ? -2.0f * g.W[2] : 0.0f);
        uint32_t j0, j1;
        cell_range(table, row + (uint32_t)nz, g.cap, j0, j1);
        for (uint32_t j = j0; j < j1; ++j) f(j, shx, shz);
      }
    }
  }
}

// Image code of a recorded pair: bits 0-1 x shift, bits 2-3 z shift (1 = +2W, 2 = -2W).
__device__ __forceinline__ uint32_t image_code(float shx, float shz) {
  return (shx > 0.f ? 1u : (shx < 0.f ? 2u : 0u)) | ((shz > 0.f ? 1u : (shz < 0.f ? 2u : 0u)) << 2);
}
__device__ __forceinline__ void image_shift(const GridK& g, uint32_t code, float& shx, float& shz) {
  const uint32_t cx = code & 3u, cz = (code >> 2) & 3u;
  shx = cx == 1u ? 2.0f * g.W[0] : (cx == 2u ? -2.0f * g.W[0] : 0.0f);
  shz = cz == 1u ? 2.0f * g.W[2] : (cz == 2u ? -2.0f * g.W[2] : 0.0f);
}

// Filter pass over the clouds neighbourhood: add(entry) for each candidate within h2, in
// visiting order.  Each (x, y) row's three z cells are read from the table together and
// visited as one range where they are contiguous with the same image shift (all but the
// z-wrapped cells at the box faces), eight position loads in flight.  The pair test rounds
// every operation explicitly (xi - xj, minus the image shift, then two fused multiply-adds, as
// within_radius does), so every kernel this is inlined into records the same pairs.  (A
// separate loop without the shift subtractions for unshifted runs was measured: 6 % slower
// clouds steps.)
template <class ADD>
__device__ __forceinline__ void filter_cloud_neighbours(const GridK& g, const uint2* __restrict__ table,
                                                        const float4* __restrict__ pos, float4 xi, float h2,
                                                        ADD&& add) {
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  auto wrap = [](int u, int R) { return u < 0 ? u + R : (u >= R ? u - R : u); };
  auto shift = [](int u, int R, float w) { return u >= R ? 2.0f * w : (u < 0 ? -2.0f * w : 0.0f); };
  const uint32_t z0 = (uint32_t)wrap(cz - 1, g.R[2]), z1 = (uint32_t)wrap(cz, g.R[2]), z2 = (uint32_t)wrap(cz + 1, g.R[2]);
  const float s0 = shift(cz - 1, g.R[2], g.W[2]), s1 = shift(cz, g.R[2], g.W[2]), s2 = shift(cz + 1, g.R[2], g.W[2]);
#pragma unroll 1
  for (int dx = -1; dx <= 1; ++dx) {
    const int ux = cx + dx;
    const int nx = wrap(ux, g.R[0]);
    const float shx = shift(ux, g.R[0], g.W[0]);
#pragma unroll 1
    for (int dy = -1; dy <= 1; ++dy) {
      const int ny = cy + dy;
      if (ny >= g.R[1] || ny < 0) continue;
      const uint32_t row = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2];
      uint32_t b0, e0, b1, e1, b2, e2;
      cell_range(table, row + z0, g.cap, b0, e0);
      cell_range(table, row + z1, g.cap, b1, e1);
      cell_range(table, row + z2, g.cap, b2, e2);
      auto run = [&](uint32_t b, uint32_t e, float shz) {
        const uint32_t code = image_code(shx, shz) << 28;
        visit_range_x8(b, e, [&](uint32_t j) { return ld4(pos + j); }, [&](uint32_t j, float4 xj) {
          const float4 xs = f4(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z), 0.0f);
          const float vx = __fsub_rn(xs.x, shx), vz = __fsub_rn(xs.z, shz);
          if (__fmaf_rn(vz, vz, __fmaf_rn(xs.y, xs.y, __fmul_rn(vx, vx))) < h2) add(j | code);
        });
      };
      // Cells in visiting order, joined while contiguous with the same shift.
      uint32_t cb = b0, ce = e0;
      float cs = s0;
      const uint32_t rb[2] = {b1, b2}, re[2] = {e1, e2};
      const float rs[2] = {s1, s2};
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        if (rb[r] == re[r]) continue;
        if (cb == ce) {
          cb = rb[r];
          ce = re[r];
          cs = rs[r];
        } else if (ce == rb[r] && cs == rs[r]) {
          ce = re[r];
        } else {
          run(cb, ce, cs);
          cb = rb[r];
          ce = re[r];
          cs = rs[r];
        }
      }
      if (cb != ce) run(cb, ce, cs);
    }
  }
}

// Records add(entry) into the device list of particle i; returns the count.
struct ListWriter {
  const PairList& L;
  uint32_t* lst;
  uint32_t n = 0;
  __device__ __forceinline__ ListWriter(const PairList& l, uint32_t i) : L(l), lst(l.idx + i) {}
  __device__ __forceinline__ void operator()(uint32_t e) {
    if (n < L.K) lst[(size_t)n * L.stride] = e;
    ++n;
  }
  __device__ __forceinline__ bool ok() const { return n <= L.K; }
  __device__ __forceinline__ uint32_t at(uint32_t k) const { return lst[(size_t)k * L.stride]; }
};

// Visits the recorded pairs of particle i on lane q of its quad (f(j, shx, shz)), or its
// 27 cells on lane 0 when the list overflowed.
template <class F>
__device__ __forceinline__ void quad_cloud_pairs(const GridK& g, const uint2* __restrict__ table, const PairList& L,
                                                 uint32_t i, uint32_t q, float4 xi, F&& f) {
  const uint32_t c = __ldg(L.count + i);
  if (c != kListOverflow) {
    const uint32_t* base = L.idx + i;
    auto visit = [&](uint32_t e) {
      float shx, shz;
      image_shift(g, e >> 28, shx, shz);
      f(e & 0x0FFFFFFFu, shx, shz);
    };
    uint32_t kk = q;
    for (; kk + 3 * kQuad < c; kk += 4 * kQuad) {  // four entries in flight
      const uint32_t e0 = __ldg(base + (size_t)kk * L.stride), e1 = __ldg(base + (size_t)(kk + kQuad) * L.stride);
      const uint32_t e2 = __ldg(base + (size_t)(kk + 2 * kQuad) * L.stride);
      const uint32_t e3 = __ldg(base + (size_t)(kk + 3 * kQuad) * L.stride);
      visit(e0);
      visit(e1);
      visit(e2);
      visit(e3);
    }
    for (; kk < c; kk += kQuad) visit(__ldg(base + (size_t)kk * L.stride));
  } else if (q == 0) {
    for_each_cloud_neighbour(g, table, xi, f);
  }
}

// Ground temperature: bilinear in the groundNx x groundNz table over the box floor.
__device__ __forceinline__ float ground_temp(const CloudK& c, const GridK& g, float x, float z) {
  if (!c.ground) return c.T0;
  const float u = fminf(fmaxf((x + g.W[0]) / (2.0f * g.W[0]), 0.0f), 1.0f) * (float)(c.nx - 1);
  const float v = fminf(fmaxf((z + g.W[2]) / (2.0f * g.W[2]), 0.0f), 1.0f) * (float)(c.nz - 1);
  const uint32_t i0 = min((uint32_t)floorf(u), c.nx - 2), k0 = min((uint32_t)floorf(v), c.nz - 2);
  const float fu = u - (float)i0, fv = v - (float)k0;
  const float a = __ldg(c.ground + i0 * c.nz + k0), b = __ldg(c.ground + i0 * c.nz + k0 + 1);
  const float cc = __ldg(c.ground + (i0 + 1) * c.nz + k0), d = __ldg(c.ground + (i0 + 1) * c.nz + k0 + 1);
  const float ab = a + (b - a) * fv, cd = cc + (d - cc) * fv;
  return ab + (cd - ab) * fu;
}
// environmentTemp (clouds.cl:80-89).
__device__ __forceinline__ float env_temp(const CloudK& c, const GridK& g, float4 p) {
  return -c.lapse * (p.y + g.W[1]) + ground_temp(c, g, p.x, p.z);
}
// saturationVaporDensity (clouds.cl:94-99): double literals, evaluated in double.
__device__ __forceinline__ float qsat(float T) { return (float)(217.0 * exp(19.5 - 4303.4 / ((double)T - 29.5)) / (double)T); }

// cld_applyMixedBoundaryConditions (clouds.cl:279-299).
__device__ __forceinline__ float4 mixed_bc(const GridK& g, float4 np) {
  float4 r = np;
  if (fabsf(np.x) > g.W[0]) r.x = np.x - 2.0f * fminf(fmaxf(np.x, -g.W[0]), g.W[0]);
  if (fabsf(np.y) > g.W[1]) r.y = fminf(fmaxf(np.y, -g.W[1]), g.W[1]);
  if (fabsf(np.z) > g.W[2]) r.z = np.z - 2.0f * fminf(fmaxf(np.z, -g.W[2]), g.W[2]);
  return r;
}

__global__ void __launch_bounds__(kKeyThreads) k_cloud_thermo_predict(
    GridK g, CloudK c, const float4* __restrict__ pos, const float4* __restrict__ vel, uint32_t n,
    float* __restrict__ temp, float* __restrict__ vapor, float* __restrict__ cloud, float* __restrict__ buoy,
    float4* __restrict__ pred, float4* __restrict__ tot, uint32_t* __restrict__ keys, int bits0,
    uint32_t* __restrict__ hist0, ZeroJob zero) {
  pdl_enter();
  __shared__ uint32_t s_hist[kMaxBins];
  zero_job(zero);
  TileHistogram th;
  th.init(s_hist, bits0);
  const float dt = c.dt;
  const uint32_t base = blockIdx.x * kSortTile;
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t i = base + k * kKeyThreads + threadIdx.x;
    if (i >= n) continue;
    const float4 p = ld4(pos + i), v = ld4(vel + i);
    const float tIn = temp[i];
    // cld_heatFromGround (clouds.cl:159-168).
    const float heat = fminf(fmaxf(expf(-(p.y + g.W[1]) / c.heatDecay), 0.0f), 1.0f);
    const float t1 = fminf(tIn + heat * c.groundHeat * dt, 313.0f);
    // cld_computeBuoyancy (clouds.cl:173-184).
    const float envT = env_temp(c, g, p);
    const float b = c.buoyancy * (t1 - envT) / envT - c.gravCoeff * kAbsGravityY * cloud[i];
    // cld_applyAdiabaticCooling (clouds.cl:189-198).
    const float t2 = fmaxf(t1 - c.adiabatic * v.y * dt, 223.0f);
    // cld_generateCloud (clouds.cl:207-221), cld_applyPhaseTransition (:226-238).
    const float gen = c.phaseRate * (vapor[i] - qsat(t2));
    cloud[i] = fmaxf(cloud[i] + gen * dt, 0.0f);
    vapor[i] = fmaxf(vapor[i] - gen * dt, 0.0f);
    // cld_applyLatentHeat (clouds.cl:243-252).
    temp[i] = t2 + fmaxf(c.latent * gen * dt, 0.0f);
    buoy[i] = b;
    // cld_predictPosition (clouds.cl:257-273) + mixed boundary (Clouds.cpp:537-538).
    const float4 pv = f4(v.x, v.y + b * dt, v.z, v.w);
    tot[i] = pv * dt;
    const float4 pp = mixed_bc(g, p + pv * dt);
    pred[i] = pp;
    const uint32_t key = cell_key(g, pp);
    keys[i] = key;
    th.add(key);
  }
  th.store(hist0);
}

// cld_computeLaplacianTemp + cld_computeConstraintFactorTemp, on p_pos (Clouds.cpp:253-255);
// records the pairs within h of p_pos for k_cloud_temp_correct.
__global__ void __launch_bounds__(kSweepThreads, 16) k_cloud_temp_lambda(GridK g, CloudK c, const float4* __restrict__ pos,
                                                                         const float* __restrict__ temp,
                                                                         const uint2* __restrict__ table, uint32_t n,
                                                                         float* __restrict__ lamT, PairList pl,
                                                                         float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Sph k(g);
  const float4 xi = ld4(pos + i);
  const float ti = __ldg(temp + i);
  ListWriter lw(pl, i);
  filter_cloud_neighbours(g, table, pos, xi, k.h2, lw);
  float lap = 0.0f, sg = 0.0f, ssq = 0.0f;
  auto body_at = [&](float4 xj, float tj, float shx, float shz) {
    const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      float r;
      const float s = k.gs(r2, r);
      const float vg = r2 * s;  // dot(vec, gradSpiky(vec))
      lap += (ti - tj) * vg / (r2 + kFloatEps);
      const float d = vg / (r2 * c.cloudRho0 + kFloatEps);
      sg += d;
      ssq += d * d;
    }
  };
  auto body = [&](uint32_t j, float shx, float shz) { body_at(ld4(pos + j), __ldg(temp + j), shx, shz); };
  if (lw.ok())
    visit_list_x4(0, lw.n, 1, [&](uint32_t kk) { return lw.at(kk); },
                  [&](uint32_t e) { return Pair4{ld4(pos + (e & 0x0FFFFFFFu)), __ldg(temp + (e & 0x0FFFFFFFu))}; },
                  [&](uint32_t e, Pair4 a) {
                    float shx, shz;
                    image_shift(g, e >> 28, shx, shz);
                    body_at(a.x, a.s, shx, shz);
                  });
  else
    for_each_cloud_neighbour(g, table, xi, body);
  pl.count[i] = lw.ok() ? lw.n : kListOverflow;
  lap /= c.cloudRho0;
  ssq += sg * sg;
  const float lt = -lap / (ssq + c.cloudRelax);
  lamT[i] = lt;
  packed[i] = f4(xi.x, xi.y, xi.z, lt);
}

// cld_computeConstraintCorrectionTemp + cld_correctTemperature (in place: the sweep reads
// only lamT and positions of the neighbours, both from `packed` = (x, y, z, lamT) written by
// k_cloud_temp_lambda).  kQuad lanes per particle.
__global__ void __launch_bounds__(128, 8) k_cloud_temp_correct(GridK g, CloudK c, const float4* __restrict__ pos,
                                                            const float* __restrict__ lamT,
                                                            const uint2* __restrict__ table, uint32_t n,
                                                            float* __restrict__ temp, PairList pl,
                                                            const float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  float corr = 0.0f;
  if (active) {
    const Sph k(g);
    const float4 xi = ld4(pos + i);
    const float li = __ldg(lamT + i);
    quad_cloud_pairs(g, table, pl, i, q, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(packed + j);
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        const float d = r2 * s / (r2 * c.cloudRho0 + kFloatEps);
        corr += (li + xj.w) * d;
      }
    });
  }
  corr = quad_sum(corr);
  if (active && q == 0) temp[i] += 0.3f * corr;
}

// cld_computeDensity + cld_computeConstraintFactor; records the pairs within h.
__global__ void __launch_bounds__(kSweepThreads, 16) k_cloud_lambda(GridK g, FluidK p, const float4* __restrict__ pred,
                                                                    const uint2* __restrict__ table, uint32_t n,
                                                                    float* __restrict__ lambda,
                                                                    float* __restrict__ density, PairList pl,
                                                                    float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Sph k(g);
  const float4 xi = ld4(pred + i);
  ListWriter lw(pl, i);
  filter_cloud_neighbours(g, table, pred, xi, k.h2, lw);
  float rho = 0.0f, sgx = 0.0f, sgy = 0.0f, sgz = 0.0f, ssq = 0.0f;
  auto body_at = [&](float4 xj, float shx, float shz) {
    const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      rho += k.w(r2);
      float r;
      const float s = k.gs(r2, r);
      const float a = vx * s, b = vy * s, cc = vz * s;
      sgx += a;
      sgy += b;
      sgz += cc;
      ssq += a * a + b * b + cc * cc;
    }
  };
  auto body = [&](uint32_t j, float shx, float shz) { body_at(ld4(pred + j), shx, shz); };
  if (lw.ok())
    visit_list_x4(0, lw.n, 1, [&](uint32_t kk) { return lw.at(kk); },
                  [&](uint32_t e) { return ld4(pred + (e & 0x0FFFFFFFu)); }, [&](uint32_t e, float4 xj) {
                    float shx, shz;
                    image_shift(g, e >> 28, shx, shz);
                    body_at(xj, shx, shz);
                  });
  else
    for_each_cloud_neighbour(g, table, xi, body);
  pl.count[i] = lw.ok() ? lw.n : kListOverflow;
  const float C = rho / p.rho0 - 1.0f;
  ssq += sgx * sgx + sgy * sgy + sgz * sgz;
  ssq *= p.invRho0Sq;
  const float lam = -C / (ssq + p.relaxCFM);
  lambda[i] = lam;
  density[i] = rho;
  packed[i] = f4(xi.x, xi.y, xi.z, lam);
}

// ---- learned warm start of the clouds solve (new: the reference's Jacobi loop,
// Clouds.cpp:570-587, starts every substep from a zero correction) -----------------------
// The fluids method (warmstart.cu) on the clouds sweep: the first density / lambda sweep of a
// substep also sums the network's features (layout in rtp.h: the fluids features with the x
// and z wall proximities, always 0 under the periodic boundary, replaced by the buoyant
// displacement of the step and the temperature above the environment), then each warp
// evaluates the network and relaxes lambda by omega(y) in (0, 3), omega(0) = 1 exactly.
constexpr int kCwsRecord = 0, kCwsInfer = 1;

__device__ __forceinline__ float cws_omega(float y) { return 1.0f + tanhf(y) * (y > 0.0f ? 2.0f : 1.0f); }
__device__ __forceinline__ float cws_omega_grad(float y) {
  const float t = tanhf(y);
  return (1.0f - t * t) * (y > 0.0f ? 2.0f : 1.0f);
}

// kCwsRecord: plain lambda into lambda, (x, y, z, lambda) into packed, the features of every
// particle into feats (rows of kMlpIn).  kCwsInfer: omega(network) lambda into lambda and packed.
// Both record the pairs within h (entries with image codes) into pl.
template <int MODE>
__global__ void __launch_bounds__(kSweepThreads, MODE == kCwsRecord ? 16 : 14)
    k_cloud_ws_lambda(GridK g, FluidK p, CloudK c, const float4* __restrict__ pred, const float4* __restrict__ velS,
                      const float* __restrict__ tempS, const float* __restrict__ buoyS,
                      const uint2* __restrict__ table, uint32_t n, float* __restrict__ lambda,
                      float* __restrict__ density, PairList pl, float4* __restrict__ packed,
                      float* __restrict__ feats, MlpDev m) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  float f[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) f[k] = 0.0f;
  float lam = 0.0f;
  float4 xi = f4(0.f, 0.f, 0.f, 0.f);
  if (active) {
    const Sph k(g);
    xi = ld4(pred + i);
    const float4 vi = ld4(velS + i);
    ListWriter lw(pl, i);
    filter_cloud_neighbours(g, table, pred, xi, k.h2, lw);
    float rho = 0.0f, sgx = 0.0f, sgy = 0.0f, sgz = 0.0f, ssq = 0.0f, div = 0.0f;
    uint32_t cnt = 0;
    auto body_at = [&](uint32_t j, float4 xj, float4 vj, float shx, float shz) {
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        rho += k.w(r2);
        float r;
        const float s = k.gs(r2, r);
        const float a = vx * s, b = vy * s, cc = vz * s;
        sgx += a;
        sgy += b;
        sgz += cc;
        ssq += a * a + b * b + cc * cc;
        if (j != i || shx != 0.0f || shz != 0.0f) {
          ++cnt;
          div += (vj.x - vi.x) * a + (vj.y - vi.y) * b + (vj.z - vi.z) * cc;
        }
      }
    };
    if (lw.ok())
      visit_list_x4(0, lw.n, 1, [&](uint32_t kk) { return lw.at(kk); },
                    [&](uint32_t e) { return Pair44{ld4(pred + (e & 0x0FFFFFFFu)), ld4(velS + (e & 0x0FFFFFFFu))}; },
                    [&](uint32_t e, Pair44 a) {
                      float shx, shz;
                      image_shift(g, e >> 28, shx, shz);
                      body_at(e & 0x0FFFFFFFu, a.x, a.v, shx, shz);
                    });
    else
      for_each_cloud_neighbour(g, table, xi, [&](uint32_t j, float shx, float shz) {
        body_at(j, ld4(pred + j), ld4(velS + j), shx, shz);
      });
    pl.count[i] = lw.ok() ? lw.n : kListOverflow;
    // cld_computeConstraintFactor, same operations as k_cloud_lambda.
    const float C = rho / p.rho0 - 1.0f;
    const float ssqRaw = ssq;
    ssq += sgx * sgx + sgy * sgy + sgz * sgz;
    ssq *= p.invRho0Sq;
    lam = -C / (ssq + p.relaxCFM);
    density[i] = rho;
    const float hr = g.h * p.invRho0, invH = 1.0f / g.h;
    f[0] = (float)cnt;
    f[1] = C;
    f[2] = sgx * hr;
    f[3] = sgy * hr;
    f[4] = sgz * hr;
    f[5] = ssqRaw * hr * hr;
    f[6] = div * (p.dt * p.invRho0);
    f[7] = __ldg(buoyS + i) * p.dt * p.dt * invH;
    f[8] = fminf(fmaxf(2.0f - (xi.y + g.W[1]) * invH, 0.0f), 2.0f) - fminf(fmaxf(2.0f - (g.W[1] - xi.y) * invH, 0.0f), 2.0f);
    f[9] = (__ldg(tempS + i) - env_temp(c, g, xi)) * 0.1f;
    f[10] = lam;
    f[11] = sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * p.dt * invH;
  }
  if constexpr (MODE == kCwsRecord) {
    if (!active) return;
    lambda[i] = lam;
    packed[i] = f4(xi.x, xi.y, xi.z, lam);
    float* o = feats + (size_t)i * kMlpIn;
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) o[k] = f[k];
  } else {
    __shared__ uint32_t s_stage[kSweepThreads / 32][32 * 9];
    float x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = active ? (f[k] - __ldg(m.inMean + k)) * __ldg(m.inScale + k) : 0.0f;
    __syncwarp();
    float y[kMlpOut];
    mlp_warp_forward(m, x, y, s_stage[threadIdx.x >> 5]);
    if (!active) return;
    const float lw = cws_omega(y[0] * __ldg(m.outScale + 0)) * lam;
    lambda[i] = lw;
    packed[i] = f4(xi.x, xi.y, xi.z, lw);
  }
}

// Backward of L = invN sum C'^2 to the corrected positions x' (the clouds density sweep at x'
// recorded pl2 and rho2): g_m = 2 invN / rho0 sum_j (C'_m + C'_j) gradW_poly6(x'_m - x'_j -
// image shift), zero in y where the mixed boundary held x' on a y wall.  lossPart[block] = sum
// of C'^2 over its particles.
__global__ void __launch_bounds__(128) k_cloud_ws_loss_grad_x(GridK g, FluidK p, const float4* __restrict__ xp,
                                                              const float* __restrict__ rho2,
                                                              const uint2* __restrict__ table, uint32_t n, PairList pl2,
                                                              float invN, float4* __restrict__ gOut,
                                                              float* __restrict__ lossPart) {
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
  if (active)
    quad_cloud_pairs(g, table, pl2, i, q, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(xp + j);
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        const float d = k.h2 - r2;
        const float f = (ci + (__ldg(rho2 + j) * p.invRho0 - 1.0f)) * (-6.0f * k.poly6 * d * d);
        gx += vx * f;
        gy += vy * f;
        gz += vz * f;
      }
    });
  gx = quad_sum(gx);
  gy = quad_sum(gy);
  gz = quad_sum(gz);
  const float sc = 2.0f * invN * p.invRho0;
  if (q == 0) s_loss[threadIdx.x / kQuad] = active ? ci * ci : 0.0f;
  if (active && q == 0) {
    const bool held = fabsf(xi.y) >= g.W[1];
    gOut[i] = f4(gx * sc, held ? 0.0f : gy * sc, gz * sc, 0.0f);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.0f;
    for (int u = 0; u < 128 / kQuad; ++u) a += s_loss[u];
    lossPart[blockIdx.x] = a;
  }
}

// dL/dy_k = omega'(y_k) lambda_k / rho0 sum_j (g_k - g_j) . gradSpiky(x*_k - x*_j - image shift),
// rows of kMlpOut (output 0).
__global__ void __launch_bounds__(128) k_cloud_ws_grad_y(GridK g, FluidK p, const float4* __restrict__ xs,
                                                         const float* __restrict__ lam, const float* __restrict__ y,
                                                         const float4* __restrict__ gIn,
                                                         const uint2* __restrict__ table, uint32_t n, PairList pl,
                                                         float* __restrict__ dy) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;
  const Sph k(g);
  const float4 xi = ld4(xs + ii), gi = ld4(gIn + ii);
  float acc = 0.0f;
  if (active)
    quad_cloud_pairs(g, table, pl, i, q, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(xs + j), gj = ld4(gIn + j);
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        acc += ((gi.x - gj.x) * vx + (gi.y - gj.y) * vy + (gi.z - gj.z) * vz) * s;
      }
    });
  acc = quad_sum(acc);
  if (!active || q != 0) return;
  *reinterpret_cast<float4*>(dy + (size_t)i * kMlpOut) =
      f4(cws_omega_grad(__ldg(y + (size_t)i * kMlpOut)) * __ldg(lam + i) * p.invRho0 * acc, 0.0f, 0.0f, 0.0f);
}

// Per-block sums of |rho_i / rho0 - 1| at pos (the solver statistics of a clouds step).
__global__ void __launch_bounds__(kSweepThreads) k_cloud_density_error(GridK g, FluidK p, const float4* __restrict__ pos,
                                                                       const uint2* __restrict__ table, uint32_t n,
                                                                       float* __restrict__ errPartial) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float err = 0.0f;
  if (i < n) {
    const Sph k(g);
    const float4 xi = ld4(pos + i);
    float rho = 0.0f;
    for_each_cloud_neighbour(g, table, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(pos + j);
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) rho += k.w(r2);
    });
    err = fabsf(rho / p.rho0 - 1.0f);
  }
  block_error_partial(err, errPartial);
}

// cld_computeConstraintCorrection, cld_correctPosition x2 and the mixed boundary
// (Clouds.cpp:577-586); LAST adds cld_updateVel (clouds.cl:958-966).  kQuad lanes.
template <bool LAST>
__global__ void __launch_bounds__(128, 8) k_cloud_deltap(GridK g, FluidK p, const float4* __restrict__ pred,
                                                      const float* __restrict__ lambda, const uint2* __restrict__ table,
                                                      uint32_t n, float4* __restrict__ predOut, float4* __restrict__ tot,
                                                      float4* __restrict__ velS, PairList pl,
                                                      const float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  float4 xi = f4(0.f, 0.f, 0.f, 0.f);
  if (active) {
    const Sph k(g);
    xi = ld4(pred + i);
    const float li = __ldg(lambda + i);
    quad_cloud_pairs(g, table, pl, i, q, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(packed + j);  // (x, y, z, lambda) from k_cloud_lambda
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        float sc = 0.0f;
        if (p.artPressure) sc = -p.apCoeff * powi(k.w(r2) * p.apInvWq, p.apExp);
        const float f = (li + xj.w + sc) * s;
        ax += vx * f;
        ay += vy * f;
        az += vz * f;
      }
    });
  }
  ax = quad_sum(ax);
  ay = quad_sum(ay);
  az = quad_sum(az);
  if (!active || q != 0) return;
  const float4 dp = f4(ax * p.invRho0, ay * p.invRho0, az * p.invRho0, 0.0f);
  predOut[i] = mixed_bc(g, xi + dp);
  const float4 tt = tot[i] + dp;
  tot[i] = tt;
  if (LAST) {
    const float d = p.dt + kFloatEps;
    velS[i] = clamp4s(f4(__fdiv_rn(tt.x, d), __fdiv_rn(tt.y, d), __fdiv_rn(tt.z, d), __fdiv_rn(tt.w, d)), -g.maxVel,
                      g.maxVel);
  }
}

__global__ void k_cloud_update_vel(GridK g, FluidK p, const float4* __restrict__ tot, uint32_t n,
                                   float4* __restrict__ velS) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 t = ld4(tot + i);
  const float d = p.dt + kFloatEps;
  velS[i] = clamp4s(f4(__fdiv_rn(t.x, d), __fdiv_rn(t.y, d), __fdiv_rn(t.z, d), __fdiv_rn(t.w, d)), -g.maxVel, g.maxVel);
}

// cld_computeVorticity (clouds.cl:727-785); records the pairs within h of the final
// positions for confinement and XSPH.
__global__ void __launch_bounds__(kSweepThreads, 16) k_cloud_vorticity(GridK g, const float4* __restrict__ pred,
                                                                       const float4* __restrict__ velS,
                                                                       const uint2* __restrict__ table, uint32_t n,
                                                                       float4* __restrict__ vort, PairList pl,
                                                                       float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Sph k(g);
  const float4 xi = ld4(pred + i), vi = ld4(velS + i);
  ListWriter lw(pl, i);
  filter_cloud_neighbours(g, table, pred, xi, k.h2, lw);
  float4 w = f4(0.f, 0.f, 0.f, 0.f);
  auto body_at = [&](float4 xj, float4 vj, float shx, float shz) {
    const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      float r;
      const float s = k.gs(r2, r);
      w = w + cross4(vj - vi, f4(vx * s, vy * s, vz * s, 0.0f));
    }
  };
  auto body = [&](uint32_t j, float shx, float shz) { body_at(ld4(pred + j), ld4(velS + j), shx, shz); };
  if (lw.ok())
    visit_list_x4(0, lw.n, 1, [&](uint32_t kk) { return lw.at(kk); },
                  [&](uint32_t e) { return Pair44{ld4(pred + (e & 0x0FFFFFFFu)), ld4(velS + (e & 0x0FFFFFFFu))}; },
                  [&](uint32_t e, Pair44 a) {
                    float shx, shz;
                    image_shift(g, e >> 28, shx, shz);
                    body_at(a.x, a.v, shx, shz);
                  });
  else
    for_each_cloud_neighbour(g, table, xi, body);
  pl.count[i] = lw.ok() ? lw.n : kListOverflow;
  vort[i] = w;
  packed[i] = f4(xi.x, xi.y, xi.z, sqrtf(dot4(w, w)));
}

// cld_applyVorticityConfinement (clouds.cl:790-850).  kQuad lanes per particle.
__global__ void __launch_bounds__(128, 8) k_cloud_confine(GridK g, FluidK p, const float4* __restrict__ pred,
                                                       const float4* __restrict__ vort, const uint2* __restrict__ table,
                                                       uint32_t n, float4* __restrict__ velS, PairList pl,
                                                       const float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  if (active) {
    const Sph k(g);
    const float4 xi = ld4(pred + i);
    quad_cloud_pairs(g, table, pl, i, q, xi, [&](uint32_t j, float shx, float shz) {
      const float4 xj = ld4(packed + j);  // (x, y, z, |omega|) from k_cloud_vorticity
      const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        const float f = xj.w * s;
        ex += vx * f;
        ey += vy * f;
        ez += vz * f;
      }
    });
  }
  ex = quad_sum(ex);
  ey = quad_sum(ey);
  ez = quad_sum(ez);
  if (!active || q != 0) return;
  const float4 cr = cross4(normalize0(f4(ex, ey, ez, 0.0f)), ld4(vort + i));
  const float s = p.vortCoeff * p.dt;
  float4 v = velS[i];
  v.x += cr.x * s;
  v.y += cr.y * s;
  v.z += cr.z * s;
  velS[i] = v;
}

// cld_applyXsphViscosityCorrection (clouds.cl:856-915) + cld_updatePosition (:942-953);
// writes the canonical state (pos, vel, temp, vapor, cloud, buoyancy, ids).  kQuad lanes.
__global__ void __launch_bounds__(128, 8) k_cloud_final(GridK g, FluidK p, CloudK c, const float4* __restrict__ pred,
                                                     const float4* __restrict__ velS, const uint2* __restrict__ table,
                                                     uint32_t n, CloudState s, PairList pl) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / kQuad, q = t % kQuad;
  const bool active = i < n;
  float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
  float4 xi = f4(0.f, 0.f, 0.f, 0.f), vi = xi;
  if (active) {
    xi = ld4(pred + i);
    vi = ld4(velS + i);
    if (p.vorticity) {
      const Sph k(g);
      quad_cloud_pairs(g, table, pl, i, q, xi, [&](uint32_t j, float shx, float shz) {
        const float4 xj = ld4(pred + j);
        const float vx = xi.x - xj.x - shx, vy = xi.y - xj.y, vz = xi.z - xj.z - shz;
        const float r2 = vx * vx + vy * vy + vz * vz;
        if (r2 < k.h2) {
          const float wv = k.w(r2);
          const float4 vj = ld4(velS + j);
          ax += (vj.x - vi.x) * wv;
          ay += (vj.y - vi.y) * wv;
          az += (vj.z - vi.z) * wv;
          aw += (vj.w - vi.w) * wv;
        }
      });
    }
  }
  ax = quad_sum(ax);
  ay = quad_sum(ay);
  az = quad_sum(az);
  aw = quad_sum(aw);
  if (!active || q != 0) return;
  s.vel[i] = p.vorticity ? f4(vi.x + p.xsph * ax, vi.y + p.xsph * ay, vi.z + p.xsph * az, vi.w + p.xsph * aw) : vi;
  float4 x = xi;
  const float alt = xi.y + g.W[1];
  x.x += (1.0f - expf(-alt * c.windX)) * c.wind * c.dt * (float)(c.dim - 2u);
  x.z += (1.0f - expf(-alt * c.windZ)) * 0.7f * c.wind * c.dt;
  s.pos[i] = x;
  s.temp[i] = __ldg(s.tempS + i);
  s.vapor[i] = __ldg(s.vaporS + i);
  s.cloud[i] = __ldg(s.cloudS + i);
  s.buoy[i] = __ldg(s.buoyS + i);
  if (s.ids) s.ids[i] = __ldg(s.idsS + i);
}

// cld_initTemperature + cld_initVaporDensity (clouds.cl:116-135); cloud = 0.
__global__ void k_cloud_init(GridK g, CloudK c, const float4* __restrict__ pos, uint32_t n, float* __restrict__ temp,
                             float* __restrict__ vapor, float* __restrict__ cloud, float* __restrict__ buoy) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float t = env_temp(c, g, ld4(pos + i));
  temp[i] = t;
  vapor[i] = c.initVapor * qsat(t);
  cloud[i] = 0.0f;
  buoy[i] = 0.0f;
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}
static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

int cloud_presort(const GridK& g, const CloudK& c, const float4* pos, const float4* vel, uint32_t n, float* temp,
                  float* vapor, float* cloud, float* buoy, float4* pred, float4* tot, uint32_t* keys,
                  const SortPlan& plan, uint32_t* hist0, Launcher& L, const ZeroJob& zero) {
  L.begin("cld_thermo_predict");
  launch(L, k_cloud_thermo_predict, dim3(plan.tiles), dim3(kKeyThreads), g, c, pos, vel, n, temp, vapor, cloud, buoy, pred,
                                                                    tot, keys, plan.bits[0], hist0, zero);
  L.end("cld_thermo_predict");
  return check("k_cloud_thermo_predict");
}

int cloud_temperature(const GridK& g, const CloudK& c, const float4* posS, float* tempS, float* lamT, const uint2* table,
                      uint32_t n, const PairList& pl, Launcher& L, float4* packed) {
  L.begin("cld_temp_lambda");
  launch(L, k_cloud_temp_lambda, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, c, posS, tempS, table, n, lamT, pl,
         packed);
  L.end("cld_temp_lambda");
  int rc = check("k_cloud_temp_lambda");
  if (rc) return rc;
  L.begin("cld_temp_correct");
  launch(L, k_cloud_temp_correct, dim3(blocks(n * kQuad, 128)), dim3(128), g, c, posS, lamT, table, n, tempS, pl,
         packed);
  L.end("cld_temp_correct");
  return check("k_cloud_temp_correct");
}

int cloud_iteration(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, float4* totS,
                    const uint2* table, uint32_t n, float* lambda, float* density, bool last, float4* velS,
                    const PairList& pl, Launcher& L, float4* packed) {
  L.begin("cld_lambda");
  launch(L, k_cloud_lambda, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, predIn, table, n, lambda, density, pl,
         packed);
  L.end("cld_lambda");
  int rc = check("k_cloud_lambda");
  if (rc) return rc;
  L.begin(last ? "cld_deltap_vel" : "cld_deltap");
  if (last)
    launch(L, k_cloud_deltap<true>, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, predIn, lambda, table, n, predOut, totS, velS,
                                                                        pl, packed);
  else
    launch(L, k_cloud_deltap<false>, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, predIn, lambda, table, n, predOut, totS,
                                                                         velS, pl, packed);
  L.end(last ? "cld_deltap_vel" : "cld_deltap");
  return check("k_cloud_deltap");
}

int cloud_ws_lambda(const GridK& g, const FluidK& p, const CloudK& c, const float4* pred, const float4* velS,
                    const float* tempS, const float* buoyS, const uint2* table, uint32_t n, float* lambda,
                    float* density, const PairList& pl, float4* packed, float* feats, const void* mlpBlock,
                    Launcher& L) {
  if (n == 0) return RTP_OK;
  if (feats) {
    MlpDev m{};
    L.begin("cld_ws_features");
    launch(L, k_cloud_ws_lambda<kCwsRecord>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, c, pred, velS,
           tempS, buoyS, table, n, lambda, density, pl, packed, feats, m);
    L.end("cld_ws_features");
  } else {
    L.begin("cld_ws_lambda_mlp");
    launch(L, k_cloud_ws_lambda<kCwsInfer>, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, c, pred, velS,
           tempS, buoyS, table, n, lambda, density, pl, packed, (float*)nullptr, mlp_dev(mlpBlock));
    L.end("cld_ws_lambda_mlp");
  }
  return check("k_cloud_ws_lambda");
}

int cloud_deltap(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, float4* totS,
                 const float* lambda, const uint2* table, uint32_t n, bool last, float4* velS, const PairList& pl,
                 Launcher& L, const float4* packed) {
  L.begin(last ? "cld_deltap_vel" : "cld_deltap");
  if (last)
    launch(L, k_cloud_deltap<true>, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, predIn, lambda, table, n, predOut,
           totS, velS, pl, packed);
  else
    launch(L, k_cloud_deltap<false>, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, predIn, lambda, table, n, predOut,
           totS, velS, pl, packed);
  L.end(last ? "cld_deltap_vel" : "cld_deltap");
  return check("k_cloud_deltap");
}

int cloud_density(const GridK& g, const FluidK& p, const float4* pred, const uint2* table, uint32_t n, float* lambda,
                  float* density, const PairList& pl, float4* packed, Launcher& L) {
  L.begin("cld_lambda");
  launch(L, k_cloud_lambda, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, pred, table, n, lambda, density,
         pl, packed);
  L.end("cld_lambda");
  return check("k_cloud_lambda");
}

int cloud_ws_loss_grad_x(const GridK& g, const FluidK& p, const float4* xp, const float* rho2, const uint2* table,
                         uint32_t n, const PairList& pl2, float4* gOut, float* lossPart, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_cloud_ws_loss_grad_x, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, xp, rho2, table, n, pl2,
         (float)(1.0 / (double)n), gOut, lossPart);
  return check("k_cloud_ws_loss_grad_x");
}

int cloud_ws_grad_y(const GridK& g, const FluidK& p, const float4* xs, const float* lam, const float* y,
                    const float4* gIn, const uint2* table, uint32_t n, const PairList& pl, float* dy, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_cloud_ws_grad_y, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, xs, lam, y, gIn, table, n, pl, dy);
  return check("k_cloud_ws_grad_y");
}

int cloud_density_error(const GridK& g, const FluidK& p, const float4* pos, const uint2* table, uint32_t n,
                        float* errPartial, Launcher& L) {
  if (n == 0) return RTP_OK;
  L.begin("cld_density_error");
  launch(L, k_cloud_density_error, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, p, pos, table, n, errPartial);
  L.end("cld_density_error");
  return check("k_cloud_density_error");
}

int cloud_update_vel(const GridK& g, const FluidK& p, const float4* totS, uint32_t n, float4* velS, Launcher& L) {
  L.begin("cld_updateVel");
  launch(L, k_cloud_update_vel, dim3(blocks(n, 256)), dim3(256), g, p, totS, n, velS);
  L.end("cld_updateVel");
  return check("k_cloud_update_vel");
}

int cloud_post(const GridK& g, const FluidK& p, const CloudK& c, const float4* pred, float4* velS, float4* vort,
               const uint2* table, uint32_t n, const CloudState& s, const PairList& pl, Launcher& L, float4* packed) {
  if (p.vorticity) {
    L.begin("cld_vorticity");
    launch(L, k_cloud_vorticity, dim3(blocks(n, kSweepThreads)), dim3(kSweepThreads), g, pred, velS, table, n, vort, pl,
           packed);
    L.end("cld_vorticity");
    int rc = check("k_cloud_vorticity");
    if (rc) return rc;
    L.begin("cld_confine");
    launch(L, k_cloud_confine, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, pred, vort, table, n, velS, pl, packed);
    L.end("cld_confine");
    rc = check("k_cloud_confine");
    if (rc) return rc;
  }
  L.begin("cld_xsph_final");
  launch(L, k_cloud_final, dim3(blocks(n * kQuad, 128)), dim3(128), g, p, c, pred, velS, table, n, s, pl);
  L.end("cld_xsph_final");
  return check("k_cloud_final");
}

int cloud_init(const GridK& g, const CloudK& c, const float4* pos, uint32_t n, float* temp, float* vapor, float* cloud,
               float* buoy, Launcher& L) {
  if (n == 0) return RTP_OK;
  L.begin("cld_init");
  launch(L, k_cloud_init, dim3(blocks(n, 256)), dim3(256), g, c, pos, n, temp, vapor, cloud, buoy);
  L.end("cld_init");
  return check("k_cloud_init");
}

}  // namespace rtp
