// fluids.cu - position-based fluids step (GB300, sm_103a).
//
// Replaces kernels/fluids.cl driven by Fluids::update (physics/ocl/Fluids.cpp:400-457).
// Per substep (I Jacobi iterations, vorticity on):
//   k_fluid_predict       fld_predictPosition + fillCellIDs + sort-tile histogram
//   sort passes           RadixSort::sort of {pos, vel, predPos} (+ particle ids)
//   cell table            resetStartEndCell / fillStartCell / fillEndCell (+ cap on read)
//   I x k_fluid_lambda    fld_applyBoundaryCondition (clamp on load) + fld_computeDensity
//                         + fld_computeConstraintFactor; records the pairs within h
//   I x k_fluid_deltap    fld_computeConstraintCorrection + fld_correctPosition into a
//                         second buffer (Jacobi), over the recorded pairs; the last one
//                         also does fld_updateVel
//   k_fluid_vorticity     fld_computeVorticity; records the pairs within h of the final
//                         positions
//   k_fluid_confine       fld_applyVorticityConfinement (in place: reads only vort of others)
//   k_fluid_xsph_final    fld_applyXsphViscosityCorrection + fld_updatePosition, writing
//                         the state back to the canonical pos/vel buffers
// The 27-cell searches (fluids.cl:101-123) run in two phases: a filter pass that only
// compares distances and records the pairs within h, then the SPH arithmetic over that
// compact list, so lanes do not all pay for the arithmetic whenever any lane of the warp
// has a neighbour.  The list sweeps give 4 lanes to each particle.
#include "fluids.cuh"

namespace rtp {

// fld_predictPosition (fluids.cl:62-74) + fillCellIDs (grid.cl:76-86) + digit-0 histogram.
// Round-to-nearest intrinsics make predPos, and so the cell keys, bit-identical to the CPU.
// With io.inPos / io.inVel the inputs come from host memory and are mirrored into pos / vel.
template <bool BATCH>
__global__ void __launch_bounds__(kKeyThreads) k_fluid_predict(GridK g0, FluidK p0, float4* __restrict__ pos,
                                                                float4* __restrict__ vel, uint32_t n,
                                                                float4* __restrict__ pred, uint32_t* __restrict__ keys,
                                                                int bits0, uint32_t* __restrict__ hist0, int clampOut,
                                                                ZeroJob zero, HostIO io) {
  pdl_enter();
  __shared__ uint32_t s_hist[kMaxBins];
  zero_job(zero);
  TileHistogram th;
  th.init(s_hist, bits0);
  const float dt = p0.dt;
  const float gx = __fmul_rn(0.0f, dt), gy = __fmul_rn(-kAbsGravityY, dt);
  const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll 2
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t i = base + k * kKeyThreads + threadIdx.x;
    if (i < n) {
      GridK g = g0;
      FluidK p = p0;
      scene_of<BATCH>(i, g, p);
      float4 x, v;
      if (io.inPos) {
        x = io.inPos[i];
        pos[i] = x;
      } else {
        x = ld4(pos + i);
      }
      if (io.inVel) {
        v = io.inVel[i];
        vel[i] = v;
      } else {
        v = ld4(vel + i);
      }
      const float4 nv = f4(__fadd_rn(v.x, gx), __fadd_rn(v.y, gy), __fadd_rn(v.z, gx), __fadd_rn(v.w, gx));
      const float4 pp = f4(__fadd_rn(x.x, __fmul_rn(nv.x, dt)), __fadd_rn(x.y, __fmul_rn(nv.y, dt)),
                           __fadd_rn(x.z, __fmul_rn(nv.z, dt)), __fadd_rn(x.w, __fmul_rn(nv.w, dt)));
      // The key comes from the unclamped prediction (fillCellIDs runs before the first
      // fld_applyBoundaryCondition); the stored copy is clamped already when a Jacobi
      // iteration (which starts with that clamp) consumes it.
      pred[i] = clampOut ? bc_clamp(p, pp) : pp;
      const uint32_t key = cell_key(g, pp);
      keys[i] = key;
      th.add(key);
    }
  }
  th.store(hist0);
}

// The sums of fld_computeDensity / fld_computeConstraintFactor over the pairs of particle i.
struct LambdaSums {
  float rho = 0.0f, sgx = 0.0f, sgy = 0.0f, sgz = 0.0f, ssq = 0.0f;
  __device__ __forceinline__ void add(const Sph& k, float4 xi, float4 xj) {
    const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      rho += k.w(r2);
      float r;
      const float s = k.gs(r2, r);
      const float gxx = vx * s, gyy = vy * s, gzz = vz * s;
      sgx += gxx;
      sgy += gyy;
      sgz += gzz;
      ssq += gxx * gxx + gyy * gyy + gzz * gzz;
    }
  }
};

// lambda_i from the sums (fld_computeConstraintFactor) and the sweep's outputs.
__device__ __forceinline__ void lambda_finish(const FluidK& p, uint32_t i, float4 xi, LambdaSums sm,
                                              float* __restrict__ lambda, float* __restrict__ density,
                                              float* __restrict__ lamTot, int totMode, float4* __restrict__ packed,
                                              const float* __restrict__ omega) {
  const float C = sm.rho / p.rho0 - 1.0f;
  float ssq = sm.ssq + (sm.sgx * sm.sgx + sm.sgy * sm.sgy + sm.sgz * sm.sgz);
  ssq *= p.invRho0Sq;
  float lam = -C / (ssq + p.relaxCFM);
  if (omega) lam *= __ldg(omega + i);  // warm start relaxing every iteration
  lambda[i] = lam;
  density[i] = sm.rho;
  if (packed) packed[i] = f4(xi.x, xi.y, xi.z, lam);
  // Total lambda of the step (warm start): kTotWrite starts it, kTotAdd accumulates.
  if (totMode == kTotWrite) lamTot[i] = lam;
  else if (totMode == kTotAdd) lamTot[i] += lam;
}

// The lambda sweep of particle i at xi from global memory: a filter pass over the 27 cells
// writes the pairs within h to the device list, then the sums run over that list (over the
// 27 cells again when the list overflowed).
template <bool MASK>
__device__ __forceinline__ void fluid_lambda_global(const GridK& g, const FluidK& p, const float4* __restrict__ pred,
                                                    const uint2* __restrict__ table, uint32_t i, float4 xi,
                                                    const PairList& pl, float* __restrict__ lambda,
                                                    float* __restrict__ density, float* __restrict__ lamTot,
                                                    int totMode, float4* __restrict__ packed,
                                                    const float* __restrict__ omega) {
  const Sph k(g);
  uint32_t cnt = 0;
  uint32_t* lst = pl.idx + i;
  filter_fluid_neighbours_to<MASK>(g, table, xi, k.h2, [&](uint32_t j) { return ld4(pred + j); }, [&](uint32_t j) {
    if (cnt < pl.K) lst[(size_t)cnt * pl.stride] = j;
    ++cnt;
  });
  LambdaSums sm;
  auto ldp = [&](uint32_t j) { return ld4(pred + j); };
  auto body = [&](uint32_t, float4 xj) { sm.add(k, xi, xj); };
  if (cnt <= pl.K)
    visit_list_x4(0, cnt, 1, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ldp, body);
  else
    for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { body(j, ldp(j)); });
  pl.count[i] = cnt <= pl.K ? cnt : kListOverflow;
  lambda_finish(p, i, xi, sm, lambda, density, lamTot, totMode, packed, omega);
}

// fld_applyBoundaryCondition + fld_computeDensity + fld_computeConstraintFactor; records
// the pairs within h for k_fluid_deltap.  One thread per particle (fluid_lambda_global).
template <bool BATCH, bool MASK>
__global__ void __launch_bounds__(kSweepThreads, BATCH ? 12 : 16) k_fluid_lambda(GridK g, FluidK p, const float4* __restrict__ pred,
                                                                const uint2* __restrict__ table, uint32_t n,
                                                                float* __restrict__ lambda,
                                                                float* __restrict__ density, PairList pl,
                                                                float* __restrict__ lamTot, int totMode,
                                                                float4* __restrict__ packed,
                                                                const float* __restrict__ omega) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  scene_of<BATCH>(i, g, p);
  fluid_lambda_global<MASK>(g, p, pred, table, i, ld4(pred + i), pl, lambda, density, lamTot, totMode, packed, omega);
}

// ---- the lambda sweep tiled by bricks of cells (one scene, every grid axis >= 6 cells) ------
// The grid is cut into bricks of kBrick^3 cells; one CTA per brick stages the sorted
// positions of the brick and its one-cell halo (kHalo^3 cells, each cell's capped range, in
// the key order: x, then y, then z fastest) in shared memory with coalesced loads, then runs
// the filter pass of the particles stored in the brick's cells from there (the sums walk the
// recorded list, whose positions the staging brought into L1).  The
// three z cells of a halo row around a particle are consecutive in shared memory, so every
// particle visits its 27 cells in the order of fluid_lambda_global and writes the same list
// (its sums can differ from the one-lane sweep's in the last bit where the compiler fuses the
// two kernels' multiply-adds differently).  A particle whose current cell (positions move between
// Jacobi iterations) is not inside its brick, and every particle of a brick whose halo holds
// more than kBrickCap particles, takes fluid_lambda_global.  The extra last CTA takes the
// particles stored in no cell's range: the first sorted one (left out of its cell as
// fillStartCell does) and those with keys past the grid.
constexpr int kBrick = 4;
constexpr int kHalo = kBrick + 2;
constexpr int kHaloCells = kHalo * kHalo * kHalo;
constexpr int kOwnCells = kBrick * kBrick * kBrick;
constexpr uint32_t kBrickThreads = 256;
constexpr uint32_t kBrickCap = 2560;
constexpr size_t kBrickSmem =
    (size_t)kBrickCap * sizeof(float4) + (size_t)(kHaloCells + 1 + kHaloCells + kOwnCells + 1 + kOwnCells) * sizeof(uint32_t);

__device__ __forceinline__ int wrap_halo(int v, int R) { return v < 0 ? v + R : (v >= R ? v - R : v); }

// Exclusive scan of a (threads < 256) over the CTA: returns the prefix; *total gets the sum.
__device__ __forceinline__ uint32_t brick_scan(uint32_t a, uint32_t* s_warp, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  uint32_t x = a;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_warp[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t v = lane < kBrickThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= (uint32_t)o) v += y;
    }
    if (lane < kBrickThreads / 32) s_warp[lane] = v;
  }
  __syncthreads();
  const uint32_t before = w ? s_warp[w - 1] : 0u;
  *total = s_warp[kBrickThreads / 32 - 1];
  __syncthreads();
  return before + x - a;
}

// Largest c in [0, count) with beg[c] <= s (beg ascending, beg[0] <= s).
__device__ __forceinline__ uint32_t brick_find(const uint32_t* beg, uint32_t count, uint32_t s) {
  uint32_t lo = 0, hi = count;
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (beg[mid] <= s) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <bool MASK>
__global__ void __launch_bounds__(kBrickThreads, 4)
    k_fluid_lambda_brick(GridK g, FluidK p, const float4* __restrict__ pred, const uint2* __restrict__ table,
                         const uint32_t* __restrict__ keys, uint32_t n, int nbx, int nby, int nbz,
                         float* __restrict__ lambda, float* __restrict__ density, PairList pl,
                         float* __restrict__ lamTot, int totMode, float4* __restrict__ packed,
                         const float* __restrict__ omega) {
  extern __shared__ __align__(16) unsigned char brick_smem[];
  float4* s_pos = reinterpret_cast<float4*>(brick_smem);
  uint32_t* s_beg = reinterpret_cast<uint32_t*>(s_pos + kBrickCap);
  uint32_t* s_glob = s_beg + (kHaloCells + 1);
  uint32_t* s_own = s_glob + kHaloCells;
  uint32_t* s_ownStart = s_own + (kOwnCells + 1);
  __shared__ uint32_t s_warp[kBrickThreads / 32];
  pdl_enter();
  const uint32_t t = threadIdx.x;
  const uint32_t nBricks = (uint32_t)(nbx * nby * nbz);
  if (blockIdx.x == nBricks) {
    if (t == 0 && n > 0 && __ldg(keys) < g.nc)
      fluid_lambda_global<MASK>(g, p, pred, table, 0, ld4(pred), pl, lambda, density, lamTot, totMode, packed, omega);
    for (int64_t i = (int64_t)n - 1 - t; i >= 0; i -= kBrickThreads) {
      if (__ldg(keys + i) < g.nc) break;
      fluid_lambda_global<MASK>(g, p, pred, table, (uint32_t)i, ld4(pred + i), pl, lambda, density, lamTot, totMode,
                                packed, omega);
    }
    return;
  }
  const int bz = (int)(blockIdx.x % (uint32_t)nbz), by = (int)((blockIdx.x / (uint32_t)nbz) % (uint32_t)nby);
  const int bx = (int)(blockIdx.x / (uint32_t)(nbz * nby));
  const int x0 = bx * kBrick, y0 = by * kBrick, z0 = bz * kBrick;
  // Halo cells (capped ranges, staged) and own cells (full ranges, processed).
  uint32_t cnt = 0, own = 0;
  if (t < (uint32_t)kHaloCells) {
    const int hz = (int)t % kHalo, hy = ((int)t / kHalo) % kHalo, hx = (int)t / (kHalo * kHalo);
    const int x = wrap_halo(x0 - 1 + hx, g.R[0]), y = wrap_halo(y0 - 1 + hy, g.R[1]), z = wrap_halo(z0 - 1 + hz, g.R[2]);
    uint32_t b, e;
    cell_range(table, g.base + ((uint32_t)x * g.R[1] + (uint32_t)y) * g.R[2] + (uint32_t)z, g.cap, b, e);
    cnt = e - b;
    s_glob[t] = b;
  }
  if (t < (uint32_t)kOwnCells) {
    const int rz = (int)t % kBrick, ry = ((int)t / kBrick) % kBrick, rx = (int)t / (kBrick * kBrick);
    const int x = x0 + rx, y = y0 + ry, z = z0 + rz;
    uint32_t st = 0;
    if (x < g.R[0] && y < g.R[1] && z < g.R[2]) {
      const uint2 se = __ldg(table + g.base + ((uint32_t)x * g.R[1] + (uint32_t)y) * g.R[2] + (uint32_t)z);
      own = se.y > se.x ? se.y - se.x : 0u;
      st = se.x;
    }
    s_ownStart[t] = st;
  }
  uint32_t haloTotal, ownTotal;
  const uint32_t hb = brick_scan(cnt, s_warp, &haloTotal);
  const uint32_t ob = brick_scan(own, s_warp, &ownTotal);
  if (t < (uint32_t)kHaloCells) s_beg[t] = hb;
  if (t == 0) s_beg[kHaloCells] = haloTotal;
  if (t < (uint32_t)kOwnCells) s_own[t] = ob;
  if (t == 0) s_own[kOwnCells] = ownTotal;
  if (ownTotal == 0) return;  // uniform over the CTA
  const bool staged = haloTotal <= kBrickCap;
  __syncthreads();
  if (staged)
    for (uint32_t s = t; s < haloTotal; s += kBrickThreads) {
      const uint32_t c = brick_find(s_beg, kHaloCells, s);
      const uint32_t j = s_glob[c] + (s - s_beg[c]);
      const float4 v = ld4(pred + j);
      s_pos[s] = f4(v.x, v.y, v.z, __uint_as_float(j));
    }
  __syncthreads();
  const Sph k(g);
  for (uint32_t o = t; o < ownTotal; o += kBrickThreads) {
    const uint32_t c = brick_find(s_own, kOwnCells, o);
    const uint32_t i = s_ownStart[c] + (o - s_own[c]);
    const float4 xi = ld4(pred + i);
    int cx, cy, cz;
    cell3(g, xi, cx, cy, cz);
    const int rx = cx - x0, ry = cy - y0, rz = cz - z0;
    if (!staged || (uint32_t)rx >= (uint32_t)kBrick || (uint32_t)ry >= (uint32_t)kBrick ||
        (uint32_t)rz >= (uint32_t)kBrick) {
      fluid_lambda_global<MASK>(g, p, pred, table, i, xi, pl, lambda, density, lamTot, totMode, packed, omega);
      continue;
    }
    uint32_t m = 0;
    uint32_t* lst = pl.idx + i;
    auto test = [&](uint32_t, float4 xj) {
      if (within_radius(xi, xj, k.h2)) {
        if (m < pl.K) lst[(size_t)m * pl.stride] = __float_as_uint(xj.w);
        ++m;
      }
    };
    auto lds = [&](uint32_t s) { return s_pos[s]; };
#pragma unroll 1
    for (int a = 0; a < 3; ++a)
#pragma unroll 1
      for (int b = 0; b < 3; ++b) {
        const int row = ((rx + a) * kHalo + (ry + b)) * kHalo + rz;
        visit_range_x8(s_beg[row], s_beg[row + 3], lds, test);
      }
    // The sums over the list from global memory (the positions this CTA staged are in L1).
    LambdaSums sm;
    auto ldp = [&](uint32_t j) { return ld4(pred + j); };
    auto body = [&](uint32_t, float4 xj) { sm.add(k, xi, xj); };
    if (m <= pl.K)
      visit_list_x4(0, m, 1, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ldp, body);
    else
      for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { body(j, ldp(j)); });
    pl.count[i] = m <= pl.K ? m : kListOverflow;
    lambda_finish(p, i, xi, sm, lambda, density, lamTot, totMode, packed, omega);
  }
}

// k_fluid_lambda with a group of LW lanes per particle (particle counts too small to keep the
// GPU busy with one lane each): the group filters the 27 cells together (filter_fluid_group)
// and sums the SPH terms over the list, one entry per lane.
template <bool BATCH, int LW>
__global__ void __launch_bounds__(128) k_fluid_lambda_group(GridK g, FluidK p, const float4* __restrict__ pred,
                                                            const uint2* __restrict__ table, uint32_t n,
                                                            float* __restrict__ lambda, float* __restrict__ density,
                                                            PairList pl, float* __restrict__ lamTot, int totMode,
                                                            float4* __restrict__ packed, const float* __restrict__ omega) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, q = t % LW;
  if ((t & ~31u) / LW >= n) return;  // the whole warp is past the last particle
  const bool live = t / LW < n;
  const uint32_t i = live ? t / LW : n - 1u;  // a group past the end shadows the last particle
  scene_of<BATCH>(i, g, p);
  const Sph k(g);
  const float4 xi = ld4(pred + i);
  auto ldp = [&](uint32_t j) { return ld4(pred + j); };
  uint32_t* lst = pl.idx + i;
  const uint32_t cnt = filter_fluid_group<LW>(g, table, xi, live, k.h2, ldp, lst, pl.stride, pl.K);
  float rho = 0.0f, sgx = 0.0f, sgy = 0.0f, sgz = 0.0f, ssq = 0.0f;
  auto body = [&](uint32_t, float4 xj) {
    const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
    const float r2 = vx * vx + vy * vy + vz * vz;
    if (r2 < k.h2) {
      rho += k.w(r2);
      float r;
      const float s = k.gs(r2, r);
      const float gxx = vx * s, gyy = vy * s, gzz = vz * s;
      sgx += gxx;
      sgy += gyy;
      sgz += gzz;
      ssq += gxx * gxx + gyy * gyy + gzz * gzz;
    }
  };
  walk_list_group<LW>(cnt <= pl.K ? cnt : 0u, i, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ldp,
                      body);
  if (cnt > pl.K && q == 0) for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { body(j, ldp(j)); });
  rho = quad_sum<LW>(rho);
  sgx = quad_sum<LW>(sgx);
  sgy = quad_sum<LW>(sgy);
  sgz = quad_sum<LW>(sgz);
  ssq = quad_sum<LW>(ssq);
  if (q != 0 || !live) return;
  pl.count[i] = cnt <= pl.K ? cnt : kListOverflow;
  const float C = rho / p.rho0 - 1.0f;
  ssq += sgx * sgx + sgy * sgy + sgz * sgz;
  ssq *= p.invRho0Sq;
  float lam = -C / (ssq + p.relaxCFM);
  if (omega) lam *= __ldg(omega + i);  // warm start relaxing every iteration
  lambda[i] = lam;
  density[i] = rho;
  if (packed) packed[i] = f4(xi.x, xi.y, xi.z, lam);
  if (totMode == kTotWrite) lamTot[i] = lam;
  else if (totMode == kTotAdd) lamTot[i] += lam;
}

// fld_computeConstraintCorrection + fld_correctPosition (Jacobi: writes a second buffer);
// LAST adds fld_updateVel (fluids.cl:263-273).  LANES lanes per particle.  Input positions
// are already clamped by fld_applyBoundaryCondition (done by their producer).
// PACKED: the neighbours' positions and lambdas come from one float4 array (x, y, z, lambda)
// written by the lambda sweep, one load per pair instead of two.
template <bool LAST, bool BATCH, int LANES, bool PACKED>
__global__ void __launch_bounds__(128, BATCH ? 1 : 12) k_fluid_deltap(GridK g, FluidK p, const float4* __restrict__ pred,
                                                      const float* __restrict__ lambda, const uint2* __restrict__ table,
                                                      uint32_t n, float4* __restrict__ predOut,
                                                      const float4* __restrict__ posS, float4* __restrict__ velS,
                                                      PairList pl, const float4* __restrict__ res,
                                                      const float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / LANES, q = t % LANES;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;  // a lane past the end shadows the last particle
  float cx = 0.0f, cy = 0.0f, cz = 0.0f;
  float4 xi;
  {
    scene_of<BATCH>(ii, g, p);
    const Sph k(g);
    xi = ld4(pred + ii);  // clamped by the producer
    const float li = PACKED ? ld4(packed + ii).w : __ldg(lambda + ii);
    auto ld = [&](uint32_t j) {
      if constexpr (PACKED) {
        const float4 a = ld4(packed + j);
        return Pair4{a, a.w};
      } else {
        return Pair4{ld4(pred + j), __ldg(lambda + j)};
      }
    };
    quad_pairs_sync<LANES, !BATCH>(g, table, pl, ii, q, active, xi, ld, [&](uint32_t, Pair4 a) {
      const float4 xj = a.x;
      const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        float sc = 0.0f;
        if (p.artPressure) sc = -p.apCoeff * powi(k.w(r2) * p.apInvWq, p.apExp);
        const float f = (li + a.s + sc) * s;
        cx += vx * f;
        cy += vy * f;
        cz += vz * f;
      }
    });
  }
  cx = quad_sum<LANES>(cx);
  cy = quad_sum<LANES>(cy);
  cz = quad_sum<LANES>(cz);
  if (!active || q != 0) return;
  float4 out = f4(xi.x + cx * p.invRho0, xi.y + cy * p.invRho0, xi.z + cz * p.invRho0, xi.w);
  if (res) {  // warm start: the network's residual displacement
    const float4 r = ld4(res + i);
    out.x += r.x;
    out.y += r.y;
    out.z += r.z;
  }
  // The next iteration starts with fld_applyBoundaryCondition: store its result directly.
  // After the last iteration the unclamped position is kept (fld_updateVel, fluids.cl:263).
  predOut[i] = LAST ? out : bc_clamp(p, out);
  if (LAST) {
    const float4 x0 = ld4(posS + i);
    const float d = p.dt + kFloatEps;
    velS[i] = clamp4s(f4(__fdiv_rn(out.x - x0.x, d), __fdiv_rn(out.y - x0.y, d), __fdiv_rn(out.z - x0.z, d),
                         __fdiv_rn(out.w - x0.w, d)),
                      -g.maxVel, g.maxVel);
  }
}

// fld_updateVel alone (only used when the solver runs zero iterations).
template <bool BATCH>
__global__ void k_fluid_update_vel(GridK g, FluidK p, const float4* __restrict__ pred, const float4* __restrict__ posS,
                                   uint32_t n, float4* __restrict__ velS) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  scene_of<BATCH>(i, g, p);
  const float4 a = ld4(pred + i), b = ld4(posS + i);
  const float d = p.dt + kFloatEps;
  velS[i] = clamp4s(f4(__fdiv_rn(a.x - b.x, d), __fdiv_rn(a.y - b.y, d), __fdiv_rn(a.z - b.z, d), __fdiv_rn(a.w - b.w, d)),
                    -g.maxVel, g.maxVel);
}

// fld_computeVorticity (fluids.cl:278-324); records the pairs within h of the final
// positions for confinement and XSPH (same two-phase scheme as k_fluid_lambda).
// GUARD also evaluates fld_computeDensity at those positions and writes each block's sum
// of |rho_i / rho0 - 1| to errPartial[blockIdx.x] (warm-start guard, solver statistics).
template <bool GUARD, bool BATCH, bool MASK>
__global__ void __launch_bounds__(kSweepThreads, BATCH ? 12 : 16) k_fluid_vorticity(GridK g, FluidK p, const float4* __restrict__ pred,
                                                                    const float4* __restrict__ velS,
                                                                    const uint2* __restrict__ table, uint32_t n,
                                                                    float4* __restrict__ vort, PairList pl,
                                                                    float* __restrict__ errPartial,
                                                                    float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float err = 0.0f;
  if (i < n) {
    scene_of<BATCH>(i, g, p);
    const Sph k(g);
    const float4 xi = ld4(pred + i), vi = ld4(velS + i);
    uint32_t cnt = 0;
    uint32_t* lst = pl.idx + i;
    filter_fluid_neighbours_to<MASK>(g, table, xi, k.h2, [&](uint32_t j) { return ld4(pred + j); }, [&](uint32_t j) {
      if (cnt < pl.K) lst[(size_t)cnt * pl.stride] = j;
      ++cnt;
    });
    float4 w = f4(0.0f, 0.0f, 0.0f, 0.0f);
    float rho = 0.0f;
    auto ld = [&](uint32_t j) { return Pair44{ld4(pred + j), ld4(velS + j)}; };
    auto body = [&](uint32_t, Pair44 a) {
      const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        if (GUARD) rho += k.w(r2);
        float r;
        const float s = k.gs(r2, r);
        w = w + cross4(a.v - vi, f4(vx * s, vy * s, vz * s, 0.0f));
      }
    };
    if (cnt <= pl.K)
      visit_list_x4(0, cnt, 1, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ld, body);
    else
      for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { body(j, ld(j)); });
    pl.count[i] = cnt <= pl.K ? cnt : kListOverflow;
    vort[i] = w;
    if (packed) packed[i] = f4(xi.x, xi.y, xi.z, sqrtf(dot4(w, w)));
    if (GUARD) err = fabsf(rho / p.rho0 - 1.0f);
  }
  if (GUARD) block_error_partial(err, errPartial);
}

// Threads of a guarded k_fluid_vorticity_group block: 64 particles of LW lanes, at most 1024.
template <int LW>
constexpr int kGuardGroupThreads = 64 * LW < 1024 ? 64 * LW : 1024;

// k_fluid_vorticity with a group of LW lanes per particle.  Without GUARD a block is 128
// threads.  With GUARD a block covers the 64 particles of one errPartial entry (particle
// blockIdx.x * 64 + r * P + t / LW, P = blockDim.x / LW, for r < 64 / P) and sums their
// errors in a fixed order; a particle's vorticity is the same either way.
template <bool GUARD, bool BATCH, int LW>
__global__ void __launch_bounds__(GUARD ? kGuardGroupThreads<LW> : 128) k_fluid_vorticity_group(
    GridK g, FluidK p, const float4* __restrict__ pred, const float4* __restrict__ velS,
    const uint2* __restrict__ table, uint32_t n, float4* __restrict__ vort, PairList pl,
    float* __restrict__ errPartial, float4* __restrict__ packed) {
  pdl_enter();
  constexpr uint32_t P = (GUARD ? kGuardGroupThreads<LW> : 128) / LW;  // particles per pass of the block
  constexpr uint32_t R = GUARD ? 64 / P : 1;
  static_assert(!GUARD || R * P == 64, "64 particles per guarded block");
  const uint32_t q = threadIdx.x % LW, slot = threadIdx.x / LW;
  __shared__ float s_err[GUARD ? 64 : 1];
  if (GUARD && q == 0)  // each entry is zeroed and later written by the same thread
    for (uint32_t r = 0; r < R; ++r) s_err[r * P + slot] = 0.0f;
#pragma unroll 1
  for (uint32_t r = 0; r < R; ++r) {
    const uint32_t i0 = GUARD ? blockIdx.x * 64u + r * P : blockIdx.x * P;  // first particle of the pass
    const uint32_t warpFirst = i0 + (slot & ~(32u / LW - 1u));                   // first of this warp
    if (warpFirst >= n) break;  // the whole warp is past the last particle
    const bool live = i0 + slot < n;
    const uint32_t i = live ? i0 + slot : n - 1u;  // a group past the end shadows the last particle
    GridK gi = g;
    FluidK pi = p;
    scene_of<BATCH>(i, gi, pi);
    const Sph k(gi);
    const float4 xi = ld4(pred + i), vi = ld4(velS + i);
    uint32_t* lst = pl.idx + i;
    const uint32_t cnt = filter_fluid_group<LW>(gi, table, xi, live, k.h2,
                                                [&](uint32_t j) { return ld4(pred + j); }, lst, pl.stride, pl.K);
    float4 w = f4(0.0f, 0.0f, 0.0f, 0.0f);
    float rho = 0.0f;
    auto ld = [&](uint32_t j) { return Pair44{ld4(pred + j), ld4(velS + j)}; };
    auto body = [&](uint32_t, Pair44 a) {
      const float vx = xi.x - a.x.x, vy = xi.y - a.x.y, vz = xi.z - a.x.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        if (GUARD) rho += k.w(r2);
        float rr;
        const float s = k.gs(r2, rr);
        w = w + cross4(a.v - vi, f4(vx * s, vy * s, vz * s, 0.0f));
      }
    };
    walk_list_group<LW>(cnt <= pl.K ? cnt : 0u, i, [&](uint32_t kk) { return lst[(size_t)kk * pl.stride]; }, ld,
                        body);
    if (cnt > pl.K && q == 0) for_each_fluid_neighbour(gi, table, xi, [&](uint32_t j) { body(j, ld(j)); });
    w.x = quad_sum<LW>(w.x);
    w.y = quad_sum<LW>(w.y);
    w.z = quad_sum<LW>(w.z);
    w.w = quad_sum<LW>(w.w);
    if (GUARD) rho = quad_sum<LW>(rho);
    if (q == 0 && live) {
      pl.count[i] = cnt <= pl.K ? cnt : kListOverflow;
      vort[i] = w;
      if (packed) packed[i] = f4(xi.x, xi.y, xi.z, sqrtf(dot4(w, w)));
      if (GUARD) s_err[r * P + slot] = fabsf(rho / pi.rho0 - 1.0f);
    }
  }
  if (GUARD) {
    __syncthreads();
    if (threadIdx.x == 0) {
      float e = 0.0f;
      for (int u = 0; u < 64; ++u) e += s_err[u];
      errPartial[blockIdx.x] = e;
    }
  }
}

// fld_applyVorticityConfinement (fluids.cl:329-377), LANES lanes per particle.  PACKED: each
// neighbour's position and |omega| come from one float4 (x, y, z, |omega|) written by the
// vorticity sweep.
template <bool BATCH, int LANES, bool PACKED>
__global__ void __launch_bounds__(128) k_fluid_confine(GridK g, FluidK p, const float4* __restrict__ pred,
                                                       const float4* __restrict__ vort, const uint2* __restrict__ table,
                                                       uint32_t n, float4* __restrict__ velS, PairList pl,
                                                       const float4* __restrict__ packed) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / LANES, q = t % LANES;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;  // a lane past the end shadows the last particle
  float ex = 0.0f, ey = 0.0f, ez = 0.0f;
  {
    scene_of<BATCH>(ii, g, p);
    const Sph k(g);
    const float4 xi = ld4(pred + ii);
    auto ld = [&](uint32_t j) {
      if constexpr (PACKED) {
        const float4 a = ld4(packed + j);
        return Pair4{a, a.w};
      } else {
        const float4 wj = ld4(vort + j);
        return Pair4{ld4(pred + j), sqrtf(dot4(wj, wj))};
      }
    };
    quad_pairs_sync<LANES, !BATCH>(g, table, pl, ii, q, active, xi, ld, [&](uint32_t, Pair4 a) {
      const float4 xj = a.x;
      const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        float r;
        const float s = k.gs(r2, r);
        const float f = a.s * s;
        ex += vx * f;
        ey += vy * f;
        ez += vz * f;
      }
    });
  }
  ex = quad_sum<LANES>(ex);
  ey = quad_sum<LANES>(ey);
  ez = quad_sum<LANES>(ez);
  if (!active || q != 0) return;
  const float4 c = cross4(normalize0(f4(ex, ey, ez, 0.0f)), ld4(vort + i));
  const float s = p.vortCoeff * p.dt;
  float4 v = velS[i];
  v.x += c.x * s;
  v.y += c.y * s;
  v.z += c.z * s;
  velS[i] = v;
}

// fld_applyXsphViscosityCorrection (fluids.cl:383-430) + fld_updatePosition (:444-450),
// writing the canonical state buffers.  LANES lanes per particle.
template <bool BATCH, int LANES>
__global__ void __launch_bounds__(128) k_fluid_xsph_final(GridK g, FluidK p, const float4* __restrict__ pred,
                                                          const float4* __restrict__ velS,
                                                          const uint2* __restrict__ table, uint32_t n,
                                                          const uint32_t* __restrict__ idsS, float4* __restrict__ pos,
                                                          float4* __restrict__ vel, uint32_t* __restrict__ ids,
                                                          PairList pl, HostIO io) {
  pdl_enter();
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t / LANES, q = t % LANES;
  const bool active = i < n;
  const uint32_t ii = active ? i : n - 1u;  // a lane past the end shadows the last particle
  float ax = 0.0f, ay = 0.0f, az = 0.0f, aw = 0.0f;
  float4 xi, vi;
  {
    scene_of<BATCH>(ii, g, p);
    const Sph k(g);
    xi = ld4(pred + ii);
    vi = ld4(velS + ii);
    auto ld = [&](uint32_t j) { return Pair44{ld4(pred + j), ld4(velS + j)}; };
    quad_pairs_sync<LANES, !BATCH>(g, table, pl, ii, q, active, xi, ld, [&](uint32_t, Pair44 a) {
      const float4 xj = a.x;
      const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        const float wv = k.w(r2);
        const float4 vj = a.v;
        ax += (vj.x - vi.x) * wv;
        ay += (vj.y - vi.y) * wv;
        az += (vj.z - vi.z) * wv;
        aw += (vj.w - vi.w) * wv;
      }
    });
  }
  ax = quad_sum<LANES>(ax);
  ay = quad_sum<LANES>(ay);
  az = quad_sum<LANES>(az);
  aw = quad_sum<LANES>(aw);
  if (!active || q != 0) return;
  const float4 vo = f4(vi.x + p.xsph * ax, vi.y + p.xsph * ay, vi.z + p.xsph * az, vi.w + p.xsph * aw);
  vel[i] = vo;
  pos[i] = xi;
  if (io.outVel) io.outVel[i] = vo;
  if (io.outPos) io.outPos[i] = xi;
  if (ids) ids[i] = __ldg(idsS + i);
}

// fld_updatePosition alone (vorticity confinement disabled: Fluids.cpp:444 skips XSPH too).
__global__ void k_fluid_final(const float4* __restrict__ pred, const float4* __restrict__ velS, uint32_t n,
                              const uint32_t* __restrict__ idsS, float4* __restrict__ pos, float4* __restrict__ vel,
                              uint32_t* __restrict__ ids, HostIO io) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = ld4(pred + i), v = ld4(velS + i);
  pos[i] = x;
  vel[i] = v;
  if (io.outPos) io.outPos[i] = x;
  if (io.outVel) io.outVel[i] = v;
  if (ids) ids[i] = __ldg(idsS + i);
}

// Step metrics: density (as fld_computeDensity) at the current positions with the step's
// table, neighbour counts, kinetic energy.
template <bool BATCH>
__global__ void __launch_bounds__(128) k_fluid_metrics(GridK g, FluidK p, const float4* __restrict__ pos,
                                                       const float4* __restrict__ vel, const uint2* __restrict__ table,
                                                       uint32_t n, double* __restrict__ acc, uint32_t* __restrict__ hist) {
  pdl_enter();
  // acc: [0] sum |rho/rho0 - 1|, [1] kinetic energy, [2] neighbour count, [3] sum max(rho/rho0 - 1, 0);
  // hist[64] = max error bits.
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  double err = 0.0, ke = 0.0, nb = 0.0, comp = 0.0;
  float mx = 0.0f;
  if (i < n) {
    scene_of<BATCH>(i, g, p);
    const Sph k(g);
    const float4 xi = ld4(pos + i);
    float rho = 0.0f;
    uint32_t cnt = 0;
    for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) {
      const float4 xj = ld4(pos + j);
      const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
      const float r2 = vx * vx + vy * vy + vz * vz;
      if (r2 < k.h2) {
        rho += k.w(r2);
        if (j != i) ++cnt;
      }
    });
    const float cdev = rho / p.rho0 - 1.0f;
    const float e = fabsf(cdev);
    err = e;
    comp = fmaxf(cdev, 0.0f);
    mx = e;
    const float4 v = ld4(vel + i);
    ke = 0.5 * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
    nb = cnt;
    atomicAdd(hist + min(cnt, 63u), 1u);
  }
  // Warp reduction, one atomic per warp.
  for (int o = 16; o > 0; o >>= 1) {
    err += __shfl_down_sync(0xffffffffu, err, o);
    ke += __shfl_down_sync(0xffffffffu, ke, o);
    nb += __shfl_down_sync(0xffffffffu, nb, o);
    comp += __shfl_down_sync(0xffffffffu, comp, o);
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc + 0, err);
    atomicAdd(acc + 1, ke);
    atomicAdd(acc + 2, nb);
    atomicAdd(acc + 3, comp);
    atomicMax(hist + 64, __float_as_uint(mx));  // mx >= 0: uint order == float order
  }
}

// Pair-list statistics: overflowed particles and the longest list (diagnostics).
__global__ void k_pair_list_stats(const uint32_t* __restrict__ count, uint32_t n, uint32_t* __restrict__ out) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = __ldg(count + i);
  if (c == kListOverflow) atomicAdd(out, 1u);
  else atomicMax(out + 1, c);
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}

static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

// From this many particles the full sweeps record hits through a bit mask per eight
// candidates (measured: 4 % faster at 4.2M, 3 % slower at 131k).
constexpr uint32_t kMaskFilterParticles = 1u << 20;
// Lanes per particle of the full sweeps (density / lambda and vorticity): a group of lanes
// (k_fluid_lambda_group, k_fluid_vorticity_group) while the particles are too few to keep
// the GPU busy one lane each, 0 for the lane-per-particle kernels.  Measured PBF steps (dam
// break, 3 iterations), us per step for one lane / 2 / 4 / 8 / 16 lanes: 16k 182 / 148 / 125 /
// 119 / 145; 32k 200 / 172 / 161 / 169 / 220; 65k 252 / 254 / 256 / 273 / 385; 131k 342 /
// 406 / 420 / 467 / 697.
static inline int sweep_group_lanes(uint32_t n) {
  if (n <= 24576u) return 8;
  if (n <= 49152u) return 4;
  return 0;
}
template <class F>
static inline void dispatch_group(int lw, F&& f) {
  if (lw == 8) f(std::integral_constant<int, 8>{});
  else f(std::integral_constant<int, 4>{});
}

int fluid_presort(const GridK& g, const FluidK& p, float4* pos, float4* vel, uint32_t n, float4* pred,
                  uint32_t* keys, const SortPlan& plan, uint32_t* hist0, bool clampOut, Launcher& L, const ZeroJob& zero,
                  const HostIO& io) {
  L.begin("fld_predict");
  if (p.bt.scenes)
    launch(L, k_fluid_predict<true>, dim3(plan.tiles), dim3(kKeyThreads), g, p, pos, vel, n, pred, keys, plan.bits[0], hist0,
                                                                     clampOut ? 1 : 0, zero, io);
  else
    launch(L, k_fluid_predict<false>, dim3(plan.tiles), dim3(kKeyThreads), g, p, pos, vel, n, pred, keys, plan.bits[0],
                                                                      hist0, clampOut ? 1 : 0, zero, io);
  L.end("fld_predict");
  return check("k_fluid_predict");
}

int fluid_iteration(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, const uint2* table, uint32_t n,
                    float* lambda, float* density, bool last, const float4* posS, float4* velS, const PairList& pl,
                    Launcher& L, float* lamTot, int totMode, float4* packed, const float* omega) {
  const int rc = fluid_lambda_sweep(g, p, predIn, table, n, lambda, density, pl, L, lamTot, totMode, packed, omega);
  if (rc) return rc;
  return fluid_deltap(g, p, predIn, predOut, lambda, table, n, last, posS, velS, pl, nullptr, L, packed);
}

// The brick-tiled sweep runs for one scene of enough particles whose grid has at least 6
// cells on every axis (so that the halo cells of a brick are distinct cells).
static bool brick_sweep_applies(const GridK& g, const FluidK& p, uint32_t n) {
  return p.tiles && !p.bt.scenes && p.sortedKeys && n > 49152u && g.R[0] >= kHalo && g.R[1] >= kHalo &&
         g.R[2] >= kHalo;
}

int fluid_lambda_sweep(const GridK& g, const FluidK& p, const float4* predIn, const uint2* table, uint32_t n,
                       float* lambda, float* density, const PairList& pl, Launcher& L, float* lamTot, int totMode,
                       float4* packed, const float* omega) {
  L.begin("fld_lambda");
  const dim3 nb(blocks(n, kSweepThreads)), nt(kSweepThreads);
  const bool mask = n >= kMaskFilterParticles;
  if (brick_sweep_applies(g, p, n)) {
    const int nbx = (g.R[0] + kBrick - 1) / kBrick, nby = (g.R[1] + kBrick - 1) / kBrick,
              nbz = (g.R[2] + kBrick - 1) / kBrick;
    const dim3 bg((unsigned)(nbx * nby * nbz + 1)), bt(kBrickThreads);
    if (mask)
      launch_smem(L, k_fluid_lambda_brick<true>, bg, bt, kBrickSmem, g, p, predIn, table, p.sortedKeys, n, nbx, nby, nbz,
                  lambda, density, pl, lamTot, totMode, packed, omega);
    else
      launch_smem(L, k_fluid_lambda_brick<false>, bg, bt, kBrickSmem, g, p, predIn, table, p.sortedKeys, n, nbx, nby,
                  nbz, lambda, density, pl, lamTot, totMode, packed, omega);
  } else if (const int lw = sweep_group_lanes(n)) {
    dispatch_group(lw, [&](auto LW) {
      const dim3 gb(blocks(n, 128 / LW)), gt(128);
      if (p.bt.scenes)
        launch(L, k_fluid_lambda_group<true, LW>, gb, gt, g, p, predIn, table, n, lambda, density, pl, lamTot, totMode,
               packed, omega);
      else
        launch(L, k_fluid_lambda_group<false, LW>, gb, gt, g, p, predIn, table, n, lambda, density, pl, lamTot,
               totMode, packed, omega);
    });
  } else if (p.bt.scenes && mask)
    launch(L, k_fluid_lambda<true, true>, nb, nt, g, p, predIn, table, n, lambda, density, pl, lamTot, totMode, packed,
           omega);
  else if (p.bt.scenes)
    launch(L, k_fluid_lambda<true, false>, nb, nt, g, p, predIn, table, n, lambda, density, pl, lamTot, totMode, packed,
           omega);
  else if (mask)
    launch(L, k_fluid_lambda<false, true>, nb, nt, g, p, predIn, table, n, lambda, density, pl, lamTot, totMode, packed,
           omega);
  else
    launch(L, k_fluid_lambda<false, false>, nb, nt, g, p, predIn, table, n, lambda, density, pl, lamTot, totMode,
           packed, omega);
  L.end("fld_lambda");
  return check("k_fluid_lambda");
}

int fluid_deltap(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, const float* lambda,
                 const uint2* table, uint32_t n, bool last, const float4* posS, float4* velS, const PairList& pl,
                 const float4* res, Launcher& L, const float4* packed) {
  L.begin(last ? "fld_deltap_vel" : "fld_deltap");
  dispatch_fluid(p, [&](auto B, auto LN) {
    constexpr bool BATCH = decltype(B)::value;
    constexpr int LANES = decltype(LN)::value;
    const dim3 gb(blocks(n * LANES, 128)), gt(128);
    if (last && packed)
      launch(L, k_fluid_deltap<true, BATCH, LANES, true>, gb, gt, g, p, predIn, lambda, table, n, predOut, posS, velS,
             pl, res, packed);
    else if (last)
      launch(L, k_fluid_deltap<true, BATCH, LANES, false>, gb, gt, g, p, predIn, lambda, table, n, predOut, posS, velS,
             pl, res, packed);
    else if (packed)
      launch(L, k_fluid_deltap<false, BATCH, LANES, true>, gb, gt, g, p, predIn, lambda, table, n, predOut, posS,
             velS, pl, res, packed);
    else
      launch(L, k_fluid_deltap<false, BATCH, LANES, false>, gb, gt, g, p, predIn, lambda, table, n, predOut, posS,
             velS, pl, res, packed);
  });
  L.end(last ? "fld_deltap_vel" : "fld_deltap");
  return check("k_fluid_deltap");
}

int fluid_update_vel(const GridK& g, const FluidK& p, const float4* pred, const float4* posS, uint32_t n, float4* velS,
                     Launcher& L) {
  L.begin("fld_updateVel");
  if (p.bt.scenes)
    launch(L, k_fluid_update_vel<true>, dim3(blocks(n, 256)), dim3(256), g, p, pred, posS, n, velS);
  else
    launch(L, k_fluid_update_vel<false>, dim3(blocks(n, 256)), dim3(256), g, p, pred, posS, n, velS);
  L.end("fld_updateVel");
  return check("k_fluid_update_vel");
}

int fluid_vorticity(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, float4* vort,
                    const uint2* table, uint32_t n, const PairList& pl, float* errPartial, Launcher& L,
                    float4* packed) {
  L.begin("fld_vorticity");
  const uint32_t nb = blocks(n, kSweepThreads);
  auto go = [&](auto GUARD, auto BATCH, auto MASK) {
    launch(L, k_fluid_vorticity<decltype(GUARD)::value, decltype(BATCH)::value, decltype(MASK)::value>, dim3(nb),
           dim3(kSweepThreads), g, p, pred, velS, table, n, vort, pl, errPartial, packed);
  };
  using T = std::true_type;
  using F = std::false_type;
  const bool mask = n >= kMaskFilterParticles;
  const bool guard = errPartial != nullptr, batch = p.bt.scenes != nullptr;
  if (const int lw = sweep_group_lanes(n)) {
    dispatch_group(lw, [&](auto LW) {
      if (guard) {  // 64 particles per block: one errPartial entry each
        const dim3 gb(blocks(n, 64)), gt(kGuardGroupThreads<LW>);
        if (batch)
          launch(L, k_fluid_vorticity_group<true, true, LW>, gb, gt, g, p, pred, velS, table, n, vort, pl, errPartial,
                 packed);
        else
          launch(L, k_fluid_vorticity_group<true, false, LW>, gb, gt, g, p, pred, velS, table, n, vort, pl, errPartial,
                 packed);
      } else {
        const dim3 gb(blocks(n, 128 / LW)), gt(128);
        if (batch)
          launch(L, k_fluid_vorticity_group<false, true, LW>, gb, gt, g, p, pred, velS, table, n, vort, pl, errPartial,
                 packed);
        else
          launch(L, k_fluid_vorticity_group<false, false, LW>, gb, gt, g, p, pred, velS, table, n, vort, pl,
                 errPartial, packed);
      }
    });
  } else if (guard) {
    if (batch) mask ? go(T{}, T{}, T{}) : go(T{}, T{}, F{});
    else mask ? go(T{}, F{}, T{}) : go(T{}, F{}, F{});
  } else {
    if (batch) mask ? go(F{}, T{}, T{}) : go(F{}, T{}, F{});
    else mask ? go(F{}, F{}, T{}) : go(F{}, F{}, F{});
  }
  L.end("fld_vorticity");
  return check("k_fluid_vorticity");
}

int fluid_post(const GridK& g, const FluidK& p, const float4* pred, float4* velS, float4* vort, const uint2* table,
               uint32_t n, const uint32_t* idsS, float4* pos, float4* vel, uint32_t* ids, const PairList& pl,
               Launcher& L, bool vorticityDone, const HostIO& io, float4* packed) {
  if (p.vorticity) {
    int rc = RTP_OK;
    if (!vorticityDone) {
      rc = fluid_vorticity(g, p, pred, velS, vort, table, n, pl, nullptr, L, packed);
      if (rc) return rc;
    }
    L.begin("fld_confine");
    dispatch_fluid(p, [&](auto B, auto LN) {
      constexpr bool BATCH = decltype(B)::value;
      constexpr int LANES = decltype(LN)::value;
      const dim3 gb(blocks(n * LANES, 128)), gt(128);
      if (packed)
        launch(L, k_fluid_confine<BATCH, LANES, true>, gb, gt, g, p, pred, vort, table, n, velS, pl, packed);
      else
        launch(L, k_fluid_confine<BATCH, LANES, false>, gb, gt, g, p, pred, vort, table, n, velS, pl, packed);
    });
    L.end("fld_confine");
    rc = check("k_fluid_confine");
    if (rc) return rc;
    L.begin("fld_xsph_final");
    dispatch_fluid(p, [&](auto B, auto LN) {
      constexpr bool BATCH = decltype(B)::value;
      constexpr int LANES = decltype(LN)::value;
      launch(L, k_fluid_xsph_final<BATCH, LANES>, dim3(blocks(n * LANES, 128)), dim3(128), g, p, pred, velS, table, n, idsS,
                                                                                      pos, vel, ids, pl, io);
    });
    L.end("fld_xsph_final");
    return check("k_fluid_xsph_final");
  }
  L.begin("fld_final");
  launch(L, k_fluid_final, dim3(blocks(n, 256)), dim3(256), pred, velS, n, idsS, pos, vel, ids, io);
  L.end("fld_final");
  return check("k_fluid_final");
}

int fluid_metrics(const GridK& g, const FluidK& p, const float4* pos, const float4* vel, const uint2* table, uint32_t n,
                  double* acc, uint32_t* hist, Launcher& L) {
  if (n == 0) return RTP_OK;
  L.begin("fld_metrics");
  if (p.bt.scenes)
    launch(L, k_fluid_metrics<true>, dim3(blocks(n, 128)), dim3(128), g, p, pos, vel, table, n, acc, hist);
  else
    launch(L, k_fluid_metrics<false>, dim3(blocks(n, 128)), dim3(128), g, p, pos, vel, table, n, acc, hist);
  L.end("fld_metrics");
  return check("k_fluid_metrics");
}

}  // namespace rtp

namespace rtp {
int pair_list_stats(const PairList& pl, uint32_t n, uint32_t* out2, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_pair_list_stats, dim3((n + 255) / 256), dim3(256), pl.count, n, out2);
  return check("k_pair_list_stats");
}
}  // namespace rtp
