// boids.cu - 3D boids step (GB300, sm_103a).
//
// Replaces kernels/boids.cl driven by Boids::update (physics/ocl/Boids.cpp:323-377):
//   k_boids_keys          fillCellIDs(pos) + sort-tile histogram
//   sort passes           RadixSort::sort of {pos, vel} (+ ids); acc is recomputed each step
//   cell table            start/end (cap 3000, Boids.cpp:78)
//   k_boids_rules_update  bd_applyBoidsRulesWithGrid3D (2D models: ...Grid2D) + bd_addTargetRule when the
//                         target is on + bd_updateVel + the boundary
//                         condition (bd_updatePosAndApplyPeriodicBC / ...WallBC), reading
//                         the sorted copies and writing the canonical pos/vel buffers.
#include "boids.cuh"

namespace rtp {

// With io.inPos / io.inVel the state comes from host memory and is mirrored into pos / vel.
__global__ void __launch_bounds__(kKeyThreads) k_boids_keys(GridK g, float4* __restrict__ pos,
                                                             float4* __restrict__ vel, uint32_t n,
                                                             uint32_t* __restrict__ keys, int bits0,
                                                             uint32_t* __restrict__ hist0, ZeroJob zero,
                                                             float4* __restrict__ track, HostIO io) {
  pdl_enter();
  __shared__ uint32_t s_hist[kMaxBins];
  zero_job(zero);
  if (track && blockIdx.x == 0 && threadIdx.x == 0) {
    uint32_t* step = reinterpret_cast<uint32_t*>(track);
    *step = *step + 1u;  // this step's slot of the target track
  }
  TileHistogram th;
  th.init(s_hist, bits0);
  const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll 2
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t i = base + k * kKeyThreads + threadIdx.x;
    if (i < n) {
      float4 x;
      if (io.inPos) {
        x = io.inPos[i];
        pos[i] = x;
      } else {
        x = ld4(pos + i);
      }
      if (io.inVel) vel[i] = io.inVel[i];
      const uint32_t key = cell_key(g, x);
      keys[i] = key;
      th.add(key);
    }
  }
  th.store(hist0);
}

// A neighbour's position and velocity, loaded ahead of use.
struct PosVel {
  float4 x, v;
};

__device__ __forceinline__ float4 fnorm(float4 a) {
  const float d = dot4(a, a);
  if (d == 0.0f) return a;
  return a * rsqrtf(d);
}

template <bool PERIODIC, bool DIM2>
__global__ void __launch_bounds__(128) k_boids_rules_update(GridK g, BoidsK p, const float4* __restrict__ posS,
                                                            const float4* __restrict__ velS,
                                                            const uint2* __restrict__ table, uint32_t n,
                                                            const uint32_t* __restrict__ idsS, float4* __restrict__ pos,
                                                            float4* __restrict__ vel, float4* __restrict__ acc,
                                                            uint32_t* __restrict__ ids, TargetK tk, HostIO io) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = ld4(posS + i);
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  int count = 0;
  float4 sp = f4(0.f, 0.f, 0.f, 0.f), sv = sp, sr = sp;
  auto rule = [&](uint32_t j0, uint32_t j1) {
    for (uint32_t j = j0; j < j1; ++j) {
      const float4 xj = ld4(posS + j);
      const float4 v = xi - xj;
      const float sq = dot4(v, v);
      if (sq < g.boidsR2 && sq > kFloatEps) {
        sp = sp + xj;
        sv = sv + fnorm(ld4(velS + j));
        sr = sr + v * (1.0f / sq);
        ++count;
      }
    }
  };
  if (DIM2) {
    // bd_applyBoidsRulesWithGrid2D (boids.cl:167-212): the 9 cells (0, dy, dz), every index
    // checked against GRID_RES_X, cells taken in the x = GRID_RES_X / 2 plane.
    const int R = g.R[0];
    if (cx >= 0 && cx < R) {
      for (int dy = -1; dy <= 1; ++dy) {
        const int ny = cy + dy;
        if (ny < 0 || ny >= R) continue;
        for (int dz = -1; dz <= 1; ++dz) {
          const int nz = cz + dz;
          if (nz < 0 || nz >= R) continue;
          uint32_t j0, j1;
          cell_range(table, (uint32_t)((R / 2 * R + ny) * g.R[1] + nz), g.cap, j0, j1);
          rule(j0, j1);
        }
      }
    }
  } else {
    // bd_applyBoidsRulesWithGrid3D (boids.cl:78-113): 27 cells, no wrap.  Two phases: the
    // row ranges (a row's z cells joined where contiguous, four position loads in flight)
    // are filtered into a per-thread list of the boids inside the radius, then the rules are
    // summed over that list in the same order, so the lanes of a warp do not all pay for the
    // neighbour body whenever one of them has a neighbour.  More than kBoidHits neighbours:
    // the sums run inline over the rows instead.
    constexpr int kBoidHits = 32;
    uint32_t hits[kBoidHits];
    int nh = 0;
    bool inline_sums = false;
    auto add = [&](uint32_t j, float4 xj) {
      const float4 v = xi - xj;
      const float sq = dot4(v, v);
      if (sq < g.boidsR2 && sq > kFloatEps) {
        sp = sp + xj;
        sv = sv + fnorm(ld4(velS + j));
        sr = sr + v * (1.0f / sq);
        ++count;
      }
    };
    auto filt = [&](uint32_t j, float4 xj) {
      const float4 v = xi - xj;
      const float sq = dot4(v, v);
      if (sq < g.boidsR2 && sq > kFloatEps) {
        if (nh < kBoidHits) hits[nh] = j;
        ++nh;
      }
    };
    auto ldp = [&](uint32_t j) { return ld4(posS + j); };
    auto rows = [&](auto&& test) {
#pragma unroll 1
      for (int dx = -1; dx <= 1; ++dx) {
        const int nx = cx + dx;
        if (nx < 0 || nx >= g.R[0]) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
          const int ny = cy + dy;
          if (ny < 0 || ny >= g.R[1]) continue;
          const uint32_t row = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2];
          uint32_t cb = 0, ce = 0;
#pragma unroll
          for (int dz = -1; dz <= 1; ++dz) {
            const int nz = cz + dz;
            if (nz < 0 || nz >= g.R[2]) continue;
            uint32_t j0, j1;
            cell_range(table, row + (uint32_t)nz, g.cap, j0, j1);
            if (j0 == j1) continue;
            if (cb == ce) {
              cb = j0;
              ce = j1;
            } else if (ce == j0) {
              ce = j1;
            } else {
              visit_range_x4(cb, ce, ldp, test);
              cb = j0;
              ce = j1;
            }
          }
          if (cb != ce) visit_range_x4(cb, ce, ldp, test);
        }
      }
    };
    rows(filt);
    inline_sums = nh > kBoidHits;
    if (inline_sums) {
      rows(add);
    } else {
      // The recorded boids, four at a time: their positions and velocities loaded together.
      visit_list_x4(
          0u, (uint32_t)nh, 1u, [&](uint32_t k) { return hits[k]; },
          [&](uint32_t j) { return PosVel{ld4(posS + j), ld4(velS + j)}; },
          [&](uint32_t, PosVel a) {
            const float4 v = xi - a.x;
            const float sq = dot4(v, v);
            sp = sp + a.x;
            sv = sv + fnorm(a.v);
            sr = sr + v * (1.0f / sq);
            ++count;
          });
    }
  }
  float4 a = f4(0.f, 0.f, 0.f, 0.f);
  if (count != 0) {
    float4 coh = sp * (1.0f / (float)count) - xi;
    coh = fnorm(coh) * p.velocityScale;
    const float4 ali = fnorm(sv) * p.velocityScale;
    const float4 sep = fnorm(sr) * p.velocityScale;
    a = ali * p.alignmentScale + sep * p.separationScale + coh * p.cohesionScale;
  }
  if (tk.track) {
    // bd_addTargetRule (boids.cl:226-241): inside the radius, adds sign x vec x
    // clamp(1.3 / |vec|, 0, 1.4 x MAX_STEERING) with vec = target - x (lengths over four lanes).
    const uint32_t s = min(*reinterpret_cast<const uint32_t*>(tk.track), tk.cap - 1u);
    const float4 vec = ld4(tk.track + 1 + s) - xi;
    const float dist = sqrtf(dot4(vec, vec));
    if (dist < tk.radius) a = a + (vec * tk.sign) * fminf(fmaxf(1.3f / dist, 0.0f), 0.7f);
  }
  acc[i] = a;
  // bd_updateVel (boids.cl:246-259).
  const float4 nv = ld4(velS + i) + a * p.dt;
  const float norm = fminf(fmaxf(sqrtf(dot4(nv, nv)), 0.2f * p.maxVelocity), p.maxVelocity);
  float4 v = fnorm(nv) * norm;
  const float4 np = xi + v * p.dt;
  const float4 lo = f4(-g.W[0], -g.W[1], -g.W[2], 0.0f), hi = f4(g.W[0], g.W[1], g.W[2], 0.0f);
  float4 cp = clamp4(np, lo, hi);
  if (PERIODIC) {
    // bd_updatePosAndApplyPeriodicBC (boids.cl:289-315).
    if (!(cp.x == np.x)) cp.x *= -1.0f;
    if (!(cp.y == np.y)) cp.y *= -1.0f;
    if (!(cp.z == np.z)) cp.z *= -1.0f;
  } else {
    // bd_updatePosAndApplyWallBC (boids.cl:264-284).
    if (!(cp.x == np.x && cp.y == np.y && cp.z == np.z)) v = v * -0.5f;
  }
  pos[i] = cp;
  vel[i] = v;
  if (io.outPos) io.outPos[i] = cp;
  if (io.outVel) io.outVel[i] = v;
  if (ids) ids[i] = __ldg(idsS + i);
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}

int boids_presort(const GridK& g, float4* pos, float4* vel, uint32_t n, uint32_t* keys, const SortPlan& plan,
                  uint32_t* hist0, Launcher& L, const ZeroJob& zero, const TargetK& tk, const HostIO& io) {
  L.begin("bd_keys");
  launch(L, k_boids_keys, dim3(plan.tiles), dim3(kKeyThreads), g, pos, vel, n, keys, plan.bits[0], hist0, zero, tk.track,
         io);
  L.end("bd_keys");
  return check("k_boids_keys");
}

int boids_rules_update(const GridK& g, const BoidsK& p, bool periodic, bool dim2, const float4* posS,
                       const float4* velS, const uint2* table, uint32_t n, const uint32_t* idsS, float4* pos,
                       float4* vel, float4* acc, uint32_t* ids, Launcher& L, const TargetK& tk, const HostIO& io) {
  const uint32_t b = (n + 127) / 128;
  L.begin("bd_rules_update");
  if (periodic && dim2)
    launch(L, k_boids_rules_update<true, true>, dim3(b), dim3(128), g, p, posS, velS, table, n, idsS, pos, vel, acc, ids, tk, io);
  else if (periodic)
    launch(L, k_boids_rules_update<true, false>, dim3(b), dim3(128), g, p, posS, velS, table, n, idsS, pos, vel, acc, ids, tk, io);
  else if (dim2)
    launch(L, k_boids_rules_update<false, true>, dim3(b), dim3(128), g, p, posS, velS, table, n, idsS, pos, vel, acc, ids, tk, io);
  else
    launch(L, k_boids_rules_update<false, false>, dim3(b), dim3(128), g, p, posS, velS, table, n, idsS, pos, vel, acc,
           ids, tk, io);
  L.end("bd_rules_update");
  return check("k_boids_rules_update");
}

}  // namespace rtp
