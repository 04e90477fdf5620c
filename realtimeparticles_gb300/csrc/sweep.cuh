// sweep.cuh - neighbour-sweep building blocks shared by the fluids and clouds kernels.
//
// The reference visits, for particle i, the 27 cells around i's cell and every particle of
// each cell's (capped) range in ascending order.  Two kernels of a step often see the same
// positions (lambda and deltap of one Jacobi iteration; vorticity, confinement and XSPH after
// the solver), so the first of them records the pairs inside the effect radius, in visiting
// order, and the others walk that list instead of the 27 cells.
#pragma once

#include "rtp_common.cuh"

namespace rtp {

// Pairs within the effect radius recorded by one sweep.  idx is [K][stride] so that the
// lanes of a warp read one row coalesced; a particle with more than K pairs is marked
// kListOverflow and searches its 27 cells again.  The top 4 bits of an entry may carry a
// periodic-image code (clouds), so particle indices must stay below 2^28.
struct PairList {
  uint32_t* idx;
  uint32_t* count;
  uint32_t stride;
  uint32_t K;
};
constexpr uint32_t kListOverflow = 0xFFFFFFFFu;
constexpr uint32_t kPairListK = 64;        // entries per particle in the device list
constexpr uint32_t kSweepThreads = 64;     // block size of the two-phase sweeps (one wave at 131k)
constexpr uint32_t kQuad = 4;              // default lanes per particle in the list sweeps

// The filter passes' pair test |xi - xj|^2 < h2 with the rounding spelled out (two fused
// multiply-adds), so that every filter pass (one lane, lane group, brick-tiled) accepts the
// same pairs whatever code the compiler generates around it.
__device__ __forceinline__ bool within_radius(float4 xi, float4 xj, float h2) {
  const float vx = __fsub_rn(xi.x, xj.x), vy = __fsub_rn(xi.y, xj.y), vz = __fsub_rn(xi.z, xj.z);
  return __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, __fmul_rn(vx, vx))) < h2;
}

// Visits [b0,e0) [b1,e1) [b2,e2) in that order, joining ranges that touch so that the
// usual case (three consecutive non-empty cells of one z column) is a single loop.
template <class F>
__device__ __forceinline__ void visit_ranges3(uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2,
                                              uint32_t e2, F&& f) {
  uint32_t cb = b0, ce = e0;
  const uint32_t rb[2] = {b1, b2}, re[2] = {e1, e2};
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    if (rb[r] == re[r]) continue;
    if (cb == ce) {
      cb = rb[r];
      ce = re[r];
    } else if (ce == rb[r]) {
      ce = re[r];
    } else {
      for (uint32_t j = cb; j < ce; ++j) f(j);
      cb = rb[r];
      ce = re[r];
    }
  }
  for (uint32_t j = cb; j < ce; ++j) f(j);
}

// The last 1..N indices [j, e) of a range in one round: N loads in flight, the indices past
// e - 1 loading e - 1 again (a line already being fetched) and not visited.
template <int N, class G, class F>
__device__ __forceinline__ void visit_tail(uint32_t j, uint32_t e, G&& g, F&& f) {
  decltype(g(j)) a[N];
#pragma unroll
  for (int u = 0; u < N; ++u) a[u] = g(min(j + u, e - 1u));
#pragma unroll
  for (int u = 0; u < N; ++u)
    if (j + u < e) f(j + u, a[u]);
}

// Visits every index of [b, e) with f(j), four loads in flight: g(j) loads what f needs for
// candidate j, f(j, loaded) consumes it.  Order of f calls = ascending j.  The last 1-3
// indices take one round, not one round each.
template <class G, class F>
__device__ __forceinline__ void visit_range_x4(uint32_t b, uint32_t e, G&& g, F&& f) {
  uint32_t j = b;
  for (; j + 4 <= e; j += 4) {
    const auto a0 = g(j), a1 = g(j + 1), a2 = g(j + 2), a3 = g(j + 3);
    f(j, a0);
    f(j + 1, a1);
    f(j + 2, a2);
    f(j + 3, a3);
  }
  if (j < e) visit_tail<3>(j, e, g, f);
}

// As visit_range_x4 with eight loads in flight first (the distance-only filter passes, whose
// per-candidate work is small enough to keep eight positions in registers).
template <class G, class F>
__device__ __forceinline__ void visit_range_x8(uint32_t b, uint32_t e, G&& g, F&& f) {
  uint32_t j = b;
  for (; j + 8 <= e; j += 8) {
    const auto a0 = g(j), a1 = g(j + 1), a2 = g(j + 2), a3 = g(j + 3);
    const auto a4 = g(j + 4), a5 = g(j + 5), a6 = g(j + 6), a7 = g(j + 7);
    f(j, a0);
    f(j + 1, a1);
    f(j + 2, a2);
    f(j + 3, a3);
    f(j + 4, a4);
    f(j + 5, a5);
    f(j + 6, a6);
    f(j + 7, a7);
  }
  visit_range_x4(j, e, g, f);
}

// Filter of [b, e): hit(loaded) tests a candidate, add(j) records it, in ascending j.  Eight
// candidates are loaded and tested at a time into a bit mask, then the hits are recorded from
// the mask, so a warp pays the recording once per hit of its busiest lane rather than once per
// candidate slot.
template <class G, class H, class A>
__device__ __forceinline__ void filter_range_x8(uint32_t b, uint32_t e, G&& g, H&& hit, A&& add) {
  uint32_t j = b;
  for (; j + 8 <= e; j += 8) {
    const auto a0 = g(j), a1 = g(j + 1), a2 = g(j + 2), a3 = g(j + 3);
    const auto a4 = g(j + 4), a5 = g(j + 5), a6 = g(j + 6), a7 = g(j + 7);
    uint32_t m = (hit(a0) ? 1u : 0u) | (hit(a1) ? 2u : 0u) | (hit(a2) ? 4u : 0u) | (hit(a3) ? 8u : 0u) |
                 (hit(a4) ? 16u : 0u) | (hit(a5) ? 32u : 0u) | (hit(a6) ? 64u : 0u) | (hit(a7) ? 128u : 0u);
    while (m) {
      add(j + (uint32_t)(__ffs(m) - 1));
      m &= m - 1u;
    }
  }
  if (j + 4 <= e) {
    const auto a0 = g(j), a1 = g(j + 1), a2 = g(j + 2), a3 = g(j + 3);
    uint32_t m = (hit(a0) ? 1u : 0u) | (hit(a1) ? 2u : 0u) | (hit(a2) ? 4u : 0u) | (hit(a3) ? 8u : 0u);
    while (m) {
      add(j + (uint32_t)(__ffs(m) - 1));
      m &= m - 1u;
    }
    j += 4;
  }
  if (j < e) {  // 1-3 left: one round (past the end re-load e - 1 and do not count)
    const uint32_t last = e - 1u;
    const auto a0 = g(j), a1 = g(min(j + 1u, last)), a2 = g(min(j + 2u, last));
    uint32_t m = (hit(a0) ? 1u : 0u) | (j + 1u < e && hit(a1) ? 2u : 0u) | (j + 2u < e && hit(a2) ? 4u : 0u);
    while (m) {
      add(j + (uint32_t)(__ffs(m) - 1));
      m &= m - 1u;
    }
  }
}

// Walks list entries begin, begin + step, ... < end in order, four at a time: the four
// indices idx(kk) are loaded, then g(j) loads each pair's operands, then f(j, loaded)
// consumes them, so a lane keeps several dependent load chains in flight.
template <class IDX, class G, class F>
__device__ __forceinline__ void visit_list_x4(uint32_t begin, uint32_t end, uint32_t step, IDX&& idx, G&& g, F&& f) {
  uint32_t kk = begin;
  for (; kk + 3 * step < end; kk += 4 * step) {
    const uint32_t j0 = idx(kk), j1 = idx(kk + step), j2 = idx(kk + 2 * step), j3 = idx(kk + 3 * step);
    const auto a0 = g(j0), a1 = g(j1), a2 = g(j2), a3 = g(j3);
    f(j0, a0);
    f(j1, a1);
    f(j2, a2);
    f(j3, a3);
  }
  if (kk < end) {  // 1-3 entries left: one round of index loads, one of operand loads
    const uint32_t last = kk + (end - 1u - kk) / step * step;
    const uint32_t j0 = idx(kk), j1 = idx(min(kk + step, last)), j2 = idx(min(kk + 2 * step, last));
    const auto a0 = g(j0), a1 = g(j1), a2 = g(j2);
    f(j0, a0);
    if (kk + step < end) f(j1, a1);
    if (kk + 2 * step < end) f(j2, a2);
  }
}

// c + d for d in {-1, 0, 1} wrapped into [0, R): the same cell as (c + d + R) % R for the
// c in [0, R] that cell3 can return (c = R is the aliased +W wall).
__device__ __forceinline__ int wrap_cell(int c, int d, int R) {
  int v = c + d;
  if (v < 0) v += R;
  else if (v >= R) v -= R;
  return v;
}

// The 27 cells of the fluids neighbourhood (fluids.cl:101-123), wrapped modulo the
// resolution, as 9 (x, y) rows of three z cells each, visited x-major then y then z.
template <class R>
__device__ __forceinline__ void for_each_fluid_row(const GridK& g, const uint2* __restrict__ table, float4 xi, R&& row_fn) {
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  const uint32_t z0 = (uint32_t)wrap_cell(cz, -1, g.R[2]), z1 = (uint32_t)wrap_cell(cz, 0, g.R[2]),
                 z2 = (uint32_t)wrap_cell(cz, 1, g.R[2]);
#pragma unroll 1
  for (int a = -1; a <= 1; ++a) {
    const int x = wrap_cell(cx, a, g.R[0]);
#pragma unroll 1
    for (int b = -1; b <= 1; ++b) {
      const int y = wrap_cell(cy, b, g.R[1]);
      const uint32_t row = g.base + ((uint32_t)x * g.R[1] + (uint32_t)y) * g.R[2];
      uint32_t b0, e0, b1, e1, b2, e2;
      cell_range(table, row + z0, g.cap, b0, e0);
      cell_range(table, row + z1, g.cap, b1, e1);
      cell_range(table, row + z2, g.cap, b2, e2);
      row_fn(b0, e0, b1, e1, b2, e2);
    }
  }
}

template <class F>
__device__ __forceinline__ void for_each_fluid_neighbour(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                         F&& f) {
  for_each_fluid_row(g, table, xi, [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
    visit_ranges3(b0, e0, b1, e1, b2, e2, f);
  });
}

// Filter pass over the fluids neighbourhood: calls add(j), in visiting order, for each
// candidate with |xi - ld(j)|^2 < h2 (ld loads j's position).  MASK records the hits of
// each eight candidates from a bit mask (faster with millions of particles, slower at 131k
// where fewer warps hide the extra loop).
template <bool MASK = false, class LD, class ADD>
__device__ __forceinline__ void filter_fluid_neighbours_to(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                           float h2, LD&& ld, ADD&& add) {
  auto hit = [&](float4 xj) { return within_radius(xi, xj, h2); };
  auto test = [&](uint32_t j, float4 xj) {
    if (hit(xj)) add(j);
  };
  auto range = [&](uint32_t b, uint32_t e) {
    if constexpr (MASK)
      filter_range_x8(b, e, ld, hit, add);
    else
      visit_range_x8(b, e, ld, test);
  };
  for_each_fluid_row(g, table, xi, [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
    uint32_t cb = b0, ce = e0;
    const uint32_t rb[2] = {b1, b2}, re[2] = {e1, e2};
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (rb[r] == re[r]) continue;
      if (cb == ce) {
        cb = rb[r];
        ce = re[r];
      } else if (ce == rb[r]) {
        ce = re[r];
      } else {
        range(cb, ce);
        cb = rb[r];
        ce = re[r];
      }
    }
    range(cb, ce);
  });
}

// The filter pass with a group of LW lanes (LW = 4 ... 32, aligned in the warp) on one
// particle, the warp's 32 / LW groups in lockstep: every group walks the same 9 rows and, per
// row, as many chunks as the group with the most candidates there needs, so all 32 lanes
// stay converged (a group whose own candidates are done tests nothing).  Within a row lane q
// of a group tests candidates q, q + LW, ... of the row's three z cells taken in order, four
// chunks of LW at a time, and a warp ballot compacts the group's hits into lst[0..K)
// (stride apart) in visiting order, the list the one-lane pass writes.  Returns the number
// of pairs within h2 on every lane of the group.  The whole warp must call; a group with
// live = false (past the last particle) records nothing.  For particle counts too small to
// keep the GPU busy with one lane each.
template <int LW, class LD>
__device__ __forceinline__ uint32_t filter_fluid_group(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                       bool live, float h2, LD&& ld, uint32_t* lst, uint32_t stride,
                                                       uint32_t K) {
  static_assert(LW >= 2 && LW <= 32 && (LW & (LW - 1)) == 0, "power-of-two group");
  const uint32_t lane = threadIdx.x & 31u, q = lane & (LW - 1u), first = lane - q;
  const uint32_t gbits = LW == 32 ? 0xffffffffu : (1u << LW) - 1u;
  const uint32_t below = (1u << q) - 1u;
  uint32_t cnt = 0;
  for_each_fluid_row(g, table, xi, [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
    const uint32_t n0 = e0 - b0, n01 = n0 + (e1 - b1), tot = live ? n01 + (e2 - b2) : 0u;
    const uint32_t most = __reduce_max_sync(0xffffffffu, tot);
    for (uint32_t c0 = 0; c0 < most; c0 += 4u * LW) {
      uint32_t j[4];
      float4 x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t c = c0 + u * LW + q;
        j[u] = c < n0 ? b0 + c : (c < n01 ? b1 + (c - n0) : b2 + (c - n01));
        if (c < tot) x[u] = ld(j[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        bool hit = false;
        if (c0 + u * LW + q < tot) hit = within_radius(xi, x[u], h2);
        const uint32_t m = (__ballot_sync(0xffffffffu, hit) >> first) & gbits;
        if (hit) {
          const uint32_t at = cnt + __popc(m & below);
          if (at < K) lst[(size_t)at * stride] = j[u];
        }
        cnt += __popc(m);
      }
    }
  });
  __syncwarp();  // the entries other lanes of the group wrote are visible to it
  return cnt;
}

// The list walk of a lane group in lockstep with the warp's other groups: lane q visits
// entries q, q + LW, ... of a list of cnt entries (idx(kk) loads entry kk), four at a time,
// for as many rounds as the warp's longest list needs, so the lanes stay converged and every
// round has four loads in flight.  A slot past the lane's own list loads particle `self`
// (any valid index) and is not visited.  The whole warp must call; cnt = 0 visits nothing.
template <int LW, class IDX, class G, class F>
__device__ __forceinline__ void walk_list_group(uint32_t cnt, uint32_t self, IDX&& idx, G&& ld, F&& f) {
  const uint32_t q = threadIdx.x & (LW - 1u);
  const uint32_t most = __reduce_max_sync(0xffffffffu, cnt);
  for (uint32_t k0 = q; k0 < most; k0 += 4u * LW) {
    uint32_t j[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) j[u] = k0 + u * LW < cnt ? idx(k0 + u * LW) : self;
    const auto a0 = ld(j[0]), a1 = ld(j[1]), a2 = ld(j[2]), a3 = ld(j[3]);
    if (k0 < cnt) f(j[0], a0);
    if (k0 + LW < cnt) f(j[1], a1);
    if (k0 + 2 * LW < cnt) f(j[2], a2);
    if (k0 + 3 * LW < cnt) f(j[3], a3);
  }
}

// Visits the pairs recorded for particle i, one in LANES per lane (lane q takes entries
// q, q + LANES, ...); an overflowed particle searches its 27 cells on lane 0.
template <int LANES = kQuad, class G, class F>
__device__ __forceinline__ void quad_pairs(const GridK& g, const uint2* __restrict__ table, const PairList& L,
                                           uint32_t i, uint32_t q, float4 xi, G&& ld, F&& f) {
  const uint32_t c = __ldg(L.count + i);
  if (c != kListOverflow) {
    const uint32_t* base = L.idx + i;
    visit_list_x4(q, c, LANES, [&](uint32_t kk) { return __ldg(base + (size_t)kk * L.stride); }, ld, f);
  } else if (q == 0) {
    for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { f(j, ld(j)); });
  }
}

// quad_pairs called by every lane of the warp (a lane past the last particle with active =
// false visits nothing).  SYNC walks the warp's particles in lockstep (walk_list_group):
// measured 0.5 % faster on the 131k dam break and 1.8 % at 16k, but 1.5 % slower for 48
// batched scenes, whose larger kernels spill under it; !SYNC is quad_pairs on the active lanes.
template <int LANES, bool SYNC, class G, class F>
__device__ __forceinline__ void quad_pairs_sync(const GridK& g, const uint2* __restrict__ table, const PairList& L,
                                                uint32_t i, uint32_t q, bool active, float4 xi, G&& ld, F&& f) {
  if constexpr (SYNC) {
    const uint32_t c = active ? __ldg(L.count + i) : 0u;
    const uint32_t* base = L.idx + i;
    walk_list_group<LANES>(c != kListOverflow ? c : 0u, i,
                           [&](uint32_t kk) { return __ldg(base + (size_t)kk * L.stride); }, ld, f);
    if (c == kListOverflow && q == 0) for_each_fluid_neighbour(g, table, xi, [&](uint32_t j) { f(j, ld(j)); });
  } else if (active) {
    quad_pairs<LANES>(g, table, L, i, q, xi, ld, f);
  }
}

// Sum of v over the LANES lanes of a particle (all 32 lanes of the warp must call).
template <int LANES = kQuad>
__device__ __forceinline__ float quad_sum(float v) {
#pragma unroll
  for (int o = 1; o < LANES; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace rtp
