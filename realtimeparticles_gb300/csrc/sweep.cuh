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
constexpr uint32_t kSweepThreads = 128;    // block size of the two-phase sweeps
constexpr uint32_t kSmemK = 64;            // entries per thread in the shared-memory list
constexpr uint32_t kQuad = 4;              // lanes per particle in the list sweeps

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

// Visits every index of [b, e) with f(j), four loads in flight: g(j) loads what f needs for
// candidate j, f(j, loaded) consumes it.  Order of f calls = ascending j.
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
  for (; j < e; ++j) f(j, g(j));
}

// The 27 cells of the fluids neighbourhood (fluids.cl:101-123), wrapped modulo the
// resolution, as 9 (x, y) rows of three z cells each, visited x-major then y then z.
template <class R>
__device__ __forceinline__ void for_each_fluid_row(const GridK& g, const uint2* __restrict__ table, float4 xi, R&& row_fn) {
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  const int z0 = (cz - 1 + g.R[2]) % g.R[2], z1 = cz % g.R[2], z2 = (cz + 1) % g.R[2];
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    const int x = (cx + a - 1 + g.R[0]) % g.R[0];
#pragma unroll 1
    for (int b = 0; b < 3; ++b) {
      const int y = (cy + b - 1 + g.R[1]) % g.R[1];
      const uint32_t row = ((uint32_t)x * g.R[1] + (uint32_t)y) * g.R[2];
      uint32_t b0, e0, b1, e1, b2, e2;
      cell_range(table, row + (uint32_t)z0, g.cap, b0, e0);
      cell_range(table, row + (uint32_t)z1, g.cap, b1, e1);
      cell_range(table, row + (uint32_t)z2, g.cap, b2, e2);
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

// Shared-memory pair list of the calling thread: entry k at s[k * blockDim + tid].
struct SmemList {
  uint32_t* s;
  uint32_t n = 0;
  __device__ __forceinline__ explicit SmemList(uint32_t* base) : s(base + threadIdx.x) {}
  __device__ __forceinline__ void add(uint32_t j) {
    if (n < kSmemK) s[n * kSweepThreads] = j;
    ++n;
  }
  __device__ __forceinline__ bool overflow() const { return n > kSmemK; }
  __device__ __forceinline__ uint32_t at(uint32_t k) const { return s[k * kSweepThreads]; }
};

// Filter pass over the fluids neighbourhood: records, in visiting order, the candidates j
// with |xi - ld(j)|^2 < h2 (ld loads j's position, clamped where the sweep clamps).
template <class LD>
__device__ __forceinline__ void filter_fluid_neighbours(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                        float h2, LD&& ld, SmemList& sl) {
  auto test = [&](uint32_t j, float4 xj) {
    const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
    if (vx * vx + vy * vy + vz * vz < h2) sl.add(j);
  };
  for_each_fluid_row(g, table, xi, [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
    // Join touching ranges (visiting order unchanged), then scan each with 4 loads in flight.
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
        visit_range_x4(cb, ce, ld, test);
        cb = rb[r];
        ce = re[r];
      }
    }
    visit_range_x4(cb, ce, ld, test);
  });
}

// Copies a thread's shared-memory list to the device list (or marks overflow).
__device__ __forceinline__ void publish(const PairList& L, uint32_t i, const SmemList& sl) {
  if (sl.overflow() || sl.n > L.K) {
    L.count[i] = kListOverflow;
    return;
  }
  for (uint32_t k = 0; k < sl.n; ++k) L.idx[(size_t)k * L.stride + i] = sl.at(k);
  L.count[i] = sl.n;
}

// ---- quad-lane 27-cell sweeps ----------------------------------------------------------
// Lane q < 3 of a particle's quad owns the x-plane dx = q - 1 of the 27 cells (three rows);
// lane 3 has none.  Each lane keeps the pairs of its plane in a shared-memory segment of
// kSegK entries (entry k at s[k * blockDim + tid]).
constexpr uint32_t kSegK = 32;

struct QuadSeg {
  uint32_t* s;
  uint32_t n = 0;
  __device__ __forceinline__ explicit QuadSeg(uint32_t* base) : s(base + threadIdx.x) {}
  __device__ __forceinline__ void add(uint32_t j) {
    if (n < kSegK) s[n * blockDim.x] = j;
    ++n;
  }
  __device__ __forceinline__ bool overflow() const { return n > kSegK; }
  __device__ __forceinline__ uint32_t at(uint32_t k) const { return s[k * blockDim.x]; }
};

// The three rows of x-plane dx = q - 1 of the fluids neighbourhood.
template <class R>
__device__ __forceinline__ void for_each_fluid_plane_row(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                         uint32_t q, R&& row_fn) {
  if (q > 2) return;
  int cx, cy, cz;
  cell3(g, xi, cx, cy, cz);
  const int z0 = (cz - 1 + g.R[2]) % g.R[2], z1 = cz % g.R[2], z2 = (cz + 1) % g.R[2];
  const int x = (cx + (int)q - 1 + g.R[0]) % g.R[0];
#pragma unroll 1
  for (int b = 0; b < 3; ++b) {
    const int y = (cy + b - 1 + g.R[1]) % g.R[1];
    const uint32_t row = ((uint32_t)x * g.R[1] + (uint32_t)y) * g.R[2];
    uint32_t b0, e0, b1, e1, b2, e2;
    cell_range(table, row + (uint32_t)z0, g.cap, b0, e0);
    cell_range(table, row + (uint32_t)z1, g.cap, b1, e1);
    cell_range(table, row + (uint32_t)z2, g.cap, b2, e2);
    row_fn(b0, e0, b1, e1, b2, e2);
  }
}

// Every candidate of lane q's plane, in visiting order.
template <class F>
__device__ __forceinline__ void for_each_fluid_plane_neighbour(const GridK& g, const uint2* __restrict__ table,
                                                               float4 xi, uint32_t q, F&& f) {
  for_each_fluid_plane_row(g, table, xi, q,
                           [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
                             visit_ranges3(b0, e0, b1, e1, b2, e2, f);
                           });
}

// Filter pass of lane q's plane: candidates with |xi - ld(j)|^2 < h2 into the segment.
template <class LD>
__device__ __forceinline__ void filter_fluid_plane(const GridK& g, const uint2* __restrict__ table, float4 xi,
                                                   uint32_t q, float h2, LD&& ld, QuadSeg& seg) {
  auto test = [&](uint32_t j, float4 xj) {
    const float vx = xi.x - xj.x, vy = xi.y - xj.y, vz = xi.z - xj.z;
    if (vx * vx + vy * vy + vz * vz < h2) seg.add(j);
  };
  for_each_fluid_plane_row(g, table, xi, q,
                           [&](uint32_t b0, uint32_t e0, uint32_t b1, uint32_t e1, uint32_t b2, uint32_t e2) {
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
                                 visit_range_x4(cb, ce, ld, test);
                                 cb = rb[r];
                                 ce = re[r];
                               }
                             }
                             visit_range_x4(cb, ce, ld, test);
                           });
}

// Publishes the quad's segments as particle i's device list (planes in visiting order), or
// marks it overflowed.  All 32 lanes of the warp must call.
__device__ __forceinline__ void quad_publish(const PairList& L, uint32_t i, uint32_t q, bool active,
                                             const QuadSeg& seg) {
  const uint32_t lane = threadIdx.x & 31u, base = lane & ~3u;
  const uint32_t mine = active ? (seg.overflow() ? 0xFFFFu : seg.n) : 0u;
  const uint32_t n0 = __shfl_sync(0xffffffffu, mine, base), n1 = __shfl_sync(0xffffffffu, mine, base + 1),
                 n2 = __shfl_sync(0xffffffffu, mine, base + 2);
  if (!active) return;
  const uint32_t total = n0 + n1 + n2;
  if (total > L.K) {
    if (q == 0) L.count[i] = kListOverflow;
    return;
  }
  const uint32_t off = q == 0 ? 0u : (q == 1 ? n0 : (q == 2 ? n0 + n1 : total));
  for (uint32_t k = 0; k < seg.n && q < 3; ++k) L.idx[(size_t)(off + k) * L.stride + i] = seg.at(k);
  if (q == 0) L.count[i] = total;
}

// Sum of v over the kQuad lanes of a particle (all 32 lanes of the warp must call).
__device__ __forceinline__ float quad_sum(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}

}  // namespace rtp
