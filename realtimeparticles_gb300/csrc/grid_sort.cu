// grid_sort.cu - uniform grid and stable radix sort (GB300, sm_103a).
//
// Replaces grid.cl (cell ids, start/end table) and RadixSort (physics/utils/RadixSort.cpp,
// kernels/radixSort.cl).  The reference sorts all maxNb keys in 4 passes of 8 bits with
// 512 work-items that each scan N/512 keys serially; here each pass is a tile-parallel
// reduce-then-scan LSD pass:
//   * digit histogram per 2048-key tile (pass 0: fused into the kernel that computes the
//     keys; pass p > 0: accumulated by pass p-1's scatter with warp-aggregated atomics),
//   * per-digit exclusive scan over tiles (k_sort_scan),
//   * stable rank inside the tile with __match_any_sync (warp w owns a contiguous chunk,
//     items processed in index order) and scatter; the last pass gathers the payloads
//     (pos, vel, ...) directly, so no permutation array round trip is needed.
// Only ceil(keyBits / 9) passes run: cell keys need 17 bits on a 40^3 grid.
#include <algorithm>
#include <cstring>

#include "rtp_internal.hpp"

namespace rtp {

SortPlan make_sort_plan(uint32_t n, uint32_t keyBits) {
  SortPlan p;
  p.n = n;
  p.keyBits = std::max<uint32_t>(1u, std::min<uint32_t>(keyBits, 32u));
  p.passes = (int)((p.keyBits + kMaxRadixBits - 1) / kMaxRadixBits);
  const int per = (int)((p.keyBits + p.passes - 1) / p.passes);
  int shift = 0;
  for (int i = 0; i < p.passes; ++i) {
    p.shift[i] = shift;
    p.bits[i] = std::min(per, (int)p.keyBits - shift);
    shift += p.bits[i];
  }
  p.tiles = (n + kSortTile - 1) / kSortTile;
  if (p.tiles == 0) p.tiles = 1;
  return p;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Up to this many tiles the scatter passes run 16-warp blocks (measured: faster over few
// tiles, slower at millions of keys where the larger shared footprint limits residency).
constexpr uint32_t kWidePassTiles = 256;

// Tile groups of the two-kernel digit scan (1 = the single-kernel scan).
static uint32_t scan_groups(uint32_t tiles) {
  return std::min<uint32_t>(kScanGroupsMax, (tiles + kScanTilesPerGroup - 1) / kScanTilesPerGroup);
}

size_t sort_scratch_bytes(const SortPlan& p) {
  const size_t nk = align256(sizeof(uint32_t) * (size_t)std::max<uint32_t>(p.n, 1));
  const size_t h = align256(sizeof(uint32_t) * (size_t)p.passes * p.tiles * kMaxBins);
  const size_t t = align256(sizeof(uint32_t) * (size_t)p.passes * kMaxBins);
  const size_t g = align256(sizeof(uint32_t) * (size_t)scan_groups(p.tiles) * kMaxBins);
  return 4 * nk + h + t + g;
}

void sort_scratch_carve(const SortPlan& p, void* base, SortScratch& s) {
  char* b = (char*)base;
  const size_t nk = align256(sizeof(uint32_t) * (size_t)std::max<uint32_t>(p.n, 1));
  s.keysA = (uint32_t*)b;
  b += nk;
  s.keysB = (uint32_t*)b;
  b += nk;
  s.idxA = (uint32_t*)b;
  b += nk;
  s.idxB = (uint32_t*)b;
  b += nk;
  s.hist = (uint32_t*)b;
  b += align256(sizeof(uint32_t) * (size_t)p.passes * p.tiles * kMaxBins);
  s.totals = (uint32_t*)b;
  b += align256(sizeof(uint32_t) * (size_t)p.passes * kMaxBins);
  s.scanPart = (uint32_t*)b;
}

// fillCellIDs (grid.cl:76-86).
__global__ void k_fill_cell_ids(GridK g, const float4* __restrict__ pos, uint32_t n, uint32_t* __restrict__ keys) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = cell_key(g, ld4(pos + i));
}

// Per-tile histogram of the digit at `shift` (pass 0 of externally supplied keys).
__global__ void __launch_bounds__(kKeyThreads) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                            int bits, uint32_t* __restrict__ hist) {
  pdl_enter();
  __shared__ uint32_t s_hist[kMaxBins];
  TileHistogram th;
  th.init(s_hist, bits);
  const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
  for (int k = 0; k < kKeyItems; ++k) {
    const uint32_t e = base + k * kKeyThreads + threadIdx.x;
    if (e < n) th.add(__ldg(keys + e) >> shift);
  }
  th.store(hist);
}

// In-place exclusive scan over tiles of each digit's column; totals[d] = column sum.
// Block = 8 warps, lane = digit within a group of 32, warp = contiguous range of tiles.
// Used when the tiles fit one block per digit group (up to kScanTilesPerGroup tiles).
__global__ void __launch_bounds__(256) k_sort_scan(uint32_t* __restrict__ hist, uint32_t tiles, int bins,
                                                   uint32_t* __restrict__ totals) {
  pdl_enter();
  __shared__ uint32_t s_part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  const uint32_t chunk = (tiles + 7) / 8;  // at most kScanChunk (tiles <= kScanTilesPerGroup)
  const uint32_t t0 = min(tiles, warp * chunk), t1 = min(tiles, t0 + chunk);
  // The warp's column slice, loaded once (all loads in flight) and kept for the rewrite.
  constexpr int kScanChunk = (int)kScanTilesPerGroup / 8;
  uint32_t v[kScanChunk];
  uint32_t sum = 0;
#pragma unroll
  for (int u = 0; u < kScanChunk; ++u) {
    v[u] = (d < bins && t0 + u < t1) ? hist[(size_t)(t0 + u) * kMaxBins + d] : 0u;
    sum += v[u];
  }
  s_part[warp][lane] = sum;
  __syncthreads();
  if (warp == 0) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      const uint32_t v = s_part[w][lane];
      s_part[w][lane] = run;
      run += v;
    }
    if (d < bins) totals[d] = run;
  }
  __syncthreads();
  if (d < bins) {
    uint32_t run = s_part[warp][lane];
#pragma unroll
    for (int u = 0; u < kScanChunk; ++u) {
      if (t0 + u < t1) hist[(size_t)(t0 + u) * kMaxBins + d] = run;
      run += v[u];
    }
  }
}

// Large tile counts: the tiles are split into blockIdx.y groups.  Pass 1 sums each
// (digit group, tile group) into part[group][digit]; pass 2 starts each group from the sum
// of the groups before it and scans in place (the last group also writes the totals).
__device__ __forceinline__ void scan_group_range(uint32_t tiles, uint32_t groups, uint32_t g, uint32_t& t0,
                                                 uint32_t& t1) {
  const uint32_t per = (tiles + groups - 1) / groups;
  t0 = min(tiles, g * per);
  t1 = min(tiles, t0 + per);
}

__global__ void __launch_bounds__(256) k_sort_scan_part(const uint32_t* __restrict__ hist, uint32_t tiles, int bins,
                                                        uint32_t* __restrict__ part) {
  pdl_enter();
  __shared__ uint32_t s_part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  uint32_t g0, g1;
  scan_group_range(tiles, gridDim.y, blockIdx.y, g0, g1);
  const uint32_t chunk = (g1 - g0 + 7) / 8;
  const uint32_t t0 = min(g1, g0 + warp * chunk), t1 = min(g1, t0 + chunk);
  uint32_t sum = 0;
  if (d < bins)
    for (uint32_t t = t0; t < t1; ++t) sum += __ldg(hist + (size_t)t * kMaxBins + d);
  s_part[warp][lane] = sum;
  __syncthreads();
  if (warp == 0 && d < bins) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) run += s_part[w][lane];
    part[(size_t)blockIdx.y * kMaxBins + d] = run;
  }
}

__global__ void __launch_bounds__(256) k_sort_scan_final(uint32_t* __restrict__ hist, uint32_t tiles, int bins,
                                                         const uint32_t* __restrict__ part,
                                                         uint32_t* __restrict__ totals) {
  pdl_enter();
  __shared__ uint32_t s_part[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  uint32_t g0, g1;
  scan_group_range(tiles, gridDim.y, blockIdx.y, g0, g1);
  const uint32_t chunk = (g1 - g0 + 7) / 8;
  const uint32_t t0 = min(g1, g0 + warp * chunk), t1 = min(g1, t0 + chunk);
  uint32_t sum = 0;
  if (d < bins)
    for (uint32_t t = t0; t < t1; ++t) sum += hist[(size_t)t * kMaxBins + d];
  s_part[warp][lane] = sum;
  __syncthreads();
  if (warp == 0) {
    uint32_t run = 0;
    if (d < bins)
      for (uint32_t gg = 0; gg < blockIdx.y; ++gg) run += __ldg(part + (size_t)gg * kMaxBins + d);
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      const uint32_t v = s_part[w][lane];
      s_part[w][lane] = run;
      run += v;
    }
    if (d < bins && blockIdx.y == gridDim.y - 1) totals[d] = run;
  }
  __syncthreads();
  if (d < bins) {
    uint32_t run = s_part[warp][lane];
    for (uint32_t t = t0; t < t1; ++t) {
      const size_t at = (size_t)t * kMaxBins + d;
      const uint32_t v = hist[at];
      hist[at] = run;
      run += v;
    }
  }
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan of a[2 t], a[2 t + 1] over the block (WARPS warps, 2 values per thread):
// returns the prefixes of both values; s_wsum holds WARPS words of scratch.
template <int WARPS>
__device__ __forceinline__ void block_scan2(uint32_t v0, uint32_t v1, uint32_t* s_wsum, uint32_t& e0, uint32_t& e1) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v0 + v1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_wsum[warp] = x;
  __syncthreads();
  uint32_t wpre = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) wpre += (w < warp) ? s_wsum[w] : 0u;
  e0 = wpre + x - (v0 + v1);
  e1 = e0 + v0;
  __syncthreads();  // s_wsum may be reused
}

// One LSD pass over a tile of kSortTile keys.  hist holds, for this pass, the exclusive
// prefix over tiles per digit (k_sort_scan); totals the per-digit totals.
// The tile's keys are ranked stably (warp w owns a contiguous chunk, items in index order),
// placed in shared memory in tile-local digit order, and written out from there, so that
// consecutive threads write consecutive addresses of each digit's run.  WARPS warps per
// block, kSortTile / (32 WARPS) keys per lane: 16 warps at small tile counts (more threads
// in flight over few tiles), 8 at large ones (smaller shared-memory footprint).  The 8-warp
// plain pass is held to 48 registers so that five blocks fit an SM (measured at 16.7M keys:
// 263 -> 221 us for two passes); the 8-warp gathering pass keeps more registers for its staged
// loads; 16-warp blocks keep two per SM (64 registers).
template <bool LAST, int WARPS>
__global__ void __launch_bounds__(32 * WARPS, WARPS == 16 ? 2 : (LAST ? 1 : 5)) k_sort_pass(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ idx_in, uint32_t n, int shift, int bits,
    const uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals, uint32_t* __restrict__ keys_out,
    uint32_t* __restrict__ idx_out, uint32_t* __restrict__ hist_next, int next_shift, int next_bits, GatherList g) {
  pdl_enter();
  constexpr int ITEMS = kSortTile / (32 * WARPS), THREADS = 32 * WARPS;
  __shared__ uint32_t s_base[kMaxBins];    // global start of (this tile, digit)
  __shared__ uint32_t s_lstart[kMaxBins];  // tile-local start of each digit
  __shared__ uint32_t s_wc[WARPS][kMaxBins];
  __shared__ uint32_t s_wsum[WARPS];
  __shared__ uint2 s_ks[kSortTile];  // (key, source index) in tile-local sorted order
  const int bins = 1 << bits;
  const uint32_t mask = (uint32_t)(bins - 1);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t tile = blockIdx.x;

  // Exclusive scan of the digit totals (2 digits per thread) + this tile's prefix.
  {
    const int d0 = 2 * tid, d1 = 2 * tid + 1;
    const uint32_t v0 = d0 < bins ? __ldg(totals + d0) : 0u;
    const uint32_t v1 = d1 < bins ? __ldg(totals + d1) : 0u;
    uint32_t e0, e1;
    block_scan2<WARPS>(v0, v1, s_wsum, e0, e1);
    const uint32_t* tp = hist + (size_t)tile * kMaxBins;
    if (d0 < bins) s_base[d0] = e0 + __ldg(tp + d0);
    if (d1 < bins) s_base[d1] = e1 + __ldg(tp + d1);
  }
  for (int i = tid; i < WARPS * bins; i += THREADS) s_wc[i / bins][i % bins] = 0;
  __syncthreads();

  // Stable rank within the warp's contiguous chunk, items in index order.
  const uint32_t wbase = tile * kSortTile + warp * (32 * ITEMS);
  const uint32_t ltmask = lanemask_lt();
  uint32_t key[ITEMS], dig[ITEMS], rank[ITEMS], srcI[ITEMS];
  // All of the lane's keys and source indices are loaded before the ranking starts.
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t e = wbase + k * 32 + lane;
    const bool valid = e < n;
    key[k] = valid ? __ldg(keys_in + e) : 0u;
    srcI[k] = (valid && idx_in) ? __ldg(idx_in + e) : e;
  }
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t e = wbase + k * 32 + lane;
    const bool valid = e < n;
    dig[k] = valid ? ((key[k] >> shift) & mask) : 0xFFFFFFFFu;
    // The lowest lane of each digit's peer group adds the group to the warp's counter and
    // hands the previous count to its peers.
    const uint32_t peers = __match_any_sync(0xffffffffu, dig[k]);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (valid && lane == leader) old = atomicAdd(&s_wc[warp][dig[k]], (uint32_t)__popc(peers));
    old = __shfl_sync(0xffffffffu, old, leader);
    rank[k] = old + __popc(peers & ltmask);
  }
  __syncthreads();
  // Per digit: exclusive offsets over warps, then the tile-local digit starts.
  {
    uint32_t c[2] = {0u, 0u};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int d = 2 * tid + q;
      if (d < bins) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
          const uint32_t t = s_wc[w][d];
          s_wc[w][d] = run;
          run += t;
        }
        c[q] = run;
      }
    }
    uint32_t e0, e1;
    block_scan2<WARPS>(c[0], c[1], s_wsum, e0, e1);
    // s_base becomes the output offset of tile-local slot 0 for each digit.
    if (2 * tid < bins) {
      s_lstart[2 * tid] = e0;
      s_base[2 * tid] -= e0;
    }
    if (2 * tid + 1 < bins) {
      s_lstart[2 * tid + 1] = e1;
      s_base[2 * tid + 1] -= e1;
    }
  }
  __syncthreads();
  // Place each key (and its source index) at its tile-local sorted slot.
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t e = wbase + k * 32 + lane;
    if (e < n) {
      const uint32_t d = dig[k];
      const uint32_t lp = s_lstart[d] + s_wc[warp][d] + rank[k];
      s_ks[lp] = make_uint2(key[k], srcI[k]);
    }
  }
  __syncthreads();

  const uint32_t count = min((uint32_t)kSortTile, n - tile * kSortTile);
  static_assert(ITEMS % 2 == 0, "the gathering pass takes elements in pairs");
  if constexpr (LAST) {
    // Two elements per round: all payload loads of both are issued before their stores (to the
    // compiler the destinations may alias the sources, so interleaved load/store pairs would
    // each wait for a full load round trip).
#pragma unroll 1
    for (int it = 0; it < ITEMS; it += 2) {
      uint32_t kk[2], pos[2], src[2];
      bool ok[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const uint32_t j = (it + u) * THREADS + tid;
        const bool valid = j < count;
        kk[u] = 0u;
        pos[u] = 0u;
        src[u] = 0u;
        if (valid) {
          const uint2 ks = s_ks[j];
          kk[u] = ks.x;
          src[u] = ks.y;
          pos[u] = s_base[(kk[u] >> shift) & mask] + j;  // wraps back into [0, n) for a consistent histogram
        }
        // A consistent histogram gives pos < n.  An inconsistent one (a bug, or offsets supplied
        // from outside) must not write out of bounds: the element is not written and the fault
        // word is raised, which the handle reports at its next synchronisation.
        ok[u] = valid && pos[u] < n;
        if (valid && !ok[u] && g.fault) atomicOr(g.fault, 1u);
      }
      float4 v4[2][GatherList::kMax4];
      uint32_t v1[2][GatherList::kMax1];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
#pragma unroll
        for (int b = 0; b < GatherList::kMax4; ++b)
          if (ok[u] && b < g.n4) v4[u][b] = __ldg(g.src4[b] + src[u]);
#pragma unroll
        for (int b = 0; b < GatherList::kMax1; ++b)
          if (ok[u] && b < g.n1) v1[u][b] = __ldg(g.src1[b] + src[u]);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (!ok[u]) continue;
        keys_out[pos[u]] = kk[u];
#pragma unroll
        for (int b = 0; b < GatherList::kMax4; ++b)
          if (b < g.n4) g.dst4[b][pos[u]] = v4[u][b];
#pragma unroll
        for (int b = 0; b < GatherList::kMax1; ++b)
          if (b < g.n1) g.dst1[b][pos[u]] = v1[u][b];
        if (g.perm) g.perm[pos[u]] = src[u];
      }
    }
    return;
  }
  const uint32_t nmask = (1u << next_bits) - 1u;
#pragma unroll 2
  for (int it = 0; it < ITEMS; ++it) {
    const uint32_t j = it * THREADS + tid;
    const bool valid = j < count;
    uint32_t kk = 0, pos = 0, src = 0;
    if (valid) {
      const uint2 ks = s_ks[j];
      kk = ks.x;
      src = ks.y;
      pos = s_base[(kk >> shift) & mask] + j;  // wraps back into [0, n) for a consistent histogram
    }
    // A consistent histogram gives pos < n.  An inconsistent one (a bug, or offsets supplied
    // from outside) must not write out of bounds: the element is not written and the fault
    // word is raised, which the handle reports at its next synchronisation.
    const bool ok = valid && pos < n;
    if (valid && !ok && g.fault) atomicOr(g.fault, 1u);
    if (ok) {
      keys_out[pos] = kk;
      idx_out[pos] = src;
    }
    // Next pass's tile histogram, aggregated over lanes hitting the same (tile, digit).
    const uint32_t slot = ok ? (pos / kSortTile) * kMaxBins + ((kk >> next_shift) & nmask) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, slot);
    if (ok && (peers & ltmask) == 0) atomicAdd(hist_next + slot, (uint32_t)__popc(peers));
  }
}

// Cell table fill (grid.cl:91-138) in the [begin, endExcl) encoding; the table was zeroed.
// fillStartCell skips ID 0, so the reset value start = 1 stays for that cell: the first
// sorted particle begins its cell at index 1.  In a batch (sceneOf != nullptr) that holds
// for the first slot of every scene.
__global__ void k_cell_table_fill(const uint32_t* __restrict__ sk, uint32_t n, uint32_t nc, uint2* __restrict__ table,
                                  const uint16_t* __restrict__ sceneOf) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = __ldg(sk + i);
  if (k >= nc) return;
  uint32_t* t = reinterpret_cast<uint32_t*>(table + k);
  const bool sceneFirst = i == 0 || (sceneOf && __ldg(sceneOf + i - 1) != __ldg(sceneOf + i));
  if (sceneFirst) t[0] = i + 1u;
  else if (__ldg(sk + i - 1) != k) t[0] = i;
  const uint32_t right = (i + 1 < n) ? __ldg(sk + i + 1) : 0xFFFFFFFFu;
  if (right != k) t[1] = i + 1;
}

// Internal encoding -> reference format (start, end inclusive, capped; empty = (1, 0)).
// In place is allowed: each thread reads and writes only its own cell.
__global__ void k_cell_table_ref(const uint2* table, uint32_t nc, uint32_t cap, uint2* out) {
  pdl_enter();
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const uint2 se = table[c];
  const uint32_t cnt = se.y > se.x ? min(se.y - se.x, cap + 1u) : 0u;
  out[c] = cnt ? make_uint2(se.x, se.x + cnt - 1u) : make_uint2(1u, 0u);
}

static int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return RTP_OK;
}

// resetCellIDs (grid.cl:65-71): a key above every cell for each slot; the slots a step does not
// fill keep theirs, so they stay at the tail of the sorted keys in slot order.
__global__ void k_reset_cell_ids(uint32_t* __restrict__ keys, uint32_t n, uint32_t base) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keys[i] = base + i;
}

int launch_reset_cell_ids(uint32_t* keys, uint32_t n, uint32_t numCells, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_reset_cell_ids, dim3((n + 255) / 256), dim3(256), keys, n, 2u * numCells);
  return check_launch("k_reset_cell_ids");
}

int launch_fill_cell_ids(const GridK& g, const float4* pos, uint32_t n, uint32_t* keys, Launcher& L) {
  if (n == 0) return RTP_OK;
  L.begin("fillCellIDs");
  launch(L, k_fill_cell_ids, dim3((n + 255) / 256), dim3(256), g, pos, n, keys);
  L.end("fillCellIDs");
  return check_launch("k_fill_cell_ids");
}

int launch_sort_histogram(const SortPlan& p, const uint32_t* keys, const SortScratch& s, Launcher& L) {
  L.begin("sort_hist0");
  launch(L, k_sort_hist, dim3(p.tiles), dim3(kKeyThreads), keys, p.n, 0, p.bits[0], s.hist);
  L.end("sort_hist0");
  return check_launch("k_sort_hist");
}

ZeroJob step_zero_job(const SortPlan& p, const SortScratch& s, uint2* table, uint32_t nc) {
  ZeroJob z;
  if (p.passes > 1) {
    const size_t per = (size_t)p.tiles * kMaxBins;
    z.p[0] = s.hist + per;
    z.n[0] = (uint32_t)(per * (p.passes - 1));
  }
  z.p[1] = reinterpret_cast<uint32_t*>(table);
  z.n[1] = 2u * nc;
  return z;
}

int launch_sort_clear(const SortPlan& p, const SortScratch& s, Launcher& L) {
  if (p.passes <= 1) return RTP_OK;
  const size_t per = (size_t)p.tiles * kMaxBins;
  L.begin("sort_clear");
  RTP_CUDA(cudaMemsetAsync(s.hist + per, 0, sizeof(uint32_t) * per * (p.passes - 1), L.stream));
  L.end("sort_clear");
  return RTP_OK;
}

static_assert(RTP_SORT_TILE == kSortTile && RTP_SORT_BINS == kMaxBins, "keep rtp.h in step with the sort tiles");

int launch_sort_one_pass(const uint32_t* keys_in, uint32_t n, int shift, int bits, const uint32_t* hist,
                         const uint32_t* totals, uint32_t* keys_out, const GatherList& g, Launcher& L) {
  if (n == 0) return RTP_OK;
  const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
  if (tiles <= kWidePassTiles)
    launch(L, k_sort_pass<true, 16>, dim3(tiles), dim3(512), keys_in, (const uint32_t*)nullptr, n, shift, bits, hist,
           totals, keys_out, (uint32_t*)nullptr, (uint32_t*)nullptr, 0, 0, g);
  else
    launch(L, k_sort_pass<true, 8>, dim3(tiles), dim3(256), keys_in, (const uint32_t*)nullptr, n, shift, bits, hist,
           totals, keys_out, (uint32_t*)nullptr, (uint32_t*)nullptr, 0, 0, g);
  return check_launch("k_sort_pass");
}

int launch_sort_passes(const SortPlan& p, const uint32_t* keys_in, uint32_t* keys_out, const SortScratch& s,
                       const GatherList& g, Launcher& L) {
  if (g.n4 < 0 || g.n4 > GatherList::kMax4 || g.n1 < 0 || g.n1 > GatherList::kMax1)
    return fail(RTP_ERR_INVALID_ARGUMENT, "sort: too many gathered arrays");
  if (p.n == 0) return RTP_OK;
  const size_t per = (size_t)p.tiles * kMaxBins;
  const uint32_t* kin = keys_in;
  const uint32_t* iin = nullptr;
  for (int pass = 0; pass < p.passes; ++pass) {
    const bool last = pass == p.passes - 1;
    uint32_t* hist = s.hist + per * pass;
    uint32_t* totals = s.totals + (size_t)kMaxBins * pass;
    const int bins = 1 << p.bits[pass];
    const uint32_t groups = scan_groups(p.tiles);
    const bool wide = p.tiles <= kWidePassTiles;
    L.begin("sort_scan");
    if (groups <= 1) {
      launch(L, k_sort_scan, dim3((bins + 31) / 32), dim3(256), hist, p.tiles, bins, totals);
    } else {
      const dim3 grid((bins + 31) / 32, groups);
      launch(L, k_sort_scan_part, dim3(grid), dim3(256), hist, p.tiles, bins, s.scanPart);
      launch(L, k_sort_scan_final, dim3(grid), dim3(256), hist, p.tiles, bins, s.scanPart, totals);
    }
    L.end("sort_scan");
    int rc = check_launch("k_sort_scan");
    if (rc) return rc;
    uint32_t* kout = last ? keys_out : ((pass % 2 == 0) ? s.keysB : s.keysA);
    uint32_t* iout = last ? nullptr : ((pass % 2 == 0) ? s.idxB : s.idxA);
    if (!last && kout == kin) kout = (kout == s.keysA) ? s.keysB : s.keysA;
    if (last) {
      L.begin("sort_pass_gather");
      if (wide)
        launch(L, k_sort_pass<true, 16>, dim3(p.tiles), dim3(512), kin, iin, p.n, p.shift[pass], p.bits[pass], hist,
               totals, kout, nullptr, nullptr, 0, 1, g);
      else
        launch(L, k_sort_pass<true, kSortWarps>, dim3(p.tiles), dim3(kSortThreads), kin, iin, p.n, p.shift[pass],
               p.bits[pass], hist, totals, kout, nullptr, nullptr, 0, 1, g);
      L.end("sort_pass_gather");
    } else {
      L.begin("sort_pass");
      if (wide)
        launch(L, k_sort_pass<false, 16>, dim3(p.tiles), dim3(512), kin, iin, p.n, p.shift[pass], p.bits[pass], hist,
               totals, kout, iout, hist + per, p.shift[pass + 1], p.bits[pass + 1], g);
      else
        launch(L, k_sort_pass<false, kSortWarps>, dim3(p.tiles), dim3(kSortThreads), kin, iin, p.n, p.shift[pass],
               p.bits[pass], hist, totals, kout, iout, hist + per, p.shift[pass + 1], p.bits[pass + 1], g);
      L.end("sort_pass");
    }
    rc = check_launch("k_sort_pass");
    if (rc) return rc;
    kin = kout;
    iin = iout;
  }
  return RTP_OK;
}

int launch_cell_table(const GridK& g, const uint32_t* sorted_keys, uint32_t n, uint2* table, Launcher& L,
                      const uint16_t* sceneOf, bool cleared) {
  if (!cleared) {
    L.begin("cellTableClear");
    RTP_CUDA(cudaMemsetAsync(table, 0, sizeof(uint2) * g.nc, L.stream));
    L.end("cellTableClear");
  }
  if (n == 0) return RTP_OK;
  L.begin("cellTable");
  launch(L, k_cell_table_fill, dim3((n + 255) / 256), dim3(256), sorted_keys, n, g.nc, table, sceneOf);
  L.end("cellTable");
  return check_launch("k_cell_table_fill");
}

int launch_cell_table_to_reference(const GridK& g, const uint2* table, uint2* out, Launcher& L) {
  L.begin("cellTableRef");
  launch(L, k_cell_table_ref, dim3((g.nc + 255) / 256), dim3(256), table, g.nc, g.cap, out);
  L.end("cellTableRef");
  return check_launch("k_cell_table_ref");
}

}  // namespace rtp

using namespace rtp;

extern "C" {

int rtp_fill_cell_ids(const rtp_grid_constants* c, const float* d_pos4, uint32_t n, uint32_t* d_keys, void* stream) {
  if (!c || (n && (!d_pos4 || !d_keys))) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_fill_cell_ids: null argument");
  Launcher L;
  L.stream = (cudaStream_t)stream;
  return launch_fill_cell_ids(make_gridk(*c), reinterpret_cast<const float4*>(d_pos4), n, d_keys, L);
}

int rtp_radix_sort_scratch_bytes(uint32_t n, uint32_t keyBits, size_t* bytes) {
  if (!bytes || keyBits > 32) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort_scratch_bytes: bad argument");
  *bytes = sort_scratch_bytes(make_sort_plan(n, keyBits));
  return RTP_OK;
}

int rtp_radix_sort(const uint32_t* d_keys_in, uint32_t n, uint32_t keyBits, uint32_t* d_keys_out, uint32_t* d_perm_out,
                   void* d_scratch, size_t scratch_bytes, void* stream) {
  if (keyBits > 32) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort: keyBits > 32");
  if (n == 0) return RTP_OK;
  if (!d_keys_in || !d_keys_out || !d_scratch) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort: null pointer");
  const SortPlan p = make_sort_plan(n, keyBits);
  if (scratch_bytes < sort_scratch_bytes(p)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort: scratch too small");
  if ((reinterpret_cast<uintptr_t>(d_scratch) & 255u) != 0)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort: scratch must be 256-byte aligned");
  SortScratch s;
  sort_scratch_carve(p, d_scratch, s);
  Launcher L;
  L.stream = (cudaStream_t)stream;
  int rc = launch_sort_clear(p, s, L);
  if (rc) return rc;
  rc = launch_sort_histogram(p, d_keys_in, s, L);
  if (rc) return rc;
  GatherList g;
  g.perm = d_perm_out;
  return launch_sort_passes(p, d_keys_in, d_keys_out, s, g, L);
}

int rtp_radix_sort_pass(const uint32_t* d_keys_in, uint32_t n, uint32_t shift, uint32_t bits,
                        const uint32_t* d_tile_offsets, const uint32_t* d_digit_totals, uint32_t* d_keys_out,
                        uint32_t* d_perm_out, uint32_t* d_fault, void* stream) {
  if (bits < 1 || bits > (uint32_t)kMaxRadixBits || shift > 31)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort_pass: bits must be 1..9 and shift < 32");
  if (n == 0) return RTP_OK;
  if (!d_keys_in || !d_keys_out || !d_tile_offsets || !d_digit_totals || !d_fault)
    return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_radix_sort_pass: null pointer");
  Launcher L;
  L.stream = (cudaStream_t)stream;
  GatherList g;
  g.perm = d_perm_out;
  g.fault = d_fault;
  return launch_sort_one_pass(d_keys_in, n, (int)shift, (int)bits, d_tile_offsets, d_digit_totals, d_keys_out, g, L);
}

int rtp_build_cell_table(const rtp_grid_constants* c, const uint32_t* d_sorted_keys, uint32_t n, uint32_t* d_table2,
                         void* stream) {
  if (!c || !d_table2 || (n && !d_sorted_keys)) return fail(RTP_ERR_INVALID_ARGUMENT, "rtp_build_cell_table: null argument");
  const GridK g = make_gridk(*c);
  Launcher L;
  L.stream = (cudaStream_t)stream;
  uint2* t = reinterpret_cast<uint2*>(d_table2);
  const int rc = launch_cell_table(g, d_sorted_keys, n, t, L);
  return rc ? rc : launch_cell_table_to_reference(g, t, t, L);
}

}  // extern "C"
