// rtp_internal.hpp - host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/rtp.h"
#include "rtp_common.cuh"

namespace rtp {

// Thread-local error message (rtp_last_error).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define RTP_CUDA(call)                                    \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return ::rtp::cuda_fail(_e, #call); \
  } while (0)

// Kernel launch bookkeeping: names each launch so the profiler can attribute time.
struct Launcher {
  cudaStream_t stream = nullptr;
  bool profiling = false;
  void* owner = nullptr;  // Handle* when profiling
  bool pdl = false;       // launch with programmatic dependent launch allowed
  int begin(const char* name);
  int end(const char* name);
};

// Launches kernel k on L's stream (errors are reported by cudaGetLastError, as for <<< >>>).
// With L.pdl the launch allows programmatic dependent launch; every kernel launched here calls
// pdl_enter() before it reads anything, so it never reads a predecessor's output early.
template <class... P, class... A>
inline void launch(const Launcher& L, void (*k)(P...), dim3 grid, dim3 block, A&&... a) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = L.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = L.pdl ? 1u : 0u;
  (void)cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(a)...);
}

// Raises kernel k's dynamic shared memory limit to `bytes` on the current device (once per
// kernel and device).
void ensure_dynamic_smem(const void* k, size_t bytes);

// launch() with `smem` bytes of dynamic shared memory.
template <class... P, class... A>
inline void launch_smem(const Launcher& L, void (*k)(P...), dim3 grid, dim3 block, size_t smem, A&&... a) {
  ensure_dynamic_smem(reinterpret_cast<const void*>(k), smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = L.pdl ? 1u : 0u;
  (void)cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(a)...);
}

// ---- Radix sort ---------------------------------------------------------------------
struct SortPlan {
  uint32_t n = 0;
  uint32_t keyBits = 0;
  int passes = 0;
  int bits[4] = {0, 0, 0, 0};
  int shift[4] = {0, 0, 0, 0};
  uint32_t tiles = 0;
};
SortPlan make_sort_plan(uint32_t n, uint32_t keyBits);
// Scratch layout for a plan: keys ping-pong, index ping-pong, histograms, totals.
struct SortScratch {
  uint32_t* keysA = nullptr;
  uint32_t* keysB = nullptr;
  uint32_t* idxA = nullptr;
  uint32_t* idxB = nullptr;
  uint32_t* hist = nullptr;      // passes x tiles x kMaxBins
  uint32_t* totals = nullptr;    // passes x kMaxBins
  uint32_t* scanPart = nullptr;  // tile groups x kMaxBins (two-kernel digit scan)
};
// Tile groups of the digit scan: one block column per kScanTilesPerGroup tiles, at most
// kScanGroupsMax (beyond that the groups grow).
constexpr uint32_t kScanTilesPerGroup = 128;
constexpr uint32_t kScanGroupsMax = 64;
size_t sort_scratch_bytes(const SortPlan& p);
void sort_scratch_carve(const SortPlan& p, void* base, SortScratch& s);

// Values carried by the last sort pass: dst[pos] = src[perm[pos]].
struct GatherList {
  // The most any step gathers (clouds: pos, vel, predicted pos, total correction; temperature,
  // buoyancy, vapour, cloud, id).  The gathering pass stages every entry in registers.
  static constexpr int kMax4 = 4;
  static constexpr int kMax1 = 5;
  const float4* src4[kMax4];
  float4* dst4[kMax4];
  const uint32_t* src1[kMax1];
  uint32_t* dst1[kMax1];
  int n4 = 0;
  int n1 = 0;
  uint32_t* perm = nullptr;  // optional: write the permutation
  // Optional fault word: a pass that computes a position outside [0, n) for an element (a digit
  // offset table inconsistent with the keys) does not write it and ORs 1 into *fault instead.
  uint32_t* fault = nullptr;
};

// Histogram of digit 0 of `keys` per tile (used when keys come from outside a model step).
int launch_sort_histogram(const SortPlan& p, const uint32_t* keys, const SortScratch& s, Launcher& L);
// Passes 0..passes-1: keys (already histogrammed for pass 0) -> sorted keys in keys_out,
// values gathered by `g` in the last pass.  keys_in may alias s.keysA.
int launch_sort_passes(const SortPlan& p, const uint32_t* keys_in, uint32_t* keys_out, const SortScratch& s,
                       const GatherList& g, Launcher& L);
// Zero the histogram area (the first pass reads it after the producer kernel filled it).
int launch_sort_clear(const SortPlan& p, const SortScratch& s, Launcher& L);
// One scatter pass over all tiles with caller-supplied digit offsets: hist = exclusive prefix
// over tiles per digit ([tile][kMaxBins]), totals = per-digit totals (kMaxBins).
int launch_sort_one_pass(const uint32_t* keys_in, uint32_t n, int shift, int bits, const uint32_t* hist,
                         const uint32_t* totals, uint32_t* keys_out, const GatherList& g, Launcher& L);

// Cell table in the internal [begin, endExcl) encoding from sorted keys (sceneOf: the scene
// of every slot of a batch, or nullptr).
// cleared: the table was zeroed already (by the key-producing kernel's ZeroJob).
int launch_cell_table(const GridK& g, const uint32_t* sorted_keys, uint32_t n, uint2* table, Launcher& L,
                      const uint16_t* sceneOf = nullptr, bool cleared = false);
// What the key-producing kernel of a model step clears: the histograms of sort passes >= 1
// (instead of launch_sort_clear) and the cell table (instead of its memset).
ZeroJob step_zero_job(const SortPlan& p, const SortScratch& s, uint2* table, uint32_t nc);
// Internal encoding -> the reference's inclusive (start, end) with (1, 0) for empty cells.
int launch_cell_table_to_reference(const GridK& g, const uint2* table, uint2* out, Launcher& L);
int launch_fill_cell_ids(const GridK& g, const float4* pos, uint32_t n, uint32_t* keys, Launcher& L);
// resetCellIDs (grid.cl:65-71): key[i] = 2 * numCells + i for the n slots.
int launch_reset_cell_ids(uint32_t* keys, uint32_t n, uint32_t numCells, Launcher& L);

}  // namespace rtp
