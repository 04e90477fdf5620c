// rtp_common.cuh - device helpers shared by the grid/sort, fluids, boids and clouds kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rtp.h"

namespace rtp {

constexpr float kFloatEps = 0.00000001f;   // FLOAT_EPS, kernels/define.cl:6
constexpr float kAbsGravityY = 9.81f;      // ABS_GRAVITY_ACC_Y, kernels/define.cl:8
constexpr int kSortTile = 2048;            // keys per sort tile
constexpr int kSortWarps = 8;              // warps of a scatter-pass block at large tile counts
constexpr int kSortItems = kSortTile / (32 * kSortWarps);  // keys per lane
constexpr int kSortThreads = kSortWarps * 32;
constexpr int kKeyThreads = 1024;          // threads of the key-producing kernels (one tile each;
                                           // 64 tiles at 131k occupy 64 SMs, so more warps per tile)
constexpr int kKeyItems = kSortTile / kKeyThreads;
constexpr int kMaxRadixBits = 9;
constexpr int kMaxBins = 1 << kMaxRadixBits;

// Programmatic dependent launch.  Every kernel of a step starts here: under a launch with the
// programmatic-serialization attribute it waits until the kernel before it has completed and
// its writes are visible (the dependent kernel is released as this one's CTAs exit); without
// the attribute it is a no-op.  Measured on the 131k PBF and boids steps: within 1 % of plain
// serialisation; releasing dependents at kernel entry instead cost 10 %.  Off by default
// (Launcher::pdl).
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The reference's JIT -D constants (Fluids.cpp:104-119), passed by value to kernels.
struct GridK {
  float W[3];      // ABS_WALL_X/Y/Z
  int R[3];        // GRID_RES_X/Y/Z
  float cell;      // GRID_CELL_SIZE_XYZ
  uint32_t nc;     // GRID_NUM_CELLS
  uint32_t cap;    // NUM_MAX_PARTS_IN_CELL
  float h;         // EFFECT_RADIUS
  float boidsR2;   // EFFECT_RADIUS_SQUARED
  float poly6;     // POLY6_COEFF
  float spiky;     // SPIKY_COEFF
  float maxVel;    // MAX_VEL
  uint32_t base;   // first key / table entry of this grid (0; scene offset in a batch)
};

inline GridK make_gridk(const rtp_grid_constants& c) {
  GridK g;
  for (int a = 0; a < 3; ++a) {
    g.W[a] = c.absWall[a];
    g.R[a] = (int)c.gridRes[a];
  }
  g.cell = c.cellSize;
  g.nc = c.numCells;
  g.cap = c.maxPartsInCell;
  g.h = c.effectRadius;
  g.boidsR2 = c.effectRadiusSquared;
  g.poly6 = c.poly6Coeff;
  g.spiky = c.spikyCoeff;
  g.maxVel = c.maxVel;
  g.base = 0;
  return g;
}

// getCell3DIndexFromPos (grid.cl:14-24): clamp to the walls, shift by +W, floor of an IEEE
// division by the cell size.  Round-to-nearest intrinsics keep it bit-identical to the CPU.
__device__ __forceinline__ void cell3(const GridK& g, float4 p, int& cx, int& cy, int& cz) {
  const float qx = __fadd_rn(fminf(fmaxf(p.x, -g.W[0]), g.W[0]), g.W[0]);
  const float qy = __fadd_rn(fminf(fmaxf(p.y, -g.W[1]), g.W[1]), g.W[1]);
  const float qz = __fadd_rn(fminf(fmaxf(p.z, -g.W[2]), g.W[2]), g.W[2]);
  cx = (int)(uint32_t)floorf(__fdiv_rn(qx, g.cell));
  cy = (int)(uint32_t)floorf(__fdiv_rn(qy, g.cell));
  cz = (int)(uint32_t)floorf(__fdiv_rn(qz, g.cell));
}

// getCell1DIndexFromPos (grid.cl:29-38), offset by the grid's base key.
__device__ __forceinline__ uint32_t cell_key(const GridK& g, float4 p) {
  int cx, cy, cz;
  cell3(g, p, cx, cy, cz);
  return g.base + ((uint32_t)cx * (uint32_t)g.R[2] * (uint32_t)g.R[1] + (uint32_t)cy * (uint32_t)g.R[2] + (uint32_t)cz);
}

// Batched scenes: each scene's own grid and wall-clamp bounds, and the scene of every
// particle slot (scenes occupy fixed contiguous slot ranges; the global sort keeps them so,
// because scene s's keys lie in [base_s, base_s + keyBound_s), below scene s + 1's).
struct SceneK {
  GridK g;
  float4 lo, hi;  // fld_applyBoundaryCondition bounds of the scene
};
struct BatchK {
  const SceneK* scenes = nullptr;  // nullptr: a single scene, parameters from the kernel arguments
  const uint16_t* sceneOf = nullptr;
};

// Cell table entry as stored on the device: [begin, endExcl).  Empty cells are (0, 0) so a
// memset clears the table.  The reference stores (start, end) inclusive with (1, 0) for
// empty cells and start = 1 for the cell of sorted index 0 (grid.cl:91-116); the fill
// kernel reproduces that by writing begin = 1 for that cell.  The per-cell cap
// (adjustEndCell, grid.cl:143-152) is applied when a range is read.
__device__ __forceinline__ void cell_range(const uint2* __restrict__ table, uint32_t c, uint32_t cap,
                                           uint32_t& b, uint32_t& e) {
  const uint2 se = __ldg(table + c);
  b = se.x;
  const uint32_t n = se.y > se.x ? min(se.y - se.x, cap + 1u) : 0u;
  e = se.x + n;
}

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

__device__ __forceinline__ float4 f4(float x, float y, float z, float w) { return make_float4(x, y, z, w); }
__device__ __forceinline__ float4 operator+(float4 a, float4 b) { return f4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 operator-(float4 a, float4 b) { return f4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ float4 operator*(float4 a, float s) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float4 operator*(float s, float4 a) { return f4(a.x * s, a.y * s, a.z * s, a.w * s); }
__device__ __forceinline__ float dot3(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ float4 cross4(float4 a, float4 b) {
  return f4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
// normalize / fast_normalize with the zero vector mapped to itself.
__device__ __forceinline__ float4 normalize0(float4 a) {
  const float d = dot4(a, a);
  if (d == 0.0f) return a;
  return a * rsqrtf(d);
}
__device__ __forceinline__ float4 clamp4(float4 v, float4 lo, float4 hi) {
  return f4(fminf(fmaxf(v.x, lo.x), hi.x), fminf(fmaxf(v.y, lo.y), hi.y), fminf(fmaxf(v.z, lo.z), hi.z),
            fminf(fmaxf(v.w, lo.w), hi.w));
}
__device__ __forceinline__ float4 clamp4s(float4 v, float lo, float hi) {
  return f4(fminf(fmaxf(v.x, lo), hi), fminf(fmaxf(v.y, lo), hi), fminf(fmaxf(v.z, lo), hi), fminf(fmaxf(v.w, lo), hi));
}
__device__ __forceinline__ float powi(float x, uint32_t k) {
  float r = 1.0f;
  for (uint32_t i = 0; i < k; ++i) r *= x;
  return r;
}

// SPH kernels (sph.cl:10-34) evaluated from r^2.  Contributions at r >= h are exactly zero
// in the reference (step mask), so callers skip them.
struct Sph {
  float h, h2, poly6, spiky;
  __device__ __forceinline__ explicit Sph(const GridK& g) : h(g.h), h2(g.h * g.h), poly6(g.poly6), spiky(g.spiky) {}
  // poly6 at distance^2 r2 (r < h).
  __device__ __forceinline__ float w(float r2) const {
    const float q = h2 - r2;
    return poly6 * q * q * q;
  }
  // Scalar s with gradSpiky(v) = v * s; zero at r <= FLOAT_EPS (sph.cl:30-31).
  __device__ __forceinline__ float gs(float r2, float& r) const {
    const float inv = rsqrtf(r2);
    r = r2 * inv;
    if (!(r > kFloatEps)) return 0.0f;
    const float q = h - r;
    return -3.0f * spiky * q * q * inv;
  }
};

// Device memory a key-producing kernel clears on its way (grid-stride), so that a step needs
// no memset nodes: the tile histograms the next sort passes accumulate into, and the cell
// table.  Word counts; each span 16-byte aligned.
struct ZeroJob {
  uint32_t* p[2] = {nullptr, nullptr};
  uint32_t n[2] = {0u, 0u};
};
__device__ __forceinline__ void zero_job(const ZeroJob& z) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    if (!z.p[q]) continue;
    uint4* v = reinterpret_cast<uint4*>(z.p[q]);
    const uint32_t n4 = z.n[q] / 4;
    for (uint32_t k = t; k < n4; k += stride) v[k] = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t k = n4 * 4 + t; k < z.n[q]; k += stride) z.p[q][k] = 0u;
  }
}

// Host-resident input and output of one step (pinned host memory, device-visible pointers):
// the step's first kernel reads pos / vel from inPos / inVel (and mirrors them into the
// canonical device buffers), its last kernel also writes the results to outPos / outVel.
// A null pointer leaves that transfer to the device buffers alone.
struct HostIO {
  const float4* inPos = nullptr;
  const float4* inVel = nullptr;
  float4* outPos = nullptr;
  float4* outVel = nullptr;
};

// Sort-tile histogram of digit 0, for the kernels that produce the keys.  The calling
// block has kKeyThreads threads and handles tile blockIdx.x: element
// blockIdx.x * kSortTile + k * kKeyThreads + threadIdx.x for k < kKeyItems.
struct TileHistogram {
  uint32_t* s;
  int mask;
  __device__ __forceinline__ void init(uint32_t* smem, int bits) {
    s = smem;
    mask = (1 << bits) - 1;
    for (int d = threadIdx.x; d <= mask; d += blockDim.x) s[d] = 0;
    __syncthreads();
  }
  __device__ __forceinline__ void add(uint32_t key) { atomicAdd(&s[key & (uint32_t)mask], 1u); }
  __device__ __forceinline__ void store(uint32_t* hist0) {
    __syncthreads();
    for (int d = threadIdx.x; d <= mask; d += blockDim.x) hist0[(size_t)blockIdx.x * kMaxBins + d] = s[d];
  }
};

}  // namespace rtp
