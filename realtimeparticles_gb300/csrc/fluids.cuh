// fluids.cuh - PBF kernel parameters and launchers (fluids.cu), shared with clouds.cu.
#pragma once

#include "rtp_internal.hpp"
#include "sweep.cuh"

#include <type_traits>

namespace rtp {

// FluidParams (kernels/define.cl:13-25) with the derived values the kernels use.
struct FluidK {
  float rho0, invRho0, invRho0Sq, relaxCFM, dt;
  float4 lo, hi;      // fld_applyBoundaryCondition bounds (fluids.cl:437-438)
  int artPressure;
  float apCoeff;      // artPressureCoeff
  float apInvWq;      // 1 / poly6L(artPressureRadius * h)
  uint32_t apExp;
  int vorticity;
  float vortCoeff;
  float xsph;
  BatchK bt;        // batched scenes (bt.scenes == nullptr: one scene, the fields above)
  int lanes = 4;    // lanes per particle of the list sweeps: 2, 4 or 8
  int tiles = 0;    // 1: the lambda sweep tiled by bricks of cells where the grid allows
  const uint32_t* sortedKeys = nullptr;  // the step's sorted cell keys (the brick sweep's leftovers)
};

FluidK make_fluidk(const rtp_grid_constants& c, const rtp_fluid_params& p);

#ifdef __CUDACC__
__device__ __forceinline__ float4 bc_clamp(const FluidK& p, float4 x) { return clamp4(x, p.lo, p.hi); }

// Parameters of particle slot i: the kernel's own (one scene) or its scene's (batch).
template <bool BATCH>
__device__ __forceinline__ void scene_of(uint32_t i, GridK& g, FluidK& p) {
  if constexpr (BATCH) {
    const SceneK* sc = p.bt.scenes + __ldg(p.bt.sceneOf + i);
    g = sc->g;
    p.lo = sc->lo;
    p.hi = sc->hi;
  }
}

// Calls f(std::integral_constant<bool, batch>, std::integral_constant<int, lanes>) for the
// batch mode and lane count of p.
template <class F>
inline void dispatch_fluid(const FluidK& p, F&& f) {
  using T = std::true_type;
  using N = std::false_type;
  const bool b = p.bt.scenes != nullptr;
  switch (p.lanes) {
    case 2:
      b ? f(T{}, std::integral_constant<int, 2>{}) : f(N{}, std::integral_constant<int, 2>{});
      break;
    case 8:
      b ? f(T{}, std::integral_constant<int, 8>{}) : f(N{}, std::integral_constant<int, 8>{});
      break;
    default:
      b ? f(T{}, std::integral_constant<int, 4>{}) : f(N{}, std::integral_constant<int, 4>{});
  }
}

// Operands of one pair loaded ahead of use: a position and a scalar, or two float4.
struct Pair4 {
  float4 x;
  float s;
};
struct Pair44 {
  float4 x, v;
};

// Block sum of v (blockDim.x == kSweepThreads, every thread of the block calls once)
// written to out[blockIdx.x].
__device__ __forceinline__ void block_error_partial(float v, float* out) {
  static_assert(kSweepThreads == 64, "two warps per block");
  __shared__ float s_part[2];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = s_part[0] + s_part[1];
}
#endif

// Total-lambda bookkeeping of k_fluid_lambda (warm start).
constexpr int kTotNone = 0, kTotWrite = 1, kTotAdd = 2;

// pos / vel are the canonical device buffers (written only to mirror io.inPos / io.inVel).
int fluid_presort(const GridK& g, const FluidK& p, float4* pos, float4* vel, uint32_t n, float4* pred,
                  uint32_t* keys, const SortPlan& plan, uint32_t* hist0, bool clampOut, Launcher& L,
                  const ZeroJob& zero = ZeroJob{}, const HostIO& io = HostIO{});
int fluid_iteration(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, const uint2* table,
                    uint32_t n, float* lambda, float* density, bool last, const float4* posS, float4* velS,
                    const PairList& pl, Launcher& L, float* lamTot = nullptr, int totMode = kTotNone,
                    float4* packed = nullptr, const float* omega = nullptr);
// The density / lambda sweep of one iteration alone (fld_applyBoundaryCondition is the
// producer's; fld_computeDensity + fld_computeConstraintFactor), recording the pairs into pl.
// With omega (per particle) the lambdas are relaxed by it (the warm start in every iteration).
int fluid_lambda_sweep(const GridK& g, const FluidK& p, const float4* predIn, const uint2* table, uint32_t n,
                       float* lambda, float* density, const PairList& pl, Launcher& L, float* lamTot = nullptr,
                       int totMode = kTotNone, float4* packed = nullptr, const float* omega = nullptr);
// Position correction alone with given lambdas (+ an optional residual displacement).  With
// `packed` (x, y, z, lambda per particle, written by the lambda sweep) the neighbours' data
// come from there.
int fluid_deltap(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, const float* lambda,
                 const uint2* table, uint32_t n, bool last, const float4* posS, float4* velS, const PairList& pl,
                 const float4* res, Launcher& L, const float4* packed = nullptr);
// fld_computeVorticity; with errPartial also the per-block density-error sums; with `packed`
// also (x, y, z, |omega|) per particle for the confinement sweep (fluid_post with the same
// `packed`).
int fluid_vorticity(const GridK& g, const FluidK& p, const float4* pred, const float4* velS, float4* vort,
                    const uint2* table, uint32_t n, const PairList& pl, float* errPartial, Launcher& L,
                    float4* packed = nullptr);
int fluid_update_vel(const GridK& g, const FluidK& p, const float4* pred, const float4* posS, uint32_t n, float4* velS,
                     Launcher& L);
int fluid_post(const GridK& g, const FluidK& p, const float4* pred, float4* velS, float4* vort, const uint2* table,
               uint32_t n, const uint32_t* idsS, float4* pos, float4* vel, uint32_t* ids, const PairList& pl,
               Launcher& L, bool vorticityDone = false, const HostIO& io = HostIO{}, float4* packed = nullptr);
int fluid_metrics(const GridK& g, const FluidK& p, const float4* pos, const float4* vel, const uint2* table, uint32_t n,
                  double* acc, uint32_t* hist, Launcher& L);

int pair_list_stats(const PairList& pl, uint32_t n, uint32_t* out2, Launcher& L);

}  // namespace rtp
