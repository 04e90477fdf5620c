// fluids.cuh - PBF kernel parameters and launchers (fluids.cu), shared with clouds.cu.
#pragma once

#include "rtp_internal.hpp"
#include "sweep.cuh"

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
};

FluidK make_fluidk(const rtp_grid_constants& c, const rtp_fluid_params& p);



int fluid_presort(const GridK& g, const FluidK& p, const float4* pos, const float4* vel, uint32_t n, float4* pred,
                  uint32_t* keys, const SortPlan& plan, uint32_t* hist0, bool clampOut, Launcher& L);
int fluid_iteration(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, const uint2* table,
                    uint32_t n, float* lambda, float* density, bool last, const float4* posS, float4* velS,
                    const PairList& pl, Launcher& L);
int fluid_update_vel(const GridK& g, const FluidK& p, const float4* pred, const float4* posS, uint32_t n, float4* velS,
                     Launcher& L);
int fluid_post(const GridK& g, const FluidK& p, const float4* pred, float4* velS, float4* vort, const uint2* table,
               uint32_t n, const uint32_t* idsS, float4* pos, float4* vel, uint32_t* ids, const PairList& pl,
               Launcher& L);
int fluid_metrics(const GridK& g, const FluidK& p, const float4* pos, const float4* vel, const uint2* table, uint32_t n,
                  double* acc, uint32_t* hist, Launcher& L);

int pair_list_stats(const PairList& pl, uint32_t n, uint32_t* out2, Launcher& L);

}  // namespace rtp
