// clouds.cuh - clouds kernel parameters and launchers (clouds.cu).
#pragma once

#include "fluids.cuh"

namespace rtp {

// CloudParams (kernels/clouds.cl:19-33) + the environment constants of clouds.cl:72-89
// and :951-952 (rtp_cloud_env), with the ground-temperature table on the device.
struct CloudK {
  uint32_t dim;
  float dt;
  float cloudRho0;   // CloudParams.restDensity (temperature constraint)
  float cloudRelax;  // CloudParams.relaxCFM
  float groundHeat, buoyancy, gravCoeff, adiabatic, phaseRate, latent, initVapor, wind;
  int smoothing;
  float T0, lapse, heatDecay, windX, windZ;
  const float* ground;
  uint32_t nx, nz;
};

// Buffers written by the last clouds kernel.
struct CloudState {
  float4* pos;
  float4* vel;
  float *temp, *vapor, *cloud, *buoy;
  const float *tempS, *vaporS, *cloudS, *buoyS;
  uint32_t* ids;
  const uint32_t* idsS;
};

int cloud_presort(const GridK& g, const CloudK& c, const float4* pos, const float4* vel, uint32_t n, float* temp,
                  float* vapor, float* cloud, float* buoy, float4* pred, float4* tot, uint32_t* keys,
                  const SortPlan& plan, uint32_t* hist0, Launcher& L, const ZeroJob& zero = ZeroJob{});
// `packed` (one float4 per particle) carries (x, y, z, lamT), then (x, y, z, lambda), then
// (x, y, z, |omega|) from each full sweep to the list sweep after it.
int cloud_temperature(const GridK& g, const CloudK& c, const float4* posS, float* tempS, float* lamT, const uint2* table,
                      uint32_t n, const PairList& pl, Launcher& L, float4* packed);
int cloud_iteration(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, float4* totS,
                    const uint2* table, uint32_t n, float* lambda, float* density, bool last, float4* velS,
                    const PairList& pl, Launcher& L, float4* packed);
int cloud_update_vel(const GridK& g, const FluidK& p, const float4* totS, uint32_t n, float4* velS, Launcher& L);
int cloud_post(const GridK& g, const FluidK& p, const CloudK& c, const float4* pred, float4* velS, float4* vort,
               const uint2* table, uint32_t n, const CloudState& s, const PairList& pl, Launcher& L, float4* packed);
int cloud_init(const GridK& g, const CloudK& c, const float4* pos, uint32_t n, float* temp, float* vapor, float* cloud,
               float* buoy, Launcher& L);

// Defined in runtime.cu (needs the handle).
struct Handle;
int record_clouds_step(Handle* h, Launcher& L);

}  // namespace rtp
