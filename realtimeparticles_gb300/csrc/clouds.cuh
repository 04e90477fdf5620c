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
// Learned warm start of the clouds solve (clouds.cu): with feats, the plain first-iteration
// sweep that also writes every particle's features (rows of RTP_MLP_IN); without, the network
// (packed block) relaxes lambda by omega.  Both write lambda, density, packed, pairs.
int cloud_ws_lambda(const GridK& g, const FluidK& p, const CloudK& c, const float4* pred, const float4* velS,
                    const float* tempS, const float* buoyS, const uint2* table, uint32_t n, float* lambda,
                    float* density, const PairList& pl, float4* packed, float* feats, const void* mlpBlock,
                    Launcher& L);
// The correction sweep alone (cld_computeConstraintCorrection + cld_correctPosition x2 + the
// mixed boundary; last: + cld_updateVel), and the density / lambda sweep alone.
int cloud_deltap(const GridK& g, const FluidK& p, const float4* predIn, float4* predOut, float4* totS,
                 const float* lambda, const uint2* table, uint32_t n, bool last, float4* velS, const PairList& pl,
                 Launcher& L, const float4* packed);
int cloud_density(const GridK& g, const FluidK& p, const float4* pred, const uint2* table, uint32_t n, float* lambda,
                  float* density, const PairList& pl, float4* packed, Launcher& L);
// Backward sweeps of the warm start's training loss on the clouds solve (rows of RTP_MLP_OUT).
int cloud_ws_loss_grad_x(const GridK& g, const FluidK& p, const float4* xp, const float* rho2, const uint2* table,
                         uint32_t n, const PairList& pl2, float4* gOut, float* lossPart, Launcher& L);
int cloud_ws_grad_y(const GridK& g, const FluidK& p, const float4* xs, const float* lam, const float* y,
                    const float4* gIn, const uint2* table, uint32_t n, const PairList& pl, float* dy, Launcher& L);
// Per-block sums of |rho / rho0 - 1| (kSweepThreads particles per block) at pos.
int cloud_density_error(const GridK& g, const FluidK& p, const float4* pos, const uint2* table, uint32_t n,
                        float* errPartial, Launcher& L);
int cloud_post(const GridK& g, const FluidK& p, const CloudK& c, const float4* pred, float4* velS, float4* vort,
               const uint2* table, uint32_t n, const CloudState& s, const PairList& pl, Launcher& L, float4* packed);
int cloud_init(const GridK& g, const CloudK& c, const float4* pos, uint32_t n, float* temp, float* vapor, float* cloud,
               float* buoy, Launcher& L);

// Defined in runtime.cu (needs the handle).
struct Handle;
int record_clouds_step(Handle* h, Launcher& L);

}  // namespace rtp
