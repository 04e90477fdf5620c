// boids.cuh - boids kernel parameters and launchers (boids.cu).
#pragma once

#include "rtp_internal.hpp"

namespace rtp {

// BoidsRuleParams (kernels/boids.cl:12-17) + the bd_updateVel arguments (boids.cl:246-252).
struct BoidsK {
  float velocityScale, alignmentScale, separationScale, cohesionScale;
  float dt;           // Boids.cpp:334 hard-codes 0.1
  float maxVelocity;  // = velocityScale (Boids.cpp:217)
};

int boids_presort(const GridK& g, const float4* pos, uint32_t n, uint32_t* keys, const SortPlan& plan, uint32_t* hist0,
                  Launcher& L, const ZeroJob& zero = ZeroJob{});
int boids_rules_update(const GridK& g, const BoidsK& p, bool periodic, bool dim2, const float4* posS, const float4* velS,
                       const uint2* table, uint32_t n, const uint32_t* idsS, float4* pos, float4* vel, float4* acc,
                       uint32_t* ids, Launcher& L);

}  // namespace rtp
