// boids.cuh - boids kernel parameters and launchers (boids.cu).
#pragma once

#include "rtp_internal.hpp"
#include "sweep.cuh"

namespace rtp {

// BoidsRuleParams (kernels/boids.cl:12-17) + the bd_updateVel arguments (boids.cl:246-252).
struct BoidsK {
  float velocityScale, alignmentScale, separationScale, cohesionScale;
  float dt;           // Boids.cpp:334 hard-codes 0.1
  float maxVelocity;  // = velocityScale (Boids.cpp:217)
};

// TargetParams (boids.cl:19-22) and the target positions of the steps of one upload.
// track[0].x holds the step counter as bits (the keys kernel of each step adds one, from
// 0xffffffff before the first); track[1 + s] is the target of step s, w = 0.
struct TargetK {
  float4* track = nullptr;  // null: no target rule
  uint32_t cap = 0;         // positions in the track
  float radius = 0.0f;
  float sign = 0.0f;        // (float)targetSignEffect
};

// pos / vel are the canonical device buffers (written only to mirror io.inPos / io.inVel).
int boids_presort(const GridK& g, float4* pos, float4* vel, uint32_t n, uint32_t* keys, const SortPlan& plan,
                  uint32_t* hist0, Launcher& L, const ZeroJob& zero = ZeroJob{}, const TargetK& tk = TargetK{},
                  const HostIO& io = HostIO{});
int boids_rules_update(const GridK& g, const BoidsK& p, bool periodic, bool dim2, const float4* posS, const float4* velS,
                       const uint2* table, uint32_t n, const uint32_t* idsS, float4* pos, float4* vel, float4* acc,
                       uint32_t* ids, Launcher& L, const TargetK& tk = TargetK{}, const HostIO& io = HostIO{});

}  // namespace rtp
