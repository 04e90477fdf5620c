// target.hpp - host state of the boids target attractor (target.cpp).
//
// The target moves on the host, as Physics::Target does (physics/utils/Target.cpp:27-50):
// three Perlin noises sampled along a straight line drive a position in spherical
// coordinates inside 0.48 x the box width.  Compiled with -ffp-contract=off so every
// position is the same float on x86-64 and aarch64.
#pragma once

#include <cstdint>

namespace rtp {

// Improved Perlin noise (K. Perlin, "Improving Noise", SIGGRAPH 2002) over the permutation
// the reference draws for a seed (physics/utils/PerlinNoise.cpp:10-25), mapped to [0, 1].
class PerlinNoise3 {
 public:
  explicit PerlinNoise3(int seed);
  float operator()(float x, float y, float z) const;

 private:
  uint8_t perm_[256];
  int p(int i) const { return perm_[i & 255]; }
};

class TargetTrajectory {
 public:
  explicit TargetTrajectory(float boxWidth);
  // One Target::updatePos: advances the noise coordinates and recomputes the position.
  void advance(bool dim3, float particlesVel);
  const float* pos() const { return pos_; }

 private:
  PerlinNoise3 theta_, beta_, radius_;
  float maxRadius_;
  float walk_[3] = {0.0f, 0.0f, 0.0f};
  float pos_[3] = {0.0f, 0.0f, 0.0f};
};

}  // namespace rtp
