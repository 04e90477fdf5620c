// target.cpp - boids target attractor trajectory (host).
#include "target.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>

namespace rtp {

namespace {

// Quintic fade 6t^5 - 15t^4 + 10t^3 in the Horner form of Perlin's published method.
inline float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
inline float mix(float t, float a, float b) { return a + t * (b - a); }

// Dot product of (x, y, z) with one of the 12 cube-edge gradients picked by the low four
// bits of the hash (Perlin 2002; the four extra codes repeat four of the twelve).
inline float edge_gradient(int hash, float x, float y, float z) {
  const int h = hash & 15;
  const float a = h < 8 ? x : y;
  const float b = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
  return ((h & 1) ? -a : a) + ((h & 2) ? -b : b);
}

}  // namespace

// The permutation: 0..255 shuffled by std::shuffle with std::default_random_engine(seed),
// the draw of PerlinNoise.cpp:10-25 (libstdc++ on both host architectures).
PerlinNoise3::PerlinNoise3(int seed) {
  int v[256];
  std::iota(v, v + 256, 0);
  std::default_random_engine engine(seed);
  std::shuffle(v, v + 256, engine);
  for (int i = 0; i < 256; ++i) perm_[i] = (uint8_t)v[i];
}

// Noise in [-1, 1] at (x, y, z), returned as (n + 1) / 2 (PerlinNoise.cpp:28-68): corner
// hashes p[p[p[X + i] + Y + j] + Z + k] of the unit cell, gradients blended along x, then
// y, then z with the fade weights.
float PerlinNoise3::operator()(float x, float y, float z) const {
  const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
  x -= fx;
  y -= fy;
  z -= fz;
  const float u = fade(x), v = fade(y), w = fade(z);
  float alongY[2];
  for (int k = 0; k < 2; ++k) {
    float alongX[2];
    for (int j = 0; j < 2; ++j) {
      const int h0 = p(p(p(X) + Y + j) + Z + k);
      const int h1 = p(p(p(X + 1) + Y + j) + Z + k);
      const float yj = j ? y - 1.0f : y, zk = k ? z - 1.0f : z;
      alongX[j] = mix(u, edge_gradient(h0, x, yj, zk), edge_gradient(h1, x - 1.0f, yj, zk));
    }
    alongY[k] = mix(v, alongX[0], alongX[1]);
  }
  return (mix(w, alongY[0], alongY[1]) + 1.0f) / 2.0f;
}

// Target.cpp:11-22: noises seeded 1 (theta), 29 (beta) and 246 (radius); the radius bound
// is 0.48 x the box width; position and walk start at the origin.
TargetTrajectory::TargetTrajectory(float boxWidth)
    : theta_(1), beta_(29), radius_(246), maxRadius_(0.48f * boxWidth) {}

// Target::updatePos (Target.cpp:27-50).  The angles use the reference's 3.14 for pi and its
// velocity ratio (particle velocity / 9.5); a 2D model keeps x = 0.
void TargetTrajectory::advance(bool dim3, float particlesVel) {
  constexpr float kPi = 3.14f;
  walk_[0] += 0.001f;
  walk_[1] += 0.002f;
  walk_[2] += 0.01f;
  const float nTheta = theta_(walk_[0], walk_[1], walk_[2]);
  const float nBeta = beta_(walk_[0], walk_[1], walk_[2]);
  const float nR = radius_(walk_[0], walk_[1], walk_[2]);
  const float velRatio = particlesVel / 9.5f;
  const float r = maxRadius_ * std::cos(12.0f * velRatio * kPi * nR);
  const float beta = 5.0f * velRatio * kPi * nBeta;
  const float theta = 4.0f * velRatio * kPi * nTheta;
  pos_[0] = dim3 ? r * std::cos(beta) : 0.0f;
  pos_[1] = r * std::sin(beta) * std::cos(theta);
  pos_[2] = r * std::sin(beta) * std::sin(theta);
}

}  // namespace rtp
