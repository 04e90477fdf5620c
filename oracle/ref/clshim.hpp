// clshim.hpp - enough of OpenCL C, as C++, to compile the reference's step kernels for the
// CPU (test infrastructure: checks the oracle against the reference's own kernel code).
//
// Vector types with the operators the kernels use, .xyz on float4, the address-space
// qualifiers as no-ops, get_global_id() from a thread-local index set by the driver, and
// the builtins evaluated exactly as the oracle documents them (oracle/oracle.cpp header):
//   fast_length / length = sqrt of the 4-lane dot, normalize / fast_normalize(v) =
//   v / sqrt(dot(v, v)) with 0 -> 0, pow(x, integer y) = repeated multiplication, other pow
//   = std::pow, clamp = fmin(fmax()), step, isequal (vector form: -1 / 0 lanes), all, any.
#pragma once

#include <cmath>
#include <cstdint>

namespace clshim {

typedef unsigned int uint;
typedef unsigned long ulong;

extern thread_local uint g_global_id;
extern thread_local uint g_global_size;

inline uint get_global_id(int) { return g_global_id; }
inline uint get_global_size(int) { return g_global_size; }

struct float3 {
  float x, y, z;
};
struct int3 {
  int x, y, z;
};
struct uint3 {
  uint x, y, z;
};
struct uint2 {
  uint x, y;
};
struct float4 {
  union {
    struct {
      float x, y, z, w;
    };
    float3 xyz;
  };
};
struct float8 {
  float s[8];
  float8() = default;
  float8(float v) {
    for (int i = 0; i < 8; ++i) s[i] = v;
  }
};

inline float4 make_float4(float a, float b, float c, float d) {
  float4 r;
  r.x = a;
  r.y = b;
  r.z = c;
  r.w = d;
  return r;
}
inline float4 make_float4(float a) { return make_float4(a, a, a, a); }
inline float3 make_float3(float a, float b, float c) { return float3{a, b, c}; }
inline float3 make_float3(float a) { return float3{a, a, a}; }
inline int3 make_int3(int a, int b, int c) { return int3{a, b, c}; }
inline int3 make_int3(int a) { return int3{a, a, a}; }
inline uint2 make_uint2(uint a, uint b) { return uint2{a, b}; }
inline uint2 make_uint2(uint a) { return uint2{a, a}; }
inline float8 make_float8(float a) { return float8(a); }

// float4 arithmetic (lane-wise, left to right as written in the kernels).
inline float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator*(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator*(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator*(float4 a, int s) { return a * (float)s; }
inline float4 operator*(int s, float4 a) { return (float)s * a; }
inline float4 operator/(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4 operator/(float4 a, int s) { return a / (float)s; }
inline float4 operator-(float4 a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
inline float4& operator+=(float4& a, float4 b) { return a = a + b; }
inline float4& operator-=(float4& a, float4 b) { return a = a - b; }
inline float4& operator*=(float4& a, float s) { return a = a * s; }
inline float4& operator/=(float4& a, float s) { return a = a / s; }
inline float4& operator/=(float4& a, int s) { return a = a / s; }

inline float3 operator+(float3 a, float3 b) { return float3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return float3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(float3 a, float s) { return float3{a.x * s, a.y * s, a.z * s}; }
inline float3 operator*(float s, float3 a) { return float3{s * a.x, s * a.y, s * a.z}; }
inline float3 operator*(float3 a, float3 b) { return float3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float3 operator/(float3 a, float s) { return float3{a.x / s, a.y / s, a.z / s}; }
inline float3 operator-(float3 a, float s) { return float3{a.x - s, a.y - s, a.z - s}; }

inline int3 operator+(int3 a, int3 b) { return int3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline int3 operator%(int3 a, int3 b) { return int3{a.x % b.x, a.y % b.y, a.z % b.z}; }
inline int3 operator<(int3 a, int3 b) { return int3{a.x < b.x ? -1 : 0, a.y < b.y ? -1 : 0, a.z < b.z ? -1 : 0}; }
inline int3 operator>=(int3 a, int3 b) { return int3{a.x >= b.x ? -1 : 0, a.y >= b.y ? -1 : 0, a.z >= b.z ? -1 : 0}; }
inline int any(int3 a) { return (a.x < 0 || a.y < 0 || a.z < 0) ? 1 : 0; }
inline int all(int3 a) { return (a.x < 0 && a.y < 0 && a.z < 0) ? 1 : 0; }

inline int3 convert_int3(uint3 a) { return int3{(int)a.x, (int)a.y, (int)a.z}; }
inline uint3 convert_uint3(float3 a) { return uint3{(uint)a.x, (uint)a.y, (uint)a.z}; }

// Scalar and vector builtins.
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float3 clamp(float3 v, float3 lo, float3 hi) {
  return float3{clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y), clamp(v.z, lo.z, hi.z)};
}
inline float4 clamp(float4 v, float4 lo, float4 hi) {
  return make_float4(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y), clamp(v.z, lo.z, hi.z), clamp(v.w, lo.w, hi.w));
}
inline float4 clamp(float4 v, float lo, float hi) {
  return make_float4(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi), clamp(v.w, lo, hi));
}
inline float fabs(float x) { return std::fabs(x); }
inline float floor(float x) { return std::floor(x); }
inline float3 floor(float3 v) { return float3{std::floor(v.x), std::floor(v.y), std::floor(v.z)}; }
// exp(double) is the global ::exp (double literals in clouds.cl:98 are evaluated in double).
inline float exp(float x) { return std::exp(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }

inline float ipow(float x, long k) {
  if (k == 0) return 1.0f;
  float r = x;
  for (long i = 1; i < k; ++i) r = r * x;
  return r;
}
inline float pow(float x, float y) {
  if (y >= 0.0f && y <= 16.0f && std::floor(y) == y) return ipow(x, (long)y);
  return std::pow(x, y);
}
inline float pow(float x, int y) { return y >= 0 ? ipow(x, y) : std::pow(x, (float)y); }
inline float pow(float x, uint y) { return ipow(x, (long)y); }

inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float4 a) { return std::sqrt(dot(a, a)); }
inline float length(float3 a) { return std::sqrt(dot(a, a)); }
inline float fast_length(float4 a) { return std::sqrt(dot(a, a)); }
inline float4 normalize(float4 a) {
  const float d = dot(a, a);
  if (d == 0.0f) return a;
  return a / std::sqrt(d);
}
inline float4 fast_normalize(float4 a) { return normalize(a); }
inline float4 cross(float4 a, float4 b) {
  return make_float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
inline int isequal(float a, float b) { return a == b ? 1 : 0; }
inline int3 isequal(float3 a, float3 b) {
  return int3{a.x == b.x ? -1 : 0, a.y == b.y ? -1 : 0, a.z == b.z ? -1 : 0};
}

}  // namespace clshim

#define __kernel
#define __global
#define __local
#define __constant const
