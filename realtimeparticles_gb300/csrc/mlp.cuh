// mlp.cuh - the warm-start network on the tensor cores (BF16 operands, FP32 accumulate).
//
// Network: 12 inputs -> 64 GELU -> 64 GELU -> 4, weights as rtp_mlp (row-major [out][in]).
// Every layer is a chain of mma.sync.m16n8k16 over 16-row tiles (a row = a particle or a
// training sample).  The weights are pre-packed by pack_mlp() into the per-lane B-fragment
// order, so a warp fetches each (n-tile, k-step) fragment with one coalesced 8-byte load per
// lane, and one layer's accumulator fragments are re-packed in registers as the next layer's
// A fragments (the m16n8 D layout of n-tiles 2k, 2k+1 is the m16k16 A layout of k-step k).
//
// Fragment layouts (PTX ISA, mma.m16n8k16 with .bf16, g = lane / 4, c = lane % 4):
//   A (16x16, row): a0 = A[g][2c..2c+1]   a1 = A[g+8][2c..2c+1]
//                   a2 = A[g][2c+8..+9]   a3 = A[g+8][2c+8..+9]
//   B (16x8, col):  b0 = B[2c..2c+1][g]   b1 = B[2c+8..2c+9][g]
//   D (16x8):       d0,d1 = D[g][2c..2c+1]   d2,d3 = D[g+8][2c..2c+1]
#pragma once

#include <cuda_bf16.h>

#include "rtp_common.cuh"

namespace rtp {

constexpr int kMlpIn = 12;
constexpr int kMlpK1 = 16;  // inputs padded to one k-step
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 4;
constexpr int kMlpH8 = kMlpHidden / 8;   // n-tiles of a hidden layer
constexpr int kMlpH16 = kMlpHidden / 16; // k-steps over a hidden layer

// Packed forward fragments: one uint2 per lane per (n-tile, k-step).
//   w1f[8 ntiles][1 kstep][32], w2f[8][4][32], w3f[1][4][32]
// Packed backward fragments (B = W itself, k = output index, n = input index):
//   w2b[8 ntiles over inputs][4 ksteps over outputs][32], w3b[8][1 kstep (4 outputs + 12 zero)][32]
// Biases are FP32.
struct MlpDev {
  const uint2* w1f;
  const uint2* w2f;
  const uint2* w3f;
  const uint2* w2b;
  const uint2* w3b;
  const float* b1;
  const float* b2;
  const float* b3;
  const float* inMean;
  const float* inScale;
  const float* outScale;
};

// Byte layout of the packed network block (one device allocation).
struct MlpLayout {
  static constexpr size_t w1f = 0;
  static constexpr size_t w2f = w1f + 8 * 1 * 32 * sizeof(uint2);
  static constexpr size_t w3f = w2f + 8 * 4 * 32 * sizeof(uint2);
  static constexpr size_t w2b = w3f + 1 * 4 * 32 * sizeof(uint2);
  static constexpr size_t w3b = w2b + 8 * 4 * 32 * sizeof(uint2);
  static constexpr size_t b1 = w3b + 8 * 1 * 32 * sizeof(uint2);
  static constexpr size_t b2 = b1 + kMlpHidden * sizeof(float);
  static constexpr size_t b3 = b2 + kMlpHidden * sizeof(float);
  static constexpr size_t inMean = b3 + 8 * sizeof(float);
  static constexpr size_t inScale = inMean + 16 * sizeof(float);
  static constexpr size_t outScale = inScale + 16 * sizeof(float);
  static constexpr size_t bytes = outScale + 8 * sizeof(float);
};

inline MlpDev mlp_dev(const void* block) {
  const char* b = (const char*)block;
  MlpDev d;
  d.w1f = (const uint2*)(b + MlpLayout::w1f);
  d.w2f = (const uint2*)(b + MlpLayout::w2f);
  d.w3f = (const uint2*)(b + MlpLayout::w3f);
  d.w2b = (const uint2*)(b + MlpLayout::w2b);
  d.w3b = (const uint2*)(b + MlpLayout::w3b);
  d.b1 = (const float*)(b + MlpLayout::b1);
  d.b2 = (const float*)(b + MlpLayout::b2);
  d.b3 = (const float*)(b + MlpLayout::b3);
  d.inMean = (const float*)(b + MlpLayout::inMean);
  d.inScale = (const float*)(b + MlpLayout::inScale);
  d.outScale = (const float*)(b + MlpLayout::outScale);
  return d;
}

// FP32 master parameters, in the order of rtp_mlp's trainable fields.
struct MlpParamOffsets {
  static constexpr int w1 = 0;
  static constexpr int b1 = w1 + kMlpHidden * kMlpIn;
  static constexpr int w2 = b1 + kMlpHidden;
  static constexpr int b2 = w2 + kMlpHidden * kMlpHidden;
  static constexpr int w3 = b2 + kMlpHidden;
  static constexpr int b3 = w3 + kMlpOut * kMlpHidden;
  static constexpr int count = b3 + kMlpOut;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half), .y = hi
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// GELU, tanh form (Hendrycks & Gimpel, 2016): 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
constexpr float kGeluA = 0.7978845608028654f;
constexpr float kGeluB = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  const float t = tanhf(kGeluA * (x + kGeluB * x * x * x));
  return 0.5f * x * (1.0f + t);
}
// d gelu / dx.
__device__ __forceinline__ float gelu_grad(float x) {
  const float t = tanhf(kGeluA * (x + kGeluB * x * x * x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGeluA * (1.0f + 3.0f * kGeluB * x * x);
}

// Layer 1 for one 16-row tile: z[nt] = A x W1^T + b1 (8 n-tiles of 16x8).
__device__ __forceinline__ void mlp_layer1(const MlpDev& m, const uint32_t (&a)[4], float (&z)[kMlpH8][4],
                                           uint32_t lane) {
  const uint32_t c = lane & 3;
#pragma unroll
  for (int nt = 0; nt < kMlpH8; ++nt) {
    const float2 bb = __ldg(reinterpret_cast<const float2*>(m.b1 + nt * 8 + 2 * c));
    z[nt][0] = bb.x;
    z[nt][1] = bb.y;
    z[nt][2] = bb.x;
    z[nt][3] = bb.y;
    mma_bf16(z[nt], a, __ldg(m.w1f + nt * 32 + lane));
  }
}

// Re-packs GELU(z) of 8 n-tiles as the 4 k-step A fragments of the next layer.
__device__ __forceinline__ void gelu_to_a(const float (&z)[kMlpH8][4], uint32_t (&a)[kMlpH16][4]) {
#pragma unroll
  for (int ks = 0; ks < kMlpH16; ++ks) {
    a[ks][0] = pack_bf16(gelu(z[2 * ks][0]), gelu(z[2 * ks][1]));
    a[ks][1] = pack_bf16(gelu(z[2 * ks][2]), gelu(z[2 * ks][3]));
    a[ks][2] = pack_bf16(gelu(z[2 * ks + 1][0]), gelu(z[2 * ks + 1][1]));
    a[ks][3] = pack_bf16(gelu(z[2 * ks + 1][2]), gelu(z[2 * ks + 1][3]));
  }
}

// Layer 2 for n-tiles [nt0, nt0 + NT): z = H1 x W2^T + b2.
template <int NT>
__device__ __forceinline__ void mlp_layer2(const MlpDev& m, const uint32_t (&h)[kMlpH16][4], int nt0,
                                           float (&z)[NT][4], uint32_t lane) {
  const uint32_t c = lane & 3;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int nt = nt0 + t;
    const float2 bb = __ldg(reinterpret_cast<const float2*>(m.b2 + nt * 8 + 2 * c));
    z[t][0] = bb.x;
    z[t][1] = bb.y;
    z[t][2] = bb.x;
    z[t][3] = bb.y;
#pragma unroll
    for (int ks = 0; ks < kMlpH16; ++ks) mma_bf16(z[t], h[ks], __ldg(m.w2f + (nt * kMlpH16 + ks) * 32 + lane));
  }
}

// Network inference for one 16-row tile whose layer-1 A fragment is `a`; returns the D
// fragment of the output layer (columns 0..3 hold the 4 outputs in network units).
// Layer 2 is done in two halves of 4 n-tiles to bound the live registers: each half's GELU
// output is the A fragment of two k-steps of layer 3.
__device__ __forceinline__ void mlp_tile_forward(const MlpDev& m, const uint32_t (&a)[4], float (&y)[4],
                                                 uint32_t lane) {
  const uint32_t c = lane & 3;
  uint32_t h1[kMlpH16][4];
  {
    float z1[kMlpH8][4];
    mlp_layer1(m, a, z1, lane);
    gelu_to_a(z1, h1);
  }
  const float2 b3 = c < 2 ? __ldg(reinterpret_cast<const float2*>(m.b3 + 2 * c)) : make_float2(0.f, 0.f);
  y[0] = b3.x;
  y[1] = b3.y;
  y[2] = b3.x;
  y[3] = b3.y;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float z2[4][4];
    mlp_layer2<4>(m, h1, half * 4, z2, lane);
#pragma unroll
    for (int k2 = 0; k2 < 2; ++k2) {
      uint32_t a3[4];
      a3[0] = pack_bf16(gelu(z2[2 * k2][0]), gelu(z2[2 * k2][1]));
      a3[1] = pack_bf16(gelu(z2[2 * k2][2]), gelu(z2[2 * k2][3]));
      a3[2] = pack_bf16(gelu(z2[2 * k2 + 1][0]), gelu(z2[2 * k2 + 1][1]));
      a3[3] = pack_bf16(gelu(z2[2 * k2 + 1][2]), gelu(z2[2 * k2 + 1][3]));
      mma_bf16(y, a3, __ldg(m.w3f + (half * 2 + k2) * 32 + lane));
    }
  }
}

// Per-warp inference over the warp's 32 rows (a row per lane).  Each lane passes its
// normalised inputs x[0..11]; on return out[0..3] holds its row's outputs in network units.
// `stage` is this warp's 32 x 9 words of shared memory.  All 32 lanes must call.
__device__ __forceinline__ void mlp_warp_forward(const MlpDev& m, const float (&x)[kMlpIn], float (&out)[kMlpOut],
                                                 uint32_t* stage) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t g = lane >> 2, c = lane & 3;
  constexpr int S = 9;  // padded row stride in words
#pragma unroll
  for (int k = 0; k < kMlpIn / 2; ++k) stage[lane * S + k] = pack_bf16(x[2 * k], x[2 * k + 1]);
  stage[lane * S + 6] = 0u;
  stage[lane * S + 7] = 0u;
  __syncwarp();
  float y[2][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const uint32_t r0 = mt * 16 + g, r1 = r0 + 8;
    uint32_t a[4];
    a[0] = stage[r0 * S + c];
    a[1] = stage[r1 * S + c];
    a[2] = stage[r0 * S + c + 4];
    a[3] = stage[r1 * S + c + 4];
    mlp_tile_forward(m, a, y[mt], lane);
  }
  __syncwarp();
  // D columns 2c, 2c+1 of rows g, g+8: outputs 0..3 live in lanes with c < 2.
  float* fs = reinterpret_cast<float*>(stage);
  if (c < 2) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const uint32_t r0 = mt * 16 + g, r1 = r0 + 8;
      fs[r0 * S + 2 * c] = y[mt][0];
      fs[r0 * S + 2 * c + 1] = y[mt][1];
      fs[r1 * S + 2 * c] = y[mt][2];
      fs[r1 * S + 2 * c + 1] = y[mt][3];
    }
  }
  __syncwarp();
#pragma unroll
  for (int o = 0; o < kMlpOut; ++o) out[o] = fs[lane * S + o];
  __syncwarp();
}

}  // namespace rtp
