// side.cu - headless side outputs of a step (render-only in the reference: colours, the
// camera-distance draw order, the grid occupancy detector), as device buffers.
//
// Round-to-nearest intrinsics keep every value bit-identical to the CPU evaluation.
#include "side.cuh"

namespace rtp {

// fld_fillFluidColor (fluids.cl:458-478).
__global__ void k_fluid_color(const float* __restrict__ density, uint32_t n, float restDensity,
                              float4* __restrict__ col) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 blue = f4(0.0f, 0.1f, 1.0f, 0.5f);
  const float4 lightBlue = f4(0.7f, 0.7f, 1.0f, 0.5f);
  const float4 darkBlue = f4(0.0f, 0.0f, 0.8f, 0.5f);
  const float c = __fsub_rn(1.0f, __fdiv_rn(__ldg(density + i), restDensity));
  float4 color = blue;
  if (c > 0.0f || c < 0.0f) {
    const float4 d = c > 0.0f ? f4(__fsub_rn(lightBlue.x, blue.x), __fsub_rn(lightBlue.y, blue.y),
                                   __fsub_rn(lightBlue.z, blue.z), __fsub_rn(lightBlue.w, blue.w))
                              : f4(__fsub_rn(blue.x, darkBlue.x), __fsub_rn(blue.y, darkBlue.y),
                                   __fsub_rn(blue.z, darkBlue.z), __fsub_rn(blue.w, darkBlue.w));
    color = f4(__fadd_rn(color.x, __fdiv_rn(__fmul_rn(c, d.x), 0.35f)),
               __fadd_rn(color.y, __fdiv_rn(__fmul_rn(c, d.y), 0.35f)),
               __fadd_rn(color.z, __fdiv_rn(__fmul_rn(c, d.z), 0.35f)),
               __fadd_rn(color.w, __fdiv_rn(__fmul_rn(c, d.w), 0.35f)));
  }
  col[i] = color;
}

// fillColorFloat (utils.cl): the quantity mapped to [0, 1] between minVal and maxVal, 0
// outside, as a grey level in all four channels.
__global__ void k_color_float(const float* __restrict__ q, uint32_t n, float minVal, float maxVal,
                              float4* __restrict__ col) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float v = __fdiv_rn(__fsub_rn(__ldg(q + i), minVal), __fsub_rn(maxVal, minVal));
  v = __fmul_rn(v, v < 0.0f ? 0.0f : 1.0f);  // step(0, v)
  v = __fmul_rn(v, 1.0f < v ? 0.0f : 1.0f);  // step(v, 1)
  col[i] = f4(v, v, v, v);
}

// resetCameraDist (maxNb slots) + fillCameraDist (utils.cl) for the first n slots.
__global__ void k_camera_dist(const float4* __restrict__ pos, uint32_t n, uint32_t maxN, float cx, float cy, float cz,
                              uint32_t* __restrict__ dist) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= maxN) return;
  if (i >= n) {
    dist[i] = (uint32_t)kFarDist;
    return;
  }
  const float4 p = ld4(pos + i);
  const float dx = __fsub_rn(p.x, cx), dy = __fsub_rn(p.y, cy), dz = __fsub_rn(p.z, cz);
  const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
  dist[i] = (uint32_t)fmaxf(__fsub_rn(kFarDist, __fmul_rn(len, 100.0f)), 0.0f);
}

// fillGridDetector (grid.cl:51-60): every component of an occupied cell's float8 set to 1
// (the detector was reset to 0).
__global__ void k_grid_detector(GridK g, const float4* __restrict__ pos, uint32_t n, float* __restrict__ det) {
  pdl_enter();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = cell_key(g, ld4(pos + i));
  if (c < g.nc) {
    float4* d = reinterpret_cast<float4*>(det + (size_t)c * 8);
    d[0] = f4(1.0f, 1.0f, 1.0f, 1.0f);
    d[1] = f4(1.0f, 1.0f, 1.0f, 1.0f);
  }
}

static int check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RTP_OK : cuda_fail(e, what);
}
static inline uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

int side_fluid_color(const float* density, uint32_t n, float restDensity, float4* col, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_fluid_color, dim3(blocks(n, 256)), dim3(256), density, n, restDensity, col);
  return check("k_fluid_color");
}

int side_color_float(const float* q, uint32_t n, float minVal, float maxVal, float4* col, Launcher& L) {
  if (n == 0) return RTP_OK;
  launch(L, k_color_float, dim3(blocks(n, 256)), dim3(256), q, n, minVal, maxVal, col);
  return check("k_color_float");
}

int side_camera_dist(const float4* pos, uint32_t n, uint32_t maxN, const float cam[3], uint32_t* dist, Launcher& L) {
  if (maxN == 0) return RTP_OK;
  launch(L, k_camera_dist, dim3(blocks(maxN, 256)), dim3(256), pos, n, maxN, cam[0], cam[1], cam[2], dist);
  return check("k_camera_dist");
}

int side_grid_detector(const GridK& g, const float4* pos, uint32_t n, float* det, Launcher& L) {
  RTP_CUDA(cudaMemsetAsync(det, 0, sizeof(float) * 8 * (size_t)g.nc, L.stream));  // resetGridDetector
  if (n == 0) return RTP_OK;
  launch(L, k_grid_detector, dim3(blocks(n, 256)), dim3(256), g, pos, n, det);
  return check("k_grid_detector");
}

}  // namespace rtp
