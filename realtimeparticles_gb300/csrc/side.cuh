// side.cuh - headless side outputs (side.cu).
#pragma once

#include "rtp_internal.hpp"

namespace rtp {

constexpr float kFarDist = 1000000.0f;  // FAR_DIST, kernels/define.cl:9

int side_fluid_color(const float* density, uint32_t n, float restDensity, float4* col, Launcher& L);
int side_color_float(const float* q, uint32_t n, float minVal, float maxVal, float4* col, Launcher& L);
int side_camera_dist(const float4* pos, uint32_t n, uint32_t maxN, const float cam[3], uint32_t* dist, Launcher& L);
int side_grid_detector(const GridK& g, const float4* pos, uint32_t n, float* det, Launcher& L);

}  // namespace rtp
