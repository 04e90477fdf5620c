// oracle.cpp - CPU restatement of the RealTimeParticles simulation step.
//
// TEST INFRASTRUCTURE ONLY (the checker): loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU legs, never by the product.  Each function follows one reference kernel
// (physics/ocl/kernels/*.cl) or host sequence (physics/ocl/*.cpp) in the same order of
// operations, so that float results agree with the reference's kernels compiled for a CPU.
// Build: oracle/Makefile (-ffp-contract=off, OpenMP over particles).
//
// OpenCL builtins are evaluated with standard C++ math:
//   fast_length(v)   = sqrt(dot(v, v))                   (dot over all four lanes)
//   fast_normalize(v), normalize(v) = v / sqrt(dot(v, v)), and v itself when dot(v, v) == 0
//   pow(x, k) for the integer-valued exponents used here (2, 3, artPressureExp) = repeated
//                      multiplication, which keeps the sign of a negative base as pow must.
//   step(e, x) = x < e ? 0 : 1;  clamp(x, a, b) = fmin(fmax(x, a), b)
//   double literals in saturationVaporDensity (clouds.cl:98) are evaluated in double.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct f4 {
  float x, y, z, w;
};

inline f4 mk(float x, float y, float z, float w) { return f4{x, y, z, w}; }
inline f4 splat(float v) { return f4{v, v, v, v}; }
inline f4 operator+(f4 a, f4 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline f4 operator-(f4 a, f4 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline f4 operator*(f4 a, float s) { return mk(a.x * s, a.y * s, a.z * s, a.w * s); }
inline f4 operator*(float s, f4 a) { return mk(s * a.x, s * a.y, s * a.z, s * a.w); }
inline f4 operator/(f4 a, float s) { return mk(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float dot(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float flen(f4 a) { return std::sqrt(dot(a, a)); }
inline f4 fnormalize(f4 a) {
  const float d = dot(a, a);
  if (d == 0.0f) return a;
  return a / std::sqrt(d);
}
// OpenCL cross() on float4: w = 0.
inline f4 cross(f4 a, f4 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline f4 clamp4(f4 v, f4 lo, f4 hi) {
  return mk(clampf(v.x, lo.x, hi.x), clampf(v.y, lo.y, hi.y), clampf(v.z, lo.z, hi.z),
            clampf(v.w, lo.w, hi.w));
}
inline f4 clamp4s(f4 v, float lo, float hi) {
  return mk(clampf(v.x, lo, hi), clampf(v.y, lo, hi), clampf(v.z, lo, hi), clampf(v.w, lo, hi));
}
inline float stepf(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float powi(float x, uint32_t k) {
  if (k == 0) return 1.0f;
  float r = x;
  for (uint32_t i = 1; i < k; ++i) r = r * x;
  return r;
}

inline f4 ld4(const float* a, size_t i) { return mk(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]); }
inline void st4(float* a, size_t i, f4 v) {
  a[4 * i] = v.x;
  a[4 * i + 1] = v.y;
  a[4 * i + 2] = v.z;
  a[4 * i + 3] = v.w;
}

constexpr float FLOAT_EPS = 0.00000001f;    // define.cl:6
constexpr float ABS_GRAVITY_ACC_Y = 9.81f;  // define.cl:8
constexpr float PI_F = 3.1415927f;          // utils/Math.hpp:69

// Utils::FloatToStr (utils/Utils.cpp:24-28) prints a float with 10 fixed decimals; the
// OpenCL compiler parses that literal back to a float.
float round_trip(float v) {
  char buf[128];
  std::snprintf(buf, sizeof buf, "%.10f", (double)v);
  return std::strtof(buf, nullptr);
}

struct Grid {
  float W[3];
  int R[3];
  float cell;
  uint32_t nc;
  uint32_t cap;
  explicit Grid(const rtp_grid_constants* c) {
    for (int a = 0; a < 3; ++a) {
      W[a] = c->absWall[a];
      R[a] = (int)c->gridRes[a];
    }
    cell = c->cellSize;
    nc = c->numCells;
    cap = c->maxPartsInCell;
  }
  // getCell3DIndexFromPos, grid.cl:14-24.
  inline void cell3(f4 p, uint32_t out[3]) const {
    const float v[3] = {p.x, p.y, p.z};
    for (int a = 0; a < 3; ++a) {
      const float q = clampf(v[a], -W[a], W[a]) + W[a];
      out[a] = (uint32_t)std::floor(q / cell);
    }
  }
  // getCell1DIndexFromPos, grid.cl:29-38.
  inline uint32_t cell1(f4 p) const {
    uint32_t c[3];
    cell3(p, c);
    return c[0] * (uint32_t)R[2] * (uint32_t)R[1] + c[1] * (uint32_t)R[2] + c[2];
  }
};

// Neighbour loop of the fluids kernels (fluids.cl:101-123): 27 cells wrapped modulo the
// grid resolution, then every e in the cell's inclusive range.
template <class F>
inline void fluid_neighbours(const Grid& g, const uint32_t* table, f4 pos, F&& f) {
  uint32_t c3[3];
  g.cell3(pos, c3);
  const int cx = (int)c3[0], cy = (int)c3[1], cz = (int)c3[2];
  for (int iX = -1; iX <= 1; ++iX)
    for (int iY = -1; iY <= 1; ++iY)
      for (int iZ = -1; iZ <= 1; ++iZ) {
        const int nx = (cx + iX + g.R[0]) % g.R[0];
        const int ny = (cy + iY + g.R[1]) % g.R[1];
        const int nz = (cz + iZ + g.R[2]) % g.R[2];
        if (nx < 0 || ny < 0 || nz < 0 || nx >= g.R[0] || ny >= g.R[1] || nz >= g.R[2]) continue;
        const uint32_t c1 = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2] + (uint32_t)nz;
        const uint32_t s = table[2 * c1], e = table[2 * c1 + 1];
        for (uint32_t k = s; k <= e; ++k) f(k);
      }
}

// Neighbour loop of the clouds kernels (clouds.cl:326-356): x and z periodic with an image
// shift of 2W * sign, y walls (out-of-range cells skipped).
template <class F>
inline void cloud_neighbours(const Grid& g, const uint32_t* table, f4 pos, F&& f) {
  uint32_t c3[3];
  g.cell3(pos, c3);
  const int cx = (int)c3[0], cy = (int)c3[1], cz = (int)c3[2];
  for (int iX = -1; iX <= 1; ++iX)
    for (int iY = -1; iY <= 1; ++iY)
      for (int iZ = -1; iZ <= 1; ++iZ) {
        f4 sign = splat(0.0f);
        const int nx = (cx + iX + g.R[0]) % g.R[0];
        const int ny = (cy + iY + g.R[1]) % g.R[1];
        const int nz = (cz + iZ + g.R[2]) % g.R[2];
        if ((cx + iX) >= g.R[0]) sign.x = 2.0f;
        else if ((cx + iX) < 0) sign.x = -2.0f;
        if (((cy + iY) >= g.R[1]) || ((cy + iY) < 0)) continue;
        if ((cz + iZ) >= g.R[2]) sign.z = 2.0f;
        else if ((cz + iZ) < 0) sign.z = -2.0f;
        const uint32_t c1 = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2] + (uint32_t)nz;
        const uint32_t s = table[2 * c1], e = table[2 * c1 + 1];
        const f4 shift = mk(g.W[0] * sign.x, g.W[1] * sign.y, g.W[2] * sign.z, 0.0f * sign.w);
        for (uint32_t k = s; k <= e; ++k) f(k, shift);
      }
}

// Neighbour loop of the boids kernel (boids.cl:78-113): no wrap, out-of-range cells skipped.
template <class F>
inline void boid_neighbours(const Grid& g, const uint32_t* table, f4 pos, F&& f) {
  uint32_t c3[3];
  g.cell3(pos, c3);
  for (int iX = -1; iX <= 1; ++iX)
    for (int iY = -1; iY <= 1; ++iY)
      for (int iZ = -1; iZ <= 1; ++iZ) {
        const int nx = (int)c3[0] + iX, ny = (int)c3[1] + iY, nz = (int)c3[2] + iZ;
        if (nx < 0 || ny < 0 || nz < 0 || nx >= g.R[0] || ny >= g.R[1] || nz >= g.R[2]) continue;
        const uint32_t c1 = ((uint32_t)nx * g.R[1] + (uint32_t)ny) * g.R[2] + (uint32_t)nz;
        const uint32_t s = table[2 * c1], e = table[2 * c1 + 1];
        for (uint32_t k = s; k <= e; ++k) f(k);
      }
}

// Neighbour loop of the 2D boids kernel (boids.cl:167-212): the 9 cells (0, iY, iZ) around the
// particle's cell, all three indices range-checked against GRID_RES_X, and the cell index
// taken in the x = GRID_RES_X / 2 plane: (GRID_RES_X / 2 * GRID_RES_X + y) * GRID_RES_Y + z.
template <class F>
inline void boid_neighbours_2d(const Grid& g, const uint32_t* table, f4 pos, F&& f) {
  uint32_t c3[3];
  g.cell3(pos, c3);
  for (int iY = -1; iY <= 1; ++iY)
    for (int iZ = -1; iZ <= 1; ++iZ) {
      const int nx = (int)c3[0], ny = (int)c3[1] + iY, nz = (int)c3[2] + iZ;
      if (nx < 0 || ny < 0 || nz < 0 || nx >= g.R[0] || ny >= g.R[0] || nz >= g.R[0]) continue;
      const uint32_t c1 = (uint32_t)((g.R[0] / 2 * g.R[0] + ny) * g.R[1] + nz);
      const uint32_t s = table[2 * c1], e = table[2 * c1 + 1];
      for (uint32_t k = s; k <= e; ++k) f(k);
    }
}

struct Sph {
  float h, poly6c, spikyc;
  explicit Sph(const rtp_grid_constants* c) : h(c->effectRadius), poly6c(c->poly6Coeff), spikyc(c->spikyCoeff) {}
  // poly6 / poly6L, sph.cl:10-19.
  inline float poly6L(float L) const { return (1.0f - stepf(h, L)) * poly6c * powi(h * h - L * L, 3); }
  inline float poly6(f4 v) const { return poly6L(flen(v)); }
  // gradSpiky, sph.cl:26-34.
  inline f4 grad(f4 v) const {
    const float L = flen(v);
    if (L <= FLOAT_EPS) return splat(0.0f);
    return v * (1.0f - stepf(h, L)) * spikyc * -3.0f * powi(h - L, 2) / L;
  }
  // artPressure, fluids.cl:51-57 (== clouds.cl:105-111).
  inline float artPressure(f4 v, const rtp_fluid_params* p) const {
    if (p->isArtPressureEnabled == 0) return 0.0f;
    return -p->artPressureCoeff * powi(poly6(v) / poly6L(p->artPressureRadius * h), p->artPressureExp);
  }
};

#define OR_PARALLEL_FOR _Pragma("omp parallel for schedule(static)")

void sort_and_table(const rtp_grid_constants* c, uint32_t n, std::vector<uint32_t>& keys,
                    std::vector<uint32_t>& perm, uint32_t* sorted_keys_out, uint32_t* table) {
  std::vector<uint32_t> sk(n);
  perm.resize(n);
  or_stable_sort(keys.data(), n, sk.data(), perm.data());
  or_cell_table(c, sk.data(), n, table);
  if (sorted_keys_out) std::memcpy(sorted_keys_out, sk.data(), sizeof(uint32_t) * n);
  keys.swap(sk);
}

void gather4(float* a, const std::vector<uint32_t>& perm, uint32_t n) {
  if (!a) return;
  std::vector<float> t(a, a + 4 * (size_t)n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) st4(a, i, ld4(t.data(), perm[i]));
}
template <class T>
void gather1(T* a, const std::vector<uint32_t>& perm, uint32_t n) {
  if (!a) return;
  std::vector<T> t(a, a + n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) a[i] = t[perm[i]];
}

}  // namespace

extern "C" {

void or_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
  (void)n;
#endif
}

int or_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int or_derive_constants(int model, const rtp_model_params* p, rtp_grid_constants* c) {
  if (!p || !c) return RTP_ERR_INVALID_ARGUMENT;
  std::memset(c, 0, sizeof *c);
  for (int a = 0; a < 3; ++a) {
    if (p->gridRes[a] == 0 || !(p->boxSize[a] > 0.0f)) return RTP_ERR_INVALID_ARGUMENT;
    c->gridRes[a] = p->gridRes[a];
    c->absWall[a] = round_trip(p->boxSize[a] / 2.0f);  // Fluids.cpp:108-110
  }
  const float bx = p->boxSize[0];
  const float rx = (float)p->gridRes[0];
  c->cellSize = round_trip(bx / rx);  // Fluids.cpp:114
  c->numCells = p->gridRes[0] * p->gridRes[1] * p->gridRes[2];
  const float effectRadius = bx / rx;  // Fluids.cpp:104
  c->effectRadius = round_trip(effectRadius);
  c->effectRadiusSquared =
      round_trip(1.0f * bx * bx / (float)(p->gridRes[0] * p->gridRes[0]));  // Boids.cpp:104
  c->poly6Coeff = round_trip(315.0f / (64.0f * PI_F * std::pow(effectRadius, 9.f)));  // :117
  c->spikyCoeff = round_trip(15.0f / (PI_F * std::pow(effectRadius, 6.f)));           // :118
  c->maxVel = round_trip(30.0f);                                                      // :119
  uint32_t cap = p->maxNbPartsInCell;
  if (cap == 0) cap = (model == RTP_MODEL_BOIDS) ? 3000u : 100u;  // Boids.cpp:78, Fluids.cpp:79
  c->maxPartsInCell = cap;
  // Largest key: every axis at +W (grid.cl:33-35 aliases index == GRID_RES).
  Grid g(c);
  const f4 top = mk(c->absWall[0], c->absWall[1], c->absWall[2], 0.0f);
  c->keyBound = g.cell1(top) + 1u;
  uint32_t bits = 0;
  while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)c->keyBound) ++bits;
  c->keyBits = bits;
  return RTP_OK;
}

void or_fill_cell_ids(const rtp_grid_constants* c, const float* pos4, uint32_t n, uint32_t* keys) {
  const Grid g(c);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) keys[i] = g.cell1(ld4(pos4, i));
}

void or_stable_sort(const uint32_t* keys, uint32_t n, uint32_t* keys_out, uint32_t* perm) {
  std::vector<uint32_t> idx(n);
  for (uint32_t i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  for (uint32_t i = 0; i < n; ++i) {
    perm[i] = idx[i];
    keys_out[i] = keys[idx[i]];
  }
}

void or_cell_table(const rtp_grid_constants* c, const uint32_t* k, uint32_t n, uint32_t* t) {
  const uint32_t nc = c->numCells;
  // resetStartEndCell, grid.cl:91-96.
  for (uint32_t i = 0; i < nc; ++i) {
    t[2 * i] = 1;
    t[2 * i + 1] = 0;
  }
  // fillStartCell, grid.cl:101-116: ID 0 never starts a cell.
  for (uint32_t i = 1; i < n; ++i)
    if (k[i] < nc && k[i] != k[i - 1]) t[2 * k[i]] = i;
  // fillEndCell, grid.cl:121-138: index n holds an inactive sentinel key.
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t right = (i + 1 < n) ? k[i + 1] : 0xFFFFFFFFu;
    if (k[i] < nc && k[i] != right) t[2 * k[i] + 1] = i;
  }
  // adjustEndCell, grid.cl:143-152.
  for (uint32_t i = 0; i < nc; ++i) {
    const uint32_t s = t[2 * i], e = t[2 * i + 1];
    if (e > s) t[2 * i + 1] = s + std::min(e - s, c->maxPartsInCell);
  }
}

void or_fld_density(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* pred,
                    const uint32_t* table, uint32_t n, float* density) {
  (void)p;
  const Grid g(c);
  const Sph k(c);
  // fld_computeDensity, fluids.cl:80-126.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 pos = ld4(pred, i);
    float rho = 0.0f;
    fluid_neighbours(g, table, pos, [&](uint32_t e) { rho += k.poly6(pos - ld4(pred, e)); });
    density[i] = rho;
  }
}

void or_fld_lambda(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* pred,
                   const float* density, const uint32_t* table, uint32_t n, float* lambda) {
  const Grid g(c);
  const Sph k(c);
  // fld_computeConstraintFactor, fluids.cl:131-193.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 pos = ld4(pred, i);
    const float densityC = density[i] / p->restDensity - 1.0f;
    f4 sumGradCi = splat(0.0f);
    float sumSqGradC = 0.0f;
    fluid_neighbours(g, table, pos, [&](uint32_t e) {
      const f4 grad = k.grad(pos - ld4(pred, e));
      sumGradCi = sumGradCi + grad;
      sumSqGradC += dot(grad, grad);
    });
    sumSqGradC += dot(sumGradCi, sumGradCi);
    sumSqGradC /= p->restDensity * p->restDensity;
    lambda[i] = -densityC / (sumSqGradC + p->relaxCFM);
  }
}

void or_fld_correction(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* pred,
                       const float* lambda, const uint32_t* table, uint32_t n, float* corr) {
  const Grid g(c);
  const Sph k(c);
  // fld_computeConstraintCorrection, fluids.cl:198-247.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 pos = ld4(pred, i);
    const float lambdaI = lambda[i];
    f4 acc = splat(0.0f);
    fluid_neighbours(g, table, pos, [&](uint32_t e) {
      const f4 vec = pos - ld4(pred, e);
      acc = acc + (lambdaI + lambda[e] + k.artPressure(vec, p)) * k.grad(vec);
    });
    st4(corr, i, acc / p->restDensity);
  }
}

}  // extern "C"

namespace {

// Fluids.cpp:412-424: fld_predictPosition, fillCellIDs(predPos), sort of {pos, col, vel,
// predPos} (col is render-only) + ids + `extra` (one float per particle), cell table.
void fluid_presort(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t n, or_state* s,
                   std::vector<uint32_t>& table, float* extra) {
  const float dt = p->timeStep;
  float* pos = s->pos;
  float* vel = s->vel;
  float* pred = s->predPos;
  // fld_predictPosition, fluids.cl:62-74.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 gdt = mk(0.0f * dt, -ABS_GRAVITY_ACC_Y * dt, 0.0f * dt, 0.0f * dt);
    const f4 newVel = ld4(vel, i) + gdt;
    st4(pred, i, ld4(pos, i) + newVel * dt);
  }
  std::vector<uint32_t> keys(n), perm;
  or_fill_cell_ids(c, pred, n, keys.data());
  table.assign(2 * (size_t)c->numCells, 0u);
  sort_and_table(c, n, keys, perm, s->cellId, table.data());
  gather4(pos, perm, n);
  gather4(vel, perm, n);
  gather4(pred, perm, n);
  gather1(s->id, perm, n);
  gather1(extra, perm, n);
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());
}

struct Bounds {
  f4 lo, hi;
  explicit Bounds(const Grid& g)
      : lo(mk(-g.W[0] + 0.01f, -g.W[1] + 0.01f, -g.W[2] + 0.01f, 0.0f)),
        hi(mk(g.W[0] - 0.1f, g.W[1] - 0.1f, g.W[2] - 0.1f, 0.0f)) {}
};

// Jacobi loop, Fluids.cpp:427-439 (`iters` iterations on pred).  With lamTot the lambdas
// of the iterations are added to it.
void fluid_jacobi(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t iters, float* pred,
                  const uint32_t* table, uint32_t n, std::vector<float>& density, std::vector<float>& lambda,
                  float* lamTot, const float* omega = nullptr) {
  const Grid g(c);
  const Bounds b(g);
  std::vector<float> corr(4 * (size_t)n);
  for (uint32_t it = 0; it < iters; ++it) {
    // fld_applyBoundaryCondition, fluids.cl:435-439.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) st4(pred, i, clamp4(ld4(pred, i), b.lo, b.hi));
    or_fld_density(c, p, pred, table, n, density.data());
    or_fld_lambda(c, p, pred, density.data(), table, n, lambda.data());
    if (omega)  // the warm start's relaxation in every iteration (warmstart.cu, relaxAllIterations)
      for (uint32_t i = 0; i < n; ++i) lambda[i] *= omega[i];
    or_fld_correction(c, p, pred, lambda.data(), table, n, corr.data());
    // fld_correctPosition, fluids.cl:252-258.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) st4(pred, i, ld4(pred, i) + ld4(corr.data(), i));
    if (lamTot)
      for (uint32_t i = 0; i < n; ++i) lamTot[i] += lambda[i];
  }
}

// fld_updateVel (Fluids.cpp:442), vorticity confinement + XSPH (:444-454), updatePosition.
void fluid_post(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t n, or_state* s,
                const uint32_t* table) {
  const Grid g(c);
  const Sph k(c);
  const float dt = p->timeStep;
  float* pos = s->pos;
  float* vel = s->vel;
  float* pred = s->predPos;
  // fld_updateVel, fluids.cl:263-273.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i)
    st4(vel, i, clamp4s((ld4(pred, i) - ld4(pos, i)) / (dt + FLOAT_EPS), -c->maxVel, c->maxVel));

  if (p->isVorticityConfEnabled) {  // Fluids.cpp:444-454
    std::vector<float> vort(4 * (size_t)n), velIn(4 * (size_t)n);
    // fld_computeVorticity, fluids.cl:278-324.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), v = ld4(vel, i);
      f4 w = splat(0.0f);
      fluid_neighbours(g, table, x, [&](uint32_t e) { w = w + cross(ld4(vel, e) - v, k.grad(x - ld4(pred, e))); });
      st4(vort.data(), i, w);
    }
    // fld_applyVorticityConfinement, fluids.cl:329-377 (writes only vel[ID]).
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), w = ld4(vort.data(), i);
      f4 eta = splat(0.0f);
      fluid_neighbours(g, table, x, [&](uint32_t e) { eta = eta + flen(ld4(vort.data(), e)) * k.grad(x - ld4(pred, e)); });
      st4(vel, i, ld4(vel, i) + p->vorticityConfCoeff * cross(fnormalize(eta), w) * dt);
    }
    // copyBuffer(p_vel, p_velInViscosity), Fluids.cpp:451.
    std::memcpy(velIn.data(), vel, sizeof(float) * 4 * n);
    // fld_applyXsphViscosityCorrection, fluids.cl:383-430.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), v = ld4(velIn.data(), i);
      f4 visc = splat(0.0f);
      fluid_neighbours(g, table, x, [&](uint32_t e) { visc = visc + (ld4(velIn.data(), e) - v) * k.poly6(x - ld4(pred, e)); });
      st4(vel, i, v + p->xsphViscosityCoeff * visc);
    }
    if (s->vort) std::memcpy(s->vort, vort.data(), sizeof(float) * 4 * n);
  }
  // fld_updatePosition, fluids.cl:444-450.
  std::memcpy(pos, pred, sizeof(float) * 4 * n);
}

}  // namespace

extern "C" {

int or_fluids_step(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t iters,
                   uint32_t n, or_state* s) {
  if (!c || !p || !s || !s->pos || !s->vel || !s->predPos) return RTP_ERR_INVALID_ARGUMENT;
  std::vector<uint32_t> table;
  fluid_presort(c, p, n, s, table, nullptr);
  std::vector<float> density(n), lambda(n);
  fluid_jacobi(c, p, iters, s->predPos, table.data(), n, density, lambda, nullptr);
  if (s->density) std::memcpy(s->density, density.data(), sizeof(float) * n);
  if (s->lambda) std::memcpy(s->lambda, lambda.data(), sizeof(float) * n);
  fluid_post(c, p, n, s, table.data());
  return RTP_OK;
}

// ---- learned warm start (new: no reference counterpart) ---------------------------------
// Restates the GPU method of warmstart.cu / mlp.cuh / mlp_train.cu: the feature sums of the
// first lambda sweep, the network (optionally with the GPU's BF16 operand rounding), its
// loss gradient, and the warm-started step with the density-error guard.

}  // extern "C"

namespace {

// Round-to-nearest-even to bfloat16 (the upper 16 bits of an IEEE float).
inline float bf16r(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  std::memcpy(&x, &u, 4);
  return x;
}
inline double q(double v, bool emu) { return emu ? (double)bf16r((float)v) : v; }

// GELU, tanh form (Hendrycks & Gimpel 2016), and its derivative.
constexpr double kGA = 0.7978845608028654, kGB = 0.044715;
inline double gelu(double x) { return 0.5 * x * (1.0 + std::tanh(kGA * (x + kGB * x * x * x))); }
inline double gelu_grad(double x) {
  const double t = std::tanh(kGA * (x + kGB * x * x * x));
  return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * kGA * (1.0 + 3.0 * kGB * x * x);
}

struct NetD {
  const rtp_mlp* n;
  bool emu;
  // Operand copies of the weights (rounded to BF16 when emulating).
  std::vector<double> w1, w2, w3;
  NetD(const rtp_mlp* net, bool e) : n(net), emu(e), w1(64 * 12), w2(64 * 64), w3(4 * 64) {
    for (int o = 0; o < 64; ++o)
      for (int k = 0; k < 12; ++k) w1[o * 12 + k] = q(net->w1[o][k], emu);
    for (int o = 0; o < 64; ++o)
      for (int k = 0; k < 64; ++k) w2[o * 64 + k] = q(net->w2[o][k], emu);
    for (int o = 0; o < 4; ++o)
      for (int k = 0; k < 64; ++k) w3[o * 64 + k] = q(net->w3[o][k], emu);
  }
  struct Act {
    double x[12], z1[64], h1[64], z2[64], h2[64], y[4];
  };
  void forward(const float* f, Act& a) const {
    for (int k = 0; k < 12; ++k) a.x[k] = q((double)((f[k] - n->inMean[k]) * n->inScale[k]), emu);
    for (int o = 0; o < 64; ++o) {
      double z = 0.0;
      for (int k = 0; k < 12; ++k) z += a.x[k] * w1[o * 12 + k];
      a.z1[o] = z + n->b1[o];
      a.h1[o] = q(gelu(a.z1[o]), emu);
    }
    for (int o = 0; o < 64; ++o) {
      double z = 0.0;
      for (int k = 0; k < 64; ++k) z += a.h1[k] * w2[o * 64 + k];
      a.z2[o] = z + n->b2[o];
      a.h2[o] = q(gelu(a.z2[o]), emu);
    }
    for (int o = 0; o < 4; ++o) {
      double z = 0.0;
      for (int k = 0; k < 64; ++k) z += a.h2[k] * w3[o * 64 + k];
      a.y[o] = z + n->b3[o];
    }
  }
};

// The network's relaxation of the plain lambda (warmstart.cu ws_omega): 1 + tanh(y) * (2 for
// y > 0, 1 otherwise), and its derivative.
inline float ws_omega(float y) { return 1.0f + std::tanh(y) * (y > 0.0f ? 2.0f : 1.0f); }
inline double ws_omega_d(double y) { return 1.0 + std::tanh(y) * (y > 0.0 ? 2.0 : 1.0); }
inline double ws_omega_grad(double y) {
  const double t = std::tanh(y);
  return (1.0 - t * t) * (y > 0.0 ? 2.0 : 1.0);
}

// Backward of one sample through the network: G += d/dparams of sum_o dy[o] y_o (dy already
// rounded as the GPU stores it when emulating).
void mlp_backward_one(const NetD& d, const NetD::Act& a, const double dy[4], bool emu, std::vector<double>& G) {
  const int W1 = 0, B1 = W1 + 768, W2 = B1 + 64, B2 = W2 + 4096, W3 = B2 + 64, B3 = W3 + 256;
  double dz2[64], dz1[64];
  for (int h = 0; h < 64; ++h) {
    double v = 0.0;
    for (int o = 0; o < 4; ++o) v += dy[o] * d.w3[o * 64 + h];
    dz2[h] = q(v * gelu_grad(a.z2[h]), emu);
  }
  for (int h = 0; h < 64; ++h) {
    double v = 0.0;
    for (int o = 0; o < 64; ++o) v += dz2[o] * d.w2[o * 64 + h];
    dz1[h] = q(v * gelu_grad(a.z1[h]), emu);
  }
  for (int o = 0; o < 4; ++o) {
    for (int h = 0; h < 64; ++h) G[W3 + o * 64 + h] += dy[o] * a.h2[h];
    G[B3 + o] += dy[o];
  }
  for (int o = 0; o < 64; ++o) {
    for (int h = 0; h < 64; ++h) G[W2 + o * 64 + h] += dz2[o] * a.h1[h];
    G[B2 + o] += dz2[o];
    for (int k = 0; k < 12; ++k) G[W1 + o * 12 + k] += dz1[o] * a.x[k];
    G[B1 + o] += dz1[o];
  }
}

// Feature sums of particle i at x0 (warmstart.cu ws_sweep + k_ws_lambda), using the
// reference's neighbour loop and kernels.
void ws_features_one(const Grid& g, const Sph& k, const rtp_fluid_params* p, const float* x0, const float* vel,
                     const uint32_t* table, int64_t i, float lo[3], float hi[3], float* f, float* lambda0) {
  const f4 pos = ld4(x0, i), vi = ld4(vel, i);
  float rho = 0.0f, ssq = 0.0f, div = 0.0f;
  f4 sg = splat(0.0f);
  uint32_t cnt = 0;
  const float h2 = k.h * k.h;
  fluid_neighbours(g, table, pos, [&](uint32_t e) {
    const f4 v = pos - ld4(x0, e);
    rho += k.poly6(v);
    const f4 gr = k.grad(v);
    sg = sg + gr;
    ssq += dot(gr, gr);
    const float r2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if ((int64_t)e != i && r2 < h2) {
      ++cnt;
      const f4 dv = ld4(vel, e) - vi;
      div += dv.x * gr.x + dv.y * gr.y + dv.z * gr.z;
    }
  });
  const float C = rho / p->restDensity - 1.0f;
  float sq = ssq + dot(sg, sg);
  sq /= p->restDensity * p->restDensity;
  const float lam = -C / (sq + p->relaxCFM);
  const float hr = k.h / p->restDensity, invH = 1.0f / k.h;
  auto prox = [&](float x, float l, float u) {
    return std::fmin(std::fmax(2.0f - (x - l) * invH, 0.0f), 2.0f) - std::fmin(std::fmax(2.0f - (u - x) * invH, 0.0f), 2.0f);
  };
  f[0] = (float)cnt;
  f[1] = C;
  f[2] = sg.x * hr;
  f[3] = sg.y * hr;
  f[4] = sg.z * hr;
  f[5] = ssq * hr * hr;
  f[6] = div * (p->timeStep / p->restDensity);
  f[7] = prox(pos.x, lo[0], hi[0]);
  f[8] = prox(pos.y, lo[1], hi[1]);
  f[9] = prox(pos.z, lo[2], hi[2]);
  f[10] = lam;
  f[11] = std::sqrt(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * p->timeStep * invH;
  if (lambda0) *lambda0 = lam;
}

// Mean |rho / rho0 - 1| at x (fld_computeDensity with the step's table).
double mean_density_error(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* x,
                          const uint32_t* table, uint32_t n) {
  std::vector<float> rho(n);
  or_fld_density(c, p, x, table, n, rho.data());
  double s = 0.0;
  for (uint32_t i = 0; i < n; ++i) s += std::fabs(rho[i] / p->restDensity - 1.0f);
  return n ? s / n : 0.0;
}

}  // namespace

extern "C" {

void or_ws_features(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* x0, const float* vel,
                    const uint32_t* table, uint32_t n, float* feats) {
  const Grid g(c);
  const Sph k(c);
  const Bounds b(g);
  float lo[3] = {b.lo.x, b.lo.y, b.lo.z}, hi[3] = {b.hi.x, b.hi.y, b.hi.z};
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i)
    ws_features_one(g, k, p, x0, vel, table, i, lo, hi, feats + 12 * i, nullptr);
}

void or_mlp_forward(const rtp_mlp* net, const float* feats, uint64_t n, int emulate, float* out) {
  const NetD d(net, emulate != 0);
  OR_PARALLEL_FOR
  for (int64_t s = 0; s < (int64_t)n; ++s) {
    NetD::Act a;
    d.forward(feats + 12 * s, a);
    for (int o = 0; o < 4; ++o) out[4 * s + o] = (float)(a.y[o] * net->outScale[o]);
  }
}

void or_mlp_loss_grad(const rtp_mlp* net, const float* lossW, const float* feats, const float* targets, uint64_t n,
                      int emulate, double* loss, double* grad) {
  // grad: w1 (64x12), b1 (64), w2 (64x64), b2 (64), w3 (4x64), b3 (4) = 5252 doubles.
  const bool emu = emulate != 0;
  const NetD d(net, emu);
  const int NP = 5252;
  std::vector<double> G(NP, 0.0);
  double L = 0.0;
  const double invN = 1.0 / (double)n;
  for (uint64_t s = 0; s < n; ++s) {
    NetD::Act a;
    d.forward(feats + 12 * s, a);
    double dy[4];
    for (int o = 0; o < 4; ++o) {
      const double t = (double)(targets[4 * s + o] / net->outScale[o]);
      const double e = a.y[o] - t;
      L += lossW[o] * e * e;
      dy[o] = q(2.0 * lossW[o] * e * invN, emu);
    }
    mlp_backward_one(d, a, dy, emu, G);
  }
  *loss = L * invN;
  std::memcpy(grad, G.data(), sizeof(double) * NP);
}

void or_mlp_backward(const rtp_mlp* net, const float* feats, const float* dy, uint64_t n, int emulate, double* grad) {
  const bool emu = emulate != 0;
  const NetD d(net, emu);
  std::vector<double> G(5252, 0.0);
  for (uint64_t s = 0; s < n; ++s) {
    NetD::Act a;
    d.forward(feats + 12 * s, a);
    double g4[4];
    for (int o = 0; o < 4; ++o) g4[o] = q((double)dy[4 * s + o], emu);
    mlp_backward_one(d, a, g4, emu, G);
  }
  std::memcpy(grad, G.data(), sizeof(double) * G.size());
}

// Loss of the warm start through the solve and its gradient to the network's output
// (warmstart.cu k_ws_loss_grad_x, k_ws_grad_y; runtime.cu ws_train_pass), in double:
//   x* = clamp(predicted positions), sorted and tabled as the step does;
//   y = network(features at x*) (BF16 operand rounding when emulating), omega = omega(y);
//   x' = clamp(x* + dp(omega lambda)), dp as fld_computeConstraintCorrection;
//   L = 1/n sum (rho(x') / rho0 - 1)^2, rho over the 27 cells of x*'s table around x';
//   dL/dy_k = omega'(y_k) lambda_k / rho0 sum_j (g_k - g_j) . gradSpiky(x*_k - x*_j), with
//   g = dL/dx' (2 / (n rho0) sum_j (C'_m + C'_j) gradPoly6(x'_m - x'_j)), zero on a clamped
//   coordinate.  The state `s` is advanced by the presort only (sorted copies, ids).  dy and
//   omega are written at index = particle id.
int or_ws_loss_grad(const rtp_grid_constants* c, const rtp_fluid_params* p, const rtp_mlp* net, int emulate,
                    uint32_t n, or_state* s, double* loss, double* dyById, double* omegaById) {
  if (!c || !p || !net || !s || !s->pos || !s->vel || !s->predPos || !s->id || !loss) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Sph k(c);
  const Bounds b(g);
  std::vector<uint32_t> table;
  fluid_presort(c, p, n, s, table, nullptr);
  std::vector<float> x0(4 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) st4(x0.data(), i, clamp4(ld4(s->predPos, i), b.lo, b.hi));
  std::vector<float> feats(12 * (size_t)n);
  or_ws_features(c, p, x0.data(), s->vel, table.data(), n, feats.data());
  const NetD d(net, emulate != 0);
  std::vector<double> y(n), om(n), lamE(n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    NetD::Act a;
    d.forward(feats.data() + 12 * i, a);
    y[i] = a.y[0] * net->outScale[0];
    om[i] = ws_omega_d(y[i]);
    lamE[i] = om[i] * (double)feats[12 * i + 10];
  }
  const double rho0 = p->restDensity, h = k.h, h2 = h * h;
  const double lo[3] = {b.lo.x, b.lo.y, b.lo.z}, hi[3] = {b.hi.x, b.hi.y, b.hi.z};
  std::vector<double> xp(3 * (size_t)n);
  std::vector<float> xpf(4 * (size_t)n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 xi = ld4(x0.data(), i);
    double dp[3] = {0.0, 0.0, 0.0};
    fluid_neighbours(g, table.data(), xi, [&](uint32_t e) {
      const f4 v = xi - ld4(x0.data(), e);
      const f4 gr = k.grad(v);
      const double f = lamE[i] + lamE[e] + (double)k.artPressure(v, p);
      dp[0] += f * gr.x;
      dp[1] += f * gr.y;
      dp[2] += f * gr.z;
    });
    const double xi3[3] = {xi.x, xi.y, xi.z};
    for (int a = 0; a < 3; ++a) xp[3 * i + a] = std::min(std::max(xi3[a] + dp[a] / rho0, lo[a]), hi[a]);
    st4(xpf.data(), i, mk((float)xp[3 * i], (float)xp[3 * i + 1], (float)xp[3 * i + 2], 0.0f));
  }
  // rho(x') and C'.
  std::vector<double> C(n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    double rho = 0.0;
    fluid_neighbours(g, table.data(), ld4(xpf.data(), i), [&](uint32_t e) {
      double r2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        const double v = xp[3 * i + a] - xp[3 * e + a];
        r2 += v * v;
      }
      if (r2 < h2) rho += (double)k.poly6c * (h2 - r2) * (h2 - r2) * (h2 - r2);
    });
    C[i] = rho / rho0 - 1.0;
  }
  double L = 0.0;
  for (uint32_t i = 0; i < n; ++i) L += C[i] * C[i];
  *loss = L / n;
  // g = dL/dx'.
  std::vector<double> gx(3 * (size_t)n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    double acc[3] = {0.0, 0.0, 0.0};
    fluid_neighbours(g, table.data(), ld4(xpf.data(), i), [&](uint32_t e) {
      double v[3], r2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        v[a] = xp[3 * i + a] - xp[3 * e + a];
        r2 += v[a] * v[a];
      }
      if (r2 < h2) {
        const double f = (C[i] + C[e]) * (-6.0 * (double)k.poly6c * (h2 - r2) * (h2 - r2));
        for (int a = 0; a < 3; ++a) acc[a] += f * v[a];
      }
    });
    for (int a = 0; a < 3; ++a) {
      const bool held = xp[3 * i + a] == lo[a] || xp[3 * i + a] == hi[a];
      gx[3 * i + a] = held ? 0.0 : 2.0 / ((double)n * rho0) * acc[a];
    }
  }
  // dL/dy.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 xi = ld4(x0.data(), i);
    double acc = 0.0;
    fluid_neighbours(g, table.data(), xi, [&](uint32_t e) {
      const f4 gr = k.grad(xi - ld4(x0.data(), e));
      acc += (gx[3 * i] - gx[3 * e]) * gr.x + (gx[3 * i + 1] - gx[3 * e + 1]) * gr.y +
             (gx[3 * i + 2] - gx[3 * e + 2]) * gr.z;
    });
    const uint32_t id = s->id[i];
    if (dyById) dyById[id] = ws_omega_grad(y[i]) * (double)feats[12 * i + 10] / rho0 * acc;
    if (omegaById) omegaById[id] = om[i];
  }
  return RTP_OK;
}

int or_ws_step(const rtp_grid_constants* c, const rtp_fluid_params* p, const rtp_mlp* net, uint32_t extraIters,
               float guardTol, uint32_t plainIters, uint32_t n, or_state* s, float* lamTot, double* solverErr,
               int* rerun, int relaxAll) {
  if (!c || !p || !net || !s || !s->pos || !s->vel || !s->predPos || !lamTot) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Sph k(c);
  const Bounds b(g);
  std::vector<uint32_t> table;
  fluid_presort(c, p, n, s, table, nullptr);
  float* pred = s->predPos;
  // x0 = fld_applyBoundaryCondition(predPos) (the first iteration's clamp).
  std::vector<float> x0(4 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) st4(x0.data(), i, clamp4(ld4(pred, i), b.lo, b.hi));
  // Features and the network (BF16 operand rounding as on the GPU).
  std::vector<float> feats(12 * (size_t)n), out(4 * (size_t)n);
  or_ws_features(c, p, x0.data(), s->vel, table.data(), n, feats.data());
  or_mlp_forward(net, feats.data(), n, 1, out.data());
  std::vector<float> lam(n), corr(4 * (size_t)n), density(n), lambdaBuf(n), om(n);
  // The network relaxes the plain first-iteration lambda (feature 10): lambda <- omega(y) lambda.
  for (uint32_t i = 0; i < n; ++i) {
    om[i] = ws_omega(out[4 * i]);
    lam[i] = om[i] * feats[12 * (size_t)i + 10];
  }
  // x1 = x0 + dp(omega lambda); clamped when iterations follow (they start with the clamp).
  or_fld_correction(c, p, x0.data(), lam.data(), table.data(), n, corr.data());
  for (uint32_t i = 0; i < n; ++i) {
    st4(pred, i, ld4(x0.data(), i) + ld4(corr.data(), i));
    lamTot[i] = lam[i];
  }
  fluid_jacobi(c, p, extraIters, pred, table.data(), n, density, lambdaBuf, lamTot, relaxAll ? om.data() : nullptr);
  double err = mean_density_error(c, p, pred, table.data(), n);
  int rr = 0;
  if (guardTol > 0.0f && err > (double)guardTol) {
    rr = 1;
    std::memcpy(pred, x0.data(), sizeof(float) * 4 * n);
    std::fill(lamTot, lamTot + n, 0.0f);
    fluid_jacobi(c, p, plainIters, pred, table.data(), n, density, lambdaBuf, lamTot);
    err = mean_density_error(c, p, pred, table.data(), n);
  }
  if (solverErr) *solverErr = err;
  if (rerun) *rerun = rr;
  fluid_post(c, p, n, s, table.data());
  return RTP_OK;
}

int or_ws_record_step(const rtp_grid_constants* c, const rtp_fluid_params* p, uint32_t iters, uint32_t stride,
                      uint32_t phase, uint32_t n, or_state* s, float* lamTot, float* feats, float* targets,
                      uint32_t* count) {
  if (!c || !p || !s || !lamTot || stride == 0 || iters == 0) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Bounds b(g);
  std::vector<uint32_t> table;
  fluid_presort(c, p, n, s, table, nullptr);
  float* pred = s->predPos;
  std::vector<float> x0(4 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) st4(x0.data(), i, clamp4(ld4(pred, i), b.lo, b.hi));
  std::vector<float> f(12 * (size_t)n);
  or_ws_features(c, p, x0.data(), s->vel, table.data(), n, f.data());
  std::fill(lamTot, lamTot + n, 0.0f);
  std::vector<float> density(n), lambda(n);
  fluid_jacobi(c, p, iters, pred, table.data(), n, density, lambda, lamTot);
  // Targets: total lambda and xFinal - x0 - dp(total lambda) at x0.
  std::vector<float> corr(4 * (size_t)n);
  or_fld_correction(c, p, x0.data(), lamTot, table.data(), n, corr.data());
  uint32_t m = 0;
  for (uint32_t i = phase; i < n; i += stride, ++m) {
    std::memcpy(feats + 12 * (size_t)m, f.data() + 12 * (size_t)i, 12 * sizeof(float));
    const f4 d = ld4(pred, i) - (ld4(x0.data(), i) + ld4(corr.data(), i));
    targets[4 * m] = lamTot[i];
    targets[4 * m + 1] = d.x;
    targets[4 * m + 2] = d.y;
    targets[4 * m + 3] = d.z;
  }
  *count = m;
  if (s->density) std::memcpy(s->density, density.data(), sizeof(float) * n);
  if (s->lambda) std::memcpy(s->lambda, lambda.data(), sizeof(float) * n);
  fluid_post(c, p, n, s, table.data());
  return RTP_OK;
}

// ---- side outputs (render-only in the reference) -------------------------------------------

void or_fill_fluid_color(const float* density, uint32_t n, float restDensity, float* col) {
  // fld_fillFluidColor, fluids.cl:458-478.
  const f4 blue = mk(0.0f, 0.1f, 1.0f, 0.5f), lightBlue = mk(0.7f, 0.7f, 1.0f, 0.5f), darkBlue = mk(0.0f, 0.0f, 0.8f, 0.5f);
  for (uint32_t i = 0; i < n; ++i) {
    const float constraint = (1.0f - density[i] / restDensity);
    f4 color = blue;
    if (constraint > 0.0f) color = color + (constraint * (lightBlue - blue)) / 0.35f;
    else if (constraint < 0.0f) color = color + (constraint * (blue - darkBlue)) / 0.35f;
    st4(col, i, color);
  }
}

void or_fill_color_float(const float* q, uint32_t n, float minVal, float maxVal, float* col) {
  // fillColorFloat, utils.cl.
  for (uint32_t i = 0; i < n; ++i) {
    float val = (q[i] - minVal) / (maxVal - minVal);
    val *= stepf(0.0f, val);
    val *= stepf(val, 1.0f);
    st4(col, i, mk(val, val, val, val));
  }
}

void or_fill_camera_dist(const float* pos, uint32_t n, uint32_t maxN, const float cam[3], uint32_t* dist) {
  // resetCameraDist + fillCameraDist, utils.cl.
  const float FAR = 1000000.0f;  // FAR_DIST, define.cl:9
  for (uint32_t i = 0; i < maxN; ++i) {
    if (i >= n) {
      dist[i] = (uint32_t)FAR;
      continue;
    }
    const float dx = pos[4 * i] - cam[0], dy = pos[4 * i + 1] - cam[1], dz = pos[4 * i + 2] - cam[2];
    const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
    dist[i] = (uint32_t)std::fmax(FAR - len * 100.0f, 0.0f);
  }
}

void or_fill_grid_detector(const rtp_grid_constants* c, const float* pos, uint32_t n, float* det) {
  // resetGridDetector + fillGridDetector, grid.cl:43-60.
  const Grid g(c);
  std::fill(det, det + 8 * (size_t)c->numCells, 0.0f);
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t k = g.cell1(ld4(pos, i));
    if (k < c->numCells) std::fill(det + 8 * (size_t)k, det + 8 * (size_t)k + 8, 1.0f);
  }
}

void or_fluid_metrics(const rtp_grid_constants* c, const rtp_fluid_params* p, const float* pred,
                      const float* vel, const uint32_t* table, uint32_t n, rtp_metrics* m) {
  std::memset(m, 0, sizeof *m);
  if (n == 0) return;
  const Grid g(c);
  const Sph k(c);
  std::vector<float> rho(n);
  std::vector<uint32_t> nb(n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 x = ld4(pred, i);
    float r = 0.0f;
    uint32_t cnt = 0;
    fluid_neighbours(g, table, x, [&](uint32_t e) {
      const f4 v = x - ld4(pred, e);
      r += k.poly6(v);
      if ((int64_t)e != i && flen(v) < k.h) ++cnt;
    });
    rho[i] = r;
    nb[i] = cnt;
  }
  double sum = 0.0, mx = 0.0, ke = 0.0, nsum = 0.0, comp = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    const double cdev = (double)rho[i] / (double)p->restDensity - 1.0;
    const double err = std::fabs(cdev);
    sum += err;
    comp += std::max(cdev, 0.0);
    mx = std::max(mx, err);
    const f4 v = ld4(vel, i);
    ke += 0.5 * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
    nsum += nb[i];
    m->neighbourHist[std::min<uint32_t>(nb[i], 63)]++;
  }
  m->meanDensityError = sum / n;
  m->maxDensityError = mx;
  m->kineticEnergy = ke;
  m->meanNeighbours = nsum / n;
  m->meanCompression = comp / n;
}

int or_boids_step(const rtp_grid_constants* c, const rtp_boids_params* p, float dt, int boundary,
                  uint32_t n, or_state* s) {
  return or_boids_step_target(c, p, dt, boundary, 3, nullptr, 0.0f, 0, n, s);
}

int or_boids_step_dim(const rtp_grid_constants* c, const rtp_boids_params* p, float dt, int boundary, int dim,
                      uint32_t n, or_state* s) {
  return or_boids_step_target(c, p, dt, boundary, dim, nullptr, 0.0f, 0, n, s);
}

// Physics::PerlinNoise (PerlinNoise.cpp:10-85): Perlin's improved noise over the permutation
// of 0..255 that std::shuffle draws with std::default_random_engine(seed), mapped to [0, 1].
float or_perlin_noise(int seed, float x, float y, float z) {
  std::vector<int> perm(256);
  std::iota(perm.begin(), perm.end(), 0);
  std::default_random_engine engine(seed);
  std::shuffle(perm.begin(), perm.end(), engine);
  perm.insert(perm.end(), perm.begin(), perm.end());
  auto fade = [](float t) { return t * t * t * (t * (t * 6 - 15) + 10); };
  auto lerp = [](float t, float a, float b) { return a + t * (b - a); };
  auto grad = [](int hash, float gx, float gy, float gz) {
    const int h = hash & 15;
    const float u = h < 8 ? gx : gy;
    const float v = h < 4 ? gy : (h == 12 || h == 14) ? gx : gz;
    return ((h & 1) == 0 ? u : -u) + ((h & 2) == 0 ? v : -v);
  };
  const int X = (int)std::floor(x) & 255, Y = (int)std::floor(y) & 255, Z = (int)std::floor(z) & 255;
  x -= std::floor(x);
  y -= std::floor(y);
  z -= std::floor(z);
  const float u = fade(x), v = fade(y), w = fade(z);
  const int A = perm[X] + Y, AA = perm[A] + Z, AB = perm[A + 1] + Z;
  const int B = perm[X + 1] + Y, BA = perm[B] + Z, BB = perm[B + 1] + Z;
  const float z0 = lerp(v, lerp(u, grad(perm[AA], x, y, z), grad(perm[BA], x - 1, y, z)),
                        lerp(u, grad(perm[AB], x, y - 1, z), grad(perm[BB], x - 1, y - 1, z)));
  const float z1 = lerp(v, lerp(u, grad(perm[AA + 1], x, y, z - 1), grad(perm[BA + 1], x - 1, y, z - 1)),
                        lerp(u, grad(perm[AB + 1], x, y - 1, z - 1), grad(perm[BB + 1], x - 1, y - 1, z - 1)));
  return (lerp(w, z0, z1) + 1.0f) / 2.0f;
}

// Target::updatePos (Target.cpp:27-50) nsteps times from a new Target (Target.cpp:11-22,
// box width boxWidth): out[3 * s + k] = coordinate k after step s.
void or_target_trajectory(float boxWidth, int dim, float particlesVel, uint32_t nsteps, float* out) {
  const float maxRadius = 0.48f * boxWidth;
  float px = 0.0f, py = 0.0f, pz = 0.0f;
  const float PI = 3.14f;
  for (uint32_t s = 0; s < nsteps; ++s) {
    px += 0.001f;
    py += 0.002f;
    pz += 0.01f;
    const float nTheta = or_perlin_noise(1, px, py, pz);
    const float nBeta = or_perlin_noise(29, px, py, pz);
    const float nR = or_perlin_noise(246, px, py, pz);
    const float velRatio = particlesVel / 9.5f;
    const float radius = maxRadius * std::cos(12 * velRatio * PI * nR);
    out[3 * s + 0] = dim == 3 ? radius * std::cos(5 * velRatio * PI * nBeta) : 0.0f;
    out[3 * s + 1] = radius * std::sin(5 * velRatio * PI * nBeta) * std::cos(4 * velRatio * PI * nTheta);
    out[3 * s + 2] = radius * std::sin(5 * velRatio * PI * nBeta) * std::sin(4 * velRatio * PI * nTheta);
  }
}

int or_boids_step_target(const rtp_grid_constants* c, const rtp_boids_params* p, float dt, int boundary, int dim,
                         const float* target, float targetRadius, int targetSign, uint32_t n, or_state* s) {
  if (!c || !p || !s || !s->pos || !s->vel || (dim != 2 && dim != 3)) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  float* pos = s->pos;
  float* vel = s->vel;
  // fillCellIDs(pos), Boids.cpp:335; sort {pos, col, vel, acc} (:337); table (:339-344).
  std::vector<uint32_t> keys(n), perm;
  or_fill_cell_ids(c, pos, n, keys.data());
  std::vector<uint32_t> table(2 * (size_t)c->numCells);
  sort_and_table(c, n, keys, perm, s->cellId, table.data());
  gather4(pos, perm, n);
  gather4(vel, perm, n);
  gather1(s->id, perm, n);
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());

  std::vector<float> acc(4 * (size_t)n);
  const float R2 = c->effectRadiusSquared;
  // bd_applyBoidsRulesWithGrid3D, boids.cl:46-132 (2D: bd_applyBoidsRulesWithGrid2D, :137-221;
  // Boids.cpp:346-349 picks it when the model is 2D).
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 x = ld4(pos, i);
    int count = 0;
    f4 newAcc = splat(0.0f), avgPos = splat(0.0f), avgVel = splat(0.0f), repulse = splat(0.0f);
    auto rule = [&](uint32_t e) {
      const f4 posN = ld4(pos, e);
      const f4 vec = x - posN;
      const float sq = dot(vec, vec);
      if (sq < R2 && sq > FLOAT_EPS) {
        avgPos = avgPos + posN;
        avgVel = avgVel + fnormalize(ld4(vel, e));
        repulse = repulse + vec / sq;
        ++count;
      }
    };
    if (dim == 2)
      boid_neighbours_2d(g, table.data(), x, rule);
    else
      boid_neighbours(g, table.data(), x, rule);
    if (count != 0) {
      avgPos = avgPos / (float)count;
      avgPos = avgPos - x;
      avgPos = fnormalize(avgPos) * p->velocityScale;
      avgVel = fnormalize(avgVel) * p->velocityScale;
      repulse = fnormalize(repulse) * p->velocityScale;
      newAcc = avgVel * p->alignmentScale + repulse * p->separationScale + avgPos * p->cohesionScale;
    }
    st4(acc.data(), i, newAcc);
  }
  if (target) {
    // bd_addTargetRule, boids.cl:226-241 (Boids.cpp:351-358): target w = 0.
    const f4 tp = mk(target[0], target[1], target[2], 0.0f);
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 vec = tp - ld4(pos, i);
      const float dist = flen(vec);
      if (dist < targetRadius)
        st4(acc.data(), i, ld4(acc.data(), i) + ((float)targetSign * vec) * clampf(1.3f / dist, 0.0f, 1.4f * 0.5f));
    }
  }
  // bd_updateVel, boids.cl:246-259 (maxVelocity = velocityScale, Boids.cpp:217).
  const float vmax = p->velocityScale;
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 nv = ld4(vel, i) + ld4(acc.data(), i) * dt;
    const float norm = clampf(flen(nv), 0.2f * vmax, vmax);
    st4(vel, i, fnormalize(nv) * norm);
  }
  const f4 lo = mk(-g.W[0], -g.W[1], -g.W[2], 0.0f), hi = mk(g.W[0], g.W[1], g.W[2], 0.0f);
  if (boundary == RTP_BOUNDARY_CYCLIC_WALL) {
    // bd_updatePosAndApplyPeriodicBC, boids.cl:289-315.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 np = ld4(pos, i) + ld4(vel, i) * dt;
      f4 cp = clamp4(np, lo, hi);
      if (!(cp.x == np.x)) cp.x *= -1.0f;
      if (!(cp.y == np.y)) cp.y *= -1.0f;
      if (!(cp.z == np.z)) cp.z *= -1.0f;
      st4(pos, i, cp);
    }
  } else {
    // bd_updatePosAndApplyWallBC, boids.cl:264-284.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 np = ld4(pos, i) + ld4(vel, i) * dt;
      const f4 cp = clamp4(np, lo, hi);
      st4(pos, i, cp);
      if (!(cp.x == np.x && cp.y == np.y && cp.z == np.z)) st4(vel, i, ld4(vel, i) * -0.5f);
    }
  }
  if (s->acc) std::memcpy(s->acc, acc.data(), sizeof(float) * 4 * n);
  return RTP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Clouds (clouds.cl, Clouds.cpp:503-610).
namespace {

struct CloudEnv {
  float W[3];
  float T0, lapse, heatDecay, windX, windZ;
  const float* ground;
  uint32_t nx, nz;
  CloudEnv(const rtp_grid_constants* c, const rtp_cloud_env* e, const float* g) {
    for (int a = 0; a < 3; ++a) W[a] = c->absWall[a];
    T0 = e->groundTemp0;
    lapse = e->lapseRate;
    heatDecay = e->heatDecay;
    windX = e->windDecayX;
    windZ = e->windDecayZ;
    ground = (g && e->groundNx >= 2 && e->groundNz >= 2) ? g : nullptr;
    nx = e->groundNx;
    nz = e->groundNz;
  }
  // Ground temperature at (x, z): bilinear in a nx x nz table spanning the box floor.
  inline float groundTemp(float x, float z) const {
    if (!ground) return T0;
    const float u = clampf((x + W[0]) / (2.0f * W[0]), 0.0f, 1.0f) * (float)(nx - 1);
    const float v = clampf((z + W[2]) / (2.0f * W[2]), 0.0f, 1.0f) * (float)(nz - 1);
    const uint32_t i0 = std::min((uint32_t)std::floor(u), nx - 2);
    const uint32_t k0 = std::min((uint32_t)std::floor(v), nz - 2);
    const float fu = u - (float)i0, fv = v - (float)k0;
    const float a = ground[i0 * nz + k0], b = ground[i0 * nz + k0 + 1];
    const float cc = ground[(i0 + 1) * nz + k0], d = ground[(i0 + 1) * nz + k0 + 1];
    const float ab = a + (b - a) * fv;
    const float cd = cc + (d - cc) * fv;
    return ab + (cd - ab) * fu;
  }
  // environmentTemp, clouds.cl:80-89.
  inline float envTemp(f4 p) const { return -lapse * (p.y + W[1]) + groundTemp(p.x, p.z); }
  // externalHeatSource, clouds.cl:72-75.
  inline float heatSource(float alt) const { return clampf(std::exp(-(alt + W[1]) / heatDecay), 0.0f, 1.0f); }
};

// saturationVaporDensity, clouds.cl:94-99 (double literals -> double arithmetic).
inline float qsat(float T) { return (float)(217 * std::exp(19.5 - 4303.4 / ((double)T - 29.5)) / (double)T); }

// cld_applyMixedBoundaryConditions, clouds.cl:279-299.
inline f4 mixed_bc(const Grid& g, f4 np) {
  const f4 cp = clamp4(np, mk(-g.W[0], -g.W[1], -g.W[2], 0.0f), mk(g.W[0], g.W[1], g.W[2], 0.0f));
  f4 r = np;
  if (std::fabs(np.x) > g.W[0]) r.x = np.x - 2 * cp.x;
  if (std::fabs(np.y) > g.W[1]) r.y = cp.y;
  if (std::fabs(np.z) > g.W[2]) r.z = np.z - 2 * cp.z;
  return r;
}

}  // namespace

extern "C" {

void or_clouds_init(const rtp_grid_constants* c, const rtp_cloud_params* cp, const rtp_cloud_env* env,
                    const float* ground, uint32_t n, or_state* s) {
  const CloudEnv E(c, env, ground);
  for (uint32_t i = 0; i < n; ++i) {
    const f4 p = ld4(s->pos, i);
    s->temp[i] = E.envTemp(p);                                  // cld_initTemperature
    s->vapor[i] = cp->initVaporDensityCoeff * qsat(s->temp[i]);  // cld_initVaporDensity
    s->cloud[i] = 0.0f;                                          // Clouds.cpp:487-488
    if (s->buoyancy) s->buoyancy[i] = 0.0f;
  }
}

}  // extern "C"

namespace {

bool clouds_state_ok(const or_state* s) {
  return s && s->pos && s->vel && s->predPos && s->totCorrPos && s->temp && s->vapor && s->cloud && s->buoyancy;
}

// Clouds.cpp:516-567: thermodynamics, predicted positions under the mixed boundary, the sort
// of every particle array by cell and the temperature smoothing.  `table` is the step's cell
// table.
void clouds_presort(const rtp_grid_constants* c, const rtp_cloud_params* cp, const CloudEnv& E, uint32_t n,
                    or_state* s, std::vector<uint32_t>& table) {
  const Grid g(c);
  const Sph k(c);
  float* pos = s->pos;
  float* vel = s->vel;
  float* pred = s->predPos;
  float* tot = s->totCorrPos;
  float* temp = s->temp;
  float* vapor = s->vapor;
  float* cloud = s->cloud;
  float* buoy = s->buoyancy;
  const float dt = cp->timeStep;

  // Thermodynamics, Clouds.cpp:516-529.
  std::vector<float> tempIn(temp, temp + n), cloudGen(n);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 p = ld4(pos, i);
    // cld_heatFromGround, clouds.cl:159-168.
    temp[i] = std::fmin(tempIn[i] + E.heatSource(p.y) * cp->groundHeatCoeff * dt, 313.0f);
    // cld_computeBuoyancy, clouds.cl:173-184.
    const float envT = E.envTemp(p);
    buoy[i] = cp->buoyancyCoeff * (temp[i] - envT) / envT - cp->gravCoeff * ABS_GRAVITY_ACC_Y * cloud[i];
    // cld_applyAdiabaticCooling, clouds.cl:189-198.
    tempIn[i] = std::fmax(temp[i] - cp->adiabaticLapseRate * ld4(vel, i).y * dt, 223.0f);
    // cld_generateCloud, clouds.cl:207-221.
    cloudGen[i] = cp->phaseTransitionRate * (vapor[i] - qsat(tempIn[i]));
    // cld_applyPhaseTransition, clouds.cl:226-238 (inputs are copies, Clouds.cpp:525-526).
    const float cIn = cloud[i], vIn = vapor[i];
    cloud[i] = std::fmax(cIn + cloudGen[i] * dt, 0.0f);
    vapor[i] = std::fmax(vIn - cloudGen[i] * dt, 0.0f);
    // cld_applyLatentHeat, clouds.cl:243-252.
    temp[i] = tempIn[i] + std::fmax(cp->latentHeatCoeff * cloudGen[i] * dt, 0.0f);
  }
  // cld_predictPosition, clouds.cl:257-273, then the mixed BC (Clouds.cpp:534-538).
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 predVel = ld4(vel, i) + mk(0.0f, buoy[i], 0.0f, 0.0f) * dt;
    st4(tot, i, predVel * dt);
    st4(pred, i, mixed_bc(g, ld4(pos, i) + predVel * dt));
  }
  // fillCellIDs + sort {pos, col, vel, predPos, totCorrPos}, {temp, buoyancy, vapor,
  // cloud, partID} (Clouds.cpp:541-543), table (:545-550).
  std::vector<uint32_t> keys(n), perm;
  or_fill_cell_ids(c, pred, n, keys.data());
  table.assign(2 * (size_t)c->numCells, 0u);
  sort_and_table(c, n, keys, perm, s->cellId, table.data());
  gather4(pos, perm, n);
  gather4(vel, perm, n);
  gather4(pred, perm, n);
  gather4(tot, perm, n);
  gather1(temp, perm, n);
  gather1(buoy, perm, n);
  gather1(vapor, perm, n);
  gather1(cloud, perm, n);
  gather1(s->id, perm, n);
  if (s->table) std::memcpy(s->table, table.data(), sizeof(uint32_t) * table.size());
  const uint32_t* T = table.data();

  if (cp->isTempSmoothingEnabled) {  // Clouds.cpp:554-567, on p_pos
    std::vector<float> lap(n), lamT(n);
    // cld_computeLaplacianTemp, clouds.cl:508-569.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pos, i);
      const float Ti = temp[i];
      float l = 0.0f;
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        const f4 vec = x - ld4(pos, e) - sh;
        l += (Ti - temp[e]) * dot(vec, k.grad(vec)) / (dot(vec, vec) + FLOAT_EPS);
      });
      lap[i] = l / cp->restDensity;
    }
    // cld_computeConstraintFactorTemp, clouds.cl:575-648.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pos, i);
      float sumG = 0.0f, sumSq = 0.0f;
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        const f4 vec = x - ld4(pos, e) - sh;
        const f4 gr = k.grad(vec);
        const float d = dot(vec, gr) / (dot(vec, vec) * cp->restDensity + FLOAT_EPS);
        sumG += d;
        sumSq += d * d;
      });
      sumSq += sumG * sumG;
      lamT[i] = -lap[i] / (sumSq + cp->relaxCFM);
    }
    // cld_computeConstraintCorrectionTemp, clouds.cl:654-722, cld_correctTemperature :931-937.
    std::vector<float> corrT(n);
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pos, i);
      const float li = lamT[i];
      float cr = 0.0f;
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        const f4 vec = x - ld4(pos, e) - sh;
        const f4 gr = k.grad(vec);
        const float d = dot(vec, gr) / (dot(vec, vec) * cp->restDensity + FLOAT_EPS);
        cr += (li + lamT[e]) * d;
      });
      corrT[i] = cr;
    }
    for (uint32_t i = 0; i < n; ++i) temp[i] += 0.3f * corrT[i];
  }
}

// cld_computeDensity (clouds.cl:305-360) and cld_computeConstraintFactor (:365-436) at pred.
void cloud_lambda(const Grid& g, const Sph& k, const rtp_fluid_params* fp, const float* pred, const uint32_t* T,
                  uint32_t n, float* density, float* lambda) {
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 x = ld4(pred, i);
    float rho = 0.0f;
    cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) { rho += k.poly6(x - ld4(pred, e) - sh); });
    density[i] = rho;
  }
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 x = ld4(pred, i);
    const float densityC = density[i] / fp->restDensity - 1.0f;
    f4 sg = splat(0.0f);
    float sq = 0.0f;
    cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
      const f4 gr = k.grad(x - ld4(pred, e) - sh);
      sg = sg + gr;
      sq += dot(gr, gr);
    });
    sq += dot(sg, sg);
    sq /= fp->restDensity * fp->restDensity;
    lambda[i] = -densityC / (sq + fp->relaxCFM);
  }
}

// cld_computeConstraintCorrection (clouds.cl:441-502), then cld_correctPosition on predPos
// and totCorrPos and the mixed boundary (Clouds.cpp:579-586).
void cloud_correct(const Grid& g, const Sph& k, const rtp_fluid_params* fp, float* pred, float* tot,
                   const float* lambda, const uint32_t* T, uint32_t n, float* corr) {
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 x = ld4(pred, i);
    const float li = lambda[i];
    f4 a = splat(0.0f);
    cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
      const f4 vec = x - ld4(pred, e) - sh;
      a = a + (li + lambda[e] + k.artPressure(vec, fp)) * k.grad(vec);
    });
    st4(corr, i, a / fp->restDensity);
  }
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const f4 cr = ld4(corr, i);
    st4(pred, i, ld4(pred, i) + cr);
    st4(tot, i, ld4(tot, i) + cr);
    st4(pred, i, mixed_bc(g, ld4(pred, i)));
  }
}

// The Jacobi loop of Clouds.cpp:570-587; density and lambda keep the last sweep's values.
void cloud_jacobi(const Grid& g, const Sph& k, const rtp_fluid_params* fp, uint32_t iters, float* pred, float* tot,
                  const uint32_t* T, uint32_t n, std::vector<float>& density, std::vector<float>& lambda) {
  std::vector<float> corr(4 * (size_t)n);
  for (uint32_t it = 0; it < iters; ++it) {
    cloud_lambda(g, k, fp, pred, T, n, density.data(), lambda.data());
    cloud_correct(g, k, fp, pred, tot, lambda.data(), T, n, corr.data());
  }
}

// Clouds.cpp:590-610: velocities from the total correction, vorticity confinement and XSPH
// viscosity, the wind drift into the new positions.
void clouds_post(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                 const CloudEnv& E, uint32_t n, or_state* s, const uint32_t* T) {
  const Grid g(c);
  const Sph k(c);
  float* pos = s->pos;
  float* vel = s->vel;
  const float* pred = s->predPos;
  const float* tot = s->totCorrPos;
  const float fdt = fp->timeStep;
  // cld_updateVel, clouds.cl:958-966.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i)
    st4(vel, i, clamp4s(ld4(tot, i) / (fdt + FLOAT_EPS), -c->maxVel, c->maxVel));

  if (fp->isVorticityConfEnabled) {  // Clouds.cpp:592-602
    std::vector<float> vort(4 * (size_t)n), velIn(4 * (size_t)n);
    // cld_computeVorticity, clouds.cl:727-785.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), v = ld4(vel, i);
      f4 w = splat(0.0f);
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        w = w + cross(ld4(vel, e) - v, k.grad(x - ld4(pred, e) - sh));
      });
      st4(vort.data(), i, w);
    }
    // cld_applyVorticityConfinement, clouds.cl:790-850.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), w = ld4(vort.data(), i);
      f4 eta = splat(0.0f);
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        eta = eta + flen(ld4(vort.data(), e)) * k.grad(x - ld4(pred, e) - sh);
      });
      st4(vel, i, ld4(vel, i) + fp->vorticityConfCoeff * cross(fnormalize(eta), w) * fdt);
    }
    std::memcpy(velIn.data(), vel, sizeof(float) * 4 * n);
    // cld_applyXsphViscosityCorrection, clouds.cl:856-915.
    OR_PARALLEL_FOR
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      const f4 x = ld4(pred, i), v = ld4(velIn.data(), i);
      f4 visc = splat(0.0f);
      cloud_neighbours(g, T, x, [&](uint32_t e, f4 sh) {
        visc = visc + (ld4(velIn.data(), e) - v) * k.poly6(x - ld4(pred, e) - sh);
      });
      st4(vel, i, v + fp->xsphViscosityCoeff * visc);
    }
    if (s->vort) std::memcpy(s->vort, vort.data(), sizeof(float) * 4 * n);
  }
  // cld_updatePosition, clouds.cl:942-953.
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    f4 p = ld4(pred, i);
    const float alt = p.y + g.W[1];
    p.x += (1 - std::exp(-alt * E.windX)) * cp->windCoeff * cp->timeStep * (float)(cp->dim - 2);
    p.z += (1 - std::exp(-alt * E.windZ)) * 0.7f * cp->windCoeff * cp->timeStep;
    st4(pos, i, p);
  }
}

// Feature sums of the clouds warm start for particle i at x0 (clouds.cu k_cloud_ws_lambda):
// the neighbour count (self excluded, periodic images included), C, h/rho0 sum gradW,
// (h/rho0)^2 sum |gradW|^2, dt/rho0 sum (v_j - v_i).gradW, the buoyancy's displacement
// b dt^2 / h, the y-wall proximity, (T - T_env) / 10, the plain lambda and |v| dt / h.
void cloud_ws_features_one(const Grid& g, const Sph& k, const rtp_fluid_params* p, const CloudEnv& E,
                           const float* x0, const float* vel, const float* temp, const float* buoy,
                           const uint32_t* T, int64_t i, float* f) {
  const f4 pos = ld4(x0, i), vi = ld4(vel, i);
  float rho = 0.0f, ssq = 0.0f, div = 0.0f;
  f4 sg = splat(0.0f);
  uint32_t cnt = 0;
  const float h2 = k.h * k.h;
  cloud_neighbours(g, T, pos, [&](uint32_t e, f4 sh) {
    const f4 v = pos - ld4(x0, e) - sh;
    rho += k.poly6(v);
    const f4 gr = k.grad(v);
    sg = sg + gr;
    ssq += dot(gr, gr);
    const float r2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (((int64_t)e != i || sh.x != 0.0f || sh.z != 0.0f) && r2 < h2) {
      ++cnt;
      const f4 dv = ld4(vel, e) - vi;
      div += dv.x * gr.x + dv.y * gr.y + dv.z * gr.z;
    }
  });
  const float C = rho / p->restDensity - 1.0f;
  float sq = ssq + dot(sg, sg);
  sq /= p->restDensity * p->restDensity;
  const float hr = k.h / p->restDensity, invH = 1.0f / k.h;
  f[0] = (float)cnt;
  f[1] = C;
  f[2] = sg.x * hr;
  f[3] = sg.y * hr;
  f[4] = sg.z * hr;
  f[5] = ssq * hr * hr;
  f[6] = div * (p->timeStep / p->restDensity);
  f[7] = buoy[i] * p->timeStep * p->timeStep * invH;
  f[8] = std::fmin(std::fmax(2.0f - (pos.y + g.W[1]) * invH, 0.0f), 2.0f) -
         std::fmin(std::fmax(2.0f - (g.W[1] - pos.y) * invH, 0.0f), 2.0f);
  f[9] = (temp[i] - E.envTemp(pos)) * 0.1f;
  f[10] = -C / (sq + p->relaxCFM);
  f[11] = std::sqrt(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z) * p->timeStep * invH;
}

}  // namespace

extern "C" {

int or_clouds_step(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                   const rtp_cloud_env* env, const float* ground, uint32_t iters, uint32_t n,
                   or_state* s) {
  if (!c || !fp || !cp || !env || !clouds_state_ok(s)) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Sph k(c);
  const CloudEnv E(c, env, ground);
  std::vector<uint32_t> table;
  clouds_presort(c, cp, E, n, s, table);
  std::vector<float> density(n), lambda(n);
  cloud_jacobi(g, k, fp, iters, s->predPos, s->totCorrPos, table.data(), n, density, lambda);
  if (s->density) std::memcpy(s->density, density.data(), sizeof(float) * n);
  if (s->lambda) std::memcpy(s->lambda, lambda.data(), sizeof(float) * n);
  clouds_post(c, fp, cp, E, n, s, table.data());
  return RTP_OK;
}

void or_clouds_ws_features(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_env* env,
                           const float* ground, const float* x0, const float* vel, const float* temp,
                           const float* buoy, const uint32_t* table, uint32_t n, float* feats) {
  const Grid g(c);
  const Sph k(c);
  const CloudEnv E(c, env, ground);
  OR_PARALLEL_FOR
  for (int64_t i = 0; i < (int64_t)n; ++i)
    cloud_ws_features_one(g, k, fp, E, x0, vel, temp, buoy, table, i, feats + 12 * i);
}

// The training loss of the clouds warm start (runtime.cu cloud_train_pass): after the step's
// presort, L = mean (rho(x') / rho0 - 1)^2 at x' = the relaxed first correction of x* under
// the mixed boundary, with the step's cell table.  s advances through the presort.
int or_clouds_ws_loss(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                      const rtp_cloud_env* env, const float* ground, const rtp_mlp* net, int emulate, uint32_t n,
                      or_state* s, double* loss, float* featsOut) {
  if (!c || !fp || !cp || !env || !net || !loss || !clouds_state_ok(s)) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Sph k(c);
  const CloudEnv E(c, env, ground);
  std::vector<uint32_t> table;
  clouds_presort(c, cp, E, n, s, table);
  std::vector<float> feats(12 * (size_t)n), out(4 * (size_t)n), lam(n), corr(4 * (size_t)n), rho(n), lamOut(n);
  or_clouds_ws_features(c, fp, env, ground, s->predPos, s->vel, s->temp, s->buoyancy, table.data(), n, feats.data());
  or_mlp_forward(net, feats.data(), n, emulate, out.data());
  for (uint32_t i = 0; i < n; ++i) lam[i] = ws_omega(out[4 * (size_t)i]) * feats[12 * (size_t)i + 10];
  cloud_correct(g, k, fp, s->predPos, s->totCorrPos, lam.data(), table.data(), n, corr.data());
  cloud_lambda(g, k, fp, s->predPos, table.data(), n, rho.data(), lamOut.data());
  double acc = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    const double C = (double)(rho[i] / fp->restDensity - 1.0f);
    acc += C * C;
  }
  *loss = n ? acc / n : 0.0;
  if (featsOut) std::memcpy(featsOut, feats.data(), sizeof(float) * feats.size());
  return RTP_OK;
}

// The warm-started clouds step (runtime.cu clouds_solve_post with a network): the network
// relaxes the plain first-iteration lambda, lambda <- omega(y) lambda, then extraIters plain
// iterations follow.  feats/omega (optional, rows by sorted index) return the network's
// inputs and relaxations.
int or_clouds_ws_step(const rtp_grid_constants* c, const rtp_fluid_params* fp, const rtp_cloud_params* cp,
                      const rtp_cloud_env* env, const float* ground, const rtp_mlp* net, uint32_t extraIters,
                      uint32_t n, or_state* s, float* featsOut, float* omegaOut) {
  if (!c || !fp || !cp || !env || !net || !clouds_state_ok(s)) return RTP_ERR_INVALID_ARGUMENT;
  const Grid g(c);
  const Sph k(c);
  const CloudEnv E(c, env, ground);
  std::vector<uint32_t> table;
  clouds_presort(c, cp, E, n, s, table);
  std::vector<float> feats(12 * (size_t)n), out(4 * (size_t)n), lam(n), corr(4 * (size_t)n);
  or_clouds_ws_features(c, fp, env, ground, s->predPos, s->vel, s->temp, s->buoyancy, table.data(), n, feats.data());
  or_mlp_forward(net, feats.data(), n, 1, out.data());
  for (uint32_t i = 0; i < n; ++i) {
    const float om = ws_omega(out[4 * (size_t)i]);
    lam[i] = om * feats[12 * (size_t)i + 10];
    if (omegaOut) omegaOut[i] = om;
  }
  if (featsOut) std::memcpy(featsOut, feats.data(), sizeof(float) * feats.size());
  cloud_correct(g, k, fp, s->predPos, s->totCorrPos, lam.data(), table.data(), n, corr.data());
  std::vector<float> density(n), lambda(n);
  cloud_jacobi(g, k, fp, extraIters, s->predPos, s->totCorrPos, table.data(), n, density, lambda);
  clouds_post(c, fp, cp, E, n, s, table.data());
  return RTP_OK;
}

}  // extern "C"
