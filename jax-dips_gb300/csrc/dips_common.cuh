// Shared helpers for the dips_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dips.h"

namespace dips {

// Thread-local error text returned by dips_last_error().
void set_error(const char* fmt, ...);

// Map a CUDA error to a status code and record its text.
int cuda_status(cudaError_t e, const char* where);

#define DIPS_CHECK_LAUNCH(where)                                   \
  do {                                                             \
    cudaError_t _e = cudaGetLastError();                           \
    if (_e != cudaSuccess) return ::dips::cuda_status(_e, where);  \
  } while (0)

#define DIPS_REQUIRE(cond, code, ...)        \
  do {                                       \
    if (!(cond)) {                           \
      ::dips::set_error(__VA_ARGS__);        \
      return code;                           \
    }                                        \
  } while (0)

constexpr int kStencil = 7;   // ijk, i-1, i+1, j-1, j+1, k-1, k+1
constexpr int kCube = 27;     // 3x3x3 regression cube, x fastest
constexpr int kCubeCentre = 13;

// Job code: stencil point j (0..6) and cube vertex k (0..26) -> j*27 + k; bit 15 marks the
// u+ network (phi >= 0 at the evaluation point).
__host__ __device__ inline uint16_t job_code(int j, int k, bool net_p) {
  return (uint16_t)((j * kCube + k) | (net_p ? 0x8000 : 0));
}
__host__ __device__ inline int job_stencil(uint16_t c) { return (c & 0x7fff) / kCube; }
__host__ __device__ inline int job_vertex(uint16_t c) { return (c & 0x7fff) % kCube; }
__host__ __device__ inline bool job_net_p(uint16_t c) { return (c & 0x8000) != 0; }

// Stencil point j of point p at spacing h, with the reference's float32 operations
// (discretization.py:347-353): the shifted coordinate is p[a] -/+ h[a].
__device__ __forceinline__ void stencil_point(const float p[3], const float h[3], int j, float s[3]) {
  // selects over the three axes (no run-time array index, which would put p, h and s in local
  // memory); p - h is computed as p + (-h), the same rounded value
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const bool moved = j > 0 && ((j - 1) >> 1) == a;
    s[a] = moved ? __fadd_rn(p[a], ((j - 1) & 1) ? h[a] : -h[a]) : p[a];
  }
}

// Offset of cube vertex k (discretization.py:164-197): components in {-h, 0, +h}.
__device__ __forceinline__ float cube_offset(int k, int a, const float h[3]) {
  int o = (a == 0) ? (k % 3) : (a == 1 ? (k / 3) % 3 : k / 9);
  return o == 0 ? -h[a] : (o == 2 ? h[a] : 0.0f);
}

// Coordinates of job code c relative to point p: stencil point, then + cube offset
// (the vertex list s + X_ijk of discretization.py:441).
__device__ __forceinline__ void job_coords(const float p[3], const float h[3], uint16_t c, float x[3]) {
  int j = job_stencil(c);
  int k = job_vertex(c);
  float s[3];
  stencil_point(p, h, j, s);
  if (k == kCubeCentre) {
    x[0] = s[0];
    x[1] = s[1];
    x[2] = s[2];
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) x[a] = __fadd_rn(s[a], cube_offset(k, a, h));
  }
}

__device__ __forceinline__ float nan_to_num(float v) {
  if (isnan(v)) return 0.0f;
  if (isinf(v)) return v > 0 ? 3.402823466e38f : -3.402823466e38f;
  return v;
}

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace dips
