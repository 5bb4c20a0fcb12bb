// Trilinear level-set interpolant, device side (domain/interpolate.py:906-1021).
// Compiled only in translation units built with -fmad=false, so every float32
// operation rounds exactly like the reference's element-wise float32 arithmetic.
#pragma once

#include "dips_common.cuh"

namespace dips {

struct LevelSet {
  const float* g;  // ghosted cube [(nx+2)][(ny+2)][(nz+2)]
  const float* xg;
  const float* yg;
  const float* zg;
  int n0, n1, n2;  // ghosted sizes
  float dx0, dy0, dz0;  // xg[1]-xg[0] etc.: the spacing used for the cell index
  float xmin, xmax, ymin, ymax, zmin, zmax;
};

inline LevelSet make_levelset(const dips_levelset_t& s) {
  LevelSet L;
  L.g = s.phi_gh;
  L.xg = s.xg;
  L.yg = s.yg;
  L.zg = s.zg;
  L.n0 = s.nx + 2;
  L.n1 = s.ny + 2;
  L.n2 = s.nz + 2;
  L.dx0 = L.dy0 = L.dz0 = 0.0f;  // set on the device by levelset_init()
  L.xmin = s.xmin;
  L.xmax = s.xmax;
  L.ymin = s.ymin;
  L.ymax = s.ymax;
  L.zmin = s.zmin;
  L.zmax = s.zmax;
  return L;
}

// Read the ghosted spacings x[1]-x[0] (the ``dx`` of find_lower_left_cell_idx) on the device.
__device__ __forceinline__ void levelset_init(LevelSet& L) {
  L.dx0 = __fsub_rn(__ldg(L.xg + 1), __ldg(L.xg));
  L.dy0 = __fsub_rn(__ldg(L.yg + 1), __ldg(L.yg));
  L.dz0 = __fsub_rn(__ldg(L.zg + 1), __ldg(L.zg));
}

// Lower-left ghosted cell index: i32((p - a0)/d), then clamped to [2, n-2]
// (find_lower_left_cell_idx, interpolate.py:939-958).
__device__ __forceinline__ int ll_index(float p, float a0, float d, int n) {
  float q = __fdiv_rn(__fsub_rn(p, a0), d);
  if (!isfinite(q)) q = 0.0f;
  int i = __float2int_rz(q);
  if (i >= n - 1) i = n - 2;
  if (i <= 1) i = 2;
  return i;
}

__device__ __forceinline__ float lerp1(float a, float b, float t) {
  // a*(1-t) + b*t with each product and the sum rounded separately
  return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t));
}

__device__ __forceinline__ float phi_at(const LevelSet& L, float xp, float yp, float zp) {
  const int i = ll_index(xp, L.xg[0], L.dx0, L.n0);
  const int j = ll_index(yp, L.yg[0], L.dy0, L.n1);
  const int k = ll_index(zp, L.zg[0], L.dz0, L.n2);
  const float xi = L.xg[i], xi1 = L.xg[i + 1];
  const float yj = L.yg[j], yj1 = L.yg[j + 1];
  const float zk = L.zg[k], zk1 = L.zg[k + 1];
  const float xd = __fdiv_rn(__fsub_rn(xp, xi), __fsub_rn(xi1, xi));
  const float yd = __fdiv_rn(__fsub_rn(yp, yj), __fsub_rn(yj1, yj));
  const float zd = __fdiv_rn(__fsub_rn(zp, zk), __fsub_rn(zk1, zk));
  const int64_t s1 = L.n2, s0 = (int64_t)L.n1 * L.n2;
  const int64_t b = (int64_t)i * s0 + (int64_t)j * s1 + k;
  const float c000 = __ldg(L.g + b);
  const float c001 = __ldg(L.g + b + 1);
  const float c010 = __ldg(L.g + b + s1);
  const float c011 = __ldg(L.g + b + s1 + 1);
  const float c100 = __ldg(L.g + b + s0);
  const float c101 = __ldg(L.g + b + s0 + 1);
  const float c110 = __ldg(L.g + b + s0 + s1);
  const float c111 = __ldg(L.g + b + s0 + s1 + 1);
  const float c00 = lerp1(c000, c100, xd);
  const float c01 = lerp1(c001, c101, xd);
  const float c10 = lerp1(c010, c110, xd);
  const float c11 = lerp1(c011, c111, xd);
  const float c0 = lerp1(c00, c10, yd);
  const float c1 = lerp1(c01, c11, yd);
  return lerp1(c0, c1, zd);
}

__device__ __forceinline__ float phi_at(const LevelSet& L, const float x[3]) { return phi_at(L, x[0], x[1], x[2]); }

// Value of the ghosted field at (i, j, k) with every index clamped into the cube (the
// reference's out-of-range gathers clamp), and its second difference along one axis.
__device__ __forceinline__ float field_at(const LevelSet& L, int i, int j, int k) {
  i = min(max(i, 0), L.n0 - 1);
  j = min(max(j, 0), L.n1 - 1);
  k = min(max(k, 0), L.n2 - 1);
  return __ldg(L.g + ((int64_t)i * L.n1 + j) * L.n2 + k);
}
__device__ __forceinline__ float second_diff(const LevelSet& L, int i, int j, int k, int di, int dj, int dk) {
  // c[+1] - 2 c[0] + c[-1], left to right
  return __fadd_rn(__fsub_rn(field_at(L, i + di, j + dj, k + dk), __fmul_rn(2.0f, field_at(L, i, j, k))),
                   field_at(L, i - di, j - dj, k - dk));
}

// Non-oscillatory quadratic interpolant (Min & Gibou 2007 eqs. 12-13 as the reference writes it,
// interpolate.py:572-759): the trilinear value minus, per axis, 0.5 t (1 - t) times the smallest
// |second difference| along that axis over the cell's 8 corners.
__device__ __forceinline__ float quad_at(const LevelSet& L, float xp, float yp, float zp) {
  const int i = ll_index(xp, L.xg[0], L.dx0, L.n0);
  const int j = ll_index(yp, L.yg[0], L.dy0, L.n1);
  const int k = ll_index(zp, L.zg[0], L.dz0, L.n2);
  const float xd = __fdiv_rn(__fsub_rn(xp, L.xg[i]), __fsub_rn(L.xg[i + 1], L.xg[i]));
  const float yd = __fdiv_rn(__fsub_rn(yp, L.yg[j]), __fsub_rn(L.yg[j + 1], L.yg[j]));
  const float zd = __fdiv_rn(__fsub_rn(zp, L.zg[k]), __fsub_rn(L.zg[k + 1], L.zg[k]));
  float mx = INFINITY, my = INFINITY, mz = INFINITY;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        mx = fminf(mx, fabsf(second_diff(L, i + a, j + b, k + c, 1, 0, 0)));
        my = fminf(my, fabsf(second_diff(L, i + a, j + b, k + c, 0, 1, 0)));
        mz = fminf(mz, fabsf(second_diff(L, i + a, j + b, k + c, 0, 0, 1)));
      }
  float v = phi_at(L, xp, yp, zp);
  v = __fsub_rn(v, __fmul_rn(__fmul_rn(__fmul_rn(mx, 0.5f), xd), __fsub_rn(1.0f, xd)));
  v = __fsub_rn(v, __fmul_rn(__fmul_rn(__fmul_rn(my, 0.5f), yd), __fsub_rn(1.0f, yd)));
  v = __fsub_rn(v, __fmul_rn(__fmul_rn(__fmul_rn(mz, 0.5f), zd), __fsub_rn(1.0f, zd)));
  return v;
}

}  // namespace dips
