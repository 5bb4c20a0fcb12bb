// Per-point geometry and residual records of the jump-condition FV stencil (sm_103a).
//
// Build with -fmad=false: every float32 expression below is a sequence of separately
// rounded operations in the reference's order, so each discrete decision (cell
// crossing, interface-vertex positions, isclose face tests, stable argsorts, sign
// masks) is taken exactly as the float32 restatement of the reference takes it.
//
// Reference: geometry/geometric_integrations_per_point.py (cell decomposition, areas,
// volumes, interface quadrature) and solvers/poisson/discretization.py:164-519
// (regression extrapolation across the interface and the FV assembly).

#include <math.h>

#include "dips_common.cuh"
#include "levelset.cuh"

namespace dips {

// corner offsets P_000, P_100, P_101, P_001, P_010, P_110, P_011, P_111 (geom_pp.py:214-226)
__constant__ int8_t c_corner_sign[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, -1, 1}, {-1, -1, 1},
                                            {-1, 1, -1}, {1, 1, -1},  {-1, 1, 1}, {1, 1, 1}};
// tetrahedra S1..S5 as corner indices (geom_pp.py:311-322)
__constant__ int8_t c_tets[5][4] = {{0, 1, 4, 3}, {5, 1, 4, 7}, {2, 1, 7, 3}, {6, 7, 4, 3}, {7, 1, 4, 3}};

// ----------------------------------------------------------------------------------------
// small float32 helpers (every op rounded on its own)
// ----------------------------------------------------------------------------------------
__device__ __forceinline__ float dot3(const float* a, const float* b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}

// 0.5*sqrt|det(D D^T)|, D = [v1-v0; v2-v0]  (area_fn, geom_pp.py:377-380)
__device__ float tri_area(const float v0[3], const float v1[3], const float v2[3]) {
  float d[2][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    d[0][c] = __fsub_rn(v1[c], v0[c]);
    d[1][c] = __fsub_rn(v2[c], v0[c]);
  }
  float g00 = dot3(d[0], d[0]), g01 = dot3(d[0], d[1]), g10 = dot3(d[1], d[0]), g11 = dot3(d[1], d[1]);
  float det = __fsub_rn(__fmul_rn(g00, g11), __fmul_rn(g01, g10));
  return __fmul_rn(0.5f, __fsqrt_rn(fabsf(nan_to_num(det))));
}

// (1/6)*sqrt|det(D D^T)|, D = [v1-v0; v2-v0; v3-v0]  (vol_fn, geom_pp.py:370-374), with
// jax's closed-form 3x3 determinant.
__device__ float tet_volume(const float v[4][3]) {
  float d[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) d[a][c] = __fsub_rn(v[a + 1][c], v[0][c]);
  float g[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) g[a][b] = dot3(d[a], d[b]);
  float t1 = __fmul_rn(__fmul_rn(g[0][0], g[1][1]), g[2][2]);
  float t2 = __fmul_rn(__fmul_rn(g[0][1], g[1][2]), g[2][0]);
  float t3 = __fmul_rn(__fmul_rn(g[0][2], g[1][0]), g[2][1]);
  float t4 = __fmul_rn(__fmul_rn(g[0][2], g[1][1]), g[2][0]);
  float t5 = __fmul_rn(__fmul_rn(g[0][0], g[1][2]), g[2][1]);
  float t6 = __fmul_rn(__fmul_rn(g[0][1], g[1][0]), g[2][2]);
  float det = __fsub_rn(__fsub_rn(__fsub_rn(__fadd_rn(__fadd_rn(t1, t2), t3), t4), t5), t6);
  return __fmul_rn((float)(1.0 / 6.0), __fsqrt_rn(fabsf(nan_to_num(det))));
}

// jnp.isclose(a, b, atol=atol, rtol=1e-5) in float32
__device__ __forceinline__ bool isclose32(float a, float b, float atol) {
  if (isnan(a) || isnan(b)) return false;
  if (isinf(a) || isinf(b)) return a == b;
  return fabsf(__fsub_rn(a, b)) <= __fadd_rn(atol, __fmul_rn(1e-5f, fabsf(b)));
}

// ----------------------------------------------------------------------------------------
// the h-cube of a point and its five-tetrahedron decomposition
// ----------------------------------------------------------------------------------------
struct Cell {
  float c[8][3];
  float phi[8];
  int crossed;  // -1 / 0 / +1 (is_point_cell_crossed_by_interface)
};

__device__ void cell_corners(const float p[3], const float h[3], float c[8][3]) {
#pragma unroll
  for (int v = 0; v < 8; ++v)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float off = __fmul_rn(__fmul_rn((float)c_corner_sign[v][a], h[a]), 0.5f);
      c[v][a] = __fadd_rn(p[a], off);
    }
}

__device__ __forceinline__ int crossed_of(const float phi[8]) {
  int eta = 0;
#pragma unroll
  for (int v = 0; v < 8; ++v) eta += (phi[v] < 0.0f);
  if (eta == 0 || eta == 8) return phi[0] > 0.0f ? 1 : (phi[0] < 0.0f ? -1 : 0);
  return 0;
}

__device__ void cell_eval(const LevelSet& L, const float p[3], const float h[3], Cell& cell) {
  cell_corners(p, h, cell.c);
#pragma unroll
  for (int v = 0; v < 8; ++v) cell.phi[v] = phi_at(L, cell.c[v]);
  cell.crossed = crossed_of(cell.phi);
}

__device__ int crossed_at(const LevelSet& L, const float p[3], const float h[3]) {
  float c[8][3];
  cell_corners(p, h, c);
  float ph[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) ph[v] = phi_at(L, c[v]);
  return crossed_of(ph);
}

// stable ascending argsort of 4 keys
__device__ __forceinline__ void argsort4(const float key[4], int o[4]) {
  o[0] = 0;
  o[1] = 1;
  o[2] = 2;
  o[3] = 3;
#pragma unroll
  for (int i = 1; i < 4; ++i) {
    int kk = o[i];
    int j = i - 1;
    while (j >= 0 && key[o[j]] > key[kk]) {
      o[j + 1] = o[j];
      --j;
    }
    o[j + 1] = kk;
  }
}

struct Tet {
  float S[4][3];  // sorted vertices
  float ps[4];    // sorted level-set values
  int eta;        // number of negative vertices
};

// sort a tetrahedron's vertices by key (phi or -phi) and keep the sorted keys
__device__ void tet_sorted(const Cell& cell, int t, bool negate, Tet& T) {
  float key[4];
  int eta = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float v = cell.phi[c_tets[t][q]];
    eta += (v < 0.0f);
    key[q] = negate ? -v : v;
  }
  int o[4];
  argsort4(key, o);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int ci = c_tets[t][o[q]];
    T.ps[q] = key[o[q]];
#pragma unroll
    for (int a = 0; a < 3; ++a) T.S[q][a] = cell.c[ci][a];
  }
  T.eta = eta;
}

// (phi_i*S_j - phi_j*S_i)/(phi_i - phi_j)
__device__ __forceinline__ void lerp_vertex(const Tet& T, int i, int j, float out[3]) {
  float den = __fsub_rn(T.ps[i], T.ps[j]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float num = __fsub_rn(__fmul_rn(T.ps[i], T.S[j][a]), __fmul_rn(T.ps[j], T.S[i][a]));
    out[a] = __fdiv_rn(num, den);
  }
}

__device__ __forceinline__ void cpy3(float d[3], const float s[3]) {
  d[0] = s[0];
  d[1] = s[1];
  d[2] = s[2];
}

// Interface triangles of tetrahedron t (get_vertices_S_intersect_Gamma, geom_pp.py:52-107).
// Returns the number of real triangles (0, 1 or 2); the rest are the reference's zero padding.
__device__ int tet_gamma(const Cell& cell, int t, float tri[2][3][3]) {
  Tet T;
  tet_sorted(cell, t, false, T);
  int eta = T.eta;
  if (eta == 1) {
    lerp_vertex(T, 0, 1, tri[0][0]);
    lerp_vertex(T, 0, 2, tri[0][1]);
    lerp_vertex(T, 0, 3, tri[0][2]);
    return 1;
  }
  if (eta == 2) {
    float q0[3], q1[3], q2[3], q5[3];
    lerp_vertex(T, 0, 2, q0);
    lerp_vertex(T, 0, 3, q1);
    lerp_vertex(T, 1, 3, q2);
    lerp_vertex(T, 1, 2, q5);
    cpy3(tri[0][0], q0);
    cpy3(tri[0][1], q1);
    cpy3(tri[0][2], q2);
    cpy3(tri[1][0], q0);
    cpy3(tri[1][1], q5);
    cpy3(tri[1][2], q2);
    return 2;
  }
  if (eta == 3) {
    Tet N;
    tet_sorted(cell, t, true, N);
    lerp_vertex(N, 0, 1, tri[0][0]);
    lerp_vertex(N, 0, 2, tri[0][1]);
    lerp_vertex(N, 0, 3, tri[0][2]);
    return 1;
  }
  return 0;
}

// Omega^- sub-tetrahedra of tetrahedron t (get_vertices_S_intersect_Omega_m, geom_pp.py:110-198).
// Returns the number of non-padding sub-tets; padding entries are zero vertices.
__device__ int tet_omega(const Cell& cell, int t, float om[3][4][3]) {
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int a = 0; a < 3; ++a) om[q][v][a] = 0.0f;
  Tet T;
  tet_sorted(cell, t, false, T);
  int eta = T.eta;
  if (eta == 4) {
#pragma unroll
    for (int v = 0; v < 4; ++v) cpy3(om[0][v], cell.c[c_tets[t][v]]);
    return 1;
  }
  if (eta == 1) {
    cpy3(om[0][0], T.S[0]);
    lerp_vertex(T, 0, 1, om[0][1]);
    lerp_vertex(T, 0, 2, om[0][2]);
    lerp_vertex(T, 0, 3, om[0][3]);
    return 1;
  }
  if (eta == 2) {
    float Q2[3], Q3[3], Q4[3], Q5[3];
    lerp_vertex(T, 0, 2, Q2);
    lerp_vertex(T, 1, 3, Q3);
    lerp_vertex(T, 1, 2, Q4);
    lerp_vertex(T, 0, 3, Q5);
    cpy3(om[0][0], T.S[0]);
    cpy3(om[0][1], T.S[1]);
    cpy3(om[0][2], Q2);
    cpy3(om[0][3], Q3);
    cpy3(om[1][0], Q4);
    cpy3(om[1][1], T.S[1]);
    cpy3(om[1][2], Q2);
    cpy3(om[1][3], Q3);
    cpy3(om[2][0], T.S[0]);
    cpy3(om[2][1], Q5);
    cpy3(om[2][2], Q2);
    cpy3(om[2][3], Q3);
    return 3;
  }
  if (eta == 3) {
    float R3[3], R4[3], R5[3];
    lerp_vertex(T, 1, 3, R3);
    lerp_vertex(T, 0, 3, R4);
    lerp_vertex(T, 2, 3, R5);
    cpy3(om[0][0], T.S[0]);
    cpy3(om[0][1], T.S[1]);
    cpy3(om[0][2], T.S[2]);
    cpy3(om[0][3], R3);
    cpy3(om[1][0], T.S[0]);
    cpy3(om[1][1], R4);
    cpy3(om[1][2], T.S[2]);
    cpy3(om[1][3], R3);
    cpy3(om[2][0], R5);
    cpy3(om[2][1], R4);
    cpy3(om[2][2], T.S[2]);
    cpy3(om[2][3], R3);
    return 3;
  }
  return 0;
}

// Omega^- area of one sub-tet's face on the plane x_axis = fc (compute_area_from_partitions.comp,
// geom_pp.py:590-626): exactly 3 vertices on the face -> their triangle, ordered by x.
__device__ float subtet_face_area(const float v[4][3], int axis, float fc, float atol) {
  int on[4];
  int cnt = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    on[q] = isclose32(v[q][axis], fc, atol);
    cnt += on[q];
  }
  if (cnt != 3) return 0.0f;
  // stable argsort by x with off-face vertices at the sentinel 200 (always last)
  float key[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) key[q] = on[q] ? v[q][0] : 200.0f;
  int o[4];
  argsort4(key, o);
  float a[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
#pragma unroll
    for (int c = 0; c < 3; ++c) a[q][c] = on[o[q]] ? v[o[q]][c] : 200.0f;
  }
  return tri_area(a[0], a[1], a[2]);
}

__device__ float partition_face_area(const Cell& cell, int t, int axis, float fc, float atol) {
  float om[3][4][3];
  tet_omega(cell, t, om);
  float s = subtet_face_area(om[0], axis, fc, atol);
  s = __fadd_rn(s, subtet_face_area(om[1], axis, fc, atol));
  s = __fadd_rn(s, subtet_face_area(om[2], axis, fc, atol));
  return s;
}

__device__ __forceinline__ float face_area_m(const Cell& cell, int ta, int tb, int axis, float fc, float hax) {
  float atol = __fmul_rn(1e-10f, hax);
  return __fadd_rn(partition_face_area(cell, ta, axis, fc, atol), partition_face_area(cell, tb, axis, fc, atol));
}

__device__ __forceinline__ float pos_or_zero(float v) { return v < 0.0f ? 0.0f : v; }

// The 26 cell coefficients of a cell that the interface does not cross (crossed = -1 or +1):
// full faces and volume on its side
__device__ __forceinline__ void face_coefficients_uncrossed(int crossed, const float h[3], const float mm[6],
                                                            const float mp[6], float out[26]) {
  const float dx = h[0], dy = h[1], dz = h[2];
  const float vol = __fmul_rn(__fmul_rn(dx, dy), dz);
  const float ax = __fmul_rn(dy, dz), ay = __fmul_rn(dx, dz), az = __fmul_rn(dx, dy);
  const float sm = crossed < 0 ? 1.0f : 0.0f;
  const float sp = crossed > 0 ? 1.0f : 0.0f;
  const float nom[6] = {ax, ax, ay, ay, az, az};
  const float hh[6] = {dx, dx, dy, dy, dz, dz};
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    out[2 * f] = __fdiv_rn(__fmul_rn(nom[f], __fmul_rn(mm[f], sm)), hh[f]);
    out[2 * f + 1] = __fdiv_rn(__fmul_rn(nom[f], __fmul_rn(mp[f], sp)), hh[f]);
    out[14 + 2 * f] = __fmul_rn(nom[f], sm);
    out[14 + 2 * f + 1] = __fmul_rn(nom[f], sp);
  }
  out[12] = __fmul_rn(vol, sm);
  out[13] = __fmul_rn(vol, sp);
}

// The 26 cell coefficients of compute_face_centroids_values_plus_minus_at_point
// (geom_pp.py:514-1007); mu at the 6 face centres are caller-supplied samples.
__device__ void face_coefficients(const Cell& cell, const float p[3], const float h[3], const float mm[6],
                                  const float mp[6], float out[26]) {
  const float dx = h[0], dy = h[1], dz = h[2];
  const float vol = __fmul_rn(__fmul_rn(dx, dy), dz);
  const float ax = __fmul_rn(dy, dz), ay = __fmul_rn(dx, dz), az = __fmul_rn(dx, dy);
  if (cell.crossed == 0) {
    float vol_m = 0.0f;
    bool first = true;
    for (int t = 0; t < 5; ++t) {
      float om[3][4][3];
      tet_omega(cell, t, om);
      for (int q = 0; q < 3; ++q) {
        float v = tet_volume(om[q]);
        vol_m = first ? v : __fadd_rn(vol_m, v);
        first = false;
      }
    }
    const float vol_p = pos_or_zero(__fsub_rn(vol, vol_m));
    const float half = 0.5f;
    float am[6];
    am[0] = face_area_m(cell, 0, 3, 0, __fsub_rn(p[0], __fmul_rn(half, dx)), dx);
    am[1] = face_area_m(cell, 1, 2, 0, __fadd_rn(p[0], __fmul_rn(half, dx)), dx);
    am[2] = face_area_m(cell, 0, 2, 1, __fsub_rn(p[1], __fmul_rn(half, dy)), dy);
    am[3] = face_area_m(cell, 1, 3, 1, __fadd_rn(p[1], __fmul_rn(half, dy)), dy);
    am[4] = face_area_m(cell, 0, 1, 2, __fsub_rn(p[2], __fmul_rn(half, dz)), dz);
    am[5] = face_area_m(cell, 2, 3, 2, __fadd_rn(p[2], __fmul_rn(half, dz)), dz);
    const float nom[6] = {ax, ax, ay, ay, az, az};
    const float hh[6] = {dx, dx, dy, dy, dz, dz};
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      float ap = pos_or_zero(__fsub_rn(nom[f], am[f]));
      out[2 * f] = __fdiv_rn(__fmul_rn(am[f], mm[f]), hh[f]);
      out[2 * f + 1] = __fdiv_rn(__fmul_rn(ap, mp[f]), hh[f]);
      out[14 + 2 * f] = am[f];
      out[14 + 2 * f + 1] = ap;
    }
    out[12] = vol_m;
    out[13] = vol_p;
  } else {
    face_coefficients_uncrossed(cell.crossed, h, mm, mp, out);
  }
}

// ----------------------------------------------------------------------------------------
// least-squares regression at a crossed stencil point (discretization.py:199-296)
// ----------------------------------------------------------------------------------------
// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations (float32; only for
// cells whose stencil spacing differs between axes, see lsq_operator).
__device__ void jacobi_eig3f(float a[3][3], float v[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? 1.0f : 0.0f;
  for (int sweep = 0; sweep < 10; ++sweep) {
    const float off = fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]);
    const float scale = fabsf(a[0][0]) + fabsf(a[1][1]) + fabsf(a[2][2]);
    if (off == 0.0f || off <= 1e-9f * scale) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        const float apq = a[p][q];
        if (apq == 0.0f) continue;
        const float theta = (a[q][q] - a[p][p]) / (2.0f * apq);
        const float t = (theta >= 0.0f ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
        const float c = 1.0f / sqrtf(t * t + 1.0f), sn = t * c;
        for (int k = 0; k < 3; ++k) {
          const float akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - sn * akq;
          a[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const float apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - sn * aqk;
          a[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const float vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - sn * vkq;
          v[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}

__device__ __forceinline__ int cube_o(int k, int a) { return (a == 0 ? k % 3 : (a == 1 ? (k / 3) % 3 : k / 9)) - 1; }

// D = pinv(X^T W X)(W X)^T (3 x 27) under the reference's pinv rule: jnp.linalg.pinv drops the
// singular values at or below 10 * 3 * eps_f32 * sigma_max (discretization.py:257-258).
//
// X's rows are the cube offsets o_k h (o_k in {-1, 0, 1}^3, x fastest; get_Xijk,
// discretization.py:164-197), so X^T W X = S N S with S = diag(h) and N = sum_k w_k o_k o_k^T,
// an integer matrix with diagonal entries <= 18.  Its rank follows exactly from integer
// invariants: det N, s = the sum of its principal 2x2 minors and t = tr N (rank 3, 2 or 1 for the
// first of them that is nonzero).  These are the ranks the cutoff keeps: for a positive
// semidefinite integer N of rank 3, lambda_min >= det / lambda_max^2 >= 1 / lambda_max^2 and
// lambda_max <= t <= 54, so lambda_min / lambda_max >= 1 / 54^3 = 6.4e-6 > 3.6e-6; for rank 2 the
// smaller nonzero eigenvalue is >= s / lambda_max >= 1 / 54, a ratio >= 3.4e-4; and a zero
// eigenvalue comes out of a float32 SVD at about eps * lambda_max, below the cutoff.
//
// With the same spacing on every axis (the reference's grids), pinv(X^T W X) = pinv(N) / h^2 and
// pinv(N) is an integer matrix over an integer: adj(N) / det N (rank 3); by Cayley-Hamilton on
// the range, ((t^2 - s) N - t N^2) / s^2 (rank 2); N / t^2 (rank 1).  D[i][k] = w_k (P o_k)_i /
// (den h) is then one float32 division of exact integers followed by the division by h.  With
// spacings that differ between axes, S N S is decomposed by float32 Jacobi rotations and its r
// largest eigenpairs (r the exact rank) are inverted.  Float32 throughout.
__device__ void lsq_operator(const float h[3], const bool w[27], float D[3][27]) {
  int N[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = 0; k < 27; ++k) {
    if (!w[k]) continue;
    const int o[3] = {cube_o(k, 0), cube_o(k, 1), cube_o(k, 2)};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) N[i][j] += o[i] * o[j];
  }
  const int t = N[0][0] + N[1][1] + N[2][2];
  const int m01 = N[0][0] * N[1][1] - N[0][1] * N[1][0];
  const int m02 = N[0][0] * N[2][2] - N[0][2] * N[2][0];
  const int m12 = N[1][1] * N[2][2] - N[1][2] * N[2][1];
  const int sm = m01 + m02 + m12;
  int adj[3][3];
  adj[0][0] = m12;
  adj[1][1] = m02;
  adj[2][2] = m01;
  adj[0][1] = adj[1][0] = N[0][2] * N[2][1] - N[0][1] * N[2][2];
  adj[0][2] = adj[2][0] = N[0][1] * N[1][2] - N[0][2] * N[1][1];
  adj[1][2] = adj[2][1] = N[0][2] * N[1][0] - N[0][0] * N[1][2];
  const int det = N[0][0] * adj[0][0] + N[0][1] * adj[1][0] + N[0][2] * adj[2][0];
  const int rank = det != 0 ? 3 : (sm != 0 ? 2 : (t != 0 ? 1 : 0));
  if (rank == 0) {
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 27; ++k) D[i][k] = 0.0f;
    return;
  }
  if (h[0] == h[1] && h[1] == h[2]) {
    int P[3][3];
    int den;
    if (rank == 3) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P[i][j] = adj[i][j];
      den = det;
    } else if (rank == 2) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const int n2 = N[i][0] * N[0][j] + N[i][1] * N[1][j] + N[i][2] * N[2][j];
          P[i][j] = (t * t - sm) * N[i][j] - t * n2;
        }
      den = sm * sm;
    } else {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) P[i][j] = N[i][j];
      den = t * t;
    }
    const float fden = (float)den;
    for (int k = 0; k < 27; ++k) {
      const int o[3] = {cube_o(k, 0), cube_o(k, 1), cube_o(k, 2)};
      for (int i = 0; i < 3; ++i) {
        const int num = w[k] ? P[i][0] * o[0] + P[i][1] * o[1] + P[i][2] * o[2] : 0;
        D[i][k] = __fdiv_rn(__fdiv_rn((float)num, fden), h[0]);
      }
    }
    return;
  }
  float A[3][3], V[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i][j] = (float)N[i][j] * h[i] * h[j];
  jacobi_eig3f(A, V);
  // the `rank` largest eigenvalues
  float lam[3] = {A[0][0], A[1][1], A[2][2]};
  bool keep[3] = {false, false, false};
  for (int r = 0; r < rank; ++r) {
    int best = -1;
    for (int e = 0; e < 3; ++e)
      if (!keep[e] && (best < 0 || lam[e] > lam[best])) best = e;
    keep[best] = true;
  }
  float P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int e = 0; e < 3; ++e) {
    if (!keep[e]) continue;
    const float inv = 1.0f / lam[e];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P[i][j] += V[i][e] * V[j][e] * inv;
  }
  for (int k = 0; k < 27; ++k)
    for (int i = 0; i < 3; ++i) {
      float s = 0.0f;
      if (w[k])
        for (int j = 0; j < 3; ++j) s += P[i][j] * ((float)cube_o(k, j) * h[j]);
      D[i][k] = s;
    }
}

struct StencilRegression {
  float phi_s;       // phi(s)
  float n[3];        // central-difference unit normal
  float rproj[3];    // s - phi(s) n
  float phi_v[27];   // phi at the cube vertices s + X_k
};

__device__ void regression_geometry(const LevelSet& L, const float s[3], const float h[3], StencilRegression& R) {
  R.phi_s = phi_at(L, s);
  float d[3];
  for (int a = 0; a < 3; ++a) {
    float sp[3] = {s[0], s[1], s[2]};
    float sm[3] = {s[0], s[1], s[2]};
    sp[a] = __fadd_rn(s[a], h[a]);
    sm[a] = __fsub_rn(s[a], h[a]);
    d[a] = __fdiv_rn(__fsub_rn(phi_at(L, sp), phi_at(L, sm)), __fmul_rn(2.0f, h[a]));
  }
  float norm = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
  for (int a = 0; a < 3; ++a) {
    R.n[a] = __fdiv_rn(d[a], norm);
    R.rproj[a] = __fsub_rn(s[a], __fmul_rn(R.phi_s, R.n[a]));
  }
  for (int k = 0; k < 27; ++k) {
    float v[3];
    for (int a = 0; a < 3; ++a) v[a] = __fadd_rn(s[a], cube_offset(k, a, h));
    R.phi_v[k] = phi_at(L, v);
  }
}

__device__ __forceinline__ bool is_box_boundary(const LevelSet& L, const float p[3], const float h[3]) {
  const float lo[3] = {L.xmin, L.ymin, L.zmin};
  const float hi[3] = {L.xmax, L.ymax, L.zmax};
  bool b = false;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float tol = __fmul_rn(1e-6f, h[a]);
    b |= fabsf(__fsub_rn(p[a], lo[a])) < tol;
    b |= fabsf(__fsub_rn(p[a], hi[a])) < tol;
  }
  return b;
}

__device__ __forceinline__ void load_point(const float* pts, int64_t i, float p[3]) {
  p[0] = pts[3 * i];
  p[1] = pts[3 * i + 1];
  p[2] = pts[3 * i + 2];
}

__device__ __forceinline__ uint32_t enc_crossed(int c) { return (uint32_t)(c + 1); }
__device__ __forceinline__ int dec_crossed(uint32_t f, int shift) { return (int)((f >> shift) & 3u) - 1; }

// flag word layout (see dips.h)
constexpr int kFlagBnd = 0;
constexpr int kFlagCrossedP = 1;
constexpr int kFlagCrossedS = 4;   // 2 bits per stencil point
constexpr int kFlagNetS = 18;      // 1 bit per stencil point

// ----------------------------------------------------------------------------------------
// kernels
// ----------------------------------------------------------------------------------------
__global__ void k_ghost_layer(const float* __restrict__ c, int nx, int ny, int nz, float* __restrict__ g) {
  const int64_t n0 = nx + 2, n1 = ny + 2, n2 = nz + 2;
  const int64_t total = n0 * n1 * n2;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total; idx += (int64_t)gridDim.x * blockDim.x) {
    int K = (int)(idx % n2);
    int J = (int)((idx / n2) % n1);
    int I = (int)(idx / (n1 * n2));
    auto C = [&](int i, int j, int k) { return c[((int64_t)i * ny + j) * nz + k]; };
    // X(I,J,K) for J in [1,ny], K in [1,nz]
    auto X = [&](int I_, int J_, int K_) -> float {
      if (I_ == 0) return __fsub_rn(__fmul_rn(2.0f, C(0, J_ - 1, K_ - 1)), C(1, J_ - 1, K_ - 1));
      if (I_ == nx + 1) return __fsub_rn(__fmul_rn(2.0f, C(nx - 1, J_ - 1, K_ - 1)), C(nx - 2, J_ - 1, K_ - 1));
      return C(I_ - 1, J_ - 1, K_ - 1);
    };
    auto Y = [&](int I_, int J_, int K_) -> float {
      if (J_ == 0) return __fsub_rn(__fmul_rn(2.0f, X(I_, 1, K_)), X(I_, 2, K_));
      if (J_ == ny + 1) return __fsub_rn(__fmul_rn(2.0f, X(I_, ny, K_)), X(I_, ny - 1, K_));
      return X(I_, J_, K_);
    };
    float v;
    if (K == 0)
      v = __fsub_rn(__fmul_rn(2.0f, Y(I, J, 1)), Y(I, J, 2));
    else if (K == nz + 1)
      v = __fsub_rn(__fmul_rn(2.0f, Y(I, J, nz)), Y(I, J, nz - 1));
    else
      v = Y(I, J, K);
    g[idx] = v;
  }
}

__global__ void k_trilinear(LevelSet L0, const float* __restrict__ pts, int64_t n, float* __restrict__ out) {
  LevelSet L = L0;
  levelset_init(L);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[3];
    load_point(pts, i, p);
    out[i] = phi_at(L, p);
  }
}

__global__ void k_quadratic(LevelSet L0, const float* __restrict__ pts, int64_t n, float* __restrict__ out) {
  LevelSet L = L0;
  levelset_init(L);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[3];
    load_point(pts, i, p);
    out[i] = quad_at(L, p[0], p[1], p[2]);
  }
}

struct H3 {
  float v[3];
};

__global__ void k_classify(LevelSet L0, const float* __restrict__ pts, int64_t n, H3 hh, uint32_t* __restrict__ flags,
                           int32_t* __restrict__ n_tri, int32_t* __restrict__ n_xs, int32_t* __restrict__ job_cap) {
  LevelSet L = L0;
  levelset_init(L);
  const float* h = hh.v;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[3];
    load_point(pts, i, p);
    const bool bnd = is_box_boundary(L, p, h);
    uint32_t f = (bnd ? 1u : 0u) << kFlagBnd;
    int nx = 0;
    for (int j = 0; j < kStencil; ++j) {
      float s[3];
      stencil_point(p, h, j, s);
      int c = crossed_at(L, s, h);
      bool net = phi_at(L, s) >= 0.0f;
      f |= enc_crossed(c) << (kFlagCrossedS + 2 * j);
      f |= (net ? 1u : 0u) << (kFlagNetS + j);
      if (j == 0) f |= enc_crossed(c) << kFlagCrossedP;
      nx += (c == 0);
    }
    int ntri = 0;  // counted for box-boundary points too: assemble integrates beta on every crossed cell
    if (dec_crossed(f, kFlagCrossedP) == 0) {
      Cell cell;
      cell_eval(L, p, h, cell);
      for (int t = 0; t < 5; ++t) {
        int eta = 0;
        for (int q = 0; q < 4; ++q) eta += (cell.phi[c_tets[t][q]] < 0.0f);
        ntri += (eta == 1 || eta == 3) ? 1 : (eta == 2 ? 2 : 0);
      }
    }
    if (bnd) nx = 0;
    flags[i] = f;
    n_tri[i] = ntri;
    n_xs[i] = nx;
    job_cap[i] = bnd ? 1 : (kStencil + (kCube - 1) * nx);
  }
}

// Passes of k_assemble: every point in one pass (kAllPoints), or two passes that keep the heavy
// points together: kDeferHeavy does the points without an interface stencil point and lists
// the others; kListed does the listed points.  A point with interface stencil points costs
// about a hundred times a bulk point (regression, five-tetrahedron clipping) and such points come
// a few to a warp of 32 consecutive points, so in one pass most of a warp idles while its heavy
// lanes run; listed, 32 heavy points share a warp.
enum AssemblePass { kAllPoints = 0, kDeferHeavy = 1, kListed = 2 };

__device__ __forceinline__ bool heavy_point(uint32_t f) {
  bool x = false;
#pragma unroll
  for (int j = 0; j < kStencil; ++j) x |= dec_crossed(f, kFlagCrossedS + 2 * j) == 0;
  return x;
}

// The points with an interface stencil point (the only ones with queries or regression work),
// listed so that a pass over them runs 32 of them to a warp
__global__ void k_heavy_list(const uint32_t* __restrict__ flags, int64_t n, int32_t* __restrict__ list,
                             int32_t* __restrict__ count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool heavy = heavy_point(flags[i]);
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, heavy);
    if (!m) continue;
    const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(act, base, leader);
    if (heavy) list[base + __popc(m & ((1u << lane) - 1))] = (int32_t)i;
  }
}

// the queries of every point (LISTED = false) or of the listed points (the others have none)
template <bool LISTED>
__global__ void k_queries(LevelSet L0, const float* __restrict__ pts, int64_t n, H3 hh, const uint32_t* __restrict__ flags,
                          const int64_t* __restrict__ tri_off, const int64_t* __restrict__ xs_off, float* __restrict__ tri_pts,
                          float* __restrict__ xs_pts, float* __restrict__ xr_pts, const int32_t* __restrict__ list,
                          const int32_t* __restrict__ count) {
  LevelSet L = L0;
  levelset_init(L);
  const float* h = hh.v;
  const int64_t end = LISTED ? (int64_t)*count : n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < end; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = LISTED ? (int64_t)list[t] : t;
    const uint32_t f = flags[i];
    float p[3];
    load_point(pts, i, p);
    if (dec_crossed(f, kFlagCrossedP) == 0) {
      Cell cell;
      cell_eval(L, p, h, cell);
      int64_t o = tri_off[i] * 3;
      for (int t = 0; t < 5; ++t) {
        float tri[2][3][3];
        int nt = tet_gamma(cell, t, tri);
        for (int q = 0; q < nt; ++q)
          for (int v = 0; v < 3; ++v, ++o)
            for (int a = 0; a < 3; ++a) tri_pts[3 * o + a] = tri[q][v][a];
      }
    }
    if ((f >> kFlagBnd) & 1u) continue;  // box-boundary points have no stencil queries
    int64_t ox = xs_off[i];
    for (int j = 0; j < kStencil; ++j) {
      if (dec_crossed(f, kFlagCrossedS + 2 * j) != 0) continue;
      float s[3];
      stencil_point(p, h, j, s);
      StencilRegression R;
      regression_geometry(L, s, h, R);
      for (int a = 0; a < 3; ++a) {
        xs_pts[3 * ox + a] = s[a];
        xr_pts[3 * ox + a] = R.rproj[a];
      }
      ++ox;
    }
  }
}

// tangent sample (0 where the direction leaves that coefficient unchanged)
__device__ __forceinline__ float tsample(const float* a, int64_t i) { return a ? a[i] : 0.0f; }

// Records of each point (discretization.py:356-424 with the extrapolation of :464-513).
// With TAN the kernel writes, instead of the records, their derivative along a direction in
// coefficient space: dco holds d(sample) of every coefficient sample (NULL arrays: zero) and
// lhs0_out, diag_out, rod_out, A_out receive d lhs0, d diag, d rod and d A (same job order as
// the records; code_out, cnt_out, cntm_out, coeff26_out, beta_int_out are not written).  The
// geometry is the same in both modes and the branches (which phase is extrapolated, which cube
// vertices have a weight) are the records' own, so the tangent is the exact derivative of the
// records as a function of the coefficients.
template <bool TAN, int PASS = kAllPoints>
__global__ void k_assemble(LevelSet L0, const float* __restrict__ pts, int64_t n, H3 hh, const uint32_t* __restrict__ flags,
                           const int64_t* __restrict__ tri_off, const int64_t* __restrict__ xs_off,
                           const int64_t* __restrict__ job_off, dips_coeffs_t co, dips_coeffs_t dco,
                           float* __restrict__ lhs0_out, float* __restrict__ diag_out, float* __restrict__ rod_out,
                           int32_t* __restrict__ cnt_out, int32_t* __restrict__ cntm_out, uint16_t* __restrict__ code_out,
                           float* __restrict__ A_out, float* __restrict__ coeff26_out, float* __restrict__ beta_int_out,
                           float* __restrict__ nl_pt_out, float* __restrict__ nl_w_out,
                           int32_t* __restrict__ heavy_list = nullptr, int32_t* __restrict__ heavy_count = nullptr) {
  LevelSet L = L0;
  levelset_init(L);
  const float* h = hh.v;
  const int64_t end = PASS == kListed ? (int64_t)*heavy_count : n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < end; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = PASS == kListed ? (int64_t)heavy_list[t] : t;
    const uint32_t f = flags[i];
    if (PASS == kDeferHeavy) {
      const bool heavy = heavy_point(f);
      const unsigned act = __activemask();
      const unsigned m = __ballot_sync(act, heavy);
      if (m) {
        const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(heavy_count, __popc(m));
        base = __shfl_sync(act, base, leader);
        if (heavy) heavy_list[base + __popc(m & ((1u << lane) - 1))] = (int32_t)i;
      }
      if (heavy) continue;
    }
    float p[3];
    load_point(pts, i, p);
    const float V = __fmul_rn(__fmul_rn(h[0], h[1]), h[2]);
    int64_t wm = job_off[i];          // u- jobs from the front
    int64_t wp = job_off[i + 1] - 1;  // u+ jobs from the back
    int nm = 0, np = 0;
    // A: the job's coefficient, or its tangent; xm, xp: the job's weights in u- and u+ at the
    // point itself (the nonlinear operator's arguments; only the centre stencil point's jobs
    // have any)
    auto emit = [&](int j, int k, bool netp, float A, float xm = 0.0f, float xp = 0.0f) {
      const int64_t o = netp ? wp : wm;
      if (!TAN) code_out[o] = job_code(j, k, netp);
      A_out[o] = A;
      if (!TAN && nl_w_out) {
        nl_w_out[2 * o] = xm;
        nl_w_out[2 * o + 1] = xp;
      }
      if (netp) {
        --wp;
        ++np;
      } else {
        ++wm;
        ++nm;
      }
    };
    Cell cell;
    // The centre cell's crossing is in the flags (k_classify evaluates the same corners with the
    // same arithmetic).  Off the interface nothing below reads the corners, so they are sampled
    // only for a crossed cell: 8 trilinear phi samples saved at 98 % of the points.
    // (the kDeferHeavy pass sees no crossed cell or stencil point: its instance leaves out that
    // code, so it needs fewer registers)
    const int cpc = dec_crossed(f, kFlagCrossedP);
    if (PASS != kDeferHeavy && cpc == 0)
      cell_eval(L, p, h, cell);
    else
      cell.crossed = cpc;
    float mm[6], mp[6], tmm[6], tmp[6];
    for (int q = 0; q < 6; ++q) {
      mm[q] = co.mu_m_face[6 * i + q];
      mp[q] = co.mu_p_face[6 * i + q];
      tmm[q] = TAN ? tsample(dco.mu_m_face, 6 * i + q) : 0.0f;
      tmp[q] = TAN ? tsample(dco.mu_p_face, 6 * i + q) : 0.0f;
    }
    float c26[26], t26[26];
    if (PASS == kDeferHeavy)
      face_coefficients_uncrossed(cell.crossed, h, mm, mp, c26);
    else
      face_coefficients(cell, p, h, mm, mp, c26);
    if (TAN) {
      // the face fluxes (entries 0..11) are linear in the face mu's; the rest is geometry
      face_coefficients(cell, p, h, tmm, tmp, t26);
      for (int q = 12; q < 26; ++q) t26[q] = 0.0f;
    }
    // interface integral of beta (integrate_over_interface_at_point, geom_pp.py:383-420)
    float bint = 0.0f, tbint = 0.0f;
    if (PASS != kDeferHeavy && cell.crossed == 0) {
      const float b0 = co.beta_origin;
      const float pad_mean = __fdiv_rn(__fadd_rn(__fadd_rn(b0, b0), b0), 3.0f);
      const float pad_term = __fmul_rn(0.0f, pad_mean);
      int64_t o = tri_off[i] * 3;
      bool first = true;
      for (int t = 0; t < 5; ++t) {
        float tri[2][3][3];
        int nt = tet_gamma(cell, t, tri);
        for (int q = 0; q < 2; ++q) {
          float term;
          if (q < nt) {
            float a = tri_area(tri[q][0], tri[q][1], tri[q][2]);
            float b1 = co.beta_tri[o], b2 = co.beta_tri[o + 1], b3 = co.beta_tri[o + 2];
            if (TAN)
              tbint += a * (tsample(dco.beta_tri, o) + tsample(dco.beta_tri, o + 1) + tsample(dco.beta_tri, o + 2)) /
                       3.0f;
            o += 3;
            term = __fmul_rn(a, __fdiv_rn(__fadd_rn(__fadd_rn(b1, b2), b3), 3.0f));
          } else {
            term = pad_term;
          }
          bint = first ? term : __fadd_rn(bint, term);
          first = false;
        }
      }
    }
    if (!TAN && coeff26_out)
      for (int q = 0; q < 26; ++q) coeff26_out[26 * i + q] = c26[q];
    if (!TAN && beta_int_out) beta_int_out[i] = bint;

    if ((f >> kFlagBnd) & 1u) {  // box boundary: lhs = u*V, rhs = g*V (discretization.py:389-393, :410-411)
      const bool net = (f >> kFlagNetS) & 1u;
      emit(0, kCubeCentre, net, TAN ? 0.0f : V);
      lhs0_out[i] = 0.0f;
      if (!TAN && nl_pt_out)  // no nonlinear term on the box boundary (discretization.py:389-393)
        reinterpret_cast<float4*>(nl_pt_out)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (TAN) {
        diag_out[i] = 0.0f;
        rod_out[i] = isfinite(__fdiv_rn(__fmul_rn(co.g[i], V), V)) ? tsample(dco.g, i) : 0.0f;
      } else {
        diag_out[i] = V;
        rod_out[i] = nan_to_num(__fdiv_rn(__fmul_rn(co.g[i], V), V));
        cnt_out[i] = nm + np;
        cntm_out[i] = nm;
      }
      continue;
    }
    const float Vm = c26[12], Vp = c26[13];
    const float km = co.k_m[i], kp = co.k_p[i];
    const float tkm = TAN ? tsample(dco.k_m, i) : 0.0f, tkp = TAN ? tsample(dco.k_p, i) : 0.0f;
    float se = c26[0], so = c26[1], tse = t26[0], tso = t26[1];
    for (int q = 1; q < 6; ++q) {
      se = __fadd_rn(se, c26[2 * q]);
      so = __fadd_rn(so, c26[2 * q + 1]);
      if (TAN) {
        tse += t26[2 * q];
        tso += t26[2 * q + 1];
      }
    }
    const float diag =
        __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(kp, Vp), __fmul_rn(km, Vm)), se), so);
    float rhs = __fadd_rn(__fmul_rn(co.f_m[i], Vm), __fmul_rn(co.f_p[i], Vp));
    rhs = __fadd_rn(rhs, bint);
    float tdiag = 0.0f, trhs = 0.0f;
    if (TAN) {
      tdiag = tkp * Vp + tkm * Vm + tse + tso;
      trhs = tsample(dco.f_m, i) * Vm + tsample(dco.f_p, i) * Vp + tbint;
    }
    float Am[kStencil], Ap[kStencil], tAm[kStencil], tAp[kStencil];
    Am[0] = __fadd_rn(__fmul_rn(km, Vm), se);
    Ap[0] = __fadd_rn(__fmul_rn(kp, Vp), so);
    tAm[0] = tkm * Vm + tse;
    tAp[0] = tkp * Vp + tso;
    for (int j = 1; j < kStencil; ++j) {
      Am[j] = -c26[2 * (j - 1)];
      Ap[j] = -c26[2 * (j - 1) + 1];
      tAm[j] = -t26[2 * (j - 1)];
      tAp[j] = -t26[2 * (j - 1) + 1];
    }
    float lhs0 = 0.0f, tlhs0 = 0.0f;
    // the nonlinear operator's arguments at the point (discretization.py:369 with u_mp_at_point,
    // :426-519): u- = Km + sum of the jobs' xm weights times their values, u+ likewise.  A point
    // off the interface has u- = u (in Omega-) and u+ = 0, or the reverse.
    float nlK[2] = {0.0f, 0.0f};
    int64_t ox = xs_off[i];
    for (int j = 0; j < kStencil; ++j) {
      const int cj = dec_crossed(f, kFlagCrossedS + 2 * j);
      const bool netj = (f >> (kFlagNetS + j)) & 1u;
      if (cj == -1) {
        emit(j, kCubeCentre, netj, TAN ? tAm[j] : Am[j], j == 0 ? 1.0f : 0.0f, 0.0f);
        continue;
      }
      if (cj == 1) {
        emit(j, kCubeCentre, netj, TAN ? tAp[j] : Ap[j], 0.0f, j == 0 ? 1.0f : 0.0f);
        continue;
      }
      if (PASS == kDeferHeavy) continue;  // not reached: such points are listed
      // interface stencil point: extrapolate the other phase (discretization.py:464-513)
      float s[3];
      stencil_point(p, h, j, s);
      StencilRegression R;
      regression_geometry(L, s, h, R);
      bool wpos[27], wneg[27];
      for (int k = 0; k < 27; ++k) {
        wpos[k] = R.phi_v[k] > 0.0f;
        wneg[k] = R.phi_v[k] < 0.0f;
      }
      const float mus_m = co.mu_m_s[ox], mus_p = co.mu_p_s[ox];
      const float alpha = co.alpha_r[ox], beta = co.beta_r[ox];
      const float mur_m = co.mu_m_r[ox], mur_p = co.mu_p_r[ox];
      const float tmus_m = TAN ? tsample(dco.mu_m_s, ox) : 0.0f, tmus_p = TAN ? tsample(dco.mu_p_s, ox) : 0.0f;
      const float talpha = TAN ? tsample(dco.alpha_r, ox) : 0.0f, tbeta = TAN ? tsample(dco.beta_r, ox) : 0.0f;
      const float tmur_m = TAN ? tsample(dco.mu_m_r, ox) : 0.0f, tmur_p = TAN ? tsample(dco.mu_p_r, ox) : 0.0f;
      ++ox;
      const bool mbig = mus_m > mus_p;
      const float delta = R.phi_s;
      const bool pos = delta > 0.0f;
      // regression on the phase whose normal derivative enters the extrapolation:
      // mu- > mu+ uses Omega^- (C^-), otherwise Omega^+ (C^+)
      float D[3][27];
      lsq_operator(h, mbig ? wneg : wpos, D);
      float C[27];
      for (int k = 0; k < 27; ++k)
        C[k] = __fadd_rn(__fadd_rn(__fmul_rn(R.n[0], D[0][k]), __fmul_rn(R.n[1], D[1][k])), __fmul_rn(R.n[2], D[2][k]));
      // zeta^-_pqm = ((mu+ - mu-)/mu+) phi C^- ; zeta^+_pqm = ((mu+ - mu-)/mu-) phi C^+
      const float mden = mbig ? mus_p : mus_m, tmden = mbig ? tmus_p : tmus_m;
      const float fac = __fmul_rn(__fdiv_rn(__fsub_rn(mus_p, mus_m), mden), delta);
      const float tfac = TAN ? delta * ((tmus_p - tmus_m) / mden - (mus_p - mus_m) * tmden / (mden * mden)) : 0.0f;
      float Z[27];
      float zsum = 0.0f, csum_off = 0.0f;
      for (int k = 0; k < 27; ++k) {
        Z[k] = __fmul_rn(fac, C[k]);
        zsum = (k == 0) ? Z[k] : __fadd_rn(zsum, Z[k]);
        if (k != kCubeCentre) csum_off += C[k];
      }
      const float zeta = -__fsub_rn(zsum, Z[kCubeCentre]);
      const float tzeta = -tfac * csum_off;
      // gamma^-_pqm = zeta^-_pqm / (1 - zeta^-); gamma^+_pqm = zeta^+_pqm / (1 + zeta^+)
      const bool use_gamma = (mbig && pos) || (!mbig && !pos);
      float G[27];
      float g;
      float tg = tzeta, den = 1.0f, tden = 0.0f;
      if (use_gamma) {
        den = mbig ? __fsub_rn(1.0f, zeta) : __fadd_rn(1.0f, zeta);
        tden = mbig ? -tzeta : tzeta;
        float gsum = 0.0f;
        tg = 0.0f;
        for (int k = 0; k < 27; ++k) {
          G[k] = __fdiv_rn(Z[k], den);
          gsum = (k == 0) ? G[k] : __fadd_rn(gsum, G[k]);
          if (TAN && k != kCubeCentre) tg -= (tfac * C[k]) / den - Z[k] * tden / (den * den);
        }
        g = -__fsub_rn(gsum, G[kCubeCentre]);
      } else {
        for (int k = 0; k < 27; ++k) G[k] = Z[k];
        g = zeta;
      }
      // tangent of G[k]
      auto tG = [&](int k) -> float {
        return use_gamma ? (tfac * C[k]) / den - Z[k] * tden / (den * den) : tfac * C[k];
      };
      // constant term of the extrapolated value
      const float mur = mbig ? mur_p : mur_m, tmur = mbig ? tmur_p : tmur_m;
      const float bmu = __fdiv_rn(beta, mur);
      const float jump = __fadd_rn(alpha, __fmul_rn(delta, bmu));
      const float tjump = talpha + delta * (tbeta / mur - beta * tmur / (mur * mur));
      float K, tK;
      if (mbig) {
        K = pos ? __fmul_rn(__fmul_rn(-1.0f, __fsub_rn(1.0f, g)), jump) : jump;
        tK = pos ? tg * jump - (1.0f - g) * tjump : tjump;
      } else {
        K = pos ? __fmul_rn(-1.0f, jump) : __fmul_rn(__fsub_rn(1.0f, g), jump);
        tK = pos ? -tjump : -tg * jump + (1.0f - g) * tjump;
      }
      const float Ax = pos ? Am[j] : Ap[j];  // coefficient of the extrapolated component
      const float Ao = pos ? Ap[j] : Am[j];  // coefficient of u itself
      const float tAx = pos ? tAm[j] : tAp[j], tAo = pos ? tAp[j] : tAm[j];
      const float wc = __fadd_rn(__fsub_rn(__fmul_rn(Ax, __fadd_rn(__fsub_rn(1.0f, g), G[kCubeCentre])),
                                           __fmul_rn(Ax, G[kCubeCentre])),
                                 Ao);
      // at the centre stencil point: the extrapolated component (u- if pos, else u+) weighs the
      // point's own value by (1 - g + G[centre]) - G[centre] and vertex k by -G[k], plus K; the
      // other component is the point's own value
      const bool c0 = j == 0;
      const float xself = c0 ? __fsub_rn(__fadd_rn(__fsub_rn(1.0f, g), G[kCubeCentre]), G[kCubeCentre]) : 0.0f;
      // d wc: Ax (1 - g) + Ao as a function (the G[centre] terms cancel)
      emit(j, kCubeCentre, netj, TAN ? tAx * (1.0f - g) - Ax * tg + tAo : wc, c0 ? (pos ? xself : 1.0f) : 0.0f,
           c0 ? (pos ? 1.0f : xself) : 0.0f);
      for (int k = 0; k < 27; ++k) {
        if (k == kCubeCentre || G[k] == 0.0f) continue;
        const float xk = c0 ? -G[k] : 0.0f;
        emit(j, k, R.phi_v[k] >= 0.0f, TAN ? -(tAx * G[k] + Ax * tG(k)) : -__fmul_rn(Ax, G[k]), pos ? xk : 0.0f,
             pos ? 0.0f : xk);
      }
      if (c0) nlK[pos ? 0 : 1] = K;
      lhs0 = __fadd_rn(lhs0, __fmul_rn(Ax, K));
      if (TAN) tlhs0 += tAx * K + Ax * tK;
    }
    if (TAN) {
      const float q = __fdiv_rn(rhs, diag);
      lhs0_out[i] = tlhs0;
      diag_out[i] = tdiag;
      rod_out[i] = isfinite(q) ? (trhs - q * tdiag) / diag : 0.0f;
    } else {
      lhs0_out[i] = lhs0;
      diag_out[i] = diag;
      rod_out[i] = nan_to_num(__fdiv_rn(rhs, diag));
      cnt_out[i] = nm + np;
      cntm_out[i] = nm;
      if (nl_pt_out) reinterpret_cast<float4*>(nl_pt_out)[i] = make_float4(nlK[0], nlK[1], Vm, Vp);
    }
  }
}

static int grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g > 152 * 64) g = 152 * 64;
  if (g < 1) g = 1;
  return (int)g;
}

static int make_ls(const dips_levelset_t* ls, LevelSet* L, cudaStream_t stream) {
  (void)stream;
  DIPS_REQUIRE(ls && ls->phi_gh && ls->xg && ls->yg && ls->zg, DIPS_E_ARG, "levelset: null pointer");
  DIPS_REQUIRE(ls->nx >= 2 && ls->ny >= 2 && ls->nz >= 2, DIPS_E_ARG, "levelset: need at least 2 samples per axis");
  *L = make_levelset(*ls);
  return DIPS_OK;
}

}  // namespace dips

using namespace dips;

extern "C" int dips_phi_ghost_layer(const float* phi, int32_t nx, int32_t ny, int32_t nz, float* phi_gh,
                                    cudaStream_t stream) {
  DIPS_REQUIRE(phi && phi_gh, DIPS_E_ARG, "dips_phi_ghost_layer: null pointer");
  DIPS_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, DIPS_E_ARG, "dips_phi_ghost_layer: need at least 2 samples per axis");
  int64_t total = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
  k_ghost_layer<<<grid_for(total, 256), 256, 0, stream>>>(phi, nx, ny, nz, phi_gh);
  DIPS_CHECK_LAUNCH("dips_phi_ghost_layer");
  return DIPS_OK;
}

extern "C" int dips_phi_trilinear(const dips_levelset_t* ls, const float* pts, int64_t n, float* out,
                                  cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0, DIPS_E_ARG, "dips_phi_trilinear: negative n");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && out, DIPS_E_ARG, "dips_phi_trilinear: null pointer");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  k_trilinear<<<grid_for(n, 256), 256, 0, stream>>>(L, pts, n, out);
  DIPS_CHECK_LAUNCH("dips_phi_trilinear");
  return DIPS_OK;
}

extern "C" int dips_phi_quadratic(const dips_levelset_t* ls, const float* pts, int64_t n, float* out,
                                  cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0, DIPS_E_ARG, "dips_phi_quadratic: negative n");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && out, DIPS_E_ARG, "dips_phi_quadratic: null pointer");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  k_quadratic<<<grid_for(n, 256), 256, 0, stream>>>(L, pts, n, out);
  DIPS_CHECK_LAUNCH("dips_phi_quadratic");
  return DIPS_OK;
}

static H3 make_h(const float h[3]) {
  H3 r;
  r.v[0] = h[0];
  r.v[1] = h[1];
  r.v[2] = h[2];
  return r;
}

extern "C" int dips_geometry_classify(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                      uint32_t* flags, int32_t* n_tri, int32_t* n_xs, int32_t* job_cap,
                                      cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0 && h, DIPS_E_ARG, "dips_geometry_classify: bad n or h");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && flags && n_tri && n_xs && job_cap, DIPS_E_ARG, "dips_geometry_classify: null pointer");
  DIPS_REQUIRE(h[0] > 0 && h[1] > 0 && h[2] > 0, DIPS_E_ARG, "dips_geometry_classify: spacing must be positive");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  k_classify<<<grid_for(n, 128), 128, 0, stream>>>(L, pts, n, make_h(h), flags, n_tri, n_xs, job_cap);
  DIPS_CHECK_LAUNCH("dips_geometry_classify");
  return DIPS_OK;
}

extern "C" int dips_geometry_queries(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                     const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                     float* tri_pts, float* xs_pts, float* xr_pts, cudaStream_t stream) {
  return dips_geometry_queries_ex(ls, pts, n, h, flags, tri_off, xs_off, tri_pts, xs_pts, xr_pts, nullptr, 0, stream);
}

extern "C" int dips_geometry_queries_ex(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                        const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                        float* tri_pts, float* xs_pts, float* xr_pts, void* scratch,
                                        size_t scratch_bytes, cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0 && h, DIPS_E_ARG, "dips_geometry_queries: bad n or h");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && flags && tri_off && xs_off, DIPS_E_ARG, "dips_geometry_queries: null pointer");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  if (!scratch) {
    k_queries<false><<<grid_for(n, 128), 128, 0, stream>>>(L, pts, n, make_h(h), flags, tri_off, xs_off, tri_pts,
                                                           xs_pts, xr_pts, nullptr, nullptr);
    DIPS_CHECK_LAUNCH("dips_geometry_queries");
    return DIPS_OK;
  }
  DIPS_REQUIRE(scratch_bytes >= dips_geometry_assemble_scratch_bytes(n) && ((uintptr_t)scratch & 3) == 0,
               DIPS_E_WORKSPACE, "dips_geometry_queries_ex: scratch too small or misaligned");
  int32_t* count = static_cast<int32_t*>(scratch);
  int32_t* list = count + 1;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int32_t), stream);
  if (e != cudaSuccess) return cuda_status(e, "dips_geometry_queries_ex: scratch counter");
  k_heavy_list<<<grid_for(n, 256), 256, 0, stream>>>(flags, n, list, count);
  k_queries<true><<<grid_for(n, 128), 128, 0, stream>>>(L, pts, n, make_h(h), flags, tri_off, xs_off, tri_pts, xs_pts,
                                                        xr_pts, list, count);
  DIPS_CHECK_LAUNCH("dips_geometry_queries_ex");
  return DIPS_OK;
}

extern "C" int dips_geometry_assemble(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                      const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                      const int64_t* job_off, const dips_coeffs_t* co, float* lhs0, float* diag,
                                      float* rod, int32_t* cnt, int32_t* cnt_m, uint16_t* job_code, float* job_A,
                                      float* coeff26, float* beta_int, cudaStream_t stream) {
  return dips_geometry_assemble_ex(ls, pts, n, h, flags, tri_off, xs_off, job_off, co, lhs0, diag, rod, cnt, cnt_m,
                                   job_code, job_A, coeff26, beta_int, nullptr, nullptr, nullptr, 0, stream);
}

extern "C" size_t dips_geometry_assemble_scratch_bytes(int64_t n) {
  return n <= 0 ? 0 : (size_t)(n + 1) * sizeof(int32_t);
}

extern "C" int dips_geometry_assemble_ex(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                         const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                         const int64_t* job_off, const dips_coeffs_t* co, float* lhs0, float* diag,
                                         float* rod, int32_t* cnt, int32_t* cnt_m, uint16_t* job_code, float* job_A,
                                         float* coeff26, float* beta_int, float* nl_pt, float* nl_w, void* scratch,
                                         size_t scratch_bytes, cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0 && h && co, DIPS_E_ARG, "dips_geometry_assemble: bad n, h or coeffs");
  DIPS_REQUIRE((nl_pt == nullptr) == (nl_w == nullptr), DIPS_E_ARG,
               "dips_geometry_assemble_ex: nl_pt and nl_w are given together");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && flags && tri_off && xs_off && job_off && lhs0 && diag && rod && cnt && cnt_m && job_code && job_A,
               DIPS_E_ARG, "dips_geometry_assemble: null pointer");
  DIPS_REQUIRE(co->mu_m_face && co->mu_p_face && co->k_m && co->k_p && co->f_m && co->f_p && co->g, DIPS_E_ARG,
               "dips_geometry_assemble: null dense coefficient pointer");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  dips_coeffs_t none{};
  if (!scratch) {
    k_assemble<false><<<grid_for(n, 64), 64, 0, stream>>>(L, pts, n, make_h(h), flags, tri_off, xs_off, job_off, *co,
                                                          none, lhs0, diag, rod, cnt, cnt_m, job_code, job_A, coeff26,
                                                          beta_int, nl_pt, nl_w);
    DIPS_CHECK_LAUNCH("dips_geometry_assemble");
    return DIPS_OK;
  }
  DIPS_REQUIRE(scratch_bytes >= dips_geometry_assemble_scratch_bytes(n) && ((uintptr_t)scratch & 3) == 0,
               DIPS_E_WORKSPACE, "dips_geometry_assemble_ex: scratch too small or misaligned");
  int32_t* count = static_cast<int32_t*>(scratch);
  int32_t* list = count + 1;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int32_t), stream);
  if (e != cudaSuccess) return cuda_status(e, "dips_geometry_assemble_ex: scratch counter");
  k_assemble<false, kDeferHeavy><<<grid_for(n, 64), 64, 0, stream>>>(
      L, pts, n, make_h(h), flags, tri_off, xs_off, job_off, *co, none, lhs0, diag, rod, cnt, cnt_m, job_code, job_A,
      coeff26, beta_int, nl_pt, nl_w, list, count);
  k_assemble<false, kListed><<<grid_for(n, 64), 64, 0, stream>>>(
      L, pts, n, make_h(h), flags, tri_off, xs_off, job_off, *co, none, lhs0, diag, rod, cnt, cnt_m, job_code, job_A,
      coeff26, beta_int, nl_pt, nl_w, list, count);
  DIPS_CHECK_LAUNCH("dips_geometry_assemble_ex");
  return DIPS_OK;
}

extern "C" int dips_geometry_assemble_tangent(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                              const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                              const int64_t* job_off, const dips_coeffs_t* co, const dips_coeffs_t* dco,
                                              float* d_lhs0, float* d_diag, float* d_rod, float* d_job_A,
                                              cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0 && h && co && dco, DIPS_E_ARG, "dips_geometry_assemble_tangent: bad n, h or coeffs");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(pts && flags && tri_off && xs_off && job_off && d_lhs0 && d_diag && d_rod && d_job_A, DIPS_E_ARG,
               "dips_geometry_assemble_tangent: null pointer");
  DIPS_REQUIRE(co->mu_m_face && co->mu_p_face && co->k_m && co->k_p && co->f_m && co->f_p && co->g, DIPS_E_ARG,
               "dips_geometry_assemble_tangent: null dense coefficient pointer");
  LevelSet L;
  int st = make_ls(ls, &L, stream);
  if (st) return st;
  k_assemble<true><<<grid_for(n, 64), 64, 0, stream>>>(L, pts, n, make_h(h), flags, tri_off, xs_off, job_off, *co,
                                                       *dco, d_lhs0, d_diag, d_rod, nullptr, nullptr, nullptr, d_job_A,
                                                       nullptr, nullptr, nullptr, nullptr);
  DIPS_CHECK_LAUNCH("dips_geometry_assemble_tangent");
  return DIPS_OK;
}
