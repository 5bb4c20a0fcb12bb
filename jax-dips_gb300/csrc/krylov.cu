// Plain method: matrix-free BiCGSTAB on the same FV stencil records (sm_103a).
//
// The reference's discrete operator (compute_Ax_and_b_discrete_fn,
// solvers/poisson/discretization.py:522-741, wrapped as Trainer.residual_vector,
// solvers/poisson/trainer.py:883-890) evaluates the FV residual of a nodal vector u on a
// grid that is also the training and level-set grid.  Its u values at stencil and cube
// points are grid-node values, so row p of the residual reads the same per-point records
// as the NBM path with each job's network value replaced by u at the job's grid node:
//     r_p(u) = nan_to_num((lhs0_p + sum_j A_j u[node_j]) / diag_p) - rod_p
// which is affine in u: r(u) = K u - b.  BiCGSTAB solves K u = b with float32 vectors and
// FP64 inner products; the scalar recurrences stay on the device, and the iterations between
// two host checks run in one cooperative launch (k_bicg_coop).
//
// At a node of the lowest layer of an axis the reference's operator does not read the nodal
// value: its quadratic interpolant (interpolate.py:572-759) clamps the first cell and
// extrapolates 2 u_1 - u_2 + min|second difference|, which is not linear in u.  Here every
// job reads its node's value, so K is linear (as BiCGSTAB needs) and equals the reference's
// operator on every row whose stencil and regression cube stay off those layers.

#include <math.h>

#include <cooperative_groups.h>

#include "dips_common.cuh"

namespace dips {

constexpr int kKThreads = 256;
constexpr int kKGrid = 152 * 8;
constexpr int kGenGrid = 152 * 8;  // blocks of the general-row kernels (8 warps each, a warp per row)

struct Grid3 {
  int nx, ny, nz;
};

// grid node of job code c of the row at (i, j, k): stencil offset + cube offset, clamped to the
// grid (the row's coordinates are computed once per row, so a job costs no integer division
// beyond the constant ones that decode its code)
__device__ __forceinline__ int64_t job_node(int i, int j, int k, uint16_t c, const Grid3& g) {
  const int st = job_stencil(c), v = job_vertex(c);
  if (st > 0) {
    const int a = (st - 1) >> 1, d = ((st - 1) & 1) ? 1 : -1;
    if (a == 0) i += d;
    if (a == 1) j += d;
    if (a == 2) k += d;
  }
  i += v % 3 - 1;
  j += (v / 3) % 3 - 1;
  k += v / 9 - 1;
  i = i < 0 ? 0 : (i >= g.nx ? g.nx - 1 : i);
  j = j < 0 ? 0 : (j >= g.ny ? g.ny - 1 : j);
  k = k < 0 ? 0 : (k >= g.nz ? g.nz - 1 : k);
  return ((int64_t)i * g.ny + j) * g.nz + k;
}

// A bulk row: 7 stencil jobs of one network (interior), with its packed record.
__device__ __forceinline__ bool bulk_row(const dips_records_t& rec, int64_t p) {
  const int c = rec.cnt[p], m = rec.cnt_m[p];
  return rec.bulk_rec && c == kStencil && (m == kStencil || m == 0);
}

// (K x)_p of a bulk row: the 7 coefficients in stencil order and diag from the packed record,
// the 7 neighbouring nodes of the grid directly
__device__ __forceinline__ float bulk_apply(const dips_records_t& rec, const Grid3& g, int64_t p,
                                            const float* __restrict__ x) {
  const float4* r4 = reinterpret_cast<const float4*>(rec.bulk_rec + p * 16);
  const float4 a = __ldg(r4 + 1), b = __ldg(r4 + 2);  // A0..A3; A4..A6, diag
  const int64_t sj = g.nz, si = (int64_t)g.ny * g.nz;
  float acc = a.x * __ldg(x + p);
  acc = fmaf(a.y, __ldg(x + p - si), acc);
  acc = fmaf(a.z, __ldg(x + p + si), acc);
  acc = fmaf(a.w, __ldg(x + p - sj), acc);
  acc = fmaf(b.x, __ldg(x + p + sj), acc);
  acc = fmaf(b.y, __ldg(x + p - 1), acc);
  acc = fmaf(b.z, __ldg(x + p + 1), acc);
  const float v = acc / b.w;
  return isfinite(v) ? v : 0.0f;
}

// (K x)_gp of any row by the whole warp, the lanes splitting its jobs (up to 7 x 27); every lane
// gets the value
__device__ __forceinline__ float general_apply_warp(const dips_records_t& rec, const Grid3& g, int64_t gp,
                                                    const float* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  const int64_t o0 = rec.job_off[gp], o1 = rec.job_off[gp + 1];
  const int cm = rec.cnt_m[gp], n = rec.cnt[gp];
  const int k = (int)(gp % g.nz);
  const int j = (int)((gp / g.nz) % g.ny);
  const int i = (int)(gp / ((int64_t)g.ny * g.nz));
  float part = 0.0f;
  for (int q = lane; q < n; q += 32) {
    const int64_t o = q < cm ? o0 + q : o1 - n + q;  // u- jobs at the front, u+ jobs at the back
    part = fmaf(rec.job_A[o], __ldg(x + job_node(i, j, k, rec.job_code[o], g)), part);
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) part += __shfl_xor_sync(0xffffffffu, part, s);
  const float v = part / rec.diag[gp];
  return isfinite(v) ? v : 0.0f;
}

// (K x)_gp of any row by one thread, its jobs in order (u- jobs at the front, u+ at the back)
__device__ __forceinline__ float general_apply_thread(const dips_records_t& rec, const Grid3& g, int64_t gp,
                                                      const float* __restrict__ x) {
  const int64_t o0 = rec.job_off[gp], o1 = rec.job_off[gp + 1];
  const int cm = rec.cnt_m[gp], n = rec.cnt[gp];
  const int k = (int)(gp % g.nz);
  const int j = (int)((gp / g.nz) % g.ny);
  const int i = (int)(gp / ((int64_t)g.ny * g.nz));
  float acc = 0.0f;
  for (int q = 0; q < n; ++q) {
    const int64_t o = q < cm ? o0 + q : o1 - n + q;
    acc = fmaf(rec.job_A[o], __ldg(x + job_node(i, j, k, rec.job_code[o], g)), acc);
  }
  const float v = acc / rec.diag[gp];
  return isfinite(v) ? v : 0.0f;
}

// (K x)_p of the rows p of one warp (valid lanes): bulk rows inline, the others one at a time
// by the whole warp.  All 32 lanes call it.
__device__ __forceinline__ float warp_apply(const dips_records_t& rec, const Grid3& g, int64_t p, bool valid,
                                            const float* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  float out = 0.0f;
  bool gen = false;
  if (valid) {
    if (bulk_row(rec, p))
      out = bulk_apply(rec, g, p, x);
    else
      gen = true;
  }
  unsigned todo = __ballot_sync(0xffffffffu, gen);
  while (todo) {
    const int owner = __ffs(todo) - 1;
    todo &= todo - 1;
    const int64_t gp = __shfl_sync(0xffffffffu, p, owner);
    const float v = general_apply_warp(rec, g, gp, x);
    if (lane == owner) out = v;
  }
  return out;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  return v;
}

// block-reduce up to 3 doubles and write one partial per block
__device__ __forceinline__ void block_partials(double a, double b, double c, double* part, int nvals) {
  __shared__ double s[3][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  if (lane == 0) {
    s[0][wid] = a;
    s[1][wid] = b;
    s[2][wid] = c;
  }
  __syncthreads();
  if (wid == 0) {
    double x0 = lane < nw ? s[0][lane] : 0.0, x1 = lane < nw ? s[1][lane] : 0.0, x2 = lane < nw ? s[2][lane] : 0.0;
    x0 = warp_sum(x0);
    x1 = warp_sum(x1);
    x2 = warp_sum(x2);
    if (lane == 0) {
      part[blockIdx.x * 3 + 0] = x0;
      if (nvals > 1) part[blockIdx.x * 3 + 1] = x1;
      if (nvals > 2) part[blockIdx.x * 3 + 2] = x2;
    }
  }
}

// residual of a nodal vector: out = K u - b (linear_only: K u)
// rows of a warp-aligned grid-stride loop: the stride is a multiple of 32, so the warps stay whole
#define DIPS_ROWS(p, valid, n)                                                                               \
  for (int64_t p##0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31), p = p##0 + (threadIdx.x & 31); \
       p##0 < (n); p##0 += (int64_t)gridDim.x * blockDim.x, p = p##0 + (threadIdx.x & 31))                   \
    if (const bool valid = p < (n); true)

__global__ void k_fv_residual(dips_records_t rec, Grid3 g, const float* __restrict__ u, int linear_only,
                              float* __restrict__ out) {
  DIPS_ROWS(p, valid, rec.n_pts) {
    const float Ku = warp_apply(rec, g, p, valid, u);
    if (!valid) continue;
    if (linear_only) {
      out[p] = Ku;
    } else {
      const float d = rec.diag[p];
      const float c = nan_to_num(rec.lhs0[p] / d);
      out[p] = Ku + c - rec.rod[p];
    }
  }
}

// BiCGSTAB state on the device: scalars in double
struct KState {
  double rho, alpha, omega, beta;
  double rhat_v, ts, tt, rho_new, rr, bb;
  int64_t breakdown;
};

struct KVecs {
  float *x, *r, *rhat, *p, *v, *s, *t;
  double* part;     // [(kKGrid + kGenGrid) * 3]: per-block partial inner products
  int32_t* glist;   // [n] the general rows (found once per solve)
  int32_t* gcount;  // their number
  KState* st;
  float* err_part;  // [kKGrid] max |x - u_exact|
  float4* coef;     // [n][2] bulk rows: A_0..A_6 (stencil order) and diag, packed once per solve
  uint8_t* gen;     // [n] 1 for a general row (warp path), 0 for a bulk row
};


// The rows whose product needs the warp-cooperative path, listed once per solve (the order of
// the list depends on the warps' arrival; each row's value does not)
__global__ void k_general_rows(dips_records_t rec, int32_t* __restrict__ list, int32_t* __restrict__ count) {
  const int lane = threadIdx.x & 31;
  DIPS_ROWS(p, valid, rec.n_pts) {
    const bool gen = valid && !bulk_row(rec, p);
    const unsigned m = __ballot_sync(0xffffffffu, gen);
    if (!m) continue;
    int base = 0;
    if (lane == 0) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (gen) list[base + __popc(m & ((1u << lane) - 1))] = (int32_t)p;
  }
}

// what a product feeds, per row i with (K x)_i = kx
enum KMode {
  kInit = 0,    // r = b - K x, rhat = r, p = v = 0; partials (r, r), (b, b)
  kApplyV = 1,  // v = K p; partial (rhat, v)
  kApplyT = 2,  // t = K s; partials (t, s), (t, t)
};

template <int MODE>
__device__ __forceinline__ void row_done(const dips_records_t& rec, const KVecs& V, int64_t i, float kx, double& a0,
                                         double& a1) {
  if (MODE == kInit) {
    const float d = rec.diag[i];
    const float b = rec.rod[i] - nan_to_num(rec.lhs0[i] / d);
    const float r = b - kx;
    V.r[i] = r;
    V.rhat[i] = r;
    V.p[i] = 0.0f;
    V.v[i] = 0.0f;
    a0 += (double)r * r;
    a1 += (double)b * b;
  } else if (MODE == kApplyV) {
    V.v[i] = kx;
    a0 += (double)V.rhat[i] * kx;
  } else {
    V.t[i] = kx;
    a0 += (double)kx * V.s[i];
    a1 += (double)kx * kx;
  }
}

// the bulk rows of the product (a thread per row); partials in V.part[0, kKGrid)
template <int MODE>
__global__ void k_apply_bulk(dips_records_t rec, Grid3 g, const float* __restrict__ x, KVecs V) {
  double a0 = 0.0, a1 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rec.n_pts; i += (int64_t)gridDim.x * blockDim.x)
    if (bulk_row(rec, i)) row_done<MODE>(rec, V, i, bulk_apply(rec, g, i, x), a0, a1);
  block_partials(a0, a1, 0.0, V.part, 2);
}

// the listed general rows (a warp per row); partials in V.part[kKGrid, kKGrid + kGenGrid)
template <int MODE>
__global__ void k_apply_general(dips_records_t rec, Grid3 g, const float* __restrict__ x, KVecs V) {
  const int lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int64_t cnt = *V.gcount;
  double a0 = 0.0, a1 = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * nw + (threadIdx.x >> 5); k < cnt; k += (int64_t)gridDim.x * nw) {
    const int64_t gp = V.glist[k];
    const float kx = general_apply_warp(rec, g, gp, x);
    if (lane == 0) row_done<MODE>(rec, V, gp, kx, a0, a1);
  }
  block_partials(a0, a1, 0.0, V.part + 3 * kKGrid, 2);
}

__global__ void k_bicg_init_scalars(KVecs V, int nblk) {
  double rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    rr += V.part[3 * i];
    bb += V.part[3 * i + 1];
  }
  __shared__ double s[2][32];
  rr = warp_sum(rr);
  bb = warp_sum(bb);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s[0][wid] = rr;
    s[1][wid] = bb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int q = 0; q < nw; ++q) {
      a += s[0][q];
      b += s[1][q];
    }
    V.st->rho = 1.0;
    V.st->alpha = 1.0;
    V.st->omega = 1.0;
    V.st->rho_new = a;  // (rhat, r) = (r, r) at start
    V.st->rr = a;
    V.st->bb = b;
    V.st->beta = 0.0;
    V.st->breakdown = 0;
  }
}

// ---- persistent BiCGSTAB ------------------------------------------------------------------------
// The whole iteration runs in one cooperative launch (check_every iterations per launch): its
// phases are separated by grid-wide barriers (all blocks co-resident by the cooperative launch),
// and every block reduces the per-block inner-product partials itself, in one fixed order, so
// all blocks hold the same recurrence scalars without another barrier and the result does not
// depend on timing.  Per iteration: 2 matrix-free products and 5 barriers, no host work.

// packs each bulk row's 7 stencil coefficients and diag (32 bytes, from its packed record) and
// flags the general rows, once per solve
__global__ void k_krylov_pack(dips_records_t rec, float4* __restrict__ coef, uint8_t* __restrict__ gen) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rec.n_pts; i += (int64_t)gridDim.x * blockDim.x) {
    const bool b = bulk_row(rec, i);
    gen[i] = b ? 0 : 1;
    if (b) {
      const float4* r4 = reinterpret_cast<const float4*>(rec.bulk_rec + i * 16);
      coef[2 * i] = r4[1];
      coef[2 * i + 1] = r4[2];
    }
  }
}

// (K x)_i of a bulk row from its packed coefficients (the same operations as bulk_apply)
__device__ __forceinline__ float coef_apply(const float4* __restrict__ coef, const Grid3& g, int64_t p,
                                            const float* __restrict__ x) {
  const float4 a = __ldg(coef + 2 * p), b = __ldg(coef + 2 * p + 1);
  const int64_t sj = g.nz, si = (int64_t)g.ny * g.nz;
  float acc = a.x * __ldg(x + p);
  acc = fmaf(a.y, __ldg(x + p - si), acc);
  acc = fmaf(a.z, __ldg(x + p + si), acc);
  acc = fmaf(a.w, __ldg(x + p - sj), acc);
  acc = fmaf(b.x, __ldg(x + p + sj), acc);
  acc = fmaf(b.y, __ldg(x + p - 1), acc);
  acc = fmaf(b.z, __ldg(x + p + 1), acc);
  const float v = acc / b.w;
  return isfinite(v) ? v : 0.0f;
}

// sum of the first `nv` columns of the grid's partials, in one fixed order; every thread of the
// block gets the sums
__device__ __forceinline__ void reduce_all(const double* part, int nblk, int nv, double out[3]) {
  __shared__ double s[3][32];
  __shared__ double res[3];
  double a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += part[3 * i];
    if (nv > 1) b += part[3 * i + 1];
    if (nv > 2) c += part[3 * i + 2];
  }
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s[0][wid] = a;
    s[1][wid] = b;
    s[2][wid] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x0 = 0, x1 = 0, x2 = 0;
    for (int q = 0; q < nw; ++q) {
      x0 += s[0][q];
      x1 += s[1][q];
      x2 += s[2][q];
    }
    res[0] = x0;
    res[1] = x1;
    res[2] = x2;
  }
  __syncthreads();
  out[0] = res[0];
  out[1] = res[1];
  out[2] = res[2];
  __syncthreads();
}

// one product over all rows (bulk rows a thread each, listed general rows a warp each), with the
// row's follow-up of MODE; per-block partials into part
template <int MODE>
__device__ __forceinline__ void coop_apply(const dips_records_t& rec, const Grid3& g, const float* __restrict__ x,
                                           const KVecs& V, int64_t n, int64_t gcnt, double* part) {
  double a0 = 0.0, a1 = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    if (!V.gen[i]) row_done<MODE>(rec, V, i, coef_apply(V.coef, g, i, x), a0, a1);
  // general rows a thread each: about one row per thread at 128^3 (136,680 rows, 15 jobs on
  // average), so their dependent loads overlap across the grid instead of queueing per warp
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < gcnt; k += stride) {
    const int64_t gp = V.glist[k];
    row_done<MODE>(rec, V, gp, general_apply_thread(rec, g, gp, x), a0, a1);
  }
  block_partials(a0, a1, 0.0, part, 2);
}

// `iters` BiCGSTAB iterations (it0 = the global number of the first); the recurrence state is
// read from and written back to V.st (block 0)
__global__ void __launch_bounds__(kKThreads, 4) k_bicg_coop(dips_records_t rec, Grid3 g, KVecs V, int64_t n, int it0,
                                                         int iters) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  const int nblk = gridDim.x;
  const int64_t gcnt = *V.gcount;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // two partial buffers: the x/r update writes its partials right after the blocks read the
  // t-product's, with no barrier in between, so the two use different buffers
  double* partA = V.part;                // products (v, then t)
  double* partB = V.part + 3 * kKGrid;   // the x/r update
  KState S = *V.st;
  double red[3];
  for (int q = 0; q < iters && !S.breakdown; ++q) {
    // beta = (rho_new / rho)(alpha / omega); rho <- rho_new; p = r (first) or r + beta (p - omega v)
    const bool first = it0 + q == 1;
    S.beta = (S.rho_new / S.rho) * (S.alpha / S.omega);
    S.rho = S.rho_new;
    if (!isfinite(S.beta) || S.rho == 0.0) {  // every block takes the same decision
      S.breakdown = 1;
      break;
    }
    const float fb = (float)S.beta, fw = (float)S.omega;
    for (int64_t i = i0; i < n; i += stride) V.p[i] = first ? V.r[i] : V.r[i] + fb * (V.p[i] - fw * V.v[i]);
    grid.sync();
    // v = K p; alpha = rho / (rhat, v); s = r - alpha v
    coop_apply<kApplyV>(rec, g, V.p, V, n, gcnt, partA);
    grid.sync();
    reduce_all(partA, nblk, 1, red);
    S.rhat_v = red[0];
    S.alpha = S.rho / S.rhat_v;
    if (!isfinite(S.alpha)) {
      S.breakdown = 1;
      break;
    }
    const float fa = (float)S.alpha;
    for (int64_t i = i0; i < n; i += stride) V.s[i] = V.r[i] - fa * V.v[i];
    grid.sync();
    // t = K s; omega = (t, s) / (t, t)
    coop_apply<kApplyT>(rec, g, V.s, V, n, gcnt, partA);
    grid.sync();
    reduce_all(partA, nblk, 2, red);
    S.ts = red[0];
    S.tt = red[1];
    S.omega = S.tt > 0.0 ? S.ts / S.tt : 0.0;
    if (S.omega == 0.0) {
      S.breakdown = 1;
      break;
    }
    // x += alpha p + omega s; r = s - omega t; (rhat, r), (r, r)
    const float w = (float)S.omega;
    double rr = 0.0, rh = 0.0;
    for (int64_t i = i0; i < n; i += stride) {
      const float sv = V.s[i];
      V.x[i] = V.x[i] + fa * V.p[i] + w * sv;
      const float r = sv - w * V.t[i];
      V.r[i] = r;
      rh += (double)V.rhat[i] * r;
      rr += (double)r * r;
    }
    block_partials(rh, rr, 0.0, partB, 2);
    grid.sync();
    reduce_all(partB, nblk, 2, red);
    S.rho_new = red[0];
    S.rr = red[1];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *V.st = S;
}

// max |x - u_exact| / max |u_exact| partials
__global__ void k_err(int64_t n, const float* __restrict__ x, const float* __restrict__ ex, float* __restrict__ part) {
  __shared__ float s[2][32];
  float e = 0.0f, m = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    e = fmaxf(e, fabsf(x[i] - ex[i]));
    m = fmaxf(m, fabsf(ex[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    e = fmaxf(e, __shfl_down_sync(0xffffffffu, e, o));
    m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    s[0][wid] = e;
    s[1][wid] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0, b = 0;
    for (int q = 0; q < nw; ++q) {
      a = fmaxf(a, s[0][q]);
      b = fmaxf(b, s[1][q]);
    }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t kcarve(KVecs* V, char* base, int64_t n) {
  size_t off = 0;
  auto take = [&](size_t b) {
    char* p = base ? base + off : nullptr;
    off = al(off + b);
    return p;
  };
  KVecs v;
  v.r = (float*)take(4 * n);
  v.rhat = (float*)take(4 * n);
  v.p = (float*)take(4 * n);
  v.v = (float*)take(4 * n);
  v.s = (float*)take(4 * n);
  v.t = (float*)take(4 * n);
  v.part = (double*)take(sizeof(double) * 3 * (kKGrid + kGenGrid));
  v.glist = (int32_t*)take(sizeof(int32_t) * n);
  v.gcount = (int32_t*)take(sizeof(int32_t));
  v.st = (KState*)take(sizeof(KState));
  v.err_part = (float*)take(sizeof(float) * 2 * kKGrid);
  v.coef = (float4*)take(sizeof(float4) * 2 * n);
  v.gen = (uint8_t*)take(n);
  v.x = nullptr;
  if (V) *V = v;
  return off;
}

// blocks of the cooperative BiCGSTAB launch on the current device (all co-resident), cached
static int coop_grid_size(int* out) {
  static int cached[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "bicgstab: cudaGetDevice");
  if (dev >= 0 && dev < 64 && cached[dev]) {
    *out = cached[dev];
    return DIPS_OK;
  }
  int coop = 0, sms = 0, per_sm = 0;
  e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bicg_coop, kKThreads, 0);
  if (e != cudaSuccess) return cuda_status(e, "bicgstab: cooperative launch attributes");
  DIPS_REQUIRE(coop && per_sm > 0, DIPS_E_CUDA, "bicgstab: the device does not support the cooperative launch");
  int grid = sms * per_sm;
  if (grid > kKGrid) grid = kKGrid;
  if (dev >= 0 && dev < 64) cached[dev] = grid;
  *out = grid;
  return DIPS_OK;
}

static int check_grid(const dips_records_t* rec, int nx, int ny, int nz) {
  DIPS_REQUIRE(rec && rec->job_off && rec->job_code && rec->job_A && rec->cnt && rec->cnt_m && rec->diag && rec->rod &&
                   rec->lhs0,
               DIPS_E_ARG, "krylov: null record pointer");
  DIPS_REQUIRE(nx > 0 && ny > 0 && nz > 0 && (int64_t)nx * ny * nz == rec->n_pts, DIPS_E_ARG,
               "krylov: records must be the %d x %d x %d grid nodes in C order (n_pts = %lld)", nx, ny, nz,
               (long long)rec->n_pts);
  return DIPS_OK;
}

}  // namespace dips

using namespace dips;

extern "C" size_t dips_bicgstab_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  return kcarve(nullptr, nullptr, n) + 256;
}

extern "C" int dips_fv_residual(const dips_records_t* rec, int32_t nx, int32_t ny, int32_t nz, const float* u,
                                int32_t linear_only, float* out, cudaStream_t stream) {
  int st = check_grid(rec, nx, ny, nz);
  if (st) return st;
  DIPS_REQUIRE(u && out, DIPS_E_ARG, "dips_fv_residual: null vector");
  Grid3 g{nx, ny, nz};
  k_fv_residual<<<kKGrid, kKThreads, 0, stream>>>(*rec, g, u, linear_only, out);
  DIPS_CHECK_LAUNCH("dips_fv_residual");
  return DIPS_OK;
}

extern "C" int dips_bicgstab(const dips_records_t* rec, int32_t nx, int32_t ny, int32_t nz, float* x,
                             const float* u_exact, int32_t max_iter, double rtol, int32_t check_every,
                             float target_rel_linf, void* workspace, size_t ws_bytes, dips_krylov_stats_t* stats,
                             cudaStream_t stream) {
  int st = check_grid(rec, nx, ny, nz);
  if (st) return st;
  DIPS_REQUIRE(x && workspace && max_iter >= 0 && check_every >= 1, DIPS_E_ARG, "dips_bicgstab: bad argument");
  const int64_t n = rec->n_pts;
  DIPS_REQUIRE(ws_bytes >= dips_bicgstab_workspace_bytes(n), DIPS_E_WORKSPACE, "dips_bicgstab: workspace too small");
  KVecs V;
  kcarve(&V, (char*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255), n);
  V.x = x;
  Grid3 g{nx, ny, nz};
  const int G = kKGrid, T = kKThreads, GP = kKGrid + kGenGrid;
  cudaError_t ez = cudaMemsetAsync(V.gcount, 0, sizeof(int32_t), stream);
  if (ez != cudaSuccess) return cuda_status(ez, "bicgstab general-row count");
  k_general_rows<<<G, T, 0, stream>>>(*rec, V.glist, V.gcount);
  if (rec->bulk_rec) {
    k_krylov_pack<<<G, T, 0, stream>>>(*rec, V.coef, V.gen);
  } else {  // no packed records: every row takes the warp path
    cudaError_t eg = cudaMemsetAsync(V.gen, 1, n, stream);
    if (eg != cudaSuccess) return cuda_status(eg, "bicgstab row kinds");
  }
  k_apply_bulk<kInit><<<G, T, 0, stream>>>(*rec, g, V.x, V);
  k_apply_general<kInit><<<kGenGrid, T, 0, stream>>>(*rec, g, V.x, V);
  k_bicg_init_scalars<<<1, 1024, 0, stream>>>(V, GP);
  DIPS_CHECK_LAUNCH("bicgstab init");
  KState hs;
  float herr[2 * kKGrid];
  dips_krylov_stats_t S;
  S.iterations = 0;
  S.rel_residual = 1.0;
  S.rel_linf = -1.0f;
  S.target_iteration = -1;
  S.breakdown = 0;
  auto read_state = [&]() -> int {
    cudaError_t e = cudaMemcpyAsync(&hs, V.st, sizeof(KState), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? 0 : cuda_status(e, "bicgstab state read");
  };
  auto read_err = [&](float* rel) -> int {
    k_err<<<G, T, 0, stream>>>(n, x, u_exact, V.err_part);
    cudaError_t e = cudaMemcpyAsync(herr, V.err_part, sizeof(float) * 2 * G, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_status(e, "bicgstab error read");
    float a = 0, b = 0;
    for (int q = 0; q < G; ++q) {
      a = fmaxf(a, herr[2 * q]);
      b = fmaxf(b, herr[2 * q + 1]);
    }
    *rel = b > 0 ? a / b : a;
    return 0;
  };
  if ((st = read_state())) return st;
  const double bnorm = sqrt(hs.bb > 0 ? hs.bb : 1.0);
  S.rel_residual = sqrt(hs.rr) / bnorm;
  if (u_exact) {
    if ((st = read_err(&S.rel_linf))) return st;
    if (S.rel_linf <= target_rel_linf) S.target_iteration = 0;
  }
  // with an exact solution and a positive target the solve stops once the target is met
  const bool stop_at_target = u_exact != nullptr && target_rel_linf > 0.0f;
  // the iterations between two host checks run in one cooperative launch: as many blocks as
  // fit on the device at once (so that the grid-wide barriers are legal), at most kKGrid
  int coop_grid = 0;
  if ((st = coop_grid_size(&coop_grid))) return st;
  for (int it = 1; it <= max_iter && S.rel_residual > rtol && !(stop_at_target && S.target_iteration >= 0);) {
    int chunk = check_every - (it - 1) % check_every;
    if (chunk > max_iter - it + 1) chunk = max_iter - it + 1;
    int64_t n_arg = n;
    int it0 = it;
    void* args[] = {(void*)rec, (void*)&g, (void*)&V, (void*)&n_arg, (void*)&it0, (void*)&chunk};
    cudaError_t el = cudaLaunchCooperativeKernel((const void*)k_bicg_coop, dim3(coop_grid), dim3(kKThreads), args, 0,
                                                 stream);
    if (el != cudaSuccess) return cuda_status(el, "bicgstab cooperative launch");
    it += chunk;
    S.iterations = it - 1;
    {
      if ((st = read_state())) return st;
      S.rel_residual = sqrt(hs.rr) / bnorm;
      if (hs.breakdown) {
        S.breakdown = 1;
        break;
      }
      if (u_exact && S.target_iteration < 0) {
        if ((st = read_err(&S.rel_linf))) return st;
        if (S.rel_linf <= target_rel_linf) S.target_iteration = it - 1;
      }
    }
  }
  if (u_exact) {
    if ((st = read_err(&S.rel_linf))) return st;
  }
  if (stats) *stats = S;
  return DIPS_OK;
}
