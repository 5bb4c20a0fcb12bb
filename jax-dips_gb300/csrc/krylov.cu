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
constexpr int kGenGrid = 152 * 8;  // blocks of the initial residual's general rows (8 warps each, a warp per row)

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

// (K x)_gp of any row by the whole warp, the lanes splitting its jobs (up to 7 x 27: lane l takes
// jobs l, l + 32, ...); every lane gets the value.  Two rounds of 32 jobs issue their loads
// together (each lane still adds its jobs in order).
__device__ __forceinline__ float general_apply_warp(const dips_records_t& rec, const Grid3& g, int64_t gp,
                                                    const float* __restrict__ x) {
  const int lane = threadIdx.x & 31;
  const int64_t o0 = rec.job_off[gp], o1 = rec.job_off[gp + 1];
  const int cm = rec.cnt_m[gp], n = rec.cnt[gp];
  const int k = (int)(gp % g.nz);
  const int j = (int)((gp / g.nz) % g.ny);
  const int i = (int)(gp / ((int64_t)g.ny * g.nz));
  float part = 0.0f;
  for (int q0 = lane; q0 < n; q0 += 64) {
    const int q1 = q0 + 32;
    const int64_t oa = q0 < cm ? o0 + q0 : o1 - n + q0;  // u- jobs at the front, u+ jobs at the back
    const float aa = __ldg(rec.job_A + oa);
    const float xa = __ldg(x + job_node(i, j, k, __ldg(rec.job_code + oa), g));
    float ab = 0.0f, xb = 0.0f;
    if (q1 < n) {
      const int64_t ob = q1 < cm ? o0 + q1 : o1 - n + q1;
      ab = __ldg(rec.job_A + ob);
      xb = __ldg(x + job_node(i, j, k, __ldg(rec.job_code + ob), g));
    }
    part = fmaf(aa, xa, part);
    if (q1 < n) part = fmaf(ab, xb, part);
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) part += __shfl_xor_sync(0xffffffffu, part, s);
  const float v = part / rec.diag[gp];
  return isfinite(v) ? v : 0.0f;
}

// A general row's header, packed once per solve (32 bytes, one sector) so that the product reads
// it before the row's jobs: job q of the row is at o0 + q (q < cm, u- jobs) or op + q (u+ jobs).
struct alignas(16) GenRowRec {
  int64_t o0;        // job_off[gp]
  int64_t op;        // job_off[gp + 1] - n
  int32_t gp;        // the row
  int32_t cmn;       // its u- jobs | its jobs << 16
  float diag;        // its diagonal coefficient
  int32_t interior;  // 1: the row lies two or more nodes inside the grid on every axis, so every
                     // job's node (stencil shift + cube shift, at most 2 per axis) needs no clamp
};

struct GenRow {
  int64_t o0, op;
  int gp, cm, n;
  float diag;
  bool interior;
};

__device__ __forceinline__ GenRow load_row(const GenRowRec* rows, int64_t k) {
  const int4* p = reinterpret_cast<const int4*>(rows + k);
  const int4 a = __ldg(p), b = __ldg(p + 1);
  GenRow r;
  r.o0 = (int64_t)(((uint64_t)(uint32_t)a.y << 32) | (uint32_t)a.x);
  r.op = (int64_t)(((uint64_t)(uint32_t)a.w << 32) | (uint32_t)a.z);
  r.gp = b.x;
  r.cm = b.y & 0xffff;
  r.n = (int)((uint32_t)b.y >> 16);
  r.diag = __int_as_float(b.z);
  r.interior = b.w != 0;
  return r;
}

// Grid-node offset of each job code (stencil shift + cube shift) for rows that need no clamp,
// filled by every block of the cooperative launch into shared memory.
constexpr int kCodes = kStencil * kCube;
__device__ __forceinline__ void fill_code_offsets(int* off, const Grid3& g) {
  for (int c = threadIdx.x; c < kCodes; c += blockDim.x) {
    const int st = c / kCube, v = c % kCube;
    int di = v % 3 - 1, dj = (v / 3) % 3 - 1, dk = v / 9 - 1;
    if (st > 0) {
      const int ax = (st - 1) >> 1, d = ((st - 1) & 1) ? 1 : -1;
      if (ax == 0) di += d;
      if (ax == 1) dj += d;
      if (ax == 2) dk += d;
    }
    off[c] = (di * g.ny + dj) * g.nz + dk;
  }
}

// (K x) of a row of at most kLightJobs jobs by one thread, its jobs in order (u- jobs at the
// front, u+ at the back).  The loads have no branch around them (a slot past the row's last job
// reloads that job and is left out of the sum), so all of them issue before the first one returns.
constexpr int kLightJobs = 8;
__device__ __forceinline__ float general_apply_thread(const dips_records_t& rec, const Grid3& g, const GenRow& r,
                                                      const float* __restrict__ x) {
  if (r.n <= 0) return 0.0f;
  const int k = r.gp % g.nz;
  const int j = (r.gp / g.nz) % g.ny;
  const int i = r.gp / (g.ny * g.nz);
  float a[kLightJobs], xv[kLightJobs];
  uint16_t c[kLightJobs];
#pragma unroll
  for (int q = 0; q < kLightJobs; ++q) {
    const int qq = q < r.n ? q : r.n - 1;
    const int64_t o = (qq < r.cm ? r.o0 : r.op) + qq;
    a[q] = __ldg(rec.job_A + o);
    c[q] = __ldg(rec.job_code + o);
  }
#pragma unroll
  for (int q = 0; q < kLightJobs; ++q) xv[q] = __ldg(x + job_node(i, j, k, c[q], g));
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < kLightJobs; ++q)
    if (q < r.n) acc = fmaf(a[q], xv[q], acc);
  const float v = acc / r.diag;
  return isfinite(v) ? v : 0.0f;
}

// (K x) of a heavy row (more than kLightJobs jobs) by a group of kGroup lanes: sub-lane l adds jobs
// l, l + kGroup, ... in order, kGroupBatch rounds of kGroup jobs at a time whose loads issue
// together (no branch around them: a slot past the row's last job reloads that job and is left
// out of the sum); then the group sums its lanes in a fixed butterfly.  Sub-lane 0's value is
// the row's (the other lanes may round differently).
constexpr int kGroup = 8;
constexpr int kGroupBatch = 4;
__device__ __forceinline__ float general_apply_group(const dips_records_t& rec, const Grid3& g, const GenRow& r,
                                                     const int* __restrict__ code_off, const float* __restrict__ x) {
  const int sl = threadIdx.x & (kGroup - 1);
  float part = 0.0f;
  if (r.interior) {  // the node of a job is the row plus its code's offset
    for (int q0 = sl; q0 < r.n; q0 += kGroupBatch * kGroup) {
      float a[kGroupBatch], xv[kGroupBatch];
      uint16_t c[kGroupBatch];
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u) {
        const int q = q0 + u * kGroup;
        const int qq = q < r.n ? q : r.n - 1;
        const int64_t o = (qq < r.cm ? r.o0 : r.op) + qq;
        a[u] = __ldg(rec.job_A + o);
        c[u] = __ldg(rec.job_code + o);
      }
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u) xv[u] = __ldg(x + (r.gp + code_off[c[u] & 0x7fff]));
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u)
        if (q0 + u * kGroup < r.n) part = fmaf(a[u], xv[u], part);
    }
  } else {
    const int k = r.gp % g.nz;
    const int j = (r.gp / g.nz) % g.ny;
    const int i = r.gp / (g.ny * g.nz);
    for (int q0 = sl; q0 < r.n; q0 += kGroupBatch * kGroup) {
      float a[kGroupBatch], xv[kGroupBatch];
      uint16_t c[kGroupBatch];
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u) {
        const int q = q0 + u * kGroup;
        const int qq = q < r.n ? q : r.n - 1;
        const int64_t o = (qq < r.cm ? r.o0 : r.op) + qq;
        a[u] = __ldg(rec.job_A + o);
        c[u] = __ldg(rec.job_code + o);
      }
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u) xv[u] = __ldg(x + job_node(i, j, k, c[u], g));
#pragma unroll
      for (int u = 0; u < kGroupBatch; ++u)
        if (q0 + u * kGroup < r.n) part = fmaf(a[u], xv[u], part);
    }
  }
#pragma unroll
  for (int s = kGroup / 2; s > 0; s >>= 1) part += __shfl_xor_sync(0xffffffffu, part, s, kGroup);
  const float v = part / r.diag;
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
  GenRowRec* grows; // [n] the general rows' headers, binned by their number of jobs (once per solve)
  int32_t* gcount;  // [2 kRowBins] the bins' sizes, then their scatter cursors
  KState* st;
  unsigned* arrive;  // [3] blocks that have written their partials, per reduction of an iteration
  double* sums;      // [3][3] the grid's sums of those reductions
  float* err_part;  // [kKGrid] max |x - u_exact|
  float4* coef;     // [n][2] bulk rows: A_0..A_6 (stencil order) and diag, packed once per solve
  uint8_t* gen;     // [n] 1 for a general row (listed in grows), 0 for a bulk row
};


// The general rows (those without a packed bulk record) are listed once per solve, in bins:
// bin 0 holds the rows of at most kLightJobs jobs (a thread each in the cooperative product),
// bin b >= 1 the rows that take b rounds of 32 jobs (a group of kGroup lanes each).  The list
// holds bin 0, then the bins of the most rounds first, so that the groups striding over the heavy
// rows get similar mixes.  counts[0, kRowBins) are the bins' sizes, counts[kRowBins, 2 kRowBins)
// scatter cursors.
// The order within a bin depends on the warps' arrival; each row's value does not.
constexpr int kRowBins = 16;  // rows of up to 15 x 32 jobs

__device__ __forceinline__ int row_bin(int cnt) {
  if (cnt <= kLightJobs) return 0;
  const int b = (cnt + 31) >> 5;
  return b < kRowBins ? b : kRowBins - 1;
}

__global__ void k_general_count(dips_records_t rec, int32_t* __restrict__ counts) {
  __shared__ int h[kRowBins];
  for (int t = threadIdx.x; t < kRowBins; t += blockDim.x) h[t] = 0;
  __syncthreads();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < rec.n_pts; p += (int64_t)gridDim.x * blockDim.x)
    if (!bulk_row(rec, p)) atomicAdd(&h[row_bin(rec.cnt[p])], 1);
  __syncthreads();
  for (int t = threadIdx.x; t < kRowBins; t += blockDim.x)
    if (h[t]) atomicAdd(counts + t, h[t]);
}

__global__ void k_general_rows(dips_records_t rec, Grid3 g, GenRowRec* __restrict__ list, int32_t* __restrict__ counts) {
  __shared__ int start[kRowBins];
  if (threadIdx.x == 0) {
    int s = counts[0];
    start[0] = 0;
    for (int b = kRowBins - 1; b >= 1; --b) {
      start[b] = s;
      s += counts[b];
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  DIPS_ROWS(p, valid, rec.n_pts) {
    const bool gen = valid && !bulk_row(rec, p);
    const int b = gen ? row_bin(rec.cnt[p]) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (gen && lane == leader) base = atomicAdd(counts + kRowBins + b, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (gen) {
      GenRowRec r;
      const int n = rec.cnt[p];
      r.o0 = rec.job_off[p];
      r.op = rec.job_off[p + 1] - n;
      r.gp = (int32_t)p;
      r.cmn = rec.cnt_m[p] | (n << 16);
      r.diag = rec.diag[p];
      const int k = (int)(p % g.nz), j = (int)((p / g.nz) % g.ny), i = (int)(p / ((int64_t)g.ny * g.nz));
      r.interior = i >= 2 && i < g.nx - 2 && j >= 2 && j < g.ny - 2 && k >= 2 && k < g.nz - 2;
      list[start[b] + base + __popc(peers & ((1u << lane) - 1))] = r;
    }
  }
}

// number of light (bin 0) and heavy general rows
__device__ __forceinline__ void general_counts(const int32_t* counts, int64_t& light, int64_t& heavy) {
  light = counts[0];
  heavy = 0;
  for (int b = 1; b < kRowBins; ++b) heavy += counts[b];
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
  int64_t light, heavy;
  general_counts(V.gcount, light, heavy);
  const int64_t cnt = light + heavy;
  double a0 = 0.0, a1 = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * nw + (threadIdx.x >> 5); k < cnt; k += (int64_t)gridDim.x * nw) {
    const int64_t gp = V.grows[k].gp;
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

// the follow-up of a product row in the cooperative iteration, with its other operand loaded by
// the caller ((rhat)_i for v = K p, s_i for t = K s)
template <int MODE>
__device__ __forceinline__ void row_finish(const KVecs& V, int64_t i, float kx, float other, double& a0, double& a1) {
  if (MODE == kApplyV) {
    V.v[i] = kx;
    a0 += (double)other * kx;
  } else {
    V.t[i] = kx;
    a0 += (double)kx * other;
    a1 += (double)kx * kx;
  }
}

// sum of the first `nv` columns of the grid's partials, in one fixed order; every thread of the
// block gets the sums
__device__ __forceinline__ void reduce_all(const double* part, int nblk, int nv, double out[3]) {
  __shared__ double s[3][32];
  __shared__ double res[3];
  double a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {  // written by other blocks: read from L2
    a += __ldcg(part + 3 * i);
    if (nv > 1) b += __ldcg(part + 3 * i + 1);
    if (nv > 2) c += __ldcg(part + 3 * i + 2);
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

// After the block's partials are written (block_partials): the last block to arrive sums the
// grid's partials in block order (reduce_all) and publishes the sums, before the grid-wide
// barrier, so that after it every block reads nv numbers instead of summing nblk partials itself.
// The counter is reset by that last block; its next use comes after another barrier.
__device__ __forceinline__ void publish_sums(const double* part, int nblk, int nv, unsigned* arrive, double* sums) {
  __shared__ int s_last;
  if (threadIdx.x == 0) {  // thread 0 wrote the block's partials
    __threadfence();
    s_last = atomicAdd(arrive, 1u) == (unsigned)nblk - 1;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    double red[3];
    reduce_all(part, nblk, nv, red);
    if (threadIdx.x == 0) {
      for (int v = 0; v < nv; ++v) sums[v] = red[v];
      *arrive = 0;
    }
  }
}

// the published sums, after the grid-wide barrier
__device__ __forceinline__ void read_sums(const double* sums, int nv, double red[3]) {
  for (int v = 0; v < nv; ++v) red[v] = __ldcg(sums + v);
}

// one product over all rows, with the row's follow-up of MODE; per-block partials into part.
// Bulk rows and light general rows take a thread each; heavy general rows (more than kLightJobs
// jobs, up to 7 x 27) a group of kGroup lanes each, the lanes reading the row's consecutive jobs
// together.  A thread walking a heavy row alone (measured at 128^3: 40,000 rows of 9-112 jobs)
// left the threads that drew the longest rows running for about 70 us after the rest of the grid
// had reached the next barrier; binning the rows by length and striding the groups over the bins
// gives every group a similar share.
template <int MODE>
__device__ __forceinline__ void coop_apply(const dips_records_t& rec, const Grid3& g, const float* __restrict__ x,
                                           const KVecs& V, int64_t n, int64_t glight, int64_t gheavy,
                                           const int* code_off, double* part) {
  double a0 = 0.0, a1 = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t i = i0; i < n; i += stride)
    if (!V.gen[i]) row_done<MODE>(rec, V, i, coef_apply(V.coef, g, i, x), a0, a1);
  for (int64_t k = i0; k < glight; k += stride) {
    const GenRow r = load_row(V.grows, k);
    row_done<MODE>(rec, V, r.gp, general_apply_thread(rec, g, r, x), a0, a1);
  }
  // group w of kGroup lanes takes heavy rows w, w + W, ... (W groups in the grid); the loop bound
  // is uniform over the group, and whole warps leave it together or keep their lanes in step
  const int64_t gstride = stride / kGroup;
  const int64_t w0 = i0 / kGroup;
  const int64_t rounds = (gheavy + gstride - 1) / gstride;  // the same for every lane of the grid
  // A group past the last row computes row 0 again and drops it.  The next row's header and the
  // row's own follow-up operand ((rhat)_i or s_i) load while its jobs are read.
  GenRow r = {};
  if (rounds > 0) r = load_row(V.grows, glight + (w0 < gheavy ? w0 : 0));  // (no heavy rows: nothing listed)
  for (int64_t t = 0; t < rounds; ++t) {
    const int64_t w = w0 + t * gstride, wn = w + gstride;
    const GenRow rn = load_row(V.grows, glight + (wn < gheavy ? wn : 0));
    const float other = MODE == kApplyV ? V.rhat[r.gp] : V.s[r.gp];
    const float kx = general_apply_group(rec, g, r, code_off, x);
    if (w < gheavy && (threadIdx.x & (kGroup - 1)) == 0) row_finish<MODE>(V, r.gp, kx, other, a0, a1);
    r = rn;
  }
  block_partials(a0, a1, 0.0, part, 2);
}

// `iters` BiCGSTAB iterations (it0 = the global number of the first); the recurrence state is
// read from and written back to V.st (block 0)
__global__ void __launch_bounds__(kKThreads, 3) k_bicg_coop(dips_records_t rec, Grid3 g, KVecs V, int64_t n, int it0,
                                                         int iters) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  const int nblk = gridDim.x;
  int64_t glight, gheavy;
  general_counts(V.gcount, glight, gheavy);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // two partial buffers: the x/r update's partials and the t-product's
  double* partA = V.part;                // products (v, then t)
  double* partB = V.part + 3 * kKGrid;   // the x/r update
  KState S = *V.st;
  double red[3];
  __shared__ int s_off[kCodes];
  fill_code_offsets(s_off, g);
  __syncthreads();
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
    // the vector updates take a thread's rows four at a time, their loads issued first, so that
    // enough loads are in flight to stream from HBM
    {
      int64_t i = i0;
      for (; i + 3 * stride < n; i += 4 * stride) {
        float rv[4], pv[4], vv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          rv[u] = V.r[i + u * stride];
          pv[u] = first ? 0.0f : V.p[i + u * stride];
          vv[u] = first ? 0.0f : V.v[i + u * stride];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) V.p[i + u * stride] = first ? rv[u] : rv[u] + fb * (pv[u] - fw * vv[u]);
      }
      for (; i < n; i += stride) V.p[i] = first ? V.r[i] : V.r[i] + fb * (V.p[i] - fw * V.v[i]);
    }
    grid.sync();
    // v = K p; alpha = rho / (rhat, v); s = r - alpha v
    coop_apply<kApplyV>(rec, g, V.p, V, n, glight, gheavy, s_off, partA);
    publish_sums(partA, nblk, 1, V.arrive, V.sums);
    grid.sync();
    read_sums(V.sums, 1, red);
    S.rhat_v = red[0];
    S.alpha = S.rho / S.rhat_v;
    if (!isfinite(S.alpha)) {
      S.breakdown = 1;
      break;
    }
    const float fa = (float)S.alpha;
    {
      int64_t i = i0;
      for (; i + 3 * stride < n; i += 4 * stride) {
        float rv[4], vv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          rv[u] = V.r[i + u * stride];
          vv[u] = V.v[i + u * stride];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) V.s[i + u * stride] = rv[u] - fa * vv[u];
      }
      for (; i < n; i += stride) V.s[i] = V.r[i] - fa * V.v[i];
    }
    grid.sync();
    // t = K s; omega = (t, s) / (t, t)
    coop_apply<kApplyT>(rec, g, V.s, V, n, glight, gheavy, s_off, partA);
    publish_sums(partA, nblk, 2, V.arrive + 1, V.sums + 3);
    grid.sync();
    read_sums(V.sums + 3, 2, red);
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
    {
      int64_t i = i0;
      for (; i + stride < n; i += 2 * stride) {  // two rows at a time, in the same order
        float sv[2], xv[2], pv[2], tv[2], hv[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          sv[u] = V.s[i + u * stride];
          xv[u] = V.x[i + u * stride];
          pv[u] = V.p[i + u * stride];
          tv[u] = V.t[i + u * stride];
          hv[u] = V.rhat[i + u * stride];
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          V.x[i + u * stride] = xv[u] + fa * pv[u] + w * sv[u];
          const float r = sv[u] - w * tv[u];
          V.r[i + u * stride] = r;
          rh += (double)hv[u] * r;
          rr += (double)r * r;
        }
      }
      for (; i < n; i += stride) {
        const float sv = V.s[i];
        V.x[i] = V.x[i] + fa * V.p[i] + w * sv;
        const float r = sv - w * V.t[i];
        V.r[i] = r;
        rh += (double)V.rhat[i] * r;
        rr += (double)r * r;
      }
    }
    block_partials(rh, rr, 0.0, partB, 2);
    publish_sums(partB, nblk, 2, V.arrive + 2, V.sums + 6);
    grid.sync();
    read_sums(V.sums + 6, 2, red);
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
  v.grows = (GenRowRec*)take(sizeof(GenRowRec) * n);
  v.gcount = (int32_t*)take(sizeof(int32_t) * 2 * kRowBins);
  v.st = (KState*)take(sizeof(KState));
  v.arrive = (unsigned*)take(sizeof(unsigned) * 4);
  v.sums = (double*)take(sizeof(double) * 9);
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
  DIPS_REQUIRE(!rec->nl_pt, DIPS_E_ARG, "krylov: the operator with nonlinear terms is not linear (no BiCGSTAB)");
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
  DIPS_REQUIRE(n < ((int64_t)1 << 31), DIPS_E_ARG, "dips_bicgstab: at most 2^31 - 1 rows (32-bit row indices)");
  DIPS_REQUIRE(ws_bytes >= dips_bicgstab_workspace_bytes(n), DIPS_E_WORKSPACE, "dips_bicgstab: workspace too small");
  KVecs V;
  kcarve(&V, (char*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255), n);
  V.x = x;
  Grid3 g{nx, ny, nz};
  const int G = kKGrid, T = kKThreads, GP = kKGrid + kGenGrid;
  cudaError_t ez = cudaMemsetAsync(V.gcount, 0, sizeof(int32_t) * 2 * kRowBins, stream);
  if (ez == cudaSuccess) ez = cudaMemsetAsync(V.arrive, 0, sizeof(unsigned) * 4, stream);
  if (ez != cudaSuccess) return cuda_status(ez, "bicgstab general-row count");
  k_general_count<<<G, T, 0, stream>>>(*rec, V.gcount);
  k_general_rows<<<G, T, 0, stream>>>(*rec, g, V.grows, V.gcount);
  if (rec->bulk_rec) {
    k_krylov_pack<<<G, T, 0, stream>>>(*rec, V.coef, V.gen);
  } else {  // no packed records: every row is a general row
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
