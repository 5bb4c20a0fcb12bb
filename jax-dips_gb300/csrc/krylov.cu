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
// FP64 inner products; the scalar recurrences stay on the device.

#include <math.h>

#include "dips_common.cuh"

namespace dips {

constexpr int kKThreads = 256;
constexpr int kKGrid = 152 * 8;
constexpr int kGenGrid = 152 * 8;  // blocks of the general-row kernels (8 warps each, a warp per row)

struct Grid3 {
  int nx, ny, nz;
};

// grid node of job code c of row p (stencil offset + cube offset, clamped to the grid)
__device__ __forceinline__ int64_t job_node(int64_t p, uint16_t c, const Grid3& g) {
  int k = (int)(p % g.nz);
  int j = (int)((p / g.nz) % g.ny);
  int i = (int)(p / ((int64_t)g.ny * g.nz));
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
  float part = 0.0f;
  for (int q = lane; q < n; q += 32) {
    const int64_t o = q < cm ? o0 + q : o1 - n + q;  // u- jobs at the front, u+ jobs at the back
    part = fmaf(rec.job_A[o], __ldg(x + job_node(gp, rec.job_code[o], g)), part);
  }
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) part += __shfl_xor_sync(0xffffffffu, part, s);
  const float v = part / rec.diag[gp];
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
  double* part;     // [(kKGrid + kGenGrid) * 3]: bulk-row blocks, then general-row blocks
  int32_t* glist;   // [n] the general rows (found once per solve)
  int32_t* gcount;  // their number
  KState* st;
  float* err_part;  // [kKGrid] max |x - u_exact|
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

// reduce the first `nv` partial columns into the given state slots
__device__ void reduce_partials(const double* part, int nblk, int nv, double* out0, double* out1, double* out2) {
  __shared__ double s[3][32];
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
    *out0 = x0;
    if (nv > 1) *out1 = x1;
    if (nv > 2) *out2 = x2;
  }
}

// beta = (rho_new/rho)(alpha/omega); rho = rho_new;  p = r + beta (p - omega v)
__global__ void k_bicg_p(int64_t n, KVecs V) {
  const KState S = *V.st;
  const double beta = (S.rho_new / S.rho) * (S.alpha / S.omega);
  const float fb = (float)beta, fw = (float)S.omega;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    V.p[i] = V.r[i] + fb * (V.p[i] - fw * V.v[i]);
}

__global__ void k_bicg_rho_shift(KVecs V) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    KState& S = *V.st;
    S.beta = (S.rho_new / S.rho) * (S.alpha / S.omega);
    S.rho = S.rho_new;
    if (!isfinite(S.beta) || S.rho == 0.0) S.breakdown = 1;
  }
}


__global__ void k_bicg_alpha(KVecs V, int nblk) {
  reduce_partials(V.part, nblk, 1, &V.st->rhat_v, nullptr, nullptr);
  __syncthreads();
  if (threadIdx.x == 0) {
    KState& S = *V.st;
    S.alpha = S.rho / S.rhat_v;
    if (!isfinite(S.alpha)) S.breakdown = 1;
  }
}

// s = r - alpha v
__global__ void k_bicg_s(int64_t n, KVecs V) {
  const float a = (float)V.st->alpha;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    V.s[i] = V.r[i] - a * V.v[i];
}


__global__ void k_bicg_omega(KVecs V, int nblk) {
  reduce_partials(V.part, nblk, 2, &V.st->ts, &V.st->tt, nullptr);
  __syncthreads();
  if (threadIdx.x == 0) {
    KState& S = *V.st;
    S.omega = S.tt > 0.0 ? S.ts / S.tt : 0.0;
    if (S.omega == 0.0) S.breakdown = 1;
  }
}

// x += alpha p + omega s;  r = s - omega t;  partials (rhat, r), (r, r)
__global__ void k_bicg_xr(int64_t n, KVecs V) {
  const float a = (float)V.st->alpha, w = (float)V.st->omega;
  double rr = 0.0, rh = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float s = V.s[i];
    V.x[i] = V.x[i] + a * V.p[i] + w * s;
    const float r = s - w * V.t[i];
    V.r[i] = r;
    rh += (double)V.rhat[i] * r;
    rr += (double)r * r;
  }
  block_partials(rh, rr, 0.0, V.part, 2);
}

__global__ void k_bicg_rho(KVecs V, int nblk) { reduce_partials(V.part, nblk, 2, &V.st->rho_new, &V.st->rr, nullptr); }

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
  v.x = nullptr;
  if (V) *V = v;
  return off;
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
  for (int it = 1; it <= max_iter && S.rel_residual > rtol && !(stop_at_target && S.target_iteration >= 0); ++it) {
    if (it > 1) {
      k_bicg_p<<<G, T, 0, stream>>>(n, V);
      k_bicg_rho_shift<<<1, 32, 0, stream>>>(V);
    } else {
      // first iteration: p = r
      k_bicg_rho_shift<<<1, 32, 0, stream>>>(V);
      cudaError_t e = cudaMemcpyAsync(V.p, V.r, sizeof(float) * n, cudaMemcpyDeviceToDevice, stream);
      if (e != cudaSuccess) return cuda_status(e, "bicgstab p = r");
    }
    k_apply_bulk<kApplyV><<<G, T, 0, stream>>>(*rec, g, V.p, V);
    k_apply_general<kApplyV><<<kGenGrid, T, 0, stream>>>(*rec, g, V.p, V);
    k_bicg_alpha<<<1, 1024, 0, stream>>>(V, GP);
    k_bicg_s<<<G, T, 0, stream>>>(n, V);
    k_apply_bulk<kApplyT><<<G, T, 0, stream>>>(*rec, g, V.s, V);
    k_apply_general<kApplyT><<<kGenGrid, T, 0, stream>>>(*rec, g, V.s, V);
    k_bicg_omega<<<1, 1024, 0, stream>>>(V, GP);
    k_bicg_xr<<<G, T, 0, stream>>>(n, V);
    k_bicg_rho<<<1, 1024, 0, stream>>>(V, G);
    DIPS_CHECK_LAUNCH("bicgstab iteration");
    S.iterations = it;
    if (it % check_every == 0 || it == max_iter) {
      if ((st = read_state())) return st;
      S.rel_residual = sqrt(hs.rr) / bnorm;
      if (hs.breakdown) {
        S.breakdown = 1;
        break;
      }
      if (u_exact && S.target_iteration < 0) {
        if ((st = read_err(&S.rel_linf))) return st;
        if (S.rel_linf <= target_rel_linf) S.target_iteration = it;
      }
    }
  }
  if (u_exact) {
    if ((st = read_err(&S.rel_linf))) return st;
  }
  if (stats) *stats = S;
  return DIPS_OK;
}
