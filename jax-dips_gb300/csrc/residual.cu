// Arch-independent part of the fused NBM residual step and the C API (sm_103a).
//
// Work unit: a "job" is one evaluation of a u-/u+ network at a stencil or regression-cube
// point of a training point.  A point's residual is affine in its job values:
//     r = nan_to_num((lhs0 + sum_j A_j u(x_j)) / diag) - rod
// (the records come from geometry.cu).  One step:
//   expand   batch -> job list, u- jobs first (padded to a multiple of 32), then u+ jobs
//   forward  thread per job (residual_arch.cuh)
//   residual thread per batch point: r, loss partials (FP64), dL/dlhs
//   adjoint  thread per job (residual_arch.cuh): one partial gradient row per CTA
//   reduce   partial rows -> gradient;  adam: clip -> Adam -> schedule -> apply
//
// Reference: Trainer.loss / update (solvers/poisson/trainer.py:783-789, :892-912),
// chained_adam (solvers/optimizers.py:33-54).

#include <math.h>

#include <vector>

#include "residual_common.cuh"

namespace dips {

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t carve(Workspace* w, char* base, int64_t B, int64_t max_jobs, int P, int pre_n) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off = align256(off + bytes);
    return p;
  };
  Workspace W;
  W.B = B;
  W.nblk = (B + kScanBlock - 1) / kScanBlock;
  W.nres = (B + 255) / 256;
  W.jcap = max_jobs + 64;
  W.grid = kAdjGrid;
  W.fgrid = kFusedGrid;
  W.n_params = P;
  W.ctl = (Ctl*)take(sizeof(Ctl));
  W.cm = (int32_t*)take(sizeof(int32_t) * B);
  W.cp = (int32_t*)take(sizeof(int32_t) * B);
  W.om = (int64_t*)take(sizeof(int64_t) * B);
  W.op = (int64_t*)take(sizeof(int64_t) * B);
  W.bk = (int32_t*)take(sizeof(int32_t) * B);
  W.ob = (int64_t*)take(sizeof(int64_t) * B);
  W.bulk = (int32_t*)take(sizeof(int32_t) * 2 * B);
  W.gs = (float*)take(sizeof(float) * B);
  W.blk = (int64_t*)take(sizeof(int64_t) * 4 * (W.nblk + 1));
  W.lossp = (double*)take(sizeof(double) * W.nres);
  W.floss = (double*)take(sizeof(double) * 2 * kLossSlots);
  W.jslot = (int32_t*)take(sizeof(int32_t) * W.jcap);
  W.jcode = (uint16_t*)take(sizeof(uint16_t) * W.jcap);
  W.jA = (float*)take(sizeof(float) * W.jcap);
  W.ju = (float*)take(sizeof(float) * W.jcap);
  W.jx = (float4*)take(sizeof(float4) * W.jcap);
  W.jg = (float*)take(sizeof(float) * W.jcap);
  W.brec = (float*)take(sizeof(float) * kRecFloats * 2 * B);
  W.pre_n = pre_n;
  W.pre_P = pre_n ? (float*)take(sizeof(float) * B) : nullptr;
  W.pre_r0 = pre_n ? (float*)take(sizeof(float) * B) : nullptr;
  W.pre_partials = pre_n ? (float*)take(sizeof(float) * (size_t)kPreGrid * pre_n) : nullptr;
  W.partials = (float*)take(sizeof(float) * (size_t)(W.grid + W.fgrid) * P);
  W.grad = (float*)take(sizeof(float) * P);
  W.sqp = (double*)take(sizeof(double) * ((P + 31) / 32));
  if (w) *w = W;
  return off;
}

// ----------------------------------------------------------------------------------------
// expansion of a batch: bulk points into two slot lists, the others into jobs
// ----------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, s);
    if (lane >= s) v += t;
  }
  return v;
}

// exclusive block scan of four counters; block totals in tot
__device__ __forceinline__ void block_scan4(const int64_t v[4], int64_t ex[4], int64_t tot[4]) {
  __shared__ int64_t ws[4][32], ts[4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t inc[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    inc[k] = warp_incl_scan(v[k], lane);
    if (lane == 31) ws[k][wid] = inc[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int64_t a = lane < nw ? ws[k][lane] : 0;
      const int64_t sa = warp_incl_scan(a, lane);
      if (lane < nw) ws[k][lane] = sa - a;
      if (lane == nw - 1) ts[k] = sa;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    ex[k] = ws[k][wid] + inc[k] - v[k];
    tot[k] = ts[k];
  }
  __syncthreads();
}

// A point is "bulk" when it has exactly 7 jobs (its stencil points, no cube vertices) all of
// one network; the fused kernel handles it.  bx: this block's index within the instance.
__device__ __forceinline__ void count_body(const int32_t* __restrict__ ids, int64_t B, int64_t n_pts,
                                           const int32_t* __restrict__ cnt, const int32_t* __restrict__ cnt_m,
                                           int bulk_ok, const Workspace& w, int bx) {
  const int64_t b = bx * (int64_t)blockDim.x + threadIdx.x;
  int64_t v[4] = {0, 0, 0, 0};  // bulk u-, bulk u+, general u- jobs, general u+ jobs
  if (b < B) {
    const int64_t pid = batch_pid(ids, b);
    int kind = 3;                   // an out-of-range id gets no work and a NaN residual
    if (pid >= 0 && pid < n_pts) {
      const int c = cnt[pid], m = cnt_m[pid];
      if (bulk_ok && c == kStencil && (m == kStencil || m == 0)) {
        kind = m ? 1 : 2;
        v[0] = m ? 1 : 0;  // selects, not a run-time index (which would put v in local memory)
        v[1] = m ? 0 : 1;
      } else {
        kind = 0;
        v[2] = m;
        v[3] = c - m;
      }
    }
    w.bk[b] = kind;
    w.cm[b] = (int32_t)v[2];
    w.cp[b] = (int32_t)v[3];
  }
  int64_t ex[4], tot[4];
  block_scan4(v, ex, tot);
  if (b < B) {
    w.ob[b] = v[0] ? ex[0] : ex[1];
    w.om[b] = ex[2];
    w.op[b] = ex[3];
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; ++k) w.blk[4 * bx + k] = tot[k];
}

__global__ void k_count(const int32_t* __restrict__ ids, int64_t B, int64_t n_pts, const int32_t* __restrict__ cnt,
                        const int32_t* __restrict__ cnt_m, int bulk_ok, const __grid_constant__ Workspace w) {
  count_body(ids, B, n_pts, cnt, cnt_m, bulk_ok, w, blockIdx.x);
}

// instance blockIdx.y of the table
__global__ void k_count_multi(const Inst* __restrict__ T, int bulk_ok) {
  const Inst& I = T[blockIdx.y];
  if ((int64_t)blockIdx.x >= I.w.nblk) return;
  count_body(I.ids, I.B, I.rec.n_pts, I.rec.cnt, I.rec.cnt_m, bulk_ok && !I.rec.nl_pt, I.w, blockIdx.x);
}

__device__ __forceinline__ void scan_body(const Workspace& w) {
  int64_t carry[4] = {0, 0, 0, 0};
  for (int64_t base = 0; base < w.nblk; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int64_t v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = i < w.nblk ? w.blk[4 * i + k] : 0;
    int64_t ex[4], tot[4];
    block_scan4(v, ex, tot);
    if (i < w.nblk)
#pragma unroll
      for (int k = 0; k < 4; ++k) w.blk[4 * i + k] = ex[k] + carry[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) carry[k] += tot[k];
  }
  if (threadIdx.x == 0) {
    const int64_t jm = carry[2], jp = carry[3];
    const int64_t jm_pad = (jm + 31) / 32 * 32;
    const bool over = jm_pad + jp > w.jcap;
    // on overflow no job is expanded or evaluated and every residual becomes NaN
    w.ctl->overflow = over ? 1 : 0;
    w.ctl->engine_error = 0;
    w.ctl->floss_n[0] = w.ctl->floss_n[1] = 0;
    w.ctl->grad_rows[0] = w.ctl->grad_rows[1] = 0;
    w.ctl->reduce_done = 0;
    w.ctl->nbm = over ? 0 : carry[0];
    w.ctl->nbp = over ? 0 : carry[1];
    w.ctl->jm = over ? 0 : jm;
    w.ctl->jp = over ? 0 : jp;
    w.ctl->jm_pad = over ? 0 : jm_pad;
    w.ctl->total = over ? 0 : jm_pad + jp;
  }
}

__global__ void k_scan_blocks(const __grid_constant__ Workspace w) { scan_body(w); }

// one block per instance
__global__ void k_scan_blocks_multi(const Inst* __restrict__ T) { scan_body(T[blockIdx.x].w); }

// Record of bulk point pid (network net): point, lhs0, the coefficient of each of its 7
// stencil jobs in stencil order, diag, rod (layout kRec*; the slot and padding are zero).
__device__ __forceinline__ void gather_bulk_record(const dips_records_t& rec, int64_t pid, int net,
                                                   float (&v)[kRecFloats]) {
  const int64_t jb = net ? rec.job_off[pid + 1] - kStencil : rec.job_off[pid];
  float A[kStencil];
#pragma unroll
  for (int t = 0; t < kStencil; ++t) A[t] = 0.0f;
#pragma unroll
  for (int q = 0; q < kStencil; ++q) {
    const int sj = job_stencil(rec.job_code[jb + q]);
    const float a = rec.job_A[jb + q];
#pragma unroll
    for (int t = 0; t < kStencil; ++t)
      if (sj == t) A[t] = a;
  }
#pragma unroll
  for (int k = 0; k < kRecFloats; ++k) v[k] = 0.0f;
  v[kRecP] = rec.pts[3 * pid];
  v[kRecP + 1] = rec.pts[3 * pid + 1];
  v[kRecP + 2] = rec.pts[3 * pid + 2];
  v[kRecLhs0] = rec.lhs0[pid];
#pragma unroll
  for (int t = 0; t < kStencil; ++t) v[kRecA + t] = A[t];
  v[kRecDiag] = rec.diag[pid];
  v[kRecRod] = rec.rod[pid];
}

__global__ void k_pack_bulk(dips_records_t rec, float* __restrict__ out) {
  for (int64_t pid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pid < rec.n_pts;
       pid += (int64_t)gridDim.x * blockDim.x) {
    const int c = rec.cnt[pid], m = rec.cnt_m[pid];
    if (c != kStencil || (m != kStencil && m != 0)) continue;
    float v[kRecFloats];
    gather_bulk_record(rec, pid, m ? 0 : 1, v);
    float4* o = reinterpret_cast<float4*>(out + pid * kRecFloats);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  }
}

// a point has at most 7 x 27 jobs (each stencil point: its cube's centre and 26 neighbours)
constexpr int kMaxJobRounds = (kStencil * kCube + 31) / 32;  // a point's jobs over 32 lanes

__device__ __forceinline__ void emit_body(const int32_t* __restrict__ ids, int64_t B, const dips_records_t& rec,
                                          const Workspace& w, int bx) {
  const int64_t b = bx * (int64_t)blockDim.x + threadIdx.x;
  if (w.ctl->overflow) return;
  const int64_t jm = w.ctl->jm, jm_pad = w.ctl->jm_pad;
  if (b == 0) {  // padding jobs between the u- and u+ segments
    for (int64_t j = jm; j < jm_pad; ++j) {
      w.jslot[j] = -1;
      w.jcode[j] = job_code(0, kCubeCentre, false);
      w.jA[j] = 0.0f;
      w.jx[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      w.jg[j] = 0.0f;
    }
  }
  const int kind = b < B ? w.bk[b] : 3;
  if (kind == 1 || kind == 2) {
    const int net = kind - 1;
    const int64_t pos = net * B + w.ob[b] + w.blk[4 * bx + net];
    w.bulk[pos] = (int32_t)b;
    // the point's record, so that the tile engine reads one contiguous 64-byte block
    const int64_t pid = batch_pid(ids, b);
    float4* r4 = reinterpret_cast<float4*>(w.brec + pos * kRecFloats);
    if (rec.bulk_rec) {  // packed once per level: one 64-byte read
      const float4* s4 = reinterpret_cast<const float4*>(rec.bulk_rec + pid * kRecFloats);
      const float4 a = __ldg(s4), c = __ldg(s4 + 1), d = __ldg(s4 + 2), e = __ldg(s4 + 3);
      r4[0] = a;
      r4[1] = c;
      r4[2] = d;
      r4[3] = make_float4(e.x, __int_as_float((int32_t)b), 0.0f, 0.0f);
    } else {
      float v[kRecFloats];
      gather_bulk_record(rec, pid, net, v);
      r4[0] = make_float4(v[0], v[1], v[2], v[3]);
      r4[1] = make_float4(v[4], v[5], v[6], v[7]);
      r4[2] = make_float4(v[8], v[9], v[10], v[11]);
      r4[3] = make_float4(v[12], __int_as_float((int32_t)b), 0.0f, 0.0f);
    }
  }
  // general points: their u- jobs go to [om, om + cm), their u+ jobs to [op, op + cp); the
  // source jobs are the first cm and the last cp of [job_off[pid], job_off[pid + 1]) (the
  // capacity may exceed the count).  A point has up to 7 x 27 jobs, so each warp expands its
  // general points one at a time with the 32 lanes taking the jobs.
  const bool gen = kind == 0;
  int64_t om = 0, op = 0, src = 0, srcp = 0;
  int cm = 0, n = 0;
  float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f;
  if (gen) {
    const int64_t pid = batch_pid(ids, b);
    om = w.om[b] + w.blk[4 * bx + 2];
    op = w.op[b] + w.blk[4 * bx + 3] + jm_pad;
    w.om[b] = om;
    w.op[b] = op;
    cm = w.cm[b];
    n = cm + w.cp[b];
    src = rec.job_off[pid];
    srcp = rec.job_off[pid + 1] - n;  // job q >= cm comes from srcp + q (the last n - cm slots)
    p0 = rec.pts[3 * pid];
    p1 = rec.pts[3 * pid + 1];
    p2 = rec.pts[3 * pid + 2];
  }
  const int lane = threadIdx.x & 31;
  const float h[3] = {rec.h[0], rec.h[1], rec.h[2]};
  unsigned todo = __ballot_sync(0xffffffffu, gen);
  while (todo) {
    const int l = __ffs(todo) - 1;
    todo &= todo - 1;
    const int64_t g_om = __shfl_sync(0xffffffffu, om, l), g_op = __shfl_sync(0xffffffffu, op, l);
    const int64_t g_src = __shfl_sync(0xffffffffu, src, l), g_srcp = __shfl_sync(0xffffffffu, srcp, l);
    const int g_cm = __shfl_sync(0xffffffffu, cm, l), g_n = __shfl_sync(0xffffffffu, n, l);
    const int32_t g_b = (int32_t)__shfl_sync(0xffffffffu, b, l);
    const float p[3] = {__shfl_sync(0xffffffffu, p0, l), __shfl_sync(0xffffffffu, p1, l),
                        __shfl_sync(0xffffffffu, p2, l)};
    // all of the point's source jobs are loaded before the first store, so that a point costs
    // one memory round trip rather than one per 32 jobs (the stores may alias the loads as
    // far as the compiler knows)
    uint16_t code[kMaxJobRounds];
    float a[kMaxJobRounds];
#pragma unroll
    for (int k = 0; k < kMaxJobRounds; ++k) {
      const int q = lane + 32 * k;
      code[k] = 0;
      a[k] = 0.0f;
      if (q < g_n) {
        const int64_t sq = (q < g_cm ? g_src : g_srcp) + q;
        code[k] = __ldg(rec.job_code + sq);
        a[k] = __ldg(rec.job_A + sq);
      }
    }
#pragma unroll
    for (int k = 0; k < kMaxJobRounds; ++k) {
      const int q = lane + 32 * k;
      if (q < g_n) {
        const int64_t dst = q < g_cm ? g_om + q : g_op + (q - g_cm);
        float x[3];
        job_coords(p, h, code[k], x);
        w.jslot[dst] = g_b;
        w.jcode[dst] = code[k];
        w.jA[dst] = a[k];
        w.jx[dst] = make_float4(x[0], x[1], x[2], 0.0f);
      }
    }
  }
}

// Measured: capping k_emit (and k_residual) at 32 registers for full occupancy did not shorten
// them (the spills cost what the occupancy gained); the batched job loads above did (expansion
// of a 2^18 batch at 128^3: 61 -> 55 us).
__global__ void k_emit(const int32_t* __restrict__ ids, int64_t B, const __grid_constant__ dips_records_t rec,
                       const __grid_constant__ Workspace w) {
  emit_body(ids, B, rec, w, blockIdx.x);
}

__global__ void k_emit_multi(const Inst* __restrict__ T) {
  const Inst& I = T[blockIdx.y];
  if ((int64_t)blockIdx.x >= I.w.nblk) return;
  emit_body(I.ids, I.B, I.rec, I.w, blockIdx.x);
}

// ----------------------------------------------------------------------------------------
// residual and loss of the general points
// ----------------------------------------------------------------------------------------
__device__ __forceinline__ double block_sum_d(double v) {
  __shared__ double ws[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (wid == 0) {
    t = lane < nw ? ws[lane] : 0.0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) t += __shfl_down_sync(0xffffffffu, t, s);
  }
  __syncthreads();
  return t;
}

// One warp handles its general points one at a time, the 32 lanes splitting the point's jobs
// (up to 7 x 27): lhs = lhs0 + sum_j A_j u_j, r = P (lhs/diag - rhs/diag), dL/du_j = dL/dlhs A_j.
// Each lane first loads its own point's records, so that a point's turn costs one round trip
// for its jobs.
//
// With nonlinear operators (rec.nl_pt set) lhs also gets N-(u-) V- + N+(u+) V+ with u-/+ at the
// point = K-/+ + sum_j x-/+_j u_j (discretization.py:369), and dL/du_j gets
// dL/dlhs (N-'(u-) V- x-_j + N+'(u+) V+ x+_j).

// N(u) and N'(u) of a nonlinear operator kind
__device__ __forceinline__ void nl_eval(int kind, float c, float u, float& f, float& df) {
  if (kind == DIPS_NL_SINH) {
    f = c * sinhf(u);
    df = c * coshf(u);
  } else {
    f = 0.0f;
    df = 0.0f;
  }
}

template <bool NL>
__device__ __forceinline__ void residual_body(const int32_t* __restrict__ ids, int64_t B, const dips_records_t& rec,
                                              const Workspace& w, float* __restrict__ residual_out, int bx) {
  const int64_t b = bx * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool overflow = w.ctl->overflow != 0;
  const int kind = b < B ? (overflow ? 3 : w.bk[b]) : -1;
  double l = 0.0;
  if (kind == 3) {
    if (residual_out) residual_out[b] = nanf("");
    l = nan("");
  }
  int64_t om = 0, op = 0;
  int cm = 0, n = 0;
  float lhs0 = 0.0f, diag = 1.0f, rod = 0.0f, Pv = 1.0f;
  constexpr bool nl = NL;  // (the records then carry nl_pt and nl_w; the launch checks it)
  float4 nlp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int64_t ro0 = 0, rop = 0;  // the point's jobs in the records (for their nonlinear weights)
  if (kind == 0) {
    const int64_t pid = batch_pid(ids, b);
    om = w.om[b];
    op = w.op[b];
    cm = w.cm[b];
    n = cm + w.cp[b];
    lhs0 = rec.lhs0[pid];
    diag = rec.diag[pid];
    rod = rec.rod[pid];
    // the learned preconditioner scales both lhs/diag and rhs/diag (discretization.py:419-420)
    if (w.pre_P) Pv = w.pre_P[b];
    if (nl) {
      nlp = reinterpret_cast<const float4*>(rec.nl_pt)[pid];
      ro0 = rec.job_off[pid];
      rop = rec.job_off[pid + 1] - n;
    }
  }
  unsigned todo = __ballot_sync(0xffffffffu, kind == 0);
  while (todo) {
    const int owner = __ffs(todo) - 1;
    todo &= todo - 1;
    const int64_t g_om = __shfl_sync(0xffffffffu, om, owner), g_op = __shfl_sync(0xffffffffu, op, owner);
    const int g_cm = __shfl_sync(0xffffffffu, cm, owner), g_n = __shfl_sync(0xffffffffu, n, owner);
    float av[kMaxJobRounds], xm[kMaxJobRounds], xp[kMaxJobRounds];
    float part = 0.0f, pm = 0.0f, pp = 0.0f;
    if (nl) {
      const int64_t g_ro0 = __shfl_sync(0xffffffffu, ro0, owner), g_rop = __shfl_sync(0xffffffffu, rop, owner);
#pragma unroll
      for (int k = 0; k < kMaxJobRounds; ++k) {
        const int q = lane + 32 * k;
        av[k] = xm[k] = xp[k] = 0.0f;
        if (q < g_n) {
          const int64_t j = q < g_cm ? g_om + q : g_op + (q - g_cm);
          const int64_t r = q < g_cm ? g_ro0 + q : g_rop + q;
          av[k] = w.jA[j];
          const float u = w.ju[j];
          const float2 x = reinterpret_cast<const float2*>(rec.nl_w)[r];
          xm[k] = x.x;
          xp[k] = x.y;
          part = fmaf(av[k], u, part);
          pm = fmaf(x.x, u, pm);
          pp = fmaf(x.y, u, pp);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kMaxJobRounds; ++k) {
        const int q = lane + 32 * k;
        av[k] = xm[k] = xp[k] = 0.0f;
        if (q < g_n) {
          const int64_t j = q < g_cm ? g_om + q : g_op + (q - g_cm);
          av[k] = w.jA[j];
          part = fmaf(av[k], w.ju[j], part);
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (nl) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        pm += __shfl_xor_sync(0xffffffffu, pm, o);
        pp += __shfl_xor_sync(0xffffffffu, pp, o);
      }
    }
    float gs = 0.0f, gm = 0.0f, gp = 0.0f;
    if (lane == owner) {
      float lhs = lhs0 + part;
      float dm = 0.0f, dp = 0.0f;
      if (nl) {
        float fm, fp;
        nl_eval(rec.nl_kind[0], rec.nl_c[0], nlp.x + pm, fm, dm);
        nl_eval(rec.nl_kind[1], rec.nl_c[1], nlp.y + pp, fp, dp);
        lhs += fm * nlp.z + fp * nlp.w;
        dm *= nlp.z;
        dp *= nlp.w;
      }
      const float qv = lhs / diag;
      const float r0 = nan_to_num(qv) - rod;
      const float r = Pv * r0;
      // d(mean 0.5 r^2)/d lhs; nan_to_num has zero derivative where lhs/diag is not finite
      gs = isfinite(qv) ? (r / (float)B) * Pv / diag : 0.0f;
      gm = gs * dm;
      gp = gs * dp;
      w.gs[b] = gs;
      if (w.pre_P) w.pre_r0[b] = r0;
      if (residual_out) residual_out[b] = r;
      l = 0.5 * (double)r * (double)r;
    }
    gs = __shfl_sync(0xffffffffu, gs, owner);
    gm = __shfl_sync(0xffffffffu, gm, owner);
    gp = __shfl_sync(0xffffffffu, gp, owner);
#pragma unroll
    for (int k = 0; k < kMaxJobRounds; ++k) {
      const int q = lane + 32 * k;
      if (q < g_n) w.jg[q < g_cm ? g_om + q : g_op + (q - g_cm)] = nl ? fmaf(gp, xp[k], fmaf(gm, xm[k], gs * av[k]))
                                                                        : gs * av[k];
    }
  }
  const double t = block_sum_d(l);
  if (threadIdx.x == 0) w.lossp[bx] = t;
}

template <bool NL>
__global__ void k_residual(const int32_t* __restrict__ ids, int64_t B, const __grid_constant__ dips_records_t rec,
                           const __grid_constant__ Workspace w, float* __restrict__ residual_out) {
  residual_body<NL>(ids, B, rec, w, residual_out, blockIdx.x);
}

__global__ void k_residual_multi(const Inst* __restrict__ T) {
  const Inst& I = T[blockIdx.y];
  if ((int64_t)blockIdx.x >= I.w.nres) return;
  residual_body<false>(I.ids, I.B, I.rec, I.w, nullptr, blockIdx.x);  // instances have no nonlinear operators
}

__global__ void k_loss_final(Workspace w, int64_t B, double* __restrict__ loss_out) {
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < w.nres; i += blockDim.x) v += w.lossp[i];
  for (int net = 0; net < 2; ++net)
    for (int64_t i = threadIdx.x; i < w.ctl->floss_n[net]; i += blockDim.x) v += w.floss[net * kLossSlots + i];
  const double t = block_sum_d(v);
  if (threadIdx.x == 0) *loss_out = w.ctl->engine_error ? nan("") : t / (double)B;
}

// columns [0, Pm) belong to the u- network and [Pm, Psol) to the u+ network, with
// Ctl::grad_rows partial rows each; columns [Psol, P) to the preconditioner (kPreGrid rows)
__global__ void k_grad_reduce(Workspace w, int P, int Pm, int Psol, float* __restrict__ grad_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  if (i >= Psol) {
    float v = 0.0f;
    for (int c = 0; c < kPreGrid; ++c) v += w.pre_partials[(size_t)c * w.pre_n + (i - Psol)];
    grad_out[i] = w.ctl->engine_error ? nanf("") : v;
    return;
  }
  const int64_t rows = w.ctl->grad_rows[i < Pm ? 0 : 1];
  float v = 0.0f;
  for (int64_t c = 0; c < rows; ++c) v += w.partials[(size_t)c * P + i];
  grad_out[i] = w.ctl->engine_error ? nanf("") : v;
}

// d loss / d theta along a direction theta in coefficient space, the networks held fixed: with
// trec holding d lhs0, d diag, d rod and d A of the records (dips_geometry_assemble_tangent),
//   d r = (d lhs0 + sum_j dA_j u_j) / diag - (lhs / diag) d diag / diag - d rod
// (the first two terms vanish where lhs / diag is not finite, as nan_to_num's derivative does),
// d loss = sum_b (r_b / B) d r_b.  Every batch point is general here (the expansion ran with
// bulk points off), so ju holds u of all its jobs.  One warp per point at a time, the lanes
// splitting its jobs as in k_residual.
__global__ void k_coeff_dot(const int32_t* __restrict__ ids, int64_t B, dips_records_t rec, dips_records_t trec,
                            Workspace w) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool overflow = w.ctl->overflow != 0;
  const int kind = b < B ? (overflow ? 3 : w.bk[b]) : -1;
  double l = kind == 3 ? nan("") : 0.0;
  unsigned todo = __ballot_sync(0xffffffffu, kind == 0);
  while (todo) {
    const int owner = __ffs(todo) - 1;
    todo &= todo - 1;
    const int64_t gb = __shfl_sync(0xffffffffu, b, owner);
    const int64_t om = w.om[gb], op = w.op[gb];
    const int cm = w.cm[gb], n = cm + w.cp[gb];
    const int64_t pid = batch_pid(ids, gb);
    const int64_t srcm = rec.job_off[pid], srcp = rec.job_off[pid + 1] - n;
    float part = 0.0f, tpart = 0.0f;
    for (int q = lane; q < n; q += 32) {
      const int64_t j = q < cm ? om + q : op + (q - cm);
      const int64_t src = (q < cm ? srcm : srcp) + q;
      const float u = w.ju[j];
      part = fmaf(w.jA[j], u, part);
      tpart = fmaf(trec.job_A[src], u, tpart);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      part += __shfl_xor_sync(0xffffffffu, part, o);
      tpart += __shfl_xor_sync(0xffffffffu, tpart, o);
    }
    if (lane == owner) {
      const float lhs = rec.lhs0[pid] + part;
      const float diag = rec.diag[pid];
      const float qv = lhs / diag;
      const float r = nan_to_num(qv) - rec.rod[pid];
      double dr = -(double)trec.rod[pid];
      if (isfinite(qv)) dr += ((double)trec.lhs0[pid] + tpart - (double)qv * trec.diag[pid]) / diag;
      l = (double)r / (double)B * dr;
    }
  }
  const double t = block_sum_d(l);
  if (threadIdx.x == 0) w.lossp[blockIdx.x] = t;
}

__global__ void k_coeff_final(Workspace w, double* __restrict__ out) {
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < w.nres; i += blockDim.x) v += w.lossp[i];
  const double t = block_sum_d(v);
  if (threadIdx.x == 0) *out = t;
}

// The optax chain (clip_by_global_norm, scale_by_adam, exponential-decay schedule, scale by
// -1; solvers/optimizers.py:33-54) over P parameters by one block, given the squared gradient
// norm; or optax.rmsprop, or the polynomial schedule (dips_adam_t).  Thread 0 increments the
// step counter.
__device__ void adam_update(const dips_adam_t& hp, int P, float gsq, float* __restrict__ params,
                            const float* __restrict__ grad, float* __restrict__ mu, float* __restrict__ nu,
                            int64_t* __restrict__ count) {
  __shared__ int64_t s_count;
  if (threadIdx.x == 0) s_count = *count;
  __syncthreads();
  const float gn = sqrtf(gsq);
  // clip_by_global_norm: keep g when gnorm < max_norm, else g / gnorm * max_norm
  const float gnorm = (gn < hp.max_norm) ? -1.0f : gn;
  const int64_t cnt0 = s_count;
  const float cnt1 = (float)(cnt0 + 1);
  const float bc1 = 1.0f - powf(hp.b1, cnt1);
  const float bc2 = 1.0f - powf(hp.b2, cnt1);
  float step;
  if (hp.schedule == DIPS_SCHED_POLYNOMIAL)
    step = hp.lr * (1.0f - fminf((float)cnt0, hp.transition_steps) / hp.transition_steps);
  else
    step = hp.lr * powf(hp.decay_rate, (float)cnt0 / hp.transition_steps);
  if (hp.kind == DIPS_OPT_RMSPROP) {
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
      float g = __ldcg(grad + i);
      if (gnorm >= 0.0f) g = (g / gnorm) * hp.max_norm;
      const float v = (1.0f - hp.b2) * (g * g) + hp.b2 * nu[i];
      nu[i] = v;
      const float upd = g / sqrtf(v + hp.eps);
      params[i] = params[i] + (upd * step) * -1.0f;
    }
    if (threadIdx.x == 0) *count = cnt0 + 1;
    return;
  }
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    float g = __ldcg(grad + i);  // L2: other blocks of k_reduce_adam wrote it in this launch
    if (gnorm >= 0.0f) g = (g / gnorm) * hp.max_norm;
    const float m = (1.0f - hp.b1) * g + hp.b1 * mu[i];
    const float v = (1.0f - hp.b2) * (g * g) + hp.b2 * nu[i];
    mu[i] = m;
    nu[i] = v;
    const float upd = (m / bc1) / (sqrtf(v / bc2) + hp.eps);
    params[i] = params[i] + (upd * step) * -1.0f;
  }
  if (threadIdx.x == 0) *count = cnt0 + 1;
}

__global__ void k_adam(dips_adam_t hp, int P, float* __restrict__ params, const float* __restrict__ grad,
                       float* __restrict__ mu, float* __restrict__ nu, int64_t* __restrict__ count) {
  __shared__ float red[32];
  __shared__ float s_sq;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float ss = 0.0f;
  for (int i = threadIdx.x; i < P; i += blockDim.x) ss = fmaf(grad[i], grad[i], ss);
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, s);
  if (lane == 0) red[wid] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int q = 0; q < nw; ++q) t += red[q];
    s_sq = t;
  }
  __syncthreads();
  adam_update(hp, P, s_sq, params, grad, mu, nu, count);
}

// The tail of a training step in one launch.  Each block sums 32 gradient columns over the
// partial rows, the rows split over its 32 warps (a few loads per thread instead of a
// latency-bound column walk), and adds up the squares of its columns; the last block to finish
// writes the loss (as k_loss_final) and applies the optax chain to all P parameters.
__device__ __forceinline__ void reduce_adam_body(const Workspace& w, int P, int Pm, int Psol, float* __restrict__ grad,
                                                 const dips_adam_t& hp, float* __restrict__ params,
                                                 float* __restrict__ mu, float* __restrict__ nu,
                                                 int64_t* __restrict__ count, int64_t B, double* __restrict__ loss_out,
                                                 int bx, int nb) {
  __shared__ float part[32][33];
  __shared__ bool s_last;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i = bx * 32 + tx;
  const bool err = w.ctl->engine_error != 0;
  float v = 0.0f;
  if (i < P) {
    if (i >= Psol) {
      for (int c = ty; c < kPreGrid; c += 32) v += w.pre_partials[(size_t)c * w.pre_n + (i - Psol)];
    } else {
      const int64_t rows = w.ctl->grad_rows[i < Pm ? 0 : 1];
      for (int64_t c = ty; c < rows; c += 32) v += w.partials[(size_t)c * P + i];
    }
  }
  part[ty][tx] = v;
  __syncthreads();
  if (ty == 0) {
    float t = 0.0f;
#pragma unroll 8
    for (int k = 0; k < 32; ++k) t += part[k][tx];
    if (err) t = nanf("");
    if (i < P) {
      grad[i] = t;
      __threadfence();  // visible to the last block before this block is counted
    }
    double sq = i < P ? (double)t * (double)t : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (tx == 0) {
      w.sqp[bx] = sq;
      __threadfence();
      const unsigned long long n = atomicAdd(reinterpret_cast<unsigned long long*>(&w.ctl->reduce_done), 1ull);
      s_last = n == (unsigned long long)(nb - 1);
    }
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // loss of the batch (the FP64 partials of the residual kernels)
  double l = 0.0;
  for (int64_t k = threadIdx.x; k < w.nres; k += blockDim.x) l += w.lossp[k];
  for (int net = 0; net < 2; ++net)
    for (int64_t k = threadIdx.x; k < w.ctl->floss_n[net]; k += blockDim.x) l += w.floss[net * kLossSlots + k];
  double g2 = 0.0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) g2 += __ldcg(w.sqp + k);
  const double lt = block_sum_d(l);
  const double gt = block_sum_d(g2);
  if (threadIdx.x == 0 && loss_out) *loss_out = err ? nan("") : lt / (double)B;
  __shared__ float s_g2;
  if (threadIdx.x == 0) s_g2 = (float)gt;
  __syncthreads();
  adam_update(hp, P, s_g2, params, grad, mu, nu, count);
}

__global__ void __launch_bounds__(kReduceThreads) k_reduce_adam(const __grid_constant__ Workspace w, int P, int Pm,
                                                                int Psol, float* __restrict__ grad, dips_adam_t hp,
                                                                float* __restrict__ params, float* __restrict__ mu,
                                                                float* __restrict__ nu, int64_t* __restrict__ count,
                                                                int64_t B, double* __restrict__ loss_out) {
  reduce_adam_body(w, P, Pm, Psol, grad, hp, params, mu, nu, count, B, loss_out, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kReduceThreads) k_reduce_adam_multi(const Inst* __restrict__ T, int P, int Pm,
                                                                      int Psol, dips_adam_t hp) {
  const Inst& I = T[blockIdx.y];
  reduce_adam_body(I.w, P, Pm, Psol, I.grad, hp, I.params, I.mu, I.nu, I.count, I.B, I.loss_out, blockIdx.x,
                   gridDim.x);
}

// ----------------------------------------------------------------------------------------
// seeded bijective permutation (4-round Feistel network with cycle walking)
// ----------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint64_t feistel(uint64_t v, int half, uint64_t key) {
  const uint64_t mask = (1ull << half) - 1;
  uint64_t l = v >> half, r = v & mask;
#pragma unroll
  for (int round = 0; round < 4; ++round) {
    const uint32_t f = mix32((uint32_t)r ^ (uint32_t)(key >> (round * 8)) ^ (uint32_t)(round * 0x9e3779b9u) ^
                             (uint32_t)(key >> 32));
    const uint64_t nl = r;
    r = (l ^ f) & mask;
    l = nl;
  }
  return (l << half) | r;
}

__global__ void k_batch_ids(int64_t n, uint64_t key, int half, int64_t start, int64_t B, int32_t* __restrict__ ids) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  uint64_t v = (uint64_t)(start + b);
  // cycle walking: iterate the permutation of [0, 2^(2*half)) until the value lands in [0, n)
  for (int it = 0; it < (1 << 24); ++it) {
    v = feistel(v, half, key);
    if (v < (uint64_t)n) break;
  }
  ids[b] = (int32_t)v;
}

// batch ids from a device step counter (graph-replay friendly): step = *counter,
// batch = step % nb, epoch = step / nb.  mode 0: consecutive ranges (the reference's fixed
// sequential batches, data_management.py:104-159); mode 1: a per-epoch seeded permutation.
__device__ __forceinline__ void batch_ids_body(int64_t n, int64_t B, int64_t nb, uint64_t seed, int mode, int half,
                                               const int64_t* __restrict__ counter, int32_t* __restrict__ ids,
                                               int64_t b) {
  if (b >= B) return;
  const int64_t step = *counter;
  const int64_t bi = step % nb, epoch = step / nb;
  if (mode == 0) {
    ids[b] = (int32_t)(bi * B + b);
    return;
  }
  const uint64_t key = seed * 0x9E3779B97F4A7C15ull ^ (uint64_t)(epoch + 1) * 0xD1B54A32D192ED03ull;
  uint64_t v = (uint64_t)(bi * B + b);
  for (int it = 0; it < (1 << 24); ++it) {
    v = feistel(v, half, key);
    if (v < (uint64_t)n) break;
  }
  ids[b] = (int32_t)v;
}

__global__ void k_batch_ids_dev(int64_t n, int64_t B, int64_t nb, uint64_t seed, int mode, int half,
                                const int64_t* __restrict__ counter, int32_t* __restrict__ ids) {
  batch_ids_body(n, B, nb, seed, mode, half, counter, ids, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

__global__ void k_batch_ids_multi(const Inst* __restrict__ T) {
  const Inst& I = T[blockIdx.y];
  if (I.ids_mode < 0) return;
  batch_ids_body(I.rec.n_pts, I.B, I.n_batches, I.seed, I.ids_mode, I.ids_half, I.count, I.ids,
                 blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// ----------------------------------------------------------------------------------------
// network-shape table
// ----------------------------------------------------------------------------------------
const ArchOps* arch_ops_1_1_2_10();
const ArchOps* arch_ops_2_8_2_8();
const ArchOps* arch_ops_2_16_2_16();
const ArchOps* arch_ops_3_32_3_32();
const ArchOps* arch_ops_4_64_4_64();

static const ArchOps* find_arch(const dips_arch_t* a) {
  if (!a) {
    set_error("null arch");
    return nullptr;
  }
  const ArchOps* table[] = {arch_ops_1_1_2_10(), arch_ops_2_8_2_8(), arch_ops_2_16_2_16(), arch_ops_3_32_3_32(),
                            arch_ops_4_64_4_64()};
  for (const ArchOps* o : table)
    if (o->m_layers == a->m_layers && o->m_width == a->m_width && o->p_layers == a->p_layers &&
        o->p_width == a->p_width)
      return o;
  set_error("no kernel compiled for DoubleMLP m=%dx%d p=%dx%d (supported: 1x1/2x10, 2x8/2x8, 2x16/2x16, 3x32/3x32, "
            "4x64/4x64)",
            a->m_layers, a->m_width, a->p_layers, a->p_width);
  return nullptr;
}

static int net_params(int L, int W) { return 3 * W + W + (L - 1) * (W * W + W) + W + 1; }

// parameters of the learned preconditioner (0 when it is off, -1 for an unsupported shape)
static int arch_pre_params(const dips_arch_t* a) {
  if (!a || a->pre_layers <= 0) return 0;
  return pre_supported(a->pre_layers, a->pre_width) ? pre_num_params(a->pre_layers, a->pre_width) : -1;
}

static int arch_params(const dips_arch_t* a) {
  if (!a || a->m_layers < 1 || a->p_layers < 1 || a->m_width < 1 || a->p_width < 1) return -1;
  const int pre = arch_pre_params(a);
  if (pre < 0) return -1;
  return net_params(a->m_layers, a->m_width) + net_params(a->p_layers, a->p_width) + pre;
}

static int check_rec(const dips_records_t* rec, int64_t B) {
  DIPS_REQUIRE(rec && rec->pts && rec->lhs0 && rec->diag && rec->rod && rec->cnt && rec->cnt_m && rec->job_off &&
                   rec->job_code && rec->job_A,
               DIPS_E_ARG, "records: null pointer");
  DIPS_REQUIRE(B > 0 && B <= 0x7fffffff, DIPS_E_ARG, "batch size must be in [1, 2^31)");
  DIPS_REQUIRE((rec->nl_pt == nullptr) == (rec->nl_w == nullptr), DIPS_E_ARG,
               "records: nl_pt and nl_w are given together");
  if (rec->nl_pt)
    for (int k = 0; k < 2; ++k)
      DIPS_REQUIRE(rec->nl_kind[k] == DIPS_NL_ZERO || rec->nl_kind[k] == DIPS_NL_SINH, DIPS_E_ARG,
                   "records: unknown nonlinear operator kind %d", rec->nl_kind[k]);
  return DIPS_OK;
}

static PtsH make_ph(const dips_records_t* rec) {
  PtsH ph;
  ph.pts = rec->pts;
  ph.h[0] = rec->h[0];
  ph.h[1] = rec->h[1];
  ph.h[2] = rec->h[2];
  return ph;
}

static int prep_ws(const dips_arch_t* arch, const float* params, int64_t B, void* ws, size_t ws_bytes, Workspace* W) {
  const int P = arch_params(arch);
  DIPS_REQUIRE(P > 0, DIPS_E_ARG, "invalid arch");
  DIPS_REQUIRE(ws != nullptr, DIPS_E_ARG, "null workspace");
  const int pre_n = arch_pre_params(arch);
  const size_t fixed = carve(nullptr, nullptr, B, 0, P, pre_n);
  DIPS_REQUIRE(ws_bytes >= fixed + 256, DIPS_E_WORKSPACE, "workspace too small: %zu < %zu", ws_bytes, fixed + 256);
  char* base = (char*)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
  const size_t avail = ws_bytes - (size_t)(base - (char*)ws);
  // largest job capacity whose layout fits
  int64_t lo = 0, hi = (int64_t)(avail / 14) + 1;
  while (lo + 1 < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (carve(nullptr, nullptr, B, mid, P, pre_n) <= avail)
      lo = mid;
    else
      hi = mid;
  }
  carve(W, base, B, lo, P, pre_n);
  W->params = params;
  return DIPS_OK;
}

static int expand(const dips_records_t* rec, const int32_t* ids, int64_t B, Workspace& W, int bulk_ok,
                  const Marks* mk, cudaStream_t s) {
  const int nblk = (int)W.nblk;
  mark(mk, kMarkStart, s);
  // with nonlinear operators every point takes the general path
  k_count<<<nblk, kScanBlock, 0, s>>>(ids, B, rec->n_pts, rec->cnt, rec->cnt_m, bulk_ok && !rec->nl_pt, W);
  k_scan_blocks<<<1, kScanBlock, 0, s>>>(W);
  k_emit<<<nblk, kScanBlock, 0, s>>>(ids, B, *rec, W);
  DIPS_CHECK_LAUNCH("batch expansion");
  mark(mk, kMarkExpand, s);
  return DIPS_OK;
}

// expansion, general forward + residual, fused bulk kernel (with or without its gradient)
static int run_forward(const ArchOps* ops, const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                       const int32_t* ids, int64_t B, Workspace& W, double* loss_out, float* residual_out,
                       bool fused_bwd, const Marks* mk, cudaStream_t s) {
  int st = expand(rec, ids, B, W, ops->bulk_ok, mk, s);
  if (st) return st;
  if (W.pre_n) {  // the preconditioner's value per slot, read by every residual kernel
    st = precond_forward(*arch, params + ops->n_params, *rec, ids, B, W, s);
    if (st) return st;
  }
  st = ops->job_forward(make_ph(rec), ids, W, mk, s);
  if (st) return st;
  if (rec->nl_pt)  // the nonlinear operators' variant (more registers) only where they are given
    k_residual<true><<<(int)W.nres, 256, 0, s>>>(ids, B, *rec, W, residual_out);
  else
    k_residual<false><<<(int)W.nres, 256, 0, s>>>(ids, B, *rec, W, residual_out);
  DIPS_CHECK_LAUNCH("residual");
  mark(mk, kMarkResidual, s);
  st = ops->bulk_fused(make_ph(rec), ids, W, *rec, residual_out, fused_bwd, mk, s);
  if (st) return st;
  if (loss_out) k_loss_final<<<1, 256, 0, s>>>(W, B, loss_out);
  DIPS_CHECK_LAUNCH("loss");
  mark(mk, kMarkLoss, s);
  return DIPS_OK;
}

// general adjoint (shapes without the tile engine) and the preconditioner's backward
static int run_adjoint(const ArchOps* ops, const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                       const int32_t* ids, int64_t B, Workspace& W, const Marks* mk, cudaStream_t s) {
  int st = ops->job_adjoint(make_ph(rec), ids, W, mk, s);
  if (st) return st;
  if (W.pre_n) {
    st = precond_backward(*arch, params + ops->n_params, *rec, ids, B, W, s);
    if (st) return st;
  }
  return DIPS_OK;
}

// general adjoint and the reduction of all partial gradient rows
static int run_backward(const ArchOps* ops, const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                        const int32_t* ids, int64_t B, Workspace& W, float* grad_out, const Marks* mk,
                        cudaStream_t s) {
  int st = run_adjoint(ops, arch, params, rec, ids, B, W, mk, s);
  if (st) return st;
  const int Pm = ops->n_params - net_params(ops->p_layers, ops->p_width);
  const int P = ops->n_params + W.pre_n;
  k_grad_reduce<<<div_up(P, 256), 256, 0, s>>>(W, P, Pm, ops->n_params, grad_out);
  DIPS_CHECK_LAUNCH("gradient reduction");
  mark(mk, kMarkReduce, s);
  return DIPS_OK;
}

}  // namespace dips

using namespace dips;

extern "C" int32_t dips_num_params(const dips_arch_t* arch) { return arch_params(arch); }

extern "C" int32_t dips_arch_supported(const dips_arch_t* arch) { return find_arch(arch) ? 1 : 0; }

extern "C" size_t dips_step_workspace_bytes(const dips_arch_t* arch, int64_t batch, int64_t max_jobs) {
  const int P = arch_params(arch);
  if (P <= 0 || batch <= 0 || max_jobs < 0) return 0;
  return carve(nullptr, nullptr, batch, max_jobs, P, arch_pre_params(arch)) + 256;
}

extern "C" int dips_residual_fwd(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                                 const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                                 double* loss_out, float* residual_out, cudaStream_t stream) {
  int st = check_rec(rec, batch);
  if (st) return st;
  DIPS_REQUIRE(params, DIPS_E_ARG, "null params");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  Workspace W;
  st = prep_ws(arch, params, batch, workspace, ws_bytes, &W);
  if (st) return st;
  st = ops->load_params(params, 0, stream);
  if (st) return st;
  return run_forward(ops, arch, params, rec, batch_ids, batch, W, loss_out, residual_out, false, nullptr, stream);
}

extern "C" int dips_residual_bwd(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                                 const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                                 float* grad_out, cudaStream_t stream) {
  int st = check_rec(rec, batch);
  if (st) return st;
  DIPS_REQUIRE(params && grad_out, DIPS_E_ARG, "null params or grad_out");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  Workspace W;
  st = prep_ws(arch, params, batch, workspace, ws_bytes, &W);
  if (st) return st;
  st = ops->load_params(params, 0, stream);
  if (st) return st;
  // the bulk points' gradient comes from the fused kernel, run again with its backward half
  st = ops->bulk_fused(make_ph(rec), batch_ids, W, *rec, nullptr, true, nullptr, stream);
  if (st) return st;
  return run_backward(ops, arch, params, rec, batch_ids, batch, W, grad_out, nullptr, stream);
}

extern "C" int dips_pack_bulk_records(const dips_records_t* rec, float* out, cudaStream_t stream) {
  DIPS_REQUIRE(rec && out && rec->pts && rec->lhs0 && rec->diag && rec->rod && rec->cnt && rec->cnt_m &&
                   rec->job_off && rec->job_code && rec->job_A,
               DIPS_E_ARG, "dips_pack_bulk_records: null pointer");
  DIPS_REQUIRE(((uintptr_t)out & 15) == 0, DIPS_E_ARG, "dips_pack_bulk_records: out must be 16-byte aligned");
  if (rec->n_pts <= 0) return DIPS_OK;
  int64_t grid = div_up(rec->n_pts, 256);
  if (grid > 152 * 32) grid = 152 * 32;
  k_pack_bulk<<<(int)grid, 256, 0, stream>>>(*rec, out);
  DIPS_CHECK_LAUNCH("dips_pack_bulk_records");
  return DIPS_OK;
}

extern "C" int dips_loss_coeff_tangent(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                                       const dips_records_t* trec, const int32_t* batch_ids, int64_t batch,
                                       void* workspace, size_t ws_bytes, double* dloss_out, cudaStream_t stream) {
  int st = check_rec(rec, batch);
  if (st) return st;
  DIPS_REQUIRE(arch && params && dloss_out && trec, DIPS_E_ARG, "null arch, params, trec or dloss_out");
  DIPS_REQUIRE(trec->lhs0 && trec->diag && trec->rod && trec->job_A, DIPS_E_ARG, "null tangent record array");
  DIPS_REQUIRE(arch->pre_layers == 0, DIPS_E_UNSUPPORTED,
               "dips_loss_coeff_tangent: the learned preconditioner's dependence on the coefficients is not "
               "differentiated");
  DIPS_REQUIRE(!rec->nl_pt, DIPS_E_UNSUPPORTED,
               "dips_loss_coeff_tangent: the nonlinear operators' terms are not differentiated along a coefficient");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  Workspace W;
  st = prep_ws(arch, params, batch, workspace, ws_bytes, &W);
  if (st) return st;
  st = ops->load_params(params, 0, stream);
  if (st) return st;
  st = expand(rec, batch_ids, batch, W, 0, nullptr, stream);  // every point general: u of all jobs
  if (st) return st;
  st = ops->job_forward(make_ph(rec), batch_ids, W, nullptr, stream);
  if (st) return st;
  k_coeff_dot<<<(int)W.nres, 256, 0, stream>>>(batch_ids, batch, *rec, *trec, W);
  k_coeff_final<<<1, 256, 0, stream>>>(W, dloss_out);
  DIPS_CHECK_LAUNCH("dips_loss_coeff_tangent");
  return DIPS_OK;
}

static int check_hp(const dips_adam_t* hp) {
  DIPS_REQUIRE(hp, DIPS_E_ARG, "null optimizer hyperparameters");
  DIPS_REQUIRE(hp->kind == DIPS_OPT_ADAM || hp->kind == DIPS_OPT_RMSPROP, DIPS_E_ARG, "unknown optimizer kind %d",
               hp->kind);
  DIPS_REQUIRE(hp->schedule == DIPS_SCHED_EXPONENTIAL || hp->schedule == DIPS_SCHED_POLYNOMIAL, DIPS_E_ARG,
               "unknown schedule %d", hp->schedule);
  DIPS_REQUIRE(hp->transition_steps > 0.0f, DIPS_E_ARG, "transition_steps must be positive");
  return DIPS_OK;
}

extern "C" int dips_adam_step(const dips_arch_t* arch, const dips_adam_t* hp, float* params, const float* grad,
                              float* mu, float* nu, int64_t* count, cudaStream_t stream) {
  const int P = arch_params(arch);
  DIPS_REQUIRE(P > 0 && hp && params && grad && mu && nu && count, DIPS_E_ARG, "dips_adam_step: bad argument");
  int sth = check_hp(hp);
  if (sth) return sth;
  k_adam<<<1, 1024, 0, stream>>>(*hp, P, params, grad, mu, nu, count);
  DIPS_CHECK_LAUNCH("dips_adam_step");
  return DIPS_OK;
}

static int train_step(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu, float* nu,
                      int64_t* count, const dips_records_t* rec, const int32_t* batch_ids, int64_t batch,
                      void* workspace, size_t ws_bytes, double* loss_out, float* grad_out, const Marks* mk,
                      cudaStream_t stream) {
  int st = check_rec(rec, batch);
  if (st) return st;
  DIPS_REQUIRE(hp && params && mu && nu && count, DIPS_E_ARG, "dips_train_step: null pointer");
  st = check_hp(hp);
  if (st) return st;
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  Workspace W;
  st = prep_ws(arch, params, batch, workspace, ws_bytes, &W);
  if (st) return st;
  st = ops->load_params(params, 0, stream);
  if (st) return st;
  // the loss is written by the step's last kernel (k_reduce_adam), before the update
  st = run_forward(ops, arch, params, rec, batch_ids, batch, W, nullptr, nullptr, true, mk, stream);
  if (st) return st;
  float* g = grad_out ? grad_out : W.grad;
  st = run_adjoint(ops, arch, params, rec, batch_ids, batch, W, mk, stream);
  if (st) return st;
  const int Pm = ops->n_params - net_params(ops->p_layers, ops->p_width);
  const int P = ops->n_params + W.pre_n;
  k_reduce_adam<<<div_up(P, 32), kReduceThreads, 0, stream>>>(W, P, Pm, ops->n_params, g, *hp, params, mu, nu,
                                                               count, batch, loss_out);
  DIPS_CHECK_LAUNCH("dips_train_step gradient reduction and adam");
  mark(mk, kMarkReduce, stream);
  mark(mk, kMarkAdam, stream);
  return DIPS_OK;
}

extern "C" int dips_train_step(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu, float* nu,
                               int64_t* count, const dips_records_t* rec, const int32_t* batch_ids, int64_t batch,
                               void* workspace, size_t ws_bytes, double* loss_out, float* grad_out,
                               cudaStream_t stream) {
  return train_step(arch, hp, params, mu, nu, count, rec, batch_ids, batch, workspace, ws_bytes, loss_out, grad_out,
                    nullptr, stream);
}

extern "C" int dips_train_step_profiled(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu,
                                        float* nu, int64_t* count, const dips_records_t* rec,
                                        const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                                        double* loss_out, float* grad_out, cudaEvent_t* events, int32_t n_events,
                                        cudaStream_t stream) {
  DIPS_REQUIRE(events && n_events >= 0, DIPS_E_ARG, "dips_train_step_profiled: null event array");
  const Marks mk = {events, n_events < kMarkCount ? n_events : (int)kMarkCount};
  return train_step(arch, hp, params, mu, nu, count, rec, batch_ids, batch, workspace, ws_bytes, loss_out, grad_out,
                    &mk, stream);
}

extern "C" int dips_autotune(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                             const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                             int32_t* choice_out, cudaStream_t stream) {
  int st = check_rec(rec, batch);
  if (st) return st;
  DIPS_REQUIRE(params, DIPS_E_ARG, "dips_autotune: null params");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  Workspace W;
  st = prep_ws(arch, params, batch, workspace, ws_bytes, &W);
  if (st) return st;
  st = ops->load_params(params, 0, stream);
  if (st) return st;
  int chosen = 0;
  if (ops->autotune) {
    // the forward prepares what the timed launches read (job lists, records, dL/du)
    st = run_forward(ops, arch, params, rec, batch_ids, batch, W, nullptr, nullptr, false, nullptr, stream);
    if (st) return st;
    st = ops->autotune(make_ph(rec), batch_ids, W, *rec, stream, &chosen);
    if (st) return st;
  }
  if (choice_out) *choice_out = chosen;
  return DIPS_OK;
}

extern "C" size_t dips_instances_table_bytes(int32_t n) { return n > 0 ? sizeof(Inst) * (size_t)n : 0; }

static int feistel_half(int64_t n) {
  int bits = 1;
  while ((1ll << bits) < n) ++bits;
  return (bits + 1) / 2;
}

extern "C" int dips_instances_prepare(const dips_arch_t* arch, const dips_instance_t* inst, int32_t n, void* table,
                                      size_t table_bytes, cudaStream_t stream) {
  DIPS_REQUIRE(arch && inst && table && n > 0 && n <= 256, DIPS_E_ARG, "dips_instances_prepare: bad argument");
  DIPS_REQUIRE(table_bytes >= sizeof(Inst) * (size_t)n, DIPS_E_WORKSPACE, "dips_instances_prepare: table too small");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  std::vector<Inst> host((size_t)n);
  for (int i = 0; i < n; ++i) {
    const dips_instance_t& d = inst[i];
    int st = check_rec(d.rec, d.batch);
    if (st) return st;
    DIPS_REQUIRE(d.params && d.mu && d.nu && d.count && d.batch_ids, DIPS_E_ARG,
                 "dips_instances_prepare: instance %d: null pointer", i);
    DIPS_REQUIRE(!d.rec->nl_pt, DIPS_E_UNSUPPORTED,
                 "dips_instances_prepare: instance %d: nonlinear operators take the single-instance step", i);
    DIPS_REQUIRE(d.ids_mode >= -1 && d.ids_mode <= 1, DIPS_E_ARG, "dips_instances_prepare: instance %d: ids_mode", i);
    if (d.ids_mode >= 0)
      DIPS_REQUIRE(d.n_batches > 0 && d.n_batches * d.batch <= d.rec->n_pts && d.rec->n_pts <= 0x7fffffff, DIPS_E_ARG,
                   "dips_instances_prepare: instance %d: %lld batches of %lld exceed n=%lld", i,
                   (long long)d.n_batches, (long long)d.batch, (long long)d.rec->n_pts);
    Inst& I = host[(size_t)i];
    st = prep_ws(arch, d.params, d.batch, d.workspace, d.ws_bytes, &I.w);
    if (st) return st;
    I.rec = *d.rec;
    I.ids = d.batch_ids;
    I.B = d.batch;
    I.n_batches = d.n_batches;
    I.seed = d.seed;
    I.ids_mode = d.ids_mode;
    I.ids_half = feistel_half(d.rec->n_pts);
    I.params = d.params;
    I.mu = d.mu;
    I.nu = d.nu;
    I.count = d.count;
    I.grad = d.grad_out ? d.grad_out : I.w.grad;
    I.loss_out = d.loss_out;
  }
  cudaError_t e = cudaMemcpyAsync(table, host.data(), sizeof(Inst) * (size_t)n, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  return e == cudaSuccess ? DIPS_OK : cuda_status(e, "dips_instances_prepare: table copy");
}

extern "C" int dips_train_step_instances(const dips_arch_t* arch, const dips_adam_t* hp, const void* table, int32_t n,
                                         int64_t max_batch, cudaStream_t stream) {
  if (hp) {
    const int sth = check_hp(hp);
    if (sth) return sth;
  }
  DIPS_REQUIRE(arch && hp && table && n > 0 && n <= 256 && max_batch > 0 && max_batch <= 0x7fffffff, DIPS_E_ARG,
               "dips_train_step_instances: bad argument");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  DIPS_REQUIRE(ops->multi_forward && ops->multi_train && arch->pre_layers == 0, DIPS_E_UNSUPPORTED,
               "dips_train_step_instances: needs a tile-engine shape (3x32, 2x16) without the preconditioner");
  const Inst* T = static_cast<const Inst*>(table);
  const int nblk = div_up(max_batch, kScanBlock), nres = div_up(max_batch, 256);
  k_batch_ids_multi<<<dim3(div_up(max_batch, 256), n), 256, 0, stream>>>(T);
  k_count_multi<<<dim3(nblk, n), kScanBlock, 0, stream>>>(T, ops->bulk_ok);
  k_scan_blocks_multi<<<n, kScanBlock, 0, stream>>>(T);
  k_emit_multi<<<dim3(nblk, n), kScanBlock, 0, stream>>>(T);
  DIPS_CHECK_LAUNCH("dips_train_step_instances expansion");
  int st = ops->multi_forward(T, n, stream);
  if (st) return st;
  k_residual_multi<<<dim3(nres, n), 256, 0, stream>>>(T);
  DIPS_CHECK_LAUNCH("dips_train_step_instances residual");
  st = ops->multi_train(T, n, stream);
  if (st) return st;
  const int Pm = ops->n_params - net_params(ops->p_layers, ops->p_width);
  const int P = ops->n_params;
  k_reduce_adam_multi<<<dim3(div_up(P, 32), n), kReduceThreads, 0, stream>>>(T, P, Pm, ops->n_params, *hp);
  DIPS_CHECK_LAUNCH("dips_train_step_instances gradient tail");
  return DIPS_OK;
}

extern "C" int dips_batch_ids(int64_t n, int64_t epoch_index, uint64_t seed, int64_t batch_index, int64_t batch,
                              int32_t* ids, cudaStream_t stream) {
  DIPS_REQUIRE(n > 0 && n <= 0x7fffffff && batch > 0 && ids && batch_index >= 0, DIPS_E_ARG,
               "dips_batch_ids: bad argument");
  DIPS_REQUIRE((batch_index + 1) * batch <= n, DIPS_E_ARG, "dips_batch_ids: batch %lld of size %lld exceeds n=%lld",
               (long long)batch_index, (long long)batch, (long long)n);
  int bits = 1;
  while ((1ll << bits) < n) ++bits;
  const int half = (bits + 1) / 2;
  const uint64_t key = seed * 0x9E3779B97F4A7C15ull ^ (uint64_t)(epoch_index + 1) * 0xD1B54A32D192ED03ull;
  k_batch_ids<<<div_up(batch, 256), 256, 0, stream>>>(n, key, half, batch_index * batch, batch, ids);
  DIPS_CHECK_LAUNCH("dips_batch_ids");
  return DIPS_OK;
}

extern "C" int dips_batch_ids_device(int64_t n, int64_t batch, int64_t n_batches, uint64_t seed, int32_t mode,
                                     const int64_t* step_counter, int32_t* ids, cudaStream_t stream) {
  DIPS_REQUIRE(n > 0 && n <= 0x7fffffff && batch > 0 && n_batches > 0 && step_counter && ids && (mode == 0 || mode == 1),
               DIPS_E_ARG, "dips_batch_ids_device: bad argument");
  DIPS_REQUIRE(n_batches * batch <= n, DIPS_E_ARG, "dips_batch_ids_device: %lld batches of %lld exceed n=%lld",
               (long long)n_batches, (long long)batch, (long long)n);
  int bits = 1;
  while ((1ll << bits) < n) ++bits;
  k_batch_ids_dev<<<div_up(batch, 256), 256, 0, stream>>>(n, batch, n_batches, seed, mode, (bits + 1) / 2,
                                                          step_counter, ids);
  DIPS_CHECK_LAUNCH("dips_batch_ids_device");
  return DIPS_OK;
}

extern "C" int dips_mlp_eval(const dips_arch_t* arch, const float* params, const float* pts, const float* phi_at,
                             int64_t n, float* u_out, float* grad_out, cudaStream_t stream) {
  DIPS_REQUIRE(n >= 0, DIPS_E_ARG, "dips_mlp_eval: negative n");
  if (n == 0) return DIPS_OK;
  DIPS_REQUIRE(params && pts && phi_at && u_out, DIPS_E_ARG, "dips_mlp_eval: null pointer");
  const ArchOps* ops = find_arch(arch);
  if (!ops) return DIPS_E_UNSUPPORTED;
  int st = ops->load_params(params, 1, stream);
  if (st) return st;
  return ops->mlp_eval(params, pts, phi_at, n, u_out, grad_out, stream);
}
