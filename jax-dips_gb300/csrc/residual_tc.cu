// DoubleMLP 4x64 (four tanh hidden layers of width 64 per phase) on the fifth-generation tensor
// cores: tcgen05.mma kind::tf32 with FP32 accumulation in tensor memory (TMEM).
//
// Reference: DoubleMLP (nn/mlp/MLP.py:93-139) inside the NBM loss and its gradient
// (solvers/poisson/trainer.py:783-789, :892-912).  Every point of this shape is expanded into
// jobs (no bulk kernel); two kernels per network do the work:
//
//   k_tc_forward   u at every job of the network (feeds the residual of every point)
//   k_tc_adjoint   forward again (the activations are recomputed, not stored between kernels),
//                  then dL/dtheta accumulated over all jobs of the network
//
// One CTA of 256 threads owns a tile of 128 jobs at a time.  Job t is TMEM lane t; it is served
// by two threads, warps w and w + 4 (w = t / 32), which take features [0, 32) and [32, 64).
// Per hidden-hidden layer the product [128 jobs x 64] x [64 x 64] is one tcgen05.mma group
// (M = 128, N = 64, eight K = 8 steps) whose A operand (the activations, job-major) sits in
// TMEM and whose B operand (the weights) sits in shared memory.  The bias, tanh and the
// (1 - h^2) factors run on the FP32 pipe, thread per job, on values read with tcgen05.ld.
//
// Weight gradients are products over the jobs of the tile (K = 128): dW_l^T = delta_l^T h_{l-1}
// with M = 64 output features and N = 72 = 64 inputs + a constant-one row (the bias gradient)
// + 7 zero rows.  Both operands are feature-major copies in shared memory, written thread per
// job (one column each) with a 144-byte K-chunk stride that keeps those stores bank-conflict
// free.  All gradients accumulate in TMEM over every tile the CTA processes and are read out
// once, as the CTA's partial gradient row.  The input layer (3 -> 64) and the output layer
// (64 -> 1) run on the FP32 pipe in the forward; their gradients come from two small MMAs
// whose 8-row operand ([x, y, z, 1] or [g]) is replicated over M = 64 (row-group stride 0).
//
// Operands are rounded to TF32 (cvt.rna) when written; the accumulators are FP32.  Every wait
// on an mbarrier is bounded: on a timeout the CTA records Ctl::engine_error (the loss and the
// gradient then come out NaN), stops at the next barrier, waits (bounded) for the MMAs it has in
// flight and frees its TMEM.

#include <atomic>

#include "residual_common.cuh"

namespace dips {
namespace tcnet {

constexpr int W = 64, L = 4;
constexpr int kNetParams = 3 * W + W + (L - 1) * (W * W + W) + W + 1;  // 12801
constexpr int kParams = 2 * kNetParams;
constexpr int kOut = 4 * W + (L - 1) * (W * W + W);  // offset of the output weights in a network
__host__ __device__ constexpr int layer_off(int l) { return l == 0 ? 0 : 4 * W + (l - 1) * (W * W + W); }

constexpr int kThreads = 256;  // forward kernel: two threads per job, features [0, 32) and [32, 64)
constexpr int kTile = 128;
constexpr int kHalf = 32;
// adjoint kernel: four threads per job (warps w, w + 4, w + 8, w + 12), 16 features each, so that
// 16 warps share the SM and hide each other's tcgen05.ld, mbarrier and MUFU latencies
constexpr int kAdjThreads = 512;
constexpr int kAQ = 16;
constexpr int kGrid = kTileGrid;
// polls of an mbarrier wait before the CTA gives up (kernel argument; dips_tc_set_wait_limit
// changes it for tests of the timeout path); the wait for MMAs still in flight after a give-up
// always uses kWaitLimit
constexpr uint32_t kWaitLimit = 1u << 24;

// ---- shared-memory operand layouts ---------------------------------------------------------
// weights (64 x 64, K-major): core matrices of 8 rows x 16 B, K-chunks 128 B apart, row groups
// 2048 B apart
constexpr int kWBytes = W * W * 4;
__device__ __forceinline__ int woff(int r, int k) { return (r >> 3) * 2048 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4; }
// feature-major job matrices (rows = features, K = the tile's 128 jobs): K-chunks 144 B apart
constexpr int kLboJ = 144, kSboJ = 32 * kLboJ;  // 4608
constexpr int kFM72 = 9 * kSboJ;                // 72 rows
constexpr int kFM8 = kSboJ;                     // 8 rows
__device__ __forceinline__ int foff(int r, int j) { return (r >> 3) * kSboJ + (j >> 2) * kLboJ + (r & 7) * 16 + (j & 3) * 4; }

// TMEM columns: D (results of the job-major products), A (job-major activations / deltas), then
// the weight-gradient accumulators of the adjoint
constexpr uint32_t cD = 0, cA = 64, cW2 = 128, cW3 = 200, cW4 = 272, cW1 = 344, cWO = 352;
constexpr uint32_t kFwdCols = 128, kAdjCols = 512;
constexpr int kFwdCtasPerSm = 2;  // 2 x 256 threads at <= 128 registers

// small tables (floats) shared by both kernels: W1[3][64], b[4][64], wo[64], bo
constexpr int kSmallFloats = 3 * W + 4 * W + W + 4;

// ---- PTX wrappers ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the sm_100 family; no swizzle, base offset 0
  return d;
}

// instruction descriptor: FP32 accumulator, TF32 A and B, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_ss(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
               ::"r"(d), "l"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void mma_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n"
               ::"r"(d), "r"(a), "l"(b), "r"(id), "r"(acc));
}
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar)));
}
__device__ __forceinline__ bool wait_phase(uint64_t* bar, uint32_t phase, uint32_t limit) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < limit && !done; ++it)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(saddr(bar)), "r"(phase));
  return done != 0;
}
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tld16(uint32_t ta, float* v) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}
__device__ __forceinline__ void tld8(uint32_t ta, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(ta));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}
__device__ __forceinline__ void tst16(uint32_t ta, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
               ::"r"(ta), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
                 "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
                 "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
                 "r"(__float_as_uint(v[15]))
               : "memory");
}
__device__ __forceinline__ void tst_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ float tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// tanh(z) = 1 - 2/(1 + e^{2z}) with the hardware exp2 and reciprocal approximations
__device__ __forceinline__ float tanh_f(float z) {
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(z * 2.8853900817779268f));
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
  return fmaf(-2.0f, r, 1.0f);
}

// ---- CTA set-up -------------------------------------------------------------------------------
// forward operands WF[l-2][n = out][k = in] = W_l[in][out]; backward operands WB[l-2][n = in][k = out]
template <bool BWD>
__device__ void load_weights(const float* __restrict__ net, unsigned char* wf, unsigned char* wb, float* small) {
  for (int e = threadIdx.x; e < 3 * W * W; e += blockDim.x) {
    const int l = e / (W * W), r = e % (W * W), i = r / W, o = r % W;
    const float v = tf32(net[layer_off(l + 1) + r]);
    *reinterpret_cast<float*>(wf + l * kWBytes + woff(o, i)) = v;
    if (BWD) *reinterpret_cast<float*>(wb + l * kWBytes + woff(i, o)) = v;
  }
  for (int e = threadIdx.x; e < 3 * W; e += blockDim.x) small[e] = net[e];  // W1
  for (int e = threadIdx.x; e < 4 * W; e += blockDim.x) {
    const int l = e / W, o = e % W;
    small[3 * W + e] = net[layer_off(l) + (l == 0 ? 3 : W) * W + o];  // b_l
  }
  for (int e = threadIdx.x; e < W + 1; e += blockDim.x) small[7 * W + e] = net[kOut + e];  // wo, bo
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t cols) {
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols));
}

// After a give-up (s_abort): every thread left its loop at the barrier before the next issue,
// so at most one commit group is in flight, the one of the wait that gave up, whose parity is
// phase ^ 1 (each wait flips phase).  Thread 0 waits for it (bounded, kWaitLimit polls; a
// completed phase returns at once) before the CTA frees its TMEM.
__device__ __forceinline__ void drain_after_abort(uint64_t* bar, uint32_t phase, const int& s_abort) {
  __syncthreads();
  if (s_abort && threadIdx.x == 0) (void)wait_phase(bar, phase ^ 1u, kWaitLimit);
  __syncthreads();
}

// h1 = tanh(W1^T x + b1) for features [f0, f0 + NQ), on the FP32 pipe
template <int NQ = kHalf>
__device__ __forceinline__ void layer1(const float* small, const float x[3], float* h, int f0) {
#pragma unroll
  for (int o = 0; o < NQ; ++o) {
    float z = small[3 * W + f0 + o];
    z = fmaf(x[0], small[f0 + o], z);
    z = fmaf(x[1], small[W + f0 + o], z);
    z = fmaf(x[2], small[2 * W + f0 + o], z);
    h[o] = tanh_f(z);
  }
}

// this thread's NQ values into its TMEM lane, columns [col, col + NQ), rounded to TF32
template <int NQ = kHalf>
__device__ __forceinline__ void to_tmem(uint32_t lane_base, uint32_t col, const float* v) {
#pragma unroll
  for (int c = 0; c < NQ; c += 16) {
    float t[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) t[q] = tf32(v[c + q]);
    tst16(lane_base + col + c, t);
  }
}
template <int NQ = kHalf>
__device__ __forceinline__ void from_tmem(uint32_t lane_base, uint32_t col, float* v) {
#pragma unroll
  for (int c = 0; c < NQ; c += 16) tld16(lane_base + col + c, v + c);
}
// rows [f0, f0 + NQ) of column t (this thread's job) of a feature-major matrix
template <int NQ = kHalf>
__device__ __forceinline__ void to_fm(unsigned char* m, int t, const float* v, int f0) {
#pragma unroll
  for (int r = 0; r < NQ; ++r) *reinterpret_cast<float*>(m + foff(f0 + r, t)) = tf32(v[r]);
}
__device__ __forceinline__ float fm_at(const unsigned char* m, int r, int t) {
  return *reinterpret_cast<const float*>(m + foff(r, t));
}

// CTA barrier that also orders tcgen05 and generic-proxy shared-memory writes before the
// MMAs issued after it
__device__ __forceinline__ void sync_for_mma() {
  tst_wait();
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
}

// one hidden-hidden forward layer: D = A(TMEM) x WF[l]
// The descriptors of consecutive K steps differ only in the start-address field (bits 0-13,
// the byte address >> 4).  Shared-memory addresses stay below 2^18 bytes, so adding the step
// there cannot carry into the other fields: each group builds one descriptor per operand and
// adds, and the issuing thread (alone while the CTA waits) runs a few instructions per MMA.
__device__ __forceinline__ void issue_fwd(uint32_t tb, const unsigned char* wf_l) {
  const uint64_t b0 = sdesc(saddr(wf_l), 128, 2048);
#pragma unroll
  for (int s = 0; s < W / 8; ++s) mma_ts(tb + cD, tb + cA + 8 * s, b0 + (uint64_t)(16 * s), idesc(128, W), s > 0);
}
// delta GEMM: D = A(TMEM, delta_l job-major) x WB[l]   (W_l delta_l per job)
__device__ __forceinline__ void issue_delta(uint32_t tb, const unsigned char* wb_l) {
  const uint64_t b0 = sdesc(saddr(wb_l), 128, 2048);
#pragma unroll
  for (int s = 0; s < W / 8; ++s) mma_ts(tb + cD, tb + cA + 8 * s, b0 + (uint64_t)(16 * s), idesc(128, W), s > 0);
}
// weight gradient: acc (M = 64 out features, N) += A (feature-major, a_rows rows) x B^T (feature-major, N rows)
__device__ __forceinline__ void issue_dw(uint32_t d, const unsigned char* a, uint32_t a_sbo, const unsigned char* b, int N,
                                         bool accumulate) {
  const uint64_t a0 = sdesc(saddr(a), kLboJ, a_sbo), b0 = sdesc(saddr(b), kLboJ, kSboJ);
  constexpr uint64_t kStep = (2 * kLboJ) >> 4;  // two K-chunks of the 144-byte stride per K = 8 step
#pragma unroll
  for (int s = 0; s < kTile / 8; ++s)
    mma_ss(d, a0 + kStep * s, b0 + kStep * s, idesc(64, N), (accumulate || s > 0) ? 1u : 0u);
}

// ---- forward kernel -------------------------------------------------------------------------
constexpr size_t kFwdSmem = 3 * kWBytes + sizeof(float) * kSmallFloats + 64;

__global__ void __launch_bounds__(kThreads, kFwdCtasPerSm) k_tc_forward(const float* __restrict__ params, int off,
                                                                        Workspace w, int net_p, uint32_t wait_limit) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* wf = sm;
  float* small = reinterpret_cast<float*>(sm + 3 * kWBytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(small + kSmallFloats);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  __shared__ int s_abort;
  __shared__ float s_u[kTile];  // partial output sums of the features [32, 64)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int job = 32 * (warp & 3) + lane, f0 = kHalf * (warp >> 2);
  load_weights<false>(params + off, wf, nullptr, small);
  if (threadIdx.x == 0) {
    s_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  tmem_alloc(slot, kFwdCols);
  sync_for_mma();
  const uint32_t tb = *slot;
  const uint32_t lb = tb + ((uint32_t)(32 * (warp & 3)) << 16);  // this warp's TMEM lane quarter
  const Ctl ctl = *w.ctl;
  const int64_t jbeg = net_p ? ctl.jm_pad : 0, jend = net_p ? ctl.total : ctl.jm;
  const int64_t ntiles = (jend - jbeg + kTile - 1) / kTile;
  uint32_t phase = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t j = jbeg + tile * kTile + job;
    float x[3] = {0.0f, 0.0f, 0.0f};
    if (j < jend) {
      const float4 xv = w.jx[j];
      x[0] = xv.x;
      x[1] = xv.y;
      x[2] = xv.z;
    }
    float h[kHalf];
    layer1(small, x, h, f0);
    for (int l = 0; l < 3; ++l) {
      to_tmem(lb, cA + f0, h);
      sync_for_mma();
      if (s_abort) break;
      if (threadIdx.x == 0) {
        issue_fwd(tb, wf + l * kWBytes);
        commit(bar);
      }
      if (!wait_phase(bar, phase, wait_limit)) {
        s_abort = 1;
        w.ctl->engine_error = 1;
      }
      phase ^= 1;
      fence_after();
      from_tmem(lb, cD + f0, h);
#pragma unroll
      for (int o = 0; o < kHalf; ++o) h[o] = tanh_f(h[o] + small[3 * W + (l + 1) * W + f0 + o]);
    }
    // (an abort is acted on at the next barrier, where every thread sees the flag)
    float u = 0.0f;
#pragma unroll
    for (int o = 0; o < kHalf; ++o) u = fmaf(small[7 * W + f0 + o], h[o], u);
    if (f0) s_u[job] = u;
    __syncthreads();
    if (!f0 && j < jend) w.ju[j] = u + s_u[job] + small[8 * W];
  }
  drain_after_abort(bar, phase, s_abort);
  fence_before();
  __syncthreads();
  fence_after();
  tmem_free(tb, kFwdCols);
}

// ---- adjoint kernel --------------------------------------------------------------------------
constexpr int kOffWF = 0;
constexpr int kOffWB = kOffWF + 3 * kWBytes;
constexpr int kOffH2 = kOffWB + 3 * kWBytes;
constexpr int kOffH3 = kOffH2 + kFM72;
constexpr int kOffZ = kOffH3 + kFM72;
constexpr int kOffGX = kOffZ + kFM72;
constexpr int kOffSmall = kOffGX + kFM8;
constexpr size_t kAdjSmem = kOffSmall + sizeof(float) * kSmallFloats + 64;

// Bulk points (7 stencil jobs of this network) come in tiles of 18 points = 126 jobs (lanes 126
// and 127 idle): after the forward the CTA forms their residuals and dL/du in shared memory, so
// that their network values need no separate forward launch.  General jobs follow in tiles of
// 128 with dL/du from the general residual.  BWD = false: bulk tiles only, forward, residual
// and loss (the forward-only path); BWD = true: the backward of every tile as well.
constexpr int kBulkPts = 18;
static_assert(kBulkPts <= 32, "the bulk residuals of a tile are formed by warp 0");

template <bool BWD>
__global__ void __launch_bounds__(kAdjThreads, 1) k_tc_adjoint(const float* __restrict__ params, int off, Workspace w,
                                                            int net_p, PtsH ph, float* __restrict__ residual_out,
                                                            uint32_t wait_limit) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* wf = sm + kOffWF;
  unsigned char* wb = sm + kOffWB;
  unsigned char* H2 = sm + kOffH2;  // h2^T, then (backward) nothing new
  unsigned char* H3 = sm + kOffH3;  // h3^T, then h1^T (recomputed)
  unsigned char* Z = sm + kOffZ;    // h4^T, then delta_l^T
  unsigned char* GX = sm + kOffGX;  // [g, 0..] then [x, y, z, 1, 0..]
  float* small = reinterpret_cast<float*>(sm + kOffSmall);
  uint64_t* bar = reinterpret_cast<uint64_t*>(small + kSmallFloats);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  int& s_abort = *reinterpret_cast<int*>(slot + 1);  // in the dynamic block's slack (static shared memory is full)
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int job = 32 * (warp & 3) + lane, part = warp >> 2, f0 = kAQ * part;
  load_weights<true>(params + off, wf, wb, small);
  // constant rows: 64 = ones (the bias input) and 65..71 = 0 in the 72-row matrices; rows 1..7
  // of GX and rows 64..71 of the 72-row matrices are never rewritten
  for (int e = t; e < 8 * kTile; e += blockDim.x) {
    const int r = 64 + e / kTile, jj = e % kTile;
    const float v = r == 64 ? 1.0f : 0.0f;
    *reinterpret_cast<float*>(H2 + foff(r, jj)) = v;
    *reinterpret_cast<float*>(H3 + foff(r, jj)) = v;
    *reinterpret_cast<float*>(Z + foff(r, jj)) = v;
    *reinterpret_cast<float*>(GX + foff(e / kTile, jj)) = 0.0f;
  }
  if (t == 0) {
    s_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  tmem_alloc(slot, kAdjCols);
  sync_for_mma();
  const uint32_t tb = *slot;
  const uint32_t lb = tb + ((uint32_t)(32 * (warp & 3)) << 16);
  const Ctl ctl = *w.ctl;
  const int64_t jbeg = net_p ? ctl.jm_pad : 0, jend = net_p ? ctl.total : ctl.jm;
  const int64_t nb = net_p ? ctl.nbp : ctl.nbm;
  const int64_t nbt = (nb + kBulkPts - 1) / kBulkPts;
  const int64_t ntiles = nbt + (BWD ? (jend - jbeg + kTile - 1) / kTile : 0);
  const float* recs = w.brec + (size_t)(net_p ? w.B : 0) * kRecFloats;
  const float hh[3] = {ph.h[0], ph.h[1], ph.h[2]};
  const float Bf = (float)w.B;
  __shared__ float s_part[2][kTile], s_au[kTile], s_g[kTile];
  // the fourth quarter's partial output sums use s_g, which is written only after they are read
  // (static + dynamic shared memory must stay within the 227 KB a CTA may have)
  float* const s_part3 = s_g;
  double lsum = 0.0;
  uint32_t phase = 0;
  bool first = true;
  auto wait = [&]() {
    if (!wait_phase(bar, phase, wait_limit)) {
      s_abort = 1;
      w.ctl->engine_error = 1;
    }
    phase ^= 1;
    fence_after();
  };
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const bool bulk = tile < nbt;
    float x[3] = {0.0f, 0.0f, 0.0f};
    float g = 0.0f;
    const int pl = job / kStencil, sj = job - kStencil * pl;  // bulk tile: point and stencil point
    const int64_t pidx = tile * kBulkPts + pl;
    const bool bvalid = bulk && job < kBulkPts * kStencil && pidx < nb;
    // threads 0..17 of a bulk tile: their point's record, loaded now so that the loads run under
    // the forward's MMAs rather than between the barriers of the residual step
    const int64_t qpt = tile * kBulkPts + t;
    const bool rvalid = bulk && t < kBulkPts && qpt < nb;
    float r_lhs0 = 0.0f, r_diag = 1.0f, r_rod = 0.0f, r_P = 1.0f, r_A[kStencil];
    int32_t rslot = 0;
#pragma unroll
    for (int k = 0; k < kStencil; ++k) r_A[k] = 0.0f;
    if (rvalid) {
      const float* r = recs + qpt * kRecFloats;
      r_lhs0 = r[kRecLhs0];
      r_diag = r[kRecDiag];
      r_rod = r[kRecRod];
      rslot = __float_as_int(r[kRecSlot]);
#pragma unroll
      for (int k = 0; k < kStencil; ++k) r_A[k] = r[kRecA + k];
      if (w.pre_P) r_P = w.pre_P[rslot];
    }
    if (bulk) {
      if (bvalid) {
        const float* r = recs + pidx * kRecFloats;
        const float p[3] = {r[kRecP], r[kRecP + 1], r[kRecP + 2]};
        stencil_point(p, hh, sj, x);
      }
    } else {
      const int64_t j = jbeg + (tile - nbt) * kTile + job;
      if (j < jend) {
        const float4 xv = w.jx[j];
        x[0] = xv.x;
        x[1] = xv.y;
        x[2] = xv.z;
        g = w.jg[j];
      }
    }
    // ---- forward, keeping h2^T and h3^T
    float h[kAQ];
    layer1<kAQ>(small, x, h, f0);
    to_tmem<kAQ>(lb, cA + f0, h);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_fwd(tb, wf);
      commit(bar);
    }
    wait();
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] = tanh_f(h[o] + small[4 * W + f0 + o]);
    to_tmem<kAQ>(lb, cA + f0, h);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_fwd(tb, wf + kWBytes);
      commit(bar);
    }
    // h2^T for dW3 while the layer-3 MMA runs (its last reader, the previous tile's dW3, is done)
    to_fm<kAQ>(H2, job, h, f0);
    wait();
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] = tanh_f(h[o] + small[5 * W + f0 + o]);
    to_tmem<kAQ>(lb, cA + f0, h);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_fwd(tb, wf + 2 * kWBytes);
      commit(bar);
    }
    to_fm<kAQ>(H3, job, h, f0);  // h3^T for dW4, likewise under the layer-4 MMA
    wait();
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] = tanh_f(h[o] + small[6 * W + f0 + o]);  // h4
    if (bulk) {
      // u of every job, A_j u_j, the residual of each of the tile's points, then dL/du
      float u = 0.0f;
#pragma unroll
      for (int o = 0; o < kAQ; ++o) u = fmaf(small[7 * W + f0 + o], h[o], u);
      if (part == 0) s_au[job] = u;
      if (part == 1) s_part[0][job] = u;
      if (part == 2) s_part[1][job] = u;
      if (part == 3) s_part3[job] = u;
      __syncthreads();
      if (t < kBulkPts) {
        if (rvalid) {
          // u of the point's 7 jobs from the four partial sums, then lhs0 + sum A_j u_j (each
          // product rounded before it is added)
          float lhs = r_lhs0;
#pragma unroll
          for (int k = 0; k < kStencil; ++k) {
            const int jj = kStencil * t + k;
            const float uj = ((s_au[jj] + s_part[0][jj]) + (s_part[1][jj] + s_part3[jj])) + small[8 * W];
            lhs += __fmul_rn(r_A[k], uj);
          }
          const float qv = lhs / r_diag;
          const float r0 = nan_to_num(qv) - r_rod;
          const float rr = r_P * r0;  // learned preconditioner (1 without it)
          if (w.pre_P) w.pre_r0[rslot] = r0;
          const float gc = isfinite(qv) ? (rr / Bf) * r_P / r_diag : 0.0f;
          lsum += 0.5 * (double)rr * (double)rr;
          if (residual_out) residual_out[rslot] = rr;
#pragma unroll
          for (int k = 0; k < kStencil; ++k) s_g[kStencil * t + k] = gc * r_A[k];
        } else {
#pragma unroll
          for (int k = 0; k < kStencil; ++k) s_g[kStencil * t + k] = 0.0f;
        }
      }
      // h4^T for dWo while warp 0 forms the residuals (Z's last reader, the previous tile's dW1,
      // is done)
      if (BWD) to_fm<kAQ>(Z, job, h, f0);
      __syncthreads();
      g = bvalid ? s_g[job] : 0.0f;
    }
    if (!BWD) continue;
    // ---- output layer: dWo, dbo = sum_j g_j [h4, 1]  (A = [g] replicated, B = h4^T with its ones row)
    if (!bulk) to_fm<kAQ>(Z, job, h, f0);
    if (!f0) {
      *reinterpret_cast<float*>(GX + foff(0, job)) = tf32(g);
      *reinterpret_cast<float*>(GX + foff(1, job)) = 0.0f;
      *reinterpret_cast<float*>(GX + foff(2, job)) = 0.0f;
      *reinterpret_cast<float*>(GX + foff(3, job)) = 0.0f;
    }
    sync_for_mma();
    if (s_abort) break;
    // Work that does not depend on an MMA in flight runs while it runs (between the issue and
    // the wait): the next delta where it needs no product, the factors read from H2/H3 (which
    // the MMA may read at the same time), and the rewrite of a buffer that the MMAs completed
    // at an earlier wait (GX after dWo, H3 after dW4).
    if (t == 0) {
      issue_dw(tb + cWO, GX, 0, Z, 72, !first);
      commit(bar);
    }
    // delta4 = g wo (1 - h4^2) into TMEM A (the dWo MMA reads only shared memory)
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] = g * small[7 * W + f0 + o] * fmaf(-h[o], h[o], 1.0f);
    to_tmem<kAQ>(lb, cA + f0, h);
    wait();
    to_fm<kAQ>(Z, job, h, f0);  // Z held h4^T for dWo until the wait
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_dw(tb + cW4, Z, kSboJ, H3, 72, !first);  // dW4^T | db4
      issue_delta(tb, wb + 2 * kWBytes);             // W4 delta4
      commit(bar);
    }
    float fac[kAQ];
#pragma unroll
    for (int o = 0; o < kAQ; ++o) {
      const float a = fm_at(H3, f0 + o, job);
      fac[o] = fmaf(-a, a, 1.0f);
    }
    if (!f0) {  // [x, y, z, 1] for dW1 (GX's last reader, dWo, completed at the previous wait)
      *reinterpret_cast<float*>(GX + foff(0, job)) = tf32(x[0]);
      *reinterpret_cast<float*>(GX + foff(1, job)) = tf32(x[1]);
      *reinterpret_cast<float*>(GX + foff(2, job)) = tf32(x[2]);
      *reinterpret_cast<float*>(GX + foff(3, job)) = 1.0f;
    }
    wait();
    // delta3 = (W4 delta4) (1 - h3^2)
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] *= fac[o];
    to_tmem<kAQ>(lb, cA + f0, h);
    to_fm<kAQ>(Z, job, h, f0);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_dw(tb + cW3, Z, kSboJ, H2, 72, !first);  // dW3^T | db3
      issue_delta(tb, wb + kWBytes);                 // W3 delta3
      commit(bar);
    }
#pragma unroll
    for (int o = 0; o < kAQ; ++o) {
      const float a = fm_at(H2, f0 + o, job);
      fac[o] = fmaf(-a, a, 1.0f);
    }
    // h1 recomputed into H3 (its last reader, dW4, completed at the previous wait)
    float h1[kAQ];
    layer1<kAQ>(small, x, h1, f0);
    to_fm<kAQ>(H3, job, h1, f0);
    wait();
    // delta2 = (W3 delta3) (1 - h2^2)
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] *= fac[o];
    to_tmem<kAQ>(lb, cA + f0, h);
    to_fm<kAQ>(Z, job, h, f0);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_dw(tb + cW2, Z, kSboJ, H3, 72, !first);  // dW2^T | db2
      issue_delta(tb, wb);                           // W2 delta2
      commit(bar);
    }
#pragma unroll
    for (int o = 0; o < kAQ; ++o) fac[o] = fmaf(-h1[o], h1[o], 1.0f);
    {  // the next tile's inputs into L2 (its first loads then wait on L2, not DRAM)
      const int64_t nt = tile + gridDim.x;
      if (nt < nbt) {
        const int64_t q = nt * kBulkPts + t;
        if (t < kBulkPts && q < nb) prefetch_l2(recs + q * kRecFloats);
      } else if (nt < ntiles) {
        const int64_t j = jbeg + (nt - nbt) * kTile + (t & (kTile - 1));
        if (j < jend) {
          if (t < kTile) prefetch_l2(w.jx + j);
          else if (t < 2 * kTile) prefetch_l2(w.jg + j);
        }
      }
    }
    wait();
    // delta1 = (W2 delta2) (1 - h1^2); dW1^T | db1 = delta1^T [x, y, z, 1]
    from_tmem<kAQ>(lb, cD + f0, h);
#pragma unroll
    for (int o = 0; o < kAQ; ++o) h[o] *= fac[o];
    to_fm<kAQ>(Z, job, h, f0);
    sync_for_mma();
    if (s_abort) break;
    if (t == 0) {
      issue_dw(tb + cW1, Z, kSboJ, GX, 8, !first);
      commit(bar);
    }
    wait();
    first = false;
  }
  drain_after_abort(bar, phase, s_abort);
  // ---- loss partial of the bulk points of this CTA (only threads 0..17, in warp 0, hold any)
  if (warp == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (t == 0) {
      w.floss[net_p * kLossSlots + blockIdx.x] = lsum;
      if (blockIdx.x == 0) w.ctl->floss_n[net_p] = gridDim.x;
    }
  }
  __syncthreads();
  if (!BWD) {
    fence_before();
    __syncthreads();
    fence_after();
    tmem_free(tb, kAdjCols);
    return;
  }
  // ---- partial gradient row of this CTA (columns of this network)
  float* row = w.partials + (size_t)blockIdx.x * w.n_params + off;
  if (t == 0 && blockIdx.x == 0) w.ctl->grad_rows[net_p] = gridDim.x;
  fence_before();
  __syncthreads();
  fence_after();
  if (first || s_abort) {
    for (int i = t; i < kNetParams; i += blockDim.x) row[i] = 0.0f;
  } else if (warp < 4) {
    // M = 64 accumulators: row o sits in lane 32*(o/16) + o%16; lanes 16..31 of each warp idle
    const int o = 16 * warp + lane;
    const bool have = lane < 16;
    float v[16];
    const uint32_t regions[3] = {cW2, cW3, cW4};
    for (int q = 0; q < 3; ++q) {
      const int lo = layer_off(q + 1);
      for (int c = 0; c < 64; c += 16) {
        tld16(lb + regions[q] + c, v);
        if (have)
          for (int i = 0; i < 16; ++i) row[lo + (c + i) * W + o] = v[i];
      }
      tld8(lb + regions[q] + 64, v);
      if (have) row[lo + W * W + o] = v[0];
    }
    tld8(lb + cW1, v);
    if (have) {
      row[0 * W + o] = v[0];
      row[1 * W + o] = v[1];
      row[2 * W + o] = v[2];
      row[3 * W + o] = v[3];
    }
    for (int c = 0; c < 64; c += 16) {
      tld16(lb + cWO + c, v);
      if (t == 0)
        for (int i = 0; i < 16; ++i) row[kOut + c + i] = v[i];
    }
    tld8(lb + cWO + 64, v);
    if (t == 0) row[kOut + W] = v[0];
  }
  fence_before();
  __syncthreads();
  fence_after();
  tmem_free(tb, kAdjCols);
}

// ---- u and grad u at points (evaluation; FP32 pipe, one thread per point) --------------------
__global__ void __launch_bounds__(128) k_tc_eval(const float* __restrict__ params, int off, const float* __restrict__ pts,
                                                 const float* __restrict__ phi, int64_t n, float* __restrict__ u_out,
                                                 float* __restrict__ g_out, int net_p) {
  const float* net = params + off;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if ((phi[i] >= 0.0f) != (net_p != 0)) continue;
    const float x[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    float act[L][W];
    for (int o = 0; o < W; ++o) {
      float z = net[3 * W + o];
      for (int c = 0; c < 3; ++c) z = fmaf(x[c], net[c * W + o], z);
      act[0][o] = tanhf(z);
    }
    for (int l = 1; l < L; ++l) {
      const float* Wl = net + layer_off(l);
      for (int o = 0; o < W; ++o) {
        float z = Wl[W * W + o];
        for (int k = 0; k < W; ++k) z = fmaf(act[l - 1][k], Wl[k * W + o], z);
        act[l][o] = tanhf(z);
      }
    }
    float u = net[kOut + W];
    for (int k = 0; k < W; ++k) u = fmaf(act[L - 1][k], net[kOut + k], u);
    u_out[i] = u;
    if (g_out) {
      float d[W], dn[W];
      for (int k = 0; k < W; ++k) d[k] = net[kOut + k] * (1.0f - act[L - 1][k] * act[L - 1][k]);
      for (int l = L - 1; l >= 1; --l) {
        const float* Wl = net + layer_off(l);
        for (int k = 0; k < W; ++k) {
          float s = 0.0f;
          for (int o = 0; o < W; ++o) s = fmaf(Wl[k * W + o], d[o], s);
          dn[k] = s * (1.0f - act[l - 1][k] * act[l - 1][k]);
        }
        for (int k = 0; k < W; ++k) d[k] = dn[k];
      }
      for (int c = 0; c < 3; ++c) {
        float s = 0.0f;
        for (int o = 0; o < W; ++o) s = fmaf(net[c * W + o], d[o], s);
        g_out[3 * i + c] = s;
      }
    }
  }
}

// ---- ArchOps ------------------------------------------------------------------------------------
// The weights stay in global memory (25,602 floats do not fit the constant bank); every call
// passes them through load_params, which records the pointer for the launches that follow on
// the calling thread.
thread_local const float* t_params = nullptr;
std::atomic<uint32_t> g_wait_limit{kWaitLimit};

static int load_params(const float* params, int, cudaStream_t) {
  t_params = params;
  return DIPS_OK;
}

static int set_smem(const void* fn, size_t bytes, bool* done) {
  if (*done) return DIPS_OK;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(tcgen05 kernel smem)");
  *done = true;
  return DIPS_OK;
}

static int job_forward(const PtsH&, const int32_t*, const Workspace& w, const Marks* mk, cudaStream_t s) {
  static bool attr = false;
  int st = set_smem((const void*)k_tc_forward, kFwdSmem, &attr);
  if (st) return st;
  const uint32_t lim = g_wait_limit.load();
  k_tc_forward<<<kGrid * kFwdCtasPerSm, kThreads, kFwdSmem, s>>>(t_params, 0, w, 0, lim);
  mark(mk, kMarkFwdM, s);
  k_tc_forward<<<kGrid * kFwdCtasPerSm, kThreads, kFwdSmem, s>>>(t_params, kNetParams, w, 1, lim);
  mark(mk, kMarkFwdP, s);
  DIPS_CHECK_LAUNCH("tcgen05 forward");
  return DIPS_OK;
}

// the backward of every job is part of the bulk launch
static int job_adjoint(const PtsH&, const int32_t*, const Workspace&, const Marks* mk, cudaStream_t s) {
  mark(mk, kMarkAdjM, s);
  mark(mk, kMarkAdjP, s);
  return DIPS_OK;
}

template <bool BWD>
static int adjoint_pair(const PtsH& ph, const Workspace& w, float* residual_out, const Marks* mk, cudaStream_t s) {
  static bool attr = false;
  int st = set_smem((const void*)k_tc_adjoint<BWD>, kAdjSmem, &attr);
  if (st) return st;
  const uint32_t lim = g_wait_limit.load();
  k_tc_adjoint<BWD><<<kGrid, kAdjThreads, kAdjSmem, s>>>(t_params, 0, w, 0, ph, residual_out, lim);
  mark(mk, kMarkFusedM, s);
  k_tc_adjoint<BWD><<<kGrid, kAdjThreads, kAdjSmem, s>>>(t_params, kNetParams, w, 1, ph, residual_out, lim);
  mark(mk, kMarkFusedP, s);
  DIPS_CHECK_LAUNCH("tcgen05 bulk / adjoint");
  return DIPS_OK;
}

// bulk points' forward, residual and loss (and, with bwd, the backward of every job)
static int bulk_fused(const PtsH& ph, const int32_t*, const Workspace& w, const dips_records_t&, float* residual_out,
                      bool bwd, const Marks* mk, cudaStream_t s) {
  return bwd ? adjoint_pair<true>(ph, w, residual_out, mk, s) : adjoint_pair<false>(ph, w, residual_out, mk, s);
}

static int mlp_eval(const float*, const float* pts, const float* phi, int64_t n, float* u, float* g, cudaStream_t s) {
  int64_t grid = (n + 127) / 128;
  if (grid > 152 * 16) grid = 152 * 16;
  k_tc_eval<<<(int)grid, 128, 0, s>>>(t_params, 0, pts, phi, n, u, g, 0);
  k_tc_eval<<<(int)grid, 128, 0, s>>>(t_params, kNetParams, pts, phi, n, u, g, 1);
  DIPS_CHECK_LAUNCH("4x64 evaluation");
  return DIPS_OK;
}

}  // namespace tcnet

// Polls of the tensor-core engine's mbarrier waits (default 2^24), for tests of the timeout
// path; returns the previous value.  Affects launches made after the call, from any thread.
extern "C" uint32_t dips_tc_set_wait_limit(uint32_t polls) { return tcnet::g_wait_limit.exchange(polls); }

const ArchOps* arch_ops_4_64_4_64() {
  static const ArchOps ops = {4, 64, 4, 64, tcnet::kParams, 1, tcnet::load_params, tcnet::job_forward,
                              tcnet::job_adjoint, tcnet::bulk_fused, tcnet::mlp_eval, nullptr, nullptr,
                              nullptr};
  return &ops;
}

}  // namespace dips
