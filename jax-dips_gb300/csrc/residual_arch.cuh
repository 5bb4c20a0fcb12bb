// Per-network-shape kernels of the residual path (included once per shape by the
// residual_a*.cu translation units, which define DIPS_LM, DIPS_WM, DIPS_LP, DIPS_WP).
//
// Everything runs on the FP32 pipe.  The shapes 3x32 and 2x16 run every launch of the step, the
// multi-instance step and the evaluation on the register-blocked tile engine (mlp_tile.cuh),
// which reads the weights from the parameter buffer.  The other shapes use the kernels below;
// each network (u- and u+) gets its own launches, so a kernel holds one network's fully
// unrolled code:
//   forward  one thread per job; the weights are broadcast shared-memory operands
//   adjoint  one thread per job recomputes the activations and stages them in the warp's
//            shared-memory tile; the output gradients propagate thread-per-job (again with
//            broadcast shared-memory weights) and overwrite the tile in place; each layer's dW is a warp
//            GEMM over the tile's 32 jobs (lane = output unit, broadcast float4 rows)
//            accumulated with shared-memory atomics into one CTA accumulator, written out
//            as one partial gradient row per CTA.
// Reference: DoubleMLP (nn/mlp/MLP.py:93-139), value_and_grad in Trainer.update
// (solvers/poisson/trainer.py:783-789).

#include <math.h>

#include <atomic>
#include <mutex>

#include "residual_common.cuh"

namespace dips {
namespace DIPS_NS {

// The weights of both networks, copied from the call's parameter buffer (Workspace::params, or
// the evaluation's params argument) into shared memory by every kernel that reads them, before
// anything else (load_weights).  Two copies: forward operands at 0 and backward operands at
// kParams, the offsets the device functions below index.  Each launch reads its own call's
// parameters, so calls on different streams or threads share no state.
constexpr int kArchParams = (3 * DIPS_WM + DIPS_WM + (DIPS_LM - 1) * (DIPS_WM * DIPS_WM + DIPS_WM) + DIPS_WM + 1) +
                            (3 * DIPS_WP + DIPS_WP + (DIPS_LP - 1) * (DIPS_WP * DIPS_WP + DIPS_WP) + DIPS_WP + 1);
static __shared__ float c_w[2 * kArchParams];

__device__ __forceinline__ void load_weights(const float* __restrict__ params) {
  for (int i = threadIdx.x; i < kArchParams; i += blockDim.x) {
    const float v = __ldg(params + i);
    c_w[i] = v;
    c_w[kArchParams + i] = v;
  }
  __syncthreads();
}

constexpr int kThreads = kAdjThreads;
constexpr int kWarps = kThreads / 32;

// tanh: 1 - 2/(1 + e^{2x}) with the hardware exp2 and reciprocal approximations (relative
// error <= 2^-22 each); absolute error below 3e-7, the size of the FP32 rounding of the
// activations themselves.  Against the oracle's tanh it moves the loss by < 1e-7 and the
// gradient by < 3e-6 relative (measured on the parity cases), and it costs three FMA-pipe
// and two MUFU instructions.
__device__ __forceinline__ float act_tanh(float x) {
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(x * 2.8853900817779268f));  // e^{2x}
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
  return fmaf(-2.0f, r, 1.0f);
}

// ----------------------------------------------------------------------------------------
// network shapes and parameter offsets (flat layout documented in dips.h)
// ----------------------------------------------------------------------------------------
template <int L, int W>
struct Net {
  static constexpr int kL = L;
  static constexpr int kW = W;
  static constexpr int kParams = 3 * W + W + (L - 1) * (W * W + W) + W + 1;
  static constexpr int kOut = 4 * W + (L - 1) * (W * W + W);
  __host__ __device__ static constexpr int layer_off(int l) { return l == 0 ? 0 : 4 * W + (l - 1) * (W * W + W); }
  // shared-memory tile, one row per job: width-32 rows are 32 floats with their eight float4
  // chunks XOR-swizzled by the row index (conflict-free row stores and broadcast chunk
  // loads); other widths use an unswizzled stride of W rounded up to 4, plus 4
  static constexpr bool kSwz = (W == 32);
  static constexpr int kRow = kSwz ? 32 : (W + 3) / 4 * 4 + 4;
  static constexpr int kTileFloats = 32 * 4 + L * 32 * kRow + 32;  // x, activations / deltas, g
  // offset of float4 chunk c of row e
  __device__ static __forceinline__ int chunk(int e, int c) { return kSwz ? e * 32 + ((c ^ (e & 7)) << 2) : e * kRow + 4 * c; }
  // offset of element i of row e
  __device__ static __forceinline__ int elem(int e, int i) { return chunk(e, i >> 2) + (i & 3); }
};

template <int LM, int WM, int LP, int WP>
struct Arch {
  using M = Net<LM, WM>;
  using P = Net<LP, WP>;
  static constexpr int kOffP = M::kParams;
  static constexpr int kParams = M::kParams + P::kParams;
};

#include "mlp_tile.cuh"

// forward, activations discarded
template <class N, int OFF>
__device__ __forceinline__ float net_forward(const float x[3]) {
  constexpr int W = N::kW, L = N::kL;
  float h[W];
#pragma unroll
  for (int o = 0; o < W; ++o) {
    float z = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) z = fmaf(x[i], c_w[OFF + i * W + o], z);
    h[o] = act_tanh(z + c_w[OFF + 3 * W + o]);
  }
#pragma unroll
  for (int l = 1; l < L; ++l) {
    const int off = OFF + N::layer_off(l);
    float t[W];
#pragma unroll
    for (int o = 0; o < W; ++o) t[o] = 0.0f;
#pragma unroll
    for (int i = 0; i < W; ++i)
#pragma unroll
      for (int o = 0; o < W; ++o) t[o] = fmaf(h[i], c_w[off + i * W + o], t[o]);
#pragma unroll
    for (int o = 0; o < W; ++o) h[o] = act_tanh(t[o] + c_w[off + W * W + o]);
  }
  float u = 0.0f;
#pragma unroll
  for (int i = 0; i < W; ++i) u = fmaf(h[i], c_w[OFF + N::kOut + i], u);
  return u + c_w[OFF + N::kOut + W];
}

// row e of a tile buffer (layout of network N)
template <class N>
__device__ __forceinline__ void store_row(float* buf, int e, const float* v) {
  constexpr int W = N::kW;
  if constexpr (W % 4 == 0) {
#pragma unroll
    for (int c = 0; c < W / 4; ++c)
      *reinterpret_cast<float4*>(buf + N::chunk(e, c)) = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) buf[N::elem(e, i)] = v[i];
  }
}

template <class N>
__device__ __forceinline__ void load_row(const float* buf, int e, float* v) {
  constexpr int W = N::kW;
  if constexpr (W % 4 == 0) {
#pragma unroll
    for (int c = 0; c < W / 4; ++c) {
      const float4 q = *reinterpret_cast<const float4*>(buf + N::chunk(e, c));
      v[4 * c] = q.x;
      v[4 * c + 1] = q.y;
      v[4 * c + 2] = q.z;
      v[4 * c + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] = buf[N::elem(e, i)];
  }
}

// forward of one job, staging x and every hidden activation in the warp tile row `lane`;
// returns the last hidden activation in h.
template <class N, int OFF>
__device__ __forceinline__ void net_forward_stage(const float x[3], float* X, float* B, int lane, float h[N::kW]) {
  constexpr int W = N::kW, L = N::kL;
  *reinterpret_cast<float4*>(X + 4 * lane) = make_float4(x[0], x[1], x[2], 0.0f);
#pragma unroll
  for (int o = 0; o < W; ++o) {
    float z = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) z = fmaf(x[i], c_w[OFF + i * W + o], z);
    h[o] = act_tanh(z + c_w[OFF + 3 * W + o]);
  }
  store_row<N>(B, lane, h);
#pragma unroll
  for (int l = 1; l < L; ++l) {
    const int off = OFF + N::layer_off(l);
    float t[W];
#pragma unroll
    for (int o = 0; o < W; ++o) t[o] = 0.0f;
#pragma unroll
    for (int i = 0; i < W; ++i)
#pragma unroll
      for (int o = 0; o < W; ++o) t[o] = fmaf(h[i], c_w[off + i * W + o], t[o]);
#pragma unroll
    for (int o = 0; o < W; ++o) h[o] = act_tanh(t[o] + c_w[off + W * W + o]);
    store_row<N>(B + l * 32 * N::kRow, lane, h);
  }
}

// dW[i][o] += sum_e H[e][i] D[e][o], db[o] += sum_e D[e][o] over the tile's 32 rows, H rows
// read as broadcast float4 chunks.  lane = o; when OUT < 32 the lane groups split the rows.
// Shared-memory atomics add the tile's contribution into the CTA accumulator.
// XH = true: H is the x buffer (3 inputs in a float4 per row).
template <class N, int IN, bool XH>
__device__ __forceinline__ void tile_gemm(const float* H, const float* D, float* accW, float* accb, int lane) {
  constexpr int OUT = N::kW;
  constexpr int G = 32 / OUT;
  const int o = lane % OUT, q = lane / OUT;
  if (q >= G) return;
  const int e0 = (q * 32) / G, e1 = ((q + 1) * 32) / G;
  float s[IN];
#pragma unroll
  for (int i = 0; i < IN; ++i) s[i] = 0.0f;
  float sb = 0.0f;
#pragma unroll 4
  for (int e = e0; e < e1; ++e) {
    const float dv = D[N::elem(e, o)];
    sb += dv;
    if constexpr (XH) {
      const float4 v = *reinterpret_cast<const float4*>(H + 4 * e);
      s[0] = fmaf(v.x, dv, s[0]);
      s[1] = fmaf(v.y, dv, s[1]);
      s[2] = fmaf(v.z, dv, s[2]);
    } else if constexpr (IN % 4 == 0) {
#pragma unroll
      for (int c = 0; c < IN / 4; ++c) {
        const float4 v = *reinterpret_cast<const float4*>(H + N::chunk(e, c));
        s[4 * c] = fmaf(v.x, dv, s[4 * c]);
        s[4 * c + 1] = fmaf(v.y, dv, s[4 * c + 1]);
        s[4 * c + 2] = fmaf(v.z, dv, s[4 * c + 2]);
        s[4 * c + 3] = fmaf(v.w, dv, s[4 * c + 3]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < IN; ++i) s[i] = fmaf(H[N::elem(e, i)], dv, s[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < IN; ++i) atomicAdd(accW + i * OUT + o, s[i]);
  atomicAdd(accb + o, sb);
}

// Backward half of a tile whose activations are staged in `tile` (h = last hidden layer of
// this lane's job, g = d loss / d u of this lane's job): output-layer grads, then for each
// hidden layer the delta (thread per job, shared-memory weights) and the dW warp GEMM.
template <class N, int OFF, int BOFF>
__device__ __forceinline__ void net_backward_tile(const float h[N::kW], float g, float* tile, float* acc, int lane) {
  constexpr int W = N::kW, L = N::kL, BUF = 32 * N::kRow;
  float* X = tile;
  float* B = tile + 32 * 4;
  float* gs = B + L * BUF;
  gs[lane] = g;
  __syncwarp();
  // output layer u = sum_i Wo[i] h[i] + bo: dWo[i] += sum_e h[e][i] g[e] (lane = i)
  {
    const float* HL = B + (L - 1) * BUF;
    if (lane < W) {
      float s0 = 0.0f, s1 = 0.0f;
#pragma unroll 8
      for (int e = 0; e < 32; e += 2) {
        s0 = fmaf(HL[N::elem(e, lane)], gs[e], s0);
        s1 = fmaf(HL[N::elem(e + 1, lane)], gs[e + 1], s1);
      }
      atomicAdd(acc + N::kOut + lane, s0 + s1);
    }
    if (lane == 0) {
      float sb = 0.0f;
      for (int e = 0; e < 32; ++e) sb += gs[e];
      atomicAdd(acc + N::kOut + W, sb);
    }
  }
  float d[W];
#pragma unroll
  for (int i = 0; i < W; ++i) d[i] = g * c_w[BOFF + OFF + N::kOut + i] * fmaf(-h[i], h[i], 1.0f);
  __syncwarp();
  store_row<N>(B + (L - 1) * BUF, lane, d);  // the last buffer now holds delta_{L-1}
  __syncwarp();
#pragma unroll
  for (int l = L - 1; l >= 1; --l) {
    const int off = N::layer_off(l);
    float* Hin = B + (l - 1) * BUF;
    // delta_{l-1} = (W_l delta_l) * (1 - a^2) first, so that only it stays live in the GEMM
    float dn[W];
    {
      float a[W];
      load_row<N>(Hin, lane, a);
#pragma unroll
      for (int i = 0; i < W; ++i) {
        float s = 0.0f;
#pragma unroll
        for (int o = 0; o < W; ++o) s = fmaf(c_w[BOFF + OFF + off + i * W + o], d[o], s);
        dn[i] = s * fmaf(-a[i], a[i], 1.0f);
      }
    }
    tile_gemm<N, W, false>(Hin, B + l * BUF, acc + off, acc + off + W * W, lane);
    __syncwarp();
    store_row<N>(Hin, lane, dn);
    __syncwarp();
#pragma unroll
    for (int i = 0; i < W; ++i) d[i] = dn[i];
  }
  tile_gemm<N, 3, true>(X, B, acc, acc + 3 * W, lane);
  __syncwarp();
}

// one tile of 32 jobs of network N: forward recompute, backpropagation of g, dW accumulation
template <class N, int OFF, int BOFF>
__device__ __forceinline__ void net_adjoint_tile(const float x[3], float g, float* tile, float* acc, int lane) {
  float h[N::kW];
  net_forward_stage<N, OFF>(x, tile, tile + 32 * 4, lane, h);
  net_backward_tile<N, OFF, BOFF>(h, g, tile, acc, lane);
}

template <class N, int OFF>
__global__ void __launch_bounds__(256) k_job_forward(PtsH ph, const int32_t* __restrict__ ids, Workspace w, int net_p) {
  load_weights(w.params);
  const Ctl ctl = *w.ctl;
  const int64_t begin = net_p ? ctl.jm_pad : 0;
  const int64_t end = net_p ? ctl.total : ctl.jm;
  for (int64_t j = begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < end; j += (int64_t)gridDim.x * blockDim.x) {
    const float4 xv = w.jx[j];
    const float x[3] = {xv.x, xv.y, xv.z};
    w.ju[j] = net_forward<N, OFF>(x);
  }
}

template <class N>
constexpr size_t adj_smem_bytes() {
  return sizeof(float) * ((size_t)(N::kParams + 3) / 4 * 4 + (size_t)kWarps * N::kTileFloats);
}

template <class N, int OFF, int BOFF>
__global__ void __launch_bounds__(kThreads, 2) k_job_adjoint(PtsH ph, const int32_t* __restrict__ ids, Workspace w,
                                                             int net_p) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* acc = smem;
  float* tile = smem + (N::kParams + 3) / 4 * 4 + warp * N::kTileFloats;
  for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) acc[i] = 0.0f;
  load_weights(w.params);
  const Ctl ctl = *w.ctl;
  const int64_t begin = net_p ? ctl.jm_pad : 0;
  const int64_t end = net_p ? ctl.total : ctl.jm;
  const int64_t tiles = (end - begin + 31) / 32;
  for (int64_t t = (int64_t)blockIdx.x * kWarps + warp; t < tiles; t += (int64_t)gridDim.x * kWarps) {
    const int64_t j = begin + t * 32 + lane;
    float x[3] = {0.0f, 0.0f, 0.0f};
    float g = 0.0f;
    if (j < end) {
      const float4 xv = w.jx[j];
      x[0] = xv.x;
      x[1] = xv.y;
      x[2] = xv.z;
      g = w.jg[j];
    }
    net_adjoint_tile<N, OFF, BOFF>(x, g, tile, acc, lane);
  }
  __syncthreads();
  float* row = w.partials + (size_t)blockIdx.x * w.n_params + OFF;
  for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) row[i] = acc[i];
}

// ----------------------------------------------------------------------------------------
// fused kernel for bulk points (7 jobs of one network: the stencil points)
// ----------------------------------------------------------------------------------------
// CTA = 7 warps; warp j evaluates stencil point j of 32 consecutive bulk points (lane = point).
// One forward gives both the residual and the staged activations; the residual goes
// through shared memory; with BWD the backward half of the adjoint tile follows.
template <class N>
constexpr size_t fused_smem_bytes() {
  return sizeof(float) * ((size_t)(N::kParams + 3) / 4 * 4 + (size_t)kStencil * N::kTileFloats + kStencil * 32);
}

template <class N, int OFF, int BOFF, bool BWD>
__global__ void __launch_bounds__(kFusedThreads, 2) k_bulk_fused(PtsH ph, const int32_t* __restrict__ ids, Workspace w,
                                                                 dips_records_t rec, int net_p,
                                                                 float* __restrict__ residual_out) {
  constexpr int W = N::kW;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;  // warp = stencil point
  float* acc = smem;
  float* tile = smem + (N::kParams + 3) / 4 * 4 + warp * N::kTileFloats;
  float* sU = smem + (N::kParams + 3) / 4 * 4 + kStencil * N::kTileFloats;  // [7][32] A_j u_j
  if (BWD)
    for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) acc[i] = 0.0f;
  load_weights(w.params);
  const int64_t nb = net_p ? w.ctl->nbp : w.ctl->nbm;
  const int32_t* list = w.bulk + (net_p ? w.B : 0);
  const float Bf = (float)w.B;
  double lsum = 0.0;
  for (int64_t base = (int64_t)blockIdx.x * 32; base < nb; base += (int64_t)gridDim.x * 32) {
    const int64_t idx = base + lane;
    const bool valid = idx < nb;
    const int32_t slot = valid ? list[idx] : 0;
    const int64_t pid = valid ? batch_pid(ids, slot) : 0;
    float x[3] = {0.0f, 0.0f, 0.0f};
    float A = 0.0f;
    if (valid) {
      const float p[3] = {ph.pts[3 * pid], ph.pts[3 * pid + 1], ph.pts[3 * pid + 2]};
      stencil_point(p, ph.h, warp, x);
      const int64_t jb = net_p ? rec.job_off[pid + 1] - kStencil : rec.job_off[pid];
#pragma unroll
      for (int q = 0; q < kStencil; ++q)
        if (job_stencil(rec.job_code[jb + q]) == warp) A = rec.job_A[jb + q];
    }
    float h[W];
    net_forward_stage<N, OFF>(x, tile, tile + 32 * 4, lane, h);
    float u = 0.0f;
#pragma unroll
    for (int i = 0; i < W; ++i) u = fmaf(h[i], c_w[OFF + N::kOut + i], u);
    u += c_w[OFF + N::kOut + W];
    sU[warp * 32 + lane] = valid ? A * u : 0.0f;
    __syncthreads();
    float gc = 0.0f;
    if (valid) {
      float lhs = rec.lhs0[pid];
#pragma unroll
      for (int j = 0; j < kStencil; ++j) lhs += sU[j * 32 + lane];
      const float diag = rec.diag[pid];
      const float qv = lhs / diag;
      const float r0 = nan_to_num(qv) - rec.rod[pid];
      const float Pv = w.pre_P ? w.pre_P[slot] : 1.0f;  // learned preconditioner
      const float r = Pv * r0;
      gc = isfinite(qv) ? (r / Bf) * Pv / diag : 0.0f;
      if (warp == 0) {
        lsum += 0.5 * (double)r * (double)r;
        if (residual_out) residual_out[slot] = r;
        if (w.pre_P) w.pre_r0[slot] = r0;
      }
    }
    __syncthreads();  // sU is rewritten by the next group
    if (BWD) net_backward_tile<N, OFF, BOFF>(h, gc * A, tile, acc, lane);
  }
  // loss partial of this CTA (warp 0 holds the sums)
  if (warp == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0) w.floss[net_p * kLossSlots + blockIdx.x] = lsum;
    if (lane == 0 && blockIdx.x == 0) {
      w.ctl->floss_n[net_p] = gridDim.x;
      if (BWD) w.ctl->grad_rows[net_p] = w.grid + gridDim.x;  // adjoint rows, then these
    }
  }
  if (BWD) {
    __syncthreads();
    float* row = w.partials + (size_t)(w.grid + blockIdx.x) * w.n_params + OFF;
    for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) row[i] = acc[i];
  }
}

// ----------------------------------------------------------------------------------------
// network evaluation with input gradient
// ----------------------------------------------------------------------------------------
template <class N, int OFF, int BOFF>
__device__ __forceinline__ float net_eval_grad(const float x[3], float gx[3]) {
  constexpr int W = N::kW, L = N::kL;
  float act[L][W];
#pragma unroll
  for (int o = 0; o < W; ++o) {
    float z = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i) z = fmaf(x[i], c_w[OFF + i * W + o], z);
    act[0][o] = act_tanh(z + c_w[OFF + 3 * W + o]);
  }
#pragma unroll
  for (int l = 1; l < L; ++l) {
    const int off = OFF + N::layer_off(l);
    float t[W];
#pragma unroll
    for (int o = 0; o < W; ++o) t[o] = 0.0f;
#pragma unroll
    for (int i = 0; i < W; ++i)
#pragma unroll
      for (int o = 0; o < W; ++o) t[o] = fmaf(act[l - 1][i], c_w[off + i * W + o], t[o]);
#pragma unroll
    for (int o = 0; o < W; ++o) act[l][o] = act_tanh(t[o] + c_w[off + W * W + o]);
  }
  float u = 0.0f;
#pragma unroll
  for (int i = 0; i < W; ++i) u = fmaf(act[L - 1][i], c_w[OFF + N::kOut + i], u);
  u += c_w[OFF + N::kOut + W];
  float d[W];
#pragma unroll
  for (int i = 0; i < W; ++i) {
    const float hv = act[L - 1][i];
    d[i] = c_w[BOFF + OFF + N::kOut + i] * fmaf(-hv, hv, 1.0f);
  }
#pragma unroll
  for (int l = L - 1; l >= 1; --l) {
    const int off = BOFF + OFF + N::layer_off(l);
    float dn[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      float s = 0.0f;
#pragma unroll
      for (int o = 0; o < W; ++o) s = fmaf(c_w[off + i * W + o], d[o], s);
      const float hv = act[l - 1][i];
      dn[i] = s * fmaf(-hv, hv, 1.0f);
    }
#pragma unroll
    for (int i = 0; i < W; ++i) d[i] = dn[i];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float s = 0.0f;
#pragma unroll
    for (int o = 0; o < W; ++o) s = fmaf(c_w[BOFF + OFF + c * W + o], d[o], s);
    gx[c] = s;
  }
  return u;
}

template <class N, int OFF, int BOFF>
__global__ void __launch_bounds__(128) k_mlp_eval(const float* __restrict__ params, const float* __restrict__ pts,
                                                  const float* __restrict__ phi, int64_t n, float* __restrict__ u_out,
                                                  float* __restrict__ g_out, int net_p) {
  load_weights(params);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if ((phi[i] >= 0.0f) != (net_p != 0)) continue;
    const float x[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    float gx[3];
    const float u = net_eval_grad<N, OFF, BOFF>(x, gx);
    u_out[i] = u;
    if (g_out) {
      g_out[3 * i] = gx[0];
      g_out[3 * i + 1] = gx[1];
      g_out[3 * i + 2] = gx[2];
    }
  }
}

using A = Arch<DIPS_LM, DIPS_WM, DIPS_LP, DIPS_WP>;

// both networks on the register-blocked tile engine (one shape for both), one launch per phase
constexpr bool kTileArch = tile::supported<typename A::M>() && tile::supported<typename A::P>() &&
                           A::M::kW == A::P::kW && A::M::kL == A::P::kL;

// Every kernel reads the parameters of its own call (Workspace::params or an argument): nothing
// to stage per call, and no state shared between calls.
static_assert(kArchParams == A::kParams, "parameter count");
static_assert(kTileArch || 2 * A::kParams * sizeof(float) <= 16 * 1024, "per-job kernels: weights in shared memory");
static int load_params(const float*, int, cudaStream_t) { return DIPS_OK; }


// CTA widths of the tile engine (warps per CTA): width 32 fills an SM with one CTA of 12, 10 or 8
// warps; width 16 runs 24 warps per SM as 2 x 12, 3 x 8 or 4 x 6.  dips_autotune picks one per
// device; the first is the default.
constexpr int kTileCand[3] = {12, A::M::kW == 32 ? 10 : 8, A::M::kW == 32 ? 8 : 6};
constexpr int kMaxDevices = 64;
static std::atomic<int> g_tile_nw[kMaxDevices];
static std::mutex g_tune_mu;

static int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
  return dev;
}

static int tile_nw() {
  const int dev = current_device();
  const int v = dev < 0 ? 0 : g_tile_nw[dev].load(std::memory_order_relaxed);
  return v ? v : kTileCand[0];
}

template <class N, int MODE, int NW>
static int tile_launch_nw(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec,
                          float* residual_out, cudaStream_t s) {
  static_assert(N::kParams == A::P::kParams, "tile engine: both networks of one shape");
  constexpr size_t bytes = tile::CtaLayout<N, NW>::kBytes;
  static_assert(bytes <= 227 * 1024, "tile engine: shared memory");
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(tile::k_tile<N, MODE, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(tile engine smem)");
    attr_done = true;
  }
  constexpr int ctas_per_sm = tile::warps_per_sm<N>() / NW;
  static_assert(kTileGrid * ctas_per_sm <= kLossSlots && kTileGrid * ctas_per_sm <= kAdjGrid + kFusedGrid,
                "tile engine: more CTAs than loss slots or partial gradient rows");
  static_assert(ctas_per_sm * (bytes + 1024) <= 228 * 1024, "tile engine: CTAs per SM do not fit in shared memory");
  tile::k_tile<N, MODE, NW><<<kTileGrid * ctas_per_sm, 32 * NW, bytes, s>>>(ph, ids, w, rec, A::kOffP, residual_out);
  return DIPS_OK;
}

// (TILE is a template parameter so that the engine is instantiated for tile archs only)
template <int MODE, bool TILE = kTileArch>
static int tile_launch(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec,
                       float* residual_out, cudaStream_t s) {
  if constexpr (TILE) {
    using N = typename A::M;
    const int nw = tile_nw();
    if (nw == kTileCand[1]) return tile_launch_nw<N, MODE, kTileCand[1]>(ph, ids, w, rec, residual_out, s);
    if (nw == kTileCand[2]) return tile_launch_nw<N, MODE, kTileCand[2]>(ph, ids, w, rec, residual_out, s);
    return tile_launch_nw<N, MODE, kTileCand[0]>(ph, ids, w, rec, residual_out, s);
  } else {
    ::dips::set_error("tile engine: network shape without the engine");
    return DIPS_E_UNSUPPORTED;
  }
}

template <class N, int MODE, int NW>
static int tile_multi_launch_nw(const Inst* T, int n, cudaStream_t s) {
  constexpr size_t bytes = tile::CtaLayout<N, NW>::kBytes;
  constexpr int ctas_per_sm = tile::warps_per_sm<N>() / NW;
  constexpr size_t static_bytes = sizeof(int64_t) * (tile::kMaxInstances + 2) + 2 * sizeof(tile::NetTiles);
  static_assert(ctas_per_sm * (bytes + static_bytes + 1024) <= 228 * 1024,
                "multi-instance tile engine: CTAs per SM do not fit in shared memory");
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(tile::k_tile_multi<N, MODE, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(multi-instance tile engine smem)");
    attr_done = true;
  }
  tile::k_tile_multi<N, MODE, NW><<<kTileGrid * ctas_per_sm, 32 * NW, bytes, s>>>(T, n, A::kOffP);
  return DIPS_OK;
}

template <int MODE, bool TILE = kTileArch>
static int tile_multi(const Inst* T, int n, cudaStream_t s) {
  if constexpr (TILE) {
    using N = typename A::M;
    if (n > tile::kMaxInstances) {
      ::dips::set_error("multi-instance step: %d instances, at most %d per launch", n, tile::kMaxInstances);
      return DIPS_E_ARG;
    }
    const int nw = tile_nw();
    if (nw == kTileCand[1]) return tile_multi_launch_nw<N, MODE, kTileCand[1]>(T, n, s);
    if (nw == kTileCand[2]) return tile_multi_launch_nw<N, MODE, kTileCand[2]>(T, n, s);
    return tile_multi_launch_nw<N, MODE, kTileCand[0]>(T, n, s);
  } else {
    ::dips::set_error("multi-instance step: network shape without the tile engine");
    return DIPS_E_UNSUPPORTED;
  }
}

static int multi_forward(const Inst* T, int n, cudaStream_t s) {
  const int st = tile_multi<tile::kForwardGeneral>(T, n, s);
  if (st) return st;
  DIPS_CHECK_LAUNCH("multi-instance general forward");
  return DIPS_OK;
}

static int multi_train(const Inst* T, int n, cudaStream_t s) {
  const int st = tile_multi<tile::kTrain>(T, n, s);
  if (st) return st;
  DIPS_CHECK_LAUNCH("multi-instance training launch");
  return DIPS_OK;
}

static int job_forward(const PtsH& ph, const int32_t* ids, const Workspace& w, const Marks* mk, cudaStream_t s) {
  if constexpr (kTileArch) {  // both networks' general jobs in one tile-engine launch
    mark(mk, kMarkFwdM, s);
    const dips_records_t none{};
    const int st = tile_launch<tile::kForwardGeneral>(ph, ids, w, none, nullptr, s);
    if (st) return st;
  } else {  // one thread per job, the weights in shared memory
    k_job_forward<typename A::M, 0><<<152 * 24, 256, 0, s>>>(ph, ids, w, 0);
    mark(mk, kMarkFwdM, s);
    k_job_forward<typename A::P, A::kOffP><<<152 * 24, 256, 0, s>>>(ph, ids, w, 1);
  }
  mark(mk, kMarkFwdP, s);
  DIPS_CHECK_LAUNCH("job forward");
  return DIPS_OK;
}

template <class N, int OFF>
static int adjoint_launch(const PtsH& ph, const int32_t* ids, const Workspace& w, int net_p, cudaStream_t s) {
  constexpr size_t bytes = adj_smem_bytes<N>();
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(k_job_adjoint<N, OFF, A::kParams>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(adjoint smem)");
    attr_done = true;
  }
  k_job_adjoint<N, OFF, A::kParams><<<w.grid, kThreads, bytes, s>>>(ph, ids, w, net_p);
  return DIPS_OK;
}

static int job_adjoint(const PtsH& ph, const int32_t* ids, const Workspace& w, const Marks* mk, cudaStream_t s) {
  // on the tile engine the general jobs' backward is part of the bulk launch
  int st = DIPS_OK;
  if constexpr (!kTileArch) st = adjoint_launch<typename A::M, 0>(ph, ids, w, 0, s);
  if (st) return st;
  mark(mk, kMarkAdjM, s);
  if constexpr (!kTileArch) st = adjoint_launch<typename A::P, A::kOffP>(ph, ids, w, 1, s);
  if (st) return st;
  mark(mk, kMarkAdjP, s);
  DIPS_CHECK_LAUNCH("job adjoint");
  return DIPS_OK;
}

template <class N, int OFF, bool BWD>
static int fused_launch(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec,
                        float* residual_out, int net_p, cudaStream_t s) {
  constexpr size_t bytes = fused_smem_bytes<N>();
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(k_bulk_fused<N, OFF, A::kParams, BWD>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(fused smem)");
    attr_done = true;
  }
  k_bulk_fused<N, OFF, A::kParams, BWD><<<w.fgrid, kFusedThreads, bytes, s>>>(ph, ids, w, rec, net_p, residual_out);
  return DIPS_OK;
}

static int bulk_fused(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec,
                      float* residual_out, bool bwd, const Marks* mk, cudaStream_t s) {
  int st;
  if constexpr (kTileArch) {
    mark(mk, kMarkFusedM, s);
    st = bwd ? tile_launch<tile::kTrain>(ph, ids, w, rec, residual_out, s)
             : tile_launch<tile::kForwardBulk>(ph, ids, w, rec, residual_out, s);
  } else if (bwd) {
    st = fused_launch<typename A::M, 0, true>(ph, ids, w, rec, residual_out, 0, s);
    if (!st) mark(mk, kMarkFusedM, s);
    if (!st) st = fused_launch<typename A::P, A::kOffP, true>(ph, ids, w, rec, residual_out, 1, s);
  } else {
    st = fused_launch<typename A::M, 0, false>(ph, ids, w, rec, residual_out, 0, s);
    if (!st) mark(mk, kMarkFusedM, s);
    if (!st) st = fused_launch<typename A::P, A::kOffP, false>(ph, ids, w, rec, residual_out, 1, s);
  }
  if (st) return st;
  mark(mk, kMarkFusedP, s);
  DIPS_CHECK_LAUNCH("fused bulk kernel");
  return DIPS_OK;
}

template <class N, int NW>
static int tile_eval_nw(const float* params, const float* pts, const float* phi, int64_t n, float* u, float* g,
                        cudaStream_t s) {
  constexpr size_t bytes = tile::CtaLayout<N, NW>::kBytes;
  constexpr int ctas_per_sm = tile::warps_per_sm<N>() / NW;
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(tile::k_tile_eval<N, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(tile evaluation smem)");
    attr_done = true;
  }
  tile::k_tile_eval<N, NW><<<kTileGrid * ctas_per_sm, 32 * NW, bytes, s>>>(pts, phi, n, params, A::kOffP, u, g);
  DIPS_CHECK_LAUNCH("tile evaluation");
  return DIPS_OK;
}

template <bool TILE = kTileArch>
static int tile_eval(const float* params, const float* pts, const float* phi, int64_t n, float* u, float* g,
                     cudaStream_t s) {
  if constexpr (TILE) {
    return tile_eval_nw<typename A::M, kTileCand[0]>(params, pts, phi, n, u, g, s);
  } else {
    ::dips::set_error("tile evaluation: network shape without the tile engine");
    return DIPS_E_UNSUPPORTED;
  }
}

static int mlp_eval(const float* params, const float* pts, const float* phi, int64_t n, float* u, float* g,
                    cudaStream_t s) {
  if constexpr (kTileArch) return tile_eval(params, pts, phi, n, u, g, s);
  int64_t grid = (n + 127) / 128;
  if (grid > 152 * 16) grid = 152 * 16;
  k_mlp_eval<typename A::M, 0, A::kParams><<<(int)grid, 128, 0, s>>>(params, pts, phi, n, u, g, 0);
  k_mlp_eval<typename A::P, A::kOffP, A::kParams><<<(int)grid, 128, 0, s>>>(params, pts, phi, n, u, g, 1);
  DIPS_CHECK_LAUNCH("mlp eval");
  return DIPS_OK;
}


// Times the training launch of the tile engine under each CTA width (one warm-up, then three
// timed repetitions on the caller's stream, which is synchronised) and keeps the fastest for
// the current device.
static int autotune(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec, cudaStream_t s,
                    int* chosen) {
  *chosen = 0;
  if constexpr (!kTileArch) {
    return DIPS_OK;
  } else {
    const int dev = current_device();
    DIPS_REQUIRE(dev >= 0, DIPS_E_CUDA, "autotune: no current device");
    std::lock_guard<std::mutex> lock(g_tune_mu);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
      return cuda_status(cudaGetLastError(), "autotune: cudaEventCreate");
    const int* cand = kTileCand;
    float best = 3.4e38f;
    int best_nw = kTileCand[0];
    int st = DIPS_OK;
    for (int ci = 0; ci < 3; ++ci) {
      const int c = cand[ci];
      g_tile_nw[dev].store(c);
      for (int r = 0; r < 4 && !st; ++r) {
        if (r == 1) cudaEventRecord(e0, s);
        st = bulk_fused(ph, ids, w, rec, nullptr, true, nullptr, s);
      }
      cudaEventRecord(e1, s);
      cudaError_t e = cudaEventSynchronize(e1);
      if (st || e != cudaSuccess) {
        if (!st) st = cuda_status(e, "autotune: timing");
        break;
      }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        best_nw = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_tile_nw[dev].store(st ? 0 : best_nw);
    if (!st) *chosen = best_nw;
    return st;
  }
}

}  // namespace DIPS_NS

const ArchOps* DIPS_GETTER() {
  static const ArchOps ops = {DIPS_LM,           DIPS_WM,          DIPS_LP,
                              DIPS_WP,           DIPS_NS::A::kParams,
                              1,
                              DIPS_NS::load_params,
                              DIPS_NS::job_forward, DIPS_NS::job_adjoint, DIPS_NS::bulk_fused,
                              DIPS_NS::mlp_eval, DIPS_NS::autotune,
                              DIPS_NS::kTileArch ? DIPS_NS::multi_forward : nullptr,
                              DIPS_NS::kTileArch ? DIPS_NS::multi_train : nullptr};
  return &ops;
}

}  // namespace dips
