// Per-network-shape kernels of the residual path (included once per shape by the
// residual_a_*.cu translation units, which define DIPS_LM, DIPS_WM, DIPS_LP, DIPS_WP).
//
// Forward and adjoint run one thread per job on the FP32 pipe: the weights are read as
// constant-bank operands of FFMA; dW is accumulated with a per-warp shared-memory
// outer-product GEMM and reduced to one partial gradient row per CTA.
// Reference: DoubleMLP (nn/mlp/MLP.py:93-139), value_and_grad in Trainer.update
// (solvers/poisson/trainer.py:783-789).

#include <math.h>

#include "residual_common.cuh"

namespace dips {
namespace DIPS_NS {

constexpr int kMaxConstParams = 15360;  // 60 KB of the 64 KB constant bank
static __constant__ float c_w[kMaxConstParams];

constexpr int kThreads = kAdjThreads;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ float act_tanh(float z) { return tanhf(z); }

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
};

template <int LM, int WM, int LP, int WP>
struct Arch {
  using M = Net<LM, WM>;
  using P = Net<LP, WP>;
  static constexpr int kOffP = M::kParams;
  static constexpr int kParams = M::kParams + P::kParams;
  static constexpr int kMaxW = WM > WP ? WM : WP;
};

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

// forward keeping every hidden activation
template <class N, int OFF>
__device__ __forceinline__ float net_forward_act(const float x[3], float act[N::kL][N::kW]) {
  constexpr int W = N::kW, L = N::kL;
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
  return u + c_w[OFF + N::kOut + W];
}

// ----------------------------------------------------------------------------------------
// per-warp outer-product accumulation  accW[i][o] += sum_lanes in[i]*d[o],  accb[o] += sum d[o]
// ----------------------------------------------------------------------------------------
constexpr int kStageIn = 36;   // float4-aligned row stride of the staged inputs (<= 32 used)
constexpr int kStageD = 33;    // row stride of the staged output gradients
constexpr int kStageFloats = 32 * kStageIn + 32 * kStageD;

template <int IN, int OUT>
__device__ __forceinline__ void warp_stage(const float* in, const float* d, float* sIn, float* sD, int lane) {
#pragma unroll
  for (int i = 0; i < IN; ++i) sIn[lane * kStageIn + i] = in[i];
#pragma unroll
  for (int o = 0; o < OUT; ++o) sD[lane * kStageD + o] = d[o];
  __syncwarp();
}

// accW[i][o] += sum_e sIn[e][i] * sD[e][o];  accb[o] += sum_e sD[e][o]  (e = the warp's 32 lanes)
template <int IN, int OUT>
__device__ __forceinline__ void warp_gemm_acc(const float* sIn, const float* sD, float* accW, float* accb, int lane) {
  constexpr int IG = 32 / OUT;            // lane groups splitting the inputs
  constexpr int CH = (IN + IG - 1) / IG;  // inputs per lane
  constexpr int CK = CH > 16 ? 16 : CH;   // inputs per pass (bounds live accumulators)
  const int o = lane % OUT;
  const int ig = lane / OUT;
  if (ig < IG) {
    const int i0 = ig * CH;
#pragma unroll
    for (int c0 = 0; c0 < CH; c0 += CK) {
      float s[CK];
#pragma unroll
      for (int c = 0; c < CK; ++c) s[c] = 0.0f;
      float sb = 0.0f;
#pragma unroll 4
      for (int e = 0; e < 32; ++e) {
        const float dv = sD[e * kStageD + o];
        if (c0 == 0) sb += dv;
        const float* row = sIn + e * kStageIn + i0 + c0;
        if constexpr (CK % 4 == 0) {
#pragma unroll
          for (int c = 0; c < CK; c += 4) {
            const float4 v = *reinterpret_cast<const float4*>(row + c);
            s[c] = fmaf(v.x, dv, s[c]);
            s[c + 1] = fmaf(v.y, dv, s[c + 1]);
            s[c + 2] = fmaf(v.z, dv, s[c + 2]);
            s[c + 3] = fmaf(v.w, dv, s[c + 3]);
          }
        } else {
#pragma unroll
          for (int c = 0; c < CK; ++c)
            if (i0 + c0 + c < IN) s[c] = fmaf(row[c], dv, s[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < CK; ++c)
        if (c0 + c < CH && i0 + c0 + c < IN) accW[(i0 + c0 + c) * OUT + o] += s[c];
      if (c0 == 0 && ig == 0) accb[o] += sb;
    }
  }
  __syncwarp();
}

// backpropagate g = dL/du through network N at x, accumulating into the warp's accumulator
// The backward pass reads the weights from a second copy in the constant bank (offset BOFF):
// with a single copy the compiler keeps every weight used by both passes in registers.
template <class N, int OFF, int BOFF>
__device__ __forceinline__ void net_adjoint(const float x[3], float g, float* sIn, float* sD, float* acc, int lane) {
  constexpr int W = N::kW, L = N::kL;
  float act[L][W];
  net_forward_act<N, OFF>(x, act);
  float d[W];
  // output layer u = sum_i Wo[i] h[i] + bo
  {
    const float gg[1] = {g};
    warp_stage<W, 1>(act[L - 1], gg, sIn, sD, lane);
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const float hv = act[L - 1][i];
      d[i] = g * c_w[BOFF + OFF + N::kOut + i] * fmaf(-hv, hv, 1.0f);
    }
    warp_gemm_acc<W, 1>(sIn, sD, acc + N::kOut, acc + N::kOut + W, lane);
  }
#pragma unroll
  for (int l = L - 1; l >= 1; --l) {
    const int off = N::layer_off(l);
    warp_stage<W, W>(act[l - 1], d, sIn, sD, lane);
    float dn[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      float s = 0.0f;
#pragma unroll
      for (int o = 0; o < W; ++o) s = fmaf(c_w[BOFF + OFF + off + i * W + o], d[o], s);
      const float hv = act[l - 1][i];
      dn[i] = s * fmaf(-hv, hv, 1.0f);
    }
    warp_gemm_acc<W, W>(sIn, sD, acc + off, acc + off + W * W, lane);
#pragma unroll
    for (int i = 0; i < W; ++i) d[i] = dn[i];
  }
  warp_stage<3, W>(x, d, sIn, sD, lane);
  warp_gemm_acc<3, W>(sIn, sD, acc, acc + 3 * W, lane);
}

template <class A>
__global__ void __launch_bounds__(256) k_job_forward(PtsH ph, const int32_t* __restrict__ ids, Workspace w) {
  const Ctl ctl = *w.ctl;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ctl.total; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t slot = w.jslot[j];
    float u = 0.0f;
    if (slot >= 0) {
      float x[3];
      job_point(ph, ids, slot, w.jcode[j], x);
      if (j < ctl.jm_pad)
        u = net_forward<typename A::M, 0>(x);
      else
        u = net_forward<typename A::P, A::kOffP>(x);
    }
    w.ju[j] = u;
  }
}

// ----------------------------------------------------------------------------------------
// adjoint over jobs
// ----------------------------------------------------------------------------------------
template <class A>
struct AdjSmem {
  static constexpr int kAccM = A::M::kParams;
  static constexpr int kAccP = A::P::kParams;
  static constexpr int kAcc = kAccM > kAccP ? kAccM : kAccP;
  static constexpr int kPerWarp = kStageFloats + (kAcc + 3) / 4 * 4;  // keeps float4 rows aligned
  static constexpr size_t kBytes = sizeof(float) * (size_t)kPerWarp * kWarps;
};

template <class A>
__global__ void __launch_bounds__(kThreads, 1) k_job_adjoint(PtsH ph, const int32_t* __restrict__ ids, Workspace w) {
  extern __shared__ float smem[];
  using S = AdjSmem<A>;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* sIn = smem + warp * S::kPerWarp;
  float* sD = sIn + 32 * kStageIn;
  float* acc = sD + 32 * kStageD;
  for (int i = lane; i < S::kAcc; i += 32) acc[i] = 0.0f;
  __syncwarp();

  const Ctl ctl = *w.ctl;
  const int64_t tiles_m = ctl.jm_pad / 32;
  const int64_t tiles_p = (ctl.jp + 31) / 32;
  const int64_t tiles = tiles_m + tiles_p;
  // CTAs [0, gm) take u- tiles, the rest take u+ tiles (in proportion to the tile counts)
  int gm = 0;
  if (tiles > 0) {
    gm = (int)((tiles_m * (int64_t)gridDim.x + tiles / 2) / tiles);
    if (tiles_m > 0 && gm < 1) gm = 1;
    if (tiles_p > 0 && gm > (int)gridDim.x - 1) gm = gridDim.x - 1;
    if (tiles_p == 0) gm = gridDim.x;
  }
  const bool net_p = (int)blockIdx.x >= gm;
  const int64_t my_tiles = net_p ? tiles_p : tiles_m;
  const int64_t cta = net_p ? blockIdx.x - gm : blockIdx.x;
  const int64_t nctas = net_p ? (int64_t)gridDim.x - gm : gm;
  const int64_t base = net_p ? ctl.jm_pad : 0;
  const int64_t end = net_p ? ctl.total : ctl.jm;

  if (nctas > 0) {
    for (int64_t t = cta * kWarps + warp; t < my_tiles; t += nctas * kWarps) {
      const int64_t j = base + t * 32 + lane;
      float x[3] = {0.0f, 0.0f, 0.0f};
      float g = 0.0f;
      if (j < end) {
        const int32_t slot = w.jslot[j];
        if (slot >= 0) {
          job_point(ph, ids, slot, w.jcode[j], x);
          g = w.gs[slot] * w.jA[j];
        }
      }
      if (net_p)
        net_adjoint<typename A::P, A::kOffP, A::kParams>(x, g, sIn, sD, acc, lane);
      else
        net_adjoint<typename A::M, 0, A::kParams>(x, g, sIn, sD, acc, lane);
    }
  }
  __syncthreads();
  // fixed-order reduction of the warps' accumulators into this CTA's partial row
  const int np = net_p ? A::P::kParams : A::M::kParams;
  const int off = net_p ? A::kOffP : 0;
  float* row = w.partials + (size_t)blockIdx.x * A::kParams;
  for (int i = threadIdx.x; i < A::kParams; i += blockDim.x) {
    float v = 0.0f;
    const int li = i - off;
    if (li >= 0 && li < np && nctas > 0) {
      for (int q = 0; q < kWarps; ++q) v += smem[q * S::kPerWarp + kStageFloats + li];
    }
    row[i] = v;
  }
}

// ----------------------------------------------------------------------------------------
// network evaluation with input gradient
// ----------------------------------------------------------------------------------------
template <class N, int OFF, int BOFF>
__device__ __forceinline__ float net_eval_grad(const float x[3], float gx[3]) {
  constexpr int W = N::kW, L = N::kL;
  float act[L][W];
  const float u = net_forward_act<N, OFF>(x, act);
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

template <class A>
__global__ void __launch_bounds__(128) k_mlp_eval(const float* __restrict__ pts, const float* __restrict__ phi, int64_t n,
                                                  float* __restrict__ u_out, float* __restrict__ g_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float x[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    float gx[3];
    float u;
    if (phi[i] >= 0.0f)
      u = net_eval_grad<typename A::P, A::kOffP, A::kParams>(x, gx);
    else
      u = net_eval_grad<typename A::M, 0, A::kParams>(x, gx);
    u_out[i] = u;
    if (g_out) {
      g_out[3 * i] = gx[0];
      g_out[3 * i + 1] = gx[1];
      g_out[3 * i + 2] = gx[2];
    }
  }
}


using A = Arch<DIPS_LM, DIPS_WM, DIPS_LP, DIPS_WP>;

static int load_params(const float* params, cudaStream_t s) {
  static_assert(2 * A::kParams <= kMaxConstParams, "network too large for the constant bank");
  // two copies: forward-pass operands at 0, backward-pass operands at kParams
  cudaError_t e = cudaMemcpyToSymbolAsync(c_w, params, sizeof(float) * A::kParams, 0, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(c_w, params, sizeof(float) * A::kParams, sizeof(float) * A::kParams,
                                cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? DIPS_OK : cuda_status(e, "cudaMemcpyToSymbolAsync(params)");
}

static int job_forward(const PtsH& ph, const int32_t* ids, const Workspace& w, cudaStream_t s) {
  k_job_forward<A><<<152 * 8, 256, 0, s>>>(ph, ids, w);
  DIPS_CHECK_LAUNCH("job forward");
  return DIPS_OK;
}

static int job_adjoint(const PtsH& ph, const int32_t* ids, const Workspace& w, cudaStream_t s) {
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e =
        cudaFuncSetAttribute(k_job_adjoint<A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AdjSmem<A>::kBytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(adjoint smem)");
    attr_done = true;
  }
  k_job_adjoint<A><<<w.grid, kThreads, AdjSmem<A>::kBytes, s>>>(ph, ids, w);
  DIPS_CHECK_LAUNCH("job adjoint");
  return DIPS_OK;
}

static int mlp_eval(const float* pts, const float* phi, int64_t n, float* u, float* g, cudaStream_t s) {
  int64_t grid = (n + 127) / 128;
  if (grid > 152 * 16) grid = 152 * 16;
  k_mlp_eval<A><<<(int)grid, 128, 0, s>>>(pts, phi, n, u, g);
  DIPS_CHECK_LAUNCH("mlp eval");
  return DIPS_OK;
}

}  // namespace DIPS_NS

const ArchOps* DIPS_GETTER() {
  static const ArchOps ops = {DIPS_LM, DIPS_WM, DIPS_LP, DIPS_WP, DIPS_NS::A::kParams,
                              DIPS_NS::load_params, DIPS_NS::job_forward, DIPS_NS::job_adjoint, DIPS_NS::mlp_eval};
  return &ops;
}

}  // namespace dips
