// Learned preconditioner of the residual (nn/preconditioner.py:10-35, trainer.py:229-243,
// discretization.py:339, :419-420): P(c) = 0.5 + s * sigmoid(MLP(c)) over the point's 26 cell
// coefficients c (geom_pp.py:873-901), multiplying lhs/diag and rhs/diag, i.e. the residual.
//
//   k_pre_fwd  one thread per batch slot: P, kept in the workspace for the residual kernels
//   k_pre_bwd  one warp per 32 slots: dL/dP = P r0^2 / B (r0 = the residual before P), back
//              through the MLP; the weight gradients are warp GEMMs over the 32 slots
//              (lane = output unit), kept in registers for all the warp's chunks and added into
//              one partial row per CTA at the end
//
// Hidden widths are uniform (8, 16 or 32) over 1 to 3 tanh layers.  Parameters (after the two
// solution networks): per hidden layer W[in][out] then b[out], then w_o[width] then b_o.

#include "residual_common.cuh"

namespace dips {

template <int L, int W>
struct Pre {
  static constexpr int kParams = kPreIn * W + W + (L - 1) * (W * W + W) + W + 1;
  static constexpr int kOut = kPreIn * W + W + (L - 1) * (W * W + W);
  __host__ __device__ static constexpr int off(int l) { return l == 0 ? 0 : kPreIn * W + W + (l - 1) * (W * W + W); }
  __host__ __device__ static constexpr int in(int l) { return l == 0 ? kPreIn : W; }
};

int pre_num_params(int layers, int width) {
  if (layers <= 0) return 0;
  return kPreIn * width + width + (layers - 1) * (width * width + width) + width + 1;
}

bool pre_supported(int layers, int width) {
  return layers >= 1 && layers <= 3 && (width == 8 || width == 16 || width == 32);
}

__device__ __forceinline__ float sigm(float y) { return 1.0f / (1.0f + __expf(-y)); }

// forward of one slot; a[l][i] = activations of hidden layer l (kept for the backward)
template <int L, int W>
__device__ __forceinline__ float pre_forward(const float* __restrict__ prm, const float* c, float (&a)[L][W]) {
  using N = Pre<L, W>;
#pragma unroll
  for (int o = 0; o < W; ++o) {
    float z = __ldg(prm + kPreIn * W + o);
#pragma unroll
    for (int i = 0; i < kPreIn; ++i) z = fmaf(c[i], __ldg(prm + i * W + o), z);
    a[0][o] = tanhf(z);
  }
#pragma unroll
  for (int l = 1; l < L; ++l) {
    const float* Wl = prm + N::off(l);
#pragma unroll
    for (int o = 0; o < W; ++o) {
      float z = __ldg(Wl + W * W + o);
#pragma unroll
      for (int i = 0; i < W; ++i) z = fmaf(a[l - 1][i], __ldg(Wl + i * W + o), z);
      a[l][o] = tanhf(z);
    }
  }
  float y = __ldg(prm + N::kOut + W);
#pragma unroll
  for (int i = 0; i < W; ++i) y = fmaf(a[L - 1][i], __ldg(prm + N::kOut + i), y);
  return y;
}

template <int L, int W>
__global__ void __launch_bounds__(256) k_pre_fwd(const float* __restrict__ prm, float scale, const int32_t* __restrict__ ids,
                                                 int64_t B, int64_t n_pts, const float* __restrict__ c26,
                                                 float* __restrict__ P) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int64_t pid = batch_pid(ids, b);
  if (pid < 0 || pid >= n_pts) {
    P[b] = 1.0f;
    return;
  }
  float c[kPreIn];
#pragma unroll
  for (int i = 0; i < kPreIn; ++i) c[i] = c26[pid * kPreIn + i];
  float a[L][W];
  const float y = pre_forward<L, W>(prm, c, a);
  P[b] = 0.5f + scale * sigm(y);
}

constexpr int kPreWarps = 4;

template <int L, int W>
__global__ void __launch_bounds__(32 * kPreWarps) k_pre_bwd(const float* __restrict__ prm, float scale,
                                                            const int32_t* __restrict__ ids, int64_t B, int64_t n_pts,
                                                            const float* __restrict__ c26, const float* __restrict__ P,
                                                            const float* __restrict__ r0, float* __restrict__ partials,
                                                            int pre_n) {
  using N = Pre<L, W>;
  // per warp: inputs [32][27], activations [L][32][W+1], deltas [L][32][W+1], output delta [32]
  // (odd row strides: the per-slot row writes and reads are bank-conflict free)
  constexpr int kCS = kPreIn + 1, kS = W + 1;
  constexpr int kWarpFloats = 32 * kCS + 2 * L * 32 * kS + 32;
  extern __shared__ float smp[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* acc = smp;  // [kParams] CTA accumulator
  float* wsm = smp + (N::kParams + 3) / 4 * 4 + warp * kWarpFloats;
  float* C = wsm;
  float* Aa = C + 32 * kCS;
  float* Dd = Aa + L * 32 * kS;
  float* Do = Dd + L * 32 * kS;
  for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) acc[i] = 0.0f;
  __syncthreads();
  // gradient accumulators, lane = output unit o (lanes >= W idle in the hidden layers)
  float gW0[kPreIn], gW[L > 1 ? L - 1 : 1][W], gb[L], gwo = 0.0f, gbo = 0.0f;
#pragma unroll
  for (int i = 0; i < kPreIn; ++i) gW0[i] = 0.0f;
#pragma unroll
  for (int l = 0; l < (L > 1 ? L - 1 : 1); ++l)
#pragma unroll
    for (int i = 0; i < W; ++i) gW[l][i] = 0.0f;
#pragma unroll
  for (int l = 0; l < L; ++l) gb[l] = 0.0f;
  const float invB = 1.0f / (float)B;
  const int64_t chunks = (B + 31) / 32;
  for (int64_t ch = (int64_t)blockIdx.x * kPreWarps + warp; ch < chunks; ch += (int64_t)gridDim.x * kPreWarps) {
    const int64_t b = ch * 32 + lane;
    float c[kPreIn];
#pragma unroll
    for (int i = 0; i < kPreIn; ++i) c[i] = 0.0f;
    float dP = 0.0f;
    const int64_t pid = b < B ? batch_pid(ids, b) : -1;
    if (pid >= 0 && pid < n_pts) {
      const float rv = r0[b];
      if (isfinite(rv)) {
#pragma unroll
        for (int i = 0; i < kPreIn; ++i) c[i] = c26[pid * kPreIn + i];
        dP = P[b] * rv * rv * invB;  // d(0.5 mean (P r0)^2) / dP
      }
    }
    float dy;
    {
      float a[L][W];
      const float sg = sigm(pre_forward<L, W>(prm, c, a));
      dy = dP * scale * sg * (1.0f - sg);
      // stage inputs and activations of the 32 slots (row = slot)
#pragma unroll
      for (int i = 0; i < kPreIn; ++i) C[lane * kCS + i] = c[i];
#pragma unroll
      for (int l = 0; l < L; ++l)
#pragma unroll
        for (int i = 0; i < W; ++i) Aa[(l * 32 + lane) * kS + i] = a[l][i];
    }
    // deltas, layer by layer from the top (activations read back from the staging rows)
    float d[W];
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const float av = Aa[((L - 1) * 32 + lane) * kS + i];
      d[i] = dy * __ldg(prm + N::kOut + i) * fmaf(-av, av, 1.0f);
    }
#pragma unroll
    for (int l = L - 1; l >= 0; --l) {
#pragma unroll
      for (int i = 0; i < W; ++i) Dd[(l * 32 + lane) * kS + i] = d[i];
      if (l > 0) {
        const float* Wl = prm + N::off(l);
        float dn[W];
#pragma unroll
        for (int i = 0; i < W; ++i) {
          float s = 0.0f;
#pragma unroll
          for (int o = 0; o < W; ++o) s = fmaf(__ldg(Wl + i * W + o), d[o], s);
          const float av = Aa[((l - 1) * 32 + lane) * kS + i];
          dn[i] = s * fmaf(-av, av, 1.0f);
        }
#pragma unroll
        for (int i = 0; i < W; ++i) d[i] = dn[i];
      }
    }
    Do[lane] = dy;
    __syncwarp();
    // weight gradients over the chunk: lane o of layer l sums in_l inputs x delta
    if (lane < W) {
      for (int s = 0; s < 32; ++s) {
        const float d0 = Dd[(0 * 32 + s) * kS + lane];
        gb[0] += d0;
#pragma unroll
        for (int i = 0; i < kPreIn; ++i) gW0[i] = fmaf(C[s * kCS + i], d0, gW0[i]);
#pragma unroll
        for (int l = 1; l < L; ++l) {
          const float dl = Dd[(l * 32 + s) * kS + lane];
          gb[l] += dl;
#pragma unroll
          for (int i = 0; i < W; ++i) gW[l - 1][i] = fmaf(Aa[((l - 1) * 32 + s) * kS + i], dl, gW[l - 1][i]);
        }
        gwo = fmaf(Aa[((L - 1) * 32 + s) * kS + lane], Do[s], gwo);
      }
    }
    if (lane == 0)
      for (int s = 0; s < 32; ++s) gbo += Do[s];
    __syncwarp();
  }
  // CTA sum of the warps, then one partial row
  if (lane < W) {
#pragma unroll
    for (int i = 0; i < kPreIn; ++i) atomicAdd(acc + i * W + lane, gW0[i]);
    atomicAdd(acc + kPreIn * W + lane, gb[0]);
#pragma unroll
    for (int l = 1; l < L; ++l) {
#pragma unroll
      for (int i = 0; i < W; ++i) atomicAdd(acc + N::off(l) + i * W + lane, gW[l - 1][i]);
      atomicAdd(acc + N::off(l) + W * W + lane, gb[l]);
    }
    atomicAdd(acc + N::kOut + lane, gwo);
  }
  if (lane == 0) atomicAdd(acc + N::kOut + W, gbo);
  __syncthreads();
  float* row = partials + (size_t)blockIdx.x * pre_n;
  for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) row[i] = acc[i];
}

template <int L, int W>
static int pre_launch(bool bwd, const dips_arch_t& a, const float* prm, const dips_records_t& rec, const int32_t* ids,
                      int64_t B, const Workspace& w, cudaStream_t s) {
  if (!bwd) {
    k_pre_fwd<L, W><<<div_up(B, 256), 256, 0, s>>>(prm, a.pre_scaling, ids, B, rec.n_pts, rec.coeff26, w.pre_P);
    DIPS_CHECK_LAUNCH("preconditioner forward");
    return DIPS_OK;
  }
  using N = Pre<L, W>;
  constexpr size_t bytes = sizeof(float) * ((size_t)(N::kParams + 3) / 4 * 4 +
                                            (size_t)kPreWarps * (32 * (kPreIn + 1) + 2 * L * 32 * (W + 1) + 32));
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_pre_bwd<L, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(preconditioner backward)");
    attr = true;
  }
  k_pre_bwd<L, W><<<kPreGrid, 32 * kPreWarps, bytes, s>>>(prm, a.pre_scaling, ids, B, rec.n_pts, rec.coeff26, w.pre_P,
                                                         w.pre_r0, w.pre_partials, w.pre_n);
  DIPS_CHECK_LAUNCH("preconditioner backward");
  return DIPS_OK;
}

static int pre_dispatch(bool bwd, const dips_arch_t& a, const float* prm, const dips_records_t& rec, const int32_t* ids,
                        int64_t B, const Workspace& w, cudaStream_t s) {
  DIPS_REQUIRE(rec.coeff26, DIPS_E_ARG, "the learned preconditioner needs records.coeff26");
  DIPS_REQUIRE(a.pre_scaling > 0.0f, DIPS_E_ARG, "preconditioner scaling must be positive");
#define DIPS_PRE_CASE(LL, WW) \
  if (a.pre_layers == LL && a.pre_width == WW) return pre_launch<LL, WW>(bwd, a, prm, rec, ids, B, w, s);
  DIPS_PRE_CASE(1, 8) DIPS_PRE_CASE(1, 16) DIPS_PRE_CASE(1, 32)
  DIPS_PRE_CASE(2, 8) DIPS_PRE_CASE(2, 16) DIPS_PRE_CASE(2, 32)
  DIPS_PRE_CASE(3, 8) DIPS_PRE_CASE(3, 16) DIPS_PRE_CASE(3, 32)
#undef DIPS_PRE_CASE
  set_error("preconditioner shape %d x %d not compiled (1-3 layers of width 8, 16 or 32)", a.pre_layers, a.pre_width);
  return DIPS_E_UNSUPPORTED;
}

int precond_forward(const dips_arch_t& a, const float* prm, const dips_records_t& rec, const int32_t* ids, int64_t B,
                    const Workspace& w, cudaStream_t s) {
  return pre_dispatch(false, a, prm, rec, ids, B, w, s);
}

int precond_backward(const dips_arch_t& a, const float* prm, const dips_records_t& rec, const int32_t* ids, int64_t B,
                     const Workspace& w, cudaStream_t s) {
  return pre_dispatch(true, a, prm, rec, ids, B, w, s);
}

}  // namespace dips
