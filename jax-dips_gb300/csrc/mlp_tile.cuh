// Register-blocked engine for DoubleMLP networks of 3 hidden layers of width 32 or 2 hidden
// layers of width 16 (nn/mlp/MLP.py:93-139): residual, adjoint and weight gradient of the NBM
// loss (solvers/poisson/trainer.py:783-789, :892-912) for bulk points and for general jobs.
//
// Included by residual_arch.cuh inside the per-shape namespace (after Net, Workspace and
// act_tanh are defined).
//
// Work unit: one warp owns a tile of 32 jobs and runs it through the whole network with
// __syncwarp only.  Every layer is a [32 jobs x W] x [W x W] product computed as 4 x NT
// register blocks (NT = W/4): lane = jbl + 8*ob holds jobs 4*jbl..4*jbl+3 and features
// ob + 4t (t < NT).  Activations and deltas sit in two warp-private shared buffers,
// feature-major ([feature][job], row stride 36 floats, so that the blocked row loads of the
// weight-gradient product are bank-conflict free).  The weights are copied once per CTA into
// shared memory, permuted so that a lane's NT features are contiguous (NT/4 float4 loads per k
// step); the forward copies are pre-scaled by 2*log2(e), the argument scale of the exp2 tanh.
//
// Per tile (3 x 32; the 2 x 16 form drops the middle layer and needs no recompute):
// forward (layer 1 from the job coordinates, layers 2 and 3 from the buffers),
// u = w_o . h3 + b_o, then the loss gradient g of each job, then
//   delta3 = g w_o (1 - h3^2)              -> buffer A (over h1)
//   dW3 += h2^T delta3                     (register accumulators)
//   delta2 = (delta3 W3^T) (1 - h2^2)      -> buffer B (over h2)
//   h1 recomputed from x                   -> buffer A
//   dW2 += h1^T delta2
//   delta1 = (delta2 W2^T) (1 - h1^2);  dW1 += x^T delta1
// The W x W weight gradients stay in registers for all tiles a warp processes (W*W/32 per lane
// and layer); bias, input-layer and output-layer gradients are reduce-scattered over the 8
// lanes that share a feature block and kept as one register each.  At the end the CTA adds its
// warps' accumulators into shared memory and writes one partial gradient row.  3 x 32: 12 warps
// per SM (168 registers), one CTA of 12, 10 or 8 warps; 2 x 16: 24 warps per SM as 2, 3 or 4
// CTAs; dips_autotune picks the CTA width.
//
// Tiles: bulk tiles hold 4 bulk points x 7 stencil points (lanes 0..27; lane = 7*point +
// stencil), whose residual is formed inside the warp from the 7 network values, plus (in the
// backward) 4 general jobs in lanes 28..31; general tiles hold 32 consecutive jobs of the
// expanded job list.  General jobs come with their coordinates and dL/du precomputed (jx, jg).

namespace tile {

template <class N>
constexpr bool supported() {
  return (N::kW == 32 && N::kL == 3) || (N::kW == 16 && N::kL == 2);
}
// warps per SM: the register budget of one thread (168 for 3 x 32, 85 for 2 x 16)
template <class N>
constexpr int warps_per_sm() {
  return N::kW == 32 ? 12 : 24;
}
constexpr int kRS = 36;  // buffer row stride (floats)
constexpr float kTanhScale = 2.8853900817779268f;  // 2 log2(e): tanh(z) = 1 - 2/(1 + 2^(kTanhScale z))

template <class N>
struct Layout {
  static_assert(supported<N>(), "tile engine: 3 hidden layers of width 32 or 2 of width 16");
  static constexpr int W = N::kW, L = N::kL;
  static constexpr int NT = W / 4;  // features per lane in a register block
  static constexpr int R = W / 8;   // weight-gradient rows per lane
  // CTA-shared, permuted weights (floats)
  static constexpr int kWF = 0;                     // [L-1][k = in][NT*ob + t] = c * W_l[k][ob + 4t]
  static constexpr int kWT = kWF + (L - 1) * W * W;  // [L-1][k = out][NT*ib + t] = W_l[ib + 4t][k]
  static constexpr int kW1 = kWT + (L - 1) * W * W;  // [3][NT*ob + t] = c * W_1[c][ob + 4t]
  static constexpr int kB = kW1 + 3 * W;            // [L][NT*ob + t] = c * b_l[ob + 4t]
  static constexpr int kWO = kB + L * W;            // [NT*ob + t] = w_o[ob + 4t]
  static constexpr int kBO = kWO + W;               // b_o
  static constexpr int kShared = kBO + 4;
  static constexpr int kNetW = (kShared + 3) / 4 * 4;  // one network's tables; u- then u+
  // warp-private region
  static constexpr int kX = 0;                  // [4][32] job coordinates (x, y, z, unused)
  static constexpr int kA = kX + 4 * 32;        // [W][kRS]
  static constexpr int kBB = kA + W * kRS;      // [W][kRS]
  static constexpr int kG = kBB + W * kRS;      // [32] dL/du per job
  static constexpr int kU = kG + 32;            // [32] A_j u_j of bulk tiles
  static constexpr int kAv = kU + 32;           // [32] A_j of bulk tiles
  static constexpr int kStage = kAv + 32;       // [2][160] inputs of the current and the next tile
  static constexpr int kStageFloats = 160;
  static constexpr int kWarpFloats = kStage + 2 * kStageFloats;
  static constexpr int kWarp0 = 2 * kNetW;
};

// the CTA-level parts of the layout, for NW warps per CTA
template <class N, int NW>
struct CtaLayout {
  using Lay = Layout<N>;
  static constexpr int kAccStride = (N::kParams + 3) / 4 * 4;
  static constexpr int kAcc = Lay::kWarp0 + NW * Lay::kWarpFloats;  // [2][kParams] CTA gradient accumulators
  static constexpr int kLoss = kAcc + 2 * kAccStride;                 // [NW][2] doubles
  static constexpr size_t kBytes = sizeof(float) * (size_t)kLoss + sizeof(double) * 2 * NW;
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}

// asynchronous global -> shared copies (zero-filled when !valid; src must still be mapped)
__device__ __forceinline__ void cp_async16(float* dst, const void* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async4(float* dst, const void* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// tanh of a pre-scaled argument y = 2 log2(e) z: 1 - 2/(1 + 2^y), hardware exp2 and
// reciprocal approximations (the same arithmetic as act_tanh)
__device__ __forceinline__ float tanh_scaled(float y) {
  float e;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(y));
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
  return fmaf(-2.0f, r, 1.0f);
}

// NT consecutive floats (NT a multiple of 4) into v
template <int NT>
__device__ __forceinline__ void ldrow(float (&v)[NT], const float* p) {
#pragma unroll
  for (int c = 0; c < NT / 4; ++c) {
    const float4 b = ld4(p + 4 * c);
    v[4 * c] = b.x;
    v[4 * c + 1] = b.y;
    v[4 * c + 2] = b.z;
    v[4 * c + 3] = b.w;
  }
}

// Two FP32 fused multiply-adds in one instruction (fma.rn.f32x2, sm_100 and later).  Each half
// rounds like fmaf, so a loop written with it gives bit-identical results to the scalar loop
// in half the issue slots.
using f32x2 = unsigned long long;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(f32x2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// z[q][t] += sum_k A[k][jc + q] * Bm[k][bc + t] over k < K (A row stride AS, Bm row stride 4 NT).
// The features of a lane come in adjacent pairs (t, t + 1), one packed FMA per pair and job.
template <int K, int AS, int NT>
__device__ __forceinline__ void gemm(float (&z)[4][NT], const float* A, int jc, const float* Bm, int bc) {
  f32x2 zz[4][NT / 2];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT / 2; ++t) zz[q][t] = pk2(z[q][2 * t], z[q][2 * t + 1]);
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    const float4 a = ld4(A + k * AS + jc);
    const float av[4] = {a.x, a.y, a.z, a.w};
    float bv[NT];
    ldrow(bv, Bm + k * 4 * NT + bc);
    f32x2 bp[NT / 2];
#pragma unroll
    for (int t = 0; t < NT / 2; ++t) bp[t] = pk2(bv[2 * t], bv[2 * t + 1]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const f32x2 aq = pk2(av[q], av[q]);
#pragma unroll
      for (int t = 0; t < NT / 2; ++t) zz[q][t] = fma2(aq, bp[t], zz[q][t]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT / 2; ++t) upk2(zz[q][t], z[q][2 * t], z[q][2 * t + 1]);
}

template <int NT>
__device__ __forceinline__ void store_blk(float* buf, int ob, int jc, const float (&z)[4][NT]) {
#pragma unroll
  for (int t = 0; t < NT; ++t) st4(buf + (ob + 4 * t) * kRS + jc, z[0][t], z[1][t], z[2][t], z[3][t]);
}

template <int NT>
__device__ __forceinline__ void load_blk(const float* buf, int ob, int jc, float (&z)[4][NT]) {
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const float4 v = ld4(buf + (ob + 4 * t) * kRS + jc);
    z[0][t] = v.x;
    z[1][t] = v.y;
    z[2][t] = v.z;
    z[3][t] = v.w;
  }
}

template <int NT>
__device__ __forceinline__ void fill_rows(float (&z)[4][NT], const float* b) {
  float bv[NT];
  ldrow(bv, b);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT; ++t) z[q][t] = bv[t];
}

template <int NT>
__device__ __forceinline__ void zero_blk(float (&z)[4][NT]) {
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT; ++t) z[q][t] = 0.0f;
}

template <int NT>
__device__ __forceinline__ void tanh_blk(float (&z)[4][NT]) {
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT; ++t) z[q][t] = tanh_scaled(z[q][t]);
}

// z *= 1 - a^2 with a this lane's block of `buf`
template <int NT>
__device__ __forceinline__ void times_dtanh(float (&z)[4][NT], const float* buf, int ob, int jc) {
  float a[4][NT];
  load_blk(buf, ob, jc, a);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT; ++t) z[q][t] *= fmaf(-a[q][t], a[q][t], 1.0f);
}

// Reduce-scatter of v[0..7] over the 8 lanes that share lane bits 3..4: returns the sum of
// v[jbl] over those lanes (jbl = lane bits 0..2).
__device__ __forceinline__ float rs(const float (&v)[8], int jbl) {
  const bool b2 = jbl & 4, b1 = jbl & 2, b0 = jbl & 1;
  float w[4], y[2];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float send = b2 ? v[q] : v[q + 4], keep = b2 ? v[q + 4] : v[q];
    w[q] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float send = b1 ? w[q] : w[q + 2], keep = b1 ? w[q + 2] : w[q];
    y[q] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  const float send = b0 ? y[0] : y[1], keep = b0 ? y[1] : y[0];
  return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

// The same for v[0..3]: the sum over the 8 lanes of v[jbl & 3]; lanes jbl and jbl ^ 4 hold the
// same value.
__device__ __forceinline__ float rs(const float (&v)[4], int jbl) {
  const bool b1 = jbl & 2, b0 = jbl & 1;
  float w[4], y[2];
#pragma unroll
  for (int q = 0; q < 4; ++q) w[q] = v[q] + __shfl_xor_sync(0xffffffffu, v[q], 4);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float send = b1 ? w[q] : w[q + 2], keep = b1 ? w[q + 2] : w[q];
    y[q] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  const float send = b0 ? y[0] : y[1], keep = b0 ? y[1] : y[0];
  return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

// feature of the reduce-scattered values of a lane, and whether the lane adds it in
template <int NT>
__device__ __forceinline__ int rs_feature(int lane) {
  return (lane >> 3) + 4 * (NT == 8 ? (lane & 7) : (lane & 3));
}
template <int NT>
__device__ __forceinline__ bool rs_owner(int lane) {
  return NT == 8 || (lane & 4) == 0;
}

// sum over this lane's 4 jobs, per feature
template <int NT>
__device__ __forceinline__ float colsum_rs(const float (&d)[4][NT], int jbl) {
  float v[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) v[t] = (d[0][t] + d[1][t]) + (d[2][t] + d[3][t]);
  return rs(v, jbl);
}

// acc[r][t] += sum over the tile's 32 jobs of H[row jbl + 8r][j] * D[row ob + 4t][j]
template <int R, int NT>
__device__ __forceinline__ void dw(float (&acc)[R][NT], const float* H, const float* D, int jbl, int ob) {
#pragma unroll 1  // measured: 1.2 % faster than 2, 1.2 % than 4 (3x32 training launch)
  for (int s = 0; s < 8; ++s) {
    float hv[R][4], dv[NT][4];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float4 v = ld4(H + (jbl + 8 * r) * kRS + 4 * s);
      hv[r][0] = v.x;
      hv[r][1] = v.y;
      hv[r][2] = v.z;
      hv[r][3] = v.w;
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const float4 v = ld4(D + (ob + 4 * t) * kRS + 4 * s);
      dv[t][0] = v.x;
      dv[t][1] = v.y;
      dv[t][2] = v.z;
      dv[t][3] = v.w;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int t = 0; t < NT; ++t) acc[r][t] = fmaf(hv[r][q], dv[t][q], acc[r][t]);
  }
}

// Gradient accumulators of one warp (see the file comment for the lane ownership).
template <class N>
struct Acc {
  static constexpr int L = N::kL, R = N::kW / 8, NT = N::kW / 4;
  float wh[L - 1][R][NT];  // dW of the hidden-to-hidden layers: rows jbl + 8r, columns ob + 4t
  float b[L];              // db of each hidden layer, feature rs_feature(lane)
  float w1[3];             // dW of the input layer, feature rs_feature(lane)
  float wo;                // dw_o, feature rs_feature(lane)
  float bo;                // db_o (every lane holds the total)
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int m = 0; m < L - 1; ++m)
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int t = 0; t < NT; ++t) wh[m][r][t] = 0.0f;
#pragma unroll
    for (int l = 0; l < L; ++l) b[l] = 0.0f;
    w1[0] = w1[1] = w1[2] = wo = bo = 0.0f;
  }
};

// Backward modes of one tile
enum TileBwd {
  kBwdNone = 0,   // forward only
  kBwdTrain = 1,  // dL/du from G; weight gradients into the accumulators
  kBwdInput = 2,  // du/dx: the backward with dL/du = 1 down to the input, no weight gradients
};

// One tile: forward of the 32 jobs whose coordinates are in X, then the backward of mode BM.
// EPI(u[4]) runs between the two: it receives this lane's 4 network values (jobs jc..jc+3) and,
// for kBwdTrain, must leave G filled for the warp (it may synchronise the warp).  With
// kBwdInput, gin[q][c] receives du/dx_c of job jc + q (every lane of the job's block).
template <class N, int BM, class Epi>
__device__ __forceinline__ void run_tile(const float* sm, float* wp, Acc<N>& acc, int lane, Epi epi,
                                         float (&gin)[4][3]) {
  using Lay = Layout<N>;
  constexpr int W = Lay::W, L = Lay::L, NT = Lay::NT;
  constexpr bool TRAIN = BM == kBwdTrain;
  const int jbl = lane & 7, ob = lane >> 3, jc = 4 * jbl, bc = NT * ob;
  float* X = wp + Lay::kX;
  float* bufA = wp + Lay::kA;
  float* bufB = wp + Lay::kBB;
  float* G = wp + Lay::kG;
  float h[4][NT];
  // layer 1: x -> bufA
  fill_rows(h, sm + Lay::kB + bc);
  gemm<3, 32>(h, X, jc, sm + Lay::kW1, bc);
  tanh_blk(h);
  store_blk(bufA, ob, jc, h);
  __syncwarp();
  if constexpr (L == 3) {
    // layer 2: bufA -> bufB
    fill_rows(h, sm + Lay::kB + W + bc);
    gemm<W, kRS>(h, bufA, jc, sm + Lay::kWF, bc);
    tanh_blk(h);
    store_blk(bufB, ob, jc, h);
    __syncwarp();
  }
  // last hidden layer: h_{L-1} (bufB for 3 layers, bufA for 2) -> registers
  float* hprev = L == 3 ? bufB : bufA;
  fill_rows(h, sm + Lay::kB + (L - 1) * W + bc);
  gemm<W, kRS>(h, hprev, jc, sm + Lay::kWF + (L - 2) * W * W, bc);
  tanh_blk(h);
  // output layer, reduced over the 4 feature blocks
  float wo[NT];
  ldrow(wo, sm + Lay::kWO + bc);
  const float bo = sm[Lay::kBO];
  float u[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float s = 0.0f;
#pragma unroll
    for (int t = 0; t < NT; ++t) s = fmaf(h[q][t], wo[t], s);
    s += __shfl_xor_sync(0xffffffffu, s, 8);
    s += __shfl_xor_sync(0xffffffffu, s, 16);
    u[q] = s + bo;
  }
  epi(u);
  if (BM == kBwdNone) {
    __syncwarp();
    return;
  }
  __syncwarp();
  float gv[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  if constexpr (TRAIN) {
    const float4 g4 = ld4(G + jc);
    gv[0] = g4.x;
    gv[1] = g4.y;
    gv[2] = g4.z;
    gv[3] = g4.w;
    float v[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) v[t] = fmaf(gv[0], h[0][t], gv[1] * h[1][t]) + fmaf(gv[2], h[2][t], gv[3] * h[3][t]);
    acc.wo += rs(v, jbl);
    float gs = (gv[0] + gv[1]) + (gv[2] + gv[3]);
    gs += __shfl_xor_sync(0xffffffffu, gs, 1);
    gs += __shfl_xor_sync(0xffffffffu, gs, 2);
    gs += __shfl_xor_sync(0xffffffffu, gs, 4);
    acc.bo += gs;
  }
  // delta_L = g w_o (1 - h_L^2) over the buffer that held h_{L-2} (3 layers: h1) or is free
  float* dbuf = L == 3 ? bufA : bufB;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < NT; ++t) h[q][t] = gv[q] * wo[t] * fmaf(-h[q][t], h[q][t], 1.0f);
  if constexpr (TRAIN) acc.b[L - 1] += colsum_rs(h, jbl);
  store_blk(dbuf, ob, jc, h);
  __syncwarp();
  if constexpr (TRAIN) dw(acc.wh[L - 2], hprev, dbuf, jbl, ob);
  // delta_{L-1} = (delta_L W_L^T) (1 - h_{L-1}^2)
  zero_blk(h);
  gemm<W, kRS>(h, dbuf, jc, sm + Lay::kWT + (L - 2) * W * W, bc);
  times_dtanh(h, hprev, ob, jc);
  if constexpr (TRAIN) acc.b[L - 2] += colsum_rs(h, jbl);
  if constexpr (L == 3) {
    __syncwarp();
    store_blk(bufB, ob, jc, h);  // delta2 over h2
    {  // h1 again, over delta3
      float h1[4][NT];
      fill_rows(h1, sm + Lay::kB + bc);
      gemm<3, 32>(h1, X, jc, sm + Lay::kW1, bc);
      tanh_blk(h1);
      store_blk(bufA, ob, jc, h1);
    }
    __syncwarp();
    if constexpr (TRAIN) dw(acc.wh[0], bufA, bufB, jbl, ob);
    // delta1 = (delta2 W2^T) (1 - h1^2)
    zero_blk(h);
    gemm<W, kRS>(h, bufB, jc, sm + Lay::kWT, bc);
    times_dtanh(h, bufA, ob, jc);
    if constexpr (TRAIN) acc.b[0] += colsum_rs(h, jbl);
  }
  if constexpr (TRAIN) {
    // h = delta1: dW1 += x^T delta1
    const float4 x0 = ld4(X + jc), x1 = ld4(X + 32 + jc), x2 = ld4(X + 64 + jc);
    float v[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) v[t] = fmaf(x0.x, h[0][t], fmaf(x0.y, h[1][t], fmaf(x0.z, h[2][t], x0.w * h[3][t])));
    acc.w1[0] += rs(v, jbl);
#pragma unroll
    for (int t = 0; t < NT; ++t) v[t] = fmaf(x1.x, h[0][t], fmaf(x1.y, h[1][t], fmaf(x1.z, h[2][t], x1.w * h[3][t])));
    acc.w1[1] += rs(v, jbl);
#pragma unroll
    for (int t = 0; t < NT; ++t) v[t] = fmaf(x2.x, h[0][t], fmaf(x2.y, h[1][t], fmaf(x2.z, h[2][t], x2.w * h[3][t])));
    acc.w1[2] += rs(v, jbl);
  } else if constexpr (BM == kBwdInput) {
    // du/dx_c = sum_f W_1[c][f] delta1_f; the table holds c W_1, scaled for the exp2 tanh
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float w1[NT];
      ldrow(w1, sm + Lay::kW1 + c * W + bc);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float s = 0.0f;
#pragma unroll
        for (int t = 0; t < NT; ++t) s = fmaf(h[q][t], w1[t], s);
        s += __shfl_xor_sync(0xffffffffu, s, 8);
        s += __shfl_xor_sync(0xffffffffu, s, 16);
        gin[q][c] = s * (1.0f / kTanhScale);
      }
    }
  }
  __syncwarp();  // the next tile overwrites X, G and both buffers
}

template <class N, bool BWD, class Epi>
__device__ __forceinline__ void run_tile(const float* sm, float* wp, Acc<N>& acc, int lane, Epi epi) {
  float unused[4][3];
  run_tile<N, BWD ? kBwdTrain : kBwdNone>(sm, wp, acc, lane, epi, unused);
}

// Copy network N's weights (flat layout at params + OFF, global memory) into the CTA's permuted
// tables.  Global rather than constant-bank loads: the permuted reads differ across a warp,
// which the constant cache would serialise.
template <class N>
__device__ __forceinline__ void load_weights(float* sm, const float* __restrict__ params, int OFF) {
  using Lay = Layout<N>;
  constexpr int W = Lay::W, L = Lay::L, NT = Lay::NT;
  const float c = kTanhScale;
  const float* pw = params + OFF;
  for (int e = threadIdx.x; e < (L - 1) * W * W; e += blockDim.x) {
    const int l = e / (W * W), r = e % (W * W), k = r / W, col = r % W, hi = col / NT, t = col % NT;
    const float* wl = pw + N::layer_off(l + 1);
    sm[Lay::kWF + e] = c * __ldg(wl + k * W + hi + 4 * t);
    sm[Lay::kWT + e] = __ldg(wl + (hi + 4 * t) * W + k);
  }
  for (int e = threadIdx.x; e < 3 * W; e += blockDim.x) {
    const int col = e % W, f = col / NT + 4 * (col % NT);
    sm[Lay::kW1 + e] = c * __ldg(pw + (e / W) * W + f);
  }
  for (int e = threadIdx.x; e < L * W; e += blockDim.x) {
    const int l = e / W, col = e % W, f = col / NT + 4 * (col % NT);
    const int boff = l == 0 ? N::layer_off(0) + 3 * W : N::layer_off(l) + W * W;
    sm[Lay::kB + e] = c * __ldg(pw + boff + f);
  }
  for (int e = threadIdx.x; e < W; e += blockDim.x) sm[Lay::kWO + e] = __ldg(pw + N::kOut + e / NT + 4 * (e % NT));
  if (threadIdx.x == 0) sm[Lay::kBO] = __ldg(pw + N::kOut + W);
}

// Add a warp's accumulators into the CTA accumulator (flat layout of network N).
template <class N>
__device__ __forceinline__ void flush_acc(float* cta, const Acc<N>& a, int lane) {
  using Lay = Layout<N>;
  constexpr int W = Lay::W, L = Lay::L, NT = Lay::NT, R = Lay::R;
  const int jbl = lane & 7, ob = lane >> 3;
#pragma unroll
  for (int m = 0; m < L - 1; ++m)
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int t = 0; t < NT; ++t) atomicAdd(cta + N::layer_off(m + 1) + (jbl + 8 * r) * W + ob + 4 * t, a.wh[m][r][t]);
  if (rs_owner<NT>(lane)) {
    const int f = rs_feature<NT>(lane);
    atomicAdd(cta + N::kOut + f, a.wo);
#pragma unroll
    for (int l = 0; l < L; ++l) atomicAdd(cta + (l == 0 ? 3 * W : N::layer_off(l) + W * W) + f, a.b[l]);
#pragma unroll
    for (int c = 0; c < 3; ++c) atomicAdd(cta + c * W + f, a.w1[c]);
  }
  if (lane == 0) atomicAdd(cta + N::kOut + W, a.bo);
}

// Launch modes of the engine.  One launch covers both networks (u- tiles first, then u+).
enum TileMode {
  kTrain = 0,           // bulk tiles (forward, residual, loss, backward) and general tiles (backward)
  kForwardBulk = 1,     // bulk tiles: forward, residual and loss only
  kForwardGeneral = 2,  // general tiles over every job of the job list: u into Workspace::ju
};

// Tiles of one network of one batch: bulk points, bulk tiles, job range [jb, je) and the first
// job of the general tiles (after the jobs the bulk tiles' spare lanes carry).
struct NetTiles {
  int64_t nb, nbt, jb, je, gf, tiles;
};

template <int MODE>
__device__ __forceinline__ NetTiles net_tiles(const Ctl& c, int q) {
  NetTiles t;
  t.nb = q ? c.nbp : c.nbm;
  t.jb = q ? c.jm_pad : 0;
  t.je = q ? c.total : c.jm;
  t.nbt = MODE == kForwardGeneral ? 0 : (t.nb + 3) / 4;
  const int64_t rest = MODE == kForwardGeneral ? t.je - t.jb : t.je - t.jb - 4 * t.nbt;
  const int64_t ngt = MODE == kForwardBulk || rest <= 0 ? 0 : (rest + 31) / 32;
  t.gf = t.jb + (MODE == kTrain ? 4 * t.nbt : 0);
  t.tiles = t.nbt + ngt;
  return t;
}

// Stage layout.  Bulk tile: 4 point records [0, 64), spare-lane coordinates [64, 80) and dL/du
// [80, 84).  General tile: coordinates [0, 128), dL/du [128, 160).  Issues this lane's part of
// tile lt (of network net) into st and commits a cp.async group (an empty one when !valid).
template <int MODE>
__device__ __forceinline__ void issue_tile(const Workspace& w, const NetTiles& nt, int net, int64_t lt, bool valid,
                                           float* st, int lane) {
  constexpr bool BWD = MODE == kTrain;
  if (valid) {
    if (lt < nt.nbt) {
      const float* recs = w.brec + (size_t)(net ? w.B : 0) * kRecFloats;
      if (lane < 16) {
        const int64_t pidx = lt * 4 + (lane >> 2);
        const bool ok = pidx < nt.nb;
        cp_async16(st + 4 * lane, recs + (ok ? pidx : 0) * kRecFloats + 4 * (lane & 3), ok);
      } else if (BWD && lane < 20) {
        const int64_t j = nt.jb + 4 * lt + (lane - 16);
        const bool ok = j < nt.je;
        cp_async16(st + 64 + 4 * (lane - 16), w.jx + (ok ? j : 0), ok);
      } else if (BWD && lane < 24) {
        const int64_t j = nt.jb + 4 * lt + (lane - 20);
        const bool ok = j < nt.je;
        cp_async4(st + 80 + (lane - 20), w.jg + (ok ? j : 0), ok);
      }
    } else {
      const int64_t j = nt.gf + (lt - nt.nbt) * 32 + lane;
      const bool ok = j < nt.je;
      cp_async16(st + 4 * lane, w.jx + (ok ? j : 0), ok);
      if (BWD) cp_async4(st + 128 + lane, w.jg + (ok ? j : 0), ok);
    }
  }
  cp_commit();
}

// Tile lt of network net, its inputs staged in st: forward, bulk residual and loss, and (kTrain)
// the backward into acc.  lsum: this lane's loss partial of the network.
template <class N, int MODE>
__device__ __forceinline__ void do_tile(const Workspace& w, const float* hh, const NetTiles& nt, int net, int64_t lt,
                                        const float* wsm, float* wp, const float* st, Acc<N>& acc, int lane,
                                        double& lsum, float* __restrict__ residual_out) {
  using Lay = Layout<N>;
  constexpr bool BWD = MODE == kTrain;
  float* X = wp + Lay::kX;
  float* G = wp + Lay::kG;
  float* U = wp + Lay::kU;
  float* Av = wp + Lay::kAv;
  const int jc = 4 * (lane & 7);
  const bool lead = (lane >> 3) == 0;  // lanes holding u of jobs jc..jc+3 after the reduction
  if (lt < nt.nbt) {
    // ---- bulk tile: lane = 7 * point + stencil point; with BWD, lanes 28..31 carry four
    // general jobs (their dL/du is known) instead of idling
    const int pl = lane / kStencil, s = lane - kStencil * pl;
    float x[3] = {0.0f, 0.0f, 0.0f};
    float A = 0.0f;
    if (lane < 4 * kStencil) {
      if (lt * 4 + pl < nt.nb) {
        const float* r = st + pl * kRecFloats;
        const float p[3] = {r[kRecP], r[kRecP + 1], r[kRecP + 2]};
        stencil_point(p, hh, s, x);
        A = r[kRecA + s];
      }
    } else if (BWD) {
      const float* xv = st + 64 + 4 * (lane - 4 * kStencil);
      x[0] = xv[0];
      x[1] = xv[1];
      x[2] = xv[2];
      G[lane] = st[80 + lane - 4 * kStencil];
    }
    // the residual's point records, for lanes 0..3 (point `lane` of the tile)
    int32_t rslot = -1;
    float r_lhs0 = 0.0f, r_diag = 1.0f, r_rod = 0.0f;
    if (lane < 4 && lt * 4 + lane < nt.nb) {
      const float* r = st + lane * kRecFloats;
      rslot = __float_as_int(r[kRecSlot]);
      r_lhs0 = r[kRecLhs0];
      r_diag = r[kRecDiag];
      r_rod = r[kRecRod];
    }
    X[lane] = x[0];
    X[32 + lane] = x[1];
    X[64 + lane] = x[2];
    Av[lane] = A;
    __syncwarp();
    const float Bf = (float)w.B;
    run_tile<N, BWD>(wsm, wp, acc, lane, [&](const float (&u)[4]) {
      if (lead) st4(U + jc, u[0] * Av[jc], u[1] * Av[jc + 1], u[2] * Av[jc + 2], u[3] * Av[jc + 3]);
      __syncwarp();
      // lanes 0..3: residual of point `lane`; then dL/du of its 7 jobs
      if (lane < 4) {
        float gc = 0.0f;
        if (rslot >= 0) {
          float lhs = r_lhs0;
#pragma unroll
          for (int q = 0; q < kStencil; ++q) lhs += U[kStencil * lane + q];
          const float qv = lhs / r_diag;
          const float r0 = nan_to_num(qv) - r_rod;
          const float Pv = w.pre_P ? w.pre_P[rslot] : 1.0f;  // learned preconditioner
          const float r = Pv * r0;
          if (w.pre_P) w.pre_r0[rslot] = r0;
          gc = isfinite(qv) ? (r / Bf) * Pv / r_diag : 0.0f;
          lsum += 0.5 * (double)r * (double)r;
          if (residual_out) residual_out[rslot] = r;
        }
        if (BWD) {
#pragma unroll
          for (int q = 0; q < kStencil; ++q) G[kStencil * lane + q] = gc * Av[kStencil * lane + q];
        }
      }
    });
  } else {
    // ---- general tile: 32 jobs of the job list; kTrain: dL/du known from the residual;
    // kForwardGeneral: u of each job to ju
    X[lane] = st[4 * lane];
    X[32 + lane] = st[4 * lane + 1];
    X[64 + lane] = st[4 * lane + 2];
    if (BWD) G[lane] = st[128 + lane];
    __syncwarp();
    const int64_t j0 = nt.gf + (lt - nt.nbt) * 32 + jc, je = nt.je;
    run_tile<N, BWD>(wsm, wp, acc, lane, [&](const float (&u)[4]) {
      if (MODE == kForwardGeneral && lead) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (j0 + q < je) w.ju[j0 + q] = u[q];
      }
    });
  }
}

// One launch for both networks.  Bulk tiles hold 4 points x 7 stencil jobs (residual and loss
// formed in the warp); general tiles hold 32 jobs of the job list.  Writes the per-CTA loss
// partials floss[net][blockIdx.x], residual_out of the bulk slots and, in kTrain, the partial
// gradient row blockIdx.x (both networks' columns).
template <class N, int MODE, int NW>
__global__ void __launch_bounds__(32 * NW, warps_per_sm<N>() / NW) k_tile(PtsH ph, const int32_t* __restrict__ ids,
                                                                         const __grid_constant__ Workspace w,
                                                                         dips_records_t rec, int off_p,
                                                                         float* __restrict__ residual_out) {
  using Lay = Layout<N>;
  using Cta = CtaLayout<N, NW>;
  constexpr bool BWD = MODE == kTrain;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  load_weights<N>(sm, w.params, 0);
  load_weights<N>(sm + Lay::kNetW, w.params, off_p);
  if (BWD)
    for (int i = threadIdx.x; i < 2 * Cta::kAccStride; i += blockDim.x) sm[Cta::kAcc + i] = 0.0f;
  // per network (u- then u+); read per tile from shared memory, not held in registers
  __shared__ NetTiles s_nt[2];
  if (threadIdx.x < 2) s_nt[threadIdx.x] = net_tiles<MODE>(*w.ctl, threadIdx.x);
  __syncthreads();
  float* wp = sm + Lay::kWarp0 + warp * Lay::kWarpFloats;
  Acc<N> acc;
  acc.clear();
  const int64_t tiles_m = s_nt[0].tiles, tiles = tiles_m + s_nt[1].tiles;
  const volatile NetTiles* snt = s_nt;
  auto nt_of = [&](int net) {
    NetTiles t;
    t.nb = snt[net].nb;
    t.nbt = snt[net].nbt;
    t.jb = snt[net].jb;
    t.je = snt[net].je;
    t.gf = snt[net].gf;
    t.tiles = 0;
    return t;
  };
  const float hh[3] = {ph.h[0], ph.h[1], ph.h[2]};  // registers, not a local copy of ph
  double lsum0 = 0.0, lsum1 = 0.0;

  float* stage0 = wp + Lay::kStage;
  auto issue = [&](int64_t t, float* st) {
    const int net = t >= tiles_m ? 1 : 0;
    issue_tile<MODE>(w, nt_of(net), net, net ? t - tiles_m : t, t < tiles, st, lane);
  };
  const int64_t stride = (int64_t)gridDim.x * NW;
  int64_t tile = (int64_t)blockIdx.x * NW + warp;
  issue(tile, stage0);
  int sidx = 0;
  int cur = -1;  // network of the accumulators
  for (; tile < tiles; tile += stride, sidx ^= 1) {
    issue(tile + stride, stage0 + (sidx ^ 1) * Lay::kStageFloats);
    cp_wait<1>();  // this tile's copies have landed
    __syncwarp();
    const int net = tile < tiles_m ? 0 : 1;
    if (BWD && net != cur) {  // tiles come in increasing order: at most one switch, u- to u+
      if (cur >= 0) {
        flush_acc<N>(sm + Cta::kAcc + cur * Cta::kAccStride, acc, lane);
        acc.clear();
      }
      cur = net;
    }
    do_tile<N, MODE>(w, hh, nt_of(net), net, net ? tile - tiles_m : tile, sm + net * Lay::kNetW, wp,
                     stage0 + sidx * Lay::kStageFloats, acc, lane, net ? lsum1 : lsum0, residual_out);
  }
  cp_wait<0>();
  // loss partials of the CTA, per network
  double* wl = reinterpret_cast<double*>(sm + Cta::kLoss);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    double v = q ? lsum1 : lsum0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) wl[2 * warp + q] = v;
  }
  if (BWD && cur >= 0) flush_acc<N>(sm + Cta::kAcc + cur * Cta::kAccStride, acc, lane);
  __syncthreads();
  if (MODE != kForwardGeneral && threadIdx.x < 2) {
    const int q = threadIdx.x;
    double t = 0.0;
    for (int k = 0; k < NW; ++k) t += wl[2 * k + q];
    w.floss[q * kLossSlots + blockIdx.x] = t;
    if (blockIdx.x == 0) {
      w.ctl->floss_n[q] = gridDim.x;
      if (BWD) w.ctl->grad_rows[q] = gridDim.x;
    }
  }
  if (BWD) {
    float* row = w.partials + (size_t)blockIdx.x * w.n_params;
    for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) {
      row[i] = sm[Cta::kAcc + i];
      row[off_p + i] = sm[Cta::kAcc + Cta::kAccStride + i];
    }
  }
}

constexpr int kMaxInstances = 256;  // instances per multi-instance launch

// The persistent launch of a multi-instance step: one launch for every tile of every instance
// of the table.  Work comes in chunks of NW consecutive tiles of one instance (one tile per
// warp); each CTA takes one contiguous range of chunks, so that it meets an instance in one run
// and crosses few instance boundaries (each costs a weight reload and a row write).  On
// entering an instance the CTA loads its two networks' weights; on leaving it, it adds its loss
// partials and (kTrain) its gradient row into the next free slot of that instance
// (Ctl::floss_n, Ctl::grad_rows, counted with atomics; the per-step expansion reset them).
template <class N, int MODE, int NW>
__global__ void __launch_bounds__(32 * NW, warps_per_sm<N>() / NW) k_tile_multi(const Inst* __restrict__ T, int n_inst,
                                                                               int off_p) {
  using Lay = Layout<N>;
  using Cta = CtaLayout<N, NW>;
  constexpr bool BWD = MODE == kTrain;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ int64_t s_chunk0[kMaxInstances + 1];  // first chunk of each instance
  __shared__ NetTiles s_nt[2];
  if (threadIdx.x == 0) {
    int64_t c = 0;
    for (int i = 0; i < n_inst; ++i) {
      s_chunk0[i] = c;
      const Ctl& ct = *T[i].w.ctl;
      const int64_t tiles = net_tiles<MODE>(ct, 0).tiles + net_tiles<MODE>(ct, 1).tiles;
      c += (tiles + NW - 1) / NW;
    }
    s_chunk0[n_inst] = c;
  }
  __syncthreads();
  const int64_t chunks = s_chunk0[n_inst];
  float* wp = sm + Lay::kWarp0 + warp * Lay::kWarpFloats;
  double* wl = reinterpret_cast<double*>(sm + Cta::kLoss);
  Acc<N> acc;
  acc.clear();
  double lsum0 = 0.0, lsum1 = 0.0;
  int cur = -1;   // network of the warp's accumulators
  int inst = -1;  // the CTA's instance
  const volatile NetTiles* snt = s_nt;
  auto nt_of = [&](int net) {
    NetTiles t;
    t.nb = snt[net].nb;
    t.nbt = snt[net].nbt;
    t.jb = snt[net].jb;
    t.je = snt[net].je;
    t.gf = snt[net].gf;
    t.tiles = snt[net].tiles;
    return t;
  };
  // leave instance `inst`: warps add their accumulators and loss partials into the CTA's, which
  // go to the instance's next free slots
  __shared__ int64_t s_row;
  auto leave = [&]() {
    const Workspace& w = T[inst].w;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      double v = q ? lsum1 : lsum0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) wl[2 * warp + q] = v;
    }
    lsum0 = lsum1 = 0.0;
    if (BWD && cur >= 0) flush_acc<N>(sm + Cta::kAcc + cur * Cta::kAccStride, acc, lane);
    acc.clear();
    cur = -1;
    __syncthreads();
    if (MODE != kForwardGeneral && threadIdx.x < 2) {
      const int q = threadIdx.x;
      double t = 0.0;
      for (int k = 0; k < NW; ++k) t += wl[2 * k + q];
      const unsigned long long slot =
          atomicAdd(reinterpret_cast<unsigned long long*>(&w.ctl->floss_n[q]), 1ull);
      w.floss[q * kLossSlots + slot] = t;
      if (BWD) {
        const unsigned long long r =
            atomicAdd(reinterpret_cast<unsigned long long*>(&w.ctl->grad_rows[q]), 1ull);
        if (q == 0) s_row = (int64_t)r;
      }
    }
    if (BWD) {
      __syncthreads();
      float* row = w.partials + (size_t)s_row * w.n_params;
      for (int i = threadIdx.x; i < N::kParams; i += blockDim.x) {
        row[i] = sm[Cta::kAcc + i];
        row[off_p + i] = sm[Cta::kAcc + Cta::kAccStride + i];
        sm[Cta::kAcc + i] = 0.0f;
        sm[Cta::kAcc + Cta::kAccStride + i] = 0.0f;
      }
    }
    __syncthreads();
  };
  if (BWD)
    for (int i = threadIdx.x; i < 2 * Cta::kAccStride; i += blockDim.x) sm[Cta::kAcc + i] = 0.0f;
  float* stage0 = wp + Lay::kStage;
  int next_inst = 0;
  int sidx = 0;
  bool have = false;  // stage sidx already holds this chunk's tile (prefetched in the last round)
  // a contiguous range of chunks per CTA: it crosses at most a few instance boundaries
  const int64_t per = (chunks + gridDim.x - 1) / gridDim.x;
  const int64_t c_end = min(chunks, (int64_t)(blockIdx.x + 1) * per);
  for (int64_t c = (int64_t)blockIdx.x * per; c < c_end; ++c, sidx ^= 1) {
    while (next_inst < n_inst && c >= s_chunk0[next_inst + 1]) ++next_inst;  // instance of chunk c
    if (next_inst != inst) {
      if (inst >= 0) leave();
      inst = next_inst;
      const Inst& I = T[inst];
      load_weights<N>(sm, I.w.params, 0);
      load_weights<N>(sm + Lay::kNetW, I.w.params, off_p);
      if (threadIdx.x < 2) s_nt[threadIdx.x] = net_tiles<MODE>(*I.w.ctl, threadIdx.x);
      __syncthreads();
      have = false;
    }
    const Inst& I = T[inst];
    const int64_t tiles_m = snt[0].tiles, tiles = tiles_m + snt[1].tiles;
    auto where = [&](int64_t cc, int& net, int64_t& lt) {  // network and net-local tile of chunk cc
      const int64_t t = (cc - s_chunk0[inst]) * NW + warp;
      net = t < tiles_m ? 0 : 1;
      lt = net ? t - tiles_m : t;
      return t;
    };
    int net;
    int64_t lt;
    const int64_t tile = where(c, net, lt);
    const NetTiles nt = nt_of(net);
    if (!have) issue_tile<MODE>(I.w, nt, net, lt, tile < tiles, stage0 + sidx * Lay::kStageFloats, lane);
    // the next chunk of this CTA, when it is in the same instance: its copies run under this tile
    const int64_t c2 = c + 1;
    have = c2 < c_end && c2 < s_chunk0[inst + 1];
    {
      int net2 = 0;
      int64_t lt2 = 0;
      const int64_t t2 = have ? where(c2, net2, lt2) : tiles;
      issue_tile<MODE>(I.w, nt_of(net2), net2, lt2, t2 < tiles, stage0 + (sidx ^ 1) * Lay::kStageFloats, lane);
    }
    cp_wait<1>();  // this chunk's copies have landed
    __syncwarp();
    if (tile < tiles) {
      if (BWD && net != cur) {
        if (cur >= 0) {
          flush_acc<N>(sm + Cta::kAcc + cur * Cta::kAccStride, acc, lane);
          acc.clear();
        }
        cur = net;
      }
      const float hh[3] = {I.rec.h[0], I.rec.h[1], I.rec.h[2]};
      do_tile<N, MODE>(I.w, hh, nt, net, lt, sm + net * Lay::kNetW, wp, stage0 + sidx * Lay::kStageFloats, acc, lane,
                       net ? lsum1 : lsum0, nullptr);
    }
  }
  cp_wait<0>();
  if (inst >= 0) leave();
}

// u and du/dx at n points (evaluate_solution_and_gradients, trainer.py:929-977): tiles of 32
// consecutive points, the network of each point chosen by the sign of phi.  A tile whose points
// all lie on one side runs that network once; a tile that straddles the interface runs both
// and keeps each point's own.
template <class N, int NW>
__global__ void __launch_bounds__(32 * NW, warps_per_sm<N>() / NW) k_tile_eval(const float* __restrict__ pts,
                                                                              const float* __restrict__ phi, int64_t n,
                                                                              const float* __restrict__ params,
                                                                              int off_p, float* __restrict__ u_out,
                                                                              float* __restrict__ g_out) {
  using Lay = Layout<N>;
  extern __shared__ float4 smem4[];
  float* sm = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  load_weights<N>(sm, params, 0);
  load_weights<N>(sm + Lay::kNetW, params, off_p);
  __syncthreads();
  float* wp = sm + Lay::kWarp0 + warp * Lay::kWarpFloats;
  float* X = wp + Lay::kX;
  const int jc = 4 * (lane & 7);
  const bool lead = (lane >> 3) == 0;
  Acc<N> unused;
  const int64_t tiles = (n + 31) / 32;
  for (int64_t tile = (int64_t)blockIdx.x * NW + warp; tile < tiles; tile += (int64_t)gridDim.x * NW) {
    const int64_t i = tile * 32 + lane;
    const bool ok = i < n;
    X[lane] = ok ? pts[3 * i] : 0.0f;
    X[32 + lane] = ok ? pts[3 * i + 1] : 0.0f;
    X[64 + lane] = ok ? pts[3 * i + 2] : 0.0f;
    const bool side = ok && phi[i] >= 0.0f;
    const unsigned on_p = __ballot_sync(0xffffffffu, side), on_m = __ballot_sync(0xffffffffu, ok && !side);
    __syncwarp();
#pragma unroll 1
    for (int net = 0; net < 2; ++net) {
      const unsigned mine = net ? on_p : on_m;
      if (!mine) continue;
      float gin[4][3];
      float uv[4];
      run_tile<N, kBwdInput>(sm + net * Lay::kNetW, wp, unused, lane,
                             [&](const float (&u)[4]) {
#pragma unroll
                               for (int q = 0; q < 4; ++q) uv[q] = u[q];
                             },
                             gin);
      if (lead) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (!((mine >> (jc + q)) & 1u)) continue;
          const int64_t j = tile * 32 + jc + q;
          u_out[j] = uv[q];
          if (g_out) {
            g_out[3 * j] = gin[q][0];
            g_out[3 * j + 1] = gin[q][1];
            g_out[3 * j + 2] = gin[q][2];
          }
        }
      }
    }
  }
}

}  // namespace tile
