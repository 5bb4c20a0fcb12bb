// Types shared by the arch-independent and the per-network-shape translation units of the
// residual path: the step workspace and the per-shape kernel table.
#pragma once

#include "dips_common.cuh"

namespace dips {

constexpr int kScanBlock = 1024;
constexpr int kAdjThreads = 256;     // adjoint CTA: 8 warps
constexpr int kAdjGrid = 152 * 2;    // two adjoint CTAs per SM (GB300 has 152 SMs)

// ----------------------------------------------------------------------------------------
// workspace
// ----------------------------------------------------------------------------------------
struct Ctl {
  int64_t jm, jp, jm_pad, total;
  int64_t overflow;  // 1 when the batch's jobs exceed the workspace's job capacity
};

struct Workspace {
  Ctl* ctl;
  int32_t* cm;
  int32_t* cp;
  int64_t* om;
  int64_t* op;
  float* gs;
  float* res;
  int64_t* blk;      // [2*nblk] block sums, then block offsets
  double* lossp;     // [nres] loss partials
  int32_t* jslot;
  uint16_t* jcode;
  float* jA;
  float* ju;
  float* partials;   // [grid][P]
  float* grad;       // [P]
  int64_t nblk, nres, jcap;
  int grid;
  int n_params;      // row stride of partials
};

struct PtsH {
  const float* pts;
  float h[3];
};

__device__ __forceinline__ int64_t batch_pid(const int32_t* ids, int64_t b) { return ids ? (int64_t)ids[b] : b; }

__device__ __forceinline__ void job_point(const PtsH& ph, const int32_t* ids, int32_t slot, uint16_t code, float x[3]) {
  const int64_t pid = batch_pid(ids, slot);
  const float p[3] = {ph.pts[3 * pid], ph.pts[3 * pid + 1], ph.pts[3 * pid + 2]};
  job_coords(p, ph.h, code, x);
}

// Kernels and launches of one DoubleMLP shape (one translation unit per shape, each with
// its own constant-bank copy of the weights).
struct ArchOps {
  int m_layers, m_width, p_layers, p_width;
  int n_params;
  int (*load_params)(const float* params, cudaStream_t s);
  int (*job_forward)(const PtsH& ph, const int32_t* ids, const Workspace& w, cudaStream_t s);
  int (*job_adjoint)(const PtsH& ph, const int32_t* ids, const Workspace& w, cudaStream_t s);
  int (*mlp_eval)(const float* pts, const float* phi, int64_t n, float* u, float* g, cudaStream_t s);
};

}  // namespace dips
