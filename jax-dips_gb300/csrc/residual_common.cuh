// Types shared by the arch-independent and the per-network-shape translation units of the
// residual path: the step workspace and the per-shape kernel table.
#pragma once

#include "dips_common.cuh"

namespace dips {

constexpr int kScanBlock = 1024;
constexpr int kAdjThreads = 256;     // adjoint CTA: 8 warps
constexpr int kAdjGrid = 152 * 2;    // two adjoint CTAs per SM (GB300 has 152 SMs)
constexpr int kFusedThreads = 224;   // fused bulk CTA: one warp per stencil point
constexpr int kFusedGrid = 152 * 2;
constexpr int kTileGrid = 152;  // register-blocked engine: 12 warps per SM (one CTA of 12 by default)
constexpr int kLossSlots = 1024;  // per-network capacity of the per-CTA loss partials
constexpr int kPreGrid = 304;    // CTAs of the preconditioner's backward (partial rows)
constexpr int kPreIn = 26;       // preconditioner input: the cell coefficients

// bulk point record (16 floats): point, lhs0, A of stencil points 0..6, diag, rod, batch slot
constexpr int kReduceThreads = 1024;  // k_reduce_adam: 32 gradient columns x 32 row groups per block
constexpr int kRecP = 0, kRecLhs0 = 3, kRecA = 4, kRecDiag = 11, kRecRod = 12, kRecSlot = 13, kRecFloats = 16;

// ----------------------------------------------------------------------------------------
// workspace
// ----------------------------------------------------------------------------------------
struct Ctl {
  int64_t jm, jp, jm_pad, total;  // jobs of the general points: u-, u+, padded u- count, all
  int64_t overflow;               // 1 when the batch's jobs exceed the workspace's job capacity
  int64_t nbm, nbp;               // bulk points (7 jobs of one network) of the u- / u+ network
  int64_t engine_error;           // nonzero when a tensor-core wait gave up (the loss and gradient become NaN)
  int64_t floss_n[2];             // per-CTA loss partials written by the point kernels of each network
  int64_t grad_rows[2];           // partial gradient rows written for each network
  uint64_t reduce_done;           // blocks of k_reduce_adam that have finished their columns
};

// Step workspace, carved from one caller-owned buffer.  Bulk points go to the fused kernel
// through two slot lists; the other ("general") points are expanded into jobs.
struct Workspace {
  Ctl* ctl;
  int32_t* cm;       // [B] general u- jobs of the slot
  int32_t* cp;       // [B] general u+ jobs
  int64_t* om;       // [B] first u- job
  int64_t* op;       // [B] first u+ job
  int32_t* bk;       // [B] 0 general, 1 bulk u-, 2 bulk u+, 3 invalid id
  int64_t* ob;       // [B] position in its bulk list
  int32_t* bulk;     // [2][B] bulk slot lists (u- then u+)
  float* gs;         // [B] d loss / d lhs of general slots
  int64_t* blk;      // [4*(nblk+1)] block sums, then block offsets
  double* lossp;     // [nres] loss partials of general slots
  double* floss;     // [2][kLossSlots] per-CTA loss partials of the point kernels (count in Ctl::floss_n)
  int32_t* jslot;
  uint16_t* jcode;
  float* jA;
  float* ju;
  float4* jx;        // [jcap] job coordinates (w unused)
  float* jg;         // [jcap] d loss / d u of the job
  float* brec;       // [2][B][16] bulk point records, in bulk-list order (layout: kRec* below)
  float* pre_P;      // [B] learned preconditioner value per slot; NULL when it is off
  float* pre_r0;     // [B] residual before preconditioning (its backward reads it)
  float* pre_partials;  // [kPreGrid][pre_n] partial gradient rows of the preconditioner
  float* partials;   // [grid + fgrid][P] partial gradient rows (count per network in Ctl::grad_rows)
  float* grad;       // [P]
  double* sqp;       // [ceil(P / 32)] squares of the gradient, per block of k_reduce_adam
  const float* params;  // the call's parameters (device): u- net, u+ net, preconditioner
  int64_t nblk, nres, jcap, B;
  int grid, fgrid;
  int n_params;      // row stride of partials
  int pre_n;         // preconditioner parameters (0 when it is off); they follow the networks'
};

struct PtsH {
  const float* pts;
  float h[3];
};

// One problem of a multi-instance step (many instances trained together, one launch per phase
// for all of them): what its kernels need, in a device table that the per-step kernels index
// with blockIdx.y and the persistent tile launch walks.
struct Inst {
  Workspace w;        // carved from the instance's workspace; w.params = its parameters
  dips_records_t rec;  // its level
  int32_t* ids;       // [B] batch ids (drawn on the device when ids_mode >= 0)
  int64_t B;
  int64_t n_batches;  // batches per epoch, for ids drawn from *count
  uint64_t seed;
  int32_t ids_mode;   // -1: ids given; 0: consecutive ranges; 1: seeded permutation per epoch
  int32_t ids_half;   // half-width of the permutation's Feistel network
  float* params;
  float* mu;
  float* nu;
  int64_t* count;
  float* grad;        // [P] (the workspace's when the caller gave none)
  double* loss_out;   // device double, may be NULL
};

__device__ __forceinline__ int64_t batch_pid(const int32_t* ids, int64_t b) { return ids ? (int64_t)ids[b] : b; }

__device__ __forceinline__ void job_point(const PtsH& ph, const int32_t* ids, int32_t slot, uint16_t code, float x[3]) {
  const int64_t pid = batch_pid(ids, slot);
  const float p[3] = {ph.pts[3 * pid], ph.pts[3 * pid + 1], ph.pts[3 * pid + 2]};
  job_coords(p, ph.h, code, x);
}

// Kernels and launches of one DoubleMLP shape (one translation unit per shape).
// Optional CUDA events recorded on the launching stream at the step's phase boundaries
// (slot numbers as in dips_train_step_profiled).  A null Marks pointer records nothing.
struct Marks {
  cudaEvent_t* ev;
  int n;
};
enum MarkSlot {
  kMarkStart = 0,
  kMarkExpand,
  kMarkFwdM,
  kMarkFwdP,
  kMarkResidual,
  kMarkFusedM,
  kMarkFusedP,
  kMarkLoss,
  kMarkAdjM,
  kMarkAdjP,
  kMarkReduce,
  kMarkAdam,
  kMarkCount
};
inline void mark(const Marks* m, int slot, cudaStream_t s) {
  if (m && slot < m->n && m->ev[slot]) cudaEventRecord(m->ev[slot], s);
}

struct ArchOps {
  int m_layers, m_width, p_layers, p_width;
  int n_params;
  int bulk_ok;  // 0: no bulk-point kernel; every point is expanded into jobs
  // hands params to the launches that follow on the calling thread, for a shape whose kernels do
  // not take them from the Workspace (the tcgen05 engine records the pointer); for_eval: the call
  // comes from mlp_eval.  The FP32 shapes read their own call's parameters and do nothing here.
  int (*load_params)(const float* params, int for_eval, cudaStream_t s);
  int (*job_forward)(const PtsH& ph, const int32_t* ids, const Workspace& w, const Marks* mk, cudaStream_t s);
  int (*job_adjoint)(const PtsH& ph, const int32_t* ids, const Workspace& w, const Marks* mk, cudaStream_t s);
  // bulk points: forward, residual, loss partials, residual_out (may be NULL) and, with bwd,
  // the gradient partial rows
  int (*bulk_fused)(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec,
                    float* residual_out, bool bwd, const Marks* mk, cudaStream_t s);
  int (*mlp_eval)(const float* params, const float* pts, const float* phi, int64_t n, float* u, float* g,
                  cudaStream_t s);
  // times the shape's tunable launch configurations on a prepared workspace and keeps the
  // fastest for the current device (NULL: nothing to tune); *chosen = the choice (0: none)
  int (*autotune)(const PtsH& ph, const int32_t* ids, const Workspace& w, const dips_records_t& rec, cudaStream_t s,
                  int* chosen);
  // multi-instance step (tile-engine shapes; NULL otherwise): the general forward and the
  // training launch of every instance of the device table T[0..n) in one persistent launch
  int (*multi_forward)(const Inst* T, int n, cudaStream_t s);
  int (*multi_train)(const Inst* T, int n, cudaStream_t s);
};

// learned preconditioner (implemented in precond.cu)
int pre_num_params(int layers, int width);
bool pre_supported(int layers, int width);
int precond_forward(const dips_arch_t& a, const float* pre_params, const dips_records_t& rec, const int32_t* ids,
                    int64_t B, const Workspace& w, cudaStream_t s);
int precond_backward(const dips_arch_t& a, const float* pre_params, const dips_records_t& rec, const int32_t* ids,
                     int64_t B, const Workspace& w, cudaStream_t s);

}  // namespace dips
