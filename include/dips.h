/*
 * dips.h -- C ABI of the GB300 (sm_103a) NBM jump-condition finite-volume residual.
 *
 * Every pointer argument is a device pointer owned by the caller (torch tensors, XLA
 * buffers, cudaMalloc'd memory) unless the comment says "host".  Work runs on the
 * cudaStream_t passed in; no entry point synchronises the device.  Each function
 * returns 0 on success or a nonzero DIPS_E_* code; dips_last_error() gives the text
 * of the last failure on the calling thread.  No C++ exception crosses this ABI.
 *
 * Layouts
 *   points      float32 [n][3], row-major (x, y, z)               (domain/mesh.py:125-129)
 *   level set   ghosted float32 cube [(nx+2)][(ny+2)][(nz+2)], C order, built by
 *               dips_phi_ghost_layer from the [nx][ny][nz] samples  (domain/interpolate.py:762-816)
 *   params      float32 flat vector: net u- then net u+; per net and hidden layer
 *               W[in][out] row-major then b[out]; output layer W[width] then b[1].
 *               This is the haiku tree order of double_mlp/~mlp_{m,p}_fn/linear{,_1,..}
 *               (nn/mlp/MLP.py:101-139) with w before b.  With the learned preconditioner
 *               its parameters follow, in the same per-layer order (first layer 26 x width).
 *   job code    uint16: stencil point j (0..6: ijk, i-1, i+1, j-1, j+1, k-1, k+1) times 27
 *               plus regression-cube vertex k (0..26, x fastest), bit 15 set when the
 *               u+ network evaluates the point (phi >= 0, nn/mlp/MLP.py:98).
 */
#ifndef DIPS_H_
#define DIPS_H_

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DIPS_OK = 0,
  DIPS_E_ARG = 1,        /* invalid argument (null pointer, bad size, unsupported shape) */
  DIPS_E_CUDA = 2,       /* a CUDA call failed */
  DIPS_E_WORKSPACE = 3,  /* workspace too small */
  DIPS_E_UNSUPPORTED = 4 /* network shape without a compiled kernel, or a feature the entry
                            point does not take (nonlinear records, the learned preconditioner) */
};

/* Level-set grid: ghosted samples and ghosted coordinates (n+2 each). */
typedef struct {
  const float* phi_gh;
  const float* xg;
  const float* yg;
  const float* zg;
  int32_t nx, ny, nz; /* unghosted sizes */
  /* bounds of the level-set grid, used by the box-boundary test
     (solvers/poisson/discretization.py:60-65, :319-333) */
  float xmin, xmax, ymin, ymax, zmin, zmax;
} dips_levelset_t;

/* Coefficient samples at the query points the geometry kernels emit (the user's
   coefficient callables are evaluated by the host between classify/queries and assemble). */
typedef struct {
  const float* mu_m_face; /* [n][6] face centres imh, iph, jmh, jph, kmh, kph */
  const float* mu_p_face; /* [n][6] */
  const float* k_m;       /* [n] */
  const float* k_p;       /* [n] */
  const float* f_m;       /* [n] */
  const float* f_p;       /* [n] */
  const float* g;         /* [n] Dirichlet value at the point */
  const float* beta_tri;  /* [3 * sum n_tri] beta at interface-triangle vertices */
  const float* mu_m_s;    /* [sum n_xs] mu- at crossed stencil points */
  const float* mu_p_s;    /* [sum n_xs] mu+ at crossed stencil points */
  const float* alpha_r;   /* [sum n_xs] alpha at the projection r = s - phi(s) n */
  const float* beta_r;    /* [sum n_xs] beta at r */
  const float* mu_m_r;    /* [sum n_xs] mu- at r */
  const float* mu_p_r;    /* [sum n_xs] mu+ at r */
  float beta_origin;      /* beta(0,0,0): the reference also integrates its zero-padding triangles */
} dips_coeffs_t;

/* Per-point residual records of one stencil spacing h (one "level"). */
typedef struct {
  const float* pts;         /* [n][3] */
  int64_t n_pts;
  float h[3];
  const float* lhs0;        /* [n] constant part of lhs (jump terms) */
  const float* diag;        /* [n] diagonal coefficient (discretization.py:381-386) */
  const float* rod;         /* [n] nan_to_num(rhs / diag) */
  const int32_t* cnt;       /* [n] jobs of the point */
  const int32_t* cnt_m;     /* [n] of which u- network jobs */
  const int64_t* job_off;   /* [n+1] the jobs of point i live in [job_off[i], job_off[i+1]):
                               its cnt_m u- jobs at the start, its cnt - cnt_m u+ jobs at the end */
  const uint16_t* job_code; /* [jobs] */
  const float* job_A;       /* [jobs] lhs coefficient of the network value at the job point */
  const float* coeff26;     /* [n][26] cell coefficients (geom_pp.py:873-901); read only by the
                               learned preconditioner, may be NULL without it */
  const float* bulk_rec;    /* [n][16] optional: each bulk point's packed record
                               (dips_pack_bulk_records), one 64-byte read per point per step;
                               NULL: gathered from the arrays above every step */
  /* Optional nonlinear operators (trainer.py:992-1017; the residual adds
     N-(u-) V- + N+(u+) V+ at an interior point, discretization.py:369).  NULL nl_pt: none.
     With them every point takes the general path (no bulk points); the plain method refuses the
     records (DIPS_E_ARG), the coefficient derivative and the batched instance step
     (dips_instances_prepare) too (DIPS_E_UNSUPPORTED). */
  const float* nl_pt;       /* [n][4] K-, K+, V-, V+ (dips_geometry_assemble_ex): u-/+ at the point
                               = K-/+ + sum over its jobs of the job's weight times its value */
  const float* nl_w;        /* [jobs][2] the job's weights in u- and u+ at the point */
  int32_t nl_kind[2];       /* per network (u-, u+): DIPS_NL_ZERO or DIPS_NL_SINH */
  float nl_c[2];            /* DIPS_NL_SINH: N(u) = c sinh(u) */
} dips_records_t;

#define DIPS_NL_ZERO 0
#define DIPS_NL_SINH 1

typedef struct {
  int32_t m_layers, m_width, p_layers, p_width; /* DoubleMLP hidden layers and widths, tanh */
  /* learned preconditioner (nn/preconditioner.py:10-35, trainer.py:229-243): pre_layers tanh
     layers of width pre_width over the 26 cell coefficients, then one output y, and
     P = 0.5 + pre_scaling * sigmoid(y) multiplies the point's residual
     (discretization.py:339, :419-420).  pre_layers = 0 disables it; widths 8, 16 or 32,
     1 to 3 layers. */
  int32_t pre_layers, pre_width;
  float pre_scaling;
} dips_arch_t;

/* The optimizers of get_optimizer (solvers/optimizers.py:13-97).
   kind DIPS_OPT_ADAM: clip_by_global_norm(max_norm) -> scale_by_adam(b1, b2, eps) ->
     scale_by_schedule -> scale(-1) (chained_adam, :33-54; optax.adam is max_norm = inf and a
     constant rate, decay_rate = 1);
   kind DIPS_OPT_RMSPROP: optax.rmsprop (:82-87): nu = (1 - b2) g^2 + b2 nu (b2 = the rms decay,
     0.9), update -rate g / sqrt(nu + eps), with max_norm clipping if finite; mu is not used.
   schedule DIPS_SCHED_EXPONENTIAL: rate = lr decay_rate^(count / transition_steps);
   DIPS_SCHED_POLYNOMIAL: rate = lr (1 - min(count, transition_steps) / transition_steps)
     (optax.polynomial_schedule with end value 0 and power 1, :25-28).
   A struct with kind and schedule zero is the chained Adam with the exponential schedule. */
typedef struct {
  float lr, decay_rate, transition_steps, max_norm, b1, b2, eps;
  int32_t kind, schedule;
} dips_adam_t;

#define DIPS_OPT_ADAM 0
#define DIPS_OPT_RMSPROP 1
#define DIPS_SCHED_EXPONENTIAL 0
#define DIPS_SCHED_POLYNOMIAL 1

/* ---- errors ------------------------------------------------------------------------- */
/* Text of the last failure on this thread (static storage; never NULL). */
const char* dips_last_error(void);
/* Library version string (host). */
const char* dips_version(void);

/* FP32 FMA throughput probe (the roofline denominator of the FP32-pipe kernels; no
   counterpart in the reference): `blocks` blocks of 256 threads, each thread 8 independent
   chains of 16*iters FMAs (2 FLOP each); out: [blocks*256]. */
int dips_fp32_fma_probe(float* out, int32_t blocks, int32_t iters, cudaStream_t stream);

/* ---- level set: replaces domain/interpolate.py:762-816 and :906-1021 ------------------ */
/* Ghost layer of linear extrapolation around the [nx][ny][nz] samples. */
int dips_phi_ghost_layer(const float* phi, int32_t nx, int32_t ny, int32_t nz, float* phi_gh,
                         cudaStream_t stream);
/* Trilinear interpolation of the ghosted cube at n points (multilinear_interpolation). */
int dips_phi_trilinear(const dips_levelset_t* ls, const float* pts, int64_t n, float* out,
                       cudaStream_t stream);
/* Non-oscillatory quadratic interpolant of the same ghosted field at n points: the trilinear
   value minus 0.5 t (1 - t) min|second difference| per axis over the cell's corners
   (nonoscillatory_quadratic_interpolation, domain/interpolate.py:572-759). */
int dips_phi_quadratic(const dips_levelset_t* ls, const float* pts, int64_t n, float* out, cudaStream_t stream);

/* ---- geometry: replaces geometry/geometric_integrations_per_point.py:201-1009 and
        solvers/poisson/discretization.py:164-519 (the parameter-independent part) ------- */
/* Pass 1: per point, flags (bit 0 box boundary, bits 1-2 crossed(p) as 0/1/2 for -1/0/+1,
   bits 4..17 crossed(s_j) two bits per stencil point, bits 18..24 phi(s_j) >= 0),
   number of real interface triangles of the point's cell, number of interface-crossed
   stencil points, and an upper bound of its jobs. */
int dips_geometry_classify(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                           uint32_t* flags, int32_t* n_tri, int32_t* n_xs, int32_t* job_cap,
                           cudaStream_t stream);
/* Pass 2: query coordinates for the coefficient callables: interface-triangle vertices
   (3 per triangle, at tri_off[i]*3), crossed stencil points and their projections onto
   the interface (at xs_off[i]); offsets are exclusive prefix sums of pass-1 counts. */
int dips_geometry_queries(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                          const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                          float* tri_pts, float* xs_pts, float* xr_pts, cudaStream_t stream);
/* dips_geometry_queries that lists the points with queries (those with an interface stencil
   point) in scratch (dips_geometry_assemble_scratch_bytes(n) bytes, 4-byte aligned, device
   memory) and runs them 32 to a warp; NULL scratch: one pass over every point.  Same outputs. */
int dips_geometry_queries_ex(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                             const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                             float* tri_pts, float* xs_pts, float* xr_pts, void* scratch, size_t scratch_bytes,
                             cudaStream_t stream);
/* Pass 3: the per-point residual records.  job_off ([n+1]) is the exclusive prefix sum of
   job_cap; cnt[i] <= job_cap[i] jobs are written (u- jobs from the front of the point's
   range, u+ jobs from its back).  coeff26
   ([n][26], may be NULL) receives compute_face_centroids_values_plus_minus_at_point and
   beta_int ([n], may be NULL) the interface integral of beta. */
int dips_geometry_assemble(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                           const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                           const int64_t* job_off, const dips_coeffs_t* co, float* lhs0, float* diag,
                           float* rod, int32_t* cnt, int32_t* cnt_m, uint16_t* job_code, float* job_A,
                           float* coeff26, float* beta_int, cudaStream_t stream);
/* dips_geometry_assemble with two optional parts:
   - nl_pt ([n][4]: K-, K+, V-, V+) and nl_w ([jobs][2], job order of job_code): the nonlinear
     operators' arguments as dips_records_t describes them (u_mp_at_point at the point,
     discretization.py:426-519); both NULL: none;
   - scratch (dips_geometry_assemble_scratch_bytes(n) bytes, 4-byte aligned, device memory):
     the points with an interface stencil point are listed there and assembled by a second
     launch, 32 to a warp, instead of a few per warp among bulk points; NULL: one launch.
   The records are the same either way. */
size_t dips_geometry_assemble_scratch_bytes(int64_t n);
int dips_geometry_assemble_ex(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                              const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                              const int64_t* job_off, const dips_coeffs_t* co, float* lhs0, float* diag,
                              float* rod, int32_t* cnt, int32_t* cnt_m, uint16_t* job_code, float* job_A,
                              float* coeff26, float* beta_int, float* nl_pt, float* nl_w, void* scratch,
                              size_t scratch_bytes, cudaStream_t stream);

/* Derivative of the records along a direction in coefficient space (no counterpart in the
   reference, which would take jax.jvp of its assembly): dco holds the derivative of every
   coefficient sample of `co` along the direction (same layout; NULL arrays are zero, e.g. only
   mu_p_face, mu_p_s and mu_p_r set to 1 for d/d mu+ of a constant mu+).  Writes d lhs0, d diag,
   d rod [n] and d job_A [jobs] (job order of dips_geometry_assemble).  The geometry and the
   discrete branches are the records' own, so this is the exact derivative of the records. */
int dips_geometry_assemble_tangent(const dips_levelset_t* ls, const float* pts, int64_t n, const float h[3],
                                   const uint32_t* flags, const int64_t* tri_off, const int64_t* xs_off,
                                   const int64_t* job_off, const dips_coeffs_t* co, const dips_coeffs_t* dco,
                                   float* d_lhs0, float* d_diag, float* d_rod, float* d_job_A, cudaStream_t stream);

/* Packs the record of every bulk point (7 jobs, all of one network) of `rec` into out [n][16]
   (float32: point, lhs0, the 7 stencil coefficients, diag, rod); other points' rows are left
   unwritten.  Pass `out` as rec->bulk_rec afterwards. */
int dips_pack_bulk_records(const dips_records_t* rec, float* out, cudaStream_t stream);

/* ---- residual, loss, adjoint, optimizer: replace Trainer.loss (trainer.py:892-912),
        value_and_grad in Trainer.update (:783-789) and the optax chain ---------------- */
int32_t dips_num_params(const dips_arch_t* arch);
/* 1 if a kernel is compiled for this network shape. */
int32_t dips_arch_supported(const dips_arch_t* arch);
/* Workspace bytes for a step over `batch` points whose jobs total at most max_jobs. */
size_t dips_step_workspace_bytes(const dips_arch_t* arch, int64_t batch, int64_t max_jobs);
/* Loss over a batch: point ids batch_ids[0..B) (NULL = 0..B-1).  loss_out: device double.
   residual_out ([B], may be NULL) receives lhs/diag - rhs/diag per batch slot. */
int dips_residual_fwd(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                      const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                      double* loss_out, float* residual_out, cudaStream_t stream);
/* Gradient of the loss of the preceding dips_residual_fwd call (same workspace) with
   respect to the params: grad_out [num_params]. */
int dips_residual_bwd(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                      const int32_t* batch_ids, int64_t batch, void* workspace, size_t ws_bytes,
                      float* grad_out, cudaStream_t stream);
/* d loss / d theta of the dips_residual_fwd loss along a coefficient direction theta, the
   params fixed (the gradient of the total loss with respect to a physical coefficient such as
   mu+): trec carries the tangent records from dips_geometry_assemble_tangent in its lhs0, diag,
   rod and job_A fields (its other fields are ignored).  dloss_out: device double.  Not for
   arch with the learned preconditioner (DIPS_E_UNSUPPORTED). */
int dips_loss_coeff_tangent(const dips_arch_t* arch, const float* params, const dips_records_t* rec,
                            const dips_records_t* trec, const int32_t* batch_ids, int64_t batch, void* workspace,
                            size_t ws_bytes, double* dloss_out, cudaStream_t stream);
/* One chained-Adam update of params (in place) from grad; mu, nu: [num_params];
   count: device int64 step counter (incremented). */
int dips_adam_step(const dips_arch_t* arch, const dips_adam_t* hp, float* params, const float* grad,
                   float* mu, float* nu, int64_t* count, cudaStream_t stream);
/* Fused training step = residual_fwd + residual_bwd + adam_step.  loss_out: device double. */
int dips_train_step(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu, float* nu,
                    int64_t* count, const dips_records_t* rec, const int32_t* batch_ids, int64_t batch,
                    void* workspace, size_t ws_bytes, double* loss_out, float* grad_out,
                    cudaStream_t stream);
/* Diagnostic form of dips_train_step: same work, plus events[i] (i < n_events; NULL entries
   skipped) recorded on `stream` at the phase boundaries, so that each kernel can be timed live:
   0 start, 1 batch expansion (count, scan, emit), 2 general forward u-, 3 general forward u+,
   4 general residual, 5 fused bulk kernel u-, 6 fused bulk kernel u+, 7 loss, 8 general adjoint
   u-, 9 general adjoint u+, 10 gradient reduction, 11 Adam.  No counterpart in the reference. */
#define DIPS_STEP_EVENTS 12
int dips_train_step_profiled(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu, float* nu,
                             int64_t* count, const dips_records_t* rec, const int32_t* batch_ids, int64_t batch,
                             void* workspace, size_t ws_bytes, double* loss_out, float* grad_out,
                             cudaEvent_t* events, int32_t n_events, cudaStream_t stream);
/* Polls of the 4x64 tensor-core engine's mbarrier waits before a CTA gives up (default 2^24);
   returns the previous value.  A give-up sets the step's error flag: the loss and gradient come
   out NaN, the CTA waits (with the default bound) for its MMAs in flight and frees its tensor
   memory, and the next call starts clean.  For tests of that path; it applies to launches made
   after the call, from any thread.  No counterpart in the reference. */
uint32_t dips_tc_set_wait_limit(uint32_t polls);
/* dips_train_step without a workspace argument, for callers that cannot allocate device
   memory (e.g. an XLA custom-call handler, which gets only the buffers XLA planned for it).
   No counterpart in the reference.  The scratch is a 64 MiB device array inside the library:
   every GPU that loads it keeps the 64 MiB until exit; batches whose workspace for max_jobs
   jobs (dips_step_workspace_bytes) exceeds it fail with DIPS_E_WORKSPACE; the first call on a
   device resolves the array's address (make it before any stream capture) and keeps it for the
   life of the process, so it is invalid after cudaDeviceReset (or any other teardown of the
   device's primary context): do not reset a device between calls; all calls share the array,
   so calls that overlap on the GPU race.  Allocates nothing. */
int dips_train_step_noalloc(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu, float* nu,
                            int64_t* count, const dips_records_t* rec, const int32_t* batch_ids, int64_t batch,
                            int64_t max_jobs, double* loss_out, float* grad_out, cudaStream_t stream);
/* ---- XLA custom calls: replace Trainer.loss (trainer.py:892-912) and its value_and_grad in
        Trainer.update (:783-789) inside a jitted JAX program, as the forward and backward of a
        jax.custom_vjp.  XLA's GPU custom-call ABI with a status argument
        (API_VERSION_STATUS_RETURNING); buffers are device pointers XLA planned:
          dips_xla_loss_fwd  operands: params f32[P], batch ids i32[B]
                             results:  loss f32[], residual f32[B], workspace u8[ws_bytes]
          dips_xla_loss_bwd  operands: params f32[P], batch ids i32[B], cotangent of the loss f32[]
                             results:  d loss/d params (times the cotangent) f32[P], workspace u8[ws_bytes]
        opaque = the bytes of a dips_xla_desc_t.  The handlers allocate nothing (the workspace is
        an XLA result the caller discards); the backward recomputes the forward.  A failure is
        reported through XlaCustomCallStatusSetFailure (found in the process's global symbol
        scope, or set with dips_xla_set_status_fn) and dips_last_error. ------------------------ */
typedef struct XlaCustomCallStatus_ XlaCustomCallStatus; /* opaque, owned by XLA */
typedef void (*dips_xla_status_fn)(XlaCustomCallStatus* status, const char* message, size_t message_len);
#define DIPS_XLA_MAGIC 0x44495053u /* "DIPS" */
typedef struct {
  uint32_t magic;               /* DIPS_XLA_MAGIC */
  uint32_t version;             /* 1 */
  dips_arch_t arch;
  const dips_records_t* rec;    /* host pointer to the level's records, alive while the program runs */
  int64_t batch;                /* B */
  int64_t max_jobs;             /* job bound of any batch of B points of this level */
  uint64_t ws_bytes;            /* size of the workspace result (dips_xla_workspace_bytes) */
} dips_xla_desc_t;
size_t dips_xla_workspace_bytes(const dips_arch_t* arch, int64_t batch, int64_t max_jobs);
int dips_xla_make_desc(const dips_arch_t* arch, const dips_records_t* rec, int64_t batch, int64_t max_jobs,
                       dips_xla_desc_t* out);
void dips_xla_set_status_fn(dips_xla_status_fn fn);
void dips_xla_loss_fwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                       XlaCustomCallStatus* status);
void dips_xla_loss_bwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                       XlaCustomCallStatus* status);

/* ---- many instances trained together (configuration 4; no counterpart in the reference,
        whose LPBE example trains its molecules one after another): each instance has its own
        records, batch, parameters, optimizer state and workspace; all share the network shape
        and the Adam hyper-parameters ----------------------------------------------------- */
typedef struct {
  const dips_records_t* rec;  /* the instance's level (read when the table is prepared) */
  int32_t* batch_ids;         /* [batch] device; drawn by each step when ids_mode >= 0 */
  int64_t batch;
  int64_t n_batches;          /* batches per epoch, for ids drawn from *count (ids_mode >= 0) */
  uint64_t seed;
  int32_t ids_mode;           /* -1: batch_ids given by the caller; 0: consecutive ranges;
                                 1: a seeded permutation per epoch (as dips_batch_ids_device) */
  float* params;
  float* mu;
  float* nu;
  int64_t* count;
  void* workspace;            /* dips_step_workspace_bytes(arch, batch, max jobs) bytes */
  size_t ws_bytes;
  double* loss_out;           /* device double, may be NULL */
  float* grad_out;            /* [num_params] device, may be NULL */
} dips_instance_t;
/* Device bytes of the instance table of n instances. */
size_t dips_instances_table_bytes(int32_t n);
/* Writes the instance table (device memory, dips_instances_table_bytes(n)) and waits for the
   copy (not capturable: call it once, before capturing steps).  n <= 256. */
int dips_instances_prepare(const dips_arch_t* arch, const dips_instance_t* inst, int32_t n, void* table,
                           size_t table_bytes, cudaStream_t stream);
/* One training step of every instance of a prepared table: per phase one launch for all
   instances (batch ids, expansion, the general forward, the general residual, the training
   launch, the gradient tail); the two tile-engine launches are persistent over all instances'
   tiles.  max_batch: the largest batch of the table.  Tile-engine shapes (3x32, 2x16) without
   the learned preconditioner; others return DIPS_E_UNSUPPORTED. */
int dips_train_step_instances(const dips_arch_t* arch, const dips_adam_t* hp, const void* table, int32_t n,
                              int64_t max_batch, cudaStream_t stream);

/* Autotuner (no counterpart in the reference): runs the residual forward on this batch, then
   times each launch configuration of the shape's tunable point kernel (for 3x32: the
   register-blocked engine, one CTA per SM of 12, 10 or 8 warps) and keeps the fastest for
   the current device, process-wide.  Synchronises `stream`; call it before capturing a graph.
   *choice_out (host, may be NULL) receives the warps per CTA chosen, 0 when the shape has
   nothing to tune.  The workspace is left in an unspecified state. */
int dips_autotune(const dips_arch_t* arch, const float* params, const dips_records_t* rec, const int32_t* batch_ids,
                  int64_t batch, void* workspace, size_t ws_bytes, int32_t* choice_out, cudaStream_t stream);

/* Batch ids of batch `index` of an epoch: a seeded bijective permutation of 0..n-1
   (uniform minibatches without replacement), written to ids[0..B).  epoch_index and
   seed select the permutation. */
int dips_batch_ids(int64_t n, int64_t epoch_index, uint64_t seed, int64_t batch_index, int64_t batch,
                   int32_t* ids, cudaStream_t stream);

/* Graph-replay form of dips_batch_ids: the step index is read from the device
   (step_counter, e.g. the Adam step count), batch = step % n_batches and
   epoch = step / n_batches.  mode 0 writes consecutive ranges batch*B + [0, B) (the
   reference's fixed sequential batches, data/data_management.py:104-159); mode 1 the
   seeded per-epoch permutation of dips_batch_ids. */
int dips_batch_ids_device(int64_t n, int64_t batch, int64_t n_batches, uint64_t seed, int32_t mode,
                          const int64_t* step_counter, int32_t* ids, cudaStream_t stream);

/* ---- network evaluation: replaces Trainer.evaluate_solution_fn (trainer.py:836-844)
        and compute_gradient_solution_neural_network (:953-957) --------------------------- */
/* u and grad u (grad_out [n][3], may be NULL) at n points; the network is chosen by
   phi_at (phi >= 0 -> u+). */
int dips_mlp_eval(const dips_arch_t* arch, const float* params, const float* pts, const float* phi_at,
                  int64_t n, float* u_out, float* grad_out, cudaStream_t stream);

/* ---- plain method: the FV system of a nodal vector (replaces Trainer.residual_vector,
        trainer.py:883-890, over compute_Ax_and_b_discrete_fn, discretization.py:522-741)
        and a matrix-free BiCGSTAB on it ---------------------------------------------- */
typedef struct {
  int32_t iterations;       /* BiCGSTAB iterations run */
  int32_t target_iteration; /* first checked iteration with rel_linf <= target, -1 if never */
  int32_t breakdown;        /* 1 if a recurrence scalar became 0 or non-finite */
  double rel_residual;      /* ||b - K x|| / ||b|| at the last check */
  float rel_linf;           /* max|x - u_exact| / max|u_exact| (-1 without u_exact) */
} dips_krylov_stats_t;

/* Residual of a nodal vector u on the grid whose nodes (C order, nx*ny*nz == n_pts) are the
   records' points: out = K u - b, or K u when linear_only is nonzero. */
int dips_fv_residual(const dips_records_t* rec, int32_t nx, int32_t ny, int32_t nz, const float* u,
                     int32_t linear_only, float* out, cudaStream_t stream);
size_t dips_bicgstab_workspace_bytes(int64_t n);
/* Solve K x = b from the initial x (in place).  Every check_every iterations the host reads
   the residual norm (and, with u_exact, the relative max error); the solve stops at
   ||r||/||b|| <= rtol, at max_iter, or -- with u_exact and target_rel_linf > 0 -- as soon as
   the relative max error reaches the target.  stats: host pointer, may be NULL. */
int dips_bicgstab(const dips_records_t* rec, int32_t nx, int32_t ny, int32_t nz, float* x, const float* u_exact,
                  int32_t max_iter, double rtol, int32_t check_every, float target_rel_linf, void* workspace,
                  size_t ws_bytes, dips_krylov_stats_t* stats, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* DIPS_H_ */
