// XLA custom-call handlers for the residual loss and its parameter gradient: the two calls a
// jax.custom_vjp of Trainer.loss binds (solvers/poisson/trainer.py:892-912 forward,
// value_and_grad in Trainer.update :783-789 backward).
//
// ABI: XLA's GPU custom-call convention with a status argument ("API_VERSION_STATUS_RETURNING"):
//   void handler(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len,
//                XlaCustomCallStatus* status)
// `buffers` lists the operands, then the results, as device pointers XLA planned.  `opaque`
// carries a dips_xla_desc_t (dips_xla_make_desc) that names the network shape, the level's
// records and the batch.  A handler allocates nothing: its scratch is one more result buffer
// (dips_xla_workspace_bytes bytes) that XLA allocates with the others and the caller discards.
//
// Failures go to XlaCustomCallStatusSetFailure, which the host process provides (jaxlib): the
// function is looked up once with dlsym in the process's global scope, or given explicitly with
// dips_xla_set_status_fn (for a process whose jaxlib was loaded with local symbol scope).  The
// text is also kept for dips_last_error on the calling thread.
#include <dlfcn.h>
#include <string.h>

#include <atomic>

#include "dips_common.cuh"

namespace {

std::atomic<dips_xla_status_fn> g_status_fn{nullptr};
std::atomic<int> g_status_looked_up{0};

dips_xla_status_fn status_fn() {
  dips_xla_status_fn f = g_status_fn.load();
  if (f) return f;
  if (!g_status_looked_up.exchange(1)) {
    void* sym = dlsym(RTLD_DEFAULT, "XlaCustomCallStatusSetFailure");
    if (sym) {
      dips_xla_status_fn expected = nullptr;
      g_status_fn.compare_exchange_strong(expected, reinterpret_cast<dips_xla_status_fn>(sym));
    }
  }
  return g_status_fn.load();
}

void fail(XlaCustomCallStatus* status, int code) {
  (void)code;
  const char* msg = dips_last_error();
  dips_xla_status_fn f = status_fn();
  if (f && status) f(status, msg, strlen(msg));
}

// the double loss the residual kernels write lives at the start of the workspace result;
// the library's workspace follows at a 256-byte offset
constexpr size_t kHead = 256;

__global__ void k_loss_out(const double* __restrict__ loss64, float* __restrict__ loss) { *loss = (float)*loss64; }

__global__ void k_scale_grad(float* __restrict__ grad, int n, const float* __restrict__ g) {
  const float s = *g;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) grad[i] *= s;
}

int check_desc(const char* opaque, size_t opaque_len, const dips_xla_desc_t** out) {
  DIPS_REQUIRE(opaque && opaque_len == sizeof(dips_xla_desc_t), DIPS_E_ARG,
               "dips_xla: opaque is %zu bytes, a dips_xla_desc_t is %zu", opaque_len, sizeof(dips_xla_desc_t));
  const dips_xla_desc_t* d = reinterpret_cast<const dips_xla_desc_t*>(opaque);
  DIPS_REQUIRE(d->magic == DIPS_XLA_MAGIC && d->version == 1, DIPS_E_ARG,
               "dips_xla: opaque is not a dips_xla_desc_t (magic %08x, version %u)", d->magic, d->version);
  DIPS_REQUIRE(d->rec && d->batch > 0 && d->max_jobs >= 0, DIPS_E_ARG, "dips_xla: descriptor without records or batch");
  const size_t need = dips_step_workspace_bytes(&d->arch, d->batch, d->max_jobs);
  DIPS_REQUIRE(need > 0, DIPS_E_UNSUPPORTED, "dips_xla: unsupported network shape");
  DIPS_REQUIRE(d->ws_bytes >= need + kHead, DIPS_E_WORKSPACE,
               "dips_xla: workspace result of %llu bytes, the batch needs %zu", (unsigned long long)d->ws_bytes,
               need + kHead);
  *out = d;
  return DIPS_OK;
}

int loss_fwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len) {
  const dips_xla_desc_t* d = nullptr;
  int st = check_desc(opaque, opaque_len, &d);
  if (st) return st;
  DIPS_REQUIRE(buffers, DIPS_E_ARG, "dips_xla_loss_fwd: no buffers");
  const float* params = static_cast<const float*>(buffers[0]);
  const int32_t* ids = static_cast<const int32_t*>(buffers[1]);
  float* loss = static_cast<float*>(buffers[2]);
  float* residual = static_cast<float*>(buffers[3]);
  unsigned char* ws = static_cast<unsigned char*>(buffers[4]);
  DIPS_REQUIRE(params && ids && loss && residual && ws, DIPS_E_ARG, "dips_xla_loss_fwd: null buffer");
  double* loss64 = reinterpret_cast<double*>(ws);
  st = dips_residual_fwd(&d->arch, params, d->rec, ids, d->batch, ws + kHead, d->ws_bytes - kHead, loss64, residual,
                         stream);
  if (st) return st;
  k_loss_out<<<1, 1, 0, stream>>>(loss64, loss);
  DIPS_CHECK_LAUNCH("dips_xla_loss_fwd");
  return DIPS_OK;
}

int loss_bwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len) {
  const dips_xla_desc_t* d = nullptr;
  int st = check_desc(opaque, opaque_len, &d);
  if (st) return st;
  DIPS_REQUIRE(buffers, DIPS_E_ARG, "dips_xla_loss_bwd: no buffers");
  const float* params = static_cast<const float*>(buffers[0]);
  const int32_t* ids = static_cast<const int32_t*>(buffers[1]);
  const float* g = static_cast<const float*>(buffers[2]);
  float* grad = static_cast<float*>(buffers[3]);
  unsigned char* ws = static_cast<unsigned char*>(buffers[4]);
  DIPS_REQUIRE(params && ids && g && grad && ws, DIPS_E_ARG, "dips_xla_loss_bwd: null buffer");
  double* loss64 = reinterpret_cast<double*>(ws);
  // the forward is recomputed here (the adjoint recomputes activations rather than storing them)
  st = dips_residual_fwd(&d->arch, params, d->rec, ids, d->batch, ws + kHead, d->ws_bytes - kHead, loss64, nullptr,
                         stream);
  if (st) return st;
  st = dips_residual_bwd(&d->arch, params, d->rec, ids, d->batch, ws + kHead, d->ws_bytes - kHead, grad, stream);
  if (st) return st;
  const int n = dips_num_params(&d->arch);
  const int blocks = dips::div_up(n, 256) < 152 ? dips::div_up(n, 256) : 152;
  k_scale_grad<<<blocks, 256, 0, stream>>>(grad, n, g);
  DIPS_CHECK_LAUNCH("dips_xla_loss_bwd");
  return DIPS_OK;
}

}  // namespace

extern "C" void dips_xla_set_status_fn(dips_xla_status_fn fn) { g_status_fn.store(fn); }

extern "C" size_t dips_xla_workspace_bytes(const dips_arch_t* arch, int64_t batch, int64_t max_jobs) {
  const size_t need = dips_step_workspace_bytes(arch, batch, max_jobs);
  return need ? need + kHead : 0;
}

extern "C" int dips_xla_make_desc(const dips_arch_t* arch, const dips_records_t* rec, int64_t batch, int64_t max_jobs,
                                  dips_xla_desc_t* out) {
  DIPS_REQUIRE(arch && rec && out && batch > 0 && max_jobs >= 0, DIPS_E_ARG, "dips_xla_make_desc: bad argument");
  const size_t ws = dips_xla_workspace_bytes(arch, batch, max_jobs);
  DIPS_REQUIRE(ws > 0, DIPS_E_UNSUPPORTED, "dips_xla_make_desc: unsupported network shape");
  memset(out, 0, sizeof(*out));
  out->magic = DIPS_XLA_MAGIC;
  out->version = 1;
  out->arch = *arch;
  out->rec = rec;
  out->batch = batch;
  out->max_jobs = max_jobs;
  out->ws_bytes = ws;
  return DIPS_OK;
}

extern "C" void dips_xla_loss_fwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                                  XlaCustomCallStatus* status) {
  const int st = loss_fwd(stream, buffers, opaque, opaque_len);
  if (st) fail(status, st);
}

extern "C" void dips_xla_loss_bwd(cudaStream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                                  XlaCustomCallStatus* status) {
  const int st = loss_bwd(stream, buffers, opaque, opaque_len);
  if (st) fail(status, st);
}
