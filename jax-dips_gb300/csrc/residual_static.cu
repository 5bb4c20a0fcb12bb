// Training step whose scratch memory is a fixed device array inside this library.
//
// Some callers cannot allocate device memory.  An XLA custom-call handler, for example,
// receives only the operand and result buffers that XLA planned for it, plus a stream: XLA owns
// every byte of device memory, and a handler that called cudaMalloc would block on and disturb
// XLA's asynchronous stream.  Frameworks that reserve the whole device for their own pool
// are in the same position.  dips_train_step_noalloc serves them: it runs exactly the
// dips_train_step pipeline, but its workspace is g_step_scratch below instead of a
// caller-allocated buffer.
//
// Properties a caller must know:
//  * Size limit: kStepScratchBytes (64 MiB).  A batch whose workspace (as computed by
//    dips_step_workspace_bytes for the caller's job bound) exceeds it is rejected with
//    DIPS_E_WORKSPACE before anything is launched.
//  * Every GPU that loads this module keeps the 64 MiB until the process exits.
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call before any
//    stream capture.  The address is kept for the life of the process: after cudaDeviceReset
//    (or any other teardown of the device's primary context) the module is loaded again and
//    the cached address is stale, so do not reset a device between calls.
//  * All calls share the one array and it keeps the previous call's contents.  The step
//    writes every scratch byte it later reads within the same call, so nothing has to be
//    cleared; but two calls that overlap on the GPU (different streams, no ordering between
//    them) race on the array and corrupt each other.
//  * The call itself allocates nothing: no cudaMalloc, cudaFree or allocating library call.

#include <mutex>

#include "dips_common.cuh"

namespace {

constexpr size_t kStepScratchBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

// The scratch.  In host code this name is only a host-side stand-in for the device array:
// a kernel must be given the address returned by cudaGetSymbolAddress, never &g_step_scratch.
static __device__ __align__(256) unsigned char g_step_scratch[kStepScratchBytes];

std::mutex g_mu;
void* g_dev_ptr[kMaxDevices] = {nullptr};

// Device address of g_step_scratch on the current device (resolved once per device).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dips::cuda_status(e, "dips_train_step_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    dips::set_error("dips_train_step_noalloc: device index %d out of range", dev);
    return DIPS_E_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_dev_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_step_scratch);
    if (e != cudaSuccess) return dips::cuda_status(e, "dips_train_step_noalloc: cudaGetSymbolAddress");
    g_dev_ptr[dev] = p;
  }
  *out = g_dev_ptr[dev];
  return DIPS_OK;
}

}  // namespace

extern "C" int dips_train_step_noalloc(const dips_arch_t* arch, const dips_adam_t* hp, float* params, float* mu,
                                       float* nu, int64_t* count, const dips_records_t* rec, const int32_t* batch_ids,
                                       int64_t batch, int64_t max_jobs, double* loss_out, float* grad_out,
                                       cudaStream_t stream) {
  DIPS_REQUIRE(batch > 0 && max_jobs >= 0, DIPS_E_ARG, "dips_train_step_noalloc: bad batch or job bound");
  const size_t need = dips_step_workspace_bytes(arch, batch, max_jobs);
  DIPS_REQUIRE(need > 0, DIPS_E_ARG, "dips_train_step_noalloc: invalid network shape");
  DIPS_REQUIRE(need <= kStepScratchBytes, DIPS_E_WORKSPACE,
               "dips_train_step_noalloc: a batch of %lld points with up to %lld jobs needs %zu bytes of scratch, "
               "more than the built-in %zu bytes; use dips_train_step with a caller-allocated workspace",
               (long long)batch, (long long)max_jobs, need, kStepScratchBytes);
  void* ws = nullptr;
  int st = scratch_address(&ws);
  if (st) return st;
  return dips_train_step(arch, hp, params, mu, nu, count, rec, batch_ids, batch, ws, kStepScratchBytes, loss_out,
                         grad_out, stream);
}
