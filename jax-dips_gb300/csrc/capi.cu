// Error state and version of the dips_gb300 C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "dips_common.cuh"

namespace dips {

static thread_local char g_err[512] = "no error";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
  return DIPS_E_CUDA;
}

}  // namespace dips

extern "C" const char* dips_last_error(void) { return dips::g_err; }

extern "C" const char* dips_version(void) { return "dips_gb300 0.1 (sm_103a)"; }

// FP32 FMA throughput probe: the FP32-pipe roofline denominator (not on the training path).
// Each thread runs 8 independent FMA chains of `iters` steps; out receives one value per
// thread so the chains are not optimised away.
__global__ void k_fma_probe(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-3f, x2 = x0 + 2e-3f, x3 = x0 + 3e-3f;
  float x4 = x0 + 4e-3f, x5 = x0 + 5e-3f, x6 = x0 + 6e-3f, x7 = x0 + 7e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fmaf(x0, a, b);
      x1 = fmaf(x1, a, b);
      x2 = fmaf(x2, a, b);
      x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b);
      x5 = fmaf(x5, a, b);
      x6 = fmaf(x6, a, b);
      x7 = fmaf(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

extern "C" int dips_fp32_fma_probe(float* out, int32_t blocks, int32_t iters, cudaStream_t stream) {
  DIPS_REQUIRE(out && blocks > 0 && iters > 0, DIPS_E_ARG, "dips_fp32_fma_probe: bad argument");
  k_fma_probe<<<blocks, 256, 0, stream>>>(out, iters, 0.999999f, 1e-7f);
  DIPS_CHECK_LAUNCH("dips_fp32_fma_probe");
  return DIPS_OK;
}
