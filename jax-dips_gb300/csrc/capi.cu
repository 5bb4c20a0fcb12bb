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
