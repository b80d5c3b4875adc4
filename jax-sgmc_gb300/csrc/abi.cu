// Error plumbing shared by every entry point: a thread-local message for the
// last failing call and a helper that turns a CUDA launch error into a status.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace gbsgmc {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    return set_error(GBSGMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  return GBSGMC_OK;
}

}  // namespace gbsgmc

extern "C" const char* gbsgmc_last_error(void) { return gbsgmc::g_last_error; }

extern "C" int gbsgmc_version(void) { return 100; }  // 0.1.0
