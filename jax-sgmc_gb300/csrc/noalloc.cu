// The fused SGLD step for callers that cannot allocate device memory.
//
// gbsgmc_sgld_glm_step needs scratch for the per-slice partial gradients,
// partial sums and ticket counters, and expects the caller to allocate it.
// Some callers cannot do that: code running inside another runtime's device
// memory pool (an XLA FFI handler whose framework has already reserved most
// of HBM, so a cudaMalloc beside it fails or fragments the pool), code issued
// while a CUDA graph is being captured (cudaMalloc/cudaFree are not stream
// work and cudaFree synchronises the device), and latency-bound loops that
// must not pay for allocation.  This entry point takes the scratch from a
// fixed-size array compiled into the library instead.  The array lives in
// every GPU's memory from the moment the library's module is loaded on that
// GPU until the process exits.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr size_t kStaticScratchBytes = GBSGMC_STATIC_SCRATCH_BYTES;

// The scratch itself.  In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_sgld_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (with that device current) and cached.
int scratch_on_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "sgld_glm_step_noalloc: cudaGetDevice: %s",
                     cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(GBSGMC_ERR_UNSUPPORTED,
                     "sgld_glm_step_noalloc: device ordinal %d >= %d", dev,
                     kMaxDevices);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sgld_scratch);
    if (e != cudaSuccess || p == nullptr)
      return set_error(GBSGMC_ERR_CUDA,
                       "sgld_glm_step_noalloc: cudaGetSymbolAddress: %s",
                       cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return GBSGMC_OK;
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_sgld_glm_step_noalloc(
    const gbsgmc_glm* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, float* w_dev, float* v_dev, float alpha, float lmbd,
    const gbsgmc_sched* sched, const gbsgmc_noise* noise, double* U_dev,
    double* lk_var_dev, float* samples_dev, double* sample_lik_dev,
    int* status_dev, gbsgmc_stream_t stream) {
  if (model == nullptr)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step_noalloc: null model");
  if (chains < 0 || n < 0 || model->d < 1)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step_noalloc: bad size");
  if (chains == 0 || n == 0) return GBSGMC_OK;
  const size_t need = glm_ws_bytes(chains, n, model->d);
  if (need > kStaticScratchBytes)
    return set_error(GBSGMC_ERR_SHAPE,
                     "sgld_glm_step_noalloc: %d chains x %d rows x d=%d need "
                     "%zu bytes of scratch; the static scratch holds %zu",
                     chains, n, model->d, need, kStaticScratchBytes);
  void* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc != GBSGMC_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The array keeps whatever the previous call left: clear the part this
  // call uses (the ticket counters must start at zero).
  const cudaError_t e = cudaMemsetAsync(scratch, 0, need, s);
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "sgld_glm_step_noalloc: memset: %s",
                     cudaGetErrorString(e));
  return glm_sgld_step(model, chains, n, idx_dev, idx_stride, w_dev, v_dev,
                       alpha, lmbd, sched, noise, U_dev, lk_var_dev,
                       samples_dev, sample_lik_dev, scratch,
                       kStaticScratchBytes, status_dev, s, GlmTune{});
}
