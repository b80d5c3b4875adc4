// The fused SGLD step for callers that cannot allocate device memory.
//
// gbsgmc_sgld_glm_step needs scratch for the per-slice partial gradients,
// partial sums and ticket counters, and expects the caller to allocate it.
// Some callers cannot do that: code running inside another runtime's device
// memory pool (an XLA FFI handler whose framework has already reserved most
// of HBM, so a cudaMalloc beside it fails or fragments the pool), host code
// that only receives device pointers from its framework and has no allocator
// of its own, and latency-bound loops that must not pay for cudaMalloc and
// the device-wide synchronisation of cudaFree.  This entry point takes the
// scratch from a fixed-size array compiled into the library instead.  The
// array lives in every GPU's memory from the moment the library's module is
// loaded on that GPU until the process exits.
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr size_t kStaticScratchBytes = GBSGMC_STATIC_SCRATCH_BYTES;

// The scratch itself.  In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_sgld_scratch[kStaticScratchBytes];

// Driver calls that identify the current context, resolved at run time
// through the runtime (the library links no libcuda).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct CtxFns {
  CtxGetCurrentFn current = nullptr;
  CtxGetIdFn id = nullptr;
};

const CtxFns& ctx_fns() {
  static CtxFns fns;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fns.current = reinterpret_cast<CtxGetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fns.id = reinterpret_cast<CtxGetIdFn>(p);
  });
  return fns;
}

// The scratch's device address belongs to the module instance of one CUDA
// context: a cudaDeviceReset, or a context the caller made with the driver
// API, loads the module again at another address.  Addresses are therefore
// cached per context, keyed by the context's process-unique id (cuCtxGetId),
// or by the device ordinal where the driver offers no context ids.
struct ScratchEntry {
  unsigned long long key;
  void* addr;
};
constexpr int kMaxEntries = 64;
std::mutex g_scratch_mutex;
ScratchEntry g_scratch[kMaxEntries];
int g_scratch_used = 0;
int g_scratch_next = 0;   // entry replaced when the table is full

int context_key(unsigned long long* key) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "sgld_glm_step_noalloc: cudaGetDevice: %s",
                     cudaGetErrorString(e));
  // With no context current yet (the runtime makes the device's primary
  // context current on its first call that needs one), the key is the
  // device ordinal; the lookup is then repeated once the context exists.
  const CtxFns& f = ctx_fns();
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (f.current != nullptr && f.id != nullptr && f.current(&ctx) == CUDA_SUCCESS &&
      ctx != nullptr && f.id(ctx, &id) == CUDA_SUCCESS) {
    *key = id << 1;   // even: a context id
    return GBSGMC_OK;
  }
  *key = (static_cast<unsigned long long>(dev) << 1) | 1ull;   // odd: an ordinal
  return GBSGMC_OK;
}

// Device address of the scratch in the current context, looked up once per
// context (with its device current) and cached.
int scratch_in_current_context(void** out) {
  unsigned long long key = 0;
  int rc = context_key(&key);
  if (rc != GBSGMC_OK) return rc;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  for (int i = 0; i < g_scratch_used; ++i)
    if (g_scratch[i].key == key) {
      *out = g_scratch[i].addr;
      return GBSGMC_OK;
    }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_sgld_scratch);
  if (e != cudaSuccess || p == nullptr)
    return set_error(GBSGMC_ERR_CUDA,
                     "sgld_glm_step_noalloc: cudaGetSymbolAddress: %s",
                     cudaGetErrorString(e));
  int slot = g_scratch_used;
  if (slot < kMaxEntries) {
    ++g_scratch_used;
  } else {
    slot = g_scratch_next;
    g_scratch_next = (g_scratch_next + 1) % kMaxEntries;
  }
  g_scratch[slot] = ScratchEntry{key, p};
  *out = p;
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
  int rc = scratch_in_current_context(&scratch);
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
