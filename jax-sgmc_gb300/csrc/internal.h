// Declarations shared between the translation units of libgbsgmc (not ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbsgmc.h"

namespace gbsgmc {

int set_error(int code, const char* fmt, ...);
int check_launch(const char* what);

// glm.cu
// Launch shape of the GLM kernel; 0 lets the library choose.
struct GlmTune {
  int slices = 0;         // CTAs per chain
  int rows_per_warp = 0;  // 2, 4 or 8 (d <= 256 only)
  int warps = 0;          // warps per CTA: 8 or 16
  int prefetch = 0;       // 1: two register tiles in flight per warp
};

size_t glm_ws_bytes(int chains, int n, int d);
// Launch shapes chosen by the plan autotuner, per problem shape.
bool glm_tune_lookup(int chains, int n, int d, int64_t ld, GlmTune* out);
void glm_tune_store(int chains, int n, int d, int64_t ld, GlmTune t);
int glm_prepare();
int glm_sgld_step(const gbsgmc_glm* model, int chains, int n,
                  const int32_t* idx_dev, int64_t idx_stride, float* w_dev,
                  float* v_dev, float alpha, float lmbd,
                  const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                  double* U_dev, double* lk_var_dev, float* samples_dev,
                  double* sample_lik_dev, void* ws, size_t ws_size,
                  int* status_dev, cudaStream_t stream, GlmTune tune);

// rng.cu
int launch_philox_index(uint64_t seed, int chain_base, int chains,
                        const int64_t* base, int64_t first_step, int steps,
                        int per_step, int64_t n_obs, int32_t* idx,
                        int64_t chain_stride, int64_t step_stride,
                        cudaStream_t stream);

}  // namespace gbsgmc
