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
  int dynamic = 0;        // 1: warps claim items of `slices` per chain
  int multistep = 0;      // 1: plans run a block of steps in one launch
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
                  int* status_dev, cudaStream_t stream, GlmTune tune,
                  int steps = 1, int64_t idx_step_stride = 0,
                  const int32_t* ident_dev = nullptr);
// The exchange of reSGLD (normal, hot) pairs on the device after a step of
// all 2 * pairs chains (normal chain p in slot p, its hot partner in slot
// pairs + p): solver.parallel_tempering's rule per pair in FP64, and for a
// pair that exchanges, its rows of x (and v), U, var and chain identities
// swapped; then, at kept steps, the normal slots' rows and -U stored as the
// step's samples.  Pair p's uniform is Philox(counter (0, k + 1), key
// (seed << 32) | pair_chain[p]).
// The MLP's value and gradient (gbsgmc_mlp_value_and_grad) where row c of
// the batch reads its minibatch from row ident_dev[c] of idx.
int mlp_value_and_grad_ident(const gbsgmc_mlp* model, int chains, int n, const int32_t* idx,
                             int64_t idx_stride, const int32_t* ident_dev, const float* w,
                             double* U, float* grad, double* lk_var, void* ws, size_t ws_bytes,
                             int* status, cudaStream_t st);
int resgld_pairs_exchange(int pairs, int d, float* x, float* v, double* U,
                          double* var, int32_t* ident, const gbsgmc_sched* sched,
                          double F, uint64_t seed, const int32_t* pair_chain,
                          double* ssq, int64_t* k, int32_t* counts, float* samples,
                          double* sample_lik, cudaStream_t stream);

// update.cu: fusions of the integrator updates used by the network plans.
struct UpdateFusion {
  float prior_pf = 0.f;       // adds pf * x to the gradient (the prior term)
  void* mirror = nullptr;     // BF16 copy of the new x[0, mirror_count) of
  int64_t mirror_count = 0;   //   each chain, chain stride mirror_stride
  int64_t mirror_stride = 0;  //   (elements; both multiples of 4)
  double* sq_parts = nullptr; // per-block sums of squares of the new x,
                              //   [chains, update_blocks(chains, P)]
  const int32_t* ident = nullptr;  // [chains] noise chain of each row (row
                                   //   c draws as chain ident[c]); null: c
};
int update_blocks(int chains, int64_t P);
// At the schedule's kept steps: row 0 of x to samples[slot], -U[0] to
// sample_lik[slot] (may be null).
int keep_row(int64_t P, const float* x, const double* U, const gbsgmc_sched* sched,
             float* samples, double* sample_lik, cudaStream_t st);
int sgld_update_fused(int chains, int64_t P, float* x, const float* g, float* v,
                      float alpha, float lmbd, const gbsgmc_sched* sched,
                      const gbsgmc_noise* noise, const UpdateFusion& f,
                      cudaStream_t st);
int obabo_first_fused(int chains, int64_t P, float* x, float* p, const float* g1,
                      const float* mass, float friction, double* ke_start,
                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                      const UpdateFusion& f, cudaStream_t st);
int obabo_second_fused(int chains, int64_t P, const float* x, float* p,
                       const float* g2, const float* mass, float friction,
                       double* ke_end, const gbsgmc_sched* sched,
                       const gbsgmc_noise* noise, const UpdateFusion& f,
                       cudaStream_t st);
// Step k's second OBABO half (gradient g2) then step k + 1's first half
// (gradient g1, taken at the same positions) in one pass: the same values as
// obabo_second_fused at step k followed by obabo_first_fused at step k + 1.
int obabo_second_first_fused(int chains, int64_t P, float* x, float* p, const float* g2,
                             const float* g1, const float* mass, float friction,
                             double* ke_end, double* ke_start, const gbsgmc_sched* sched,
                             const gbsgmc_noise* noise, const UpdateFusion& f,
                             cudaStream_t st);
int sghmc_position_fused(int chains, int64_t P, float* x, float* p, const float* mass,
                         float friction, const gbsgmc_sched* sched,
                         const UpdateFusion& f, cudaStream_t st);
int sghmc_momentum_fused(int chains, int64_t P, const float* x, float* p,
                         const float* g, float friction, const gbsgmc_sched* sched,
                         const gbsgmc_noise* noise, const UpdateFusion& f,
                         cudaStream_t st);
// The mirror and squares of x itself (before the first fused update).
int mirror_fused(int chains, int64_t P, const float* x, const UpdateFusion& f,
                 cudaStream_t st);

// mlp.cu: the value and likelihood gradient with the weights' BF16 copy and
// sums of squares supplied by the integrator (UpdateFusion), the prior's
// gradient left to the update.
int mlp_mirror_region(const gbsgmc_mlp* model, int chains, int n, void* ws,
                      void** mirror, int64_t* count, int64_t* stride);
int mlp_value_and_grad_fused(const gbsgmc_mlp* model, int chains, int n,
                             const int32_t* idx, int64_t idx_stride, const float* w,
                             double* U, float* grad, double* lk_var, void* ws,
                             size_t ws_bytes, int* status, cudaStream_t st,
                             const double* sq_parts, int sq_count);

// rng.cu
int launch_philox_index(uint64_t seed, int chain_base, int chains,
                        const int64_t* base, int64_t first_step, int steps,
                        int per_step, int64_t n_obs, int32_t* idx,
                        int64_t chain_stride, int64_t step_stride,
                        cudaStream_t stream);

}  // namespace gbsgmc
