/*
 * gbsgmc.h -- C ABI of the GB300 SG-MCMC hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (GBSGMC_OK == 0) and never throws.  Pointers named `*_dev` or
 * documented as "device" are CUDA device pointers owned by the caller; the
 * library only owns the memory behind a gbsgmc_plan handle.  Launches are
 * ordered on the caller's stream and never synchronise the host, except the
 * plan calls, which say so.  Errors raised inside a kernel (an observation
 * index outside [0, N), a non-finite potential, a bounded wait that gave up)
 * are written to a caller-owned device status word `status_dev`; the first
 * error code written wins (atomicCAS from 0).
 *
 * The reference (jax_sgmc 0.1.5) has no C ABI: its boundary is the Python API.
 * Each declaration below names the reference function whose arithmetic it
 * replaces (paths relative to the jax-sgmc project root).
 */
#ifndef GBSGMC_H_
#define GBSGMC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t, passed as an opaque pointer (NULL = legacy default stream). */
typedef void* gbsgmc_stream_t;

/* Status codes (return values and device status words). */
#define GBSGMC_OK 0
#define GBSGMC_ERR_ARG 1         /* null pointer, negative size, bad stride   */
#define GBSGMC_ERR_SHAPE 2       /* shape outside the supported range         */
#define GBSGMC_ERR_INDEX 3       /* observation index outside [0, N)          */
#define GBSGMC_ERR_NONFINITE 4   /* potential or gradient is NaN / Inf        */
#define GBSGMC_ERR_TIMEOUT 5     /* a bounded device wait gave up             */
#define GBSGMC_ERR_CUDA 6        /* CUDA runtime error (message in last_error) */
#define GBSGMC_ERR_UNSUPPORTED 7 /* feature not available in this library      */

/* Likelihood families of the generalised-linear kernels. */
#define GBSGMC_GLM_LINEAR_GAUSSIAN 0 /* lk = log N(y | x.w, sigma^2)          */
#define GBSGMC_GLM_LOGISTIC 1        /* lk = y*z - softplus(z), z = x.w       */
#define GBSGMC_GLM_LINEAR 2          /* lk = z = x.w (y unused)               */

/* Noise stream tags (fourth Philox counter word). */
#define GBSGMC_TAG_SGLD 0u
#define GBSGMC_TAG_OBABO_1 1u
#define GBSGMC_TAG_OBABO_2 2u
#define GBSGMC_TAG_SGHMC_RESAMPLE 3u
#define GBSGMC_TAG_SGHMC_STEP 4u
#define GBSGMC_TAG_SWAP 5u
#define GBSGMC_TAG_INDEX 6u
#define GBSGMC_TAG_AMAGOLD 7u
#define GBSGMC_TAG_AMAGOLD_INIT 8u
#define GBSGMC_TAG_MH 9u

/* Thread-local message for the last non-zero status returned on this thread. */
const char* gbsgmc_last_error(void);
/* ABI version (major*10000 + minor*100 + patch). */
int gbsgmc_version(void);

/* ------------------------------------------------------------------------ */
/* Random streams                                                            */
/* ------------------------------------------------------------------------ */

/* numpy PCG64 bit-generator state (numpy's bit_generator.state dict:
 * state.state, state.inc, has_uint32, uinteger), 128-bit words split in
 * 64-bit halves.  40 bytes, 8-byte aligned. */
typedef struct gbsgmc_pcg64 {
  uint64_t state_hi, state_lo;
  uint64_t inc_hi, inc_lo;
  uint32_t has_uint32, uinteger;
} gbsgmc_pcg64;

/* Host function: the fresh gbsgmc_pcg64 words ([count, 5] uint64: state
 * high/low, increment high/low, buffered half 0) of the numpy PCG64 streams
 * numpy.random.default_rng(SeedSequence(seed).spawn(1)[0]) starts with, for
 * seeds seeds_lo[c] + 2^64 seeds_hi[c] (seeds_hi may be NULL: seeds below
 * 2^64).  The index streams NumpyDataLoader.register_random_pipeline gives
 * its chains (jax_sgmc/data/numpy_loader.py:261-265). */
int gbsgmc_pcg64_seed(const uint64_t* seeds_lo, const uint64_t* seeds_hi, int count,
                      uint64_t* words);

/* Draws `draws` indices in [0, n_obs) for each of `chains` numpy PCG64 streams,
 * bit-identical to numpy's Generator.choice(arange(n_obs), draws,
 * replace=True) (== Generator.integers(0, n_obs, dtype=int64)), and advances
 * `states_dev` exactly as numpy would.  Draw j of chain c is written to
 * idx_dev[c*chain_stride + (j / per_step)*step_stride + j % per_step].
 * n_obs in [1, 2^31).
 * Replaces NumpyDataLoader._draw_indices (jax_sgmc/data/numpy_loader.py:382-389)
 * called cache_size times by _get_indices (numpy_loader.py:342-355). */
int gbsgmc_index_draw_pcg64(gbsgmc_pcg64* states_dev, int chains,
                            int64_t n_obs, int64_t draws, int per_step,
                            int32_t* idx_dev, int64_t chain_stride,
                            int64_t step_stride, int* status_dev,
                            gbsgmc_stream_t stream);

/* Counter-based index draws: idx = floor(u32 * n_obs / 2^32) with u32 from
 * Philox4x32-10(counter = (j/4, step, chain_base + c, TAG_INDEX),
 * key = seed).  `steps` consecutive steps starting at `first_step`, `per_step`
 * draws each, laid out as in gbsgmc_index_draw_pcg64.
 * Replaces DeviceNumpyDataLoader.get_random_data
 * (jax_sgmc/data/numpy_loader.py:128-141), whose threefry stream is not
 * reproduced. */
int gbsgmc_index_draw_philox(uint64_t seed, int chain_base, int chains,
                             int64_t first_step, int steps, int per_step,
                             int64_t n_obs, int32_t* idx_dev,
                             int64_t chain_stride, int64_t step_stride,
                             gbsgmc_stream_t stream);

/* Standard normals from the production noise stream: out[c*stride + j] =
 * N(0,1) from Philox4x32-10(counter = (j/4, step, chain_base + c, tag),
 * key = seed) through Box-Muller on the pairs (u0,u1), (u2,u3).
 * Replaces integrator.random_tree (jax_sgmc/integrator.py:119-135). */
int gbsgmc_philox_normal(uint64_t seed, int chain_base, int chains,
                         int64_t step, uint32_t tag, int64_t count,
                         float* out_dev, int64_t stride,
                         gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Generalised-linear minibatch potential and its adjoint                    */
/* ------------------------------------------------------------------------ */

/* Model + dataset description (all pointers are device pointers). */
typedef struct gbsgmc_glm {
  int family;          /* GBSGMC_GLM_*                                       */
  int d;               /* features = parameters per chain, 1..1024            */
  int64_t n_obs;       /* N of the N/n scale (observations in the dataset)   */
  int64_t ld;          /* row stride of X in floats (>= d)                    */
  const float* X;      /* [n_obs, ld] fp32 features                           */
  const float* y;      /* [n_obs] fp32 targets                                */
  float sigma;         /* linear-Gaussian noise sd                            */
  float prior_scale;   /* Gaussian prior N(0, s^2 I) sd; <= 0: flat prior     */
  float temperature;   /* potential temperature T: U = (-N/n sum lk - log p)/T */
  int y_inline;        /* 1: the target of row i is X[i*ld + d] (y unused and
                          ld >= d+1); 0: the target is y[i]                 */
  int64_t n_rows;      /* rows of X and y (index bound); 0 means n_obs        */
} gbsgmc_glm;

/* Bytes of workspace needed by gbsgmc_glm_value_and_grad for `chains` chains of
 * minibatch size n.  The workspace must be zero-filled before its first use;
 * calls leave it zeroed again. */
size_t gbsgmc_glm_workspace_bytes(int chains, int n, int d);

/* For each chain c: U[c] = (-N/n * sum_i m_i lk_i - log p(w_c)) / T,
 * grad[c] = dU/dw_c, lk[c, i] = lk_i and lk_var[c] = var_i(lk_i), where row i
 * of the minibatch is observation idx[c*idx_stride + i] and m_i = mask[c*n+i]
 * (all ones when mask is NULL).  grad, lk, lk_var may be NULL.
 * Replaces minibatch_potential's potential_function
 * (jax_sgmc/potential.py:159-214) under jax.value_and_grad
 * (jax_sgmc/integrator.py:792) plus jnp.var(likelihoods) (integrator.py:880). */
int gbsgmc_glm_value_and_grad(const gbsgmc_glm* model, int chains, int n,
                              const int32_t* idx_dev, int64_t idx_stride,
                              const float* mask_dev, const float* w_dev,
                              double* U_dev, float* grad_dev, float* lk_dev,
                              double* lk_var_dev, void* workspace_dev,
                              size_t workspace_bytes, int* status_dev,
                              gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Integrator updates (elementwise over [chains, P])                         */
/* ------------------------------------------------------------------------ */

/* Per-step schedule read on the device, so that captured launches can be
 * replayed: step k = (*base_dev) + offset (base_dev NULL: k = offset);
 * h = step_size_dev[k] (or step_size when NULL), T likewise. */
typedef struct gbsgmc_sched {
  const float* step_size_dev;
  const float* temperature_dev;
  const int64_t* base_dev;
  const int32_t* keep_slot_dev; /* sample slot of step k, -1 = not kept */
  int64_t offset;
  float step_size;
  float temperature;
  /* Per-chain factor of the temperature (replica c runs at T_k * f[c]), or
   * NULL for 1: the temperature ladder of tempering replicas. */
  const float* chain_temperature_dev;
} gbsgmc_sched;

/* Noise source: injected normals noise_dev[c*noise_stride + j] when noise_dev
 * is not NULL, else Philox normals (seed, chain_base + c, step k, tag). */
typedef struct gbsgmc_noise {
  const float* noise_dev;
  int64_t noise_stride;
  uint64_t seed;
  int chain_base;
  int _pad;
} gbsgmc_noise;

/* SGLD step with optional RMSprop on [chains, P]:
 *   v <- alpha v + (1-alpha) g^2;  G = 1/(lmbd + sqrt v)         (rms_prop)
 *   x <- x + G (-h g) + sqrt(G) sqrt(2 T h) xi                    (rms_prop)
 *   x <- x + (-h g) + sqrt(2 T h) xi                              (plain)
 * `v_dev` NULL selects plain SGLD.  When the step is kept, the new x is copied
 * to samples_dev[slot*chains*P + c*P + j].
 * Replaces langevin_diffusion.update_fn (jax_sgmc/integrator.py:860-922) and
 * adaption.rms_prop update/get (jax_sgmc/adaption.py:254-291). */
int gbsgmc_sgld_update(int chains, int64_t P, float* x_dev, const float* g_dev,
                       float* v_dev, float alpha, float lmbd,
                       const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                       float* samples_dev, gbsgmc_stream_t stream);

/* OBABO, first half: O (p <- sqrt(e^{-f h}) p + sqrt((1-e^{-f h}) T) sqrt(m) xi1),
 * ke_start[c] += 0.5 p.p/m, B (p <- p - h/2 g1), A (x <- x + h p/m).
 * `mass_dev` [P] NULL = unit mass.  Noise tag GBSGMC_TAG_OBABO_1.
 * Replaces obabo._leapfrog_steps up to the second gradient
 * (jax_sgmc/integrator.py:209-241). */
int gbsgmc_obabo_first(int chains, int64_t P, float* x_dev, float* p_dev,
                       const float* g1_dev, const float* mass_dev,
                       float friction, double* ke_start_dev,
                       const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                       gbsgmc_stream_t stream);

/* OBABO, second half: B (p <- p - h/2 g2), ke_end[c] += 0.5 p.p/m, O with xi2.
 * Noise tag GBSGMC_TAG_OBABO_2.  Replaces jax_sgmc/integrator.py:243-273. */
int gbsgmc_obabo_second(int chains, int64_t P, float* p_dev,
                        const float* g2_dev, const float* mass_dev,
                        float friction, double* ke_end_dev,
                        const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                        gbsgmc_stream_t stream);

/* SGHMC momentum resample p = sqrt(m) xi (tag GBSGMC_TAG_SGHMC_RESAMPLE).
 * Replaces friction_leapfrog.integrate (jax_sgmc/integrator.py:735-738). */
int gbsgmc_sghmc_resample(int chains, int64_t P, float* p_dev,
                          const float* mass_dev, const gbsgmc_sched* sched,
                          const gbsgmc_noise* noise, gbsgmc_stream_t stream);

/* SGHMC position update x <- x + h p/m and friction decay
 * p <- p - h f (p/m).  Replaces jax_sgmc/integrator.py:610-619. */
int gbsgmc_sghmc_position(int chains, int64_t P, float* x_dev, float* p_dev,
                          const float* mass_dev, const float* friction_dev,
                          float friction, const gbsgmc_sched* sched,
                          gbsgmc_stream_t stream);

/* SGHMC force and noise: p <- p - h g + f sqrt(2h) xi (tag
 * GBSGMC_TAG_SGHMC_STEP).  `friction_dev` [P] or NULL (scalar friction).
 * Replaces jax_sgmc/integrator.py:621-655 (noise_model = None). */
int gbsgmc_sghmc_momentum(int chains, int64_t P, float* p_dev,
                          const float* g_dev, const float* friction_dev,
                          float friction, const gbsgmc_sched* sched,
                          const gbsgmc_noise* noise, gbsgmc_stream_t stream);

/* SGHMC force and noise under a noise model (integrator.py:630-647):
 * p <- p - h g + sqrt(2h) (cb_diff_sqrt * xi), cb_diff_sqrt [chains, P]
 * from gbsgmc_glm_fisher_noise, xi of tag GBSGMC_TAG_SGHMC_STEP. */
int gbsgmc_sghmc_momentum_noise_model(int chains, int64_t P, float* p_dev,
                                      const float* g_dev, const float* cb_diff_sqrt_dev,
                                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                                      gbsgmc_stream_t stream);

/* The empirical-Fisher noise model of fisher_information(diagonal=True)
 * (jax_sgmc/adaption.py:371-457) on a generalised-linear likelihood, per
 * chain: with G = grad_dev (dU/dw of the minibatch potential at w) and the
 * per-observation likelihood gradients lk'(z_i) x_i of the n rows idx,
 *   ssq = sum_i (lk'(z_i) x_i - G / N)^2,  b = 0.5 step_size ssq / (n - 1),
 *   corr = friction - b, corr <= 0 replaced by the chain's smallest positive
 *   corr;  cb_diff_sqrt = sqrt(corr),  b_sqrt = sqrt(friction - corr)
 * (b_sqrt_dev may be NULL).  friction_dev [d] or NULL (scalar friction).
 * 2 <= n <= 4096; fp32 like the reference. */
int gbsgmc_glm_fisher_noise(const gbsgmc_glm* model, int chains, int n,
                            const int32_t* idx_dev, int64_t idx_stride, const float* w_dev,
                            const float* grad_dev, const float* friction_dev, float friction,
                            float step_size, float* cb_diff_sqrt_dev, float* b_sqrt_dev,
                            int* status_dev, gbsgmc_stream_t stream);

/* The dense form, fisher_information(diagonal=False)
 * (jax_sgmc/adaption.py:441-452): with d_i = lk'(z_i) x_i - G / N,
 *   b = 0.5 step_size / (n - 1) sum_i d_i d_i^T       (d x d),
 *   cb_diff_sqrt = u sqrt(s) for (u, s, .) = svd(diag(friction) - b),
 *   b_sqrt = u sqrt(s) for (u, s, .) = svd(b),
 * each a d-vector (the left singular vectors times the root singular
 * values, which the integrator applies elementwise, as the reference does).
 * The SVDs of these symmetric matrices come from their eigendecompositions
 * (gbsgmc_sym_eig's method and sign convention; the signs of LAPACK's
 * singular vectors are not specified, and these vectors depend on them).
 * d <= 128, 2 <= n <= 4096 (n * 8 bytes + 8 d^2 bytes of shared memory
 * within 227 KB); fp32. */
int gbsgmc_glm_fisher_noise_dense(const gbsgmc_glm* model, int chains, int n,
                                  const int32_t* idx_dev, int64_t idx_stride,
                                  const float* w_dev, const float* grad_dev,
                                  const float* friction_dev, float friction,
                                  float step_size, float* cb_diff_sqrt_dev,
                                  float* b_sqrt_dev, int* status_dev,
                                  gbsgmc_stream_t stream);

/* Eigendecomposition of `batch` symmetric P x P matrices (A_dev [batch, P,
 * P], row-major; the symmetric part (A + A^T) / 2 is used): eigenvalues in
 * ascending order to w_dev [batch, P] and the eigenvectors as the columns of
 * V_dev [batch, P, P], each scaled so that its largest-magnitude component
 * (the first of equal ones) is positive.  Cyclic Jacobi with the
 * round-robin ordering, one CTA per matrix, fp32; P <= 128.
 * Replaces jnp.linalg.eigh in mass_matrix(diagonal=False)
 * (jax_sgmc/adaption.py:316). */
int gbsgmc_sym_eig(int batch, int P, const float* A_dev, float* w_dev,
                   float* V_dev, gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Reversible leapfrog (AMAGOLD) and Metropolis-Hastings corrections         */
/* ------------------------------------------------------------------------ */

/* x <- x + (scale h_k) p / m: the half (scale 0.5) and full (scale 1) position
 * steps of reversible_leapfrog (jax_sgmc/integrator.py:383-388). */
int gbsgmc_leapfrog_position(int chains, int64_t P, float* x_dev,
                             const float* p_dev, const float* mass_dev,
                             float scale, const gbsgmc_sched* sched,
                             gbsgmc_stream_t stream);

/* One momentum step of reversible_leapfrog (jax_sgmc/integrator.py:402-458):
 *   p' = ((1 - h f) p - h g + sqrt(4 f h) sqrt(m) xi) / (1 + h f)
 * with xi the Philox normals of tag GBSGMC_TAG_AMAGOLD at step k, and
 * energy_dev[c] += 0.5 h sum (p + p') g / m (may be NULL). */
int gbsgmc_amagold_momentum(int chains, int64_t P, float* p_dev,
                            const float* g_dev, const float* mass_dev,
                            float friction, double* energy_dev,
                            const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                            gbsgmc_stream_t stream);

#define GBSGMC_MH_AMAGOLD 0
#define GBSGMC_MH_SGGMC 1

/* FP64 Metropolis-Hastings decision per chain of solver.amagold
 * (jax_sgmc/solver.py:368-395: log a = U_old - U_new + energy) or
 * solver.sggmc (jax_sgmc/solver.py:508-528: log a = -(U_new - U_old +
 * ke_end - ke_start) / T_k), capped at 0; accept when log u < log a with
 * u = u_dev[c] or the 53-bit Philox uniform (seed, counter (chain_base + c,
 * k, 0, GBSGMC_TAG_MH)).  Writes accept_dev[c] (0/1), ratio_dev[c] =
 * exp(log a) and U_keep_dev[c] (U_new if accepted, else U_old); the last two
 * may be NULL. */
int gbsgmc_mh_accept(int chains, int kind, const double* U_old_dev,
                     const double* U_new_dev, const double* energy_dev,
                     const double* ke_start_dev, const double* ke_end_dev,
                     const gbsgmc_sched* sched, const double* u_dev,
                     uint64_t seed, int chain_base, int32_t* accept_dev,
                     double* ratio_dev, double* U_keep_dev,
                     gbsgmc_stream_t stream);

/* After gbsgmc_mh_accept: rejected chains return to x_old and
 * reject_momentum_sign * p_old (AMAGOLD flips the momentum: -1; SGGMC: +1;
 * p_dev NULL leaves momenta alone); accepted chains keep the proposal. */
int gbsgmc_mh_select(int chains, int64_t P, const int32_t* accept_dev,
                     float* x_dev, const float* x_old_dev, float* p_dev,
                     const float* p_old_dev, float reject_momentum_sign,
                     gbsgmc_stream_t stream);

/* Dense mass matrices.  The reference's integrators multiply by the inverse
 * mass and the root mass as matrices when those are P x P (tensor_matmul of
 * a Tensor with ndim 2, jax_sgmc/util/tree_util.py:38-56), which is what
 * mass_matrix(diagonal=False) adapts.  These are the updates of
 * gbsgmc_leapfrog_position, gbsgmc_amagold_momentum, gbsgmc_obabo_first and
 * gbsgmc_obabo_second with m^-1 p, m^-1 g and sqrt(m) xi replaced by the
 * products with minv_dev [P, P] and msqrt_dev [P, P] (row-major, shared by
 * all chains), and the same noise streams.  One CTA per chain, P <= 8192
 * (meant for small P: each update reads the matrices once per chain). */
int gbsgmc_leapfrog_position_dense(int chains, int64_t P, float* x_dev,
                                   const float* p_dev, const float* minv_dev,
                                   float scale, const gbsgmc_sched* sched,
                                   gbsgmc_stream_t stream);
int gbsgmc_amagold_momentum_dense(int chains, int64_t P, float* p_dev,
                                  const float* g_dev, const float* minv_dev,
                                  const float* msqrt_dev, float friction,
                                  double* energy_dev, const gbsgmc_sched* sched,
                                  const gbsgmc_noise* noise,
                                  gbsgmc_stream_t stream);
int gbsgmc_obabo_first_dense(int chains, int64_t P, float* x_dev, float* p_dev,
                             const float* g1_dev, const float* minv_dev,
                             const float* msqrt_dev, float friction,
                             double* ke_start_dev, const gbsgmc_sched* sched,
                             const gbsgmc_noise* noise, gbsgmc_stream_t stream);
int gbsgmc_obabo_second_dense(int chains, int64_t P, float* p_dev,
                              const float* g2_dev, const float* minv_dev,
                              const float* msqrt_dev, float friction,
                              double* ke_end_dev, const gbsgmc_sched* sched,
                              const gbsgmc_noise* noise, gbsgmc_stream_t stream);

/* y[c] = M x[c] for c < chains (M [P, P] row-major, x and y [chains, P]);
 * the initial AMAGOLD momentum sqrt(M) xi under a dense mass
 * (jax_sgmc/solver.py:352).  P <= 8192. */
int gbsgmc_dense_matvec(int chains, int64_t P, const float* m_dev,
                        const float* x_dev, float* y_dev, gbsgmc_stream_t stream);

/* One update of mass_matrix(diagonal=False) (jax_sgmc/adaption.py:296-368)
 * with the `iteration`-th sample x (1-based), fp32 in the reference's
 * operation order:  mean' = (i-1)/i mean + 1/i x;
 * ssq += (x - mean)(x - mean')^T  (ssq_dev [P, P]).  When iteration ==
 * burn_in: inv = ssq / i and, from the eigendecomposition (w, V) of inv
 * (gbsgmc_sym_eig into eig_w_dev [P] and eig_v_dev [P, P]),
 * sqrt = V^T diag(sqrt(max(w, 0))) V, the product adaption.py:317 forms.
 * P <= 128. */
int gbsgmc_mass_adapt_dense(int64_t P, int iteration, int burn_in,
                            const float* x_dev, float* mean_dev, float* ssq_dev,
                            float* inv_dev, float* sqrt_dev, float* eig_w_dev,
                            float* eig_v_dev, gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Sample statistics                                                         */
/* ------------------------------------------------------------------------ */

/* FP64 posterior moments of kept samples (replaces collecting every sample
 * on the host through io.py:626-771 to take moments there).  Adds `count`
 * samples of each chain -- sample k of chain c at
 * samples_dev[k * slot_stride + c * chain_stride + j] -- to the shifted sums
 * of [chains, P]: shift (fp32, the first sample, written when seen == 0),
 * s1 = sum (x - shift), s2 = sum (x - shift)^2 (fp64).  `seen` is the number
 * of samples already in the sums. */
int gbsgmc_moments_accumulate(int chains, int64_t P, int count, const float* samples_dev,
                              int64_t slot_stride, int64_t chain_stride, int64_t seen,
                              float* shift_dev, double* s1_dev, double* s2_dev,
                              gbsgmc_stream_t stream);

/* Mean and population variance (ddof 0) of n samples from the sums above:
 * mean = shift + s1 / n, var = max((s2 - s1 (s1 / n)) / n, 0). */
int gbsgmc_moments_finalize(int chains, int64_t P, int64_t n, const float* shift_dev,
                            const double* s1_dev, const double* s2_dev, double* mean_dev,
                            double* var_dev, gbsgmc_stream_t stream);

/* Diagonal mass adaption (adaption.py:296-368, mass_matrix(diagonal=True)),
 * one update with the `iteration`-th sample x (1-based), fp32:
 *   mean' = (i-1)/i mean + 1/i x;  ssq += (x - mean)(x - mean')
 * and when iteration == burn_in: inv = ssq / i, sqrt = sqrt(i / ssq) and,
 * when mass_dev is not NULL, the mass i / ssq that the integrator kernels
 * take as `mass_dev`. */
int gbsgmc_mass_adapt(int64_t P, int iteration, int burn_in, const float* x_dev,
                      float* mean_dev, float* ssq_dev, float* inv_dev, float* sqrt_dev,
                      float* mass_dev, gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Replica exchange                                                          */
/* ------------------------------------------------------------------------ */

/* reSGLD exchange for `pairs` (normal, hot) replica pairs, in FP64:
 *   k += 1;  ssq <- (1 - 1/k) ssq + (1/k) var_normal
 *   dbeta = 1/T_normal - 1/T_hot
 *   log_s = dbeta (U_normal - U_hot - dbeta ssq / F)
 *   swapped = !(log u < log s)      (the reference keeps the pair when
 *                                    log u < log s and exchanges otherwise)
 * u is given in u_dev[pair] (uniform in (0,1)), or drawn from Philox
 * (tag GBSGMC_TAG_SWAP, counter (pair, step)) when u_dev is NULL.
 * perm_dev[pair] receives 1 when the pair exchanged its states.  The caller
 * exchanges the replica buffers (gbsgmc_swap_rows).
 * Replaces solver.parallel_tempering.update (jax_sgmc/solver.py:264-293). */
int gbsgmc_resgld_swap_f64(int pairs, const double* U_normal_dev,
                           const double* U_hot_dev,
                           const double* var_normal_dev, const double* T_normal_dev,
                           const double* T_hot_dev, double F, double* ssq_dev,
                           int64_t* k_dev, const double* u_dev, uint64_t seed,
                           int64_t step, double* log_s_dev, int32_t* perm_dev,
                           gbsgmc_stream_t stream);

/* Exchanges rows a[pair] <-> b[pair] ([pairs, width] fp32) where
 * perm_dev[pair] == 1.  Used for positions, RMSprop state and potentials. */
int gbsgmc_swap_rows(int pairs, int64_t width, float* a_dev, float* b_dev,
                     const int32_t* perm_dev, gbsgmc_stream_t stream);

/* Replica-exchange over a temperature ladder of R replicas (rows of [R, P]
 * arrays, coldest first), the adjacent-pair generalisation of
 * solver.parallel_tempering (jax_sgmc/solver.py:264-293), which pairs one
 * normal and one hot chain.  Pair r = (r, r + 1) keeps its own estimate
 * ssq[r] of the variance, fed by replica r's var(lk) as the reference feeds
 * it the normal chain's:
 *   k += 1;  ssq[r] <- (1 - 1/k) ssq[r] + (1/k) var[r]     (every step) */
int gbsgmc_resgld_sa_update(int replicas, const double* lk_var_dev,
                            double* ssq_dev, int64_t* k_dev,
                            gbsgmc_stream_t stream);

/* Exchange attempt at step k = sched's step (the caller attempts when
 * (k + 1) % every == 0): round = (k + 1) / every selects the pairs r of
 * parity round % 2 (alternating even and odd pairs).  For each, in FP64,
 *   dbeta = 1/T(k, r) - 1/T(k, r+1),  T(k, c) = t_k * chain_temperature[c]
 *   log_s = dbeta (U[r] - U[r+1] - dbeta ssq[r] / F)
 *   exchanged = !(log u < log s)    (the reference's lax.cond rule)
 * with u = u_dev[r], or Philox (seed, counter (r, round, 0, GBSGMC_TAG_SWAP))
 * when u_dev is NULL.  An exchanging pair swaps its rows of x (and v when
 * not NULL), U and lk_var; flags_dev[r] = 1 for it, counts_dev[r] (may be
 * NULL) counts exchanges, log_s_dev (may be NULL) receives log s. */
int gbsgmc_resgld_exchange_adjacent(int replicas, int64_t P, float* x_dev,
                                    float* v_dev, double* U_dev,
                                    double* lk_var_dev,
                                    const gbsgmc_sched* sched, int every,
                                    const double* ssq_dev, double F,
                                    uint64_t seed, const double* u_dev,
                                    int32_t* flags_dev, int32_t* counts_dev,
                                    double* log_s_dev, gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Tensor-core GEMM (building block of the network likelihoods)              */
/* ------------------------------------------------------------------------ */

/* C[b] = A[b] * B[b]^T for b < batch on the tcgen05 tensor cores: A is M x K
 * and B is N x K, both BF16 row-major with K contiguous (leading dimensions
 * lda, ldb, multiples of 8; base addresses 16-byte aligned); C is M x N fp32
 * (ldc a multiple of 4).  Needs M % 128 == 0, N % 128 == 0, K % 64 == 0.
 * Replaces the XLA dot_general that jax.grad of a dense-network likelihood
 * lowers to (the reference's likelihood is user code, e.g.
 * examples/cifar.md:203-210). */
int gbsgmc_gemm_bf16_nt(const void* A_dev, int64_t lda, int64_t a_batch_stride,
                        const void* B_dev, int64_t ldb, int64_t b_batch_stride,
                        float* C_dev, int64_t ldc, int64_t c_batch_stride,
                        int batch, int M, int N, int K, int* status_dev,
                        gbsgmc_stream_t stream);

/* As gbsgmc_gemm_bf16_nt with a choice of operand layout: a_mn != 0 means A
 * is stored transposed (K x M, row-major with M contiguous, lda >= M),
 * b_mn != 0 that B is stored K x N (ldb >= N).  The transposed forms let the
 * adjoint GEMMs of a network (X^T G, Z^T G) read activations where the
 * forward pass wrote them. */
int gbsgmc_gemm_bf16(int a_mn, int b_mn, const void* A_dev, int64_t lda,
                     int64_t a_batch_stride, const void* B_dev, int64_t ldb,
                     int64_t b_batch_stride, float* C_dev, int64_t ldc,
                     int64_t c_batch_stride, int batch, int M, int N, int K,
                     int* status_dev, gbsgmc_stream_t stream);

/* As gbsgmc_gemm_bf16 with C stored as BF16 (rounded to nearest even; ldc and
 * the C batch stride multiples of 8 elements, C 16-byte aligned). */
int gbsgmc_gemm_bf16_c16(int a_mn, int b_mn, const void* A_dev, int64_t lda,
                         int64_t a_batch_stride, const void* B_dev, int64_t ldb,
                         int64_t b_batch_stride, void* C_dev, int64_t ldc,
                         int64_t c_batch_stride, int batch, int M, int N, int K,
                         int* status_dev, gbsgmc_stream_t stream);

/* As gbsgmc_gemm_bf16 with the bound of each wait for pipeline progress (the
 * TMA operands of a stage, a free stage, a finished or drained TMEM
 * accumulator) given in nanoseconds instead of the default 1 s.  A CTA whose
 * wait runs out writes GBSGMC_ERR_TIMEOUT to *status_dev, stops issuing
 * copies and MMAs, waits (up to 1 s) for those it issued, frees its TMEM and
 * returns; C is then incomplete, and the device stays usable.  No reference
 * counterpart: the bounded waits are this library's failure detection. */
int gbsgmc_gemm_bf16_wait_limit(int a_mn, int b_mn, const void* A_dev,
                                int64_t lda, int64_t a_batch_stride,
                                const void* B_dev, int64_t ldb,
                                int64_t b_batch_stride, float* C_dev,
                                int64_t ldc, int64_t c_batch_stride, int batch,
                                int M, int N, int K, uint64_t wait_limit_ns,
                                int* status_dev, gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Dense tanh network (MLP) with a Gaussian likelihood                       */
/* ------------------------------------------------------------------------ */

/* out(x) = W3^T tanh(W2^T tanh(W1^T x + b1) + b2) + b3 with
 * lk = log N(y | out(x), sigma^2).  The flat parameter vector of a chain is
 * the ravel of the pytree {W1 [d_in,h1], W2 [h1,h2], W3 [h2,1], b1 [h1],
 * b2 [h2], b3 [1]} in sorted key order:
 *   W1 | W2 | W3 | b1 | b2 | b3,  P = d_in h1 + h1 h2 + h2 + h1 + h2 + 1.
 * GEMMs run in BF16 with FP32 accumulation on the tensor cores; tanh uses the
 * hardware approximation.  Needs d_in % 64 == 0, h1 % 256 == 0,
 * h2 % 256 == 0, n % 128 == 0. */
typedef struct gbsgmc_mlp {
  int d_in, h1, h2;
  int y_inline;        /* 1: target of row i at X[i*ld + d_in]; 0: y[i]     */
  int64_t n_obs;       /* N of the N/n scale                                */
  int64_t n_rows;      /* rows of X (index bound); 0 means n_obs           */
  int64_t ld;          /* row stride of X in floats                         */
  const float* X;
  const float* y;
  float sigma, prior_scale, temperature;
  int _reserved;
} gbsgmc_mlp;

int64_t gbsgmc_mlp_param_count(const gbsgmc_mlp* model);
size_t gbsgmc_mlp_workspace_bytes(const gbsgmc_mlp* model, int chains, int n);

/* As gbsgmc_glm_value_and_grad for the dense network: U[c], grad[c] = dU/dw_c
 * (grad may be NULL: value only), lk[c, i] and lk_var[c] for `chains` chains
 * whose flat parameters are the rows of w [chains, P].  The workspace needs
 * no initialisation.  Replaces minibatch_potential (jax_sgmc/potential.py:
 * 159-214) under jax.value_and_grad (jax_sgmc/integrator.py:166,593,792) for
 * a dense-network likelihood. */
int gbsgmc_mlp_value_and_grad(const gbsgmc_mlp* model, int chains, int n,
                              const int32_t* idx_dev, int64_t idx_stride,
                              const float* mask_dev, const float* w_dev,
                              double* U_dev, float* grad_dev, float* lk_dev,
                              double* lk_var_dev, void* workspace_dev,
                              size_t workspace_bytes, int* status_dev,
                              gbsgmc_stream_t stream);

/* As gbsgmc_mlp_value_and_grad with a minibatch of n_dev[c] rows for chain c
 * (1 <= n_dev[c] <= n_max, device memory): row i of chain c is observation
 * idx[c*idx_stride + i] for i < n_dev[c]; the N/n scale, the sums and
 * var(lk) of chain c use its own n_dev[c], lk[c, i >= n_dev[c]] is 0.  The
 * tensor cores only work on each chain's own rows (rounded up to 128).  The
 * workspace is gbsgmc_mlp_workspace_bytes(model, chains, n_max), n_max a
 * multiple of 128.  For tempering replicas that draw minibatches of
 * different sizes; no reference counterpart (its replicas share one batch
 * size). */
int gbsgmc_mlp_value_and_grad_ragged(const gbsgmc_mlp* model, int chains,
                                     int n_max, const int32_t* n_dev,
                                     const int32_t* idx_dev, int64_t idx_stride,
                                     const float* mask_dev, const float* w_dev,
                                     double* U_dev, float* grad_dev,
                                     float* lk_dev, double* lk_var_dev,
                                     void* workspace_dev, size_t workspace_bytes,
                                     int* status_dev, gbsgmc_stream_t stream);

/* The empirical-Fisher noise model of fisher_information(diagonal=True)
 * (jax_sgmc/adaption.py:371-457) on the MLP likelihood, per chain: with
 * G = grad_dev (dU/dw at w) and the per-observation gradients d_i of the
 * likelihoods lk_i of the n rows idx,
 *   ssq = sum_i (d_i - G / N)^2 = S2 - 2 (G / N) S1 + n (G / N)^2,
 *   S1 = sum_i d_i, S2 = sum_i d_i^2 (clamped at 0 against rounding),
 *   b = 0.5 step_size ssq / (n - 1), corr = friction - b, corr <= 0 replaced
 *   by the chain's smallest positive corr; cb_diff_sqrt = sqrt(corr),
 *   b_sqrt = sqrt(friction - corr)   (both [chains, P], both required).
 * S1 comes from the adjoint GEMMs seeded with d lk_i / d out, S2 from GEMMs
 * on the squared BF16 operands ((Z1^2)^T (G2^2), (G1^2)^T (X^2)) on the
 * tcgen05 tensor cores.  friction_dev [P] or NULL (scalar friction).  n a
 * positive multiple of 128; workspace gbsgmc_mlp_fisher_workspace_bytes. */
size_t gbsgmc_mlp_fisher_workspace_bytes(const gbsgmc_mlp* model, int chains, int n);
int gbsgmc_mlp_fisher_noise(const gbsgmc_mlp* model, int chains, int n,
                            const int32_t* idx_dev, int64_t idx_stride,
                            const float* w_dev, const float* grad_dev,
                            const float* friction_dev, float friction,
                            float step_size, float* cb_diff_sqrt_dev,
                            float* b_sqrt_dev, void* workspace_dev,
                            size_t workspace_bytes, int* status_dev,
                            gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Convolutional classifier with a softmax likelihood (CNN)                  */
/* ------------------------------------------------------------------------ */

/* x [32,32,3] -> conv3x3(32) ReLU maxpool2 -> conv3x3(64) ReLU maxpool2 ->
 * conv3x3(128) ReLU maxpool2 -> flatten (h, w, c) -> dense(10), SAME padding;
 * lk = logits[label] - logsumexp(logits).  Flat parameters (sorted ravel of
 * {conv1: {b, w}, conv2: {b, w}, conv3: {b, w}, linear: {b, w}}, w in HWIO
 * and [in, out]): b1 | W1 | b2 | W2 | b3 | W3 | bd | Wd, P = 113,738.
 * Image of row r: X[r*ld .. r*ld + 3072) (NHWC floats); its label (a class
 * index stored as a float) at labels[r*label_ld]. */
typedef struct gbsgmc_cnn {
  int64_t n_obs, n_rows, ld;
  const float* X;
  const float* labels;
  int64_t label_ld;
  float prior_scale, temperature;
} gbsgmc_cnn;

int64_t gbsgmc_cnn_param_count(void);
/* n must be even. */
size_t gbsgmc_cnn_workspace_bytes(int chains, int n);

/* As gbsgmc_glm_value_and_grad for the CNN: U[c], grad[c] (may be NULL),
 * lk[c, i] (may be NULL) and lk_var[c] for chains whose parameters are the
 * rows of w [chains, P].  The convolutions run as BF16 GEMMs with fp32
 * accumulation on the tensor cores.  Replaces minibatch_potential
 * (jax_sgmc/potential.py:159-214) under jax.value_and_grad for a
 * classifier likelihood such as examples/cifar.md:203-210. */
int gbsgmc_cnn_value_and_grad(const gbsgmc_cnn* model, int chains, int n,
                              const int32_t* idx_dev, int64_t idx_stride,
                              const float* mask_dev, const float* w_dev,
                              double* U_dev, float* grad_dev, float* lk_dev,
                              double* lk_var_dev, void* workspace_dev,
                              size_t workspace_bytes, int* status_dev,
                              gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Fused SGLD step for the generalised-linear families                       */
/* ------------------------------------------------------------------------ */

/* One fused launch: gather of the minibatch rows (128-bit loads straight
 * into registers), likelihood, adjoint, N/n-scaled reduction, Gaussian prior,
 * RMSprop, noise and the SGLD update of every chain, plus on-device sample
 * collection (samples_dev[slot, c, :] = new w, sample_lik_dev[slot, c] =
 * -U(old w)).  U_dev / lk_var_dev receive the potential at the pre-update
 * position and the variance of the per-observation log-likelihoods.
 * `v_dev` NULL = plain SGLD.
 * Replaces one lax.scan iteration of solver.mcmc over
 * langevin_diffusion.update_fn (jax_sgmc/solver.py:94-123,
 * jax_sgmc/integrator.py:860-922, jax_sgmc/adaption.py:254-291,
 * jax_sgmc/potential.py:159-214). */
int gbsgmc_sgld_glm_step(const gbsgmc_glm* model, int chains, int n,
                         const int32_t* idx_dev, int64_t idx_stride,
                         float* w_dev, float* v_dev, float alpha, float lmbd,
                         const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                         double* U_dev, double* lk_var_dev, float* samples_dev,
                         double* sample_lik_dev, void* workspace_dev,
                         size_t workspace_bytes, int* status_dev,
                         gbsgmc_stream_t stream);

/* `steps` consecutive fused SGLD steps in one launch, step j drawing chain
 * c's rows from idx_dev[j * idx_step_stride + c * idx_stride + i] and using
 * schedule step (counter + offset + j).  With one CTA per chain (n <= 1024
 * and the launch shape a plan's autotuner may choose) every CTA runs its
 * chain's steps back to back, so the steps pay no launch gap or grid tail;
 * other shapes issue one launch per step.  Results equal `steps` calls of
 * gbsgmc_sgld_glm_step with the same shape.  Injected noise (noise_dev) is
 * one draw and is rejected when steps > 1.  samples_dev / sample_lik_dev
 * receive the steps whose keep slot is set.  Replaces `steps` iterations of
 * the lax.scan in solver.mcmc (jax_sgmc/solver.py:152-160). */
int gbsgmc_sgld_glm_steps(const gbsgmc_glm* model, int chains, int n,
                          const int32_t* idx_dev, int64_t idx_stride,
                          int64_t idx_step_stride, int steps, float* w_dev,
                          float* v_dev, float alpha, float lmbd,
                          const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                          double* U_dev, double* lk_var_dev, float* samples_dev,
                          double* sample_lik_dev, void* workspace_dev,
                          size_t workspace_bytes, int* status_dev,
                          gbsgmc_stream_t stream);

/* Size of the scratch array compiled into the library for
 * gbsgmc_sgld_glm_step_noalloc (8 MiB per GPU that loads the library). */
#define GBSGMC_STATIC_SCRATCH_BYTES (8u << 20)

/* gbsgmc_sgld_glm_step for callers that cannot allocate device memory --
 * code running inside another runtime's memory pool (which has reserved the
 * GPU's memory for itself), host code that receives device pointers but owns
 * no allocator, or loops that must not pay for cudaMalloc/cudaFree.
 * It has no counterpart in the reference.  Same arguments and results as
 * gbsgmc_sgld_glm_step minus the workspace: the scratch is an array of
 * GBSGMC_STATIC_SCRATCH_BYTES inside the library, held by every GPU that loads
 * it until the process exits.  Shapes whose scratch
 * (gbsgmc_glm_workspace_bytes(chains, n, d)) exceeds that size are rejected
 * with GBSGMC_ERR_SHAPE (256 chains with d <= 256 and n <= 16384 fit).  It
 * calls no cudaMalloc, cudaFree or other allocating routine.
 *   - The first call in each CUDA context (normally once per device, with
 *     that device current) looks up the array's device address
 *     (cudaGetSymbolAddress) and caches it; make that first call before any
 *     stream capture.
 *   - Each call clears the part of the array it uses, on `stream`.
 *   - All calls share the one array: calls that may overlap on the GPU
 *     (different streams without an ordering between them) race and must be
 *     serialised by the caller. */
int gbsgmc_sgld_glm_step_noalloc(const gbsgmc_glm* model, int chains, int n,
                                 const int32_t* idx_dev, int64_t idx_stride,
                                 float* w_dev, float* v_dev, float alpha,
                                 float lmbd, const gbsgmc_sched* sched,
                                 const gbsgmc_noise* noise, double* U_dev,
                                 double* lk_var_dev, float* samples_dev,
                                 double* sample_lik_dev, int* status_dev,
                                 gbsgmc_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Plans: many steps replayed from a CUDA graph                              */
/* ------------------------------------------------------------------------ */

typedef struct gbsgmc_plan gbsgmc_plan;

/* Index source of a plan: numpy-identical PCG64 streams (pcg_dev != NULL,
 * advanced in place), Philox indices from index_seed, or, with external != 0,
 * indices the caller supplies before each run of at most one block
 * (gbsgmc_plan_set_indices; e.g. the shuffled streams of
 * jax_sgmc/data/numpy_loader.py:391-460, drawn by the host loader). */
typedef struct gbsgmc_index_src {
  gbsgmc_pcg64* pcg_dev;
  uint64_t index_seed;
  int chain_base;
  int external;
} gbsgmc_index_src;

/* Builds a plan that runs SGLD(+RMSprop) on a GLM for `chains` chains: per
 * block of `block_steps` steps one index-draw launch and `block_steps` fused
 * step launches, captured once into a CUDA graph on an internal stream.  All
 * pointers are baked into the graph and must stay valid while the plan
 * lives.  The schedule tables in `sched` must hold every step that will be
 * run.  Replaces solver.mcmc's jit(lax.scan) driver (jax_sgmc/solver.py:152-185)
 * for alias.sgld (jax_sgmc/alias.py:30-120). */
int gbsgmc_sgld_glm_plan_create(gbsgmc_plan** plan, const gbsgmc_glm* model,
                                int chains, int n, float* w_dev, float* v_dev,
                                float alpha, float lmbd,
                                const gbsgmc_sched* sched,
                                const gbsgmc_noise* noise,
                                const gbsgmc_index_src* index_src,
                                double* U_dev, double* lk_var_dev,
                                float* samples_dev, double* sample_lik_dev,
                                int block_steps, int* status_dev);

/* Integrator of a network plan. */
#define GBSGMC_INTEGRATOR_SGLD 0  /* langevin_diffusion, rms_prop when aux != NULL */
#define GBSGMC_INTEGRATOR_OBABO 1 /* obabo: two minibatches per step             */
#define GBSGMC_INTEGRATOR_SGHMC 2 /* friction_leapfrog: one minibatch per step   */

typedef struct gbsgmc_integrator {
  int kind;
  int leapfrog_steps; /* SGHMC: steps between momentum resamples (>= 1)     */
  float friction;     /* OBABO and SGHMC                                    */
  float alpha, lmbd;  /* rms_prop of SGLD                                   */
  int _pad;
  const float* mass_dev; /* diagonal mass [P] or NULL (identity)            */
} gbsgmc_integrator;

/* Builds a plan that runs `chains` chains of an integrator on the dense
 * network: per step the index draw(s), gbsgmc_mlp_value_and_grad over all
 * chains and the integrator's elementwise update(s), `block_steps` steps per
 * captured CUDA graph.  x_dev [chains, P] holds the positions; aux_dev the
 * rms_prop state (SGLD, may be NULL) or the momentum (OBABO, SGHMC; the
 * caller initialises it).  After each step U_dev [chains] holds the
 * potential (OBABO: the mean of its two evaluations), lk_var_dev [chains]
 * (may be NULL) the variance of the last evaluation's lk, and ke_dev
 * [2 * chains] (OBABO, may be NULL) accumulates the kinetic energies after
 * the first and before the last quarter step.  For SGHMC the momentum is
 * resampled every leapfrog_steps steps, so plan_run's first step and step
 * count must be multiples of it.  Replaces solver.mcmc's scan
 * (jax_sgmc/solver.py:152-185) over alias.sgld / obabo / sghmc
 * (jax_sgmc/alias.py) for this likelihood. */
int gbsgmc_mlp_plan_create(gbsgmc_plan** plan, const gbsgmc_mlp* model,
                           int chains, int n, const gbsgmc_integrator* integrator,
                           float* x_dev, float* aux_dev,
                           const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                           const gbsgmc_index_src* index_src, double* U_dev,
                           double* lk_var_dev, double* ke_dev, int block_steps,
                           int* status_dev);

/* As gbsgmc_mlp_plan_create for the CNN classifier (n even). */
int gbsgmc_cnn_plan_create(gbsgmc_plan** plan, const gbsgmc_cnn* model,
                           int chains, int n, const gbsgmc_integrator* integrator,
                           float* x_dev, float* aux_dev,
                           const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                           const gbsgmc_index_src* index_src, double* U_dev,
                           double* lk_var_dev, double* ke_dev, int block_steps,
                           int* status_dev);

/* As gbsgmc_mlp_plan_create for the generalised-linear families (P = d):
 * per step gbsgmc_glm_value_and_grad over all chains and the integrator's
 * updates.  Meant for OBABO and SGHMC; SGLD on these families has its own
 * fused step (gbsgmc_sgld_glm_plan_create), in which the update runs inside
 * the likelihood kernel. */
int gbsgmc_glm_plan_create(gbsgmc_plan** plan, const gbsgmc_glm* model,
                           int chains, int n, const gbsgmc_integrator* integrator,
                           float* x_dev, float* aux_dev,
                           const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                           const gbsgmc_index_src* index_src, double* U_dev,
                           double* lk_var_dev, double* ke_dev, int block_steps,
                           int* status_dev);

/* Tempering of a network plan: replica r of R runs at the schedule's
 * temperature times chain_temperature_dev[r] (set in the plan's sched), and
 * every `every` steps adjacent replicas attempt an exchange
 * (gbsgmc_resgld_exchange_adjacent).  ssq_dev [R - 1], k_dev [1] (the SA
 * counter) and counts_dev [R - 1] are the caller's and persist across runs;
 * flags_dev [R - 1] receives the last round's exchanges. */
typedef struct gbsgmc_tempering {
  int every;
  int _pad;
  double F;
  uint64_t seed;
  double* ssq_dev;
  int64_t* k_dev;
  int32_t* counts_dev;
  int32_t* flags_dev;
} gbsgmc_tempering;

/* reSGLD on the dense network: R replicas of SGLD (+ rms_prop when v_dev is
 * not NULL) with per-replica minibatch sizes n_dev[r] <= n_max (device
 * memory, fixed for the plan's life), per-replica temperatures and the
 * adjacent exchanges above, `block_steps` steps per captured CUDA graph
 * (a multiple of `every`; plan_run's first step and step count must be
 * multiples of `every`).  Per step: index draws of n_max per replica (the
 * first n_dev[r] are used), gbsgmc_mlp_value_and_grad_ragged, the SGLD
 * update, the SA variance update, and at exchange steps the exchange.
 * Replaces alias.re_sgld (jax_sgmc/alias.py:121-229) run through
 * solver.mcmc, generalised from 2 replicas to R. */
int gbsgmc_mlp_resgld_plan_create(gbsgmc_plan** plan, const gbsgmc_mlp* model,
                                  int replicas, int n_max, const int32_t* n_dev,
                                  float* x_dev, float* v_dev, float alpha,
                                  float lmbd, const gbsgmc_sched* sched,
                                  const gbsgmc_noise* noise,
                                  const gbsgmc_index_src* index_src,
                                  const gbsgmc_tempering* tempering,
                                  double* U_dev, double* lk_var_dev,
                                  int block_steps, int* status_dev);

/* As gbsgmc_mlp_resgld_plan_create with kept samples: at the steps whose
 * keep slot (sched->keep_slot_dev) is >= 0, after that step's exchange
 * attempt, replica 0's positions go to samples_dev [slot, P] and its -U to
 * sample_lik_dev [slot] (may be NULL).  A keep table needs a sample buffer
 * and the other way round.  This is the ladder that alias.re_sgld_ladder
 * runs; the reference samples pairs of one normal and one hot chain only. */
int gbsgmc_mlp_resgld_plan_create_keep(gbsgmc_plan** plan, const gbsgmc_mlp* model,
                                       int replicas, int n_max, const int32_t* n_dev,
                                       float* x_dev, float* v_dev, float alpha, float lmbd,
                                       const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                                       const gbsgmc_index_src* index_src,
                                       const gbsgmc_tempering* tempering, double* U_dev,
                                       double* lk_var_dev, float* samples_dev,
                                       double* sample_lik_dev, int block_steps,
                                       int* status_dev);

/* reSGLD on a generalised-linear potential as alias.re_sgld runs it: `pairs`
 * pairs of a normal and a hot chain, plain SGLD (rms_prop when v_dev is not
 * NULL), and after every step each pair's exchange in FP64 with the rule of
 * solver.parallel_tempering.update (jax_sgmc/solver.py:264-293, the SA
 * schedule 1/k):  k_p += 1;  ssq_p <- (1 - 1/k_p) ssq_p + (1/k_p) var_normal;
 * log s = dbeta (U_normal - U_hot - dbeta ssq_p / F); the pair exchanges its
 * states unless log u < log s.  Chains are slots of [2 pairs, d] arrays
 * (x_dev, v_dev, U_dev, lk_var_dev): normal chain p in slot p, its hot
 * partner in slot pairs + p, each at the temperature T_k *
 * sched->chain_temperature_dev[slot].  An exchange swaps the two slots' x, v,
 * U, var(lk) and chain identities ident_dev[slot]: identity i (0 <= i <
 * 2 pairs) is the chain with index stream index_src->pcg_dev[i] and noise
 * chain id noise->chain_base + i, so streams travel with the states as the
 * reference's whole-state exchange moves them.  Pair p's uniform is
 * Philox(counter (0, k + 1, 0, GBSGMC_TAG_SWAP), key (tempering->seed << 32)
 * | pair_chain_dev[p]).  At kept steps the normal slots' x and -U go to
 * samples_dev [slot, pairs, d] and sample_lik_dev [slot, pairs]; swap counts
 * are added to tempering->counts_dev [pairs] when it is not NULL
 * (tempering->every and flags_dev are not used).  Per step: one fused SGLD
 * launch for all 2 pairs chains and one exchange launch; per block one
 * index-draw launch, replayed from a CUDA graph.
 * Replaces alias.re_sgld (jax_sgmc/alias.py:122-208) through solver.mcmc. */
int gbsgmc_glm_resgld_plan_create(gbsgmc_plan** plan, const gbsgmc_glm* model,
                                  int pairs, int n, float* x_dev, float* v_dev,
                                  float alpha, float lmbd,
                                  const gbsgmc_sched* sched,
                                  const gbsgmc_noise* noise,
                                  const gbsgmc_index_src* index_src,
                                  const gbsgmc_tempering* tempering,
                                  const int32_t* pair_chain_dev,
                                  int32_t* ident_dev, double* U_dev,
                                  double* lk_var_dev, float* samples_dev,
                                  double* sample_lik_dev, int block_steps,
                                  int* status_dev);

/* As gbsgmc_glm_resgld_plan_create on the dense network (MLP): the same pair
 * layout, identities, exchange rule, uniforms, kept samples and counts; per
 * step one batched value-and-gradient of all 2 pairs chains (row c reads its
 * minibatch from identity ident_dev[c]'s index stream), one SGLD update
 * (noise drawn as identity ident_dev[c]) and one exchange launch.  n a
 * positive multiple of 128.  Replaces alias.re_sgld (jax_sgmc/alias.py:
 * 122-208) through solver.mcmc on a network likelihood. */
int gbsgmc_mlp_resgld_pairs_plan_create(gbsgmc_plan** plan, const gbsgmc_mlp* model,
                                        int pairs, int n, float* x_dev, float* v_dev,
                                        float alpha, float lmbd, const gbsgmc_sched* sched,
                                        const gbsgmc_noise* noise,
                                        const gbsgmc_index_src* index_src,
                                        const gbsgmc_tempering* tempering,
                                        const int32_t* pair_chain_dev, int32_t* ident_dev,
                                        double* U_dev, double* lk_var_dev, float* samples_dev,
                                        double* sample_lik_dev, int block_steps,
                                        int* status_dev);

/* Runs steps [first_step, first_step + steps) of the plan, ordered after prior
 * work on `stream`; later work on `stream` waits for it.  Does not block the
 * host. */
int gbsgmc_plan_run(gbsgmc_plan* plan, int64_t first_step, int64_t steps,
                    gbsgmc_stream_t stream);

/* The launch shape the plan's autotuner chose for the fused step: CTAs per
 * chain, rows per warp, warps per CTA, whether each warp keeps two row tiles
 * in flight, whether the dynamically scheduled kernel runs (then `slices`
 * is the number of row items per chain that warps claim), and the steps one
 * launch runs (1, or the plan's block of steps); 0 = the library default.  The autotuner times a few
 * candidate shapes on scratch copies of the chain state when the plan is
 * created (GBSGMC_AUTOTUNE=0 disables it) and caches the choice per problem
 * shape for the process.  Network plans report zeros.  No reference
 * counterpart: launch configuration only. */
int gbsgmc_plan_launch_shape(const gbsgmc_plan* plan, int* slices,
                             int* rows_per_warp, int* warps, int* prefetch,
                             int* dynamic, int* steps_per_launch);

/* Kernel launches one plan_run of `steps` steps performs (for accounting). */
int64_t gbsgmc_plan_launches(const gbsgmc_plan* plan, int64_t steps);

/* Plans with an external index source (GLM SGLD, network and GLM OBABO /
 * SGHMC / SGLD plans): copies the indices of the next `steps` steps
 * (1 <= steps <= block_steps) into the plan, stream-ordered on `stream`.
 * src (host, pinned or pageable, or device) is [steps, chains, k * n]
 * int32, k the minibatches of one step (2 for OBABO, else 1), in the order
 * the chain's loader hands them out.  The next gbsgmc_plan_run on `stream`
 * must cover at most `steps` steps. */
int gbsgmc_plan_set_indices(gbsgmc_plan* plan, const int32_t* src, int steps,
                            gbsgmc_stream_t stream);

/* Releases the plan's graphs, stream and workspace (synchronises the plan's
 * internal stream first). */
int gbsgmc_plan_destroy(gbsgmc_plan* plan);

/* ------------------------------------------------------------------------ */
/* Plain (unfused) one-chain form, kept as the GPU comparison baseline       */
/* ------------------------------------------------------------------------ */

/* One SGLD(+RMSprop) step of ONE chain as separate kernels, the way an
 * op-by-op compiler lays it out: gather rows into a buffer, forward GEMV,
 * link, backward GEMV, reductions, prior, RMSprop, noise, update (8 launches).
 * `buf_dev` must hold gbsgmc_plain_buffer_bytes(n, d) bytes. */
size_t gbsgmc_plain_buffer_bytes(int n, int d);
int gbsgmc_plain_sgld_glm_step(const gbsgmc_glm* model, int n,
                               const int32_t* idx_dev, float* w_dev,
                               float* v_dev, float alpha, float lmbd,
                               const gbsgmc_sched* sched,
                               const gbsgmc_noise* noise, double* U_dev,
                               void* buf_dev, int* status_dev,
                               gbsgmc_stream_t stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* GBSGMC_H_ */
