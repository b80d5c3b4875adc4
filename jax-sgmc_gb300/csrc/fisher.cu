// The empirical-Fisher noise model of SGHMC on the generalised-linear
// families (adaption.py:371-457, fisher_information(diagonal=True)), and the
// SGHMC momentum update that uses it (integrator.py:630-647).
//
// For a minibatch of n rows and the potential's gradient G = dU/dw at w:
//   gbar = G / N
//   ssq_j = sum_i (d lk_i / d w_j - gbar_j)^2,  d lk_i / d w = lk'(z_i) x_i
//   v = ssq / (n - 1),  b = 0.5 h v,  corr = friction - b
//   corr <= 0 is replaced by the smallest positive corr of the chain
//   cb_diff_sqrt = sqrt(corr),  b_sqrt = sqrt(friction - corr)
// (the per-observation gradients are of the likelihood, not the potential,
// and are compared with gbar as the reference writes it).  One CTA per
// chain: first z_i and lk'(z_i) of every row (a warp per row), then each
// thread sums its features over the rows; fp32 throughout like the
// reference.
#include <algorithm>
#include <cfloat>

#include "common.cuh"
#include "eig.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxRows = 4096;  // rows and their derivatives in shared memory

struct FisherArgs {
  int family, d;
  int64_t ld, n_rows;
  const float* X;
  const float* y;
  int y_inline;
  float inv_s2;  // 1 / sigma^2 (linear-Gaussian)
  int n;
  const int32_t* idx;
  int64_t idx_stride;
  const float* w;     // [chains, d]
  const float* grad;  // [chains, d], dU/dw
  float n_obs;
  const float* fric;  // [d] or null
  float friction;
  float h;
  float* cb;          // [chains, d]
  float* bs;          // [chains, d] or null
  int* status;
};

__global__ void __launch_bounds__(kThreads) glm_fisher_kernel(FisherArgs a) {
  __shared__ int32_t rows[kMaxRows];
  __shared__ float dlk[kMaxRows];
  __shared__ float red[32];
  const int c = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* wc = a.w + static_cast<int64_t>(c) * a.d;
  // Pass 1: the likelihood derivative of every row.
  for (int i = warp; i < a.n; i += kThreads / 32) {
    int32_t o = a.idx[static_cast<int64_t>(c) * a.idx_stride + i];
    if (o < 0 || o >= a.n_rows) {
      if (lane == 0) raise_status(a.status, GBSGMC_ERR_INDEX);
      o = -1;
    }
    float z = 0.f;
    if (o >= 0) {
      const float* xr = a.X + static_cast<int64_t>(o) * a.ld;
      for (int j = lane; j < a.d; j += 32) z = fmaf(xr[j], wc[j], z);
    }
    z = warp_sum(z);
    if (lane == 0) {
      float g = 0.f;
      if (o >= 0 && a.family == GBSGMC_GLM_LINEAR) {
        g = 1.0f;  // lk = z: y is not read
      } else if (o >= 0) {
        const float yv = a.y_inline ? a.X[static_cast<int64_t>(o) * a.ld + a.d] : a.y[o];
        g = a.family == GBSGMC_GLM_LINEAR_GAUSSIAN ? (yv - z) * a.inv_s2
                                                   : yv - 1.0f / (1.0f + expf(-z));
      }
      rows[i] = o;
      dlk[i] = g;
    }
  }
  __syncthreads();
  // Pass 2: per feature, the squared deviations summed over the rows.
  const float scale_v = 1.0f / static_cast<float>(a.n - 1);
  float corr[1024 / kThreads];
  float minpos = FLT_MAX;
  bool any_pos = false;
#pragma unroll
  for (int q = 0; q < 1024 / kThreads; ++q) {
    const int j = threadIdx.x + q * kThreads;
    corr[q] = 0.f;
    if (j >= a.d) continue;
    const float gbar = a.grad[static_cast<int64_t>(c) * a.d + j] / a.n_obs;
    float ssq = 0.f;
    for (int i = 0; i < a.n; ++i) {
      const int32_t o = rows[i];
      const float xij = o >= 0 ? a.X[static_cast<int64_t>(o) * a.ld + j] : 0.f;
      const float dev = dlk[i] * xij - gbar;
      ssq = fmaf(dev, dev, ssq);
    }
    const float v = scale_v * ssq;
    const float b = 0.5f * a.h * v;
    const float f = a.fric != nullptr ? a.fric[j] : a.friction;
    corr[q] = f - b;
    if (corr[q] > 0.f) {
      any_pos = true;
      minpos = fminf(minpos, corr[q]);
    }
  }
  // The chain's smallest positive correction (infinity when there is none).
  float m = any_pos ? minpos : INFINITY;
  for (int s = 16; s > 0; s >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, s));
  if (lane == 0) red[warp] = m;
  __syncthreads();
  float smallest = INFINITY;
  for (int w = 0; w < kThreads / 32; ++w) smallest = fminf(smallest, red[w]);
#pragma unroll
  for (int q = 0; q < 1024 / kThreads; ++q) {
    const int j = threadIdx.x + q * kThreads;
    if (j >= a.d) continue;
    const float f = a.fric != nullptr ? a.fric[j] : a.friction;
    const float pc = corr[q] <= 0.f ? smallest : corr[q];
    a.cb[static_cast<int64_t>(c) * a.d + j] = sqrtf(pc);
    if (a.bs != nullptr) a.bs[static_cast<int64_t>(c) * a.d + j] = sqrtf(f - pc);
  }
}

// The dense form (fisher_information(diagonal=False), adaption.py:441-452):
// with d_i = lk'(z_i) x_i - gbar,
//   b = 0.5 h / (n - 1) sum_i d_i d_i^T                        [d, d]
//   (u, s) = svd(diag(friction) - b),  cb_diff_sqrt = u sqrt(s)  [d]
//   (u, s) = svd(b),                   b_sqrt = u sqrt(s)        [d]
// (the products of the left singular vectors with the root singular values
// are vectors, which the integrator then applies elementwise).  Both
// matrices are symmetric, so their SVDs come from one eigendecomposition
// each: singular values |lambda|, left singular vectors the eigenvectors,
// with the eigenvector signs of eig.cuh (LAPACK's are not specified).  One
// CTA per chain, d <= kMaxEigDim: the rows' derivatives, then b accumulated
// tile by tile in shared memory, then the two Jacobi solves.
constexpr int kDenseTile = 16;

size_t dense_fisher_smem(int n, int Pp) {
  return sizeof(int32_t) * n + sizeof(float) * n +              // rows, dlk
         sizeof(float) * 2 * static_cast<size_t>(Pp) * Pp +     // A, V
         sizeof(float) * kDenseTile * Pp + sizeof(float) * Pp + // tile, gbar
         sizeof(float) * Pp + sizeof(float2) * (Pp / 2) +       // friction, rot
         sizeof(float) * 32;                                    // red
}

// out[k] = sum_j sign_j V[k, j] sqrt(|shift - A[j, j]|) over the d real
// eigenpairs (shift 0 and the eigenvalues of A themselves, or, for
// shift * I - A, its eigenvalues with A's eigenvectors).
__device__ void root_combination(const float* A, const float* V, int Pp, int d,
                                 float shift, float sign, float* out) {
  for (int k = threadIdx.x; k < d; k += blockDim.x) {
    float acc = 0.f;
    for (int j = 0; j < d; ++j)
      acc = fmaf(eigvec_sign(V, Pp, d, j) * V[k * Pp + j],
                 sqrtf(fabsf(shift + sign * A[j * Pp + j])), acc);
    out[k] = acc;
  }
}

__global__ void __launch_bounds__(kThreads) glm_fisher_dense_kernel(FisherArgs a, int Pp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = a.n, d = a.d;
  float* A = reinterpret_cast<float*>(smem_raw);
  float* V = A + Pp * Pp;
  float* tile = V + Pp * Pp;
  float* gbar = tile + kDenseTile * Pp;
  float* fr = gbar + Pp;
  float2* rot = reinterpret_cast<float2*>(fr + Pp);
  float* red = reinterpret_cast<float*>(rot + Pp / 2);
  float* dlk = red + 32;
  int32_t* rows = reinterpret_cast<int32_t*>(dlk + n);
  const int c = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float* wc = a.w + static_cast<int64_t>(c) * d;
  // The likelihood derivative of every row (as the diagonal kernel).
  for (int i = warp; i < n; i += kThreads / 32) {
    int32_t o = a.idx[static_cast<int64_t>(c) * a.idx_stride + i];
    if (o < 0 || o >= a.n_rows) {
      if (lane == 0) raise_status(a.status, GBSGMC_ERR_INDEX);
      o = -1;
    }
    float z = 0.f;
    if (o >= 0) {
      const float* xr = a.X + static_cast<int64_t>(o) * a.ld;
      for (int j = lane; j < d; j += 32) z = fmaf(xr[j], wc[j], z);
    }
    z = warp_sum(z);
    if (lane == 0) {
      float g = 0.f;
      if (o >= 0 && a.family == GBSGMC_GLM_LINEAR) {
        g = 1.0f;
      } else if (o >= 0) {
        const float yv = a.y_inline ? a.X[static_cast<int64_t>(o) * a.ld + d] : a.y[o];
        g = a.family == GBSGMC_GLM_LINEAR_GAUSSIAN ? (yv - z) * a.inv_s2
                                                   : yv - 1.0f / (1.0f + expf(-z));
      }
      rows[i] = o;
      dlk[i] = g;
    }
  }
  for (int j = threadIdx.x; j < Pp; j += kThreads) {
    gbar[j] = j < d ? a.grad[static_cast<int64_t>(c) * d + j] / a.n_obs : 0.f;
    fr[j] = j < d ? (a.fric != nullptr ? a.fric[j] : a.friction) : 0.f;
  }
  for (int e = threadIdx.x; e < Pp * Pp; e += kThreads) A[e] = 0.f;
  __syncthreads();
  // sum_i d_i d_i^T, kDenseTile rows at a time.
  for (int i0 = 0; i0 < n; i0 += kDenseTile) {
    const int rn = min(kDenseTile, n - i0);
    for (int e = threadIdx.x; e < kDenseTile * Pp; e += kThreads) {
      const int r = e / Pp, j = e - r * Pp;
      float v = 0.f;
      if (r < rn && j < d) {
        const int32_t o = rows[i0 + r];
        const float xij = o >= 0 ? a.X[static_cast<int64_t>(o) * a.ld + j] : 0.f;
        v = dlk[i0 + r] * xij - gbar[j];
      }
      tile[e] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < Pp * Pp; e += kThreads) {
      const int j = e / Pp, k = e - j * Pp;
      float acc = A[e];
      for (int r = 0; r < rn; ++r) acc = fmaf(tile[r * Pp + j], tile[r * Pp + k], acc);
      A[e] = acc;
    }
    __syncthreads();
  }
  // b, kept in A; its eigendecomposition gives b_sqrt.
  const float scale = 0.5f * a.h / static_cast<float>(n - 1);
  for (int e = threadIdx.x; e < Pp * Pp; e += kThreads) A[e] *= scale;
  __syncthreads();
  jacobi_eig(A, V, rot, red, Pp);
  if (a.bs != nullptr)
    root_combination(A, V, Pp, d, 0.f, 1.f, a.bs + static_cast<int64_t>(c) * d);
  // With one friction for every parameter, f I - b has b's eigenvectors and
  // the eigenvalues f - lambda: no second solve (whose nearly equal
  // eigenvalues would make its eigenvectors inaccurate in fp32).
  bool uniform = true;
  for (int j = 1; j < d; ++j) uniform = uniform && fr[j] == fr[0];
  if (uniform) {
    root_combination(A, V, Pp, d, fr[0], -1.f, a.cb + static_cast<int64_t>(c) * d);
    return;
  }
  __syncthreads();
  // diag(friction) - b = diag(friction) - V diag(lambda) V^T, then its own
  // eigendecomposition gives cb_diff_sqrt.
  float* lam = gbar;  // gbar is no longer needed
  for (int j = threadIdx.x; j < Pp; j += kThreads) lam[j] = j < d ? A[j * Pp + j] : 0.f;
  __syncthreads();
  for (int e = threadIdx.x; e < Pp * Pp; e += kThreads) {
    const int j = e / Pp, k = e - j * Pp;
    float acc = 0.f;
    for (int m = 0; m < d; ++m) acc = fmaf(V[j * Pp + m] * lam[m], V[k * Pp + m], acc);
    A[e] = (j == k ? fr[j] : 0.f) - acc;
  }
  __syncthreads();
  jacobi_eig(A, V, rot, red, Pp);
  root_combination(A, V, Pp, d, 0.f, 1.f, a.cb + static_cast<int64_t>(c) * d);
}

// p <- p - h g + sqrt(2h) (cb_diff_sqrt * xi), xi from tag GBSGMC_TAG_SGHMC_STEP
// (integrator.py:621-647 with a noise model).
__global__ void sghmc_momentum_model_kernel(int64_t P, float* p, const float* g,
                                            const float* cb, Sched sched, Noise noise) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float root = sqrtf(2.0f * h);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float xi[4];
    noise4(noise, c, 4 * q, P, k, GBSGMC_TAG_SGHMC_STEP, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t j = 4 * q + e;
      if (j >= P) break;
      float pj = p[off + j] + (-h) * g[off + j];
      pj = pj + root * (cb[off + j] * xi[e]);
      p[off + j] = pj;
    }
  }
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_glm_fisher_noise(const gbsgmc_glm* m, int chains, int n,
                                       const int32_t* idx_dev, int64_t idx_stride,
                                       const float* w_dev, const float* grad_dev,
                                       const float* friction_dev, float friction,
                                       float step_size, float* cb_diff_sqrt_dev,
                                       float* b_sqrt_dev, int* status_dev,
                                       gbsgmc_stream_t stream) {
  if (m == nullptr || idx_dev == nullptr || w_dev == nullptr || grad_dev == nullptr ||
      cb_diff_sqrt_dev == nullptr || status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise: null pointer");
  if (m->family != GBSGMC_GLM_LINEAR_GAUSSIAN && m->family != GBSGMC_GLM_LOGISTIC &&
      m->family != GBSGMC_GLM_LINEAR)
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise: unknown family %d", m->family);
  if (m->d < 1 || m->d > 1024 || m->ld < m->d + (m->y_inline ? 1 : 0) || m->n_obs < 1 ||
      m->X == nullptr ||
      (m->family != GBSGMC_GLM_LINEAR && !m->y_inline && m->y == nullptr))
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise: bad model");
  if (chains < 0 || chains > 65535 || n < 2 || n > kMaxRows || idx_stride < n)
    return set_error(GBSGMC_ERR_SHAPE,
                     "glm_fisher_noise: needs 2 <= n <= %d and idx_stride >= n", kMaxRows);
  if (m->family == GBSGMC_GLM_LINEAR_GAUSSIAN && !(m->sigma > 0.0f))
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise: sigma must be positive");
  if (chains == 0) return GBSGMC_OK;
  FisherArgs a;
  a.family = m->family;
  a.d = m->d;
  a.ld = m->ld;
  a.n_rows = m->n_rows > 0 ? m->n_rows : m->n_obs;
  a.X = m->X;
  a.y = m->y;
  a.y_inline = m->y_inline ? 1 : 0;
  a.inv_s2 = m->family == GBSGMC_GLM_LINEAR_GAUSSIAN ? 1.0f / (m->sigma * m->sigma) : 0.f;
  a.n = n;
  a.idx = idx_dev;
  a.idx_stride = idx_stride;
  a.w = w_dev;
  a.grad = grad_dev;
  a.n_obs = static_cast<float>(m->n_obs);
  a.fric = friction_dev;
  a.friction = friction;
  a.h = step_size;
  a.cb = cb_diff_sqrt_dev;
  a.bs = b_sqrt_dev;
  a.status = status_dev;
  glm_fisher_kernel<<<chains, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
  return check_launch("glm_fisher_noise");
}

extern "C" int gbsgmc_glm_fisher_noise_dense(const gbsgmc_glm* m, int chains, int n,
                                             const int32_t* idx_dev, int64_t idx_stride,
                                             const float* w_dev, const float* grad_dev,
                                             const float* friction_dev, float friction,
                                             float step_size, float* cb_diff_sqrt_dev,
                                             float* b_sqrt_dev, int* status_dev,
                                             gbsgmc_stream_t stream) {
  if (m == nullptr || idx_dev == nullptr || w_dev == nullptr || grad_dev == nullptr ||
      cb_diff_sqrt_dev == nullptr || status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise_dense: null pointer");
  if (m->family != GBSGMC_GLM_LINEAR_GAUSSIAN && m->family != GBSGMC_GLM_LOGISTIC &&
      m->family != GBSGMC_GLM_LINEAR)
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise_dense: unknown family %d",
                     m->family);
  if (m->d < 1 || m->ld < m->d + (m->y_inline ? 1 : 0) || m->n_obs < 1 || m->X == nullptr ||
      (m->family != GBSGMC_GLM_LINEAR && !m->y_inline && m->y == nullptr))
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise_dense: bad model");
  if (m->d > kMaxEigDim)
    return set_error(GBSGMC_ERR_SHAPE,
                     "glm_fisher_noise_dense: the dense noise model needs d <= %d (got %d)",
                     kMaxEigDim, m->d);
  if (chains < 0 || chains > 65535 || n < 2 || n > kMaxRows || idx_stride < n)
    return set_error(GBSGMC_ERR_SHAPE,
                     "glm_fisher_noise_dense: needs 2 <= n <= %d and idx_stride >= n",
                     kMaxRows);
  if (m->family == GBSGMC_GLM_LINEAR_GAUSSIAN && !(m->sigma > 0.0f))
    return set_error(GBSGMC_ERR_ARG, "glm_fisher_noise_dense: sigma must be positive");
  if (chains == 0) return GBSGMC_OK;
  FisherArgs a;
  a.family = m->family;
  a.d = m->d;
  a.ld = m->ld;
  a.n_rows = m->n_rows > 0 ? m->n_rows : m->n_obs;
  a.X = m->X;
  a.y = m->y;
  a.y_inline = m->y_inline ? 1 : 0;
  a.inv_s2 = m->family == GBSGMC_GLM_LINEAR_GAUSSIAN ? 1.0f / (m->sigma * m->sigma) : 0.f;
  a.n = n;
  a.idx = idx_dev;
  a.idx_stride = idx_stride;
  a.w = w_dev;
  a.grad = grad_dev;
  a.n_obs = static_cast<float>(m->n_obs);
  a.fric = friction_dev;
  a.friction = friction;
  a.h = step_size;
  a.cb = cb_diff_sqrt_dev;
  a.bs = b_sqrt_dev;
  a.status = status_dev;
  const int Pp = m->d + (m->d & 1);
  const size_t smem = dense_fisher_smem(n, Pp);
  if (smem > 227 * 1024)
    return set_error(GBSGMC_ERR_SHAPE,
                     "glm_fisher_noise_dense: d = %d with n = %d needs %zu bytes of shared "
                     "memory", m->d, n, smem);
  const cudaError_t e = cudaFuncSetAttribute(
      glm_fisher_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
      static_cast<int>(smem));
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "glm_fisher_noise_dense: %s", cudaGetErrorString(e));
  glm_fisher_dense_kernel<<<chains, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(a, Pp);
  return check_launch("glm_fisher_noise_dense");
}

extern "C" int gbsgmc_sghmc_momentum_noise_model(int chains, int64_t P, float* p_dev,
                                                 const float* g_dev,
                                                 const float* cb_diff_sqrt_dev,
                                                 const gbsgmc_sched* sched,
                                                 const gbsgmc_noise* noise,
                                                 gbsgmc_stream_t stream) {
  if (chains < 0 || chains > 65535 || P < 0)
    return set_error(GBSGMC_ERR_ARG, "sghmc_momentum_noise_model: bad chains/P");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  if (!p_dev || !g_dev || !cb_diff_sqrt_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "sghmc_momentum_noise_model: null pointer");
  const int64_t groups = (P + 3) / 4;
  int64_t bx = std::min<int64_t>((groups + kThreads - 1) / kThreads,
                                 std::max<int64_t>(4, (152 * 8 + chains - 1) / chains));
  bx = std::max<int64_t>(1, std::min<int64_t>(bx, 65535));
  const dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(chains));
  sghmc_momentum_model_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      P, p_dev, g_dev, cb_diff_sqrt_dev, to_sched(sched), to_noise(noise));
  return check_launch("sghmc_momentum_noise_model");
}
