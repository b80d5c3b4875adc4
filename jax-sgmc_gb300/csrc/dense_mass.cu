// Dense mass matrices for the MH samplers: the integrator updates of the
// reversible leapfrog (AMAGOLD) and OBABO (SGGMC) with a full inverse mass
// M^-1 [P, P] and root mass M^1/2 [P, P] (the reference's tensor_matmul of
// a Tensor with ndim 2, util/tree_util.py:38-56, as integrator.py:170-273
// and 376-460 use it), and the adaption that estimates them
// (mass_matrix(diagonal=False), adaption.py:296-368).
//
// One CTA per chain: the chain's vectors (momentum, gradient, noise) are
// staged in shared memory, and each matrix-vector product is one warp per
// row reading the row coalesced from global memory (the matrices stay in
// L2 for the small P these are meant for).  The elementwise arithmetic is
// that of the diagonal kernels in update.cu with m^-1 p and sqrt(m) xi
// replaced by the products.
#include <algorithm>

#include "common.cuh"
#include "eig.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kDT = 256;
constexpr int64_t kMaxDenseP = 8192;  // four P-vectors in shared memory

// Row j of M [P, P] dotted with the shared-memory vector v, by one warp;
// every lane receives the sum.
__device__ __forceinline__ float row_dot(const float* __restrict__ M, int64_t P, int64_t j,
                                         const float* v, int lane) {
  const float* r = M + j * P;
  float acc = 0.f;
  for (int64_t k = lane; k < P; k += 32) acc = fmaf(__ldg(r + k), v[k], acc);
  return warp_sum(acc);
}

// Normals of the chain's noise stream (tag, step k) for all P entries.
__device__ __forceinline__ void stage_noise(const Noise& noise, int c, int64_t P, int64_t k,
                                            uint32_t tag, float* xi) {
  for (int64_t q = threadIdx.x; 4 * q < P; q += blockDim.x) {
    float v[4];
    noise4(noise, c, 4 * q, P, k, tag, v);
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (4 * q + e < P) xi[4 * q + e] = v[e];
  }
}

__device__ __forceinline__ void add_block(double* acc, int c, float part) {
  if (acc == nullptr) return;
  __shared__ double red[32];
  const double tot = block_sum(static_cast<double>(part), red);
  if (threadIdx.x == 0) atomicAdd(acc + c, tot);
}

// x <- x + (scale h) M^-1 p.
__global__ void __launch_bounds__(kDT) dense_position_kernel(int64_t P, float* x, const float* p,
                                                             const float* Minv, float scale,
                                                             Sched sched) {
  extern __shared__ float sv[];
  const int c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t off = static_cast<int64_t>(c) * P;
  const float s = scale * sched.step_size(sched.step());
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) sv[j] = p[off + j];
  __syncthreads();
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float m = row_dot(Minv, P, j, sv, lane);
    if (lane == 0) x[off + j] = x[off + j] + s * m;
  }
}

// p' = ((1 - h f) p - h g + sqrt(4 f h) (M^1/2 xi)) / (1 + h f) and
// energy[c] += 0.5 h sum_j (p_j + p'_j) (M^-1 g)_j, xi of tag AMAGOLD.
__global__ void __launch_bounds__(kDT) dense_amagold_kernel(int64_t P, float* p, const float* g,
                                                            const float* Minv,
                                                            const float* Msqrt, float friction,
                                                            double* energy, Sched sched,
                                                            Noise noise) {
  extern __shared__ float sv[];
  float* xi = sv;
  float* pv = sv + P;
  float* gv = sv + 2 * P;
  const int c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t off = static_cast<int64_t>(c) * P;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float decay = 1.0f - h * friction;
  const float inv = 1.0f / (1.0f + h * friction);
  const float ns = sqrtf(4.0f * friction * h);
  stage_noise(noise, c, P, k, GBSGMC_TAG_AMAGOLD, xi);
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    pv[j] = p[off + j];
    gv[j] = g[off + j];
  }
  __syncthreads();
  float part = 0.f;
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float n = row_dot(Msqrt, P, j, xi, lane);
    const float u = row_dot(Minv, P, j, gv, lane);
    if (lane == 0) {
      const float pn = inv * ((decay * pv[j] + (-h) * gv[j]) + ns * n);
      p[off + j] = pn;
      part += (pv[j] + pn) * u;
    }
  }
  add_block(energy, c, 0.5f * h * part);
}

struct DenseObabo {
  float h, keep, inject, half;
};
__device__ __forceinline__ DenseObabo dense_obabo_coef(const Sched& sched, int64_t k, int c,
                                                       float friction) {
  DenseObabo q;
  q.h = sched.step_size(k);
  const float T = sched.temperature(k, c);
  const float permanence = expf(-friction * q.h);
  q.keep = sqrtf(permanence);
  q.inject = sqrtf((1.0f - permanence) * T);
  q.half = 0.5f * q.h;
  return q;
}

// O (p <- keep p + inject M^1/2 xi1), ke_start += 0.5 p . M^-1 p,
// B (p <- p - h/2 g1), A (x <- x + h M^-1 p).
__global__ void __launch_bounds__(kDT) dense_obabo_first_kernel(
    int64_t P, float* x, float* p, const float* g1, const float* Minv, const float* Msqrt,
    float friction, double* ke_start, Sched sched, Noise noise) {
  extern __shared__ float sv[];
  float* xi = sv;      // the noise, then the momentum after B
  float* pv = sv + P;  // the momentum
  float* po = sv + 2 * P;  // the momentum after O
  const int c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t off = static_cast<int64_t>(c) * P;
  const int64_t k = sched.step();
  const DenseObabo q = dense_obabo_coef(sched, k, c, friction);
  stage_noise(noise, c, P, k, GBSGMC_TAG_OBABO_1, xi);
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) pv[j] = p[off + j];
  __syncthreads();
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float n = row_dot(Msqrt, P, j, xi, lane);
    if (lane == 0) po[j] = __fmaf_rn(q.keep, pv[j], __fmul_rn(q.inject, n));
  }
  __syncthreads();
  float ke = 0.f;
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float u = row_dot(Minv, P, j, po, lane);
    if (lane == 0) {
      ke = __fmaf_rn(__fmul_rn(0.5f, po[j]), u, ke);
      xi[j] = __fmaf_rn(-q.half, g1[off + j], po[j]);  // B
    }
  }
  __syncthreads();
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float u = row_dot(Minv, P, j, xi, lane);
    if (lane == 0) {
      x[off + j] = __fmaf_rn(q.h, u, x[off + j]);
      p[off + j] = xi[j];
    }
  }
  add_block(ke_start, c, ke);
}

// B (p <- p - h/2 g2), ke_end += 0.5 p . M^-1 p, O (p <- keep p + inject
// M^1/2 xi2).
__global__ void __launch_bounds__(kDT) dense_obabo_second_kernel(
    int64_t P, float* p, const float* g2, const float* Minv, const float* Msqrt,
    float friction, double* ke_end, Sched sched, Noise noise) {
  extern __shared__ float sv[];
  float* xi = sv;
  float* pb = sv + P;
  const int c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t off = static_cast<int64_t>(c) * P;
  const int64_t k = sched.step();
  const DenseObabo q = dense_obabo_coef(sched, k, c, friction);
  stage_noise(noise, c, P, k, GBSGMC_TAG_OBABO_2, xi);
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x)
    pb[j] = __fmaf_rn(-q.half, g2[off + j], p[off + j]);
  __syncthreads();
  float ke = 0.f;
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float u = row_dot(Minv, P, j, pb, lane);
    const float n = row_dot(Msqrt, P, j, xi, lane);
    if (lane == 0) {
      ke = __fmaf_rn(__fmul_rn(0.5f, pb[j]), u, ke);
      p[off + j] = __fmaf_rn(q.keep, pb[j], __fmul_rn(q.inject, n));
    }
  }
  add_block(ke_end, c, ke);
}

// y[c] = M x[c].
__global__ void __launch_bounds__(kDT) dense_matvec_kernel(int64_t P, const float* M,
                                                           const float* x, float* y) {
  extern __shared__ float sv[];
  const int c = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) sv[j] = x[off + j];
  __syncthreads();
  for (int64_t j = warp; j < P; j += blockDim.x / 32) {
    const float m = row_dot(M, P, j, sv, lane);
    if (lane == 0) y[off + j] = m;
  }
}

// One update of the dense mass adaption (adaption.py:342-362), fp32 in the
// reference's operation order: mean' = (i-1)/i mean + 1/i x and
// ssq += (x - mean) (x - mean')^T.  The mean is replaced by a second launch
// once every entry of ssq has read the old one.
__global__ void dense_ssq_kernel(int64_t P, int iteration, const float* x, const float* mean,
                                 float* ssq) {
  const float it = static_cast<float>(iteration);
  const float a = static_cast<float>(iteration - 1) / it;
  const float b = 1.0f / it;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < P * P;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j = e / P, k = e - j * P;
    const float nk = __fadd_rn(__fmul_rn(a, mean[k]), __fmul_rn(b, x[k]));
    ssq[e] = __fadd_rn(ssq[e], __fmul_rn(__fsub_rn(x[j], mean[j]), __fsub_rn(x[k], nk)));
  }
}

__global__ void dense_mean_kernel(int64_t P, int iteration, const float* x, float* mean,
                                  const float* ssq, float* inv, int finalize) {
  const float it = static_cast<float>(iteration);
  const float a = static_cast<float>(iteration - 1) / it;
  const float b = 1.0f / it;
  const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t j = tid; j < P; j += stride)
    mean[j] = __fadd_rn(__fmul_rn(a, mean[j]), __fmul_rn(b, x[j]));
  if (finalize)
    for (int64_t e = tid; e < P * P; e += stride) inv[e] = ssq[e] / it;
}

// sqrt = V^T diag(sqrt(w)) V from the eigendecomposition of inv, the
// product adaption.py:317 writes (with the eigenvectors as the columns of
// V); eigenvalues below zero (rounding of a rank-deficient estimate) count
// as zero.
__global__ void dense_root_kernel(int64_t P, const float* w, const float* V, float* out) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < P * P;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j = e / P, k = e - j * P;
    float acc = 0.f;
    for (int64_t m = 0; m < P; ++m)
      acc = fmaf(V[m * P + j] * sqrtf(fmaxf(w[m], 0.f)), V[m * P + k], acc);
    out[e] = acc;
  }
}

// Allows `bytes` of dynamic shared memory for kernel k (above the 48 KB
// default).
template <class K>
int allow_smem(K k, size_t bytes, const char* what) {
  if (bytes <= 48 * 1024) return GBSGMC_OK;
  const cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
  if (e != cudaSuccess) return set_error(GBSGMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return GBSGMC_OK;
}

int check_dense(int chains, int64_t P, const void* a, const void* b, const char* what) {
  if (chains < 0 || chains > 65535 || P < 1 || P > kMaxDenseP)
    return set_error(GBSGMC_ERR_SHAPE, "%s: needs 1 <= P <= %lld", what,
                     static_cast<long long>(kMaxDenseP));
  if (a == nullptr || b == nullptr) return set_error(GBSGMC_ERR_ARG, "%s: null pointer", what);
  return GBSGMC_OK;
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_leapfrog_position_dense(int chains, int64_t P, float* x_dev,
                                              const float* p_dev, const float* minv_dev,
                                              float scale, const gbsgmc_sched* sched,
                                              gbsgmc_stream_t stream) {
  int rc = check_dense(chains, P, x_dev, p_dev, "leapfrog_position_dense");
  if (rc != GBSGMC_OK) return rc;
  if (minv_dev == nullptr || sched == nullptr)
    return set_error(GBSGMC_ERR_ARG, "leapfrog_position_dense: null pointer");
  if (chains == 0) return GBSGMC_OK;
  if ((rc = allow_smem(dense_position_kernel, sizeof(float) * P, "leapfrog_position_dense"))) return rc;
  dense_position_kernel<<<chains, kDT, sizeof(float) * P, static_cast<cudaStream_t>(stream)>>>(
      P, x_dev, p_dev, minv_dev, scale, to_sched(sched));
  return check_launch("leapfrog_position_dense");
}

extern "C" int gbsgmc_amagold_momentum_dense(int chains, int64_t P, float* p_dev,
                                             const float* g_dev, const float* minv_dev,
                                             const float* msqrt_dev, float friction,
                                             double* energy_dev, const gbsgmc_sched* sched,
                                             const gbsgmc_noise* noise, gbsgmc_stream_t stream) {
  int rc = check_dense(chains, P, p_dev, g_dev, "amagold_momentum_dense");
  if (rc != GBSGMC_OK) return rc;
  if (minv_dev == nullptr || msqrt_dev == nullptr || sched == nullptr || noise == nullptr)
    return set_error(GBSGMC_ERR_ARG, "amagold_momentum_dense: null pointer");
  if (noise->noise_dev != nullptr)
    return set_error(GBSGMC_ERR_ARG, "amagold_momentum_dense: injected noise is not supported");
  if (chains == 0) return GBSGMC_OK;
  if ((rc = allow_smem(dense_amagold_kernel, 3 * sizeof(float) * P, "amagold_momentum_dense"))) return rc;
  dense_amagold_kernel<<<chains, kDT, 3 * sizeof(float) * P,
                         static_cast<cudaStream_t>(stream)>>>(
      P, p_dev, g_dev, minv_dev, msqrt_dev, friction, energy_dev, to_sched(sched),
      to_noise(noise));
  return check_launch("amagold_momentum_dense");
}

extern "C" int gbsgmc_obabo_first_dense(int chains, int64_t P, float* x_dev, float* p_dev,
                                        const float* g1_dev, const float* minv_dev,
                                        const float* msqrt_dev, float friction,
                                        double* ke_start_dev, const gbsgmc_sched* sched,
                                        const gbsgmc_noise* noise, gbsgmc_stream_t stream) {
  int rc = check_dense(chains, P, x_dev, p_dev, "obabo_first_dense");
  if (rc != GBSGMC_OK) return rc;
  if (g1_dev == nullptr || minv_dev == nullptr || msqrt_dev == nullptr || sched == nullptr ||
      noise == nullptr)
    return set_error(GBSGMC_ERR_ARG, "obabo_first_dense: null pointer");
  if (noise->noise_dev != nullptr)
    return set_error(GBSGMC_ERR_ARG, "obabo_first_dense: injected noise is not supported");
  if (chains == 0) return GBSGMC_OK;
  if ((rc = allow_smem(dense_obabo_first_kernel, 3 * sizeof(float) * P, "obabo_first_dense"))) return rc;
  dense_obabo_first_kernel<<<chains, kDT, 3 * sizeof(float) * P,
                             static_cast<cudaStream_t>(stream)>>>(
      P, x_dev, p_dev, g1_dev, minv_dev, msqrt_dev, friction, ke_start_dev, to_sched(sched),
      to_noise(noise));
  return check_launch("obabo_first_dense");
}

extern "C" int gbsgmc_obabo_second_dense(int chains, int64_t P, float* p_dev,
                                         const float* g2_dev, const float* minv_dev,
                                         const float* msqrt_dev, float friction,
                                         double* ke_end_dev, const gbsgmc_sched* sched,
                                         const gbsgmc_noise* noise, gbsgmc_stream_t stream) {
  int rc = check_dense(chains, P, p_dev, g2_dev, "obabo_second_dense");
  if (rc != GBSGMC_OK) return rc;
  if (minv_dev == nullptr || msqrt_dev == nullptr || sched == nullptr || noise == nullptr)
    return set_error(GBSGMC_ERR_ARG, "obabo_second_dense: null pointer");
  if (noise->noise_dev != nullptr)
    return set_error(GBSGMC_ERR_ARG, "obabo_second_dense: injected noise is not supported");
  if (chains == 0) return GBSGMC_OK;
  if ((rc = allow_smem(dense_obabo_second_kernel, 2 * sizeof(float) * P, "obabo_second_dense"))) return rc;
  dense_obabo_second_kernel<<<chains, kDT, 2 * sizeof(float) * P,
                              static_cast<cudaStream_t>(stream)>>>(
      P, p_dev, g2_dev, minv_dev, msqrt_dev, friction, ke_end_dev, to_sched(sched),
      to_noise(noise));
  return check_launch("obabo_second_dense");
}

extern "C" int gbsgmc_dense_matvec(int chains, int64_t P, const float* m_dev,
                                   const float* x_dev, float* y_dev, gbsgmc_stream_t stream) {
  int rc = check_dense(chains, P, m_dev, x_dev, "dense_matvec");
  if (rc != GBSGMC_OK) return rc;
  if (y_dev == nullptr) return set_error(GBSGMC_ERR_ARG, "dense_matvec: null pointer");
  if (chains == 0) return GBSGMC_OK;
  if ((rc = allow_smem(dense_matvec_kernel, sizeof(float) * P, "dense_matvec"))) return rc;
  dense_matvec_kernel<<<chains, kDT, sizeof(float) * P, static_cast<cudaStream_t>(stream)>>>(
      P, m_dev, x_dev, y_dev);
  return check_launch("dense_matvec");
}

extern "C" int gbsgmc_mass_adapt_dense(int64_t P, int iteration, int burn_in,
                                       const float* x_dev, float* mean_dev, float* ssq_dev,
                                       float* inv_dev, float* sqrt_dev, float* eig_w_dev,
                                       float* eig_v_dev, gbsgmc_stream_t stream) {
  if (P < 1 || P > kMaxEigDim)
    return set_error(GBSGMC_ERR_SHAPE, "mass_adapt_dense: needs 1 <= P <= %d", kMaxEigDim);
  if (iteration < 1)
    return set_error(GBSGMC_ERR_ARG, "mass_adapt_dense: iteration counts from 1");
  if (!x_dev || !mean_dev || !ssq_dev || !inv_dev || !sqrt_dev)
    return set_error(GBSGMC_ERR_ARG, "mass_adapt_dense: null pointer");
  const bool fin = iteration == burn_in;
  if (fin && (eig_w_dev == nullptr || eig_v_dev == nullptr))
    return set_error(GBSGMC_ERR_ARG, "mass_adapt_dense: the final update needs eig buffers");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int blocks = static_cast<int>(std::min<int64_t>((P * P + 255) / 256, 1024));
  dense_ssq_kernel<<<blocks, 256, 0, s>>>(P, iteration, x_dev, mean_dev, ssq_dev);
  int rc = check_launch("mass_adapt_dense");
  if (rc != GBSGMC_OK) return rc;
  dense_mean_kernel<<<blocks, 256, 0, s>>>(P, iteration, x_dev, mean_dev, ssq_dev, inv_dev,
                                           fin ? 1 : 0);
  if ((rc = check_launch("mass_adapt_dense"))) return rc;
  if (!fin) return GBSGMC_OK;
  if ((rc = gbsgmc_sym_eig(1, static_cast<int>(P), inv_dev, eig_w_dev, eig_v_dev, stream)))
    return rc;
  dense_root_kernel<<<blocks, 256, 0, s>>>(P, eig_w_dev, eig_v_dev, sqrt_dev);
  return check_launch("mass_adapt_dense");
}
