// Batched symmetric eigendecomposition (the jnp.linalg.eigh of
// mass_matrix(diagonal=False), jax_sgmc/adaption.py:316), one CTA per
// matrix, by the round-robin cyclic Jacobi method of eig.cuh.
#include <algorithm>

#include "common.cuh"
#include "eig.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kEigThreads = 256;

size_t eig_smem(int Pp) {
  return sizeof(float) * 2 * static_cast<size_t>(Pp) * Pp + sizeof(float2) * (Pp / 2) +
         sizeof(float) * 32;
}

// Matrix b: load (zero-padded to Pp), diagonalise, then eigenvalue j goes to
// position rank(j) (ascending; equal values keep index order) with its
// sign-normalised eigenvector.
__global__ void __launch_bounds__(kEigThreads) sym_eig_kernel(int P, int Pp, const float* A_in,
                                                             float* w_out, float* V_out) {
  extern __shared__ __align__(16) float sm[];
  float* A = sm;
  float* V = A + Pp * Pp;
  float2* rot = reinterpret_cast<float2*>(V + Pp * Pp);
  float* red = reinterpret_cast<float*>(rot + Pp / 2);
  const int b = blockIdx.x;
  const float* src = A_in + static_cast<int64_t>(b) * P * P;
  for (int e = threadIdx.x; e < Pp * Pp; e += blockDim.x) {
    const int j = e / Pp, k = e % Pp;
    // The symmetric part, so that a slightly asymmetric input is well defined.
    A[e] = (j < P && k < P) ? 0.5f * (src[j * P + k] + src[k * P + j]) : 0.f;
  }
  __syncthreads();
  jacobi_eig(A, V, rot, red, Pp);
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    const float lj = A[j * Pp + j];
    int rank = 0;
    for (int k = 0; k < P; ++k) {
      const float lk = A[k * Pp + k];
      rank += (lk < lj || (lk == lj && k < j)) ? 1 : 0;
    }
    w_out[static_cast<int64_t>(b) * P + rank] = lj;
    const float sgn = eigvec_sign(V, Pp, P, j);
    float* dst = V_out + static_cast<int64_t>(b) * P * P;
    for (int k = 0; k < P; ++k) dst[k * P + rank] = sgn * V[k * Pp + j];
  }
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_sym_eig(int batch, int P, const float* A_dev, float* w_dev,
                              float* V_dev, gbsgmc_stream_t stream) {
  if (batch < 0 || batch > 65535 || P < 1 || P > kMaxEigDim)
    return set_error(GBSGMC_ERR_SHAPE, "sym_eig: needs 1 <= P <= %d (got %d)", kMaxEigDim, P);
  if (batch == 0) return GBSGMC_OK;
  if (A_dev == nullptr || w_dev == nullptr || V_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "sym_eig: null pointer");
  const int Pp = P + (P & 1);
  const size_t smem = eig_smem(Pp);
  cudaError_t e = cudaFuncSetAttribute(sym_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "sym_eig: %s", cudaGetErrorString(e));
  sym_eig_kernel<<<batch, kEigThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      P, Pp, A_dev, w_dev, V_dev);
  return check_launch("sym_eig");
}
