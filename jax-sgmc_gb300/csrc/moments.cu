// Statistics of kept samples on the device: FP64 posterior moments of the
// sample buffers (the reference streams every sample to the host,
// io.py:626-771, and leaves the moments to the user) and the diagonal mass
// matrix adaption of the MH samplers (adaption.py:296-368).
//
// Moments use shifted sums: for each parameter the first kept sample is the
// shift s (fp32), and the sums S1 = sum (x - s), S2 = sum (x - s)^2 run in
// fp64.  The difference d = x - s of two fp32 values is exact in fp64
// whenever their exponents differ by less than 29; its square can need up to
// twice d's significant bits, so S2 += d*d is one fma that rounds once (a
// relative error of at most 2^-53 per added term).  The other roundings are
// the fp64 additions of S1 and the final mean = s + S1 / n,
// variance = (S2 - S1 (S1 / n)) / n.
// Accumulating more samples later just continues the sums.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kThreads = 256;

// Grid (blocks over P, chains): one thread per parameter, striding over P;
// for each parameter the K samples are read at slot stride, each read
// coalesced across the warp.
__global__ void moments_accumulate_kernel(int64_t P, int K, const float* __restrict__ samples,
                                          int64_t slot_stride, int64_t chain_stride,
                                          int64_t seen, float* __restrict__ shift,
                                          double* __restrict__ s1, double* __restrict__ s2) {
  const int c = blockIdx.y;
  const float* base = samples + static_cast<int64_t>(c) * chain_stride;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < P;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float sh;
    double a1, a2;
    if (seen == 0) {
      sh = base[j];
      shift[off + j] = sh;
      a1 = 0.0;
      a2 = 0.0;
    } else {
      sh = shift[off + j];
      a1 = s1[off + j];
      a2 = s2[off + j];
    }
    const double shd = static_cast<double>(sh);
    for (int k = 0; k < K; ++k) {
      const double d = static_cast<double>(base[k * slot_stride + j]) - shd;
      a1 += d;
      a2 = fma(d, d, a2);
    }
    s1[off + j] = a1;
    s2[off + j] = a2;
  }
}

__global__ void moments_finalize_kernel(int64_t total, double n, const float* __restrict__ shift,
                                        const double* __restrict__ s1,
                                        const double* __restrict__ s2,
                                        double* __restrict__ mean, double* __restrict__ var) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double m1 = s1[i] / n;
    mean[i] = static_cast<double>(shift[i]) + m1;
    const double v = (s2[i] - s1[i] * m1) / n;
    var[i] = v > 0.0 ? v : 0.0;
  }
}

// One adaption update of the diagonal mass (adaption.py:342-362), fp32 as
// the reference computes it, the operations in its order and unfused:
//   mean' = (i - 1) / i * mean + 1 / i * x
//   ssq  += (x - mean) (x - mean')
// and at i == burn_in the inverse mass ssq / i and its root's reciprocal
// sqrt(i / ssq) (adaption.py:309-319), with the mass itself i / ssq.
__global__ void mass_adapt_kernel(int64_t P, int iteration, int burn_in,
                                  const float* __restrict__ x, float* __restrict__ mean,
                                  float* __restrict__ ssq, float* __restrict__ inv,
                                  float* __restrict__ sqrt_m, float* __restrict__ mass) {
  const float it = static_cast<float>(iteration);
  const float a = static_cast<float>(iteration - 1) / it;
  const float b = 1.0f / it;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < P;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float xj = x[j], mj = mean[j];
    const float nm = __fadd_rn(__fmul_rn(a, mj), __fmul_rn(b, xj));
    const float s = __fadd_rn(ssq[j], __fmul_rn(__fsub_rn(xj, mj), __fsub_rn(xj, nm)));
    mean[j] = nm;
    ssq[j] = s;
    if (iteration == burn_in) {
      inv[j] = s / it;
      const float r = it / s;
      sqrt_m[j] = sqrtf(r);
      if (mass != nullptr) mass[j] = r;
    }
  }
}

int grid_x(int chains, int64_t P) {
  int64_t bx = (P + kThreads - 1) / kThreads;
  const int64_t fill = std::max<int64_t>(1, (152 * 8 + chains - 1) / std::max(chains, 1));
  bx = std::min<int64_t>(std::min<int64_t>(bx, fill), 65535);
  return static_cast<int>(std::max<int64_t>(bx, 1));
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_moments_accumulate(int chains, int64_t P, int count,
                                         const float* samples_dev, int64_t slot_stride,
                                         int64_t chain_stride, int64_t seen,
                                         float* shift_dev, double* s1_dev, double* s2_dev,
                                         gbsgmc_stream_t stream) {
  if (chains < 0 || chains > 65535 || P < 0 || count < 0 || seen < 0)
    return set_error(GBSGMC_ERR_ARG, "moments_accumulate: bad chains/P/count/seen");
  if (chains == 0 || P == 0 || count == 0) return GBSGMC_OK;
  if (!samples_dev || !shift_dev || !s1_dev || !s2_dev)
    return set_error(GBSGMC_ERR_ARG, "moments_accumulate: null pointer");
  if ((count > 1 && slot_stride < P) || (chains > 1 && chain_stride < P))
    return set_error(GBSGMC_ERR_ARG, "moments_accumulate: strides below P");
  const dim3 grid(grid_x(chains, P), chains);
  moments_accumulate_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      P, count, samples_dev, slot_stride, chain_stride, seen, shift_dev, s1_dev, s2_dev);
  return check_launch("moments_accumulate");
}

extern "C" int gbsgmc_moments_finalize(int chains, int64_t P, int64_t n,
                                       const float* shift_dev, const double* s1_dev,
                                       const double* s2_dev, double* mean_dev,
                                       double* var_dev, gbsgmc_stream_t stream) {
  if (chains < 0 || P < 0 || n < 1)
    return set_error(GBSGMC_ERR_ARG, "moments_finalize: bad chains/P/n");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  if (!shift_dev || !s1_dev || !s2_dev || !mean_dev || !var_dev)
    return set_error(GBSGMC_ERR_ARG, "moments_finalize: null pointer");
  const int64_t total = static_cast<int64_t>(chains) * P;
  const int blocks = static_cast<int>(std::min<int64_t>((total + kThreads - 1) / kThreads,
                                                        152 * 16));
  moments_finalize_kernel<<<blocks, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      total, static_cast<double>(n), shift_dev, s1_dev, s2_dev, mean_dev, var_dev);
  return check_launch("moments_finalize");
}

extern "C" int gbsgmc_mass_adapt(int64_t P, int iteration, int burn_in, const float* x_dev,
                                 float* mean_dev, float* ssq_dev, float* inv_dev,
                                 float* sqrt_dev, float* mass_dev, gbsgmc_stream_t stream) {
  if (P < 0 || iteration < 1)
    return set_error(GBSGMC_ERR_ARG, "mass_adapt: bad P/iteration");
  if (P == 0) return GBSGMC_OK;
  if (!x_dev || !mean_dev || !ssq_dev || !inv_dev || !sqrt_dev)
    return set_error(GBSGMC_ERR_ARG, "mass_adapt: null pointer");
  mass_adapt_kernel<<<grid_x(1, P), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      P, iteration, burn_in, x_dev, mean_dev, ssq_dev, inv_dev, sqrt_dev, mass_dev);
  return check_launch("mass_adapt");
}
