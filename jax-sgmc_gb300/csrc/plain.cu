// The plain one-chain form of an SGLD(+RMSprop) step on a GLM, kept as the
// GPU comparison baseline: the operations an op-by-op compiler emits for the
// reference's update_fn, each its own launch over its own buffer --
// gather of the minibatch rows, forward GEMV, link, backward GEMV, likelihood
// reduction, prior and gradient scaling, noise, RMSprop + update.
#include <cmath>

#include "common.cuh"

namespace gbsgmc {
namespace {

struct PlainBuf {
  float* xb;    // [n, d] gathered rows
  float* yb;    // [n]
  float* z;     // [n]
  float* lk;    // [n]
  float* dz;    // [n]
  float* gl;    // [d]
  float* grad;  // [d]
  float* xi;    // [d]
  double* sums; // [2]
};

size_t al(size_t x) { return (x + 255) / 256 * 256; }

PlainBuf carve(void* buf, int n, int d) {
  char* p = static_cast<char*>(buf);
  PlainBuf b;
  b.xb = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * n * d);
  b.yb = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * n);
  b.z = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * n);
  b.lk = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * n);
  b.dz = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * n);
  b.gl = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * d);
  b.grad = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * d);
  b.xi = reinterpret_cast<float*>(p);
  p += al(sizeof(float) * d);
  b.sums = reinterpret_cast<double*>(p);
  return b;
}

__global__ void gather_kernel(const float* X, int64_t ld, const float* y,
                              int y_inline, const int32_t* idx, int n, int d,
                              int64_t n_obs, float* xb, float* yb, int* status) {
  const int i = blockIdx.x;
  int32_t o = idx[i];
  if (o < 0 || o >= n_obs) {
    if (threadIdx.x == 0) raise_status(status, GBSGMC_ERR_INDEX);
    o = 0;
  }
  for (int j = threadIdx.x; j < d; j += blockDim.x)
    xb[static_cast<int64_t>(i) * d + j] = X[o * ld + j];
  if (threadIdx.x == 0)
    yb[i] = y_inline ? X[o * ld + d] : (y != nullptr ? y[o] : 0.0f);
}

__global__ void gemv_kernel(const float* xb, const float* w, int n, int d,
                            float* z) {
  const int i = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  float acc = 0.0f;
  for (int j = lane; j < d; j += 32) acc += xb[static_cast<int64_t>(i) * d + j] * w[j];
  acc = warp_sum(acc);
  if (lane == 0) z[i] = acc;
}

__global__ void link_kernel(int family, const float* z, const float* yb,
                            int n, float inv_s2, float log_norm, float* lk,
                            float* dz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float zi = z[i], yi = yb[i];
  if (family == GBSGMC_GLM_LOGISTIC) {
    const float sp = fmaxf(zi, 0.0f) + log1pf(expf(-fabsf(zi)));
    lk[i] = yi * zi - sp;
    dz[i] = yi - 1.0f / (1.0f + expf(-zi));
  } else if (family == GBSGMC_GLM_LINEAR) {
    lk[i] = zi;
    dz[i] = 1.0f;
  } else {
    const float r = yi - zi;
    lk[i] = -0.5f * r * r * inv_s2 - log_norm;
    dz[i] = r * inv_s2;
  }
}

__global__ void gemv_t_kernel(const float* xb, const float* dz, int n, int d,
                              float* gl) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  float acc = 0.0f;
  for (int i = 0; i < n; ++i) acc += dz[i] * xb[static_cast<int64_t>(i) * d + j];
  gl[j] = acc;
}

__global__ void reduce_kernel(const float* lk, int n, const float* w, int d,
                              double* sums) {
  __shared__ double scratch[32];
  double s = 0.0, ww = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += lk[i];
  for (int j = threadIdx.x; j < d; j += blockDim.x) ww += static_cast<double>(w[j]) * w[j];
  s = block_sum(s, scratch);
  ww = block_sum(ww, scratch);
  if (threadIdx.x == 0) {
    sums[0] = s;
    sums[1] = ww;
  }
}

__global__ void grad_kernel(const float* gl, const float* w, int d, float scale,
                            float inv_p2, float inv_temp, const double* sums,
                            double n_obs, double n_count, double prior_const,
                            double* U, float* grad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < d) grad[j] = (-scale * gl[j] + w[j] * inv_p2) * inv_temp;
  if (j == 0 && U != nullptr) {
    const double log_prior = -0.5 * sums[1] * inv_p2 - prior_const;
    U[0] = (-n_obs * (sums[0] / n_count) - log_prior) * inv_temp;
  }
}

__global__ void noise_kernel(int d, int64_t step, Noise nz, float* xi) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (4 * q >= d) return;
  float z[4];
  noise4(nz, 0, 4 * q, d, step, GBSGMC_TAG_SGLD, z);
  for (int e = 0; e < 4; ++e)
    if (4 * q + e < d) xi[4 * q + e] = z[e];
}

__global__ void update_kernel(int d, float* w, float* v, const float* grad,
                              const float* xi, float alpha, float lmbd,
                              Sched sched) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float T = sched.temperature(k, 0);
  const float g = grad[j];
  const float sgrad = -h * g;
  const float snoise = sqrtf(2.0f * T * h) * xi[j];
  if (v != nullptr) {
    const float vn = alpha * v[j] + (1.0f - alpha) * (g * g);
    const float G = 1.0f / (lmbd + sqrtf(vn));
    v[j] = vn;
    w[j] = w[j] + ((0.0f + G * sgrad) + sqrtf(G) * snoise);
  } else {
    w[j] = w[j] + (sgrad + snoise);
  }
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" size_t gbsgmc_plain_buffer_bytes(int n, int d) {
  if (n <= 0 || d <= 0) return 0;
  return al(sizeof(float) * n * d) + 4 * al(sizeof(float) * n) +
         3 * al(sizeof(float) * d) + al(2 * sizeof(double));
}

extern "C" int gbsgmc_plain_sgld_glm_step(
    const gbsgmc_glm* m, int n, const int32_t* idx_dev, float* w_dev,
    float* v_dev, float alpha, float lmbd, const gbsgmc_sched* sched,
    const gbsgmc_noise* noise, double* U_dev, void* buf_dev, int* status_dev,
    gbsgmc_stream_t stream) {
  if (!m || !idx_dev || !w_dev || !sched || !noise || !buf_dev)
    return set_error(GBSGMC_ERR_ARG, "plain_sgld_glm_step: null argument");
  if (m->d < 1 || n < 1 || m->ld < m->d)
    return set_error(GBSGMC_ERR_ARG, "plain_sgld_glm_step: bad shape");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int d = m->d;
  PlainBuf b = carve(buf_dev, n, d);
  const double sg = m->sigma > 0.0f ? m->sigma : 1.0;
  const float inv_s2 = static_cast<float>(1.0 / (sg * sg));
  const float log_norm = static_cast<float>(std::log(sg) + 0.5 * std::log(2.0 * M_PI));
  float inv_p2 = 0.0f;
  double prior_const = 0.0;
  if (m->prior_scale > 0.0f) {
    inv_p2 = static_cast<float>(1.0 / (static_cast<double>(m->prior_scale) * m->prior_scale));
    prior_const = d * (std::log(static_cast<double>(m->prior_scale)) + 0.5 * std::log(2.0 * M_PI));
  }
  const double n_over = static_cast<double>(m->n_obs) / n;
  const Sched sc = to_sched(sched);
  gather_kernel<<<n, 128, 0, s>>>(m->X, m->ld, m->y, m->y_inline, idx_dev, n, d,
                                  m->n_rows > 0 ? m->n_rows : m->n_obs, b.xb,
                                  b.yb, status_dev);
  gemv_kernel<<<(n + 7) / 8, 256, 0, s>>>(b.xb, w_dev, n, d, b.z);
  link_kernel<<<(n + 255) / 256, 256, 0, s>>>(m->family, b.z, b.yb, n, inv_s2,
                                              log_norm, b.lk, b.dz);
  gemv_t_kernel<<<(d + 255) / 256, 256, 0, s>>>(b.xb, b.dz, n, d, b.gl);
  reduce_kernel<<<1, 256, 0, s>>>(b.lk, n, w_dev, d, b.sums);
  grad_kernel<<<(d + 255) / 256, 256, 0, s>>>(
      b.gl, w_dev, d, static_cast<float>(n_over), inv_p2, 1.0f / m->temperature,
      b.sums, static_cast<double>(m->n_obs), static_cast<double>(n),
      prior_const, U_dev, b.grad);
  // The noise launch needs the step on the host: this form takes it in
  // `offset` (no device counter).
  const int64_t host_step = sc.base == nullptr ? sc.offset : -1;
  if (host_step < 0)
    return set_error(GBSGMC_ERR_ARG,
                     "plain_sgld_glm_step: the schedule must give the step "
                     "in `offset` (base_dev NULL)");
  noise_kernel<<<(d / 4 + 1 + 127) / 128, 128, 0, s>>>(d, host_step,
                                                       to_noise(noise), b.xi);
  update_kernel<<<(d + 255) / 256, 256, 0, s>>>(d, w_dev, v_dev, b.grad, b.xi,
                                                alpha, lmbd, sc);
  return check_launch("plain_sgld_glm_step");
}
