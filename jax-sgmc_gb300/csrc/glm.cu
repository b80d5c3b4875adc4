// Generalised-linear minibatch potential, its adjoint, and the fused SGLD step.
//
// Grid (slices, chains).  CTA (s, c) owns rows [s*R, (s+1)*R) of chain c's
// minibatch.  One producer warp stages the gathered rows X[idx_i] into a ring
// of shared-memory stages with cp.async.bulk (one 16-byte-aligned copy per
// row, completing on the stage's mbarrier); eight consumer warps each take a
// row at a time: z = x.w by a warp reduction, the family's log-likelihood
// lk(z, y) and dlk/dz, and acc += dlk/dz * x kept in registers.  The warp
// partials are reduced through shared memory.  With several slices per chain,
// each CTA writes its partial gradient and partial sums to the workspace and
// the last CTA of the chain to finish (ticket counter) adds them in slice
// order -- the result does not depend on which CTA finishes last -- and runs
// the epilogue:
//   U = (-N/n sum_i m_i lk_i - log p(w)) / T_pot
//   g = (-N/n sum_i m_i dlk_i/dw + w / s^2) / T_pot
// then either stores (U, g) or applies the SGLD(+RMSprop) update in place.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace gbsgmc {
namespace {

constexpr int kConsumerWarps = 8;
constexpr int kThreads = (kConsumerWarps + 1) * 32;
constexpr int kRowsPerWarpStage = 2;
constexpr int kRowsPerStage = kConsumerWarps * kRowsPerWarpStage;
constexpr int kMaxRowsPerSlice = 1024;
constexpr int kMinSlicesAlloc = 16;
constexpr size_t kRingBudget = 96 * 1024;

enum Mode { kValueGrad = 0, kSgldStep = 1 };

struct GlmArgs {
  int family, d, dq;
  int64_t n_obs, n_rows, ld;
  const float* X;
  const float* y;
  float inv_s2;     // 1/sigma^2 (linear-Gaussian)
  float log_norm;   // log sigma + 0.5 log 2 pi (linear-Gaussian)
  float inv_p2;     // 1/prior_scale^2, 0 for a flat prior
  double prior_const;  // d * (log s + 0.5 log 2 pi), 0 for a flat prior
  float inv_temp;
  int chains, n, slices, rows_per_slice;
  const int32_t* idx;
  int64_t idx_stride;
  const float* mask;
  int mode;
  float* w;
  float* v;
  float alpha, lmbd;
  Sched sched;
  Noise noise;
  double* U;
  float* grad;
  float* lk;
  double* lk_var;
  float* samples;
  double* sample_lik;
  float4* ws_part;
  double* ws_sums;
  unsigned* ws_ticket;
  int* status;
  int bulk;
  int stages;
};

struct SmemLayout {
  size_t bars, abort_flag, idx, y, m, ring, red, sums, total;
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) {
  return (x + a - 1) / a * a;
}

__host__ __device__ inline SmemLayout smem_layout(int rows_per_slice, int dq,
                                                  int stages) {
  SmemLayout L;
  size_t o = 0;
  L.bars = o;
  o += sizeof(uint64_t) * 2 * stages;
  L.abort_flag = o;
  o += 16;
  o = align_up(o, 16);
  L.idx = o;
  o += sizeof(int32_t) * rows_per_slice;
  o = align_up(o, 16);
  L.y = o;
  o += sizeof(float) * rows_per_slice;
  o = align_up(o, 16);
  L.m = o;
  o += sizeof(float) * rows_per_slice;
  o = align_up(o, 128);
  L.ring = o;
  o += static_cast<size_t>(stages) * kRowsPerStage * dq * 16;
  o = align_up(o, 16);
  L.red = o;
  o += static_cast<size_t>(kConsumerWarps) * dq * 16;
  o = align_up(o, 16);
  L.sums = o;
  o += sizeof(double) * 4 * (kConsumerWarps + 1);
  L.total = o;
  return L;
}

__device__ __forceinline__ float softplusf(float z) {
  return fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z)));
}

__device__ __forceinline__ float sigmoidf(float z) {
  if (z >= 0.0f) return 1.0f / (1.0f + expf(-z));
  const float e = expf(z);
  return e / (1.0f + e);
}

template <int QPL>
__global__ void __launch_bounds__(kThreads)
    glm_kernel(const GlmArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const SmemLayout L = smem_layout(a.rows_per_slice, a.dq, a.stages);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars);
  uint64_t* empty = full + a.stages;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L.abort_flag);
  int* is_last = reinterpret_cast<int*>(smem + L.abort_flag + 4);
  int32_t* idx_s = reinterpret_cast<int32_t*>(smem + L.idx);
  float* y_s = reinterpret_cast<float*>(smem + L.y);
  float* m_s = reinterpret_cast<float*>(smem + L.m);
  float4* ring = reinterpret_cast<float4*>(smem + L.ring);
  float4* red = reinterpret_cast<float4*>(smem + L.red);
  double* sums = reinterpret_cast<double*>(smem + L.sums);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = blockIdx.x, c = blockIdx.y;
  const int row0 = s * a.rows_per_slice;
  const int R = max(0, min(a.rows_per_slice, a.n - row0));
  const int dq = a.dq;

  if (tid == 0) {
    for (int i = 0; i < a.stages; ++i) {
      mbar_init(&full[i], a.bulk ? 1u : 32u);
      mbar_init(&empty[i], static_cast<uint32_t>(kConsumerWarps));
    }
    *abort_flag = 0;
    *is_last = 0;
    mbar_fence_init();
  }
  // Indices, targets and mask weights of this slice.
  for (int r = tid; r < R; r += kThreads) {
    const int i = row0 + r;
    int32_t o = __ldg(a.idx + c * a.idx_stride + i);
    if (o < 0 || o >= a.n_rows) {
      raise_status(a.status, GBSGMC_ERR_INDEX);
      o = -1;
    }
    idx_s[r] = o;
    y_s[r] = (o >= 0 && a.y != nullptr) ? __ldg(a.y + o) : 0.0f;
    m_s[r] = a.mask != nullptr ? __ldg(a.mask + static_cast<int64_t>(c) * a.n + i)
                               : 1.0f;
  }
  __syncthreads();

  const int n_stages = (R + kRowsPerStage - 1) / kRowsPerStage;
  const uint32_t row_bytes = static_cast<uint32_t>(dq) * 16u;

  double my_mlk = 0.0, my_lk = 0.0, my_lk2 = 0.0;

  if (warp == kConsumerWarps) {
    // ------------------------------ producer ------------------------------
    int issued = 0;
    for (int st = 0; st < n_stages; ++st) {
      const int slot = st % a.stages;
      const uint32_t ph = static_cast<uint32_t>(st / a.stages) & 1u;
      if (!mbar_wait_bounded(&empty[slot], ph ^ 1u, abort_flag)) {
        if (lane == 0) {
          raise_status(a.status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
        }
        break;
      }
      const int r0 = st * kRowsPerStage;
      const int cnt = min(kRowsPerStage, R - r0);
      float4* dst = ring + static_cast<size_t>(slot) * kRowsPerStage * dq;
      if (a.bulk) {
        if (lane == 0) {
          uint32_t bytes = 0;
          for (int r = 0; r < cnt; ++r) bytes += idx_s[r0 + r] >= 0 ? row_bytes : 0u;
          mbar_arrive_expect_tx(&full[slot], bytes);
          for (int r = 0; r < cnt; ++r) {
            const int32_t o = idx_s[r0 + r];
            if (o >= 0)
              bulk_g2s(dst + static_cast<size_t>(r) * dq, a.X + o * a.ld,
                       row_bytes, &full[slot]);
          }
        }
      } else {
        float* dsts = reinterpret_cast<float*>(dst);
        for (int r = 0; r < cnt; ++r) {
          const int32_t o = idx_s[r0 + r];
          for (int j = lane; j < dq * 4; j += 32)
            dsts[r * dq * 4 + j] =
                (o >= 0 && j < a.d) ? __ldg(a.X + o * a.ld + j) : 0.0f;
        }
        mbar_arrive(&full[slot]);
      }
      issued = st + 1;
    }
    if (*abort_flag && a.bulk && lane == 0) {
      // Let the copies already issued land before the CTA exits.
      for (int st = max(0, issued - a.stages); st < issued; ++st)
        mbar_wait_bounded(&full[st % a.stages],
                          static_cast<uint32_t>(st / a.stages) & 1u, nullptr);
    }
  } else {
    // ------------------------------ consumers -----------------------------
    float4 wq[QPL];
    float4 acc[QPL];
    const float* wc = a.w + static_cast<int64_t>(c) * a.d;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int j = 4 * (lane + 32 * k);
      wq[k].x = j + 0 < a.d ? wc[j + 0] : 0.0f;
      wq[k].y = j + 1 < a.d ? wc[j + 1] : 0.0f;
      wq[k].z = j + 2 < a.d ? wc[j + 2] : 0.0f;
      wq[k].w = j + 3 < a.d ? wc[j + 3] : 0.0f;
      acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float* lk_out = a.lk != nullptr ? a.lk + static_cast<int64_t>(c) * a.n + row0
                                    : nullptr;
    for (int st = 0; st < n_stages; ++st) {
      const int slot = st % a.stages;
      const uint32_t ph = static_cast<uint32_t>(st / a.stages) & 1u;
      if (!mbar_wait_bounded(&full[slot], ph, abort_flag)) {
        if (lane == 0) {
          raise_status(a.status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
        }
        break;
      }
      const float4* src = ring + static_cast<size_t>(slot) * kRowsPerStage * dq;
#pragma unroll
      for (int rr = 0; rr < kRowsPerWarpStage; ++rr) {
        const int r = rr * kConsumerWarps + warp;
        const int row = st * kRowsPerStage + r;
        if (row >= R || idx_s[row] < 0) continue;
        const float4* xr = src + static_cast<size_t>(r) * dq;
        float4 xv[QPL];
        float z = 0.0f;
#pragma unroll
        for (int k = 0; k < QPL; ++k) {
          const int q = lane + 32 * k;
          if (q < dq) {
            xv[k] = xr[q];
            z = fmaf(xv[k].x, wq[k].x, z);
            z = fmaf(xv[k].y, wq[k].y, z);
            z = fmaf(xv[k].z, wq[k].z, z);
            z = fmaf(xv[k].w, wq[k].w, z);
          } else {
            xv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
        z = warp_sum(z);
        const float yv = y_s[row];
        float lkv, dz;
        if (a.family == GBSGMC_GLM_LOGISTIC) {
          lkv = yv * z - softplusf(z);
          dz = yv - sigmoidf(z);
        } else if (a.family == GBSGMC_GLM_LINEAR) {
          lkv = z;
          dz = 1.0f;
        } else {
          const float res = yv - z;
          lkv = -0.5f * res * res * a.inv_s2 - a.log_norm;
          dz = res * a.inv_s2;
        }
        const float mw = m_s[row];
        const float coef = mw * dz;
#pragma unroll
        for (int k = 0; k < QPL; ++k) {
          acc[k].x = fmaf(coef, xv[k].x, acc[k].x);
          acc[k].y = fmaf(coef, xv[k].y, acc[k].y);
          acc[k].z = fmaf(coef, xv[k].z, acc[k].z);
          acc[k].w = fmaf(coef, xv[k].w, acc[k].w);
        }
        if (lane == 0) {
          my_mlk += static_cast<double>(mw) * lkv;
          my_lk += lkv;
          my_lk2 += static_cast<double>(lkv) * lkv;
          if (lk_out != nullptr) lk_out[row] = lkv;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[slot]);
    }
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = lane + 32 * k;
      if (q < dq) red[warp * dq + q] = acc[k];
    }
    if (lane == 0) {
      sums[warp * 4 + 0] = my_mlk;
      sums[warp * 4 + 1] = my_lk;
      sums[warp * 4 + 2] = my_lk2;
    }
  }
  __syncthreads();

  // Reduce the warp partials in a fixed order: partial gradient in red[0..dq).
  for (int q = tid; q < dq; q += kThreads) {
    float4 t = red[q];
    for (int w = 1; w < kConsumerWarps; ++w) {
      const float4 u = red[w * dq + q];
      t.x += u.x;
      t.y += u.y;
      t.z += u.z;
      t.w += u.w;
    }
    red[q] = t;
  }
  if (tid == 0) {
    double t0 = 0.0, t1 = 0.0, t2 = 0.0;
    for (int w = 0; w < kConsumerWarps; ++w) {
      t0 += sums[w * 4 + 0];
      t1 += sums[w * 4 + 1];
      t2 += sums[w * 4 + 2];
    }
    sums[kConsumerWarps * 4 + 0] = t0;
    sums[kConsumerWarps * 4 + 1] = t1;
    sums[kConsumerWarps * 4 + 2] = t2;
  }
  __syncthreads();

  if (a.slices > 1) {
    const int64_t pc = static_cast<int64_t>(c) * a.slices + s;
    for (int q = tid; q < dq; q += kThreads) a.ws_part[pc * dq + q] = red[q];
    if (tid == 0) {
      a.ws_sums[pc * 4 + 0] = sums[kConsumerWarps * 4 + 0];
      a.ws_sums[pc * 4 + 1] = sums[kConsumerWarps * 4 + 1];
      a.ws_sums[pc * 4 + 2] = sums[kConsumerWarps * 4 + 2];
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      const unsigned ticket = atomicAdd(a.ws_ticket + c, 1u);
      const int last = ticket == static_cast<unsigned>(a.slices - 1);
      if (last) a.ws_ticket[c] = 0u;  // ready for the next launch
      *is_last = last;
    }
    __syncthreads();
    if (!*is_last) return;
    __threadfence();
    const float4* part = a.ws_part + static_cast<int64_t>(c) * a.slices * dq;
    for (int q = tid; q < dq; q += kThreads) {
      float4 t = __ldcg(part + q);
      for (int k = 1; k < a.slices; ++k) {
        const float4 u = __ldcg(part + static_cast<int64_t>(k) * dq + q);
        t.x += u.x;
        t.y += u.y;
        t.z += u.z;
        t.w += u.w;
      }
      red[q] = t;
    }
    if (tid == 0) {
      const double* ps = a.ws_sums + static_cast<int64_t>(c) * a.slices * 4;
      double t0 = 0.0, t1 = 0.0, t2 = 0.0;
      for (int k = 0; k < a.slices; ++k) {
        t0 += __ldcg(ps + k * 4 + 0);
        t1 += __ldcg(ps + k * 4 + 1);
        t2 += __ldcg(ps + k * 4 + 2);
      }
      sums[kConsumerWarps * 4 + 0] = t0;
      sums[kConsumerWarps * 4 + 1] = t1;
      sums[kConsumerWarps * 4 + 2] = t2;
    }
    __syncthreads();
  }

  // ------------------------------ epilogue ---------------------------------
  const double sum_mlk = sums[kConsumerWarps * 4 + 0];
  const double sum_lk = sums[kConsumerWarps * 4 + 1];
  const double sum_lk2 = sums[kConsumerWarps * 4 + 2];
  float* wc = a.w + static_cast<int64_t>(c) * a.d;
  const float scale = static_cast<float>(static_cast<double>(a.n_obs) / a.n);

  double ww = 0.0;
  if (a.inv_p2 > 0.0f) {
    for (int j = tid; j < a.d; j += kThreads) {
      const double wj = wc[j];
      ww += wj * wj;
    }
  }
  // Reuse the per-warp sums area as block-reduction scratch (9 warps).
  ww = block_sum(ww, sums);
  const double log_prior = -0.5 * ww * a.inv_p2 - a.prior_const;
  // -N * mean(lk) without a mask, -N/n * (lk . mask) with one, as written in
  // potential.py:183-185 (the unmasked form is exact for integer sums).
  const double lik = a.mask == nullptr
                         ? -static_cast<double>(a.n_obs) * (sum_mlk / a.n)
                         : -(static_cast<double>(a.n_obs) / a.n) * sum_mlk;
  const double U = (lik - log_prior) * a.inv_temp;
  const double mean_lk = sum_lk / a.n;
  const double var_lk = fmax(sum_lk2 / a.n - mean_lk * mean_lk, 0.0);
  if (!isfinite(U)) raise_status(a.status, GBSGMC_ERR_NONFINITE);

  const float* gl = reinterpret_cast<const float*>(red);
  if (a.mode == kValueGrad) {
    if (a.grad != nullptr) {
      float* gc = a.grad + static_cast<int64_t>(c) * a.d;
      for (int j = tid; j < a.d; j += kThreads)
        gc[j] = (-scale * gl[j] + wc[j] * a.inv_p2) * a.inv_temp;
    }
    if (tid == 0) {
      a.U[c] = U;
      if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    }
    return;
  }

  // SGLD (+RMSprop) update of chain c, four parameters per thread.
  const int64_t k = a.sched.step();
  const float h = a.sched.step_size(k);
  const float T = a.sched.temperature(k);
  const int slot = a.sched.keep_slot(k);
  const float noise_scale = sqrtf(2.0f * T * h);
  float* vc = a.v != nullptr ? a.v + static_cast<int64_t>(c) * a.d : nullptr;
  float* smp = slot >= 0 ? a.samples + (static_cast<int64_t>(slot) * a.chains + c) * a.d
                         : nullptr;
  bool bad = false;
  for (int q = tid; q < dq; q += kThreads) {
    float xi[4];
    noise4(a.noise, c, 4 * q, a.d, k, GBSGMC_TAG_SGLD, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int j = 4 * q + e;
      if (j >= a.d) break;
      const float x = wc[j];
      const float g = (-scale * gl[j] + x * a.inv_p2) * a.inv_temp;
      bad |= !isfinite(g);
      const float scaled_gradient = -h * g;
      const float scaled_noise = noise_scale * xi[e];
      float x_new;
      if (vc != nullptr) {
        const float vn = a.alpha * vc[j] + (1.0f - a.alpha) * (g * g);
        const float G = 1.0f / (a.lmbd + sqrtf(vn));
        const float sG = sqrtf(G);
        vc[j] = vn;
        x_new = x + ((0.0f + G * scaled_gradient) + sG * scaled_noise);
      } else {
        x_new = x + (scaled_gradient + scaled_noise);
      }
      wc[j] = x_new;
      if (smp != nullptr) smp[j] = x_new;
    }
  }
  if (bad) raise_status(a.status, GBSGMC_ERR_NONFINITE);
  if (tid == 0) {
    if (a.U != nullptr) a.U[c] = U;
    if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    if (slot >= 0 && a.sample_lik != nullptr)
      a.sample_lik[static_cast<int64_t>(slot) * a.chains + c] = -U;
  }
}

// ---------------------------------------------------------------------------
// Host side: argument checks, slice choice, launch.
// ---------------------------------------------------------------------------

int slices_alloc(int n) {
  return std::max(kMinSlicesAlloc, ceil_div(n, kMaxRowsPerSlice));
}

struct WsView {
  float4* part;
  double* sums;
  unsigned* ticket;
};

size_t ws_bytes(int chains, int n, int d) {
  const int dq = (d + 3) / 4;
  const size_t S = static_cast<size_t>(slices_alloc(n));
  size_t b = align_up(static_cast<size_t>(chains) * S * dq * 16, 256);
  b += align_up(static_cast<size_t>(chains) * S * 4 * sizeof(double), 256);
  b += align_up(static_cast<size_t>(chains) * sizeof(unsigned), 256);
  return b;
}

WsView ws_view(void* ws, int chains, int n, int d) {
  const int dq = (d + 3) / 4;
  const size_t S = static_cast<size_t>(slices_alloc(n));
  char* p = static_cast<char*>(ws);
  WsView v;
  v.part = reinterpret_cast<float4*>(p);
  p += align_up(static_cast<size_t>(chains) * S * dq * 16, 256);
  v.sums = reinterpret_cast<double*>(p);
  p += align_up(static_cast<size_t>(chains) * S * 4 * sizeof(double), 256);
  v.ticket = reinterpret_cast<unsigned*>(p);
  return v;
}

int sm_count() {
  static int cached = 0;
  if (cached == 0) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) ==
            cudaSuccess &&
        n > 0)
      cached = n;
    else
      cached = 152;
  }
  return cached;
}

int choose_stages(int dq) {
  const size_t stage_bytes = static_cast<size_t>(kRowsPerStage) * dq * 16;
  int st = static_cast<int>(kRingBudget / stage_bytes);
  return std::max(2, std::min(8, st));
}

// Slices per chain: enough CTAs for about three waves of two CTAs per SM,
// at most kMaxRowsPerSlice rows and at least 32 rows per slice.
int choose_slices(int chains, int n) {
  const int need = ceil_div(n, kMaxRowsPerSlice);
  const int target = 3 * 2 * sm_count();
  int s = std::max(1, ceil_div(target, std::max(chains, 1)));
  s = std::min(s, std::max(1, n / 32));
  s = std::max(s, need);
  s = std::min(s, slices_alloc(n));
  return s;
}

constexpr int kMaxDynSmem = 227 * 1024;

template <int QPL>
int prepare_q() {
  static int done = 0;
  if (done) return GBSGMC_OK;
  const cudaError_t e = cudaFuncSetAttribute(
      glm_kernel<QPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
  if (e != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "glm: cudaFuncSetAttribute: %s",
                     cudaGetErrorString(e));
  done = 1;
  return GBSGMC_OK;
}

template <int QPL>
int launch_q(const GlmArgs& a, size_t smem, cudaStream_t st) {
  const int rc = prepare_q<QPL>();
  if (rc != GBSGMC_OK) return rc;
  dim3 grid(a.slices, a.chains);
  glm_kernel<QPL><<<grid, kThreads, smem, st>>>(a);
  return check_launch("glm_kernel");
}

int launch_glm(GlmArgs& a, cudaStream_t st) {
  if (a.chains == 0 || a.n == 0) return GBSGMC_OK;
  a.stages = choose_stages(a.dq);
  const SmemLayout L = smem_layout(a.rows_per_slice, a.dq, a.stages);
  if (L.total > 227 * 1024)
    return set_error(GBSGMC_ERR_SHAPE, "glm: shared memory %zu too large",
                     L.total);
  if (a.dq <= 32) return launch_q<1>(a, L.total, st);
  if (a.dq <= 64) return launch_q<2>(a, L.total, st);
  if (a.dq <= 128) return launch_q<4>(a, L.total, st);
  return launch_q<8>(a, L.total, st);
}

int fill_common(GlmArgs& a, const gbsgmc_glm* m, int chains, int n,
                const int32_t* idx, int64_t idx_stride, const float* mask,
                void* ws, size_t ws_size, int* status, int slices_override = 0) {
  if (m == nullptr || m->X == nullptr || idx == nullptr ||
      (m->y == nullptr && m->family != GBSGMC_GLM_LINEAR))
    return set_error(GBSGMC_ERR_ARG, "glm: null model, data or index pointer");
  if (m->family != GBSGMC_GLM_LINEAR_GAUSSIAN && m->family != GBSGMC_GLM_LOGISTIC &&
      m->family != GBSGMC_GLM_LINEAR)
    return set_error(GBSGMC_ERR_ARG, "glm: unknown family %d", m->family);
  if (m->d < 1 || m->d > 1024)
    return set_error(GBSGMC_ERR_SHAPE, "glm: d must be in [1, 1024], got %d", m->d);
  if (m->ld < m->d || m->n_obs < 1 || m->n_rows < 0 ||
      m->n_rows >= (1ll << 31) || (m->n_rows == 0 && m->n_obs >= (1ll << 31)))
    return set_error(GBSGMC_ERR_ARG, "glm: bad ld, n_obs or n_rows");
  if (chains < 0 || n < 0 || n > kMaxRowsPerSlice * 64)
    return set_error(GBSGMC_ERR_SHAPE, "glm: chains/n out of range");
  if (idx_stride < n) return set_error(GBSGMC_ERR_ARG, "glm: idx_stride < n");
  if (m->family == GBSGMC_GLM_LINEAR_GAUSSIAN && !(m->sigma > 0.0f))
    return set_error(GBSGMC_ERR_ARG, "glm: sigma must be positive");
  if (!(m->temperature > 0.0f))
    return set_error(GBSGMC_ERR_ARG, "glm: temperature must be positive");
  int S = choose_slices(chains, n);
  if (slices_override > 0)
    S = std::min(std::max(slices_override, ceil_div(n, kMaxRowsPerSlice)),
                 std::min(slices_alloc(n), std::max(1, n)));
  if (S > 1) {
    if (ws == nullptr || ws_size < ws_bytes(chains, n, m->d))
      return set_error(GBSGMC_ERR_ARG, "glm: workspace missing or too small "
                                       "(need %zu bytes)",
                       ws_bytes(chains, n, m->d));
  }
  a.family = m->family;
  a.d = m->d;
  a.dq = (m->d + 3) / 4;
  a.n_obs = m->n_obs;
  a.n_rows = m->n_rows > 0 ? m->n_rows : m->n_obs;
  a.ld = m->ld;
  a.X = m->X;
  a.y = m->y;
  const double sg = m->sigma > 0.0f ? m->sigma : 1.0;
  a.inv_s2 = static_cast<float>(1.0 / (sg * sg));
  a.log_norm = static_cast<float>(std::log(sg) + 0.5 * std::log(2.0 * M_PI));
  if (m->prior_scale > 0.0f) {
    const double ps = m->prior_scale;
    a.inv_p2 = static_cast<float>(1.0 / (ps * ps));
    a.prior_const = m->d * (std::log(ps) + 0.5 * std::log(2.0 * M_PI));
  } else {
    a.inv_p2 = 0.0f;
    a.prior_const = 0.0;
  }
  a.inv_temp = 1.0f / m->temperature;
  a.chains = chains;
  a.n = n;
  a.slices = S;
  a.rows_per_slice = ceil_div(n, S);
  a.idx = idx;
  a.idx_stride = idx_stride;
  a.mask = mask;
  if (S > 1) {
    const WsView v = ws_view(ws, chains, n, m->d);
    a.ws_part = v.part;
    a.ws_sums = v.sums;
    a.ws_ticket = v.ticket;
  } else {
    a.ws_part = nullptr;
    a.ws_sums = nullptr;
    a.ws_ticket = nullptr;
  }
  a.status = status;
  const bool aligned = (reinterpret_cast<uintptr_t>(m->X) % 16 == 0) &&
                       (m->ld % 4 == 0) && (m->d % 4 == 0);
  a.bulk = aligned ? 1 : 0;
  a.lk = nullptr;
  a.lk_var = nullptr;
  a.grad = nullptr;
  a.U = nullptr;
  a.samples = nullptr;
  a.sample_lik = nullptr;
  a.v = nullptr;
  a.alpha = 0.9f;
  a.lmbd = 1e-5f;
  a.sched = Sched{nullptr, nullptr, nullptr, nullptr, 0, 0.0f, 1.0f};
  a.noise = Noise{nullptr, 0, 0, 0};
  return GBSGMC_OK;
}

}  // namespace

// Shared with the plan implementation.
size_t glm_ws_bytes(int chains, int n, int d) { return ws_bytes(chains, n, d); }

int glm_prepare() {
  int rc = prepare_q<1>();
  if (rc == GBSGMC_OK) rc = prepare_q<2>();
  if (rc == GBSGMC_OK) rc = prepare_q<4>();
  if (rc == GBSGMC_OK) rc = prepare_q<8>();
  return rc;
}

int glm_default_slices(int chains, int n) { return choose_slices(chains, n); }

int glm_sgld_step(const gbsgmc_glm* model, int chains, int n,
                  const int32_t* idx_dev, int64_t idx_stride, float* w_dev,
                  float* v_dev, float alpha, float lmbd,
                  const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                  double* U_dev, double* lk_var_dev, float* samples_dev,
                  double* sample_lik_dev, void* ws, size_t ws_size,
                  int* status_dev, cudaStream_t stream, int slices) {
  GlmArgs a;
  int rc = fill_common(a, model, chains, n, idx_dev, idx_stride, nullptr, ws,
                       ws_size, status_dev, slices);
  if (rc != GBSGMC_OK) return rc;
  if (w_dev == nullptr || sched == nullptr || noise == nullptr)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step: null w, sched or noise");
  if (sched->keep_slot_dev != nullptr && samples_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "sgld_glm_step: keep table given without sample buffer");
  if (noise->noise_dev != nullptr && noise->noise_stride < model->d)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step: noise_stride < d");
  a.mode = kSgldStep;
  a.w = w_dev;
  a.v = v_dev;
  a.alpha = alpha;
  a.lmbd = lmbd;
  a.sched = to_sched(sched);
  a.noise = to_noise(noise);
  a.U = U_dev;
  a.lk_var = lk_var_dev;
  a.samples = samples_dev;
  a.sample_lik = sample_lik_dev;
  return launch_glm(a, stream);
}

}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" size_t gbsgmc_glm_workspace_bytes(int chains, int n, int d) {
  if (chains <= 0 || n <= 0 || d <= 0) return 0;
  return ws_bytes(chains, n, d);
}

extern "C" int gbsgmc_glm_value_and_grad(
    const gbsgmc_glm* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, const float* mask_dev, const float* w_dev,
    double* U_dev, float* grad_dev, float* lk_dev, double* lk_var_dev,
    void* workspace_dev, size_t workspace_bytes, int* status_dev,
    gbsgmc_stream_t stream) {
  GlmArgs a;
  int rc = fill_common(a, model, chains, n, idx_dev, idx_stride, mask_dev,
                       workspace_dev, workspace_bytes, status_dev);
  if (rc != GBSGMC_OK) return rc;
  if (w_dev == nullptr || U_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "glm_value_and_grad: null w or U");
  a.mode = kValueGrad;
  a.w = const_cast<float*>(w_dev);
  a.U = U_dev;
  a.grad = grad_dev;
  a.lk = lk_dev;
  a.lk_var = lk_var_dev;
  return launch_glm(a, static_cast<cudaStream_t>(stream));
}

extern "C" int gbsgmc_sgld_glm_step(
    const gbsgmc_glm* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, float* w_dev, float* v_dev, float alpha, float lmbd,
    const gbsgmc_sched* sched, const gbsgmc_noise* noise, double* U_dev,
    double* lk_var_dev, float* samples_dev, double* sample_lik_dev,
    void* workspace_dev, size_t workspace_bytes, int* status_dev,
    gbsgmc_stream_t stream) {
  return glm_sgld_step(model, chains, n, idx_dev, idx_stride, w_dev, v_dev,
                       alpha, lmbd, sched, noise, U_dev, lk_var_dev,
                       samples_dev, sample_lik_dev, workspace_dev,
                       workspace_bytes, status_dev,
                       static_cast<cudaStream_t>(stream), 0);
}
