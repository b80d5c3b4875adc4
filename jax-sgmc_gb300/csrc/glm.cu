// Generalised-linear minibatch potential, its adjoint, and the fused SGLD step.
//
// Grid (slices, chains).  CTA (s, c) owns rows [s*R, (s+1)*R) of chain c's
// minibatch; its 8 warps take tiles of RW rows in turn.  A warp gathers the
// RW rows of its tile straight from HBM with 128-bit loads that do not
// allocate in L1 (each row is read once), every lane holding RW x QPL float4
// of x in registers, so RW rows' worth of loads are in flight per warp:
//   * each lane forms partial dot products x.w over its columns for the RW
//     rows; a transposed butterfly (log2 RW halving exchanges, then plain
//     xor steps) leaves lane group g = lane / (32/RW) with z of row g --
//     6 shuffles for 4 rows instead of 20;
//   * each lane group evaluates the family's lk(z, y) and dlk/dz for its row,
//     so the link function runs once per row, not 32 times;
//   * the RW coefficients are broadcast back and acc += coef * x accumulates
//     the gradient from the rows still held in registers.
// The target comes either from its own vector (the layout the Python
// package uploads: 4 bytes per observation, small enough to stay in L2 while
// the rows stream past) or from column d of the feature row (y_inline).
// (Staging rows through shared memory with one cp.async.bulk per 1 KB row
// was measured slower: per-request cost held it near 13 GB/s per SM.)
// The warp partials are reduced through shared memory in a fixed order.  With
// several slices per chain, each CTA writes its partial gradient and partial
// sums to the workspace and the last CTA of the chain to finish (ticket
// counter) adds them in slice order -- the result does not depend on which
// CTA finishes last -- and runs the epilogue:
//   U = (-N/n sum_i m_i lk_i - log p(w)) / T_pot
//   g = (-N/n sum_i m_i dlk_i/dw + w / s^2) / T_pot
// then either stores (U, g) or applies the SGLD(+RMSprop) update in place.
// With one CTA per chain, one launch can run several SGLD steps back to back
// (glm_kernel's step loop).  glm_dyn_kernel is a dynamically scheduled form
// of the same step (warps claim row items of any chain).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kMaxWarps = 16;   // warps per CTA: 8 or 16 (a kernel parameter)
constexpr int kMaxRowsPerSlice = 1024;
constexpr int kMinSlicesAlloc = 16;

enum Mode { kValueGrad = 0, kSgldStep = 1 };

struct GlmArgs {
  int family, d, dq;
  int y_inline;
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
  int steps;                // SGLD steps per launch (> 1: one CTA per chain)
  int64_t idx_step_stride;  // elements between the index sets of two steps
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
  void* ws_base;
  size_t ws_size;
  int slices_fixed;   // > 0: slices per chain chosen by the caller
  int rw_fixed;       // > 0: rows per warp chosen by the caller
  int warps_fixed;    // > 0: warps per CTA chosen by the caller
  int pf_fixed;       // 1: prefetching variant, -1: not, 0: library choice
  int dyn_fixed;      // 1: dynamically scheduled kernel, -1: not, 0: library choice
  int* status;
  int vec4;   // rows are 16-byte aligned: 128-bit loads
  // Replica exchange: chain c's index row and noise stream belong to chain
  // ident[c] (the states that moved into c with an exchange); NULL: c itself.
  const int32_t* ident;
};

// The chain whose index row and noise stream chain (slot) c uses.
__device__ __forceinline__ int ident_of(const GlmArgs& a, int c) {
  return a.ident != nullptr ? __ldg(a.ident + c) : c;
}

struct SmemLayout {
  size_t flags, idx, idx2, m, red, sums, wbuf, total;
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) {
  return (x + a - 1) / a * a;
}

__host__ __device__ inline SmemLayout smem_layout(int rows_per_slice, int dq,
                                                  int warps) {
  SmemLayout L;
  size_t o = 0;
  L.flags = o;
  o += 16;
  L.idx = o;
  o += sizeof(int32_t) * rows_per_slice;
  o = align_up(o, 16);
  L.idx2 = o;  // the next step's indices (multi-step launches)
  o += sizeof(int32_t) * rows_per_slice;
  o = align_up(o, 16);
  L.m = o;
  o += sizeof(float) * rows_per_slice;
  o = align_up(o, 16);
  L.red = o;
  o += static_cast<size_t>(warps) * dq * 16;
  o = align_up(o, 16);
  L.sums = o;
  o += sizeof(double) * 4 * (warps + 1);
  o = align_up(o, 16);
  L.wbuf = o;  // w between the steps of a multi-step launch
  o += static_cast<size_t>(dq) * 16;
  L.total = o;
  return L;
}

// Bernoulli-logit log-likelihood y z - softplus(z) and its derivative
// y - sigmoid(z), from one exponential: e = exp(-|z|),
// softplus(z) = max(z, 0) + log1p(e), sigmoid(z) = 1/(1+e) or e/(1+e).
__device__ __forceinline__ void logistic_link(float z, float y, float& lk,
                                              float& dz) {
  const float e = expf(-fabsf(z));
  const float r = 1.0f / (1.0f + e);
  lk = y * z - (fmaxf(z, 0.0f) + log1pf(e));
  dz = y - (z >= 0.0f ? r : e * r);
}

// 128-bit read-only load that does not allocate in L1 (rows are read once).
__device__ __forceinline__ float4 ld_row4(const float* p) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}

__device__ __forceinline__ float ld_row1(const float* p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// 4-byte asynchronous copy global -> shared (completes in the background;
// cp_async_wait_all waits for the calling thread's copies).
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gmem_src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int RW>
struct Log2;
template <>
struct Log2<1> { static constexpr int v = 0; };
template <>
struct Log2<2> { static constexpr int v = 1; };
template <>
struct Log2<4> { static constexpr int v = 2; };
template <>
struct Log2<8> { static constexpr int v = 3; };

// Sum of p[r] over the 32 lanes for RW rows at once.  Returns, in every lane
// of group g = lane >> (5 - log2 RW), the full sum of row g.
template <int RW>
__device__ __forceinline__ float transposed_warp_sum(float (&p)[RW], int lane) {
  constexpr int LOG = Log2<RW>::v;
#pragma unroll
  for (int t = 0; t < LOG; ++t) {
    const int o = 16 >> t;
    const int half = RW >> (t + 1);
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float send = upper ? p[i] : p[i + half];
      const float keep = upper ? p[i + half] : p[i];
      p[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  float z = p[0];
#pragma unroll
  for (int o = 16 >> LOG; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
  return z;
}

// Issues every load of the tile of rows [r0, r0 + RW): x of the RW rows and
// the target of this lane's row r0 + g.  Rows past R or with an invalid
// index read as zero.
template <int QPL, int RW>
__device__ __forceinline__ void load_tile(const GlmArgs& a, const int32_t* idx_s,
                                          int R, int r0, int lane, int g,
                                          float4 (&xv)[RW][QPL], float& yv,
                                          int& og) {
#pragma unroll
  for (int r = 0; r < RW; ++r) {
    const int o = r0 + r < R ? idx_s[r0 + r] : -1;
    const float* row = a.X + static_cast<int64_t>(o) * a.ld;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = lane + 32 * k;
      if (o >= 0 && q < a.dq) {
        if (a.vec4) {
          xv[r][k] = ld_row4(row + 4 * q);
        } else {
          const int j = 4 * q;
          xv[r][k].x = ld_row1(row + j);
          xv[r][k].y = j + 1 < a.d ? ld_row1(row + j + 1) : 0.0f;
          xv[r][k].z = j + 2 < a.d ? ld_row1(row + j + 2) : 0.0f;
          xv[r][k].w = j + 3 < a.d ? ld_row1(row + j + 3) : 0.0f;
        }
      } else {
        xv[r][k] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  }
  og = r0 + g < R ? idx_s[r0 + g] : -1;
  yv = 0.0f;
  if (og >= 0) {
    if (a.y_inline) {
      yv = ld_row1(a.X + static_cast<int64_t>(og) * a.ld + a.d);
    } else if (a.y != nullptr) {
      yv = ld_row1(a.y + og);
    }
  }
}

// Per-lane accumulators of one CTA row stream.  The likelihood sums stay in
// fp32 per lane (a lane sees a few dozen rows); they are widened to fp64 for
// the warp and block reductions.  GB300's fp64 pipe runs at a small fraction
// of the fp32 rate, so per-row fp64 arithmetic would throttle the kernel.
//
// The sum of the (masked) likelihoods that makes U is compensated: each
// addition's rounding error is carried in mlk_c (Neumaier's variant of
// Kahan summation, A. Neumaier 1974), so a lane's sum is good to about one
// rounding of its total whatever its row count.  Once the sum overflows the
// correction is dropped, so an infinite likelihood sum stays infinite (the
// MH tests reject such a proposal) instead of turning into inf - inf.
//
// The variance needs E[lk^2] - E[lk]^2, which cancels badly when |lk| is
// large, so each lane sums around its first value K: s1 = sum(lk - K),
// s2 = sum((lk - K)^2); the widening to fp64 restores sum(lk) and sum(lk^2).
template <int QPL>
struct Accum {
  float4 acc[QPL];
  float mlk, mlk_c, K, s1, s2;
  int cnt;
};

__device__ __forceinline__ void neumaier_add(float& sum, float& comp, float x) {
  const float t = sum + x;
  const float e = fabsf(sum) >= fabsf(x) ? (sum - t) + x : (x - t) + sum;
  comp += isfinite(t) ? e : 0.0f;
  sum = t;
}

// Likelihood, adjoint and accumulation for a loaded tile (see load_tile).
template <int QPL, int RW>
__device__ __forceinline__ void consume_tile(const GlmArgs& a, const float* m_s,
                                             float* lk_out, int r0, int lane,
                                             int g, bool leader,
                                             const float4 (&wq)[QPL],
                                             const float4 (&xv)[RW][QPL],
                                             float yv, int og, Accum<QPL>& A) {
  constexpr int GROUP = 32 / RW;
  float p[RW];
#pragma unroll
  for (int r = 0; r < RW; ++r) {
    float z = 0.0f;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      z = fmaf(xv[r][k].x, wq[k].x, z);
      z = fmaf(xv[r][k].y, wq[k].y, z);
      z = fmaf(xv[r][k].z, wq[k].z, z);
      z = fmaf(xv[r][k].w, wq[k].w, z);
    }
    p[r] = z;
  }
  const float z = transposed_warp_sum<RW>(p, lane);
  const bool ok = og >= 0;
  const int row = r0 + g;
  const float mw = (ok && a.mask != nullptr) ? m_s[row] : 1.0f;
  float lkv, dz;
  if (a.family == GBSGMC_GLM_LOGISTIC) {
    logistic_link(z, yv, lkv, dz);
  } else if (a.family == GBSGMC_GLM_LINEAR) {
    lkv = z;
    dz = 1.0f;
  } else {
    const float res = yv - z;
    lkv = -0.5f * res * res * a.inv_s2 - a.log_norm;
    dz = res * a.inv_s2;
  }
  const float coef = ok ? mw * dz : 0.0f;
  if (ok && leader) {
    neumaier_add(A.mlk, A.mlk_c, mw * lkv);
    if (A.cnt == 0) A.K = lkv;
    const float dk = lkv - A.K;
    A.s1 += dk;
    A.s2 = fmaf(dk, dk, A.s2);
    A.cnt += 1;
    if (lk_out != nullptr) lk_out[row] = lkv;
  }
#pragma unroll
  for (int r = 0; r < RW; ++r) {
    const float cr = __shfl_sync(0xffffffffu, coef, r * GROUP);
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      A.acc[k].x = fmaf(cr, xv[r][k].x, A.acc[k].x);
      A.acc[k].y = fmaf(cr, xv[r][k].y, A.acc[k].y);
      A.acc[k].z = fmaf(cr, xv[r][k].z, A.acc[k].z);
      A.acc[k].w = fmaf(cr, xv[r][k].w, A.acc[k].w);
    }
  }
}

// Step j of a launch (see glm_kernel): indices at idx + j * idx_step_stride,
// schedule step counter + offset + j.
template <int QPL, int RW, bool PF, int WARPS>
__device__ __forceinline__ void glm_step(const GlmArgs& a, int j, unsigned char* smem) {
  constexpr int LOG = Log2<RW>::v;
  constexpr int GROUP = 32 >> LOG;  // lanes per row in the link phase
  const int dq = a.dq;
  const SmemLayout L = smem_layout(a.rows_per_slice, dq, WARPS);
  int* is_last = reinterpret_cast<int*>(smem + L.flags);
  // Multi-step launches alternate two index buffers: step j reads buffer
  // j & 1 while the copies of step j + 1 fill the other.
  const bool multi = a.steps > 1;
  int32_t* idx_s = reinterpret_cast<int32_t*>(smem + ((multi && (j & 1)) ? L.idx2 : L.idx));
  int32_t* idx_next = reinterpret_cast<int32_t*>(smem + ((j & 1) ? L.idx : L.idx2));
  float* m_s = reinterpret_cast<float*>(smem + L.m);
  float4* red = reinterpret_cast<float4*>(smem + L.red);
  double* sums = reinterpret_cast<double*>(smem + L.sums);
  float4* w_s = reinterpret_cast<float4*>(smem + L.wbuf);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = blockIdx.x, c = blockIdx.y;
  const int row0 = s * a.rows_per_slice;
  const int R = max(0, min(a.rows_per_slice, a.n - row0));

  if (tid == 0) *is_last = 0;
  // Observation indices (and mask weights) of this slice.  In a multi-step
  // launch the indices of step j > 0 were copied asynchronously during step
  // j - 1 (each thread the same entries r), so they are only checked here.
  const int32_t* idx_j = a.idx + j * a.idx_step_stride;
  if (multi && j > 0) {
    cp_async_wait_all();
    for (int r = tid; r < R; r += (WARPS * 32)) {
      const int32_t o = idx_s[r];
      if (o < 0 || o >= a.n_rows) {
        raise_status(a.status, GBSGMC_ERR_INDEX);
        idx_s[r] = -1;
      }
    }
  } else {
    for (int r = tid; r < R; r += (WARPS * 32)) {
      int32_t o = __ldg(idx_j + ident_of(a, c) * a.idx_stride + row0 + r);
      if (o < 0 || o >= a.n_rows) {
        raise_status(a.status, GBSGMC_ERR_INDEX);
        o = -1;
      }
      idx_s[r] = o;
      if (a.mask != nullptr)
        m_s[r] = __ldg(a.mask + static_cast<int64_t>(c) * a.n + row0 + r);
    }
  }
  __syncthreads();
  if (multi && j + 1 < a.steps) {
    const int32_t* src = idx_j + a.idx_step_stride + ident_of(a, c) * a.idx_stride + row0;
    for (int r = tid; r < R; r += (WARPS * 32)) cp_async4(idx_next + r, src + r);
    asm volatile("cp.async.commit_group;" ::: "memory");
  }

  // w of the chain: from global memory at the first step of a launch, then
  // from the copy the previous step's update left in shared memory.
  float4 wq[QPL];
  Accum<QPL> A;
  const float* w_in = a.w + static_cast<int64_t>(c) * a.d;
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = lane + 32 * k;
    const int e0 = 4 * q;
    if (multi && j > 0) {
      wq[k] = q < dq ? w_s[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      wq[k].x = e0 + 0 < a.d ? w_in[e0 + 0] : 0.0f;
      wq[k].y = e0 + 1 < a.d ? w_in[e0 + 1] : 0.0f;
      wq[k].z = e0 + 2 < a.d ? w_in[e0 + 2] : 0.0f;
      wq[k].w = e0 + 3 < a.d ? w_in[e0 + 3] : 0.0f;
    }
    A.acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  A.mlk = A.mlk_c = A.K = A.s1 = A.s2 = 0.0f;
  A.cnt = 0;
  // What the epilogue needs, loaded now so that the latency overlaps the row
  // stream instead of stalling the step after it: the schedule at this step
  // (counter, then table entries), the chain's RMSprop state for this
  // thread's parameters (q = tid), and sum(w^2) for the prior (warp 0, from
  // the w just loaded; zero past d).
  int64_t k_step = 0;
  float h_step = 0.0f, t_step = 1.0f;
  int slot = -1;
  float4 vq = make_float4(0.f, 0.f, 0.f, 0.f);
  if (a.mode == kSgldStep) {
    k_step = a.sched.step() + j;
    h_step = a.sched.step_size(k_step);
    t_step = a.sched.temperature(k_step, c);
    slot = a.sched.keep_slot(k_step);
    if (a.v != nullptr && tid < dq) {
      const float* vc = a.v + static_cast<int64_t>(c) * a.d + 4 * tid;
      const int e0 = 4 * tid;
      vq.x = vc[0];
      vq.y = e0 + 1 < a.d ? vc[1] : 0.0f;
      vq.z = e0 + 2 < a.d ? vc[2] : 0.0f;
      vq.w = e0 + 3 < a.d ? vc[3] : 0.0f;
    }
  }
  if (a.inv_p2 > 0.0f && warp == 0) {
    double ww = 0.0;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const double e[4] = {wq[k].x, wq[k].y, wq[k].z, wq[k].w};
#pragma unroll
      for (int i = 0; i < 4; ++i) ww += e[i] * e[i];
    }
    ww = warp_sum(ww);
    if (lane == 0) sums[WARPS * 4 + 3] = ww;
  }
  const int g = lane >> (5 - LOG);           // my row in the link phase
  const bool leader = (lane & (GROUP - 1)) == 0;
  float* lk_out = a.lk != nullptr ? a.lk + static_cast<int64_t>(c) * a.n + row0
                                  : nullptr;
  constexpr int kStride = WARPS * RW;
  if (PF) {
    // Two register tiles: the loads of the next tile are in flight while
    // the current one is consumed.
    float4 xa[RW][QPL], xb[RW][QPL];
    float ya, yb;
    int oa, ob;
    int r0 = warp * RW;
    load_tile<QPL, RW>(a, idx_s, R, r0, lane, g, xa, ya, oa);
    while (r0 < R) {
      load_tile<QPL, RW>(a, idx_s, R, r0 + kStride, lane, g, xb, yb, ob);
      consume_tile<QPL, RW>(a, m_s, lk_out, r0, lane, g, leader, wq, xa, ya, oa, A);
      r0 += kStride;
      if (r0 >= R) break;
      load_tile<QPL, RW>(a, idx_s, R, r0 + kStride, lane, g, xa, ya, oa);
      consume_tile<QPL, RW>(a, m_s, lk_out, r0, lane, g, leader, wq, xb, yb, ob, A);
      r0 += kStride;
    }
  } else {
    for (int r0 = warp * RW; r0 < R; r0 += kStride) {
      float4 xv[RW][QPL];
      float yv;
      int og;
      load_tile<QPL, RW>(a, idx_s, R, r0, lane, g, xv, yv, og);
      consume_tile<QPL, RW>(a, m_s, lk_out, r0, lane, g, leader, wq, xv, yv, og, A);
    }
  }
  // Widen once: sum(lk) = s1 + n K, sum(lk^2) = s2 + 2 K s1 + n K^2.
  const double K = A.K, n_l = A.cnt;
  double my_mlk = static_cast<double>(A.mlk) + A.mlk_c;
  double my_lk = static_cast<double>(A.s1) + n_l * K;
  double my_lk2 = static_cast<double>(A.s2) + 2.0 * K * A.s1 + n_l * K * K;
  my_mlk = warp_sum(my_mlk);
  my_lk = warp_sum(my_lk);
  my_lk2 = warp_sum(my_lk2);
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = lane + 32 * k;
    if (q < dq) red[warp * dq + q] = A.acc[k];
  }
  if (lane == 0) {
    sums[warp * 4 + 0] = my_mlk;
    sums[warp * 4 + 1] = my_lk;
    sums[warp * 4 + 2] = my_lk2;
  }
  __syncthreads();

  // Reduce the warp partials in a fixed order: partial gradient in red[0..dq).
  for (int q = tid; q < dq; q += (WARPS * 32)) {
    float4 t = red[q];
    for (int w = 1; w < WARPS; ++w) {
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
    for (int w = 0; w < WARPS; ++w) {
      t0 += sums[w * 4 + 0];
      t1 += sums[w * 4 + 1];
      t2 += sums[w * 4 + 2];
    }
    sums[WARPS * 4 + 0] = t0;
    sums[WARPS * 4 + 1] = t1;
    sums[WARPS * 4 + 2] = t2;
  }
  __syncthreads();

  if (a.slices > 1) {
    const int64_t pc = static_cast<int64_t>(c) * a.slices + s;
    for (int q = tid; q < dq; q += (WARPS * 32)) a.ws_part[pc * dq + q] = red[q];
    if (tid == 0) {
      a.ws_sums[pc * 4 + 0] = sums[WARPS * 4 + 0];
      a.ws_sums[pc * 4 + 1] = sums[WARPS * 4 + 1];
      a.ws_sums[pc * 4 + 2] = sums[WARPS * 4 + 2];
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
    for (int q = tid; q < dq; q += (WARPS * 32)) {
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
      sums[WARPS * 4 + 0] = t0;
      sums[WARPS * 4 + 1] = t1;
      sums[WARPS * 4 + 2] = t2;
    }
    __syncthreads();
  }

  // ------------------------------ epilogue ---------------------------------
  const double sum_mlk = sums[WARPS * 4 + 0];
  const double sum_lk = sums[WARPS * 4 + 1];
  const double sum_lk2 = sums[WARPS * 4 + 2];
  float* wc = a.w + static_cast<int64_t>(c) * a.d;
  const float scale = static_cast<float>(static_cast<double>(a.n_obs) / a.n);

  const double ww = a.inv_p2 > 0.0f ? sums[WARPS * 4 + 3] : 0.0;
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
      for (int j = tid; j < a.d; j += (WARPS * 32))
        gc[j] = (-scale * gl[j] + wc[j] * a.inv_p2) * a.inv_temp;
    }
    if (tid == 0) {
      a.U[c] = U;
      if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    }
    return;
  }

  // SGLD (+RMSprop) update of chain c: thread tid < dq owns the four
  // parameters 4 tid .. 4 tid + 3, whose w is in its warp's wq[tid / 32]
  // (dq <= 32 QPL <= WARPS * 32).
  const float noise_scale = sqrtf(2.0f * t_step * h_step);
  float* vc = a.v != nullptr ? a.v + static_cast<int64_t>(c) * a.d : nullptr;
  float* smp = slot >= 0 ? a.samples + (static_cast<int64_t>(slot) * a.chains + c) * a.d
                         : nullptr;
  bool bad = false;
  if (tid < dq) {
    const int q = tid;
    float4 xq = wq[0];
#pragma unroll
    for (int k = 1; k < QPL; ++k)
      if (warp == k) xq = wq[k];
    const float xs[4] = {xq.x, xq.y, xq.z, xq.w};
    const float vs[4] = {vq.x, vq.y, vq.z, vq.w};
    float xi[4];
    noise4(a.noise, ident_of(a, c), 4 * q, a.d, k_step, GBSGMC_TAG_SGLD, xi);
    float xn[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int jj = 4 * q + e;
      if (jj >= a.d) break;
      const float x = xs[e];
      const float g = (-scale * gl[jj] + x * a.inv_p2) * a.inv_temp;
      bad |= !isfinite(g);
      const float scaled_gradient = -h_step * g;
      const float scaled_noise = noise_scale * xi[e];
      float x_new;
      if (vc != nullptr) {
        const float vn = a.alpha * vs[e] + (1.0f - a.alpha) * (g * g);
        const float G = 1.0f / (a.lmbd + sqrtf(vn));
        const float sG = sqrtf(G);
        vc[jj] = vn;
        x_new = x + ((0.0f + G * scaled_gradient) + sG * scaled_noise);
      } else {
        x_new = x + (scaled_gradient + scaled_noise);
      }
      wc[jj] = x_new;
      xn[e] = x_new;
      if (smp != nullptr) smp[jj] = x_new;
    }
    if (multi) w_s[q] = make_float4(xn[0], xn[1], xn[2], xn[3]);
  }
  if (bad) raise_status(a.status, GBSGMC_ERR_NONFINITE);
  if (tid == 0) {
    if (a.U != nullptr) a.U[c] = U;
    if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    if (slot >= 0 && a.sample_lik != nullptr)
      a.sample_lik[static_cast<int64_t>(slot) * a.chains + c] = -U;
  }
}

// One launch runs a.steps consecutive SGLD steps (a.steps > 1 only with one
// CTA per chain: a chain's step depends on nothing but its own previous
// step, so the CTA that owns the chain runs them back to back).  Chains drift
// out of phase, so one CTA's index loads and update overlap the row streams
// of the others, and the steps pay no launch gap or grid tail.
template <int QPL, int RW, bool PF, int MINB, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, MINB)
    glm_kernel(const GlmArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  for (int j = 0; j < a.steps; ++j) {
    if (j > 0) __syncthreads();  // step j-1's update of w is visible
    glm_step<QPL, RW, PF, WARPS>(a, j, smem);
  }
}

// ---------------------------------------------------------------------------
// Dynamically scheduled form.  The rows of one launch are cut into items of
// rows_per_slice rows of one chain (item u = chain * items + item), and every
// warp of a persistent grid claims items from a counter in the workspace
// until none are left: all SMs stay busy until the last item, whatever the
// ratio of chains to SMs (256 chains on 152 SMs leave a static grid with one
// or two CTAs per SM).  A warp loads the chain's w into registers, streams
// the item's rows through the same tile loads and link as glm_kernel, and
// writes the item's partial gradient and sums to the workspace.  The warp
// that completes a chain's last item (per-chain ticket) adds the chain's
// partials in item order -- the order does not depend on scheduling -- and
// runs the epilogue and update of that chain alone.  The last warp to leave
// the grid resets the claim counter for the next launch.
// ---------------------------------------------------------------------------

// Epilogue of chain c run by one warp: gq gets the chain's summed partial
// gradient; wq holds the chain's w (lane's float4 columns q = lane + 32 k).
template <int QPL>
__device__ __forceinline__ void dyn_epilogue(const GlmArgs& a, int c, int lane,
                                             const float4 (&wq)[QPL]) {
  const int dq = a.dq, ipc = a.slices;
  const float4* part = a.ws_part + static_cast<int64_t>(c) * ipc * dq;
  float gl[QPL][4];
  double ww = 0.0;
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = lane + 32 * k;
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    if (q < dq) {
      t = __ldcg(part + q);
      for (int s = 1; s < ipc; ++s) {
        const float4 u = __ldcg(part + static_cast<int64_t>(s) * dq + q);
        t.x += u.x;
        t.y += u.y;
        t.z += u.z;
        t.w += u.w;
      }
    }
    gl[k][0] = t.x;
    gl[k][1] = t.y;
    gl[k][2] = t.z;
    gl[k][3] = t.w;
    if (a.inv_p2 > 0.0f) {
      const float wv[4] = {wq[k].x, wq[k].y, wq[k].z, wq[k].w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const double wj = wv[e];  // zero past d
        ww += wj * wj;
      }
    }
  }
  double t0 = 0.0, t1 = 0.0, t2 = 0.0;
  const double* ps = a.ws_sums + static_cast<int64_t>(c) * ipc * 4;
  for (int s = lane; s < ipc; s += 32) {
    t0 += __ldcg(ps + s * 4 + 0);
    t1 += __ldcg(ps + s * 4 + 1);
    t2 += __ldcg(ps + s * 4 + 2);
  }
  const double sum_mlk = warp_sum(t0);
  const double sum_lk = warp_sum(t1);
  const double sum_lk2 = warp_sum(t2);
  ww = warp_sum(ww);

  float* wc = a.w + static_cast<int64_t>(c) * a.d;
  const float scale = static_cast<float>(static_cast<double>(a.n_obs) / a.n);
  const double log_prior = -0.5 * ww * a.inv_p2 - a.prior_const;
  const double lik = a.mask == nullptr
                         ? -static_cast<double>(a.n_obs) * (sum_mlk / a.n)
                         : -(static_cast<double>(a.n_obs) / a.n) * sum_mlk;
  const double U = (lik - log_prior) * a.inv_temp;
  const double mean_lk = sum_lk / a.n;
  const double var_lk = fmax(sum_lk2 / a.n - mean_lk * mean_lk, 0.0);
  if (lane == 0 && !isfinite(U)) raise_status(a.status, GBSGMC_ERR_NONFINITE);

  if (a.mode == kValueGrad) {
    if (a.grad != nullptr) {
      float* gc = a.grad + static_cast<int64_t>(c) * a.d;
#pragma unroll
      for (int k = 0; k < QPL; ++k) {
        const float wv[4] = {wq[k].x, wq[k].y, wq[k].z, wq[k].w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = 4 * (lane + 32 * k) + e;
          if (j < a.d) gc[j] = (-scale * gl[k][e] + wv[e] * a.inv_p2) * a.inv_temp;
        }
      }
    }
    if (lane == 0) {
      a.U[c] = U;
      if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    }
    return;
  }

  const int64_t k_step = a.sched.step();
  const float h = a.sched.step_size(k_step);
  const float T = a.sched.temperature(k_step, c);
  const int slot = a.sched.keep_slot(k_step);
  const float noise_scale = sqrtf(2.0f * T * h);
  float* vc = a.v != nullptr ? a.v + static_cast<int64_t>(c) * a.d : nullptr;
  float* smp = slot >= 0 ? a.samples + (static_cast<int64_t>(slot) * a.chains + c) * a.d
                         : nullptr;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < QPL; ++k) {
    const int q = lane + 32 * k;
    if (q >= dq) continue;
    float xi[4];
    noise4(a.noise, ident_of(a, c), 4 * q, a.d, k_step, GBSGMC_TAG_SGLD, xi);
    const float wv[4] = {wq[k].x, wq[k].y, wq[k].z, wq[k].w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int j = 4 * q + e;
      if (j >= a.d) break;
      const float x = wv[e];
      const float g = (-scale * gl[k][e] + x * a.inv_p2) * a.inv_temp;
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
  if (lane == 0) {
    if (a.U != nullptr) a.U[c] = U;
    if (a.lk_var != nullptr) a.lk_var[c] = var_lk;
    if (slot >= 0 && a.sample_lik != nullptr)
      a.sample_lik[static_cast<int64_t>(slot) * a.chains + c] = -U;
  }
}

// Shared memory of the dynamic kernel: per warp, the indices and mask
// weights of its current item.
__host__ __device__ inline size_t dyn_smem_bytes(int item_rows, int warps) {
  return static_cast<size_t>(warps) * item_rows * (sizeof(int32_t) + sizeof(float));
}

template <int QPL, int RW, int MINB, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, MINB)
    glm_dyn_kernel(const GlmArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int LOG = Log2<RW>::v;
  constexpr int GROUP = 32 >> LOG;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int IR = a.rows_per_slice;
  int32_t* idx_s = reinterpret_cast<int32_t*>(smem) + static_cast<size_t>(warp) * IR;
  float* m_s = reinterpret_cast<float*>(smem) + static_cast<size_t>(WARPS + warp) * IR;
  const int ipc = a.slices;
  const int total = a.chains * ipc;
  unsigned* claim = a.ws_ticket + a.chains;
  unsigned* exits = claim + 1;
  const int g = lane >> (5 - LOG);
  const bool leader = (lane & (GROUP - 1)) == 0;

  int u = 0;
  if (lane == 0) u = static_cast<int>(atomicAdd(claim, 1u));
  u = __shfl_sync(0xffffffffu, u, 0);
  while (u < total) {
    // The next item is claimed now; its number is needed only at the end.
    int un = 0;
    if (lane == 0) un = static_cast<int>(atomicAdd(claim, 1u));
    const int c = u / ipc, s = u - c * ipc;
    const int row0 = s * IR;
    const int R = max(0, min(IR, a.n - row0));
    __syncwarp();  // the previous item's reads of idx_s / m_s are done
    for (int r = lane; r < R; r += 32) {
      int32_t o = __ldg(a.idx + ident_of(a, c) * a.idx_stride + row0 + r);
      if (o < 0 || o >= a.n_rows) {
        raise_status(a.status, GBSGMC_ERR_INDEX);
        o = -1;
      }
      idx_s[r] = o;
      if (a.mask != nullptr)
        m_s[r] = __ldg(a.mask + static_cast<int64_t>(c) * a.n + row0 + r);
    }
    float4 wq[QPL];
    Accum<QPL> A;
    const float* w_in = a.w + static_cast<int64_t>(c) * a.d;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int j = 4 * (lane + 32 * k);
      wq[k].x = j + 0 < a.d ? w_in[j + 0] : 0.0f;
      wq[k].y = j + 1 < a.d ? w_in[j + 1] : 0.0f;
      wq[k].z = j + 2 < a.d ? w_in[j + 2] : 0.0f;
      wq[k].w = j + 3 < a.d ? w_in[j + 3] : 0.0f;
      A.acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    A.mlk = A.mlk_c = A.K = A.s1 = A.s2 = 0.0f;
    A.cnt = 0;
    __syncwarp();
    float* lk_out = a.lk != nullptr ? a.lk + static_cast<int64_t>(c) * a.n + row0
                                    : nullptr;
    for (int r0 = 0; r0 < R; r0 += RW) {
      float4 xv[RW][QPL];
      float yv;
      int og;
      load_tile<QPL, RW>(a, idx_s, R, r0, lane, g, xv, yv, og);
      consume_tile<QPL, RW>(a, m_s, lk_out, r0, lane, g, leader, wq, xv, yv, og, A);
    }
    const double K = A.K, n_l = A.cnt;
    const double my_mlk = warp_sum(static_cast<double>(A.mlk) + A.mlk_c);
    const double my_lk = warp_sum(static_cast<double>(A.s1) + n_l * K);
    const double my_lk2 =
        warp_sum(static_cast<double>(A.s2) + 2.0 * K * A.s1 + n_l * K * K);
    const int64_t pc = static_cast<int64_t>(c) * ipc + s;
#pragma unroll
    for (int k = 0; k < QPL; ++k) {
      const int q = lane + 32 * k;
      if (q < a.dq) a.ws_part[pc * a.dq + q] = A.acc[k];
    }
    if (lane == 0) {
      a.ws_sums[pc * 4 + 0] = my_mlk;
      a.ws_sums[pc * 4 + 1] = my_lk;
      a.ws_sums[pc * 4 + 2] = my_lk2;
    }
    __threadfence();
    __syncwarp();
    int last = 0;
    if (lane == 0) {
      const unsigned ticket = atomicAdd(a.ws_ticket + c, 1u);
      last = ticket == static_cast<unsigned>(ipc - 1);
      if (last) a.ws_ticket[c] = 0u;  // ready for the next launch
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence();
      dyn_epilogue<QPL>(a, c, lane, wq);
    }
    u = __shfl_sync(0xffffffffu, un, 0);
  }
  // Every claim of this warp precedes its exit; the last warp to leave sees
  // all claims done and resets both counters.
  __threadfence();
  if (lane == 0) {
    const unsigned e = atomicAdd(exits, 1u);
    if (e == gridDim.x * static_cast<unsigned>(WARPS) - 1u) {
      atomicExch(claim, 0u);
      atomicExch(exits, 0u);
    }
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
  // Per-chain tickets, then the claim and exit counters of glm_dyn_kernel.
  b += align_up((static_cast<size_t>(chains) + 2) * sizeof(unsigned), 256);
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

// Rows a warp holds at once, and the CTAs per SM the register budget is set
// for, per float4-column count QPL.  More rows per warp cut the per-row
// instruction count (one transposed reduction and one link evaluation per
// lane group) at the price of registers and resident warps; for d <= 256 the
// measured best is 4 rows per warp at 3 CTAs/SM.  Plans autotune this.
__host__ __device__ constexpr int default_rows_per_warp(int qpl) {
  return qpl <= 2 ? 4 : (qpl == 4 ? 2 : 1);
}

int qpl_for(int dq) { return dq <= 32 ? 1 : (dq <= 64 ? 2 : (dq <= 128 ? 4 : 8)); }

int env_int(const char* name, int fallback) {
  const char* v = std::getenv(name);
  if (v == nullptr || *v == 0) return fallback;
  const int x = std::atoi(v);
  return x > 0 ? x : fallback;
}

int clamp_slices(int s, int n) {
  return std::min(std::max(s, ceil_div(n, kMaxRowsPerSlice)),
                  std::min(slices_alloc(n), std::max(1, n)));
}

// Slices per chain when the caller does not choose: enough rows per CTA to
// amortise its prologue and epilogue (about 384 KB of rows; the per-CTA fixed
// cost was measured at tens of rows), but at least one CTA per SM for small
// problems so that their latency is spread.  Plans autotune this choice.
int choose_slices(int chains, int n, int row_bytes) {
  const int forced = env_int("GBSGMC_GLM_SLICES", 0);
  if (forced > 0) return clamp_slices(forced, n);
  const double target = 384.0 * 1024.0;
  int s = static_cast<int>(std::ceil(static_cast<double>(n) * row_bytes / target));
  if (static_cast<int64_t>(chains) * s < sm_count())
    s = std::max(s, std::min(ceil_div(sm_count(), std::max(chains, 1)), n / 32));
  return clamp_slices(std::max(s, 1), n);
}

constexpr int kMaxDynSmem = 227 * 1024;

template <int QPL, int RW, bool PF, int MINB, int WARPS>
struct Variant {
  static int prepare() {
    static int done = 0;
    if (done) return GBSGMC_OK;
    const cudaError_t e = cudaFuncSetAttribute(
        glm_kernel<QPL, RW, PF, MINB, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        kMaxDynSmem);
    if (e != cudaSuccess)
      return set_error(GBSGMC_ERR_CUDA, "glm: cudaFuncSetAttribute: %s",
                       cudaGetErrorString(e));
    done = 1;
    return GBSGMC_OK;
  }
  // Resident CTAs per SM for this variant at `smem` bytes (cached per size).
  static int occupancy(size_t smem) {
    static size_t last_smem = 0;
    static int last = 0;
    if (last > 0 && last_smem == smem) return last;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, glm_kernel<QPL, RW, PF, MINB, WARPS>, WARPS * 32, smem) != cudaSuccess ||
        nb < 1)
      nb = 1;
    last_smem = smem;
    last = nb;
    return nb;
  }
  static int launch(GlmArgs a, size_t smem, cudaStream_t st) {
    const int rc = prepare();
    if (rc != GBSGMC_OK) return rc;
    a.slices = a.slices_fixed > 0
                   ? clamp_slices(a.slices_fixed, a.n)
                   : choose_slices(a.chains, a.n,
                                   static_cast<int>(std::min<int64_t>(a.ld, 1 << 20)) * 4);
    a.rows_per_slice = ceil_div(a.n, a.slices);
    if (a.slices > 1) {
      if (a.ws_base == nullptr || a.ws_size < ws_bytes(a.chains, a.n, a.d))
        return set_error(GBSGMC_ERR_ARG,
                         "glm: workspace missing or too small (need %zu bytes)",
                         ws_bytes(a.chains, a.n, a.d));
      const WsView v = ws_view(a.ws_base, a.chains, a.n, a.d);
      a.ws_part = v.part;
      a.ws_sums = v.sums;
      a.ws_ticket = v.ticket;
    }
    dim3 grid(a.slices, a.chains);
    if (a.steps > 1 && a.slices > 1) {
      // Several CTAs per chain: one launch per step.
      GlmArgs b = a;
      b.steps = 1;
      for (int j = 0; j < a.steps; ++j) {
        b.idx = a.idx + j * a.idx_step_stride;
        b.sched.offset = a.sched.offset + j;
        glm_kernel<QPL, RW, PF, MINB, WARPS><<<grid, WARPS * 32, smem, st>>>(b);
        const int rc2 = check_launch("glm_kernel");
        if (rc2 != GBSGMC_OK) return rc2;
      }
      return GBSGMC_OK;
    }
    glm_kernel<QPL, RW, PF, MINB, WARPS><<<grid, WARPS * 32, smem, st>>>(a);
    return check_launch("glm_kernel");
  }
};

// The dynamically scheduled kernel: `slices` is the number of items per
// chain, the grid is as many CTAs as fit on the SMs at once (no more than the
// items need).
template <int QPL, int RW, int MINB, int WARPS>
struct DynVariant {
  static int prepare() {
    static int done = 0;
    if (done) return GBSGMC_OK;
    const cudaError_t e = cudaFuncSetAttribute(
        glm_dyn_kernel<QPL, RW, MINB, WARPS>,
        cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem);
    if (e != cudaSuccess)
      return set_error(GBSGMC_ERR_CUDA, "glm: cudaFuncSetAttribute: %s",
                       cudaGetErrorString(e));
    done = 1;
    return GBSGMC_OK;
  }
  static int occupancy(size_t smem) {
    static size_t last_smem = 0;
    static int last = 0;
    if (last > 0 && last_smem == smem) return last;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, glm_dyn_kernel<QPL, RW, MINB, WARPS>, WARPS * 32, smem) != cudaSuccess ||
        nb < 1)
      nb = 1;
    last_smem = smem;
    last = nb;
    return nb;
  }
  static int launch(GlmArgs a, cudaStream_t st) {
    const int rc = prepare();
    if (rc != GBSGMC_OK) return rc;
    const int want = a.slices_fixed > 0 ? a.slices_fixed : kMinSlicesAlloc;
    const int ipc0 = clamp_slices(want, a.n);
    a.rows_per_slice = ceil_div(a.n, ipc0);
    a.slices = ceil_div(a.n, a.rows_per_slice);  // no empty items
    if (a.ws_base == nullptr || a.ws_size < ws_bytes(a.chains, a.n, a.d))
      return set_error(GBSGMC_ERR_ARG,
                       "glm: workspace missing or too small (need %zu bytes)",
                       ws_bytes(a.chains, a.n, a.d));
    const WsView v = ws_view(a.ws_base, a.chains, a.n, a.d);
    a.ws_part = v.part;
    a.ws_sums = v.sums;
    a.ws_ticket = v.ticket;
    const size_t smem = dyn_smem_bytes(a.rows_per_slice, WARPS);
    const int64_t items = static_cast<int64_t>(a.chains) * a.slices;
    const int64_t need = (items + WARPS - 1) / WARPS;
    const int grid = static_cast<int>(
        std::max<int64_t>(1, std::min<int64_t>(need,
                                               static_cast<int64_t>(sm_count()) *
                                                   occupancy(smem))));
    GlmArgs b = a;
    b.steps = 1;
    for (int j = 0; j < a.steps; ++j) {
      b.idx = a.idx + j * a.idx_step_stride;
      b.sched.offset = a.sched.offset + j;
      glm_dyn_kernel<QPL, RW, MINB, WARPS><<<grid, WARPS * 32, smem, st>>>(b);
      const int rc2 = check_launch("glm_dyn_kernel");
      if (rc2 != GBSGMC_OK) return rc2;
    }
    return GBSGMC_OK;
  }
};

// Launch-shape overrides for experiments: GBSGMC_GLM_RW (2 or 4 rows per
// warp, d <= 256), GBSGMC_GLM_WARPS (8 or 16 warps per CTA),
// GBSGMC_GLM_SLICES (CTAs per chain, or items per chain with
// GBSGMC_GLM_DYN=1: the dynamically scheduled kernel).
int rows_override() { return env_int("GBSGMC_GLM_RW", 0); }
int warps_override() { return env_int("GBSGMC_GLM_WARPS", 0); }
int prefetch_override() { return env_int("GBSGMC_GLM_PF", -1); }
int dynamic_override() { return env_int("GBSGMC_GLM_DYN", -1); }

// Dispatch over the tuned shape: rows per warp (RW) and warps per CTA.  The
// register budget (MINB) is 3 CTAs/SM for 8-warp CTAs with RW = 4, otherwise
// what fits without spilling.
template <int QPL>
int launch_q(const GlmArgs& a, size_t smem, cudaStream_t st) {
  const int warps = a.warps_fixed > 0 ? a.warps_fixed
                    : (warps_override() > 0 ? warps_override() : 8);
  const bool big = warps >= 16;
  if constexpr (QPL <= 2) {
    const int rw = a.rw_fixed > 0 ? a.rw_fixed
                   : (rows_override() > 0 ? rows_override()
                                          : default_rows_per_warp(QPL));
    const bool dyn = a.dyn_fixed > 0 || (a.dyn_fixed == 0 && dynamic_override() > 0);
    if (dyn) {
      if (rw == 8) return DynVariant<QPL, 8, 2, 8>::launch(a, st);
      if (rw == 4) return DynVariant<QPL, 4, 3, 8>::launch(a, st);
      return DynVariant<QPL, 2, 4, 8>::launch(a, st);
    }
    const int pfo = prefetch_override();
    const bool pf = a.pf_fixed > 0 || (a.pf_fixed == 0 && pfo > 0);
    // Prefetching variants hold two tiles in registers, so they get the
    // register budget of fewer resident CTAs.
    if (rw == 8) return Variant<QPL, 8, false, 2, 8>::launch(a, smem, st);
    if (rw == 4) {
      if (pf) return big ? Variant<QPL, 4, true, 1, 16>::launch(a, smem, st)
                         : Variant<QPL, 4, true, 2, 8>::launch(a, smem, st);
      return big ? Variant<QPL, 4, false, 1, 16>::launch(a, smem, st)
                 : Variant<QPL, 4, false, 3, 8>::launch(a, smem, st);
    }
    if (pf) return Variant<QPL, 2, true, 3, 8>::launch(a, smem, st);
    return big ? Variant<QPL, 2, false, 2, 16>::launch(a, smem, st)
               : Variant<QPL, 2, false, 4, 8>::launch(a, smem, st);
  } else if constexpr (QPL == 4) {
    return big ? Variant<4, 2, false, 1, 16>::launch(a, smem, st)
               : Variant<4, 2, false, 2, 8>::launch(a, smem, st);
  } else {
    return big ? Variant<8, 1, false, 1, 16>::launch(a, smem, st)
               : Variant<8, 1, false, 2, 8>::launch(a, smem, st);
  }
}

int launch_glm(GlmArgs& a, cudaStream_t st) {
  if (a.chains == 0 || a.n == 0) return GBSGMC_OK;
  const int qpl = qpl_for(a.dq);
  // Shared memory sized for the largest slice any choice can give.
  const SmemLayout L = smem_layout(std::min(a.n, kMaxRowsPerSlice), a.dq, kMaxWarps);
  if (L.total > 227 * 1024)
    return set_error(GBSGMC_ERR_SHAPE, "glm: shared memory %zu too large",
                     L.total);
  if (qpl == 1) return launch_q<1>(a, L.total, st);
  if (qpl == 2) return launch_q<2>(a, L.total, st);
  if (qpl == 4) return launch_q<4>(a, L.total, st);
  return launch_q<8>(a, L.total, st);
}

int fill_common(GlmArgs& a, const gbsgmc_glm* m, int chains, int n,
                const int32_t* idx, int64_t idx_stride, const float* mask,
                void* ws, size_t ws_size, int* status, GlmTune tune = GlmTune{}) {
  if (m == nullptr || m->X == nullptr || idx == nullptr ||
      (m->y == nullptr && !m->y_inline && m->family != GBSGMC_GLM_LINEAR))
    return set_error(GBSGMC_ERR_ARG, "glm: null model, data or index pointer");
  if (m->y_inline && m->ld < static_cast<int64_t>(m->d) + 1)
    return set_error(GBSGMC_ERR_ARG, "glm: y_inline needs ld >= d + 1");
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
  a.family = m->family;
  a.d = m->d;
  a.dq = (m->d + 3) / 4;
  a.y_inline = m->y_inline ? 1 : 0;
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
  a.slices = 0;
  a.rows_per_slice = 0;
  if (tune.slices == 0 && tune.rows_per_warp == 0 && tune.warps == 0)
    glm_tune_lookup(chains, n, m->d, m->ld, &tune);
  a.slices_fixed = tune.slices;
  a.rw_fixed = tune.rows_per_warp;
  a.warps_fixed = tune.warps;
  a.pf_fixed = tune.prefetch > 0 ? 1 : (tune.rows_per_warp > 0 ? -1 : 0);
  a.dyn_fixed = tune.dynamic > 0 ? 1 : (tune.rows_per_warp > 0 ? -1 : 0);
  a.ws_base = ws;
  a.ws_size = ws_size;
  a.ws_part = nullptr;
  a.ws_sums = nullptr;
  a.ws_ticket = nullptr;
  a.idx = idx;
  a.idx_stride = idx_stride;
  a.steps = 1;
  a.idx_step_stride = 0;
  a.mask = mask;
  a.status = status;
  // 128-bit row loads need every row 16-byte aligned.
  a.vec4 = (reinterpret_cast<uintptr_t>(m->X) % 16 == 0) && (m->ld % 4 == 0) ? 1 : 0;
  a.lk = nullptr;
  a.lk_var = nullptr;
  a.grad = nullptr;
  a.U = nullptr;
  a.samples = nullptr;
  a.sample_lik = nullptr;
  a.v = nullptr;
  a.alpha = 0.9f;
  a.lmbd = 1e-5f;
  a.sched = Sched{nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0.0f, 1.0f};
  a.noise = Noise{nullptr, 0, 0, 0};
  a.ident = nullptr;
  return GBSGMC_OK;
}

struct TuneKey {
  int chains, n, d;
  int64_t ld;
  bool operator<(const TuneKey& o) const {
    return std::tie(chains, n, d, ld) < std::tie(o.chains, o.n, o.d, o.ld);
  }
};
std::mutex g_tune_mutex;
std::map<TuneKey, GlmTune> g_tune_cache;

}  // namespace

bool glm_tune_lookup(int chains, int n, int d, int64_t ld, GlmTune* out) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tune_cache.find(TuneKey{chains, n, d, ld});
  if (it == g_tune_cache.end()) return false;
  *out = it->second;
  return true;
}

void glm_tune_store(int chains, int n, int d, int64_t ld, GlmTune t) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_cache[TuneKey{chains, n, d, ld}] = t;
}

// Shared with the plan implementation.
size_t glm_ws_bytes(int chains, int n, int d) { return ws_bytes(chains, n, d); }

int glm_prepare() {
  // Sets the shared-memory attribute of every variant before any stream
  // capture.
  int rc = Variant<1, 4, false, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 8, false, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 4, true, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 4, true, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 2, true, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 8, false, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 4, true, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 4, true, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 2, true, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 4, false, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 2, false, 4, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<1, 2, false, 2, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 4, false, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 4, false, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 2, false, 4, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<2, 2, false, 2, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<4, 2, false, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<4, 2, false, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<8, 1, false, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = Variant<8, 1, false, 1, 16>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<1, 8, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<1, 4, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<1, 2, 4, 8>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<2, 8, 2, 8>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<2, 4, 3, 8>::prepare();
  if (rc == GBSGMC_OK) rc = DynVariant<2, 2, 4, 8>::prepare();
  return rc;
}

int glm_sgld_step(const gbsgmc_glm* model, int chains, int n,
                  const int32_t* idx_dev, int64_t idx_stride, float* w_dev,
                  float* v_dev, float alpha, float lmbd,
                  const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                  double* U_dev, double* lk_var_dev, float* samples_dev,
                  double* sample_lik_dev, void* ws, size_t ws_size,
                  int* status_dev, cudaStream_t stream, GlmTune tune, int steps,
                  int64_t idx_step_stride, const int32_t* ident_dev) {
  GlmArgs a;
  int rc = fill_common(a, model, chains, n, idx_dev, idx_stride, nullptr, ws,
                       ws_size, status_dev, tune);
  if (rc != GBSGMC_OK) return rc;
  if (w_dev == nullptr || sched == nullptr || noise == nullptr)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step: null w, sched or noise");
  if (sched->keep_slot_dev != nullptr && samples_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG,
                     "sgld_glm_step: keep table given without sample buffer");
  if (noise->noise_dev != nullptr && noise->noise_stride < model->d)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_step: noise_stride < d");
  if (steps < 1 || idx_step_stride < 0 || (steps > 1 && noise->noise_dev != nullptr))
    return set_error(GBSGMC_ERR_ARG,
                     "sgld_glm_steps: steps < 1, negative index step stride, or "
                     "injected noise with several steps");
  if (steps > 1 && chains == 0) return GBSGMC_OK;
  if (ident_dev != nullptr && steps > 1)
    return set_error(GBSGMC_ERR_ARG, "sgld_glm_steps: chain identities need one step "
                                     "per launch");
  a.ident = ident_dev;
  a.steps = steps;
  a.idx_step_stride = steps > 1 ? idx_step_stride : 0;
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
                       static_cast<cudaStream_t>(stream), GlmTune{}, 1, 0);
}

extern "C" int gbsgmc_sgld_glm_steps(
    const gbsgmc_glm* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, int64_t idx_step_stride, int steps, float* w_dev,
    float* v_dev, float alpha, float lmbd, const gbsgmc_sched* sched,
    const gbsgmc_noise* noise, double* U_dev, double* lk_var_dev,
    float* samples_dev, double* sample_lik_dev, void* workspace_dev,
    size_t workspace_bytes, int* status_dev, gbsgmc_stream_t stream) {
  return glm_sgld_step(model, chains, n, idx_dev, idx_stride, w_dev, v_dev,
                       alpha, lmbd, sched, noise, U_dev, lk_var_dev,
                       samples_dev, sample_lik_dev, workspace_dev,
                       workspace_bytes, status_dev,
                       static_cast<cudaStream_t>(stream), GlmTune{}, steps,
                       idx_step_stride);
}
