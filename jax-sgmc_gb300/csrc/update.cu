// Elementwise integrator updates over [chains, P] and the reSGLD exchange.
//
// Each kernel mirrors the operation order of the reference tree arithmetic so
// that fp32 results agree to rounding: e.g. the OBABO refresh is
// sqrt(e^{-f h}) p + sqrt((1 - e^{-f h}) T) (sqrt(m) xi), evaluated as the
// reference's _momentum_resampling writes it.  Grid: (groups, chains), four
// parameters per thread so that one Philox call feeds one thread.
#include <algorithm>

#include <cuda_bf16.h>

#include "common.cuh"
#include "internal.h"

namespace gbsgmc {
namespace {

constexpr int kThreads = 256;

struct Grid4 {
  dim3 grid;
  int64_t groups;
};

// Blocks per chain: enough to fill the GPU about eight times over with all
// chains together, and no more -- the threads then stride over their chain's
// parameters, so per-chain reductions (kinetic energies) take one atomic
// per block rather than one per warp.
Grid4 grid4(int chains, int64_t P) {
  Grid4 g;
  g.groups = (P + 3) / 4;
  int64_t bx = (g.groups + kThreads - 1) / kThreads;
  const int64_t fill = std::max<int64_t>(4, (152 * 8 + chains - 1) / std::max(chains, 1));
  bx = std::min<int64_t>(std::min<int64_t>(bx, fill), 65535);
  g.grid = dim3(static_cast<unsigned>(std::max<int64_t>(bx, 1)),
                static_cast<unsigned>(chains));
  return g;
}

__device__ __forceinline__ float mass_inv(const float* m, int64_t j) {
  return m != nullptr ? 1.0f / __ldg(m + j) : 1.0f;
}
__device__ __forceinline__ float mass_sqrt(const float* m, int64_t j) {
  return m != nullptr ? sqrtf(__ldg(m + j)) : 1.0f;
}

// Optional fusions of an update (see UpdateFusion): the prior term added to
// the gradient, a BF16 mirror of the new positions and per-block sums of
// their squares.
struct Fuse {
  float pf;
  uint32_t* mirror;  // BF16 pairs
  int64_t mcount, mstride;
  double* sq;
  const int32_t* ident;  // noise chain of each row, or null
};

Fuse to_fuse(const UpdateFusion* f) {
  Fuse r{0.f, nullptr, 0, 0, nullptr, nullptr};
  if (f != nullptr) {
    r.pf = f->prior_pf;
    r.mirror = static_cast<uint32_t*>(f->mirror);
    r.mcount = f->mirror_count;
    r.mstride = f->mirror_stride;
    r.sq = f->sq_parts;
    r.ident = f->ident;
  }
  return r;
}

// New positions xn[0..3] of parameters j0..j0+3 of chain c (j < P valid).
__device__ __forceinline__ void fuse_store(const Fuse& f, int c, int64_t j0, int64_t P,
                                           const float (&xn)[4], float& sq) {
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (j0 + e < P) sq = fmaf(xn[e], xn[e], sq);
  if (f.mirror != nullptr && j0 < f.mcount) {  // mcount % 4 == 0: whole groups
    const __nv_bfloat162 a = __floats2bfloat162_rn(xn[0], xn[1]);
    const __nv_bfloat162 b = __floats2bfloat162_rn(xn[2], xn[3]);
    uint2 w;
    w.x = *reinterpret_cast<const uint32_t*>(&a);
    w.y = *reinterpret_cast<const uint32_t*>(&b);
    *reinterpret_cast<uint2*>(f.mirror + (static_cast<int64_t>(c) * f.mstride + j0) / 2) = w;
  }
}

__device__ __forceinline__ void fuse_finish(const Fuse& f, int c, float sq) {
  if (f.sq == nullptr) return;
  __shared__ double red[32];
  const double tot = block_sum(static_cast<double>(sq), red);
  if (threadIdx.x == 0) f.sq[static_cast<int64_t>(c) * gridDim.x + blockIdx.x] = tot;
}

// The 4 parameters j0..j0+3 of a chain row (those below P): all loads of a
// group are issued before any store, so they overlap.
__device__ __forceinline__ void load4(const float* __restrict__ a, int64_t j0, int64_t P,
                                      float (&v)[4]) {
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = j0 + e < P ? a[j0 + e] : 0.f;
}
__device__ __forceinline__ void store4(float* __restrict__ a, int64_t j0, int64_t P,
                                       const float (&v)[4]) {
#pragma unroll
  for (int e = 0; e < 4; ++e)
    if (j0 + e < P) a[j0 + e] = v[e];
}

__global__ void mirror_kernel(int64_t P, const float* x, Fuse f) {
  const int c = blockIdx.y;
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float sq = 0.f;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float xn[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) xn[e] = 4 * q + e < P ? x[off + 4 * q + e] : 0.f;
    fuse_store(f, c, 4 * q, P, xn, sq);
  }
  fuse_finish(f, c, sq);
}

// Four resident blocks per SM (64 registers instead of 72): more loads in
// flight for this memory-bound stream (measured 1 % faster in the reSGLD
// plan; the OBABO kernels measured no gain from the same bound).
__global__ void __launch_bounds__(kThreads, 4)
sgld_update_kernel(int chains, int64_t P, float* x, const float* g, float* v, float alpha,
                   float lmbd, Sched sched, Noise noise, float* samples, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float T = sched.temperature(k, c);
  const int slot = sched.keep_slot(k);
  const float noise_scale = sqrtf(2.0f * T * h);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float sq = 0.f;
  float* __restrict__ xc = x + off;
  const float* __restrict__ gc = g + off;
  float* __restrict__ vc = v != nullptr ? v + off : nullptr;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j0 = 4 * q;
    float xv[4], gv[4], vv[4] = {0.f, 0.f, 0.f, 0.f}, xi[4];
    load4(xc, j0, P, xv);
    load4(gc, j0, P, gv);
    if (vc != nullptr) load4(vc, j0, P, vv);
    noise4(noise, fz.ident != nullptr ? __ldg(fz.ident + c) : c, j0, P, k, GBSGMC_TAG_SGLD, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float gj = fz.pf != 0.f ? fmaf(fz.pf, xv[e], gv[e]) : gv[e];
      const float scaled_gradient = -h * gj;
      const float scaled_noise = noise_scale * xi[e];
      if (vc != nullptr) {
        const float vn = alpha * vv[e] + (1.0f - alpha) * (gj * gj);
        const float G = 1.0f / (lmbd + sqrtf(vn));
        vv[e] = vn;
        xv[e] = xv[e] + ((0.0f + G * scaled_gradient) + sqrtf(G) * scaled_noise);
      } else {
        xv[e] = xv[e] + (scaled_gradient + scaled_noise);
      }
    }
    if (vc != nullptr) store4(vc, j0, P, vv);
    store4(xc, j0, P, xv);
    if (slot >= 0)
      store4(samples + (static_cast<int64_t>(slot) * chains + c) * P, j0, P, xv);
    fuse_store(fz, c, j0, P, xv, sq);
  }
  fuse_finish(fz, c, sq);
}

// Per-thread kinetic-energy partials are fp32; the block sum and the
// accumulation across blocks are fp64, one atomic per block.
__device__ __forceinline__ void add_ke(double* ke, int c, float part) {
  if (ke == nullptr) return;
  __shared__ double red[32];
  const double tot = block_sum(static_cast<double>(part), red);
  if (threadIdx.x == 0) atomicAdd(ke + c, tot);
}

// The OBABO halves of one parameter (integrator.py:192-273), with every
// rounding spelled out (__fmaf_rn / __fmul_rn) so that the separate kernels
// and the fused second-then-first kernel compute the same bits.
struct ObaboCoef {
  float h, keep, inject, half;
};
__device__ __forceinline__ ObaboCoef obabo_coef(const Sched& sched, int64_t k, int c,
                                                float friction) {
  ObaboCoef q;
  q.h = sched.step_size(k);
  const float T = sched.temperature(k, c);
  const float permanence = expf(-friction * q.h);
  q.keep = sqrtf(permanence);
  q.inject = sqrtf((1.0f - permanence) * T);
  q.half = 0.5f * q.h;
  return q;
}
// O, kinetic energy, B, A: p, x updated, ke accumulates.
__device__ __forceinline__ void obabo_first_elem(const ObaboCoef& q, float mi, float ms,
                                                 float g, float xi, float& p, float& x,
                                                 float& ke) {
  float pj = __fmaf_rn(q.keep, p, __fmul_rn(q.inject, __fmul_rn(ms, xi)));
  ke = __fmaf_rn(__fmul_rn(0.5f, pj), __fmul_rn(mi, pj), ke);
  pj = __fmaf_rn(-q.half, g, pj);
  p = pj;
  x = __fmaf_rn(q.h, __fmul_rn(mi, pj), x);
}
// B, kinetic energy, O: p updated, ke accumulates.
__device__ __forceinline__ void obabo_second_elem(const ObaboCoef& q, float mi, float ms,
                                                  float g, float xi, float& p, float& ke) {
  const float pj = __fmaf_rn(-q.half, g, p);
  ke = __fmaf_rn(__fmul_rn(0.5f, pj), __fmul_rn(mi, pj), ke);
  p = __fmaf_rn(q.keep, pj, __fmul_rn(q.inject, __fmul_rn(ms, xi)));
}

__global__ void obabo_first_kernel(
    int chains, int64_t P, float* x, float* p, const float* g1, const float* mass,
    float friction, double* ke_start, Sched sched, Noise noise, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const ObaboCoef qc = obabo_coef(sched, k, c, friction);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float ke = 0.0f, sq = 0.0f;
  float* __restrict__ xc = x + off;
  float* __restrict__ pc = p + off;
  const float* __restrict__ gc = g1 + off;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j0 = 4 * q;
    float xv[4], pv[4], gv[4], xi[4];
    load4(xc, j0, P, xv);
    load4(pc, j0, P, pv);
    load4(gc, j0, P, gv);
    noise4(noise, c, j0, P, k, GBSGMC_TAG_OBABO_1, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (j0 + e >= P) break;
      const float gj = fz.pf != 0.f ? __fmaf_rn(fz.pf, xv[e], gv[e]) : gv[e];
      obabo_first_elem(qc, mass_inv(mass, j0 + e), mass_sqrt(mass, j0 + e), gj, xi[e],
                       pv[e], xv[e], ke);
    }
    store4(pc, j0, P, pv);
    store4(xc, j0, P, xv);
    fuse_store(fz, c, j0, P, xv, sq);
  }
  add_ke(ke_start, c, ke);
  fuse_finish(fz, c, sq);
}

__global__ void obabo_second_kernel(
    int chains, int64_t P, const float* x, float* p, const float* g2, const float* mass,
    float friction, double* ke_end, Sched sched, Noise noise, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const ObaboCoef qc = obabo_coef(sched, k, c, friction);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float ke = 0.0f;
  float* __restrict__ pc = p + off;
  const float* __restrict__ gc = g2 + off;
  const float* __restrict__ xc = fz.pf != 0.f ? x + off : nullptr;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j0 = 4 * q;
    float pv[4], gv[4], xv[4] = {0.f, 0.f, 0.f, 0.f}, xi[4];
    load4(pc, j0, P, pv);
    load4(gc, j0, P, gv);
    if (xc != nullptr) load4(xc, j0, P, xv);
    noise4(noise, c, j0, P, k, GBSGMC_TAG_OBABO_2, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (j0 + e >= P) break;
      const float gj = xc != nullptr ? __fmaf_rn(fz.pf, xv[e], gv[e]) : gv[e];
      obabo_second_elem(qc, mass_inv(mass, j0 + e), mass_sqrt(mass, j0 + e), gj, xi[e],
                        pv[e], ke);
    }
    store4(pc, j0, P, pv);
  }
  add_ke(ke_end, c, ke);
}

// The second half of step k and the first half of step k + 1 in one pass
// (their gradients g2 of step k and g1 of step k + 1 are both taken at the
// same positions): per parameter exactly the operations of
// obabo_second_kernel (step k) then obabo_first_kernel (step k + 1).
__global__ void obabo_second_first_kernel(
    int chains, int64_t P, float* x, float* p, const float* g2, const float* g1,
    const float* mass, float friction, double* ke_end, double* ke_start, Sched sched,
    Noise noise, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const ObaboCoef q2 = obabo_coef(sched, k, c, friction);
  const ObaboCoef q1 = obabo_coef(sched, k + 1, c, friction);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float ke2 = 0.0f, ke1 = 0.0f, sq = 0.0f;
  float* __restrict__ xc = x + off;
  float* __restrict__ pc = p + off;
  const float* __restrict__ g2c = g2 + off;
  const float* __restrict__ g1c = g1 + off;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t j0 = 4 * q;
    float xv[4], pv[4], gv2[4], gv1[4], xi2[4], xi1[4];
    load4(xc, j0, P, xv);
    load4(pc, j0, P, pv);
    load4(g2c, j0, P, gv2);
    load4(g1c, j0, P, gv1);
    noise4(noise, c, j0, P, k, GBSGMC_TAG_OBABO_2, xi2);
    noise4(noise, c, j0, P, k + 1, GBSGMC_TAG_OBABO_1, xi1);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if (j0 + e >= P) break;
      const float mi = mass_inv(mass, j0 + e), ms = mass_sqrt(mass, j0 + e);
      const float ga = fz.pf != 0.f ? __fmaf_rn(fz.pf, xv[e], gv2[e]) : gv2[e];
      obabo_second_elem(q2, mi, ms, ga, xi2[e], pv[e], ke2);
      const float gb = fz.pf != 0.f ? __fmaf_rn(fz.pf, xv[e], gv1[e]) : gv1[e];
      obabo_first_elem(q1, mi, ms, gb, xi1[e], pv[e], xv[e], ke1);
    }
    store4(pc, j0, P, pv);
    store4(xc, j0, P, xv);
    fuse_store(fz, c, j0, P, xv, sq);
  }
  add_ke(ke_end, c, ke2);
  add_ke(ke_start, c, ke1);
  fuse_finish(fz, c, sq);
}

__global__ void sghmc_resample_kernel(int chains, int64_t P, float* p,
                                      const float* mass, Sched sched,
                                      Noise noise) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float xi[4];
    noise4(noise, c, 4 * q, P, k, GBSGMC_TAG_SGHMC_RESAMPLE, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t j = 4 * q + e;
      if (j >= P) break;
      p[off + j] = mass_sqrt(mass, j) * xi[e];
    }
  }
}

__global__ void sghmc_position_kernel(int chains, int64_t P, float* x,
                                      float* p, const float* mass,
                                      const float* fric, float friction,
                                      Sched sched, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float sq = 0.f;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float xs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t j = 4 * q + e;
      if (j >= P) break;
      const float f = fric != nullptr ? __ldg(fric + j) : friction;
      const float pj = p[off + j];
      const float sm = mass_inv(mass, j) * pj;
      xs[e] = x[off + j] + h * sm;
      x[off + j] = xs[e];
      p[off + j] = pj + (-h * f) * sm;
    }
    fuse_store(fz, c, 4 * q, P, xs, sq);
  }
  fuse_finish(fz, c, sq);
}

__global__ void sghmc_momentum_kernel(int chains, int64_t P, const float* x, float* p,
                                      const float* g, const float* fric,
                                      float friction, Sched sched,
                                      Noise noise, Fuse fz) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float noise_scale = sqrtf(2.0f * h);
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
      const float f = fric != nullptr ? __ldg(fric + j) : friction;
      const float gj = fz.pf != 0.f ? fmaf(fz.pf, x[off + j], g[off + j]) : g[off + j];
      float pj = p[off + j] + (-h) * gj;
      pj = pj + f * (noise_scale * xi[e]);
      p[off + j] = pj;
    }
  }
}

// Uniform in (0, 1) with 53 random bits from Philox (seed, counter (pair,
// step, 0, GBSGMC_TAG_SWAP)).
__device__ __forceinline__ double swap_uniform(uint64_t seed, uint32_t pair, uint32_t step) {
  const U32x4 r = philox4x32_10(U32x4{pair, step, 0u, GBSGMC_TAG_SWAP},
                                static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
  const uint64_t bits = ((static_cast<uint64_t>(r.x) >> 5) << 26) |
                        (static_cast<uint64_t>(r.y) >> 6);
  return (static_cast<double>(bits) + 0.5) * (1.0 / 9007199254740992.0);
}

__global__ void resgld_swap_kernel(int pairs, const double* Un,
                                   const double* Uh, const double* var_n,
                                   const double* Tn, const double* Th,
                                   double F, double* ssq, int64_t* kc,
                                   const double* u_in, uint64_t seed,
                                   int64_t step, double* log_s_out,
                                   int32_t* perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pairs) return;
  const int64_t k = kc[i] + 1;
  kc[i] = k;
  const double sa = 1.0 / static_cast<double>(k);
  const double s2 = (1.0 - sa) * ssq[i] + sa * var_n[i];
  ssq[i] = s2;
  const double dbeta = 1.0 / Tn[i] - 1.0 / Th[i];
  const double correction = dbeta * s2 / F;
  const double log_s = dbeta * (Un[i] - Uh[i] - correction);
  const double u = u_in != nullptr
                       ? u_in[i]
                       : swap_uniform(seed, static_cast<uint32_t>(i), static_cast<uint32_t>(step));
  if (log_s_out != nullptr) log_s_out[i] = log_s;
  perm[i] = (log(u) < log_s) ? 0 : 1;
}

// One CTA per (normal, hot) pair: the decision of resgld_swap_kernel at the
// pair's own counter k, the swap of the pair's slots, then the kept sample
// of the normal slot.
__global__ void resgld_pairs_kernel(int pairs, int d, float* x, float* v, double* U,
                                    double* var, int32_t* ident, Sched sched, double F,
                                    uint64_t seed, const int32_t* pair_chain, double* ssq,
                                    int64_t* kc, int32_t* counts, float* samples,
                                    double* sample_lik) {
  const int p = blockIdx.x;
  const int sn = p, sh = pairs + p;
  const int64_t k = sched.step();
  __shared__ int swapped;
  if (threadIdx.x == 0) {
    const int64_t kk = kc[p] + 1;
    kc[p] = kk;
    const double sa = 1.0 / static_cast<double>(kk);
    const double s2 = (1.0 - sa) * ssq[p] + sa * var[sn];
    ssq[p] = s2;
    const double Tn = sched.temperature(k, sn), Th = sched.temperature(k, sh);
    const double dbeta = 1.0 / Tn - 1.0 / Th;
    const double log_s = dbeta * (U[sn] - U[sh] - dbeta * s2 / F);
    const uint64_t key = (seed << 32) | static_cast<uint32_t>(__ldg(pair_chain + p));
    const double u = swap_uniform(key, 0u, static_cast<uint32_t>(k + 1));
    // The reference keeps the pair when log u < log s (lax.cond true branch).
    const int sw = (log(u) < log_s) ? 0 : 1;
    swapped = sw;
    if (sw) {
      double t = U[sn];
      U[sn] = U[sh];
      U[sh] = t;
      t = var[sn];
      var[sn] = var[sh];
      var[sh] = t;
      const int32_t i = ident[sn];
      ident[sn] = ident[sh];
      ident[sh] = i;
      if (counts != nullptr) counts[p] += 1;
    }
  }
  __syncthreads();
  float* xn = x + static_cast<int64_t>(sn) * d;
  float* xh = x + static_cast<int64_t>(sh) * d;
  if (swapped) {
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
      const float t = xn[j];
      xn[j] = xh[j];
      xh[j] = t;
      if (v != nullptr) {
        float* vn = v + static_cast<int64_t>(sn) * d;
        float* vh = v + static_cast<int64_t>(sh) * d;
        const float tv = vn[j];
        vn[j] = vh[j];
        vh[j] = tv;
      }
    }
  }
  const int slot = sched.keep_slot(k);
  if (slot >= 0) {
    float* dst = samples + (static_cast<int64_t>(slot) * pairs + p) * d;
    for (int j = threadIdx.x; j < d; j += blockDim.x) dst[j] = xn[j];
    if (threadIdx.x == 0 && sample_lik != nullptr)
      sample_lik[static_cast<int64_t>(slot) * pairs + p] = -U[sn];
  }
}

__global__ void swap_rows_kernel(int pairs, int64_t width, float* a, float* b,
                                 const int32_t* perm) {
  const int i = blockIdx.y;
  if (perm[i] == 0) return;
  const int64_t off = static_cast<int64_t>(i) * width;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       j < width; j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float t = a[off + j];
    a[off + j] = b[off + j];
    b[off + j] = t;
  }
}

// Stochastic-approximation update of the adjacent-pair variance estimates
// (one block): k += 1, ssq[r] = (1 - 1/k) ssq[r] + (1/k) var[r].
__global__ void resgld_sa_kernel(int replicas, const double* var, double* ssq, int64_t* kc) {
  const int64_t k = kc[0] + 1;
  __syncthreads();
  if (threadIdx.x == 0) kc[0] = k;
  const double sa = 1.0 / static_cast<double>(k);
  for (int r = threadIdx.x; r < replicas - 1; r += blockDim.x)
    ssq[r] = (1.0 - sa) * ssq[r] + sa * var[r];
}

// Exchange decisions between adjacent replicas (r, r + 1) at step k, for the
// pairs r = parity, parity + 2, ... with parity = round & 1, round =
// (k + 1) / every.  Replica r runs at T(k, r) = t_k f_r (the schedule's
// per-chain temperature).  The rule of solver.py:273-291 per pair, in FP64;
// a pair that exchanges swaps its U and var here and its rows in
// swap_adjacent_rows_kernel.
__global__ void resgld_decide_kernel(int replicas, Sched sched, int every, double* U,
                                     double* var, const double* ssq, double F, uint64_t seed,
                                     const double* u_in, int32_t* flags, int32_t* counts,
                                     double* log_s_out) {
  const int64_t k = sched.step();
  const int64_t round = (k + 1) / every;
  const int parity = static_cast<int>(round & 1);
  for (int r = threadIdx.x; r < replicas - 1; r += blockDim.x) {
    int swapped = 0;
    if ((r & 1) == parity) {
      const double Tn = sched.temperature(k, r), Th = sched.temperature(k, r + 1);
      const double dbeta = 1.0 / Tn - 1.0 / Th;
      const double log_s = dbeta * (U[r] - U[r + 1] - dbeta * ssq[r] / F);
      const double u = u_in != nullptr
                           ? u_in[r]
                           : swap_uniform(seed, static_cast<uint32_t>(r),
                                          static_cast<uint32_t>(round));
      // The reference keeps the pair when log u < log s (lax.cond true branch).
      swapped = (log(u) < log_s) ? 0 : 1;
      if (log_s_out != nullptr) log_s_out[r] = log_s;
    }
    flags[r] = swapped;
  }
  __syncthreads();
  // Pairs of one parity are disjoint, so the swaps do not interfere.
  for (int r = threadIdx.x; r < replicas - 1; r += blockDim.x) {
    if (flags[r] == 0) continue;
    double t = U[r];
    U[r] = U[r + 1];
    U[r + 1] = t;
    if (var != nullptr) {
      t = var[r];
      var[r] = var[r + 1];
      var[r + 1] = t;
    }
    if (counts != nullptr) counts[r] += 1;
  }
}

__global__ void swap_adjacent_rows_kernel(int64_t width, float* a, const int32_t* flags) {
  const int r = blockIdx.y;
  if (flags[r] == 0) return;
  float* x = a + static_cast<int64_t>(r) * width;
  float* y = x + width;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < width;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const float t = x[j];
    x[j] = y[j];
    y[j] = t;
  }
}

// ---------------------------------------------------------------------------
// Reversible leapfrog (AMAGOLD) and Metropolis-Hastings corrections.
// ---------------------------------------------------------------------------

// x <- x + (scale h) p / m at the schedule's step.
__global__ void leapfrog_position_kernel(int chains, int64_t P, float* x, const float* p,
                                         const float* mass, float scale, Sched sched) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float s = scale * sched.step_size(k);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t j = 4 * q + e;
      if (j >= P) break;
      const float sm = mass_inv(mass, j) * p[off + j];
      x[off + j] = x[off + j] + s * sm;
    }
  }
}

// One momentum step of the reversible leapfrog, with the noise of tag
// GBSGMC_TAG_AMAGOLD at the schedule's step:
//   p' = ((1 - h f) p - h g + sqrt(4 f h) sqrt(m) xi) / (1 + h f)
// and energy[c] += 0.5 h sum_j (p_j + p'_j) g_j / m_j.
__global__ void amagold_momentum_kernel(int chains, int64_t P, float* p, const float* g,
                                        const float* mass, float friction, double* energy,
                                        Sched sched, Noise noise) {
  const int c = blockIdx.y;
  const int64_t k = sched.step();
  const float h = sched.step_size(k);
  const float decay = 1.0f - h * friction;
  const float inv = 1.0f / (1.0f + h * friction);
  const float ns = sqrtf(4.0f * friction * h);
  const int64_t groups = (P + 3) / 4;
  const int64_t off = static_cast<int64_t>(c) * P;
  float part = 0.f;
  for (int64_t q = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       q < groups; q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float xi[4];
    noise4(noise, c, 4 * q, P, k, GBSGMC_TAG_AMAGOLD, xi);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int64_t j = 4 * q + e;
      if (j >= P) break;
      const float pj = p[off + j], gj = g[off + j];
      const float noise_j = ns * (mass_sqrt(mass, j) * xi[e]);
      const float pn = inv * ((decay * pj + (-h) * gj) + noise_j);
      p[off + j] = pn;
      part += (pj + pn) * (mass_inv(mass, j) * gj);
    }
  }
  add_ke(energy, c, 0.5f * h * part);
}

// The MH decision of chain c in FP64:
//   AMAGOLD (kind 0): log a = U_old - U_new + energy
//   SGGMC   (kind 1): log a = -(U_new - U_old + ke_end - ke_start) / T_k
// capped at 0 as the reference caps it (AMAGOLD keeps a NaN, SGGMC maps it
// to 0); the proposal is accepted when log u < log a, u from Philox (seed,
// counter (chain_base + c, step, 0, GBSGMC_TAG_MH)) or u_dev[c].  Writes
// accept[c], ratio[c] = exp(log a) and the potential the chain keeps.
__global__ void mh_accept_kernel(int chains, int kind, const double* U_old,
                                 const double* U_new, const double* energy,
                                 const double* ke_start, const double* ke_end, Sched sched,
                                 const double* u_in, uint64_t seed, int chain_base,
                                 int32_t* accept, double* ratio, double* U_keep) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= chains) return;
  const int64_t k = sched.step();
  double la;
  if (kind == 0) {
    la = U_old[c] - U_new[c] + energy[c];
    la = la > 0.0 ? 0.0 : la;
  } else {
    const double T = static_cast<double>(sched.temperature(k, c));
    la = -1.0 / T * (U_new[c] - U_old[c] + ke_end[c] - ke_start[c]);
    la = la <= 0.0 ? la : 0.0;
  }
  double u;
  if (u_in != nullptr) {
    u = u_in[c];
  } else {
    const U32x4 r = philox4x32_10(
        U32x4{static_cast<uint32_t>(chain_base + c), static_cast<uint32_t>(k), 0u,
              GBSGMC_TAG_MH},
        static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint64_t bits = ((static_cast<uint64_t>(r.x) >> 5) << 26) |
                          (static_cast<uint64_t>(r.y) >> 6);
    u = (static_cast<double>(bits) + 0.5) * (1.0 / 9007199254740992.0);
  }
  const int acc = log(u) < la ? 1 : 0;
  accept[c] = acc;
  if (ratio != nullptr) ratio[c] = exp(la);
  if (U_keep != nullptr) U_keep[c] = acc ? U_new[c] : U_old[c];
}

// Rejected chains go back to (x_old, sign * p_old); accepted ones keep the
// proposal in x, p.
__global__ void mh_select_kernel(int chains, int64_t P, const int32_t* accept, float* x,
                                 const float* x_old, float* p, const float* p_old,
                                 float sign) {
  const int c = blockIdx.y;
  if (accept[c]) return;
  const int64_t off = static_cast<int64_t>(c) * P;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < P;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    x[off + j] = x_old[off + j];
    if (p != nullptr) p[off + j] = sign * p_old[off + j];
  }
}

int check_ec(int chains, int64_t P, const char* what) {
  if (chains < 0 || P < 0 || chains > 65535)
    return set_error(GBSGMC_ERR_ARG, "%s: bad chains/P", what);
  return GBSGMC_OK;
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int gbsgmc_sgld_update(int chains, int64_t P, float* x_dev,
                                  const float* g_dev, float* v_dev,
                                  float alpha, float lmbd,
                                  const gbsgmc_sched* sched,
                                  const gbsgmc_noise* noise,
                                  float* samples_dev, gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "sgld_update");
  if (rc) return rc;
  if (!x_dev || !g_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "sgld_update: null pointer");
  if (sched->keep_slot_dev && !samples_dev)
    return set_error(GBSGMC_ERR_ARG, "sgld_update: keep table without samples");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  sgld_update_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, x_dev, g_dev, v_dev, alpha, lmbd, to_sched(sched),
      to_noise(noise), samples_dev, to_fuse(nullptr));
  return check_launch("sgld_update");
}

extern "C" int gbsgmc_obabo_first(int chains, int64_t P, float* x_dev,
                                  float* p_dev, const float* g1_dev,
                                  const float* mass_dev, float friction,
                                  double* ke_start_dev,
                                  const gbsgmc_sched* sched,
                                  const gbsgmc_noise* noise,
                                  gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "obabo_first");
  if (rc) return rc;
  if (!x_dev || !p_dev || !g1_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "obabo_first: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  obabo_first_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, x_dev, p_dev, g1_dev, mass_dev, friction, ke_start_dev,
      to_sched(sched), to_noise(noise), to_fuse(nullptr));
  return check_launch("obabo_first");
}

extern "C" int gbsgmc_obabo_second(int chains, int64_t P, float* p_dev,
                                   const float* g2_dev, const float* mass_dev,
                                   float friction, double* ke_end_dev,
                                   const gbsgmc_sched* sched,
                                   const gbsgmc_noise* noise,
                                   gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "obabo_second");
  if (rc) return rc;
  if (!p_dev || !g2_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "obabo_second: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  obabo_second_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, nullptr, p_dev, g2_dev, mass_dev, friction, ke_end_dev,
      to_sched(sched), to_noise(noise), to_fuse(nullptr));
  return check_launch("obabo_second");
}

extern "C" int gbsgmc_sghmc_resample(int chains, int64_t P, float* p_dev,
                                     const float* mass_dev,
                                     const gbsgmc_sched* sched,
                                     const gbsgmc_noise* noise,
                                     gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "sghmc_resample");
  if (rc) return rc;
  if (!p_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "sghmc_resample: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  sghmc_resample_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, p_dev, mass_dev, to_sched(sched), to_noise(noise));
  return check_launch("sghmc_resample");
}

extern "C" int gbsgmc_sghmc_position(int chains, int64_t P, float* x_dev,
                                     float* p_dev, const float* mass_dev,
                                     const float* friction_dev, float friction,
                                     const gbsgmc_sched* sched,
                                     gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "sghmc_position");
  if (rc) return rc;
  if (!x_dev || !p_dev || !sched)
    return set_error(GBSGMC_ERR_ARG, "sghmc_position: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  sghmc_position_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, x_dev, p_dev, mass_dev, friction_dev, friction,
      to_sched(sched), to_fuse(nullptr));
  return check_launch("sghmc_position");
}

extern "C" int gbsgmc_sghmc_momentum(int chains, int64_t P, float* p_dev,
                                     const float* g_dev,
                                     const float* friction_dev, float friction,
                                     const gbsgmc_sched* sched,
                                     const gbsgmc_noise* noise,
                                     gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "sghmc_momentum");
  if (rc) return rc;
  if (!p_dev || !g_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "sghmc_momentum: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  sghmc_momentum_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, nullptr, p_dev, g_dev, friction_dev, friction, to_sched(sched),
      to_noise(noise), to_fuse(nullptr));
  return check_launch("sghmc_momentum");
}

extern "C" int gbsgmc_leapfrog_position(int chains, int64_t P, float* x_dev,
                                        const float* p_dev, const float* mass_dev,
                                        float scale, const gbsgmc_sched* sched,
                                        gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "leapfrog_position");
  if (rc) return rc;
  if (!x_dev || !p_dev || !sched)
    return set_error(GBSGMC_ERR_ARG, "leapfrog_position: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  leapfrog_position_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, x_dev, p_dev, mass_dev, scale, to_sched(sched));
  return check_launch("leapfrog_position");
}

extern "C" int gbsgmc_amagold_momentum(int chains, int64_t P, float* p_dev,
                                       const float* g_dev, const float* mass_dev,
                                       float friction, double* energy_dev,
                                       const gbsgmc_sched* sched,
                                       const gbsgmc_noise* noise,
                                       gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "amagold_momentum");
  if (rc) return rc;
  if (!p_dev || !g_dev || !sched || !noise)
    return set_error(GBSGMC_ERR_ARG, "amagold_momentum: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, P);
  amagold_momentum_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, p_dev, g_dev, mass_dev, friction, energy_dev, to_sched(sched),
      to_noise(noise));
  return check_launch("amagold_momentum");
}

extern "C" int gbsgmc_mh_accept(int chains, int kind, const double* U_old_dev,
                                const double* U_new_dev, const double* energy_dev,
                                const double* ke_start_dev, const double* ke_end_dev,
                                const gbsgmc_sched* sched, const double* u_dev,
                                uint64_t seed, int chain_base, int32_t* accept_dev,
                                double* ratio_dev, double* U_keep_dev,
                                gbsgmc_stream_t stream) {
  if (chains < 0 || (kind != GBSGMC_MH_AMAGOLD && kind != GBSGMC_MH_SGGMC))
    return set_error(GBSGMC_ERR_ARG, "mh_accept: bad chains or kind");
  if (!U_old_dev || !U_new_dev || !sched || !accept_dev ||
      (kind == GBSGMC_MH_AMAGOLD && !energy_dev) ||
      (kind == GBSGMC_MH_SGGMC && (!ke_start_dev || !ke_end_dev)))
    return set_error(GBSGMC_ERR_ARG, "mh_accept: null pointer");
  if (chains == 0) return GBSGMC_OK;
  mh_accept_kernel<<<(chains + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, kind, U_old_dev, U_new_dev, energy_dev, ke_start_dev, ke_end_dev,
      to_sched(sched), u_dev, seed, chain_base, accept_dev, ratio_dev, U_keep_dev);
  return check_launch("mh_accept");
}

extern "C" int gbsgmc_mh_select(int chains, int64_t P, const int32_t* accept_dev,
                                float* x_dev, const float* x_old_dev, float* p_dev,
                                const float* p_old_dev, float reject_momentum_sign,
                                gbsgmc_stream_t stream) {
  int rc = check_ec(chains, P, "mh_select");
  if (rc) return rc;
  if (!accept_dev || !x_dev || !x_old_dev || (p_dev != nullptr && p_old_dev == nullptr))
    return set_error(GBSGMC_ERR_ARG, "mh_select: null pointer");
  if (chains == 0 || P == 0) return GBSGMC_OK;
  const Grid4 g = grid4(chains, (P + 3) / 4 * 4);
  mh_select_kernel<<<g.grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      chains, P, accept_dev, x_dev, x_old_dev, p_dev, p_old_dev, reject_momentum_sign);
  return check_launch("mh_select");
}

extern "C" int gbsgmc_resgld_swap_f64(
    int pairs, const double* U_normal_dev, const double* U_hot_dev,
    const double* var_normal_dev, const double* T_normal_dev,
    const double* T_hot_dev, double F, double* ssq_dev, int64_t* k_dev,
    const double* u_dev, uint64_t seed, int64_t step, double* log_s_dev,
    int32_t* perm_dev, gbsgmc_stream_t stream) {
  if (pairs < 0) return set_error(GBSGMC_ERR_ARG, "resgld_swap: pairs < 0");
  if (pairs == 0) return GBSGMC_OK;
  if (!U_normal_dev || !U_hot_dev || !var_normal_dev || !T_normal_dev ||
      !T_hot_dev || !ssq_dev || !k_dev || !perm_dev)
    return set_error(GBSGMC_ERR_ARG, "resgld_swap: null pointer");
  if (!(F != 0.0)) return set_error(GBSGMC_ERR_ARG, "resgld_swap: F == 0");
  resgld_swap_kernel<<<(pairs + 127) / 128, 128, 0,
                       static_cast<cudaStream_t>(stream)>>>(
      pairs, U_normal_dev, U_hot_dev, var_normal_dev, T_normal_dev, T_hot_dev,
      F, ssq_dev, k_dev, u_dev, seed, step, log_s_dev, perm_dev);
  return check_launch("resgld_swap");
}

namespace gbsgmc {

int resgld_pairs_exchange(int pairs, int d, float* x, float* v, double* U,
                          double* var, int32_t* ident, const gbsgmc_sched* sched,
                          double F, uint64_t seed, const int32_t* pair_chain,
                          double* ssq, int64_t* k, int32_t* counts, float* samples,
                          double* sample_lik, cudaStream_t stream) {
  if (pairs <= 0 || d <= 0) return GBSGMC_OK;
  if (sched->keep_slot_dev != nullptr && samples == nullptr)
    return set_error(GBSGMC_ERR_ARG, "resgld pairs: keep table without sample buffer");
  resgld_pairs_kernel<<<pairs, 128, 0, stream>>>(pairs, d, x, v, U, var, ident,
                                                 to_sched(sched), F, seed, pair_chain, ssq,
                                                 k, counts, samples, sample_lik);
  return check_launch("resgld_pairs");
}

}  // namespace gbsgmc

extern "C" int gbsgmc_swap_rows(int pairs, int64_t width, float* a_dev,
                                float* b_dev, const int32_t* perm_dev,
                                gbsgmc_stream_t stream) {
  if (pairs < 0 || width < 0 || pairs > 65535)
    return set_error(GBSGMC_ERR_ARG, "swap_rows: bad size");
  if (pairs == 0 || width == 0) return GBSGMC_OK;
  if (!a_dev || !b_dev || !perm_dev)
    return set_error(GBSGMC_ERR_ARG, "swap_rows: null pointer");
  int64_t bx = std::min<int64_t>((width + kThreads - 1) / kThreads, 4096);
  dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(pairs));
  swap_rows_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      pairs, width, a_dev, b_dev, perm_dev);
  return check_launch("swap_rows");
}

extern "C" int gbsgmc_resgld_sa_update(int replicas, const double* lk_var_dev, double* ssq_dev,
                                       int64_t* k_dev, gbsgmc_stream_t stream) {
  if (replicas < 2 || replicas > 65536 || lk_var_dev == nullptr || ssq_dev == nullptr ||
      k_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "resgld_sa_update: bad arguments");
  resgld_sa_kernel<<<1, 256, 0, static_cast<cudaStream_t>(stream)>>>(replicas, lk_var_dev,
                                                                     ssq_dev, k_dev);
  return check_launch("resgld_sa_update");
}

extern "C" int gbsgmc_resgld_exchange_adjacent(
    int replicas, int64_t P, float* x_dev, float* v_dev, double* U_dev, double* lk_var_dev,
    const gbsgmc_sched* sched, int every, const double* ssq_dev, double F, uint64_t seed,
    const double* u_dev, int32_t* flags_dev, int32_t* counts_dev, double* log_s_dev,
    gbsgmc_stream_t stream) {
  if (replicas < 2 || replicas > 65536 || P < 0 || x_dev == nullptr || U_dev == nullptr ||
      sched == nullptr || ssq_dev == nullptr || flags_dev == nullptr || every < 1 || !(F > 0))
    return set_error(GBSGMC_ERR_ARG, "resgld_exchange_adjacent: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  resgld_decide_kernel<<<1, 256, 0, st>>>(replicas, to_sched(sched), every, U_dev, lk_var_dev,
                                         ssq_dev, F, seed, u_dev, flags_dev, counts_dev,
                                         log_s_dev);
  int rc = check_launch("resgld_exchange_adjacent: decide");
  if (rc != GBSGMC_OK || P == 0) return rc;
  const int chunks = static_cast<int>(std::min<int64_t>((P + 1023) / 1024, 64));
  dim3 grid(chunks, replicas - 1);
  swap_adjacent_rows_kernel<<<grid, 256, 0, st>>>(P, x_dev, flags_dev);
  if (v_dev != nullptr) swap_adjacent_rows_kernel<<<grid, 256, 0, st>>>(P, v_dev, flags_dev);
  return check_launch("resgld_exchange_adjacent: rows");
}

namespace gbsgmc {

int update_blocks(int chains, int64_t P) { return static_cast<int>(grid4(chains, P).grid.x); }

// At kept steps (the schedule's keep slot >= 0) row 0 of x [., P] is copied to
// samples [slot, P] and -U[0] to sample_lik[slot].
__global__ void keep_row_kernel(int64_t P, const float* __restrict__ x,
                                const double* __restrict__ U, Sched sched, float* samples,
                                double* sample_lik) {
  const int slot = sched.keep_slot(sched.step());
  if (slot < 0) return;
  for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < P;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    samples[static_cast<int64_t>(slot) * P + j] = x[j];
  if (blockIdx.x == 0 && threadIdx.x == 0 && sample_lik != nullptr)
    sample_lik[slot] = -U[0];
}

int keep_row(int64_t P, const float* x, const double* U, const gbsgmc_sched* sched,
             float* samples, double* sample_lik, cudaStream_t st) {
  const int blocks = static_cast<int>(std::min<int64_t>((P + 1023) / 1024, 1024));
  keep_row_kernel<<<blocks, 256, 0, st>>>(P, x, U, to_sched(sched), samples, sample_lik);
  return check_launch("keep_row");
}

int sgld_update_fused(int chains, int64_t P, float* x, const float* g, float* v,
                      float alpha, float lmbd, const gbsgmc_sched* sched,
                      const gbsgmc_noise* noise, const UpdateFusion& f, cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  sgld_update_kernel<<<gr.grid, kThreads, 0, st>>>(chains, P, x, g, v, alpha, lmbd,
                                                   to_sched(sched), to_noise(noise), nullptr,
                                                   to_fuse(&f));
  return check_launch("sgld_update (fused)");
}

int obabo_first_fused(int chains, int64_t P, float* x, float* p, const float* g1,
                      const float* mass, float friction, double* ke_start,
                      const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                      const UpdateFusion& f, cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  obabo_first_kernel<<<gr.grid, kThreads, 0, st>>>(chains, P, x, p, g1, mass, friction,
                                                   ke_start, to_sched(sched), to_noise(noise),
                                                   to_fuse(&f));
  return check_launch("obabo_first (fused)");
}

int obabo_second_fused(int chains, int64_t P, const float* x, float* p, const float* g2,
                       const float* mass, float friction, double* ke_end,
                       const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                       const UpdateFusion& f, cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  obabo_second_kernel<<<gr.grid, kThreads, 0, st>>>(chains, P, x, p, g2, mass, friction,
                                                    ke_end, to_sched(sched), to_noise(noise),
                                                    to_fuse(&f));
  return check_launch("obabo_second (fused)");
}

int obabo_second_first_fused(int chains, int64_t P, float* x, float* p, const float* g2,
                             const float* g1, const float* mass, float friction,
                             double* ke_end, double* ke_start, const gbsgmc_sched* sched,
                             const gbsgmc_noise* noise, const UpdateFusion& f,
                             cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  obabo_second_first_kernel<<<gr.grid, kThreads, 0, st>>>(
      chains, P, x, p, g2, g1, mass, friction, ke_end, ke_start, to_sched(sched),
      to_noise(noise), to_fuse(&f));
  return check_launch("obabo_second_first (fused)");
}

int sghmc_position_fused(int chains, int64_t P, float* x, float* p, const float* mass,
                         float friction, const gbsgmc_sched* sched, const UpdateFusion& f,
                         cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  sghmc_position_kernel<<<gr.grid, kThreads, 0, st>>>(chains, P, x, p, mass, nullptr,
                                                      friction, to_sched(sched), to_fuse(&f));
  return check_launch("sghmc_position (fused)");
}

int sghmc_momentum_fused(int chains, int64_t P, const float* x, float* p, const float* g,
                         float friction, const gbsgmc_sched* sched, const gbsgmc_noise* noise,
                         const UpdateFusion& f, cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  sghmc_momentum_kernel<<<gr.grid, kThreads, 0, st>>>(chains, P, x, p, g, nullptr, friction,
                                                      to_sched(sched), to_noise(noise),
                                                      to_fuse(&f));
  return check_launch("sghmc_momentum (fused)");
}

int mirror_fused(int chains, int64_t P, const float* x, const UpdateFusion& f,
                 cudaStream_t st) {
  const Grid4 gr = grid4(chains, P);
  mirror_kernel<<<gr.grid, kThreads, 0, st>>>(P, x, to_fuse(&f));
  return check_launch("mirror (fused)");
}

}  // namespace gbsgmc
