// Shared device helpers of the gbsgmc kernels: status words, the schedule and
// noise readers, Philox4x32-10 + Box-Muller, 128-bit LCG arithmetic for the
// numpy PCG64 stream, and mbarrier / bulk-copy wrappers with bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbsgmc.h"

namespace gbsgmc {

// ---------------------------------------------------------------------------
// Host-side error reporting (defined in abi.cu).
// ---------------------------------------------------------------------------
int set_error(int code, const char* fmt, ...);
int check_launch(const char* what);

// ---------------------------------------------------------------------------
// Device status word: the first error wins.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void raise_status(int* status, int code) {
  if (status != nullptr) atomicCAS(status, 0, code);
}

// Nanosecond global timer, used to bound every spin-wait.
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A spin-wait gives up after this long and reports GBSGMC_ERR_TIMEOUT.
constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s

// ---------------------------------------------------------------------------
// Schedule and noise readers.
// ---------------------------------------------------------------------------
struct Sched {
  const float* h_tab;
  const float* t_tab;
  const int64_t* base;
  const int32_t* keep;
  const float* chain_t;
  int64_t offset;
  float h, t;

  __device__ __forceinline__ int64_t step() const {
    return (base != nullptr ? __ldg(base) : 0) + offset;
  }
  __device__ __forceinline__ float step_size(int64_t k) const {
    return h_tab != nullptr ? __ldg(h_tab + k) : h;
  }
  // Temperature of chain c at step k.
  __device__ __forceinline__ float temperature(int64_t k, int c) const {
    const float tk = t_tab != nullptr ? __ldg(t_tab + k) : t;
    return chain_t != nullptr ? tk * __ldg(chain_t + c) : tk;
  }
  __device__ __forceinline__ int keep_slot(int64_t k) const {
    return keep != nullptr ? __ldg(keep + k) : -1;
  }
};

inline Sched to_sched(const gbsgmc_sched* s) {
  Sched r;
  r.h_tab = s->step_size_dev;
  r.t_tab = s->temperature_dev;
  r.base = s->base_dev;
  r.keep = s->keep_slot_dev;
  r.chain_t = s->chain_temperature_dev;
  r.offset = s->offset;
  r.h = s->step_size;
  r.t = s->temperature;
  return r;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the
// multiply-xor round function with the published multipliers and Weyl key
// increments.
// ---------------------------------------------------------------------------
struct U32x4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U32x4 philox4x32_10(U32x4 c, uint32_t k0,
                                               uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    const uint32_t lo0 = M0 * c.x, hi0 = __umulhi(M0, c.x);
    const uint32_t lo1 = M1 * c.z, hi1 = __umulhi(M1, c.z);
    U32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
  }
  return c;
}

// Uniform in (0,1): the top 23 bits plus one half, (2m+1)/2^24, which fp32
// represents exactly over the whole interval.
__device__ __forceinline__ float u32_to_open01(uint32_t v) {
  return (static_cast<float>(v >> 9) + 0.5f) * (1.0f / 8388608.0f);
}

// Box-Muller: (a, b) uniform words -> two standard normals.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0,
                                           float& z1) {
  const float u1 = u32_to_open01(a);
  const float u2 = u32_to_open01(b);
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

// Four normals of group g (params 4g..4g+3) of one chain, step and tag.
__device__ __forceinline__ void philox_normal4(uint64_t seed, uint32_t group,
                                               uint32_t step, uint32_t chain,
                                               uint32_t tag, float out[4]) {
  U32x4 c{group, step, chain, tag};
  U32x4 r = philox4x32_10(c, static_cast<uint32_t>(seed),
                          static_cast<uint32_t>(seed >> 32));
  box_muller(r.x, r.y, out[0], out[1]);
  box_muller(r.z, r.w, out[2], out[3]);
}

struct Noise {
  const float* buf;
  int64_t stride;
  uint64_t seed;
  int chain_base;
};

inline Noise to_noise(const gbsgmc_noise* n) {
  Noise r;
  r.buf = n->noise_dev;
  r.stride = n->noise_stride;
  r.seed = n->seed;
  r.chain_base = n->chain_base;
  return r;
}

// Four normals for params j0..j0+3 (j0 % 4 == 0) of chain c.
__device__ __forceinline__ void noise4(const Noise& nz, int c, int64_t j0,
                                       int64_t P, int64_t step, uint32_t tag,
                                       float out[4]) {
  if (nz.buf != nullptr) {
    const float* p = nz.buf + static_cast<int64_t>(c) * nz.stride + j0;
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = (j0 + q < P) ? __ldg(p + q) : 0.0f;
  } else {
    philox_normal4(nz.seed, static_cast<uint32_t>(j0 >> 2),
                   static_cast<uint32_t>(step),
                   static_cast<uint32_t>(nz.chain_base + c), tag, out);
  }
}

// ---------------------------------------------------------------------------
// 128-bit LCG arithmetic for numpy's PCG64 (O'Neill 2014, XSL-RR output).
// ---------------------------------------------------------------------------
struct U128 {
  uint64_t hi, lo;
};

__device__ __forceinline__ U128 mul128(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo * b.lo;
  r.hi = __umul64hi(a.lo, b.lo) + a.lo * b.hi + a.hi * b.lo;
  return r;
}

__device__ __forceinline__ U128 add128(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ull : 0ull);
  return r;
}

// Affine map s -> A s + C of the LCG.
struct Affine {
  U128 a, c;
};

// Apply f then g: s -> g.a (f.a s + f.c) + g.c.
__device__ __forceinline__ Affine compose(Affine f, Affine g) {
  Affine r;
  r.a = mul128(g.a, f.a);
  r.c = add128(mul128(g.a, f.c), g.c);
  return r;
}

__device__ __forceinline__ U128 apply(Affine f, U128 s) {
  return add128(mul128(f.a, s), f.c);
}

// PCG XSL-RR 128/64 output of a state.
__device__ __forceinline__ uint64_t pcg_output(U128 s) {
  const uint64_t x = s.hi ^ s.lo;
  const unsigned rot = static_cast<unsigned>(s.hi >> 58);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}

// The 128-bit PCG multiplier.
__device__ __forceinline__ U128 pcg_multiplier() {
  return U128{0x2360ED051FC65DA4ull, 0x4385DF649FCCF645ull};
}

// ---------------------------------------------------------------------------
// mbarrier and bulk-copy wrappers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity.  Returns false after
// limit_ns (kWaitLimitNs unless given) or when *abort becomes non-zero.
// try_wait may itself suspend the thread for a while, so the clock and the
// abort flag are checked after every unsuccessful try.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar,
                                                  uint32_t parity,
                                                  volatile int* abort,
                                                  uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (abort != nullptr && *abort) return false;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from
// global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// Warp / block reductions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; every thread receives the result.  `scratch` holds at
// least blockDim.x / 32 doubles.  Contains __syncthreads.
__device__ __forceinline__ double block_sum(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < nw; ++i) t += scratch[i];
  return t;
}

inline int ceil_div(int64_t a, int64_t b) {
  return static_cast<int>((a + b - 1) / b);
}

}  // namespace gbsgmc
