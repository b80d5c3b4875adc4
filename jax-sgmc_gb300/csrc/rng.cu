// Index and noise streams.
//
// * gbsgmc_index_draw_pcg64 reproduces numpy's Generator.choice(arange(N), n,
//   replace=True) bit for bit.  numpy draws each index as a 32-bit Lemire
//   bounded integer (Lemire 2019, "Fast random integer generation in an
//   interval"): x = next_uint32(); m = x * N; accept when (m mod 2^32) >=
//   2^32 mod N, the index being m >> 32.  next_uint32 hands out the low half
//   of a fresh PCG64 output and keeps the high half for the next call.  The
//   accept test depends only on the 32-bit value, so a CTA expands 2048 PCG64
//   outputs at once (each thread jumps ahead to its own 8 consecutive steps
//   by LCG jump-ahead, Brown 1994, "Random number generation with arbitrary
//   strides"), tests the 4096 halves, and compacts the accepted ones with a
//   block scan.  The chain's stream state (128-bit LCG state,
//   buffered half) is advanced exactly as numpy advances it.
// * gbsgmc_index_draw_philox and gbsgmc_philox_normal use Philox4x32-10.
#include "common.cuh"

namespace gbsgmc {
namespace {

constexpr int kDrawThreads = 256;
constexpr int kDrawPerThread = 8;   // consecutive LCG outputs per thread per round
constexpr int kDrawLog2Round = 11;  // log2(kDrawThreads * kDrawPerThread)

// Block-wide exclusive scan of small non-negative ints; returns the exclusive
// prefix and sets *total.  Contains __syncthreads.
__device__ __forceinline__ int block_excl_scan(int v, int* warp_tot,
                                               int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  __syncthreads();
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  int before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kDrawThreads / 32; ++w) {
    const int t = warp_tot[w];
    before += (w < warp) ? t : 0;
    all += t;
  }
  *total = all;
  return before + incl - v;
}

__global__ void __launch_bounds__(kDrawThreads)
    pcg64_draw_kernel(gbsgmc_pcg64* states, int64_t n_obs, int64_t draws,
                      int per_step, int32_t* idx, int64_t chain_stride,
                      int64_t step_stride) {
  // The LCG map applied 1, 2, 4, ..., 2^kDrawLog2Round times.
  __shared__ Affine pow2[kDrawLog2Round + 1];
  __shared__ int warp_tot[kDrawThreads / 32];

  const int c = blockIdx.x;
  const int t = threadIdx.x;
  gbsgmc_pcg64* st = states + c;
  int32_t* out = idx + static_cast<int64_t>(c) * chain_stride;
  auto put = [&](int64_t pos, int32_t v) {
    out[(pos / per_step) * step_stride + pos % per_step] = v;
  };

  if (draws <= 0) return;
  if (n_obs == 1) {  // numpy returns the offset without consuming randomness
    for (int64_t j = t; j < draws; j += kDrawThreads) put(j, 0);
    return;
  }

  U128 s{st->state_hi, st->state_lo};
  const U128 inc{st->inc_hi, st->inc_lo};
  uint32_t has = st->has_uint32;
  const uint32_t buffered = st->uinteger;
  const uint64_t N = static_cast<uint64_t>(n_obs);
  const uint32_t threshold = static_cast<uint32_t>((1ull << 32) % N);

  if (t == 0) {
    pow2[0].a = pcg_multiplier();
    pow2[0].c = inc;
    for (int i = 1; i <= kDrawLog2Round; ++i) pow2[i] = compose(pow2[i - 1], pow2[i - 1]);
  }
  __syncthreads();
  // A round is kDrawThreads * kDrawPerThread LCG steps; this thread's
  // outputs are steps t*K + 1 .. t*K + K of the round (K = kDrawPerThread),
  // so the thread order of the scan is the stream order.
  Affine jump{U128{0, 1}, U128{0, 0}};
  {
    const int k = t * kDrawPerThread + 1;
    for (int i = 0; i <= kDrawLog2Round; ++i)
      if ((k >> i) & 1) jump = compose(jump, pow2[i]);
  }
  const Affine step1 = pow2[0];
  const Affine round_jump = pow2[kDrawLog2Round];

  int64_t produced = 0;
  if (has) {  // the half buffered by the previous call comes first
    const bool acc = static_cast<uint32_t>(buffered * N) >= threshold;
    if (acc) {
      if (t == 0) put(0, static_cast<int32_t>((buffered * N) >> 32));
      produced = 1;
    }
    has = 0;
    if (produced == draws) {
      __syncthreads();
      if (t == 0) st->has_uint32 = 0u;
      return;
    }
  }

  for (;;) {
    U128 sj[kDrawPerThread];
    uint32_t lo[kDrawPerThread], hi[kDrawPerThread];
    unsigned acc = 0;  // bit 2i: low half i accepted, bit 2i+1: high half i
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < kDrawPerThread; ++i) {
      sj[i] = i == 0 ? apply(jump, s) : apply(step1, sj[i - 1]);
      const uint64_t o = pcg_output(sj[i]);
      lo[i] = static_cast<uint32_t>(o);
      hi[i] = static_cast<uint32_t>(o >> 32);
      const unsigned a0 = static_cast<uint32_t>(lo[i] * N) >= threshold ? 1u : 0u;
      const unsigned a1 = static_cast<uint32_t>(hi[i] * N) >= threshold ? 1u : 0u;
      acc |= (a0 << (2 * i)) | (a1 << (2 * i + 1));
      cnt += static_cast<int>(a0 + a1);
    }
    int total;
    const int excl = block_excl_scan(cnt, warp_tot, &total);
    // Output position pos = q * per_step + r, advanced without divisions.
    int64_t pos = produced + excl;
    int64_t q = pos / per_step;
    int r = static_cast<int>(pos - q * per_step);
    int32_t* dst = out + q * step_stride;
#pragma unroll
    for (int i = 0; i < kDrawPerThread; ++i) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if ((acc >> (2 * i + h)) & 1u) {
          const uint32_t v = h ? hi[i] : lo[i];
          if (pos < draws) dst[r] = static_cast<int32_t>((v * N) >> 32);
          ++pos;
          if (++r == per_step) {
            r = 0;
            dst += step_stride;
          }
        }
      }
    }
    if (produced + total >= draws) {
      // The thread holding the last value used stores the stream state after
      // its output, and buffers the high half if the low half was the last.
      const int64_t last = draws - 1 - produced;  // rank of the last value used
      if (cnt > 0 && last >= excl && last < excl + cnt) {
        int64_t rank = excl;
#pragma unroll
        for (int i = 0; i < kDrawPerThread; ++i) {
          if ((acc >> (2 * i)) & 1u) {
            if (rank == last) {
              st->state_hi = sj[i].hi;
              st->state_lo = sj[i].lo;
              st->has_uint32 = 1u;
              st->uinteger = hi[i];
            }
            ++rank;
          }
          if ((acc >> (2 * i + 1)) & 1u) {
            if (rank == last) {
              st->state_hi = sj[i].hi;
              st->state_lo = sj[i].lo;
              st->has_uint32 = 0u;
              st->uinteger = hi[i];
            }
            ++rank;
          }
        }
      }
      return;
    }
    produced += total;
    s = apply(round_jump, s);
  }
}

__global__ void philox_index_kernel(uint64_t seed, int chain_base, int chains,
                                    const int64_t* base, int64_t first_step,
                                    int steps,
                                    int per_step, int64_t n_obs, int32_t* idx,
                                    int64_t chain_stride,
                                    int64_t step_stride) {
  // One thread per pair of draws: a 64-bit uniform per draw keeps the
  // multiply-shift bias below n_obs / 2^64.
  const int pairs = (per_step + 1) / 2;
  const int64_t total = static_cast<int64_t>(chains) * steps * pairs;
  const uint64_t N = static_cast<uint64_t>(n_obs);
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       g < total; g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int p = static_cast<int>(g % pairs);
    const int64_t cs = g / pairs;
    const int sidx = static_cast<int>(cs % steps);
    const int c = static_cast<int>(cs / steps);
    const int64_t step = (base != nullptr ? *base : 0) + first_step + sidx;
    const U32x4 r = philox4x32_10(
        U32x4{static_cast<uint32_t>(p), static_cast<uint32_t>(step),
              static_cast<uint32_t>(chain_base + c), GBSGMC_TAG_INDEX},
        static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint64_t u0 = (static_cast<uint64_t>(r.y) << 32) | r.x;
    const uint64_t u1 = (static_cast<uint64_t>(r.w) << 32) | r.z;
    int32_t* o = idx + c * chain_stride + sidx * step_stride;
    const int j0 = 2 * p;
    o[j0] = static_cast<int32_t>(__umul64hi(u0, N));
    if (j0 + 1 < per_step) o[j0 + 1] = static_cast<int32_t>(__umul64hi(u1, N));
  }
}

__global__ void philox_normal_kernel(uint64_t seed, int chain_base,
                                     int chains, int64_t step, uint32_t tag,
                                     int64_t count, float* out,
                                     int64_t stride) {
  const int64_t groups = (count + 3) / 4;
  const int64_t total = groups * chains;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
       g < total; g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(g / groups);
    const int64_t q = g % groups;
    float z[4];
    philox_normal4(seed, static_cast<uint32_t>(q), static_cast<uint32_t>(step),
                   static_cast<uint32_t>(chain_base + c), tag, z);
    float* o = out + c * stride + 4 * q;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (4 * q + i < count) o[i] = z[i];
  }
}

int grid_for(int64_t work, int threads) {
  int64_t b = (work + threads - 1) / threads;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return static_cast<int>(b);
}

}  // namespace

int launch_philox_index(uint64_t seed, int chain_base, int chains,
                        const int64_t* base, int64_t first_step, int steps,
                        int per_step, int64_t n_obs, int32_t* idx,
                        int64_t chain_stride, int64_t step_stride,
                        cudaStream_t stream) {
  const int64_t work =
      static_cast<int64_t>(chains) * steps * ((per_step + 1) / 2);
  if (work == 0) return GBSGMC_OK;
  philox_index_kernel<<<grid_for(work, 256), 256, 0, stream>>>(
      seed, chain_base, chains, base, first_step, steps, per_step, n_obs, idx,
      chain_stride, step_stride);
  return check_launch("index_draw_philox");
}

}  // namespace gbsgmc

using namespace gbsgmc;

// Fresh numpy PCG64 streams of chains registered with the given seeds: the
// generator numpy.random.default_rng(SeedSequence(seed).spawn(1)[0]) starts
// with.  SeedSequence is M. O'Neill's seed_seq_fe entropy mixer ("Developing
// a seed_seq Alternative", 2015) over a pool of four 32-bit words with its
// published hash and mix constants; the assembled entropy of a chain is its
// seed as four little-endian 32-bit words (zero-padded to the pool size, as
// SeedSequence does when a spawn key follows) and the spawn key word 0.  Four 64-bit words generated from the pool seed
// PCG64 as numpy does: state = 0, inc = 2 initseq + 1, one LCG step,
// state += initstate, one LCG step.
namespace {

struct SeedSeqFe {
  uint32_t hash_a = 0x43B0D7E5u;
  uint32_t hashmix(uint32_t v) {
    v ^= hash_a;
    hash_a *= 0x931E8875u;
    v *= hash_a;
    return v ^ (v >> 16);
  }
  static uint32_t mix(uint32_t x, uint32_t y) {
    const uint32_t r = 0xCA01F9DDu * x - 0x4973F715u * y;
    return r ^ (r >> 16);
  }
};

void pcg64_seed_one(uint64_t lo, uint64_t hi, uint64_t (&out)[5]) {
  // With a spawn key the run entropy is zero-padded to the pool size, so
  // the assembled entropy is always the four seed limbs and the key word.
  const int n = 5;
  const uint32_t ent[5] = {static_cast<uint32_t>(lo), static_cast<uint32_t>(lo >> 32),
                           static_cast<uint32_t>(hi), static_cast<uint32_t>(hi >> 32),
                           0u};  // spawn key (0,)
  SeedSeqFe h;
  uint32_t pool[4];
  for (int i = 0; i < 4; ++i) pool[i] = h.hashmix(ent[i]);
  for (int s = 0; s < 4; ++s)
    for (int d = 0; d < 4; ++d)
      if (s != d) pool[d] = SeedSeqFe::mix(pool[d], h.hashmix(pool[s]));
  for (int i = 4; i < n; ++i)
    for (int d = 0; d < 4; ++d) pool[d] = SeedSeqFe::mix(pool[d], h.hashmix(ent[i]));
  uint32_t hash_b = 0x8B51F9DDu;
  uint32_t w[8];
  for (int i = 0; i < 8; ++i) {
    uint32_t v = pool[i % 4] ^ hash_b;
    hash_b *= 0x58F38DEDu;
    v *= hash_b;
    w[i] = v ^ (v >> 16);
  }
  using u128 = unsigned __int128;
  const auto word64 = [&](int k) {
    return static_cast<uint64_t>(w[2 * k]) | (static_cast<uint64_t>(w[2 * k + 1]) << 32);
  };
  const u128 initstate = (static_cast<u128>(word64(0)) << 64) | word64(1);
  const u128 initseq = (static_cast<u128>(word64(2)) << 64) | word64(3);
  const u128 mult = (static_cast<u128>(0x2360ED051FC65DA4ull) << 64) | 0x4385DF649FCCF645ull;
  const u128 inc = (initseq << 1) | 1u;
  u128 state = inc;                 // 0 * mult + inc
  state += initstate;
  state = state * mult + inc;
  out[0] = static_cast<uint64_t>(state >> 64);
  out[1] = static_cast<uint64_t>(state);
  out[2] = static_cast<uint64_t>(inc >> 64);
  out[3] = static_cast<uint64_t>(inc);
  out[4] = 0;  // no buffered 32-bit half
}

}  // namespace

extern "C" int gbsgmc_pcg64_seed(const uint64_t* seeds_lo, const uint64_t* seeds_hi, int count,
                                 uint64_t* words) {
  if (count < 0) return set_error(GBSGMC_ERR_ARG, "pcg64_seed: negative count");
  if (count > 0 && (seeds_lo == nullptr || words == nullptr))
    return set_error(GBSGMC_ERR_ARG, "pcg64_seed: null pointer");
  for (int c = 0; c < count; ++c) {
    uint64_t out[5];
    pcg64_seed_one(seeds_lo[c], seeds_hi != nullptr ? seeds_hi[c] : 0, out);
    for (int k = 0; k < 5; ++k) words[5 * static_cast<int64_t>(c) + k] = out[k];
  }
  return GBSGMC_OK;
}

extern "C" int gbsgmc_index_draw_pcg64(gbsgmc_pcg64* states_dev, int chains,
                                       int64_t n_obs, int64_t draws,
                                       int per_step, int32_t* idx_dev,
                                       int64_t chain_stride,
                                       int64_t step_stride, int* status_dev,
                                       gbsgmc_stream_t stream) {
  (void)status_dev;
  if (states_dev == nullptr || idx_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "index_draw_pcg64: null pointer");
  if (chains < 0 || draws < 0 || per_step <= 0)
    return set_error(GBSGMC_ERR_ARG, "index_draw_pcg64: negative size");
  if (n_obs < 1 || n_obs >= (1ll << 31))
    return set_error(GBSGMC_ERR_SHAPE,
                     "index_draw_pcg64: n_obs must be in [1, 2^31), got %lld",
                     static_cast<long long>(n_obs));
  if (chains == 0 || draws == 0) return GBSGMC_OK;
  pcg64_draw_kernel<<<chains, kDrawThreads, 0,
                      static_cast<cudaStream_t>(stream)>>>(
      states_dev, n_obs, draws, per_step, idx_dev, chain_stride, step_stride);
  return check_launch("index_draw_pcg64");
}

extern "C" int gbsgmc_index_draw_philox(uint64_t seed, int chain_base,
                                        int chains, int64_t first_step,
                                        int steps, int per_step, int64_t n_obs,
                                        int32_t* idx_dev, int64_t chain_stride,
                                        int64_t step_stride,
                                        gbsgmc_stream_t stream) {
  if (idx_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "index_draw_philox: null pointer");
  if (chains < 0 || steps < 0 || per_step <= 0)
    return set_error(GBSGMC_ERR_ARG, "index_draw_philox: negative size");
  if (n_obs < 1 || n_obs >= (1ll << 31))
    return set_error(GBSGMC_ERR_SHAPE,
                     "index_draw_philox: n_obs must be in [1, 2^31)");
  return launch_philox_index(seed, chain_base, chains, nullptr, first_step,
                             steps, per_step, n_obs, idx_dev, chain_stride,
                             step_stride, static_cast<cudaStream_t>(stream));
}

extern "C" int gbsgmc_philox_normal(uint64_t seed, int chain_base, int chains,
                                    int64_t step, uint32_t tag, int64_t count,
                                    float* out_dev, int64_t stride,
                                    gbsgmc_stream_t stream) {
  if (out_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "philox_normal: null pointer");
  if (chains < 0 || count < 0 || stride < count)
    return set_error(GBSGMC_ERR_ARG, "philox_normal: bad size or stride");
  const int64_t work = static_cast<int64_t>(chains) * ((count + 3) / 4);
  if (work == 0) return GBSGMC_OK;
  philox_normal_kernel<<<grid_for(work, 256), 256, 0,
                         static_cast<cudaStream_t>(stream)>>>(
      seed, chain_base, chains, step, tag, count, out_dev, stride);
  return check_launch("philox_normal");
}
