// Shared declarations of the tcgen05 GEMM (tc_gemm.cu) and its users.
#pragma once

#include <cuda.h>
#include <stddef.h>
#include <stdint.h>

#include <type_traits>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace gbsgmc {

constexpr int kGemmBM = 128;     // rows of a CTA tile (UMMA M)
constexpr int kGemmBK = 64;      // K per stage: one 128-byte swizzle row
constexpr int kGemmStages = 4;   // shared-memory ring depth at BN = 256
// Ring depth of the single-CTA kernel: as many stages as fit beside the
// epilogue staging (one CTA per SM either way), so that short-N GEMMs keep
// more copies in flight: 4 at BN = 256 (48 KB stages), 6 at BN = 128, 8 at
// BN = 64.
__host__ __device__ constexpr int gemm_stages(int bn) {
  return bn == 256 ? kGemmStages : bn == 128 ? 6 : 8;
}
constexpr int kGemmSplit = 2;    // epilogue warps per TMEM lane quarter
constexpr int kGemmEpiWarps = 4 * kGemmSplit;
constexpr int kGemmThreads = 64 + 32 * kGemmEpiWarps;  // producer, MMA, epilogue
constexpr int kStageWords = 32 * 32;  // per-warp staging tile (32 x 32 words, 4 KB)

// Epilogue staging helpers.  A warp's 32 lanes own 32 consecutive
// accumulator rows; these move a 32-row block between that row-per-lane form
// and row-contiguous global memory through the warp's 4 KB staging tile
// (1024-byte aligned), so that every global access is one 128-byte row
// segment.  Word j of row r sits at r * 32 + (j ^ r): a row written by one
// lane and a column read across lanes both touch 32 distinct banks.  The
// tile may also hold a TMA store's box (store_box); the helpers that write
// it first wait until such a store has read it.
namespace epi {

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Waits until the warp's last TMA store (store_box) has read the staging
// tile; warp-collective.
__device__ __forceinline__ void reclaim() {
  if (lane_id() == 0) tc::bulk_wait_read();
  __syncwarp();
}

// Lane l's 32 words go to staging row l; afterwards any lane may read row r.
__device__ __forceinline__ void put_rows(uint32_t* st, const uint32_t (&w)[32]) {
  const int l = lane_id();
  reclaim();
#pragma unroll
  for (int j = 0; j < 32; ++j) st[l * 32 + (j ^ l)] = w[j];
  __syncwarp();
}

// Word `lane` of staging row r.
__device__ __forceinline__ uint32_t get(const uint32_t* st, int r) {
  return st[r * 32 + (lane_id() ^ r)];
}

// The reverse: word `lane` of row r was written by the whole warp (set,
// after reclaim), and lane l collects its own row.
__device__ __forceinline__ void set(uint32_t* st, int r, uint32_t v) {
  st[r * 32 + (lane_id() ^ r)] = v;
}
__device__ __forceinline__ void get_row(const uint32_t* st, uint32_t (&w)[32]) {
  const int l = lane_id();
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 32; ++j) w[j] = st[l * 32 + (j ^ l)];
  __syncwarp();
}

// Stores the warp's 32 rows of 128 bytes (lane l's words w = row l) as one
// box of a tensor map with a 128-byte swizzle and a box of 128 bytes x 32
// rows, at coordinates (x, y, z): the rows are written to the staging tile
// in the swizzled order (16-byte chunk q of row r at chunk q ^ (r & 7)) and
// one lane issues the TMA store, which runs on while the warp continues.
// The epilogue kernels wait for the stores before they exit.
__device__ __forceinline__ void store_box(uint32_t* st, const uint32_t (&w)[32],
                                          const CUtensorMap* map, int x, int y, int z) {
  const int l = lane_id();
  reclaim();
  uint8_t* row = reinterpret_cast<uint8_t*>(st) + l * 128;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    tc::sts128(row + ((q ^ (l & 7)) << 4), w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
  tc::fence_async_shared();
  __syncwarp();
  if (l == 0) {
    tc::tma_store_3d(map, st, x, y, z);
    tc::bulk_commit();
  }
}

// The reverse of store_box for a warp's reads: copies a block of 32 rows of
// 128 bytes (row r at src + r * ld_bytes, 16-byte aligned) into the staging
// tile in store_box's swizzled order with asynchronous 16-byte copies
// (eight per lane, 8 lanes per row), once the tile's last TMA store has read
// it; fetch_wait completes them for the whole warp and read_row gives lane
// l its row.
__device__ __forceinline__ void fetch_box(uint32_t* st, const void* src, int64_t ld_bytes) {
  const int l = lane_id(), q = l & 7;
  reclaim();
  uint8_t* tile = reinterpret_cast<uint8_t*>(st);
  const char* s = static_cast<const char*>(src);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int r = 4 * i + (l >> 3);
    tc::cp_async16(tile + r * 128 + ((q ^ (r & 7)) << 4), s + r * ld_bytes + q * 16);
  }
  tc::cp_async_commit();
}
__device__ __forceinline__ void fetch_wait() {
  tc::cp_async_wait_all();
  __syncwarp();
}
__device__ __forceinline__ void read_row(const uint32_t* st, uint32_t (&w)[32]) {
  const int l = lane_id();
  const uint8_t* row = reinterpret_cast<const uint8_t*>(st) + l * 128;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const uint4 x = tc::lds128(row + ((q ^ (l & 7)) << 4));
    w[4 * q] = x.x;
    w[4 * q + 1] = x.y;
    w[4 * q + 2] = x.z;
    w[4 * q + 3] = x.w;
  }
}

}  // namespace epi

// 3-D BF16 tensor map (cols innermost, rows, batch) with a 128-byte swizzled
// box of box_cols x box_rows; strides in elements.
int make_tmap_bf16_3d(CUtensorMap* map, const void* base, int64_t cols,
                      int64_t rows, int64_t batch, int64_t row_stride,
                      int64_t batch_stride, int box_cols, int box_rows);

// 4-D BF16 tensor map (dims[0] innermost, strides of dims 1..3 in elements)
// with a 128-byte swizzled box; dims[0] x 2 bytes of a box row must be 128.
int make_tmap_bf16_4d(CUtensorMap* map, const void* base, const int64_t (&dims)[4],
                      const int64_t (&strides)[3], const int (&box)[4]);

// 4-D BF16 tensor map without swizzle (dims[0] innermost, strides of dims
// 1..3 in elements), for the unswizzled operand layouts: a box row of
// box[0] BF16 (a multiple of 8) lands as box[0] * 2 contiguous bytes.
int make_tmap_bf16_4d_plain(CUtensorMap* map, const void* base, const int64_t (&dims)[4],
                            const int64_t (&strides)[3], const int (&box)[4]);

// 3-D tensor map (cols innermost, rows, batch) of an epilogue's output for
// epi::store_box: 128-byte swizzle, boxes of 128 bytes x 32 rows (64 BF16 or
// 32 fp32 columns); strides in elements.
int make_tmap_rows(CUtensorMap* map, const void* base, bool f32, int64_t cols, int64_t rows,
                   int64_t batch, int64_t row_stride, int64_t batch_stride);

size_t gemm_smem_bytes(int bn);

// Operand loaders.  An epilogue type may replace the tiled 3-D loads of the
// single-CTA GEMM's operands: with `static constexpr bool kLoadA = true` and
//   load_a(dst, map, k0, m0, b, bar)  (a K-major 128 x 64 A tile)
// and with `kLoadB = true` and
//   load_b(dst, map, n, k0, b, bar)   (a B tile: for an MN-major B one
//                                      64 x 64 block starting at column n,
//                                      for a K-major B the BN x 64 tile)
// the producer calls these instead, e.g. to read shifted boxes of an NHWC
// map for an implicit convolution.  They must load the bytes the default
// loads would.
// Partial stages.  An epilogue type whose loaders fill only part of a stage
// (rows of A or columns of B whose products it never stores) declares the
// bytes they deliver per stage as `static constexpr uint32_t kStageBytes`;
// the producer expects that many instead of the full A and B tiles.  An
// MN-major A is then loaded by its load_a too.
template <class E, class = void>
struct StageBytes : std::integral_constant<uint32_t, 0> {};
template <class E>
struct StageBytes<E, std::void_t<decltype(E::kStageBytes)>>
    : std::integral_constant<uint32_t, E::kStageBytes> {};

// Unswizzled operand layouts.  With `static constexpr bool kInterleaveA =
// true` (kInterleaveB) the epilogue type's load_a (load_b) fills the stage in
// the unswizzled core-matrix layout instead of the 128-byte swizzle: for a
// K-major operand of R rows (128 for A, BN for B) the core matrix of row
// group g and K group j (8 rows x 8 BF16) at j * R * 16 + g * 128 bytes; for
// an MN-major B the core matrix of N group j and K group g at j * 1024 +
// g * 128 (each 64-row K slice of 8 N columns is 1 KB).
template <class E, class = void>
struct InterleaveA : std::false_type {};
template <class E>
struct InterleaveA<E, std::void_t<decltype(E::kInterleaveA)>>
    : std::bool_constant<E::kInterleaveA> {};
template <class E, class = void>
struct InterleaveB : std::false_type {};
template <class E>
struct InterleaveB<E, std::void_t<decltype(E::kInterleaveB)>>
    : std::bool_constant<E::kInterleaveB> {};

template <class E, class = void>
struct LoadsA : std::false_type {};
template <class E>
struct LoadsA<E, std::void_t<decltype(E::kLoadA)>> : std::bool_constant<E::kLoadA> {};
template <class E, class = void>
struct LoadsB : std::false_type {};
template <class E>
struct LoadsB<E, std::void_t<decltype(E::kLoadB)>> : std::bool_constant<E::kLoadB> {};

// CTA-pair GEMM (tc_gemm2_kernel): shared-memory ring depth, bytes, and
// whether it is used where it applies (the GBSGMC_GEMM_PAIR environment
// variable set to 0 turns it off; read at each launch).
constexpr int kGemm2Stages = 6;
size_t gemm2_smem_bytes(int bn);
bool gemm_pair_enabled();

// Ragged batches: chain b may use only the first m_b rows (row-ragged: its
// output tiles are counted by tile_prefix[b + 1] - tile_prefix[b]) or only
// the first kblocks[b] 64-wide K slices (K-ragged).  Null pointers mean the
// uniform batch.  Both arrays live in device memory.
struct GemmRagged {
  const int* tile_prefix = nullptr;  // [batch + 1], tile_prefix[0] = 0
  const int* kblocks = nullptr;      // [batch]
  // Split-K (uniform batches only): each output tile is computed as ksplit
  // partial products over consecutive K ranges by different CTAs; the
  // epilogue sees batch index b * ksplit + s for split s.
  int ksplit = 1;
  // Bound of each wait for pipeline progress (a stage's operands, a free
  // stage or accumulator, a finished accumulator).  The waits of the clean-up
  // after a timeout (copies and MMAs already issued) keep kWaitLimitNs.
  uint64_t wait_ns = kWaitLimitNs;
};

__device__ __forceinline__ int ragged_batch(const GemmRagged& rg, int t, int per_batch,
                                            int batch) {
  if (rg.tile_prefix == nullptr) return t / per_batch;
  int lo = 0, hi = batch;  // largest b with tile_prefix[b] <= t
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(rg.tile_prefix + mid) <= t) lo = mid; else hi = mid;
  }
  return lo;
}

// Persistent batched GEMM C[b] = A[b] * B[b]^T on the tcgen05 tensor cores.
//
// A is M x K and B is N x K, BF16; each is either K-major (rows of K
// contiguous elements, A_MN / B_MN false) or MN-major (stored transposed:
// rows of M or N contiguous elements).  The grid holds at most one CTA per
// resident slot; CTA i takes output tiles i, i + gridDim.x, ... in the order
// (batch, M tile, N tile), N fastest.  Roles:
//   warp 0 (one lane)  TMA producer into a gemm_stages(BN)-deep ring of 64-wide
//                      K slices (128-byte swizzle)
//   warp 1             allocates two BN-column TMEM accumulators; one lane
//                      issues tcgen05.mma (M=128, N=BN, K=16) into them
//   warps 2..          epilogue, kGemmSplit warps per TMEM lane quarter:
//                      warp w reads lanes 32 (w % 4) .. + 31 of the finished
//                      accumulator, columns [h NC, (h + 1) NC) with
//                      h = (w - 2) / 4 and NC = BN / kGemmSplit, while the
//                      MMA warp fills the other accumulator with the next tile
// Each epilogue lane owns one accumulator row and the warp calls
//   epi.template tile<NC>(batch, row0, col0, load, stage)
// with row0 the first of the warp's 32 rows (lane l holds row row0 + l),
// col0 its first column, load(c, v) filling v[32] with columns
// [32c, 32c + 32) of the lane's row (warp-collective), and stage a private
// 4 KB shared-memory tile (1024-byte aligned) for the epi:: helpers.
//
// Every wait is bounded (rg.wait_ns, kWaitLimitNs by default): on a timeout
// the CTA records GBSGMC_ERR_TIMEOUT, stops issuing work, waits (bounded by
// kWaitLimitNs) for the copies and MMAs it issued, frees its TMEM and
// returns.
template <int BN, bool A_MN, bool B_MN, class Epi>
__global__ void __launch_bounds__(kGemmThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                   const __grid_constant__ CUtensorMap tb, int M, int N, int K,
                   int batch, int* status, const __grid_constant__ Epi epi, GemmRagged rg) {
  constexpr int BM = kGemmBM, BK = kGemmBK, STAGES = gemm_stages(BN);
  constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  constexpr uint32_t BLOCK_BYTES = 64 * BK * 2;  // one 64 x 64 MN-major box
  constexpr uint32_t TMEM_COLS = 2 * BN;
  static_assert(BN == 64 || BN == 128 || BN == 256, "BN");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sa = smem;
  uint8_t* sb = smem + STAGES * A_BYTES;
  uint32_t* stage_all = reinterpret_cast<uint32_t*>(sb + STAGES * B_BYTES);
  uint64_t* full = reinterpret_cast<uint64_t*>(stage_all + kGemmEpiWarps * kStageWords);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;  // [2] accumulator ready for the epilogue
  uint64_t* tempty = tfull + 2;      // [2] accumulator drained by the epilogue
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_n = N / BN, per_batch = (M / BM) * tiles_n;
  const int vbatch = batch * rg.ksplit;
  const int tiles = rg.tile_prefix != nullptr ? __ldg(rg.tile_prefix + batch)
                                              : per_batch * vbatch;
  // (Virtual) batch of tile t, its index within the batch, its K slices and
  // the first of them.
  auto decode = [&](int t, int& b, int& r, int& KB, int& kb0) {
    b = ragged_batch(rg, t, per_batch, vbatch);
    r = t - (rg.tile_prefix != nullptr ? __ldg(rg.tile_prefix + b) : b * per_batch);
    KB = rg.kblocks != nullptr ? __ldg(rg.kblocks + b) : K / BK / rg.ksplit;
    kb0 = (b % rg.ksplit) * KB;
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], kGemmEpiWarps);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    mbar_fence_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x) {
        int bv, r, KB, kb0;
        decode(t, bv, r, KB, kb0);
        const int b = bv / rg.ksplit;
        const int m0 = (r / tiles_n) * BM, n0 = (r % tiles_n) * BN;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!mbar_wait_bounded(&empty[s], ph ^ 1u, abort_flag, rg.wait_ns)) {
            raise_status(status, GBSGMC_ERR_TIMEOUT);
            *abort_flag = 1;
            ok = false;
            break;
          }
          constexpr uint32_t TX =
              StageBytes<Epi>::value != 0 ? StageBytes<Epi>::value : A_BYTES + B_BYTES;
          mbar_arrive_expect_tx(&full[s], TX);
          const int k0 = (kb0 + kb) * BK;
          if constexpr (A_MN && LoadsA<Epi>::value) {
            epi.load_a(sa + s * A_BYTES, &ta, k0, m0, b, &full[s]);
          } else if constexpr (A_MN) {
#pragma unroll
            for (int j = 0; j < BM / 64; ++j)
              tc::tma_load_3d(sa + s * A_BYTES + j * BLOCK_BYTES, &ta, m0 + 64 * j, k0, b,
                              &full[s]);
          } else if constexpr (LoadsA<Epi>::value) {
            epi.load_a(sa + s * A_BYTES, &ta, k0, m0, b, &full[s]);
          } else {
            tc::tma_load_3d(sa + s * A_BYTES, &ta, k0, m0, b, &full[s]);
          }
          if constexpr (B_MN) {
#pragma unroll
            for (int j = 0; j < BN / 64; ++j) {
              if constexpr (LoadsB<Epi>::value)
                epi.load_b(sb + s * B_BYTES + j * BLOCK_BYTES, &tb, n0 + 64 * j, k0, b,
                           &full[s]);
              else
                tc::tma_load_3d(sb + s * B_BYTES + j * BLOCK_BYTES, &tb, n0 + 64 * j, k0, b,
                                &full[s]);
            }
          } else if constexpr (LoadsB<Epi>::value) {
            epi.load_b(sb + s * B_BYTES, &tb, n0, k0, b, &full[s]);
          } else {
            tc::tma_load_3d(sb + s * B_BYTES, &tb, k0, n0, b, &full[s]);
          }
        }
      }
      if (!ok) {
        // Let the copies still in flight land before the CTA exits.
        for (uint32_t i = (it > STAGES ? it - STAGES : 0); i < it; ++i)
          mbar_wait_bounded(&full[i % STAGES], (i / STAGES) & 1u, nullptr);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN, A_MN, B_MN);
      uint32_t it = 0, acc = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x, ++acc) {
        int b, r, KB, kb0;
        decode(t, b, r, KB, kb0);
        const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
        if (!mbar_wait_bounded(&tempty[buf], aph ^ 1u, abort_flag, rg.wait_ns)) {
          raise_status(status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        tc::fence_after_sync();
        const uint32_t d = tmem + buf * BN;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!mbar_wait_bounded(&full[s], ph, abort_flag, rg.wait_ns)) {
            raise_status(status, GBSGMC_ERR_TIMEOUT);
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc::fence_after_sync();
          constexpr bool IA = InterleaveA<Epi>::value, IB = InterleaveB<Epi>::value;
          static_assert(!(IA && A_MN), "an unswizzled A is K-major");
          // Descriptor steps per K = 16 slice, in 16-byte units: 32 bytes
          // along a swizzled K-major row, two 8-row groups (2048 bytes) of a
          // swizzled MN-major tile, two K groups of an unswizzled tile.
          constexpr uint32_t step_a = IA ? 2 * BM : A_MN ? 128 : 2;
          constexpr uint32_t step_b = IB ? (B_MN ? 16 : 2 * BN) : B_MN ? 128 : 2;
          const uint64_t a0 = IA     ? tc::sdesc_none(sa + s * A_BYTES, BM * 16, 128)
                              : A_MN ? tc::sdesc_mn_sw128(sa + s * A_BYTES, BLOCK_BYTES)
                                     : tc::sdesc_k_sw128(sa + s * A_BYTES);
          const uint64_t b0 = IB     ? (B_MN ? tc::sdesc_none(sb + s * B_BYTES, 128, 1024)
                                             : tc::sdesc_none(sb + s * B_BYTES, BN * 16, 128))
                              : B_MN ? tc::sdesc_mn_sw128(sb + s * B_BYTES, BLOCK_BYTES)
                                     : tc::sdesc_k_sw128(sb + s * B_BYTES);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint64_t da = static_cast<uint64_t>(step_a) * k;
            const uint64_t db = static_cast<uint64_t>(step_b) * k;
            tc::mma_bf16(d, a0 + da, b0 + db, idesc, (kb | k) != 0);
          }
          tc::mma_commit(&empty[s]);
        }
        if (ok) tc::mma_commit(&tfull[buf]);
      }
      // Every MMA issued by this CTA has completed once `drain` flips.
      tc::mma_commit(drain);
      mbar_wait_bounded(drain, 0, nullptr);
    }
  } else {
    constexpr int NC = BN / kGemmSplit;
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int h = (warp - 2) >> 2;
    uint32_t* stage = stage_all + (warp - 2) * kStageWords;
    uint32_t acc = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++acc) {
      const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
      const bool ok = mbar_wait_bounded(&tfull[buf], aph, abort_flag, rg.wait_ns);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0 && !*abort_flag) {
          raise_status(status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
        }
        break;
      }
      tc::fence_after_sync();
      int b, r, KB, kb0;
      decode(t, b, r, KB, kb0);
      const int row0 = (r / tiles_n) * BM + q * 32;
      const uint32_t tbase =
          tmem + buf * BN + h * NC + (static_cast<uint32_t>(q * 32) << 16);
      const tc::TmemRows load{tbase};
      epi.template tile<NC>(b, row0, (r % tiles_n) * BN + h * NC, load, stage);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[buf]);
    }
    if (lane == 0) tc::bulk_wait();  // the epilogue's TMA stores
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Launches the persistent GEMM on `st`: one CTA per resident slot (at most
// one per output tile of the uniform batch; with a ragged batch M and K are
// the largest chain's).  ta / tb: tensor maps made by make_tmap_bf16_3d with
// boxes of 64 x 128 (A, K-major), 64 x BN (B, K-major) or 64 x 64 (MN-major).
template <int BN, bool A_MN, bool B_MN, class Epi>
int launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, int batch, int M,
                int N, int K, int* status, const Epi& epi, cudaStream_t st,
                GemmRagged rg = GemmRagged{}) {
  auto kern = tc_gemm_kernel<BN, A_MN, B_MN, Epi>;
  const size_t smem = gemm_smem_bytes(BN);
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGemmThreads, smem);
    if (e != cudaSuccess || per_sm < 1)
      return set_error(GBSGMC_ERR_CUDA, "gemm: cannot configure the kernel: %s",
                       cudaGetErrorString(e));
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "gemm: cannot query the device");
  const int64_t tiles = static_cast<int64_t>(M / kGemmBM) * (N / BN) * batch * rg.ksplit;
  const int grid = static_cast<int>(tiles < int64_t(sms) * per_sm ? tiles : int64_t(sms) * per_sm);
  kern<<<grid, kGemmThreads, smem, st>>>(ta, tb, M, N, K, batch, status, epi, rg);
  return check_launch("tc_gemm_kernel");
}

// Persistent batched GEMM on CTA pairs (tcgen05 .cta_group::2): each
// cluster of two CTAs computes 256 x BN output tiles, C[b] = A[b] B[b]^T as
// tc_gemm_kernel, with the same operand layouts and epilogue interface.
// Per pair tile and 64-wide K slice, CTA r (its rank in the cluster) loads
// rows [128 r, 128 r + 128) of the tile's A rows and rows [BN/2 r, BN/2 r +
// BN/2) of its B rows into its own ring stage; both CTAs' copies complete on
// the leader's (rank 0) `full` barrier.  The leader's MMA warp issues
// M = 256 x N = BN MMAs that read both CTAs' halves and accumulate rows
// [128 r, 128 r + 128) in CTA r's TMEM, and commits to the `empty` and
// `tfull` barriers of both CTAs at once.  Each CTA's epilogue warps drain
// their own TMEM rows and report to the leader's `tempty` barrier.  Against
// the single-CTA kernel a B row is read once per 256 output rows instead of
// once per 128, halving the B operand's shared-memory reads and copies, and
// a stage holds 32 KB, so the ring is six stages deep.
//
// Every wait is bounded as in tc_gemm_kernel; a CTA that times out sets its
// own and its partner's abort flags, and both leave their loops, wait 2 ms
// for copies in flight, meet at a cluster barrier, free the TMEM and return.
template <int BN, bool A_MN, bool B_MN, class Epi>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kGemmThreads, 1)
    tc_gemm2_kernel(const __grid_constant__ CUtensorMap ta,
                    const __grid_constant__ CUtensorMap tb, int M, int N, int K, int batch,
                    int* status, const __grid_constant__ Epi epi, uint64_t wait_ns) {
  constexpr int BM = 2 * kGemmBM;  // rows of a pair tile, kGemmBM per CTA
  constexpr int BK = kGemmBK, STAGES = kGemm2Stages;
  constexpr int BNH = BN / 2;      // B rows held by each CTA
  constexpr uint32_t A_BYTES = kGemmBM * BK * 2, B_BYTES = BNH * BK * 2;
  constexpr uint32_t BLOCK_BYTES = 64 * BK * 2;  // one 64 x 64 MN-major box
  constexpr uint32_t TMEM_COLS = 2 * BN;
  static_assert(BN == 256, "pair tiles are 256 x 256");
  static_assert(!LoadsA<Epi>::value && !LoadsB<Epi>::value && !InterleaveA<Epi>::value &&
                    !InterleaveB<Epi>::value,
                "pair tiles take no operand loaders");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sa = smem;
  uint8_t* sb = smem + STAGES * A_BYTES;
  uint32_t* stage_all = reinterpret_cast<uint32_t*>(sb + STAGES * B_BYTES);
  uint64_t* full = reinterpret_cast<uint64_t*>(stage_all + kGemmEpiWarps * kStageWords);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;  // [2] accumulator ready (both CTAs)
  uint64_t* tempty = tfull + 2;      // [2] accumulator drained (leader: both CTAs' warps)
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const uint32_t rank = tc::cluster_rank();
  const bool leader = rank == 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_n = N / BN, per_batch = (M / BM) * tiles_n;
  const int tiles = per_batch * batch;
  const int KB = K / BK;
  const int first = static_cast<int>(tc::cluster_id());
  const int step = static_cast<int>(tc::cluster_count());
  const uint32_t peer_abort = tc::peer_addr(const_cast<int*>(abort_flag), rank ^ 1u);
  auto fail = [&]() {
    raise_status(status, GBSGMC_ERR_TIMEOUT);
    *abort_flag = 1;
    tc::st_cluster_u32(peer_abort, 1u);
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], 2 * kGemmEpiWarps);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    mbar_fence_init();
  }
  if (warp == 1) {
    tc::tmem_alloc2(tmem_slot, TMEM_COLS);
    tc::tmem_relinquish2();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::cluster_sync();  // both CTAs' barriers and flags are initialised
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int t = first; ok && t < tiles; t += step) {
        const int b = t / per_batch, r = t % per_batch;
        const int m0 = (r / tiles_n) * BM + kGemmBM * static_cast<int>(rank);
        const int n0 = (r % tiles_n) * BN + BNH * static_cast<int>(rank);
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!mbar_wait_bounded(&empty[s], ph ^ 1u, abort_flag, wait_ns)) {
            fail();
            ok = false;
            break;
          }
          const uint32_t fb = tc::peer_addr(&full[s], 0);
          if (leader) mbar_arrive_expect_tx(&full[s], 2 * (A_BYTES + B_BYTES));
          const int k0 = kb * BK;
          if constexpr (A_MN) {
#pragma unroll
            for (int j = 0; j < kGemmBM / 64; ++j)
              tc::tma_load_3d_pair(sa + s * A_BYTES + j * BLOCK_BYTES, &ta, m0 + 64 * j, k0, b, fb);
          } else {
            tc::tma_load_3d_pair(sa + s * A_BYTES, &ta, k0, m0, b, fb);
          }
          if constexpr (B_MN) {
#pragma unroll
            for (int j = 0; j < BNH / 64; ++j)
              tc::tma_load_3d_pair(sb + s * B_BYTES + j * BLOCK_BYTES, &tb, n0 + 64 * j, k0, b, fb);
          } else {
            tc::tma_load_3d_pair(sb + s * B_BYTES, &tb, k0, n0, b, fb);
          }
        }
      }
    }
  } else if (warp == 1) {
    if (leader && lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN, A_MN, B_MN);
      uint32_t it = 0, acc = 0;
      bool ok = true;
      for (int t = first; ok && t < tiles; t += step, ++acc) {
        const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
        if (!tc::mbar_wait_cluster_bounded(&tempty[buf], aph ^ 1u, abort_flag, wait_ns)) {
          fail();
          break;
        }
        tc::fence_after_sync();
        const uint32_t d = tmem + buf * BN;
        for (int kb = 0; kb < KB; ++kb, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!mbar_wait_bounded(&full[s], ph, abort_flag, wait_ns)) {
            fail();
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint64_t a0 = A_MN ? tc::sdesc_mn_sw128(sa + s * A_BYTES, BLOCK_BYTES)
                                   : tc::sdesc_k_sw128(sa + s * A_BYTES);
          const uint64_t b0 = B_MN ? tc::sdesc_mn_sw128(sb + s * B_BYTES, BLOCK_BYTES)
                                   : tc::sdesc_k_sw128(sb + s * B_BYTES);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint64_t da = A_MN ? 128u * k : 2u * k;
            const uint64_t db = B_MN ? 128u * k : 2u * k;
            tc::mma2_bf16(d, a0 + da, b0 + db, idesc, (kb | k) != 0);
          }
          tc::mma2_commit_multicast(&empty[s], 0x3);
        }
        if (ok) tc::mma2_commit_multicast(&tfull[buf], 0x3);
      }
      tc::mma2_commit(drain);
      mbar_wait_bounded(drain, 0, nullptr);
    }
  } else {
    constexpr int NC = BN / kGemmSplit;
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    uint32_t* stage = stage_all + (warp - 2) * kStageWords;
    const uint32_t drained0 = tc::peer_addr(&tempty[0], 0);
    const uint32_t drained1 = tc::peer_addr(&tempty[1], 0);
    uint32_t acc = 0;
    for (int t = first; t < tiles; t += step, ++acc) {
      const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
      const bool ok = mbar_wait_bounded(&tfull[buf], aph, abort_flag, wait_ns);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0 && !*abort_flag) fail();
        break;
      }
      tc::fence_after_sync();
      const int b = t / per_batch, r = t % per_batch;
      const int row0 = (r / tiles_n) * BM + kGemmBM * static_cast<int>(rank) + q * 32;
      const uint32_t tbase =
          tmem + buf * BN + h * NC + (static_cast<uint32_t>(q * 32) << 16);
      const tc::TmemRows load{tbase};
      epi.template tile<NC>(b, row0, (r % tiles_n) * BN + h * NC, load, stage);
      tc::fence_before_sync();
      __syncwarp();
      // The accumulator's rows are in registers (tcgen05.wait::ld): nothing
      // else has to be ordered before the leader may overwrite them.
      if (lane == 0) tc::mbar_arrive_cluster_relaxed(buf ? drained1 : drained0);
    }
    if (lane == 0) tc::bulk_wait();  // the epilogue's TMA stores
  }
  tc::fence_before_sync();
  __syncthreads();
  if (*abort_flag && threadIdx.x == 0) {
    // Copies already issued complete within microseconds.
    const uint64_t t0 = global_ns();
    while (global_ns() - t0 < 2000000ull) {
    }
  }
  __syncthreads();
  tc::cluster_sync();  // no further access to the partner's shared memory
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc2(tmem, TMEM_COLS);
  }
}

// Launches the pair GEMM on `st` (uniform batches; M a multiple of 256, N of
// BN, K of 64): one cluster per co-resident pair slot, at most one per pair
// tile.  Tensor maps as for launch_gemm except that a K-major B map has
// boxes of 64 x BN/2.
template <int BN, bool A_MN, bool B_MN, class Epi>
int launch_gemm2(const CUtensorMap& ta, const CUtensorMap& tb, int batch, int M, int N, int K,
                 int* status, const Epi& epi, cudaStream_t st,
                 uint64_t wait_ns = kWaitLimitNs) {
  auto kern = tc_gemm2_kernel<BN, A_MN, B_MN, Epi>;
  const size_t smem = gemm2_smem_bytes(BN);
  static int max_clusters = 0;
  if (max_clusters == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * (sms / 2), 1, 1);
      cfg.blockDim = dim3(kGemmThreads, 1, 1);
      cfg.dynamicSmemBytes = smem;
      e = cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg);
    }
    if (e != cudaSuccess || max_clusters < 1) {
      max_clusters = 0;
      return set_error(GBSGMC_ERR_CUDA, "gemm (pairs): cannot configure the kernel: %s",
                       cudaGetErrorString(e));
    }
  }
  if (M % (2 * kGemmBM) != 0 || N % BN != 0 || K % kGemmBK != 0)
    return set_error(GBSGMC_ERR_SHAPE, "gemm (pairs): needs M %% 256, N %% %d, K %% 64", BN);
  const int64_t tiles = static_cast<int64_t>(M / (2 * kGemmBM)) * (N / BN) * batch;
  const int clusters = static_cast<int>(tiles < max_clusters ? tiles : max_clusters);
  kern<<<2 * clusters, kGemmThreads, smem, st>>>(ta, tb, M, N, K, batch, status, epi, wait_ns);
  return check_launch("tc_gemm2_kernel");
}

}  // namespace gbsgmc
