// Shared declarations of the tcgen05 GEMM (tc_gemm.cu) and its users.
#pragma once

#include <cuda.h>
#include <stddef.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace gbsgmc {

constexpr int kGemmBM = 128;       // rows of a CTA tile (UMMA M)
constexpr int kGemmBK = 64;        // K per stage: one 128-byte swizzle row
constexpr int kGemmStages = 4;     // shared-memory ring depth
constexpr int kGemmThreads = 192;  // producer, MMA, 4 epilogue warps

// 3-D BF16 tensor map (cols innermost, rows, batch) with a 128-byte swizzled
// box of box_cols x box_rows; strides in elements.
int make_tmap_bf16_3d(CUtensorMap* map, const void* base, int64_t cols,
                      int64_t rows, int64_t batch, int64_t row_stride,
                      int64_t batch_stride, int box_cols, int box_rows);

size_t gemm_smem_bytes(int bn);

// Batched GEMM kernel C[b] = A[b] * B[b]^T (see tc_gemm.cu).  Each epilogue
// thread owns one accumulator row of the CTA tile and calls
//   epi.template tile<BN>(batch, row, first column of the tile, load)
// where load(c, v) fills v[16] with columns [16c, 16c + 16) of that row
// (warp-collective: all 32 lanes must call it with the same c).
template <int BN, class Epi>
__global__ void __launch_bounds__(kGemmThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap ta,
                   const __grid_constant__ CUtensorMap tb, int K, int* status,
                   Epi epi) {
  constexpr int BM = kGemmBM, BK = kGemmBK, STAGES = kGemmStages;
  constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint8_t* sa = smem;
  uint8_t* sb = smem + STAGES * A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sb + STAGES * B_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tile = blockIdx.x, m_tile = blockIdx.y, b = blockIdx.z;
  const int KB = K / BK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(accum, 1);
    *abort_flag = 0;
    mbar_fence_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, BN);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = static_cast<uint32_t>(kb / STAGES) & 1u;
        if (!mbar_wait_bounded(&empty[s], ph ^ 1u, abort_flag)) {
          raise_status(status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        mbar_arrive_expect_tx(&full[s], A_BYTES + B_BYTES);
        tc::tma_load_3d(sa + s * A_BYTES, &ta, kb * BK, m_tile * BM, b, &full[s]);
        tc::tma_load_3d(sb + s * B_BYTES, &tb, kb * BK, n_tile * BN, b, &full[s]);
        issued = kb + 1;
      }
      if (*abort_flag) {
        for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb)
          mbar_wait_bounded(&full[kb % STAGES],
                            static_cast<uint32_t>(kb / STAGES) & 1u, nullptr);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = static_cast<uint32_t>(kb / STAGES) & 1u;
        if (!mbar_wait_bounded(&full[s], ph, abort_flag)) {
          raise_status(status, GBSGMC_ERR_TIMEOUT);
          *abort_flag = 1;
          break;
        }
        tc::fence_after_sync();
        const uint64_t a0 = tc::sdesc_k_sw128(sa + s * A_BYTES);
        const uint64_t b0 = tc::sdesc_k_sw128(sb + s * B_BYTES);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)
          tc::mma_bf16(tmem, a0 + 2 * k, b0 + 2 * k, idesc, (kb | k) != 0);
        tc::mma_commit(&empty[s]);
      }
      // Signals the epilogue; also lets every issued MMA finish on abort.
      tc::mma_commit(accum);
      if (*abort_flag) mbar_wait_bounded(accum, 0, nullptr);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const bool ok = mbar_wait_bounded(accum, 0, abort_flag);
    if (!ok && lane == 0) {
      raise_status(status, GBSGMC_ERR_TIMEOUT);
      *abort_flag = 1;
    }
    if (__all_sync(0xffffffffu, ok)) {
      tc::fence_after_sync();
      const int row = m_tile * BM + q * 32 + lane;
      const uint32_t tbase = tmem + (static_cast<uint32_t>(q * 32) << 16);
      auto load = [tbase](int c, float(&v)[16]) {
        tc::tmem_ld16(tbase + static_cast<uint32_t>(c * 16), v);
      };
      epi.template tile<BN>(b, row, n_tile * BN, load);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, BN);
  }
}

template <int BN, class Epi>
int launch_gemm(const CUtensorMap& ta, const CUtensorMap& tb, int batch, int M,
                int N, int K, int* status, const Epi& epi, cudaStream_t st) {
  const size_t smem = gemm_smem_bytes(BN);
  static bool attr = false;
  if (!attr) {
    const cudaError_t e = cudaFuncSetAttribute(
        tc_gemm_kernel<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(smem));
    if (e != cudaSuccess)
      return set_error(GBSGMC_ERR_CUDA, "gemm: cudaFuncSetAttribute: %s",
                       cudaGetErrorString(e));
    attr = true;
  }
  dim3 grid(N / BN, M / kGemmBM, batch);
  tc_gemm_kernel<BN, Epi><<<grid, kGemmThreads, smem, st>>>(ta, tb, K, status, epi);
  return check_launch("tc_gemm_kernel");
}

}  // namespace gbsgmc
