// Batched BF16 GEMM on the 5th-generation tensor cores:
//   C[b] (M x N, fp32) = A[b] (M x K) * B[b] (N x K)^T,
// A and B row-major with K contiguous ("K-major"), both BF16.
//
// One CTA computes a 128 x BN tile of one batch entry.  Warp 0 (one lane)
// streams 128x64 A tiles and BNx64 B tiles into a 4-stage shared-memory ring
// with TMA (128-byte swizzle), warp 1 allocates BN TMEM columns and one of
// its lanes issues tcgen05.mma (M=128, N=BN, K=16, four per 64-wide K tile),
// committing each stage back to the producer; warps 2-5 read the 128 x BN
// fp32 accumulator out of TMEM (each warp its 32-lane quarter, tcgen05.ld
// 32x32b) and hand 16 columns at a time to the epilogue.  Every wait is
// bounded: after kWaitLimitNs the CTA records GBSGMC_ERR_TIMEOUT, lets the
// work it issued drain, frees its TMEM and returns.
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"
#include "tc_gemm.cuh"

namespace gbsgmc {

namespace {

// Signature of the driver's cuTensorMapEncodeTiled (resolved at run time).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t,
                                   void*, const cuuint64_t*, const cuuint64_t*,
                                   const cuuint32_t*, const cuuint32_t*,
                                   CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

}  // namespace

int make_tmap_bf16_3d(CUtensorMap* map, const void* base, int64_t cols,
                      int64_t rows, int64_t batch, int64_t row_stride,
                      int64_t batch_stride, int box_cols, int box_rows) {
  auto fn = encode_fn();
  if (fn == nullptr)
    return set_error(GBSGMC_ERR_CUDA, "tensor map: cuTensorMapEncodeTiled unavailable");
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || row_stride % 8 != 0 ||
      batch_stride % 8 != 0)
    return set_error(GBSGMC_ERR_ARG,
                     "tensor map: base must be 16-byte aligned and strides "
                     "multiples of 8 elements");
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(cols),
                              static_cast<cuuint64_t>(rows),
                              static_cast<cuuint64_t>(batch)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(row_stride) * 2,
                                 static_cast<cuuint64_t>(batch_stride) * 2};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(box_cols),
                             static_cast<cuuint32_t>(box_rows), 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                        const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(GBSGMC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)",
                     static_cast<int>(r));
  return GBSGMC_OK;
}

namespace {

// Plain fp32 store of the accumulator.
struct StoreF32 {
  float* C;
  int64_t ldc, batch_stride;
  __device__ __forceinline__ void operator()(int b, int row, int col0,
                                             const float (&v)[16]) const {
    float4* out = reinterpret_cast<float4*>(C + b * batch_stride + row * ldc + col0);
#pragma unroll
    for (int i = 0; i < 4; ++i)
      out[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  }
};

}  // namespace

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
#pragma unroll 1
      for (int c = 0; c < BN / 16; ++c) {
        float v[16];
        tc::tmem_ld16(tbase + static_cast<uint32_t>(c * 16), v);
        epi(b, row, n_tile * BN + c * 16, v);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, BN);
  }
}

size_t gemm_smem_bytes(int bn) {
  return 1024 + static_cast<size_t>(kGemmStages) *
                    (kGemmBM * kGemmBK * 2 + static_cast<size_t>(bn) * kGemmBK * 2) +
         (2 * kGemmStages + 1) * 8 + 16;
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

using namespace gbsgmc;

extern "C" int gbsgmc_gemm_bf16_nt(const void* A_dev, int64_t lda,
                                   int64_t a_batch_stride, const void* B_dev,
                                   int64_t ldb, int64_t b_batch_stride,
                                   float* C_dev, int64_t ldc,
                                   int64_t c_batch_stride, int batch, int M,
                                   int N, int K, int* status_dev,
                                   gbsgmc_stream_t stream) {
  if (A_dev == nullptr || B_dev == nullptr || C_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16_nt: null pointer");
  if (batch <= 0 || M <= 0 || N <= 0 || K <= 0)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16_nt: sizes must be positive");
  if (M % kGemmBM != 0 || N % 128 != 0 || K % kGemmBK != 0)
    return set_error(GBSGMC_ERR_SHAPE,
                     "gemm_bf16_nt: needs M %% 128 == 0, N %% 128 == 0, "
                     "K %% 64 == 0 (got %d, %d, %d)", M, N, K);
  if (lda < K || ldb < K || ldc < N || ldc % 4 != 0 ||
      reinterpret_cast<uintptr_t>(C_dev) % 16 != 0)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16_nt: bad leading dimension");
  const bool wide = N % 256 == 0;
  CUtensorMap ta, tb;
  int rc = make_tmap_bf16_3d(&ta, A_dev, K, M, batch, lda, a_batch_stride,
                             kGemmBK, kGemmBM);
  if (rc != GBSGMC_OK) return rc;
  rc = make_tmap_bf16_3d(&tb, B_dev, K, N, batch, ldb, b_batch_stride, kGemmBK,
                         wide ? 256 : 128);
  if (rc != GBSGMC_OK) return rc;
  const StoreF32 epi{C_dev, ldc, c_batch_stride};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return wide ? launch_gemm<256>(ta, tb, batch, M, N, K, status_dev, epi, st)
              : launch_gemm<128>(ta, tb, batch, M, N, K, status_dev, epi, st);
}
