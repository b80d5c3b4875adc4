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
  template <int BN, class Load>
  __device__ __forceinline__ void tile(int b, int row, int col0,
                                       const Load& load) const {
    float* dst = C + b * batch_stride + static_cast<int64_t>(row) * ldc + col0;
#pragma unroll 1
    for (int c = 0; c < BN / 16; ++c) {
      float v[16];
      load(c, v);
      float4* out = reinterpret_cast<float4*>(dst + 16 * c);
#pragma unroll
      for (int i = 0; i < 4; ++i)
        out[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
  }
};

}  // namespace

size_t gemm_smem_bytes(int bn) {
  return 1024 + static_cast<size_t>(kGemmStages) *
                    (kGemmBM * kGemmBK * 2 + static_cast<size_t>(bn) * kGemmBK * 2) +
         (2 * kGemmStages + 1) * 8 + 16;
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
