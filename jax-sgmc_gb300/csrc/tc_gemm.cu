// Batched BF16 GEMM on the 5th-generation tensor cores:
//   C[b] (M x N, fp32) = A[b] (M x K) * B[b] (N x K)^T,
// with each operand stored K-major (row-major with K contiguous) or
// MN-major (stored transposed).  The kernel itself (persistent, TMA ring,
// double-buffered TMEM accumulators) is in tc_gemm.cuh so that other
// translation units instantiate it with fused epilogues; this file holds
// the tensor-map encoder and the plain fp32-output entry points.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdlib>
#include <cstring>
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

// Plain fp32 store of the accumulator, one 128-byte row segment per store.
struct StoreF32 {
  float* C;
  int64_t ldc, batch_stride;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    float* dst = C + b * batch_stride + static_cast<int64_t>(row0) * ldc + col0 + epi::lane_id();
#pragma unroll 1
    for (int c = 0; c < NC / 32; ++c) {
      float v[32];
      uint32_t w[32];
      load(c, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) w[j] = __float_as_uint(v[j]);
      epi::put_rows(st, w);
#pragma unroll 4
      for (int r = 0; r < 32; ++r) dst[r * ldc + 32 * c] = __uint_as_float(epi::get(st, r));
    }
  }
};

// Plain BF16 store of the accumulator (round to nearest even): each 64-column
// block of the warp's 32 rows is one TMA store box of `map` (C as [batch,
// M, N]).
struct StoreBF16 {
  CUtensorMap map;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
#pragma unroll 1
    for (int blk = 0; blk < NC / 64; ++blk) {
      float v[64];
      uint32_t w[32];
      load.wide(blk, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        w[j] = *reinterpret_cast<const uint32_t*>(&pr);
      }
      epi::store_box(st, w, &map, col0 + 64 * blk, row0, b);
    }
  }
};

}  // namespace

int make_tmap_bf16_4d_plain(CUtensorMap* map, const void* base, const int64_t (&dims)[4],
                            const int64_t (&strides)[3], const int (&box)[4]) {
  auto fn = encode_fn();
  if (fn == nullptr)
    return set_error(GBSGMC_ERR_CUDA, "tensor map: cuTensorMapEncodeTiled unavailable");
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || strides[0] % 8 != 0 ||
      strides[1] % 8 != 0 || strides[2] % 8 != 0 || box[0] % 8 != 0)
    return set_error(GBSGMC_ERR_ARG,
                     "tensor map (4-D, unswizzled): base 16-byte aligned, strides multiples "
                     "of 8 elements, box rows of whole 16-byte units");
  cuuint64_t d[4], st[3];
  cuuint32_t bx[4], es[4] = {1, 1, 1, 1};
  for (int i = 0; i < 4; ++i) {
    d[i] = static_cast<cuuint64_t>(dims[i]);
    bx[i] = static_cast<cuuint32_t>(box[i]);
  }
  for (int i = 0; i < 3; ++i) st[i] = static_cast<cuuint64_t>(strides[i]) * 2;
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), d,
                        st, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(GBSGMC_ERR_CUDA, "cuTensorMapEncodeTiled (4-D, unswizzled) failed (%d)",
                     static_cast<int>(r));
  return GBSGMC_OK;
}

int make_tmap_rows(CUtensorMap* map, const void* base, bool f32, int64_t cols, int64_t rows,
                   int64_t batch, int64_t row_stride, int64_t batch_stride) {
  auto fn = encode_fn();
  if (fn == nullptr)
    return set_error(GBSGMC_ERR_CUDA, "tensor map: cuTensorMapEncodeTiled unavailable");
  const int es = f32 ? 4 : 2;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || (row_stride * es) % 16 != 0 ||
      (batch_stride * es) % 16 != 0 || (cols * es) % 128 != 0 || rows % 32 != 0)
    return set_error(GBSGMC_ERR_ARG,
                     "output tensor map: base 16-byte aligned, 16-byte strides, rows of "
                     "whole 128-byte boxes, 32-row boxes");
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows),
                              static_cast<cuuint64_t>(batch)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(row_stride) * es,
                                 static_cast<cuuint64_t>(batch_stride) * es};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(128 / es), 32, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r =
      fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
         const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(GBSGMC_ERR_CUDA, "cuTensorMapEncodeTiled (output) failed (%d)",
                     static_cast<int>(r));
  return GBSGMC_OK;
}

int make_tmap_bf16_4d(CUtensorMap* map, const void* base, const int64_t (&dims)[4],
                      const int64_t (&strides)[3], const int (&box)[4]) {
  auto fn = encode_fn();
  if (fn == nullptr)
    return set_error(GBSGMC_ERR_CUDA, "tensor map: cuTensorMapEncodeTiled unavailable");
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || strides[0] % 8 != 0 ||
      strides[1] % 8 != 0 || strides[2] % 8 != 0 || box[0] * 2 != 128)
    return set_error(GBSGMC_ERR_ARG,
                     "tensor map (4-D): base 16-byte aligned, strides multiples of 8 "
                     "elements, 128-byte box rows");
  cuuint64_t d[4], st[3];
  cuuint32_t bx[4], es[4] = {1, 1, 1, 1};
  for (int i = 0; i < 4; ++i) {
    d[i] = static_cast<cuuint64_t>(dims[i]);
    bx[i] = static_cast<cuuint32_t>(box[i]);
  }
  for (int i = 0; i < 3; ++i) st[i] = static_cast<cuuint64_t>(strides[i]) * 2;
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), d,
                        st, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(GBSGMC_ERR_CUDA, "cuTensorMapEncodeTiled (4-D) failed (%d)",
                     static_cast<int>(r));
  return GBSGMC_OK;
}

size_t gemm_smem_bytes(int bn) {
  const int stages = gemm_stages(bn);
  return 1024 + static_cast<size_t>(stages) *
                    (kGemmBM * kGemmBK * 2 + static_cast<size_t>(bn) * kGemmBK * 2) +
         static_cast<size_t>(kGemmEpiWarps) * kStageWords * 4 + (2 * stages + 5) * 8 + 16;
}

size_t gemm2_smem_bytes(int bn) {
  return 1024 + static_cast<size_t>(kGemm2Stages) *
                    (kGemmBM * kGemmBK * 2 + static_cast<size_t>(bn / 2) * kGemmBK * 2) +
         static_cast<size_t>(kGemmEpiWarps) * kStageWords * 4 + (2 * kGemm2Stages + 5) * 8 + 16;
}

bool gemm_pair_enabled() {
  const char* v = std::getenv("GBSGMC_GEMM_PAIR");
  return v == nullptr || std::strcmp(v, "0") != 0;
}

}  // namespace gbsgmc

using namespace gbsgmc;

namespace {

template <class Epi>
int dispatch_pair(bool a_mn, bool b_mn, const CUtensorMap& ta, const CUtensorMap& tb,
                  int batch, int M, int N, int K, int* status, const Epi& epi,
                  cudaStream_t st, uint64_t wait_ns) {
  if (a_mn)
    return b_mn ? launch_gemm2<256, true, true>(ta, tb, batch, M, N, K, status, epi, st, wait_ns)
                : launch_gemm2<256, true, false>(ta, tb, batch, M, N, K, status, epi, st, wait_ns);
  return b_mn ? launch_gemm2<256, false, true>(ta, tb, batch, M, N, K, status, epi, st, wait_ns)
              : launch_gemm2<256, false, false>(ta, tb, batch, M, N, K, status, epi, st, wait_ns);
}

template <int BN, class Epi>
int dispatch_layout(bool a_mn, bool b_mn, const CUtensorMap& ta, const CUtensorMap& tb,
                    int batch, int M, int N, int K, int* status, const Epi& epi,
                    cudaStream_t st, const GemmRagged& rg) {
  if (a_mn)
    return b_mn ? launch_gemm<BN, true, true>(ta, tb, batch, M, N, K, status, epi, st, rg)
                : launch_gemm<BN, true, false>(ta, tb, batch, M, N, K, status, epi, st, rg);
  return b_mn ? launch_gemm<BN, false, true>(ta, tb, batch, M, N, K, status, epi, st, rg)
              : launch_gemm<BN, false, false>(ta, tb, batch, M, N, K, status, epi, st, rg);
}

}  // namespace

extern "C" int gbsgmc_gemm_bf16(int a_mn, int b_mn, const void* A_dev, int64_t lda,
                                int64_t a_batch_stride, const void* B_dev, int64_t ldb,
                                int64_t b_batch_stride, float* C_dev, int64_t ldc,
                                int64_t c_batch_stride, int batch, int M, int N, int K,
                                int* status_dev, gbsgmc_stream_t stream) {
  return gbsgmc_gemm_bf16_wait_limit(a_mn, b_mn, A_dev, lda, a_batch_stride, B_dev, ldb,
                                     b_batch_stride, C_dev, ldc, c_batch_stride, batch, M,
                                     N, K, kWaitLimitNs, status_dev, stream);
}

namespace {

// The plain GEMM with C in fp32 (StoreF32) or BF16 (StoreBF16): checks,
// tensor maps, and the pair or single-CTA kernel.
template <class Epi>
int plain_gemm(int a_mn, int b_mn, const void* A_dev, int64_t lda, int64_t a_batch_stride,
               const void* B_dev, int64_t ldb, int64_t b_batch_stride, const void* C_dev,
               int64_t ldc, int64_t c_batch_stride, int batch, int M, int N, int K,
               uint64_t wait_limit_ns, int* status_dev, gbsgmc_stream_t stream,
               const Epi& epi) {
  if (A_dev == nullptr || B_dev == nullptr || C_dev == nullptr || status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16: null pointer");
  if (batch <= 0 || M <= 0 || N <= 0 || K <= 0 || batch > (1 << 20))
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16: sizes must be positive");
  if (M % kGemmBM != 0 || N % 128 != 0 || K % kGemmBK != 0)
    return set_error(GBSGMC_ERR_SHAPE,
                     "gemm_bf16: needs M %% 128 == 0, N %% 128 == 0, "
                     "K %% 64 == 0 (got %d, %d, %d)", M, N, K);
  if (lda < (a_mn ? M : K) || ldb < (b_mn ? N : K) || ldc < N || ldc % 4 != 0 ||
      reinterpret_cast<uintptr_t>(C_dev) % 16 != 0 || c_batch_stride % 4 != 0)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16: bad leading dimension");
  const int bn = N % 256 == 0 ? 256 : 128;
  // CTA pairs for 256 x 256 tiles; a K-major B is then loaded in halves.
  const bool pair = bn == 256 && M % 256 == 0 && gemm_pair_enabled();
  CUtensorMap ta, tb;
  int rc = a_mn ? make_tmap_bf16_3d(&ta, A_dev, M, K, batch, lda, a_batch_stride, 64, 64)
                : make_tmap_bf16_3d(&ta, A_dev, K, M, batch, lda, a_batch_stride,
                                    kGemmBK, kGemmBM);
  if (rc != GBSGMC_OK) return rc;
  rc = b_mn ? make_tmap_bf16_3d(&tb, B_dev, N, K, batch, ldb, b_batch_stride, 64, 64)
            : make_tmap_bf16_3d(&tb, B_dev, K, N, batch, ldb, b_batch_stride, kGemmBK,
                                pair ? bn / 2 : bn);
  if (rc != GBSGMC_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (pair)
    return dispatch_pair(a_mn, b_mn, ta, tb, batch, M, N, K, status_dev, epi, st, wait_limit_ns);
  GemmRagged rg;
  rg.wait_ns = wait_limit_ns;
  return bn == 256
             ? dispatch_layout<256>(a_mn, b_mn, ta, tb, batch, M, N, K, status_dev, epi, st, rg)
             : dispatch_layout<128>(a_mn, b_mn, ta, tb, batch, M, N, K, status_dev, epi, st, rg);
}

}  // namespace

extern "C" int gbsgmc_gemm_bf16_wait_limit(
    int a_mn, int b_mn, const void* A_dev, int64_t lda, int64_t a_batch_stride,
    const void* B_dev, int64_t ldb, int64_t b_batch_stride, float* C_dev, int64_t ldc,
    int64_t c_batch_stride, int batch, int M, int N, int K, uint64_t wait_limit_ns,
    int* status_dev, gbsgmc_stream_t stream) {
  const StoreF32 epi{C_dev, ldc, c_batch_stride};
  return plain_gemm(a_mn, b_mn, A_dev, lda, a_batch_stride, B_dev, ldb, b_batch_stride, C_dev,
                    ldc, c_batch_stride, batch, M, N, K, wait_limit_ns, status_dev, stream, epi);
}

extern "C" int gbsgmc_gemm_bf16_c16(int a_mn, int b_mn, const void* A_dev, int64_t lda,
                                    int64_t a_batch_stride, const void* B_dev, int64_t ldb,
                                    int64_t b_batch_stride, void* C_dev, int64_t ldc,
                                    int64_t c_batch_stride, int batch, int M, int N, int K,
                                    int* status_dev, gbsgmc_stream_t stream) {
  if (ldc % 8 != 0 || c_batch_stride % 8 != 0)
    return set_error(GBSGMC_ERR_ARG, "gemm_bf16_c16: ldc and the C batch stride must be "
                     "multiples of 8");
  if (batch > 0 && M > 0 && N > 0 && ldc >= N && c_batch_stride >= 0 &&
      (M % 32 != 0 || N % 64 != 0 || reinterpret_cast<uintptr_t>(C_dev) % 16 != 0))
    return set_error(GBSGMC_ERR_SHAPE, "gemm_bf16_c16: needs M %% 32, N %% 64 and a 16-byte "
                     "aligned C");
  StoreBF16 epi;
  if (batch > 0 && M > 0 && N > 0 && ldc >= N && C_dev != nullptr) {
    const int rc = make_tmap_rows(&epi.map, C_dev, false, N, M, batch, ldc,
                                  batch > 1 ? c_batch_stride : int64_t(M) * ldc);
    if (rc != GBSGMC_OK) return rc;
  }
  return plain_gemm(a_mn, b_mn, A_dev, lda, a_batch_stride, B_dev, ldb, b_batch_stride, C_dev,
                    ldc, c_batch_stride, batch, M, N, K, kWaitLimitNs, status_dev, stream, epi);
}

extern "C" int gbsgmc_gemm_bf16_nt(const void* A_dev, int64_t lda,
                                   int64_t a_batch_stride, const void* B_dev,
                                   int64_t ldb, int64_t b_batch_stride,
                                   float* C_dev, int64_t ldc,
                                   int64_t c_batch_stride, int batch, int M,
                                   int N, int K, int* status_dev,
                                   gbsgmc_stream_t stream) {
  return gbsgmc_gemm_bf16(0, 0, A_dev, lda, a_batch_stride, B_dev, ldb, b_batch_stride,
                          C_dev, ldc, c_batch_stride, batch, M, N, K, status_dev, stream);
}
