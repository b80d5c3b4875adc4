// Shared declarations of the tcgen05 GEMM (tc_gemm.cu) and its users.
#pragma once

#include <cuda.h>
#include <stddef.h>
#include <stdint.h>

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

}  // namespace gbsgmc
