// Dense tanh network with a Gaussian likelihood: U, dU/dw, lk and var(lk)
// for many chains at once, the contractions on the tcgen05 tensor cores.
//
// Per chain, with the minibatch X [n, D] (rows gathered by index) and the
// flat parameters W1 [D,H1] | W2 [H1,H2] | W3 [H2] | b1 [H1] | b2 [H2] | b3:
//   forward   A1 = X W1 + b1, Z1 = tanh A1, A2 = Z1 W2 + b2, Z2 = tanh A2,
//             out = Z2 W3 + b3, lk = log N(y | out, sigma^2)
//   adjoint   g  = dU/dout = -(N / (n T)) m (y - out) / sigma^2
//             G2 = (g W3^T) * (1 - Z2^2),  G1 = (G2 W2^T) * (1 - Z1^2)
//             dW3 = Z2^T g, dW2 = Z1^T G2, dW1 = X^T G1, db = column sums,
//             each plus the prior term w / (s^2 T).
// This is the chain rule of jax.value_and_grad over minibatch_potential
// (jax_sgmc/potential.py:159-214, integrator.py:166,593,792) written out by
// hand.  Nothing of the forward pass is kept beyond the BF16 activations the
// adjoint GEMMs consume.
//
// Launch sequence (each batched over chains; GEMMs are C = A B^T on the
// tcgen05 tensor cores, BF16 operands read K-major or MN-major straight from
// where the previous step wrote them, fp32 accumulation in TMEM):
//   1 mlp_prep_kernel     W1 | W2 -> BF16 copy Wb, partial sums of w^2
//   2 mlp_gather_kernel   X rows -> Xb [n,D] (BF16), targets
//   3 GEMM Xb . W1        epilogue tanh(+b1) -> Z1 [n,H1]
//   4 GEMM Z1 . W2        epilogue tanh(+b2) -> Z2 [n,H2], partial Z2 . W3
//   5 mlp_out_kernel      out, lk, g; G2 in place of Z2, partial column sums
//                         for dW3 and db2
//   6 GEMM Z1^T . G2      epilogue -> dW2
//   7 GEMM G2 . W2^T      epilogue *(1 - Z1^2) -> G1 in place of Z1,
//                         partial db1
//   8 GEMM G1^T . Xb      epilogue -> dW1 (written transposed)
//   (steps 6 and 8 add the prior's w / (s^2 T) in their epilogues)
//   9 mlp_finalize_kernel db1, db2, dW3, db3 (with their prior terms), U and
//                         var(lk)
// Without a gradient only 1-5 and 9 run.
//
// The empirical-Fisher noise model (fisher_information(diagonal=True),
// adaption.py:371-457) runs the same sequence with the adjoint seeded by
// d lk_i / d out = (y - out) / sigma^2 (the likelihood's, unscaled), so that
// the GEMMs sum the per-observation gradients d_i, and adds GEMMs on
// squared operands for sum_i d_i^2: (Z1^2)^T (G2^2) after step 6 and
// (G1^2)^T (Xb^2) after step 8 (the squares of the BF16 operands, rounded
// to BF16 by mlp_square_kernel), the output layer's and the biases' sums of
// squares in mlp_out_kernel and mlp_square_kernel.  Then
//   ssq = sum_i (d_i - gbar)^2 = S2 - 2 gbar S1 + n gbar^2,  gbar = G / N
// (clamped at 0 against rounding), and the reference's correction.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.h"
#include "tc_gemm.cuh"

namespace gbsgmc {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTile = 64;      // rows / columns of a prep, gather or out tile
constexpr int kBN = 256;       // N tile of the H1- and H2-wide GEMMs
constexpr int kSlot = kBN / kGemmSplit;  // columns of one epilogue warp

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ void unpack_bf16x2(uint32_t u, float& lo, float& hi) {
  __nv_bfloat162 p = *reinterpret_cast<__nv_bfloat162*>(&u);
  const float2 f = __bfloat1622float2(p);
  lo = f.x;
  hi = f.y;
}

// Sum over the 32 lanes of each of v[0..15]; lane l returns the total of
// column l >> 1 (a transposed butterfly: 16 shuffles instead of 80).
__device__ __forceinline__ float warp_colsum16(const float (&v)[16], int lane) {
  const unsigned full = 0xffffffffu;
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const bool up = lane & 16;
    const float keep = up ? v[j + 8] : v[j], send = up ? v[j] : v[j + 8];
    a[j] = keep + __shfl_xor_sync(full, send, 16);
  }
  float b[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const bool up = lane & 8;
    const float keep = up ? a[j + 4] : a[j], send = up ? a[j] : a[j + 4];
    b[j] = keep + __shfl_xor_sync(full, send, 8);
  }
  float c[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const bool up = lane & 4;
    const float keep = up ? b[j + 2] : b[j], send = up ? b[j] : b[j + 2];
    c[j] = keep + __shfl_xor_sync(full, send, 4);
  }
  const bool up = lane & 2;
  float d = (up ? c[1] : c[0]) + __shfl_xor_sync(full, up ? c[0] : c[1], 2);
  d += __shfl_xor_sync(full, d, 1);
  return d;
}

// Offsets (in floats) of the leaves in a chain's flat parameter vector.
struct MlpShape {
  int D, H1, H2;
  int64_t oW1, oW2, oW3, ob1, ob2, ob3, P;
};

MlpShape mlp_shape(int D, int H1, int H2) {
  MlpShape s;
  s.D = D;
  s.H1 = H1;
  s.H2 = H2;
  s.oW1 = 0;
  s.oW2 = s.oW1 + static_cast<int64_t>(D) * H1;
  s.oW3 = s.oW2 + static_cast<int64_t>(H1) * H2;
  s.ob1 = s.oW3 + H2;
  s.ob2 = s.ob1 + H1;
  s.ob3 = s.ob2 + H2;
  s.P = s.ob3 + 1;
  return s;
}

constexpr int kPrepPairs = 16;                   // weight pairs per prep thread
constexpr int kPrepPerBlock = 2 * 256 * kPrepPairs;  // weights per prep block

__host__ __device__ inline int64_t matrix_params(const MlpShape& s) { return s.oW3; }  // |W1| + |W2|

int prep_blocks(const MlpShape& s) {
  return static_cast<int>((matrix_params(s) + kPrepPerBlock - 1) / kPrepPerBlock) + 1;
}

// Workspace regions, each [chains, per-chain size], 256-byte aligned.
struct MlpLayout {
  size_t wb, xb, z1, z2g;           // BF16
  size_t yv, outp, pw3, pb2, pb1;   // fp32
  size_t psq, plk;                  // fp64
  size_t rag;                       // int tables of a ragged batch
  // Fisher noise model only: squared operands (BF16), partial sums of
  // squares (fp32), U and the smallest positive correction per chain.
  size_t sqa, sqb, pw3sq, pb2sq, pb1sq, fU, fmin;
  size_t total;
};

MlpLayout mlp_layout(const MlpShape& s, int chains, int n, bool fisher = false) {
  MlpLayout L;
  size_t off = 0;
  auto take = [&](size_t bytes_per_chain) {
    const size_t at = off;
    off += (bytes_per_chain * static_cast<size_t>(chains) + 255) & ~static_cast<size_t>(255);
    return at;
  };
  const size_t D = s.D, H1 = s.H1, H2 = s.H2, N = n;
  L.wb = take(2 * static_cast<size_t>(matrix_params(s)));
  L.xb = take(2 * N * D);
  L.z1 = take(2 * N * H1);
  L.z2g = take(2 * N * H2);
  L.yv = take(4 * N);
  L.outp = take(4 * (H2 / kSlot) * N);
  L.pw3 = take(4 * (N / kTile) * H2);
  L.pb2 = take(4 * (N / kTile) * H2);
  L.pb1 = take(4 * (N / 32) * H1);
  L.psq = take(8 * static_cast<size_t>(prep_blocks(s)));
  L.plk = take(8 * 4 * (N / kTile));
  L.rag = take(4 * 5);  // tile prefixes [C + 1] x 2, K slices [C]
  L.sqa = L.sqb = L.pw3sq = L.pb2sq = L.pb1sq = L.fU = L.fmin = 0;
  if (fisher) {
    L.sqa = take(2 * N * H1);
    L.sqb = take(2 * N * (H2 > D ? H2 : D));
    L.pw3sq = take(4 * (N / kTile) * H2);
    L.pb2sq = take(4 * (N / kTile) * H2);
    L.pb1sq = take(4 * (N / kTile) * H1);
    L.fU = take(8);
    L.fmin = take(4);
  }
  L.total = off;
  return L;
}

struct MlpArgs {
  MlpShape s;
  int chains, n, y_inline, want_grad;
  int64_t n_obs, n_rows, ld, idx_stride;
  const float* X;
  const float* y;
  const float* mask;
  const int32_t* idx;
  const float* w;
  float sigma, prior_scale, temperature;
  double* U;
  float* grad;
  float* lk;
  double* lk_var;
  int* status;
  // Ragged batch: rows of chain c are n_true[c] <= n (null: all n).
  const int32_t* n_true;
  // Row c of the batch reads its minibatch from row ident[c] of idx (null: c).
  const int32_t* ident;
  // Fused with the integrator: the BF16 weights and the sums of squares
  // (sq_count per chain in psq) are supplied, the prior's gradient is the
  // update's.
  int fused, sq_count;
  // Fisher noise model: the adjoint is the likelihood's (grad receives
  // sum_i d_i), grad_sq receives sum_i d_i^2.
  int fisher;
  float* grad_sq;
  float *pw3sq, *pb2sq, *pb1sq;
  bf16 *sqa, *sqb;
  uint32_t* fmin;
  int *prefix1, *prefix2, *kblocks;
  // workspace views
  bf16 *wb, *xb, *z1, *z2g;
  float *yv, *outp, *pw3, *pb2, *pb1;
  double *psq, *plk;
};

// Rows of chain c, and the rows its GEMMs cover (a multiple of 128).
__device__ __forceinline__ int chain_rows(const MlpArgs& a, int c) {
  if (a.n_true == nullptr) return a.n;
  const int v = __ldg(a.n_true + c);
  return v < 1 ? 1 : (v > a.n ? a.n : v);
}
__device__ __forceinline__ int chain_rows_padded(const MlpArgs& a, int c) {
  return (chain_rows(a, c) + 127) & ~127;
}

// Tile tables of a ragged batch for the GEMMs (one thread).
__global__ void mlp_ragged_kernel(const MlpArgs a) {
  int p1 = 0, p2 = 0;
  a.prefix1[0] = 0;
  a.prefix2[0] = 0;
  for (int c = 0; c < a.chains; ++c) {
    const int v = __ldg(a.n_true + c);
    if (v < 1 || v > a.n) raise_status(a.status, GBSGMC_ERR_SHAPE);
    const int np = chain_rows_padded(a, c);
    p1 += (np / 128) * (a.s.H1 / kBN);
    p2 += (np / 128) * (a.s.H2 / kBN);
    a.prefix1[c + 1] = p1;
    a.prefix2[c + 1] = p2;
    a.kblocks[c] = np / kGemmBK;
  }
}

// ---------------------------------------------------------------------------
// 1. W1 | W2 to BF16 (same layout) and partial sums of squares of every
//    parameter.  Grid (prep_blocks, chains); the last block of a chain sums
//    the vector leaves W3 | b1 | b2 | b3.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_prep_kernel(const MlpArgs a) {
  __shared__ double red[32];
  const MlpShape& s = a.s;
  const int c = blockIdx.y, blk = blockIdx.x, t = threadIdx.x;
  const float* w = a.w + static_cast<int64_t>(c) * s.P;
  const int64_t pw = matrix_params(s);
  float sq = 0.f;
  if (blk + 1 < static_cast<int>(gridDim.x)) {
    uint32_t* dst = reinterpret_cast<uint32_t*>(a.wb + static_cast<int64_t>(c) * pw);
    const int64_t e0 = static_cast<int64_t>(blk) * kPrepPerBlock + 2 * t;
    float v0[kPrepPairs], v1[kPrepPairs];
#pragma unroll
    for (int k = 0; k < kPrepPairs; ++k) {  // pw is even: pairs never straddle the end
      const int64_t e = e0 + 512 * k;
      v0[k] = e < pw ? __ldg(w + e) : 0.f;
      v1[k] = e < pw ? __ldg(w + e + 1) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kPrepPairs; ++k) {
      const int64_t e = e0 + 512 * k;
      sq = fmaf(v0[k], v0[k], fmaf(v1[k], v1[k], sq));
      if (e < pw) dst[e >> 1] = pack_bf16x2(v0[k], v1[k]);
    }
  } else {
    for (int64_t i = pw + t; i < s.P; i += 256) {
      const float v = __ldg(w + i);
      sq = fmaf(v, v, sq);
    }
  }
  const double tot = block_sum(static_cast<double>(sq), red);
  if (t == 0) a.psq[static_cast<int64_t>(c) * gridDim.x + blk] = tot;
}

// ---------------------------------------------------------------------------
// 2. Minibatch rows to BF16 plus targets.
//    Grid (n/64, D/64, chains).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_gather_kernel(const MlpArgs a) {
  __shared__ int64_t rows[kTile];
  const MlpShape& s = a.s;
  const int i0 = blockIdx.x * kTile, f0 = blockIdx.y * kTile, c = blockIdx.z;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int nc = chain_rows(a, c);
  if (i0 >= chain_rows_padded(a, c)) return;
  if (t < kTile) {
    // Rows past the chain's minibatch (ragged batches) are zero.
    int64_t o = -1;
    if (i0 + t < nc) {
      const int ic = a.ident != nullptr ? __ldg(a.ident + c) : c;
      o = a.idx[static_cast<int64_t>(ic) * a.idx_stride + i0 + t];
      if (o < 0 || o >= a.n_rows) {
        raise_status(a.status, GBSGMC_ERR_INDEX);
        o = 0;
      }
    }
    rows[t] = o;
    if (blockIdx.y == 0) {
      const float yy = o < 0 ? 0.f : a.y_inline ? __ldg(a.X + o * a.ld + s.D) : __ldg(a.y + o);
      a.yv[static_cast<int64_t>(c) * a.n + i0 + t] = yy;
    }
  }
  __syncthreads();
  bf16* xb = a.xb + static_cast<int64_t>(c) * a.n * s.D;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int r = warp * 8 + j;
    float v0 = 0.f, v1 = 0.f;
    if (rows[r] >= 0) {
      const float* src = a.X + rows[r] * a.ld + f0;
      v0 = __ldg(src + lane);
      v1 = __ldg(src + 32 + lane);
    }
    bf16* d = xb + static_cast<int64_t>(i0 + r) * s.D + f0;
    d[lane] = __float2bfloat16_rn(v0);
    d[lane + 32] = __float2bfloat16_rn(v1);
  }
}

// ---------------------------------------------------------------------------
// GEMM epilogues.
// ---------------------------------------------------------------------------

// Bias + tanh over one 64-column block of the lane's row, packed to BF16
// pairs: pk[j] holds columns 2j, 2j + 1 of the block.  With w3 the fp32 dot
// product of the block with w3 is added to `dot`.  The column vectors are
// read once per 32 columns, lane l holding column l, and broadcast by
// shuffles (a load per element kept the warps waiting on L1).
template <class Load>
__device__ __forceinline__ void tanh_block(const Load& load, int blk, const float* bias,
                                           uint32_t (&pk)[32], const float* w3, float& dot) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  float dot2 = 0.f;  // odd columns: two independent FMA chains
  const float bl0 = __ldg(bias + 64 * blk + lane);
  const float bl1 = __ldg(bias + 64 * blk + 32 + lane);
  const float wl0 = w3 != nullptr ? __ldg(w3 + 64 * blk + lane) : 0.f;
  const float wl1 = w3 != nullptr ? __ldg(w3 + 64 * blk + 32 + lane) : 0.f;
  float vv[64];
  load.wide(blk, vv);  // one wait for the block's 64 columns
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const float bl = half ? bl1 : bl0;
    const float wl = half ? wl1 : wl0;
    const float* v = vv + 32 * half;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float z0 = tanh_approx(v[2 * j] + __shfl_sync(full, bl, 2 * j));
      const float z1 = tanh_approx(v[2 * j + 1] + __shfl_sync(full, bl, 2 * j + 1));
      if (w3 != nullptr) {
        dot = fmaf(z0, __shfl_sync(full, wl, 2 * j), dot);
        dot2 = fmaf(z1, __shfl_sync(full, wl, 2 * j + 1), dot2);
      }
      pk[16 * half + j] = pack_bf16x2(z0, z1);
    }
  }
  dot += dot2;
}

// 3: Z1 = tanh(acc + b1) -> Z1 [n, H1]; each packed 64-column block of the
//    warp's rows leaves as one TMA store box of zmap (Z1 as [chains, n, H1]).
struct EpiHidden1 {
  const float* w;
  int64_t P, ob1;
  CUtensorMap zmap;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    const float* b1 = w + b * P + ob1 + col0;
    float unused = 0.f;
#pragma unroll 1
    for (int blk = 0; blk < NC / 64; ++blk) {
      uint32_t pk[32];
      tanh_block(load, blk, b1, pk, nullptr, unused);
      epi::store_box(st, pk, &zmap, col0 + 64 * blk, row0, b);
    }
  }
};

// 4: Z2 = tanh(acc + b2) -> Z2 [n, H2] (TMA store boxes of zmap, Z2 as
//    [chains, n, H2]); the fp32 partial Z2 . W3 over the warp's NC columns
//    -> outp [H2 / NC, n].
struct EpiHidden2 {
  const float* w;
  int64_t P, ob2, oW3;
  int H2, n;
  float* outp;
  CUtensorMap zmap;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    const float* b2 = w + b * P + ob2 + col0;
    const float* w3 = w + b * P + oW3 + col0;
    float dot = 0.f;
#pragma unroll 1
    for (int blk = 0; blk < NC / 64; ++blk) {
      uint32_t pk[32];
      tanh_block(load, blk, b2, pk, w3, dot);
      epi::store_box(st, pk, &zmap, col0 + 64 * blk, row0, b);
    }
    outp[(static_cast<int64_t>(b) * (H2 / NC) + col0 / NC) * n + row0 + epi::lane_id()] = dot;
  }
};

// 7: G1 = acc * (1 - Z1^2) written over Z1 [n, H1] (the block is read with
//    asynchronous copies into the warp's staging tile and rewritten, as a
//    TMA store box, by the same warp); per-warp column sums -> pb1
//    [n/32, H1].
struct EpiAdjoint1 {
  bf16* z1;
  float* pb1;
  int H1, n;
  CUtensorMap zmap;  // Z1 as [chains, n, H1], boxes of 64 columns x 32 rows
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    const int lane = epi::lane_id();
    const char* zsrc = reinterpret_cast<const char*>(z1 + (static_cast<int64_t>(b) * n + row0) * H1 +
                                                     col0);
    float* part = pb1 + (static_cast<int64_t>(b) * (n / 32) + row0 / 32) * H1 + col0;
#pragma unroll 1
    for (int blk = 0; blk < NC / 64; ++blk) {
      // The Z1 block is copied into the staging tile (cp.async) and the
      // accumulator's 64 columns requested; both arrive together.
      epi::fetch_box(st, zsrc + 128 * blk, static_cast<int64_t>(H1) * 2);
      uint32_t acc[64];
      load.wide_start(blk, acc);
      uint32_t zw[32];
      epi::fetch_wait();
      epi::read_row(st, zw);
      tc::tmem_ld64_wait(acc);
      float vv[64];
#pragma unroll
      for (int i = 0; i < 64; ++i) vv[i] = __uint_as_float(acc[i]);
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        float* v = vv + 32 * half;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float za, zb;
          unpack_bf16x2(zw[16 * half + j], za, zb);
          v[2 * j] *= 1.f - za * za;
          v[2 * j + 1] *= 1.f - zb * zb;
          zw[16 * half + j] = pack_bf16x2(v[2 * j], v[2 * j + 1]);
        }
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          float v16[16];
#pragma unroll
          for (int k = 0; k < 16; ++k) v16[k] = v[16 * g + k];
          const float cs = warp_colsum16(v16, lane);
          if ((lane & 1) == 0) part[64 * blk + 32 * half + 16 * g + (lane >> 1)] = cs;
        }
      }
      epi::store_box(st, zw, &zmap, col0 + 64 * blk, row0, b);
    }
  }
};

// 6: gradient of a row-major weight matrix (GEMM row = matrix row),
//    grad[b*P + off + row*ld + col] = acc + pf w at the same index (pf the
//    prior's 1 / (s^2 T); 0 leaves the likelihood term alone and reads no w).
struct EpiGradRows {
  float* grad;
  int64_t P, off, ld;
  const float* w = nullptr;
  float pf = 0.f;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    const int64_t at = b * P + off + row0 * ld + col0 + epi::lane_id();
    float* dst = grad + at;
    const float* src = w + at;
#pragma unroll 1
    for (int c = 0; c < NC / 32; ++c) {
      // The prior's w of the 32 x 32 block (row r in wv[r], lane = column)
      // is requested before the accumulator load, whose wait covers it.
      float wv[32];
      if (pf != 0.f) {
#pragma unroll
        for (int r = 0; r < 32; ++r) wv[r] = __ldg(src + r * ld + 32 * c);
      }
      float v[32];
      uint32_t u[32];
      load(c, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) u[j] = __float_as_uint(v[j]);
      epi::put_rows(st, u);
      if (pf != 0.f) {
#pragma unroll
        for (int r = 0; r < 32; ++r)
          dst[r * ld + 32 * c] = fmaf(pf, wv[r], __uint_as_float(epi::get(st, r)));
      } else {
#pragma unroll 4
        for (int r = 0; r < 32; ++r) dst[r * ld + 32 * c] = __uint_as_float(epi::get(st, r));
      }
    }
  }
};

// 8: gradient of a matrix stored transposed to the GEMM (GEMM row = matrix
//    column): grad[b*P + off + col*ld + row] = acc + pf w; lanes hold
//    consecutive rows, so each access is already one contiguous segment.
struct EpiGradCols {
  float* grad;
  int64_t P, off, ld;
  const float* w = nullptr;
  float pf = 0.f;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t*) const {
    const int64_t at = b * P + off + row0 + epi::lane_id();
    float* dst = grad + at;
    const float* src = w + at;
#pragma unroll 1
    for (int c = 0; c < NC / 32; ++c) {
      float wv[32];
      if (pf != 0.f) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
          wv[j] = __ldg(src + static_cast<int64_t>(col0 + 32 * c + j) * ld);
      }
      float v[32];
      load(c, v);
      if (pf != 0.f) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
          dst[static_cast<int64_t>(col0 + 32 * c + j) * ld] = fmaf(pf, wv[j], v[j]);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) dst[static_cast<int64_t>(col0 + 32 * c + j) * ld] = v[j];
      }
    }
  }
};

// ---------------------------------------------------------------------------
// 5. Output layer, likelihood and the first adjoint for 64 rows of a chain.
//    Grid (n/64, chains).  With a gradient the block then streams its
//    64 x H2 block of Z2 in 16-byte vectors, writes G2 over it and leaves
//    per-block column sums for dW3 (sum_i g_i Z2_ij) and db2 (sum_i G2_ij).
// ---------------------------------------------------------------------------
template <bool kFisher>
__global__ void __launch_bounds__(256) mlp_out_kernel(const MlpArgs a) {
  constexpr int kParts = kFisher ? 4 : 2;
  __shared__ float g_s[kTile];
  __shared__ double red[2][4];
  __shared__ float colp[kParts][256 * 8];
  const MlpShape& s = a.s;
  const int c = blockIdx.y, rb = blockIdx.x, i0 = rb * kTile;
  const int t = threadIdx.x, lane = t & 31;
  const float* w = a.w + static_cast<int64_t>(c) * s.P;
  const int nc = chain_rows(a, c);
  if (i0 >= chain_rows_padded(a, c)) {
    if (a.lk != nullptr && t < kTile) a.lk[static_cast<int64_t>(c) * a.n + i0 + t] = 0.f;
    return;
  }
  if (a.want_grad) {
    // The block's 64 x H2 tile of Z2 is brought into L2 while the output
    // layer below runs (one 128-byte line per prefetch).
    const char* zt = reinterpret_cast<const char*>(a.z2g + (static_cast<int64_t>(c) * a.n + i0) *
                                                              s.H2);
    const int lines = kTile * s.H2 * 2 / 128;
    for (int q = t; q < lines; q += 256)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(zt + static_cast<int64_t>(q) * 128));
  }
  if (t < kTile) {
    const float inv_s2 = 1.f / (a.sigma * a.sigma);
    const float scale = static_cast<float>(static_cast<double>(a.n_obs) / nc / a.temperature);
    const int i = i0 + t;
    const bool live = i < nc;  // rows past a ragged chain's minibatch add nothing
    const int nslot = s.H2 / kSlot;
    float out = __ldg(w + s.ob3);
    for (int q = 0; q < nslot; ++q) out += a.outp[(static_cast<int64_t>(c) * nslot + q) * a.n + i];
    const float r = a.yv[static_cast<int64_t>(c) * a.n + i] - out;
    const float lk = -0.5f * r * r * inv_s2 - logf(a.sigma) - 0.91893853320467274f;
    const float m = !live ? 0.f
                    : a.mask != nullptr ? __ldg(a.mask + static_cast<int64_t>(c) * a.n + i)
                                        : 1.f;
    // The Fisher model differentiates lk_i itself: d lk_i / d out = r / s^2.
    const float g = kFisher ? (live ? r * inv_s2 : 0.f) : -scale * m * r * inv_s2;
    g_s[t] = g;
    if (a.lk != nullptr) a.lk[static_cast<int64_t>(c) * a.n + i] = live ? lk : 0.f;
    // var(lk) is over all n values, masked or not (jnp.var, integrator.py:880).
    const double lkl = live ? lk : 0.0;
    // Slot 0 is sum_i g_i^2 (b3's sum of squares) in the Fisher model.
    double v4[4] = {kFisher ? static_cast<double>(g) * g : static_cast<double>(m) * lkl, lkl,
                    lkl * lkl, g};
#pragma unroll
    for (int k = 0; k < 4; ++k) v4[k] = warp_sum(v4[k]);
    if (lane == 0)
      for (int k = 0; k < 4; ++k) red[t >> 5][k] = v4[k];
  }
  __syncthreads();
  if (t == 0) {
    double* p = a.plk + (static_cast<int64_t>(c) * (a.n / kTile) + rb) * 4;
    for (int k = 0; k < 4; ++k) p[k] = red[0][k] + red[1][k];
  }
  if (!a.want_grad) return;
  // Threads: CT column threads (8 columns each) x RG row groups.
  const int cpr = s.H2 / 8;
  const int CT = cpr < 256 ? cpr : 256, RG = 256 / CT;
  const int ct = t % CT, rg = t / CT;
  uint4* z2 = reinterpret_cast<uint4*>(a.z2g + (static_cast<int64_t>(c) * a.n + i0) * s.H2);
  // Every thread runs the same number of passes (the barriers below).
  for (int base = 0; base < cpr; base += CT) {
    const int ch = base + ct;
    const bool active = ch < cpr;
    float w3[8], aw[8], ab[8], aw2[8], ab2[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      w3[k] = active ? __ldg(w + s.oW3 + 8 * ch + k) : 0.f;
      aw[k] = 0.f;
      ab[k] = 0.f;
      aw2[k] = 0.f;
      ab2[k] = 0.f;
    }
    for (int r0 = rg; active && r0 < kTile; r0 += 8 * RG) {
      uint4 cell[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (r0 + k * RG < kTile) cell[k] = z2[static_cast<int64_t>(r0 + k * RG) * cpr + ch];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int r = r0 + k * RG;
        if (r >= kTile) break;
        const float g = g_s[r];
        uint32_t* u = reinterpret_cast<uint32_t*>(&cell[k]);
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float za, zb;
          unpack_bf16x2(u[h], za, zb);
          const float ga = g * w3[2 * h] * (1.f - za * za);
          const float gb = g * w3[2 * h + 1] * (1.f - zb * zb);
          aw[2 * h] = fmaf(g, za, aw[2 * h]);
          aw[2 * h + 1] = fmaf(g, zb, aw[2 * h + 1]);
          ab[2 * h] += ga;
          ab[2 * h + 1] += gb;
          if (kFisher) {
            const float da = g * za, db = g * zb;
            aw2[2 * h] = fmaf(da, da, aw2[2 * h]);
            aw2[2 * h + 1] = fmaf(db, db, aw2[2 * h + 1]);
            ab2[2 * h] = fmaf(ga, ga, ab2[2 * h]);
            ab2[2 * h + 1] = fmaf(gb, gb, ab2[2 * h + 1]);
          }
          u[h] = pack_bf16x2(ga, gb);
        }
        z2[static_cast<int64_t>(r) * cpr + ch] = cell[k];
      }
    }
    // Column sums over the RG row groups.
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      colp[0][t * 8 + k] = aw[k];
      colp[1][t * 8 + k] = ab[k];
      if (kFisher) {
        colp[kParts - 2][t * 8 + k] = aw2[k];
        colp[kParts - 1][t * 8 + k] = ab2[k];
      }
    }
    __syncthreads();
    if (rg == 0 && active) {
      const int64_t pr = (static_cast<int64_t>(c) * (a.n / kTile) + rb) * s.H2 + 8 * ch;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        float sw = 0.f, sb = 0.f, sw2 = 0.f, sb2 = 0.f;
        for (int q = 0; q < RG; ++q) {
          sw += colp[0][(q * CT + ct) * 8 + k];
          sb += colp[1][(q * CT + ct) * 8 + k];
          if (kFisher) {
            sw2 += colp[kParts - 2][(q * CT + ct) * 8 + k];
            sb2 += colp[kParts - 1][(q * CT + ct) * 8 + k];
          }
        }
        a.pw3[pr + k] = sw;
        a.pb2[pr + k] = sb;
        if (kFisher) {
          a.pw3sq[pr + k] = sw2;
          a.pb2sq[pr + k] = sb2;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 9. Bias and output-layer gradients, U and var(lk).  Grid
//    (ceil(max(H1,H2)/256), chains) with a gradient, (1, chains) without.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_finalize_kernel(const MlpArgs a, int nprep) {
  __shared__ double red[32];
  const MlpShape& s = a.s;
  const int c = blockIdx.y, t = threadIdx.x;
  const float* w = a.w + static_cast<int64_t>(c) * s.P;
  const double s2 = static_cast<double>(a.prior_scale) * a.prior_scale;
  const float pf = a.prior_scale > 0.f && !a.fused && !a.fisher
                       ? static_cast<float>(1.0 / (s2 * a.temperature))
                       : 0.f;
  const int nc = chain_rows(a, c), npad = chain_rows_padded(a, c);
  const int nb64 = npad / kTile, nb32 = npad / 32;
  if (a.want_grad) {
    float* g = a.grad + static_cast<int64_t>(c) * s.P;
    const int j = blockIdx.x * 256 + t;
    if (j < s.H1) {
      const float* p = a.pb1 + static_cast<int64_t>(c) * (a.n / 32) * s.H1 + j;
      float acc = 0.f;
      for (int r = 0; r < nb32; ++r) acc += p[static_cast<int64_t>(r) * s.H1];
      g[s.ob1 + j] = fmaf(pf, __ldg(w + s.ob1 + j), acc);
      if (a.fisher) {
        const float* q = a.pb1sq + static_cast<int64_t>(c) * (a.n / kTile) * s.H1 + j;
        float sq = 0.f;
        for (int r = 0; r < nb64; ++r) sq += q[static_cast<int64_t>(r) * s.H1];
        a.grad_sq[static_cast<int64_t>(c) * s.P + s.ob1 + j] = sq;
      }
    }
    if (j < s.H2) {
      const int64_t base = static_cast<int64_t>(c) * (a.n / kTile) * s.H2 + j;
      float acc2 = 0.f, acc3 = 0.f;
      for (int r = 0; r < nb64; ++r) {
        acc2 += a.pb2[base + static_cast<int64_t>(r) * s.H2];
        acc3 += a.pw3[base + static_cast<int64_t>(r) * s.H2];
      }
      g[s.ob2 + j] = fmaf(pf, __ldg(w + s.ob2 + j), acc2);
      g[s.oW3 + j] = fmaf(pf, __ldg(w + s.oW3 + j), acc3);
      if (a.fisher) {
        float sq2 = 0.f, sq3 = 0.f;
        for (int r = 0; r < nb64; ++r) {
          sq2 += a.pb2sq[base + static_cast<int64_t>(r) * s.H2];
          sq3 += a.pw3sq[base + static_cast<int64_t>(r) * s.H2];
        }
        a.grad_sq[static_cast<int64_t>(c) * s.P + s.ob2 + j] = sq2;
        a.grad_sq[static_cast<int64_t>(c) * s.P + s.oW3 + j] = sq3;
      }
    }
  }
  if (blockIdx.x != 0) return;
  double sq = 0.0, lm = 0.0, l1 = 0.0, l2 = 0.0, gs = 0.0;
  for (int i = t; i < nprep; i += 256) sq += a.psq[static_cast<int64_t>(c) * nprep + i];
  for (int i = t; i < nb64; i += 256) {
    const double* p = a.plk + (static_cast<int64_t>(c) * (a.n / kTile) + i) * 4;
    lm += p[0];
    l1 += p[1];
    l2 += p[2];
    gs += p[3];
  }
  sq = block_sum(sq, red);
  lm = block_sum(lm, red);
  l1 = block_sum(l1, red);
  l2 = block_sum(l2, red);
  gs = block_sum(gs, red);
  if (t != 0) return;
  if (a.fisher) {
    // b3: sum_i g_i and sum_i g_i^2; the correction's minimum starts at +inf.
    a.grad[static_cast<int64_t>(c) * s.P + s.ob3] = static_cast<float>(gs);
    a.grad_sq[static_cast<int64_t>(c) * s.P + s.ob3] = static_cast<float>(lm);
    a.fmin[c] = 0x7f800000u;
    return;
  }
  double log_prior = 0.0;
  if (a.prior_scale > 0.f)
    log_prior = -0.5 * sq / s2 -
                static_cast<double>(s.P) * (log(static_cast<double>(a.prior_scale)) +
                                            0.91893853320467274178);
  // -N * mean(lk) without a mask, -N/n * (lk . mask) with one (potential.py:183-185).
  const double lik = -static_cast<double>(a.n_obs) * (lm / nc);
  const double U = (lik - log_prior) / a.temperature;
  a.U[c] = U;
  if (a.lk_var != nullptr) {
    const double mean = l1 / nc;
    a.lk_var[c] = fmax(l2 / nc - mean * mean, 0.0);
  }
  if (!isfinite(U)) raise_status(a.status, GBSGMC_ERR_NONFINITE);
  if (a.want_grad)
    a.grad[static_cast<int64_t>(c) * s.P + s.ob3] =
        static_cast<float>(gs) + pf * __ldg(w + s.ob3);
}

// Squares of a BF16 matrix [n, H] per chain (blockIdx.z), rounded to BF16,
// and with `colsq` the fp32 column sums of the squares of each 64-row block
// -> colsq [chains, n / 64, H].  Grid (n / 64, H / 64, chains).
__global__ void __launch_bounds__(256) mlp_square_kernel(const bf16* __restrict__ src,
                                                         bf16* __restrict__ dst, int n, int H,
                                                         float* colsq) {
  __shared__ float part[32][65];
  const int t = threadIdx.x, cc = t & 7, rg = t >> 3;
  const int64_t base = static_cast<int64_t>(blockIdx.z) * n * H;
  const int r0 = blockIdx.x * kTile, col = blockIdx.y * 64 + 8 * cc;
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int64_t e = base + static_cast<int64_t>(r0 + rg + 32 * k) * H + col;
    uint4 v = *reinterpret_cast<const uint4*>(src + e);
    uint32_t* u = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      float x0, x1;
      unpack_bf16x2(u[h], x0, x1);
      const float q0 = x0 * x0, q1 = x1 * x1;  // exact: 8-bit significands
      acc[2 * h] += q0;
      acc[2 * h + 1] += q1;
      u[h] = pack_bf16x2(q0, q1);
    }
    *reinterpret_cast<uint4*>(dst + e) = v;
  }
  if (colsq == nullptr) return;
#pragma unroll
  for (int k = 0; k < 8; ++k) part[rg][8 * cc + k] = acc[k];
  __syncthreads();
  if (t < 64) {
    float sum = 0.f;
    for (int r = 0; r < 32; ++r) sum += part[r][t];
    colsq[(static_cast<int64_t>(blockIdx.z) * (n / kTile) + blockIdx.x) * H + blockIdx.y * 64 + t] =
        sum;
  }
}

// Fisher noise, first pass: with S1 = sum_i d_i (in bs) and S2 = sum_i d_i^2
// (in cb), corr = friction - 0.5 h max(S2 - 2 gbar S1 + n gbar^2, 0) / (n - 1)
// is written over S2 and the chain's smallest positive corr is kept in
// fmin (as its bit pattern: positive floats order like their bits).  Grid
// (blocks over P, chains).
__global__ void __launch_bounds__(256) mlp_fisher_corr_kernel(
    int64_t P, int n, float n_obs, float h, const float* __restrict__ grad,
    const float* __restrict__ fric, float friction, const float* __restrict__ s1, float* s2,
    uint32_t* fmin) {
  __shared__ float red[8];
  const int c = blockIdx.y;
  const float scale_v = 1.0f / static_cast<float>(n - 1);
  const float nf = static_cast<float>(n);
  float m = INFINITY;
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x; p < P;
       p += static_cast<int64_t>(gridDim.x) * 256) {
    const int64_t e = static_cast<int64_t>(c) * P + p;
    const float gbar = grad[e] / n_obs;
    const float ssq = fmaxf(fmaf(nf * gbar, gbar, fmaf(-2.0f * gbar, s1[e], s2[e])), 0.f);
    const float b = 0.5f * h * (scale_v * ssq);
    const float corr = (fric != nullptr ? fric[p] : friction) - b;
    s2[e] = corr;
    if (corr > 0.f) m = fminf(m, corr);
  }
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) m = fminf(m, red[w]);
    if (m < INFINITY) atomicMin(fmin + c, __float_as_uint(m));
  }
}

// Second pass: corr <= 0 -> the smallest positive corr (+inf when none, as
// jnp.min over an all-inf array gives); cb = sqrt(corr), bs = sqrt(f - corr).
__global__ void __launch_bounds__(256) mlp_fisher_apply_kernel(int64_t P,
                                                               const float* __restrict__ fric,
                                                               float friction,
                                                               const uint32_t* __restrict__ fmin,
                                                               float* cb, float* bs) {
  const int c = blockIdx.y;
  const float smallest = __uint_as_float(fmin[c]);
  for (int64_t p = static_cast<int64_t>(blockIdx.x) * 256 + threadIdx.x; p < P;
       p += static_cast<int64_t>(gridDim.x) * 256) {
    const int64_t e = static_cast<int64_t>(c) * P + p;
    const float corr = cb[e];
    const float pc = corr <= 0.f ? smallest : corr;
    cb[e] = sqrtf(pc);
    bs[e] = sqrtf((fric != nullptr ? fric[p] : friction) - pc);
  }
}

}  // namespace
}  // namespace gbsgmc

namespace gbsgmc {
namespace {

int check_model(const gbsgmc_mlp* m, const char* who) {
  if (m == nullptr || m->X == nullptr)
    return set_error(GBSGMC_ERR_ARG, "%s: null model or data", who);
  if (m->d_in < 64 || m->d_in % 64 != 0 || m->h1 < 256 || m->h1 % 256 != 0 ||
      m->h2 < 256 || m->h2 % 256 != 0 || m->d_in > 4096 || m->h1 > 16384 ||
      m->h2 > 16384)
    return set_error(GBSGMC_ERR_SHAPE,
                     "%s: needs d_in %% 64 == 0, h1 %% 256 == 0, h2 %% 256 == 0 "
                     "(got %d, %d, %d)", who, m->d_in, m->h1, m->h2);
  if (m->y_inline ? m->ld < m->d_in + 1 : (m->ld < m->d_in || m->y == nullptr))
    return set_error(GBSGMC_ERR_ARG, "%s: bad ld or missing targets", who);
  if (m->n_obs < 1 || m->n_rows < 0 || m->n_rows >= (1ll << 31) ||
      (m->n_rows == 0 && m->n_obs >= (1ll << 31)))
    return set_error(GBSGMC_ERR_ARG, "%s: bad n_obs or n_rows", who);
  if (!(m->sigma > 0.f) || !(m->temperature > 0.f) || !(m->prior_scale >= 0.f))
    return set_error(GBSGMC_ERR_ARG,
                     "%s: sigma and temperature must be positive, "
                     "prior_scale >= 0", who);
  return GBSGMC_OK;
}

template <class T>
T* view(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<unsigned char*>(ws) + off);
}

// A 256-wide GEMM of the network: on CTA pairs (tc_gemm2_kernel) for uniform
// batches whose M is a multiple of 256, else on single CTAs.  tb_pair is the
// B map for pairs (a K-major B is loaded in 128-row halves there).
template <bool A_MN, bool B_MN, class Epi>
int gemm256(const CUtensorMap& ta, const CUtensorMap& tb, const CUtensorMap& tb_pair, int C,
            int M, int N, int K, int* status, const Epi& e, cudaStream_t st,
            const GemmRagged& rg, bool uniform) {
  if (uniform && M % 256 == 0 && gemm_pair_enabled())
    return launch_gemm2<kBN, A_MN, B_MN>(ta, tb_pair, C, M, N, K, status, e, st);
  return launch_gemm<kBN, A_MN, B_MN>(ta, tb, C, M, N, K, status, e, st, rg);
}

int run_mlp(MlpArgs& a, const MlpLayout& L, void* ws, cudaStream_t st) {
  const MlpShape& s = a.s;
  a.wb = view<bf16>(ws, L.wb);
  a.xb = view<bf16>(ws, L.xb);
  a.z1 = view<bf16>(ws, L.z1);
  a.z2g = view<bf16>(ws, L.z2g);
  a.yv = view<float>(ws, L.yv);
  a.outp = view<float>(ws, L.outp);
  a.pw3 = view<float>(ws, L.pw3);
  a.pb2 = view<float>(ws, L.pb2);
  a.pb1 = view<float>(ws, L.pb1);
  if (!a.fused) a.psq = view<double>(ws, L.psq);
  a.plk = view<double>(ws, L.plk);
  if (a.fisher) {
    a.sqa = view<bf16>(ws, L.sqa);
    a.sqb = view<bf16>(ws, L.sqb);
    a.pw3sq = view<float>(ws, L.pw3sq);
    a.pb2sq = view<float>(ws, L.pb2sq);
    a.pb1sq = view<float>(ws, L.pb1sq);
    a.fmin = view<uint32_t>(ws, L.fmin);
  }
  a.prefix1 = view<int>(ws, L.rag);
  a.prefix2 = a.prefix1 + (a.chains + 1);
  a.kblocks = a.prefix2 + (a.chains + 1);
  const int C = a.chains, n = a.n, D = s.D, H1 = s.H1, H2 = s.H2;
  // Ragged batches: GEMM tiles only over each chain's own rows.
  GemmRagged rows_h1, rows_h2, ksl;
  if (a.n_true != nullptr) {
    mlp_ragged_kernel<<<1, 1, 0, st>>>(a);
    int rc0 = check_launch("mlp_ragged_kernel");
    if (rc0 != GBSGMC_OK) return rc0;
    rows_h1.tile_prefix = a.prefix1;
    rows_h2.tile_prefix = a.prefix2;
    ksl.kblocks = a.kblocks;
  }
  const int64_t pw = matrix_params(s);
  const int nprep = a.fused ? a.sq_count : prep_blocks(s);
  const bf16* w1b = a.wb;
  const bf16* w2b = a.wb + s.oW2;
  int rc;

  if (!a.fused) {
    mlp_prep_kernel<<<dim3(nprep, C), 256, 0, st>>>(a);
    if ((rc = check_launch("mlp_prep_kernel")) != GBSGMC_OK) return rc;
  }
  mlp_gather_kernel<<<dim3(n / kTile, D / kTile, C), 256, 0, st>>>(a);
  if ((rc = check_launch("mlp_gather_kernel")) != GBSGMC_OK) return rc;

  // Tensor maps (columns, rows, chains).  K-major operands use 64 x 128 (A)
  // or 64 x BN (B) boxes, MN-major ones 64 x 64 boxes.
  const int64_t sx = int64_t(n) * D, s1 = int64_t(n) * H1, s2 = int64_t(n) * H2;
  CUtensorMap m_xb, m_w1, m_z1, m_w2;
  if ((rc = make_tmap_bf16_3d(&m_xb, a.xb, D, n, C, D, sx, kGemmBK, kGemmBM)) ||
      (rc = make_tmap_bf16_3d(&m_w1, w1b, H1, D, C, H1, pw, 64, 64)) ||
      (rc = make_tmap_bf16_3d(&m_z1, a.z1, H1, n, C, H1, s1, kGemmBK, kGemmBM)) ||
      (rc = make_tmap_bf16_3d(&m_w2, w2b, H2, H1, C, H2, pw, 64, 64)))
    return rc;
  const bool uniform = a.n_true == nullptr;
  // 3: A1 = Xb W1 (W1 [D, H1] is the MN-major B operand).
  EpiHidden1 e1{a.w, s.P, s.ob1};
  if ((rc = make_tmap_rows(&e1.zmap, a.z1, false, H1, n, C, H1, s1))) return rc;
  if ((rc = gemm256<false, true>(m_xb, m_w1, m_w1, C, n, H1, D, a.status, e1, st, rows_h1,
                                 uniform)))
    return rc;
  // 4: A2 = Z1 W2.
  EpiHidden2 e2{a.w, s.P, s.ob2, s.oW3, H2, n, a.outp};
  if ((rc = make_tmap_rows(&e2.zmap, a.z2g, false, H2, n, C, H2, s2))) return rc;
  if ((rc = gemm256<false, true>(m_z1, m_w2, m_w2, C, n, H2, H1, a.status, e2, st, rows_h2,
                                 uniform)))
    return rc;

  if (a.fisher)
    mlp_out_kernel<true><<<dim3(n / kTile, C), 256, 0, st>>>(a);
  else
    mlp_out_kernel<false><<<dim3(n / kTile, C), 256, 0, st>>>(a);
  if ((rc = check_launch("mlp_out_kernel")) != GBSGMC_OK) return rc;

  if (a.want_grad) {
    CUtensorMap m_z1mn, m_g2mn, m_g2, m_w2k, m_w2k_half, m_xbmn;
    if ((rc = make_tmap_bf16_3d(&m_z1mn, a.z1, H1, n, C, H1, s1, 64, 64)) ||
        (rc = make_tmap_bf16_3d(&m_g2mn, a.z2g, H2, n, C, H2, s2, 64, 64)) ||
        (rc = make_tmap_bf16_3d(&m_g2, a.z2g, H2, n, C, H2, s2, kGemmBK, kGemmBM)) ||
        (rc = make_tmap_bf16_3d(&m_w2k, w2b, H2, H1, C, H2, pw, kGemmBK, kBN)) ||
        (rc = make_tmap_bf16_3d(&m_w2k_half, w2b, H2, H1, C, H2, pw, kGemmBK, kBN / 2)) ||
        (rc = make_tmap_bf16_3d(&m_xbmn, a.xb, D, n, C, D, sx, 64, 64)))
      return rc;
    const double sc2 = static_cast<double>(a.prior_scale) * a.prior_scale;
    const float pf = a.prior_scale > 0.f ? static_cast<float>(1.0 / (sc2 * a.temperature)) : 0.f;
    // 6: dW2 [H1, H2] = Z1^T G2 (both operands MN-major), before step 7
    //    overwrites Z1.
    // The prior's term pf w of W1 and W2 is added in the gradient GEMMs'
    // epilogues (not in the fused plans, whose update adds it, nor in the
    // Fisher model, which differentiates the likelihood alone).
    const float pf_epi = a.fused || a.fisher ? 0.f : pf;
    const EpiGradRows e6{a.grad, s.P, s.oW2, H2, a.w, pf_epi};
    if ((rc = gemm256<true, true>(m_z1mn, m_g2mn, m_g2mn, C, H1, H2, n, a.status, e6, st, ksl,
                                  uniform)))
      return rc;
    if (a.fisher) {
      // 6b: sum_i d_i^2 of W2 = (Z1^2)^T (G2^2).
      mlp_square_kernel<<<dim3(n / kTile, H1 / 64, C), 256, 0, st>>>(a.z1, a.sqa, n, H1, nullptr);
      if ((rc = check_launch("mlp_square_kernel")) != GBSGMC_OK) return rc;
      mlp_square_kernel<<<dim3(n / kTile, H2 / 64, C), 256, 0, st>>>(a.z2g, a.sqb, n, H2, nullptr);
      if ((rc = check_launch("mlp_square_kernel")) != GBSGMC_OK) return rc;
      CUtensorMap m_qa, m_qb;
      if ((rc = make_tmap_bf16_3d(&m_qa, a.sqa, H1, n, C, H1, s1, 64, 64)) ||
          (rc = make_tmap_bf16_3d(&m_qb, a.sqb, H2, n, C, H2, s2, 64, 64)))
        return rc;
      const EpiGradRows e6q{a.grad_sq, s.P, s.oW2, H2};
      if ((rc = gemm256<true, true>(m_qa, m_qb, m_qb, C, H1, H2, n, a.status, e6q, st, ksl,
                                    uniform)))
        return rc;
    }
    // 7: G1 = (G2 W2^T) * (1 - Z1^2); W2 [H1, H2] is the K-major B operand.
    EpiAdjoint1 e7{a.z1, a.pb1, H1, n};
    if ((rc = make_tmap_rows(&e7.zmap, a.z1, false, H1, n, C, H1, s1))) return rc;
    if ((rc = gemm256<false, false>(m_g2, m_w2k, m_w2k_half, C, n, H1, H2, a.status, e7, st,
                                    rows_h1, uniform)))
      return rc;
    // 8: dW1^T [H1, D] = G1^T Xb: GEMM row i (hidden unit), column f
    //    (feature) lands at dW1[f, i].
    const EpiGradCols e8{a.grad, s.P, s.oW1, H1, a.w, pf_epi};
    if ((rc = launch_gemm<64, true, true>(m_z1mn, m_xbmn, C, H1, D, n, a.status, e8, st, ksl)))
      return rc;
    if (a.fisher) {
      // 8b: sum_i d_i^2 of W1 = (G1^2)^T (Xb^2), and b1's sums of squares.
      mlp_square_kernel<<<dim3(n / kTile, H1 / 64, C), 256, 0, st>>>(a.z1, a.sqa, n, H1, a.pb1sq);
      if ((rc = check_launch("mlp_square_kernel")) != GBSGMC_OK) return rc;
      mlp_square_kernel<<<dim3(n / kTile, D / 64, C), 256, 0, st>>>(a.xb, a.sqb, n, D, nullptr);
      if ((rc = check_launch("mlp_square_kernel")) != GBSGMC_OK) return rc;
      CUtensorMap m_qa, m_qx;
      if ((rc = make_tmap_bf16_3d(&m_qa, a.sqa, H1, n, C, H1, s1, 64, 64)) ||
          (rc = make_tmap_bf16_3d(&m_qx, a.sqb, D, n, C, D, sx, 64, 64)))
        return rc;
      const EpiGradCols e8q{a.grad_sq, s.P, s.oW1, H1};
      if ((rc = launch_gemm<64, true, true>(m_qa, m_qx, C, H1, D, n, a.status, e8q, st, ksl)))
        return rc;
    }
  }
  const int fx = a.want_grad ? ceil_div(H1 > H2 ? H1 : H2, 256) : 1;
  mlp_finalize_kernel<<<dim3(fx, C), 256, 0, st>>>(a, nprep);
  return check_launch("mlp_finalize_kernel");
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int64_t gbsgmc_mlp_param_count(const gbsgmc_mlp* model) {
  if (model == nullptr) return -1;
  return mlp_shape(model->d_in, model->h1, model->h2).P;
}

extern "C" size_t gbsgmc_mlp_workspace_bytes(const gbsgmc_mlp* model, int chains, int n) {
  if (model == nullptr || chains <= 0 || n <= 0 || n % 128 != 0 ||
      model->d_in % 64 != 0 || model->h1 % 256 != 0 || model->h2 % 256 != 0)
    return 0;
  return mlp_layout(mlp_shape(model->d_in, model->h1, model->h2), chains, n).total;
}

namespace {

int mlp_call(const gbsgmc_mlp* model, int chains, int n, const int32_t* n_dev,
             const int32_t* idx_dev, int64_t idx_stride, const float* mask_dev,
             const float* w_dev, double* U_dev, float* grad_dev, float* lk_dev,
             double* lk_var_dev, void* workspace_dev, size_t workspace_bytes,
             int* status_dev, gbsgmc_stream_t stream, const double* sq_parts = nullptr,
             int sq_count = 0, const int32_t* ident_dev = nullptr) {
  int rc = check_model(model, "mlp_value_and_grad");
  if (rc != GBSGMC_OK) return rc;
  if (chains < 0 || n < 0)
    return set_error(GBSGMC_ERR_ARG, "mlp_value_and_grad: negative size");
  if (chains == 0) return GBSGMC_OK;
  if (n == 0 || n % 128 != 0 || chains > 65535 || n > (1 << 24))
    return set_error(GBSGMC_ERR_SHAPE,
                     "mlp_value_and_grad: n must be a positive multiple of 128 "
                     "(got %d), chains <= 65535", n);
  if (idx_dev == nullptr || w_dev == nullptr || U_dev == nullptr ||
      workspace_dev == nullptr || status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_value_and_grad: null pointer");
  if (idx_stride < n)
    return set_error(GBSGMC_ERR_ARG, "mlp_value_and_grad: idx_stride < n");
  if (reinterpret_cast<uintptr_t>(workspace_dev) % 256 != 0)
    return set_error(GBSGMC_ERR_ARG, "mlp_value_and_grad: workspace must be 256-byte aligned");
  const MlpShape s = mlp_shape(model->d_in, model->h1, model->h2);
  const MlpLayout L = mlp_layout(s, chains, n);
  if (workspace_bytes < L.total)
    return set_error(GBSGMC_ERR_ARG,
                     "mlp_value_and_grad: workspace of %zu bytes, need %zu",
                     workspace_bytes, L.total);
  MlpArgs a{};
  a.s = s;
  a.chains = chains;
  a.n = n;
  a.y_inline = model->y_inline ? 1 : 0;
  a.want_grad = grad_dev != nullptr;
  a.n_obs = model->n_obs;
  a.n_rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  a.ld = model->ld;
  a.idx_stride = idx_stride;
  a.X = model->X;
  a.y = model->y;
  a.mask = mask_dev;
  a.idx = idx_dev;
  a.w = w_dev;
  a.sigma = model->sigma;
  a.prior_scale = model->prior_scale;
  a.temperature = model->temperature;
  a.U = U_dev;
  a.grad = grad_dev;
  a.lk = lk_dev;
  a.lk_var = lk_var_dev;
  a.status = status_dev;
  a.n_true = n_dev;
  a.ident = ident_dev;
  a.fused = sq_parts != nullptr ? 1 : 0;
  a.sq_count = sq_count;
  a.psq = const_cast<double*>(sq_parts);
  return run_mlp(a, L, workspace_dev, static_cast<cudaStream_t>(stream));
}

}  // namespace

namespace gbsgmc {

int mlp_mirror_region(const gbsgmc_mlp* model, int chains, int n, void* ws, void** mirror,
                      int64_t* count, int64_t* stride) {
  const MlpShape s = mlp_shape(model->d_in, model->h1, model->h2);
  const MlpLayout L = mlp_layout(s, chains, n);
  *mirror = static_cast<unsigned char*>(ws) + L.wb;
  *count = matrix_params(s);
  *stride = matrix_params(s);
  return GBSGMC_OK;
}

int mlp_value_and_grad_ident(const gbsgmc_mlp* model, int chains, int n, const int32_t* idx,
                             int64_t idx_stride, const int32_t* ident_dev, const float* w,
                             double* U, float* grad, double* lk_var, void* ws, size_t ws_bytes,
                             int* status, cudaStream_t st) {
  if (ident_dev == nullptr) return set_error(GBSGMC_ERR_ARG, "mlp (identities): null map");
  return mlp_call(model, chains, n, nullptr, idx, idx_stride, nullptr, w, U, grad, nullptr,
                  lk_var, ws, ws_bytes, status, st, nullptr, 0, ident_dev);
}

int mlp_value_and_grad_fused(const gbsgmc_mlp* model, int chains, int n, const int32_t* idx,
                             int64_t idx_stride, const float* w, double* U, float* grad,
                             double* lk_var, void* ws, size_t ws_bytes, int* status,
                             cudaStream_t st, const double* sq_parts, int sq_count) {
  if (sq_parts == nullptr || sq_count < 1)
    return set_error(GBSGMC_ERR_ARG, "mlp (fused): missing sums of squares");
  return mlp_call(model, chains, n, nullptr, idx, idx_stride, nullptr, w, U, grad, nullptr,
                  lk_var, ws, ws_bytes, status, st, sq_parts, sq_count);
}

}  // namespace gbsgmc

extern "C" int gbsgmc_mlp_value_and_grad(
    const gbsgmc_mlp* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, const float* mask_dev, const float* w_dev,
    double* U_dev, float* grad_dev, float* lk_dev, double* lk_var_dev,
    void* workspace_dev, size_t workspace_bytes, int* status_dev,
    gbsgmc_stream_t stream) {
  return mlp_call(model, chains, n, nullptr, idx_dev, idx_stride, mask_dev, w_dev, U_dev,
                  grad_dev, lk_dev, lk_var_dev, workspace_dev, workspace_bytes, status_dev,
                  stream);
}

extern "C" int gbsgmc_mlp_value_and_grad_ragged(
    const gbsgmc_mlp* model, int chains, int n_max, const int32_t* n_dev,
    const int32_t* idx_dev, int64_t idx_stride, const float* mask_dev,
    const float* w_dev, double* U_dev, float* grad_dev, float* lk_dev,
    double* lk_var_dev, void* workspace_dev, size_t workspace_bytes,
    int* status_dev, gbsgmc_stream_t stream) {
  if (n_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_value_and_grad_ragged: null row counts");
  return mlp_call(model, chains, n_max, n_dev, idx_dev, idx_stride, mask_dev, w_dev, U_dev,
                  grad_dev, lk_dev, lk_var_dev, workspace_dev, workspace_bytes, status_dev,
                  stream);
}

extern "C" size_t gbsgmc_mlp_fisher_workspace_bytes(const gbsgmc_mlp* model, int chains, int n) {
  if (model == nullptr || chains <= 0 || n <= 0 || n % 128 != 0 ||
      model->d_in % 64 != 0 || model->h1 % 256 != 0 || model->h2 % 256 != 0)
    return 0;
  return mlp_layout(mlp_shape(model->d_in, model->h1, model->h2), chains, n, true).total;
}

extern "C" int gbsgmc_mlp_fisher_noise(const gbsgmc_mlp* model, int chains, int n,
                                       const int32_t* idx_dev, int64_t idx_stride,
                                       const float* w_dev, const float* grad_dev,
                                       const float* friction_dev, float friction,
                                       float step_size, float* cb_diff_sqrt_dev,
                                       float* b_sqrt_dev, void* workspace_dev,
                                       size_t workspace_bytes, int* status_dev,
                                       gbsgmc_stream_t stream) {
  int rc = check_model(model, "mlp_fisher_noise");
  if (rc != GBSGMC_OK) return rc;
  if (chains < 0) return set_error(GBSGMC_ERR_ARG, "mlp_fisher_noise: negative size");
  if (chains == 0) return GBSGMC_OK;
  if (n <= 0 || n % 128 != 0 || chains > 65535 || n > (1 << 24))
    return set_error(GBSGMC_ERR_SHAPE,
                     "mlp_fisher_noise: n must be a positive multiple of 128 (got %d), "
                     "chains <= 65535", n);
  if (idx_dev == nullptr || w_dev == nullptr || grad_dev == nullptr ||
      cb_diff_sqrt_dev == nullptr || b_sqrt_dev == nullptr || workspace_dev == nullptr ||
      status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "mlp_fisher_noise: null pointer");
  if (idx_stride < n) return set_error(GBSGMC_ERR_ARG, "mlp_fisher_noise: idx_stride < n");
  if (reinterpret_cast<uintptr_t>(workspace_dev) % 256 != 0)
    return set_error(GBSGMC_ERR_ARG, "mlp_fisher_noise: workspace must be 256-byte aligned");
  const MlpShape s = mlp_shape(model->d_in, model->h1, model->h2);
  const MlpLayout L = mlp_layout(s, chains, n, true);
  if (workspace_bytes < L.total)
    return set_error(GBSGMC_ERR_ARG, "mlp_fisher_noise: workspace of %zu bytes, need %zu",
                     workspace_bytes, L.total);
  MlpArgs a{};
  a.s = s;
  a.chains = chains;
  a.n = n;
  a.y_inline = model->y_inline ? 1 : 0;
  a.want_grad = 1;
  a.n_obs = model->n_obs;
  a.n_rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  a.ld = model->ld;
  a.idx_stride = idx_stride;
  a.X = model->X;
  a.y = model->y;
  a.idx = idx_dev;
  a.w = w_dev;
  a.sigma = model->sigma;
  a.prior_scale = model->prior_scale;
  a.temperature = model->temperature;
  a.U = view<double>(workspace_dev, L.fU);
  a.status = status_dev;
  a.fisher = 1;
  a.grad = b_sqrt_dev;           // S1, then b_sqrt
  a.grad_sq = cb_diff_sqrt_dev;  // S2, then corr, then cb_diff_sqrt
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((rc = run_mlp(a, L, workspace_dev, st)) != GBSGMC_OK) return rc;
  const int gx = static_cast<int>(std::min<int64_t>((s.P + 1023) / 1024, 1024));
  mlp_fisher_corr_kernel<<<dim3(gx, chains), 256, 0, st>>>(
      s.P, n, static_cast<float>(model->n_obs), step_size, grad_dev, friction_dev, friction,
      b_sqrt_dev, cb_diff_sqrt_dev, a.fmin);
  if ((rc = check_launch("mlp_fisher_corr_kernel")) != GBSGMC_OK) return rc;
  mlp_fisher_apply_kernel<<<dim3(gx, chains), 256, 0, st>>>(s.P, friction_dev, friction, a.fmin,
                                                            cb_diff_sqrt_dev, b_sqrt_dev);
  return check_launch("mlp_fisher_apply_kernel");
}
