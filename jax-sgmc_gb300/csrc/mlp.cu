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
// Launch sequence (each batched over chains; GEMMs are C = A B^T with both
// operands K-major BF16, fp32 accumulation in TMEM):
//   1 mlp_prep_kernel     W1 -> W1t [H1,D], W2 -> W2t [H2,H1] and W2b [H1,H2]
//                         (BF16), partial sums of w^2 for the prior
//   2 mlp_gather_kernel   X rows -> Xb [n,D], Xt [D,n] (BF16), targets
//   3 GEMM Xb  . W1t^T    epilogue tanh(+b1) -> Z1 [n,H1], Z1t [H1,n]
//   4 GEMM Z1  . W2t^T    epilogue tanh(+b2) -> Z2 [n,H2], partial Z2 . W3
//   5 mlp_out_kernel      out, lk, g; G2 in place of Z2, G2t [H2,n], partial
//                         column sums for dW3 and db2
//   6 GEMM G2  . W2b^T    epilogue *(1 - Z1^2) -> G1t [H1,n], partial db1
//   7 GEMM Z1t . G2t^T    epilogue + prior -> dW2
//   8 GEMM G1t . Xt^T     epilogue + prior -> dW1 (written transposed)
//   9 mlp_finalize_kernel db1, db2, dW3, db3, U and var(lk)
// Without a gradient only 1-5 and 9 run, and the transposed copies are not
// written.
#include <cuda_bf16.h>

#include <cmath>

#include "common.cuh"
#include "internal.h"
#include "tc_gemm.cuh"

namespace gbsgmc {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kTile = 64;      // rows / columns of a prep, gather or out tile
constexpr int kOutCols = 256;  // columns of an out-kernel tile
constexpr int kBN = 256;       // N tile of the H1- and H2-wide GEMMs

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

// Stores 16 floats as BF16 at a 32-byte aligned address.
__device__ __forceinline__ void store_bf16x16(bf16* dst, const float (&x)[16]) {
  uint4 a, b;
  a.x = pack_bf16x2(x[0], x[1]);
  a.y = pack_bf16x2(x[2], x[3]);
  a.z = pack_bf16x2(x[4], x[5]);
  a.w = pack_bf16x2(x[6], x[7]);
  b.x = pack_bf16x2(x[8], x[9]);
  b.y = pack_bf16x2(x[10], x[11]);
  b.z = pack_bf16x2(x[12], x[13]);
  b.w = pack_bf16x2(x[14], x[15]);
  uint4* d = reinterpret_cast<uint4*>(dst);
  d[0] = a;
  d[1] = b;
}

__device__ __forceinline__ void load_bf16x16(const bf16* src, float (&x)[16]) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  const uint4 a = s[0], b = s[1];
  unpack_bf16x2(a.x, x[0], x[1]);
  unpack_bf16x2(a.y, x[2], x[3]);
  unpack_bf16x2(a.z, x[4], x[5]);
  unpack_bf16x2(a.w, x[6], x[7]);
  unpack_bf16x2(b.x, x[8], x[9]);
  unpack_bf16x2(b.y, x[10], x[11]);
  unpack_bf16x2(b.z, x[12], x[13]);
  unpack_bf16x2(b.w, x[14], x[15]);
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

int prep_blocks(const MlpShape& s) {
  return (s.D / kTile) * (s.H1 / kTile) + (s.H1 / kTile) * (s.H2 / kTile) + 1;
}

// Workspace regions, each [chains, per-chain size], 256-byte aligned.
struct MlpLayout {
  size_t w1t, w2t, w2b, xb, xt, z1, z1t, z2g, g2t, g1t;  // BF16
  size_t yv, outp, pw3, pb2, pb1;                        // fp32
  size_t psq, plk;                                       // fp64
  size_t total;
};

MlpLayout mlp_layout(const MlpShape& s, int chains, int n) {
  MlpLayout L;
  size_t off = 0;
  auto take = [&](size_t bytes_per_chain) {
    const size_t at = off;
    off += (bytes_per_chain * static_cast<size_t>(chains) + 255) & ~static_cast<size_t>(255);
    return at;
  };
  const size_t D = s.D, H1 = s.H1, H2 = s.H2, N = n;
  L.w1t = take(2 * H1 * D);
  L.w2t = take(2 * H2 * H1);
  L.w2b = take(2 * H1 * H2);
  L.xb = take(2 * N * D);
  L.xt = take(2 * D * N);
  L.z1 = take(2 * N * H1);
  L.z1t = take(2 * H1 * N);
  L.z2g = take(2 * N * H2);
  L.g2t = take(2 * H2 * N);
  L.g1t = take(2 * H1 * N);
  L.yv = take(4 * N);
  L.outp = take(4 * (H2 / kBN) * N);
  L.pw3 = take(4 * (N / kTile) * H2);
  L.pb2 = take(4 * (N / kTile) * H2);
  L.pb1 = take(4 * (N / 32) * H1);
  L.psq = take(8 * static_cast<size_t>(prep_blocks(s)));
  L.plk = take(8 * 4 * (N / kTile));
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
  // workspace views
  bf16 *w1t, *w2t, *w2b, *xb, *xt, *z1, *z1t, *z2g, *g2t, *g1t;
  float *yv, *outp, *pw3, *pb2, *pb1;
  double *psq, *plk;
};

// ---------------------------------------------------------------------------
// 1. Weights to BF16 (W1 transposed; W2 straight and transposed) and partial
//    sums of squares of every parameter.  Grid (prep_blocks, chains).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_prep_kernel(const MlpArgs a) {
  __shared__ float tile[kTile][kTile + 1];
  __shared__ double red[32];
  const MlpShape& s = a.s;
  const int c = blockIdx.y, blk = blockIdx.x, t = threadIdx.x;
  const float* w = a.w + static_cast<int64_t>(c) * s.P;
  const int nt1 = (s.D / kTile) * (s.H1 / kTile);
  const int nt2 = (s.H1 / kTile) * (s.H2 / kTile);
  float sq = 0.f;
  if (blk < nt1 + nt2) {
    const bool first = blk < nt1;
    const int tt = first ? blk : blk - nt1;
    const int R = first ? s.D : s.H1, Cc = first ? s.H1 : s.H2;
    const int ti = tt / (Cc / kTile), tj = tt % (Cc / kTile);
    const float* src = w + (first ? s.oW1 : s.oW2);
    const int col = t & 63;
    bf16* straight = (!first && a.want_grad)
                         ? a.w2b + static_cast<int64_t>(c) * s.H1 * s.H2
                         : nullptr;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const int r = (t >> 6) + 4 * k;
      const int64_t e = static_cast<int64_t>(ti * kTile + r) * Cc + tj * kTile + col;
      const float v = __ldg(src + e);
      sq = fmaf(v, v, sq);
      tile[r][col] = v;
      if (straight != nullptr) straight[e] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    bf16* dstT = first ? a.w1t + static_cast<int64_t>(c) * s.H1 * s.D
                       : a.w2t + static_cast<int64_t>(c) * s.H2 * s.H1;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int i = t + 256 * k;
      const int cc = i >> 5, r2 = (i & 31) * 2;
      const int64_t e = static_cast<int64_t>(tj * kTile + cc) * R + ti * kTile + r2;
      *reinterpret_cast<uint32_t*>(dstT + e) = pack_bf16x2(tile[r2][cc], tile[r2 + 1][cc]);
    }
  } else {
    const int64_t tail = s.P - s.oW3;
    for (int64_t i = t; i < tail; i += 256) {
      const float v = __ldg(w + s.oW3 + i);
      sq = fmaf(v, v, sq);
    }
  }
  const double tot = block_sum(static_cast<double>(sq), red);
  if (t == 0) a.psq[static_cast<int64_t>(c) * gridDim.x + blk] = tot;
}

// ---------------------------------------------------------------------------
// 2. Minibatch rows to BF16, row-major and transposed, plus targets.
//    Grid (n/64, D/64, chains).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_gather_kernel(const MlpArgs a) {
  __shared__ float tile[kTile][kTile + 1];
  __shared__ int64_t rows[kTile];
  const MlpShape& s = a.s;
  const int i0 = blockIdx.x * kTile, f0 = blockIdx.y * kTile, c = blockIdx.z;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < kTile) {
    int64_t o = a.idx[static_cast<int64_t>(c) * a.idx_stride + i0 + t];
    if (o < 0 || o >= a.n_rows) {
      raise_status(a.status, GBSGMC_ERR_INDEX);
      o = 0;
    }
    rows[t] = o;
    if (blockIdx.y == 0) {
      const float yy = a.y_inline ? __ldg(a.X + o * a.ld + s.D) : __ldg(a.y + o);
      a.yv[static_cast<int64_t>(c) * a.n + i0 + t] = yy;
    }
  }
  __syncthreads();
  bf16* xb = a.xb + static_cast<int64_t>(c) * a.n * s.D;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int r = warp * 8 + j;
    const float* src = a.X + rows[r] * a.ld + f0;
    const float v0 = __ldg(src + lane), v1 = __ldg(src + 32 + lane);
    tile[r][lane] = v0;
    tile[r][lane + 32] = v1;
    bf16* d = xb + static_cast<int64_t>(i0 + r) * s.D + f0;
    d[lane] = __float2bfloat16_rn(v0);
    d[lane + 32] = __float2bfloat16_rn(v1);
  }
  if (!a.want_grad) return;
  __syncthreads();
  bf16* xt = a.xt + static_cast<int64_t>(c) * s.D * a.n;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = t + 256 * k;
    const int f = i >> 5, r2 = (i & 31) * 2;
    *reinterpret_cast<uint32_t*>(xt + static_cast<int64_t>(f0 + f) * a.n + i0 + r2) =
        pack_bf16x2(tile[r2][f], tile[r2 + 1][f]);
  }
}

// ---------------------------------------------------------------------------
// GEMM epilogues.
// ---------------------------------------------------------------------------

// 3: Z1 = tanh(acc + b1) -> Z1 [n, H1] and (with a gradient) Z1t [H1, n].
struct EpiHidden1 {
  const float* w;
  int64_t P, ob1;
  int H1, n;
  bf16* z1;
  bf16* z1t;  // null: not written
  template <int BN, class Load>
  __device__ __forceinline__ void tile(int b, int row, int col0, const Load& load) const {
    const float* b1 = w + b * P + ob1;
    bf16* dst = z1 + (static_cast<int64_t>(b) * n + row) * H1 + col0;
#pragma unroll 1
    for (int c = 0; c < BN / 16; ++c) {
      float v[16];
      load(c, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = tanh_approx(v[k] + __ldg(b1 + col0 + 16 * c + k));
      store_bf16x16(dst + 16 * c, v);
      if (z1t != nullptr) {
        bf16* tr = z1t + (static_cast<int64_t>(b) * H1 + col0 + 16 * c) * n + row;
#pragma unroll
        for (int k = 0; k < 16; ++k) tr[static_cast<int64_t>(k) * n] = __float2bfloat16_rn(v[k]);
      }
    }
  }
};

// 4: Z2 = tanh(acc + b2) -> Z2 [n, H2]; the fp32 partial Z2 . W3 over this
//    tile's columns -> outp [H2/BN, n].
struct EpiHidden2 {
  const float* w;
  int64_t P, ob2, oW3;
  int H2, n;
  bf16* z2;
  float* outp;
  template <int BN, class Load>
  __device__ __forceinline__ void tile(int b, int row, int col0, const Load& load) const {
    const float* b2 = w + b * P + ob2;
    const float* w3 = w + b * P + oW3;
    bf16* dst = z2 + (static_cast<int64_t>(b) * n + row) * H2 + col0;
    float acc = 0.f;
#pragma unroll 1
    for (int c = 0; c < BN / 16; ++c) {
      float v[16];
      load(c, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int j = col0 + 16 * c + k;
        v[k] = tanh_approx(v[k] + __ldg(b2 + j));
        acc = fmaf(v[k], __ldg(w3 + j), acc);
      }
      store_bf16x16(dst + 16 * c, v);
    }
    outp[(static_cast<int64_t>(b) * (H2 / BN) + col0 / BN) * n + row] = acc;
  }
};

// 6: G1 = acc * (1 - Z1^2) -> G1t [H1, n]; per-warp column sums -> pb1
//    [n/32, H1].
struct EpiAdjoint1 {
  const bf16* z1;
  bf16* g1t;
  float* pb1;
  int H1, n;
  template <int BN, class Load>
  __device__ __forceinline__ void tile(int b, int row, int col0, const Load& load) const {
    const int lane = threadIdx.x & 31;
    const bf16* zr = z1 + (static_cast<int64_t>(b) * n + row) * H1 + col0;
    float* part = pb1 + (static_cast<int64_t>(b) * (n / 32) + row / 32) * H1 + col0;
#pragma unroll 1
    for (int c = 0; c < BN / 16; ++c) {
      float v[16], z[16];
      load(c, v);
      load_bf16x16(zr + 16 * c, z);
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] *= 1.f - z[k] * z[k];
      bf16* tr = g1t + (static_cast<int64_t>(b) * H1 + col0 + 16 * c) * n + row;
#pragma unroll
      for (int k = 0; k < 16; ++k) tr[static_cast<int64_t>(k) * n] = __float2bfloat16_rn(v[k]);
      const float cs = warp_colsum16(v, lane);
      if ((lane & 1) == 0) part[16 * c + (lane >> 1)] = cs;
    }
  }
};

// 7 and 8: gradient of a weight matrix plus the prior term.  Element
// (row, col) of the GEMM lands at grad[b*P + off + row*rs + col*cs].
struct EpiWeightGrad {
  const float* w;
  float* grad;
  int64_t P, off, rs, cs;
  float pf;  // 1 / (s^2 T); 0 for a flat prior
  template <int BN, class Load>
  __device__ __forceinline__ void tile(int b, int row, int col0, const Load& load) const {
    const int64_t base = b * P + off + row * rs;
#pragma unroll 1
    for (int c = 0; c < BN / 16; ++c) {
      float v[16];
      load(c, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int64_t e = base + static_cast<int64_t>(col0 + 16 * c + k) * cs;
        grad[e] = fmaf(pf, __ldg(w + e), v[k]);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// 5. Output layer, likelihood and the first adjoint.  Grid (H2/256, n/64,
//    chains) with a gradient, (1, n/64, chains) without.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mlp_out_kernel(const MlpArgs a) {
  __shared__ float g_s[kTile];
  __shared__ double red[32];
  __shared__ float colp[2][2][kOutCols];
  __shared__ __align__(16) bf16 tileT[kOutCols][kTile + 2];  // 33-word rows
  const MlpShape& s = a.s;
  const int c = blockIdx.z, rb = blockIdx.y, i0 = rb * kTile, c0 = blockIdx.x * kOutCols;
  const int t = threadIdx.x;
  const float* w = a.w + static_cast<int64_t>(c) * s.P;
  const float inv_s2 = 1.f / (a.sigma * a.sigma);
  const float scale = static_cast<float>(static_cast<double>(a.n_obs) / a.n / a.temperature);
  double lk_m = 0.0, lk_sum = 0.0, lk_sq = 0.0, g_sum = 0.0;
  if (t < kTile) {
    const int i = i0 + t;
    const int ntile = s.H2 / kBN;
    float out = __ldg(w + s.ob3);
    for (int q = 0; q < ntile; ++q)
      out += a.outp[(static_cast<int64_t>(c) * ntile + q) * a.n + i];
    const float r = a.yv[static_cast<int64_t>(c) * a.n + i] - out;
    const float lk = -0.5f * r * r * inv_s2 - logf(a.sigma) - 0.91893853320467274f;
    const float m = a.mask != nullptr ? __ldg(a.mask + static_cast<int64_t>(c) * a.n + i) : 1.f;
    const float g = -scale * m * r * inv_s2;
    g_s[t] = g;
    lk_m = static_cast<double>(m) * lk;
    lk_sum = lk;
    lk_sq = static_cast<double>(lk) * lk;
    g_sum = g;
    if (blockIdx.x == 0 && a.lk != nullptr) a.lk[static_cast<int64_t>(c) * a.n + i] = lk;
  }
  if (blockIdx.x == 0) {
    // var(lk) is over all n values, masked or not (jnp.var, integrator.py:880).
    const double s0 = block_sum(lk_m, red);
    const double s1 = block_sum(lk_sum, red);
    const double s2 = block_sum(lk_sq, red);
    const double s3 = block_sum(g_sum, red);
    if (t == 0) {
      double* p = a.plk + (static_cast<int64_t>(c) * (a.n / kTile) + rb) * 4;
      p[0] = s0;
      p[1] = s1;
      p[2] = s2;
      p[3] = s3;
    }
  }
  if (!a.want_grad) return;
  __syncthreads();
  // Thread t handles columns c0 + 2p, c0 + 2p + 1 on rows rg, rg + 2, ...
  const int p = t & 127, rg = t >> 7;
  const int j = c0 + 2 * p;
  const float w3a = __ldg(w + s.oW3 + j), w3b = __ldg(w + s.oW3 + j + 1);
  bf16* z2g = a.z2g + static_cast<int64_t>(c) * a.n * s.H2;
  float aw3a = 0.f, aw3b = 0.f, ab2a = 0.f, ab2b = 0.f;
#pragma unroll 4
  for (int r = rg; r < kTile; r += 2) {
    uint32_t* cell = reinterpret_cast<uint32_t*>(z2g + static_cast<int64_t>(i0 + r) * s.H2 + j);
    float za, zb;
    unpack_bf16x2(*cell, za, zb);
    const float g = g_s[r];
    const float ga = g * w3a * (1.f - za * za), gb = g * w3b * (1.f - zb * zb);
    *cell = pack_bf16x2(ga, gb);
    aw3a = fmaf(g, za, aw3a);
    aw3b = fmaf(g, zb, aw3b);
    ab2a += ga;
    ab2b += gb;
    tileT[2 * p][r] = __float2bfloat16_rn(ga);
    tileT[2 * p + 1][r] = __float2bfloat16_rn(gb);
  }
  colp[0][rg][2 * p] = aw3a;
  colp[0][rg][2 * p + 1] = aw3b;
  colp[1][rg][2 * p] = ab2a;
  colp[1][rg][2 * p + 1] = ab2b;
  __syncthreads();
  {
    const int64_t pr = (static_cast<int64_t>(c) * (a.n / kTile) + rb) * s.H2 + c0 + t;
    a.pw3[pr] = colp[0][0][t] + colp[0][1][t];
    a.pb2[pr] = colp[1][0][t] + colp[1][1][t];
  }
  // G2t rows: 64 contiguous BF16 (128 bytes) per column.
  bf16* g2t = a.g2t + static_cast<int64_t>(c) * s.H2 * a.n;
  const int lane = t & 31, warp = t >> 5;
#pragma unroll 4
  for (int k = 0; k < kOutCols / 8; ++k) {
    const int jj = warp * (kOutCols / 8) + k;
    *reinterpret_cast<uint32_t*>(g2t + static_cast<int64_t>(c0 + jj) * a.n + i0 + 2 * lane) =
        *reinterpret_cast<const uint32_t*>(&tileT[jj][2 * lane]);
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
  const float pf = a.prior_scale > 0.f
                       ? static_cast<float>(1.0 / (s2 * a.temperature))
                       : 0.f;
  const int nb64 = a.n / kTile, nb32 = a.n / 32;
  if (a.want_grad) {
    float* g = a.grad + static_cast<int64_t>(c) * s.P;
    const int j = blockIdx.x * 256 + t;
    if (j < s.H1) {
      const float* p = a.pb1 + static_cast<int64_t>(c) * nb32 * s.H1 + j;
      float acc = 0.f;
      for (int r = 0; r < nb32; ++r) acc += p[static_cast<int64_t>(r) * s.H1];
      g[s.ob1 + j] = fmaf(pf, __ldg(w + s.ob1 + j), acc);
    }
    if (j < s.H2) {
      const int64_t base = static_cast<int64_t>(c) * nb64 * s.H2 + j;
      float acc2 = 0.f, acc3 = 0.f;
      for (int r = 0; r < nb64; ++r) {
        acc2 += a.pb2[base + static_cast<int64_t>(r) * s.H2];
        acc3 += a.pw3[base + static_cast<int64_t>(r) * s.H2];
      }
      g[s.ob2 + j] = fmaf(pf, __ldg(w + s.ob2 + j), acc2);
      g[s.oW3 + j] = fmaf(pf, __ldg(w + s.oW3 + j), acc3);
    }
  }
  if (blockIdx.x != 0) return;
  double sq = 0.0, lm = 0.0, l1 = 0.0, l2 = 0.0, gs = 0.0;
  for (int i = t; i < nprep; i += 256) sq += a.psq[static_cast<int64_t>(c) * nprep + i];
  for (int i = t; i < nb64; i += 256) {
    const double* p = a.plk + (static_cast<int64_t>(c) * nb64 + i) * 4;
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
  double log_prior = 0.0;
  if (a.prior_scale > 0.f)
    log_prior = -0.5 * sq / s2 -
                static_cast<double>(s.P) * (log(static_cast<double>(a.prior_scale)) +
                                            0.91893853320467274178);
  // -N * mean(lk) without a mask, -N/n * (lk . mask) with one (potential.py:183-185).
  const double lik = -static_cast<double>(a.n_obs) * (lm / a.n);
  const double U = (lik - log_prior) / a.temperature;
  a.U[c] = U;
  if (a.lk_var != nullptr) {
    const double mean = l1 / a.n;
    a.lk_var[c] = fmax(l2 / a.n - mean * mean, 0.0);
  }
  if (!isfinite(U)) raise_status(a.status, GBSGMC_ERR_NONFINITE);
  if (a.want_grad)
    a.grad[static_cast<int64_t>(c) * s.P + s.ob3] =
        static_cast<float>(gs) + pf * __ldg(w + s.ob3);
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

int run_mlp(MlpArgs& a, const MlpLayout& L, void* ws, cudaStream_t st) {
  const MlpShape& s = a.s;
  a.w1t = view<bf16>(ws, L.w1t);
  a.w2t = view<bf16>(ws, L.w2t);
  a.w2b = view<bf16>(ws, L.w2b);
  a.xb = view<bf16>(ws, L.xb);
  a.xt = view<bf16>(ws, L.xt);
  a.z1 = view<bf16>(ws, L.z1);
  a.z1t = view<bf16>(ws, L.z1t);
  a.z2g = view<bf16>(ws, L.z2g);
  a.g2t = view<bf16>(ws, L.g2t);
  a.g1t = view<bf16>(ws, L.g1t);
  a.yv = view<float>(ws, L.yv);
  a.outp = view<float>(ws, L.outp);
  a.pw3 = view<float>(ws, L.pw3);
  a.pb2 = view<float>(ws, L.pb2);
  a.pb1 = view<float>(ws, L.pb1);
  a.psq = view<double>(ws, L.psq);
  a.plk = view<double>(ws, L.plk);
  const int C = a.chains, n = a.n, D = s.D, H1 = s.H1, H2 = s.H2;
  const int nprep = prep_blocks(s);
  int rc;

  mlp_prep_kernel<<<dim3(nprep, C), 256, 0, st>>>(a);
  if ((rc = check_launch("mlp_prep_kernel")) != GBSGMC_OK) return rc;
  mlp_gather_kernel<<<dim3(n / kTile, D / kTile, C), 256, 0, st>>>(a);
  if ((rc = check_launch("mlp_gather_kernel")) != GBSGMC_OK) return rc;

  // Tensor maps: (K columns, rows, chains), box 64 x {128 | BN}.
  CUtensorMap m_xb, m_w1t, m_z1, m_w2t;
  if ((rc = make_tmap_bf16_3d(&m_xb, a.xb, D, n, C, D, int64_t(n) * D, kGemmBK, kGemmBM)) ||
      (rc = make_tmap_bf16_3d(&m_w1t, a.w1t, D, H1, C, D, int64_t(H1) * D, kGemmBK, kBN)) ||
      (rc = make_tmap_bf16_3d(&m_z1, a.z1, H1, n, C, H1, int64_t(n) * H1, kGemmBK, kGemmBM)) ||
      (rc = make_tmap_bf16_3d(&m_w2t, a.w2t, H1, H2, C, H1, int64_t(H2) * H1, kGemmBK, kBN)))
    return rc;

  const EpiHidden1 e1{a.w, s.P, s.ob1, H1, n, a.z1, a.want_grad ? a.z1t : nullptr};
  if ((rc = launch_gemm<kBN>(m_xb, m_w1t, C, n, H1, D, a.status, e1, st))) return rc;
  const EpiHidden2 e2{a.w, s.P, s.ob2, s.oW3, H2, n, a.z2g, a.outp};
  if ((rc = launch_gemm<kBN>(m_z1, m_w2t, C, n, H2, H1, a.status, e2, st))) return rc;

  mlp_out_kernel<<<dim3(a.want_grad ? H2 / kOutCols : 1, n / kTile, C), 256, 0, st>>>(a);
  if ((rc = check_launch("mlp_out_kernel")) != GBSGMC_OK) return rc;

  if (a.want_grad) {
    CUtensorMap m_g2, m_w2b, m_z1t, m_g2t, m_g1t, m_xt;
    if ((rc = make_tmap_bf16_3d(&m_g2, a.z2g, H2, n, C, H2, int64_t(n) * H2, kGemmBK, kGemmBM)) ||
        (rc = make_tmap_bf16_3d(&m_w2b, a.w2b, H2, H1, C, H2, int64_t(H1) * H2, kGemmBK, kBN)) ||
        (rc = make_tmap_bf16_3d(&m_z1t, a.z1t, n, H1, C, n, int64_t(H1) * n, kGemmBK, kGemmBM)) ||
        (rc = make_tmap_bf16_3d(&m_g2t, a.g2t, n, H2, C, n, int64_t(H2) * n, kGemmBK, kBN)) ||
        (rc = make_tmap_bf16_3d(&m_g1t, a.g1t, n, H1, C, n, int64_t(H1) * n, kGemmBK, kGemmBM)) ||
        (rc = make_tmap_bf16_3d(&m_xt, a.xt, n, D, C, n, int64_t(D) * n, kGemmBK, 64)))
      return rc;
    const double s2 = static_cast<double>(a.prior_scale) * a.prior_scale;
    const float pf = a.prior_scale > 0.f ? static_cast<float>(1.0 / (s2 * a.temperature)) : 0.f;
    const EpiAdjoint1 e3{a.z1, a.g1t, a.pb1, H1, n};
    if ((rc = launch_gemm<kBN>(m_g2, m_w2b, C, n, H1, H2, a.status, e3, st))) return rc;
    // dW2[i, j] (row i of H1, column j of H2) = sum_r Z1t[i, r] G2t[j, r].
    const EpiWeightGrad e4{a.w, a.grad, s.P, s.oW2, H2, 1, pf};
    if ((rc = launch_gemm<kBN>(m_z1t, m_g2t, C, H1, H2, n, a.status, e4, st))) return rc;
    // dW1[f, i] = sum_r G1t[i, r] Xt[f, r]: GEMM row i, column f.
    const EpiWeightGrad e5{a.w, a.grad, s.P, s.oW1, 1, H1, pf};
    if ((rc = launch_gemm<64>(m_g1t, m_xt, C, H1, D, n, a.status, e5, st))) return rc;
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

extern "C" int gbsgmc_mlp_value_and_grad(
    const gbsgmc_mlp* model, int chains, int n, const int32_t* idx_dev,
    int64_t idx_stride, const float* mask_dev, const float* w_dev,
    double* U_dev, float* grad_dev, float* lk_dev, double* lk_var_dev,
    void* workspace_dev, size_t workspace_bytes, int* status_dev,
    gbsgmc_stream_t stream) {
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
  return run_mlp(a, L, workspace_dev, static_cast<cudaStream_t>(stream));
}
