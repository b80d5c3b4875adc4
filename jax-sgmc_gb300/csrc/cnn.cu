// Convolutional classifier with a softmax likelihood: U, dU/dw, lk and
// var(lk) for many chains at once, the convolutions as GEMMs on the tcgen05
// tensor cores.
//
// Network (NHWC, SAME padding, stride 1):
//   x [32,32,3] -> conv3x3 32 + b, ReLU, 2x2 max-pool -> [16,16,32]
//               -> conv3x3 64 + b, ReLU, 2x2 max-pool -> [8,8,64]
//               -> conv3x3 128 + b, ReLU, 2x2 max-pool -> [4,4,128]
//               -> flatten (h, w, c) 2048 -> dense 10 -> logits
//   lk = logits[label] - logsumexp(logits)   (the negative softmax cross
//   entropy of the reference's classifier example, examples/cifar.md:203-210)
// Flat parameters: the sorted ravel of {conv1: {b, w}, conv2: {b, w},
// conv3: {b, w}, linear: {b, w}} with w in HWIO / [in, out] layout:
//   b1 32 | W1 [3,3,3,32] | b2 64 | W2 [3,3,32,64] | b3 128 | W3 [3,3,64,128]
//   | bd 10 | Wd [2048,10],   P = 113,738.
//
// Each convolution is a GEMM over the im2col matrix Col [pixels, K] with K
// ordered (kh, kw, ci) and zero-padded to a multiple of 64:
//   forward  Y = ReLU(Col W + b)          A = Col (K-major), B = W (HWIO rows
//                                         = K, MN-major)
//   weights  dW = dY^T Col                 both MN-major; written into the
//                                         HWIO gradient directly
//   inputs   dX = sum over taps of dY shifted back by the tap times the tap's
//            W^T (the transposed convolution), A = dY (K-major), B = W
//            (K-major), then the pooling's argmax routing and the ReLU mask.
// conv1 reads its input by tap pairs from the images gathered as X8 [n, 32,
// 32, 8]: pixel (h, w) holds the 3 channels of (h, w - 1), then its own 3,
// then 2 zeros, so that one 16-byte core-matrix row of the unswizzled
// layout serves the taps (kh, 0) and (kh, 1) together and another (kh, 2):
// K = 3 kernel rows x 2 groups x 8 = 48 (padded to one 64-wide slice), each
// group a shifted (16 W, 8 H) box; its weight gradient reads the same
// boxes as an MN-major B.  Col is materialised for conv2 (32 input
// channels).  Where
// a tap's input channels fill a 128-byte row (64 BF16: conv3's input P2 and
// the output gradients dY2, dY3 of the transposed convolutions) the GEMMs
// are implicit: each 64-wide K slice of A (or 64-wide N block of dW's B) is
// one tap's box of the NHWC map, shifted by the tap and read by TMA from a
// 4-D tensor map, whose out-of-bounds zero fill is the SAME padding.  The forward GEMMs' epilogues apply bias and ReLU and
// the 2x2 max-pool to the fp32 accumulators themselves (EpiConvPool): each
// epilogue warp holds whole pool windows in its 32 rows, so it writes the
// pooled BF16 map and the argmax marks and no pre-pool activation is
// stored.  For that the rows of conv1's GEMM (32 x 32 pixels) are ordered in
// 16-pixel half rows, two image rows per 32 GEMM rows (conv1_row); conv2's
// natural order (16 x 16) and conv3's (8 x 8) already have that property.
// Everything a GEMM reads is BF16.  Channel and K padding come from the tensor maps'
// out-of-bounds zero fill; epilogues drop rows and columns past the real
// extents.  The dense layer, softmax and their adjoints are small and run on
// the CUDA cores in fp32.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.h"
#include "tc_gemm.cuh"

namespace gbsgmc {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kImg = 32, kInC = 3, kClasses = 10;
constexpr int kC1 = 32, kC2 = 64, kC3 = 128;
constexpr int kFlat = 4 * 4 * kC3;  // 2048
constexpr int kK1 = 27;  // conv1's K (3 x 3 taps x 3 channels)
constexpr int kX8 = 8;   // channels per gathered pixel: its left neighbour's 3, its own 3, 0, 0
constexpr int kG1 = 8;   // conv1's K groups of 8 (6 real: kernel row kh, columns {0, 1} or {2})
constexpr int kK1i = kG1 * kX8;  // conv1's GEMM K (one 64-wide slice)
constexpr int kK2 = 9 * kC1, kK2p = 320;
constexpr int kK3 = 9 * kC2;  // conv3 reads P2 by tap: no padded im2col
constexpr int kA1ld = kC1;  // conv1 output-gradient channels as stored (the dW1
                            // GEMM's 64-wide box reads zeros past them)

// Offsets of the leaves in a chain's flat parameter vector.
constexpr int64_t ob1 = 0, oW1 = ob1 + kC1, ob2 = oW1 + kK1 * kC1, oW2 = ob2 + kC2,
                  ob3 = oW2 + kK2 * kC2, oW3 = ob3 + kC3, obd = oW3 + kK3 * kC3,
                  oWd = obd + kClasses, kP = oWd + kFlat * kClasses;
static_assert(kP == 113738, "parameter count");

struct CnnLayout {
  size_t w1i, w2b, w3b;               // BF16 weights (conv1 unswizzled, others HWIO)
  size_t x8, p1, col2, p2, p3;        // BF16 GEMM operands
  size_t dy1, dy2, dy3;               // BF16 output gradients of the convs
  size_t m1, m2, m3;                  // uint8 argmax of each pool window
  size_t dp2, dp1;                    // fp32 input gradients of conv3, conv2
  size_t labels;                      // int32
  size_t dp3, gl;                     // fp32 dP3 [n, 2048], dlogits [n, 10]
  size_t psq, plk;                    // fp64 partial sums
  size_t part, bpart;                 // split-K weight partials, bias partials
  size_t total;
};

constexpr int kPrepBlocks = 64;  // Σw² partial sums per chain

// Split-K factors of the weight-gradient GEMMs (K = pixels of n images:
// 16n, 4n and n slices of 64 for the three layers; n is even; a factor
// divides the slice count).  Layer 2 has 5 N tiles per chain: 16 splits
// make 640 tiles for 8 chains (4.3 waves of 148 CTAs) where 8 made 320
// (2.2 waves, the third one sixth full).
inline int wsplit(int layer, int n) {
  return layer == 1 ? 32 : layer == 2 ? (n % 4 == 0 ? 16 : 8) : (n % 4 == 0 ? 4 : 2);
}

CnnLayout cnn_layout(int chains, int n) {
  CnnLayout L;
  size_t off = 0;
  auto take = [&](size_t per_chain) {
    const size_t at = off;
    off += (per_chain * static_cast<size_t>(chains) + 255) & ~static_cast<size_t>(255);
    return at;
  };
  const size_t N = n;
  L.w1i = take(2 * kG1 * 64 * kX8);
  L.w2b = take(2 * kK2 * kC2);
  L.w3b = take(2 * kK3 * kC3);
  L.x8 = take(2 * N * 1024 * kX8);
  L.dy1 = take(2 * N * 1024 * kA1ld);
  L.p1 = take(2 * N * 256 * kC1);
  L.col2 = take(2 * N * 256 * kK2p);
  L.dy2 = take(2 * N * 256 * kC2);
  L.p2 = take(2 * N * 64 * kC2);
  L.dy3 = take(2 * N * 64 * kC3);
  L.p3 = take(2 * N * 16 * kC3);
  L.m1 = take(N * 256 * kC1);
  L.m2 = take(N * 64 * kC2);
  L.m3 = take(N * 16 * kC3);
  L.dp2 = take(4 * N * 64 * kC2);
  L.dp1 = take(4 * N * 256 * kC1);
  L.labels = take(4 * N);
  L.dp3 = take(4 * N * kFlat);
  L.gl = take(4 * N * kClasses);
  L.psq = take(8 * kPrepBlocks);
  L.plk = take(8 * 4 * N);
  size_t part = 0;
  part = std::max<size_t>(part, size_t(wsplit(1, n)) * kC1 * kK1);
  part = std::max<size_t>(part, size_t(wsplit(2, n)) * kC2 * kK2);
  part = std::max<size_t>(part, size_t(wsplit(3, n)) * kC3 * kK3);
  L.part = take(4 * part);
  // Bias partials: one per unpool block and channel, 8 pooled elements per
  // thread and 256 threads per block: n*Ho*Wo*C / 2048 * C = 128 n floats
  // for each of the three layers.
  L.bpart = take(4 * 128 * N);
  L.total = off;
  return L;
}

struct CnnArgs {
  int chains, n, want_grad;
  int64_t n_obs, n_rows, ld;
  const float* X;       // image rows: 3072 floats (32x32x3 NHWC) at X + row*ld
  const float* labels;  // label of row r at labels[r * label_ld]
  int64_t label_ld;
  const float* mask;
  const int32_t* idx;
  int64_t idx_stride;
  const float* w;
  float prior_scale, temperature;
  double* U;
  float* grad;
  float* lk;
  double* lk_var;
  int* status;
  bf16 *w1i, *w2b, *w3b, *x8, *p1, *col2, *p2, *p3;
  float *dp2, *dp1;
  bf16 *dy1, *dy2, *dy3;
  uint8_t *m1, *m2, *m3;
  int32_t* lab;
  float *dp3, *gl;
  double *psq, *plk;
  float *part, *bpart;
};

__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }

// ---------------------------------------------------------------------------
// Weights to BF16 and partial sums of squares: conv2 and conv3 in HWIO
// order, conv1 as the unswizzled K-major B of its GEMM, W1i [8 K groups][64
// output channels][8 slots]: group g = 2 kh + p, slot s weighs input channel
// s % 3 of tap (kh, p + s / 3); zero for s >= 6, for (p = 1, s < 3), for
// groups >= 6 and outputs >= 32.  Grid (kPrepBlocks, chains).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) cnn_prep_kernel(const CnnArgs a) {
  __shared__ double red[32];
  const int c = blockIdx.y;
  const float* w = a.w + static_cast<int64_t>(c) * kP;
  for (int e = blockIdx.x * 256 + threadIdx.x; e < kG1 * 64 * kX8; e += kPrepBlocks * 256) {
    const int g = e / (64 * kX8), co = (e / kX8) % 64, sl = e % kX8;
    const int kh = g >> 1, pp = g & 1, kw = pp + sl / kInC, ci = sl % kInC;
    const bool real = g < 6 && co < kC1 && sl < 2 * kInC && (pp == 0 || sl >= kInC);
    const float v = real ? __ldg(w + oW1 + ((kh * 3 + kw) * kInC + ci) * kC1 + co) : 0.f;
    a.w1i[static_cast<int64_t>(c) * kG1 * 64 * kX8 + e] = __float2bfloat16_rn(v);
  }
  float sq = 0.f;
  for (int64_t i = blockIdx.x * 256 + threadIdx.x; i < kP; i += kPrepBlocks * 256) {
    const float v = __ldg(w + i);
    sq = fmaf(v, v, sq);
    if (i >= oW2 && i < ob3)
      a.w2b[static_cast<int64_t>(c) * kK2 * kC2 + (i - oW2)] = __float2bfloat16_rn(v);
    else if (i >= oW3 && i < obd)
      a.w3b[static_cast<int64_t>(c) * kK3 * kC3 + (i - oW3)] = __float2bfloat16_rn(v);
  }
  const double tot = block_sum(static_cast<double>(sq), red);
  if (threadIdx.x == 0) a.psq[c * kPrepBlocks + blockIdx.x] = tot;
}

// Row of pixel (h, w) of a 32 x 32 image in conv1's GEMM (and in its output
// gradient dY1): a 128-row tile holds the 16 columns w0 .. w0 + 15 (w0 = 0
// or 16) of image rows 8u .. 8u + 7, the (16 W, 8 H) box of one TMA load
// in row-major order.  Every 32 rows hold image rows 2k (lanes 0-15) and
// 2k + 1 (lanes 16-31), so that every 2 x 2 pool window lies in one warp's
// rows, at lanes (l, l ^ 1, l ^ 16, l ^ 17).
__host__ __device__ __forceinline__ int conv1_row(int h, int w) {
  return ((h >> 3) << 8) | ((w >> 4) << 7) | ((h & 7) << 4) | (w & 15);
}
// Its inverse: the pixel of row r (0 <= r < 1024).
__host__ __device__ __forceinline__ void conv1_pixel(int r, int& h, int& w) {
  h = ((r >> 8) << 3) | ((r >> 4) & 7);
  w = (((r >> 7) & 1) << 4) | (r & 15);
}

// ---------------------------------------------------------------------------
// Gather of the minibatch images as BF16 X8 [n, 32, 32, 8] in natural pixel
// order, pixel (h, w) holding channels 0-2 of (h, w - 1) (zero at w = 0),
// channels 0-2 of (h, w) and two zeros, plus labels.
// Grid (n*1024/256, chains): one thread per pixel, one 16-byte store each.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) cnn_gather1_kernel(const CnnArgs a) {
  const int c = blockIdx.y;
  const int p = blockIdx.x * 256 + threadIdx.x;
  if (p >= a.n * 1024) return;
  const int i = p >> 10, hw = p & 1023;
  int64_t o = a.idx[static_cast<int64_t>(c) * a.idx_stride + i];
  if (o < 0 || o >= a.n_rows) {
    raise_status(a.status, GBSGMC_ERR_INDEX);
    o = 0;
  }
  if (hw == 0) {
    const float lf = __ldg(a.labels + o * a.label_ld);
    int lab = static_cast<int>(lf);
    if (!(lf >= 0.f) || lab >= kClasses) {
      raise_status(a.status, GBSGMC_ERR_INDEX);
      lab = 0;
    }
    a.lab[static_cast<int64_t>(c) * a.n + i] = lab;
  }
  const float* px = a.X + o * a.ld + hw * kInC;
  const bool left = (hw & 31) != 0;
  const float l0 = left ? __ldg(px - 3) : 0.f, l1 = left ? __ldg(px - 2) : 0.f,
              l2 = left ? __ldg(px - 1) : 0.f;
  const __nv_bfloat162 q0 = __floats2bfloat162_rn(l0, l1);
  const __nv_bfloat162 q1 = __floats2bfloat162_rn(l2, __ldg(px));
  const __nv_bfloat162 q2 = __floats2bfloat162_rn(__ldg(px + 1), __ldg(px + 2));
  reinterpret_cast<uint4*>(a.x8)[static_cast<int64_t>(c) * a.n * 1024 + p] =
      make_uint4(*reinterpret_cast<const uint32_t*>(&q0), *reinterpret_cast<const uint32_t*>(&q1),
                 *reinterpret_cast<const uint32_t*>(&q2), 0u);
}

// ---------------------------------------------------------------------------
// im2col of a pooled map P [n, H, W, C] -> Col [n*H*W, Kp], K = (kh, kw, ci):
// the 9C real columns of each row (row stride Kp); the columns 9C..Kp-1 are
// never written (the tensor maps that read Col end at 9C, so their boxes
// read zeros there).  One thread per 8 consecutive K entries (C is a
// multiple of 8).  Grid (ceil(n*H*W*9C/8 / 256), chains).
// ---------------------------------------------------------------------------
template <int H, int W, int C, int Kp>
__global__ void __launch_bounds__(256) cnn_im2col_kernel(const bf16* Pin, bf16* Col, int n) {
  constexpr int G = 9 * C / 8;  // 8-column groups per row
  const int c = blockIdx.y;
  const int groups = n * H * W * G;
  const int e = blockIdx.x * 256 + threadIdx.x;
  if (e >= groups) return;
  const int k0 = (e % G) * 8;
  const int pix = e / G;
  const int x = pix % W, y = (pix / W) % H;
  const int i = pix / (W * H);
  uint4 v = make_uint4(0, 0, 0, 0);
  const int tap = k0 / C, ci = k0 % C;
  const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
  if (yy >= 0 && yy < H && xx >= 0 && xx < W)
    v = *reinterpret_cast<const uint4*>(Pin + static_cast<int64_t>(c) * n * H * W * C +
                                        ((i * H + yy) * W + xx) * C + ci);
  *reinterpret_cast<uint4*>(Col + (static_cast<int64_t>(c) * n * H * W + pix) * Kp + k0) = v;
}

// ---------------------------------------------------------------------------
// Dense layer, softmax likelihood and its adjoint for kDenseImgs images of a
// chain per block.  Writes lk, dlogits g = dU/dlogits (fp32), dP3 = g Wd^T
// and the per-image likelihood terms.  Grid (ceil(n / kDenseImgs), chains),
// 16 threads per image: thread (image j = t / 16, slice s = t % 16) handles
// the features f = s, s + 16, ...; an image's 16 threads are one half-warp
// and reduce by shuffles.  The block first copies Wd (80 KB) and its images'
// P3 rows (4 KB each) into shared memory with all loads in flight: a
// half-warp then reads 16 Wd rows 40 bytes apart, 16 distinct banks (the
// other half-warp the same words), and 16 consecutive P3 features.
// ---------------------------------------------------------------------------
constexpr int kDenseImgs = 16;
static_assert(oWd % 2 == 0 && kP % 2 == 0, "Wd is copied as float2");
constexpr size_t kDenseSmem =
    sizeof(float) * kFlat * kClasses + sizeof(bf16) * kDenseImgs * kFlat;

__global__ void __launch_bounds__(kDenseImgs * 16) cnn_dense_kernel(const CnnArgs a) {
  extern __shared__ float wd_s[];  // Wd [2048][10], then P3 rows [kDenseImgs][2048]
  bf16* x_s = reinterpret_cast<bf16*>(wd_s + kFlat * kClasses);
  __shared__ float g_s[kDenseImgs][kClasses];
  const unsigned full = 0xffffffffu;
  const int c = blockIdx.y, t = threadIdx.x, j = t >> 4, sl = t & 15;
  const int i = blockIdx.x * kDenseImgs + j;
  const bool live = i < a.n;
  const float* w = a.w + static_cast<int64_t>(c) * kP;
  {
    // oWd and kP are even: the chain's Wd starts 8-byte aligned.
    const float2* src = reinterpret_cast<const float2*>(w + oWd);
    float2* dst = reinterpret_cast<float2*>(wd_s);
#pragma unroll 8
    for (int e = t; e < kFlat * kClasses / 2; e += kDenseImgs * 16) dst[e] = __ldg(src + e);
    // The block's images, 16 bytes per load (rows past n are not read).
    const int i0 = blockIdx.x * kDenseImgs;
    const int rows = min(kDenseImgs, a.n - i0);
    const uint4* xs = reinterpret_cast<const uint4*>(a.p3 + (static_cast<int64_t>(c) * a.n + i0) * kFlat);
    uint4* xd = reinterpret_cast<uint4*>(x_s);
#pragma unroll 8
    for (int e = t; e < kDenseImgs * kFlat / 8; e += kDenseImgs * 16)
      if (e < rows * (kFlat / 8)) xd[e] = __ldg(xs + e);
  }
  __syncthreads();
  const bf16* x = x_s + j * kFlat;
  float acc[kClasses];
#pragma unroll
  for (int k = 0; k < kClasses; ++k) acc[k] = 0.f;
#pragma unroll 4
  for (int f = sl; f < kFlat; f += 16) {
    const float xv = live ? bf(x[f]) : 0.f;
    const float* wr = wd_s + f * kClasses;
#pragma unroll
    for (int k = 0; k < kClasses; ++k) acc[k] = fmaf(xv, wr[k], acc[k]);
  }
#pragma unroll
  for (int k = 0; k < kClasses; ++k)
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(full, acc[k], off);
  if (sl == 0 && live) {
    float logit[kClasses], mx = -INFINITY;
    for (int k = 0; k < kClasses; ++k) {
      logit[k] = acc[k] + __ldg(w + obd + k);
      mx = fmaxf(mx, logit[k]);
    }
    float se = 0.f;
    for (int k = 0; k < kClasses; ++k) se += expf(logit[k] - mx);
    const float lse = mx + logf(se);
    const int lab = a.lab[static_cast<int64_t>(c) * a.n + i];
    const float lk = logit[lab] - lse;
    const float m = a.mask != nullptr ? __ldg(a.mask + static_cast<int64_t>(c) * a.n + i) : 1.f;
    const float scale = static_cast<float>(static_cast<double>(a.n_obs) / a.n / a.temperature);
    for (int k = 0; k < kClasses; ++k) {
      const float pk = expf(logit[k] - lse);
      const float g = -scale * m * ((k == lab ? 1.f : 0.f) - pk);
      g_s[j][k] = g;
      a.gl[(static_cast<int64_t>(c) * a.n + i) * kClasses + k] = g;
    }
    if (a.lk != nullptr) a.lk[static_cast<int64_t>(c) * a.n + i] = lk;
    double* pl = a.plk + (static_cast<int64_t>(c) * a.n + i) * 4;
    pl[0] = static_cast<double>(m) * lk;
    pl[1] = lk;
    pl[2] = static_cast<double>(lk) * lk;
    pl[3] = 0.0;
  }
  if (!a.want_grad) return;
  __syncthreads();
  if (!live) return;
  float gk[kClasses];
#pragma unroll
  for (int k = 0; k < kClasses; ++k) gk[k] = g_s[j][k];
  float* dx = a.dp3 + (static_cast<int64_t>(c) * a.n + i) * kFlat;
#pragma unroll 4
  for (int f = sl; f < kFlat; f += 16) {
    const float* wr = wd_s + f * kClasses;
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < kClasses; ++k) sum = fmaf(gk[k], wr[k], sum);
    dx[f] = sum;
  }
}

// dWd [2048, 10] = sum_i P3_i (x) g_i and dbd = sum_i g_i (likelihood part).
// Grid (kFlat / 128 + 1, chains), 512 threads: feature f = 128 x + t % 128,
// image group q = t / 128 adds the images i = q (mod 4) in order; the four
// partial sums are added in group order.  dlogits are staged in shared
// memory 512 images at a time.
__global__ void __launch_bounds__(512) cnn_dense_grad_kernel(const CnnArgs a) {
  __shared__ float gs[512 * kClasses];
  __shared__ float red[3][128 * kClasses];
  const int c = blockIdx.y, t = threadIdx.x, q = t >> 7;
  float* g = a.grad + static_cast<int64_t>(c) * kP;
  const float* gl = a.gl + static_cast<int64_t>(c) * a.n * kClasses;
  if (blockIdx.x == kFlat / 128) {
    if (t < kClasses) {
      float s = 0.f;
      for (int i = 0; i < a.n; ++i) s += gl[i * kClasses + t];
      g[obd + t] = s;
    }
    return;
  }
  const int f = blockIdx.x * 128 + (t & 127);
  const bf16* x = a.p3 + static_cast<int64_t>(c) * a.n * kFlat + f;
  float acc[kClasses];
#pragma unroll
  for (int k = 0; k < kClasses; ++k) acc[k] = 0.f;
  for (int i0 = 0; i0 < a.n; i0 += 512) {
    const int cnt = min(512, a.n - i0);
    __syncthreads();
    for (int e = t; e < cnt * kClasses; e += 512) gs[e] = gl[i0 * kClasses + e];
    __syncthreads();
    int i = q;
    for (; i + 12 < cnt; i += 16) {
      float xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = bf(x[static_cast<int64_t>(i0 + i + 4 * u) * kFlat]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int k = 0; k < kClasses; ++k)
          acc[k] = fmaf(xv[u], gs[(i + 4 * u) * kClasses + k], acc[k]);
    }
    for (; i < cnt; i += 4) {
      const float xv = bf(x[static_cast<int64_t>(i0 + i) * kFlat]);
#pragma unroll
      for (int k = 0; k < kClasses; ++k) acc[k] = fmaf(xv, gs[i * kClasses + k], acc[k]);
    }
  }
  if (q > 0) {
#pragma unroll
    for (int k = 0; k < kClasses; ++k) red[q - 1][(t & 127) * kClasses + k] = acc[k];
  }
  __syncthreads();
  if (q == 0) {
#pragma unroll
    for (int k = 0; k < kClasses; ++k) {
      float s = acc[k];
      for (int r = 0; r < 3; ++r) s += red[r][t * kClasses + k];
      g[oWd + static_cast<int64_t>(f) * kClasses + k] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Pool-window routing + ReLU mask: for each pooled element (i, py, px, ch),
// the gradient dP = dp[i, py, px, ch] (fp32: the dense layer's adjoint for
// layer 3, the transposed convolution's output for layers 2 and 1) goes to
// the window element its argmax chose if that element was positive (the
// pool's mark byte, bits 0-1 and 2); the three others (and channels
// C..ld-1) get 0:  dY [n, H, W, ld] BF16 (rows in conv1_row order for
// layer 1, kConv1Rows).  One thread per pooled pixel and eight channels:
// 128-bit loads of dp, 64-bit of the marks, 128-bit stores of dY; C and ld
// are multiples of 8.  32-bit index arithmetic (per-chain counts < 2^31).
// Grid (ceil(n*Ho*Wo*C/8 / 256), chains).
// The bias gradient is the column sum of dY, i.e. the sum over pooled
// elements of the routed (BF16-rounded) values: each block adds its threads'
// values per channel in a fixed order and writes
// bpart[(chain * gridDim.x + block) * C + ch]; cnn_bias_sum_kernel adds the
// blocks.  2048 / C threads of a block share a channel group (256 * 8 is a
// multiple of C, so the channel of thread t is 8 t mod C).
// ---------------------------------------------------------------------------
template <int H, int W, int C, int ld, bool kConv1Rows = false>
__global__ void __launch_bounds__(256) cnn_unpool_kernel(bf16* dY, const uint8_t* M,
                                                        const float* dp, int n, float* bpart) {
  __shared__ float red[256 * 8];
  const int c = blockIdx.y;
  const int Ho = H / 2, Wo = W / 2;
  const int pper = n * Ho * Wo * C;
  const int e = (blockIdx.x * 256 + threadIdx.x) * 8;
  const bool active = e < pper;
  float bsum[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) {
  const int ch = e % C;
  const int pix = e / C;
  const int px = pix % Wo, py = (pix / Wo) % Ho, i = pix / (Wo * Ho);
  float g[8];
  {
    const float4* d4 = reinterpret_cast<const float4*>(dp + static_cast<int64_t>(c) * pper + e);
    const float4 u = d4[0], v = d4[1];
    g[0] = u.x; g[1] = u.y; g[2] = u.z; g[3] = u.w;
    g[4] = v.x; g[5] = v.y; g[6] = v.z; g[7] = v.w;
  }
  const uint2 mk = *reinterpret_cast<const uint2*>(M + static_cast<int64_t>(c) * pper + e);
  const uint32_t marks[2] = {mk.x, mk.y};
  const int64_t base = static_cast<int64_t>(c) * n * H * W * ld;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int y = 2 * py + (q >> 1), x = 2 * px + (q & 1);
    const int off = (kConv1Rows ? i * H * W + conv1_row(y, x) : (i * H + y) * W + x) * ld;
    __nv_bfloat162 o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t m0 = (marks[k >> 1] >> (16 * (k & 1))) & 0xffu;
      const uint32_t m1 = (marks[k >> 1] >> (16 * (k & 1) + 8)) & 0xffu;
      const float v0 = ((m0 & 3u) == static_cast<uint32_t>(q) && (m0 & 4u)) ? g[2 * k] : 0.f;
      const float v1 = ((m1 & 3u) == static_cast<uint32_t>(q) && (m1 & 4u)) ? g[2 * k + 1] : 0.f;
      o[k] = __floats2bfloat162_rn(v0, v1);
      bsum[2 * k] += __low2float(o[k]);
      bsum[2 * k + 1] += __high2float(o[k]);
    }
    *reinterpret_cast<uint4*>(dY + base + off + ch) = *reinterpret_cast<const uint4*>(o);
    for (int extra = C + ch; extra < ld; extra += C)
      *reinterpret_cast<uint4*>(dY + base + off + extra) = make_uint4(0u, 0u, 0u, 0u);
  }
  }  // active
#pragma unroll
  for (int k = 0; k < 8; ++k) red[threadIdx.x * 8 + k] = bsum[k];
  __syncthreads();
  if (static_cast<int>(threadIdx.x) < C) {
    const int t = threadIdx.x, group = t / 8, k = t % 8, groups = C / 8;
    float s = 0.f;
    for (int u = group; u < 256; u += groups) s += red[u * 8 + k];
    bpart[(static_cast<int64_t>(c) * gridDim.x + blockIdx.x) * C + t] = s;
  }
}

// Bias gradient: grad[off + ch] = sum over the unpool blocks' partials in a
// fixed order: thread t adds channel t % C of blocks t / C, t / C + kBiasT /
// C, ... (coalesced along channels, eight loads in flight), then the
// kBiasT / C partial sums of a channel are added in order.  Grid (chains),
// kBiasT threads (enough loads in flight for the few blocks this grid has);
// C divides kBiasT.
constexpr int kBiasT = 1024;

__global__ void __launch_bounds__(kBiasT) cnn_bias_sum_kernel(const float* bpart, int blocks,
                                                              int C, float* grad, int64_t off) {
  __shared__ float acc[kBiasT];
  const int c = blockIdx.x, t = threadIdx.x, ch = t % C, g0 = t / C, step = kBiasT / C;
  const float* p = bpart + static_cast<int64_t>(c) * blocks * C + ch;
  float s = 0.f;
#pragma unroll 8
  for (int q = g0; q < blocks; q += step) s += p[static_cast<int64_t>(q) * C];
  acc[t] = s;
  __syncthreads();
  if (t < C) {
    float tot = 0.f;
    for (int u = 0; u < step; ++u) tot += acc[u * C + t];
    grad[static_cast<int64_t>(c) * kP + off + t] = tot;
  }
}

// Split-K reduction of a weight gradient: grad[off + e] = sum_s part[c, s, e]
// over e < K * Cout (HWIO order).  Grid (ceil(K*Cout/256), chains).
__global__ void __launch_bounds__(256) cnn_wsum_kernel(const float* part, int splits, int count,
                                                      float* grad, int64_t off) {
  const int c = blockIdx.y, e = blockIdx.x * 256 + threadIdx.x;
  if (e >= count) return;
  const float* p = part + static_cast<int64_t>(c) * splits * count + e;
  float s = 0.f;
  for (int q = 0; q < splits; ++q) s += p[static_cast<int64_t>(q) * count];
  grad[static_cast<int64_t>(c) * kP + off + e] = s;
}

// grad += w / (s^2 T) over every parameter; U and var(lk).  Grid
// (ceil(P/256), chains); block 0 of a chain also writes U, var.
__global__ void __launch_bounds__(256) cnn_finalize_kernel(const CnnArgs a, float pf) {
  __shared__ double red[32];
  const int c = blockIdx.y, t = threadIdx.x;
  const float* w = a.w + static_cast<int64_t>(c) * kP;
  if (a.want_grad && pf != 0.f) {
    const int64_t j = static_cast<int64_t>(blockIdx.x) * 256 + t;
    if (j < kP) {
      float* g = a.grad + static_cast<int64_t>(c) * kP + j;
      *g = fmaf(pf, __ldg(w + j), *g);
    }
  }
  if (blockIdx.x != 0) return;
  double sq = 0.0, lm = 0.0, l1 = 0.0, l2 = 0.0;
  for (int i = t; i < kPrepBlocks; i += 256) sq += a.psq[c * kPrepBlocks + i];
  for (int i = t; i < a.n; i += 256) {
    const double* p = a.plk + (static_cast<int64_t>(c) * a.n + i) * 4;
    lm += p[0];
    l1 += p[1];
    l2 += p[2];
  }
  sq = block_sum(sq, red);
  lm = block_sum(lm, red);
  l1 = block_sum(l1, red);
  l2 = block_sum(l2, red);
  if (t != 0) return;
  double log_prior = 0.0;
  if (a.prior_scale > 0.f) {
    const double s2 = static_cast<double>(a.prior_scale) * a.prior_scale;
    log_prior = -0.5 * sq / s2 -
                static_cast<double>(kP) * (log(static_cast<double>(a.prior_scale)) +
                                           0.91893853320467274178);
  }
  const double U = (-static_cast<double>(a.n_obs) * (lm / a.n) - log_prior) / a.temperature;
  a.U[c] = U;
  if (a.lk_var != nullptr) {
    const double mean = l1 / a.n;
    a.lk_var[c] = fmax(l2 / a.n - mean * mean, 0.0);
  }
  if (!isfinite(U)) raise_status(a.status, GBSGMC_ERR_NONFINITE);
}

// ---------------------------------------------------------------------------
// GEMM epilogues.
// ---------------------------------------------------------------------------

// Forward: ReLU(acc + b) in fp32 and the 2 x 2 max-pool of it, straight from
// the accumulator.  A warp's 32 rows hold whole pool windows: the window of
// lane l is lanes (base, base + 1, base + V, base + V + 1), base = l & ~(V | 1),
// in row-major window order, with V = 16 for conv1 (conv1_row order) and
// conv2 (16 pixels per image row) and V = 8 for conv3 (8 per row).  Per
// output the maximum (first one in window order, as jax's max-pool argmax
// routes the gradient) goes to P [n, Ho, Wo, C] as BF16 and the mark byte
// to M: bits 0-1 the argmax, bit 2 (maximum > 0), the ReLU mask of the
// element the backward pass routes the gradient to.  The four lanes of a
// window each write 8 of every 32 channels (16-byte P stores, 8-byte mark
// stores).  Columns >= C (conv1's padding to N = 64) are skipped.  The
// window maxima of a 32-channel chunk take two exchange stages instead of
// four shuffles per channel: the two pixels of a window row swap the
// halves of the channels they do not keep (16 shuffles) and keep the
// pairwise maximum, then the two rows swap halves again (8 shuffles), so
// that each lane ends with the maxima of its 8 channels; comparisons are
// strict in window order (left before right, top before bottom), which
// keeps the first maximum of the window as the sequential scan does.
template <int H, int W, int V, bool kConv1Rows>
struct EpiConvPool {
  const float* w;
  int64_t boff;
  int C;
  bf16* P;
  uint8_t* M;
  int n;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t*) const {
    if (col0 >= C) return;  // padding columns (warp-uniform)
    const unsigned full = 0xffffffffu;
    const int lane = epi::lane_id();
    const int base = lane & ~(V | 1);
    const int wp = ((lane & V) ? 2 : 0) | (lane & 1);
    // The window's pooled pixel, from the row of its first lane.
    const int r = row0 + base;
    const int i = r / (H * W), rr = r % (H * W);
    int yp, xp;
    if (kConv1Rows) {
      int h, x;
      conv1_pixel(rr, h, x);
      yp = h >> 1;
      xp = x >> 1;
    } else {
      yp = (rr / W) >> 1;
      xp = (rr % W) >> 1;
    }
    const int64_t pix = (static_cast<int64_t>(b) * n + i) * (H / 2) * (W / 2) +
                        yp * (W / 2) + xp;
    const float* bias = w + b * kP + boff;
#pragma unroll 1
    for (int cb = 0; cb < NC / 32; ++cb) {
      const int k0 = col0 + 32 * cb;
      const float bl = __ldg(bias + k0 + lane);
      float v[32];
      load(cb, v);
      float x[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) x[j] = fmaxf(v[j] + __shfl_sync(full, bl, j), 0.f);
      // Stage 1, the window row's two pixels (lanes l, l ^ 1): keep the
      // chunks {cbit, cbit + 2} of 8 channels (kept channel i: i < 8 in
      // the first, i >= 8 in the second), send the other two.
      const bool cbit = (lane & 1) != 0, rbit = (lane & V) != 0;
      float m1[16];
      uint32_t col_bits = 0;  // bit i: kept channel i's maximum is the right pixel
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int lo = q < 8 ? q : 8 + q, hi = lo + 8;
        const float mine = cbit ? x[hi] : x[lo];
        const float other = __shfl_xor_sync(full, cbit ? x[lo] : x[hi], 1);
        const float left = cbit ? other : mine, right = cbit ? mine : other;
        const bool rt = right > left;
        m1[q] = rt ? right : left;
        col_bits |= (rt ? 1u : 0u) << q;
      }
      // Stage 2, the window's two rows (lanes l, l ^ V): the top row keeps
      // kept channels 0-7 (chunk cbit), the bottom row 8-15 (chunk
      // cbit + 2): chunk wp of the 32 channels.
      const uint32_t other_bits = __shfl_xor_sync(full, col_bits, V);
      float best_mine[8];
      uint32_t mark_mine[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int ki = rbit ? 8 + q : q;
        const float mine = rbit ? m1[8 + q] : m1[q];
        const float other = __shfl_xor_sync(full, rbit ? m1[q] : m1[8 + q], V);
        const uint32_t my_col = (col_bits >> ki) & 1u, ot_col = (other_bits >> ki) & 1u;
        const float top = rbit ? other : mine, bot = rbit ? mine : other;
        const uint32_t top_col = rbit ? ot_col : my_col, bot_col = rbit ? my_col : ot_col;
        const bool b2 = bot > top;
        const float best = b2 ? bot : top;
        best_mine[q] = best;
        mark_mine[q] = (b2 ? 2u + bot_col : top_col) | (best > 0.f ? 4u : 0u);
      }
      uint32_t pk[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(best_mine[2 * e], best_mine[2 * e + 1]);
        pk[e] = *reinterpret_cast<const uint32_t*>(&pr);
      }
      const int64_t at = pix * C + k0 + 8 * wp;
      *reinterpret_cast<uint4*>(P + at) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      uint2 mk;
      mk.x = mark_mine[0] | (mark_mine[1] << 8) | (mark_mine[2] << 16) | (mark_mine[3] << 24);
      mk.y = mark_mine[4] | (mark_mine[5] << 8) | (mark_mine[6] << 16) | (mark_mine[7] << 24);
      *reinterpret_cast<uint2*>(M + at) = mk;
    }
  }
};

// Weights: element (row = output channel co, col = im2col column k) of the
// split-K partial product of (virtual) batch bv = chain * splits + split
// lands at part[bv][k][co] (HWIO order), rows < Cout, cols < K.  With x8 the
// columns are conv1's K groups x 8 slots: column 8 g + s (g = 2 kh + p) is
// input channel s % 3 of tap (kh, p + s / 3), for g < 6, s < 6, and p = 0
// or s >= 3.
struct EpiConvGradW {
  float* part;
  int Cout, K;
  bool x8 = false;
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int bv, int row0, int col0, const Load& load,
                                       uint32_t*) const {
    const int co = row0 + epi::lane_id();
    float* dst = part + static_cast<int64_t>(bv) * K * Cout + co;
#pragma unroll 1
    for (int cb = 0; cb < NC / 32; ++cb) {
      float v[32];
      load(cb, v);
      if (co < Cout) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int k = col0 + 32 * cb + j;
          if (x8) {
            const int g = k >> 3, sl = k & 7;
            const int kw = (g & 1) + sl / kInC;
            if (g < 6 && sl < 2 * kInC && ((g & 1) == 0 || sl >= kInC))
              dst[static_cast<int64_t>(((g >> 1) * 3 + kw) * kInC + sl % kInC) * Cout] = v[j];
          } else if (k < K) {
            dst[static_cast<int64_t>(k) * Cout] = v[j];
          }
        }
      }
    }
  }
};

// The transposed convolution's output dX as fp32 [rows, C] (columns >= C of
// the N = 64 tile are skipped), one 128-byte row segment per store.
struct EpiStoreDX {
  float* dx;
  int C;
  int64_t rows;  // rows per chain
  template <int NC, class Load>
  __device__ __forceinline__ void tile(int b, int row0, int col0, const Load& load,
                                       uint32_t* st) const {
    if (col0 >= C) return;  // padding columns (warp-uniform)
    float* dst = dx + (b * rows + row0) * C + col0 + epi::lane_id();
#pragma unroll 1
    for (int cb = 0; cb < NC / 32; ++cb) {
      if (col0 + 32 * cb >= C) break;
      float v[32];
      uint32_t u[32];
      load(cb, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) u[j] = __float_as_uint(v[j]);
      epi::put_rows(st, u);
#pragma unroll 4
      for (int r = 0; r < 32; ++r) dst[r * C + 32 * cb] = __uint_as_float(epi::get(st, r));
    }
  }
};

// Implicit A operand: the K slice k0 of a GEMM over pixels (rows) and taps x
// channels (K) is tap t = k0 / Ck, channels [k0 % Ck, + 64), of the NHWC map
// shifted by the tap: the box (64 channels, W, rows / W, images) of a 4-D map
// (Ck, W, H, chains * n) at (k0 % Ck, s (kw - 1), h0 + s (kh - 1), image),
// s = +1 for a convolution and -1 for its transpose (the box reads zeros
// outside the image: SAME padding).  A tile of 128 rows covers whole image
// rows (W | 128) of one image, or whole images (H W | 128).
template <class Inner>
struct ImplicitA : Inner {
  int H, W, Ck, sign, n;
  static constexpr bool kLoadA = true;
  __device__ __forceinline__ void load_a(void* dst, const CUtensorMap* map, int k0, int m0,
                                         int b, uint64_t* bar) const {
    const int tap = k0 / Ck, c0 = k0 - tap * Ck;
    const int kh = tap / 3, kw = tap - 3 * kh;
    const int img = m0 / (H * W), h0 = (m0 - img * H * W) / W;
    tc::tma_load_4d(dst, map, c0, sign * (kw - 1), h0 + sign * (kh - 1), b * n + img, bar);
  }
};

// Implicit MN-major B operand of a weight gradient dW = dY^T Col: the
// 64-wide N block starting at column nn is tap t = nn / Ck, input channels
// [nn % Ck, + 64), and the K slice k0 is 64 pixels (whole rows of one
// image): the box (64 channels, W, 64 / W, 1) of the 4-D map of the
// layer's input, shifted by the tap.
template <class Inner>
struct ImplicitBmn : Inner {
  int H, W, Ck, n;
  static constexpr bool kLoadB = true;
  __device__ __forceinline__ void load_b(void* dst, const CUtensorMap* map, int nn, int k0,
                                         int b, uint64_t* bar) const {
    const int tap = nn / Ck, c0 = nn - tap * Ck;
    const int kh = tap / 3, kw = tap - 3 * kh;
    const int img = k0 / (H * W), h0 = (k0 - img * H * W) / W;
    tc::tma_load_4d(dst, map, c0, kw - 1, h0 + kh - 1, b * n + img, bar);
  }
};

// K-major B operand of a transposed convolution: for the K slice k0 (tap
// t = k0 / Ckb, output channels [k0 % Ckb, + 64)) the rows n.. of W^T, i.e.
// the box (64 output channels, 64 input channels, 1, 1) of the HWIO weights
// as a 4-D map (Cout, Cin, 9, chains) at (k0 % Ckb, n, t, chain); input
// channels past Cin read zeros.
template <class Inner>
struct TransposedB : Inner {
  int Ckb;
  static constexpr bool kLoadB = true;
  __device__ __forceinline__ void load_b(void* dst, const CUtensorMap* map, int nn, int k0,
                                         int b, uint64_t* bar) const {
    const int tap = k0 / Ckb, c0 = k0 - tap * Ckb;
    tc::tma_load_4d(dst, map, c0, nn, tap, b, bar);
  }
};

// conv1's operands, read by K group from the gathered images X8 and from its
// weights W1i, unswizzled: a pixel's 8 slots (16 bytes) are one core-matrix
// row.  X8 is mapped as image rows of 256 elements (32 pixels x 8 slots):
// 4-D map (256, 32, chains * n, 1) with boxes (128, R, 1, 1), 16 pixels of
// R rows (8 for the forward GEMM, 4 for the weight gradient), whose shift by
// a group's column offset is 8 elements (16 bytes) per pixel; a box is R
// rows of 256 bytes for TMA.  K group g = 2 kh + p of output pixel (h, w)
// is the pixel (h + kh - 1, w + p) of X8 (zeros outside the image).
// Groups 6 and 7 read a box wholly below the image (zeros).  W1i is mapped
// as (256, 2, 8, chains), a group's 64 x 8 weights as two rows of 256, box
// (256, 2, 8, 1).  Forward: the 128-row tile at m0 (columns w0 .. w0 + 15 of
// image rows 8u .. 8u + 7, conv1_row order) is, per group, one box 2 KB
// apart; B is the weights' box.
template <class Inner>
struct Conv1Fwd : Inner {
  int n;
  static constexpr bool kLoadA = true, kLoadB = true, kInterleaveA = true,
                        kInterleaveB = true;
  __device__ __forceinline__ void load_a(void* dst, const CUtensorMap* map, int, int m0, int b,
                                         uint64_t* bar) const {
    const int img = b * n + m0 / 1024, t = (m0 % 1024) / 128;
    const int u = t >> 1, w0 = (t & 1) * 16;
    uint8_t* d = static_cast<uint8_t*>(dst);
#pragma unroll
    for (int g = 0; g < kG1; ++g) {
      const int kh = g >> 1, dx = g & 1;
      const int y = g < 6 ? 8 * u + kh - 1 : 64;
      tc::tma_load_4d(d + g * 2048, map, (w0 + dx) * kX8, y, img, 0, bar);
    }
  }
  __device__ __forceinline__ void load_b(void* dst, const CUtensorMap* map, int nn, int, int b,
                                         uint64_t* bar) const {
    tc::tma_load_4d(dst, map, 0, nn / 32, 0, b, bar);
  }
};

// conv1's weight gradient dW1 = dY1^T Col1 with Col1 read from X8: the
// 64-pixel K slice k0 (the upper or lower 4 rows of a conv1 tile, conv1_row
// order) of the MN-major B is, per real K group (0-5), that slice's (16 W,
// 4 H) box shifted by the group, 1 KB apart.  Only the parts of the stage
// whose products are stored are loaded: A's first 64 rows (output channels;
// 32 real) and B's first 48 columns; the MMAs' other rows and columns read
// whatever the stage held and the epilogue drops them.
template <class Inner>
struct Conv1Bmn : Inner {
  int n;
  static constexpr bool kLoadA = true, kLoadB = true, kInterleaveB = true;
  static constexpr uint32_t kStageBytes = 64 * kGemmBK * 2 + 6 * 1024;
  __device__ __forceinline__ void load_a(void* dst, const CUtensorMap* map, int k0, int m0,
                                         int b, uint64_t* bar) const {
    tc::tma_load_3d(dst, map, m0, k0, b, bar);
  }
  __device__ __forceinline__ void load_b(void* dst, const CUtensorMap* map, int, int k0, int b,
                                         uint64_t* bar) const {
    const int img = b * n + k0 / 1024, rr = k0 % 1024, t = rr >> 7;
    const int h0 = 8 * (t >> 1) + 4 * ((rr >> 6) & 1), w0 = (t & 1) * 16;
    uint8_t* d = static_cast<uint8_t*>(dst);
#pragma unroll
    for (int g = 0; g < 6; ++g) {
      const int kh = g >> 1, dx = g & 1;
      tc::tma_load_4d(d + g * 1024, map, (w0 + dx) * kX8, h0 + kh - 1, img, 0, bar);
    }
  }
};

// A weight gradient whose output channels fill only the first 64 of the
// GEMM's 128 rows: A's first 64 rows are loaded (one MN-major box), the
// MMAs' other rows read whatever the stage held and the epilogue drops them.
template <class Inner>
struct HalfA : Inner {
  static constexpr bool kLoadA = true;
  static constexpr uint32_t kStageBytes = 2 * 64 * kGemmBK * 2;
  __device__ __forceinline__ void load_a(void* dst, const CUtensorMap* map, int k0, int m0,
                                         int b, uint64_t* bar) const {
    tc::tma_load_3d(dst, map, m0, k0, b, bar);
  }
};

// A transposed convolution whose output channels fill only kRows of the
// GEMM's N = 64 columns: B's box holds those kRows rows (the map's box is
// 64 x kRows), the MMAs' other columns read whatever the stage held and the
// epilogue drops them; the stage expects A's bytes and kRows rows of B.
template <class Inner, int kRows>
struct TransposedBRows : TransposedB<Inner> {
  static constexpr uint32_t kStageBytes = (kGemmBM + kRows) * kGemmBK * 2;
};

template <class T>
T* view(void* ws, size_t off) {
  return reinterpret_cast<T*>(static_cast<unsigned char*>(ws) + off);
}

int grid1(int64_t work) { return static_cast<int>((work + 255) / 256); }

int run_cnn(CnnArgs& a, const CnnLayout& L, void* ws, cudaStream_t st) {
  a.w1i = view<bf16>(ws, L.w1i);
  a.w2b = view<bf16>(ws, L.w2b);
  a.w3b = view<bf16>(ws, L.w3b);
  a.x8 = view<bf16>(ws, L.x8);
  a.dy1 = view<bf16>(ws, L.dy1);
  a.p1 = view<bf16>(ws, L.p1);
  a.col2 = view<bf16>(ws, L.col2);
  a.dy2 = view<bf16>(ws, L.dy2);
  a.p2 = view<bf16>(ws, L.p2);
  a.dy3 = view<bf16>(ws, L.dy3);
  a.p3 = view<bf16>(ws, L.p3);
  a.m1 = view<uint8_t>(ws, L.m1);
  a.m2 = view<uint8_t>(ws, L.m2);
  a.m3 = view<uint8_t>(ws, L.m3);
  a.dp2 = view<float>(ws, L.dp2);
  a.dp1 = view<float>(ws, L.dp1);
  a.lab = view<int32_t>(ws, L.labels);
  a.dp3 = view<float>(ws, L.dp3);
  a.gl = view<float>(ws, L.gl);
  a.psq = view<double>(ws, L.psq);
  a.plk = view<double>(ws, L.plk);
  a.part = view<float>(ws, L.part);
  a.bpart = view<float>(ws, L.bpart);
  const int C = a.chains, n = a.n;
  const int64_t r1 = int64_t(n) * 1024, r2 = int64_t(n) * 256, r3 = int64_t(n) * 64;
  int rc;
  auto launched = [&](const char* what) { return check_launch(what); };
  // Bias gradient of a layer from its dY [rows, ld] (C real channels).
  // Unpool of a layer (H x H before pooling, Cr channels) and its bias
  // gradient from the unpool blocks' partials.
  auto bias_sum = [&](int H, int Cr, int64_t off) {
    const int blocks = grid1(int64_t(n) * (H / 2) * (H / 2) * Cr / 8);
    cnn_bias_sum_kernel<<<C, kBiasT, 0, st>>>(a.bpart, blocks, Cr, a.grad, off);
    return launched("cnn_bias_sum_kernel");
  };
  auto unpool_grid = [&](int H, int Cr) {
    return dim3(grid1(int64_t(n) * (H / 2) * (H / 2) * Cr / 8), C);
  };
  // Weight gradient of a layer: split-K GEMM into partials, then their sum.
  auto weight_grad = [&](const CUtensorMap& mdy, const CUtensorMap& mcol, int layer, int Cout,
                         int K, int Kp, int64_t rows, int64_t off) {
    GemmRagged rg;
    rg.ksplit = wsplit(layer, n);
    if (Cout > 64) return set_error(GBSGMC_ERR_ARG, "cnn: weight gradient with %d outputs", Cout);
    const HalfA<EpiConvGradW> e{{a.part, Cout, K}};
    int r = launch_gemm<64, true, true>(mdy, mcol, C, 128, Kp, static_cast<int>(rows), a.status,
                                        e, st, rg);
    if (r) return r;
    cnn_wsum_kernel<<<dim3(grid1(int64_t(K) * Cout), C), 256, 0, st>>>(a.part, rg.ksplit,
                                                                       K * Cout, a.grad, off);
    return launched("cnn_wsum_kernel");
  };

  cnn_prep_kernel<<<dim3(kPrepBlocks, C), 256, 0, st>>>(a);
  if ((rc = launched("cnn_prep_kernel"))) return rc;
  cnn_gather1_kernel<<<dim3(grid1(r1), C), 256, 0, st>>>(a);
  if ((rc = launched("cnn_gather1_kernel"))) return rc;

  // Tensor maps (columns, rows, chains), and 4-D maps (channels, W, H,
  // images) of the NHWC maps the implicit GEMMs read by tap.
  const int64_t imgs = int64_t(C) * n;
  CUtensorMap m_x8, m_x8h, m_w1i, m_col2, m_w2, m_w3, m_p2a;
  if ((rc = make_tmap_bf16_4d_plain(&m_x8, a.x8, {32 * kX8, 32, imgs, 1},
                                    {32 * kX8, 1024 * kX8, imgs * 1024 * kX8},
                                    {16 * kX8, 8, 1, 1})) ||
      (rc = make_tmap_bf16_4d_plain(&m_x8h, a.x8, {32 * kX8, 32, imgs, 1},
                                    {32 * kX8, 1024 * kX8, imgs * 1024 * kX8},
                                    {16 * kX8, 4, 1, 1})) ||
      (rc = make_tmap_bf16_4d_plain(&m_w1i, a.w1i, {32 * kX8, 2, kG1, C},
                                    {32 * kX8, 64 * kX8, kG1 * 64 * kX8},
                                    {32 * kX8, 2, kG1, 1})) ||
      (rc = make_tmap_bf16_3d(&m_col2, a.col2, kK2, r2, C, kK2p, r2 * kK2p, kGemmBK, kGemmBM)) ||
      (rc = make_tmap_bf16_3d(&m_w2, a.w2b, kC2, kK2, C, kC2, kK2 * kC2, 64, 64)) ||
      (rc = make_tmap_bf16_3d(&m_w3, a.w3b, kC3, kK3, C, kC3, kK3 * kC3, 64, 64)) ||
      (rc = make_tmap_bf16_4d(&m_p2a, a.p2, {kC2, 8, 8, imgs}, {kC2, 8 * kC2, 64 * kC2},
                              {64, 8, 8, 2})))
    return rc;

  // conv1+pool1 (implicit) -> im2col2 -> conv2+pool2 -> conv3+pool3
  // (implicit): each conv GEMM's epilogue writes the pooled BF16 map and the
  // marks.  conv1 runs as N = 64 (W1i's zero output channels past 32) and
  // K = 8 groups x 8 slots; its epilogue skips the padding columns.
  const Conv1Fwd<EpiConvPool<32, 32, 16, true>> e1{{a.w, ob1, kC1, a.p1, a.m1, n}, n};
  if ((rc = launch_gemm<64, false, false>(m_x8, m_w1i, C, r1, 64, kK1i, a.status, e1, st)))
    return rc;
  cnn_im2col_kernel<16, 16, kC1, kK2p><<<dim3(grid1(r2 * kK2 / 8), C), 256, 0, st>>>(
      a.p1, a.col2, n);
  if ((rc = launched("cnn_im2col_kernel 2"))) return rc;
  const EpiConvPool<16, 16, 16, false> e2{a.w, ob2, kC2, a.p2, a.m2, n};
  if ((rc = launch_gemm<64, false, true>(m_col2, m_w2, C, r2, kC2, kK2p, a.status, e2, st)))
    return rc;
  // conv3, implicit: A tiles are P2's tap-shifted 2-image boxes.
  const ImplicitA<EpiConvPool<8, 8, 8, false>> e3{{a.w, ob3, kC3, a.p3, a.m3, n},
                                                   8, 8, kC2, 1, n};
  if ((rc = launch_gemm<128, false, true>(m_p2a, m_w3, C, r3, kC3, kK3, a.status, e3, st)))
    return rc;
  static const cudaError_t dense_attr = cudaFuncSetAttribute(
      cnn_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kDenseSmem));
  if (dense_attr != cudaSuccess)
    return set_error(GBSGMC_ERR_CUDA, "cnn_dense_kernel: %s", cudaGetErrorString(dense_attr));
  cnn_dense_kernel<<<dim3((n + kDenseImgs - 1) / kDenseImgs, C), kDenseImgs * 16, kDenseSmem,
                     st>>>(a);
  if ((rc = launched("cnn_dense_kernel"))) return rc;

  if (a.want_grad) {
    cnn_dense_grad_kernel<<<dim3(kFlat / 128 + 1, C), 512, 0, st>>>(a);
    if ((rc = launched("cnn_dense_grad_kernel"))) return rc;
    // Layer 3: dY3 (routing of dP3), db3, dW3 = dY3^T Col3 (implicit: B
    // blocks are P2's tap-shifted images), dP2 = the transposed convolution
    // of dY3 (implicit: A tiles are dY3's tap-shifted 2-image boxes).
    cnn_unpool_kernel<8, 8, kC3, kC3><<<unpool_grid(8, kC3), 256, 0, st>>>(
        a.dy3, a.m3, a.dp3, n, a.bpart);
    if ((rc = launched("cnn_unpool_kernel 3")) || (rc = bias_sum(8, kC3, ob3))) return rc;
    CUtensorMap m_dy3t, m_p2b, m_dy3a, m_w3t;
    if ((rc = make_tmap_bf16_3d(&m_dy3t, a.dy3, kC3, r3, C, kC3, r3 * kC3, 64, 64)) ||
        (rc = make_tmap_bf16_4d(&m_p2b, a.p2, {kC2, 8, 8, imgs}, {kC2, 8 * kC2, 64 * kC2},
                                {64, 8, 8, 1})) ||
        (rc = make_tmap_bf16_4d(&m_dy3a, a.dy3, {kC3, 8, 8, imgs}, {kC3, 8 * kC3, 64 * kC3},
                                {64, 8, 8, 2})) ||
        (rc = make_tmap_bf16_4d(&m_w3t, a.w3b, {kC3, kC2, 9, C}, {kC3, kC2 * kC3, kK3 * kC3},
                                {64, 64, 1, 1})))
      return rc;
    {
      GemmRagged rg;
      rg.ksplit = wsplit(3, n);
      const ImplicitBmn<EpiConvGradW> e{{a.part, kC3, kK3}, 8, 8, kC2, n};
      if ((rc = launch_gemm<64, true, true>(m_dy3t, m_p2b, C, 128, kK3, static_cast<int>(r3),
                                            a.status, e, st, rg)))
        return rc;
      cnn_wsum_kernel<<<dim3(grid1(int64_t(kK3) * kC3), C), 256, 0, st>>>(a.part, rg.ksplit,
                                                                          kK3 * kC3, a.grad, oW3);
      if ((rc = launched("cnn_wsum_kernel"))) return rc;
    }
    const TransposedB<ImplicitA<EpiStoreDX>> d3{{{a.dp2, kC2, r3}, 8, 8, kC3, -1, n}, kC3};
    if ((rc = launch_gemm<64, false, false>(m_dy3a, m_w3t, C, r3, kC2, 9 * kC3, a.status, d3,
                                            st)))
      return rc;
    // Layer 2: dY2 (routing of dP2), db2, dW2 = dY2^T Col2, dP1 = the
    // transposed convolution of dY2 (implicit).
    cnn_unpool_kernel<16, 16, kC2, kC2><<<unpool_grid(16, kC2), 256, 0, st>>>(
        a.dy2, a.m2, a.dp2, n, a.bpart);
    if ((rc = launched("cnn_unpool_kernel 2")) || (rc = bias_sum(16, kC2, ob2))) return rc;
    CUtensorMap m_dy2t, m_col2t, m_dy2a, m_w2t;
    if ((rc = make_tmap_bf16_3d(&m_dy2t, a.dy2, kC2, r2, C, kC2, r2 * kC2, 64, 64)) ||
        (rc = make_tmap_bf16_3d(&m_col2t, a.col2, kK2, r2, C, kK2p, r2 * kK2p, 64, 64)) ||
        (rc = make_tmap_bf16_4d(&m_dy2a, a.dy2, {kC2, 16, 16, imgs},
                                {kC2, 16 * kC2, 256 * kC2}, {64, 16, 8, 1})) ||
        (rc = make_tmap_bf16_4d(&m_w2t, a.w2b, {kC2, kC1, 9, C}, {kC2, kC1 * kC2, kK2 * kC2},
                                {64, kC1, 1, 1})))
      return rc;
    if ((rc = weight_grad(m_dy2t, m_col2t, 2, kC2, kK2, kK2p, r2, oW2))) return rc;
    const TransposedBRows<ImplicitA<EpiStoreDX>, kC1> d2{
        {{{a.dp1, kC1, r2}, 16, 16, kC2, -1, n}, kC2}};
    if ((rc = launch_gemm<64, false, false>(m_dy2a, m_w2t, C, r2, 64, 9 * kC2, a.status, d2,
                                            st)))
      return rc;
    // Layer 1.
    cnn_unpool_kernel<32, 32, kC1, kA1ld, true><<<unpool_grid(32, kC1), 256, 0, st>>>(
        a.dy1, a.m1, a.dp1, n, a.bpart);
    if ((rc = launched("cnn_unpool_kernel 1")) || (rc = bias_sum(32, kC1, ob1))) return rc;
    // dW1 = dY1^T Col1, Col1 read by K group from X8 (N = 8 groups x 8 slots).
    CUtensorMap m_dy1t;
    if ((rc = make_tmap_bf16_3d(&m_dy1t, a.dy1, kA1ld, r1, C, kA1ld, r1 * kA1ld, 64, 64)))
      return rc;
    {
      GemmRagged rg;
      rg.ksplit = wsplit(1, n);
      const Conv1Bmn<EpiConvGradW> e{{a.part, kC1, kK1, true}, n};
      if ((rc = launch_gemm<64, true, true>(m_dy1t, m_x8h, C, 128, kK1i, static_cast<int>(r1),
                                            a.status, e, st, rg)))
        return rc;
      cnn_wsum_kernel<<<dim3(grid1(int64_t(kK1) * kC1), C), 256, 0, st>>>(a.part, rg.ksplit,
                                                                          kK1 * kC1, a.grad, oW1);
      if ((rc = launched("cnn_wsum_kernel"))) return rc;
    }
  }

  const double s2 = static_cast<double>(a.prior_scale) * a.prior_scale;
  const float pf = a.prior_scale > 0.f ? static_cast<float>(1.0 / (s2 * a.temperature)) : 0.f;
  cnn_finalize_kernel<<<dim3(a.want_grad ? grid1(kP) : 1, C), 256, 0, st>>>(a, pf);
  return launched("cnn_finalize_kernel");
}

}  // namespace
}  // namespace gbsgmc

using namespace gbsgmc;

extern "C" int64_t gbsgmc_cnn_param_count(void) { return kP; }

extern "C" size_t gbsgmc_cnn_workspace_bytes(int chains, int n) {
  if (chains <= 0 || n <= 0 || n % 2 != 0) return 0;
  return cnn_layout(chains, n).total;
}

extern "C" int gbsgmc_cnn_value_and_grad(const gbsgmc_cnn* model, int chains, int n,
                                         const int32_t* idx_dev, int64_t idx_stride,
                                         const float* mask_dev, const float* w_dev,
                                         double* U_dev, float* grad_dev, float* lk_dev,
                                         double* lk_var_dev, void* workspace_dev,
                                         size_t workspace_bytes, int* status_dev,
                                         gbsgmc_stream_t stream) {
  if (model == nullptr || model->X == nullptr || model->labels == nullptr)
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: null model or data");
  if (chains < 0 || n < 0) return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: negative size");
  if (chains == 0) return GBSGMC_OK;
  if (n == 0 || n % 2 != 0 || chains > 65535 || n > 65536)
    return set_error(GBSGMC_ERR_SHAPE,
                     "cnn_value_and_grad: n must be a positive even number (got %d)", n);
  if (model->ld < kImg * kImg * kInC || model->label_ld < 1 || model->n_obs < 1 ||
      model->n_rows < 0 || model->n_rows >= (1ll << 31))
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: bad strides or sizes");
  if (!(model->temperature > 0.f) || !(model->prior_scale >= 0.f))
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: bad temperature or prior scale");
  if (idx_dev == nullptr || w_dev == nullptr || U_dev == nullptr || workspace_dev == nullptr ||
      status_dev == nullptr)
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: null pointer");
  if (idx_stride < n) return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: idx_stride < n");
  if (reinterpret_cast<uintptr_t>(workspace_dev) % 256 != 0)
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: workspace must be 256-byte aligned");
  const CnnLayout L = cnn_layout(chains, n);
  if (workspace_bytes < L.total)
    return set_error(GBSGMC_ERR_ARG, "cnn_value_and_grad: workspace of %zu bytes, need %zu",
                     workspace_bytes, L.total);
  CnnArgs a{};
  a.chains = chains;
  a.n = n;
  a.want_grad = grad_dev != nullptr;
  a.n_obs = model->n_obs;
  a.n_rows = model->n_rows > 0 ? model->n_rows : model->n_obs;
  a.ld = model->ld;
  a.X = model->X;
  a.labels = model->labels;
  a.label_ld = model->label_ld;
  a.mask = mask_dev;
  a.idx = idx_dev;
  a.idx_stride = idx_stride;
  a.w = w_dev;
  a.prior_scale = model->prior_scale;
  a.temperature = model->temperature;
  a.U = U_dev;
  a.grad = grad_dev;
  a.lk = lk_dev;
  a.lk_var = lk_var_dev;
  a.status = status_dev;
  return run_cnn(a, L, workspace_dev, static_cast<cudaStream_t>(stream));
}
