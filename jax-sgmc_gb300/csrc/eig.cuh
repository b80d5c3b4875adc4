// Symmetric eigendecomposition of small matrices, one CTA per matrix, by the
// cyclic Jacobi method with the round-robin ordering (Golub & Van Loan,
// Matrix Computations, sections 8.5.2 and 8.5.4): each round rotates Pp / 2
// disjoint index pairs at once, Pp - 1 rounds make a sweep that visits every
// pair, and sweeps repeat until the off-diagonal mass is negligible.  fp32,
// like the jnp.linalg calls it replaces.
//
// Conventions of the results (the reference's eigh / svd leave both to
// LAPACK): eigenvalues ascending; each eigenvector scaled so that its
// largest-magnitude component (the first of equal ones) is positive.
#pragma once

#include <cuda_runtime.h>

namespace gbsgmc {

// Largest matrix order: the work matrix and the eigenvectors (2 * 128^2
// floats) fill 128 KB of the CTA's shared memory.
constexpr int kMaxEigDim = 128;

// Pair i of round r of the round-robin schedule over Pp (even) indices.
__device__ __forceinline__ void jacobi_pair(int r, int i, int Pp, int& p, int& q) {
  const int m = Pp - 1;
  if (i == 0) {
    p = m;
    q = r;
  } else {
    p = (r + i) % m;
    q = (r - i + m) % m;
  }
}

// A [Pp * Pp] (row-major, symmetric; rows and columns P .. Pp - 1 zero) is
// diagonalised in place and V [Pp * Pp] receives the eigenvectors as
// columns (A_input = V diag(A) V^T).  rot holds Pp / 2 float2 and red 32
// floats.  Every thread of the block calls this.
__device__ inline void jacobi_eig(float* A, float* V, float2* rot, float* red, int Pp) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < Pp * Pp; e += nt) V[e] = (e / Pp == e % Pp) ? 1.f : 0.f;
  __syncthreads();
  for (int sweep = 0; sweep < 30; ++sweep) {
    // Off-diagonal and total squared mass.
    float off = 0.f, tot = 0.f;
    for (int e = tid; e < Pp * Pp; e += nt) {
      const float a = A[e];
      tot = fmaf(a, a, tot);
      if (e / Pp != e % Pp) off = fmaf(a, a, off);
    }
    for (int s = 16; s > 0; s >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, s);
      tot += __shfl_xor_sync(0xffffffffu, tot, s);
    }
    __syncthreads();
    if (lane == 0) {
      red[warp] = off;
      red[16 + warp] = tot;
    }
    __syncthreads();
    float o = 0.f, t = 0.f;
    for (int w = 0; w < (nt + 31) / 32; ++w) {
      o += red[w];
      t += red[16 + w];
    }
    if (!(o > 1e-13f * t)) break;  // converged (or a zero matrix)
    for (int r = 0; r < Pp - 1; ++r) {
      for (int i = tid; i < Pp / 2; i += nt) {
        int p, q;
        jacobi_pair(r, i, Pp, p, q);
        const float apq = A[p * Pp + q];
        float c = 1.f, s = 0.f;
        if (apq != 0.f) {
          const float tau = (A[q * Pp + q] - A[p * Pp + p]) / (2.f * apq);
          const float tt = copysignf(1.f, tau) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.f)));
          c = 1.f / sqrtf(fmaf(tt, tt, 1.f));
          s = tt * c;
        }
        rot[i] = make_float2(c, s);
      }
      __syncthreads();
      // Rows p, q of J^T A.
      for (int e = tid; e < (Pp / 2) * Pp; e += nt) {
        const int i = e / Pp, k = e - i * Pp;
        int p, q;
        jacobi_pair(r, i, Pp, p, q);
        const float2 cs = rot[i];
        const float ap = A[p * Pp + k], aq = A[q * Pp + k];
        A[p * Pp + k] = cs.x * ap - cs.y * aq;
        A[q * Pp + k] = cs.y * ap + cs.x * aq;
      }
      __syncthreads();
      // Columns p, q of (J^T A) J and of V J.
      for (int e = tid; e < (Pp / 2) * Pp; e += nt) {
        const int i = e / Pp, k = e - i * Pp;
        int p, q;
        jacobi_pair(r, i, Pp, p, q);
        const float2 cs = rot[i];
        const float ap = A[k * Pp + p], aq = A[k * Pp + q];
        A[k * Pp + p] = cs.x * ap - cs.y * aq;
        A[k * Pp + q] = cs.y * ap + cs.x * aq;
        const float vp = V[k * Pp + p], vq = V[k * Pp + q];
        V[k * Pp + p] = cs.x * vp - cs.y * vq;
        V[k * Pp + q] = cs.y * vp + cs.x * vq;
      }
      __syncthreads();
    }
  }
}

// +1 or -1: the sign that makes column j of V (first P rows) have its
// largest-magnitude component (the first of equal ones) positive.
__device__ __forceinline__ float eigvec_sign(const float* V, int Pp, int P, int j) {
  float best = -1.f, sgn = 1.f;
  for (int k = 0; k < P; ++k) {
    const float v = V[k * Pp + j];
    if (fabsf(v) > best) {
      best = fabsf(v);
      sgn = v < 0.f ? -1.f : 1.f;
    }
  }
  return sgn;
}

}  // namespace gbsgmc
