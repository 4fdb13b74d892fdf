// Gaussian-state glue on the device: from a pure state's xp covariance and means to the serving
// state (B, gamma) and the vacuum amplitude's ingredients, the conversions of
// thewalrus/quantum/conversions.py:69-170 (Qmat, Amat, complex_to_real_displacements) and
// fock_tensors.py:45-98 (pure_state_amplitude's prefactor):
//   Q = [[<a^+ a>, <a a>^*], [<a a>, <a^+ a>^*]] + I       (the Husimi matrix, 2M x 2M, Hermitian
//                                                          positive definite for a valid state)
//   B = -(Q^-1)[M:, :M]                                     ((X (I - Q^-1)^*)[:M, :M]^*)
//   alpha = (mu_x + i mu_p) / sqrt(2 hbar),  gamma = alpha - B alpha^*
//   <0|psi> = exp(-(|alpha|^2 - alpha^H B alpha^*) / 2) / det(Q)^(1/4)
// Q is factored by a right-looking Cholesky decomposition Q = L L^H (no pivoting: Q is Hermitian
// positive definite; a non-positive pivot means the covariance is not a physical state and is
// reported), det Q = prod |L_kk|^2, and the M columns of Q^-1 that B needs come from forward and
// backward substitution, one thread per column.  One CTA does it all in global memory (the work
// is O((2M)^3) once per state, against the sieve's exponential work per request).
#pragma once
#include <cuda_runtime.h>

#include "arith.cuh"

namespace wg {

__device__ __forceinline__ c64 cz(double re, double im) { return {re, im}; }
__device__ __forceinline__ c64 cadd_(c64 a, c64 b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ c64 csub_(c64 a, c64 b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ c64 cmul_(c64 a, c64 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ c64 cmulc_(c64 a, c64 b) {  // a * conj(b)
  return {a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im};
}
__device__ __forceinline__ c64 cconj_(c64 a) { return {a.re, -a.im}; }

// out[0] = log det Q, out[1], out[2] = quad (re, im), out[3] = max_i sum_j |B_ij| (the largest
// absolute row sum), out[4] = 0 on success or 1 + k for a non-positive Cholesky pivot k.
// Work: Q (n x n) and X (n x M), n = 2M, row-major.
static __global__ void __launch_bounds__(1024) gaussian_state_kernel(const double* __restrict__ cov,
                                                                     const double* __restrict__ mu, int M,
                                                                     double hbar, c64* __restrict__ Q,
                                                                     c64* __restrict__ X, c64* __restrict__ B,
                                                                     c64* __restrict__ gamma,
                                                                     double* __restrict__ out) {
  const int n = 2 * M;
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double s_logdet;
  __shared__ int s_fail;
  __shared__ double s_red[1024];
  if (tid == 0) {
    s_logdet = 0.0;
    s_fail = 0;
  }
  // Husimi Q from the covariance (scaled by 2 / hbar): blocks x, xp, p of the xp ordering
  const double sc = 2.0 / hbar;
  for (int e = tid; e < M * M; e += nt) {
    const int i = e / M, j = e % M;
    const double x = cov[(size_t)i * n + j] * sc, p = cov[(size_t)(M + i) * n + M + j] * sc;
    const double xp = cov[(size_t)i * n + M + j] * sc, px = cov[(size_t)j * n + M + i] * sc;  // xp^T
    const c64 adag_a = cz((x + p - (i == j ? 2.0 : 0.0)) / 4.0, (xp - px) / 4.0);
    const c64 a_a = cz((x - p) / 4.0, (xp + px) / 4.0);
    const double d = i == j ? 1.0 : 0.0;
    Q[(size_t)i * n + j] = cz(adag_a.re + d, adag_a.im);
    Q[(size_t)i * n + M + j] = cconj_(a_a);
    Q[(size_t)(M + i) * n + j] = a_a;
    Q[(size_t)(M + i) * n + M + j] = cz(adag_a.re + d, -adag_a.im);
  }
  __syncthreads();
  // right-looking Cholesky, lower triangle in place
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double dk = Q[(size_t)k * n + k].re;
      if (!(dk > 0.0)) {
        s_fail = 1 + k;
      } else {
        const double r = sqrt(dk);
        Q[(size_t)k * n + k] = cz(r, 0.0);
        s_logdet += 2.0 * log(r);
      }
    }
    __syncthreads();
    if (s_fail) break;
    const double r = Q[(size_t)k * n + k].re;
    for (int i = k + 1 + tid; i < n; i += nt) {
      const c64 v = Q[(size_t)i * n + k];
      Q[(size_t)i * n + k] = cz(v.re / r, v.im / r);
    }
    __syncthreads();
    const int w = n - k - 1;
    for (int e = tid; e < w * w; e += nt) {  // trailing update of the lower triangle
      const int i = k + 1 + e / w, j = k + 1 + e % w;
      if (j <= i) Q[(size_t)i * n + j] = csub_(Q[(size_t)i * n + j], cmulc_(Q[(size_t)i * n + k], Q[(size_t)j * n + k]));
    }
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0) out[4] = (double)s_fail;
    return;
  }
  // columns 0..M-1 of Q^-1: L y = e_c, then L^H x = y, one thread per column
  for (int c = tid; c < M; c += nt) {
    for (int i = 0; i < n; ++i) {
      c64 s = cz(i == c ? 1.0 : 0.0, 0.0);
      for (int j = 0; j < i; ++j) s = csub_(s, cmul_(Q[(size_t)i * n + j], X[(size_t)j * M + c]));
      const double r = Q[(size_t)i * n + i].re;
      X[(size_t)i * M + c] = cz(s.re / r, s.im / r);
    }
    for (int i = n - 1; i >= 0; --i) {
      c64 s = X[(size_t)i * M + c];
      for (int j = i + 1; j < n; ++j) s = csub_(s, cmul_(cconj_(Q[(size_t)j * n + i]), X[(size_t)j * M + c]));
      const double r = Q[(size_t)i * n + i].re;
      X[(size_t)i * M + c] = cz(s.re / r, s.im / r);
    }
  }
  __syncthreads();
  // B = -(Q^-1)[M:, :M]
  for (int e = tid; e < M * M; e += nt) {
    const c64 v = X[(size_t)(M + e / M) * M + e % M];
    B[e] = cz(-v.re, -v.im);
  }
  __syncthreads();
  // gamma = alpha - B alpha^*, the row sums of |B| and quad = |alpha|^2 - alpha^H B alpha^*
  const double ra = 1.0 / sqrt(2.0 * hbar);
  double rowmax = 0.0, qre = 0.0, qim = 0.0;
  for (int i = tid; i < M; i += nt) {
    const c64 ai = cz(mu[i] * ra, mu[M + i] * ra);
    c64 bs = cz(0.0, 0.0);
    double rs = 0.0;
    for (int j = 0; j < M; ++j) {
      const c64 b = B[(size_t)i * M + j];
      bs = cadd_(bs, cmul_(b, cz(mu[j] * ra, -mu[M + j] * ra)));
      rs += hypot(b.re, b.im);
    }
    gamma[i] = csub_(ai, bs);
    rowmax = fmax(rowmax, rs);
    const c64 t = cmul_(cconj_(ai), bs);  // alpha_i^* (B alpha^*)_i
    qre += ai.re * ai.re + ai.im * ai.im - t.re;
    qim -= t.im;
  }
  double vals[3] = {rowmax, qre, qim};
  for (int q = 0; q < 3; ++q) {
    s_red[tid] = vals[q];
    __syncthreads();
    for (int h = nt / 2; h > 0; h >>= 1) {
      if (tid < h) s_red[tid] = q == 0 ? fmax(s_red[tid], s_red[tid + h]) : s_red[tid] + s_red[tid + h];
      __syncthreads();
    }
    if (tid == 0) out[q == 0 ? 3 : q] = s_red[0];
    __syncthreads();
  }
  if (tid == 0) {
    out[0] = s_logdet;
    out[4] = 0.0;
  }
}

}  // namespace wg
