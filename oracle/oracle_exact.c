/*
 * Exact hafnians of integer matrices.  TEST INFRASTRUCTURE ONLY: compiled and called by the
 * test-suite and the precision leg of bench.py, never by the product path.
 *
 * The sieve of _calc_hafnian (thewalrus/_hafnian.py:415-467) is a finite sum of integers times
 * [eta^(N/2)] det(I - eta AX_S)^(-1/2), scaled by 2^-(N/2-1) for the Glynn form.  For an integer
 * matrix every one of those is an element of the field F_p once p exceeds N: det(I - eta AX_S)
 * has constant term 1, the series g = c^(-1/2) obeys n g_n = -sum_i c_i (n - i/2) g_(n-i),
 * which divides only by 2 and by n <= N/2, and the prefactors (binomials, signs, the halving of
 * the delta_0 = 0 term, the final power of 2) are integers or inverses of 2.  So this file runs
 * the reference's sieve -- the same mixed-radix term order (find_kept_edges, :162-180) and the
 * same AX_S (get_AX_S, :288-312) -- with every term's characteristic polynomial computed exactly
 * over F_p (Hessenberg reduction by elimination, then the Hessenberg determinant recurrence of
 * charpoly.py:195-282).  Python combines the residues of several 31-bit primes by the Chinese
 * remainder theorem into the exact integer (oracle/__init__.py, exact_hafnian).
 *
 * Each prime is a compile-time constant, so the reductions are multiply-shift sequences.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t u64;

#define DEFINE_EXACT(NAME, P)                                                                        \
  static inline u64 NAME##_mul(u64 a, u64 b) { return (a * b) % (P); }                             \
  static inline u64 NAME##_add(u64 a, u64 b) { u64 s = a + b; return s >= (P) ? s - (P) : s; }     \
  static inline u64 NAME##_sub(u64 a, u64 b) { return a >= b ? a - b : a + (P) - b; }              \
  static u64 NAME##_pow(u64 a, u64 e) {                                                            \
    u64 r = 1;                                                                                       \
    while (e) {                                                                                      \
      if (e & 1) r = NAME##_mul(r, a);                                                               \
      a = NAME##_mul(a, a);                                                                          \
      e >>= 1;                                                                                       \
    }                                                                                                \
    return r;                                                                                        \
  }                                                                                                  \
  static u64 NAME##_inv(u64 a) { return NAME##_pow(a, (P) - 2); }                                  \
  static u64 NAME##_of(int64_t v) {                                                                  \
    int64_t r = v % (int64_t)(P);                                                                    \
    return (u64)(r < 0 ? r + (int64_t)(P) : r);                                                      \
  }                                                                                                  \
  /* [eta^K] det(I - eta H)^(-1/2) for H (m x m, destroyed) */                                    \
  static u64 NAME##_f(u64* H, int m, int K, u64* c, u64* g, u64* cw) {                              \
    /* Hessenberg form by elimination with any nonzero pivot (a similarity) */                     \
    for (int j = 0; j + 2 < m; ++j) {                                                                \
      int piv = -1;                                                                                  \
      for (int r = j + 1; r < m; ++r)                                                                \
        if (H[r * m + j]) { piv = r; break; }                                                        \
      if (piv < 0) continue;                                                                         \
      if (piv != j + 1) {                                                                            \
        for (int cc = 0; cc < m; ++cc) {                                                             \
          u64 t = H[piv * m + cc]; H[piv * m + cc] = H[(j + 1) * m + cc]; H[(j + 1) * m + cc] = t;   \
        }                                                                                            \
        for (int r = 0; r < m; ++r) {                                                                \
          u64 t = H[r * m + piv]; H[r * m + piv] = H[r * m + j + 1]; H[r * m + j + 1] = t;           \
        }                                                                                            \
      }                                                                                              \
      const u64 inv = NAME##_inv(H[(j + 1) * m + j]);                                                \
      for (int a = j + 2; a < m; ++a) {                                                              \
        const u64 l = NAME##_mul(H[a * m + j], inv);                                                 \
        if (!l) continue;                                                                            \
        for (int cc = j; cc < m; ++cc)                                                               \
          H[a * m + cc] = NAME##_sub(H[a * m + cc], NAME##_mul(l, H[(j + 1) * m + cc]));             \
        for (int r = 0; r < m; ++r)                                                                  \
          H[r * m + j + 1] = NAME##_add(H[r * m + j + 1], NAME##_mul(l, H[r * m + a]));              \
      }                                                                                              \
    }                                                                                                \
    /* c_i[t], t <= K: det(I - eta H_i) of the leading i x i block */                              \
    const int W = K + 1;                                                                             \
    for (int t = 0; t <= K; ++t) cw[t] = t == 0;                                                     \
    for (int i = 1; i <= m; ++i) {                                                                   \
      u64* ci = cw + (size_t)i * W;                                                                  \
      const u64* cp = cw + (size_t)(i - 1) * W;                                                      \
      const u64 a = H[(i - 1) * m + (i - 1)];                                                        \
      for (int t = 0; t <= K; ++t) ci[t] = NAME##_sub(cp[t], t ? NAME##_mul(a, cp[t - 1]) : 0);     \
      u64 beta = 1;                                                                                  \
      for (int r = 1; r < i; ++r) {                                                                  \
        beta = NAME##_mul(beta, H[(i - r) * m + (i - r - 1)]);                                       \
        if (!beta) break;                                                                            \
        const u64 T = NAME##_mul(H[(i - r - 1) * m + (i - 1)], beta);                                \
        const u64* cq = cw + (size_t)(i - r - 1) * W;                                                \
        for (int t = r + 1; t <= K; ++t) ci[t] = NAME##_sub(ci[t], NAME##_mul(T, cq[t - r - 1]));  \
      }                                                                                              \
    }                                                                                                \
    memcpy(c, cw + (size_t)m * W, sizeof(u64) * W);                                                  \
    /* g = c^(-1/2): n g_n = -sum_{i=1}^{n} c_i (2n - i)/2 g_(n-i) */                             \
    const u64 inv2 = NAME##_inv(2);                                                                  \
    g[0] = 1;                                                                                        \
    for (int n = 1; n <= K; ++n) {                                                                   \
      u64 s = 0;                                                                                     \
      for (int i = 1; i <= n; ++i)                                                                   \
        s = NAME##_add(s, NAME##_mul(NAME##_mul(c[i], (u64)(2 * n - i)), g[n - i]));                 \
      g[n] = NAME##_sub(0, NAME##_mul(NAME##_mul(s, inv2), NAME##_inv((u64)n)));                     \
    }                                                                                                \
    return g[K];                                                                                     \
  }                                                                                                  \
  int oracle_exact_hafnian_##NAME(const int64_t* A, int n, const int64_t* reps, int E, int glynn,  \
                                  int nthreads, int64_t* out) {                                     \
    int N = 0, maxrep = 0;                                                                           \
    for (int i = 0; i < E; ++i) { N += 2 * (int)reps[i]; if (reps[i] > maxrep) maxrep = (int)reps[i]; } \
    const int K = N / 2;                                                                             \
    int64_t steps = 1;                                                                               \
    for (int i = 0; i < E; ++i) steps *= (i == 0 && glynn) ? (reps[0] + 2) / 2 : reps[i] + 1;       \
    const int mb = maxrep + 1;                                                                       \
    u64* binom = (u64*)calloc((size_t)mb * mb, sizeof(u64));                                        \
    for (int a = 0; a < mb; ++a) {                                                                   \
      binom[a * mb] = 1;                                                                             \
      for (int b = 1; b <= a; ++b)                                                                   \
        binom[a * mb + b] = NAME##_add(binom[(a - 1) * mb + b - 1], b <= a - 1 ? binom[(a - 1) * mb + b] : 0); \
    }                                                                                                \
    if (nthreads < 1) nthreads = 1;                                                                  \
    u64* part = (u64*)calloc((size_t)nthreads, sizeof(u64));                                        \
    _Pragma("omp parallel num_threads(nthreads)") {                                                  \
      int tid = 0, nt = 1;                                                                           \
      EXACT_THREAD_IDS                                                                               \
      const int64_t lo = steps * tid / nt, hi = steps * (tid + 1) / nt;                              \
      const int mm = n > 0 ? n : 1;                                                                  \
      u64* H = (u64*)malloc(sizeof(u64) * mm * mm);                                                  \
      u64* cw = (u64*)malloc(sizeof(u64) * (size_t)(mm + 1) * (K + 1));                             \
      u64 *c = (u64*)malloc(sizeof(u64) * (K + 1)), *g = (u64*)malloc(sizeof(u64) * (K + 1));        \
      int* rows = (int*)malloc(sizeof(int) * mm);                                                    \
      int64_t *kept = (int64_t*)malloc(sizeof(int64_t) * (E > 0 ? E : 1)),                            \
              *delta = (int64_t*)malloc(sizeof(int64_t) * (E > 0 ? E : 1)),                           \
              *dnz = (int64_t*)malloc(sizeof(int64_t) * mm);                                         \
      u64 acc = 0;                                                                                   \
      for (int64_t j = lo; j < hi; ++j) {                                                            \
        int64_t q = j; /* find_kept_edges: mixed radix, edge 0 most significant */                   \
        for (int i = E - 1; i >= 0; --i) {                                                           \
          const int64_t R = (i == 0 && glynn) ? (reps[0] + 2) / 2 : reps[i] + 1;                     \
          kept[i] = q % R;                                                                           \
          q /= R;                                                                                    \
        }                                                                                            \
        int64_t esum = 0;                                                                            \
        u64 pre = 1;                                                                                 \
        for (int i = 0; i < E; ++i) { esum += kept[i]; pre = NAME##_mul(pre, binom[reps[i] * mb + kept[i]]); } \
        int ne = 0;                                                                                  \
        for (int i = 0; i < E; ++i) {                                                                \
          delta[i] = glynn ? 2 * kept[i] - reps[i] : kept[i];                                        \
          if (delta[i]) { rows[ne] = i; dnz[ne] = delta[i]; ++ne; }                                  \
        }                                                                                            \
        for (int i = 0; i < ne; ++i) rows[ne + i] = rows[i] + E;                                     \
        const int m = 2 * ne;                                                                        \
        for (int a = 0; a < m; ++a)                                                                  \
          for (int cc = 0; cc < m; ++cc) {                                                           \
            const int src = cc < ne ? cc + ne : cc - ne;                                             \
            H[a * m + cc] = NAME##_of(A[rows[a] * n + rows[src]] * dnz[cc < ne ? cc : cc - ne]);     \
          }                                                                                          \
        u64 f = m ? NAME##_f(H, m, K, c, g, cw) : (K == 0);                                          \
        if ((K - esum) % 2) pre = NAME##_sub(0, pre);                                                \
        if (glynn && delta[0] == 0) pre = NAME##_mul(pre, NAME##_inv(2));                             \
        acc = NAME##_add(acc, NAME##_mul(pre, f));                                                   \
      }                                                                                              \
      part[tid] = acc;                                                                               \
      free(H); free(cw); free(c); free(g); free(rows); free(kept); free(delta); free(dnz);           \
    }                                                                                                \
    u64 h = 0;                                                                                       \
    for (int t = 0; t < nthreads; ++t) h = NAME##_add(h, part[t]);                                   \
    if (glynn && K > 0) h = NAME##_mul(h, NAME##_pow(NAME##_inv(2), (u64)(K - 1)));                  \
    free(part);                                                                                      \
    free(binom);                                                                                     \
    *out = (int64_t)h;                                                                               \
    return 0;                                                                                        \
  }

#ifdef _OPENMP
#define EXACT_THREAD_IDS tid = omp_get_thread_num(); nt = omp_get_num_threads();
#else
#define EXACT_THREAD_IDS
#endif

DEFINE_EXACT(p0, 2147483647ull)
DEFINE_EXACT(p1, 2147483629ull)
DEFINE_EXACT(p2, 2147483587ull)
DEFINE_EXACT(p3, 2147483579ull)
DEFINE_EXACT(p4, 2147483563ull)
