/*
 * CPU oracle for the Glynn / inclusion-exclusion hafnian sieve.  TEST INFRASTRUCTURE ONLY:
 * this file is compiled and called by the test-suite, by the smoke check and by the CPU
 * baseline leg of bench.py, never by the product path.
 *
 * It restates, in plain C, the algorithm of the reference implementation (thewalrus 0.23):
 *   - nb_binom / precompute_binoms        thewalrus/_hafnian.py:26-62
 *   - find_kept_edges (mixed radix)       thewalrus/_hafnian.py:162-180
 *   - f / f_loop / f_loop_odd             thewalrus/_hafnian.py:183-285
 *   - get_AX_S / get_submatrices          thewalrus/_hafnian.py:288-356
 *   - get_submatrix_batch_odd0            thewalrus/_hafnian.py:359-380
 *   - _calc_hafnian                       thewalrus/_hafnian.py:415-467
 *   - _calc_loop_hafnian                  thewalrus/_hafnian.py:511-577
 *   - powertrace (matmul branch, then Householder Hessenberg + La Budde + Cayley-Hamilton)
 *                                         thewalrus/charpoly.py:301-327, :42-125, :195-298
 *   - _calc_loop_hafnian_batch_even/_odd  thewalrus/loop_hafnian_batch.py:50-208
 * with the same term order, the same matrix products and the same combiners, so that the
 * double-precision build agrees with the reference to rounding, and the extended builds
 * (long double, _Float128) serve as the high-precision oracle.
 *
 * One deliberate deviation: powertrace of a 0x0 matrix (every delta zero) returns p_0 = 0
 * and zeros after it, which is what the reference's loops yield once its out-of-bounds
 * read of an empty array (charpoly.py:215-217) is taken out.
 *
 * The file is compiled once per scalar type: OR_REAL names the real type and SFX the
 * symbol suffix (_d double, _ld long double, _q _Float128).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef OR_REAL
#define OR_REAL double
#define SFX _d
#endif
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(x) CAT(x, SFX)

typedef OR_REAL R;
typedef struct { R re, im; } C;
#define CX FN(cx_t)
typedef C CX;

static inline C FN(cmk)(R a, R b) { C z; z.re = a; z.im = b; return z; }
static inline C FN(cadd)(C a, C b) { return FN(cmk)(a.re + b.re, a.im + b.im); }
static inline C FN(csub)(C a, C b) { return FN(cmk)(a.re - b.re, a.im - b.im); }
static inline C FN(cmul)(C a, C b) {
  return FN(cmk)(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline C FN(cscale)(C a, R s) { return FN(cmk)(a.re * s, a.im * s); }
static inline C FN(cconj)(C a) { return FN(cmk)(a.re, -a.im); }
static inline C FN(cdiv)(C a, C b) {
  R d = b.re * b.re + b.im * b.im;
  return FN(cmk)((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}

#if defined(OR_IS_QUAD)
static inline R FN(rsqrt_)(R x) {
  /* Newton refinement of a double seed: sqrt to full _Float128 precision without libquadmath */
  if (x == 0) return 0;
  R y = (R)sqrt((double)x);
  for (int it = 0; it < 3; ++it) y = (y + x / y) / 2;
  return y;
}
#define RSQRT(x) FN(rsqrt_)(x)
#elif defined(OR_IS_LD)
#define RSQRT(x) sqrtl(x)
#else
#define RSQRT(x) sqrt(x)
#endif

static inline R FN(cabs_)(C a) { return RSQRT(a.re * a.re + a.im * a.im); }

/* binomial coefficient table, binoms[i*(mb+1)+j] = C(i, j) for 0<=i,j<=mb (_hafnian.py:26-62) */
static R* FN(make_binoms)(int mb) {
  R* t = (R*)calloc((size_t)(mb + 1) * (mb + 1), sizeof(R));
  for (int i = 0; i <= mb; ++i)
    for (int j = 0; j <= mb; ++j) {
      if (j < 0 || j > i) { t[i * (mb + 1) + j] = 0; continue; }
      if (j == 0 || j == i) { t[i * (mb + 1) + j] = 1; continue; }
      int64_t b = 1;
      int kk = j < i - j ? j : i - j;
      for (int q = 0; q < kk; ++q) { b *= (i - q); b /= (q + 1); }
      t[i * (mb + 1) + j] = (R)b;
    }
  return t;
}

/* mixed-radix digits of j in bases reps[i]+1, most significant first (_hafnian.py:162-180) */
static void FN(kept_edges)(int64_t j, const int64_t* reps, int E, int64_t* out) {
  int64_t num = j;
  for (int i = E - 1; i >= 0; --i) {
    int64_t base = reps[i] + 1;
    out[i] = num % base;
    num /= base;
  }
}

/* ---------------- characteristic polynomial / power traces (charpoly.py) ---------------- */

/* Householder reduction to upper Hessenberg, in place, row-major m x m (charpoly.py:42-125) */
static void FN(hessenberg)(C* H, int m, C* v, C* tmp) {
  for (int k = 1; k < m - 1; ++k) {
    int sz = m - k;
    R nrm2 = 0;
    for (int i = 0; i < sz; ++i) {
      C x = H[(k + i) * m + (k - 1)];
      v[i] = x;
      nrm2 += x.re * x.re + x.im * x.im;
    }
    R sigma_abs = RSQRT(nrm2);
    C sigma = FN(cmk)(sigma_abs, 0);
    if (v[0].re != 0 || v[0].im != 0) {
      R a0 = FN(cabs_)(v[0]);
      sigma = FN(cmk)(sigma_abs * v[0].re / a0, sigma_abs * v[0].im / a0);
    }
    v[0] = FN(cadd)(v[0], sigma);
    R nv = 0;
    for (int i = 0; i < sz; ++i) nv += v[i].re * v[i].re + v[i].im * v[i].im;
    if (nv == 0) continue;
    /* vHA over columns k-1 .. m-1 */
    for (int j = 0; j < m - k + 1; ++j) {
      C s = FN(cmk)(0, 0);
      for (int l = 0; l < sz; ++l) s = FN(cadd)(s, FN(cmul)(FN(cconj)(v[l]), H[(k + l) * m + (k - 1 + j)]));
      tmp[j] = s;
    }
    for (int i = 0; i < sz; ++i)
      for (int j = 0; j < m - k + 1; ++j) {
        C t = FN(cmul)(v[i], tmp[j]);
        t = FN(cscale)(t, 2 / nv);
        H[(k + i) * m + (k - 1 + j)] = FN(csub)(H[(k + i) * m + (k - 1 + j)], t);
      }
    for (int i = 0; i < m; ++i) {
      C s = FN(cmk)(0, 0);
      for (int l = 0; l < sz; ++l) s = FN(cadd)(s, FN(cmul)(H[i * m + k + l], v[l]));
      tmp[i] = s;
    }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < sz; ++j) {
        C t = FN(cmul)(tmp[i], FN(cconj)(v[j]));
        t = FN(cscale)(t, 2 / nv);
        H[i * m + k + j] = FN(csub)(H[i * m + k + j], t);
      }
  }
}

/* La Budde's recurrence on a Hessenberg matrix (charpoly.py:195-282); writes the m
 * coefficients of det(lambda I - H) = lambda^m + poly[0] lambda^{m-1} + ... + poly[m-1]. */
static void FN(labudde)(const C* H, int m, C* c /* m*m scratch */, C* poly) {
#define Hh(i, j) H[((i) - 1) * m + ((j) - 1)]
#define cc(i, j) c[((i) - 1) * m + ((j) - 1)]
  for (int i = 0; i < m * m; ++i) c[i] = FN(cmk)(0, 0);
  int k = m;
  cc(1, 1) = FN(cmk)(-Hh(1, 1).re, -Hh(1, 1).im);
  if (m >= 2) {
    cc(2, 1) = FN(csub)(cc(1, 1), Hh(2, 2));
    cc(2, 2) = FN(csub)(FN(cmul)(Hh(1, 1), Hh(2, 2)), FN(cmul)(Hh(1, 2), Hh(2, 1)));
  }
  for (int i = 3; i <= k; ++i) {
    cc(i, 1) = FN(csub)(cc(i - 1, 1), Hh(i, i));
    for (int j = 2; j < i; ++j) {
      C suma = FN(cmk)(0, 0);
      for (int mm = 1; mm < j - 1; ++mm) {
        C bp = FN(cmk)(1, 0);
        for (int bm = i; bm > i - mm; --bm) bp = FN(cmul)(bp, Hh(bm, bm - 1));
        suma = FN(cadd)(suma, FN(cmul)(FN(cmul)(Hh(i - mm, i), bp), cc(i - mm - 1, j - mm - 1)));
      }
      C bp = FN(cmk)(1, 0);
      for (int bm = i; bm > i - j + 1; --bm) bp = FN(cmul)(bp, Hh(bm, bm - 1));
      C v = FN(csub)(cc(i - 1, j), FN(cmul)(Hh(i, i), cc(i - 1, j - 1)));
      v = FN(csub)(v, suma);
      v = FN(csub)(v, FN(cmul)(Hh(i - j + 1, i), bp));
      cc(i, j) = v;
    }
    C suma = FN(cmk)(0, 0);
    for (int mm = 1; mm < i - 1; ++mm) {
      C bp = FN(cmk)(1, 0);
      for (int bm = i; bm > i - mm; --bm) bp = FN(cmul)(bp, Hh(bm, bm - 1));
      suma = FN(cadd)(suma, FN(cmul)(FN(cmul)(Hh(i - mm, i), bp), cc(i - mm - 1, i - mm - 1)));
    }
    C bp = FN(cmk)(1, 0);
    for (int bm = i; bm > 1; --bm) bp = FN(cmul)(bp, Hh(bm, bm - 1));
    C v = FN(cmul)(Hh(i, i), cc(i - 1, i - 1));
    v = FN(cmk)(-v.re, -v.im);
    v = FN(csub)(v, suma);
    v = FN(csub)(v, FN(cmul)(Hh(1, i), bp));
    cc(i, i) = v;
  }
  for (int i = 1; i <= m; ++i) poly[i - 1] = cc(m, i);
#undef Hh
#undef cc
}

typedef struct {
  C *A1, *A2, *v, *tmp, *cpc, *poly;
} FN(ws_t);

static void FN(ws_init)(FN(ws_t) * w, int m) {
  size_t mm = (size_t)(m > 0 ? m : 1);
  w->A1 = (C*)malloc(mm * mm * sizeof(C));
  w->A2 = (C*)malloc(mm * mm * sizeof(C));
  w->v = (C*)malloc(mm * sizeof(C));
  w->tmp = (C*)malloc(mm * sizeof(C));
  w->cpc = (C*)malloc(mm * mm * sizeof(C));
  w->poly = (C*)malloc(mm * sizeof(C));
}
static void FN(ws_free)(FN(ws_t) * w) {
  free(w->A1); free(w->A2); free(w->v); free(w->tmp); free(w->cpc); free(w->poly);
}

/* power traces p_0 .. p_{n-1} of H (m x m, mutated when the charpoly branch runs),
 * charpoly.py:301-327.  out must hold max(n, 2) entries. */
static void FN(powertrace)(C* H, int m, int n, C* out, FN(ws_t) * w) {
  int minv = n < m ? n : m;
  int cnt = 0;
  C tr = FN(cmk)(0, 0);
  for (int i = 0; i < m; ++i) tr = FN(cadd)(tr, H[i * m + i]);
  out[cnt++] = FN(cmk)((R)m, 0);
  out[cnt++] = tr;
  if (m > 0) {
    memcpy(w->A1, H, sizeof(C) * m * m);
    for (int it = 0; it < minv - 2; ++it) {
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
          C s = FN(cmk)(0, 0);
          for (int l = 0; l < m; ++l) s = FN(cadd)(s, FN(cmul)(w->A1[i * m + l], H[l * m + j]));
          w->A2[i * m + j] = s;
        }
      C t = FN(cmk)(0, 0);
      for (int i = 0; i < m; ++i) t = FN(cadd)(t, w->A2[i * m + i]);
      out[cnt++] = t;
      C* sw = w->A1; w->A1 = w->A2; w->A2 = sw;
    }
  }
  if (n <= m) return;
  /* charpoly branch */
  if (m > 0) {
    FN(hessenberg)(H, m, w->v, w->tmp);
    FN(labudde)(H, m, w->cpc, w->poly);
  }
  for (int it = minv; it < n; ++it) {
    C s = FN(cmk)(0, 0);
    for (int k = 0; k < m; ++k) s = FN(csub)(s, FN(cmul)(w->poly[k], out[cnt - k - 1]));
    out[cnt++] = s;
  }
}

/* f: coefficient comb of exp(sum p_i eta^i / (2i)), _hafnian.py:183-209; returns comb[n/2] */
static C FN(f_plain)(C* AX, int m, int n, FN(ws_t) * w, C* pt, C* comb) {
  int h = n / 2;
  FN(powertrace)(AX, m, h + 1, pt, w);
  C* c0 = comb;
  C* c1 = comb + (h + 1);
  for (int i = 0; i <= h; ++i) c0[i] = c1[i] = FN(cmk)(0, 0);
  c0[0] = FN(cmk)(1, 0);
  int count = 0;
  for (int i = 1; i <= h; ++i) {
    C factor = FN(cscale)(pt[i], (R)1 / (R)(2 * i));
    C powfactor = FN(cmk)(1, 0);
    count = 1 - count;
    C* cur = count ? c1 : c0;
    C* prev = count ? c0 : c1;
    for (int q = 0; q <= h; ++q) cur[q] = prev[q];
    for (int j = 1; j <= n / (2 * i); ++j) {
      powfactor = FN(cmul)(powfactor, FN(cscale)(factor, (R)1 / (R)j));
      for (int k = i * j + 1; k <= h + 1; ++k)
        cur[k - 1] = FN(cadd)(cur[k - 1], FN(cmul)(prev[k - i * j - 1], powfactor));
    }
  }
  return (count ? c1 : c0)[h];
}

/* f_loop, _hafnian.py:212-242; returns comb[n/2] */
static C FN(f_loop)(C* AX, const C* AXS, const C* XD0, const C* DS, int m, int n, FN(ws_t) * w,
                    C* pt, C* comb, C* xd, C* xd2) {
  int h = n / 2;
  FN(powertrace)(AX, m, h + 1, pt, w);
  for (int i = 0; i < m; ++i) xd[i] = XD0[i];
  C* c0 = comb;
  C* c1 = comb + (h + 1);
  for (int i = 0; i <= h; ++i) c0[i] = c1[i] = FN(cmk)(0, 0);
  c0[0] = FN(cmk)(1, 0);
  int count = 0;
  for (int i = 1; i <= h; ++i) {
    C dot = FN(cmk)(0, 0);
    for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(xd[q], DS[q]));
    C factor = FN(cadd)(FN(cscale)(pt[i], (R)1 / (R)(2 * i)), FN(cscale)(dot, (R)1 / (R)2));
    for (int jj = 0; jj < m; ++jj) {
      C s = FN(cmk)(0, 0);
      for (int q = 0; q < m; ++q) s = FN(cadd)(s, FN(cmul)(xd[q], AXS[q * m + jj]));
      xd2[jj] = s;
    }
    for (int jj = 0; jj < m; ++jj) xd[jj] = xd2[jj];
    C powfactor = FN(cmk)(1, 0);
    count = 1 - count;
    C* cur = count ? c1 : c0;
    C* prev = count ? c0 : c1;
    for (int q = 0; q <= h; ++q) cur[q] = prev[q];
    for (int j = 1; j <= n / (2 * i); ++j) {
      powfactor = FN(cmul)(powfactor, FN(cscale)(factor, (R)1 / (R)j));
      for (int k = i * j + 1; k <= h + 1; ++k)
        cur[k - 1] = FN(cadd)(cur[k - 1], FN(cmul)(prev[k - i * j - 1], powfactor));
    }
  }
  return (count ? c1 : c0)[h];
}

/* f_loop_odd, _hafnian.py:245-285; returns comb[n] */
static C FN(f_loop_odd)(C* AX, const C* AXS, const C* XD, const C* D0, int m, int n, C oddloop,
                        const C* oddVX, FN(ws_t) * w, C* pt, C* comb, C* ds, C* ds2) {
  FN(powertrace)(AX, m, n / 2 + 1, pt, w);
  for (int i = 0; i < m; ++i) ds[i] = D0[i];
  C* c0 = comb;
  C* c1 = comb + (n + 1);
  for (int i = 0; i <= n; ++i) c0[i] = c1[i] = FN(cmk)(0, 0);
  c0[0] = FN(cmk)(1, 0);
  int count = 0;
  for (int i = 1; i <= n; ++i) {
    C factor;
    if (i == 1) {
      factor = oddloop;
    } else if (i % 2 == 0) {
      C dot = FN(cmk)(0, 0);
      for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(XD[q], ds[q]));
      factor = FN(cadd)(FN(cscale)(pt[i / 2], (R)1 / (R)i), FN(cscale)(dot, (R)1 / (R)2));
    } else {
      C dot = FN(cmk)(0, 0);
      for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(oddVX[q], ds[q]));
      factor = dot;
      for (int r = 0; r < m; ++r) {
        C s = FN(cmk)(0, 0);
        for (int q = 0; q < m; ++q) s = FN(cadd)(s, FN(cmul)(AXS[r * m + q], ds[q]));
        ds2[r] = s;
      }
      for (int r = 0; r < m; ++r) ds[r] = ds2[r];
    }
    C powfactor = FN(cmk)(1, 0);
    count = 1 - count;
    C* cur = count ? c1 : c0;
    C* prev = count ? c0 : c1;
    for (int q = 0; q <= n; ++q) cur[q] = prev[q];
    for (int j = 1; j <= n / i; ++j) {
      powfactor = FN(cmul)(powfactor, FN(cscale)(factor, (R)1 / (R)j));
      for (int k = i * j + 1; k <= n + 1; ++k)
        cur[k - 1] = FN(cadd)(cur[k - 1], FN(cmul)(prev[k - i * j - 1], powfactor));
    }
  }
  return (count ? c1 : c0)[n];
}

/* get_submatrices (_hafnian.py:315-356): rows/cols of nonzero delta, AX_S with columns scaled
 * by delta and halves swapped; XD_S, D_S, oddVX_S likewise.  Returns m. */
static int FN(submatrices)(const int64_t* delta, int E, const C* A, int n, const C* D, const C* oddV,
                           C* AXS, C* XDS, C* DS, C* oddVXS, int* rows, R* dnz) {
  int ne = 0;
  for (int i = 0; i < E; ++i)
    if (delta[i] != 0) { rows[ne] = i; dnz[ne] = (R)delta[i]; ++ne; }
  for (int i = 0; i < ne; ++i) rows[ne + i] = rows[i] + E;
  int m = 2 * ne;
  for (int a = 0; a < m; ++a)
    for (int c = 0; c < m; ++c) {
      int src = c < ne ? c + ne : c - ne;
      R s = dnz[c < ne ? c : c - ne];
      C x = A[rows[a] * n + rows[src]];
      AXS[a * m + c] = FN(cscale)(x, s);
    }
  if (D) {
    for (int a = 0; a < m; ++a) DS[a] = D[rows[a]];
    for (int a = 0; a < m; ++a) {
      int src = a < ne ? a + ne : a - ne;
      XDS[a] = FN(cscale)(DS[src], dnz[a < ne ? a : a - ne]);
    }
  }
  if (oddV) {
    for (int a = 0; a < m; ++a) {
      int src = a < ne ? a + ne : a - ne;
      oddVXS[a] = FN(cscale)(oddV[rows[src]], dnz[a < ne ? a : a - ne]);
    }
  }
  return m;
}

static int64_t FN(prod_radix)(const int64_t* reps, int E, int first_half) {
  int64_t steps = 1;
  for (int i = 0; i < E; ++i) {
    if (i == 0 && first_half) steps *= (reps[0] + 2) / 2;
    else steps *= reps[i] + 1;
  }
  return steps;
}

static void FN(load_c)(const double* src, C* dst, size_t cnt) {
  for (size_t i = 0; i < cnt; ++i) dst[i] = FN(cmk)((R)src[2 * i], (R)src[2 * i + 1]);
}

static void FN(store_dd)(C v, double* out) {
  double hr = (double)v.re, hi = (double)v.im;
  out[0] = hr;
  out[1] = hi;
  out[2] = (double)(v.re - (R)hr);
  out[3] = (double)(v.im - (R)hi);
}

/* The sum over sieve terms.  Each thread sums a contiguous range; the thread partials are then
 * added in thread order.  `kind`: 0 plain, 1 loop (even), 2 loop with odd self-loop. */
static C FN(sieve)(int kind, const C* A, const C* D, int n, const int64_t* reps, int E, C oddloop,
                   const C* oddV, int glynn, int nthreads, int64_t t_begin, int64_t t_end, int scale,
                   int absmode) {
  int N = 0;
  for (int i = 0; i < E; ++i) N += 2 * (int)reps[i];
  if (kind == 2) N += 1;
  int half_first = glynn && kind != 2;
  int64_t steps = FN(prod_radix)(reps, E, half_first);
  if (t_end < 0 || t_end > steps) t_end = steps;
  if (t_begin < 0) t_begin = 0;
  int64_t span = t_end > t_begin ? t_end - t_begin : 0;
  int64_t maxrep = 0;
  for (int i = 0; i < E; ++i) maxrep = reps[i] > maxrep ? reps[i] : maxrep;
  int mb = (int)maxrep + 1;
  R* binoms = FN(make_binoms)(mb);
  if (nthreads < 1) nthreads = 1;
  C* partial = (C*)calloc((size_t)nthreads, sizeof(C));
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0, nt = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nt = omp_get_num_threads();
#endif
    int64_t lo = t_begin + span * tid / nt, hi = t_begin + span * (tid + 1) / nt;
    int mm = n > 0 ? n : 1;
    FN(ws_t) w;
    FN(ws_init)(&w, mm);
    C* AXS = (C*)malloc(sizeof(C) * mm * mm);
    C* AXc = (C*)malloc(sizeof(C) * mm * mm);
    C *XDS = (C*)malloc(sizeof(C) * mm), *DS = (C*)malloc(sizeof(C) * mm), *OV = (C*)malloc(sizeof(C) * mm);
    C *v1 = (C*)malloc(sizeof(C) * mm), *v2 = (C*)malloc(sizeof(C) * mm);
    C* pt = (C*)malloc(sizeof(C) * (N + 4));
    C* comb = (C*)malloc(sizeof(C) * 2 * (N + 2));
    int* rows = (int*)malloc(sizeof(int) * mm);
    R* dnz = (R*)malloc(sizeof(R) * mm);
    int64_t* kept = (int64_t*)malloc(sizeof(int64_t) * (E > 0 ? E : 1));
    int64_t* delta = (int64_t*)malloc(sizeof(int64_t) * (E > 0 ? E : 1));
    C acc = FN(cmk)(0, 0);
    for (int64_t j = lo; j < hi; ++j) {
      FN(kept_edges)(j, reps, E, kept);
      int64_t esum = 0;
      R bprod = 1;
      for (int i = 0; i < E; ++i) {
        esum += kept[i];
        bprod *= binoms[reps[i] * (mb + 1) + kept[i]];
      }
      for (int i = 0; i < E; ++i) delta[i] = glynn ? 2 * kept[i] - reps[i] : kept[i];
      int m = FN(submatrices)(delta, E, A, n, D, kind == 2 ? oddV : NULL, AXS, XDS, DS, OV, rows, dnz);
      R prefac = ((N / 2 - esum) % 2 == 0) ? bprod : -bprod;
      C val;
      if (kind == 0) {
        if (glynn && delta[0] == 0) prefac *= (R)0.5;
        memcpy(AXc, AXS, sizeof(C) * m * m);
        val = FN(f_plain)(AXc, m, N, &w, pt, comb);
      } else if (kind == 1) {
        if (glynn && delta[0] == 0) prefac *= (R)0.5;
        memcpy(AXc, AXS, sizeof(C) * m * m);
        val = FN(f_loop)(AXc, AXS, XDS, DS, m, N, &w, pt, comb, v1, v2);
      } else {
        memcpy(AXc, AXS, sizeof(C) * m * m);
        val = FN(f_loop_odd)(AXc, AXS, XDS, DS, m, N, oddloop, OV, &w, pt, comb, v1, v2);
      }
      if (absmode) /* sum of |prefac * term|: the sum's condition number is that over |sum| */
        acc.re += FN(cabs_)(FN(cscale)(val, prefac));
      else
        acc = FN(cadd)(acc, FN(cscale)(val, prefac));
    }
    partial[tid] = acc;
    FN(ws_free)(&w);
    free(AXS); free(AXc); free(XDS); free(DS); free(OV); free(v1); free(v2); free(pt); free(comb);
    free(rows); free(dnz); free(kept); free(delta);
  }
  C H = FN(cmk)(0, 0);
  for (int t = 0; t < nthreads; ++t) H = FN(cadd)(H, partial[t]);
  free(partial);
  free(binoms);
  if (glynn && scale) {
    int e = (kind == 2) ? N / 2 : N / 2 - 1;
    R s = 1;
    for (int i = 0; i < e; ++i) s *= (R)0.5;
    H = FN(cscale)(H, s);
  }
  return H;
}

/* ---- exported entry points: complex inputs as interleaved doubles (re, im), outputs as
 * {re_hi, im_hi, re_lo, im_lo} so the extended builds can hand back their extra bits. ---- */

int FN(oracle_calc_hafnian)(const double* A, int n, const int64_t* edge_reps, int E, int glynn,
                            int nthreads, double* out) {
  C* Ac = (C*)malloc(sizeof(C) * (n > 0 ? n * n : 1));
  FN(load_c)(A, Ac, (size_t)n * n);
  C h = FN(sieve)(0, Ac, NULL, n, edge_reps, E, FN(cmk)(0, 0), NULL, glynn, nthreads, 0, -1, 1, 0);
  FN(store_dd)(h, out);
  free(Ac);
  return 0;
}

/* Unscaled partial sum of the plain sieve over terms [t_begin, t_end) (bounded CPU samples). */
int FN(oracle_hafnian_term_range)(const double* A, int n, const int64_t* edge_reps, int E, int glynn,
                                  int nthreads, int64_t t_begin, int64_t t_end, double* out) {
  C* Ac = (C*)malloc(sizeof(C) * (n > 0 ? n * n : 1));
  FN(load_c)(A, Ac, (size_t)n * n);
  C h = FN(sieve)(0, Ac, NULL, n, edge_reps, E, FN(cmk)(0, 0), NULL, glynn, nthreads, t_begin, t_end, 0, 0);
  FN(store_dd)(h, out);
  free(Ac);
  return 0;
}

int FN(oracle_calc_loop_hafnian)(const double* A, const double* D, int n, const int64_t* edge_reps,
                                 int E, int has_odd, const double* oddloop, const double* oddV,
                                 int glynn, int nthreads, double* out) {
  C* Ac = (C*)malloc(sizeof(C) * (n > 0 ? n * n : 1));
  C* Dc = (C*)malloc(sizeof(C) * (n > 0 ? n : 1));
  C* Vc = (C*)malloc(sizeof(C) * (n > 0 ? n : 1));
  FN(load_c)(A, Ac, (size_t)n * n);
  FN(load_c)(D, Dc, (size_t)n);
  C ol = FN(cmk)(0, 0);
  if (has_odd) {
    FN(load_c)(oddV, Vc, (size_t)n);
    ol = FN(cmk)((R)oddloop[0], (R)oddloop[1]);
  }
  C h = FN(sieve)(has_odd ? 2 : 1, Ac, Dc, n, edge_reps, E, ol, has_odd ? Vc : NULL, glynn, nthreads, 0, -1, 1, 0);
  FN(store_dd)(h, out);
  free(Ac); free(Dc); free(Vc);
  return 0;
}

/* Partial sums over sieve terms [t_begin, t_end) (mixed-radix order) of the plain or loop sieve,
 * unscaled, for checks and conditioning: kind 0 plain, 1 loop, 2 loop with an odd self-loop;
 * absmode 1 returns the sum of the terms' absolute values in the real part instead. */
int FN(oracle_sieve_term_range)(int kind, const double* A, const double* D, int n, const int64_t* edge_reps,
                                int E, const double* oddloop, const double* oddV, int glynn, int nthreads,
                                int64_t t_begin, int64_t t_end, int absmode, double* out) {
  C* Ac = (C*)malloc(sizeof(C) * (n > 0 ? n * n : 1));
  C* Dc = (C*)malloc(sizeof(C) * (n > 0 ? n : 1));
  C* Vc = (C*)malloc(sizeof(C) * (n > 0 ? n : 1));
  FN(load_c)(A, Ac, (size_t)n * n);
  if (kind > 0) FN(load_c)(D, Dc, (size_t)n);
  C ol = FN(cmk)(0, 0);
  if (kind == 2) {
    FN(load_c)(oddV, Vc, (size_t)n);
    ol = FN(cmk)((R)oddloop[0], (R)oddloop[1]);
  }
  C h = FN(sieve)(kind, Ac, kind > 0 ? Dc : NULL, n, edge_reps, E, ol, kind == 2 ? Vc : NULL, glynn, nthreads,
                  t_begin, t_end, 0, absmode);
  FN(store_dd)(h, out);
  free(Ac); free(Dc); free(Vc);
  return 0;
}

/* loop_hafnian_batch.py:50-208.  odd == 0: _calc_loop_hafnian_batch_even(A, D, fixed, batch_max,
 * odd_cutoff); odd == 1: _calc_loop_hafnian_batch_odd(A, D, fixed, batch_max, even_cutoff).
 * out receives len = 2*batch_max+cutoff+1 (+1 when odd) entries of 4 doubles each. */
int FN(oracle_calc_loop_hafnian_batch)(const double* A, const double* D, int n, const int64_t* fixed,
                                       int Ef, int batch_max, int cutoff, int odd, int glynn,
                                       int nthreads, double* out) {
  C* Ac = (C*)malloc(sizeof(C) * n * n);
  C* Dc = (C*)malloc(sizeof(C) * n);
  FN(load_c)(A, Ac, (size_t)n * n);
  FN(load_c)(D, Dc, (size_t)n);
  C oddloop = Dc[0];
  const C* oddV = Ac; /* row 0 */
  C oddloop0 = odd ? Dc[1] : FN(cmk)(0, 0);
  const C* oddV0 = odd ? Ac + n : NULL;
  int nb = odd ? 2 : 1;
  int E = Ef + nb;
  int64_t* reps = (int64_t*)malloc(sizeof(int64_t) * E);
  reps[0] = batch_max;
  if (odd) reps[1] = 1;
  for (int i = 0; i < Ef; ++i) reps[nb + i] = fixed[i];
  int Nf = 0;
  for (int i = 0; i < Ef; ++i) Nf += 2 * (int)fixed[i];
  if (odd) Nf += 1;
  int Nmax = odd ? Nf + 2 * batch_max + cutoff + 1 : Nf + 2 * batch_max + cutoff;
  int len = odd ? 2 * batch_max + cutoff + 2 : 2 * batch_max + cutoff + 1;
  int64_t steps = FN(prod_radix)(reps, E, 0);
  int64_t maxrep = 0;
  for (int i = 0; i < E; ++i) maxrep = reps[i] > maxrep ? reps[i] : maxrep;
  int mb = (int)maxrep + cutoff;
  R* binoms = FN(make_binoms)(mb);
  if (nthreads < 1) nthreads = 1;
  C* partial = (C*)calloc((size_t)nthreads * len, sizeof(C));
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0, nt = 1;
#ifdef _OPENMP
    tid = omp_get_thread_num();
    nt = omp_get_num_threads();
#endif
    int64_t lo = steps * tid / nt, hi = steps * (tid + 1) / nt;
    int mm = n;
    FN(ws_t) w;
    FN(ws_init)(&w, mm);
    C* AXS = (C*)malloc(sizeof(C) * mm * mm);
    C* AXc = (C*)malloc(sizeof(C) * mm * mm);
    C *XDS = (C*)malloc(sizeof(C) * mm), *DS = (C*)malloc(sizeof(C) * mm), *OV = (C*)malloc(sizeof(C) * mm);
    C *OV0 = (C*)malloc(sizeof(C) * mm);
    C *v1 = (C*)malloc(sizeof(C) * mm), *v2 = (C*)malloc(sizeof(C) * mm);
    C* pt = (C*)malloc(sizeof(C) * (Nmax + 4));
    C* comb = (C*)malloc(sizeof(C) * 2 * (Nmax + 2));
    int* rows = (int*)malloc(sizeof(int) * mm);
    R* dnz = (R*)malloc(sizeof(R) * mm);
    int64_t* kept = (int64_t*)malloc(sizeof(int64_t) * E);
    int64_t* delta = (int64_t*)malloc(sizeof(int64_t) * E);
    C* acc = partial + (size_t)tid * len;
    for (int64_t j = lo; j < hi; ++j) {
      FN(kept_edges)(j, reps, E, kept);
      int64_t esum = 0;
      for (int i = 0; i < E; ++i) esum += kept[i];
      R bprod = 1;
      for (int i = nb; i < E; ++i) bprod *= binoms[reps[i] * (mb + 1) + kept[i]];
      for (int i = 0; i < E; ++i) delta[i] = glynn ? 2 * kept[i] - reps[i] : kept[i];
      int m = FN(submatrices)(delta, E, Ac, n, Dc, oddV, AXS, XDS, DS, OV, rows, dnz);
      memcpy(AXc, AXS, sizeof(C) * m * m);
      if (odd && kept[0] == 0 && kept[1] == 0) {
        /* get_submatrix_batch_odd0 */
        int ne = m / 2;
        for (int a = 0; a < m; ++a) {
          int src = a < ne ? a + ne : a - ne;
          OV0[a] = FN(cscale)(oddV0[rows[src]], dnz[a < ne ? a : a - ne]);
        }
        R pm = ((Nf / 2 - esum) % 2 == 0) ? 1 : -1;
        C f0 = FN(f_loop_odd)(AXc, AXS, XDS, DS, m, Nf, oddloop0, OV0, &w, pt, comb, v1, v2);
        acc[0] = FN(cadd)(acc[0], FN(cscale)(f0, bprod * pm));
      }
      /* f_even = f_loop(..., N_max) full comb; f_odd = f_loop_odd(..., N_max) full comb */
      /* the reference keeps the whole comb arrays; recompute them here into two buffers */
      int h = Nmax / 2;
      C* feven = (C*)malloc(sizeof(C) * (h + 1));
      C* fodd = (C*)malloc(sizeof(C) * (Nmax + 1));
      {
        /* f_loop at Nmax, keep comb */
        FN(powertrace)(AXc, m, h + 1, pt, &w);
        for (int i = 0; i < m; ++i) v1[i] = XDS[i];
        C* c0 = comb;
        C* c1 = comb + (h + 1);
        for (int i = 0; i <= h; ++i) c0[i] = c1[i] = FN(cmk)(0, 0);
        c0[0] = FN(cmk)(1, 0);
        int count = 0;
        for (int i = 1; i <= h; ++i) {
          C dot = FN(cmk)(0, 0);
          for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(v1[q], DS[q]));
          C factor = FN(cadd)(FN(cscale)(pt[i], (R)1 / (R)(2 * i)), FN(cscale)(dot, (R)1 / (R)2));
          for (int jj = 0; jj < m; ++jj) {
            C s = FN(cmk)(0, 0);
            for (int q = 0; q < m; ++q) s = FN(cadd)(s, FN(cmul)(v1[q], AXS[q * m + jj]));
            v2[jj] = s;
          }
          for (int jj = 0; jj < m; ++jj) v1[jj] = v2[jj];
          C powfactor = FN(cmk)(1, 0);
          count = 1 - count;
          C* cur = count ? c1 : c0;
          C* prev = count ? c0 : c1;
          for (int q = 0; q <= h; ++q) cur[q] = prev[q];
          for (int jq = 1; jq <= Nmax / (2 * i); ++jq) {
            powfactor = FN(cmul)(powfactor, FN(cscale)(factor, (R)1 / (R)jq));
            for (int k = i * jq + 1; k <= h + 1; ++k)
              cur[k - 1] = FN(cadd)(cur[k - 1], FN(cmul)(prev[k - i * jq - 1], powfactor));
          }
        }
        for (int q = 0; q <= h; ++q) feven[q] = (count ? c1 : c0)[q];
      }
      {
        /* f_loop_odd at Nmax on the (possibly Hessenberg-reduced) AXc, keep comb */
        int nn = Nmax;
        FN(powertrace)(AXc, m, nn / 2 + 1, pt, &w);
        for (int i = 0; i < m; ++i) v1[i] = DS[i];
        C* c0 = comb;
        C* c1 = comb + (nn + 1);
        for (int i = 0; i <= nn; ++i) c0[i] = c1[i] = FN(cmk)(0, 0);
        c0[0] = FN(cmk)(1, 0);
        int count = 0;
        for (int i = 1; i <= nn; ++i) {
          C factor;
          if (i == 1) {
            factor = oddloop;
          } else if (i % 2 == 0) {
            C dot = FN(cmk)(0, 0);
            for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(XDS[q], v1[q]));
            factor = FN(cadd)(FN(cscale)(pt[i / 2], (R)1 / (R)i), FN(cscale)(dot, (R)1 / (R)2));
          } else {
            C dot = FN(cmk)(0, 0);
            for (int q = 0; q < m; ++q) dot = FN(cadd)(dot, FN(cmul)(OV[q], v1[q]));
            factor = dot;
            for (int r = 0; r < m; ++r) {
              C s = FN(cmk)(0, 0);
              for (int q = 0; q < m; ++q) s = FN(cadd)(s, FN(cmul)(AXS[r * m + q], v1[q]));
              v2[r] = s;
            }
            for (int r = 0; r < m; ++r) v1[r] = v2[r];
          }
          C powfactor = FN(cmk)(1, 0);
          count = 1 - count;
          C* cur = count ? c1 : c0;
          C* prev = count ? c0 : c1;
          for (int q = 0; q <= nn; ++q) cur[q] = prev[q];
          for (int jq = 1; jq <= nn / i; ++jq) {
            powfactor = FN(cmul)(powfactor, FN(cscale)(factor, (R)1 / (R)jq));
            for (int k = i * jq + 1; k <= nn + 1; ++k)
              cur[k - 1] = FN(cadd)(cur[k - 1], FN(cmul)(prev[k - i * jq - 1], powfactor));
          }
        }
        for (int q = 0; q <= nn; ++q) fodd[q] = (count ? c1 : c0)[q];
      }
      if (!odd) {
        for (int Nd = 2 * (int)kept[0]; Nd < len; ++Nd) {
          int Nn = Nf + Nd;
          R pm = ((Nn / 2 - esum) % 2 == 0) ? 1 : -1;
          R bb = binoms[(Nd / 2) * (mb + 1) + kept[0]] * bprod;
          C f = (Nd % 2 == 0) ? feven[Nn / 2] : fodd[Nn];
          acc[Nd] = FN(cadd)(acc[Nd], FN(cscale)(f, bb * pm));
        }
      } else {
        for (int Nd = 2 * (int)kept[0] + 1; Nd < len; ++Nd) {
          int Nn = Nf + Nd;
          R pm = ((Nn / 2 - esum) % 2 == 0) ? 1 : -1;
          R bb = binoms[((Nd - 1) / 2) * (mb + 1) + kept[0]] * bprod;
          C f = (Nn % 2 == 0) ? feven[Nn / 2] : fodd[Nn];
          acc[Nd] = FN(cadd)(acc[Nd], FN(cscale)(f, bb * pm));
        }
      }
      free(feven);
      free(fodd);
    }
    FN(ws_free)(&w);
    free(AXS); free(AXc); free(XDS); free(DS); free(OV); free(OV0); free(v1); free(v2); free(pt);
    free(comb); free(rows); free(dnz); free(kept); free(delta);
  }
  for (int q = 0; q < len; ++q) {
    C s = FN(cmk)(0, 0);
    for (int t = 0; t < nthreads; ++t) s = FN(cadd)(s, partial[(size_t)t * len + q]);
    if (glynn) {
      int x = Nf + q;
      R sc = 1;
      for (int i = 0; i < x / 2; ++i) sc *= (R)0.5;
      s = FN(cscale)(s, sc);
    }
    FN(store_dd)(s, out + 4 * q);
  }
  free(partial); free(reps); free(binoms); free(Ac); free(Dc);
  return 0;
}

/* charpoly.powertrace on its own (charpoly.py:301-327), for the La Budde known-answer tests */
int FN(oracle_powertrace)(const double* H, int m, int n, double* out) {
  C* Hc = (C*)malloc(sizeof(C) * (m > 0 ? m * m : 1));
  FN(load_c)(H, Hc, (size_t)m * m);
  FN(ws_t) w;
  FN(ws_init)(&w, m > 0 ? m : 1);
  C* pt = (C*)malloc(sizeof(C) * (n + 4));
  FN(powertrace)(Hc, m, n, pt, &w);
  for (int i = 0; i < n; ++i) FN(store_dd)(pt[i], out + 4 * i);
  free(pt); free(Hc);
  FN(ws_free)(&w);
  return 0;
}

/* charpoly.charpoly (charpoly.py:285-298): Householder Hessenberg then La Budde */
int FN(oracle_charpoly)(const double* H, int m, double* out) {
  C* Hc = (C*)malloc(sizeof(C) * m * m);
  FN(load_c)(H, Hc, (size_t)m * m);
  FN(ws_t) w;
  FN(ws_init)(&w, m);
  FN(hessenberg)(Hc, m, w.v, w.tmp);
  FN(labudde)(Hc, m, w.cpc, w.poly);
  for (int i = 0; i < m; ++i) FN(store_dd)(w.poly[i], out + 4 * i);
  free(Hc);
  FN(ws_free)(&w);
  return 0;
}
