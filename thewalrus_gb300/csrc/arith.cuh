// Scalar arithmetic for the sieve kernels.
//
// Seven scalar types share one interface (struct Ar<S>):
//   double  real FP64                 c64  complex FP64
//   dfr     real double-float (FP32)  cdf  complex double-float
//   ddr     real double-double (FP64) cdd  complex double-double
//   modp<P> residues modulo a 31-bit prime P in Montgomery form (exact integer sieves)
// A double-float value is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), giving
// a 48-bit significand from FP32 instructions only.  Products use the FMA error-free
// transformation (err = fma(a, b, -a*b)); sums use Knuth's two-sum.  Conversions to and from
// FP64 are exact for the hi part and round the lo part once.  A double-double value is the same
// construction one precision up (two doubles, a 106-bit significand from FP64 instructions), for
// sums whose terms cancel by more than FP64 can resolve.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wg {

// The double-float scalars are aligned to their size, so that one moves in a single 128-bit
// (64-bit for dfr) shared or global access (every tile, pool and series array is 16-byte
// aligned): that took df n = 40 from 173 ms to 142 ms.  The same for c64 measured 1-3 % slower,
// so it keeps the 8-byte alignment of its doubles.
struct c64 {
  double re, im;
};
struct alignas(8) dfr {
  float hi, lo;
};
struct alignas(16) cdf {
  dfr re, im;
};

__device__ __forceinline__ double neg_d(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ float neg_f(float x) { return __int_as_float(__float_as_int(x) ^ 0x80000000); }
__device__ __forceinline__ unsigned long long absbits_d(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned int absbits_f(float x) { return (unsigned)__float_as_int(x) & 0x7fffffffu; }

// Deflation threshold of a pivot column for the double-float keys (FP32 high parts): k * 2^-40,
// 0 when that leaves the normal range.  Subdiagonal candidates at or below it are rounding
// residues of an exact cancellation (terms whose matrix repeats a row, such as the two ends of
// the batch edge) and are treated as zero.  The FP64 and double-double types, whose elimination
// is normalised, compare in the classic frame instead (hessenberg_elim), at 2^-DEFLATE_BITS.
__device__ __forceinline__ unsigned long long key_shift_f(unsigned long long k) {
  constexpr unsigned long long sh = 40ull << 23;
  return k > sh ? k - sh : 0ull;
}

// 1/x for the pivots: the PTX approximate reciprocal (rcp.approx.ftz.f64) refined by one step of
// the third-order (Chebyshev / Householder) iteration r <- r (1 + e + e^2), e = 1 - x r, which
// cubes the relative error (three FMAs where two Newton steps, squaring it twice, take four);
// inputs whose exponent leaves the approximation's safe range take the IEEE division instead.
__device__ __forceinline__ double recip_newton(double x) {
  const unsigned hi = (unsigned)(__double_as_longlong(x) >> 32);
  const unsigned ex = (hi >> 20) & 0x7ffu;
  if (ex < 64u || ex > 2000u) return 1.0 / x;
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double e = ::fma(-x, r, 1.0);
  return ::fma(r, ::fma(e, e, e), r);
}

// ---------------------------------------------------------------- double-float primitives
__device__ __forceinline__ dfr df_two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ dfr df_fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return {s, e};
}
__device__ __forceinline__ dfr df_add(dfr a, dfr b) {
  dfr s = df_two_sum(a.hi, b.hi);
  float lo = s.lo + (a.lo + b.lo);
  return df_fast_two_sum(s.hi, lo);
}
__device__ __forceinline__ dfr df_neg(dfr a) { return {neg_f(a.hi), neg_f(a.lo)}; }
__device__ __forceinline__ dfr df_mul(dfr a, dfr b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// c + a*b with one renormalisation
__device__ __forceinline__ dfr df_fma(dfr a, dfr b, dfr c) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  dfr s = df_two_sum(c.hi, p);
  float lo = s.lo + (c.lo + e);
  return df_fast_two_sum(s.hi, lo);
}
// c + a*b + d*f  (two products accumulated before one renormalisation)
__device__ __forceinline__ dfr df_fma2(dfr a, dfr b, dfr d, dfr f, dfr c) {
  float p1 = a.hi * b.hi;
  float e1 = fmaf(a.hi, b.hi, -p1);
  e1 = fmaf(a.hi, b.lo, e1);
  e1 = fmaf(a.lo, b.hi, e1);
  float p2 = d.hi * f.hi;
  float e2 = fmaf(d.hi, f.hi, -p2);
  e2 = fmaf(d.hi, f.lo, e2);
  e2 = fmaf(d.lo, f.hi, e2);
  dfr s1 = df_two_sum(c.hi, p1);
  dfr s2 = df_two_sum(s1.hi, p2);
  float lo = (s1.lo + s2.lo) + (c.lo + (e1 + e2));
  return df_fast_two_sum(s2.hi, lo);
}
// a * s for a float s that is exact (the small integers and halves of the series and the gather)
__device__ __forceinline__ dfr df_mul_f(dfr a, float s) {
  float p = a.hi * s;
  float e = fmaf(a.hi, s, -p);
  e = fmaf(a.lo, s, e);
  return df_fast_two_sum(p, e);
}
// a / k for a small positive integer k: the correctly rounded float quotient q1, whose remainder
// a.hi - q1 k is exact in one FMA (a multiple of ulp(q1) of a few bits), and the quotient of
// the remainder plus a.lo as the low part (|q2| <= ulp(q1), so its rounding is ~2^-48 of a / k)
__device__ __forceinline__ dfr df_div_int(dfr a, int k) {
  const float kf = (float)k;
  const float q1 = __fdiv_rn(a.hi, kf);
  const float r = fmaf(neg_f(q1), kf, a.hi) + a.lo;
  return df_fast_two_sum(q1, __fdiv_rn(r, kf));
}
// 2^-e for a float whose magnitude bits are `bits` and |x| in [2^e, 2^(e+1)), e clamped to the
// normal range: multiplying by it is exact and brings |x| into [1, 2)
__device__ __forceinline__ float df_pow2_inv(unsigned bits) {
  int ef = 254 - (int)(bits >> 23);
  ef = ef < 1 ? 1 : (ef > 254 ? 254 : ef);
  return __int_as_float(ef << 23);
}
// 1/a for |a.hi| in [1, 8), FP32 instructions only: the correctly rounded float reciprocal r0
// and 1/a = r0 (1 + e + e^2 + ..) with e = 1 - a r0 = e0 - a.lo r0 (e0 = 1 - a.hi r0 exact in
// one FMA, the second product split exactly by another), kept as a double-float so that the
// correction r0 e is formed to ~2^-49; |e| <= 2^-23, so e^2 is the last term that counts.
// Relative error ~2^-49, as good as rounding the FP64 reciprocal: the pivot reciprocal's error
// is the same for every multiplier of a column, so it is kept well below the other roundings.
__device__ __forceinline__ dfr df_recip_unit(dfr a) {
  const float r0 = __frcp_rn(a.hi);
  const float e0 = fmaf(neg_f(a.hi), r0, 1.0f);
  const float e1 = neg_f(a.lo) * r0;
  const float e1l = fmaf(neg_f(a.lo), r0, neg_f(e1));
  dfr e = df_two_sum(e0, e1);
  e.lo += e1l;
  const float ch = r0 * e.hi;
  const float cl = fmaf(r0, e.hi, neg_f(ch)) + r0 * fmaf(e.hi, e.hi, e.lo);
  const dfr s = df_fast_two_sum(r0, ch);
  return df_fast_two_sum(s.hi, s.lo + cl);
}
// 1/a: scaled by a power of two into [1, 2), inverted, scaled back (exact unless the result
// leaves float's normal range)
__device__ __forceinline__ dfr df_recip(dfr a) {
  const float f = df_pow2_inv(absbits_f(a.hi));
  const dfr r = df_recip_unit({a.hi * f, a.lo * f});
  return {r.hi * f, r.lo * f};
}
__device__ __forceinline__ double df_to_d(dfr a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfr df_from_d(double x) {
  float h = __double2float_rn(x);
  float l = __double2float_rn(x - (double)h);
  return {h, l};
}

// ---------------------------------------------------------------- double-double primitives
// The error-free transformations of the double-float type (Knuth's two-sum, Dekker's fast
// two-sum for |a| >= |b|, the FMA two-product) on doubles.
struct alignas(16) ddr {
  double hi, lo;
};
struct cdd {
  ddr re, im;
};
__device__ __forceinline__ ddr dd_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ ddr dd_fast_two_sum(double a, double b) {
  double s = a + b;
  double e = b - (s - a);
  return {s, e};
}
__device__ __forceinline__ ddr dd_add(ddr a, ddr b) {
  ddr s = dd_two_sum(a.hi, b.hi);
  double lo = s.lo + (a.lo + b.lo);
  return dd_fast_two_sum(s.hi, lo);
}
__device__ __forceinline__ ddr dd_neg(ddr a) { return {neg_d(a.hi), neg_d(a.lo)}; }
__device__ __forceinline__ ddr dd_mul(ddr a, ddr b) {
  double p = a.hi * b.hi;
  double e = ::fma(a.hi, b.hi, -p);
  e = ::fma(a.hi, b.lo, e);
  e = ::fma(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ ddr dd_mul_d(ddr a, double s) {
  double p = a.hi * s;
  double e = ::fma(a.hi, s, -p);
  e = ::fma(a.lo, s, e);
  return dd_fast_two_sum(p, e);
}
// c + a*b with one renormalisation
__device__ __forceinline__ ddr dd_fma(ddr a, ddr b, ddr c) {
  double p = a.hi * b.hi;
  double e = ::fma(a.hi, b.hi, -p);
  e = ::fma(a.hi, b.lo, e);
  e = ::fma(a.lo, b.hi, e);
  ddr s = dd_two_sum(c.hi, p);
  double lo = s.lo + (c.lo + e);
  return dd_fast_two_sum(s.hi, lo);
}
// c + a*b + d*f  (two products accumulated before one renormalisation)
__device__ __forceinline__ ddr dd_fma2(ddr a, ddr b, ddr d, ddr f, ddr c) {
  double p1 = a.hi * b.hi;
  double e1 = ::fma(a.hi, b.hi, -p1);
  e1 = ::fma(a.hi, b.lo, e1);
  e1 = ::fma(a.lo, b.hi, e1);
  double p2 = d.hi * f.hi;
  double e2 = ::fma(d.hi, f.hi, -p2);
  e2 = ::fma(d.hi, f.lo, e2);
  e2 = ::fma(d.lo, f.hi, e2);
  ddr s1 = dd_two_sum(c.hi, p1);
  ddr s2 = dd_two_sum(s1.hi, p2);
  double lo = (s1.lo + s2.lo) + (c.lo + (e1 + e2));
  return dd_fast_two_sum(s2.hi, lo);
}
// 1/a: the FP64 reciprocal of the high part, then one Newton step r + r (1 - a r) with the
// residual 1 - a r formed exactly enough (1 - hi(a r) is exact near 1) -- relative error ~2^-104
__device__ __forceinline__ ddr dd_recip(ddr a) {
  const double r = recip_newton(a.hi);
  const ddr t = dd_mul_d(a, r);
  const double e = (1.0 - t.hi) - t.lo;
  return dd_fast_two_sum(r, r * e);
}
// a / k for a small positive integer k: a times the double-double reciprocal of k
__device__ __forceinline__ ddr dd_div_int(ddr a, int k) {
  const double r = 1.0 / (double)k;
  const ddr rk = {r, ::fma(-(double)k, r, 1.0) * r};
  return dd_mul(a, rk);
}
// ---------------------------------------------------------------- traits
template <class S>
struct Ar;

template <>
struct Ar<double> {
  using S = double;
  using Comp = double;  // reducible component type
  static constexpr int NC = 1;
  static constexpr bool cplx = false;
  static constexpr bool fp64 = true;
  static constexpr bool modular = false;
  static constexpr bool dd = false;
  static constexpr int DEFLATE_BITS = 44;  // deflation threshold 2^-44 (normalised elimination)
  __device__ static __forceinline__ S zero() { return 0.0; }
  __device__ static __forceinline__ S one() { return 1.0; }
  __device__ static __forceinline__ S add(S a, S b) { return a + b; }
  __device__ static __forceinline__ S sub(S a, S b) { return a - b; }
  __device__ static __forceinline__ S mul(S a, S b) { return a * b; }
  __device__ static __forceinline__ S fma(S a, S b, S c) { return ::fma(a, b, c); }
  __device__ static __forceinline__ S fnma(S a, S b, S c) { return ::fma(neg_d(a), b, c); }
  __device__ static __forceinline__ S neg(S a) { return neg_d(a); }
  __device__ static __forceinline__ S conj(S a) { return a; }
  __device__ static __forceinline__ S scale(S a, double s) { return a * s; }
  __device__ static __forceinline__ S scale_f(S a, float s) { return a * (double)s; }
  __device__ static __forceinline__ S from_c64(c64 v) { return v.re; }
  __device__ static __forceinline__ c64 to_c64(S a) { return {a, 0.0}; }
  __device__ static __forceinline__ unsigned long long key(S a) { return absbits_d(a); }
  // 32-bit pivot key: sign-free exponent and the top 20 mantissa bits
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)(k >> 32); }
  __device__ static __forceinline__ bool is_zero(S a) { return absbits_d(a) == 0; }
  __device__ static __forceinline__ S recip(S a) { return recip_newton(a); }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return a; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) { a = v; }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return a + b; }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  __device__ static __forceinline__ S shfl(S v, int src) { return __shfl_sync(0xffffffffu, v, src); }
};

template <>
struct Ar<c64> {
  using S = c64;
  using Comp = double;
  static constexpr int NC = 2;
  static constexpr bool cplx = true;
  static constexpr bool fp64 = true;
  static constexpr bool modular = false;
  static constexpr bool dd = false;
  static constexpr int DEFLATE_BITS = 44;
  __device__ static __forceinline__ S zero() { return {0.0, 0.0}; }
  __device__ static __forceinline__ S one() { return {1.0, 0.0}; }
  __device__ static __forceinline__ S add(S a, S b) { return {a.re + b.re, a.im + b.im}; }
  __device__ static __forceinline__ S sub(S a, S b) { return {a.re - b.re, a.im - b.im}; }
  __device__ static __forceinline__ S mul(S a, S b) {
    return {::fma(a.re, b.re, neg_d(a.im * b.im)), ::fma(a.re, b.im, a.im * b.re)};
  }
  // c + a*b : 4 DFMA
  __device__ static __forceinline__ S fma(S a, S b, S c) {
    return {::fma(a.re, b.re, ::fma(neg_d(a.im), b.im, c.re)), ::fma(a.re, b.im, ::fma(a.im, b.re, c.im))};
  }
  // c - a*b : 4 DFMA
  __device__ static __forceinline__ S fnma(S a, S b, S c) {
    return {::fma(neg_d(a.re), b.re, ::fma(a.im, b.im, c.re)), ::fma(neg_d(a.re), b.im, ::fma(neg_d(a.im), b.re, c.im))};
  }
  __device__ static __forceinline__ S neg(S a) { return {neg_d(a.re), neg_d(a.im)}; }
  __device__ static __forceinline__ S conj(S a) { return {a.re, neg_d(a.im)}; }
  __device__ static __forceinline__ S scale(S a, double s) { return {a.re * s, a.im * s}; }
  __device__ static __forceinline__ S scale_f(S a, float s) { return scale(a, (double)s); }
  __device__ static __forceinline__ S from_c64(c64 v) { return v; }
  __device__ static __forceinline__ c64 to_c64(S a) { return a; }
  __device__ static __forceinline__ unsigned long long key(S a) {
    const unsigned long long x = absbits_d(a.re), y = absbits_d(a.im);
    return x > y ? x : y;
  }
  // 32-bit pivot key: sign-free exponent and the top 20 mantissa bits
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)(k >> 32); }
  __device__ static __forceinline__ bool is_zero(S a) { return (absbits_d(a.re) | absbits_d(a.im)) == 0; }
  __device__ static __forceinline__ S recip(S a) {
    const double d = recip_newton(::fma(a.re, a.re, a.im * a.im));
    return {a.re * d, neg_d(a.im) * d};
  }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return i ? a.im : a.re; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) {
    if (i) a.im = v; else a.re = v;
  }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return a + b; }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  __device__ static __forceinline__ S shfl(S v, int src) {
    return {__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
  }
};

template <>
struct Ar<dfr> {
  using S = dfr;
  using Comp = dfr;
  static constexpr int NC = 1;
  static constexpr bool cplx = false;
  static constexpr bool fp64 = false;
  static constexpr bool modular = false;
  static constexpr bool dd = false;
  __device__ static __forceinline__ S zero() { return {0.f, 0.f}; }
  __device__ static __forceinline__ S one() { return {1.f, 0.f}; }
  __device__ static __forceinline__ S add(S a, S b) { return df_add(a, b); }
  __device__ static __forceinline__ S sub(S a, S b) { return df_add(a, df_neg(b)); }
  __device__ static __forceinline__ S mul(S a, S b) { return df_mul(a, b); }
  __device__ static __forceinline__ S fma(S a, S b, S c) { return df_fma(a, b, c); }
  __device__ static __forceinline__ S fnma(S a, S b, S c) { return df_fma(df_neg(a), b, c); }
  __device__ static __forceinline__ S neg(S a) { return df_neg(a); }
  __device__ static __forceinline__ S conj(S a) { return a; }
  __device__ static __forceinline__ S scale(S a, double s) { return df_mul(a, df_from_d(s)); }
  __device__ static __forceinline__ S scale_f(S a, float s) { return df_mul_f(a, s); }
  __device__ static __forceinline__ S div_int(S a, int k) { return df_div_int(a, k); }
  __device__ static __forceinline__ S from_c64(c64 v) { return df_from_d(v.re); }
  __device__ static __forceinline__ c64 to_c64(S a) { return {df_to_d(a), 0.0}; }
  __device__ static __forceinline__ unsigned long long key(S a) { return absbits_f(a.hi); }
  __device__ static __forceinline__ unsigned long long key_deflate(unsigned long long k) { return key_shift_f(k); }
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)k; }
  __device__ static __forceinline__ bool is_zero(S a) { return absbits_f(a.hi) == 0; }
  __device__ static __forceinline__ S recip(S a) { return df_recip(a); }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return a; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) { a = v; }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return df_add(a, b); }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
  }
  __device__ static __forceinline__ S shfl(S v, int src) {
    return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
  }
};

template <>
struct Ar<cdf> {
  using S = cdf;
  using Comp = dfr;
  static constexpr int NC = 2;
  static constexpr bool cplx = true;
  static constexpr bool fp64 = false;
  static constexpr bool modular = false;
  static constexpr bool dd = false;
  __device__ static __forceinline__ S zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
  __device__ static __forceinline__ S one() { return {{1.f, 0.f}, {0.f, 0.f}}; }
  __device__ static __forceinline__ S add(S a, S b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
  __device__ static __forceinline__ S sub(S a, S b) { return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))}; }
  __device__ static __forceinline__ S mul(S a, S b) {
    dfr z = {0.f, 0.f};
    return {df_fma2(a.re, b.re, df_neg(a.im), b.im, z), df_fma2(a.re, b.im, a.im, b.re, z)};
  }
  __device__ static __forceinline__ S fma(S a, S b, S c) {
    return {df_fma2(a.re, b.re, df_neg(a.im), b.im, c.re), df_fma2(a.re, b.im, a.im, b.re, c.im)};
  }
  __device__ static __forceinline__ S fnma(S a, S b, S c) {
    return {df_fma2(df_neg(a.re), b.re, a.im, b.im, c.re), df_fma2(df_neg(a.re), b.im, df_neg(a.im), b.re, c.im)};
  }
  __device__ static __forceinline__ S neg(S a) { return {df_neg(a.re), df_neg(a.im)}; }
  __device__ static __forceinline__ S conj(S a) { return {a.re, df_neg(a.im)}; }
  __device__ static __forceinline__ S scale(S a, double s) {
    dfr t = df_from_d(s);
    return {df_mul(a.re, t), df_mul(a.im, t)};
  }
  __device__ static __forceinline__ S scale_f(S a, float s) { return {df_mul_f(a.re, s), df_mul_f(a.im, s)}; }
  __device__ static __forceinline__ S div_int(S a, int k) { return {df_div_int(a.re, k), df_div_int(a.im, k)}; }
  __device__ static __forceinline__ S from_c64(c64 v) { return {df_from_d(v.re), df_from_d(v.im)}; }
  __device__ static __forceinline__ c64 to_c64(S a) { return {df_to_d(a.re), df_to_d(a.im)}; }
  __device__ static __forceinline__ unsigned long long key(S a) {
    const unsigned x = absbits_f(a.re.hi), y = absbits_f(a.im.hi);
    return x > y ? x : y;
  }
  __device__ static __forceinline__ unsigned long long key_deflate(unsigned long long k) { return key_shift_f(k); }
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)k; }
  __device__ static __forceinline__ bool is_zero(S a) { return (absbits_f(a.re.hi) | absbits_f(a.im.hi)) == 0; }
  __device__ static __forceinline__ S recip(S a) {
    // conj(z) / |z|^2 on z scaled by a power of two into [1, 2) (so |z|^2 in [1, 8) neither
    // overflows nor underflows), in FP32 instructions only
    const unsigned x = absbits_f(a.re.hi), y = absbits_f(a.im.hi);
    const float f = df_pow2_inv(x > y ? x : y);
    const dfr re = {a.re.hi * f, a.re.lo * f}, im = {a.im.hi * f, a.im.lo * f};
    const dfr d = df_recip_unit(df_fma2(re, re, im, im, dfr{0.f, 0.f}));
    const dfr rr = df_mul(re, d), ri = df_mul(im, d);
    return {{rr.hi * f, rr.lo * f}, {neg_f(ri.hi * f), neg_f(ri.lo * f)}};
  }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return i ? a.im : a.re; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) {
    if (i) a.im = v; else a.re = v;
  }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return df_add(a, b); }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
  }
  __device__ static __forceinline__ S shfl(S v, int src) {
    return {{__shfl_sync(0xffffffffu, v.re.hi, src), __shfl_sync(0xffffffffu, v.re.lo, src)},
            {__shfl_sync(0xffffffffu, v.im.hi, src), __shfl_sync(0xffffffffu, v.im.lo, src)}};
  }
};

// Double-double: FP64's exponent range, so the normalised (unit-subdiagonal) elimination of the
// FP64 types applies; pivot keys from the high parts.
template <>
struct Ar<ddr> {
  using S = ddr;
  using Comp = ddr;
  static constexpr int NC = 1;
  static constexpr bool cplx = false;
  static constexpr bool fp64 = true;
  static constexpr bool modular = false;
  static constexpr bool dd = true;
  static constexpr int DEFLATE_BITS = 92;
  __device__ static __forceinline__ S zero() { return {0.0, 0.0}; }
  __device__ static __forceinline__ S one() { return {1.0, 0.0}; }
  __device__ static __forceinline__ S add(S a, S b) { return dd_add(a, b); }
  __device__ static __forceinline__ S sub(S a, S b) { return dd_add(a, dd_neg(b)); }
  __device__ static __forceinline__ S mul(S a, S b) { return dd_mul(a, b); }
  __device__ static __forceinline__ S fma(S a, S b, S c) { return dd_fma(a, b, c); }
  __device__ static __forceinline__ S fnma(S a, S b, S c) { return dd_fma(dd_neg(a), b, c); }
  __device__ static __forceinline__ S neg(S a) { return dd_neg(a); }
  __device__ static __forceinline__ S conj(S a) { return a; }
  __device__ static __forceinline__ S scale(S a, double s) { return dd_mul_d(a, s); }
  __device__ static __forceinline__ S scale_f(S a, float s) { return dd_mul_d(a, (double)s); }
  __device__ static __forceinline__ S div_int(S a, int k) { return dd_div_int(a, k); }
  __device__ static __forceinline__ S from_c64(c64 v) { return {v.re, 0.0}; }
  __device__ static __forceinline__ c64 to_c64(S a) { return {a.hi, 0.0}; }
  __device__ static __forceinline__ c64 lo_c64(S a) { return {a.lo, 0.0}; }
  __device__ static __forceinline__ unsigned long long key(S a) { return absbits_d(a.hi); }
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)(k >> 32); }
  __device__ static __forceinline__ bool is_zero(S a) { return absbits_d(a.hi) == 0; }
  __device__ static __forceinline__ S recip(S a) { return dd_recip(a); }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return a; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) { a = v; }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return dd_add(a, b); }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
  }
  __device__ static __forceinline__ S shfl(S v, int src) {
    return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
  }
};

template <>
struct Ar<cdd> {
  using S = cdd;
  using Comp = ddr;
  static constexpr int NC = 2;
  static constexpr bool cplx = true;
  static constexpr bool fp64 = true;
  static constexpr bool modular = false;
  static constexpr bool dd = true;
  static constexpr int DEFLATE_BITS = 92;
  __device__ static __forceinline__ S zero() { return {{0.0, 0.0}, {0.0, 0.0}}; }
  __device__ static __forceinline__ S one() { return {{1.0, 0.0}, {0.0, 0.0}}; }
  __device__ static __forceinline__ S add(S a, S b) { return {dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
  __device__ static __forceinline__ S sub(S a, S b) { return {dd_add(a.re, dd_neg(b.re)), dd_add(a.im, dd_neg(b.im))}; }
  __device__ static __forceinline__ S mul(S a, S b) {
    const ddr z = {0.0, 0.0};
    return {dd_fma2(a.re, b.re, dd_neg(a.im), b.im, z), dd_fma2(a.re, b.im, a.im, b.re, z)};
  }
  __device__ static __forceinline__ S fma(S a, S b, S c) {
    return {dd_fma2(a.re, b.re, dd_neg(a.im), b.im, c.re), dd_fma2(a.re, b.im, a.im, b.re, c.im)};
  }
  __device__ static __forceinline__ S fnma(S a, S b, S c) {
    return {dd_fma2(dd_neg(a.re), b.re, a.im, b.im, c.re), dd_fma2(dd_neg(a.re), b.im, dd_neg(a.im), b.re, c.im)};
  }
  __device__ static __forceinline__ S neg(S a) { return {dd_neg(a.re), dd_neg(a.im)}; }
  __device__ static __forceinline__ S conj(S a) { return {a.re, dd_neg(a.im)}; }
  __device__ static __forceinline__ S scale(S a, double s) { return {dd_mul_d(a.re, s), dd_mul_d(a.im, s)}; }
  __device__ static __forceinline__ S scale_f(S a, float s) { return scale(a, (double)s); }
  __device__ static __forceinline__ S div_int(S a, int k) { return {dd_div_int(a.re, k), dd_div_int(a.im, k)}; }
  __device__ static __forceinline__ S from_c64(c64 v) { return {{v.re, 0.0}, {v.im, 0.0}}; }
  __device__ static __forceinline__ c64 to_c64(S a) { return {a.re.hi, a.im.hi}; }
  __device__ static __forceinline__ c64 lo_c64(S a) { return {a.re.lo, a.im.lo}; }
  __device__ static __forceinline__ unsigned long long key(S a) {
    const unsigned long long x = absbits_d(a.re.hi), y = absbits_d(a.im.hi);
    return x > y ? x : y;
  }
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return (unsigned)(k >> 32); }
  __device__ static __forceinline__ bool is_zero(S a) { return (absbits_d(a.re.hi) | absbits_d(a.im.hi)) == 0; }
  __device__ static __forceinline__ S recip(S a) {
    const ddr z = {0.0, 0.0};
    const ddr d = dd_recip(dd_fma2(a.re, a.re, a.im, a.im, z));
    return {dd_mul(a.re, d), dd_neg(dd_mul(a.im, d))};
  }
  __device__ static __forceinline__ Comp comp(const S& a, int i) { return i ? a.im : a.re; }
  __device__ static __forceinline__ void set_comp(S& a, int i, Comp v) {
    if (i) a.im = v; else a.re = v;
  }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return dd_add(a, b); }
  __device__ static __forceinline__ Comp shfl_xor(Comp v, int m) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
  }
  __device__ static __forceinline__ S shfl(S v, int src) {
    return {{__shfl_sync(0xffffffffu, v.re.hi, src), __shfl_sync(0xffffffffu, v.re.lo, src)},
            {__shfl_sync(0xffffffffu, v.im.hi, src), __shfl_sync(0xffffffffu, v.im.lo, src)}};
  }
};

// ---------------------------------------------------------------- residues modulo a prime
// Exact arithmetic for integer inputs: every step of the sieve (elimination with any nonzero
// pivot, La Budde, the series, the prefactors) is a field operation, so the sieve of an integer
// matrix is exact in F_P; the host combines several primes by the Chinese remainder theorem.
// Residues are held in Montgomery form x R mod P (R = 2^32): a product is one 32x32->64
// multiply and a Montgomery reduction (two more multiplies, a shift and a conditional
// subtraction), all on the integer pipe.
template <uint32_t P>
struct modp {
  uint32_t v;  // Montgomery form
};

template <uint32_t P>
struct Montgomery {
  // -P^-1 mod 2^32 by Newton's iteration x <- x (2 - P x), correct to 2^32 after five steps
  static constexpr uint32_t inv_neg() {
    uint32_t x = P;  // P x = 1 mod 2^3 for odd P
    for (int i = 0; i < 5; ++i) x *= 2u - P * x;
    return 0u - x;
  }
  static constexpr uint32_t NEG_INV = inv_neg();
  static constexpr uint32_t R1 = (uint32_t)((1ull << 32) % P);                       // R mod P
  static constexpr uint32_t R2 = (uint32_t)((unsigned __int128)R1 * R1 % P);          // R^2 mod P
  __host__ __device__ static constexpr uint32_t redc(uint64_t t) {                   // t R^-1 mod P
    const uint32_t m = (uint32_t)t * NEG_INV;
    const uint32_t u = (uint32_t)((t + (uint64_t)m * P) >> 32);
    return u >= P ? u - P : u;
  }
  __host__ __device__ static constexpr uint32_t to_mont(uint32_t x) { return redc((uint64_t)x * R2); }
};

template <uint32_t P>
struct Ar<modp<P>> {
  using S = modp<P>;
  using Comp = modp<P>;
  using M = Montgomery<P>;
  static constexpr int NC = 1;
  static constexpr bool cplx = false;
  static constexpr bool fp64 = true;  // exact zero tests, normalised (unit-subdiagonal) elimination
  static constexpr bool modular = true;
  static constexpr bool dd = false;
  __device__ static __forceinline__ S zero() { return S{0u}; }
  __device__ static __forceinline__ S one() { return S{M::R1}; }
  __device__ static __forceinline__ S add(S a, S b) {
    const uint32_t s = a.v + b.v;  // < 2^32
    return S{s >= P ? s - P : s};
  }
  __device__ static __forceinline__ S sub(S a, S b) { return S{a.v >= b.v ? a.v - b.v : a.v + P - b.v}; }
  __device__ static __forceinline__ S neg(S a) { return S{a.v ? P - a.v : 0u}; }
  __device__ static __forceinline__ S mul(S a, S b) { return S{M::redc((uint64_t)a.v * b.v)}; }
  __device__ static __forceinline__ S fma(S a, S b, S c) { return add(mul(a, b), c); }
  __device__ static __forceinline__ S fnma(S a, S b, S c) { return sub(c, mul(a, b)); }
  __device__ static __forceinline__ S conj(S a) { return a; }
  __device__ static __forceinline__ S of_int(long long k) {
    const long long r = k % (long long)P;
    return S{M::to_mont((uint32_t)(r < 0 ? r + P : r))};
  }
  __device__ static __forceinline__ S half() { return S{M::to_mont((P + 1) / 2)}; }
  // exact for the integers and half-integers the kernel scales by
  __device__ static __forceinline__ S scale(S a, double s) {
    const long long t = __double2ll_rn(2.0 * s);
    return mul(mul(a, of_int(t)), half());
  }
  __device__ static __forceinline__ S pow(S a, uint32_t e) {
    S r = one();
    while (e) {
      if (e & 1u) r = mul(r, a);
      a = mul(a, a);
      e >>= 1;
    }
    return r;
  }
  __device__ static __forceinline__ S recip(S a) { return pow(a, P - 2); }  // Fermat
  __device__ static __forceinline__ S inv_int(int k) { return recip(of_int(k)); }
  // plain residues (< 2^31) travel through FP64 slots exactly
  __device__ static __forceinline__ S from_c64(c64 z) { return of_int(__double2ll_rn(z.re)); }
  __device__ static __forceinline__ c64 to_c64(S a) { return {(double)M::redc(a.v), 0.0}; }
  __device__ static __forceinline__ unsigned long long key(S a) { return a.v; }  // any nonzero pivot
  __device__ static __forceinline__ unsigned long long key_deflate(unsigned long long) { return 0ull; }
  __device__ static __forceinline__ unsigned key32(unsigned long long k) { return k ? 0x80u : 0u; }
  __device__ static __forceinline__ bool is_zero(S a) { return a.v == 0u; }
  __device__ static __forceinline__ Comp comp(const S& a, int) { return a; }
  __device__ static __forceinline__ void set_comp(S& a, int, Comp v) { a = v; }
  __device__ static __forceinline__ Comp cadd(Comp a, Comp b) { return add(a, b); }
  __device__ static __forceinline__ Comp shfl_xor(Comp a, int m) { return S{__shfl_xor_sync(0xffffffffu, a.v, m)}; }
  __device__ static __forceinline__ S shfl(S a, int src) { return S{__shfl_sync(0xffffffffu, a.v, src)}; }
};

}  // namespace wg
