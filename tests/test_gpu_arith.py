"""The kernels' own arithmetic primitives on the GPU (``wg_check_arith``) against IEEE and exact
references.

* The pivot reciprocal (``recip_newton``: the PTX approximate reciprocal refined by one
  third-order step r(1 + e + e^2), IEEE division outside the approximation's safe exponent range)
  against numpy's correctly rounded 1/x: within 1 ulp everywhere, over magnitudes 2^-1000 ..
  2^1000 and both signs.
* The double-double primitives (reciprocal, division by a small integer, product) against exact
  rational arithmetic: relative error below 2^-100 (a double-double carries 106 bits; the
  primitives give up a few bits to their final renormalisation).
* The double-float pivot reciprocal (real and complex, FP32 instructions only: a power-of-two
  prescaling, the float reciprocal and its Newton series with the residual kept in double-float)
  against exact rationals: real within 2^-48 (emulated worst case 2^-49: as accurate as rounding
  an FP64 reciprocal), complex within 2^-45 (emulated worst case 2^-45.9: |z|^2 and the two
  products add their roundings);
  the division by a small integer of the series within 2^-46; for operands and results within
  2^+-90, where the low part of a double-float is still a normal float (below ~2^-100 it loses
  bits to underflow, in any double-float arithmetic).
"""
from fractions import Fraction

import numpy as np
import pytest

from thewalrus_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _dd_inputs(rng, count, lo_exp=-60, hi_exp=60):
    hi = np.ldexp(rng.uniform(1.0, 2.0, size=count), rng.integers(lo_exp, hi_exp, size=count))
    hi *= rng.choice([-1.0, 1.0], size=count)
    lo = hi * rng.uniform(-1.0, 1.0, size=count) * 2.0 ** -54  # |lo| <= ulp(hi) / 2
    return hi, lo


def _rel(hi, lo, exact):
    return abs(Fraction(float(hi)) + Fraction(float(lo)) - exact) / abs(exact)


def test_pivot_reciprocal_within_one_ulp():
    rng = np.random.default_rng(1)
    x = np.ldexp(rng.uniform(1.0, 2.0, size=4000), rng.integers(-1000, 1000, size=4000))
    x *= rng.choice([-1.0, 1.0], size=4000)
    x = np.concatenate([x, [1.0, -1.0, 3.0, 7.0, 1e-300, 1e300, 2.0 ** -1022, 0.1, 1 / 3]])
    got, _ = nat.check_arith(0, x)
    want = 1.0 / x
    ulps = np.abs(got - want) / np.spacing(np.abs(want))
    assert np.all(np.isfinite(got))
    assert ulps.max() <= 1.0, (ulps.max(), x[np.argmax(ulps)])


def test_double_double_reciprocal_and_division():
    rng = np.random.default_rng(2)
    hi, lo = _dd_inputs(rng, 300)
    rh, rl = nat.check_arith(1, hi, lo)
    worst = max(_rel(a, b, 1 / (Fraction(float(h)) + Fraction(float(l)))) for a, b, h, l in zip(rh, rl, hi, lo))
    assert worst < 2.0 ** -100, worst
    k = rng.integers(1, 250, size=300).astype(np.float64)
    qh, ql = nat.check_arith(2, hi, lo, k)
    worst = max(_rel(a, b, (Fraction(float(h)) + Fraction(float(l))) / int(kk))
                for a, b, h, l, kk in zip(qh, ql, hi, lo, k))
    assert worst < 2.0 ** -100, worst


def test_double_double_product():
    rng = np.random.default_rng(3)
    ah, al = _dd_inputs(rng, 300)
    bh, bl = _dd_inputs(rng, 300)
    ph, pl = nat.check_arith(3, ah, al, bh, bl)
    worst = max(_rel(p, q, (Fraction(float(a)) + Fraction(float(b))) * (Fraction(float(c)) + Fraction(float(d))))
                for p, q, a, b, c, d in zip(ph, pl, ah, al, bh, bl))
    assert worst < 2.0 ** -100, worst


def _df_inputs(rng, count, lo_exp=-90, hi_exp=90):
    hi = np.ldexp(rng.uniform(1.0, 2.0, size=count), rng.integers(lo_exp, hi_exp, size=count))
    hi = (hi * rng.choice([-1.0, 1.0], size=count)).astype(np.float32).astype(np.float64)
    lo = (hi * rng.uniform(-1.0, 1.0, size=count) * 2.0 ** -25).astype(np.float32).astype(np.float64)
    return hi, lo


def test_double_float_reciprocals_and_division():
    rng = np.random.default_rng(4)
    hi, lo = _df_inputs(rng, 400)
    hi = np.concatenate([hi, [1.0, -1.0, 3.0, 0.1, 2.0 ** -90, 2.0 ** 90, 1.5 * 2.0 ** 89]]).astype(np.float32).astype(np.float64)
    lo = np.concatenate([lo, np.zeros(7)])
    rh, rl = nat.check_arith(4, hi, lo)
    worst = max(_rel(a, b, 1 / (Fraction(float(h)) + Fraction(float(l)))) for a, b, h, l in zip(rh, rl, hi, lo))
    assert worst < 2.0 ** -48, worst
    # complex: re and im of 1 / z, z = (hi, lo) + i (yh, yl), over mixed magnitudes of the parts
    yh, yl = _df_inputs(rng, 407, -20, 20)
    yh[::5] = 0.0
    yl[::5] = 0.0
    re, im = nat.check_arith(5, hi[:407], lo[:407], yh, yl)
    for k in range(407):
        x = Fraction(float(hi[k])) + Fraction(float(lo[k]))
        y = Fraction(float(yh[k])) + Fraction(float(yl[k]))
        d = x * x + y * y
        ex, ey = x / d, -y / d
        scale = max(abs(ex), abs(ey))
        assert abs(Fraction(float(re[k])) - ex) / scale < 2.0 ** -45, (k, float(re[k]), float(ex))
        assert abs(Fraction(float(im[k])) - ey) / scale < 2.0 ** -45, (k, float(im[k]), float(ey))
    k = rng.integers(1, 250, size=407).astype(np.float64)
    qh, ql = nat.check_arith(6, hi[:407], lo[:407], k)
    worst = max(_rel(a, b, (Fraction(float(h)) + Fraction(float(l))) / int(kk))
                for a, b, h, l, kk in zip(qh, ql, hi, lo, k))
    assert worst < 2.0 ** -46, worst
