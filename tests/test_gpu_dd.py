"""Double-double terms (``precision="dd"``) on the GPU: FP64 pairs with a 106-bit significand,
and a compensated accumulation that keeps every term's low part.

For sums whose terms cancel beyond FP64's reach -- the 40-photon loop hafnian of the 20-mode
Gaussian state cancels to 1 part in 3.4e10 -- the FP64 sieve (this one or the reference's) is
good to ~1e-6..1e-8 only; double-double meets 1e-10 against the _Float128 oracle there.
Well-conditioned inputs come out far inside FP64's accuracy; the golden families of the
reference hold at 1e-10 (the reference's own values carry FP64 rounding)."""
import math
import os

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    return abs(complex(a) - complex(b)) / abs(complex(b))


def test_state20_40_photons_to_1e10():
    data = np.load(os.path.join(HERE, "golden", "metric_cases.npz"))
    A, rpt, mu = data["lhaf_state20_40/A"], data["lhaf_state20_40/rpt"], data["lhaf_state20_40/mu"]
    truth = complex(data["lhaf_state20_40/oracle_q"])
    got = tw.hafnian_repeated(A, list(rpt), mu=mu, loop=True, precision="dd")
    assert rel(got, truth) < 1e-10, (got, truth)


@pytest.mark.parametrize("n,kind", [(16, "complex"), (20, "signed"), (18, "nonneg")])
def test_vs_quad_far_below_fp64(n, kind):
    # both results are rounded to complex128 once: double-double meets the _Float128 value to the
    # last bit or two (4e-16), where the FP64 sieve is ~1e-13 away
    gen = {"complex": wl.complex_symmetric, "signed": wl.real_signed, "nonneg": wl.real_nonneg}[kind]
    A = gen(n, seed=n)
    truth = complex(oracle.hafnian(A, precision="quad"))
    assert rel(tw.hafnian(A, precision="dd"), truth) < 4e-16
    B = wl.complex_symmetric(n - 3, seed=n)
    truth = complex(oracle.hafnian(B, loop=True, precision="quad"))
    assert rel(tw.hafnian(B, loop=True, precision="dd"), truth) < 4e-16


def test_golden_families(golden):
    for c in golden["haf"]:
        assert rel(tw.hafnian(c["A"], precision="dd"), c["out"]) < 1e-10
    for c in golden["lhaf"]:
        assert rel(tw.hafnian(c["A"], loop=True, precision="dd"), c["out"]) < 1e-10
    for c in golden["rep"]:
        assert rel(tw.hafnian_repeated(c["A"], list(c["rpt"]), precision="dd"), c["out"]) < 1e-10
    for c in golden["rep_loop"]:
        got = tw.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True, precision="dd")
        assert rel(got, c["out"]) < 1e-10
    for c in golden["batch"]:
        got = tw.loop_hafnian_batch(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]), precision="dd")
        ref = c["out"]
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-10


def test_integers_round_exactly():
    # 29!! ~ 2^52.5: beyond what the FP64 sieve rounds exactly
    got = tw.hafnian(np.ones((30, 30)), precision="dd")
    assert got.real == float(math.prod(range(1, 30, 2))) and got.imag == 0.0
    A = wl.adjacency01(28, seed=5)
    assert tw.hafnian(A, precision="dd") == tw.hafnian(A)  # the exact sieve's integer
