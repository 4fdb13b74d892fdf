"""GPU parity at the benchmark sizes themselves: the 40x40 complex and real plain hafnians (seed 0,
524,288 sieve terms each) and the loop hafnian of the 20-mode Gaussian state with 40 photons
(``hafnian_repeated(A, rpt, mu=gamma, loop=True)``, 110,592 terms), against the values the
reference's own code produced for the same inputs (``tests/golden/metric_cases.npz``, written
by ``make_golden.py --metric``, which also stores the oracle's long-double values, the sieve
sum's condition number cond = sum|term| / |sum| and, where cond is large, the _Float128 value).

Tolerances.  The plain hafnians are well conditioned (cond 6.8e4 complex, 2.0e5 real): 1e-10
relative for FP64 against both the reference and the oracle.  Double-float terms carry a 48-bit
significand, so the sieve's cancellation leaves ~cond x 2^-48 (5e-10 complex, 1.4e-9 real);
they are held to 16 x cond x 2^-48, the bound ``hafnian_with_error`` states (measured: 1e-10
complex, 1.2e-9 real; a change in the order of any rounding moves the real one by up to ~10x
either way within that bound).
The 40-photon loop hafnian is not: its 110,592 terms cancel to 1 part in cond = 3.4e10, so
per-term rounding of 2^-53 can move the result by up to 3.8e-6 relative -- the reference's own
double result is 4.5e-8 from the _Float128 value.  FP64 is held to eps * cond against the
_Float128 value, and to the same bound against the reference's value.
"""
import os

import numpy as np
import pytest

import thewalrus_gb300 as tw

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RTOL = 1e-10
EPS = 2.0 ** -53
EPS_DF = 2.0 ** -48


@pytest.fixture(scope="module")
def metric():
    data = np.load(os.path.join(HERE, "golden", "metric_cases.npz"))
    out = {}
    for key in data.files:
        case, field = key.split("/")
        out.setdefault(case, {})[field] = data[key]
    return out


def rel(a, b):
    return abs(complex(a) - complex(b)) / abs(complex(b))


@pytest.mark.parametrize("case", ["haf40_complex", "haf40_real"])
@pytest.mark.parametrize("precision", ["fp64", "df"])
def test_plain_n40_vs_reference(metric, case, precision):
    c = metric[case]
    tol = RTOL if precision == "fp64" else 16 * float(c["cond"]) * EPS_DF
    got = tw.hafnian(c["A"], precision=precision)
    assert isinstance(got, np.complex128)
    assert rel(got, c["out"]) < tol, (case, precision, got, complex(c["out"]))


@pytest.mark.parametrize("case", ["haf40_complex", "haf40_real"])
def test_plain_n40_vs_oracle(metric, case):
    c = metric[case]
    assert rel(c["oracle_ld"], c["out"]) < 1e-12  # the fixture's own cross-check
    assert rel(tw.hafnian(c["A"], precision="fp64"), c["oracle_ld"]) < RTOL


def test_loop_state20_40_photons_fp64(metric):
    c = metric["lhaf_state20_40"]
    assert int(c["rpt"].sum()) == 40 and int(c["rpt"].max()) <= 3
    truth = complex(c["oracle_q"])
    tol = EPS * float(c["cond"])
    assert rel(c["out"], truth) < tol  # the reference's own double result meets the same bound
    got = tw.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True, precision="fp64")
    assert rel(got, truth) < tol, (got, truth, tol)
    assert rel(got, c["out"]) < 2 * tol


def test_batched_members_at_n40_vs_reference(metric):
    # the benchmark matrices as members of one batched plan (with smaller members beside them)
    from thewalrus_gb300 import workloads as wl
    mats = [metric["haf40_complex"]["A"], wl.complex_symmetric(12, seed=5), metric["haf40_real"]["A"],
            wl.real_nonneg(16, seed=6)]
    got = tw.hafnian_batch(mats)
    assert rel(got[0], metric["haf40_complex"]["out"]) < RTOL
    assert rel(got[2], metric["haf40_real"]["out"]) < RTOL
    assert rel(got[1], tw.hafnian(mats[1])) < 1e-13
