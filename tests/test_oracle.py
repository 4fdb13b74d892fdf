"""Pins the CPU oracle against vectors produced by the reference itself and against the
reference test-suite's known answers (thewalrus/tests/test_hafnian.py, test_hafnian_repeated.py,
test_labudde.py, test_reference.py)."""
import math
import os

import numpy as np
import pytest

import oracle
from thewalrus_gb300 import workloads as wl

T = [1, 1, 2, 4, 10, 26, 76, 232, 764, 2620, 9496]  # telephone numbers


def rel(a, b):
    return abs(complex(a) - complex(b)) / max(abs(complex(b)), 1e-300)


@pytest.mark.parametrize("prec", ["double", "quad"])
def test_plain_vs_reference(golden, prec):
    for c in golden["haf"]:
        A = c["A"]
        if prec == "quad" and A.shape[0] > 20:
            continue
        got = oracle.hafnian(A, precision=prec)
        assert rel(got, c["out"]) < 1e-11, (A.shape, got, c["out"])


def test_inclexcl_vs_reference(golden):
    for c in golden["haf_inclexcl"]:
        got = oracle.hafnian(c["A"], method="inclexcl")
        assert rel(got, c["out"]) < 1e-11


@pytest.mark.parametrize("prec", ["double", "long"])
def test_loop_vs_reference(golden, prec):
    for c in golden["lhaf"]:
        got = oracle.hafnian(c["A"], loop=True, precision=prec)
        assert rel(got, c["out"]) < 1e-11, (c["A"].shape, got, c["out"])


def test_repeated_vs_reference(golden):
    for c in golden["rep"]:
        got = oracle.hafnian_repeated(c["A"], list(c["rpt"]))
        assert rel(got, c["out"]) < 1e-11, (c["rpt"], got, c["out"])
    for c in golden["rep_loop"]:
        got = oracle.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True)
        assert rel(got, c["out"]) < 1e-11, (c["rpt"], got, c["out"])


def test_batch_vs_reference(golden):
    for c in golden["batch"]:
        got = oracle.loop_hafnian_batch(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]))
        ref = c["out"]
        assert got.shape == ref.shape
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) / scale < 1e-11


def test_batch_gamma_vs_reference(golden):
    odd_paths = 0
    for c in golden["batch_gamma"]:
        got = oracle.loop_hafnian_batch_gamma(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]))
        ref = c["out"]
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-11
        odd_paths += oracle.matched_reps(np.asarray(c["fixed"])[np.nonzero(c["fixed"])])[2] is not None
    assert 0 < odd_paths < len(golden["batch_gamma"])  # both the even and the odd pairing paths


def test_brute_force(golden):
    for c in golden["brute"]:
        A, loop = c["A"], bool(c["loop"])
        assert rel(oracle.hafnian(A, loop=loop), c["out"]) < 1e-11
        assert rel(oracle.brute_hafnian(A, loop=loop), c["out"]) < 1e-12


def test_powertrace_charpoly(golden):
    for c in golden["ptrace"]:
        got = oracle.powertrace(c["H"], int(c["n"]))
        np.testing.assert_allclose(got, c["out"], rtol=1e-10, atol=1e-10)
    for c in golden["charpoly"]:
        np.testing.assert_allclose(oracle.charpoly(c["H"]), c["out"], rtol=1e-10, atol=1e-10)


def test_labudde_known_answers():
    # thewalrus/tests/test_labudde.py:22-74
    for phi in (0.1, 0.2, 0.3):
        m = np.array([[math.cosh(phi), math.sinh(phi)], [math.sinh(phi), math.cosh(phi)]])
        cp = oracle.charpoly(m)
        assert np.allclose(cp[0], -2 * math.cosh(phi)) and np.allclose(cp[1], 1)
    mat = np.array([[1.04975523, 0.31935254, 1, 2], [0.31935254, 1.04975523, 3, 4],
                    [0.31635254, 2.444, 5, 6], [21.31935254, 3.14975523, 7, 8]])
    for n, v in ((1, 15.0995), (2, 301.18), (4, 81466.1)):
        assert np.allclose(oracle.powertrace(mat, n + 1)[-1], v)


@pytest.mark.parametrize("n", [6, 8, 12])
def test_known_answers(n):
    # haf(J_2n) = (2n)!/(n! 2^n); haf([[0,J],[J,0]]) = n!; lhaf(J_n) = T(n)
    J = np.ones((2 * n, 2 * n))
    assert oracle.hafnian(J, precision="quad").real == pytest.approx(
        math.factorial(2 * n) / (math.factorial(n) * 2**n), rel=1e-15)
    O, B = np.zeros((n, n)), np.ones((n, n))
    assert oracle.hafnian(np.block([[O, B], [B, O]])).real == pytest.approx(math.factorial(n), rel=1e-13)
    if n <= 10:
        assert oracle.hafnian(np.ones((n, n)), loop=True).real == pytest.approx(T[n], rel=1e-13)
    assert oracle.hafnian_repeated(np.array([[1.0]]), [2 * n]).real == pytest.approx(
        math.factorial(2 * n) / (math.factorial(n) * 2**n), rel=1e-13)


def test_all_ones_24_exact():
    got = oracle.hafnian(np.ones((24, 24)), precision="quad")
    assert got.real == 316234143225.0 and abs(got.lo) < 1e-3


def test_matched_reps_cases():
    x, er, odd = oracle.matched_reps([0, 0, 0, 0])
    assert x.shape == (0,) and er.shape == (0,) and odd is None
    x, er, odd = oracle.matched_reps([3])
    assert list(er) == [1] and odd == 0


def test_exact_oracle_known_values():
    import math

    for n in (4, 8, 12, 24):
        assert oracle.exact_hafnian(np.ones((n, n), dtype=np.int64)) == math.prod(range(n - 1, 0, -2))
    rng = np.random.default_rng(0)
    for n in (6, 8, 10):
        A = wl.adjacency01(n, seed=n)
        assert oracle.exact_hafnian(A) == round(oracle.brute_hafnian(A).real)
        assert oracle.exact_hafnian(A, glynn=False) == round(oracle.brute_hafnian(A).real)
        B = rng.integers(-3, 4, size=(n, n))
        B = B + B.T
        assert oracle.exact_hafnian(B) == round(oracle.brute_hafnian(B).real)
    A = rng.integers(-2, 3, size=(4, 4))
    A = A + A.T
    assert oracle.exact_hafnian(A, reps=[2, 1, 3, 2]) == round(complex(oracle.hafnian_repeated(A, [2, 1, 3, 2])).real)
    # against the _Float128 oracle on a 20-vertex graph
    A = wl.adjacency01(20, seed=4)
    assert oracle.exact_hafnian(A) == round(complex(oracle.hafnian(A, precision="quad")).real)


def test_metric_fixture_cross_checks():
    """The benchmark-size reference values (tests/golden/metric_cases.npz) against the oracle's
    values stored beside them: the well-conditioned plain hafnians agree to 1e-12; the loop
    hafnian of the 20-mode, 40-photon state (condition number ~3e10) agrees with the _Float128
    value within 2^-53 times its condition number."""
    data = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "metric_cases.npz"))
    for case in ("haf40_complex", "haf40_real"):
        out, ld = complex(data[case + "/out"]), complex(data[case + "/oracle_ld"])
        assert abs(out - ld) <= 1e-12 * abs(ld)
        assert float(data[case + "/cond"]) < 1e6
    out = complex(data["lhaf_state20_40/out"])
    q = complex(data["lhaf_state20_40/oracle_q"])
    ld = complex(data["lhaf_state20_40/oracle_ld"])
    cond = float(data["lhaf_state20_40/cond"])
    assert cond > 1e9
    assert abs(out - q) <= 2.0 ** -53 * cond * abs(q)
    assert abs(ld - q) <= 2.0 ** -64 * cond * abs(q)
