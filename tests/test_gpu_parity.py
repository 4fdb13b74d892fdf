"""GPU parity: the CUDA sieve (through the C ABI) against vectors produced by the reference and
against the CPU oracle in _Float128 arithmetic.  Tolerances: 1e-10 relative for FP64 terms;
exact integer rounding where the hafnian is an integer below 2^53."""
import math

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-10
T = [1, 1, 2, 4, 10, 26, 76, 232, 764, 2620, 9496]


def rel(a, b):
    return abs(complex(a) - complex(b)) / max(abs(complex(b)), 1e-300)


def test_plain_vs_reference(golden):
    for c in golden["haf"]:
        got = tw.hafnian(c["A"])
        assert isinstance(got, np.complex128)
        assert rel(got, c["out"]) < RTOL, (c["A"].shape, got, c["out"])


def test_inclexcl_vs_reference(golden):
    for c in golden["haf_inclexcl"]:
        assert rel(tw.hafnian(c["A"], method="inclexcl"), c["out"]) < RTOL


def test_loop_vs_reference(golden):
    for c in golden["lhaf"]:
        got = tw.hafnian(c["A"], loop=True)
        assert rel(got, c["out"]) < RTOL, (c["A"].shape, got, c["out"])


def test_repeated_vs_reference(golden):
    for c in golden["rep"]:
        got = tw.hafnian_repeated(c["A"], list(c["rpt"]))
        assert rel(got, c["out"]) < RTOL, (c["rpt"], got, c["out"])
    for c in golden["rep_loop"]:
        got = tw.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True)
        assert rel(got, c["out"]) < RTOL, (c["rpt"], got, c["out"])


def test_batch_vs_reference(golden):
    for c in golden["batch"]:
        got = tw.loop_hafnian_batch(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]))
        ref = c["out"]
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < RTOL


def test_batch_gamma_vs_reference(golden):
    for c in golden["batch_gamma"]:
        got = tw.loop_hafnian_batch_gamma(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]))
        ref = c["out"]
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < RTOL


def test_batch_gamma_rows_are_batches():
    # loop_hafnian_batch_gamma(A, D, f, c)[k] == loop_hafnian_batch(A, D[k], f, c), one plan for all rows
    B, D0, fixed, cutoff = wl.batch_loop_calls(count=1, seed=12, modes=7, cutoff=3)[0]
    D = np.array([D0 * (1 + 0.1 * k) - 0.2 * k * B[:, 0] for k in range(5)])
    got = tw.loop_hafnian_batch_gamma(B, D, list(fixed), cutoff)
    for k in range(len(D)):
        one = tw.loop_hafnian_batch(B, D[k], list(fixed), cutoff)
        assert np.max(np.abs(got[k] - one)) <= 1e-13 * np.max(np.abs(one))


def test_brute_force_small():
    for n in (6, 8, 10):
        A = wl.complex_symmetric(n, seed=70 + n)
        assert rel(tw.hafnian(A), oracle.brute_hafnian(A)) < RTOL
    for n in (5, 7, 9):
        A = wl.complex_symmetric(n, seed=80 + n)
        assert rel(tw.hafnian(A, loop=True), oracle.brute_hafnian(A, loop=True)) < RTOL


@pytest.mark.parametrize("precision", [None, "fp64"])  # None: the exact sieve for integer inputs
@pytest.mark.parametrize("n", [6, 8, 12])
def test_known_answers(n, precision):
    J = np.ones((2 * n, 2 * n))
    assert tw.hafnian(J, precision=precision).real == math.factorial(2 * n) // (math.factorial(n) * 2**n)
    O, B = np.zeros((n, n)), np.ones((n, n))
    assert round(tw.hafnian(np.block([[O, B], [B, O]]), precision=precision).real) == math.factorial(n)
    if n <= 10:
        assert tw.hafnian(np.ones((n, n)), loop=True, precision=precision).real == pytest.approx(T[n], rel=1e-13)
        assert tw.hafnian(np.ones((n + 1, n + 1)), loop=True,
                          precision=precision).real == pytest.approx(T[n + 1], rel=1e-13)
    assert tw.hafnian(np.identity(2 * n), precision=precision) == 0
    assert abs(tw.hafnian(np.identity(2 * n), loop=True, precision=precision) - 1) < 1e-12
    assert tw.hafnian_repeated(np.array([[1.0]]), [2 * n], precision=precision).real == pytest.approx(
        math.factorial(2 * n) / (math.factorial(n) * 2**n), rel=1e-13)


@pytest.mark.parametrize("precision", [None, "fp64"])
def test_all_ones_24_exact(precision):
    got = tw.hafnian(np.ones((24, 24)), precision=precision)
    assert got.real == 316234143225.0 and got.imag == 0.0


@pytest.mark.parametrize("n,kind", [(16, "complex"), (20, "signed"), (22, "nonneg"), (18, "adj")])
def test_vs_quad_oracle(n, kind):
    gen = {"complex": wl.complex_symmetric, "signed": wl.real_signed, "nonneg": wl.real_nonneg,
           "adj": wl.adjacency01}[kind]
    A = gen(n, seed=n)
    ref = oracle.hafnian(A, precision="quad")
    assert rel(tw.hafnian(A), ref) < RTOL
    if kind == "adj":  # integer hafnian below 2^53: must round to the exact count
        got = tw.hafnian(A, precision="fp64")
        assert round(got.real) == round(ref.real) and abs(got.real - round(ref.real)) < 1e-6
        assert tw.hafnian(A) == float(round(ref.real))  # default for integers: exact


def test_loop_odd_and_repeated_vs_quad():
    A, gamma, rpt = wl.gaussian_state_loop(modes=8, seed=5, photons=16, max_rep=3)
    ref = oracle.hafnian_repeated(A, list(rpt), mu=gamma, loop=True, precision="quad")
    assert rel(tw.hafnian_repeated(A, list(rpt), mu=gamma, loop=True), ref) < RTOL
    B = wl.complex_symmetric(13, seed=9)
    assert rel(tw.hafnian(B, loop=True), oracle.hafnian(B, loop=True, precision="quad")) < RTOL


def test_batch_identity():
    # loop_hafnian_batch(A, D, fixed, c)[k] == loop_hafnian(A, D, reps=fixed + [k])
    B, D, fixed, cutoff = wl.batch_loop_calls(count=1, seed=11, modes=6, cutoff=5)[0]
    got = tw.loop_hafnian_batch(B, D, list(fixed), cutoff)
    for k in range(cutoff + 1):
        ref = oracle.loop_hafnian(B, D, list(fixed) + [k], precision="quad")
        assert abs(got[k] - complex(ref)) <= RTOL * max(abs(complex(ref)), np.max(np.abs(got)) * 1e-3)


def test_hafnian_batch_uneven():
    mats = [wl.complex_symmetric(n, seed=n) for n in (6, 10, 14, 8)] + \
        [wl.real_nonneg(n, seed=n) for n in (12, 16)]
    got = tw.hafnian_batch(mats)
    for A, g in zip(mats, got):
        assert rel(g, tw.hafnian(A)) < 1e-13


def test_inputs_not_mutated():
    A = wl.complex_symmetric(10, seed=3)
    A0 = A.copy()
    tw.hafnian(A)
    tw.hafnian(A, loop=True)
    assert np.array_equal(A, A0)


def test_exact_integer_graphs():
    # random 0/1 graphs against the exact modular oracle: relative error within 1e-12, and the
    # FP64 sieve rounds to the exact perfect-matching count while the count's ulp-scaled error
    # stays well below 0.5 (counts below 2^36; at n = 32, ~2^40, the cancellation between terms
    # leaves errors of ~4e-13 relative, i.e. ~0.6 absolute)
    for n, seeds in ((24, (1, 2, 3)), (28, (1, 2)), (32, (1, 2)), (36, (1,))):
        for seed in seeds:
            A = wl.adjacency01(n, seed=seed)
            exact = oracle.exact_hafnian(A)
            got = tw.hafnian(A, precision="fp64")  # integer inputs default to the exact sieve
            assert abs(complex(got) - exact) <= 1e-12 * exact, (n, seed, got, exact)
            if exact < 2 ** 36:
                assert round(got.real) == exact and abs(got.imag) < 0.5, (n, seed, got, exact)


def test_all_ones_exact_to_n28():
    # (n-1)!! for the all-ones matrix rounds exactly up to n = 28 (27!! ~ 2^47.6); float64 and
    # complex128 inputs
    for n in (20, 24, 26, 28):
        want = math.prod(range(n - 1, 0, -2))
        for dt in (np.float64, np.complex128):
            got = tw.hafnian(np.ones((n, n), dtype=dt), precision="fp64")
            assert round(got.real) == want and abs(got.imag) < 0.5, (n, dt, got, want)
            assert tw.hafnian(np.ones((n, n), dtype=dt)) == float(want)  # default: exact for integers


@pytest.mark.parametrize("n,cplx", [(64, True), (58, True), (60, False)])
def test_large_tiles_on_a_term_prefix(n, cplx):
    """Term matrices of 58-64 rows (two whole 32-row blocks of the column update, or one block
    and a 26-28-row block) on the first 64 sieve terms: those are the terms whose leading 25+
    multiplicities sit at their first digit in both the Gray order here and the reference's
    mixed-radix order, so the shard equals the oracle's term-range sum times 2^-(n/2-1)."""
    from thewalrus_gb300 import _native as nat
    P = 64
    # the convention on a small instance first: the whole range is the hafnian
    small = tw.prepare_hafnian(wl.complex_symmetric(12, seed=3))
    whole = nat.run([small.shard(0, small.terms())])[0]
    assert rel(whole, oracle.haf_term_range(small.A, small.reps, 0, small.terms()) * 2.0 ** -5) < RTOL
    A = wl.complex_symmetric(n, seed=n) if cplx else wl.real_signed(n, seed=n)
    inst = tw.prepare_hafnian(A)
    assert inst.terms() == 2 ** (n // 2 - 1)
    got = nat.run([inst.shard(0, P)])[0]
    want = complex(oracle.haf_term_range(inst.A, inst.reps, 0, P)) * 2.0 ** -(n // 2 - 1)
    assert rel(got, want) < 1e-9, (got, want)


def test_golden_families_double_float(golden):
    """Every golden family with FP32 double-float terms (48-bit significand): 1e-8 relative, the
    bound the double-float error table supports at these sizes (n <= 24, worst seen 1.2e-9 on a
    signed real n = 20 matrix)."""
    tol = 1e-8
    for c in golden["haf"]:
        assert rel(tw.hafnian(c["A"], precision="df"), c["out"]) < tol, c["A"].shape
    for c in golden["haf_inclexcl"]:
        assert rel(tw.hafnian(c["A"], method="inclexcl", precision="df"), c["out"]) < tol
    for c in golden["lhaf"]:
        assert rel(tw.hafnian(c["A"], loop=True, precision="df"), c["out"]) < tol, c["A"].shape
    for c in golden["rep"]:
        assert rel(tw.hafnian_repeated(c["A"], list(c["rpt"]), precision="df"), c["out"]) < tol
    for c in golden["rep_loop"]:
        got = tw.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True, precision="df")
        assert rel(got, c["out"]) < tol, c["rpt"]
    for c in golden["batch"]:
        got = tw.loop_hafnian_batch(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]), precision="df")
        assert np.max(np.abs(got - c["out"])) / np.max(np.abs(c["out"])) < tol
