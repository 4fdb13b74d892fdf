"""Host-side behaviour of the public functions, no GPU: argument checks and the cases answered
before the sieve runs (thewalrus/_hafnian.py:634-665 ``input_validation``, :717-818 the special
cases of ``hafnian``, :864-936 ``hafnian_repeated``; the reference's tests
thewalrus/tests/test_hafnian.py:86-118 and :350-370 check the same), and the fast ``allclose``
these checks use against ``numpy.allclose``."""
import itertools

import numpy as np
import pytest

import thewalrus_gb300 as tw
from thewalrus_gb300 import _hafnian as H


@pytest.mark.filterwarnings("ignore:overflow encountered")  # numpy.allclose(1e308, -1e308) warns too
def test_allclose_matches_numpy():
    rng = np.random.default_rng(5)
    special = [0.0, -0.0, 1e-9, -1e-9, 1.0, np.inf, -np.inf, np.nan, 1e308, -1e308, 5e-324]
    for rtol, atol in ((1e-5, 1e-8), (0.0, 0.0), (1e-3, 0.0), (0.0, 1e-3)):
        for a, b in itertools.product(special, repeat=2):
            assert H._allclose(np.array([a]), np.array([b]), rtol, atol) == np.allclose(a, b, rtol, atol), (a, b)
            ca, cb = complex(a, 1.0), complex(1.0, b)
            assert H._allclose(np.array([ca]), np.array([cb]), rtol, atol) == np.allclose(ca, cb, rtol, atol)
        for _ in range(200):
            A = rng.normal(size=(5, 5)) * 10.0 ** rng.integers(-12, 3)
            B = A + rng.normal(size=(5, 5)) * 10.0 ** rng.integers(-14, 0)
            if rng.random() < 0.3:
                B = B + 1j * rng.normal(size=(5, 5)) * 10.0 ** rng.integers(-14, 0)
            assert H._allclose(A, B, rtol, atol) == np.allclose(A, B, rtol, atol)
            assert H._allclose(A, 0, rtol, atol) == np.allclose(A, 0, rtol, atol)


def test_argument_errors():
    with pytest.raises(TypeError):
        tw.hafnian(1)
    with pytest.raises(TypeError):
        tw.hafnian([[0.0, 1.0], [1.0, 0.0]])
    with pytest.raises(ValueError):
        tw.hafnian(np.zeros([2, 3]))
    A = np.ones([4, 4])
    A[0, 1] = 0.0
    with pytest.raises(ValueError):
        tw.hafnian(A)
    with pytest.raises(ValueError):
        tw.hafnian(np.array([[2, 1], [1, np.nan]]))
    with pytest.raises(ValueError):
        tw.hafnian(np.array([[np.inf, 1.0], [2.0, np.inf]]))
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.ones([2, 2]), [1])
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.ones([2, 2]), [1, -1])
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.ones([2, 2]), [1, 0.5])
    # symmetric within the tolerance passes
    A = np.ones([4, 4])
    A[0, 1] += 1e-9
    assert tw.input_validation(A)


def _brute(A, loop):
    """Sum over perfect matchings (with loops: matchings of any size, unmatched vertices
    weighted by their diagonal entries)."""
    n = len(A)

    def rec(free):
        if not free:
            return 1.0
        i, rest = free[0], free[1:]
        total = A[i, i] * rec(rest) if loop else 0.0
        for k, j in enumerate(rest):
            total += A[i, j] * rec(rest[:k] + rest[k + 1:])
        return total

    return rec(list(range(n)))


def test_special_cases_answered_on_the_host():
    rng = np.random.default_rng(9)
    assert tw.hafnian(np.ndarray((0, 0))) == 1
    assert tw.hafnian(np.ones([3, 3])) == 0
    assert tw.hafnian(np.ones([5, 5])) == 0
    for n in (2, 3, 4):
        for cplx in (False, True):
            A = rng.normal(size=(n, n)) + (1j * rng.normal(size=(n, n)) if cplx else 0)
            A = A + A.T
            if n != 3:
                assert np.isclose(tw.hafnian(A), _brute(A, False), rtol=1e-14, atol=0)
            assert np.isclose(tw.hafnian(A, loop=True), _brute(A, True), rtol=1e-14, atol=0)
    d = rng.normal(size=7)
    assert tw.hafnian(np.diag(d)) == 0
    assert np.isclose(tw.hafnian(np.diag(d), loop=True), np.prod(d), rtol=1e-14)
    # repeated rows: no photons, odd photon numbers, the zero matrix
    A = np.ones([2, 2])
    assert tw.hafnian_repeated(A, [0, 0]) == 1.0
    assert tw.hafnian_repeated(A, [1, 2]) == 0.0
    assert tw.hafnian_repeated(np.zeros([3, 3]), [2, 1, 1]) == 0
    mu = np.array([2.0, 3.0, 0.5])
    assert tw.hafnian_repeated(np.zeros([3, 3]), [2, 1, 3], mu=mu, loop=True) == 4.0 * 3.0 * 0.125
    assert tw.loop_hafnian(A, D=np.ones(2), reps=[0, 0]) == 1.0
    x, y, z = tw.matched_reps([0, 0, 0, 0])
    assert x.shape == (0,) and y.shape == (0,) and z is None


def test_prepared_instances_match_a_direct_construction():
    """The host preparation (edge pairing, row/column selection, the real/complex choice, the
    batch edges) against the same construction written out with numpy's generic indexing, for
    ordinary inputs (which pair balancing leaves untouched)."""
    from thewalrus_gb300 import _native as nat
    from thewalrus_gb300 import workloads as wl

    def typed(x, cplx):
        x = np.asarray(x)
        return x.astype(np.complex128) if cplx else x.real.astype(np.float64)

    rng = np.random.default_rng(21)
    for trial in range(40):
        n = int(rng.integers(2, 9))
        A = wl.complex_symmetric(n, seed=trial) if trial % 2 else wl.real_signed(n, seed=trial)
        D = rng.normal(size=n) + (1j * rng.normal(size=n) if trial % 2 else 0)
        reps = [int(r) for r in rng.integers(0, 3, size=n)]
        if sum(reps) == 0:
            reps[0] = 2
        x, er, odd = tw.matched_reps(reps)
        cplx = bool(trial % 2)  # complex_symmetric and the complex D have nonzero imaginary parts
        if sum(reps) % 2 == 0:
            inst = tw.prepare_hafnian(A, reps)
            assert inst.A.dtype == (np.complex128 if cplx else np.float64)
            assert np.array_equal(inst.A, typed(A[np.ix_(x, x)], cplx))
            assert np.array_equal(inst.reps, er)
        inst = tw.prepare_loop_hafnian(A, D, reps)
        if isinstance(inst, nat.Instance):
            assert np.array_equal(inst.A, typed(A[np.ix_(x, x)], cplx))
            assert np.array_equal(inst.D, typed(np.asarray(D)[x], cplx))
            if odd is not None:
                assert np.array_equal(inst.oddV, typed(A[odd, x], cplx))
        # loop_hafnian_batch: the fixed modes' pairing, bordered by the batch edge(s)
        fixed = reps[:-1]
        bi = tw.prepare_loop_hafnian_batch(A, D, fixed, 4)
        nz = np.nonzero(fixed + [1])[0]
        fe, fm, fodd = tw.matched_reps(np.asarray(fixed)[nz[:-1]])
        edges = H._batch_edges_even(fe) if fodd is None else H._batch_edges_odd(fe, fodd)
        assert np.array_equal(bi.A, typed(A[np.ix_(nz, nz)][np.ix_(edges, edges)], cplx))
        assert np.array_equal(bi.D, typed(np.asarray(D)[nz][edges], cplx))
        assert np.array_equal(bi.reps, fm)
