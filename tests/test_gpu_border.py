"""The loop kinds' border series (``border_prepare`` / ``border_series`` in sieve_kernel.cuh:
lambda_t = d x.H^(t-1) e_1 from La Budde's trailing determinants of the anti-transposed block)
on the paths the benchmark-size tests do not reach: more than 32 series coefficients (T = N/2 >=
33, so the coefficient and division sweeps take several 32-lane chunks), even and odd photon
numbers, and block-diagonal inputs, whose term matrices reduce to Hessenberg form with zero
subdiagonal entries (the weights x_r beta_1..beta_(r-1) stop at the first zero).

Double-double results are held to 1e-12 of the oracle's _Float128 value (these sums cancel to
cond = sum|term| / |sum| of up to 2.3e6, far inside double-double's reach).  FP64 results are
held to 32 x 2^-53 x cond: with 33 series coefficients the terms' own series cancel more than at
the benchmark sizes, and the error in units of 2^-53 x cond measured 1.1-16.3 over these inputs
(1.2-16.0 when the border data came from a Krylov sequence instead: the spread is the series',
not the border method's).  thewalrus/_hafnian.py:580-631 is the reference's loop hafnian."""
import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from oracle import matched_reps

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -53


def rel(a, b):
    return abs(complex(a) - complex(b)) / abs(complex(b))


def _inputs(trial, n=4):
    rng = np.random.default_rng(11)
    for _ in range(trial + 1):
        G = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        A = 0.3 * (G + G.T) / 2
        D = 0.5 * (rng.normal(size=n) + 1j * rng.normal(size=n))
    return A, D


def _cond(A, D, reps):
    """sum|term| / |sum| of the loop sieve (the oracle in double: enough for a tolerance)."""
    x, er, odd = matched_reps(reps)
    Ax = A[np.ix_(x, x)].astype(np.complex128)
    Dx = np.asarray(D)[x].astype(np.complex128)
    kw = {}
    if odd is not None:
        kw = dict(oddloop=complex(D[odd]), oddV=A[odd, x].astype(np.complex128))
    s = complex(oracle.sieve_term_range(Ax, er, Dx=Dx, **kw))
    a = abs(complex(oracle.sieve_term_range(Ax, er, Dx=Dx, absolute=True, **kw)))
    return a / abs(s)


@pytest.mark.parametrize("trial,reps", [(2, [17, 17, 16, 16]), (2, [17, 17, 16, 17]), (2, [20, 12, 18, 16]),
                                        (4, [17, 17, 16, 16]), (1, [17, 17, 16, 17])])
def test_more_than_32_series_coefficients(trial, reps):
    A, D = _inputs(trial)
    want = complex(oracle.hafnian_repeated(A, reps, mu=D, loop=True, precision="quad"))
    cond = _cond(A, D, reps)
    got_dd = tw.hafnian_repeated(A, reps, mu=D, loop=True, precision="dd")
    assert rel(got_dd, want) < 1e-12, (reps, got_dd, want)
    got = tw.hafnian_repeated(A, reps, mu=D, loop=True, precision="fp64")
    assert rel(got, want) < 32 * EPS * cond, (reps, got, want, cond)


@pytest.mark.parametrize("reps", [[3, 2, 3, 2], [2, 3, 2, 2], [9, 8, 9, 8], [12, 11, 12, 10]])
def test_block_diagonal_terms(reps):
    """A loop hafnian of a block-diagonal matrix is the product of its blocks' loop hafnians; the
    term matrices keep the block structure, so their reduction has zero subdiagonal entries."""
    A, D = _inputs(3)
    A[:2, 2:] = 0.0
    A[2:, :2] = 0.0
    want = complex(oracle.hafnian_repeated(A, reps, mu=D, loop=True, precision="quad"))
    blocks = complex(oracle.hafnian_repeated(A[:2, :2], reps[:2], mu=D[:2], loop=True, precision="quad")) * \
        complex(oracle.hafnian_repeated(A[2:, 2:], reps[2:], mu=D[2:], loop=True, precision="quad"))
    assert rel(blocks, want) < 1e-14  # the oracle agrees with the factorisation
    cond = _cond(A, D, reps)
    assert rel(tw.hafnian_repeated(A, reps, mu=D, loop=True, precision="dd"), want) < 1e-12
    assert rel(tw.hafnian_repeated(A, reps, mu=D, loop=True, precision="fp64"), want) < max(32 * EPS * cond, 1e-13)


def test_window_storage_in_a_mixed_plan():
    """A plain instance with an even repetition has terms with fewer than K + 1 rows, so a launch
    group holding it keeps La Budde's coefficient rows in the circular window instead of dead
    tile columns; the loop instances merged into that group read their trailing determinants
    from the window.  Every output equals the instance evaluated alone (tile storage)."""
    from thewalrus_gb300 import _native as nat
    from thewalrus_gb300 import workloads as wl

    A = wl.complex_symmetric(10, seed=5)
    plain = tw.prepare_hafnian(A, reps=[2, 1, 1, 2, 0, 1, 1, 0, 2, 0])
    B, D = _inputs(2, n=6)
    loops = [tw.prepare_loop_hafnian(B, D, [3, 2, 2, 1, 2, 2]), tw.prepare_loop_hafnian(B, D, [3, 2, 2, 1, 2, 1]),
             tw.prepare_loop_hafnian(B, D, [17, 17, 16, 16, 0, 0])]
    insts = [plain] + loops
    alone = [complex(nat.run([i])[0]) for i in insts]
    plan = nat.Plan(insts, merge_classes=True)
    try:
        plan.execute()
        mixed = plan.read()
    finally:
        plan.close()
    for a, b in zip(alone, mixed):
        assert rel(b, a) < 1e-13, (a, b)
    want = complex(oracle.hafnian_repeated(B, [17, 17, 16, 16, 0, 0], mu=D, loop=True, precision="quad"))
    assert rel(mixed[3], want) < 32 * EPS * _cond(B, D, [17, 17, 16, 16, 0, 0])
