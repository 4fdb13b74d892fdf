"""Exact sieves of integer inputs on the GPU (precision="exact": residues modulo three 31-bit
primes, Chinese remainder theorem) against the exact modular oracle, brute-force matchings and
closed forms -- exact equality, including counts beyond 2^53."""
import math

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat, workloads as wl

pytestmark = pytest.mark.gpu


def test_all_ones_exact_beyond_2_53():
    for n in (28, 30, 32, 34):
        want = math.prod(range(n - 1, 0, -2))
        got = nat.run_exact([tw.prepare_hafnian(np.ones((n, n)))])[0]
        assert got == want, (n, got, want)
        assert tw.hafnian(np.ones((n, n)), precision="exact") == float(want)


def test_graphs_vs_exact_oracle():
    for n, seed in ((24, 1), (32, 2), (36, 1), (40, 3)):
        A = wl.adjacency01(n, seed=seed)
        assert nat.run_exact([tw.prepare_hafnian(A)])[0] == oracle.exact_hafnian(A), (n, seed)


def test_signed_and_repeated_vs_exact_oracle():
    rng = np.random.default_rng(31)
    for case in range(4):
        n = 14 + 2 * case
        B = rng.integers(-3, 4, size=(n, n))
        B = B + B.T
        assert nat.run_exact([tw.prepare_hafnian(B)])[0] == oracle.exact_hafnian(B)
    for case in range(4):
        n = int(rng.integers(3, 6))
        B = rng.integers(-2, 3, size=(n, n))
        B = B + B.T
        rpt = rng.integers(1, 6, size=n)
        if rpt.sum() % 2:
            rpt[0] += 1
        got = nat.run_exact([tw.prepare_hafnian(B, list(rpt))])[0]
        assert got == oracle.exact_hafnian(B, reps=list(rpt)), rpt


def test_loop_and_batch_exact():
    rng = np.random.default_rng(37)
    for n in (5, 6, 7, 8):
        B = rng.integers(-2, 3, size=(n, n))
        B = B + B.T
        want = round(oracle.brute_hafnian(B, loop=True).real)
        assert nat.run_exact([tw.prepare_loop_hafnian(B)])[0] == want, n
    # loop_hafnian_batch on integers: every output an integer, equal to the FP64 path rounded
    B = rng.integers(-1, 2, size=(7, 7))
    B = B + B.T
    D = rng.integers(-2, 3, size=7).astype(np.float64)
    fixed = [1, 2, 0, 1, 1, 2]
    exact = nat.run_exact([tw.prepare_loop_hafnian_batch(B.astype(np.float64), D, fixed, 4)])
    ref = oracle.loop_hafnian_batch(B.astype(np.float64), D, fixed, 4)
    assert exact == [round(v.real) for v in ref]


def test_exact_rejects_non_integer_inputs():
    with pytest.raises(RuntimeError):
        tw.hafnian(np.full((6, 6), 0.5), precision="exact")
