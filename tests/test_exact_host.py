"""Host side of the exact (modular) sieve, without a GPU: the Chinese remainder step and the
magnitude bound that decides how many primes run."""
import math

import numpy as np

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat, workloads as wl


def test_crt_round_trip():
    rng = np.random.default_rng(1)
    for k in (2, 3, 5):
        M = math.prod(nat.MOD_PRIMES[:k])
        for _ in range(200):
            v = int(rng.integers(-2**62, 2**62)) * int(rng.integers(1, 2**28))
            v %= M
            if v > M // 2:
                v -= M
            assert nat.crt([v % p for p in nat.MOD_PRIMES[:k]], nat.MOD_PRIMES[:k]) == v


def test_bound_covers_exact_values():
    rng = np.random.default_rng(2)
    cases = [np.ones((n, n)) for n in (10, 20, 30)] + [wl.adjacency01(n, seed=n) for n in (12, 20, 28)]
    for n in (10, 14, 18):
        B = rng.integers(-5, 6, size=(n, n))
        cases.append((B + B.T).astype(float))
    for A in cases:
        inst = tw.prepare_hafnian(A)
        exact = oracle.exact_hafnian(A)
        assert exact == 0 or math.log2(abs(exact)) <= inst.log2_bound()
        k = nat.exact_primes([inst])
        assert k is not None and math.prod(nat.MOD_PRIMES[:k]) > 2 * abs(exact)


def test_exact_is_the_default_for_integer_inputs():
    from thewalrus_gb300._hafnian import _auto

    assert _auto(None, [tw.prepare_hafnian(np.ones((8, 8)))]) == "exact"
    assert _auto(None, [tw.prepare_hafnian(np.ones((8, 8), dtype=np.complex128))]) == "exact"
    assert _auto(None, [tw.prepare_hafnian(wl.real_signed(8, seed=1))]) == "fp64"
    assert _auto(None, [tw.prepare_hafnian(wl.complex_symmetric(8, seed=1))]) == "fp64"
    assert _auto("df", [tw.prepare_hafnian(np.ones((8, 8)))]) == "df"
