"""Term matrices that repeat a row (a mode used by several edges, the batch edge's two ends):
their exact Hessenberg form has zero subdiagonal entries, which the elimination must meet as
zeros, not as rounding residues.  GPU against the oracle on the chain-rule sampler's batch calls
and on hafnians with large repetitions."""
import math

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat, samples as smp, workloads as wl

pytestmark = pytest.mark.gpu


def test_sampler_batch_calls_vs_oracle():
    M, cutoff, K = 12, 5, 64
    cov, mean = wl.gaussian_state_cov(M, seed=21)
    chain = smp._Chain(cov, mean, 2)
    np.random.seed(1)
    draws = [chain.attempt_draws() for _ in range(K)]
    starts = [chain.start(a, b) for a, b, _ in draws]
    het = [s[0] for s in starts]
    gam = [s[1].copy() for s in starts]
    det = np.zeros((K, M), dtype=int)
    fac = np.array([math.factorial(k) for k in range(cutoff + 1)], dtype=float)
    worst = 0.0
    for mode in range(M):
        m = mode + 1
        insts, refs = [], []
        for j in range(K):
            gam[j] -= het[j][mode] * chain.B[:, mode]
            args = (chain.B[:m, :m], gam[j][:m], det[j, :mode], cutoff)
            insts.append(tw.prepare_loop_hafnian_batch(*args))
            refs.append(oracle.loop_hafnian_batch(*args))
        got = nat.run(insts, "fp64").reshape(K, cutoff + 1)
        assert np.all(np.isfinite(got)), mode
        for j in range(K):
            worst = max(worst, np.max(np.abs(got[j] - refs[j])) / np.max(np.abs(refs[j])))
            p = (refs[j] * refs[j].conj()).real / fac
            det[j, mode] = smp._choose(p / p.sum(), draws[j][2][mode])
    assert worst < 1e-10, worst


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("df", 1e-7)])
def test_large_repetitions_vs_oracle(precision, tol):
    rng = np.random.default_rng(17)
    for case in range(6):
        n = int(rng.integers(3, 6))
        A = wl.complex_symmetric(n, seed=1700 + case)
        rpt = rng.integers(2, 7, size=n)
        mu = (rng.normal(size=n) + 1j * rng.normal(size=n)) * 0.5
        got = tw.hafnian_repeated(A, list(rpt), mu=mu, loop=True, precision=precision)
        ref = complex(oracle.hafnian_repeated(A, list(rpt), mu=mu, loop=True, precision="quad"))
        assert np.isfinite(got) and abs(got - ref) <= tol * abs(ref), (rpt, got, ref)
        if rpt.sum() % 2 == 0:
            got = tw.hafnian_repeated(A, list(rpt), precision=precision)
            ref = complex(oracle.hafnian_repeated(A, list(rpt), precision="quad"))
            assert np.isfinite(got) and abs(got - ref) <= tol * abs(ref), (rpt, got, ref)
