"""Host-side pair balancing of prepared matrices (no GPU): a scaling of vertex e by s and of its
partner E + e by 1/s leaves the hafnian and every sieve term unchanged; balancing undoes such
scalings exactly (powers of two) and leaves ordinary and integer inputs untouched."""
import numpy as np

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _hafnian as H
from thewalrus_gb300 import workloads as wl


def _pair_scale(n, decades, seed):
    rng = np.random.default_rng(seed)
    x, _, _ = H.matched_reps([1] * n)
    E = n // 2
    s = 2.0 ** np.round(rng.uniform(-decades, decades, size=E) * np.log2(10))
    d = np.ones(n)
    d[x[:E]] = s
    d[x[E:]] = 1 / s
    return d


def test_balancing_undoes_pair_scaling_exactly():
    for n, decades in ((12, 4), (16, 8), (20, 12)):
        A = wl.complex_symmetric(n, seed=n)
        d = _pair_scale(n, decades, n)
        bal = tw.prepare_hafnian(d[:, None] * A * d[None, :])
        plain = tw.prepare_hafnian(A)
        assert np.array_equal(bal.A, plain.A) and np.array_equal(bal.reps, plain.reps)


def test_ordinary_and_integer_inputs_untouched():
    for A in (wl.complex_symmetric(16, seed=1), wl.real_nonneg(14, seed=2)):
        x, _, _ = H.matched_reps([1] * len(A))
        assert np.array_equal(tw.prepare_hafnian(A).A, A[np.ix_(x, x)])
    # integer inputs take the exact sieve: never rescaled, however spread
    A = wl.adjacency01(12, seed=3) * np.outer(np.arange(1, 13), np.arange(1, 13)) ** 3
    x, _, _ = H.matched_reps([1] * 12)
    assert np.array_equal(tw.prepare_hafnian(A).A, A[np.ix_(x, x)])


def test_pair_scaling_invariance_of_the_sieve():
    # the oracle (the reference algorithm) on pair-scaled prepared inputs: plain, loop, batch
    rng = np.random.default_rng(5)
    A = wl.complex_symmetric(10, seed=4)
    p = tw.prepare_hafnian(A)
    d = np.ldexp(1.0, rng.integers(-20, 20, size=5))
    d = np.concatenate([d, 1 / d])
    want = complex(oracle.haf_prepared(p.A, p.reps))
    got = complex(oracle.haf_prepared(d[:, None] * p.A * d[None, :], p.reps))
    assert abs(got - want) <= 1e-13 * abs(want)
    gamma = rng.normal(size=11) + 1j * rng.normal(size=11)
    B = wl.complex_symmetric(11, seed=6)
    q = tw.prepare_loop_hafnian(B, gamma, [1] * 11)  # odd: a self-loop vertex outside the pairs
    odd = complex(q.struct.oddloop[0], q.struct.oddloop[1])
    want = complex(oracle.loop_haf_prepared(q.A, q.D, q.reps, oddloop=odd, oddV=q.oddV))
    S = d[:, None] * q.A * d[None, :]
    got = complex(oracle.loop_haf_prepared(S, d * q.D, q.reps, oddloop=odd, oddV=d * q.oddV))
    assert abs(got - want) <= 1e-13 * abs(want)


def test_balanced_loop_values():
    # pair-scaled inputs through the public host preparation give the oracle's unscaled values
    rng = np.random.default_rng(9)
    n = 10
    A = wl.complex_symmetric(n, seed=7)
    gamma = (rng.normal(size=n) + 1j * rng.normal(size=n)) * 0.5
    d = _pair_scale(n, 6, 11)
    q = tw.prepare_loop_hafnian(d[:, None] * A * d[None, :], d * gamma, [1] * n)
    got = complex(oracle.loop_haf_prepared(q.A, q.D, q.reps))
    want = complex(oracle.loop_hafnian(A, gamma, [1] * n))
    assert abs(got - want) <= 1e-12 * abs(want)


def test_batch_balancing_leaves_the_batch_edges_alone():
    # a badly scaled fixed part: balancing scales only pairs from `first` on
    rng = np.random.default_rng(13)
    B, D, fixed, cutoff = wl.batch_loop_calls(count=1, seed=14, modes=7, cutoff=3)[0]
    inst = tw.prepare_loop_hafnian_batch(B, D, list(fixed), cutoff)
    n = inst.A.shape[0]
    E = n // 2
    first = 1 if inst.struct.kind == 3 else 2
    s = np.ldexp(1.0, rng.integers(-30, 30, size=E))
    s[:first] = 1.0
    d = np.concatenate([s, 1 / s])
    Ax, Dx = d[:, None] * inst.A * d[None, :], d * inst.D
    bal = H._pair_balance(Ax, Dx, first=first)
    assert bal is not None
    # the extra scale of vertex i from the diagonal: (d_i s_i)^2 / d_i^2
    diag = np.abs(np.diagonal(Ax)) > 0
    k = np.round(0.5 * np.log2(np.abs(np.diagonal(bal[0])[diag] / np.diagonal(Ax)[diag])))
    idx = np.flatnonzero(diag)
    fixed_ends = (idx >= first) & ((idx < E) | (idx >= E + first))
    assert not np.any(k[~fixed_ends]) and np.any(k[fixed_ends])
