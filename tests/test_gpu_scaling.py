"""Badly scaled inputs on the GPU.

* Pair scalings: vertex e of the prepared matrix scaled by s_e and its partner E + e by 1/s_e
  (the original matrix A -> diag(d) A diag(d) with d_i d_partner(i) = 1) leave the hafnian and
  every sieve term unchanged (each term matrix undergoes a diagonal similarity), yet spread the
  entries of one column over up to s^2 = 1e16 (d over [1e-8, 1e8]).  The reference's
  matrix-power traces are indifferent to such a similarity; a pivoted Hessenberg reduction is
  not.  The host undoes them by pair balancing before the sieve: results must equal haf(A) at
  1e-10 (FP64) for d spread over [1e-4, 1e4] and [1e-8, 1e8].
* General diagonal scalings diag(d) A diag(d): the hafnian scales by prod(d), but the sieve
  sum's terms carry products of the large d's that cancel only in the sum -- for n = 16 and d
  over [1e-4, 1e4] the _Float128 oracle's own sum was off from prod(d) haf(A) by 0.5 to 1e25
  relative on three seeds, so no sieve can be checked on the whole sum there.  What the
  elimination's pivoting and deflation decide is each term, so each term (a one-term shard) is
  checked against the oracle's term in _Float128 at 1e-10.
"""
import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _hafnian as H
from thewalrus_gb300 import _native as nat
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    return abs(complex(a) - complex(b)) / abs(complex(b))


def pair_scaling(n, decades, seed):
    """d over the original indices with d_i d_partner(i) = 1 for the sieve's pairing, log-uniform
    over [10^-decades, 10^decades] rounded to powers of two."""
    rng = np.random.default_rng(seed)
    x, _, _ = H.matched_reps([1] * n)
    E = n // 2
    s = 2.0 ** np.round(rng.uniform(-decades, decades, size=E) * np.log2(10))
    d = np.ones(n)
    d[x[:E]] = s
    d[x[E:]] = 1 / s
    return d, rng


@pytest.mark.parametrize("decades", [4, 8])
@pytest.mark.parametrize("n,kind", [(16, "complex"), (20, "signed"), (24, "complex")])
def test_pair_scaled_hafnian(n, kind, decades):
    A = (wl.complex_symmetric if kind == "complex" else wl.real_signed)(n, seed=n + decades)
    d, _ = pair_scaling(n, decades, 1000 * n + decades)
    S = d[:, None] * A * d[None, :]
    assert np.max(np.abs(S)) / np.min(np.abs(S)[np.abs(S) > 0]) > 10.0 ** decades
    # prod(d) = 1; the unscaled sum is well conditioned (cond ~1e2-1e4), so the oracle's double
    # arithmetic is good to ~1e-13
    want = complex(oracle.hafnian(A, precision="double"))
    assert rel(tw.hafnian(S, precision="fp64"), want) < RTOL
    assert rel(tw.hafnian(S, precision="df"), want) < 1e-8


@pytest.mark.parametrize("decades", [4, 8])
@pytest.mark.parametrize("n", [16, 21])
def test_pair_scaled_loop_hafnian(n, decades):
    # lhaf(D A D, D gamma) = prod(d) lhaf(A, gamma); the loop weights scale once, A's diagonal
    # (unused by matchings) twice
    A = wl.complex_symmetric(n, seed=n + decades)
    d, rng = pair_scaling(n, decades, 2000 * n + decades)
    gamma = (rng.normal(size=n) + 1j * rng.normal(size=n)) * 0.5
    want = complex(oracle.hafnian_repeated(A, [1] * n, mu=gamma, loop=True, precision="double"))
    S = d[:, None] * A * d[None, :]
    got = tw.hafnian_repeated(S, [1] * n, mu=d * gamma, loop=True, precision="fp64")
    assert rel(got, want * np.prod(d)) < RTOL


@pytest.mark.parametrize("decades", [4, 8])
@pytest.mark.parametrize("n,kind", [(16, "complex"), (20, "signed"), (24, "complex")])
def test_general_scaling_terms(n, kind, decades):
    A = (wl.complex_symmetric if kind == "complex" else wl.real_signed)(n, seed=n + decades)
    rng = np.random.default_rng(3000 * n + decades)
    d = 2.0 ** np.round(rng.uniform(-decades, decades, size=n) * np.log2(10))
    inst = tw.prepare_hafnian(d[:, None] * A * d[None, :])
    T = inst.terms()
    ts = sorted({0, 1, T - 1} | {int(t) for t in rng.integers(0, T, size=13)})
    got = nat.run([inst.shard(t, t + 1) for t in ts], "fp64")
    scale = 2.0 ** -(n // 2 - 1)
    for t, g in zip(ts, got):
        # term t of the binary reflected Gray order is term t ^ (t >> 1) of the mixed-radix order
        m = t ^ (t >> 1)
        want = complex(oracle.haf_term_range(inst.A, inst.reps, m, m + 1, precision="quad")) * scale
        assert rel(g, want) < RTOL, (t, g, want)


@pytest.mark.parametrize("n", [20, 24, 28, 32])
def test_small_entry_gaussian_state_loops(n):
    """Loop hafnians of a 64-mode Gaussian state's B (entries ~0.1, so every pivot is below 1):
    in the normalised elimination the subdiagonal candidates shrink by the product of the
    pivots against the rows above (1e-15 after 22 columns), which a deflation test made in that
    frame took for rounding residues -- relative errors of 0.03 at n = 20 up to 760 at n = 28
    before the test moved to the classic frame.  These sums are well conditioned (sum|term| /
    |sum| ~ 1e2..1e3), so the oracle's double arithmetic (the reference algorithm) is good to
    ~1e-13 and the bar is 1e-10."""
    from thewalrus_gb300.serving import GaussianState
    st = GaussianState.synthetic(modes=64, seed=3)
    rng = np.random.default_rng(n)
    modes = np.sort(rng.choice(64, size=n, replace=False))
    B, gamma = st.B[np.ix_(modes, modes)], st.gamma[modes]
    want = complex(oracle.hafnian_repeated(B, [1] * n, mu=gamma, loop=True, precision="double"))
    assert rel(tw.hafnian_repeated(B, [1] * n, mu=gamma, loop=True), want) < RTOL
    assert rel(tw.hafnian_repeated(B, [1] * n, mu=gamma, loop=True, precision="dd"), want) < RTOL
    want = complex(oracle.hafnian(B, precision="double"))
    assert rel(tw.hafnian(B), want) < RTOL


def test_batch_kinds_invariant_under_pair_scaling():
    """loop_hafnian_batch instances (batch edge first, the odd mode's edge second for odd
    cutoffs) give the same outputs after a pair scaling of their fixed edges -- what the host's
    pair balancing relies on for them."""
    rng = np.random.default_rng(15)
    for seed, cutoff in ((16, 4), (17, 5)):
        B, D, fixed, _ = wl.batch_loop_calls(count=1, seed=seed, modes=7, cutoff=cutoff)[0]
        inst = tw.prepare_loop_hafnian_batch(B, D, list(fixed), cutoff)
        want = nat.run([inst], "fp64")
        n = inst.A.shape[0]
        E = n // 2
        first = 1 if inst.struct.kind == nat.WG_KIND_BATCH_EVEN else 2
        s = np.ldexp(1.0, rng.integers(-20, 20, size=E))
        s[:first] = 1.0
        d = np.concatenate([s, 1 / s])
        scaled = nat.Instance(inst.struct.kind, d[:, None] * inst.A * d[None, :], inst.reps, D=d * inst.D,
                              batch_max=inst.struct.batch_max, cutoff=inst.struct.cutoff)
        got = nat.run([scaled], "fp64")
        assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want)), (seed, cutoff)
