"""Gaussian boson sampling by the chain rule over modes, on the GPU sieve.

Drop-ins for ``thewalrus.samples.generate_hafnian_sample``, ``hafnian_sample_state``,
``generate_torontonian_sample`` and ``torontonian_sample_state`` (thewalrus/samples.py:95-590),
and the graph forms ``hafnian_sample_graph`` / ``torontonian_sample_graph`` (:372-399, :591-621:
the pure Gaussian state that encodes an adjacency matrix at a given mean photon number, then the
state samplers),
the callers of ``loop_hafnian_batch`` and ``loop_hafnian_batch_gamma``.  For mode k = 1..M the
sampler evaluates the loop hafnians of the first k modes for every photon number 0..cutoff of
mode k (one batch sieve, the earlier modes fixed at their sampled counts), turns them into
conditional probabilities and draws mode k.

GPU-first structure: ``hafnian_sample_state`` advances all attempts in lockstep, so each mode
is ONE plan holding every attempt's batch instance (one persistent launch for all samples)
instead of one call per sample per mode.  Every attempt's random numbers are drawn up front, in
exactly the order the reference's sequential loop draws them (two ``normal(size=2M)`` vectors,
then one uniform per mode for ``np.random.choice``), and attempts that the reference would
discard (more than ``max_photons``, or the quirk ``pattern[-1] == cutoff`` on the re-ordered
pattern, samples.py:256-259) are discarded in the same order, so for a given ``np.random``
state the returned samples equal the reference's (up to draws that fall within ~1e-12 of a
cumulative-probability boundary) and the global random state advances identically.
The torontonian sampler stops drawing at the first click in a mode (data-dependent draw
count), so it runs attempts one after another; each mode's ``fanout`` displacement rows are
one plan.
"""
import numpy as np
from scipy.linalg import schur, sqrtm
from scipy.special import factorial

from ._hafnian import DEFAULT_PRECISION, prepare_loop_hafnian_batch, prepare_loop_hafnian_batch_gamma
from . import _native as nat

__all__ = [
    "williamson",
    "decompose_cov",
    "mu_to_alpha",
    "invert_permutation",
    "photon_means_order",
    "get_heterodyne_fanout",
    "generate_hafnian_sample",
    "hafnian_sample_state",
    "generate_torontonian_sample",
    "torontonian_sample_state",
    "adj_scaling",
    "gen_Qmat_from_graph",
    "Covmat",
    "hafnian_sample_graph",
    "torontonian_sample_graph",
]


def _sympmat(n):
    z, i = np.zeros((n, n)), np.identity(n)
    return np.block([[z, i], [-i, z]])


def williamson(V, rtol=1e-05, atol=1e-08):
    """Williamson normal form V = S diag(d, d) S^T, S symplectic (thewalrus/decompositions.py:50-102).

    Method (Houde et al., arXiv:2403.04596): with M = V^(1/2), the matrix M^-1 Omega M^-1 is real
    antisymmetric; its real Schur form is block diagonal with 2x2 blocks [[0, phi], [-phi, 0]]
    and orthogonal Schur vectors O.  Ordering each block so that its upper entry is positive and
    moving from (x1, p1, x2, p2, ...) to (x1, x2, ..., p1, p2, ...) gives d = 1/phi and
    S = M O diag(sqrt(phi), sqrt(phi)).  Returns (diag(d, d), S) like the reference.
    """
    n2, m2 = V.shape
    if n2 != m2:
        raise ValueError("The input matrix is not square")
    if not np.allclose(V, V.T, rtol=rtol, atol=atol):
        raise ValueError("The input matrix is not symmetric")
    if n2 % 2 != 0:
        raise ValueError("The input matrix must have an even number of rows/columns")
    n = n2 // 2
    if not np.all(np.linalg.eigvalsh(V) > 0):
        raise ValueError("Input matrix is not positive definite")
    root = np.real_if_close(sqrtm(V))
    root_inv = np.linalg.inv(root)
    blocks, vecs = schur(root_inv @ _sympmat(n) @ root_inv)
    cols = np.arange(2 * n)
    for i in range(n):
        if blocks[2 * i, 2 * i + 1] <= 0:  # make the block's upper entry positive
            cols[2 * i], cols[2 * i + 1] = cols[2 * i + 1], cols[2 * i]
    cols = np.concatenate([cols[0::2], cols[1::2]])
    phi = np.abs(np.diag(blocks, k=1)[::2])
    d = np.concatenate([1 / phi, 1 / phi])
    return np.diag(d), root @ vecs[:, cols] * np.sqrt(1 / d)


def decompose_cov(cov, hbar=2):
    """cov = T + W with T = (hbar/2) S S^T pure and W = sqrtW sqrtW^T >= 0 classical noise
    (thewalrus/samples.py:95-117)."""
    m = cov.shape[0] // 2
    D, S = williamson(cov)
    T = hbar / 2 * S @ S.T
    noise = D - hbar / 2 * np.eye(2 * m)
    noise[abs(noise) < 1e-10] = 0.0  # rounding can leave tiny negative values
    return T, S @ np.sqrt(noise)


def mu_to_alpha(mu, hbar=2):
    """Complex mean displacement of each mode (thewalrus/samples.py:120-137)."""
    M = len(mu) // 2
    return (mu[:M] + 1j * mu[M:]) / np.sqrt(2 * hbar)


def invert_permutation(p):
    """The inverse permutation s with s[p[i]] = i (thewalrus/samples.py:140-154)."""
    s = np.empty_like(p, dtype=int)
    s[p] = np.arange(p.size, dtype=int)
    return s


def _photon_number_means(mu, cov, hbar=2):
    """<n_j> = (mu_x^2 + mu_p^2 + cov_xx + cov_pp - hbar) / (2 hbar)
    (thewalrus/quantum/means_and_variances.py:31-66)."""
    N = len(mu) // 2
    j = np.arange(N)
    return (mu[j] ** 2 + mu[j + N] ** 2 + cov[j, j] + cov[j + N, j + N] - hbar) / (2 * hbar)


def photon_means_order(mu, cov):
    """Modes sorted by increasing mean photon number, ties by index (thewalrus/samples.py:157-175;
    the means use hbar = 2 whatever the sampler's hbar, as the reference does)."""
    means = _photon_number_means(mu, cov)
    return np.asarray([x for _, x in sorted(zip(means, range(len(means))))])


def get_heterodyne_fanout(alpha, fanout):
    """Per mode: the coherent amplitude in channel 0 and fresh complex normals in channels
    1..fanout-1, mixed by the unitary DFT (thewalrus/samples.py:178-201)."""
    M = len(alpha)
    out = np.zeros((M, fanout), dtype=np.complex128)
    for j in range(M):
        chan = np.zeros(fanout, dtype=np.complex128)
        chan[0] = alpha[j]
        chan[1:] = np.random.normal(size=fanout - 1) + 1j * np.random.normal(size=fanout - 1)
        out[j, :] = np.fft.fft(chan, norm="ortho")
    return out


def _husimi_a(cov):
    """A = X (I - Q^-1)^* of the Gaussian state with covariance ``cov`` (hbar = 2), the Husimi
    matrix Q as in thewalrus/quantum/conversions.py:70-150."""
    N = len(cov) // 2
    I = np.identity(N)
    x, xp, p = cov[:N, :N], cov[:N, N:], cov[N:, N:]
    adag_a = (x + p + 1j * (xp - xp.T) - 2 * I) / 4
    a_a = (x - p + 1j * (xp + xp.T)) / 4
    Q = np.block([[adag_a, a_a.conj()], [a_a, adag_a.conj()]]) + np.identity(2 * N)
    W = (np.identity(2 * N) - np.linalg.inv(Q)).conj()
    return np.block([[W[N:, :N], W[N:, N:]], [W[:N, :N], W[:N, N:]]])  # X @ W


def _check_cov(cov):
    if not isinstance(cov, np.ndarray):
        raise TypeError("Covariance matrix must be a NumPy array.")
    if cov.shape[0] != cov.shape[1]:
        raise ValueError("Covariance matrix must be square.")
    if np.isnan(cov).any():
        raise ValueError("Covariance matrix must not contain NaNs.")


def _choose(probs, u):
    """``np.random.choice(arange(len(probs)), p=probs)`` with its uniform draw ``u`` given: the
    same validation and cumulative-sum search as NumPy's legacy generator."""
    p = np.asarray(probs, dtype=np.float64)
    if np.isnan(p).any():
        raise ValueError("probabilities contain NaN")
    if (p < 0).any():
        raise ValueError("probabilities are not non-negative")
    if abs(p.sum() - 1.0) > np.sqrt(np.finfo(np.float64).eps):
        raise ValueError("probabilities do not sum to 1")
    cdf = p.cumsum()
    cdf /= cdf[-1]
    return int(cdf.searchsorted(u, side="right"))


class _Chain:
    """Per-state data shared by every attempt: mode order, pure part of the covariance, B."""

    def __init__(self, cov, mean, hbar):
        M = cov.shape[0] // 2
        mu = np.zeros(2 * M) if mean is None else np.asarray(mean, dtype=np.float64)
        order = photon_means_order(mu, cov)
        self.order_inv = invert_permutation(order)
        oo = np.concatenate((order, order + M))
        self.mu = mu[oo]
        cov = cov[np.ix_(oo, oo)]
        T, self.sqrtW = decompose_cov(cov, hbar=hbar)
        self.chol_T_I = np.linalg.cholesky(T + np.eye(2 * M))
        self.B = _husimi_a(T)[:M, :M]
        self.M, self.hbar = M, hbar

    def attempt_draws(self):
        """The random numbers one attempt of the reference consumes, in its order."""
        n_pure = np.random.normal(size=2 * self.M)
        n_het = np.random.normal(size=2 * self.M)
        return n_pure, n_het, np.random.random_sample(self.M)

    def start(self, n_pure, n_het):
        pure_mu = self.mu + self.sqrtW @ n_pure
        pure_alpha = mu_to_alpha(pure_mu, hbar=self.hbar)
        het_alpha = mu_to_alpha(pure_mu + self.chol_T_I @ n_het, hbar=self.hbar)
        return het_alpha, pure_alpha.conj() + self.B @ (het_alpha - pure_alpha)


def _hafnian_attempts(chain, count, cutoff, max_photons, precision):
    """``count`` attempts of generate_hafnian_sample in lockstep: one plan per mode for all."""
    M, B = chain.M, chain.B
    draws = [chain.attempt_draws() for _ in range(count)]
    starts = [chain.start(n_pure, n_het) for n_pure, n_het, _ in draws]
    het = [s[0] for s in starts]
    gam = [s[1].copy() for s in starts]
    det = np.zeros((count, M), dtype=int)
    fac = factorial(np.arange(cutoff + 1))
    for mode in range(M):
        m = mode + 1
        insts = []
        for j in range(count):
            gam[j] -= het[j][mode] * B[:, mode]
            insts.append(prepare_loop_hafnian_batch(B[:m, :m], gam[j][:m], det[j, :mode], cutoff))
        lhafs = nat.run(insts, precision).reshape(count, cutoff + 1)
        for j in range(count):
            probs = (lhafs[j] * lhafs[j].conj()).real / fac
            probs /= probs.sum()
            det[j, mode] = _choose(probs, draws[j][2][mode])
    out = []
    for j in range(count):
        pattern = det[j][chain.order_inv]
        if pattern[-1] == cutoff or pattern.sum() > max_photons:
            out.append(-1)
        else:
            out.append(list(pattern))
    return out


def generate_hafnian_sample(cov, mean=None, hbar=2, cutoff=12, max_photons=8, precision=None):
    """One photon-number sample of the Gaussian state, or -1 when it is rejected
    (thewalrus/samples.py:204-261)."""
    chain = _Chain(cov, mean, hbar)
    return _hafnian_attempts(chain, 1, cutoff, max_photons, precision or DEFAULT_PRECISION)[0]


def hafnian_sample_state(cov, samples, mean=None, hbar=2, cutoff=5, max_photons=30, parallel=False,
                         precision=None):
    """``samples`` photon-number samples (thewalrus/samples.py:264-369).  ``parallel`` is accepted
    for signature compatibility; attempts always run in lockstep on the GPU."""
    _check_cov(cov)
    chain = _Chain(cov, mean, hbar)
    got = []
    while len(got) < samples:
        # every attempt of this pass is one the sequential reference would also make
        for res in _hafnian_attempts(chain, samples - len(got), cutoff, max_photons,
                                     precision or DEFAULT_PRECISION):
            if res != -1:
                got.append(res)
    return np.vstack(got)


def generate_torontonian_sample(cov, mu=None, hbar=2, max_photons=30, fanout=10, cutoff=1, precision=None):
    """One threshold-detector (click) sample, or -1 (thewalrus/samples.py:407-481): each mode is
    split over ``fanout`` channels; per mode one ``loop_hafnian_batch_gamma`` plan covers all
    channels, and channels are drawn in order until the first click."""
    precision = precision or DEFAULT_PRECISION
    M = cov.shape[0] // 2
    mu = np.zeros(2 * M) if mu is None else np.asarray(mu, dtype=np.float64)
    order = photon_means_order(mu, cov)
    order_inv = invert_permutation(order)
    oo = np.concatenate((order, order + M))
    mu = mu[oo]
    cov = cov[np.ix_(oo, oo)]
    T, sqrtW = decompose_cov(cov, hbar=hbar)
    chol_T_I = np.linalg.cholesky(T + np.eye(2 * M))
    B = _husimi_a(T)[:M, :M] / fanout
    fac = factorial(np.arange(cutoff + 1))
    det_pattern = np.zeros(M, dtype=int)
    click_pattern = np.zeros(M, dtype=np.int8)
    pure_mu = mu + sqrtW @ np.random.normal(size=2 * M)
    pure_alpha = mu_to_alpha(pure_mu, hbar=hbar)
    het_alpha = mu_to_alpha(pure_mu + chol_T_I @ np.random.normal(size=2 * M), hbar=hbar)
    het_fan = get_heterodyne_fanout(het_alpha, fanout)
    gamma = pure_alpha.conj() / np.sqrt(fanout) + B @ (het_fan.sum(axis=1) - np.sqrt(fanout) * pure_alpha)
    gfan = np.zeros((fanout, M), dtype=np.complex128)
    for mode in range(M):
        gfan[0, :] = gamma - het_fan[mode, 0] * B[:, mode]
        for k in range(1, fanout):
            gfan[k, :] = gfan[k - 1, :] - het_fan[mode, k] * B[:, mode]
        insts = prepare_loop_hafnian_batch_gamma(B[: mode + 1, : mode + 1], gfan[:, : mode + 1],
                                                 det_pattern[:mode], cutoff)
        lhafs = nat.run(insts, precision).reshape(fanout, cutoff + 1)
        probs = (lhafs * lhafs.conj()).real / fac
        for k in range(fanout):
            gamma = gfan[k, :]
            outcome = _choose(probs[k, :] / probs[k, :].sum(), np.random.random_sample())
            det_pattern[mode] += outcome
            if outcome > 0:
                click_pattern[mode] = 1
                break
        if sum(click_pattern[order_inv]) > max_photons:
            return -1
    return list(click_pattern[order_inv])


def torontonian_sample_state(cov, samples, mu=None, hbar=2, max_photons=30, fanout=10, cutoff=1,
                             parallel=False, precision=None):
    """``samples`` click samples (thewalrus/samples.py:484-588); ``parallel`` is accepted for
    signature compatibility."""
    _check_cov(cov)
    if mu is None:
        mu = np.zeros(cov.shape[0], dtype=np.float64)
    got = []
    while len(got) < samples:
        res = generate_torontonian_sample(cov, mu, hbar=hbar, max_photons=max_photons, fanout=fanout,
                                          cutoff=cutoff, precision=precision)
        if res != -1:
            got.append(res)
    return np.vstack(got)


# ---------------------------------------------------------------------------------------------
# Graph states (thewalrus/quantum/adjacency_matrices.py:90-177, conversions.py:99-121)


def adj_scaling(A, n_mean):
    """The factor x for which the pure Gaussian state encoding x A has mean photon number
    ``n_mean``: sum_i (x s_i)^2 / (1 - (x s_i)^2) = n_mean over the singular values s_i of A,
    solved by bracketed root finding on (0, 1 / s_max) (adjacency_matrices.py:90-152)."""
    from scipy.optimize import brentq

    eps = 1e-10
    s = np.linalg.svd(np.asarray(A), compute_uv=False)
    if 1000 * eps >= s[0]:
        raise ValueError("The singular values of the matrix A are too small.")

    def excess(x):
        v = (x * s) ** 2
        return float(np.sum(v / (1.0 - v))) - n_mean

    return brentq(excess, 0.0, 1.0 / (eps + s[0]), xtol=2e-12, rtol=4 * np.finfo(float).eps, maxiter=200)


def gen_Qmat_from_graph(A, n_mean):
    """Husimi Q matrix of the pure state encoding the adjacency matrix A at mean photon number
    ``n_mean``: Q = (I - X (x A (+) conj(x A)))^-1 with X the mode-swap block matrix
    (adjacency_matrices.py:155-177)."""
    A = np.asarray(A)
    n, m = A.shape
    if n != m:
        raise ValueError("Matrix must be square.")
    Asc = adj_scaling(A, n_mean) * A
    Z = np.zeros_like(Asc)
    B = np.block([[Asc, Z], [Z, Asc.conj()]])
    idn = np.identity(n)
    X = np.block([[0 * idn, idn], [idn, 0 * idn]])
    return np.linalg.inv(np.identity(2 * n) - X @ B)


def Covmat(Q, hbar=2):
    """xp-ordered Wigner covariance matrix of the state with Husimi matrix Q
    (conversions.py:99-121)."""
    n = len(Q) // 2
    idn = np.identity(n)
    N = Q[0:n, 0:n] - idn
    M = Q[n:2 * n, 0:n]
    c11 = 2 * (N.real + M.real) + idn
    c22 = 2 * (N.real - M.real) + idn
    c12 = 2 * (M.imag + N.imag)
    return (hbar / 2) * np.block([[c11, c12], [c12.T, c22]])


def hafnian_sample_graph(A, n_mean, samples=1, cutoff=5, max_photons=30, parallel=False, precision=None):
    """Photon-number samples of the pure state encoding the adjacency matrix A at mean photon
    number ``n_mean`` (thewalrus/samples.py:372-399)."""
    cov = Covmat(gen_Qmat_from_graph(A, n_mean), hbar=2)
    return hafnian_sample_state(cov, samples, mean=None, hbar=2, cutoff=cutoff, max_photons=max_photons,
                                parallel=parallel, precision=precision)


def torontonian_sample_graph(A, n_mean, samples=1, max_photons=30, fanout=10, cutoff=1, parallel=False,
                             precision=None):
    """Click samples of the pure state encoding the adjacency matrix A at mean photon number
    ``n_mean`` (thewalrus/samples.py:591-621)."""
    cov = Covmat(gen_Qmat_from_graph(A, n_mean), hbar=2)
    return torontonian_sample_state(cov, samples, hbar=2, max_photons=max_photons, fanout=fanout, cutoff=cutoff,
                                    parallel=parallel, precision=precision)
