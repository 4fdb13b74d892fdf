"""Seeded synthetic workloads for the hafnian sieve.

Every generator is deterministic in its seed and uses NumPy's ``default_rng``.
The shapes and value distributions follow the benchmark configurations of the
hafnian / loop-hafnian path:

* ``complex_symmetric(n, seed)``: A = (G + G^T)/2 with Re G, Im G ~ N(0, 1/2) iid
  (the 24x24 and 40x40 plain-hafnian workloads).
* ``real_nonneg(n, seed)``: A = |G| + |G|^T with G ~ N(0, 1).
* ``real_signed(n, seed)``: A = (G + G^T)/2 with G ~ N(0, 1).
* ``adjacency01(n, seed, p)``: symmetric 0/1 adjacency matrix, zero diagonal, edge probability p.
* ``gaussian_state_loop(modes, seed, ...)``: reduced loop-hafnian input of a synthetic Gaussian
  state: Haar unitary U, squeezing r_i ~ U(0.3, 0.8), B = U diag(tanh r) U^T, A = B (+) B*,
  diagonal gamma ~ CN(0, 0.1) and a photon pattern with at most ``max_rep`` photons per mode.
* ``gaussian_state_cov(modes, seed, ...)``: covariance and means of a lossy squeezed, displaced
  state behind a Haar interferometer (the samplers' input).

Haar sampling follows the QR-with-phase-correction recipe that
``thewalrus/random.py:115-134`` (``random_interferometer``) uses.
"""
import numpy as np

__all__ = [
    "complex_symmetric",
    "real_nonneg",
    "real_signed",
    "adjacency01",
    "haar_unitary",
    "gaussian_state_loop",
    "gaussian_state_cov",
    "photon_pattern",
    "batch_instances",
    "batch_loop_calls",
]


def complex_symmetric(n, seed=0):
    """A = (G + G^T)/2, Re G and Im G iid N(0, 1/2)."""
    rng = np.random.default_rng(seed)
    s = np.sqrt(0.5)
    G = rng.normal(scale=s, size=(n, n)) + 1j * rng.normal(scale=s, size=(n, n))
    return (G + G.T) / 2


def real_nonneg(n, seed=0):
    """A = |G| + |G|^T with G iid N(0, 1): symmetric, entrywise non-negative."""
    rng = np.random.default_rng(seed)
    G = np.abs(rng.normal(size=(n, n)))
    return G + G.T


def real_signed(n, seed=0):
    """A = (G + G^T)/2 with G iid N(0, 1)."""
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, n))
    return (G + G.T) / 2


def adjacency01(n, seed=0, p=0.5):
    """Symmetric 0/1 adjacency matrix (zero diagonal), each edge present with probability p."""
    rng = np.random.default_rng(seed)
    U = np.triu((rng.random((n, n)) < p).astype(np.float64), 1)
    return U + U.T


def haar_unitary(modes, rng):
    """Haar-random unitary: QR of a complex Ginibre matrix with the phases of diag(R) removed."""
    Z = (rng.normal(size=(modes, modes)) + 1j * rng.normal(size=(modes, modes))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    d = np.diagonal(R)
    return Q * (d / np.abs(d))


def photon_pattern(modes, total, max_rep, rng):
    """Random photon pattern over ``modes`` with ``sum == total`` and entries <= ``max_rep``."""
    if total > modes * max_rep:
        raise ValueError("pattern cannot hold that many photons")
    pat = np.zeros(modes, dtype=np.int64)
    placed = 0
    while placed < total:
        i = rng.integers(modes)
        if pat[i] < max_rep:
            pat[i] += 1
            placed += 1
    return pat


def gaussian_state_loop(modes=20, seed=1, photons=40, max_rep=3):
    """Reduced loop-hafnian input of a synthetic pure Gaussian state.

    Returns ``(A, gamma, rpt)`` with A = B (+) B* (2*modes square, complex128) whose diagonal is
    replaced by gamma, and ``rpt`` the repetition vector over the 2*modes indices: the photon
    pattern ``nvec`` over the modes (``sum(nvec) == photons // 2``) repeated on both halves, so
    ``sum(rpt) == photons`` and every entry is at most ``max_rep``.
    """
    rng = np.random.default_rng(seed)
    U = haar_unitary(modes, rng)
    r = rng.uniform(0.3, 0.8, size=modes)
    B = U @ np.diag(np.tanh(r)) @ U.T
    Z = np.zeros_like(B)
    A = np.block([[B, Z], [Z, B.conj()]])
    gamma = (rng.normal(size=2 * modes) + 1j * rng.normal(size=2 * modes)) * np.sqrt(0.1 / 2)
    np.fill_diagonal(A, gamma)
    nvec = photon_pattern(modes, photons // 2, max_rep, rng)
    rpt = np.concatenate([nvec, nvec])
    return A, gamma, rpt


def gaussian_state_cov(modes=12, seed=21, r_range=(0.5, 0.9), transmission=0.8, disp=0.3):
    """xp-covariance (hbar = 2) and means of a synthetic lossy GBS state: single-mode squeezers
    r_i ~ U(r_range) (diag(e^-r, e^r)), a Haar interferometer ([[Re U, -Im U], [Im U, Re U]]),
    uniform transmission (cov -> t cov + (1 - t) I) and means ~ N(0, disp^2)."""
    rng = np.random.default_rng(seed)
    U = haar_unitary(modes, rng)
    r = rng.uniform(*r_range, size=modes)
    Sq = np.diag(np.concatenate([np.exp(-r), np.exp(r)]))
    O = np.block([[U.real, -U.imag], [U.imag, U.real]])
    S = O @ Sq
    cov = transmission * (S @ S.T) + (1 - transmission) * np.identity(2 * modes)
    mean = rng.normal(size=2 * modes) * disp
    return cov, mean


def batch_instances(count=4096, seed=2, n_min=8, n_max=40):
    """Independent plain-hafnian instances of uneven even size.

    Even n drawn uniformly from {n_min, ..., n_max}; the first half are real non-negative
    (``|G| + |G|^T``), the second half complex as ``complex_symmetric``.
    """
    rng = np.random.default_rng(seed)
    sizes = 2 * rng.integers(n_min // 2, n_max // 2 + 1, size=count)
    out = []
    for i, n in enumerate(sizes):
        s = int(rng.integers(1 << 31))
        out.append(real_nonneg(int(n), s) if i < count // 2 else complex_symmetric(int(n), s))
    return out


def batch_loop_calls(count=16, seed=3, modes=12, cutoff=6, max_fixed=2):
    """Arguments of ``loop_hafnian_batch`` calls on synthetic 12-mode Gaussian states.

    Each call is ``(A, D, fixed_reps, cutoff)`` with A the reduced (modes x modes) matrix of a
    pure Gaussian state (B = U diag(tanh r) U^T), D its displacement vector and ``fixed_reps``
    the photon numbers of the first ``modes - 1`` modes.
    """
    rng = np.random.default_rng(seed)
    calls = []
    for _ in range(count):
        U = haar_unitary(modes, rng)
        r = rng.uniform(0.3, 0.8, size=modes)
        B = U @ np.diag(np.tanh(r)) @ U.T
        D = (rng.normal(size=modes) + 1j * rng.normal(size=modes)) * np.sqrt(0.1 / 2)
        fixed = rng.integers(0, max_fixed + 1, size=modes - 1)
        calls.append((B, D, fixed, cutoff))
    return calls
