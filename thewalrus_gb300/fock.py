"""Fock-space elements of Gaussian states evaluated on the GPU sieve.

Drop-ins for ``thewalrus.quantum``'s ``pure_state_amplitude`` (fock_tensors.py:45-98),
``density_matrix_element`` (:191-232) and the conversions they rest on (``Xmat``, ``Qmat``,
``Amat``, ``complex_to_real_displacements``: conversions.py:46-170; ``_prefactor``:
fock_tensors.py:566-581).  An element is a (loop) hafnian of the state's A matrix (B = A[:N, :N]^*
for a pure state) with the rows of the requested pattern repeated, times a Gaussian prefactor:

    <i|psi>   = lhaf(B_i, gamma_i) e^{-(|alpha|^2 - alpha^* B alpha^*)/2} / sqrt(i! sqrt(det Q))
    <i|rho|j> = lhaf(A_{i+j}, gamma_{i+j}) e^{-beta Q^-1 beta^*/2} / sqrt(det Q) / sqrt((i+j)!)

with gamma = alpha - B alpha^* (pure) or beta^* - A beta (mixed), and no loops when the state is
not displaced.  The conversions run on the host (NumPy); the hafnian is one ``hafnian_repeated``
call, i.e. the sieve on the GPU.  ``_pure_problem`` / ``_dm_problem`` return the (matrix,
repetitions, loop weights, scale) of an element, so the host side can be checked apart from the
sieve.
"""
import numpy as np

from ._hafnian import hafnian_repeated

__all__ = ["Xmat", "Qmat", "Amat", "complex_to_real_displacements", "is_valid_cov", "is_pure_cov",
           "pure_state_amplitude", "density_matrix_element"]


def Xmat(N):
    """The 2N x 2N mode-swap matrix [[0, I], [I, 0]]."""
    idn = np.identity(N)
    zero = np.zeros_like(idn)
    return np.block([[zero, idn], [idn, zero]])


def Qmat(cov, hbar=2):
    """Husimi Q matrix of the state with xp-ordered covariance ``cov``: the blocks <a_i^+ a_j> and
    <a_i a_j> of the normal-ordered moments, plus the identity (conversions.py:69-96)."""
    cov = np.asarray(cov)
    N = len(cov) // 2
    x = cov[:N, :N] * 2 / hbar
    xp = cov[:N, N:] * 2 / hbar
    p = cov[N:, N:] * 2 / hbar
    adag_a = (x + p + 1j * (xp - xp.T) - 2 * np.identity(N)) / 4
    a_a = (x - p + 1j * (xp + xp.T)) / 4
    return np.block([[adag_a, a_a.conj()], [a_a, adag_a.conj()]]) + np.identity(2 * N)


def Amat(cov, hbar=2, cov_is_qmat=False):
    """Hamilton's A = X (I - Q^-1)^* (conversions.py:124-150)."""
    Q = np.asarray(cov) if cov_is_qmat else Qmat(cov, hbar=hbar)
    N = len(Q) // 2
    return Xmat(N) @ (np.identity(2 * N) - np.linalg.inv(Q)).conj()


def complex_to_real_displacements(mu, hbar=2):
    """(<a_1> .. <a_N>, <a_1^+> .. <a_N^+>) from the xp means (conversions.py:153-170)."""
    mu = np.asarray(mu)
    N = len(mu) // 2
    alpha = (mu[:N] + 1j * mu[N:]) / np.sqrt(2 * hbar)
    return np.concatenate([alpha, alpha.conj()])


def is_valid_cov(cov, hbar=2, rtol=1e-05, atol=1e-08):
    """Square, even, symmetric and obeying the uncertainty relation V + i hbar Omega / 2 >= 0."""
    cov = np.asarray(cov)
    n, m = cov.shape
    if n != m or n % 2:
        return False
    if not np.allclose(cov, cov.T, rtol=rtol, atol=atol):
        return False
    N = n // 2
    omega = np.block([[np.zeros((N, N)), np.identity(N)], [-np.identity(N), np.zeros((N, N))]])
    vals = np.linalg.eigvalsh(cov + 0.5j * hbar * omega)
    vals[np.abs(vals) < atol] = 0.0
    return bool(np.all(vals >= 0))


def is_pure_cov(cov, hbar=2, rtol=1e-05, atol=1e-08):
    """Valid and of purity 1 / sqrt(det(2 V / hbar)) = 1."""
    if not is_valid_cov(cov, hbar=hbar, rtol=rtol, atol=atol):
        return False
    purity = 1 / np.sqrt(np.linalg.det(2 * np.asarray(cov) / hbar))
    return bool(np.allclose(purity, 1.0, rtol=rtol, atol=atol))


def _prefactor(mu, cov, hbar=2):
    """e^{-beta Q^-1 beta^* / 2} / sqrt(det Q) (fock_tensors.py:566-581)."""
    Q = Qmat(cov, hbar=hbar)
    beta = complex_to_real_displacements(mu, hbar=hbar)
    return np.exp(-0.5 * beta @ np.linalg.inv(Q) @ beta.conj()) / np.sqrt(np.linalg.det(Q))


def _fact(rpt):
    out = 1.0
    for k in rpt:
        for v in range(2, int(k) + 1):
            out *= v
    return out


def _pure_problem(mu, cov, i, include_prefactor=True, tol=1e-10, hbar=2, check_purity=True):
    """(B, repetitions, loop weights or None, scale) of <i|psi>."""
    cov = np.asarray(cov)
    if check_purity and not is_pure_cov(cov, hbar=hbar, rtol=1e-05, atol=1e-08):
        raise ValueError("The covariance matrix does not correspond to a pure state")
    rpt = [int(k) for k in i]
    N = len(cov) // 2
    beta = complex_to_real_displacements(mu, hbar=hbar)
    Q = Qmat(cov, hbar=hbar)
    B = Amat(Q, cov_is_qmat=True)[:N, :N].conj()
    alpha = beta[:N]
    gamma = None if np.linalg.norm(alpha) < tol else alpha - B @ alpha.conj()
    scale = 1.0 / np.sqrt(_fact(rpt) * np.sqrt(np.linalg.det(Q)))
    if include_prefactor:
        scale = scale * np.exp(-0.5 * (np.linalg.norm(alpha) ** 2 - alpha.conj() @ B @ alpha.conj()))
    return B, rpt, gamma, scale


def _dm_problem(mu, cov, i, j, include_prefactor=True, tol=1e-10, hbar=2):
    """(A, repetitions, loop weights or None, scale) of <i|rho|j>."""
    rpt = [int(k) for k in list(i) + list(j)]
    beta = complex_to_real_displacements(mu, hbar=hbar)
    A = Amat(cov, hbar=hbar)
    gamma = None if np.linalg.norm(beta) < tol else beta.conj() - A @ beta
    scale = 1.0 / np.sqrt(_fact(rpt))
    if include_prefactor:
        scale = scale * _prefactor(mu, cov, hbar=hbar)
    return A, rpt, gamma, scale


def _evaluate(M, rpt, gamma, precision):
    if sum(rpt) == 0:
        return 1.0 + 0j
    if gamma is None:
        return complex(hafnian_repeated(M, rpt, precision=precision))
    return complex(hafnian_repeated(M, rpt, mu=gamma, loop=True, precision=precision))


def pure_state_amplitude(mu, cov, i, include_prefactor=True, tol=1e-10, hbar=2, check_purity=True, precision=None):
    """<i|psi> of the pure Gaussian state (mu, cov) (fock_tensors.py:45-98)."""
    B, rpt, gamma, scale = _pure_problem(mu, cov, i, include_prefactor, tol, hbar, check_purity)
    return _evaluate(B, rpt, gamma, precision) * scale


def density_matrix_element(mu, cov, i, j, include_prefactor=True, tol=1e-10, hbar=2, precision=None):
    """<i|rho|j> of the Gaussian state (mu, cov) (fock_tensors.py:191-232)."""
    A, rpt, gamma, scale = _dm_problem(mu, cov, i, j, include_prefactor, tol, hbar)
    return _evaluate(A, rpt, gamma, precision) * scale
