"""Host side of the Fock-space elements (thewalrus_gb300.fock): the conversions, the element's
matrix, repetitions, loop weights and Gaussian scale, with the hafnian taken by the oracle on the
CPU, against pure_state_amplitude / density_matrix_element values produced by the reference."""
import numpy as np
import pytest

import oracle
from thewalrus_gb300 import fock


def _oracle_element(M, rpt, gamma, scale):
    if sum(rpt) == 0:
        return scale
    if gamma is None:
        return complex(oracle.hafnian_repeated(M, rpt)) * scale
    return complex(oracle.hafnian_repeated(M, rpt, mu=gamma, loop=True)) * scale


def test_pure_state_amplitudes_vs_reference(golden):
    for c in golden["pure"]:
        parts = fock._pure_problem(c["mu"], c["cov"], list(c["pattern"]))
        got = _oracle_element(*parts)
        want = complex(c["out"])
        # elements that vanish by symmetry come out as rounding noise (~1e-18) on both sides
        assert abs(got - want) <= 1e-10 * abs(want) + 1e-15, (got, want)


def test_density_matrix_elements_vs_reference(golden):
    for c in golden["dm"]:
        parts = fock._dm_problem(c["mu"], c["cov"], list(c["i"]), list(c["j"]))
        got = _oracle_element(*parts)
        want = complex(c["out"])
        # elements that vanish by symmetry come out as rounding noise (~1e-18) on both sides
        assert abs(got - want) <= 1e-10 * abs(want) + 1e-15, (got, want)


def test_conversions_and_checks(golden):
    c = golden["dm"][0]
    cov, mu = c["cov"], c["mu"]
    Q = fock.Qmat(cov)
    assert np.allclose(Q, Q.conj().T)
    A = fock.Amat(cov)
    assert np.allclose(A, A.T)
    assert np.allclose(fock.Amat(Q, cov_is_qmat=True), A)
    beta = fock.complex_to_real_displacements(mu)
    assert np.allclose(beta[len(mu) // 2:], beta[:len(mu) // 2].conj())
    pure = golden["pure"][0]["cov"]
    assert fock.is_pure_cov(pure) and fock.is_valid_cov(pure)
    mixed = pure + 0.3 * np.eye(len(pure))
    assert fock.is_valid_cov(mixed) and not fock.is_pure_cov(mixed)
    assert not fock.is_valid_cov(0.5 * pure)  # violates the uncertainty relation
    with pytest.raises(ValueError):
        fock._pure_problem(np.zeros(len(mixed)), mixed, [1] * (len(mixed) // 2))
