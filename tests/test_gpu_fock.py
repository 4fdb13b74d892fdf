"""Fock-space elements of Gaussian states on the GPU: thewalrus_gb300.fock.pure_state_amplitude and
density_matrix_element through the sieve, against the values the reference's own
pure_state_amplitude / density_matrix_element produced (quantum/fock_tensors.py:45-98, :191-232)
for displaced and undisplaced, pure and mixed states, at 1e-10 relative (elements that vanish by
symmetry come out as rounding noise on both sides and are held to 1e-15 absolute)."""
import pytest

from thewalrus_gb300 import fock

pytestmark = pytest.mark.gpu


def _close(got, want):
    return abs(complex(got) - complex(want)) <= 1e-10 * abs(complex(want)) + 1e-15


def test_pure_state_amplitudes(golden):
    for c in golden["pure"]:
        got = fock.pure_state_amplitude(c["mu"], c["cov"], list(c["pattern"]))
        assert _close(got, c["out"]), (list(c["pattern"]), got, complex(c["out"]))


def test_density_matrix_elements(golden):
    for c in golden["dm"]:
        got = fock.density_matrix_element(c["mu"], c["cov"], list(c["i"]), list(c["j"]))
        assert _close(got, c["out"]), (list(c["i"]), list(c["j"]), got, complex(c["out"]))


def test_elements_without_prefactor_and_in_double_double(golden):
    c = golden["dm"][5]
    full = fock.density_matrix_element(c["mu"], c["cov"], list(c["i"]), list(c["j"]))
    bare = fock.density_matrix_element(c["mu"], c["cov"], list(c["i"]), list(c["j"]), include_prefactor=False)
    pref = fock._prefactor(c["mu"], c["cov"])
    assert _close(bare * pref, full)
    dd = fock.density_matrix_element(c["mu"], c["cov"], list(c["i"]), list(c["j"]), precision="dd")
    assert _close(dd, c["out"])
