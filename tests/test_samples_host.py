"""Host side of the Gaussian boson samplers (no GPU): the state decomposition, the mode order, the
Husimi A block and the categorical draw, against values produced by the reference."""
import numpy as np

from thewalrus_gb300 import samples as smp


def test_decomposition_vs_reference(golden):
    # the Williamson basis comes from LAPACK's Schur vectors: the fixtures were made on x86-64
    for c in golden["gbs_decomp"]:
        T, sqrtW = smp.decompose_cov(c["cov_ordered"])
        assert np.allclose(T, c["T"], atol=1e-12, rtol=0)
        assert np.allclose(sqrtW, c["sqrtW"], atol=1e-10, rtol=0)
        assert np.allclose(T + sqrtW @ sqrtW.T, c["cov_ordered"], atol=1e-12, rtol=0)
        M = len(T) // 2
        assert np.allclose(smp._husimi_a(T)[:M, :M], c["B"], atol=1e-12, rtol=0)
        assert np.array_equal(smp.photon_means_order(c["mean"], c["cov"]), c["order"])


def test_williamson_normal_form():
    rng = np.random.default_rng(3)
    G = rng.normal(size=(8, 8))
    V = G @ G.T + 8 * np.eye(8)
    D, S = smp.williamson(V)
    n = 4
    omega = np.block([[np.zeros((n, n)), np.eye(n)], [-np.eye(n), np.zeros((n, n))]])
    assert np.allclose(S @ D @ S.T, V, atol=1e-10)
    assert np.allclose(S @ omega @ S.T, omega, atol=1e-10)


def test_choose_matches_numpy_choice():
    rng = np.random.default_rng(5)
    for trial in range(200):
        p = rng.random(int(rng.integers(2, 9))) ** 3
        p /= p.sum()
        np.random.seed(trial)
        want = np.random.choice(np.arange(len(p)), p=p)
        np.random.seed(trial)
        assert smp._choose(p, np.random.random_sample()) == want


def test_permutation_helpers():
    p = np.array([3, 0, 2, 1])
    assert np.array_equal(smp.invert_permutation(p)[p], np.arange(4))
    mu = np.arange(6.0)
    assert np.allclose(smp.mu_to_alpha(mu, hbar=2), (mu[:3] + 1j * mu[3:]) / 2)


def test_graph_state_vs_reference(golden):
    # adj_scaling / gen_Qmat_from_graph / Covmat of the graph samplers against the reference's
    for c in golden["graph"]:
        A, n_mean = c["A"], float(c["n_mean"])
        x = smp.adj_scaling(A, n_mean)
        assert abs(x - float(c["scale"])) <= 1e-11 * abs(float(c["scale"]))
        Q = smp.gen_Qmat_from_graph(A, n_mean)
        assert np.allclose(Q, c["Q"], atol=1e-10, rtol=1e-10)
        cov = smp.Covmat(Q)
        assert np.allclose(cov, c["cov"], atol=1e-10, rtol=1e-10)
        # the state is pure and carries the requested mean photon number
        n = len(A)
        assert abs((np.trace(cov) - 2 * n) / 4 - n_mean) < 1e-8
        assert abs(np.linalg.det(cov) - 1.0) < 1e-7
