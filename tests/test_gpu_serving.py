"""GPU tests of the serving subsystem: matrices formed on the device from a resident state,
continuous batching over streams, each result the same alone and in the mix (FP64, 1e-10)."""
import numpy as np
import pytest

import oracle
from thewalrus_gb300.serving import GaussianState, ProbabilityServer, poisson_requests

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def test_served_amplitudes_match_reference(golden):
    pytest.importorskip("torch")
    cases = golden["pure"]
    st = GaussianState.from_cov(cases[0]["mu"], cases[0]["cov"])
    srv = ProbabilityServer([st], max_batch=4, streams=2)
    reqs = [(0.0, 0, np.asarray(c["pattern"])) for c in cases]
    res = srv.serve(reqs)
    for c, r in zip(cases, res):
        ref = complex(c["out"])
        assert abs(r["amplitude"] - ref) <= RTOL * abs(ref)
        assert abs(r["probability"] - abs(ref) ** 2) <= 2 * RTOL * abs(ref) ** 2


def test_same_alone_and_in_the_mix():
    pytest.importorskip("torch")
    states = [GaussianState.synthetic(modes=24, seed=s) for s in range(3)]
    reqs = poisson_requests(states, rate=2000.0, count=40, photons=(2, 16), seed=7)
    srv = ProbabilityServer(states, max_batch=8, streams=3)
    mixed = srv.serve(reqs)
    assert len({r["batch"] for r in mixed if r["batch"] >= 0}) > 1
    for j in range(0, len(reqs), 5):
        alone = srv.serve([(0.0, reqs[j][1], reqs[j][2])])[0]
        a, b = alone["probability"], mixed[j]["probability"]
        assert abs(a - b) <= RTOL * abs(a), (j, a, b)
    # and against the CPU oracle for a few requests
    for j in (0, 11, 23):
        _, s, pat = reqs[j]
        lh = complex(oracle.hafnian_repeated(states[s].B, list(pat), mu=states[s].gamma, loop=True, precision="long"))
        ref = abs(lh * states[s].norm(pat)) ** 2
        assert abs(mixed[j]["probability"] - ref) <= RTOL * ref


def test_admission_respects_memory_budget():
    pytest.importorskip("torch")
    states = [GaussianState.synthetic(modes=16, seed=9)]
    reqs = poisson_requests(states, rate=1e6, count=12, photons=(6, 10), seed=3)
    tight = ProbabilityServer.estimate_bytes(10) + 1  # one request per batch fits
    srv = ProbabilityServer(states, max_batch=64, streams=2, mem_budget=tight)
    res = srv.serve(reqs)
    assert len({r["batch"] for r in res}) == len(reqs)


def test_state_formed_on_the_device_from_the_covariance(golden):
    """wg_state_create_from_cov: the Husimi matrix, its Cholesky factor, B, gamma and the vacuum
    amplitude formed on the GPU from the covariance equal the host conversions, and the served
    amplitudes equal the reference's pure_state_amplitude values."""
    pytest.importorskip("torch")
    cases = golden["pure"]
    host = GaussianState.from_cov(cases[0]["mu"], cases[0]["cov"])
    dev = GaussianState.from_cov_on_device(cases[0]["mu"], cases[0]["cov"])
    assert np.max(np.abs(dev.B - host.B)) <= 1e-13 * np.max(np.abs(host.B))
    assert np.max(np.abs(dev.gamma - host.gamma)) <= 1e-13 * np.max(np.abs(host.gamma))
    assert abs(dev.vacuum - host.vacuum) <= 1e-13 * abs(host.vacuum)
    srv = ProbabilityServer([dev], max_batch=4, streams=2)
    res = srv.serve([(0.0, 0, np.asarray(c["pattern"])) for c in cases])
    for c, r in zip(cases, res):
        ref = complex(c["out"])
        assert abs(r["amplitude"] - ref) <= RTOL * abs(ref) + 1e-15
    # a larger synthetic state (64 modes, hbar = 1): the device conversion against the host one
    from thewalrus_gb300 import workloads as wl
    cov, mu = wl.gaussian_state_cov(64, seed=5, transmission=1.0, disp=0.2)
    host = GaussianState.from_cov(mu, cov * 0.5, hbar=1)
    dev = GaussianState.from_cov_on_device(mu, cov * 0.5, hbar=1)
    assert np.max(np.abs(dev.B - host.B)) <= 1e-12 * np.max(np.abs(host.B))
    assert abs(dev.vacuum - host.vacuum) <= 1e-12 * abs(host.vacuum)
    # a covariance whose Husimi matrix is not positive definite (negative variances) is refused
    with pytest.raises(RuntimeError):
        GaussianState.from_cov_on_device(np.zeros(8), -2.0 * np.eye(8))


def test_served_many_photon_requests_vs_double_double():
    """Served amplitudes of 26-32-photon requests on 64-mode states (12-13 sieve edges, term
    matrices of up to 26 rows plus the border) against the double-double sieve of the same loop
    hafnian: within 1e-10, or 64 eps cond where the sum's condition number cond = sum|term| /
    |sum| (the oracle's, ~1e3..1e4 here) allows more."""
    pytest.importorskip("torch")
    import thewalrus_gb300 as tw
    states = [GaussianState.synthetic(modes=64, seed=s) for s in range(2)]
    reqs = poisson_requests(states, rate=1e5, count=6, photons=(26, 32), seed=11)
    srv = ProbabilityServer(states, max_batch=8, streams=2)
    res = srv.serve(reqs)
    for (t, s, pat), r in zip(reqs, res):
        st = states[s]
        truth = complex(tw.hafnian_repeated(st.B, list(pat), mu=st.gamma, loop=True, precision="dd"))
        p = tw.prepare_loop_hafnian(st.B, st.gamma, list(pat))
        N = int(np.sum(pat))
        cond = complex(oracle.sieve_term_range(p.A, p.reps, Dx=p.D, absolute=True)).real * 0.5 ** (N // 2 - 1) / abs(truth)
        tol = max(RTOL, 64 * 2.0 ** -53 * cond)
        got = r["amplitude"] / st.norm(pat)
        assert abs(got - truth) <= tol * abs(truth), (N, got, truth, cond)
