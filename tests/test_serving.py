"""CPU checks of the serving front end: state conventions against the reference's
pure_state_amplitude (golden vectors), request generation, summaries."""
import numpy as np

import oracle
from thewalrus_gb300.serving import GaussianState, poisson_requests, summary


def test_from_cov_amplitudes_match_reference(golden):
    for c in golden["pure"]:
        st = GaussianState.from_cov(c["mu"], c["cov"])
        lhaf = complex(oracle.hafnian_repeated(st.B, list(c["pattern"]), mu=st.gamma, loop=True))
        amp = lhaf * st.norm(c["pattern"])
        assert abs(amp - complex(c["out"])) <= 1e-12 * abs(complex(c["out"]))


def test_pure_vacuum_formula_consistent(golden):
    c = golden["pure"][0]
    st = GaussianState.from_cov(c["mu"], c["cov"])
    direct = GaussianState(st.B, st.alpha)  # det(I - B B*)^(1/4) form
    assert abs(direct.vacuum - st.vacuum) <= 1e-12 * abs(st.vacuum)


def test_poisson_requests_shape():
    states = [GaussianState.synthetic(modes=16, seed=s) for s in range(2)]
    reqs = poisson_requests(states, rate=1000.0, count=50, photons=(4, 10), seed=1)
    times = [r[0] for r in reqs]
    assert times == sorted(times) and len(reqs) == 50
    for _, s, pat in reqs:
        assert 0 <= s < 2 and pat.sum() % 2 == 0 and 4 <= pat.sum() <= 10 and pat.max() <= 2
    res = [{"latency": 0.1 * i, "done": 1.0 + i, "arrival": float(i), "batch": i % 3} for i in range(10)]
    sm = summary(res)
    assert sm["requests"] == 10 and sm["batches"] == 3 and sm["p99_s"] >= sm["p50_s"]


def test_request_cost_counts_the_sieve_terms():
    from thewalrus_gb300._hafnian import matched_reps
    from thewalrus_gb300.serving import ProbabilityServer
    for k in (2, 5, 9):
        pat = np.zeros(30, dtype=np.int64)
        pat[: 2 * k] = 1
        # k edges of multiplicity 1: 2^(k-1) terms (the first radix halved), m = 2k, bordered m + 1
        assert ProbabilityServer.request_cost(matched_reps(pat)) == 2 ** (k - 1) * float(2 * k + 2) ** 3
    # an unpaired mode: no halving of the first radix
    pat = np.zeros(10, dtype=np.int64)
    pat[:3] = 1
    x, reps, odd = matched_reps(pat)
    assert odd is not None and ProbabilityServer.request_cost((x, reps, odd)) == 2.0 * 4.0 ** 3
    costs = [ProbabilityServer.request_cost(matched_reps(np.array([1] * n + [0] * (40 - n)))) for n in (8, 16, 24, 32)]
    assert costs == sorted(costs)
