"""GPU tests of the batching subsystem: one plan over many uneven instances, re-execution,
CUDA-graph replay, merged launch classes, chunk sizes and the autotuner all give the same
results as single calls."""
import numpy as np
import pytest

import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat
from thewalrus_gb300 import autotune
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _instances():
    mats = [wl.complex_symmetric(n, seed=100 + n) for n in (8, 12, 18, 24, 26)] + \
        [wl.real_nonneg(n, seed=200 + n) for n in (10, 16, 22, 28)]
    insts = [tw.prepare_hafnian(A) for A in mats]
    B, D, fixed, cut = wl.batch_loop_calls(count=1, seed=5, modes=8, cutoff=4)[0]
    insts.append(tw.prepare_loop_hafnian_batch(B, D, list(fixed), cut))
    A, g, rpt = wl.gaussian_state_loop(modes=6, seed=2, photons=12, max_rep=3)
    insts.append(tw.prepare_loop_hafnian(A, g, list(rpt)))
    return mats, insts


def _singles(insts):
    return np.concatenate([nat.run([i]) for i in insts])


def test_plan_matches_single_calls_and_reexecutes():
    _, insts = _instances()
    ref = _singles(insts)
    plan = nat.Plan(insts)
    for _ in range(3):
        plan.execute()
        got = plan.read()
        assert np.allclose(got, ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("opts", [
    {"use_graph": True},
    {"merge_classes": True, "use_graph": True},
    {"chunk_scale": 0.25},
    {"chunk_scale": 8.0, "max_warps_per_cta": 2},
])
def test_plan_options_same_results(opts):
    _, insts = _instances()
    ref = _singles(insts)
    plan = nat.Plan(insts, **opts)
    for _ in range(3):  # graph: capture on first use, replay after
        plan.execute()
        assert np.allclose(plan.read(), ref, rtol=1e-12, atol=0)


def test_autotuner_returns_valid_options():
    _, insts = _instances()
    best, table = autotune.tune(insts, candidates=[{"chunk_scale": 1.0, "max_warps_per_cta": 0,
                                                    "merge_classes": False},
                                                   {"chunk_scale": 2.0, "max_warps_per_cta": 0,
                                                    "merge_classes": True}],
                                repeats=1, use_cache=False)
    assert best in [c for c, _ in table] and all(t > 0 for _, t in table)
    plan = nat.Plan(insts, **best)
    plan.execute()
    assert np.allclose(plan.read(), _singles(insts), rtol=1e-12, atol=0)


def test_hafnian_batch_public_api():
    mats, _ = _instances()
    got = tw.hafnian_batch(mats)
    for A, g in zip(mats, got):
        assert abs(g - tw.hafnian(A)) <= 1e-12 * abs(g)
