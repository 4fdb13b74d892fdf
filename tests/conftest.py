"""Shared fixtures.  GPU tests carry ``@pytest.mark.gpu``; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_cases.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def golden():
    """Reference-produced cases: dict family -> list of dicts of arrays."""
    data = np.load(GOLDEN, allow_pickle=False)
    fam = {}
    for key in data.files:
        f, i, field = key.split("/")
        fam.setdefault(f, {}).setdefault(int(i), {})[field] = data[key]
    return {f: [v[i] for i in sorted(v)] for f, v in fam.items()}


@pytest.fixture(scope="session")
def rng():
    return np.random.default_rng(137)
