"""Term magnitudes on the GPU (``wg_plan_read_magnitudes``): per output, the sum over the sieve
terms of |prefactor x term| times the final scale.  Against the oracle's sums of the terms'
absolute values on the benchmark-size fixture (the GPU sums |re| + |im|, the oracle the complex
modulus, so their ratio lies in [1, sqrt 2], and is 1 for real terms); ``hafnian_with_error``'s
estimate against the measured error; ``precision="auto"`` keeping FP64 where it is good to
1e-10 and moving to double-double where it is not."""
import os

import numpy as np
import pytest

import thewalrus_gb300 as tw
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def metric():
    data = np.load(os.path.join(HERE, "golden", "metric_cases.npz"))
    out = {}
    for key in data.files:
        case, field = key.split("/")
        out.setdefault(case, {})[field] = data[key]
    return out


def rel(a, b):
    return abs(complex(a) - complex(b)) / abs(complex(b))


def test_magnitudes_match_the_oracle(metric):
    for case, real in (("haf40_complex", False), ("haf40_real", True)):
        c = metric[case]
        _, mag = tw.run_with_magnitudes([tw.prepare_hafnian(c["A"])])
        ratio = mag[0] / (float(c["cond"]) * abs(complex(c["oracle_ld"])))
        lo, hi = (1 - 1e-9, 1 + 1e-9) if real else (1 - 1e-9, 2 ** 0.5 + 1e-9)
        assert lo <= ratio <= hi, (case, ratio)
    c = metric["lhaf_state20_40"]
    inst = tw.prepare_loop_hafnian(c["A"], c["mu"], list(c["rpt"]))
    _, mag = tw.run_with_magnitudes([inst])
    ratio = mag[0] / (float(c["cond"]) * abs(complex(c["oracle_q"])))
    assert 1 - 1e-9 <= ratio <= 2 ** 0.5 + 1e-9, ratio
    # the exact sieve carries none
    _, mag = tw.run_with_magnitudes([tw.prepare_hafnian(np.ones((12, 12)))], "mod0")
    assert mag[0] == 0.0


def test_error_estimate_bounds_the_error(metric):
    for case in ("haf40_complex", "haf40_real"):
        c = metric[case]
        val, est, mag = tw.hafnian_with_error(c["A"])
        assert abs(complex(val) - complex(c["oracle_ld"])) <= 16 * est, (case, val, est)
    val, est, mag = tw.hafnian_with_error(wl.complex_symmetric(18, seed=4), precision="dd")
    assert est < 1e-25 * abs(complex(val))
    assert tw.hafnian_with_error(np.array([[0.0, 2.0], [2.0, 0.0]])) == (2.0, 0.0, 0.0)


def test_auto_precision(metric):
    c = metric["haf40_complex"]  # sum|term| / |sum| = 6.8e4: FP64 is kept
    got = tw.hafnian(c["A"], precision="auto")
    assert rel(got, tw.hafnian(c["A"], precision="fp64")) < 1e-14
    assert rel(got, tw.hafnian(c["A"], precision="dd")) > 1e-13  # FP64 and dd differ by ~4.4e-12 here
    c = metric["haf40_real"]  # 2.0e5: double-double
    assert rel(tw.hafnian(c["A"], precision="auto"), tw.hafnian(c["A"], precision="dd")) < 1e-15
    c = metric["lhaf_state20_40"]  # 3.4e10: double-double, to 1e-10 of the _Float128 value
    got = tw.hafnian_repeated(c["A"], list(c["rpt"]), mu=c["mu"], loop=True, precision="auto")
    assert rel(got, c["oracle_q"]) < 1e-10
    # integer inputs take the exact sieve, as the default does
    assert tw.hafnian(np.ones((16, 16)), precision="auto") == 2027025.0
    # batches: each member decided on its own
    mats = [metric["haf40_real"]["A"], wl.complex_symmetric(10, seed=1)]
    got = tw.hafnian_batch(mats, precision="auto")
    assert rel(got[0], tw.hafnian(mats[0], precision="dd")) < 1e-15
    assert rel(got[1], tw.hafnian(mats[1], precision="fp64")) < 1e-13
