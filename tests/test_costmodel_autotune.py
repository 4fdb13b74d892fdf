"""Host logic behind the measurements: the algorithmic flop counts the roofline divides by, and
the autotuner's workload signature (no GPU)."""
import numpy as np

import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat
from thewalrus_gb300 import autotune, costmodel
from thewalrus_gb300 import workloads as wl


def test_flops_per_n40_hafnian():
    # the figure bench.py reports as flops_per_launch for the n = 40 complex hafnian
    assert costmodel.plain_hafnian_flops(40) == 241969397760
    assert costmodel.plain_hafnian_flops(40, complex_input=False) * 4 == costmodel.plain_hafnian_flops(40)


def test_elimination_count_closed_form():
    # plain term, no border: the elimination's multiply-adds sum_{L=1}^{m-1} (L + (L-1)L + mL)
    # = (m-1)m(2m-1)/6 + m^2(m-1)/2, i.e. (5/6) m^3 to leading order; then La Budde and the series
    for m, K in ((8, 4), (24, 12), (40, 20)):
        hess = (m - 1) * m * (2 * m - 1) // 6 + m * m * (m - 1) // 2
        Kc = min(K, m)
        lab = sum(min(j, i) for i in range(1, m + 1) for j in range(1, min(i, Kc) + 1))
        ser = sum(min(n, Kc) for n in range(1, K + 1))
        assert costmodel.term_macs(m, K) == hess + lab + ser


def test_term_distribution_counts_every_term():
    # the histogram of term-matrix sizes covers the sieve's terms exactly (the ranges the GPU
    # enumerates), for plain, repeated and loop instances
    for reps, kind in (([1] * 10, "plain"), ([2, 1, 3, 1, 1], "plain"), ([3, 3, 2, 2, 2, 1, 1, 1], "loop"),
                       ([2, 2, 2, 1, 1], "loop")):
        n = len(reps)
        A = wl.complex_symmetric(n, seed=1)
        if kind == "plain":
            inst = tw.prepare_hafnian(A, reps=reps) if any(r != 1 for r in reps) else tw.prepare_hafnian(A)
        else:
            inst = tw.prepare_loop_hafnian(A, np.diag(A).copy(), reps)
        # the Glynn halving of the first edge applies unless a self-loop is left unpaired
        half = inst.struct.kind in (nat.WG_KIND_PLAIN, nat.WG_KIND_LOOP) and not inst.struct.has_odd
        dist = costmodel._edge_m_distribution(inst.reps, glynn=True, half_first=half)
        assert sum(dist.values()) == inst.terms()


def test_autotune_signature():
    a = [tw.prepare_hafnian(wl.complex_symmetric(n, seed=n)) for n in (8, 10, 12)]
    b = [tw.prepare_hafnian(wl.complex_symmetric(n, seed=n + 1)) for n in (12, 8, 10)]
    # a histogram of shapes: the values and the order of the instances do not matter
    assert autotune.signature(a, "fp64") == autotune.signature(b, "fp64")
    assert autotune.signature(a, "fp64") != autotune.signature(a, "df")
    assert autotune.signature(a, "fp64") != autotune.signature(a[:2], "fp64")
    assert all(set(c) == {"chunk_scale", "max_warps_per_cta", "merge_classes", "serial_groups"}
               for c in autotune.DEFAULT_CANDIDATES)
