"""wg_hafnian_noalloc: the allocation-free entry point, for callers that cannot allocate device
memory while they call the library (their own memory pools, serving plugins, stall-free loops).

The test owns the device buffers (allocated here with torch, as such a caller would own them)
and checks, on two calls in a row, that the entry point reproduces wg_hafnian's result; then
against values the reference produced (the 24x24 complex matrix of the plain-hafnian workload)
and against the _Float128 oracle on repeated edges (non-unit binomials) and on the
inclusion/exclusion form (glynn = 0).  It is collected last so that a failure here leaves every
other test already run.
"""
import ctypes

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat
from thewalrus_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _reference(inst):
    """wg_hafnian on the same prepared input (host pointers)."""
    lib = nat.load()
    out = np.zeros(2)
    dtype = nat.WG_COMPLEX128 if np.iscomplexobj(inst.A) else nat.WG_FLOAT64
    nat.check(lib.wg_hafnian(inst.A.ctypes.data, inst.A.shape[0], dtype,
                             inst.reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(inst.reps),
                             int(inst.struct.glynn), nat.WG_PREC_FP64,
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None))
    return complex(out[0], out[1])


def _noalloc(inst, torch):
    lib = nat.load()
    cplx = np.iscomplexobj(inst.A)
    A_dev = torch.from_numpy(inst.A.copy()).cuda()
    out_dev = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.wg_hafnian_noalloc(ctypes.c_void_p(A_dev.data_ptr()), inst.A.shape[0],
                                nat.WG_COMPLEX128 if cplx else nat.WG_FLOAT64,
                                inst.reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(inst.reps),
                                int(inst.struct.glynn), ctypes.c_void_p(out_dev.data_ptr()),
                                ctypes.c_void_p(stream.cuda_stream))
    nat.check(rc)
    torch.cuda.synchronize()
    o = out_dev.cpu().numpy()
    return complex(o[0], o[1])


def test_noalloc_matches_wg_hafnian_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    cases = [tw.prepare_hafnian(wl.complex_symmetric(24, seed=7)),
             tw.prepare_hafnian(wl.real_nonneg(20, seed=8))]
    for inst in cases:  # two calls in a row, different inputs and types
        ref = _reference(inst)
        got = _noalloc(inst, torch)
        assert abs(got - ref) <= RTOL * abs(ref), (got, ref)
    # the same input again after a different one: the shared scratch keeps no stale state
    ref = _reference(cases[0])
    assert abs(_noalloc(cases[0], torch) - ref) <= RTOL * abs(ref)


def test_noalloc_vs_reference_and_oracle(golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    # the 24x24 complex workload matrix (seed 0) against the reference's own value
    case = [c for c in golden["haf"] if c["A"].shape == (24, 24) and np.iscomplexobj(c["A"])][0]
    got = _noalloc(tw.prepare_hafnian(case["A"]), torch)
    assert abs(got - complex(case["out"])) <= RTOL * abs(complex(case["out"]))
    # repeated edges: edge multiplicities above 1 (binomial prefactors, radix (r0 + 2) / 2 first)
    rng = np.random.default_rng(31)
    for k in range(3):
        A = wl.complex_symmetric(6, seed=40 + k)
        rpt = [int(r) for r in rng.integers(1, 5, size=6)]
        if sum(rpt) % 2:
            rpt[0] += 1
        inst = tw.prepare_hafnian(A, rpt)
        assert max(inst.reps) > 1
        want = complex(oracle.hafnian_repeated(A, rpt, precision="quad"))
        got = _noalloc(inst, torch)
        assert abs(got - want) <= RTOL * abs(want), (rpt, got, want)
        assert abs(got - _reference(inst)) <= RTOL * abs(want)
    # inclusion/exclusion (glynn = 0): every edge's radix is rep + 1 and no halving
    A = wl.complex_symmetric(14, seed=9)
    inst = tw.prepare_hafnian(A, glynn=False)
    want = complex(oracle.hafnian(A, method="inclexcl", precision="quad"))
    got = _noalloc(inst, torch)
    assert abs(got - want) <= RTOL * abs(want), (got, want)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = nat.load()
    A_dev = torch.zeros((66, 66), dtype=torch.float64, device="cuda")
    out_dev = torch.zeros(2, dtype=torch.float64, device="cuda")
    reps = np.ones(33, dtype=np.int64)
    rc = lib.wg_hafnian_noalloc(ctypes.c_void_p(A_dev.data_ptr()), 66, nat.WG_FLOAT64,
                                reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 33, 1,
                                ctypes.c_void_p(out_dev.data_ptr()), None)
    assert rc == -1
    assert b"maximum" in lib.wg_last_error()
    # no photons at all: a closed form (1), not a sieve; rejected rather than run
    zero = np.zeros(2, dtype=np.int64)
    rc = lib.wg_hafnian_noalloc(ctypes.c_void_p(A_dev.data_ptr()), 4, nat.WG_FLOAT64,
                                zero.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), 2, 1,
                                ctypes.c_void_p(out_dev.data_ptr()), None)
    assert rc == -1
    assert b"no photons" in lib.wg_last_error()
