"""CPU checks of the native boundary and the host logic (no compute calls need a GPU here)."""
import re
import os

import numpy as np
import pytest

import oracle
import thewalrus_gb300 as tw
from thewalrus_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            syms |= set(re.findall(r"^\s*(?:const\s+)?(?:\w+[\s*]+)+(wg_\w+)\s*\(", src, re.M))
    return syms


def test_library_exports_header_symbols():
    lib = nat.load()
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert set(nat.EXPORTS) <= syms


def test_validation_errors():
    with pytest.raises(TypeError):
        tw.hafnian(1)
    with pytest.raises(ValueError):
        tw.hafnian(np.zeros([2, 3]))
    A = np.ones([4, 4]); A[0, 1] = 0.0
    with pytest.raises(ValueError):
        tw.hafnian(A)
    with pytest.raises(ValueError):
        tw.hafnian(np.array([[2, 1], [1, np.nan]]))
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.array([[2, 1], [1, 3]]), [1])
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.array([[2, 1], [1, 3]]), [1, -1])
    with pytest.raises(ValueError):
        tw.hafnian_repeated(np.array([[2, 1], [1, 3]]), [1.1, 1])
    with pytest.raises(TypeError):
        tw.hafnian_repeated(1, [1])


def test_closed_forms_without_gpu(rng):
    assert tw.hafnian(np.ndarray((0, 0))) == 1
    assert tw.hafnian(np.ones([3, 3])) == 0.0
    assert tw.hafnian(np.ones([3, 3]), loop=True) == 4.0
    A = rng.random((4, 4)) + 1j * rng.random((4, 4)); A += A.T
    assert np.allclose(tw.hafnian(A), A[0, 1] * A[2, 3] + A[0, 2] * A[1, 3] + A[0, 3] * A[1, 2])
    assert tw.hafnian(np.identity(6)) == 0
    v = rng.random(5)
    assert np.allclose(tw.hafnian(np.diag(v), loop=True), np.prod(v))
    assert tw.hafnian_repeated(np.array([[2, 1], [1, 3]]), [0, 0]) == 1.0
    assert tw.hafnian_repeated(np.ones([3, 3]), [1] * 3) == 0.0
    assert np.allclose(tw.hafnian_repeated(np.zeros((6, 6)), [1] * 6), 0)


def test_matched_reps_matches_oracle(rng):
    for _ in range(300):
        reps = list(rng.integers(0, 6, size=rng.integers(1, 9)))
        a, b = tw.matched_reps(reps), oracle.matched_reps(reps)
        assert list(a[0]) == list(b[0]) and list(a[1]) == list(b[1]) and a[2] == b[2]


def test_reduction():
    for n in (6, 8):
        res = tw.reduction(np.array([[0, 1], [1, 0]]), [n, n])
        O, B = np.zeros([n, n]), np.ones([n, n])
        assert np.all(res == np.vstack([np.hstack([O, B]), np.hstack([B, O])]))
        assert np.all(tw.reduction(np.array([0, 1]), [n, n]) == np.hstack([O[0], B[0]]))


def test_prepared_instances(golden):
    # host preparation mirrors the reference: batch instances carry the fixed edge reps
    for c in golden["batch"]:
        inst = tw.prepare_loop_hafnian_batch(c["A"], c["D"], list(c["fixed"]), int(c["cutoff"]))
        assert inst.outputs() == len(c["out"])
        assert inst.struct.n == 2 * (inst.struct.E + (2 if inst.struct.kind == nat.WG_KIND_BATCH_ODD else 1))


def test_no_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(RuntimeError):
        tw.hafnian(np.ones((6, 6)))


def test_noalloc_rejects_misaligned_pointers():
    # checked before any CUDA call: the kernels read A in 8-byte words and write the output pair
    # in one 16-byte access (the pointer values are never dereferenced)
    import ctypes
    lib = nat.load()
    reps = np.ones(3, dtype=np.int64)
    rp = reps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    for A, dtype, out in ((0x10004, nat.WG_COMPLEX128, 0x20000), (0x10004, nat.WG_FLOAT64, 0x20000),
                          (0x10000, nat.WG_COMPLEX128, 0x20008)):
        rc = lib.wg_hafnian_noalloc(ctypes.c_void_p(A), 6, dtype, rp, 3, 1, ctypes.c_void_p(out), None)
        assert rc == -1  # WG_EINVAL
        assert b"aligned" in lib.wg_last_error()
