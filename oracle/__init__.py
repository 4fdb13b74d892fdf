"""CPU oracle for the hafnian sieve path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may import
this package, and only as a checker or as the timed CPU baseline, never as part of the product.

The compiled core (``oracle_core.c``) restates the reference's sieve drivers and combiners
(thewalrus/_hafnian.py:183-577, thewalrus/charpoly.py, thewalrus/loop_hafnian_batch.py:50-208)
in double, long double and _Float128 arithmetic.  This module restates the reference's
host-side preparation around them:

* ``matched_reps``            thewalrus/_hafnian.py:80-159
* ``_haf`` / ``loop_hafnian`` thewalrus/_hafnian.py:470-508, :580-631
* ``hafnian`` special cases   thewalrus/_hafnian.py:717-818
* ``hafnian_repeated``        thewalrus/_hafnian.py:864-936
* ``add_batch_edges_*``, ``loop_hafnian_batch``  thewalrus/loop_hafnian_batch.py:211-304

Extended results come back as double-double pairs; ``precision`` selects the arithmetic:
"double", "long" (x87 80-bit on x86-64, binary128 on AArch64) or "quad" (_Float128).
Parity is pinned by ``tests/golden`` vectors that were produced by the reference itself.
"""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "hafnian",
    "hafnian_repeated",
    "loop_hafnian",
    "loop_hafnian_batch",
    "haf_prepared",
    "haf_term_range",
    "loop_haf_prepared",
    "powertrace",
    "charpoly",
    "matched_reps",
    "brute_hafnian",
]

_SFX = {"double": "_d", "long": "_ld", "quad": "_q"}
_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int64)
        for sfx in _SFX.values():
            f = getattr(lib, "oracle_calc_hafnian" + sfx)
            f.argtypes = [dp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
            f = getattr(lib, "oracle_calc_loop_hafnian" + sfx)
            f.argtypes = [dp, dp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, dp, dp,
                          ctypes.c_int, ctypes.c_int, dp]
            f = getattr(lib, "oracle_calc_loop_hafnian_batch" + sfx)
            f.argtypes = [dp, dp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                          ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
            f = getattr(lib, "oracle_hafnian_term_range" + sfx)
            f.argtypes = [dp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                          ctypes.c_int64, ctypes.c_int64, dp]
            f = getattr(lib, "oracle_sieve_term_range" + sfx)
            f.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ip, ctypes.c_int, dp, dp, ctypes.c_int,
                          ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, dp]
            f = getattr(lib, "oracle_powertrace" + sfx)
            f.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp]
            f = getattr(lib, "oracle_charpoly" + sfx)
            f.argtypes = [dp, ctypes.c_int, dp]
        for k in range(len(EXACT_PRIMES)):
            f = getattr(lib, "oracle_exact_hafnian_p%d" % k)
            f.argtypes = [ip, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip]
        _lib = lib
    return _lib


def _default_threads():
    return int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))


def _cbuf(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ibuf(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.int64))
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def _dd(out, i=0):
    """(value, low part) of the i-th complex double-double in an output buffer."""
    hi = complex(out[4 * i], out[4 * i + 1])
    lo = complex(out[4 * i + 2], out[4 * i + 3])
    return hi, lo


class DD(complex):
    """A complex128 result that also carries the low-order bits of an extended-precision value."""

    def __new__(cls, hi, lo=0j):
        obj = complex.__new__(cls, hi)
        obj.lo = complex(lo)
        return obj


def matched_reps(reps):
    """Greedy pairing of repeated rows into edges (restates thewalrus/_hafnian.py:80-159).

    Returns ``(x, edge_reps, oddmode)``: vertex order of length 2E (vertex i paired with i+E),
    edge multiplicities and the unpaired index (or None).
    """
    reps = [int(r) for r in reps]
    if sum(reps) == 0:
        return np.array([], dtype=int), np.array([], dtype=int), None
    order = sorted(zip(reps, range(len(reps))), reverse=True)
    items = [(r, i) for r, i in order if r > 0]
    ea, eb, er = [], [], []
    while len(items) > 1 or (len(items) == 1 and items[0][0] > 1):
        items.sort(reverse=True)
        r0, i0 = items[0]
        if len(items) == 1 or r0 > 2 * items[1][0]:
            ea.append(i0)
            eb.append(i0)
            er.append(r0 // 2)
            if r0 % 2 == 0:
                items = items[1:]
            else:
                items[0] = (1, i0)
        else:
            r1, i1 = items[1]
            ea.append(i0)
            eb.append(i1)
            er.append(r1)
            if r0 > r1:
                items = [(r0 - r1, i0)] + items[2:]
            else:
                items = items[2:]
    oddmode = items[0][1] if len(items) == 1 else None
    return np.asarray(ea + eb, dtype=np.int64), np.asarray(er, dtype=np.int64), oddmode


def haf_prepared(Ax, edge_reps, glynn=True, precision="double", nthreads=None):
    """_calc_hafnian on prepared inputs (reordered matrix, edge multiplicities)."""
    lib = _load()
    A, pA = _cbuf(Ax)
    r, pr = _ibuf(edge_reps)
    out = np.zeros(4)
    getattr(lib, "oracle_calc_hafnian" + _SFX[precision])(
        pA, A.shape[0], pr, len(r), int(bool(glynn)), nthreads or _default_threads(),
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return DD(*_dd(out))


def haf_term_range(Ax, edge_reps, t_begin, t_end, glynn=True, precision="double", nthreads=None):
    """Unscaled sum of the plain sieve's terms [t_begin, t_end) on prepared inputs, in the
    reference's mixed-radix term order: a bounded sample of one hafnian's CPU work."""
    lib = _load()
    A, pA = _cbuf(Ax)
    r, pr = _ibuf(edge_reps)
    out = np.zeros(4)
    getattr(lib, "oracle_hafnian_term_range" + _SFX[precision])(
        pA, A.shape[0], pr, len(r), int(bool(glynn)), nthreads or _default_threads(),
        int(t_begin), int(t_end), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return DD(*_dd(out))


def sieve_term_range(Ax, edge_reps, t_begin=0, t_end=-1, Dx=None, oddloop=None, oddV=None, glynn=True,
                     absolute=False, precision="double", nthreads=None):
    """Unscaled sum over the terms [t_begin, t_end) (t_end = -1: to the end) of the plain
    (``Dx`` None) or loop sieve on prepared inputs, in the reference's mixed-radix term order;
    ``absolute=True`` sums the terms' absolute values instead (with the absolute value of the
    scaled sum this gives the sum's condition number)."""
    lib = _load()
    A, pA = _cbuf(Ax)
    r, pr = _ibuf(edge_reps)
    kind = 0 if Dx is None else (2 if oddloop is not None else 1)
    D, pD = _cbuf(Dx if Dx is not None else np.zeros(1))
    V, pV = _cbuf(oddV if oddV is not None else np.zeros(1))
    ol = np.array([complex(oddloop or 0).real, complex(oddloop or 0).imag])
    out = np.zeros(4)
    getattr(lib, "oracle_sieve_term_range" + _SFX[precision])(
        kind, pA, pD, A.shape[0], pr, len(r), ol.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), pV,
        int(bool(glynn)), nthreads or _default_threads(), int(t_begin), int(t_end), int(bool(absolute)),
        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return DD(*_dd(out))


def loop_haf_prepared(Ax, Dx, edge_reps, oddloop=None, oddV=None, glynn=True,
                      precision="double", nthreads=None):
    """_calc_loop_hafnian on prepared inputs."""
    lib = _load()
    A, pA = _cbuf(Ax)
    D, pD = _cbuf(Dx)
    r, pr = _ibuf(edge_reps)
    has_odd = oddloop is not None
    ol, pol = _cbuf([oddloop if has_odd else 0])
    ov, pov = _cbuf(oddV if has_odd else np.zeros(max(A.shape[0], 1)))
    out = np.zeros(4)
    getattr(lib, "oracle_calc_loop_hafnian" + _SFX[precision])(
        pA, pD, A.shape[0], pr, len(r), int(has_odd), pol, pov, int(bool(glynn)),
        nthreads or _default_threads(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return DD(*_dd(out))


def _haf(A, reps=None, glynn=True, precision="double", nthreads=None):
    n = A.shape[0]
    reps = [1] * n if reps is None else list(reps)
    N = sum(reps)
    if N == 0:
        return 1.0
    if N % 2 == 1:
        return 0.0
    x, edge_reps, _ = matched_reps(reps)
    Ax = A[np.ix_(x, x)].astype(np.complex128)
    return haf_prepared(Ax, edge_reps, glynn, precision, nthreads)


def loop_hafnian(A, D=None, reps=None, glynn=True, precision="double", nthreads=None):
    """Loop hafnian with repetitions (restates thewalrus/_hafnian.py:580-631)."""
    n = A.shape[0]
    reps = [1] * n if reps is None else list(reps)
    if D is None:
        D = A.diagonal()
    N = sum(reps)
    if N == 0:
        return 1.0
    if N == 1:
        return D[np.where(np.array(reps) == 1)[0][0]]
    x, edge_reps, oddmode = matched_reps(reps)
    if oddmode is not None:
        oddloop = complex(D[oddmode])
        oddV = A[oddmode, x].astype(np.complex128)
    else:
        oddloop, oddV = None, None
    Ax = A[np.ix_(x, x)].astype(np.complex128)
    Dx = np.asarray(D)[x].astype(np.complex128)
    return loop_haf_prepared(Ax, Dx, edge_reps, oddloop, oddV, glynn, precision, nthreads)


def hafnian(A, loop=False, rtol=1e-05, atol=1e-08, method="glynn", precision="double",
            nthreads=None):
    """Public-API behaviour of thewalrus.hafnian for the sieve methods (no validation)."""
    glynn = method != "inclexcl"
    if A.shape == (0, 0):
        return 1
    if A.shape[0] % 2 != 0 and not loop:
        return 0.0
    if np.allclose(np.diag(np.diag(A)), A, rtol=rtol, atol=atol):
        return np.prod(np.diag(A)) if loop else 0
    if A.shape[0] == 2:
        return A[0, 1] + A[0, 0] * A[1, 1] if loop else A[0][1]
    if A.shape[0] == 3 and loop:
        return A[0, 0] * A[1, 2] + A[1, 1] * A[0, 2] + A[2, 2] * A[0, 1] + A[0, 0] * A[1, 1] * A[2, 2]
    if A.shape[0] == 4:
        if loop:
            return (A[0, 1] * A[2, 3] + A[0, 2] * A[1, 3] + A[0, 3] * A[1, 2]
                    + A[0, 0] * A[1, 1] * A[2, 3] + A[0, 1] * A[2, 2] * A[3, 3]
                    + A[0, 2] * A[1, 1] * A[3, 3] + A[0, 0] * A[2, 2] * A[1, 3]
                    + A[0, 0] * A[3, 3] * A[1, 2] + A[0, 3] * A[1, 1] * A[2, 2]
                    + A[0, 0] * A[1, 1] * A[2, 2] * A[3, 3])
        return A[0, 1] * A[2, 3] + A[0, 2] * A[1, 3] + A[0, 3] * A[1, 2]
    if loop:
        return loop_hafnian(A, None, None, True, precision, nthreads)
    return _haf(A, None, glynn, precision, nthreads)


def hafnian_repeated(A, rpt, mu=None, loop=False, rtol=1e-05, atol=1e-08, glynn=True,
                     precision="double", nthreads=None):
    """Public-API behaviour of thewalrus.hafnian_repeated (no validation)."""
    nud = np.array(rpt, dtype=np.int32)
    if np.all(nud == 0):
        return 1.0
    if np.sum(nud) % 2 != 0 and not loop:
        return 0.0
    if mu is None:
        mu = A.diagonal().copy()
    if np.allclose(A, 0, rtol=rtol, atol=atol):
        return np.prod(mu**rpt) if loop else 0
    if loop:
        return loop_hafnian(A, mu, rpt, glynn, precision, nthreads)
    return _haf(A, rpt, glynn, precision, nthreads)


def _batch_edges_even(fixed_edges):
    if len(fixed_edges) == 0:
        return np.array([0, 0], dtype=int)
    ne = fixed_edges.shape[0]
    new = max(fixed_edges) + 1
    return np.concatenate([[new], fixed_edges[: ne // 2], [new], fixed_edges[ne // 2:]]).astype(int)


def _batch_edges_odd(fixed_edges, oddmode):
    if len(fixed_edges) == 0:
        return np.array([1, oddmode, 1, 1], dtype=int)
    ne = fixed_edges.shape[0]
    new = max(max(fixed_edges), oddmode) + 1
    return np.concatenate([[new, oddmode], fixed_edges[: ne // 2], [new, new],
                           fixed_edges[ne // 2:]]).astype(int)


def loop_hafnian_batch(A, D, fixed_reps, N_cutoff, glynn=True, precision="double", nthreads=None,
                       return_dd=False):
    """Restates thewalrus/loop_hafnian_batch.py:260-304 (host prep) around the compiled sieve."""
    n = A.shape[0]
    nz = np.nonzero(list(fixed_reps) + [1])[0]
    Anz = A[np.ix_(nz, nz)]
    Dnz = np.asarray(D)[nz]
    fixed_reps = np.asarray(fixed_reps)
    fixed_nz = fixed_reps[nz[:-1]]
    fixed_edges, fixed_m_reps, oddmode = matched_reps(fixed_nz)
    if oddmode is None:
        batch_max, cut, odd = N_cutoff // 2, N_cutoff % 2, 0
        edges = _batch_edges_even(fixed_edges)
        length = 2 * batch_max + cut + 1
    else:
        batch_max, cut, odd = (N_cutoff - 1) // 2, 1 - (N_cutoff % 2), 1
        edges = _batch_edges_odd(fixed_edges, oddmode)
        length = 2 * batch_max + cut + 2
    Ax = Anz[np.ix_(edges, edges)].astype(np.complex128)
    Dx = Dnz[edges].astype(np.complex128)
    lib = _load()
    A_, pA = _cbuf(Ax)
    D_, pD = _cbuf(Dx)
    r, pr = _ibuf(fixed_m_reps)
    out = np.zeros(4 * length)
    getattr(lib, "oracle_calc_loop_hafnian_batch" + _SFX[precision])(
        pA, pD, A_.shape[0], pr, len(r), batch_max, cut, odd, int(bool(glynn)),
        nthreads or _default_threads(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    hi = out[0::4] + 1j * out[1::4]
    if return_dd:
        return hi, out[2::4] + 1j * out[3::4]
    return hi


def loop_hafnian_batch_gamma(A, D, fixed_reps, N_cutoff, glynn=True, precision="double", nthreads=None):
    """Restates thewalrus/loop_hafnian_batch_gamma.py:222-269: for every row k of D the inner
    loop (:99-117 even, :181-205 odd) is the loop_hafnian_batch sum with displacement D[k]
    (self-loop weights D[k, 0], D[k, 1]); rows are stacked into an (len(D), N_cutoff + 1) array."""
    D = np.asarray(D)
    n = A.shape[0]
    assert A.shape[1] == n and D.shape[1] == n and len(fixed_reps) == n - 1
    rows = [loop_hafnian_batch(A, D[k], fixed_reps, N_cutoff, glynn, precision, nthreads) for k in range(len(D))]
    return np.array(rows, dtype=np.complex128).reshape(len(D), N_cutoff + 1)


EXACT_PRIMES = (2147483647, 2147483629, 2147483587, 2147483579, 2147483563)


def exact_hafnian(A, reps=None, glynn=True, nthreads=None):
    """Exact hafnian (a Python int) of an integer-valued symmetric matrix: the sieve of
    thewalrus/_hafnian.py:415-467 evaluated over F_p for five 31-bit primes (oracle_exact.c), then
    the Chinese remainder theorem; exact while |haf| < 2^153."""
    A = np.asarray(A)
    if not np.all(np.equal(np.mod(A, 1), 0)):
        raise ValueError("exact_hafnian needs an integer-valued matrix")
    n = A.shape[0]
    reps = [1] * n if reps is None else list(reps)
    N = sum(reps)
    if N == 0:
        return 1
    if N % 2:
        return 0
    x, edge_reps, _ = matched_reps(reps)
    Ax = np.ascontiguousarray(A[np.ix_(x, x)].astype(np.int64))
    r = np.ascontiguousarray(edge_reps, dtype=np.int64)
    lib = _load()
    res = []
    for k, p in enumerate(EXACT_PRIMES):
        out = ctypes.c_int64()
        getattr(lib, "oracle_exact_hafnian_p%d" % k)(
            Ax.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), Ax.shape[0],
            r.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(r), int(bool(glynn)),
            nthreads or _default_threads(), ctypes.byref(out))
        res.append(int(out.value))
    M, v = 1, 0
    for p, a in zip(EXACT_PRIMES, res):  # CRT, incremental
        t = ((a - v) * pow(M, -1, p)) % p
        v += M * t
        M *= p
    return v - M if v > M // 2 else v


def powertrace(H, n, precision="double"):
    """charpoly.powertrace(H, n) (restates thewalrus/charpoly.py:301-327)."""
    lib = _load()
    Hc, pH = _cbuf(H)
    out = np.zeros(4 * max(n + 2, 2))
    getattr(lib, "oracle_powertrace" + _SFX[precision])(
        pH, Hc.shape[0], n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out[0: 4 * n: 4] + 1j * out[1: 4 * n: 4]


def charpoly(H, precision="double"):
    """charpoly.charpoly(H): Householder Hessenberg then La Budde (thewalrus/charpoly.py:285-298)."""
    lib = _load()
    Hc, pH = _cbuf(H)
    m = Hc.shape[0]
    out = np.zeros(4 * m)
    getattr(lib, "oracle_charpoly" + _SFX[precision])(
        pH, m, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out[0::4] + 1j * out[1::4]


def brute_hafnian(A, loop=False):
    """Sum over perfect matchings (single-pair matchings when loop) by recursion on the first
    vertex, exact for object arrays of Python ints; a small-n check independent of the sieve."""
    A = np.asarray(A)
    n = A.shape[0]

    def rec(idx):
        if not idx:
            return 1
        i, rest = idx[0], idx[1:]
        s = A[i, i] * rec(rest) if loop else 0
        for t, j in enumerate(rest):
            s = s + A[i, j] * rec(rest[:t] + rest[t + 1:])
        return s

    return rec(tuple(range(n)))
