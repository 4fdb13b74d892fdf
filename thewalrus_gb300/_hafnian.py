"""Drop-in hafnian / loop-hafnian API on the GB300 sieve kernels.

Same names, arguments, return conventions and errors as the reference's public functions:

* ``hafnian``            thewalrus/_hafnian.py:717-818
* ``hafnian_repeated``   thewalrus/_hafnian.py:864-936
* ``loop_hafnian``       thewalrus/_hafnian.py:580-631
* ``_haf``               thewalrus/_hafnian.py:470-508
* ``input_validation``   thewalrus/_hafnian.py:634-665
* ``reduction``          thewalrus/_hafnian.py:697-714
* ``matched_reps``       thewalrus/_hafnian.py:80-159
* ``loop_hafnian_batch`` thewalrus/loop_hafnian_batch.py:260-304

The host keeps validation, the closed forms for tiny matrices, edge pairing and reordering;
every sieve runs on the GPU (no CPU fallback).  Extra keyword ``precision`` selects "fp64"
(default), "df" (FP32 double-float term arithmetic), "dd" (FP64 double-double terms, for sums
that cancel beyond FP64's reach), "auto" (FP64, and double-double again for the instances whose
term magnitudes say FP64 may miss 1e-10) or "exact" (integer inputs).  Sieve results come back as
``numpy.complex128`` also for real input, as in the reference.
"""
import heapq

import numpy as np

from . import _native as nat

__all__ = [
    "hafnian",
    "hafnian_repeated",
    "loop_hafnian",
    "loop_hafnian_batch",
    "hafnian_batch",
    "input_validation",
    "reduction",
    "matched_reps",
    "prepare_hafnian",
    "prepare_loop_hafnian",
    "prepare_loop_hafnian_batch",
    "hafnian_with_error",
    "run_with_magnitudes",
]

DEFAULT_PRECISION = "fp64"


def _integral(inst):
    """True when an instance's inputs are real integers the exact sieve accepts (magnitudes
    below 2^31, edge repetitions up to 50)."""
    if not isinstance(inst, nat.Instance) or np.iscomplexobj(inst.A):
        return False
    for a in (inst.A, inst.D, inst.oddV):
        if a is not None and a.size and not (np.all(np.isfinite(a)) and np.all(a == np.round(a))
                                             and np.max(np.abs(a)) < 2 ** 31):
            return False
    if inst.struct.has_odd and inst.struct.oddloop[0] != round(inst.struct.oddloop[0]):
        return False
    return len(inst.reps) == 0 or int(np.max(inst.reps)) <= 50


def _integer_valued(*arrays):
    """True when every given array (or scalar) holds real integers: such inputs take the exact
    sieve by default, whose result no scaling could improve."""
    for a in arrays:
        if a is None:
            continue
        a = np.asarray(a)
        if a.size and (np.iscomplexobj(a) and np.any(a.imag != 0) or np.any(np.real(a) != np.round(np.real(a)))):
            return False
    return True


def _auto(precision, insts):
    """The precision of a call: the caller's, else exact for integer inputs (the sieve over
    residues modulo 31-bit primes, so integer hafnians come back exactly, rounded once to
    complex128), else FP64."""
    if precision:
        return precision
    if insts and all(_integral(i) for i in insts) and nat.exact_primes(insts) is not None:
        return "exact"
    return DEFAULT_PRECISION


def _allclose(a, b, rtol, atol):
    """``numpy.allclose(a, b, rtol, atol)``: on finite inputs its test |a - b| <= atol + rtol |b|
    without numpy's generic wrapper (~10 us a call on a small matrix), otherwise numpy's
    (NaN never close, equal infinities close)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if not (np.isfinite(a).all() and np.isfinite(b).all()):
        return bool(np.allclose(a, b, rtol=rtol, atol=atol))
    return bool((np.abs(a - b) <= atol + rtol * np.abs(b)).all())


def input_validation(A, rtol=1e-05, atol=1e-08):
    """Checks that ``A`` is a square, NaN-free, symmetric NumPy array (raises otherwise)."""
    if not isinstance(A, np.ndarray):
        raise TypeError("Input matrix must be a NumPy array.")
    n = A.shape
    if n[0] != n[1]:
        raise ValueError("Input matrix must be square.")
    if np.isnan(A).any():
        raise ValueError("Input matrix must not contain NaNs.")
    if not _allclose(A, A.T, rtol, atol):
        raise ValueError("Input matrix must be symmetric.")
    return True


def reduction(A, rpt):
    """Repeat row/column i of ``A`` rpt[i] times (vectors: entry i)."""
    rows = np.repeat(np.arange(len(rpt)), np.asarray(rpt, dtype=np.int64))
    if A.ndim == 1:
        return A[rows]
    return A[:, rows][rows]


def matched_reps(reps):
    """Pair repeated indices into edges with multiplicities.

    Greedy rule of the reference: repeatedly take the two indices with the most remaining
    repetitions; if the largest has more than twice the second (or is alone) it is paired with
    itself ``r // 2`` times, otherwise it is paired with the second as often as the second
    allows.  Returns ``(x, edge_reps, oddmode)`` with vertex ``x[i]`` matched to ``x[i + E]``.
    """
    reps = [int(r) for r in reps]
    if sum(reps) == 0:
        return np.array([], dtype=int), np.array([], dtype=int), None
    # a heap of (-count, -index): the largest count first, ties broken by the larger index first
    pool = [(-r, -i) for i, r in enumerate(reps) if r > 0]
    heapq.heapify(pool)
    left, right, mult = [], [], []
    while len(pool) > 1 or (pool and -pool[0][0] > 1):
        top_r, top_i = heapq.heappop(pool)
        top_r, top_i = -top_r, -top_i
        if not pool or top_r > 2 * -pool[0][0]:
            left.append(top_i)
            right.append(top_i)
            mult.append(top_r // 2)
            if top_r % 2:
                heapq.heappush(pool, (-1, -top_i))
        else:
            sec_r, sec_i = heapq.heappop(pool)
            sec_r, sec_i = -sec_r, -sec_i
            left.append(top_i)
            right.append(sec_i)
            mult.append(sec_r)
            if top_r > sec_r:
                heapq.heappush(pool, (-(top_r - sec_r), -top_i))
    oddmode = -pool[0][1] if len(pool) == 1 else None
    return np.asarray(left + right, dtype=np.int64), np.asarray(mult, dtype=np.int64), oddmode


def _cast(x, dt):
    x = np.asarray(x)
    return np.real(x).astype(np.float64) if dt == np.float64 else x.astype(np.complex128)


def _sub(A, idx):
    """A[idx][:, idx] (rows and columns picked by idx; ~5x cheaper than A[np.ix_(idx, idx)] on the
    small matrices the samplers prepare by thousands)."""
    return np.asarray(A).take(idx, 0).take(idx, 1)


def _is_complex(*arrays):
    """True when some input has a nonzero imaginary part: complex128 inputs with real values run
    the real sieve (a quarter of the flops, and the exact sieve for integers), with the same
    numpy.complex128 result."""
    for a in arrays:
        if a is None:
            continue
        a = np.asarray(a)
        if a.dtype.kind == "c" and np.any(a.imag):
            return True
    return False


def _pair_balance(Ax, Dx=None, oddV=None, first=0, spread=16.0, sweeps=16):
    """Balance a prepared matrix by a similarity that leaves every sieve term unchanged.

    In a prepared matrix vertex e is matched to vertex E + e.  Scaling vertex e by s_e and
    vertex E + e by 1/s_e (A -> S A S, loop weights D -> S D, the odd vertex's row oddV -> S oddV)
    multiplies the hafnian of the expanded matrix by prod_e (s_e / s_e)^r_e = 1, and each sieve
    term's matrix A X_delta by the diagonal similarity S (.) S^-1, so no term changes either.
    Such a scaling can make rows of one column differ by many orders of magnitude, which the
    term matrices' pivoted Hessenberg reduction meets as tiny pivots and threshold-size
    candidates; the reference's matrix-power traces are indifferent to it.  Choosing s_e (powers
    of two, so the scaling is exact) so that the paired rows e and E + e get equal absolute row
    sums undoes it: a few sweeps of that rule are Parlett-Reinsch balancing of the term matrix
    restricted to pair scalings.  Edges before ``first`` (the batch edge, and in the odd batch
    form the edge of the odd mode, whose unpaired copies would carry the scale) stay unscaled.
    Returns the scaled (Ax, Dx, oddV), or None when every pair's row sums (of the entries'
    moduli) already agree within ``spread`` (the usual case: inputs are then used exactly as
    given)."""
    n = Ax.shape[0]
    E = n // 2
    if E - first < 1:
        return None
    # the early test (the usual outcome) on moduli, within sqrt 2 of |re| + |im|, in plain Python
    # over the pairs: a few microseconds per instance, which the samplers prepare by thousands
    rows = np.abs(Ax).sum(axis=1)
    if Dx is not None:
        rows += np.abs(Dx)
    r = rows.tolist()
    if all(not (r[e] > 0 and r[e + E] > 0) or (r[e] <= spread * r[e + E] and r[e + E] <= spread * r[e])
           for e in range(first, E)):
        return None
    w = np.abs(Ax.real) + np.abs(Ax.imag) if np.iscomplexobj(Ax) else np.abs(Ax)
    if Dx is not None:
        wd = np.abs(Dx.real) + np.abs(Dx.imag) if np.iscomplexobj(Dx) else np.abs(Dx)
        w = np.concatenate([w, wd[:, None]], axis=1)
    k = np.zeros(n, dtype=np.int64)  # log2 of each vertex's scale
    for _ in range(sweeps):
        moved = False
        for i in range(first, E):
            d = np.ldexp(1.0, k)
            dw = d[:, None] * w[:, :n] * d[None, :]
            ra = dw[i].sum() + (d[i] * w[i, n] if Dx is not None else 0.0)
            rb = dw[i + E].sum() + (d[i + E] * w[i + E, n] if Dx is not None else 0.0)
            if ra <= 0 or rb <= 0:
                continue
            step = int(np.round(0.5 * np.log2(rb / ra)))
            if step:
                k[i] += step
                k[i + E] -= step
                moved = True
        if not moved:
            break
    if not np.any(k):
        return None
    d = np.ldexp(1.0, k)
    Ax = d[:, None] * Ax * d[None, :]
    Dx = None if Dx is None else d * Dx
    oddV = None if oddV is None else d * oddV
    return Ax, Dx, oddV


def prepare_hafnian(A, reps=None, glynn=True):
    """Host preparation of ``_haf``: returns a native instance, or a plain value when the
    sieve is not needed (no photons: 1.0; odd photon number: 0.0)."""
    n = A.shape[0]
    reps = [1] * n if reps is None else list(reps)
    N = sum(reps)
    if N == 0:
        return 1.0
    if N % 2 == 1:
        return 0.0
    assert n == len(reps)
    x, edge_reps, _ = matched_reps(reps)
    Ax = _sub(A, x)
    Ax = _cast(Ax, np.complex128 if _is_complex(Ax) else np.float64)
    if not _integer_valued(Ax):  # integer inputs run the exact sieve, which needs no balancing
        bal = _pair_balance(Ax)
        if bal is not None:
            Ax = bal[0]
    return nat.Instance(nat.WG_KIND_PLAIN, Ax, edge_reps, glynn=glynn)


def prepare_loop_hafnian(A, D=None, reps=None, glynn=True):
    """Host preparation of ``loop_hafnian``: native instance or a plain value."""
    n = A.shape[0]
    reps = [1] * n if reps is None else list(reps)
    if D is None:
        D = A.diagonal()
    N = sum(reps)
    if N == 0:
        return 1.0
    if N == 1:
        return D[np.where(np.array(reps) == 1)[0][0]]
    assert n == len(reps)
    assert D.shape[0] == n
    x, edge_reps, oddmode = matched_reps(reps)
    cplx = _is_complex(A, D)
    dt = np.complex128 if cplx else np.float64
    if oddmode is not None:
        oddloop = _cast(D[oddmode], dt)
        oddV = _cast(A[oddmode, x], dt)
    else:
        oddloop, oddV = None, None
    Ax = _cast(_sub(A, x), dt)
    Dx = _cast(np.asarray(D)[x], dt)
    # integer inputs run the exact sieve, which needs no balancing (complex ones cannot)
    if dt == np.complex128 or not _integer_valued(Ax, Dx, oddV, oddloop):
        bal = _pair_balance(Ax, Dx, oddV)
        if bal is not None:
            Ax, Dx, oddV = bal
    return nat.Instance(nat.WG_KIND_LOOP, Ax, edge_reps, glynn=glynn, D=Dx, oddV=oddV, oddloop=oddloop)


# Relative rounding of one sieve term in each term arithmetic (the unit roundoff of its
# significand) and the rule of precision="auto": FP64 first; when AUTO_FACTOR x 2^-53 x
# sum|term| exceeds AUTO_RTOL x |result| the instance runs again in double-double.  The factor
# covers the Hessenberg route's per-term rounding: on the n = 40 benchmark matrices
# (sum|term| / |sum| = 6.8e4 complex, 2.0e5 real) FP64 ends 4.4e-12 and 4.1e-11 from the
# reference's values (0.6 and 1.8 x 2^-53 x cond), on the 40-photon loop hafnian of a 20-mode
# state (3.4e10) 2.2e-6 (0.6x); the first stays FP64, the other two go to double-double.  Over
# 300 loop hafnians of 64-mode Gaussian states with 8-28 photons the error in units of
# 2^-53 x cond is at most 6.3 where cond >= 1e3; larger ratios (up to 85, rounding inside
# single terms) occur only below cond = 100, where the error is below 2e-13.
UNIT_ROUNDOFF = {"fp64": 2.0 ** -53, "df": 2.0 ** -48, "dd": 2.0 ** -104}
AUTO_FACTOR = 8.0
AUTO_RTOL = 1e-10


def run_with_magnitudes(instances, precision="fp64"):
    """Outputs of the instances with, per output, sum |prefactor x term| times the final scale
    (the size of the terms the output cancels from): (values, magnitudes)."""
    plan = nat.Plan(list(instances), precision=precision)
    try:
        plan.execute()
        return plan.read(), plan.read_magnitudes()
    finally:
        plan.close()


def _auto_run(insts):
    """precision="auto": FP64, then double-double for the instances whose FP64 rounding could
    exceed AUTO_RTOL relative (see UNIT_ROUNDOFF)."""
    vals, mags = run_with_magnitudes(insts, "fp64")
    outs = [inst.outputs() for inst in insts]
    redo, off = [], 0
    for k, n_out in enumerate(outs):
        v, m = vals[off:off + n_out], mags[off:off + n_out]
        scale = max(float(np.max(np.abs(v))), 1e-300)
        if AUTO_FACTOR * UNIT_ROUNDOFF["fp64"] * float(np.max(m)) > AUTO_RTOL * scale:
            redo.append((k, off))
        off += n_out
    if redo:
        again = nat.run([insts[k] for k, _ in redo], "dd")
        pos = 0
        for k, o in redo:
            vals[o:o + outs[k]] = again[pos:pos + outs[k]]
            pos += outs[k]
    return vals


def _run(insts, precision):
    if precision == "auto":
        if all(_integral(i) for i in insts) and nat.exact_primes(insts) is not None:
            return nat.run(insts, "exact")
        return _auto_run(insts)
    return nat.run(insts, precision)


def _finish(prep, precision):
    if not isinstance(prep, nat.Instance):
        return prep
    return np.complex128(_run([prep], precision)[0])


def hafnian_with_error(A, loop=False, rtol=1e-05, atol=1e-08, precision="fp64"):
    """(hafnian, error estimate, magnitude): the sieve result with the sum over its terms of
    |prefactor x term| (the magnitude the result cancels from) and the first-order estimate of
    its rounding error, the term arithmetic's unit roundoff times that magnitude (measured FP64
    errors: within ~2x of it on the n = 40 benchmark matrices, within 6.3x on served Gaussian-state
    loop hafnians whose cond exceeds 1e3, up to ~16x on loop hafnians with 66 photons on 4 modes,
    whose terms' own 33-coefficient series cancel).  For a small matrix answered in closed form
    the estimate and magnitude are 0.  ``precision``: "fp64", "df" or "dd"."""
    input_validation(A, rtol=rtol, atol=atol)
    done, value = _closed_form(A, loop, rtol, atol)
    prep = None if done else (prepare_loop_hafnian(A, None, None, True) if loop else prepare_hafnian(A))
    if done or not isinstance(prep, nat.Instance):
        return np.complex128(value if done else prep), 0.0, 0.0
    vals, mags = run_with_magnitudes([prep], precision)
    return np.complex128(vals[0]), float(UNIT_ROUNDOFF[precision] * mags[0]), float(mags[0])


def _haf(A, reps=None, glynn=True, precision=None):
    """Hafnian with optional repeated rows/columns (the reference's ``_haf``)."""
    prep = prepare_hafnian(A, reps, glynn)
    return _finish(prep, _auto(precision, [prep]))


def loop_hafnian(A, D=None, reps=None, glynn=True, precision=None):
    """Loop hafnian with optional repeated rows/columns."""
    prep = prepare_loop_hafnian(A, D, reps, glynn)
    return _finish(prep, _auto(precision, [prep]))


def _closed_form(A, loop, rtol, atol):
    """The reference's special cases of ``hafnian`` (empty, odd, diagonal, n <= 4);
    returns (True, value) or (False, None)."""
    matshape = A.shape
    if matshape == (0, 0):
        return True, 1
    if matshape[0] % 2 != 0 and not loop:
        return True, 0.0
    if _allclose(np.diag(np.diag(A)), A, rtol, atol):
        return True, (np.prod(np.diag(A)) if loop else 0)
    if matshape[0] == 2:
        return True, (A[0, 1] + A[0, 0] * A[1, 1] if loop else A[0][1])
    if matshape[0] == 3 and loop:
        return True, (A[0, 0] * A[1, 2] + A[1, 1] * A[0, 2] + A[2, 2] * A[0, 1]
                      + A[0, 0] * A[1, 1] * A[2, 2])
    if matshape[0] == 4:
        if loop:
            return True, (A[0, 1] * A[2, 3] + A[0, 2] * A[1, 3] + A[0, 3] * A[1, 2]
                          + A[0, 0] * A[1, 1] * A[2, 3] + A[0, 1] * A[2, 2] * A[3, 3]
                          + A[0, 2] * A[1, 1] * A[3, 3] + A[0, 0] * A[2, 2] * A[1, 3]
                          + A[0, 0] * A[3, 3] * A[1, 2] + A[0, 3] * A[1, 1] * A[2, 2]
                          + A[0, 0] * A[1, 1] * A[2, 2] * A[3, 3])
        return True, A[0, 1] * A[2, 3] + A[0, 2] * A[1, 3] + A[0, 3] * A[1, 2]
    return False, None


def _method_glynn(method):
    if method == "glynn":
        return True
    if method == "inclexcl":
        return False
    if method == "recursive":
        raise NotImplementedError("method='recursive' is not part of the GPU sieve path")
    raise ValueError("unknown hafnian method %r" % (method,))


def hafnian(A, loop=False, rtol=1e-05, atol=1e-08, approx=False, num_samples=1000, method="glynn",
            precision=None):
    """Returns the hafnian (or loop hafnian) of a symmetric matrix.

    Args and results as ``thewalrus.hafnian``; ``method`` is "glynn" or "inclexcl" (the loop
    hafnian always uses the finite-difference sieve, as in the reference).  ``precision``:
    None (exact for integer-valued real inputs, FP64 otherwise), "fp64", "df" (double-float
    terms), "dd" (double-double terms: ~14x the FP64 time, for sieve sums whose terms cancel by
    more than ~1e6, e.g. the loop hafnians of many-photon Gaussian-state patterns), "auto"
    (FP64, re-run in double-double when the sum of the terms' magnitudes says FP64 may miss
    1e-10) or "exact" (integer inputs only).
    """
    input_validation(A, rtol=rtol, atol=atol)
    glynn = _method_glynn(method) if not loop else True
    done, value = _closed_form(A, loop, rtol, atol)
    if done:
        return value
    if approx:
        raise NotImplementedError("approx=True (Barvinok sampling) is not part of the GPU sieve path")
    if loop:
        return loop_hafnian(A, D=None, reps=None, glynn=True, precision=precision)
    return _haf(A, reps=None, glynn=glynn, precision=precision)


def hafnian_repeated(A, rpt, mu=None, loop=False, rtol=1e-05, atol=1e-08, glynn=True, precision=None):
    """Hafnian of ``A`` with row/column i repeated ``rpt[i]`` times (``mu``: loop weights)."""
    input_validation(A, atol=atol, rtol=rtol)
    if len(rpt) != len(A):
        raise ValueError("the rpt argument must be 1-dimensional sequence of length len(A).")
    nud = np.array(rpt, dtype=np.int32)
    if not np.all(np.mod(rpt, 1) == 0) or np.any(nud < 0):
        raise ValueError("the rpt argument must contain non-negative integers.")
    if np.all(nud == 0):
        return 1.0
    if np.sum(nud) % 2 != 0 and not loop:
        return 0.0
    if mu is None:
        mu = A.diagonal().copy()
    if _allclose(A, 0, rtol, atol):
        if loop:
            return np.prod(mu**rpt)
        return 0
    if len(mu) != len(A):
        raise ValueError("Length of means vector must be the same length as the matrix A.")
    if loop:
        return loop_hafnian(A, D=mu, reps=rpt, glynn=glynn, precision=precision)
    return _haf(A, reps=rpt, glynn=glynn, precision=precision)


def _batch_edges_even(fixed_edges):
    if len(fixed_edges) == 0:
        return np.array([0, 0], dtype=int)
    fe = [int(v) for v in fixed_edges]
    half = len(fe) // 2
    new = max(fe) + 1
    return np.array([new] + fe[:half] + [new] + fe[half:], dtype=int)


def _batch_edges_odd(fixed_edges, oddmode):
    if len(fixed_edges) == 0:
        return np.array([1, oddmode, 1, 1], dtype=int)
    fe = [int(v) for v in fixed_edges]
    half = len(fe) // 2
    new = max(max(fe), int(oddmode)) + 1
    return np.array([new, oddmode] + fe[:half] + [new, new] + fe[half:], dtype=int)


def prepare_loop_hafnian_batch(A, D, fixed_reps, N_cutoff, glynn=True):
    """Host preparation of ``loop_hafnian_batch`` (loop_hafnian_batch.py:275-304)."""
    n = A.shape[0]
    assert A.shape[1] == n
    assert D.shape == (n,)
    assert len(fixed_reps) == n - 1
    nz = np.nonzero(list(fixed_reps) + [1])[0]
    Anz = _sub(A, nz)
    Dnz = D[nz]
    fixed_reps = np.asarray(fixed_reps)
    fixed_reps_nz = fixed_reps[nz[:-1]]
    fixed_edges, fixed_m_reps, oddmode = matched_reps(fixed_reps_nz)
    dt = np.complex128 if _is_complex(A, D) else np.float64
    if oddmode is None:
        batch_max, cutoff, kind = N_cutoff // 2, N_cutoff % 2, nat.WG_KIND_BATCH_EVEN
        edges = _batch_edges_even(fixed_edges)
    else:
        batch_max, cutoff, kind = (N_cutoff - 1) // 2, 1 - (N_cutoff % 2), nat.WG_KIND_BATCH_ODD
        edges = _batch_edges_odd(fixed_edges, oddmode)
    Ax = _cast(_sub(Anz, edges), dt)
    Dx = _cast(Dnz[edges], dt)
    # the batch edge (and the odd mode's edge) stay unscaled; integer inputs run the exact sieve
    if dt == np.complex128 or not _integer_valued(Ax, Dx):
        bal = _pair_balance(Ax, Dx, first=1 if oddmode is None else 2)
        if bal is not None:
            Ax, Dx = bal[0], bal[1]
    return nat.Instance(kind, Ax, fixed_m_reps, glynn=glynn, D=Dx, batch_max=batch_max, cutoff=cutoff)


def loop_hafnian_batch(A, D, fixed_reps, N_cutoff, glynn=True, precision=None):
    """Loop hafnians for every photon number 0..N_cutoff of the last mode, in one sieve."""
    prep = prepare_loop_hafnian_batch(A, D, fixed_reps, N_cutoff, glynn)
    return _run([prep], _auto(precision, [prep]))


def prepare_loop_hafnian_batch_gamma(A, D, fixed_reps, N_cutoff, glynn=True):
    """Host preparation of ``loop_hafnian_batch_gamma`` (loop_hafnian_batch_gamma.py:222-269).

    D holds one displacement vector per row.  The reference's inner loop over rows k
    (loop_hafnian_batch_gamma.py:99-117 and :181-205) evaluates, for each k, exactly the
    ``loop_hafnian_batch`` sum with D[k] (self-loop weights D[k, 0] and D[k, 1], the same
    AX_S and oddV), so each row becomes one batch instance; all rows run in one plan.
    """
    D = np.asarray(D)
    n = A.shape[0]
    assert A.shape[1] == n
    assert D.ndim == 2 and D.shape[1] == n
    assert len(fixed_reps) == n - 1
    return [prepare_loop_hafnian_batch(A, D[k], fixed_reps, N_cutoff, glynn) for k in range(D.shape[0])]


def loop_hafnian_batch_gamma(A, D, fixed_reps, N_cutoff, glynn=True, precision=None):
    """Loop hafnians for every photon number 0..N_cutoff of the last mode, for each row of D
    (threshold-detector sampling); returns an array of shape (len(D), N_cutoff + 1)."""
    preps = prepare_loop_hafnian_batch_gamma(A, D, fixed_reps, N_cutoff, glynn)
    if not preps:
        return np.zeros((0, N_cutoff + 1), dtype=np.complex128)
    vals = _run(preps, _auto(precision, preps))
    return vals.reshape(len(preps), -1)


def hafnian_batch(matrices, loop=False, rtol=1e-05, atol=1e-08, method="glynn", precision=None,
                  validate=True):
    """Hafnians of many matrices of uneven size in one persistent launch per arithmetic class.

    Each result equals ``hafnian(M, loop=loop, method=method)``.  Instances that the reference
    answers in closed form are answered the same way on the host; all others share one plan.
    """
    results = [None] * len(matrices)
    insts, where = [], []
    for i, A in enumerate(matrices):
        if validate:
            input_validation(A, rtol=rtol, atol=atol)
        glynn = _method_glynn(method) if not loop else True
        done, value = _closed_form(A, loop, rtol, atol)
        if done:
            results[i] = value
            continue
        prep = prepare_loop_hafnian(A, None, None, True) if loop else prepare_hafnian(A, None, glynn)
        if isinstance(prep, nat.Instance):
            insts.append(prep)
            where.append(i)
        else:
            results[i] = prep
    if insts:
        vals = _run(insts, _auto(precision, insts))
        for i, v in zip(where, vals):
            results[i] = np.complex128(v)
    return results
