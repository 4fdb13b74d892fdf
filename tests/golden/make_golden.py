"""Generate golden input/output vectors from the reference implementation itself.

Usage::

    python tests/golden/make_golden.py REFERENCE_CHECKOUT            # small cases
    python tests/golden/make_golden.py REFERENCE_CHECKOUT --metric   # benchmark-size cases
    python tests/golden/make_golden.py --metric-oracle   # re-run only their oracle cross-check

``REFERENCE_CHECKOUT`` is a source checkout of thewalrus (the directory holding the
``thewalrus`` package); the environment variable ``WALRUS_REFERENCE`` may give it instead.
numba is not needed: a stub module turns ``numba.jit`` into the identity and ``numba.prange``
into ``range``, so the reference's own Python code runs as plain NumPy.  The package
``__init__`` (which pulls in dask) is bypassed by registering a bare ``thewalrus`` package whose
path is the reference's source directory.

``--metric`` evaluates the benchmark-size inputs (the 40x40 complex and real plain hafnians,
seed 0, and the 20-mode, 40-photon Gaussian-state loop hafnian) through the reference's public
``hafnian`` / ``hafnian_repeated``.  Single-threaded that is ~1 ms per sieve term (524,288 terms
for n = 40), so the work is split over processes: in each worker the stub's ``prange(steps)``
yields only one slice of the term range, the reference's own ``_calc_hafnian`` /
``_calc_loop_hafnian`` sum that slice (their result is linear in the sum: the final
``0.5 ** (N/2 - 1)`` scale applies to each slice alike) and the slices' results are added in
term order with ``math.fsum``.  Output: ``metric_cases.npz``.

One reference quirk is guarded: ``charpoly.powertrace`` of a 0x0 matrix indexes an empty array
(thewalrus/charpoly.py:215-217); the guard returns the values the reference's loops produce
around that read (p_0 = 0 followed by zeros).

Output of the default mode: ``reference_cases.npz`` next to this script.  Keys are
``<family>/<index>/<field>``.
"""
import math
import multiprocessing as mp
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from thewalrus_gb300 import workloads as wl  # noqa: E402


_IMPORTED = {}


def import_reference(path):
    if path in _IMPORTED:
        return _IMPORTED[path]

    def mk(name):
        m = types.ModuleType(name)
        m.__path__ = []
        sys.modules[name] = m
        return m

    stub = mk("numba")

    def jit(*args, **kwargs):
        if args and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    stub.jit = jit
    stub.njit = jit
    stub.prange = range
    # the quantum package imports a numba tuple helper and dask; plain-Python stand-ins suffice
    mk("numba.cpython")
    mk("numba.cpython.unsafe")
    mk("numba.cpython.unsafe.tuple").tuple_setitem = lambda t, i, v: t[:i] + (v,) + t[i + 1:]
    dask = mk("dask")
    dask.delayed = lambda f: f
    pkg = types.ModuleType("thewalrus")
    pkg.__path__ = [os.path.join(path, "thewalrus")]
    sys.modules["thewalrus"] = pkg
    import thewalrus.quantum  # noqa: F401  (resolves the quantum <-> decompositions import cycle)
    import thewalrus.charpoly as cp
    import thewalrus._hafnian as hf
    import thewalrus.loop_hafnian_batch as lb
    import thewalrus.reference as ref
    import thewalrus._hermite_multidimensional as hm

    for name in ("hafnian", "hafnian_repeated", "reduction"):
        setattr(pkg, name, getattr(hf, name))
    for name in dir(hm):
        if not name.startswith("_"):
            setattr(pkg, name, getattr(hm, name))

    orig = cp.powertrace

    def guarded(H, n):
        if len(H) == 0:
            return np.zeros(n + 2, dtype=H.dtype)
        return orig(H, n)

    cp.powertrace = guarded
    _IMPORTED[path] = (cp, hf, lb, ref)
    return cp, hf, lb, ref


def _slice_worker(args):
    """Evaluate one slice [p/P, (p+1)/P) of the reference's sieve loop through its public API."""
    path, case, piece, pieces = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    cp, hf, lb, ref = import_reference(path)

    def prange(steps):
        return range(steps * piece // pieces, steps * (piece + 1) // pieces)

    # the reference modules keep the numba stub they were imported with (a worker process runs
    # several slices), so patch that module object
    hf.numba.prange = prange
    kind, A, extra = case
    if kind == "haf":
        val = hf.hafnian(A)
    else:
        rpt, mu = extra
        val = hf.hafnian_repeated(A, list(rpt), mu=mu, loop=True)
    return piece, complex(val)


def metric_cases(path, workers=None, pieces=256):
    """Benchmark-size reference values (see the module docstring), split over processes."""
    cases = {
        "haf40_complex": ("haf", wl.complex_symmetric(40, seed=0), None),
        "haf40_real": ("haf", wl.real_signed(40, seed=0), None),
    }
    A, gamma, rpt = wl.gaussian_state_loop(modes=20, seed=1, photons=40, max_rep=3)
    cases["lhaf_state20_40"] = ("lhaf", A, (rpt, gamma))
    workers = workers or os.cpu_count()
    out = {}
    ctx = mp.get_context("spawn")
    for name, case in cases.items():
        t0 = time.time()
        with ctx.Pool(workers) as pool:
            parts = sorted(pool.map(_slice_worker, [(path, case, p, pieces) for p in range(pieces)]))
        val = complex(math.fsum(v.real for _, v in parts), math.fsum(v.imag for _, v in parts))
        kind, A, extra = case
        out[name + "/A"] = A
        if extra is not None:
            out[name + "/rpt"] = np.asarray(extra[0])
            out[name + "/mu"] = np.asarray(extra[1])
        out[name + "/out"] = np.asarray(val)
        print("%s = %r (%.0f s on %d processes)" % (name, val, time.time() - t0, workers), flush=True)
    np.savez_compressed(os.path.join(HERE, "metric_cases.npz"), **out)
    metric_oracle_check()


def metric_oracle_check():
    """Cross-check of ``metric_cases.npz`` with the oracle, adding per case (fields already
    present are kept):

    * ``oracle_ld``: the long-double oracle's value (x87 80-bit on x86-64);
    * ``cond``: the sieve sum's condition number sum|term| / |sum| (double oracle), the factor
      by which per-term rounding reaches the result;
    * ``oracle_q``: the _Float128 oracle's value, for the cases whose ``cond`` exceeds 1e6 (there
      even the long-double result has only ~1e-19 * cond relative accuracy).
    """
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import oracle
    import thewalrus_gb300 as tw

    path = os.path.join(HERE, "metric_cases.npz")
    data = dict(np.load(path))
    for name in sorted({k.split("/")[0] for k in data}):
        A = data[name + "/A"]
        ref = complex(data[name + "/out"])
        loop = name + "/rpt" in data

        def value(precision):
            if loop:
                return complex(oracle.hafnian_repeated(A, list(data[name + "/rpt"]), mu=data[name + "/mu"],
                                                       loop=True, precision=precision))
            return complex(oracle.hafnian(A, precision=precision))

        if name + "/cond" not in data:
            t0 = time.time()
            if loop:
                p = tw.prepare_loop_hafnian(A, data[name + "/mu"], list(data[name + "/rpt"]))
                tot = oracle.sieve_term_range(p.A, p.reps, Dx=p.D, absolute=True)
                N = int(2 * np.sum(p.reps))
            else:
                p = tw.prepare_hafnian(A)
                tot = oracle.sieve_term_range(p.A, p.reps, absolute=True)
                N = int(2 * np.sum(p.reps))
            cond = complex(tot).real * 0.5 ** (N // 2 - 1) / abs(ref)
            data[name + "/cond"] = np.asarray(cond)
            print("%s: condition number %.3g (%.0f s)" % (name, cond, time.time() - t0), flush=True)
        for key, precision in (("oracle_ld", "long"), ("oracle_q", "quad")):
            if name + "/" + key in data or (key == "oracle_q" and float(data[name + "/cond"]) <= 1e6):
                continue
            t0 = time.time()
            val = value(precision)
            data[name + "/" + key] = np.asarray(val)
            print("%s: oracle (%s) %r, relative difference from the reference %.2e (%.0f s)"
                  % (name, precision, val, abs(val - ref) / abs(ref), time.time() - t0), flush=True)
            np.savez_compressed(path, **data)
    np.savez_compressed(path, **data)


def reference_path(argv):
    args = [a for a in argv if not a.startswith("--")]
    path = args[0] if args else os.environ.get("WALRUS_REFERENCE")
    if not path:
        raise SystemExit("usage: make_golden.py REFERENCE_CHECKOUT [--metric] "
                         "(or set WALRUS_REFERENCE)")
    return path


def main(path):
    cp, hf, lb, ref = import_reference(path)
    rng = np.random.default_rng(20261203)
    out = {}
    counts = {}

    def put(family, **fields):
        i = counts.get(family, 0)
        counts[family] = i + 1
        for k, v in fields.items():
            out["%s/%d/%s" % (family, i, k)] = np.asarray(v)

    t0 = time.time()
    # plain hafnian through the public API (method="glynn")
    for n in (6, 8, 10, 12, 14, 16, 18, 20):
        A = wl.complex_symmetric(n, seed=100 + n)
        put("haf", A=A, out=hf.hafnian(A))
    for n in (6, 10, 14, 16):
        A = wl.real_signed(n, seed=200 + n)
        put("haf", A=A, out=hf.hafnian(A))
    for n in (8, 12, 16):
        A = wl.real_nonneg(n, seed=300 + n)
        put("haf", A=A, out=hf.hafnian(A))
    for n in (10, 16):
        A = wl.adjacency01(n, seed=400 + n)
        put("haf", A=A, out=hf.hafnian(A))
    A = np.ones((12, 12), dtype=np.int64)
    put("haf", A=A, out=hf.hafnian(A))
    # the 24x24 plain-hafnian workload (seed 0) and the all-ones 24x24 matrix
    A = wl.complex_symmetric(24, seed=0)
    put("haf", A=A, out=hf.hafnian(A))
    A = np.ones((24, 24))
    put("haf", A=A, out=hf.hafnian(A))
    # inclusion/exclusion variant
    for n in (8, 12):
        A = wl.complex_symmetric(n, seed=500 + n)
        put("haf_inclexcl", A=A, out=hf.hafnian(A, method="inclexcl"))

    # loop hafnian through the public API
    for n in (5, 6, 7, 8, 9, 11, 12, 15, 16):
        A = wl.complex_symmetric(n, seed=600 + n)
        put("lhaf", A=A, out=hf.hafnian(A, loop=True))
    for n in (6, 9, 14):
        A = wl.real_signed(n, seed=700 + n)
        put("lhaf", A=A, out=hf.hafnian(A, loop=True))

    # hafnian_repeated, plain and loop, random repetitions 0..3
    for case in range(14):
        n = int(rng.integers(2, 8))
        A = wl.complex_symmetric(n, seed=800 + case)
        rpt = rng.integers(0, 4, size=n)
        if rpt.sum() == 0:
            rpt[0] = 2
        mu = (rng.normal(size=n) + 1j * rng.normal(size=n)) * 0.5
        if rpt.sum() % 2 == 0:
            put("rep", A=A, rpt=rpt, out=hf.hafnian_repeated(A, list(rpt)))
        put("rep_loop", A=A, rpt=rpt, mu=mu,
            out=hf.hafnian_repeated(A, list(rpt), mu=mu, loop=True))
    # repeated edges that produce all-zero deltas (0x0 term matrices)
    A = np.array([[1.0]])
    put("rep", A=A, rpt=np.array([12]), out=hf.hafnian_repeated(A, [12]))
    A = np.array([[0.0, 1.0], [1.0, 0.0]], dtype=np.complex128)
    put("rep", A=A, rpt=np.array([6, 6]), out=hf.hafnian_repeated(A, [6, 6]))

    # the loop-hafnian Gaussian-state workload at reduced size: 6 modes, 12 photons
    A, gamma, rpt = wl.gaussian_state_loop(modes=6, seed=1, photons=12, max_rep=3)
    put("rep_loop", A=A, rpt=rpt, mu=gamma,
        out=hf.hafnian_repeated(A, list(rpt), mu=gamma, loop=True))

    # loop_hafnian_batch: even and odd pairing paths
    for case in range(8):
        modes = int(rng.integers(3, 7))
        calls = wl.batch_loop_calls(count=1, seed=900 + case, modes=modes,
                                    cutoff=int(rng.integers(2, 7)), max_fixed=2)
        B, D, fixed, cutoff = calls[0]
        put("batch", A=B, D=D, fixed=fixed, cutoff=cutoff,
            out=lb.loop_hafnian_batch(B, D, fixed, cutoff))

    # loop_hafnian_batch_gamma (threshold-detector batches): several displacement rows
    import thewalrus.loop_hafnian_batch_gamma as lbg

    for case in range(6):
        modes = int(rng.integers(3, 7))
        calls = wl.batch_loop_calls(count=1, seed=950 + case, modes=modes,
                                    cutoff=int(rng.integers(1, 5)), max_fixed=2)
        B, D0, fixed, cutoff = calls[0]
        nD = int(rng.integers(2, 5))
        D = np.array([D0 - k * 0.3 * B[:, -1] for k in range(nD)])
        put("batch_gamma", A=B, D=D, fixed=fixed, cutoff=cutoff,
            out=lbg.loop_hafnian_batch_gamma(B, D, fixed, cutoff))

    # brute-force matchings from thewalrus/reference.py for small n
    for n in (4, 6, 8):
        A = wl.complex_symmetric(n, seed=1000 + n)
        put("brute", A=A, loop=False, out=ref.hafnian(A))
    for n in (3, 5, 7):
        A = wl.complex_symmetric(n, seed=1100 + n)
        put("brute", A=A, loop=True, out=ref.hafnian(A, loop=True))

    # charpoly.powertrace: matmul branch (n <= m) and La Budde branch (n > m)
    for m, n in ((4, 3), (4, 7), (6, 4), (6, 9), (8, 12)):
        H = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        put("ptrace", H=H, n=n, out=cp.powertrace(H.copy(), n))
    for m in (2, 5, 9):
        H = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        put("charpoly", H=H, out=np.array(cp.charpoly(H.copy())))

    # pure-state Fock amplitudes (thewalrus/quantum/fock_tensors.py:45-98) of a displaced,
    # squeezed 6-mode state: cov = S S^T with S = interferometer(U) squeezing(r), hbar = 2
    import thewalrus.symplectic as sy
    from thewalrus.quantum.fock_tensors import pure_state_amplitude

    M = 6
    U = wl.haar_unitary(M, np.random.default_rng(41))
    r = np.random.default_rng(42).uniform(0.3, 0.8, size=M)
    S = sy.interferometer(U) @ sy.squeezing(r)
    cov = S @ S.T
    mu = np.random.default_rng(43).normal(size=2 * M) * 0.4
    for case in range(10):
        pat = rng.integers(0, 3, size=M)
        if pat.sum() < 2:
            pat[0] += 2
        put("pure", mu=mu, cov=cov, pattern=pat, out=pure_state_amplitude(mu, cov, list(pat)))

    # Gaussian boson sampling (thewalrus/samples.py): a pure and a mixed 5-mode state; samples
    # for fixed np.random seeds, plus the decomposition the samplers start from
    import thewalrus.samples as smp
    from thewalrus.quantum.conversions import Amat

    M = 5
    U = wl.haar_unitary(M, np.random.default_rng(51))
    r = np.random.default_rng(52).uniform(0.5, 0.9, size=M)
    S = sy.interferometer(U) @ sy.squeezing(r)
    pure = S @ S.T
    mixed = 0.7 * pure + 0.3 * np.eye(2 * M) * 1.4
    mean = np.random.default_rng(53).normal(size=2 * M) * 0.3
    for name, cov in (("pure", pure), ("mixed", mixed)):
        # the samplers decompose the covariance with the modes re-ordered by mean photon number
        order = smp.photon_means_order(mean, cov)
        oo = np.concatenate((order, order + M))
        cov_r = cov[np.ix_(oo, oo)]
        T, sqrtW = smp.decompose_cov(cov_r)
        put("gbs_decomp", cov=cov, mean=mean, order=order, cov_ordered=cov_r, T=T, sqrtW=sqrtW,
            B=Amat(T)[:M, :M])
        for seed, (cutoff, maxp, count) in enumerate(((6, 12, 6), (4, 30, 5))):
            np.random.seed(1000 + seed)
            samples = smp.hafnian_sample_state(cov, count, mean=mean, cutoff=cutoff, max_photons=maxp)
            put("gbs_hafnian", cov=cov, mean=mean, seed=1000 + seed, cutoff=cutoff, max_photons=maxp,
                count=count, out=samples, next_uniform=np.random.random_sample())
        np.random.seed(77)
        samples = smp.torontonian_sample_state(cov, 4, mu=mean, fanout=4, cutoff=1, max_photons=30)
        put("gbs_threshold", cov=cov, mean=mean, seed=77, fanout=4, cutoff=1, max_photons=30, count=4,
            out=samples, next_uniform=np.random.random_sample())

    # graph states (quantum/adjacency_matrices.py, conversions.py): scaling, Q and covariance
    from thewalrus.quantum import adj_scaling, gen_Qmat_from_graph, Covmat
    grng = np.random.default_rng(61)
    for n, n_mean, weighted in ((6, 2.0, False), (8, 5.0, True), (5, 0.7, True)):
        G = np.triu((grng.random((n, n)) < 0.5).astype(float), 1)
        if weighted:
            G = G * grng.uniform(0.2, 1.5, size=(n, n))
        A = G + G.T
        Q = gen_Qmat_from_graph(A, n_mean)
        put("graph", A=A, n_mean=n_mean, scale=adj_scaling(A, n_mean), Q=Q, cov=Covmat(Q))

    # density-matrix elements of mixed, displaced and undisplaced states (fock_tensors.py:191-232)
    from thewalrus.quantum import density_matrix_element
    drng = np.random.default_rng(71)
    M = 3
    U = wl.haar_unitary(M, np.random.default_rng(72))
    S = sy.interferometer(U) @ sy.squeezing(drng.uniform(0.2, 0.6, size=M))
    for k, (thermal, disp) in enumerate(((0.0, 0.0), (0.4, 0.0), (0.4, 0.5), (0.0, 0.5))):
        cov = S @ S.T + thermal * np.eye(2 * M)
        mu = drng.normal(size=2 * M) * disp
        for i, j in (([1, 0, 1], [1, 0, 1]), ([2, 1, 0], [0, 1, 2]), ([0, 0, 0], [1, 1, 0]), ([3, 0, 1], [1, 2, 1])):
            put("dm", mu=mu, cov=cov, i=np.array(i), j=np.array(j), out=density_matrix_element(mu, cov, i, j))

    np.savez_compressed(os.path.join(HERE, "reference_cases.npz"), **out)
    print("wrote %d arrays for %s in %.1fs" % (len(out), counts, time.time() - t0))


if __name__ == "__main__":
    if "--metric-oracle" in sys.argv[1:]:
        metric_oracle_check()
    elif "--metric" in sys.argv[1:]:
        metric_cases(reference_path(sys.argv[1:]))
    else:
        main(reference_path(sys.argv[1:]))
