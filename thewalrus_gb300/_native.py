"""Build and load the native library ``libwalrus_gb300.so`` (CUDA, sm_103a) through ctypes.

The library is compiled in-tree into ``thewalrus_gb300/_build/`` with nvcc.  There is no CPU
fallback: every computing entry point fails with ``RuntimeError`` when no GPU is usable.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libwalrus_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["sieve.cu", "noalloc.cu", "kernels_c64.cu", "kernels_cdf.cu", "kernels_f64.cu", "kernels_fdf.cu",
           "kernels_cdd.cu", "kernels_fdd.cu", "kernels_mod0.cu", "kernels_mod1.cu", "kernels_mod2.cu",
           "kernels_mod3.cu", "kernels_mod4.cu"]
DEPS = SOURCES + ["sieve_kernel.cuh", "arith.cuh", "host_common.h", "kernels.h", "kernels_unit.cuh",
                  "state_glue.cuh"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-shared"]

WG_FLOAT64, WG_COMPLEX128 = 0, 1
WG_PREC_FP64, WG_PREC_DF, WG_PREC_DD = 0, 1, 7
WG_PREC_MOD = (2, 3, 4, 5, 6)
MOD_PRIMES = (2147483647, 2147483629, 2147483587, 2147483579, 2147483563)
WG_KIND_PLAIN, WG_KIND_LOOP, WG_KIND_BATCH_EVEN, WG_KIND_BATCH_ODD = 0, 1, 3, 4
PRECISIONS = {"fp64": WG_PREC_FP64, "df": WG_PREC_DF, "dd": WG_PREC_DD}
PRECISIONS.update({"mod%d" % k: v for k, v in enumerate(WG_PREC_MOD)})

_lock = threading.Lock()
_lib = None


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in DEPS] + [os.path.join(INCLUDE, "walrus_gb300.h")]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force=False, verbose=False):
    """Compile the CUDA library for sm_103a if it is missing or older than its sources."""
    with _lock:
        if not force and not _stale():
            return LIB
        os.makedirs(BUILD, exist_ok=True)
        tag = "%d" % os.getpid()
        compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]
        procs, objs = [], []
        tmp = LIB + ".tmp" + tag
        try:
            for src in SOURCES:  # translation units compile in parallel, then one link
                obj = os.path.join(BUILD, src.replace(".cu", ".%s.o" % tag))
                cmd = [_nvcc()] + compile_flags + ["-c", os.path.join(CSRC, src), "-o", obj]
                procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
                objs.append(obj)
            failed = None
            for cmd, p in procs:  # wait for every compiler before reporting the first failure
                out, _ = p.communicate()
                if p.returncode != 0 and failed is None:
                    failed = "nvcc failed:\n%s\n%s" % (" ".join(cmd), out.decode())
                elif verbose and out:
                    print(out.decode())
            if failed:
                raise RuntimeError(failed)
            cmd = [_nvcc(), "-shared", "-o", tmp] + objs
            res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if res.returncode != 0:
                raise RuntimeError("nvcc link failed:\n%s\n%s" % (" ".join(cmd), res.stdout.decode()))
            os.replace(tmp, LIB)
        finally:  # no object or half-written library outlives the build, failed or not
            for _, p in procs:  # compilers still running after an early exit (a Popen that raised)
                if p.poll() is None:
                    p.kill()
                    p.wait()
            for path in objs + [tmp]:
                if os.path.exists(path):
                    os.unlink(path)
        return LIB


class WgInstance(ctypes.Structure):
    """Mirror of ``wg_instance`` in include/walrus_gb300.h."""

    _fields_ = [
        ("kind", ctypes.c_int32),
        ("n", ctypes.c_int32),
        ("E", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("glynn", ctypes.c_int32),
        ("has_odd", ctypes.c_int32),
        ("batch_max", ctypes.c_int32),
        ("cutoff", ctypes.c_int32),
        ("edge_reps", ctypes.c_void_p),
        ("A", ctypes.c_void_p),
        ("D", ctypes.c_void_p),
        ("oddV", ctypes.c_void_p),
        ("oddloop", ctypes.c_double * 2),
        ("term_begin", ctypes.c_int64),
        ("term_end", ctypes.c_int64),
    ]


EXPORTS = [
    "wg_init", "wg_last_error", "wg_instance_outputs", "wg_hafnian", "wg_loop_hafnian",
    "wg_loop_hafnian_batch", "wg_plan_create", "wg_plan_create_ex", "wg_plan_execute", "wg_plan_read", "wg_plan_outputs",
    "wg_plan_kernel_launches", "wg_plan_partials", "wg_plan_chunk", "wg_plan_transfer_bytes",
    "wg_plan_destroy", "wg_run",
    "wg_measure_fp_peaks", "wg_hafnian_noalloc", "wg_state_create", "wg_state_destroy",
    "wg_plan_create_requests", "wg_plan_device_bytes", "wg_instance_terms", "wg_state_create_from_cov",
    "wg_check_arith", "wg_plan_read_magnitudes",
]


class WgRequest(ctypes.Structure):
    """Mirror of ``wg_request``."""

    _fields_ = [
        ("x", ctypes.c_void_p),
        ("edge_reps", ctypes.c_void_p),
        ("E", ctypes.c_int32),
        ("oddmode", ctypes.c_int32),
    ]


def load(build_if_needed=True):
    """Load the library (building it first if needed) and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        build()
    if not os.path.exists(LIB):
        raise RuntimeError("libwalrus_gb300.so is missing; run thewalrus_gb300._native.build()")
    lib = ctypes.CDLL(LIB)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
    i32 = ctypes.c_int
    lib.wg_init.argtypes = [i32]
    lib.wg_last_error.restype = ctypes.c_char_p
    lib.wg_instance_outputs.argtypes = [ctypes.POINTER(WgInstance)]
    lib.wg_instance_terms.argtypes = [ctypes.POINTER(WgInstance)]
    lib.wg_instance_terms.restype = ctypes.c_longlong
    lib.wg_hafnian.argtypes = [vp, i32, i32, ip, i32, i32, i32, dp, vp]
    lib.wg_loop_hafnian.argtypes = [vp, vp, i32, i32, ip, i32, i32, dp, vp, i32, i32, dp, vp]
    lib.wg_loop_hafnian_batch.argtypes = [vp, vp, i32, i32, ip, i32, i32, i32, i32, i32, i32, dp, vp]
    lib.wg_plan_create.argtypes = [ctypes.POINTER(WgInstance), i32, i32, ctypes.c_double,
                                   ctypes.POINTER(vp)]
    lib.wg_plan_create_ex.argtypes = [ctypes.POINTER(WgInstance), i32, i32, ctypes.POINTER(WgPlanOptions),
                                      ctypes.POINTER(vp)]
    lib.wg_plan_execute.argtypes = [vp, vp]
    lib.wg_plan_read.argtypes = [vp, dp, vp]
    lib.wg_plan_read_magnitudes.argtypes = [vp, dp, vp]
    lib.wg_plan_outputs.argtypes = [vp]
    lib.wg_plan_kernel_launches.argtypes = [vp]
    lib.wg_plan_transfer_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    lib.wg_plan_partials.argtypes = [vp, dp, i32, vp]
    lib.wg_plan_chunk.argtypes = [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                  ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    lib.wg_plan_destroy.argtypes = [vp]
    lib.wg_run.argtypes = [ctypes.POINTER(WgInstance), i32, i32, dp, vp]
    lib.wg_measure_fp_peaks.argtypes = [dp, dp]
    lib.wg_check_arith.argtypes = [i32, dp, i32, dp]
    lib.wg_hafnian_noalloc.argtypes = [vp, i32, i32, ip, i32, i32, vp, vp]
    lib.wg_state_create.argtypes = [dp, dp, i32, ctypes.POINTER(vp)]
    lib.wg_state_create_from_cov.argtypes = [dp, dp, i32, ctypes.c_double, ctypes.POINTER(vp), dp, dp, dp]
    lib.wg_state_destroy.argtypes = [vp]
    lib.wg_plan_create_requests.argtypes = [vp, ctypes.POINTER(WgRequest), i32, i32,
                                            ctypes.POINTER(WgPlanOptions), ctypes.POINTER(vp)]
    lib.wg_plan_device_bytes.argtypes = [vp]
    lib.wg_plan_device_bytes.restype = ctypes.c_longlong
    _lib = lib
    return lib


def check(rc):
    """Raise ``RuntimeError`` with the library's message on a nonzero status."""
    if rc != 0:
        msg = load(False).wg_last_error().decode(errors="replace")
        raise RuntimeError("walrus_gb300 error %d: %s" % (rc, msg))


class Instance:
    """A prepared sieve problem that keeps its NumPy buffers alive for the ctypes struct."""

    def __init__(self, kind, A, edge_reps, glynn=True, D=None, oddV=None, oddloop=None,
                 batch_max=0, cutoff=0):
        A = np.asarray(A)
        cplx = any(x is not None and np.asarray(x).dtype.kind == "c" for x in (A, D, oddV, oddloop))
        dt = np.complex128 if cplx else np.float64
        self.A = np.ascontiguousarray(A, dtype=dt)
        self.reps = np.ascontiguousarray(np.asarray(edge_reps, dtype=np.int64).reshape(-1))
        self.D = None if D is None else np.ascontiguousarray(np.asarray(D).reshape(-1), dtype=dt)
        self.oddV = None if oddV is None else np.ascontiguousarray(np.asarray(oddV).reshape(-1), dtype=dt)
        s = WgInstance()
        s.kind = kind
        s.n = self.A.shape[0] if self.A.ndim == 2 else 0
        s.E = len(self.reps)
        s.dtype = WG_COMPLEX128 if cplx else WG_FLOAT64
        s.glynn = 1 if glynn else 0
        s.has_odd = 1 if oddloop is not None and kind == WG_KIND_LOOP else 0
        s.batch_max = int(batch_max)
        s.cutoff = int(cutoff)
        s.edge_reps = self.reps.ctypes.data if len(self.reps) else None
        s.A = self.A.ctypes.data if self.A.size else None
        s.D = None if self.D is None else self.D.ctypes.data
        s.oddV = None if self.oddV is None else self.oddV.ctypes.data
        if oddloop is not None:
            z = complex(oddloop)
            s.oddloop[0], s.oddloop[1] = z.real, z.imag
        self.struct = s

    def log2_bound(self):
        """log2 of a bound on |output|: the expanded matrix (each edge end repeated rep times,
        loop weights on the diagonal) has haf^2 <= per <= prod of absolute row sums."""
        s = self.struct
        n = self.A.shape[0] if self.A.ndim == 2 else 0
        if n == 0:
            return 0.0
        reps = list(self.reps)
        if s.kind in (WG_KIND_BATCH_EVEN, WG_KIND_BATCH_ODD):  # the batch ends carry batch_max + cutoff
            extra = [s.batch_max + s.cutoff + 1] + ([1] if s.kind == WG_KIND_BATCH_ODD else [])
            reps = extra + reps
        E = len(reps)
        mult = np.array([reps[i % E] for i in range(n)], dtype=np.float64) if E else np.ones(n)
        absA = np.abs(np.real(self.A)) + np.abs(np.imag(self.A))
        rows = absA @ mult
        if self.D is not None:
            rows = rows + np.abs(self.D)
        if s.has_odd and self.oddV is not None:
            rows = rows + np.abs(self.oddV) + abs(complex(s.oddloop[0], s.oddloop[1]))
        rows = np.maximum(rows, 1.0)
        return float(0.5 * np.sum(mult * np.log2(rows))) + 1.0

    def terms(self):
        """Number of sieve terms (the range that ``shard`` partitions)."""
        n = load().wg_instance_terms(ctypes.byref(self.struct))
        if n < 0:
            check(int(n))
        return int(n)

    def shard(self, begin, end):
        """A copy restricted to sieve terms [begin, end) (non-empty); its outputs are that
        shard's share of the result, so the shards of a partition of [0, terms()) sum to the
        full outputs."""
        if not 0 <= begin < end:
            raise ValueError("a shard needs 0 <= begin < end (got [%d, %d))" % (begin, end))
        other = Instance.__new__(Instance)
        other.__dict__.update(self.__dict__)
        other.struct = WgInstance.from_buffer_copy(self.struct)
        other.struct.term_begin, other.struct.term_end = int(begin), int(end)
        return other

    def outputs(self):
        if self.struct.kind == WG_KIND_BATCH_EVEN:
            return 2 * self.struct.batch_max + self.struct.cutoff + 1
        if self.struct.kind == WG_KIND_BATCH_ODD:
            return 2 * self.struct.batch_max + self.struct.cutoff + 2
        return 1


class WgPlanOptions(ctypes.Structure):
    """Mirror of ``wg_plan_options``."""

    _fields_ = [
        ("chunk_scale", ctypes.c_double),
        ("max_warps_per_cta", ctypes.c_int32),
        ("merge_classes", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("serial_groups", ctypes.c_int32),
        ("stream", ctypes.c_void_p),
    ]


class Plan:
    """Device-resident batch of instances: create once, execute many times, read results.

    ``chunk_scale`` (term-chunk size), ``max_warps_per_cta``, ``merge_classes`` (one persistent
    launch per scalar type), ``use_graph`` (CUDA-graph replay) and ``serial_groups`` (launch the
    groups one after another on the caller's stream) map to ``wg_plan_options``.
    """

    def __init__(self, instances, precision="fp64", chunk_scale=1.0, max_warps_per_cta=0,
                 merge_classes=False, use_graph=False, serial_groups=False):
        self.lib = load()
        self.instances = list(instances)
        arr = (WgInstance * max(len(self.instances), 1))()
        for i, inst in enumerate(self.instances):
            arr[i] = inst.struct
        self._arr = arr
        opt = WgPlanOptions(float(chunk_scale), int(max_warps_per_cta), int(bool(merge_classes)),
                            int(bool(use_graph)), int(bool(serial_groups)), None)
        h = ctypes.c_void_p()
        check(self.lib.wg_plan_create_ex(arr, len(self.instances), PRECISIONS[precision],
                                         ctypes.byref(opt), ctypes.byref(h)))
        self.handle = h
        self.total_out = self.lib.wg_plan_outputs(h)
        self.kernel_launches = self.lib.wg_plan_kernel_launches(h)

    @classmethod
    def from_requests(cls, state, requests, precision="fp64", **options):
        """Plan over serving requests on a resident state; ``requests`` are (x, edge_reps,
        oddmode) triples as ``matched_reps`` returns them for each photon pattern."""
        self = cls.__new__(cls)
        self.lib = load()
        self.instances = []
        keep = []
        arr = (WgRequest * max(len(requests), 1))()
        for i, (x, reps, odd) in enumerate(requests):
            xa = np.ascontiguousarray(x, dtype=np.int32)
            ra = np.ascontiguousarray(reps, dtype=np.int64)
            keep.append((xa, ra))
            arr[i] = WgRequest(xa.ctypes.data, ra.ctypes.data, len(ra), -1 if odd is None else int(odd))
        self._keep, self._arr = keep, arr
        opt = WgPlanOptions(float(options.get("chunk_scale", 1.0)), int(options.get("max_warps_per_cta", 0)),
                            int(bool(options.get("merge_classes", False))), int(bool(options.get("use_graph", False))),
                            int(bool(options.get("serial_groups", False))), options.get("stream"))
        h = ctypes.c_void_p()
        check(self.lib.wg_plan_create_requests(state.handle, arr, len(requests), PRECISIONS[precision],
                                               ctypes.byref(opt), ctypes.byref(h)))
        self.handle = h
        self.total_out = self.lib.wg_plan_outputs(h)
        self.kernel_launches = self.lib.wg_plan_kernel_launches(h)
        return self

    def device_bytes(self):
        return int(self.lib.wg_plan_device_bytes(self.handle))

    def transfer_bytes(self):
        h, d = ctypes.c_longlong(), ctypes.c_longlong()
        check(self.lib.wg_plan_transfer_bytes(self.handle, ctypes.byref(h), ctypes.byref(d)))
        return h.value, d.value

    def partials(self, stream=0):
        """Unscaled per-chunk partial sums of the last execution, with each chunk's
        (instance, first slot, t0, t1)."""
        cnt = self.lib.wg_plan_partials(self.handle, None, 0, ctypes.c_void_p(stream))
        out = np.zeros(2 * max(cnt, 1))
        self.lib.wg_plan_partials(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  cnt, ctypes.c_void_p(stream))
        chunks = []
        a, b = ctypes.c_int(), ctypes.c_int()
        t0, t1 = ctypes.c_longlong(), ctypes.c_longlong()
        k = 0
        while True:
            n = self.lib.wg_plan_chunk(self.handle, k, ctypes.byref(a), ctypes.byref(b),
                                       ctypes.byref(t0), ctypes.byref(t1))
            if n <= k:
                break
            chunks.append((a.value, b.value, t0.value, t1.value))
            k += 1
        return (out[0::2] + 1j * out[1::2])[:cnt], chunks

    def execute(self, stream=0):
        check(self.lib.wg_plan_execute(self.handle, ctypes.c_void_p(stream)))

    def read(self, stream=0):
        out = np.zeros(2 * max(self.total_out, 1))
        check(self.lib.wg_plan_read(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    ctypes.c_void_p(stream)))
        return (out[0::2] + 1j * out[1::2])[: self.total_out]

    def read_magnitudes(self, stream=0):
        """Per output of the last execution: sum |prefactor x term| times the final scale (the
        size of the terms the output cancels from; 0 for exact precisions)."""
        out = np.zeros(max(self.total_out, 1))
        check(self.lib.wg_plan_read_magnitudes(self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               ctypes.c_void_p(stream)))
        return out[: self.total_out]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.wg_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def crt(residues, primes=MOD_PRIMES):
    """The integer in (-M/2, M/2], M = prod(primes), with the given residues."""
    M, v = 1, 0
    for p, a in zip(primes, residues):
        t = ((int(a) - v) * pow(M, -1, p)) % p
        v += M * t
        M *= p
    return v - M if v > M // 2 else v


def exact_primes(instances):
    """How many of the 31-bit primes an exact run needs: enough that the product exceeds twice
    a bound on every output's magnitude, |haf(A)| <= sqrt(prod_i r_i) with r_i the absolute row
    sums of the expanded matrix (haf^2 <= per <= product of row sums); None beyond five."""
    bits = 0.0
    for inst in instances:
        bits = max(bits, inst.log2_bound())
    k = int(np.ceil((bits + 2.0) / 30.99))
    return max(k, 2) if k <= len(MOD_PRIMES) else None


def run_exact(instances, stream=0, nprimes=None):
    """Exact outputs (Python ints) of integer-valued real instances: the sieve modulo 31-bit
    primes on the GPU (as many as ``exact_primes`` asks), combined by the Chinese remainder
    theorem."""
    k = nprimes or exact_primes(instances)
    if k is None:
        raise ValueError("exact precision: the outputs may exceed 2^153, beyond five primes")
    per_prime = [run(instances, "mod%d" % j, stream).real for j in range(k)]
    return [crt([round(float(r[i])) for r in per_prime], MOD_PRIMES[:k]) for i in range(len(per_prime[0]))]


def run(instances, precision="fp64", stream=0):
    """Run instances through one plan; returns the concatenated complex outputs.  With
    ``precision="exact"`` the exact integers, rounded to complex128."""
    if precision == "exact":
        return np.array([complex(float(v), 0.0) for v in run_exact(instances, stream)], dtype=np.complex128)
    lib = load()
    insts = list(instances)
    arr = (WgInstance * max(len(insts), 1))()
    total = 0
    for i, inst in enumerate(insts):
        arr[i] = inst.struct
        total += inst.outputs()
    out = np.zeros(2 * max(total, 1))
    check(lib.wg_run(arr, len(insts), PRECISIONS[precision],
                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_void_p(stream)))
    return (out[0::2] + 1j * out[1::2])[:total]


def check_arith(op, x, x_lo=None, y=None, y_lo=None):
    """Evaluate one of the kernels' arithmetic primitives on the device elementwise
    (``wg_check_arith``): op 0 the FP64 pivot reciprocal, 1-3 the double-double reciprocal,
    division by the integer y and product, 4-6 the double-float reciprocal, complex reciprocal
    (returns the real and imaginary parts) and division by the integer y.  Returns the (hi, lo)
    arrays."""
    x = np.asarray(x, dtype=np.float64).ravel()
    z = np.zeros_like(x)
    inp = np.ascontiguousarray(np.stack([x, z if x_lo is None else np.asarray(x_lo, dtype=np.float64).ravel(),
                                         z if y is None else np.asarray(y, dtype=np.float64).ravel(),
                                         z if y_lo is None else np.asarray(y_lo, dtype=np.float64).ravel()], axis=1))
    out = np.zeros((len(x), 2))
    dp = ctypes.POINTER(ctypes.c_double)
    check(load().wg_check_arith(int(op), inp.ctypes.data_as(dp), len(x), out.ctypes.data_as(dp)))
    return out[:, 0], out[:, 1]


def measure_fp_peaks():
    """(FP64, FP32) FMA-pipe TFLOP/s measured on the current device."""
    lib = load()
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib.wg_measure_fp_peaks(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


class DeviceState:
    """A loop-hafnian source matrix B (M x M) and loop weights gamma (M) resident on the GPU."""

    @classmethod
    def from_cov(cls, cov, mu, hbar=2.0):
        """The state formed on the device from a pure state's xp covariance and means
        (``wg_state_create_from_cov``); returns (state, vacuum amplitude, B, gamma) with host
        copies of B and gamma."""
        self = cls.__new__(cls)
        self.lib = load()
        cov = np.ascontiguousarray(cov, dtype=np.float64)
        mu = np.ascontiguousarray(mu, dtype=np.float64)
        M = cov.shape[0] // 2
        dp = ctypes.POINTER(ctypes.c_double)
        vac = np.zeros(2)
        B = np.zeros((M, M), dtype=np.complex128)
        g = np.zeros(M, dtype=np.complex128)
        h = ctypes.c_void_p()
        check(self.lib.wg_state_create_from_cov(cov.ctypes.data_as(dp), mu.ctypes.data_as(dp), M, float(hbar),
                                                ctypes.byref(h), vac.ctypes.data_as(dp), B.ctypes.data_as(dp),
                                                g.ctypes.data_as(dp)))
        self.handle = h
        self.M = M
        return self, complex(vac[0], vac[1]), B, g

    def __init__(self, B, gamma):
        self.lib = load()
        B = np.ascontiguousarray(B, dtype=np.complex128)
        g = np.ascontiguousarray(gamma, dtype=np.complex128)
        h = ctypes.c_void_p()
        dp = ctypes.POINTER(ctypes.c_double)
        check(self.lib.wg_state_create(B.ctypes.data_as(dp), g.ctypes.data_as(dp), B.shape[0], ctypes.byref(h)))
        self.handle = h
        self.M = B.shape[0]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.wg_state_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass
