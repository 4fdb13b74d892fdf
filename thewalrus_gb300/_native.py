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
SOURCES = ["sieve.cu", "noalloc.cu"]
DEPS = ["sieve.cu", "noalloc.cu", "sieve_kernel.cuh", "arith.cuh", "host_common.h"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-shared"]

WG_FLOAT64, WG_COMPLEX128 = 0, 1
WG_PREC_FP64, WG_PREC_DF = 0, 1
WG_KIND_PLAIN, WG_KIND_LOOP, WG_KIND_BATCH_EVEN, WG_KIND_BATCH_ODD = 0, 1, 3, 4
PRECISIONS = {"fp64": WG_PREC_FP64, "df": WG_PREC_DF}

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
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [_nvcc()] + NVCC_FLAGS + ["-o", tmp] + [os.path.join(CSRC, s) for s in SOURCES]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), res.stdout.decode()))
        if verbose and res.stdout:
            print(res.stdout.decode())
        os.replace(tmp, LIB)
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
    ]


EXPORTS = [
    "wg_init", "wg_last_error", "wg_instance_outputs", "wg_hafnian", "wg_loop_hafnian",
    "wg_loop_hafnian_batch", "wg_plan_create", "wg_plan_execute", "wg_plan_read", "wg_plan_outputs",
    "wg_plan_kernel_launches", "wg_plan_partials", "wg_plan_chunk", "wg_plan_transfer_bytes",
    "wg_plan_destroy", "wg_run",
    "wg_measure_fp_peaks", "wg_hafnian_noalloc",
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
    lib.wg_hafnian.argtypes = [vp, i32, i32, ip, i32, i32, i32, dp, vp]
    lib.wg_loop_hafnian.argtypes = [vp, vp, i32, i32, ip, i32, i32, dp, vp, i32, i32, dp, vp]
    lib.wg_loop_hafnian_batch.argtypes = [vp, vp, i32, i32, ip, i32, i32, i32, i32, i32, i32, dp, vp]
    lib.wg_plan_create.argtypes = [ctypes.POINTER(WgInstance), i32, i32, ctypes.c_double,
                                   ctypes.POINTER(vp)]
    lib.wg_plan_execute.argtypes = [vp, vp]
    lib.wg_plan_read.argtypes = [vp, dp, vp]
    lib.wg_plan_outputs.argtypes = [vp]
    lib.wg_plan_kernel_launches.argtypes = [vp]
    lib.wg_plan_transfer_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    lib.wg_plan_partials.argtypes = [vp, dp, i32, vp]
    lib.wg_plan_chunk.argtypes = [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                  ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    lib.wg_plan_destroy.argtypes = [vp]
    lib.wg_run.argtypes = [ctypes.POINTER(WgInstance), i32, i32, dp, vp]
    lib.wg_measure_fp_peaks.argtypes = [dp, dp]
    lib.wg_hafnian_noalloc.argtypes = [vp, i32, i32, ip, i32, i32, vp, vp]
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
        cplx = np.iscomplexobj(A) or (D is not None and np.iscomplexobj(D)) or \
            (oddV is not None and np.iscomplexobj(oddV)) or \
            (oddloop is not None and np.iscomplexobj(oddloop))
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

    def outputs(self):
        if self.struct.kind == WG_KIND_BATCH_EVEN:
            return 2 * self.struct.batch_max + self.struct.cutoff + 1
        if self.struct.kind == WG_KIND_BATCH_ODD:
            return 2 * self.struct.batch_max + self.struct.cutoff + 2
        return 1


class Plan:
    """Device-resident batch of instances: create once, execute many times, read results."""

    def __init__(self, instances, precision="fp64", chunk_scale=1.0):
        self.lib = load()
        self.instances = list(instances)
        arr = (WgInstance * max(len(self.instances), 1))()
        for i, inst in enumerate(self.instances):
            arr[i] = inst.struct
        self._arr = arr
        h = ctypes.c_void_p()
        check(self.lib.wg_plan_create(arr, len(self.instances), PRECISIONS[precision],
                                      float(chunk_scale), ctypes.byref(h)))
        self.handle = h
        self.total_out = self.lib.wg_plan_outputs(h)
        self.kernel_launches = self.lib.wg_plan_kernel_launches(h)

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

    def close(self):
        if getattr(self, "handle", None):
            self.lib.wg_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def run(instances, precision="fp64", stream=0):
    """Run instances through one plan; returns the concatenated complex outputs."""
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


def measure_fp_peaks():
    """(FP64, FP32) FMA-pipe TFLOP/s measured on the current device."""
    lib = load()
    a, b = ctypes.c_double(), ctypes.c_double()
    check(lib.wg_measure_fp_peaks(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value
