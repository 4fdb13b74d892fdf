"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle_core.c`` three times, once per scalar type (double, long double, _Float128),
and ``oracle_exact.c`` (the sieve over F_p for exact integer hafnians) into one shared library
``oracle/_build/liboracle.so``.  OpenMP threads split the sieve terms.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")

VARIANTS = [
    ("double", "_d", []),
    ("long double", "_ld", ["-DOR_IS_LD"]),
    ("_Float128", "_q", ["-DOR_IS_QUAD"]),
]


def build(force=False, verbose=False):
    """Compile the oracle if its library is missing or older than its source."""
    src = os.path.join(HERE, "oracle_core.c")
    exact = os.path.join(HERE, "oracle_exact.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src),
                                                                          os.path.getmtime(exact)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    procs = []
    for real, sfx, extra in VARIANTS:
        obj = os.path.join(OUT_DIR, "oracle%s.o" % sfx)
        cmd = ["gcc", "-O2", "-fPIC", "-fopenmp", "-std=gnu11", "-c", src, "-o", obj,
               "-DOR_REAL=%s" % real, "-DSFX=%s" % sfx] + extra
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    obj = os.path.join(OUT_DIR, "oracle_exact.o")
    cmd = ["gcc", "-O2", "-fPIC", "-fopenmp", "-std=gnu11", "-c", exact, "-o", obj]
    procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objs.append(obj)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), out.decode()))
        if verbose and out:
            sys.stdout.write(out.decode())
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-shared", "-fopenmp", "-o", tmp] + objs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
