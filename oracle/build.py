"""ORACLE build recipe -- test infrastructure only.

Builds
  oracle/_build/libxmoracle.so  from oracle/xm_oracle.c (the CPU restatement)
  oracle/_ref/libxmref.so       from the reference libxm sources, compiled in
                                place from the reference checkout (only when
                                that checkout exists, i.e. not on GPU hosts),
                                linked with oracle/ref_blas_shim.c.
Neither library is part of the product; tests/, smoke() and the CPU-baseline
leg of bench.py are the only users.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout's src/ directory: $XM_REFERENCE_SRC, else a
# checkout named "reference" beside this repository
REF_SRC = os.environ.get("XM_REFERENCE_SRC") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference", "src"))
ORACLE_SO = os.path.join(HERE, "_build", "libxmoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libxmref.so")
REF_FILES = ["alloc.c", "blockspace.c", "contract.c", "dim.c", "scalar.c",
             "tensor.c", "util.c", "xm.c"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _arch_tag(path):
    tag = path + ".arch"
    if not os.path.exists(tag):
        return None
    with open(tag) as f:
        return f.read().strip()


def build_oracle(force=False):
    src = os.path.join(HERE, "xm_oracle.c")
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    if force or _stale(ORACLE_SO, [src]) or _arch_tag(ORACLE_SO) != platform.machine():
        _run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=gnu11",
              "-o", ORACLE_SO, src, "-ldl", "-lm"])
        with open(ORACLE_SO + ".arch", "w") as f:
            f.write(platform.machine())
    return ORACLE_SO


def build_reference(force=False):
    """Compile the reference from its own sources (returns None when the
    reference checkout is not present on this machine)."""
    if not os.path.isdir(REF_SRC):
        return REF_SO if os.path.exists(REF_SO) and _arch_tag(REF_SO) == platform.machine() else None
    srcs = [os.path.join(REF_SRC, f) for f in REF_FILES]
    shim = os.path.join(HERE, "ref_blas_shim.c")
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    if force or _stale(REF_SO, srcs + [shim]) or _arch_tag(REF_SO) != platform.machine():
        _run(["gcc", "-O3", "-fopenmp", "-DNDEBUG", "-fPIC", "-shared",
              "-std=gnu11", "-w", "-I", REF_SRC, "-o", REF_SO] + srcs +
             [shim, "-ldl", "-lm", "-lpthread"])
        with open(REF_SO + ".arch", "w") as f:
            f.write(platform.machine())
    return REF_SO


def find_blas():
    """Path of numpy's bundled ILP64 OpenBLAS (scipy_?gemm_64_), or None."""
    try:
        import numpy
    except ImportError:
        return None
    base = os.path.dirname(os.path.dirname(numpy.__file__))
    for d in (os.path.join(base, "numpy.libs"), os.path.join(os.path.dirname(numpy.__file__), ".libs")):
        if os.path.isdir(d):
            for f in sorted(os.listdir(d)):
                if "openblas" in f and f.endswith(".so") or ("openblas" in f and ".so." in f):
                    return os.path.join(d, f)
    return None


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_reference(force="-f" in sys.argv))
    print(find_blas())
