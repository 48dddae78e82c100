"""Build libxm-gb300: C host sources + sm_103a CUDA kernels -> one shared
library, libxm_gb300/lib/libxmgb.so, exporting the libxm C API (include/).

Compiles in parallel, only what changed; no cmake.
"""
import concurrent.futures as cf
import glob
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "lib", "libxmgb.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(CSRC, "host"),
       "-I", os.path.join(CSRC, "cuda")]
CFLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wextra", "-Wno-unused-parameter"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"] + ARCH


def _headers():
    return (glob.glob(os.path.join(ROOT, "include", "*.h")) +
            glob.glob(os.path.join(CSRC, "*", "*.h")) +
            glob.glob(os.path.join(CSRC, "*", "*.cuh")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + INC + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["gcc"] + CFLAGS + INC + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr).strip() or None


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "host", "*.c")) +
                  glob.glob(os.path.join(CSRC, "cuda", "*.cu")))
    # the long CUDA translation units first
    srcs.sort(key=lambda s: (not s.endswith(".cu"), s))
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    for _, msg in results:
        if msg and verbose:
            print(msg)
    if _stale(LIB, objs) or _arch_tag() != platform.machine():
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + [
            "-lcudart_static", "-ldl", "-lrt", "-lpthread", "-lm",
            "-Xlinker", "-z", "-Xlinker", "defs"]   # no undefined symbols
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        with open(LIB + ".arch", "w") as f:
            f.write(platform.machine())
    return LIB


def build_sanitized(out_dir):
    """The library with its host code (the C sources and the host side of
    the CUDA sources) built with AddressSanitizer and UBSan into
    out_dir/libxmgb.so, for running the CPU test suite with the sanitizer
    runtimes preloaded:

        LD_PRELOAD="$(gcc -print-file-name=libasan.so) $(gcc -print-file-name=libubsan.so)" \
        ASAN_OPTIONS=detect_leaks=0:verify_asan_link_order=0 python -c "
        import libxm_gb300, pytest, sys
        libxm_gb300.LIB_PATH = 'OUT_DIR/libxmgb.so'
        sys.exit(pytest.main(['tests', '-q', '-m', 'not gpu']))"
    """
    os.makedirs(out_dir, exist_ok=True)
    san = ["-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer"]
    cmds = []
    for src in sorted(glob.glob(os.path.join(CSRC, "host", "*.c"))):
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        cmds.append(["gcc", "-O1", "-g", "-fPIC", "-std=gnu11"] + san + INC +
                    ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "cuda", "*.cu"))):
        # the host side of the CUDA sources (plans, work lists) too
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        cmds.append([NVCC, "-O1", "-g", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC"] + [x for f in san for x in ("-Xcompiler", f)] +
                    ARCH + INC + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds):
            if r.returncode != 0:
                raise RuntimeError("compile failed: %s\n%s" % (" ".join(r.args), r.stderr))
    objs = [c[c.index("-o") + 1] for c in cmds]
    lib = os.path.join(out_dir, "libxmgb.so")
    subprocess.run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + [
        "-lcudart_static", "-ldl", "-lrt", "-lpthread", "-lm", "-lasan", "-lubsan"], check=True)
    return lib


def _arch_tag():
    try:
        with open(LIB + ".arch") as f:
            return f.read().strip()
    except OSError:
        return None


if __name__ == "__main__":
    if "--sanitize" in sys.argv:
        print(build_sanitized(sys.argv[sys.argv.index("--sanitize") + 1]))
    else:
        print(build(verbose="-v" in sys.argv))
