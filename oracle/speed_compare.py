"""ORACLE timing recipe -- test infrastructure only.

Times the oracle port (oracle/xm_oracle.c) against the reference built from
its own sources (oracle/_ref/libxmref.so, see oracle/build.py) on the whole
uneven Z2^3 ladder (o = 96 in 6 blocks, v = 384 in 12 blocks): the same
inputs, the same OpenMP thread count (OMP_NUM_THREADS, default all cores),
OPENBLAS_NUM_THREADS=1, one warm-up call and the best of three whole
xm_contract calls for each library, and checks that both give the same
result.  Runs only where the reference checkout exists (the reference
library cannot be built elsewhere).  Prints a markdown summary:

    python oracle/speed_compare.py [--scale S] [--reps R]
"""
import argparse
import os
import platform
import sys
import time

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import oracle.build as ob  # noqa: E402
from libxm_gb300 import api, workloads as W  # noqa: E402


def load(kind):
    blas = ob.find_blas()
    if kind == "port":
        lib = api.Lib(ob.build_oracle())
        lib.dll.xmo_set_blas.argtypes = [api.C.c_char_p]
        lib.dll.xmo_set_blas(blas.encode() if blas else None)
    else:
        path = ob.build_reference()
        if path is None:
            raise SystemExit("the reference checkout is not present here")
        lib = api.Lib(path)
        lib.dll.xmref_set_blas.argtypes = [api.C.c_char_p]
        lib.dll.xmref_set_blas(blas.encode() if blas else None)
    return lib


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=1)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    threads = int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count())
    os.environ["OMP_NUM_THREADS"] = str(threads)
    rows, outs = [], {}
    for kind in ("reference", "port"):
        lib = load(kind)
        al = api.Allocator(lib)
        w = W.cfg2(lib, al, scale=args.scale)
        flops = sum(2.0 * m * n * k for _, _, m, n, k in pairs(lib, w))
        w.run()
        times = []
        for _ in range(args.reps):
            t0 = time.perf_counter()
            w.run()
            times.append(time.perf_counter() - t0)
        outs[kind] = W.read_canonical(w.c)
        rows.append((kind, min(times), float(np.mean(times)), flops / min(times) / 1e12))
        w.free()
        al.destroy()
    rel = W.rel_frobenius(outs["port"], outs["reference"])
    print("# CPU reference vs oracle port, whole xm_contract on %s"
          % ("cfg2_ladder_o96_v384_z2" if args.scale == 1 else "cfg2_ladder_scaled_%d" % args.scale))
    print()
    print("Command: `OMP_NUM_THREADS=%d python oracle/speed_compare.py%s`"
          % (threads, "" if args.scale == 1 else " --scale %d" % args.scale))
    print()
    print("Host: %s, %d OpenMP threads, OPENBLAS_NUM_THREADS=1 (numpy's bundled "
          "OpenBLAS), one warm-up then best of %d calls." % (platform.machine(), threads, args.reps))
    print()
    print("| library | best s | mean s | TFLOP/s (best) |")
    print("|---|---|---|---|")
    for kind, best, mean, tf in rows:
        print("| %s | %.3f | %.3f | %.4f |" % (
            "reference (compiled from source)" if kind == "reference" else "oracle port",
            best, mean, tf))
    print()
    print("Port / reference time: %.3f; relative Frobenius difference of the results: %.2e"
          % (rows[1][1] / rows[0][1], rel))


def pairs(lib, w):
    """Merged pair list (GEMM shapes) of lib's own xm_contract run."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import helpers as H
    if hasattr(lib.dll, "xmo_set_pair_callback"):
        lib.dll.xmo_set_plan_only(1)
        try:
            return H.pair_structure_oracle(lib, w.a, w.b, w.c.structure(), w.idxa, w.idxb, w.idxc)
        finally:
            lib.dll.xmo_set_plan_only(0)
    orc = load("port")
    oal = api.Allocator(orc)
    wo = W.cfg2(orc, oal, scale=1 if w.name.endswith("z2") else int(w.name.rsplit("_", 1)[1]),
                fill_data=False)
    orc.dll.xmo_set_plan_only(1)
    try:
        return H.pair_structure_oracle(orc, wo.a, wo.b, wo.c, wo.idxa, wo.idxb, wo.idxc)
    finally:
        orc.dll.xmo_set_plan_only(0)
        wo.free()


if __name__ == "__main__":
    main()
