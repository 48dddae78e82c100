"""Generate the golden fixtures of tests/golden from the REFERENCE libxm.

Run in a checkout where the reference sources exist (oracle/build.py
compiles them into oracle/_ref/libxmref.so); GPU hosts never run this.
Inputs are regenerated by the tests from the same numpy seeds, so only
outputs and structure logs are stored:

  contract_cases.npz  46 test-driver cases x 4 scalar types: canonical
                      output blocks for seeded inputs and scalars, and the
                      reference's GEMM call log (type, m, n, k, al) for
                      alpha=1, beta=0 with one thread (its merged pair list)
  elementwise.npz     add / copy / mul / div / dot cases of the driver
  workloads.npz       cfg1 ladder output digests and GEMM log; the uneven
                      Z2^3 ladder at 1/4 scale, full outputs and GEMM log
  example.json        the reference's example.c result matrix (2-D case)

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from libxm_gb300 import api, workloads as W  # noqa: E402
import oracle.build as ob  # noqa: E402
import cases  # noqa: E402
import helpers as H  # noqa: E402


def ref_lib():
    lib = api.Lib(ob.build_reference())
    lib.dll.xmref_set_blas.argtypes = [C.c_char_p]
    lib.dll.xmref_set_blas(ob.find_blas().encode())
    lib.dll.xmref_log_get.argtypes = [C.c_size_t] + [C.c_void_p] * 6
    lib.dll.xmref_log_count.restype = C.c_size_t
    return lib


def gemm_log(lib):
    n = lib.dll.xmref_log_count()
    out = np.zeros((n, 6))
    t, m, nn, k = C.c_int(), C.c_long(), C.c_long(), C.c_long()
    re, im = C.c_double(), C.c_double()
    for i in range(n):
        lib.dll.xmref_log_get(i, C.byref(t), C.byref(m), C.byref(nn), C.byref(k),
                              C.byref(re), C.byref(im))
        out[i] = (t.value, m.value, nn.value, k.value, re.value, im.value)
    return out


def digest(x):
    """Full vector when small, else (sum, sum |x|^2, every 97th element)."""
    x = np.asarray(x).ravel()
    if x.size <= 4096:
        return x
    return np.concatenate([[x.sum(), np.vdot(x, x).real], x[::97]])


def case_scalars(ci, dtype):
    rng = np.random.default_rng(77 + 1000 * ci + dtype)
    return H.scalar(rng, dtype), H.scalar(rng, dtype)


def main():
    assert os.environ.get("OMP_NUM_THREADS") == "1", "run with OMP_NUM_THREADS=1"
    lib = ref_lib()
    al = api.Allocator(lib)
    out = {}
    for ci, case in enumerate(cases.CONTRACT_TESTS):
        for dt in H.TYPES:
            alpha, beta = case_scalars(ci, dt)
            res = H.run_contract_case(lib, al, case, dt, 1000 * ci + dt, alpha, beta)
            out["c%02d_t%d" % (ci, dt)] = np.concatenate(
                [res[k].ravel() for k in sorted(res)]) if res else np.zeros(0)
            # structure: GEMM log at alpha = 1, beta = 0
            make, ia, ib, ic = case
            a, b, c = make(lib, al, dt)
            rng = np.random.default_rng(5)
            H.fill_random(a, rng); H.fill_random(b, rng); H.fill_random(c, rng)
            lib.dll.xmref_log_enable(1)
            api.contract(1.0, a, b, 0.0, c, ia, ib, ic)
            lib.dll.xmref_log_enable(0)
            out["log%02d_t%d" % (ci, dt)] = gemm_log(lib)
            for t in (a, b, c):
                t.free()
    np.savez_compressed(os.path.join(HERE, "contract_cases.npz"), **out)

    ew = {}
    for ci, (make, ia, ib) in enumerate(cases.ADD_TESTS):
        for dt in H.TYPES:
            for combo in range(4):
                rng = np.random.default_rng(9000 + 100 * ci + 10 * dt + combo)
                x = H.scalar(rng, dt)
                y = H.scalar(rng, dt)
                alpha = [0, 0, x, x][combo]
                beta = [0, y, 0, y][combo]
                a, b = make(lib, al, dt)
                H.fill_random(a, rng); H.fill_random(b, rng)
                api.add(alpha, a, beta, b, ia, ib)
                r = H.canon(a)
                ew["add%d_t%d_%d" % (ci, dt, combo)] = digest(np.concatenate([r[k].ravel() for k in sorted(r)]))
                a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.MUL_DIV_TESTS):
        for dt in H.TYPES:
            for op in ("mul", "div"):
                rng = np.random.default_rng(12000 + 100 * ci + 10 * dt + (op == "div"))
                a, b = make(lib, al, dt)
                H.fill_random(a, rng); H.fill_random(b, rng)
                (api.mul if op == "mul" else api.div)(a, b, ia, ib)
                r = H.canon(a)
                ew["%s%d_t%d" % (op, ci, dt)] = digest(np.concatenate([r[k].ravel() for k in sorted(r)]))
                a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.DOT_TESTS):
        for dt in H.TYPES:
            rng = np.random.default_rng(15000 + 100 * ci + dt)
            a, b = make(lib, al, dt)
            H.fill_random(a, rng); H.fill_random(b, rng)
            ew["dot%d_t%d" % (ci, dt)] = np.array([api.dot(a, b, ia, ib)])
            a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.ADD_TESTS):
        for dt in H.TYPES:
            rng = np.random.default_rng(18000 + 100 * ci + dt)
            a, b = make(lib, al, dt)
            H.fill_random(a, rng); H.fill_random(b, rng)
            s = H.scalar(rng, dt)
            api.copy(a, s, b, ia, ib)
            r = H.canon(a)
            ew["copy%d_t%d" % (ci, dt)] = digest(np.concatenate([r[k].ravel() for k in sorted(r)]))
            a.free(); b.free()
    np.savez_compressed(os.path.join(HERE, "elementwise.npz"), **ew)

    wl = {}
    w = W.cfg1(lib, al)
    lib.dll.xmref_log_enable(1)
    w.run()
    lib.dll.xmref_log_enable(0)
    wl["cfg1_log"] = gemm_log(lib)
    r = H.canon(w.c)
    keys = sorted(r)
    wl["cfg1_blocks"] = np.array(keys)
    wl["cfg1_sum"] = np.array([r[k].sum() for k in keys])
    wl["cfg1_sumsq"] = np.array([float(np.dot(r[k], r[k])) for k in keys])
    wl["cfg1_sample"] = np.concatenate([r[k][:7] for k in keys])
    w.free()
    w = W.cfg2(lib, al, scale=4)
    lib.dll.xmref_log_enable(1)
    w.run()
    lib.dll.xmref_log_enable(0)
    wl["cfg2s4_log"] = gemm_log(lib)
    r = H.canon(w.c)
    keys = sorted(r)
    wl["cfg2s4_blocks"] = np.array(keys)
    wl["cfg2s4_out"] = digest(np.concatenate([r[k] for k in keys]))
    w.free()
    np.savez_compressed(os.path.join(HERE, "workloads.npz"), **wl)

    # example.c:17-100 (a 2-D tutorial contraction) through the API
    bsa = api.BlockSpace(lib, [4, 5]).split(0, 2).split(1, 2).split(1, 3)
    bsb = api.BlockSpace(lib, [5, 3]).split(0, 2).split(0, 3)
    bsc = api.BlockSpace(lib, [4, 3]).split(0, 2)
    a = api.Tensor(lib, bsa, api.DOUBLE, al)
    b = api.Tensor(lib, bsb, api.DOUBLE, al)
    c = api.Tensor(lib, bsc, api.DOUBLE, al, canonical=True)
    a.set_canonical((0, 0)); a.write_block((0, 0), np.array([1.0, 2, 3, 4]).reshape(2, 2, order="F"))
    a.set_derivative((1, 2), (0, 0), (1, 0), -1.0)
    b.set_canonical((0, 0)); b.write_block((0, 0), np.array([6.0, 5, -4, 3, 2, -1]).reshape(2, 3, order="F"))
    b.set_derivative((2, 0), (0, 0), (0, 1), -0.5)
    api.set_all(c, 1.0)
    api.contract(2.0, a, b, 1.0, c, "ik", "kj", "ij")
    mat = [[c.get_element((i, j)).real for j in range(3)] for i in range(4)]
    with open(os.path.join(HERE, "example.json"), "w") as f:
        json.dump({"c": mat, "a": [[a.get_element((i, j)).real for j in range(5)] for i in range(4)],
                   "b": [[b.get_element((i, j)).real for j in range(3)] for i in range(5)]}, f, indent=1)
    print("golden fixtures written")


if __name__ == "__main__":
    main()
