"""Pin the oracle (CPU restatement) to the reference.

Known answers from the reference test driver (test.c:1728-1824), the
example program's result (example.c), golden fixtures produced by the
reference built from source (tests/golden/make_golden.py), and -- where
the reference checkout exists -- the live reference on the same inputs.
"""
import json
import os

import numpy as np
import pytest

import cases
import helpers as H
from libxm_gb300 import api, workloads as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gold(name):
    return np.load(os.path.join(GOLD, name))


def digest(x):
    x = np.asarray(x).ravel()
    if x.size <= 4096:
        return x
    return np.concatenate([[x.sum(), np.vdot(x, x).real], x[::97]])


@pytest.mark.parametrize("which", ["oracle", "engine"])
def test_dim_kat(which, request):
    # test.c:1728-1764: xm_dim_inc walks every index with index 0 fastest,
    # xm_dim_offset numbers them sequentially and xm_dim_from_offset
    # inverts it
    lib = request.getfixturevalue(which)
    P = api.C.POINTER(api.Dim)
    lib.dll.xm_dim_offset.restype = api.C.c_size_t
    lib.dll.xm_dim_offset.argtypes = [P, P]
    lib.dll.xm_dim_from_offset.restype = api.Dim
    lib.dll.xm_dim_from_offset.argtypes = [api.C.c_size_t, P]
    lib.dll.xm_dim_inc.restype = None
    lib.dll.xm_dim_inc.argtypes = [P, P]
    for dims in ([5, 6, 3, 1], [1, 31, 16], [5, 2, 3, 2, 1, 2, 5, 4]):
        d = api.Dim.of(dims)
        idx = api.Dim.of([0] * len(dims))
        for off, want in enumerate(np.ndindex(*dims[::-1])):
            assert idx.tolist() == list(want[::-1])
            assert lib.dll.xm_dim_offset(api.C.byref(idx), api.C.byref(d)) == off
            back = lib.dll.xm_dim_from_offset(off, api.C.byref(d))
            assert back.tolist() == idx.tolist()
            lib.dll.xm_dim_inc(api.C.byref(idx), api.C.byref(d))
    d = api.Dim.of([5, 2, 3, 2, 1, 2, 5, 4])
    lib.xm_dim_dot.restype = api.C.c_size_t
    assert lib.xm_dim_dot(api.C.byref(d)) == 5 * 2 * 3 * 2 * 2 * 5 * 4


@pytest.mark.parametrize("which", ["oracle", "reference"])
def test_blockspace_kat(which, request):
    lib = request.getfixturevalue(which)
    # test.c:1766-1824
    bs = api.BlockSpace(lib, [1, 2, 3, 4, 5, 6, 7, 8]).autosplit()
    assert bs.nblocks() == [1] * 8
    assert bs.block_dims([0] * 8) == [1, 2, 3, 4, 5, 6, 7, 8]
    bs.free()
    bs = api.BlockSpace(lib, [10, 20, 30, 40, 50, 60, 70, 80]).autosplit()
    assert bs.nblocks() == [1, 1, 1, 2, 2, 2, 3, 3]
    for blk in np.ndindex(*bs.nblocks()):
        assert all(x < 31 for x in bs.block_dims(blk))
    bs.free()
    bs = api.BlockSpace(lib, [30, 31, 32, 33, 34]).autosplit()
    assert bs.nblocks() == [1, 1, 1, 2, 2]
    assert bs.block_dims([0] * 5) == [30, 31, 32, 16, 18]
    bs.free()
    a = api.BlockSpace(lib, [102, 40, 203, 593, 15, 84, 1934])
    b = api.BlockSpace(lib, [40, 593, 83, 84, 85, 1934])
    for _ in range(2):
        eq = [lib.xm_block_space_eq1(a.h, i, b.h, j) for i, j in
              [(1, 0), (3, 1), (5, 2), (5, 3), (5, 4), (6, 5)]]
        assert eq == [1, 1, 0, 1, 0, 1]
        a.autosplit(); b.autosplit()
    a.free(); b.free()


def test_make_masks(oracle):
    assert api.make_masks(oracle, "ijcd", "cdab") == ([2, 3], [0, 1])
    assert api.make_masks(oracle, "ijab", "ijcd") == ([0, 1], [0, 1])


def test_example_known_answer(oracle):
    ex = json.load(open(os.path.join(GOLD, "example.json")))
    lib = oracle
    al = api.Allocator(lib)
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
    got = [[c.get_element((i, j)).real for j in range(3)] for i in range(4)]
    assert got == ex["c"]
    for t in (a, b, c):
        t.free()


@pytest.mark.parametrize("ci", range(len(cases.CONTRACT_TESTS)))
def test_oracle_contract_golden(oracle, ci):
    g = gold("contract_cases.npz")
    al = api.Allocator(oracle)
    for dt in H.TYPES:
        rng = np.random.default_rng(77 + 1000 * ci + dt)
        alpha, beta = H.scalar(rng, dt), H.scalar(rng, dt)
        res = H.run_contract_case(oracle, al, cases.CONTRACT_TESTS[ci], dt,
                                  1000 * ci + dt, alpha, beta)
        got = np.concatenate([res[k].ravel() for k in sorted(res)]) if res else np.zeros(0)
        ref = g["c%02d_t%d" % (ci, dt)]
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=H.TOL[dt])
        # structure: the oracle's merged pairs = the reference's GEMM calls
        make, ia, ib, ic = cases.CONTRACT_TESTS[ci]
        a, b, c = make(oracle, al, dt)
        r2 = np.random.default_rng(5)
        for t in (a, b, c):
            H.fill_random(t, r2)
        pairs = H.pair_structure_oracle(oracle, a, b, c, ia, ib, ic)
        log = g["log%02d_t%d" % (ci, dt)]
        assert len(pairs) == len(log)
        mine = sorted((min(m, n), max(m, n), k, round(z.real, 6), round(z.imag, 6))
                      for _, z, m, n, k in pairs)
        theirs = sorted((int(min(r[1], r[2])), int(max(r[1], r[2])), int(r[3]),
                         round(r[4], 6), round(r[5], 6)) for r in log)
        assert mine == theirs
        for t in (a, b, c):
            t.free()


def test_oracle_elementwise_golden(oracle):
    g = gold("elementwise.npz")
    al = api.Allocator(oracle)
    for ci, (make, ia, ib) in enumerate(cases.ADD_TESTS):
        for dt in H.TYPES:
            for combo in range(4):
                rng = np.random.default_rng(9000 + 100 * ci + 10 * dt + combo)
                x, y = H.scalar(rng, dt), H.scalar(rng, dt)
                a, b = make(oracle, al, dt)
                H.fill_random(a, rng); H.fill_random(b, rng)
                api.add([0, 0, x, x][combo], a, [0, y, 0, y][combo], b, ia, ib)
                r = H.canon(a)
                np.testing.assert_allclose(digest(np.concatenate([r[k].ravel() for k in sorted(r)])),
                                           g["add%d_t%d_%d" % (ci, dt, combo)], rtol=1e-5, atol=H.TOL[dt])
                a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.MUL_DIV_TESTS):
        for dt in H.TYPES:
            for op in ("mul", "div"):
                rng = np.random.default_rng(12000 + 100 * ci + 10 * dt + (op == "div"))
                a, b = make(oracle, al, dt)
                H.fill_random(a, rng); H.fill_random(b, rng)
                (api.mul if op == "mul" else api.div)(a, b, ia, ib)
                r = H.canon(a)
                np.testing.assert_allclose(digest(np.concatenate([r[k].ravel() for k in sorted(r)])),
                                           g["%s%d_t%d" % (op, ci, dt)], rtol=1e-4, atol=H.TOL[dt])
                a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.DOT_TESTS):
        for dt in H.TYPES:
            rng = np.random.default_rng(15000 + 100 * ci + dt)
            a, b = make(oracle, al, dt)
            H.fill_random(a, rng); H.fill_random(b, rng)
            d = api.dot(a, b, ia, ib)
            ref = g["dot%d_t%d" % (ci, dt)][0]
            assert abs(d - ref) <= (1e-3 if dt < 2 else 1e-8) * max(1.0, abs(ref))
            a.free(); b.free()
    for ci, (make, ia, ib) in enumerate(cases.ADD_TESTS):
        for dt in H.TYPES:
            rng = np.random.default_rng(18000 + 100 * ci + dt)
            a, b = make(oracle, al, dt)
            H.fill_random(a, rng); H.fill_random(b, rng)
            api.copy(a, H.scalar(rng, dt), b, ia, ib)
            r = H.canon(a)
            np.testing.assert_allclose(digest(np.concatenate([r[k].ravel() for k in sorted(r)])),
                                       g["copy%d_t%d" % (ci, dt)], rtol=1e-5, atol=H.TOL[dt])
            a.free(); b.free()


def test_oracle_workloads_golden(oracle):
    g = gold("workloads.npz")
    al = api.Allocator(oracle)
    w = W.cfg1(oracle, al)
    w.run()
    r = H.canon(w.c)
    keys = sorted(r)
    assert np.array_equal(np.array(keys), g["cfg1_blocks"])
    np.testing.assert_allclose([r[k].sum() for k in keys], g["cfg1_sum"], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose([float(np.dot(r[k], r[k])) for k in keys], g["cfg1_sumsq"], rtol=1e-12)
    np.testing.assert_allclose(np.concatenate([r[k][:7] for k in keys]), g["cfg1_sample"], rtol=0, atol=1e-11)
    w.free()
    w = W.cfg2(oracle, al, scale=4)
    w.run()
    r = H.canon(w.c)
    keys = sorted(r)
    assert np.array_equal(np.array(keys), g["cfg2s4_blocks"])
    np.testing.assert_allclose(digest(np.concatenate([r[k] for k in keys])), g["cfg2s4_out"],
                               rtol=1e-10, atol=1e-11)
    w.free()


def test_oracle_vs_live_reference(oracle, reference):
    """Same inputs through both libraries: canonical outputs agree."""
    ao, ar = api.Allocator(oracle), api.Allocator(reference)
    for ci in (35, 36, 37, 38, 39, 40, 45):
        for dt in (api.DOUBLE, api.DOUBLE_COMPLEX):
            x = H.run_contract_case(oracle, ao, cases.CONTRACT_TESTS[ci], dt, 3 + ci, 0.7, -0.3)
            y = H.run_contract_case(reference, ar, cases.CONTRACT_TESTS[ci], dt, 3 + ci, 0.7, -0.3)
            assert H.max_abs_diff(x, y) < 1e-12
