"""GPU parity: the GB300 engine against the oracle on identical inputs.

Every contraction case of the reference test driver in all four scalar
types and all alpha/beta kinds (test.c:1993-2032), the element-wise
operations, unfold/fold round trips, the measured ladders, and a pagefile
(staged) allocator.  Tolerances: the reference's own absolute bounds
(1e-8 double, 1e-4 float; test.c:48-70) and, for double, a relative
Frobenius error <= 1e-12 against the oracle in both precision modes.
"""
import os
import tempfile

import numpy as np
import pytest

import cases
import helpers as H
from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

REL_FP64 = 1e-12      # relative Frobenius bound for double results
REL_FP32 = 1e-5


@pytest.fixture(scope="module")
def gal(engine):
    return api.Allocator(engine)


@pytest.fixture(scope="module")
def oal(oracle):
    return api.Allocator(oracle)


def _alpha_beta(rng, dt, combo):
    x, y = H.scalar(rng, dt), H.scalar(rng, dt)
    return [(0, 0), (0, y), (x, 0), (x, y)][combo]


def _check(x, y, dt):
    assert x.keys() == y.keys()
    assert H.max_abs_diff(x, y) <= H.TOL[dt]
    if x:
        rel = W.rel_frobenius(x, y)
        assert rel <= (REL_FP64 if dt >= 2 else REL_FP32), rel


@pytest.mark.parametrize("prec", [api.PREC_FP64, api.PREC_AUTO])
@pytest.mark.parametrize("ci", range(len(cases.CONTRACT_TESTS)))
def test_contract_cases(engine, oracle, gal, oal, ci, prec):
    engine.check(engine.xmg_set_precision(prec))
    for dt in H.TYPES:
        for combo in range(4):
            rng = np.random.default_rng(100 * ci + 10 * dt + combo)
            alpha, beta = _alpha_beta(rng, dt, combo)
            seed = 7 + 1000 * ci + 10 * dt + combo
            x = H.run_contract_case(engine, gal, cases.CONTRACT_TESTS[ci], dt, seed, alpha, beta)
            y = H.run_contract_case(oracle, oal, cases.CONTRACT_TESTS[ci], dt, seed, alpha, beta)
            _check(x, y, dt)
    engine.check(engine.xmg_set_precision(api.PREC_AUTO))


def _ew_pair(lib, al, make, dt, seed):
    a, b = make(lib, al, dt)
    rng = np.random.default_rng(seed)
    H.fill_random(a, rng)
    H.fill_random(b, rng)
    return a, b


@pytest.mark.parametrize("ci", range(len(cases.ADD_TESTS)))
def test_add_copy(engine, oracle, gal, oal, ci):
    make, ia, ib = cases.ADD_TESTS[ci]
    for dt in H.TYPES:
        for combo in range(4):
            rng = np.random.default_rng(ci * 31 + dt * 7 + combo)
            alpha, beta = _alpha_beta(rng, dt, combo)
            res = []
            for lib, al in ((engine, gal), (oracle, oal)):
                a, b = _ew_pair(lib, al, make, dt, 5 + ci)
                api.add(alpha, a, beta, b, ia, ib)
                res.append(H.canon(a))
                api.copy(a, beta if beta else 1.5, b, ia, ib)
                res.append(H.canon(a))
                a.free(); b.free()
            _check(res[0], res[2], dt)
            _check(res[1], res[3], dt)


def test_slab_transposes(engine, oracle, gal, oal, monkeypatch):
    """Permutations that swap the two leading indices of whole blocks
    (b's "cdab" -> "dcab"): xm_copy through the slab schedule (one bulk
    copy per CTA, the transpose in shared memory) where each slice's bytes
    are a multiple of 16, the matrix schedule elsewhere (odd slices here)
    and for the other operations.  Same results as the oracle in every
    scalar type, and bit for bit the matrix schedule's (XMG_PTASK_SLAB=0)
    for xm_copy, xm_add, xm_mul and xm_div."""
    o, v = [4, 6], [6, 8, 7, 10]
    for dt in H.TYPES:
        res = {}
        for name, lib, al, slab in (("slab", engine, gal, "1"), ("matrix", engine, gal, "0"),
                                    ("oracle", oracle, oal, "1")):
            monkeypatch.setenv("XMG_PTASK_SLAB", slab)
            w = W.ladder(lib, al, o, v, seed=5, dtype=dt)
            b2 = w.b.structure()
            W.fill(b2, 77, W.LADDER_ANTISYM)
            out = []
            api.copy(b2, 1.25, w.b, "cdab", "dcab")
            out.append(H.canon(b2))
            api.add(0.5, b2, -0.75, w.b, "cdab", "dcab")
            out.append(H.canon(b2))
            api.mul(b2, w.b, "cdab", "dcab")
            out.append(H.canon(b2))
            api.div(b2, w.b, "cdab", "dcab")
            out.append(H.canon(b2))
            res[name] = out
            b2.free()
            w.free()
        for x, y, z in zip(res["slab"], res["matrix"], res["oracle"]):
            assert x.keys() == y.keys() == z.keys()
            for k in x:
                np.testing.assert_array_equal(x[k], y[k])
                np.testing.assert_allclose(x[k], z[k], rtol=1e-4 if dt < 2 else 1e-12,
                                           atol=H.TOL[dt])


@pytest.mark.parametrize("ci", range(len(cases.MUL_DIV_TESTS)))
def test_mul_div(engine, oracle, gal, oal, ci):
    make, ia, ib = cases.MUL_DIV_TESTS[ci]
    for dt in H.TYPES:
        res = []
        for lib, al in ((engine, gal), (oracle, oal)):
            a, b = _ew_pair(lib, al, make, dt, 9 + ci)
            api.mul(a, b, ia, ib)
            res.append(H.canon(a))
            api.div(a, b, ia, ib)
            res.append(H.canon(a))
            a.free(); b.free()
        _check(res[0], res[2], dt)
        for k in res[1]:      # division amplifies: compare relatively
            np.testing.assert_allclose(res[1][k], res[3][k], rtol=1e-4 if dt < 2 else 1e-10,
                                       atol=H.TOL[dt])


@pytest.mark.parametrize("ci", range(len(cases.DOT_TESTS)))
def test_dot(engine, oracle, gal, oal, ci):
    make, ia, ib = cases.DOT_TESTS[ci]
    for dt in H.TYPES:
        d = []
        for lib, al in ((engine, gal), (oracle, oal)):
            a, b = _ew_pair(lib, al, make, dt, 11 + ci)
            d.append(api.dot(a, b, ia, ib))
            a.free(); b.free()
        assert abs(d[0] - d[1]) <= (1e-3 if dt < 2 else 1e-10) * max(1.0, abs(d[1]))


def test_set(engine, oracle, gal, oal):
    # test.c:1826-1860
    for dt in H.TYPES:
        x = complex(0.25, -0.5) if dt in (1, 3) else -0.375
        outs = []
        for lib, al in ((engine, gal), (oracle, oal)):
            bs = api.BlockSpace(lib, [3, 5, 1, 6, 3, 6, 9, 4])
            for d, p in [(0, 1), (0, 1), (1, 1), (1, 2), (3, 3), (5, 4), (6, 3), (6, 7)]:
                bs.split(d, p)
            a = api.Tensor(lib, bs, dt, al, canonical=True)
            bs.free()
            api.set_all(a, x)
            outs.append(H.canon(a))
            a.free()
        _check(outs[0], outs[1], dt)
        assert all(np.all(v == np.asarray(x, dtype=v.dtype)) for v in outs[0].values())


MASKS_3456 = [((0, 1, 2, 3), ()), ((2, 0, 1, 3), ()), ((1, 3, 2), (0,)), ((3, 2, 1), (0,)),
              ((3, 2), (1, 0)), ((3, 2), (0, 1)), ((2,), (3, 0, 1)), ((2,), (1, 3, 0)),
              ((), (0, 1, 2, 3)), ((), (0, 3, 2, 1)), ((), (1, 3, 2, 0))]


@pytest.mark.parametrize("dt", H.TYPES)
def test_unfold_fold(engine, oracle, gal, oal, dt):
    """test.c:1378-1451 masks on 5^4 blocks: unfold of a derivative block
    (its permutation applied) matches the oracle bit for bit; fold of the
    canonical block inverts unfold."""
    z, one = api.Dim.of([0] * 4), api.Dim.of([1] * 4)
    for perm in [(0, 1, 2, 3), (2, 3, 0, 1), (1, 0, 3, 2), (3, 1, 0, 2)]:
        outs = []
        for lib, al in ((engine, gal), (oracle, oal)):
            bs = api.BlockSpace(lib, [10, 10, 10, 10])
            for d in range(4):
                bs.split(d, 5)
            t = api.Tensor(lib, bs, dt, al)
            bs.free()
            t.set_canonical((0, 0, 0, 0))
            t.set_derivative((1, 1, 1, 1), (0, 0, 0, 0), perm, -1.0)
            H.fill_random(t, np.random.default_rng(3))
            raw = t.read_block((0, 0, 0, 0))
            res = []
            for mi, mj in MASKS_3456:
                ni = 5 ** len(mi)
                stride = ni + 3
                nj = 5 ** len(mj)
                to = np.full(stride * nj, 7.0, dtype=raw.dtype)
                lib.xm_tensor_unfold_block(t.h, one, api.Dim.of(mi), api.Dim.of(mj),
                                           raw.ctypes.data, to.ctypes.data, stride)
                res.append(to.copy())
                lib.xm_tensor_unfold_block(t.h, z, api.Dim.of(mi), api.Dim.of(mj),
                                           raw.ctypes.data, to.ctypes.data, stride)
                back = np.zeros_like(raw)
                lib.xm_tensor_fold_block(t.h, z, api.Dim.of(mi), api.Dim.of(mj),
                                         to.ctypes.data, back.ctypes.data, stride)
                assert np.array_equal(back, raw)
            outs.append(res)
            t.free()
        for x, y in zip(*outs):
            assert np.array_equal(x, y)


def test_unfold_derivative_block(engine, oracle, gal, oal):
    """Unfold of a derivative block applies its permutation (test.c:1192-1287)."""
    for dt in H.TYPES:
        outs = []
        for lib, al in ((engine, gal), (oracle, oal)):
            bs = api.BlockSpace(lib, [5, 10]).split(1, 5)
            t = api.Tensor(lib, bs, dt, al)
            bs.free()
            t.set_canonical((0, 0))
            t.set_derivative((0, 1), (0, 0), (1, 0), -0.3)
            H.fill_random(t, np.random.default_rng(4))
            raw = t.read_block((0, 1))
            to = np.zeros_like(raw)
            lib.xm_tensor_unfold_block(t.h, api.Dim.of([0, 1]), api.Dim.of([1]), api.Dim.of([0]),
                                       raw.ctypes.data, to.ctypes.data, 5)
            outs.append(to)
            t.free()
        assert np.array_equal(outs[0], outs[1])


def test_cfg1_ladder_golden_and_oracle(engine, oracle, gal, oal):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "workloads.npz"))
    for prec in (api.PREC_FP64, api.PREC_EMU64, api.PREC_AUTO):
        engine.check(engine.xmg_set_precision(prec))
        w = W.cfg1(engine, gal)
        w.run()
        r = H.canon(w.c)
        w.free()
        keys = sorted(r)
        assert np.array_equal(np.array(keys), g["cfg1_blocks"])
        np.testing.assert_allclose([r[k].sum() for k in keys], g["cfg1_sum"], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose([float(np.dot(r[k], r[k])) for k in keys], g["cfg1_sumsq"], rtol=1e-11)
    engine.check(engine.xmg_set_precision(api.PREC_AUTO))
    wo = W.cfg1(oracle, oal)
    wo.run()
    ref = H.canon(wo.c)
    wo.free()
    for prec in (api.PREC_FP64, api.PREC_EMU64):
        engine.check(engine.xmg_set_precision(prec))
        w = W.cfg1(engine, gal)
        w.run()
        rel = W.rel_frobenius(H.canon(w.c), ref)
        w.free()
        assert rel <= REL_FP64, (prec, rel)
    engine.check(engine.xmg_set_precision(api.PREC_AUTO))


def test_cfg2_scaled_golden(engine, gal):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "workloads.npz"))
    for prec in (api.PREC_FP64, api.PREC_EMU64):
        engine.check(engine.xmg_set_precision(prec))
        w = W.cfg2(engine, gal, scale=4)
        w.run()
        r = H.canon(w.c)
        w.free()
        keys = sorted(r)
        assert np.array_equal(np.array(keys), g["cfg2s4_blocks"])
        x = np.concatenate([r[k] for k in keys])
        ref = g["cfg2s4_out"]
        if x.size > 4096:
            x = np.concatenate([[x.sum(), np.dot(x, x)], x[::97]])
        np.testing.assert_allclose(x, ref, rtol=1e-10, atol=1e-11)
    engine.check(engine.xmg_set_precision(api.PREC_AUTO))


def test_pagefile_allocator_contract(engine, oracle, oal):
    """Tensors in a host pagefile: the engine stages blocks into HBM (with
    alpha = 0 no GEMM runs and only beta is applied to c)."""
    d = tempfile.mkdtemp()
    pal = api.Allocator(engine, os.path.join(d, "xmpagefile"))
    for ci in (35, 38, 45):
        for alpha, beta in ((0.5, 0.25), (0.0, 0.25), (0.0, 0.0)):
            x = H.run_contract_case(engine, pal, cases.CONTRACT_TESTS[ci], api.DOUBLE, 1 + ci,
                                    alpha, beta)
            y = H.run_contract_case(oracle, oal, cases.CONTRACT_TESTS[ci], api.DOUBLE, 1 + ci,
                                    alpha, beta)
            _check(x, y, api.DOUBLE)
    pal.destroy()
    os.rmdir(d)
