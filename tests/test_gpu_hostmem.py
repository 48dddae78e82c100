"""GPU: tensors in page-locked host memory (xmg_allocator_create_host).

Every contraction on such tensors streams its operands through HBM: a's
(and, for beta != 0, c's) blocks and b's first batch, then the remaining
batches of b while the previous one is contracted, and c back.  Checked
against the oracle on identical inputs: every reference contraction case
in the four scalar types and the four alpha/beta kinds, the ladders and
the ring term in both precision modes; the kept streamed plan is replayed
on repeated calls (no planning) and still sees new data, new scalars and
changed structures; element-wise operations and the block list calls.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import helpers as H
from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module")
def hal(engine):
    al = api.Allocator(engine, host=True)
    yield al
    engine.xmg_plan_cache_clear()
    al.destroy()


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
        assert W.rel_frobenius(x, y) <= (REL if dt >= 2 else 1e-5)


@pytest.mark.parametrize("ci", range(len(cases.CONTRACT_TESTS)))
def test_contract_cases_host_memory(engine, oracle, hal, oal, ci):
    for dt in H.TYPES:
        for combo in range(4):
            rng = np.random.default_rng(300 * ci + 10 * dt + combo)
            alpha, beta = _alpha_beta(rng, dt, combo)
            seed = 17 + 1000 * ci + 10 * dt + combo
            x = H.run_contract_case(engine, hal, cases.CONTRACT_TESTS[ci], dt, seed, alpha, beta)
            y = H.run_contract_case(oracle, oal, cases.CONTRACT_TESTS[ci], dt, seed, alpha, beta)
            _check(x, y, dt)


@pytest.mark.parametrize("prec", [api.PREC_AUTO, api.PREC_FP64])
def test_ladder_host_memory_streamed(engine, oracle, hal, oal, prec):
    """The uneven Z2^3 ladder (block sizes / 4) with alpha and beta: b in
    several batches, each contracted while the next one is copied."""
    engine.check(engine.xmg_set_precision(prec))
    we, wo = W.cfg2(engine, hal, scale=4), W.cfg2(oracle, oal, scale=4)
    try:
        for w in (we, wo):
            W.fill(w.c, 33, W.LADDER_ANTISYM)
            w.alpha, w.beta = 0.7, -0.5
        we.run()
        wo.run()
        st = api.last_stats(engine)
        assert st.stage_batches > 1 and st.stage_bytes > 0
        assert st.precision_used == (api.PREC_EMU64 if prec == api.PREC_AUTO else api.PREC_FP64)
        assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        we.free()
        wo.free()


@pytest.mark.parametrize("dtype", [api.DOUBLE, api.DOUBLE_COMPLEX, api.FLOAT])
def test_ring_host_memory(engine, oracle, hal, oal, dtype):
    hi = {api.FLOAT: api.DOUBLE}.get(dtype, dtype)
    we = W.cfg3(engine, hal, dtype=dtype, o_blk=6, v_blk=10)
    wo = W.cfg3(oracle, oal, dtype=hi, o_blk=6, v_blk=10, fill_data=False)
    try:
        for ts, td in zip(we.tensors(), wo.tensors()):
            W.copy_data(ts, td)
        we.run()
        wo.run()
        assert api.last_stats(engine).stage_batches > 1
        rel = W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c))
        assert rel <= (REL if dtype != api.FLOAT else 1e-6), rel
    finally:
        we.free()
        wo.free()


def test_kept_streamed_plan(engine, oracle, hal, oal):
    """Repeated calls replay the kept plan (no planning after the first
    two calls) and still see new data in a and b, accumulate through beta
    every call, and a changed structure or scalar draws a new plan."""
    we, wo = W.cfg2(engine, hal, scale=4), W.cfg2(oracle, oal, scale=4)
    try:
        for w in (we, wo):
            W.fill(w.c, 35, W.LADDER_ANTISYM)
            w.alpha, w.beta = 1.25, 0.5
        plan_ms = []
        for step in range(4):
            if step == 2:
                # new data in one block of each operand
                for w in (we, wo):
                    for t, seed in ((w.a, 91), (w.b, 92)):
                        blk = t.canonical_blocks()[3]
                        t.write_block(blk, W.uniform(seed, t.block_size(blk)))
            we.run()
            wo.run()
            st = api.last_stats(engine)
            plan_ms.append(st.ms_plan)
            assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL, step
        # the first call plans; the replays plan nothing
        assert max(plan_ms[2:]) < 0.25 * plan_ms[0] + 0.5, plan_ms
        # another alpha: a new plan, still right
        for w in (we, wo):
            w.alpha = -0.75
            w.run()
        assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
        # a changed structure of c: a new plan
        for w in (we, wo):
            blk = w.c.canonical_blocks()[0]
            w.c.lib.xm_tensor_set_zero_block(w.c.h, api.Dim.of(blk))
            w.run()
        assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
    finally:
        we.free()
        wo.free()


def test_shared_a_side(engine, oracle, hal, oal, monkeypatch):
    """a's split-precision operands prepared once per call by batch 0 and
    read by the later batches (XMG_STREAM_SHARE_A=1, the default) give the
    oracle's result as splitting a in every batch does, on replays of the
    kept plan too, with less slice workspace; an Inf in a reaches every
    batch (all of them fall back to FP64) and clean data brings the
    split-precision path back."""
    slice_bytes = {}
    for share in ("0", "1"):
        monkeypatch.setenv("XMG_STREAM_SHARE_A", share)
        we, wo = W.cfg2(engine, hal, scale=4), W.cfg2(oracle, oal, scale=4)
        try:
            for w in (we, wo):
                W.fill(w.c, 37, W.LADDER_ANTISYM)
                w.alpha, w.beta = 0.9, 0.25
            for _ in range(2):
                we.run()
                wo.run()
                st = api.last_stats(engine)
                assert st.stage_batches > 1
                assert st.precision_used == api.PREC_EMU64
                assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
            slice_bytes[share] = st.slice_bytes
            for w in (we, wo):
                blk = w.a.canonical_blocks()[0]
                x = w.a.read_block(blk)
                x.flat[0] = np.inf
                w.a.write_block(blk, x)
                w.run()
            assert api.last_stats(engine).precision_used == api.PREC_FP64
            got, ref = W.read_canonical(we.c), W.read_canonical(wo.c)
            for k in ref:
                np.testing.assert_allclose(got[k], ref[k], rtol=1e-10, atol=1e-10)
            for w in (we, wo):
                W.fill(w.a, 38, W.LADDER_ANTISYM)
                W.fill(w.c, 39, W.LADDER_ANTISYM)
                w.run()
            assert api.last_stats(engine).precision_used == api.PREC_EMU64
            assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
        finally:
            we.free()
            wo.free()
    assert slice_bytes["1"] < slice_bytes["0"], slice_bytes


@pytest.mark.parametrize("order,early", [("file", "1"), ("output", "0"), ("output", "1")])
def test_stream_orders(engine, oracle, hal, oal, monkeypatch, order, early):
    """b's batches cut in file order or in the output blocks' order
    (XMG_STREAM_ORDER), c written back after the last batch or block by
    block once final (XMG_STREAM_CWRITE): the oracle's result every way,
    with beta accumulating over repeated calls of the kept plan."""
    monkeypatch.setenv("XMG_STREAM_ORDER", order)
    monkeypatch.setenv("XMG_STREAM_CWRITE", early)
    we, wo = W.cfg2(engine, hal, scale=4), W.cfg2(oracle, oal, scale=4)
    try:
        for w in (we, wo):
            W.fill(w.c, 41, W.LADDER_ANTISYM)
            w.alpha, w.beta = -1.1, 0.5
        for step in range(3):
            we.run()
            wo.run()
            assert api.last_stats(engine).stage_batches > 1
            assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL, step
    finally:
        we.free()
        wo.free()


def test_elementwise_host_memory(engine, oracle, hal, oal):
    """xm_set, xm_add with a permutation, xm_dot on host-memory tensors."""
    for dt in (api.DOUBLE, api.FLOAT_COMPLEX):
        res = []
        for lib, al in ((engine, hal), (oracle, oal)):
            a, b = cases.ADD_TESTS[3][0](lib, al, dt)
            rng = np.random.default_rng(61)
            H.fill_random(a, rng)
            H.fill_random(b, rng)
            ia, ib = cases.ADD_TESTS[3][1:]
            api.add(0.5, a, -1.5, b, ia, ib)
            res.append(H.canon(a))
            res.append(api.dot(a, b, ia, ib))
            api.set_all(b, 0.25)
            res.append(H.canon(b))
            a.free(); b.free()
        _check(res[0], res[3], dt)
        assert abs(res[1] - res[4]) <= (1e-3 if dt < 2 else 1e-10) * max(1.0, abs(res[4]))
        _check(res[2], res[5], dt)


@pytest.mark.parametrize("where", ["gpu", "host"])
def test_block_list_calls(engine, hal, where):
    """xmg_tensor_write_blocks / read_blocks round trip, against the
    one-block calls, and their argument checks."""
    al = api.Allocator(engine) if where == "gpu" else hal
    w = W.cfg2(engine, al, scale=4)          # zero, canonical and derivative blocks
    try:
        blocks = w.b.canonical_blocks()
        data = [W.uniform(200 + i, w.b.block_size(blk)) for i, blk in enumerate(blocks)]
        w.b.write_blocks(blocks, [d.ctypes.data for d in data])
        for blk, d in zip(blocks, data):
            assert np.array_equal(w.b.read_block(blk), d)
        # every nonzero block, derivative ones read their source's data
        nz = [blk for blk in np.ndindex(*w.b.nblocks()) if w.b.block_type(blk) != api.ZERO]
        outs = [np.empty(w.b.block_size(blk)) for blk in nz]
        w.b.read_blocks(nz, [o.ctypes.data for o in outs])
        for blk, o in zip(nz, outs):
            assert np.array_equal(o, w.b.read_block(blk))
        der = next(blk for blk in nz if w.b.block_type(blk) == api.DERIVATIVE)
        with pytest.raises(api.XmError, match="canonical"):
            w.b.write_blocks([der], [data[0].ctypes.data])
        zero = next(blk for blk in np.ndindex(*w.a.nblocks()) if w.a.block_type(blk) == api.ZERO)
        buf = np.empty(w.a.block_size(zero))
        with pytest.raises(api.XmError, match="zero-blocks"):
            w.a.read_blocks([zero], [buf.ctypes.data])
        with pytest.raises(api.XmError, match="out of range"):
            w.a.read_blocks([(9, 9, 9, 9)], [buf.ctypes.data])
    finally:
        w.free()
        if where == "gpu":
            al.destroy()
