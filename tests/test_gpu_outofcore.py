"""GPU: out-of-core contractions with b streamed from the pagefile.

With the staging budget forced to one byte, every pagefile contraction
streams b through two HBM regions in batches (side-stream copies, from
pinned chunks the reader threads fill or straight from the file's mapping,
overlapping the previous batch's contraction).  The regions are
made small so that the ladders split into many batches.  Results must
match the oracle (in-memory tensors, same inputs) in both precision modes
with alpha and beta applied exactly once, the out-of-core statistics must
show the batches, and a block larger than a region must be refused.
"""
import os
import tempfile

import numpy as np
import pytest

from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture()
def staging(engine):
    engine.check(engine.xmg_set_staging(1, 3 << 20))
    yield engine
    engine.check(engine.xmg_set_staging(int(180e9), int(32e9)))


@pytest.fixture()
def pagefile(engine):
    d = tempfile.mkdtemp()
    al = api.Allocator(engine, os.path.join(d, "xmpagefile"))
    yield al
    al.destroy()


def _copy_inputs(src, dst):
    for ts, td in zip(src.tensors(), dst.tensors()):
        for blk in ts.canonical_blocks():
            td.write_block(blk, ts.read_block(blk))


@pytest.mark.parametrize("mapped", ["0", "1"])
@pytest.mark.parametrize("prec", [api.PREC_AUTO, api.PREC_FP64])
def test_ladder_streamed(engine, oracle, staging, pagefile, prec, mapped, monkeypatch):
    """Both ways of reading the pagefile: reader threads through pinned
    chunks (XMG_STAGE_MMAP=0) and copies straight from the file's mapping
    (=1; the default where the device reads pageable host memory)."""
    monkeypatch.setenv("XMG_STAGE_MMAP", mapped)
    engine.check(engine.xmg_set_precision(prec))
    oal = api.Allocator(oracle)
    we, wo = W.cfg1(engine, pagefile), W.cfg1(oracle, oal)
    try:
        for w in (we, wo):
            W.fill(w.c, 31, W.LADDER_ANTISYM)
            w.alpha, w.beta = 0.7, -0.5
        _copy_inputs(wo, we)
        we.run()
        wo.run()
        st = api.last_stats(engine)
        assert st.stage_batches > 1
        assert st.stage_bytes > 0
        assert st.precision_used == (api.PREC_EMU64 if prec == api.PREC_AUTO else api.PREC_FP64)
        rel = W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c))
        assert rel <= REL, rel
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        we.free()
        wo.free()


@pytest.mark.parametrize("dtype", [api.DOUBLE, api.DOUBLE_COMPLEX])
def test_ring_streamed(engine, oracle, staging, pagefile, dtype):
    """Permuted ring term (transposes on both unfolds and the fold, beta = 1,
    pair-symmetric c) with b streamed."""
    oal = api.Allocator(oracle)
    we = W.cfg3(engine, pagefile, dtype=dtype, o_blk=6, v_blk=10)
    wo = W.cfg3(oracle, oal, dtype=dtype, o_blk=6, v_blk=10)
    try:
        _copy_inputs(we, wo)
        we.run()
        wo.run()
        assert api.last_stats(engine).stage_batches > 1
        rel = W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c))
        assert rel <= REL, rel
    finally:
        we.free()
        wo.free()


def test_streamed_equals_in_core(engine, staging, pagefile):
    """The same FP64 contraction streamed and in core (HBM tensors) agree to
    the last bits: only the batch order of the accumulation differs."""
    engine.check(engine.xmg_set_precision(api.PREC_FP64))
    gal = api.Allocator(engine)
    ws, wr = W.cfg2(engine, pagefile, scale=4), W.cfg2(engine, gal, scale=4)
    try:
        ws.run()
        assert api.last_stats(engine).stage_batches > 1
        wr.run()
        assert api.last_stats(engine).stage_batches == 0
        a, b = W.read_canonical(ws.c), W.read_canonical(wr.c)
        assert W.rel_frobenius(a, b) <= 1e-14
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        ws.free()
        wr.free()


def test_block_larger_than_region(engine, pagefile):
    engine.check(engine.xmg_set_staging(1, 4096))
    w = W.cfg1(engine, pagefile)
    try:
        with pytest.raises(api.XmError, match="staging region"):
            w.run()
    finally:
        engine.check(engine.xmg_set_staging(int(180e9), int(32e9)))
        w.free()


def test_production_ladder_streamed(engine, oracle, staging, pagefile):
    """The production ladder's structure (o = 128 as 8 x 16, v blocks of
    24..40, Z2^3 labels) with block sizes divided by 4 and its first 10 v
    blocks, b streamed in batches, against the oracle in both precision
    modes; the two modes also agree with each other."""
    oal = api.Allocator(oracle)
    we = W.cfg5(engine, pagefile, scale=4, v_blocks=10)
    wo = W.cfg5(oracle, oal, scale=4, v_blocks=10)
    try:
        wo.run()
        ref = W.read_canonical(wo.c)
        got = {}
        for prec in (api.PREC_AUTO, api.PREC_FP64):
            engine.check(engine.xmg_set_precision(prec))
            we.run()
            st = api.last_stats(engine)
            assert st.stage_batches > 1
            got[prec] = W.read_canonical(we.c)
            assert W.rel_frobenius(got[prec], ref) <= REL, prec
        assert W.rel_frobenius(got[api.PREC_AUTO], got[api.PREC_FP64]) <= REL
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        we.free()
        wo.free()
