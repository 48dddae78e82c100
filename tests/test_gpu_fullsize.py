"""Parity at the measured configurations' full sizes.

The engine runs the whole contraction; the oracle computes a seeded sample
of the canonical output blocks on identical inputs (its other output blocks
are zero blocks, so it does only the sample's work).  Covered:

* the uneven Z2^3 ladder, o = 96 in 6 blocks, v = 384 in 12 blocks, in
  split-precision and plain FP64 form (relative Frobenius error <= 1e-12);
* the permuted ring term C(i,a,j,b) += A(k,i,c,a) B(j,k,b,c), o = 64 as
  4 x 16, v = 256 as 8 x 32 (K = 512 per block pair, the reference's 512^3
  GEMMs of contract.c:193-218), in complex128 (<= 1e-12) and float32
  (compensated bf16 split <= 1e-6, plain FP32 <= 1e-5, against the FP64
  oracle on the float-rounded inputs);
* the adjoint of the ladder at full size: dA and dB on sampled canonical
  blocks against the oracle's two gradient contractions (<= 1e-11).
"""
import numpy as np
import pytest

import helpers as H
from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

SAMPLE = 48


def _sampled_rel(got, ref):
    return W.rel_frobenius({k: got[k] for k in ref}, ref)


@pytest.fixture(scope="module")
def ladder_pair(engine, oracle):
    """The full-size uneven Z2^3 ladder on the engine and its copy on the
    oracle (shared by the forward and adjoint tests)."""
    eal, oal = api.Allocator(engine), api.Allocator(oracle)
    we = W.cfg2(engine, eal)
    wo = W.cfg2(oracle, oal, fill_data=False)
    W.copy_data(we.a, wo.a)
    W.copy_data(we.b, wo.b)
    yield we, wo
    we.free()
    wo.free()
    eal.destroy()
    oal.destroy()


@pytest.mark.parametrize("prec", [api.PREC_AUTO, api.PREC_FP64])
def test_ladder_full_size(engine, ladder_pair, prec):
    we, wo = ladder_pair
    chosen = W.sample_blocks(we.c.canonical_blocks(), SAMPLE, seed=21)
    ref = W.contract_sample(wo, chosen)
    engine.check(engine.xmg_set_precision(prec))
    try:
        we.run()
        st = api.last_stats(engine)
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
    got = {blk: we.c.read_block(blk) for blk in chosen}
    rel = _sampled_rel(got, ref)
    assert rel <= 1e-12, rel
    assert st.precision_used == (api.PREC_FP64 if prec == api.PREC_FP64 else api.PREC_EMU64)


@pytest.mark.parametrize("dtype,precs", [
    (api.DOUBLE_COMPLEX, [(api.PREC_AUTO, 1e-12)]),
    (api.FLOAT, [(api.PREC_AUTO, 1e-6), (api.PREC_FP64, 1e-5)])])
def test_ring_term_full_size(engine, oracle, dtype, precs):
    hi = {api.FLOAT: api.DOUBLE}.get(dtype, dtype)
    eal, oal = api.Allocator(engine), api.Allocator(oracle)
    we = W.cfg3(engine, eal, dtype=dtype)
    wo = W.cfg3(oracle, oal, dtype=hi, fill_data=False)
    W.copy_data(we.a, wo.a)
    W.copy_data(we.b, wo.b)
    chosen = W.sample_blocks(we.c.canonical_blocks(), SAMPLE, seed=31)
    c0 = {blk: we.c.read_block(blk) for blk in chosen}
    ref = W.contract_sample(wo, chosen, {k: v.astype(wo.c.np) for k, v in c0.items()})
    try:
        for prec, tol in precs:
            engine.check(engine.xmg_set_precision(prec))
            for blk, x in c0.items():       # beta = 1: start from the same C
                we.c.write_block(blk, x)
            we.run()
            st = api.last_stats(engine)
            got = {blk: we.c.read_block(blk) for blk in chosen}
            rel = _sampled_rel(got, ref)
            assert rel <= tol, (prec, rel)
            if prec == api.PREC_AUTO:
                assert st.precision_used == api.PREC_EMU64
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        we.free()
        wo.free()
        eal.destroy()
        oal.destroy()


def test_adjoint_full_size(engine, oracle, ladder_pair):
    """xm_contract_adjoint on the full-size ladder: dA and dB on sampled
    canonical blocks against the oracle's W * B and A * W at every position
    that maps onto them, W being dC folded onto C's canonical blocks with
    its multiplicity."""
    we, wo = ladder_pair
    alpha = 1.0
    oal = wo.a.alloc        # xm_contract wants one allocator for all three
    dce = we.c.structure()
    W.fill(dce, 77, W.LADDER_ANTISYM)
    da, db = we.a.structure(), we.b.structure()
    api.set_all(da, 0)
    api.set_all(db, 0)
    engine.check(engine.xm_contract_adjoint(api.Scalar.of(alpha), we.a.h, we.b.h, dce.h,
                                            da.h, db.h, b"ijcd", b"cdab", b"ijab"))
    st = api.last_stats(engine)
    sa = W.sample_blocks(da.canonical_blocks(), SAMPLE, seed=41)
    sb = W.sample_blocks(db.canonical_blocks(), SAMPLE, seed=42)
    gda = {blk: da.read_block(blk) for blk in sa}
    gdb = {blk: db.read_block(blk) for blk in sb}

    lib = oracle
    dco = wo.c.structure()
    W.copy_data(dce, dco)
    wt = H.folded_cotangent(lib, oal, dco)
    ref_da = H.sampled_gradient(lib, oal, wo.a, wt, wo.b, "ijab", "cdab", "ijcd", alpha, sa, True)
    ref_db = H.sampled_gradient(lib, oal, wo.b, wt, wo.a, "ijab", "ijcd", "cdab", alpha, sb, False)
    rel_a = W.rel_frobenius(gda, ref_da)
    rel_b = W.rel_frobenius(gdb, ref_db)
    for x in (da, db, dce, wt, dco):
        x.free()
    assert rel_a <= 1e-11, rel_a
    assert rel_b <= 1e-11, rel_b
    assert st.precision_used == api.PREC_EMU64
