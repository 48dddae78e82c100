"""GPU: cached device plans, CUDA-graph replay and the tile autotuner.

xmg_contract keeps a device plan per (tensors, structure generations,
index strings, alpha, beta, precision) and replays its captured CUDA graph;
the first runs of a split-precision plan try each tile-orientation policy
once.  Every replay must give the oracle's result: repeated runs (all
tuning candidates included), new operand data written between replays,
beta accumulation across replays, tensors recreated at recycled addresses,
and Inf operands inside a replayed plan (FP64 fallback under AUTO, an error
under EMU64).  The ladder is cfg2's structure with block sizes divided by 4.
"""
import numpy as np
import pytest

from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

REL = 1e-12
SCALE = 4


@pytest.fixture(scope="module")
def gal(engine):
    return api.Allocator(engine)


@pytest.fixture(scope="module")
def oal(oracle):
    return api.Allocator(oracle)


def _pair(engine, oracle, gal, oal, seed=2):
    return W.cfg2(engine, gal, seed=seed, scale=SCALE), W.cfg2(oracle, oal, seed=seed, scale=SCALE)


def _rel(w, wo):
    return W.rel_frobenius(W.read_canonical(w.c), W.read_canonical(wo.c))


def test_replay_and_tuning(engine, oracle, gal, oal):
    w, wo = _pair(engine, oracle, gal, oal)
    wo.run()
    engine.check(engine.xmg_set_precision(api.PREC_EMU64))
    try:
        for r in range(6):
            n0 = engine.xmg_kernel_launches()
            w.run()
            st = api.last_stats(engine)
            assert st.precision_used == api.PREC_EMU64
            assert engine.xmg_kernel_launches() - n0 >= 3
            rel = _rel(w, wo)
            assert rel <= REL, (r, rel)
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        w.free()
        wo.free()


def test_new_operand_data_between_replays(engine, oracle, gal, oal):
    w, wo = _pair(engine, oracle, gal, oal)
    try:
        for r in range(3):
            w.run()
        for x in (w, wo):
            W.fill(x.a, 977, W.LADDER_ANTISYM)
            W.fill(x.b, 978, W.LADDER_ANTISYM)
        w.run()
        wo.run()
        assert _rel(w, wo) <= REL
    finally:
        w.free()
        wo.free()


def test_beta_accumulates_across_replays(engine, oracle, gal, oal):
    w, wo = _pair(engine, oracle, gal, oal)
    try:
        for x in (w, wo):
            W.fill(x.c, 979, W.LADDER_ANTISYM)
            x.alpha, x.beta = 0.75, 1.0
        for r in range(4):
            w.run()
            wo.run()
        assert _rel(w, wo) <= REL
    finally:
        w.free()
        wo.free()


def test_recreated_tensors_get_new_plans(engine, oracle, gal, oal):
    for seed in (2, 5, 2):
        w, wo = _pair(engine, oracle, gal, oal, seed)
        try:
            w.run()
            w.run()
            wo.run()
            assert _rel(w, wo) <= REL, seed
        finally:
            w.free()
            wo.free()


def _poison(t, value):
    blk = t.canonical_blocks()[0]
    x = t.read_block(blk)
    x.flat[0] = value
    t.write_block(blk, x)


def test_inf_operand_in_replayed_plan(engine, oracle, gal, oal):
    w, wo = _pair(engine, oracle, gal, oal)
    try:
        w.run()
        w.run()
        assert api.last_stats(engine).precision_used == api.PREC_EMU64
        for x in (w, wo):
            _poison(x.a, np.inf)
        w.run()
        wo.run()
        assert api.last_stats(engine).precision_used == api.PREC_FP64
        got, ref = W.read_canonical(w.c), W.read_canonical(wo.c)
        for k in ref:
            np.testing.assert_allclose(got[k], ref[k], rtol=1e-10, atol=1e-10)
        engine.check(engine.xmg_set_precision(api.PREC_EMU64))
        with pytest.raises(api.XmError, match="Inf/NaN"):
            w.run()
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        for x in (w, wo):
            W.fill(x.a, 7, W.LADDER_ANTISYM)
        w.run()
        wo.run()
        assert api.last_stats(engine).precision_used == api.PREC_EMU64
        assert _rel(w, wo) <= REL
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        w.free()
        wo.free()


def test_cta_pair_kernel(engine, oracle, gal, oal, monkeypatch):
    """The opt-in CTA-pair form of the split-precision GEMM (256-row tiles,
    cta_group::2 MMAs over a cluster of two CTAs) gives the oracle's result.
    The work-list policy is fixed to the pair form through the environment
    (read when a plan is built)."""
    monkeypatch.setenv("XMG_CTA_PAIR", "1")
    monkeypatch.setenv("XMG_POLICY", "3")
    w, wo = _pair(engine, oracle, gal, oal, seed=9)
    try:
        engine.check(engine.xmg_set_precision(api.PREC_EMU64))
        wo.run()
        for _ in range(2):
            w.run()
            assert api.last_stats(engine).precision_used == api.PREC_EMU64
            assert _rel(w, wo) <= REL
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        w.free()
        wo.free()


@pytest.mark.parametrize("policy", [0, 6])
def test_work_list_policies(engine, oracle, gal, oal, monkeypatch, policy):
    """A fixed work-list policy (read when a plan is built) runs and gives
    the oracle's result: 0 (one output block per tile) and 6 (stacked
    tiles: N-side tails of blocks sharing an M side in common columns,
    M-side tails of blocks sharing an N side in common lanes); the
    statistics report the policy that ran."""
    monkeypatch.setenv("XMG_POLICY", str(policy))
    w, wo = _pair(engine, oracle, gal, oal, seed=11)
    try:
        engine.check(engine.xmg_set_precision(api.PREC_EMU64))
        wo.run()
        w.run()
        st = api.last_stats(engine)
        assert st.precision_used == api.PREC_EMU64
        assert st.gemm_policy == policy
        assert _rel(w, wo) <= REL
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        w.free()
        wo.free()


def test_stacked_work_list_ring_complex(engine, oracle, monkeypatch):
    """The stacked work list on the permuted ring term in complex128 (two
    real passes, beta = 1, transposes on both unfolds and the fold)."""
    monkeypatch.setenv("XMG_POLICY", "6")
    eal, oal2 = api.Allocator(engine), api.Allocator(oracle)
    we = W.cfg3(engine, eal, dtype=api.DOUBLE_COMPLEX, o_blk=6, v_blk=10)
    wo = W.cfg3(oracle, oal2, dtype=api.DOUBLE_COMPLEX, o_blk=6, v_blk=10)
    try:
        wo.run()
        we.run()
        st = api.last_stats(engine)
        assert st.precision_used == api.PREC_EMU64 and st.gemm_policy == 6
        assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= REL
    finally:
        we.free()
        wo.free()
