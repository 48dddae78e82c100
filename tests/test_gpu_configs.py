"""The remaining measured workloads as parity cases: the permuted ring term
(float32 and complex128, beta = 1, pair-symmetric output) and the
hand-written adjoint of the ladder (checked against the oracle's
contractions and against finite differences of L = <dC, C>)."""
import numpy as np
import pytest

import helpers as H
from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [api.PREC_AUTO, api.PREC_FP64])
@pytest.mark.parametrize("dtype,tol", [(api.FLOAT, 1e-6), (api.DOUBLE_COMPLEX, 1e-12),
                                       (api.DOUBLE, 1e-12), (api.FLOAT_COMPLEX, 1e-6)])
def test_ring_term(engine, oracle, dtype, tol, prec):
    """C(i,a,j,b) += sum_{k,c} A(k,i,c,a) B(j,k,b,c) with 4 x 8 blocks of a
    reduced size (same structure as the 64 / 256 configuration), against
    an FP64 oracle on identical (for float types: float-rounded) inputs.
    Plain FP32 accumulation is held to 1e-5; the split paths to 1e-6."""
    engine.check(engine.xmg_set_precision(prec))
    hi = {api.FLOAT: api.DOUBLE, api.FLOAT_COMPLEX: api.DOUBLE_COMPLEX}.get(dtype, dtype)
    eal, oal = api.Allocator(engine), api.Allocator(oracle)
    we = W.cfg3(engine, eal, dtype=dtype, o_blk=6, v_blk=10)
    wo = W.cfg3(oracle, oal, dtype=hi, o_blk=6, v_blk=10)
    for te, to in zip(we.tensors(), wo.tensors()):
        for blk in te.canonical_blocks():
            to.write_block(blk, te.read_block(blk).astype(api.NP_TYPES[hi]))
    we.run()
    wo.run()
    rel = W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c))
    st = api.last_stats(engine)
    we.free()
    wo.free()
    engine.check(engine.xmg_set_precision(api.PREC_AUTO))
    bound = tol if (prec == api.PREC_AUTO or dtype >= 2) else 1e-5
    assert rel <= bound, (rel, st.precision_used)
    if prec == api.PREC_AUTO:
        assert st.precision_used == api.PREC_EMU64


def _loss(lib, w, dc):
    return api.dot(w.c, dc, w.idxc, w.idxc)


def test_adjoint_ladder(engine, oracle):
    """da, db from xm_contract_adjoint against (1) the oracle computing the
    two gradient contractions and folding derivative blocks back in numpy,
    (2) central differences of L = <dC, alpha * A * B>."""
    alpha = 0.75
    eal, oal = api.Allocator(engine), api.Allocator(oracle)
    res = {}
    for lib, al in ((engine, eal), (oracle, oal)):
        w = W.cfg2(lib, al, scale=4)
        w.alpha = alpha
        dc = w.c.structure()
        W.fill(dc, 77, W.LADDER_ANTISYM)
        res[lib.path] = (w, dc)
    (we, dce), (wo, dco) = res[engine.path], res[oracle.path]
    da = we.a.structure()
    db = we.b.structure()
    api.set_all(da, 0)
    api.set_all(db, 0)
    engine.check(engine.xm_contract_adjoint(api.Scalar.of(alpha), we.a.h, we.b.h, dce.h,
                                            da.h, db.h, b"ijcd", b"cdab", b"ijab"))
    gda, gdb = W.read_canonical(da), W.read_canonical(db)

    # (1) reference gradient with the oracle: W = mult * dc on canonical
    # positions, G = alpha W B (resp. alpha A W) at every nonzero position,
    # folded back through each block's permutation and scalar.
    lib = oracle
    nb = dco.nblocks()
    wt = api.Tensor(lib, None, api.DOUBLE, oal,
                    handle=lib.xm_tensor_create(lib.xm_tensor_get_block_space(dco.h), api.DOUBLE, oal.h))
    mult = {}
    for blk in np.ndindex(*nb):
        if dco.block_type(blk) == api.ZERO:
            continue
        mult.setdefault(dco.data_ptr(blk), 0.0)
        mult[dco.data_ptr(blk)] += dco.block_scalar(blk).real ** 2
    for blk in dco.canonical_blocks():
        wt.set_canonical(blk)
        wt.write_block(blk, dco.read_block(blk) * mult[dco.data_ptr(blk)])

    def full_grad_tensor(t):
        g = api.Tensor(lib, None, api.DOUBLE, oal,
                       handle=lib.xm_tensor_create(lib.xm_tensor_get_block_space(t.h), api.DOUBLE, oal.h))
        for blk in np.ndindex(*t.nblocks()):
            if t.block_type(blk) != api.ZERO:
                g.set_canonical(blk)
        return g

    def fold(t, g):
        out = {blk: np.zeros(t.block_size(blk)) for blk in t.canonical_blocks()}
        ptr2canon = {t.data_ptr(blk): blk for blk in t.canonical_blocks()}
        for blk in np.ndindex(*t.nblocks()):
            if t.block_type(blk) == api.ZERO:
                continue
            q = ptr2canon[t.data_ptr(blk)]
            dims = t.block_dims(blk)
            perm = t.block_perm(blk)
            x = g.read_block(blk).reshape(dims, order="F")
            # element e of blk <-> element permute(e, perm) of q
            y = np.transpose(x, np.argsort(perm))    # shape of q's block
            out[q] += t.block_scalar(blk).real * y.ravel(order="F")
        return out

    ga = full_grad_tensor(wo.a)
    api.contract(alpha, wt, wo.b, 0.0, ga, "ijab", "cdab", "ijcd")
    ref_da = fold(wo.a, ga)
    gb = full_grad_tensor(wo.b)
    api.contract(alpha, wo.a, wt, 0.0, gb, "ijcd", "ijab", "cdab")
    ref_db = fold(wo.b, gb)
    assert W.rel_frobenius(gda, ref_da) <= 1e-11
    assert W.rel_frobenius(gdb, ref_db) <= 1e-11

    # (2) central differences on seeded canonical elements (L is linear in
    # every element, so a unit step is exact up to rounding)
    rng = np.random.default_rng(5)
    wo.alpha = alpha
    for t, grad in ((wo.a, ref_da), (wo.b, ref_db)):
        blocks = t.canonical_blocks()
        for _ in range(6):
            blk = blocks[rng.integers(len(blocks))]
            data = t.read_block(blk)
            e = int(rng.integers(data.size))
            vals = []
            for h in (1.0, -1.0):
                d2 = data.copy()
                d2[e] += h
                t.write_block(blk, d2)
                wo.run()
                vals.append(api.dot(wo.c, dco, "ijab", "ijab").real)
            t.write_block(blk, data)
            fd = (vals[0] - vals[1]) / 2.0
            g_eng = (gda if t is wo.a else gdb)[blk][e]
            assert abs(fd - g_eng) <= 1e-9 * max(1.0, abs(fd)), (fd, g_eng)
    for x in (da, db, ga, gb, wt, dce, dco):
        x.free()
    we.free()
    wo.free()


@pytest.mark.parametrize("dims,tiles", [((44, 92), (16, 8)), ((92, 188), (32, 16))])
def test_tile_autosplit_ladder(engine, oracle, dims, tiles):
    """A Z2^3 ladder on the opt-in tile-aware autosplit's blocks
    (xmg_block_space_autosplit_tiles, every block a multiple of the
    quantum but the last) against the oracle on the same splits, in both
    precision modes."""
    o_sz = W.split_sizes(engine, dims[0], tiles)
    v_sz = W.split_sizes(engine, dims[1], tiles)
    assert sum(o_sz) == dims[0] and sum(v_sz) == dims[1]
    assert all(x % tiles[1] == 0 for x in o_sz[:-1] + v_sz[:-1])
    eal, oal = api.Allocator(engine), api.Allocator(oracle)
    we = W.autosplit_ladder(engine, eal, o_sz, v_sz)
    wo = W.autosplit_ladder(oracle, oal, o_sz, v_sz)
    wo.run()
    ref = W.read_canonical(wo.c)
    try:
        for prec in (api.PREC_AUTO, api.PREC_FP64):
            engine.check(engine.xmg_set_precision(prec))
            we.run()
            assert W.rel_frobenius(W.read_canonical(we.c), ref) <= 1e-12, prec
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        we.free()
        wo.free()


def test_adjoint_kept_intermediates(engine):
    """Repeated adjoint calls reuse W, the gradient tensors and the plans of
    the two gradient contractions: a call after new dC data equals the same
    call computed from scratch (after xmg_adjoint_release)."""
    al = api.Allocator(engine)
    w = W.cfg2(engine, al, scale=4)
    dc = w.c.structure()
    da, db = w.a.structure(), w.b.structure()

    def grads():
        api.set_all(da, 0)
        api.set_all(db, 0)
        engine.check(engine.xm_contract_adjoint(api.Scalar.of(0.5), w.a.h, w.b.h, dc.h,
                                                da.h, db.h, b"ijcd", b"cdab", b"ijab"))
        return {**{("a",) + k: v for k, v in W.read_canonical(da).items()},
                **{("b",) + k: v for k, v in W.read_canonical(db).items()}}
    try:
        W.fill(dc, 77, W.LADDER_ANTISYM)
        g1 = grads()
        W.fill(dc, 78, W.LADDER_ANTISYM)          # same structure, new data
        g2 = grads()
        engine.xmg_adjoint_release()
        g3 = grads()
        assert W.rel_frobenius(g2, g3) <= 1e-13
        assert W.rel_frobenius(g1, g3) > 1e-3
    finally:
        engine.xmg_adjoint_release()
        for x in (dc, da, db):
            x.free()
        w.free()
        al.destroy()


def _adjoint(engine, w, dc, alpha):
    da, db = w.a.structure(), w.b.structure()
    api.set_all(da, 0)
    api.set_all(db, 0)
    engine.check(engine.xm_contract_adjoint(api.Scalar.of(alpha), w.a.h, w.b.h, dc.h, da.h,
                                            db.h, w.idxa.encode(), w.idxb.encode(),
                                            w.idxc.encode()))
    out = W.read_canonical(da), W.read_canonical(db)
    da.free()
    db.free()
    return out


def test_adjoint_forms_agree(engine, monkeypatch):
    """The ladder's gradients in the symmetric form (canonical positions
    times multiplicities; the structural checks pass) equal the
    every-position form forced with XMG_ADJOINT_EVERY=1, in both precision
    modes."""
    import test_adjoint_cpu as T
    al = api.Allocator(engine)
    w = W.cfg2(engine, al, scale=4)
    dc = w.c.structure()
    W.fill(dc, 79, W.LADDER_ANTISYM)
    assert T.plan_check(engine, w.a, w.b, dc, w.idxa, w.idxb, w.idxc)[0] == [T.SYM, T.SYM]
    try:
        for prec in (api.PREC_AUTO, api.PREC_FP64):
            engine.check(engine.xmg_set_precision(prec))
            engine.xmg_adjoint_release()
            sym = _adjoint(engine, w, dc, 1.5)
            monkeypatch.setenv("XMG_ADJOINT_EVERY", "1")
            engine.xmg_adjoint_release()
            every = _adjoint(engine, w, dc, 1.5)
            monkeypatch.delenv("XMG_ADJOINT_EVERY")
            for x, y in zip(sym, every):
                assert W.rel_frobenius(x, y) <= 1e-12, prec
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        engine.xmg_adjoint_release()
        dc.free()
        w.free()


@pytest.mark.parametrize("dtype", [api.DOUBLE, api.DOUBLE_COMPLEX])
def test_adjoint_mixed_forms_vs_oracle(engine, oracle, dtype):
    """a antisymmetric in the contracted pair (c,d) with b fully canonical:
    a's gradient falls back to the every-position form, b's takes the
    symmetric one.  Both against the oracle's exact gradients."""
    import test_adjoint_cpu as T
    res = {}
    for lib in (engine, oracle):
        al = api.Allocator(lib)
        o, v = [5, 7], [6, 9, 8]
        sa = W.make_space(lib, [o, o, v, v])
        sb = W.make_space(lib, [v, v, v, v])
        a = W.symmetric_tensor(lib, al, sa, dtype, [((0, 1, 2, 3), 1.0), ((0, 1, 3, 2), -1.0)])
        b = api.Tensor(lib, sb, dtype, al, canonical=True)
        c = api.Tensor(lib, sa, dtype, al, canonical=True)
        W.fill(a, 31, [((0, 1, 2, 3), 1.0), ((0, 1, 3, 2), -1.0)])
        W.fill(b, 32)
        dc = c.structure()
        W.fill(dc, 33)
        res[lib.path] = (W.Workload("mixed", a, b, c, ("ijcd", "cdab", "ijab"), 1.0, 0.0,
                                    None, None), dc, al)
        sa.free()
        sb.free()
    (we, dce, _), (wo, dco, oal) = res[engine.path], res[oracle.path]
    assert T.plan_check(engine, we.a, we.b, dce, we.idxa, we.idxb, we.idxc)[0] == \
        [T.EVERY, T.SYM]
    try:
        gda, gdb = _adjoint(engine, we, dce, -0.5)
        ea, eb = T.exact_gradients(oracle, oal, wo, dco, -0.5)
        assert W.rel_frobenius(gda, ea) <= 1e-12
        assert W.rel_frobenius(gdb, eb) <= 1e-12
    finally:
        engine.xmg_adjoint_release()
        for w, dc, al in res.values():
            dc.free()
            w.free()
            al.destroy()
