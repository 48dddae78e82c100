"""CPU: the adjoint's structural checks and the algebra of its symmetric form.

xm_contract_adjoint computes a gradient at the canonical positions only,
times a per-block factor, when the block tables of a, b and dc carry the
contraction over (xmg_adjoint_plan_check runs those checks without a
device); otherwise at every nonzero position, folded back.  Checked here:

* which form each gradient takes for consistent structures (the
  antisymmetric ladder; operands antisymmetric in the contracted pair) and
  for inconsistent ones (an output declared symmetric where the
  contraction is antisymmetric; the ring term, whose declared output
  symmetry the independent operands do not produce; an operand symmetry
  the other operand lacks);
* the ladder's factors: the number of nonzero positions that share a
  canonical block's data;
* with the oracle doing the contractions: factor x gradient at the
  canonical positions equals the every-position gradient folded back
  (the exact form), for the ladder and the contracted-pair structure, in
  real and complex types.
"""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

import helpers as H
from libxm_gb300 import api, workloads as W

EVERY, SYM = 2, 1


@pytest.fixture()
def pagefile_alloc(engine):
    d = tempfile.mkdtemp(prefix="xmg_adj_")
    al = api.Allocator(engine, os.path.join(d, "pf"))
    yield al
    al.destroy()


def plan_check(lib, a, b, dc, ia, ib, ic):
    mode = (C.c_int * 2)()
    na = int(np.prod(a.nblocks()))
    nb = int(np.prod(b.nblocks()))
    fa = (C.c_double * (2 * na))()
    fb = (C.c_double * (2 * nb))()
    lib.check(lib.xmg_adjoint_plan_check(a.h, b.h, dc.h, ia.encode(), ib.encode(),
                                         ic.encode(), mode, fa, fb))
    fa = np.frombuffer(fa, dtype=np.complex128).copy()
    fb = np.frombuffer(fb, dtype=np.complex128).copy()
    return list(mode), fa, fb


def linear(t, blk):
    return int(np.ravel_multi_index(blk, t.nblocks(), order="F"))


def ladder(lib, al, dtype=api.DOUBLE, scale=4):
    w = W.cfg2(lib, al, scale=scale)
    if dtype != api.DOUBLE:
        w2 = W.ladder(lib, al, w.extra["o_sizes"], w.extra["v_sizes"], seed=2, dtype=dtype,
                      z2=(w.extra["o_labels"], w.extra["v_labels"]))
        w.free()
        w = w2
    return w


def test_ladder_takes_the_symmetric_form(engine, pagefile_alloc):
    w = ladder(engine, pagefile_alloc)
    dc = w.c.structure()
    mode, fa, fb = plan_check(engine, w.a, w.b, dc, w.idxa, w.idxb, w.idxc)
    assert mode == [SYM, SYM]
    for t, f in ((w.a, fa), (w.b, fb)):
        count = {}
        for blk in np.ndindex(*t.nblocks()):
            if t.block_type(blk) != api.ZERO:
                count[t.data_ptr(blk)] = count.get(t.data_ptr(blk), 0) + 1
        for blk in np.ndindex(*t.nblocks()):
            want = count[t.data_ptr(blk)] if t.block_type(blk) == api.CANONICAL else 0
            assert f[linear(t, blk)] == want, (blk, f[linear(t, blk)], want)
    dc.free()
    w.free()


def test_ring_term_keeps_every_position(engine, pagefile_alloc):
    """The ring term's output is declared pair-symmetric, (i,a) <-> (j,b),
    but with independent a and b the contraction at a derivative position
    of c is not the permuted contraction at its source: the loss pairs dc
    with c's declared blocks, so only the every-position form (dc folded
    onto c's canonical blocks) is exact."""
    w = W.cfg3(engine, pagefile_alloc, dtype=api.DOUBLE, o_blk=3, v_blk=4, no=2, nv=3)
    dc = w.c.structure()
    mode, fa, fb = plan_check(engine, w.a, w.b, dc, w.idxa, w.idxb, w.idxc)
    assert mode == [EVERY, EVERY]
    dc.free()
    w.free()


def contracted_pair(lib, al, dtype):
    """a(i,j,c,d), b(c,d,a,b) both antisymmetric in (c,d) only; c fully
    canonical: consistent, factor 2 off the c = d diagonal."""
    o, v = [3, 2], [2, 3, 2]
    sa = W.make_space(lib, [o, o, v, v])
    sb = W.make_space(lib, [v, v, v, v])
    ga = [((0, 1, 2, 3), 1.0), ((0, 1, 3, 2), -1.0)]
    gb = [((0, 1, 2, 3), 1.0), ((1, 0, 2, 3), -1.0)]
    a = W.symmetric_tensor(lib, al, sa, dtype, ga)
    b = W.symmetric_tensor(lib, al, sb, dtype, gb)
    c = api.Tensor(lib, sa, dtype, al, canonical=True)
    sa.free()
    sb.free()
    W.fill(a, 11, ga)
    W.fill(b, 12, gb)
    return W.Workload("contracted_pair", a, b, c, ("ijcd", "cdab", "ijab"), 1.0, 0.0,
                      (ga, gb, W.NO_SYM), (11, 12, 13))


def test_inconsistent_output_symmetry_falls_back(engine, pagefile_alloc):
    """dc declared symmetric (+1) in (i,j) while a is antisymmetric: the
    contraction does not follow dc's derivative blocks, so neither
    gradient may use the symmetric form."""
    o, v = [3, 2], [2, 3]
    sa = W.make_space(engine, [o, o, v, v])
    sb = W.make_space(engine, [v, v, v, v])
    bad = [((0, 1, 2, 3), 1.0), ((1, 0, 2, 3), 1.0), ((0, 1, 3, 2), -1.0),
           ((1, 0, 3, 2), -1.0)]
    a = W.symmetric_tensor(engine, pagefile_alloc, sa, api.DOUBLE, W.LADDER_ANTISYM)
    b = W.symmetric_tensor(engine, pagefile_alloc, sb, api.DOUBLE, W.LADDER_ANTISYM)
    dc = W.symmetric_tensor(engine, pagefile_alloc, sa, api.DOUBLE, bad)
    mode, fa, fb = plan_check(engine, a, b, dc, "ijcd", "cdab", "ijab")
    assert mode == [EVERY, EVERY]
    assert not fa.any() and not fb.any()
    # the same tensors with dc antisymmetric like the forward: symmetric
    dc2 = W.symmetric_tensor(engine, pagefile_alloc, sa, api.DOUBLE, W.LADDER_ANTISYM)
    assert plan_check(engine, a, b, dc2, "ijcd", "cdab", "ijab")[0] == [SYM, SYM]
    for t in (a, b, dc, dc2):
        t.free()
    sa.free()
    sb.free()


def test_operand_symmetry_without_partner_falls_back(engine, pagefile_alloc):
    """a antisymmetric in (c,d) while b is fully canonical: a's gradient
    is not equivariant under the (c,d) swap (b has no matching blocks),
    b's gradient has no derivative blocks to fold."""
    o, v = [3, 2], [2, 3]
    sa = W.make_space(engine, [o, o, v, v])
    sb = W.make_space(engine, [v, v, v, v])
    sc = W.make_space(engine, [o, o, v, v])
    a = W.symmetric_tensor(engine, pagefile_alloc, sa, api.DOUBLE,
                           [((0, 1, 2, 3), 1.0), ((0, 1, 3, 2), -1.0)])
    b = api.Tensor(engine, sb, api.DOUBLE, pagefile_alloc, canonical=True)
    c = api.Tensor(engine, sc, api.DOUBLE, pagefile_alloc, canonical=True)
    mode, fa, fb = plan_check(engine, a, b, c, "ijcd", "cdab", "ijab")
    assert mode == [EVERY, SYM]
    assert np.all(fb == 1)
    for t in (a, b, c):
        t.free()
    for s in (sa, sb, sc):
        s.free()


def exact_gradients(oracle, al, w, dc, alpha):
    """The oracle's gradients of L = <dc, alpha a b> with respect to the
    canonical blocks of a and b: at every nonzero position, folded back."""
    wt = H.folded_cotangent(oracle, al, dc)
    ga = H.sampled_gradient(oracle, al, w.a, wt, w.b, w.idxc, w.idxb, w.idxa, alpha,
                            w.a.canonical_blocks(), True)
    gb = H.sampled_gradient(oracle, al, w.b, wt, w.a, w.idxc, w.idxa, w.idxb, alpha,
                            w.b.canonical_blocks(), False)
    wt.free()
    return ga, gb


def _exact_and_symmetric(oracle, al, w, dc, alpha, factors):
    """The gradients of L = <dc, alpha a b> on the oracle, exact (every
    position, folded back) and in the symmetric form (canonical positions
    times the factors)."""
    out = []
    for k, (t, f, exact) in enumerate(zip((w.a, w.b), factors,
                                          exact_gradients(oracle, al, w, dc, alpha))):
        blocks = t.canonical_blocks()
        g = api.Tensor(oracle, None, t.dtype, al,
                       handle=oracle.xm_tensor_create(oracle.xm_tensor_get_block_space(t.h),
                                                      t.dtype, al.h))
        for blk in blocks:
            g.set_canonical(blk)
        if k == 0:
            api.contract(alpha, dc, w.b, 0.0, g, w.idxc, w.idxb, w.idxa)
        else:
            api.contract(alpha, w.a, dc, 0.0, g, w.idxa, w.idxc, w.idxb)
        sym = {blk: f[linear(t, blk)] * g.read_block(blk) for blk in blocks}
        g.free()
        out.append((exact, sym))
    return out


@pytest.mark.parametrize("dtype", [api.DOUBLE, api.DOUBLE_COMPLEX])
def test_symmetric_form_equals_exact_ladder(engine, oracle, pagefile_alloc, dtype):
    oal = api.Allocator(oracle)
    we = ladder(engine, pagefile_alloc, dtype)
    dce = we.c.structure()
    mode, fa, fb = plan_check(engine, we.a, we.b, dce, we.idxa, we.idxb, we.idxc)
    assert mode == [SYM, SYM]
    wo = ladder(oracle, oal, dtype)
    dc = wo.c.structure()
    W.fill(dc, 77, W.LADDER_ANTISYM)
    for exact, sym in _exact_and_symmetric(oracle, oal, wo, dc, 0.75, (fa, fb)):
        assert H.max_abs_diff(exact, sym) <= 1e-9 * max(1.0, max(
            float(np.max(np.abs(x))) for x in exact.values()))
    dce.free()
    we.free()
    dc.free()
    wo.free()
    oal.destroy()


@pytest.mark.parametrize("dtype", [api.DOUBLE, api.FLOAT_COMPLEX])
def test_symmetric_form_equals_exact_contracted_pair(engine, oracle, pagefile_alloc, dtype):
    oal = api.Allocator(oracle)
    we = contracted_pair(engine, pagefile_alloc, dtype)
    mode, fa, fb = plan_check(engine, we.a, we.b, we.c, we.idxa, we.idxb, we.idxc)
    assert mode == [SYM, SYM]
    assert set(np.unique(fa.real)) <= {0, 1, 2} and 2 in fa.real
    wo = contracted_pair(oracle, oal, dtype)
    dc = wo.c.structure()
    W.fill(dc, 78)
    tol = 1e-4 if dtype == api.FLOAT_COMPLEX else 1e-10
    for exact, sym in _exact_and_symmetric(oracle, oal, wo, dc, -1.25, (fa, fb)):
        assert H.max_abs_diff(exact, sym) <= tol
    dc.free()
    we.free()
    wo.free()
    oal.destroy()
