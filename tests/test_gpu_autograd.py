"""GPU: the adjoint through a torch.autograd binding (test harness only).

Ladder with the cfg2 structure at 1/4 block size, loss
L = sum over every block of W o C (the xm_dot pairing, W antisymmetric like
C) written in torch on the canonical values.  The autograd gradients must
equal (1) the adjoint called directly with dC = W, (2) central finite
differences with h = 1e-6 on 200 seeded canonical elements (100 of A, 100
of B).  L is linear in every element, so the difference quotient is exact
up to the rounding of L: with |L| ~ 1e3 and FP64 forwards that rounding is
~1e-13 / 2e-6, so the comparison is held to 1e-6 relative to the largest
gradient component."""
import numpy as np
import pytest

from libxm_gb300 import api, workloads as W

torch = pytest.importorskip("torch")
import xm_autograd as XA  # noqa: E402

pytestmark = pytest.mark.gpu


def test_autograd_adjoint_and_finite_differences(engine):
    al = api.Allocator(engine)
    w = W.cfg2(engine, al, scale=4)
    alpha = 0.75
    wt = w.c.structure()
    W.fill(wt, 77, W.LADDER_ANTISYM)
    mult = XA.multiplicity(w.c)
    wm = torch.from_numpy(np.concatenate([wt.read_block(b).ravel() * mult[w.c.data_ptr(b)]
                                          for b in w.c.canonical_blocks()]))
    try:
        a0, b0 = XA.flat(w.a), XA.flat(w.b)
        a = a0.clone().requires_grad_(True)
        b = b0.clone().requires_grad_(True)
        engine.check(engine.xmg_set_precision(api.PREC_FP64))
        c = XA.Contract.apply(a, b, w, alpha)
        loss = (c * wm).sum()
        loss.backward()
        # the pairing through the engine equals the torch loss
        lv = loss.item()
        assert abs(api.dot(w.c, wt, w.idxc, w.idxc).real - lv) <= 1e-10 * abs(lv)

        # (1) the adjoint called directly with dC = W
        da, db = w.a.structure(), w.b.structure()
        api.set_all(da, 0)
        api.set_all(db, 0)
        engine.check(engine.xm_contract_adjoint(api.Scalar.of(alpha), w.a.h, w.b.h, wt.h, da.h, db.h,
                                                b"ijcd", b"cdab", b"ijab"))
        for got, ref in ((a.grad, XA.flat(da)), (b.grad, XA.flat(db))):
            assert float((got - ref).norm() / ref.norm()) <= 1e-13
        da.free()
        db.free()

        # (2) central differences, h = 1e-6, FP64 forwards
        rng = np.random.default_rng(11)
        h = 1e-6
        for vals, grad, which in ((a0, a.grad, 0), (b0, b.grad, 1)):
            gmax = float(grad.abs().max())
            for e in rng.choice(vals.numel(), 100, replace=False):
                lv = []
                for s in (h, -h):
                    x = vals.clone()
                    x[e] += s
                    args = (x, b0) if which == 0 else (a0, x)
                    with torch.no_grad():
                        lv.append(float((XA.Contract.apply(*args, w, alpha) * wm).sum()))
                fd = (lv[0] - lv[1]) / (2 * h)
                assert abs(fd - float(grad[e])) <= 1e-6 * gmax, (which, e, fd, float(grad[e]))
    finally:
        engine.check(engine.xmg_set_precision(api.PREC_AUTO))
        wt.free()
        w.free()
