"""torch.autograd binding of xm_contract for the test harness (not part of
the library): forward runs the engine's xm_contract, backward its
hand-written adjoint xm_contract_adjoint.

Values cross the boundary as flat float64 CPU tensors holding every
canonical block of a tensor in canonical-list order (each block in its own
index-0-fastest layout).  The gradient flowing into backward is
dL/d(canonical c values); the adjoint's dc pairs with c over every block
(the xm_dot pairing), where a canonical block with k nonzero images counts
k times, so backward hands it g / k on c's structure.
"""
import numpy as np
import torch

from libxm_gb300 import api


def flat(t):
    return torch.from_numpy(np.concatenate([t.read_block(b).ravel() for b in t.canonical_blocks()]))


def scatter(t, v):
    v = v.detach().cpu().numpy()
    o = 0
    for b in t.canonical_blocks():
        n = t.block_size(b)
        t.write_block(b, v[o:o + n])
        o += n


def multiplicity(t):
    """Per canonical block: the number of nonzero blocks sharing its data,
    weighted by their squared scalars (the xm_dot pairing of t with a
    tensor of the same structure)."""
    m = {}
    for blk in np.ndindex(*t.nblocks()):
        if t.block_type(blk) != api.ZERO:
            p = t.data_ptr(blk)
            m[p] = m.get(p, 0.0) + abs(t.block_scalar(blk)) ** 2
    return m


class Contract(torch.autograd.Function):
    """c = alpha * contract(a, b) (beta = 0) over the workload's tensors."""

    @staticmethod
    def forward(ctx, a_vals, b_vals, w, alpha):
        scatter(w.a, a_vals)
        scatter(w.b, b_vals)
        api.contract(alpha, w.a, w.b, 0.0, w.c, w.idxa, w.idxb, w.idxc)
        ctx.w, ctx.alpha = w, alpha
        return flat(w.c)

    @staticmethod
    def backward(ctx, g):
        w, alpha = ctx.w, ctx.alpha
        lib = w.c.lib
        dc = w.c.structure()
        mult = multiplicity(w.c)
        g = g.detach().cpu().numpy()
        o = 0
        for blk in w.c.canonical_blocks():
            n = w.c.block_size(blk)
            dc.write_block(blk, g[o:o + n] / mult[w.c.data_ptr(blk)])
            o += n
        da, db = w.a.structure(), w.b.structure()
        api.set_all(da, 0)
        api.set_all(db, 0)
        lib.check(lib.xm_contract_adjoint(api.Scalar.of(alpha), w.a.h, w.b.h, dc.h, da.h, db.h,
                                          w.idxa.encode(), w.idxb.encode(), w.idxc.encode()))
        ga, gb = flat(da), flat(db)
        for x in (dc, da, db):
            x.free()
        return ga, gb, None, None
