"""Seeded random contractions through the host planner: random index
strings (contracted, a-only and b-only letters in random orders), random
block splits (shared by every tensor that carries a letter), zero blocks,
and (anti)symmetric dimensions stored as derivative blocks with a +-1
scalar: a transposition of two dimensions, or the exchange of two pairs of
dimensions at once.  The engine's merged pair list
(output block, merged factor, m, n, k) and its flop count must equal the
oracle's bit for bit (contract.c:161-218 of the reference), and the
split-precision GEMM's work lists and the out-of-core batch plans built
from it hold their invariants.  No device is involved: the engine plans on
a pagefile allocator.  The scalar type cycles over the four kinds."""
import itertools
import os
import tempfile

import numpy as np
import pytest

import helpers as H
from libxm_gb300 import api

LETTERS = "abcdefgh"


@pytest.fixture(scope="module")
def pagefile(engine):
    d = tempfile.mkdtemp()
    al = api.Allocator(engine, os.path.join(d, "xmpagefile"))
    yield al
    al.destroy()
    os.rmdir(d)


def _case(rng):
    nk = int(rng.integers(1, 4))
    na, nb = int(rng.integers(0, 3)), int(rng.integers(0, 3))
    if na + nb == 0:
        na = 1
    ks = list(LETTERS[:nk])
    fa = list(LETTERS[nk:nk + na])
    fb = list(LETTERS[nk + na:nk + na + nb])
    defs = {}
    for x in ks + fa + fb:
        if defs and rng.random() < 0.5:        # a twin of an earlier letter
            defs[x] = defs[list(defs)[int(rng.integers(0, len(defs)))]]
        else:
            n = int(rng.integers(2, 11))
            cuts = sorted(set(int(c) for c in rng.integers(1, n, size=int(rng.integers(0, 3)))))
            defs[x] = (n, tuple(cuts))
    perm = lambda s: "".join(s[i] for i in rng.permutation(len(s)))
    idxa, idxb, idxc = perm(ks + fa), perm(ks + fb), perm(fa + fb)
    return defs, idxa, idxb, idxc, set(ks)


def _layout(rng, defs, idx, contracted):
    """Block kinds of one tensor: {blk: ("c",) | ("z",) | ("d", src, perm, s)}.
    A symmetry over two contracted letters is preferred: when both operands
    carry it, symmetry-equivalent pairs merge."""
    nblk = [len(defs[x][1]) + 1 for x in idx]
    twins = [(p, q) for p, q in itertools.combinations(range(len(idx)), 2)
             if defs[idx[p]] == defs[idx[q]]]
    inner = [t for t in twins if idx[t[0]] in contracted and idx[t[1]] in contracted]
    if inner and rng.random() < 0.8:
        twins = inner
    # the symmetry: one transposition of twin positions, or an exchange of
    # two twin pairs at once ((p1 q1) <-> (p2 q2), like (ia|jb) = (jb|ia))
    swaps = None
    pairs2 = [(s1, s2) for s1, s2 in itertools.combinations(twins, 2)
              if len({*s1, *s2}) == 4]
    if pairs2 and rng.random() < 0.4:
        (p1, p2), (q1, q2) = pairs2[int(rng.integers(0, len(pairs2)))]
        swaps = [(p1, p2), (q1, q2)]
        key = lambda b: ((b[p1], b[q1]), (b[p2], b[q2]))
    elif twins and rng.random() < 0.8:
        swaps = [twins[int(rng.integers(0, len(twins)))]]
        key = lambda b: ((b[swaps[0][0]],), (b[swaps[0][1]],))
    sign = -1.0 if rng.random() < 0.6 else 1.0
    kinds = {}
    for blk in itertools.product(*[range(b) for b in nblk]):
        if swaps and key(blk)[0] > key(blk)[1]:
            src, p = list(blk), list(range(len(idx)))
            for u, v in swaps:
                src[u], src[v] = src[v], src[u]
                p[u], p[v] = p[v], p[u]
            kinds[blk] = ("d", tuple(src), p, sign)
        else:
            kinds[blk] = ("z",) if rng.random() < 0.2 else ("c",)
    for blk, k in kinds.items():       # a derivative of a zero block is zero
        if k[0] == "d" and kinds[k[1]][0] == "z":
            kinds[blk] = ("z",)
    return kinds


def _build(lib, alloc, defs, idx, kinds, dtype):
    bs = api.BlockSpace(lib, [defs[x][0] for x in idx])
    for d, x in enumerate(idx):
        for c in defs[x][1]:
            bs.split(d, c)
    t = api.Tensor(lib, bs, dtype, alloc)
    bs.free()
    for blk, k in kinds.items():
        if k[0] == "c":
            t.set_canonical(blk)
    for blk, k in kinds.items():
        if k[0] == "d":
            t.set_derivative(blk, k[1], k[2], k[3])
    return t


@pytest.mark.parametrize("seed", range(200))
def test_random_contractions_plan_like_the_oracle(engine, oracle, pagefile, seed):
    rng = np.random.default_rng(1000 + seed)
    defs, idxa, idxb, idxc, ks = _case(rng)
    kinds = [_layout(rng, defs, s, ks) for s in (idxa, idxb, idxc)]
    dt = (api.DOUBLE, api.DOUBLE_COMPLEX, api.FLOAT, api.FLOAT_COMPLEX)[seed % 4]
    oal = api.Allocator(oracle)
    et = [_build(engine, pagefile, defs, s, k, dt) for s, k in zip((idxa, idxb, idxc), kinds)]
    ot = [_build(oracle, oal, defs, s, k, dt) for s, k in zip((idxa, idxb, idxc), kinds)]
    try:
        for t in ot:
            H.fill_random(t, rng)
        mine = H.pair_structure_engine(engine, *et, idxa, idxb, idxc)
        ref = H.pair_structure_oracle(oracle, *ot, idxa, idxb, idxc)
        assert mine == ref, (idxa, idxb, idxc, defs)
        flops = engine.xmg_contract_flops(et[0].h, et[1].h, et[2].h, idxa.encode(),
                                          idxb.encode(), idxc.encode())
        mult = 8 if dt in (api.FLOAT_COMPLEX, api.DOUBLE_COMPLEX) else 2
        assert flops == sum(mult * m * n * k for _, _, m, n, k in ref)
        # the split-precision work lists and the out-of-core batch cut
        args = (et[0].h, et[1].h, et[2].h, idxa.encode(), idxb.encode(), idxc.encode())
        out = (api.C.c_longlong * 4)()
        for pol in (0, 1, 2, 6):
            engine.check(engine.xmg_work_list_check(*args, pol, out))
            assert out[3] == 1, pol
        for nbatch in (1, 3):
            engine.check(engine.xmg_batch_plan_check(*args, nbatch, 0, 6, out))
            assert out[3] == 1 and out[1] == len(mine), nbatch
    finally:
        for t in et + ot:
            t.free()
