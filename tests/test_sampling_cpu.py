"""The oracle-side helpers of the full-size parity tests, checked on the CPU.

W.contract_sample (the oracle computing a sample of the output blocks) must
give exactly the blocks of the whole contraction, and H.sampled_gradient
(the oracle's gradient on sampled canonical blocks) must agree with central
differences of L = <dC, alpha A B>, which are exact for a bilinear L.
"""
import numpy as np

import helpers as H
from libxm_gb300 import api, workloads as W


def test_contract_sample_equals_whole_contraction(oracle):
    al = api.Allocator(oracle)
    w = W.cfg2(oracle, al, scale=4)
    w.run()
    full = W.read_canonical(w.c)
    chosen = W.sample_blocks(w.c.canonical_blocks(), 12, seed=3)
    part = W.contract_sample(w, chosen)
    assert sorted(part) == sorted(chosen)
    for blk in chosen:
        assert np.array_equal(part[blk], full[blk]), blk
    w.free()
    # beta = 1 with a prefilled, pair-symmetric output
    w = W.cfg3(oracle, al, dtype=api.DOUBLE, o_blk=6, v_blk=10)
    c0 = W.read_canonical(w.c)
    chosen = W.sample_blocks(w.c.canonical_blocks(), 9, seed=4)
    part = W.contract_sample(w, chosen, {k: c0[k] for k in chosen})
    w.run()
    for blk in chosen:
        assert np.array_equal(part[blk], w.c.read_block(blk)), blk
    w.free()
    al.destroy()


def test_sample_blocks_is_seeded_and_ordered():
    blocks = [(i, j) for i in range(5) for j in range(7)]
    s1 = W.sample_blocks(blocks, 10, seed=8)
    assert s1 == W.sample_blocks(blocks, 10, seed=8)
    assert len(set(s1)) == 10 and s1 == sorted(s1, key=blocks.index)
    assert W.sample_blocks(blocks, 100) == blocks


def test_sampled_gradient_central_differences(oracle):
    alpha = 0.75
    al = api.Allocator(oracle)
    w = W.cfg2(oracle, al, scale=4)
    w.alpha = alpha
    dc = w.c.structure()
    W.fill(dc, 77, W.LADDER_ANTISYM)
    wt = H.folded_cotangent(oracle, al, dc)
    rng = np.random.default_rng(12)
    for t, args in ((w.a, (w.b, "ijab", "cdab", "ijcd", True)),
                    (w.b, (w.a, "ijab", "ijcd", "cdab", False))):
        other, iw, io, it, w_first = args
        sample = W.sample_blocks(t.canonical_blocks(), 3, seed=13)
        grad = H.sampled_gradient(oracle, al, t, wt, other, iw, io, it, alpha, sample, w_first)
        for blk in sample:
            data = t.read_block(blk)
            for e in rng.integers(data.size, size=2):
                vals = []
                for h in (1.0, -1.0):
                    d2 = data.copy()
                    d2[e] += h
                    t.write_block(blk, d2)
                    w.run()
                    vals.append(api.dot(w.c, dc, "ijab", "ijab").real)
                t.write_block(blk, data)
                fd = (vals[0] - vals[1]) / 2.0
                assert abs(fd - grad[blk][e]) <= 1e-9 * max(1.0, abs(fd)), (blk, e, fd, grad[blk][e])
    for x in (wt, dc):
        x.free()
    w.free()
    al.destroy()


def test_threaded_fill_gives_the_same_values(oracle):
    al = api.Allocator(oracle)
    w1 = W.cfg2(oracle, al, scale=4)
    w2 = W.cfg2(oracle, al, scale=4, fill_data=False)
    W.fill(w2.a, 7, W.LADDER_ANTISYM, threads=4)
    W.fill(w1.a, 7, W.LADDER_ANTISYM)
    for blk in w1.a.canonical_blocks():
        assert np.array_equal(w1.a.read_block(blk), w2.a.read_block(blk))
    w1.free()
    w2.free()
    al.destroy()
