"""Block structures of the reference test driver (test.c:415-1190),
restated for the Python binding so that the same cases run against the
oracle, the reference built from source and the GB300 engine.

Each make_* takes (lib, alloc, dtype) and returns tensors; the case tables
mirror test.c:1875-1959.
"""
from libxm_gb300 import api


def _space(lib, dims, splits):
    bs = api.BlockSpace(lib, dims)
    for d, x in splits:
        bs.split(d, x)
    return bs


def make_ab_1(lib, al, t):      # test.c:415-433
    bs = _space(lib, [1, 2, 3, 4, 5, 6, 7, 8], [(1, 1), (3, 2), (5, 3), (7, 2), (7, 5)])
    a = api.Tensor(lib, bs, t, al, canonical=True)
    b = api.Tensor(lib, bs, t, al, canonical=True)
    bs.free()
    return a, b


def make_ab_2(lib, al, t):      # test.c:435-452
    bs = _space(lib, [4, 4, 4, 4], [(0, 2), (1, 2), (2, 2), (3, 2)])
    a = api.Tensor(lib, bs, t, al, canonical=True)
    b = api.Tensor(lib, bs, t, al, canonical=True)
    bs.free()
    return a, b


def make_ab_3(lib, al, t):      # test.c:454-473
    bs = _space(lib, [8, 8], [(0, 4), (1, 4)])
    a = api.Tensor(lib, bs, t, al, canonical=True)
    b = api.Tensor(lib, bs, t, al)
    b.set_canonical((0, 0))
    b.set_canonical((1, 1))
    b.set_derivative((0, 1), (0, 0), (1, 0), -4)
    bs.free()
    return a, b


def make_ab_4(lib, al, t):      # test.c:475-495
    bs = _space(lib, [20, 20], [(0, 10), (1, 10)])
    a = api.Tensor(lib, bs, t, al)
    a.set_canonical((0, 0))
    a.set_canonical((1, 1))
    b = api.Tensor(lib, bs, t, al)
    b.set_canonical((0, 0))
    b.set_derivative((1, 1), (0, 0), (1, 0), -10)
    bs.free()
    return a, b


def make_ab_5(lib, al, t):      # test.c:497-518
    bs = _space(lib, [17, 31], [(0, 11), (1, 15)])
    a = api.Tensor(lib, bs, t, al)
    a.set_canonical((0, 0))
    a.set_canonical((1, 1))
    b = api.Tensor(lib, bs, t, al)
    for blk in [(0, 0), (1, 1), (0, 1), (1, 0)]:
        b.set_canonical(blk)
    bs.free()
    return a, b


def make_abc_1(lib, al, t):     # test.c:520-541
    bs = api.BlockSpace(lib, [4, 4])
    a, b, c = (api.Tensor(lib, bs, t, al) for _ in range(3))
    bs.free()
    for x in (a, b, c):
        x.set_canonical((0, 0))
    return a, b, c


def make_abc_2(lib, al, t):     # test.c:543-573
    bs = _space(lib, [4, 4], [(0, 2), (1, 2)])
    a, b, c = (api.Tensor(lib, bs, t, al, canonical=True) for _ in range(3))
    bs.free()
    return a, b, c


def make_abc_3(lib, al, t):     # test.c:575-592
    bsa = api.BlockSpace(lib, [1] * 8)
    a = api.Tensor(lib, bsa, t, al, canonical=True)
    b = api.Tensor(lib, bsa, t, al, canonical=True)
    bsc = api.BlockSpace(lib, [1, 1])
    c = api.Tensor(lib, bsc, t, al, canonical=True)
    bsa.free(); bsc.free()
    return a, b, c


def make_abc_4(lib, al, t):     # test.c:594-609
    bs = api.BlockSpace(lib, [3] * 6)
    a, b, c = (api.Tensor(lib, bs, t, al, canonical=True) for _ in range(3))
    bs.free()
    return a, b, c


def make_abc_5(lib, al, t):     # test.c:611-641
    bs = _space(lib, [4, 4], [(0, 2), (1, 2)])
    a, b, c = (api.Tensor(lib, bs, t, al) for _ in range(3))
    bs.free()
    for x in (a, b, c):
        x.set_canonical((0, 0))
    c.set_canonical((0, 1))
    c.set_canonical((1, 0))
    for x in (a, b, c):
        x.set_canonical((1, 1))
    return a, b, c


def make_abc_6(lib, al, t):     # test.c:643-676
    bsa = _space(lib, [3], [(0, 1)])
    bsb = _space(lib, [2, 5], [(1, 3)])
    bsc = _space(lib, [2, 3, 5], [(1, 1), (2, 3)])
    a = api.Tensor(lib, bsa, t, al)
    b = api.Tensor(lib, bsb, t, al)
    c = api.Tensor(lib, bsc, t, al)
    bsa.free(); bsb.free(); bsc.free()
    a.set_canonical((0,)); a.set_canonical((1,))
    b.set_canonical((0, 0)); b.set_canonical((0, 1))
    for blk in [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1)]:
        c.set_canonical(blk)
    return a, b, c


def make_abc_7(lib, al, t):     # test.c:678-737
    import numpy as np
    bsa = _space(lib, [7, 4, 11], [(0, 2), (0, 5), (1, 2), (2, 2), (2, 9)])
    a = api.Tensor(lib, bsa, t, al)
    bsa.free()
    a.set_canonical((0, 0, 0))
    a.set_canonical((1, 0, 0))
    a.set_derivative((2, 0, 0), (0, 0, 0), (2, 1, 0), -0.5)
    a.set_derivative((0, 1, 0), (0, 0, 0), (1, 0, 2), 1.5)
    a.set_canonical((1, 1, 0))
    a.set_derivative((2, 1, 0), (0, 0, 0), (2, 0, 1), 0.7)
    for blk in np.ndindex(*a.nblocks()):
        if a.block_type(blk) == api.ZERO:
            a.set_canonical(blk)
    bsb = _space(lib, [7, 4, 8], [(0, 2), (0, 5), (1, 2), (2, 2), (2, 6)])
    b = api.Tensor(lib, bsb, t, al, canonical=True)
    bsc = _space(lib, [8, 11], [(0, 2), (0, 6), (1, 2), (1, 9)])
    c = api.Tensor(lib, bsc, t, al, canonical=True)
    bsb.free(); bsc.free()
    return a, b, c


def make_abc_8(lib, al, t):     # test.c:739-776
    bsa = _space(lib, [15, 10], [(0, 5), (0, 10), (1, 5)])
    a = api.Tensor(lib, bsa, t, al)
    a.set_canonical((0, 0))
    a.set_derivative((0, 1), (0, 0), (1, 0), -0.3)
    a.set_canonical((2, 0))
    a.set_canonical((2, 1))
    bsb = _space(lib, [10], [(0, 5)])
    b = api.Tensor(lib, bsb, t, al)
    b.set_canonical((0,)); b.set_canonical((1,))
    bsc = _space(lib, [15], [(0, 5), (0, 10)])
    c = api.Tensor(lib, bsc, t, al)
    c.set_canonical((0,)); c.set_canonical((2,))
    bsa.free(); bsb.free(); bsc.free()
    return a, b, c


ANTI4 = [((1, 0, 2, 3), -1), ((0, 1, 3, 2), -1), ((1, 0, 3, 2), 1)]
PAIR8 = ANTI4 + [((2, 3, 0, 1), 1), ((3, 2, 0, 1), -1), ((2, 3, 1, 0), -1),
                 ((3, 2, 1, 0), 1)]


def _fill_sym(ts, nblk, group):
    """Set canonical + derivative blocks over nested loops with the last
    index fastest (test.c:838-895 pattern) on every tensor in ts."""
    import itertools
    for blk in itertools.product(*[range(n) for n in nblk]):
        if ts[0].block_type(blk) != api.ZERO:
            continue
        for x in ts:
            x.set_canonical(blk)
        for perm, s in group:
            b2 = tuple(blk[perm[k]] for k in range(4))
            if ts[0].block_type(b2) == api.ZERO:
                for x in ts:
                    x.set_derivative(b2, blk, perm, s)


def make_abc_9(lib, al, t):     # test.c:778-896
    bsa = _space(lib, [6, 6, 10, 10], [(0, 2), (1, 2), (0, 5), (1, 5),
                                        (2, 3), (3, 3), (2, 4), (3, 4), (2, 8), (3, 8)])
    bsb = _space(lib, [10] * 4, [(d, x) for x in (3, 4, 8) for d in range(4)])
    a = api.Tensor(lib, bsa, t, al)
    b = api.Tensor(lib, bsb, t, al)
    c = api.Tensor(lib, bsa, t, al)
    bsa.free(); bsb.free()
    _fill_sym([a, c], [3, 3, 4, 4], ANTI4)
    _fill_sym([b], [4, 4, 4, 4], PAIR8)
    return a, b, c


def make_abc_10(lib, al, t):    # test.c:898-1000
    bsa = _space(lib, [6, 6, 9, 9], [(0, 4), (1, 4), (2, 3), (3, 3), (2, 7), (3, 7)])
    a = api.Tensor(lib, bsa, t, al)
    c = api.Tensor(lib, bsa, t, al)
    bsa.free()
    _fill_sym([a, c], [2, 2, 3, 3], ANTI4)
    bsb = _space(lib, [9] * 4, [(d, x) for x in (3, 7) for d in range(4)])
    b = api.Tensor(lib, bsb, t, al)
    bsb.free()
    _fill_sym([b], [3, 3, 3, 3], PAIR8)
    return b, a, c  # swapped, as in the reference


def make_abc_11(lib, al, t):    # test.c:1002-1087
    bsa = _space(lib, [6] * 4, [(d, 2) for d in range(4)])
    a = api.Tensor(lib, bsa, t, al)
    bsa.free()
    C_, D_ = a.set_canonical, a.set_derivative
    C_((0, 0, 0, 0)); C_((1, 0, 0, 0))
    D_((0, 1, 0, 0), (1, 0, 0, 0), (1, 0, 2, 3), -1.0)
    C_((1, 1, 0, 0))
    D_((0, 0, 1, 0), (1, 0, 0, 0), (2, 3, 0, 1), 1.0)
    C_((1, 0, 1, 0))
    D_((0, 1, 1, 0), (1, 0, 1, 0), (1, 0, 2, 3), -1.0)
    C_((1, 1, 1, 0))
    D_((0, 0, 0, 1), (1, 0, 0, 0), (2, 3, 1, 0), -1.0)
    D_((1, 0, 0, 1), (1, 0, 1, 0), (0, 1, 3, 2), -1.0)
    D_((0, 1, 0, 1), (1, 0, 1, 0), (1, 0, 3, 2), 1.0)
    D_((1, 1, 0, 1), (1, 1, 1, 0), (0, 1, 3, 2), -1.0)
    D_((0, 0, 1, 1), (1, 1, 0, 0), (2, 3, 0, 1), 1.0)
    D_((1, 0, 1, 1), (1, 1, 1, 0), (2, 3, 0, 1), 1.0)
    D_((0, 1, 1, 1), (1, 1, 1, 0), (3, 2, 0, 1), -1.0)
    C_((1, 1, 1, 1))
    bsb = _space(lib, [3, 3, 6, 6], [(2, 2), (3, 2)])
    b = api.Tensor(lib, bsb, t, al)
    bsb.free()
    for blk in [(0, 0, 0, 0), (0, 0, 0, 1), (0, 0, 1, 0), (0, 0, 1, 1)]:
        b.set_canonical(blk)
    return a, b, b.structure()


def make_abc_12(lib, al, t):    # test.c:1089-1190
    bsa = _space(lib, [11] * 4, [(d, x) for x in (2, 7, 8) for d in range(4)])
    a = api.Tensor(lib, bsa, t, al)
    b = api.Tensor(lib, bsa, t, al)
    bsa.free()
    import itertools
    for blk in itertools.product(range(4), repeat=4):
        if b.block_type(blk) != api.ZERO:
            continue
        a.set_canonical(blk)
        b.set_canonical(blk)
        for perm, s in PAIR8:
            b2 = tuple(blk[perm[k]] for k in range(4))
            if b.block_type(b2) == api.ZERO:
                a.set_derivative(b2, blk, perm, s)
                b.set_derivative(b2, blk, perm, s)
    bsc = _space(lib, [11, 11], [(0, 2), (1, 2), (0, 7), (1, 7), (0, 8), (1, 8)])
    c = api.Tensor(lib, bsc, t, al, canonical=True)
    bsc.free()
    return a, b, c


# test.c:1875-1959
ADD_TESTS = [(make_ab_1, "abcdefgh", "abcdefgh"), (make_ab_2, "ijkl", "ijkl"),
             (make_ab_2, "ijkl", "ijlk"), (make_ab_2, "ijkl", "jkil"),
             (make_ab_2, "ijkl", "lkji"), (make_ab_3, "ij", "ij"),
             (make_ab_3, "ji", "ij"), (make_ab_4, "ij", "ij"), (make_ab_4, "ij", "ji")]
MUL_DIV_TESTS = ADD_TESTS[:5] + [(make_ab_5, "ij", "ij")]
DOT_TESTS = ADD_TESTS + [(make_ab_5, "ij", "ij")]
CONTRACT_TESTS = (
    [(make_abc_1, ia, ib, ic) for ia, ib, ic in
     [("ik", "kj", "ij"), ("ik", "kj", "ji"), ("ik", "jk", "ij"), ("ik", "jk", "ji"),
      ("ki", "kj", "ij"), ("ki", "kj", "ji"), ("ki", "jk", "ij"), ("ki", "jk", "ji")]] +
    [(make_abc_2, ia, ib, ic) for ia, ib, ic in
     [("ik", "kj", "ij"), ("ik", "kj", "ji"), ("ik", "jk", "ij"), ("ik", "jk", "ji"),
      ("ki", "kj", "ij"), ("ki", "kj", "ji"), ("ki", "jk", "ij"), ("ki", "jk", "ji")]] +
    [(make_abc_3, "abcdefgh", "abcdefgi", "ih"), (make_abc_3, "abcdefgi", "abcdefgh", "ih"),
     (make_abc_3, "abcdxfgh", "abcdyfgh", "xy"), (make_abc_3, "abcdefgh", "obcdefgh", "ao"),
     (make_abc_3, "abcdefgh", "obcdefgh", "oa"),
     (make_abc_4, "abcdef", "abcijk", "ijkdef"), (make_abc_4, "abcdef", "aibjck", "ijkdef"),
     (make_abc_4, "badcfe", "xyzdef", "xyzabc")] +
    [(make_abc_5, ia, ib, ic) for ia, ib, ic in
     [("ik", "kj", "ij"), ("ik", "kj", "ji"), ("ik", "jk", "ij"), ("ik", "jk", "ji"),
      ("ki", "kj", "ij"), ("ki", "kj", "ji"), ("ki", "jk", "ij"), ("ki", "jk", "ji")]] +
    [(make_abc_6, "y", "xz", "xyz"), (make_abc_7, "abc", "abd", "dc"),
     (make_abc_8, "ab", "b", "a"),
     (make_abc_9, "ijab", "abcd", "ijcd"), (make_abc_9, "ijcd", "abcd", "ijab"),
     (make_abc_10, "abcd", "ijab", "ijcd"), (make_abc_10, "cdab", "ijab", "ijcd"),
     (make_abc_11, "abcd", "ijcd", "ijab"),
     (make_abc_12, "abcf", "abce", "ef"), (make_abc_12, "abfc", "abce", "ef"),
     (make_abc_12, "fabc", "bace", "ef"), (make_abc_12, "abcf", "acbe", "fe"),
     (make_abc_12, "afbc", "eabc", "fe"), (make_abc_12, "afcb", "bace", "fe")])
assert len(CONTRACT_TESTS) == 46
