"""The allocation-free dot product against the regular xm_dot.

xmg_dot_noalloc exists for callers that cannot allocate memory when they
need the value (a host program whose pool already holds the GPU memory it
may use, or a per-iteration norm in a tight solver loop).  This file is
collected last so that a failure here cannot hide other results; it must
pass both alone in a fresh process and after every other test, and runs
each case twice in a row because all calls share one static device array.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import helpers as H
from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(lib, a, b, ia, ib):
    f = lib.dll.xmg_dot_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(api.Scalar)]
    f.restype = C.c_int
    out = api.Scalar()
    lib.check(f(a.h, b.h, ia.encode(), ib.encode(), C.byref(out)))
    return out.value()


def _close(x, ref, dt):
    # the tolerance of the dot-product parity tests
    return abs(x - ref) <= (1e-3 if dt < 2 else 1e-10) * max(1.0, abs(ref))


@pytest.mark.parametrize("ci", range(len(cases.DOT_TESTS)))
def test_noalloc_dot_matches_xm_dot(engine, ci):
    al = api.Allocator(engine)
    make, ia, ib = cases.DOT_TESTS[ci]
    for dt in H.TYPES:
        a, b = make(engine, al, dt)
        rng = np.random.default_rng(40 + ci)
        H.fill_random(a, rng)
        H.fill_random(b, rng)
        ref = api.dot(a, b, ia, ib)
        first = _noalloc(engine, a, b, ia, ib)
        second = _noalloc(engine, a, b, ia, ib)
        assert _close(first, ref, dt), (first, ref)
        assert _close(second, ref, dt), (second, ref)
        a.free()
        b.free()
    al.destroy()


def test_noalloc_dot_ladder(engine):
    """Many blocks (several batches) with derivative blocks on both sides."""
    al = api.Allocator(engine)
    w = W.cfg1(engine, al)
    W.fill(w.c, 99, W.LADDER_ANTISYM)
    ref = api.dot(w.a, w.c, "ijab", "ijab")
    for _ in range(2):
        got = _noalloc(engine, w.a, w.c, "ijab", "ijab")
        assert _close(got, ref, api.DOUBLE), (got, ref)
    got = _noalloc(engine, w.a, w.c, "ijab", "jiba")
    assert _close(got, api.dot(w.a, w.c, "ijab", "jiba"), api.DOUBLE)
    w.free()
    al.destroy()


def test_noalloc_dot_rejects_oversize_block(engine):
    al = api.Allocator(engine)
    n = 16384 * 2048 + 1
    bs = api.BlockSpace(engine, [n])
    a = api.Tensor(engine, bs, api.FLOAT, al, canonical=True)
    bs.free()
    f = engine.dll.xmg_dot_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_char_p, C.POINTER(api.Scalar)]
    out = api.Scalar()
    assert f(a.h, a.h, b"i", b"i", C.byref(out)) == 1
    assert b"exceeds the maximum" in engine.xmg_last_error()
    a.free()
    al.destroy()
