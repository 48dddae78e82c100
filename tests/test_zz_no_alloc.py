"""The allocation-free dot product against the regular xm_dot and the oracle.

xmg_dot_noalloc exists for callers that cannot allocate memory when they
need the value (a host program whose pool already holds the GPU memory it
may use, or a per-iteration norm in a tight solver loop).  This file is
collected last so that a failure here cannot hide other results; it must
pass both alone in a fresh process and after every other test, and runs
each case twice in a row because all calls share one static device array.
The first test checks the promise itself: in a fresh process the first
and the second call change neither the device's free memory nor the
engine's allocation count.
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


def _memory(lib):
    free, total = C.c_size_t(), C.c_size_t()
    lib.check(lib.xmg_device_memory(C.byref(free), C.byref(total)))
    f = lib.dll.xmgd_arena_bytes_in_use
    f.restype = C.c_size_t
    return int(free.value), int(f())


def test_noalloc_dot_allocates_nothing(engine):
    """First test of the file: in a fresh process these are the first two
    xmg_dot_noalloc calls.  The tensors (and so the engine) exist before;
    the calls must leave the device's free memory and the engine's
    allocated bytes unchanged."""
    al = api.Allocator(engine)
    w = W.cfg1(engine, al)
    W.fill(w.c, 98, W.LADDER_ANTISYM)
    engine.check(engine.xmg_synchronize())
    before = _memory(engine)
    first = _noalloc(engine, w.a, w.c, "ijab", "ijab")
    after_first = _memory(engine)
    second = _noalloc(engine, w.a, w.c, "ijab", "ijab")
    after_second = _memory(engine)
    assert after_first == before, (before, after_first)
    assert after_second == before, (before, after_second)
    ref = api.dot(w.a, w.c, "ijab", "ijab")
    assert _close(first, ref, api.DOUBLE) and _close(second, ref, api.DOUBLE), (first, second, ref)
    w.free()
    al.destroy()


@pytest.mark.parametrize("ci", range(len(cases.DOT_TESTS)))
def test_noalloc_dot_matches_xm_dot(engine, oracle, ci):
    """Against the engine's xm_dot and, on identical inputs, the oracle's."""
    al, oal = api.Allocator(engine), api.Allocator(oracle)
    make, ia, ib = cases.DOT_TESTS[ci]
    for dt in H.TYPES:
        a, b = make(engine, al, dt)
        rng = np.random.default_rng(40 + ci)
        H.fill_random(a, rng)
        H.fill_random(b, rng)
        oa, ob_ = make(oracle, oal, dt)
        rng = np.random.default_rng(40 + ci)
        H.fill_random(oa, rng)
        H.fill_random(ob_, rng)
        ref = api.dot(a, b, ia, ib)
        ref_oracle = api.dot(oa, ob_, ia, ib)
        first = _noalloc(engine, a, b, ia, ib)
        second = _noalloc(engine, a, b, ia, ib)
        for got in (first, second):
            assert _close(got, ref, dt), (got, ref)
            assert _close(got, ref_oracle, dt), (got, ref_oracle)
        for t in (a, b, oa, ob_):
            t.free()
    al.destroy()
    oal.destroy()


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


def test_noalloc_dot_rejects_bad_arguments(engine):
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
    assert f(None, a.h, b"i", b"i", C.byref(out)) == 1
    assert f(a.h, a.h, None, b"i", C.byref(out)) == 1
    assert b"NULL" in engine.xmg_last_error()
    a.free()
    al.destroy()
