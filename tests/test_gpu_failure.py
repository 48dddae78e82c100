"""GPU: failure detection without a fault.

Every pipeline wait of the GEMM kernels is bounded: on timeout the kernel
records an error code, stops its roles, waits (bounded) for its own copies
and MMAs, frees TMEM and returns, and the host reports XMG_ETIMEOUT.  The
self-test drives that path on purpose with a barrier that nothing arrives
at and a short limit; the context must stay usable afterwards (a
contraction right after it still matches the oracle)."""
import time

import pytest

from libxm_gb300 import api, workloads as W

pytestmark = pytest.mark.gpu

XMG_ETIMEOUT = 5


def test_bounded_wait_gives_up_and_device_stays_usable(engine, oracle):
    t0 = time.perf_counter()
    st = engine.xmg_selftest_bounded_wait(200000)        # 200 ms
    dt = time.perf_counter() - t0
    assert st == XMG_ETIMEOUT
    assert "gave up" in engine.xmg_last_error().decode()
    assert 0.15 <= dt < 10.0
    gal, oal = api.Allocator(engine), api.Allocator(oracle)
    we, wo = W.cfg1(engine, gal), W.cfg1(oracle, oal)
    try:
        we.run()
        wo.run()
        assert W.rel_frobenius(W.read_canonical(we.c), W.read_canonical(wo.c)) <= 1e-12
    finally:
        we.free()
        wo.free()
