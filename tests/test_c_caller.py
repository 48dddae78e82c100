"""A compiled C program calling the libxm API (tests/c/ladder_caller.c).

The program builds a small antisymmetric ladder, runs xm_contract, xm_set
+ xm_add and xm_contract with beta = 1, and compares every result with
values this test computes with the oracle on the same structure and inputs
(the program's own deterministic stream, replicated here).  On the CPU it
is linked against the oracle library, which pins the replication; on the
GPU it is linked against libxmgb.so like any user program (include/ and
-lxmgb), so the engine runs behind a C caller, not behind ctypes.
"""
import os
import subprocess

import numpy as np
import pytest

from libxm_gb300 import api, workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "ladder_caller.c")


def _stream(seed, n):
    """The program's uniform(seed, i), i = 0 .. n-1: splitmix64 in [-0.5, 0.5)."""
    return (W.splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53) - 0.5


def _expected(oracle):
    al = api.Allocator(oracle)
    so = [[4, 3], [4, 3], [5, 6], [5, 6]]
    sv = [[5, 6]] * 4
    ts = {}
    for name, spec in (("a", so), ("b", sv), ("c", so), ("a2", so)):
        bs = W.make_space(oracle, spec)
        ts[name] = W.symmetric_tensor(oracle, al, bs, api.DOUBLE, W.LADDER_ANTISYM)
        bs.free()
    for name, seed in (("a", 11), ("b", 12)):
        t = ts[name]
        blocks = t.canonical_blocks()
        vals = _stream(seed, sum(t.block_size(blk) for blk in blocks))
        pos = 0
        for blk in blocks:
            n = t.block_size(blk)
            t.write_block(blk, vals[pos:pos + n])
            pos += n
    a, b, c, a2 = ts["a"], ts["b"], ts["c"], ts["a2"]

    def dump():
        return np.concatenate([c.read_block(blk) for blk in c.canonical_blocks()])
    out = []
    api.contract(0.5, a, b, 0.0, c, "ijcd", "cdab", "ijab")
    out.append(dump())
    api.set_all(a2, 0.125)
    api.add(2.0, c, -0.5, a2, "ijab", "jiba")
    out.append(dump())
    api.contract(-1.5, a, b, 1.0, c, "ijcd", "cdab", "ijab")
    out.append(dump())
    for t in ts.values():
        t.free()
    al.destroy()
    return np.concatenate(out)


def _build_and_run(tmp_path, lib_path, expected):
    exe = str(tmp_path / "ladder_caller")
    libdir, name = os.path.split(lib_path)
    lname = name[3:].split(".so")[0]          # libxmgb.so -> xmgb
    subprocess.run(["cc", "-O2", "-std=gnu11", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", libdir, "-l" + lname, "-Wl,-rpath," + libdir, "-lm", "-o", exe],
                   check=True, capture_output=True, text=True)
    want = str(tmp_path / "expected.bin")
    expected.astype(np.float64).tofile(want)
    return subprocess.run([exe, want], capture_output=True, text=True, timeout=300)


def test_c_caller_against_oracle_library(oracle, tmp_path):
    """CPU: the program linked against the oracle library reproduces the
    expected values (the inputs are replicated correctly)."""
    r = _build_and_run(tmp_path, oracle.path, _expected(oracle))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")


@pytest.mark.gpu
def test_c_caller_on_engine(engine, oracle, tmp_path):
    """GPU: the same program linked against the engine (libxmgb.so)."""
    r = _build_and_run(tmp_path, engine.path, _expected(oracle))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "GB300" in r.stdout and r.stdout.strip().endswith("ok")
