"""CPU: the multi-rank plumbing of bench.py, run as two gloo ranks on
127.0.0.1.

The contraction path runs replicas only (one independent contraction per
GPU, no collective on the data path), so the N > 1 logic is host-side: a
barrier around the timed region, the maximum of the timed interval over the
ranks, and rank 0 alone printing the result line.  The reference arm runs
its CPU sample on rank 0 only; the other ranks exit without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks()
    r.barrier()
    m = r.max(1.5 * (rank + 1))
    r.barrier()
    q.put((rank, r.world, m))
    r.dist.destroy_process_group()


def test_two_ranks_barrier_and_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(60)
    assert [p.exitcode for p in ps] == [0, 0]
    assert res == [(0, 2, 3.0), (1, 2, 3.0)]


def test_reference_arm_two_ranks_prints_once(tmp_path):
    """torchrun with two ranks: one JSON line, from rank 0, with the
    reference arm's keys; both ranks exit 0."""
    # torchrun's own scratch directories go under the test's directory
    env = dict(os.environ, OMP_NUM_THREADS="2", TMPDIR=str(tmp_path))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--scale", "4"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    if "unavailable" not in d:
        assert d["unit"] == "TFLOP/s" and d["value"] > 0
        assert d["e2e"]["h2d_bytes_per_step"] == 0
        assert d["cpu_baseline"]["cores"] >= 1
        # one step is the whole contraction
        assert d["cpu_baseline"]["sample"].startswith("262 of 262 ")
