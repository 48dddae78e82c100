#!/usr/bin/env python3
"""Benchmark: xm_contract TFLOP/s on one GB300, split-precision (emulated
FP64 on tcgen05 tensor cores) against the plain FP64 GPU form, with the
relative Frobenius error of both against FP64 references.

Workload: the uneven-block, Z2^3-sparse FP64 ladder
    C(i,j,a,b) = sum_{c,d} A(i,j,c,d) B(c,d,a,b)
o = 96 in 6 blocks of 8..24, v = 384 in 12 blocks of 16..48, i<->j, c<->d,
a<->b antisymmetry, seeded uniform[-1,1] data (synthetic: splitmix64).
Inputs (A ~0.3 GB, B ~7.8 GB) are larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

One step = one xm_contract call over the whole workload (plan + kernels +
synchronisation) with block data resident in HBM.  e2e = the same step
through the C API with host buffers: every canonical block of A and B
written from page-locked host memory, the contraction, every canonical
block of C read back.  For N > 1 (torchrun) every rank runs an independent
replica on its own GPU (no collective on the data path; weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

from libxm_gb300 import api  # noqa: E402  (ctypes binding only)

METRIC = "xm_contract TFLOP/s on 1 GB300: split-precision vs plain FP64 at rel err ≤1e-12"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["engine", "reference"], default="engine")
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-out-of-core", action="store_true",
                   help="skip the pagefile-streamed measurement")
    p.add_argument("--no-elementwise", action="store_true",
                   help="skip the xm_set / xm_add bandwidth measurement")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the other measured configurations (cfg1, cfg3, cfg4)")
    p.add_argument("--scale", type=int, default=1, help="shrink block sizes (debug only)")
    p.add_argument("--subset", type=str, default=None,
                   help="O,V: keep the first O occupied and V virtual blocks (profiling case)")
    p.add_argument("--cfg5-v-blocks", type=int, default=0,
                   help="v blocks of the production ladder's structure streamed from a "
                        "pagefile (0: the most, up to 21, that the disk and RAM hold)")
    p.add_argument("--cfg5-region-gb", type=float, default=32.0,
                   help="HBM region size for that measurement (32: the engine's default)")
    p.add_argument("--cfg5-only", action="store_true",
                   help="only the production-ladder subset measurement (one JSON line)")
    p.add_argument("--ring-only", choices=["f32", "c128", "f64"], default=None,
                   help="only the ring term in that type (profiling case; one JSON line)")
    p.add_argument("--ladder-only", action="store_true",
                   help="only the headline ladder's device time and the adjoint of it "
                        "(tuning case; one JSON line)")
    p.add_argument("--ring-nv", type=int, default=8,
                   help="v blocks (of 32) of the ring term for --ring-only")
    return p.parse_args()


# ---------------------------------------------------------------- ranks --
class Ranks:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            import torch.distributed as dist
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)])
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


# --------------------------------------------------------------- clocks --
class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev, self.rows, self.proc = dev, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 7
                          for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm),
                "power_w_max": max((float(r[2]) for r in self.rows if len(r) >= 7
                                    and r[2].replace(".", "").isdigit()), default=None)}


# ------------------------------------------------------------- CPU side --
def cpu_lib():
    """The reference built from source when it loads on this machine, else
    the oracle port.  Returns (lib, kind)."""
    import oracle.build as ob
    from libxm_gb300 import api
    blas = ob.find_blas()
    ref = ob.build_reference()
    if ref is not None:
        try:
            lib = api.Lib(ref)
            lib.dll.xmref_set_blas.argtypes = [api.C.c_char_p]
            lib.dll.xmref_set_blas(blas.encode() if blas else None)
            return lib, "reference"
        except OSError:
            pass
    lib = api.Lib(ob.build_oracle())
    lib.dll.xmo_set_blas.argtypes = [api.C.c_char_p]
    lib.dll.xmo_set_blas(blas.encode() if blas else None)
    return lib, "port"


def cpu_contract_timed(w, reps):
    """The CPU reference's whole xm_contract on w's workload (all canonical
    output blocks): one untimed warm-up call, then `reps` timed calls.
    All host threads, OPENBLAS_NUM_THREADS=1 (the reference parallelises
    over output blocks itself).  Returns (seconds per call, best seconds,
    {block: data})."""
    api.contract(w.alpha, w.a, w.b, w.beta, w.c, w.idxa, w.idxb, w.idxc)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        api.contract(w.alpha, w.a, w.b, w.beta, w.c, w.idxa, w.idxb, w.idxc)
        times.append(time.perf_counter() - t0)
    return float(np.mean(times)), min(times), {blk: w.c.read_block(blk)
                                               for blk in w.c.canonical_blocks()}


def cpu_threads(lib):
    n = lib.dll.xmo_num_threads() if hasattr(lib.dll, "xmo_num_threads") else 0
    return int(os.environ.get("OMP_NUM_THREADS") or n or os.cpu_count())


def cpu_baseline(w, flops, reps=3):
    """The CPU reference timed on the whole workload (every canonical output
    block), best of `reps` calls after one warm-up, on the same inputs as
    the engine (the engine's A and B copied over)."""
    from libxm_gb300 import workloads as W
    lib, kind = cpu_lib()
    al = api.Allocator(lib)
    wc = make_workload(lib, al, w.scale, w.subset, fill_data=False)
    W.copy_data(w.a, wc.a)
    W.copy_data(w.b, wc.b)
    mean_s, best_s, out = cpu_contract_timed(wc, reps)
    nblk = len(out)
    res = {"value": flops / best_s / 1e12, "unit": "TFLOP/s", "cores": cpu_threads(lib),
           "kind": kind,
           "sample": "%d of %d canonical output blocks (the whole xm_contract, %.3e useful "
                     "flops), best of %d calls after one warm-up: %.2f s (mean %.2f s)"
                     % (nblk, nblk, flops, reps, best_s, mean_s)}
    wc.free()
    al.destroy()
    return res, out


def cpu_sample_error(w, chosen, c0, got):
    """CPU-baseline leg: the CPU reference's result for the chosen canonical
    output blocks of w's workload (its other output blocks zero, so it
    does only the sample's work) on the engine's inputs, with the chosen
    blocks' initial values c0 (beta != 0); relative Frobenius error of the
    engine's blocks `got` over the sample."""
    from libxm_gb300 import workloads as W
    lib, _ = cpu_lib()
    al = api.Allocator(lib)
    wc = W.cfg3(lib, al, dtype=w.a.dtype, fill_data=False)
    W.copy_data(w.a, wc.a)
    W.copy_data(w.b, wc.b)
    ref = W.contract_sample(wc, chosen, c0)
    wc.free()
    al.destroy()
    return W.rel_frobenius(got, ref)


def block_costs(w):
    """Useful flops per canonical output block (the reference's GEMM work)."""
    import oracle.build as ob
    from libxm_gb300 import api
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    lib = w.c.lib
    blocks = w.c.canonical_blocks()
    cost = [0.0] * len(blocks)
    if lib.gb:
        import helpers as H
        for l, _, m, n, k in H.pair_structure_engine(lib, w.a, w.b, w.c, w.idxa, w.idxb, w.idxc):
            cost[l] += 2.0 * m * n * k
        return cost
    # plan-only pass of the oracle on the same structure
    orc = api.Lib(ob.build_oracle())
    oal = api.Allocator(orc)
    wo = make_workload(orc, oal, w.scale, w.subset, fill_data=False)
    import helpers as H
    orc.dll.xmo_set_plan_only(1)
    for l, _, m, n, k in H.pair_structure_oracle(orc, wo.a, wo.b, wo.c, wo.idxa, wo.idxb, wo.idxc):
        cost[l] += 2.0 * m * n * k
    orc.dll.xmo_set_plan_only(0)
    wo.free()
    return cost


# DRAM bytes (read + write) of one split-precision GEMM launch on the cfg2
# ladder, from a single-pass ncu capture of that kernel on this workload
# (dram__bytes_read.sum + dram__bytes_write.sum, the stacked work list the
# tuner keeps, 256-element chunks, two K steps per pipeline stage; the
# command is in the launch-list profile)
GEMM_DRAM_BYTES = 77.56e9 + 0.93e9


def timed_calls(eng, fn, reps=3, warm=5):
    """Device time per call of fn after `warm` untimed calls (plan, tuning)."""
    for _ in range(warm):
        fn()
    eng.check(eng.xmg_synchronize())
    eng.check(eng.xmg_timer_start())
    for _ in range(reps):
        fn()
    return eng.xmg_timer_stop() / reps


def adjoint_modes(eng, api, w, dc):
    """The form xm_contract_adjoint takes for each gradient (1 symmetric,
    2 every position), from its host-only checks."""
    import ctypes
    mode = (ctypes.c_int * 2)()
    eng.check(eng.xmg_adjoint_plan_check(w.a.h, w.b.h, dc.h, w.idxa.encode(), w.idxb.encode(),
                                         w.idxc.encode(), mode, None, None))
    return list(mode)


def other_configs(eng, api, W, check=None):
    """The remaining measured configurations at full size: the plain FP64
    ladder cfg1, the permuted ring term cfg3 in float32 and complex128
    (o = 64 as 4 x 16, v = 256 as 8 x 32, beta = 1, C prefilled), and the
    adjoint of the cfg2 ladder (cfg4: dA and dB in one call).  Accuracy of
    the float32 ring term: against the same contraction in FP64 on the GPU
    (plain path) over identical, float-rounded inputs; of the complex128
    one (when `check`, the CPU-baseline leg's sample check, is given):
    against the CPU reference on 40 seeded output blocks."""
    out = {}
    al = api.Allocator(eng)
    eng.check(eng.xmg_set_precision(api.PREC_AUTO))
    # cfg1
    w = W.cfg1(eng, al)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())
    ms = timed_calls(eng, w.run)
    out["cfg1_ladder_o24_v64"] = {"ms": ms, "tflops": fl / ms / 1e9, "useful_flops": fl,
                                  "precision_used": api.last_stats(eng).precision_used}
    w.free()
    # cfg3 float32, with an FP64 twin for the error
    w = W.cfg3(eng, al, dtype=api.FLOAT)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())
    c0 = W.read_canonical(w.c)
    wd = W.cfg3(eng, al, dtype=api.DOUBLE)
    for ts, td in zip(w.tensors(), wd.tensors()):
        for blk in ts.canonical_blocks():
            td.write_block(blk, ts.read_block(blk).astype(np.float64))
    ms = timed_calls(eng, w.run)
    used = api.last_stats(eng).precision_used
    for blk, x in c0.items():           # restore C, then one more call: beta = 1
        w.c.write_block(blk, x)
    w.run()
    eng.check(eng.xmg_set_precision(api.PREC_FP64))
    wd.run()
    eng.check(eng.xmg_set_precision(api.PREC_AUTO))
    rel = W.rel_frobenius(W.read_canonical(w.c), W.read_canonical(wd.c))
    out["cfg3_ring_o64_v256_f32"] = {"ms": ms, "tflops": fl / ms / 1e9, "useful_flops": fl,
                                     "precision_used": used, "rel_err_vs_fp64": rel}
    w.free()
    wd.free()
    # cfg3 complex128
    w = W.cfg3(eng, al, dtype=api.DOUBLE_COMPLEX)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())
    chosen = W.sample_blocks(w.c.canonical_blocks(), 40, seed=31)
    c0 = {blk: w.c.read_block(blk) for blk in chosen}
    ms = timed_calls(eng, w.run)
    out["cfg3_ring_o64_v256_c128"] = {"ms": ms, "tflops": fl / ms / 1e9, "useful_flops": fl,
                                      "precision_used": api.last_stats(eng).precision_used}
    if check is not None:
        for blk in chosen:                 # beta = 1: restore the sample, one more call
            w.c.write_block(blk, c0[blk])
        w.run()
        got = {blk: w.c.read_block(blk) for blk in chosen}
        out["cfg3_ring_o64_v256_c128"]["rel_err_vs_oracle_sample"] = check(w, chosen, c0, got)
        out["cfg3_ring_o64_v256_c128"]["sample"] = "%d of %d canonical output blocks" % (
            len(chosen), len(w.c.canonical_blocks()))
    w.free()
    # cfg4: the adjoint of the cfg2 ladder, dA and dB
    w = W.cfg2(eng, al)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())
    dc = w.c.structure()
    W.fill(dc, 77, W.LADDER_ANTISYM)
    da, db = w.a.structure(), w.b.structure()

    def adj():
        eng.check(eng.xm_contract_adjoint(api.Scalar.of(1.0), w.a.h, w.b.h, dc.h, da.h, db.h,
                                          b"ijcd", b"cdab", b"ijab"))
    ms = timed_calls(eng, adj)

    def grads():
        api.set_all(da, 0)
        api.set_all(db, 0)
        adj()
        return {**{("a",) + k: v for k, v in W.read_canonical(da).items()},
                **{("b",) + k: v for k, v in W.read_canonical(db).items()}}
    g_emu = grads()
    used = api.last_stats(eng).precision_used
    # the same adjoint on the FP64 path: one call (about 9 s)
    eng.check(eng.xmg_set_precision(api.PREC_FP64))
    try:
        ms64 = timed_calls(eng, adj, reps=1, warm=1)
        g_64 = grads()
    finally:
        eng.check(eng.xmg_set_precision(api.PREC_AUTO))
    out["cfg4_adjoint_cfg2"] = {
        "ms": ms, "tflops": 2 * fl / ms / 1e9, "useful_flops": 2 * fl,
        "precision_used": used,
        "fp64_plain": {"ms": ms64, "tflops": 2 * fl / ms64 / 1e9},
        "speedup_vs_fp64_plain": ms64 / ms,
        "rel_err_vs_fp64": W.rel_frobenius(g_emu, g_64),
        "form": "symmetric" if adjoint_modes(eng, api, w, dc) == [1, 1] else "every position",
        "note": "dA and dB in one call; symmetric form: each gradient one contraction "
                "at the canonical positions of A (B), then a per-block multiplicity "
                "scale (the structural checks pass for the antisymmetric ladder)"}
    for x in (dc, da, db):
        x.free()
    w.free()
    out["tile_autosplit_ladder_o92_v376"] = tile_autosplit(eng, api, W, al)
    al.destroy()
    return out


def padding_model(eng, w):
    """Useful over issued MMA work of a contraction's merged pairs on the
    split-precision GEMM's tiles, one output block per tile: the M side in
    128-row tiles, the N side and K rounded up to 16, the orientation with
    less padding."""
    import helpers as H
    up = lambda x, q: -(-x // q) * q
    useful = issued = 0.0
    for _, _, m, n, k in H.pair_structure_engine(eng, w.a, w.b, w.c, w.idxa, w.idxb, w.idxc):
        useful += m * n * k
        issued += min(up(m, 128) * up(n, 16), up(n, 128) * up(m, 16)) * up(k, 16)
    return useful / issued if issued else None


def tile_autosplit(eng, api, W, al):
    """The opt-in tile-aware autosplit against the reference's autosplit on
    the same dimensions (o = 92, v = 376, Z2^3 labels per block, the same
    block counts): block sizes, the padding model and measured time."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    res = {}
    for name, tiles in (("reference_autosplit", None), ("tiles_32_16", (32, 16))):
        o_sz, v_sz = W.split_sizes(eng, 92, tiles), W.split_sizes(eng, 376, tiles)
        w = W.autosplit_ladder(eng, al, o_sz, v_sz)
        fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(),
                                    w.idxc.encode())
        ms = timed_calls(eng, w.run)
        res[name] = {"o": o_sz, "v": v_sz, "ms": ms, "useful_flops": fl,
                     "tflops": fl / ms / 1e9, "padding_efficiency": padding_model(eng, w),
                     "gemm_ms": api.last_stats(eng).ms_gemm}
        w.free()
    res["note"] = ("padding_efficiency = useful MMA work / issued MMA work (M side in "
                   "128-row tiles, N and K in 16s, one output block per tile); the "
                   "GEMM's stacked tiles recover part of the padding either way")
    return res


def ring_only(eng, api, W, args):
    """The ring term alone (o = 64 as 4 x 16, v = 32 * ring_nv, beta = 1):
    `warmup` untimed calls (plan, work-list tuning), then device time per
    call over `steps` calls and the last call's phases."""
    dt = {"f32": api.FLOAT, "c128": api.DOUBLE_COMPLEX, "f64": api.DOUBLE}[args.ring_only]
    al = api.Allocator(eng)
    w = W.cfg3(eng, al, dtype=dt, nv=args.ring_nv)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(),
                                w.idxc.encode())
    ms = timed_calls(eng, w.run, reps=args.steps, warm=args.warmup)
    st = api.last_stats(eng)
    out = {"workload": "ring_o64_v%d_%s" % (32 * args.ring_nv, args.ring_only), "ms": ms,
           "useful_flops": fl, "tflops": fl / ms / 1e9, "gemm_ms": st.ms_gemm,
           "split_ms": st.ms_split, "policy": st.gemm_policy,
           "precision_used": st.precision_used}
    w.free()
    al.destroy()
    return out


def ladder_only(eng, api, W, args):
    """The headline ladder (or its --subset / --scale form): device time per
    xm_contract over `steps` calls after `warmup` untimed ones, the GEMM
    and split phases of the last call, and the adjoint (dA and dB) of the
    same ladder, timed the same way."""
    al = api.Allocator(eng)
    w = make_workload(eng, al, args.scale, args.subset)
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(),
                                w.idxc.encode())
    ms = timed_calls(eng, w.run, reps=args.steps, warm=args.warmup)
    st = api.last_stats(eng)
    out = {"workload": w.name, "ms": ms, "useful_flops": fl, "tflops": fl / ms / 1e9,
           "gemm_ms": st.ms_gemm, "split_ms": st.ms_split, "policy": st.gemm_policy}
    dc = w.c.structure()
    W.fill(dc, 77, W.LADDER_ANTISYM)
    da, db = w.a.structure(), w.b.structure()

    def adj():
        eng.check(eng.xm_contract_adjoint(api.Scalar.of(1.0), w.a.h, w.b.h, dc.h, da.h, db.h,
                                          b"ijcd", b"cdab", b"ijab"))
    ams = timed_calls(eng, adj, reps=args.steps, warm=args.warmup)
    out["adjoint"] = {"ms": ams, "useful_flops": 2 * fl, "tflops": 2 * fl / ams / 1e9}
    eng.xmg_adjoint_release()
    for t in (dc, da, db):
        t.free()
    w.free()
    al.destroy()
    return out


def mem_available():
    """MemAvailable of /proc/meminfo in bytes (0 if unreadable)."""
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def cfg5_v_blocks_that_fit(W, path, most=21, least=12):
    """The most v blocks (least..most) whose canonical a, b and c fit the
    pagefile's file system (10 GB kept free) and half the available RAM
    (the page cache holds the pagefile while it is streamed)."""
    import shutil
    disk = shutil.disk_usage(path).free - 10e9
    ram = 0.5 * mem_available()
    for n in range(most, least - 1, -1):
        if sum(W.cfg5_bytes(n)) <= min(disk, ram):
            return n, disk, ram
    return 0, disk, ram


def cfg5_subset(eng, api, W, v_blocks=0, region=int(32e9)):
    """The production ladder's structure (o = 128 as 8 x 16, v blocks of
    24..40 with Z2^3 labels) on its first v_blocks v blocks (0: the most
    that the host holds, up to 21, where b is 60 GB), all tensors in a
    pagefile and b streamed through two HBM regions of `region` bytes:
    split-precision against the plain FP64 path on the same inputs, wall
    clock per xm_contract (the first split-precision call plans; the
    repeated ones reuse the kept streamed plan).  The full b (~300 GB over
    32 v blocks) exceeds the host's disk and RAM."""
    import tempfile
    tmp = tempfile.mkdtemp(prefix="xmg_cfg5_")
    if not v_blocks:
        v_blocks, disk, ram = cfg5_v_blocks_that_fit(W, tmp)
        if not v_blocks:
            os.rmdir(tmp)
            return {"skipped": "12 v blocks (%.1f GB) exceed the free disk (%.1f GB) or half "
                               "the available RAM (%.1f GB)"
                               % (sum(W.cfg5_bytes(12)) / 1e9, disk / 1e9, ram / 1e9)}
    pal = api.Allocator(eng, os.path.join(tmp, "pagefile"))
    t0 = time.perf_counter()
    w = W.cfg5(eng, pal, v_blocks=v_blocks, threads=os.cpu_count() or 1)
    setup = time.perf_counter() - t0
    fl = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(),
                                w.idxc.encode())
    nb = sum(w.b.block_size(blk) for blk in w.b.canonical_blocks()) * 8
    out = {"workload": w.name, "v_blocks": v_blocks, "b_bytes": nb, "useful_flops": fl,
           "region_bytes": region, "setup_s": setup}
    eng.check(eng.xmg_set_staging(1, region))
    try:
        res = {}
        for prec, name, reps in ((api.PREC_AUTO, "emu", 2), (api.PREC_FP64, "fp64", 1)):
            eng.check(eng.xmg_set_precision(prec))
            plan_ms = []
            if prec == api.PREC_AUTO:
                w.run()
                plan_ms.append(api.last_stats(eng).ms_plan)
            best = 1e30
            for _ in range(reps):
                t0 = time.perf_counter()
                w.run()
                best = min(best, time.perf_counter() - t0)
                plan_ms.append(api.last_stats(eng).ms_plan)
            st = api.last_stats(eng)
            res[name] = W.read_canonical(w.c)
            out[name] = {"ms": best * 1e3, "tflops": fl / best / 1e12,
                         "device_ms": st.ms_device, "batches": st.stage_batches,
                         "stage_gbs": st.stage_bytes / best / 1e9,
                         "stage_wait_ms": st.ms_stage_wait, "plan_ms": plan_ms,
                         "precision_used": "emu64" if st.precision_used == api.PREC_EMU64
                         else "fp64"}
        out["speedup_vs_fp64_plain"] = out["fp64"]["ms"] / out["emu"]["ms"]
        out["device_speedup_vs_fp64_plain"] = out["fp64"]["device_ms"] / out["emu"]["device_ms"]
        out["rel_err_vs_fp64"] = W.rel_frobenius(res["emu"], res["fp64"])
    finally:
        eng.check(eng.xmg_set_precision(api.PREC_AUTO))
        eng.check(eng.xmg_set_staging(int(180e9), int(32e9)))
        w.free()
        pal.destroy()
        os.rmdir(tmp)
    return out


def make_workload(lib, al, scale=1, subset=None, fill_data=True):
    from libxm_gb300 import workloads as W
    ob, vb = (int(x) for x in subset.split(",")) if subset else (None, None)
    w = W.cfg2(lib, al, scale=scale, o_blocks=ob, v_blocks=vb, fill_data=fill_data)
    w.scale = scale
    w.subset = subset
    return w


def workload_config(w, flops):
    """The `config` object of both arms' JSON lines (identical keys and
    values for the same workload)."""
    return {"workload": w.name, "o": w.extra["o_sizes"], "v": w.extra["v_sizes"],
            "z2_labels": {"o": w.extra["o_labels"], "v": w.extra["v_labels"]},
            "contraction": "C(ijab)=A(ijcd)B(cdab)", "useful_flops": flops,
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas"}


# --------------------------------------------------------------- engine --
def engine_arm(args, ranks):
    os.environ.setdefault("XMG_DEVICE", str(ranks.local))
    import libxm_gb300
    from libxm_gb300 import api, workloads as W
    libxm_gb300.build()
    eng = libxm_gb300.load()
    if args.ladder_only:
        if ranks.rank == 0:
            print(json.dumps({"ladder": ladder_only(eng, api, W, args)}))
        return
    if args.ring_only:
        if ranks.rank == 0:
            print(json.dumps({"ring_term": ring_only(eng, api, W, args)}))
        return
    if args.cfg5_only:
        if ranks.rank == 0:
            print(json.dumps({"cfg5_subset": cfg5_subset(
                eng, api, W, args.cfg5_v_blocks, int(args.cfg5_region_gb * 1e9))}))
        return
    al = api.Allocator(eng)
    t0 = time.perf_counter()
    w = make_workload(eng, al, args.scale, args.subset)
    setup_s = time.perf_counter() - t0
    flops = eng.xmg_contract_flops(w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())

    def timed(prec, steps, warmup):
        eng.check(eng.xmg_set_precision(prec))
        if prec != api.PREC_FP64:
            # plan building and autotuning: the first calls of a new plan
            # try each work-list candidate once (five at most)
            for _ in range(5):
                w.run()
        for _ in range(warmup):
            w.run()
        ranks.barrier()
        eng.check(eng.xmg_synchronize())
        clk = Clocks(int(os.environ["XMG_DEVICE"]))
        clk.start()
        n0 = eng.xmg_kernel_launches()
        gemm_ms, split_ms = [], []
        eng.check(eng.xmg_timer_start())
        for _ in range(steps):
            w.run()
            st = api.last_stats(eng)
            gemm_ms.append(st.ms_gemm)
            split_ms.append(st.ms_split)
        ms = eng.xmg_timer_stop()
        eng.check(eng.xmg_synchronize())
        launches = eng.xmg_kernel_launches() - n0
        ranks.barrier()
        clocks = clk.stop()
        ms = ranks.max(ms)
        return {"ms_per_step": ms / steps, "gemm_ms": float(np.mean(gemm_ms)),
                "split_ms": float(np.mean(split_ms)), "launches": launches // steps,
                "gemm_policy": api.last_stats(eng).gemm_policy,
                "clocks": clocks, "precision_used": api.last_stats(eng).precision_used,
                "out": W.read_canonical(w.c)}

    emu = timed(api.PREC_AUTO, args.steps, args.warmup)
    fp64 = timed(api.PREC_FP64, args.fp64_steps, 1)
    rel_emu_vs_fp64 = W.rel_frobenius(emu["out"], fp64["out"])

    # end to end through the C API with host buffers, two forms:
    # (1) the headline: A, B and C in page-locked host memory
    #     (xmg_allocator_create_host, the reference's RAM allocator kept in
    #     host memory); every xm_contract copies A and B in and C out, b in
    #     batches whose copies overlap the previous batch's kernels;
    # (2) A, B and C in GPU memory, written from and read back into pinned
    #     host buffers every step with the block list calls.
    e2e = None
    if True:
        eng.check(eng.xmg_set_precision(api.PREC_AUTO))
        hal = api.Allocator(eng, host=True)
        wh = make_workload(eng, hal, args.scale, args.subset, fill_data=False)
        W.copy_data(w.a, wh.a)
        W.copy_data(w.b, wh.b)
        bytes_a = sum(wh.a.block_size(blk) for blk in wh.a.canonical_blocks()) * 8
        bytes_c = sum(wh.c.block_size(blk) for blk in wh.c.canonical_blocks()) * 8
        for _ in range(3):          # plan, tune the batch plans
            wh.run()
        steps = max(1, min(args.steps, 10))
        ranks.barrier()
        acc = np.zeros(4)
        t0 = time.perf_counter()
        for _ in range(steps):
            wh.run()
            st = api.last_stats(eng)
            acc += (st.ms_device, st.ms_plan, st.ms_stage_wait, st.stage_batches)
        dt = ranks.max((time.perf_counter() - t0) / steps)
        st = api.last_stats(eng)
        rel_host = W.rel_frobenius(W.read_canonical(wh.c), emu["out"])
        e2e = {"value": ranks.world * flops / dt / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": int(bytes_a + st.stage_bytes),
               "d2h_bytes_per_step": int(bytes_c), "ms_per_step": dt * 1e3,
               "form": "A, B, C in page-locked host memory (xmg_allocator_create_host); "
                       "each xm_contract copies A and B in (B in batches overlapping the "
                       "previous batch's kernels) and C out",
               "phases_ms": {"device": acc[0] / steps, "plan": acc[1] / steps,
                             "stage_wait": acc[2] / steps},
               "batches": int(acc[3] / steps), "rel_err_vs_hbm_resident": rel_host,
               "link_h2d_floor_ms": (bytes_a + st.stage_bytes) / 212e9 * 1e3}
        wh.free()
        eng.xmg_plan_cache_clear()
        hal.destroy()

        # (2) HBM tensors, block list calls from / into pinned buffers (one
        # page-locked buffer for the inputs, one for the outputs)
        nbytes_in = sum(t.block_size(blk) for t in (w.a, w.b)
                        for blk in t.canonical_blocks()) * 8
        nbytes_out = sum(w.c.block_size(blk) for blk in w.c.canonical_blocks()) * 8
        pin_in, pin_out = eng.xmg_host_alloc(nbytes_in), eng.xmg_host_alloc(nbytes_out)
        host, outs, off = {}, {}, 0
        for t in (w.a, w.b):
            for blk in t.canonical_blocks():
                n = t.block_size(blk) * 8
                buf = np.frombuffer((api.C.c_char * n).from_address(pin_in + off),
                                    dtype=np.float64)
                buf[:] = t.read_block(blk)
                host[(id(t), blk)] = (pin_in + off, buf)
                off += n
        off = 0
        for blk in w.c.canonical_blocks():
            n = w.c.block_size(blk) * 8
            outs[blk] = (pin_out + off, n)
            off += n
        lists = [(t, api.BlockList(t.canonical_blocks(),
                                   [host[(id(t), blk)][0] for blk in t.canonical_blocks()]))
                 for t in (w.a, w.b)]
        cblocks = api.BlockList(list(outs), [outs[blk][0] for blk in outs])
        phase = np.zeros(3)

        def hbm_step():
            t0 = time.perf_counter()
            for t, bl in lists:
                t.write_blocks(bl)
            t1 = time.perf_counter()
            w.run()
            t2 = time.perf_counter()
            w.c.read_blocks(cblocks)
            phase[:] += (t1 - t0, t2 - t1, time.perf_counter() - t2)
        hbm_step()
        ranks.barrier()
        phase[:] = 0
        t0 = time.perf_counter()
        for _ in range(steps):
            hbm_step()
        dt = ranks.max((time.perf_counter() - t0) / steps)
        e2e["hbm_tensors"] = {
            "value": ranks.world * flops / dt / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": nbytes_in, "d2h_bytes_per_step": nbytes_out,
            "ms_per_step": dt * 1e3,
            "form": "A, B, C in GPU memory; every canonical block of A and B written "
                    "from pinned buffers (xmg_tensor_write_blocks) and of C read back "
                    "(xmg_tensor_read_blocks) every step",
            "phases_ms": {"h2d": phase[0] * 1e3 / steps, "contract": phase[1] * 1e3 / steps,
                          "d2h": phase[2] * 1e3 / steps},
            "copies_per_step": sum(bl.n for _, bl in lists) + cblocks.n}
        eng.xmg_host_free(pin_in)
        eng.xmg_host_free(pin_out)

    # out-of-core: the same contraction with every tensor in a host pagefile
    # and b streamed through two 2 GB HBM regions (reader threads, pinned
    # chunks, side-stream copies overlapping the previous batch)
    ooc = None
    if not args.no_out_of_core and ranks.rank == 0:
        import tempfile
        tmp = tempfile.mkdtemp(prefix="xmg_bench_")
        pal = api.Allocator(eng, os.path.join(tmp, "pagefile"))
        wp = make_workload(eng, pal, args.scale, args.subset)
        eng.check(eng.xmg_set_precision(api.PREC_AUTO))
        eng.check(eng.xmg_set_staging(1, int(2e9)))
        wp.run()
        times = []
        for _ in range(2):
            t0 = time.perf_counter()
            wp.run()
            times.append(time.perf_counter() - t0)
        st = api.last_stats(eng)
        dt = min(times)
        ooc = {"value": flops / dt / 1e12, "unit": "TFLOP/s", "ms_per_step": dt * 1e3,
               "staged_bytes": st.stage_bytes, "stage_gbs": st.stage_bytes / dt / 1e9,
               "batches": st.stage_batches, "region_bytes": int(2e9),
               "device_ms": st.ms_device, "stage_wait_ms": st.ms_stage_wait,
               "plan_ms": st.ms_plan,
               "precision_used": "emu64" if st.precision_used == api.PREC_EMU64 else "fp64",
               "note": "all tensors in a pagefile on the box's disk (page cache warm); "
                       "b streamed in batches, wall clock per xm_contract"}
        eng.check(eng.xmg_set_staging(int(180e9), int(32e9)))
        wp.free()
        pal.destroy()
        os.rmdir(tmp)
        ooc["cfg5_subset"] = cfg5_subset(eng, api, W, args.cfg5_v_blocks,
                                         int(args.cfg5_region_gb * 1e9))

    configs = None if args.no_configs or ranks.rank != 0 else other_configs(
        eng, api, W, None if args.no_cpu_baseline or ranks.world > 1 else cpu_sample_error)

    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)

    # bandwidth-bound operations on b (the largest tensor), timed on the
    # device through the public calls: xm_set (write), xm_add without and
    # with a permutation (read a, read b, write a: the gather-transpose
    # path of unfold/fold), xm_copy (read, write), xm_mul (read a, read b,
    # write a), xm_dot (read both, one scalar back)
    elem = None
    if not args.no_elementwise:
        nbytes = sum(w.b.block_size(blk) for blk in w.b.canonical_blocks()) * 8
        # xm_dot pairs every nonzero block, derivative ones included
        # (the reference's xm.c:472-497 loop)
        nbytes_all = sum(w.b.block_size(blk) for blk in np.ndindex(*w.b.nblocks())
                         if w.b.block_type(blk) != api.ZERO) * 8
        b2 = w.b.structure()
        api.set_all(b2, 0.25)
        elem = {}
        for name, fn, traffic in (
                ("xm_set", lambda: api.set_all(b2, 1.5), nbytes),
                ("xm_add", lambda: api.add(0.5, b2, 0.25, w.b, "cdab", "cdab"), 3 * nbytes),
                ("xm_add_permuted", lambda: api.add(0.5, b2, 0.25, w.b, "cdab", "dcab"), 3 * nbytes),
                ("xm_copy", lambda: api.copy(b2, 1.0, w.b, "cdab", "cdab"), 2 * nbytes),
                ("xm_copy_permuted", lambda: api.copy(b2, 1.0, w.b, "cdab", "dcab"), 2 * nbytes),
                ("xm_mul", lambda: api.mul(b2, w.b, "cdab", "cdab"), 3 * nbytes),
                ("xm_dot", lambda: api.dot(b2, w.b, "cdab", "cdab"), 2 * nbytes_all)):
            fn()
            eng.check(eng.xmg_synchronize())
            eng.check(eng.xmg_timer_start())
            reps = 5
            for _ in range(reps):
                fn()
            ms = eng.xmg_timer_stop() / reps
            gbs = traffic / (ms * 1e-3) / 1e9
            elem[name] = {"ms": ms, "bytes": traffic, "gbs": gbs, "frac_of_hbm": gbs / hbm_peak}
        elem["note"] = ("algorithmic bytes of the canonical blocks of b (%.2f GB) per call "
                        "(xm_dot: of every nonzero block, %.2f GB); device time of the public "
                        "call, host planning included; peak = measured copy bandwidth"
                        % (nbytes / 1e9, nbytes_all / 1e9))
        b2.free()
    tc_peak = peaks.get("bf16_tflops", 1900.0)
    slices = 6
    products = slices * (slices + 1) // 2
    if emu["precision_used"] == api.PREC_EMU64 and emu["gemm_ms"] > 0:
        achieved = flops * products / (emu["gemm_ms"] * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": tc_peak, "unit": "TFLOP/s",
                "frac": achieved / tc_peak,
                "traffic": GEMM_DRAM_BYTES if w.name == "cfg2_ladder_o96_v384_z2" else None,
                "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one emu_gemm "
                                "launch on this workload (ncu, one pass); the slices and c it "
                                "must touch are ~13 GB, the rest is L2 misses on re-read tiles",
                "kernel": "emu_gemm (bf16 slices, tcgen05)",
                "note": "achieved = useful FP64 flops x %d slice products / mean GEMM-kernel time; peak = measured cuBLAS bf16 burst" % products}
    else:
        achieved = flops / (emu["gemm_ms"] * 1e-3) / 1e12 if emu["gemm_ms"] > 0 else None
        roof = {"bound": "fp64", "achieved": achieved, "peak": None, "unit": "TFLOP/s",
                "frac": None, "traffic": None, "kernel": "plain_gemm_kernel<double>"}

    cpu = None
    rel_emu_vs_cpu = None
    if ranks.rank == 0 and ranks.world == 1 and not args.no_cpu_baseline:
        cpu, cpu_out = cpu_baseline(w, flops)
        sub = {k: emu["out"][k] for k in cpu_out}
        rel_emu_vs_cpu = W.rel_frobenius(sub, cpu_out)
        rel_fp64_vs_cpu = W.rel_frobenius({k: fp64["out"][k] for k in cpu_out}, cpu_out)
    value = ranks.world * flops / (emu["ms_per_step"] * 1e-3) / 1e12
    fp64_value = ranks.world * flops / (fp64["ms_per_step"] * 1e-3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": emu["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (emulated: bf16 slices, fp32 exact partials, int64 accumulation)",
        "data": "synthetic (seeded splitmix64 uniform[-1,1]; inputs larger than L2)",
        "config": workload_config(w, flops),
        "fp64_plain": {"value": fp64_value, "ms_per_step": fp64["ms_per_step"],
                       "gemm_ms": fp64["gemm_ms"]},
        "speedup_vs_fp64_plain": value / fp64_value,
        "rel_err": {"emu_vs_gpu_fp64": rel_emu_vs_fp64, "emu_vs_cpu_reference": rel_emu_vs_cpu,
                    "gpu_fp64_vs_cpu_reference": rel_fp64_vs_cpu if cpu else None},
        "precision_used": "emu64" if emu["precision_used"] == api.PREC_EMU64 else "fp64",
        "phases_ms": {"gemm": emu["gemm_ms"], "split": emu["split_ms"]},
        "gemm_work_list": {"policy": emu["gemm_policy"],
                           "note": "autotuned work-list policy of the split-precision GEMM "
                                   "(6: stacked tiles; 0-2: one output block per tile)"},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "out_of_core": ooc,
        "elementwise": elem, "other_configs": configs,
        "gpu_launches": emu["launches"], "clocks": emu["clocks"],
        "setup_s": setup_s,
    }
    if ranks.rank == 0:
        print(json.dumps(line))


def reference_arm(args, ranks):
    """The reference's CPU implementation of the path on the machine's host
    cores: one step = one whole xm_contract over the workload (every
    canonical output block), W untimed steps then K timed ones."""
    if ranks.rank != 0:
        return
    lib, kind = cpu_lib()
    al = api.Allocator(lib)
    w = make_workload(lib, al, args.scale, args.subset)
    flops = sum(block_costs(w))
    nblk = len(w.c.canonical_blocks())
    for _ in range(args.warmup):
        w.run()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        w.run()
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    value = flops / dt / 1e12
    sample = ("%d of %d canonical output blocks per step (the whole xm_contract, %.3e useful "
              "flops); mean %.2f s, best %.2f s per call" % (nblk, nblk, flops, dt, min(times)))
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64 uniform[-1,1]; inputs larger than L2)",
        "config": workload_config(w, flops),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cpu_threads(lib),
                         "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))
    w.free()
    al.destroy()


def main():
    args = parse()
    ranks = Ranks()
    if args.impl == "reference":
        reference_arm(args, ranks)
    else:
        engine_arm(args, ranks)


if __name__ == "__main__":
    main()
