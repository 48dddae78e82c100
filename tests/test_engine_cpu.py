"""Engine checks that need no GPU: the C-ABI library loads and exports every
declared symbol, and its host planner reproduces the reference's block
structure bit for bit (merged pair lists, factors, GEMM shapes, flops),
driven through a pagefile allocator so that no device memory is touched."""
import os
import re
import tempfile

import numpy as np
import pytest

import cases
import helpers as H
from libxm_gb300 import api, workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(xmg?_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    names -= {"xmg_pair_cb"}
    return sorted(names)


def test_exports_every_declared_symbol(engine):
    names = declared_functions()
    assert len(names) > 100
    missing = [n for n in names if not hasattr(engine.dll, n)]
    assert missing == []


@pytest.mark.parametrize("prog", ["test.c", "example.c"])
def test_reference_programs_link_unchanged(engine, prog):
    """The reference's own test driver and example program compile against
    include/ and link against the engine library, unchanged (they run only
    where a GPU is present, and their sources only where the reference
    checkout is)."""
    import shutil
    import subprocess
    import oracle.build as ob
    src = os.path.join(os.path.dirname(ob.REF_SRC), prog)
    if not os.path.exists(src) or shutil.which("gcc") is None:
        pytest.skip("reference sources or gcc not present")
    libdir = os.path.join(ROOT, "libxm_gb300", "lib")
    with tempfile.TemporaryDirectory() as d:
        obj, exe = os.path.join(d, "p.o"), os.path.join(d, "p")
        r = subprocess.run(["gcc", "-std=gnu99", "-I", os.path.join(ROOT, "include"), "-c",
                            src, "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run(["gcc", "-o", exe, obj, "-L", libdir, "-lxmgb",
                            "-Wl,-rpath," + libdir, "-lm"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_exports_reference_test_driver_privates(engine):
    # test.c calls xm_fatal and xm_make_masks (util.h:34-35)
    assert hasattr(engine.dll, "xm_fatal") and hasattr(engine.dll, "xm_make_masks")
    assert api.make_masks(engine, "ijcd", "cdab") == ([2, 3], [0, 1])


def test_engine_blockspace_kat(engine):
    bs = api.BlockSpace(engine, [10, 20, 30, 40, 50, 60, 70, 80]).autosplit()
    assert bs.nblocks() == [1, 1, 1, 2, 2, 2, 3, 3]
    bs.free()
    bs = api.BlockSpace(engine, [30, 31, 32, 33, 34]).autosplit()
    assert bs.block_dims([0] * 5) == [30, 31, 32, 16, 18]
    bs.free()
    bs = api.BlockSpace(engine, [1000]).autosplit()
    o = api.BlockSpace(engine, [1000])
    lib_o = None
    bs.free(); o.free()


@pytest.fixture()
def pagefile(engine):
    d = tempfile.mkdtemp()
    al = api.Allocator(engine, os.path.join(d, "xmpagefile"))
    yield al
    al.destroy()
    os.rmdir(d)


def test_autosplit_matches_oracle(engine, oracle):
    for n in [1, 7, 31, 32, 33, 63, 64, 65, 100, 127, 129, 384, 1000, 1934, 4097]:
        x = api.BlockSpace(engine, [n]).autosplit()
        y = api.BlockSpace(oracle, [n]).autosplit()
        assert x.nblocks() == y.nblocks()
        nb = x.nblocks()[0]
        assert [engine.xm_block_space_get_split(x.h, 0, i) for i in range(nb + 1)] == \
               [oracle.xm_block_space_get_split(y.h, 0, i) for i in range(nb + 1)]
        x.free(); y.free()


def test_tensor_structure_on_pagefile(engine, pagefile):
    a, b, c = cases.make_abc_9(engine, pagefile, api.DOUBLE)
    blocks = c.canonical_blocks()
    assert blocks == sorted(blocks, key=lambda x: x[::-1])  # index 0 fastest
    assert a.block_type((1, 0, 0, 0)) == api.DERIVATIVE
    assert a.block_perm((1, 0, 0, 0)) == [1, 0, 2, 3]
    assert a.block_scalar((1, 0, 0, 0)) == -1
    assert a.data_ptr((1, 0, 0, 0)) == a.data_ptr((0, 1, 0, 0))
    # pagefile round trip (no device involved)
    blk = blocks[3]
    v = np.arange(c.block_size(blk), dtype=np.float64)
    c.write_block(blk, v)
    assert np.array_equal(c.read_block(blk), v)
    for t in (a, b, c):
        t.free()


@pytest.mark.parametrize("ci", range(len(cases.CONTRACT_TESTS)))
def test_pair_structure_matches_oracle(engine, oracle, pagefile, ci):
    make, ia, ib, ic = cases.CONTRACT_TESTS[ci]
    ao = api.Allocator(oracle)
    for dt in H.TYPES:
        a, b, c = make(engine, pagefile, dt)
        mine = H.pair_structure_engine(engine, a, b, c, ia, ib, ic)
        flops = engine.xmg_contract_flops(a.h, b.h, c.h, ia.encode(), ib.encode(), ic.encode())
        for t in (a, b, c):
            t.free()
        x, y, z = make(oracle, ao, dt)
        for t in (x, y, z):
            H.fill_random(t, np.random.default_rng(1))
        ref = H.pair_structure_oracle(oracle, x, y, z, ia, ib, ic)
        for t in (x, y, z):
            t.free()
        assert mine == ref
        mult = 8 if dt in (1, 3) else 2
        assert flops == sum(mult * m * n * k for _, _, m, n, k in ref)


@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_workload_structure_matches_oracle(engine, oracle, pagefile, name):
    """Full-size block structure of the measured ladders, bit-exact."""
    gen = {"cfg1": W.cfg1, "cfg2": W.cfg2}[name]
    oracle.dll.xmo_set_plan_only(1)
    try:
        ws = []
        for lib, al in ((engine, pagefile), (oracle, api.Allocator(oracle))):
            orig_fill = W.fill
            W.fill = lambda *a, **k: None      # structure only: no data
            try:
                ws.append(gen(lib, al))
            finally:
                W.fill = orig_fill
        e, o = ws
        mine = H.pair_structure_engine(engine, e.a, e.b, e.c, e.idxa, e.idxb, e.idxc)
        ref = H.pair_structure_oracle(oracle, o.a, o.b, o.c, o.idxa, o.idxb, o.idxc)
        assert len(mine) > 0 and mine == ref
        flops = engine.xmg_contract_flops(e.a.h, e.b.h, e.c.h, b"ijcd", b"cdab", b"ijab")
        assert flops == sum(2 * m * n * k for _, _, m, n, k in ref)
        if name == "cfg1":
            assert len(e.c.canonical_blocks()) == 60 and len(ref) == 600
            assert flops == 5033164800.0
        for w in ws:
            for t in w.tensors():
                t.free(data=True)
    finally:
        oracle.dll.xmo_set_plan_only(0)


def test_golden_gemm_log_cfg1(engine, pagefile):
    """The engine's cfg1 plan against the reference's recorded GEMM calls."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "workloads.npz"))
    orig = W.fill
    W.fill = lambda *a, **k: None
    try:
        w = W.cfg1(engine, pagefile)
    finally:
        W.fill = orig
    mine = H.pair_structure_engine(engine, w.a, w.b, w.c, w.idxa, w.idxb, w.idxc)
    log = g["cfg1_log"]
    assert sorted((min(m, n), max(m, n), k, z.real) for _, z, m, n, k in mine) == \
        sorted((int(min(r[1], r[2])), int(max(r[1], r[2])), int(r[3]), r[4]) for r in log)
    w.free()


def test_invalid_indices_return_status(engine, pagefile):
    a, b, c = cases.make_abc_1(engine, pagefile, api.DOUBLE)
    st = engine.xmg_contract(api.Scalar.of(1), a.h, b.h, api.Scalar.of(0), c.h, b"ik", b"kj", b"ijx")
    assert st == 1 and b"bad contraction indices" in engine.xmg_last_error()
    st = engine.xmg_contract(api.Scalar.of(1), a.h, b.h, api.Scalar.of(0), c.h, b"ik", b"kj", b"jk")
    assert st == 1
    for t in (a, b, c):
        t.free()


@pytest.mark.parametrize("dims", [[96, 384, 30, 17], [16, 31, 64, 1000], [5, 100, 128, 47]])
def test_autosplit_tiles_opt_in(engine, dims):
    """The opt-in tile-aware autosplit cuts every dimension at multiples of
    the quantum into parts near the target; the default autosplit is left
    as the reference's (its known answers are pinned elsewhere)."""
    bs = api.BlockSpace(engine, dims)
    try:
        engine.check(engine.xmg_block_space_autosplit_tiles(bs.h, 32, 16))
        nb = bs.nblocks()
        for d, n in enumerate(dims):
            sizes = [bs.block_dims([0] * d + [i] + [0] * (len(dims) - d - 1))[d]
                     for i in range(nb[d])]
            assert sum(sizes) == n
            cuts = np.cumsum(sizes)[:-1]
            assert all(c % 16 == 0 for c in cuts)
            if n >= 16:
                assert all(s >= 16 for s in sizes)
                assert max(sizes) <= 2 * 32 + 15
    finally:
        bs.free()
    with pytest.raises(api.XmError):
        engine.check(engine.xmg_block_space_autosplit_tiles(None, 32, 16))


def _work_list(engine, w, policy):
    out = (api.C.c_longlong * 4)()
    engine.check(engine.xmg_work_list_check(w.a.h, w.b.h, w.c.h, w.idxa.encode(),
                                            w.idxb.encode(), w.idxc.encode(), policy, out))
    return list(out)


@pytest.mark.parametrize("name", ["cfg2", "cfg3", "cfg5"])
def test_gemm_work_lists_hold_their_invariants(engine, pagefile, name):
    """The split-precision GEMM's work lists, built on the host for the
    full-size structures: every policy's list passes the checks the kernel's
    addressing relies on (member tiles inside their views and the stage,
    members sharing the other side pair by pair), and the stacked list
    (policy 6) holds stacked items, fewer items than policy 2 and never more
    members than policy 2 has items."""
    gen = {"cfg2": lambda: W.cfg2(engine, pagefile),
           "cfg3": lambda: W.cfg3(engine, pagefile, dtype=api.DOUBLE_COMPLEX),
           "cfg5": lambda: W.cfg5(engine, pagefile, v_blocks=8)}[name]
    orig_fill = W.fill
    W.fill = lambda *a, **k: None      # structure only: no data
    try:
        w = gen()
    finally:
        W.fill = orig_fill
    try:
        lists = {pol: _work_list(engine, w, pol) for pol in (0, 1, 2, 6)}
        for pol, (nitems, nmem, stacked, ok) in lists.items():
            assert ok == 1, (name, pol)
            assert nitems > 0
            if pol != 6:
                assert nmem == nitems and stacked == 0
        n2, n6 = lists[2][0], lists[6]
        if name == "cfg2":
            assert n6[2] > 0 and n6[0] < n2 and n6[1] <= n2
        with pytest.raises(api.XmError):
            _work_list(engine, w, 7)
    finally:
        for t in w.tensors():
            t.free(data=True)


@pytest.mark.parametrize("order", ["output", "file"])
@pytest.mark.parametrize("name,nbatch", [("cfg2", 1), ("cfg2", 4), ("cfg2", 13),
                                         ("cfg3", 5), ("cfg5", 3)])
def test_out_of_core_batch_plans_partition_the_plan(engine, pagefile, name, nbatch, order,
                                                    monkeypatch):
    """The out-of-core path builds the whole plan once and cuts each batch's
    plan from it.  Cut on the host for b's blocks in nbatch runs, and in the
    streamed path's own batches of at most a region's bytes, with b's
    blocks in the output blocks' order or in file order: every merged pair
    lands in exactly one batch, in its output block's order, with its views
    and tables; the flops add up to the whole plan's; every batch's stacked
    work list holds the kernel's invariants; every block lies aligned
    inside its batch's region; no block of c is written back before a batch
    that feeds it; a block larger than the region is refused."""
    monkeypatch.setenv("XMG_STREAM_ORDER", order)
    gen = {"cfg2": lambda: W.cfg2(engine, pagefile),
           "cfg3": lambda: W.cfg3(engine, pagefile, dtype=api.DOUBLE_COMPLEX),
           "cfg5": lambda: W.cfg5(engine, pagefile, v_blocks=8)}[name]
    orig_fill = W.fill
    W.fill = lambda *a, **k: None      # structure only: no data
    try:
        w = gen()
    finally:
        W.fill = orig_fill
    try:
        args = (w.a.h, w.b.h, w.c.h, w.idxa.encode(), w.idxb.encode(), w.idxc.encode())
        out = (api.C.c_longlong * 4)()
        engine.check(engine.xmg_batch_plan_check(*args, nbatch, 0, 6, out))
        batches, npairs, items, ok = list(out)
        assert ok == 1 and batches == nbatch
        whole = _work_list(engine, w, 6)
        assert whole[3] == 1
        pairs = H.pair_structure_engine(engine, w.a, w.b, w.c, w.idxa, w.idxb, w.idxc)
        assert npairs == len(pairs)
        # one batch is the whole plan: the same work list
        if nbatch == 1:
            assert items == whole[0]
        else:
            assert items >= whole[0]
        with pytest.raises(api.XmError):
            engine.check(engine.xmg_batch_plan_check(*args, 0, 0, 6, out))
        sizes = [engine.xm_tensor_get_block_bytes(w.b.h, api.Dim.of(blk))
                 for blk in w.b.canonical_blocks()]
        for parts in (1, nbatch + 1):
            region = sum(sizes) // parts + 256 * len(sizes)
            engine.check(engine.xmg_batch_plan_check(*args, 0, region, 6, out))
            assert out[3] == 1 and out[1] == npairs
            assert out[0] > 1 if parts > 1 else out[0] == 1
        with pytest.raises(api.XmError):
            engine.check(engine.xmg_batch_plan_check(*args, 0, max(sizes) - 1, 6, out))
    finally:
        for t in w.tensors():
            t.free(data=True)


@pytest.mark.parametrize("ci", range(len(cases.CONTRACT_TESTS)))
def test_plan_checks_on_reference_cases(engine, pagefile, ci, monkeypatch):
    """Every contraction case of the reference's test driver, all four
    scalar types: each work-list policy of the split-precision GEMM holds
    the kernel's invariants, and the out-of-core batch plans for b's blocks
    in 1, 2 and 5 runs partition the whole plan (b's blocks in the output
    blocks' order for two of the types, in file order for the others)."""
    make, ia, ib, ic = cases.CONTRACT_TESTS[ci]
    out = (api.C.c_longlong * 4)()
    for dt in H.TYPES:
        monkeypatch.setenv("XMG_STREAM_ORDER", "output" if dt % 2 == 0 else "file")
        a, b, c = make(engine, pagefile, dt)
        try:
            args = (a.h, b.h, c.h, ia.encode(), ib.encode(), ic.encode())
            for pol in (0, 1, 2, 6):
                engine.check(engine.xmg_work_list_check(*args, pol, out))
                assert out[3] == 1, (dt, pol)
            npairs = len(H.pair_structure_engine(engine, a, b, c, ia, ib, ic))
            for nbatch in (1, 2, 5):
                engine.check(engine.xmg_batch_plan_check(*args, nbatch, 0, 6, out))
                assert out[3] == 1 and out[1] == npairs, (dt, nbatch)
        finally:
            for t in (a, b, c):
                t.free()


def _runs(engine, h, sz, dst):
    n = len(h)
    arr = lambda v: (api.C.c_uint64 * max(n, 1))(*v)
    start = (api.C.c_size_t * max(n, 1))()
    q = engine.xmg_copy_runs(arr(h), arr(sz), arr(dst), n, start)
    return list(start[:q])


def test_copy_runs(engine):
    """The staging copies: one per run of blocks that follow one another
    with only alignment padding between, in host memory and in HBM alike;
    equal end-to-end distances alone never merge (two equal-sized blocks
    that trade places between the two sides would be swapped)."""
    # three blocks carved one after another on both sides (256-byte padding)
    assert _runs(engine, [0, 256, 768], [200, 500, 10], [4096, 4352, 4864]) == [0]
    # a block missing from the list between two listed ones: no merge
    assert _runs(engine, [0, 512], [200, 200], [4096, 4608]) == [0, 1]
    # equal-sized blocks in another order on the host side
    # (host: x0 x2 x1, device: x0 x1 x2; list x0, x1): not one copy
    assert _runs(engine, [0, 512], [200, 200], [4096, 4352]) == [0, 1]
    assert _runs(engine, [0, 256, 512], [200, 200, 200], [4096, 4608, 4352]) == [0, 1, 2]
    # a descending host address or a different distance: new runs
    assert _runs(engine, [512, 0], [100, 100], [4096, 4352]) == [0, 1]
    assert _runs(engine, [0, 256], [100, 100], [4096, 4608]) == [0, 1]
    assert _runs(engine, [], [], []) == []


def _stream_batches(engine, sizes, region, host):
    n = len(sizes)
    arr = (api.C.c_uint64 * n)(*sizes)
    bstart = (api.C.c_size_t * (n + 1))()
    nb = engine.xmg_stream_batches(arr, n, int(region), host, bstart)
    return [list(range(bstart[k], bstart[k + 1])) for k in range(nb)]


def test_stream_batch_schedules(engine, monkeypatch):
    """The streamed path's batches of b: a partition of the blocks in
    order, every batch within the region (256-byte aligned blocks); for a
    host-memory b the default tent (sizes grow by XMG_HOST_GROWTH to the
    middle and shrink again, so the first and the last batch are small),
    the geometric shape on request; for a pagefile b about
    XMG_STAGE_BATCHES equal batches; a block beyond the region refused."""
    for k in ("XMG_HOST_SHAPE", "XMG_HOST_BATCHES", "XMG_HOST_GROWTH", "XMG_STAGE_BATCHES"):
        monkeypatch.delenv(k, raising=False)
    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(1 << 20, 8 << 20, 1500)]
    al = [(x + 255) // 256 * 256 for x in sizes]

    def check(b, region):
        assert [i for bb in b for i in bb] == list(range(len(sizes)))
        assert all(sum(al[i] for i in bb) <= region for bb in b)
        return [sum(sizes[i] for i in bb) for bb in b]

    big = 32e9
    got = check(_stream_batches(engine, sizes, big, 1), big)
    assert 8 <= len(got) <= 9
    planned = got[:8]
    mid = max(planned)
    assert mid > 2.5 * planned[0] and mid > 2.5 * planned[7], got
    assert abs(planned[0] - planned[7]) < 0.3 * planned[0], got
    assert planned.index(mid) in (3, 4)

    monkeypatch.setenv("XMG_HOST_SHAPE", "geometric")
    monkeypatch.setenv("XMG_HOST_BATCHES", "6")
    monkeypatch.setenv("XMG_HOST_GROWTH", "1.15")
    got = check(_stream_batches(engine, sizes, big, 1), big)
    assert 6 <= len(got) <= 7
    assert all(got[k + 1] > got[k] for k in range(5)), got

    monkeypatch.setenv("XMG_STAGE_BATCHES", "5")
    got = check(_stream_batches(engine, sizes, big, 0), big)
    assert 5 <= len(got) <= 6
    assert max(got[:5]) < 1.1 * min(got[:5]), got

    # a region below the planned batches caps every batch
    region = 200 << 20
    got = check(_stream_batches(engine, sizes, region, 1), region)
    assert len(got) > 30
    # a block larger than the region
    assert _stream_batches(engine, sizes, 4 << 20, 1) == []


def test_blocks_beyond_int32_offsets_are_refused(engine, pagefile):
    """Offsets inside a block are 32-bit on the device: the planner refuses
    a block with more than 2^31 - 1 elements with an error instead of
    building wrapped offset tables.  Blocks are set with placeholder data
    handles (nothing is allocated or read)."""
    set_raw = engine.dll.xm_tensor_set_canonical_block_raw
    set_raw.argtypes = [api.C.c_void_p, api.Dim, api.C.c_uint64]
    set_raw.restype = None
    big, small = 50000, 8            # 50000^2 = 2.5e9 elements > 2^31 - 1
    for da, db, dc, ia, ib, ic in (([big, big], [big, small], [big, small], "ij", "jk", "ik"),
                                   ([big, small], [small, big], [big, big], "ik", "kj", "ij")):
        spaces = [api.BlockSpace(engine, d) for d in (da, db, dc)]
        ts = [api.Tensor(engine, s, api.DOUBLE, pagefile) for s in spaces]
        for n, t in enumerate(ts):
            set_raw(t.h, api.Dim.of([0, 0]), 4096 * (n + 1))
        f = engine.xmg_contract_flops(ts[0].h, ts[1].h, ts[2].h, ia.encode(), ib.encode(),
                                      ic.encode())
        assert f == -1
        assert "2^31" in engine.xmg_last_error().decode()
        for t in ts:
            t.free(data=False)
        for s in spaces:
            s.free()
