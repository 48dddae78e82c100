"""Host layers checked against the reference library compiled from its own
sources (skipped where its checkout is absent).  The pagefile allocator
(alloc.c:40-145, 252-300): the same data handles as the reference's own
allocator for the same sequence of allocations and releases (first-fit
page runs, file growth, handle = page offset | pages << 32), and the bytes
written through one handle read back unchanged while every other live
handle is written too.  The tensor layer (tensor.c:26-336): the reference
test driver's tensors have the same blocks, permutations, scalars and
data handles.  No device memory is involved."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

PAGE = 512 * 1024


def _bind(lib):
    d = lib.dll
    d.xm_allocator_allocate.argtypes = [C.c_void_p, C.c_size_t]
    d.xm_allocator_allocate.restype = C.c_uint64
    d.xm_allocator_deallocate.argtypes = [C.c_void_p, C.c_uint64]
    d.xm_allocator_deallocate.restype = None
    for f in (d.xm_allocator_read, d.xm_allocator_write):
        f.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t]
        f.restype = None
    return d


def _sequence(seed, n):
    """Seeded allocate / release operations: sizes from a byte to a few
    pages, page multiples and near misses included."""
    rng = np.random.default_rng(seed)
    ops, live = [], 0
    for _ in range(n):
        if live and rng.random() < 0.35:
            ops.append(("free", int(rng.integers(0, live))))
            live -= 1
        else:
            kind = rng.integers(0, 4)
            if kind == 0:
                size = int(rng.integers(1, 4096))
            elif kind == 1:
                size = PAGE * int(rng.integers(1, 5))
            elif kind == 2:
                size = PAGE * int(rng.integers(1, 4)) + int(rng.integers(-8, 9))
            else:
                size = int(rng.integers(1, 6 * PAGE))
            ops.append(("alloc", max(1, size)))
            live += 1
    return ops


def _run(dll, path, ops):
    a = dll.xm_allocator_create(path.encode())
    assert a
    handles, live = [], []
    for op, x in ops:
        if op == "alloc":
            h = dll.xm_allocator_allocate(a, x)
            handles.append(h)
            live.append((h, x))
        else:
            h, _ = live.pop(x)
            dll.xm_allocator_deallocate(a, h)
    return a, handles, live


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_pagefile_handles_match_reference(engine, reference, seed):
    ops = _sequence(seed, 300)
    d = tempfile.mkdtemp()
    ed, rd = _bind(engine), _bind(reference)
    ea, eh, elive = _run(ed, os.path.join(d, "engine"), ops)
    ra, rh, _ = _run(rd, os.path.join(d, "reference"), ops)
    try:
        assert eh == rh
        # every live block keeps its own bytes
        rng = np.random.default_rng(seed + 100)
        data = [rng.integers(0, 256, size=n, dtype=np.uint8) for _, n in elive]
        for (h, n), v in zip(elive, data):
            ed.xm_allocator_write(ea, h, v.ctypes.data, n)
        for (h, n), v in zip(elive, data):
            back = np.empty(n, dtype=np.uint8)
            ed.xm_allocator_read(ea, h, back.ctypes.data, n)
            assert np.array_equal(back, v)
    finally:
        ed.xm_allocator_destroy(ea)
        rd.xm_allocator_destroy(ra)
        os.rmdir(d)


def _describe(t):
    """Everything the tensor layer exposes about a tensor's blocks."""
    out = {"canonical": t.canonical_blocks()}
    nb = t.nblocks()
    blocks = []
    for idx in np.ndindex(*nb):
        typ = t.block_type(idx)
        row = (idx, typ, tuple(t.block_dims(idx)))
        if typ != 0:      # XM_BLOCK_TYPE_ZERO
            row += (tuple(t.block_perm(idx)), complex(t.block_scalar(idx)), t.data_ptr(idx))
        blocks.append(row)
    out["blocks"] = blocks
    return out


@pytest.mark.parametrize("ci", range(46))
def test_tensor_layer_matches_reference(engine, reference, ci):
    """The reference test driver's tensors built through both libraries on
    pagefile allocators: canonical block lists, block types, dimensions,
    permutations, scalars and data handles are identical."""
    import cases
    from libxm_gb300 import api
    make = cases.CONTRACT_TESTS[ci][0]
    d = tempfile.mkdtemp()
    ea = api.Allocator(engine, os.path.join(d, "engine"))
    ra = api.Allocator(reference, os.path.join(d, "reference"))
    try:
        for dt in (api.FLOAT, api.FLOAT_COMPLEX, api.DOUBLE, api.DOUBLE_COMPLEX):
            et, rt = make(engine, ea, dt), make(reference, ra, dt)
            try:
                for x, y in zip(et, rt):
                    assert _describe(x) == _describe(y), (ci, dt)
            finally:
                for t in et + rt:
                    t.free()
    finally:
        ea.destroy()
        ra.destroy()
        os.rmdir(d)
