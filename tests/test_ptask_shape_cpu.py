"""Host normalisation of element-wise block tasks (xmg_ptask_shape), the
step between a block pair of xm_add / xm_copy / xm_set / unfold / fold and
the element-wise kernels' schedules.  For random shapes, permutations and
extent-1 dimensions the normalised task must visit exactly the same
(destination offset, source offset) pairs, with the destination's
unit-stride dimension first and the source's unit-stride dimension
second whenever the two differ.  No device is involved."""
import ctypes as C
import itertools

import numpy as np
import pytest


class PTask(C.Structure):
    _fields_ = [("dst", C.c_uint64), ("src", C.c_uint64),
                ("ndim", C.c_int32), ("op", C.c_int32),
                ("size", C.c_int32 * 8),
                ("dst_stride", C.c_int64 * 8), ("src_stride", C.c_int64 * 8),
                ("alpha", C.c_double * 2), ("beta", C.c_double * 2)]


def _pairs(sizes, ds, ss):
    out = []
    for idx in itertools.product(*[range(s) for s in sizes]):
        out.append((sum(i * d for i, d in zip(idx, ds)), sum(i * s for i, s in zip(idx, ss))))
    return sorted(out)


def _canon(dims):
    st, acc = [], 1
    for d in dims:
        st.append(acc)
        acc *= d
    return st


@pytest.fixture(scope="module")
def shape(engine):
    f = engine.dll.xmg_ptask_shape
    f.argtypes = [C.POINTER(PTask), C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                  C.POINTER(C.c_int64)]
    f.restype = None
    return f


def test_normalised_tasks_keep_the_element_mapping(shape):
    rng = np.random.default_rng(11)
    for _ in range(400):
        nd = int(rng.integers(0, 7))
        dims = [int(rng.choice([1, 1, 2, 3, 4, 5, 7])) for _ in range(nd)]
        # destination canonical, source a permuted canonical block (the
        # derivative / permuted-index case), as the block operations build them
        perm = list(rng.permutation(nd))
        sdims = [dims[p] for p in perm]
        sst = _canon(sdims)
        ss = [0] * nd
        for k, p in enumerate(perm):
            ss[p] = sst[k]
        ds = _canon(dims)
        if rng.random() < 0.3:      # a strided destination (row of a larger block)
            ds = [d * 3 for d in ds]
        arr = lambda v: (C.c_int64 * max(1, nd))(*v)
        t = PTask()
        shape(C.byref(t), nd, arr(dims), arr(ds), arr(ss))
        n = t.ndim
        assert 1 <= n <= max(1, nd)
        size = list(t.size[:n])
        tds, tss = list(t.dst_stride[:n]), list(t.src_stride[:n])
        assert all(s >= 1 for s in size)
        assert _pairs(size, tds, tss) == _pairs(dims, ds, ss)
        # dimension 0: the smallest destination stride
        if n > 1:
            rest = tds[2:] if tss[0] != 1 and 1 in tss[1:] else tds[1:]
            assert all(tds[0] <= d for d in rest)
        # the source's unit-stride dimension at position 1 unless it is 0
        if 1 in tss and tss[0] != 1:
            assert tss[1] == 1
