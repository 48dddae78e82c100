"""Shared test helpers: seeded fills and case runners."""
import ctypes as C

import numpy as np

from libxm_gb300 import api

TOL = {api.FLOAT: 1e-4, api.FLOAT_COMPLEX: 1e-4, api.DOUBLE: 1e-8,
       api.DOUBLE_COMPLEX: 1e-8}       # test.c:48-70 (absolute)
TYPES = [api.FLOAT, api.FLOAT_COMPLEX, api.DOUBLE, api.DOUBLE_COMPLEX]
TYPE_NAMES = {0: "float", 1: "cfloat", 2: "double", 3: "cdouble"}


def fill_random(t, rng):
    """drand48() - 0.5 style values (test.c:72-132), from a numpy stream."""
    for blk in t.canonical_blocks():
        n = t.block_size(blk)
        v = rng.random(n) - 0.5
        if t.dtype in (api.FLOAT_COMPLEX, api.DOUBLE_COMPLEX):
            v = v + 1j * (rng.random(n) - 0.5)
        t.write_block(blk, v)


def scalar(rng, dtype):
    if dtype in (api.FLOAT_COMPLEX, api.DOUBLE_COMPLEX):
        return complex(rng.random() - 0.5, rng.random() - 0.5)
    return rng.random() - 0.5


def canon(t):
    return {blk: t.read_block(blk) for blk in t.canonical_blocks()}


def max_abs_diff(x, y):
    assert x.keys() == y.keys()
    m = 0.0
    for k in x:
        if x[k].size:
            m = max(m, float(np.max(np.abs(x[k].astype(np.complex128) - y[k].astype(np.complex128)))))
    return m


def run_contract_case(lib, alloc, case, dtype, seed, alpha, beta, pagefile=None):
    """Build a reference test case on lib, fill it from seed, contract.
    Returns (outputs of c's canonical blocks, tensors)."""
    make, ia, ib, ic = case
    a, b, c = make(lib, alloc, dtype)
    rng = np.random.default_rng(seed)
    fill_random(a, rng)
    fill_random(b, rng)
    fill_random(c, rng)
    api.contract(alpha, a, b, beta, c, ia, ib, ic)
    out = canon(c)
    for t in (a, b, c):
        t.free()
    return out


PAIR_CB = C.CFUNCTYPE(None, C.c_size_t, C.c_double, C.c_double, C.c_long, C.c_long, C.c_long)


def pair_structure_oracle(lib, a, b, c, ia, ib, ic):
    """Merged pair list of the oracle (pair callback during xm_contract)."""
    out = []

    def cb(l, re, im, m, n, k):
        out.append((int(l), complex(re, im), int(m), int(n), int(k)))
    f = PAIR_CB(cb)
    lib.dll.xmo_set_pair_callback.argtypes = [PAIR_CB]
    lib.dll.xmo_set_pair_callback(f)
    api.contract(1.0, a, b, 0.0, c, ia, ib, ic)
    lib.dll.xmo_set_pair_callback(PAIR_CB())
    return sorted(out, key=lambda x: (x[0], x[4], x[2], x[3], x[1].real, x[1].imag))


def pair_structure_engine(lib, a, b, c, ia, ib, ic):
    out = []

    def cb(l, re, im, m, n, k):
        out.append((int(l), complex(re, im), int(m), int(n), int(k)))
    f = PAIR_CB(cb)
    lib.dll.xmg_contract_pairs.argtypes = [C.c_void_p] * 3 + [C.c_char_p] * 3 + [PAIR_CB]
    lib.check(lib.dll.xmg_contract_pairs(a.h, b.h, c.h, ia.encode(), ib.encode(), ic.encode(), f))
    return sorted(out, key=lambda x: (x[0], x[4], x[2], x[3], x[1].real, x[1].imag))


def folded_cotangent(lib, al, dc):
    """W = dC folded onto C's canonical blocks: every canonical block of dc
    times its multiplicity (the sum of scalar^2 over the nonzero blocks
    that share its data), on a tensor whose other blocks are zero."""
    mult = {}
    for blk in np.ndindex(*dc.nblocks()):
        if dc.block_type(blk) != api.ZERO:
            mult[dc.data_ptr(blk)] = mult.get(dc.data_ptr(blk), 0.0) + \
                dc.block_scalar(blk).real ** 2
    wt = api.Tensor(lib, None, dc.dtype, al,
                    handle=lib.xm_tensor_create(lib.xm_tensor_get_block_space(dc.h),
                                                dc.dtype, al.h))
    for blk in dc.canonical_blocks():
        wt.set_canonical(blk)
        wt.write_block(blk, dc.read_block(blk) * mult[dc.data_ptr(blk)])
    return wt


def sampled_gradient(lib, al, t, wt, other, idx_w, idx_o, idx_t, alpha, sample, w_first):
    """The oracle's gradient of L with respect to the sampled canonical
    blocks of t: G = alpha * W * other at every nonzero position of t whose
    data is a sampled block, folded back through each position's
    permutation and scalar onto its canonical block."""
    ptr2canon = {t.data_ptr(blk): blk for blk in t.canonical_blocks()}
    keep = set(sample)
    g = api.Tensor(lib, None, t.dtype, al,
                   handle=lib.xm_tensor_create(lib.xm_tensor_get_block_space(t.h), t.dtype, al.h))
    positions = []
    for blk in np.ndindex(*t.nblocks()):
        if t.block_type(blk) != api.ZERO and ptr2canon[t.data_ptr(blk)] in keep:
            g.set_canonical(blk)
            positions.append(blk)
    if w_first:
        api.contract(alpha, wt, other, 0.0, g, idx_w, idx_o, idx_t)
    else:
        api.contract(alpha, other, wt, 0.0, g, idx_o, idx_w, idx_t)
    cplx = t.dtype in (api.FLOAT_COMPLEX, api.DOUBLE_COMPLEX)
    out = {blk: np.zeros(t.block_size(blk), dtype=np.complex128 if cplx else np.float64)
           for blk in sample}
    for blk in positions:
        q = ptr2canon[t.data_ptr(blk)]
        x = g.read_block(blk).reshape(t.block_dims(blk), order="F")
        y = np.transpose(x, np.argsort(t.block_perm(blk)))
        s = t.block_scalar(blk)
        out[q] += (s if cplx else s.real) * y.ravel(order="F")
    g.free()
    return out
