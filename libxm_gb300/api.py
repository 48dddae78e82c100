"""ctypes binding of the libxm C API (include/xm.h and include/xmg.h).

The same binding drives any library exporting the libxm symbols: the GB300
engine (libxmgb.so) and, in tests only, the CPU oracle and the reference
built from source.  Block data crosses the boundary as host numpy arrays,
exactly as the C API's read/write_block do.
"""
import ctypes as C
import numpy as np

MAX_DIM = 8
FLOAT, FLOAT_COMPLEX, DOUBLE, DOUBLE_COMPLEX = 0, 1, 2, 3
ZERO, CANONICAL, DERIVATIVE = 0, 1, 2
NULL_PTR = (1 << 64) - 1
NP_TYPES = {FLOAT: np.float32, FLOAT_COMPLEX: np.complex64,
            DOUBLE: np.float64, DOUBLE_COMPLEX: np.complex128}
PREC_FP64, PREC_EMU64, PREC_AUTO = 0, 1, 2


class Dim(C.Structure):
    """xm_dim_t (dim.h:33-38)."""
    _fields_ = [("n", C.c_size_t), ("i", C.c_size_t * MAX_DIM)]

    @classmethod
    def of(cls, seq):
        d = cls()
        seq = list(seq)
        if len(seq) > MAX_DIM:
            raise ValueError("too many dimensions")
        d.n = len(seq)
        for k, v in enumerate(seq):
            d.i[k] = int(v)
        return d

    def tolist(self):
        return [int(self.i[k]) for k in range(self.n)]


class Scalar(C.Structure):
    """xm_scalar_t: C99 double complex, passed like a two-double aggregate
    on both x86-64 (SSE, SSE) and AArch64 (HFA)."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]

    @classmethod
    def of(cls, v):
        v = complex(v)
        return cls(v.real, v.imag)

    def value(self):
        return complex(self.re, self.im)


class Stats(C.Structure):
    """xmg_stats_t (include/xmg.h)."""
    _fields_ = [("flops", C.c_double), ("ms_plan", C.c_double),
                ("ms_device", C.c_double), ("ms_split", C.c_double),
                ("ms_gemm", C.c_double), ("n_cblocks", C.c_longlong),
                ("n_pairs", C.c_longlong), ("slice_bytes", C.c_longlong),
                ("precision_used", C.c_int), ("gemm_launches", C.c_int),
                ("stage_bytes", C.c_longlong), ("stage_batches", C.c_int),
                ("gemm_policy", C.c_int), ("ms_stage_wait", C.c_double)]


_P = C.c_void_p
_SIGS = {
    "xm_dim_dot": (C.c_size_t, [C.POINTER(Dim)]),
    "xm_block_space_create": (_P, [Dim]),
    "xm_block_space_clone": (_P, [_P]),
    "xm_block_space_free": (None, [_P]),
    "xm_block_space_split": (None, [_P, C.c_size_t, C.c_size_t]),
    "xm_block_space_autosplit": (None, [_P]),
    "xm_block_space_get_nblocks": (Dim, [_P]),
    "xm_block_space_get_abs_dims": (Dim, [_P]),
    "xm_block_space_get_ndims": (C.c_size_t, [_P]),
    "xm_block_space_get_block_dims": (Dim, [_P, Dim]),
    "xm_block_space_get_split": (C.c_size_t, [_P, C.c_size_t, C.c_size_t]),
    "xm_block_space_get_largest_block_size": (C.c_size_t, [_P]),
    "xm_block_space_eq1": (C.c_int, [_P, C.c_size_t, _P, C.c_size_t]),
    "xm_block_space_eq": (C.c_int, [_P, _P]),
    "xm_allocator_create": (_P, [C.c_char_p]),
    "xm_allocator_destroy": (None, [_P]),
    "xm_allocator_get_path": (C.c_char_p, [_P]),
    "xm_tensor_create": (_P, [_P, C.c_int, _P]),
    "xm_tensor_create_canonical": (_P, [_P, C.c_int, _P]),
    "xm_tensor_create_structure": (_P, [_P, C.c_int, _P]),
    "xm_tensor_free": (None, [_P]),
    "xm_tensor_free_block_data": (None, [_P]),
    "xm_tensor_get_block_space": (_P, [_P]),
    "xm_tensor_get_nblocks": (Dim, [_P]),
    "xm_tensor_get_abs_dims": (Dim, [_P]),
    "xm_tensor_get_scalar_type": (C.c_int, [_P]),
    "xm_tensor_get_block_type": (C.c_int, [_P, Dim]),
    "xm_tensor_get_block_dims": (Dim, [_P, Dim]),
    "xm_tensor_get_block_size": (C.c_size_t, [_P, Dim]),
    "xm_tensor_get_block_bytes": (C.c_size_t, [_P, Dim]),
    "xm_tensor_get_largest_block_size": (C.c_size_t, [_P]),
    "xm_tensor_get_block_data_ptr": (C.c_uint64, [_P, Dim]),
    "xm_tensor_get_block_permutation": (Dim, [_P, Dim]),
    "xm_tensor_get_block_scalar": (Scalar, [_P, Dim]),
    "xm_tensor_get_element": (Scalar, [_P, Dim]),
    "xm_tensor_set_zero_block": (None, [_P, Dim]),
    "xm_tensor_set_canonical_block": (None, [_P, Dim]),
    "xm_tensor_set_derivative_block": (None, [_P, Dim, Dim, Dim, Scalar]),
    "xm_tensor_get_canonical_block_list": (None, [_P, C.POINTER(C.POINTER(Dim)), C.POINTER(C.c_size_t)]),
    "xm_tensor_read_block": (None, [_P, Dim, _P]),
    "xm_tensor_write_block": (None, [_P, Dim, _P]),
    "xm_tensor_unfold_block": (None, [_P, Dim, Dim, Dim, _P, _P, C.c_size_t]),
    "xm_tensor_fold_block": (None, [_P, Dim, Dim, Dim, _P, _P, C.c_size_t]),
    "xm_set": (None, [_P, Scalar]),
    "xm_copy": (None, [_P, Scalar, _P, C.c_char_p, C.c_char_p]),
    "xm_add": (None, [Scalar, _P, Scalar, _P, C.c_char_p, C.c_char_p]),
    "xm_mul": (None, [_P, _P, C.c_char_p, C.c_char_p]),
    "xm_div": (None, [_P, _P, C.c_char_p, C.c_char_p]),
    "xm_dot": (Scalar, [_P, _P, C.c_char_p, C.c_char_p]),
    "xm_contract": (None, [Scalar, _P, _P, Scalar, _P, C.c_char_p, C.c_char_p, C.c_char_p]),
    "xm_make_masks": (None, [C.c_char_p, C.c_char_p, C.POINTER(Dim), C.POINTER(Dim)]),
}
_GB_SIGS = {
    "xmg_last_error": (C.c_char_p, []),
    "xmg_set_precision": (C.c_int, [C.c_int]),
    "xmg_get_precision": (C.c_int, []),
    "xmg_contract": (C.c_int, [Scalar, _P, _P, Scalar, _P, C.c_char_p, C.c_char_p, C.c_char_p]),
    "xmg_add": (C.c_int, [Scalar, _P, Scalar, _P, C.c_char_p, C.c_char_p]),
    "xmg_set": (C.c_int, [_P, Scalar]),
    "xmg_contract_flops": (C.c_double, [_P, _P, _P, C.c_char_p, C.c_char_p, C.c_char_p]),
    "xmg_work_list_check": (C.c_int, [_P, _P, _P, C.c_char_p, C.c_char_p, C.c_char_p,
                                      C.c_int, C.POINTER(C.c_longlong)]),
    "xmg_batch_plan_check": (C.c_int, [_P, _P, _P, C.c_char_p, C.c_char_p, C.c_char_p,
                                       C.c_int, C.c_longlong, C.c_int,
                                       C.POINTER(C.c_longlong)]),
    "xmg_copy_runs": (C.c_size_t, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64), C.c_size_t,
                                   C.POINTER(C.c_size_t)]),
    "xmg_stream_batches": (C.c_size_t, [C.POINTER(C.c_uint64), C.c_size_t, C.c_size_t,
                                        C.c_int, C.POINTER(C.c_size_t)]),
    "xmg_get_last_stats": (C.c_int, [C.POINTER(Stats)]),
    "xmg_synchronize": (C.c_int, []),
    "xmg_plan_cache_clear": (None, []),
    "xmg_adjoint_release": (None, []),
    "xmg_adjoint_plan_check": (C.c_int, [_P, _P, _P, C.c_char_p, C.c_char_p, C.c_char_p,
                                         _P, _P, _P]),
    "xmg_set_staging": (C.c_int, [C.c_size_t, C.c_size_t]),
    "xmg_selftest_bounded_wait": (C.c_int, [C.c_uint]),
    "xmg_block_space_autosplit_tiles": (C.c_int, [_P, C.c_size_t, C.c_size_t]),
    "xm_contract_adjoint": (C.c_int, [Scalar, _P, _P, _P, _P, _P, C.c_char_p, C.c_char_p, C.c_char_p]),
    "xmg_timer_start": (C.c_int, []),
    "xmg_timer_stop": (C.c_double, []),
    "xmg_kernel_launches": (C.c_longlong, []),
    "xmg_host_alloc": (_P, [C.c_size_t]),
    "xmg_host_free": (None, [_P]),
    "xmg_device_memory": (C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "xmg_allocator_create_host": (_P, []),
    "xmg_tensor_write_blocks": (C.c_int, [_P, C.c_size_t, C.POINTER(Dim), C.POINTER(_P)]),
    "xmg_tensor_read_blocks": (C.c_int, [_P, C.c_size_t, C.POINTER(Dim), C.POINTER(_P)]),
}


class XmError(RuntimeError):
    pass


class Lib:
    """A loaded libxm-API shared library."""

    def __init__(self, path, extra=None):
        self.path = path
        self.dll = C.CDLL(path, mode=C.RTLD_LOCAL)
        self.gb = hasattr(self.dll, "xmg_contract")
        sigs = dict(_SIGS)
        if self.gb:
            sigs.update(_GB_SIGS)
        sigs.update(extra or {})
        for name, (res, args) in sigs.items():
            if not hasattr(self.dll, name):
                continue
            f = getattr(self.dll, name)
            f.restype = res
            f.argtypes = args
            setattr(self, name, f)

    def check(self, status):
        if status != 0:
            raise XmError(self.xmg_last_error().decode())
        return status


class BlockSpace:
    def __init__(self, lib, dims):
        self.lib = lib
        self.h = lib.xm_block_space_create(Dim.of(dims))
        if not self.h:
            raise XmError("xm_block_space_create failed")

    def split(self, dim, x):
        self.lib.xm_block_space_split(self.h, dim, x)
        return self

    def autosplit(self):
        self.lib.xm_block_space_autosplit(self.h)
        return self

    def nblocks(self):
        return self.lib.xm_block_space_get_nblocks(self.h).tolist()

    def block_dims(self, blk):
        return self.lib.xm_block_space_get_block_dims(self.h, Dim.of(blk)).tolist()

    def free(self):
        if self.h:
            self.lib.xm_block_space_free(self.h)
            self.h = None


class Allocator:
    def __init__(self, lib, path=None, host=False):
        """GPU memory (path None), a pagefile (path), or, on the engine,
        page-locked host memory (host=True: xmg_allocator_create_host)."""
        self.lib = lib
        if host:
            self.h = lib.xmg_allocator_create_host()
        else:
            self.h = lib.xm_allocator_create(path.encode() if path else None)
        if not self.h:
            raise XmError("allocator creation failed")

    def destroy(self):
        if self.h:
            self.lib.xm_allocator_destroy(self.h)
            self.h = None


class BlockList:
    """The C arrays of a block list call (block indices, host addresses),
    built once for calls that repeat."""

    def __init__(self, blocks, ptrs):
        self.n = len(blocks)
        self.dims = (Dim * max(1, self.n))(*[Dim.of(b) for b in blocks])
        self.bufs = (C.c_void_p * max(1, self.n))(*ptrs)


class Tensor:
    def __init__(self, lib, bs, dtype, alloc, canonical=False, handle=None):
        self.lib = lib
        self.dtype = dtype
        self.alloc = alloc
        if handle is not None:
            self.h = handle
        else:
            fn = lib.xm_tensor_create_canonical if canonical else lib.xm_tensor_create
            self.h = fn(bs.h, dtype, alloc.h)
        self.np = NP_TYPES[dtype]

    def structure(self, dtype=None):
        dt = self.dtype if dtype is None else dtype
        h = self.lib.xm_tensor_create_structure(self.h, dt, self.alloc.h)
        return Tensor(self.lib, None, dt, self.alloc, handle=h)

    def nblocks(self):
        return self.lib.xm_tensor_get_nblocks(self.h).tolist()

    def abs_dims(self):
        return self.lib.xm_tensor_get_abs_dims(self.h).tolist()

    def block_type(self, blk):
        return self.lib.xm_tensor_get_block_type(self.h, Dim.of(blk))

    def block_dims(self, blk):
        return self.lib.xm_tensor_get_block_dims(self.h, Dim.of(blk)).tolist()

    def block_size(self, blk):
        return self.lib.xm_tensor_get_block_size(self.h, Dim.of(blk))

    def block_perm(self, blk):
        return self.lib.xm_tensor_get_block_permutation(self.h, Dim.of(blk)).tolist()

    def block_scalar(self, blk):
        return self.lib.xm_tensor_get_block_scalar(self.h, Dim.of(blk)).value()

    def data_ptr(self, blk):
        return self.lib.xm_tensor_get_block_data_ptr(self.h, Dim.of(blk))

    def set_canonical(self, blk):
        self.lib.xm_tensor_set_canonical_block(self.h, Dim.of(blk))

    def set_derivative(self, blk, src, perm, scalar):
        self.lib.xm_tensor_set_derivative_block(self.h, Dim.of(blk), Dim.of(src),
                                                Dim.of(perm), Scalar.of(scalar))

    def canonical_blocks(self):
        p = C.POINTER(Dim)()
        n = C.c_size_t()
        self.lib.xm_tensor_get_canonical_block_list(self.h, C.byref(p), C.byref(n))
        out = [tuple(p[k].tolist()) for k in range(n.value)]
        if n.value:
            C.CDLL(None).free(C.cast(p, C.c_void_p))
        return out

    def write_block(self, blk, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=self.np).ravel(order="F"))
        if a.size != self.block_size(blk):
            raise ValueError("block size mismatch")
        self.lib.xm_tensor_write_block(self.h, Dim.of(blk), a.ctypes.data)

    def read_block(self, blk):
        """Raw canonical data of the block (for a derivative block: of its
        source) as an array of shape block_dims(source) in Fortran order."""
        n = self.block_size(blk)
        a = np.empty(n, dtype=self.np)
        self.lib.xm_tensor_read_block(self.h, Dim.of(blk), a.ctypes.data)
        return a

    def write_blocks(self, blocks, ptrs=None):
        """xmg_tensor_write_blocks: blocks[i] from the host address ptrs[i]
        (or a prepared BlockList)."""
        bl = blocks if isinstance(blocks, BlockList) else BlockList(blocks, ptrs)
        self.lib.check(self.lib.xmg_tensor_write_blocks(self.h, bl.n, bl.dims, bl.bufs))

    def read_blocks(self, blocks, ptrs=None):
        """xmg_tensor_read_blocks: blocks[i] into the host address ptrs[i]
        (or a prepared BlockList)."""
        bl = blocks if isinstance(blocks, BlockList) else BlockList(blocks, ptrs)
        self.lib.check(self.lib.xmg_tensor_read_blocks(self.h, bl.n, bl.dims, bl.bufs))

    def get_element(self, idx):
        return self.lib.xm_tensor_get_element(self.h, Dim.of(idx)).value()

    def free(self, data=True):
        if self.h:
            if data:
                self.lib.xm_tensor_free_block_data(self.h)
            self.lib.xm_tensor_free(self.h)
            self.h = None


def _b(s):
    return s.encode() if isinstance(s, str) else s


def contract(alpha, a, b, beta, c, ia, ib, ic):
    lib = c.lib
    if lib.gb:
        lib.check(lib.xmg_contract(Scalar.of(alpha), a.h, b.h, Scalar.of(beta), c.h,
                                   _b(ia), _b(ib), _b(ic)))
    else:
        lib.xm_contract(Scalar.of(alpha), a.h, b.h, Scalar.of(beta), c.h, _b(ia), _b(ib), _b(ic))


def add(alpha, a, beta, b, ia, ib):
    lib = a.lib
    if lib.gb:
        lib.check(lib.xmg_add(Scalar.of(alpha), a.h, Scalar.of(beta), b.h, _b(ia), _b(ib)))
    else:
        lib.xm_add(Scalar.of(alpha), a.h, Scalar.of(beta), b.h, _b(ia), _b(ib))


def set_all(a, x):
    lib = a.lib
    if lib.gb:
        lib.check(lib.xmg_set(a.h, Scalar.of(x)))
    else:
        lib.xm_set(a.h, Scalar.of(x))


def copy(a, s, b, ia, ib):
    a.lib.xm_copy(a.h, Scalar.of(s), b.h, _b(ia), _b(ib))


def mul(a, b, ia, ib):
    a.lib.xm_mul(a.h, b.h, _b(ia), _b(ib))


def div(a, b, ia, ib):
    a.lib.xm_div(a.h, b.h, _b(ia), _b(ib))


def dot(a, b, ia, ib):
    return a.lib.xm_dot(a.h, b.h, _b(ia), _b(ib)).value()


def last_stats(lib):
    s = Stats()
    lib.check(lib.xmg_get_last_stats(C.byref(s)))
    return s


def make_masks(lib, s1, s2):
    m1, m2 = Dim(), Dim()
    lib.xm_make_masks(_b(s1), _b(s2), C.byref(m1), C.byref(m2))
    return m1.tolist(), m2.tolist()
