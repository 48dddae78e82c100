"""Error behaviour against the reference library compiled from its own
sources: for each invalid call of the reference's validation in
xm_contract (contract.c:237-280) and in xm_add / xm_copy / xm_mul /
xm_div / xm_dot (xm.c:70-95, 165-190, 257-282, 340-365, 422-446) and in
the tensor layer's block setters, reads and writes (tensor.c:255-366) both
libraries print the same `libxm: ...` line and exit with status 1.  Each
call runs in a child process (the public API exits on error,
util.c:24-35); validation precedes any device use, so no GPU is
involved."""
import os
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import os, sys
sys.path.insert(0, {root!r})
from libxm_gb300 import api
lib = api.Lib({path!r})
d = {tmp!r}
al = api.Allocator(lib, os.path.join(d, "pf"))
al2 = api.Allocator(lib, os.path.join(d, "pf2"))

def space(dims, cuts):
    bs = api.BlockSpace(lib, dims)
    for k, c in enumerate(cuts):
        if c:
            bs.split(k, c)
    return bs

def tensor(dims, cuts, dtype=api.DOUBLE, alloc=al):
    return api.Tensor(lib, space(dims, cuts), dtype, alloc)

case = {case!r}
a = tensor([6, 8], [3, 4], api.FLOAT if case == "type" else api.DOUBLE)
b = tensor([8, 5], [5 if case == "ab" else 4, 2], alloc=al2 if case == "alloc" else al)
c = tensor([6, 5], [2 if case == "ac" else 3, 3 if case == "bc" else 2])
idx = {{"length": ("ik", "kj", "ijj"),
       "letters": ("ik", "kj", "ix")}}.get(case, ("ik", "kj", "ij"))
sys.stderr.flush()
lib.xm_contract(api.Scalar.of(1), a.h, b.h, api.Scalar.of(0), c.h,
                idx[0].encode(), idx[1].encode(), idx[2].encode())
print("returned")
'''

CASES = ["length", "letters", "type", "alloc", "ab", "ac", "bc"]


def _run(path, case):
    # the child exits through the error path, so its pagefiles go with the
    # directory
    with tempfile.TemporaryDirectory() as tmp:
        r = subprocess.run([sys.executable, "-c",
                            CHILD.format(root=ROOT, path=path, case=case, tmp=tmp)],
                           capture_output=True, text=True, timeout=120)
    lines = [l for l in r.stderr.splitlines() if l.startswith("libxm:")]
    return r.returncode, lines


@pytest.mark.parametrize("case", CASES)
def test_contract_errors_match_reference(engine, reference, case):
    mine = _run(engine.path, case)
    ref = _run(reference.path, case)
    assert ref[0] == 1 and ref[1], ref
    assert mine == ref


PAIR_CHILD = r'''
import os, sys
sys.path.insert(0, {root!r})
from libxm_gb300 import api
lib = api.Lib({path!r})
d = {tmp!r}
al = api.Allocator(lib, os.path.join(d, "pf"))
al2 = api.Allocator(lib, os.path.join(d, "pf2"))

def tensor(dims, cuts, dtype=api.DOUBLE, alloc=al):
    bs = api.BlockSpace(lib, dims)
    for k, c in enumerate(cuts):
        if c:
            bs.split(k, c)
    return api.Tensor(lib, bs, dtype, alloc)

fn, case = {fn!r}, {case!r}
a = tensor([6, 8], [3, 4])
b = tensor([8 if case == "ab" else 6, 6 if case == "ab" else 8],
           [4, 3] if case == "ab" else [2 if case == "blocks" else 3, 4],
           api.FLOAT if case == "type" else api.DOUBLE,
           al2 if case == "alloc" else al)
ia, ib = {{"length": ("ij", "i"), "letters": ("ij", "ix"), "ab": ("ij", "ji")}}.get(
    case, ("ij", "ij"))
one = api.Scalar.of(1)
if fn == "xm_add":
    lib.xm_add(one, a.h, one, b.h, ia.encode(), ib.encode())
elif fn == "xm_copy":
    lib.xm_copy(a.h, one, b.h, ia.encode(), ib.encode())
elif fn == "xm_dot":
    lib.xm_dot(a.h, b.h, ia.encode(), ib.encode())
else:
    getattr(lib, fn)(a.h, b.h, ia.encode(), ib.encode())
print("returned")
'''

PAIR_CASES = ["length", "letters", "type", "alloc", "blocks"]


@pytest.mark.parametrize("fn", ["xm_add", "xm_copy", "xm_mul", "xm_div", "xm_dot"])
@pytest.mark.parametrize("case", PAIR_CASES)
def test_elementwise_errors_match_reference(engine, reference, fn, case):
    if fn == "xm_copy" and case == "type":
        pytest.skip("xm_copy takes tensors of different scalar types "
                    "(xm.c:70-95 checks none); the copy itself needs a device")
    def run(path):
        with tempfile.TemporaryDirectory() as tmp:
            r = subprocess.run([sys.executable, "-c", PAIR_CHILD.format(
                root=ROOT, path=path, tmp=tmp, fn=fn, case=case)],
                capture_output=True, text=True, timeout=120)
        return r.returncode, [l for l in r.stderr.splitlines() if l.startswith("libxm:")]
    mine, ref = run(engine.path), run(reference.path)
    assert ref[0] == 1 and ref[1], ref
    assert mine == ref


TENSOR_CHILD = r'''
import os, sys
import numpy as np
sys.path.insert(0, {root!r})
from libxm_gb300 import api
lib = api.Lib({path!r})
al = api.Allocator(lib, os.path.join({tmp!r}, "pf"))
bs = api.BlockSpace(lib, [6, 6])
bs.split(0, 3)
bs.split(1, 3)
t = api.Tensor(lib, bs, api.DOUBLE, al)
case = {case!r}
t.set_canonical((0, 1))
if case == "canonical_twice":
    t.set_canonical((0, 1))
elif case == "derivative_on_nonzero":
    t.set_derivative((0, 1), (0, 1), [1, 0], -1.0)
elif case == "derivative_of_zero":
    t.set_derivative((1, 0), (1, 1), [1, 0], -1.0)
elif case == "bad_permutation":
    t.set_derivative((1, 0), (0, 1), [0, 0], -1.0)
elif case == "read_zero":
    t.read_block((1, 1))
elif case == "write_derivative":
    t.set_derivative((1, 0), (0, 1), [1, 0], -1.0)
    t.write_block((1, 0), np.zeros(9))
print("returned")
'''

TENSOR_CASES = ["canonical_twice", "derivative_on_nonzero", "derivative_of_zero",
                "bad_permutation", "read_zero", "write_derivative"]


@pytest.mark.parametrize("case", TENSOR_CASES)
def test_tensor_errors_match_reference(engine, reference, case):
    """Block setters and block reads/writes (tensor.c:255-366)."""
    def run(path):
        with tempfile.TemporaryDirectory() as tmp:
            r = subprocess.run([sys.executable, "-c", TENSOR_CHILD.format(
                root=ROOT, path=path, tmp=tmp, case=case)],
                capture_output=True, text=True, timeout=120)
        return r.returncode, [l for l in r.stderr.splitlines() if l.startswith("libxm:")]
    mine, ref = run(engine.path), run(reference.path)
    assert ref[0] == 1 and ref[1], ref
    assert mine == ref
