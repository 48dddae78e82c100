"""Seeded synthetic block-tensor workloads built through the libxm API.

The five contraction workloads measured by this project (ladder, uneven
Z2^3-sparse ladder, permuted ring term, ladder adjoint, out-of-core
production ladder) are generated here, identically for every library that
exports the libxm API.  Values are uniform in [-1, 1] from a splitmix64
stream keyed by (tensor seed, linear block index); canonical blocks that
map onto themselves under a symmetry are projected onto the symmetric
subspace after generation (the "antisymmetrised diagonal blocks").
"""
import numpy as np

from . import api

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)

# symmetry groups as (permutation, factor); block index map b'[k] = b[perm[k]]
LADDER_ANTISYM = [((0, 1, 2, 3), 1.0), ((1, 0, 2, 3), -1.0),
                  ((0, 1, 3, 2), -1.0), ((1, 0, 3, 2), 1.0)]
PAIR_SYM = [((0, 1, 2, 3), 1.0), ((2, 3, 0, 1), 1.0)]
NO_SYM = [((0, 1, 2, 3), 1.0)]


def splitmix64(seed, n):
    """n consecutive splitmix64 outputs after state = seed."""
    with np.errstate(over="ignore"):
        x = np.uint64(seed) + GAMMA * np.arange(1, n + 1, dtype=np.uint64)
        x = (x ^ (x >> np.uint64(30))) * M1
        x = (x ^ (x >> np.uint64(27))) * M2
        x = x ^ (x >> np.uint64(31))
    return x


def uniform(seed, n):
    """n values uniform in [-1, 1) from the splitmix64 stream of seed."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -52) - 1.0


def block_seed(tseed, lin):
    return int(splitmix64((int(tseed) * 0x100000001B3 + int(lin)) & (2**64 - 1), 1)[0])


def uneven_sizes(total, nblk, lo, hi, seed):
    """Seeded block sizes in [lo, hi] summing to total."""
    r = splitmix64(seed, 4 * nblk * nblk + 16)
    sizes = [total // nblk] * nblk
    for k in range(total - sum(sizes)):
        sizes[k] += 1
    p = 0
    for _ in range(4 * nblk):
        i = int(r[p] % nblk); j = int(r[p + 1] % nblk)
        d = int(r[p + 2] % 9)
        p += 3
        if i == j:
            continue
        d = min(d, sizes[i] - lo, hi - sizes[j])
        if d > 0:
            sizes[i] -= d
            sizes[j] += d
    assert sum(sizes) == total and min(sizes) >= lo and max(sizes) <= hi
    return sizes


def labels(n, seed):
    return [int(v % 8) for v in splitmix64(seed, n)]


def make_space(lib, sizes_per_dim):
    dims = [sum(s) for s in sizes_per_dim]
    bs = api.BlockSpace(lib, dims)
    for d, sizes in enumerate(sizes_per_dim):
        x = 0
        for s in sizes[:-1]:
            x += s
            bs.split(d, x)
    return bs


def symmetric_tensor(lib, alloc, bs, dtype, group, allowed=None):
    """Canonical/derivative structure like the reference's test builders:
    visit block indices with the last position fastest; an unassigned,
    allowed block becomes canonical and its images under the group become
    derivative blocks (when still unassigned)."""
    t = api.Tensor(lib, bs, dtype, alloc)
    nb = bs.nblocks()
    for blk in np.ndindex(*nb):
        if t.block_type(blk) != api.ZERO:
            continue
        if allowed is not None and not allowed(blk):
            continue
        t.set_canonical(blk)
        for perm, s in group[1:]:
            b2 = tuple(blk[perm[k]] for k in range(len(blk)))
            if t.block_type(b2) == api.ZERO:
                t.set_derivative(b2, blk, perm, s)
    return t


def _block_values(blk, dims, nb, seed, cplx, group):
    n = int(np.prod(dims))
    lin = int(np.ravel_multi_index(blk, nb, order="F"))
    s0 = block_seed(seed, lin)
    v = uniform(s0, n)
    if cplx:
        v = v + 1j * uniform(s0 ^ 0x5555, n)
    x = v.reshape(dims, order="F")
    stab = [(p, s) for p, s in group
            if tuple(blk[p[k]] for k in range(len(blk))) == tuple(blk)]
    if len(stab) > 1:
        x = sum(s * np.transpose(x, p) for p, s in stab) / len(stab)
    return x


def fill(t, seed, group=NO_SYM, threads=1):
    """Write seeded uniform[-1,1] data into every canonical block; project
    blocks that are their own image under the group.  threads > 1
    generates the blocks' values on that many threads, a bounded window of
    blocks at a time (the same values; the writes stay on this thread)."""
    nb = t.nblocks()
    cplx = t.dtype in (api.FLOAT_COMPLEX, api.DOUBLE_COMPLEX)
    blocks = [(blk, t.block_dims(blk)) for blk in t.canonical_blocks()]
    if threads <= 1:
        for blk, dims in blocks:
            t.write_block(blk, _block_values(blk, dims, nb, seed, cplx, group))
        return
    from concurrent.futures import ThreadPoolExecutor
    win = 4 * threads
    with ThreadPoolExecutor(threads) as ex:
        for i in range(0, len(blocks), win):
            part = blocks[i:i + win]
            vals = ex.map(lambda bd: _block_values(bd[0], bd[1], nb, seed, cplx, group), part)
            for (blk, _), x in zip(part, vals):
                t.write_block(blk, x)


class Workload:
    """Three tensors and a contraction c = alpha * a * b + beta * c."""

    def __init__(self, name, a, b, c, idx, alpha, beta, groups, seeds, extra=None):
        self.name = name
        self.a, self.b, self.c = a, b, c
        self.idxa, self.idxb, self.idxc = idx
        self.alpha, self.beta = alpha, beta
        self.groups = groups
        self.seeds = seeds
        self.extra = extra or {}

    def tensors(self):
        return [self.a, self.b, self.c]

    def run(self):
        api.contract(self.alpha, self.a, self.b, self.beta, self.c,
                     self.idxa, self.idxb, self.idxc)

    def free(self):
        for t in self.tensors():
            t.free()


def ladder(lib, alloc, o_sizes, v_sizes, seed=1, dtype=api.DOUBLE, z2=None,
           with_c_fill=False, fill_data=True, threads=1):
    """C(i,j,a,b) = sum_{c,d} A(i,j,c,d) B(c,d,a,b) with i<->j, c<->d, a<->b
    antisymmetry (factor -1 derivative blocks) and optional Z2^3 labels.
    fill_data=False leaves the block data unwritten (for a copy of another
    library's tensors of the same structure)."""
    bso = [o_sizes, o_sizes, v_sizes, v_sizes]
    bsv = [v_sizes] * 4
    sa, sb = make_space(lib, bso), make_space(lib, bsv)
    alw_a = alw_b = None
    if z2 is not None:
        lo, lv = z2
        alw_a = lambda b: (lo[b[0]] ^ lo[b[1]] ^ lv[b[2]] ^ lv[b[3]]) == 0
        alw_b = lambda b: (lv[b[0]] ^ lv[b[1]] ^ lv[b[2]] ^ lv[b[3]]) == 0
    a = symmetric_tensor(lib, alloc, sa, dtype, LADDER_ANTISYM, alw_a)
    b = symmetric_tensor(lib, alloc, sb, dtype, LADDER_ANTISYM, alw_b)
    c = symmetric_tensor(lib, alloc, sa, dtype, LADDER_ANTISYM, alw_a)
    sa.free(); sb.free()
    if fill_data:
        fill(a, seed * 3 + 1, LADDER_ANTISYM, threads)
        fill(b, seed * 3 + 2, LADDER_ANTISYM, threads)
    if with_c_fill and fill_data:
        fill(c, seed * 3 + 3, LADDER_ANTISYM, threads)
    return Workload("ladder", a, b, c, ("ijcd", "cdab", "ijab"), 1.0, 0.0,
                    (LADDER_ANTISYM, LADDER_ANTISYM, LADDER_ANTISYM),
                    (seed * 3 + 1, seed * 3 + 2, seed * 3 + 3))


def cfg1(lib, alloc, seed=1):
    """Plain FP64 ladder, CPU-runnable: o = 24 as 3 x 8, v = 64 as 4 x 16."""
    w = ladder(lib, alloc, [8] * 3, [16] * 4, seed)
    w.name = "cfg1_ladder_o24_v64"
    return w


def cfg2_shape(seed=2):
    o = uneven_sizes(96, 6, 8, 24, seed * 7 + 11)
    v = uneven_sizes(384, 12, 16, 48, seed * 7 + 12)
    lo = labels(6, seed * 7 + 13)
    lv = labels(12, seed * 7 + 14)
    return o, v, lo, lv


def cfg2(lib, alloc, seed=2, scale=1, o_blocks=None, v_blocks=None, fill_data=True):
    """Uneven-block Z2^3-sparse FP64 ladder: o = 96 in 6 blocks of 8..24,
    v = 384 in 12 blocks of 16..48.  scale > 1 shrinks every block size by
    that factor (structure preserved) for quick parity runs; o_blocks /
    v_blocks keep only the first blocks of each space (block sizes
    unchanged), a smaller case with the full-size tiles for profiling."""
    o, v, lo, lv = cfg2_shape(seed)
    if scale > 1:
        o = [max(1, x // scale) for x in o]
        v = [max(1, x // scale) for x in v]
    if o_blocks:
        o, lo = o[:o_blocks], lo[:o_blocks]
    if v_blocks:
        v, lv = v[:v_blocks], lv[:v_blocks]
    w = ladder(lib, alloc, o, v, seed, z2=(lo, lv), fill_data=fill_data)
    if o_blocks or v_blocks:
        w.name = "cfg2_subset_o%d_v%d" % (len(o), len(v))
    else:
        w.name = "cfg2_ladder_o96_v384_z2" if scale == 1 else "cfg2_ladder_scaled_%d" % scale
    w.extra = {"o_sizes": o, "v_sizes": v, "o_labels": lo, "v_labels": lv}
    return w


def split_sizes(lib, dim, tiles=None):
    """Block sizes of one dimension of length dim as the library's
    autosplit cuts it: xm_block_space_autosplit (tiles None, the
    reference's rule) or, on the engine, xmg_block_space_autosplit_tiles
    with tiles = (target, quantum)."""
    bs = api.BlockSpace(lib, [dim])
    if tiles is None:
        bs.autosplit()
    else:
        lib.check(lib.xmg_block_space_autosplit_tiles(bs.h, tiles[0], tiles[1]))
    n = bs.nblocks()[0]
    cuts = [lib.xm_block_space_get_split(bs.h, 0, i) for i in range(n + 1)]
    bs.free()
    return [cuts[i + 1] - cuts[i] for i in range(n)]


def autosplit_ladder(lib, alloc, o_sizes, v_sizes, seed=4):
    """A Z2^3-sparse ladder on given block sizes (labels from the uneven
    ladder's seeds, one per block), for comparing block splittings of the
    same dimensions."""
    _, _, lo, lv = cfg2_shape(seed)
    lo = (lo * 4)[:len(o_sizes)]
    lv = (lv * 4)[:len(v_sizes)]
    w = ladder(lib, alloc, o_sizes, v_sizes, seed, z2=(lo, lv))
    w.name = "ladder_o%d_v%d_z2" % (sum(o_sizes), sum(v_sizes))
    return w


def cfg5_shape(seed=5):
    o = [16] * 8
    v = uneven_sizes(1024, 32, 24, 40, seed * 7 + 12)
    lo = labels(8, seed * 7 + 13)
    lv = labels(32, seed * 7 + 14)
    return o, v, lo, lv


def cfg5_bytes(v_blocks=None, seed=5):
    """Canonical bytes of (a, b, c) of the production ladder on its first
    v_blocks v blocks, from the shape alone: (anti)symmetric pairs keep
    one block each (first index <= second), the Z2^3 labels keep the
    blocks whose four labels xor to 0."""
    o, v, lo, lv = cfg5_shape(seed)
    if v_blocks:
        v, lv = v[:v_blocks], lv[:v_blocks]

    def pairs(sz, lab):
        # {label: sum of s_p * s_q over canonical pairs p <= q with that label}
        out = {}
        for p in range(len(sz)):
            for q in range(p, len(sz)):
                k = lab[p] ^ lab[q]
                out[k] = out.get(k, 0) + sz[p] * sz[q]
        return out

    po, pv = pairs(o, lo), pairs(v, lv)
    oo = sum(po[k] * po[k] for k in po)
    ov = sum(po[k] * pv.get(k, 0) for k in po)
    vv = sum(pv[k] * pv[k] for k in pv)
    return 8 * ov, 8 * vv, 8 * ov


def cfg5(lib, alloc, seed=5, scale=1, v_blocks=None, threads=1):
    """Production ladder: o = 128 in 8 blocks of 16, v = 1024 in 32 blocks
    of 24..40, Z2^3 labels.  The full b (vvvv) holds ~275 GB of canonical
    data; v_blocks keeps the first v blocks only (block sizes and labels
    unchanged) and scale > 1 shrinks every block size by that factor."""
    o, v, lo, lv = cfg5_shape(seed)
    if scale > 1:
        o = [max(1, x // scale) for x in o]
        v = [max(1, x // scale) for x in v]
    if v_blocks:
        v, lv = v[:v_blocks], lv[:v_blocks]
    w = ladder(lib, alloc, o, v, seed, z2=(lo, lv), threads=threads)
    w.name = "cfg5_ladder_o%d_v%d_z2%s" % (sum(o), sum(v), "" if scale == 1 else "_scaled_%d" % scale)
    w.extra = {"o_sizes": o, "v_sizes": v, "o_labels": lo, "v_labels": lv}
    return w


def cfg3(lib, alloc, dtype=api.FLOAT, seed=3, o_blk=16, v_blk=32, no=4, nv=8,
         fill_data=True):
    """Ring term C(i,a,j,b) += sum_{k,c} A(k,i,c,a) B(j,k,b,c), beta = 1,
    C prefilled; (i,a) <-> (j,b) pair symmetry (+1) on C only, A and B
    fully canonical."""
    o, v = [o_blk] * no, [v_blk] * nv
    sab = make_space(lib, [o, o, v, v])
    sc = make_space(lib, [o, v, o, v])
    a = api.Tensor(lib, sab, dtype, alloc, canonical=True)
    b = api.Tensor(lib, sab, dtype, alloc, canonical=True)
    c = symmetric_tensor(lib, alloc, sc, dtype, PAIR_SYM)
    sab.free(); sc.free()
    if fill_data:
        fill(a, seed * 3 + 1)
        fill(b, seed * 3 + 2)
        fill(c, seed * 3 + 3, PAIR_SYM)
    return Workload("cfg3_ring_o64_v256", a, b, c, ("kica", "jkbc", "iajb"),
                    1.0, 1.0, (NO_SYM, NO_SYM, PAIR_SYM),
                    (seed * 3 + 1, seed * 3 + 2, seed * 3 + 3))


def copy_data(src, dst):
    """Write every canonical block of src into dst (same structure; the
    values converted to dst's scalar type)."""
    for blk in src.canonical_blocks():
        dst.write_block(blk, src.read_block(blk).astype(dst.np))


def sample_blocks(blocks, n, seed=0):
    """A deterministic, seeded sample of n of the given blocks (all of
    them when there are no more than n), in their original order."""
    if len(blocks) <= n:
        return list(blocks)
    rng = np.random.default_rng(seed)
    return [blocks[i] for i in sorted(rng.choice(len(blocks), n, replace=False))]


def contract_sample(w, chosen, c0=None):
    """Run w's contraction for the chosen canonical output blocks only:
    the other canonical blocks of a fresh output structure are set to zero
    blocks, so that a library that computes every canonical block does only
    the chosen ones' work.  c0 gives the chosen blocks' initial values (for
    beta != 0).  Returns {block: data} of the chosen blocks."""
    c = w.c.structure()
    keep = set(chosen)
    for blk in w.c.canonical_blocks():
        if blk not in keep:
            c.lib.xm_tensor_set_zero_block(c.h, api.Dim.of(blk))
    if c0 is not None:
        for blk in chosen:
            c.write_block(blk, c0[blk])
    api.contract(w.alpha, w.a, w.b, w.beta, c, w.idxa, w.idxb, w.idxc)
    out = {blk: c.read_block(blk) for blk in chosen}
    c.free()
    return out


def read_canonical(t):
    """{block index: raw canonical data} of a tensor."""
    return {blk: t.read_block(blk) for blk in t.canonical_blocks()}


def rel_frobenius(x, ref):
    """sqrt(sum |x - ref|^2) / sqrt(sum |ref|^2) over matching blocks."""
    num = den = 0.0
    for k, r in ref.items():
        d = x[k].astype(np.complex128) - r.astype(np.complex128)
        num += float(np.vdot(d, d).real)
        den += float(np.vdot(r.astype(np.complex128), r.astype(np.complex128)).real)
    return (num ** 0.5) / (den ** 0.5 if den > 0 else 1.0)
