/*
 * Block spaces for libxm-gb300 (host metadata; no device work).
 *
 * Each dimension keeps a sorted array of split points splits[0..nblocks]
 * with splits[0] = 0 and splits[nblocks] = extent (blockspace.c:25-51).
 * Splitting is an idempotent sorted insert (blockspace.c:117-139) and the
 * automatic split reproduces the reference's even-split rule targeting 32
 * elements per block (blockspace.c:141-163) so that block structures are
 * bit-identical with the reference.
 */
#include "xmg_host.h"

#define AUTOSPLIT_TARGET 32	/* blockspace.c:23 */

struct xm_block_space {
	xm_dim_t dims, nblocks;
	size_t *splits[XM_MAX_DIM];
};

xm_block_space_t *
xm_block_space_create(xm_dim_t dims)
{
	xm_block_space_t *bs;
	size_t d;

	if (dims.n == 0 || dims.n > XM_MAX_DIM)
		xm_fatal("%s: bad number of dimensions", __func__);
	if ((bs = calloc(1, sizeof *bs)) == NULL)
		return NULL;
	bs->dims = dims;
	bs->nblocks = xm_dim_same(dims.n, 1);
	for (d = 0; d < dims.n; d++) {
		if ((bs->splits[d] = malloc(2 * sizeof(size_t))) == NULL) {
			xm_block_space_free(bs);
			return NULL;
		}
		bs->splits[d][0] = 0;
		bs->splits[d][1] = dims.i[d];
	}
	return bs;
}

xm_block_space_t *
xm_block_space_clone(const xm_block_space_t *src)
{
	xm_dim_t id = xm_dim_identity_permutation(src->dims.n);
	return xm_block_space_permute_clone(src, id);
}

xm_block_space_t *
xm_block_space_permute_clone(const xm_block_space_t *src, xm_dim_t perm)
{
	xm_block_space_t *bs;
	size_t d, to, n;

	if ((bs = calloc(1, sizeof *bs)) == NULL)
		return NULL;
	bs->dims = xm_dim_permute(&src->dims, &perm);
	bs->nblocks = xm_dim_permute(&src->nblocks, &perm);
	for (d = 0; d < src->dims.n; d++) {
		to = perm.i[d];
		n = src->nblocks.i[d] + 1;
		if ((bs->splits[to] = malloc(n * sizeof(size_t))) == NULL) {
			xm_block_space_free(bs);
			return NULL;
		}
		memcpy(bs->splits[to], src->splits[d], n * sizeof(size_t));
	}
	return bs;
}

size_t xm_block_space_get_ndims(const xm_block_space_t *bs) { return bs->dims.n; }
xm_dim_t xm_block_space_get_abs_dims(const xm_block_space_t *bs) { return bs->dims; }
xm_dim_t xm_block_space_get_nblocks(const xm_block_space_t *bs) { return bs->nblocks; }

void
xm_block_space_split(xm_block_space_t *bs, size_t dim, size_t x)
{
	size_t pos, nb, *grown;

	if (dim >= bs->dims.n || x > bs->dims.i[dim])
		xm_fatal("%s: split point out of range", __func__);
	nb = bs->nblocks.i[dim];
	/* first split point >= x */
	for (pos = 0; pos <= nb && bs->splits[dim][pos] < x; pos++)
		;
	if (pos <= nb && bs->splits[dim][pos] == x)
		return;
	if ((grown = realloc(bs->splits[dim], (nb + 2) * sizeof(size_t))) == NULL)
		return;
	bs->splits[dim] = grown;
	memmove(grown + pos + 1, grown + pos, (nb + 1 - pos) * sizeof(size_t));
	grown[pos] = x;
	bs->nblocks.i[dim] = nb + 1;
}

void
xm_block_space_autosplit(xm_block_space_t *bs)
{
	size_t d, left, nparts, p, sz, at;

	for (d = 0; d < bs->dims.n; d++) {
		left = bs->dims.i[d];
		nparts = (left + AUTOSPLIT_TARGET - 1) / AUTOSPLIT_TARGET;
		at = 0;
		for (p = 0; p + 1 < nparts; p++) {
			sz = left / (nparts - p);
			/* odd sizes are nudged to even: up when below the
			 * target, down otherwise */
			if (sz > 1 && (sz & 1))
				sz = sz < AUTOSPLIT_TARGET ? sz + 1 : sz - 1;
			left -= sz;
			at += sz;
			xm_block_space_split(bs, d, at);
		}
	}
}

/*
 * Opt-in tile-aware variant (no counterpart in the reference; the default
 * autosplit above stays bit-identical to it): every dimension is cut into
 * about dim / target parts whose sizes are whole multiples of `quantum`,
 * spread as evenly as the quanta allow, the last part also taking the
 * remainder below one quantum.  With quantum 16 the contraction's tile
 * widths (multiples of 16 rows) and 128-row M tiles waste less padding.
 */
int
xmg_block_space_autosplit_tiles(xm_block_space_t *bs, size_t target,
    size_t quantum)
{
	size_t d, nq, parts, p, at, q;

	if (bs == NULL || target == 0 || quantum == 0 || quantum > target)
		return xmg_seterr(XMG_EINVAL, "xmg_block_space_autosplit_tiles: "
		    "invalid argument");
	for (d = 0; d < bs->dims.n; d++) {
		nq = bs->dims.i[d] / quantum;
		parts = (nq * quantum + target / 2) / target;
		if (parts < 1)
			parts = 1;
		if (parts > nq)
			parts = nq > 0 ? nq : 1;
		at = 0;
		for (p = 0; p + 1 < parts; p++) {
			q = nq / parts + (p < nq % parts ? 1 : 0);
			at += q * quantum;
			xm_block_space_split(bs, d, at);
		}
	}
	return XMG_OK;
}

size_t
xm_block_space_get_split(xm_block_space_t *bs, size_t dim, size_t i)
{
	if (dim >= bs->dims.n || i > bs->nblocks.i[dim])
		xm_fatal("%s: index out of range", __func__);
	return bs->splits[dim][i];
}

xm_dim_t
xm_block_space_get_block_dims(const xm_block_space_t *bs, xm_dim_t blkidx)
{
	xm_dim_t r = xm_dim_zero(bs->dims.n);
	size_t d;

	for (d = 0; d < bs->dims.n; d++)
		r.i[d] = bs->splits[d][blkidx.i[d] + 1] - bs->splits[d][blkidx.i[d]];
	return r;
}

size_t
xm_block_space_get_block_size(const xm_block_space_t *bs, xm_dim_t blkidx)
{
	xm_dim_t dims = xm_block_space_get_block_dims(bs, blkidx);
	return xm_dim_dot(&dims);
}

size_t
xm_block_space_get_largest_block_size(const xm_block_space_t *bs)
{
	size_t d, b, w, widest, prod = 1;

	for (d = 0; d < bs->dims.n; d++) {
		widest = 0;
		for (b = 0; b < bs->nblocks.i[d]; b++) {
			w = bs->splits[d][b + 1] - bs->splits[d][b];
			if (w > widest)
				widest = w;
		}
		prod *= widest;
	}
	return prod;
}

void
xm_block_space_decompose_index(const xm_block_space_t *bs, xm_dim_t idx,
    xm_dim_t *blkidx, xm_dim_t *elidx)
{
	size_t d, b;

	*blkidx = xm_dim_zero(bs->dims.n);
	*elidx = xm_dim_zero(bs->dims.n);
	for (d = 0; d < bs->dims.n; d++) {
		for (b = 0; b < bs->nblocks.i[d]; b++) {
			if (idx.i[d] < bs->splits[d][b + 1]) {
				blkidx->i[d] = b;
				elidx->i[d] = idx.i[d] - bs->splits[d][b];
				break;
			}
		}
	}
}

int
xm_block_space_eq1(const xm_block_space_t *bsa, size_t dima,
    const xm_block_space_t *bsb, size_t dimb)
{
	size_t n;

	if (bsa->nblocks.i[dima] != bsb->nblocks.i[dimb])
		return 0;
	n = bsa->nblocks.i[dima] + 1;
	return memcmp(bsa->splits[dima], bsb->splits[dimb],
	    n * sizeof(size_t)) == 0;
}

int
xm_block_space_eq(const xm_block_space_t *bsa, const xm_block_space_t *bsb)
{
	size_t d;

	if (bsa->dims.n != bsb->dims.n)
		return 0;
	for (d = 0; d < bsa->dims.n; d++)
		if (!xm_block_space_eq1(bsa, d, bsb, d))
			return 0;
	return 1;
}

void
xm_block_space_free(xm_block_space_t *bs)
{
	size_t d;

	if (bs == NULL)
		return;
	for (d = 0; d < XM_MAX_DIM; d++)
		free(bs->splits[d]);
	free(bs);
}
