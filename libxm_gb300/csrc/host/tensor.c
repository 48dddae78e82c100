/*
 * Block tensors for libxm-gb300.
 *
 * The block table mirrors the reference's struct xm_block
 * (tensor.c:26-39): zero blocks carry nothing, canonical blocks an
 * allocator handle, derivative blocks a permutation, a scalar and the
 * linear index of their canonical source.  All validation rules and the
 * index-0-fastest canonical block order are kept so that block lists,
 * canonical mapping and sparsity are identical to the reference's.
 *
 * Block data lives in HBM (or a pagefile); unfold/fold run as CUDA kernels.
 */
#include "xmg_host.h"

size_t
xmg_tensor_block_linear(const xm_tensor_t *t, xm_dim_t blkidx)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs);

	if (blkidx.n != nb.n || !xm_dim_less(&blkidx, &nb))
		xm_fatal("%s: block index out of range", __func__);
	return xm_dim_offset(&blkidx, &nb);
}

struct xmg_block *
xmg_tensor_block(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return &t->blocks[xmg_tensor_block_linear(t, blkidx)];
}

void
xmg_canon_strides(const xm_dim_t *dims, int64_t s[XM_MAX_DIM])
{
	size_t k;
	int64_t acc = 1;

	for (k = 0; k < dims->n; k++) {
		s[k] = acc;
		acc *= (int64_t)dims->i[k];
	}
}

void
xmg_tensor_block_strides(const xm_tensor_t *t, xm_dim_t blkidx,
    int64_t strides[XM_MAX_DIM])
{
	struct xmg_block *b = xmg_tensor_block(t, blkidx);
	xm_dim_t dims, cdims;
	int64_t cs[XM_MAX_DIM];
	size_t k;

	/* The source block's dims are this block's dims permuted
	 * (tensor.c:300-304); element el of this block is element
	 * permute(el, perm) of the source (tensor.c:167-171). */
	dims = xm_block_space_get_block_dims(t->bs, blkidx);
	cdims = xm_dim_permute(&dims, &b->perm);
	xmg_canon_strides(&cdims, cs);
	for (k = 0; k < dims.n; k++)
		strides[k] = cs[b->perm.i[k]];
}

/* Every block-table change draws a fresh generation number, so a cached
 * contraction plan keyed on (tensor address, generation) can never match a
 * tensor that changed or a new tensor at a recycled address. */
static uint64_t g_gen;

void
xmg_tensor_touch(xm_tensor_t *t)
{
	t->gen = __atomic_add_fetch(&g_gen, 1, __ATOMIC_RELAXED);
}

xm_tensor_t *
xm_tensor_create(const xm_block_space_t *bs, xm_scalar_type_t type,
    xm_allocator_t *allocator)
{
	xm_tensor_t *t;
	xm_dim_t nb;
	size_t i;

	if (bs == NULL || allocator == NULL)
		xm_fatal("%s: invalid argument", __func__);
	if (!xm_scalar_check_type(type))
		xm_fatal("%s: unexpected scalar type", __func__);
	if ((t = calloc(1, sizeof *t)) == NULL ||
	    (t->bs = xm_block_space_clone(bs)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	t->type = type;
	t->allocator = allocator;
	nb = xm_block_space_get_nblocks(bs);
	t->nblocks_total = xm_dim_dot(&nb);
	if ((t->blocks = calloc(t->nblocks_total, sizeof *t->blocks)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < t->nblocks_total; i++) {
		t->blocks[i].type = XM_BLOCK_TYPE_ZERO;
		t->blocks[i].perm = xm_dim_identity_permutation(nb.n);
		t->blocks[i].scalar = 0;
		t->blocks[i].data = XM_NULL_PTR;
	}
	xmg_tensor_touch(t);
	return t;
}

xm_tensor_t *
xm_tensor_create_canonical(const xm_block_space_t *bs, xm_scalar_type_t type,
    xm_allocator_t *allocator)
{
	xm_tensor_t *t = xm_tensor_create(bs, type, allocator);
	xm_dim_t nb = xm_block_space_get_nblocks(bs), idx = xm_dim_zero(nb.n);

	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb))
		xm_tensor_set_canonical_block(t, idx);
	return t;
}

xm_tensor_t *
xm_tensor_create_structure(const xm_tensor_t *src, xm_scalar_type_t type,
    xm_allocator_t *allocator)
{
	xm_tensor_t *t;
	xm_dim_t nb, idx;
	size_t i;

	t = xm_tensor_create(src->bs, type,
	    allocator ? allocator : src->allocator);
	nb = xm_block_space_get_nblocks(src->bs);
	idx = xm_dim_zero(nb.n);
	for (i = 0; i < t->nblocks_total; i++, xm_dim_inc(&idx, &nb)) {
		t->blocks[i] = src->blocks[i];
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL) {
			t->blocks[i].type = XM_BLOCK_TYPE_ZERO;
			xm_tensor_set_canonical_block(t, idx);
		}
	}
	xmg_tensor_touch(t);
	return t;
}

const xm_block_space_t *xm_tensor_get_block_space(const xm_tensor_t *t) { return t->bs; }
xm_scalar_type_t xm_tensor_get_scalar_type(const xm_tensor_t *t) { return t->type; }
xm_allocator_t *xm_tensor_get_allocator(const xm_tensor_t *t) { return t->allocator; }
xm_dim_t xm_tensor_get_abs_dims(const xm_tensor_t *t) { return xm_block_space_get_abs_dims(t->bs); }
xm_dim_t xm_tensor_get_nblocks(const xm_tensor_t *t) { return xm_block_space_get_nblocks(t->bs); }

xm_block_type_t
xm_tensor_get_block_type(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xmg_tensor_block(t, blkidx)->type;
}

xm_dim_t
xm_tensor_get_block_dims(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xm_block_space_get_block_dims(t->bs, blkidx);
}

size_t
xm_tensor_get_block_size(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xm_block_space_get_block_size(t->bs, blkidx);
}

size_t
xm_tensor_get_block_bytes(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xm_tensor_get_block_size(t, blkidx) * xm_scalar_sizeof(t->type);
}

size_t
xm_tensor_get_largest_block_size(const xm_tensor_t *t)
{
	return xm_block_space_get_largest_block_size(t->bs);
}

size_t
xm_tensor_get_largest_block_bytes(const xm_tensor_t *t)
{
	return xm_tensor_get_largest_block_size(t) * xm_scalar_sizeof(t->type);
}

uint64_t
xm_tensor_get_block_data_ptr(const xm_tensor_t *t, xm_dim_t blkidx)
{
	struct xmg_block *b = xmg_tensor_block(t, blkidx);

	if (b->type == XM_BLOCK_TYPE_CANONICAL)
		return b->data;
	if (b->type == XM_BLOCK_TYPE_DERIVATIVE)
		return t->blocks[b->data].data;
	return XM_NULL_PTR;
}

xm_dim_t
xm_tensor_get_block_permutation(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xmg_tensor_block(t, blkidx)->perm;
}

xm_scalar_t
xm_tensor_get_block_scalar(const xm_tensor_t *t, xm_dim_t blkidx)
{
	return xmg_tensor_block(t, blkidx)->scalar;
}

xm_scalar_t
xm_tensor_get_element(const xm_tensor_t *t, xm_dim_t idx)
{
	xm_dim_t blkidx, elidx;
	struct xmg_block *b;
	int64_t st[XM_MAX_DIM], off = 0;
	size_t k, esz = xm_scalar_sizeof(t->type);
	double buf[2] = {0, 0};
	xm_scalar_t v;

	xm_block_space_decompose_index(t->bs, idx, &blkidx, &elidx);
	b = xmg_tensor_block(t, blkidx);
	if (b->type == XM_BLOCK_TYPE_ZERO)
		return 0;
	xmg_tensor_block_strides(t, blkidx, st);
	for (k = 0; k < elidx.n; k++)
		off += (int64_t)elidx.i[k] * st[k];
	xmg_die_on(xmg_alloc_read_range(t->allocator,
	    xm_tensor_get_block_data_ptr(t, blkidx), (size_t)off * esz,
	    buf, esz));
	v = xm_scalar_get_element(buf, 0, t->type);
	return xm_scalar_mul(b->scalar, v, t->type);
}

void
xm_tensor_set_zero_block(xm_tensor_t *t, xm_dim_t blkidx)
{
	struct xmg_block *b = xmg_tensor_block(t, blkidx);

	b->type = XM_BLOCK_TYPE_ZERO;
	b->perm = xm_dim_identity_permutation(blkidx.n);
	b->scalar = 0;
	b->data = XM_NULL_PTR;
	xmg_tensor_touch(t);
}

void
xm_tensor_set_canonical_block(xm_tensor_t *t, xm_dim_t blkidx)
{
	uint64_t h;

	if (xm_tensor_get_block_type(t, blkidx) != XM_BLOCK_TYPE_ZERO)
		xm_fatal("%s: block must be zero", __func__);
	h = xm_allocator_allocate(t->allocator,
	    xm_tensor_get_block_bytes(t, blkidx));
	if (h == XM_NULL_PTR)
		xm_fatal("%s: unable to allocate block data", __func__);
	xm_tensor_set_canonical_block_raw(t, blkidx, h);
}

void
xm_tensor_set_canonical_block_raw(xm_tensor_t *t, xm_dim_t blkidx,
    uint64_t data_ptr)
{
	struct xmg_block *b;

	if (data_ptr == XM_NULL_PTR)
		xm_fatal("%s: unexpected null data pointer", __func__);
	if (xm_tensor_get_block_type(t, blkidx) != XM_BLOCK_TYPE_ZERO)
		xm_fatal("%s: block must be zero", __func__);
	b = xmg_tensor_block(t, blkidx);
	b->type = XM_BLOCK_TYPE_CANONICAL;
	b->perm = xm_dim_identity_permutation(blkidx.n);
	b->scalar = 1;
	b->data = data_ptr;
	xmg_tensor_touch(t);
}

void
xm_tensor_set_derivative_block(xm_tensor_t *t, xm_dim_t blkidx,
    xm_dim_t source_blkidx, xm_dim_t permutation, xm_scalar_t scalar)
{
	struct xmg_block *b;
	xm_dim_t d1, d2;

	if (xm_tensor_get_block_type(t, blkidx) != XM_BLOCK_TYPE_ZERO)
		xm_fatal("%s: block must be zero", __func__);
	if (xm_tensor_get_block_type(t, source_blkidx) !=
	    XM_BLOCK_TYPE_CANONICAL)
		xm_fatal("%s: derivative blocks must have canonical source "
		    "blocks", __func__);
	d1 = xm_block_space_get_block_dims(t->bs, blkidx);
	d1 = xm_dim_permute(&d1, &permutation);
	d2 = xm_block_space_get_block_dims(t->bs, source_blkidx);
	if (xm_dim_ne(&d1, &d2))
		xm_fatal("%s: invalid block permutation", __func__);
	b = xmg_tensor_block(t, blkidx);
	b->type = XM_BLOCK_TYPE_DERIVATIVE;
	b->perm = permutation;
	b->scalar = scalar;
	b->data = xmg_tensor_block_linear(t, source_blkidx);
	xmg_tensor_touch(t);
}

void
xm_tensor_get_canonical_block_list(const xm_tensor_t *t, xm_dim_t **blklist,
    size_t *nblklist)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs), idx, *list = NULL;
	size_t i, n = 0;

	for (i = 0; i < t->nblocks_total; i++)
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL)
			n++;
	if (n > 0 && (list = malloc(n * sizeof *list)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	n = 0;
	idx = xm_dim_zero(nb.n);
	for (i = 0; i < t->nblocks_total; i++, xm_dim_inc(&idx, &nb))
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL)
			list[n++] = idx;
	*blklist = list;
	*nblklist = n;
}

void
xm_tensor_read_block(const xm_tensor_t *t, xm_dim_t blkidx, void *buf)
{
	if (xm_tensor_get_block_type(t, blkidx) == XM_BLOCK_TYPE_ZERO)
		xm_fatal("%s: cannot read data from zero-blocks", __func__);
	xm_allocator_read(t->allocator, xm_tensor_get_block_data_ptr(t, blkidx),
	    buf, xm_tensor_get_block_bytes(t, blkidx));
}

void
xm_tensor_write_block(xm_tensor_t *t, xm_dim_t blkidx, const void *buf)
{
	if (xm_tensor_get_block_type(t, blkidx) != XM_BLOCK_TYPE_CANONICAL)
		xm_fatal("%s: can only write to canonical blocks", __func__);
	xm_allocator_write(t->allocator, xm_tensor_get_block_data_ptr(t, blkidx),
	    buf, xm_tensor_get_block_bytes(t, blkidx));
}

/* index check without exiting (the xmg_ list calls return a status) */
static int
block_of(const xm_tensor_t *t, xm_dim_t blkidx, const char *fn,
    struct xmg_block **out)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs);

	if (blkidx.n != nb.n || !xm_dim_less(&blkidx, &nb))
		return xmg_seterr(XMG_EINVAL, "%s: block index out of range", fn);
	*out = &t->blocks[xm_dim_offset(&blkidx, &nb)];
	return XMG_OK;
}

/*
 * n blocks in one call.  For tensors in GPU memory every block's copy is
 * queued on the engine stream (one cudaMemcpyAsync each) and the call
 * waits once, at the end; the caller's buffers may be reused on return,
 * as after xm_tensor_write_block.  Pagefile and host-memory tensors write
 * block by block.
 */
int
xmg_tensor_write_blocks(xm_tensor_t *t, size_t n, const xm_dim_t *blks,
    const void *const *bufs)
{
	const char *fn = "xmg_tensor_write_blocks";
	struct xmg_block *b;
	size_t i;
	int st = XMG_OK, s2;

	if (t == NULL || (n > 0 && (blks == NULL || bufs == NULL)))
		return xmg_seterr(XMG_EINVAL, "%s: NULL argument", fn);
	for (i = 0; i < n; i++) {
		if ((st = block_of(t, blks[i], fn, &b)) != XMG_OK)
			return st;
		if (b->type != XM_BLOCK_TYPE_CANONICAL)
			return xmg_seterr(XMG_EINVAL, "%s: can only write to "
			    "canonical blocks", fn);
		if (bufs[i] == NULL)
			return xmg_seterr(XMG_EINVAL, "%s: NULL buffer", fn);
	}
	for (i = 0; st == XMG_OK && i < n; i++) {
		b = xmg_tensor_block(t, blks[i]);
		size_t bytes = xm_tensor_get_block_bytes(t, blks[i]);
		st = xmg_alloc_is_device(t->allocator) ?
		    xmgd_h2d_async(b->data, bufs[i], bytes) :
		    xmg_alloc_io(t->allocator, b->data, (void *)bufs[i], bytes, 1);
	}
	if (xmg_alloc_is_device(t->allocator) && n > 0 &&
	    (s2 = xmgd_sync()) != XMG_OK && st == XMG_OK)
		st = s2;
	return st;
}

/* n nonzero blocks into n host buffers, the copies queued and waited for
 * once as in xmg_tensor_write_blocks (derivative blocks read their
 * source's data, as xm_tensor_read_block does) */
int
xmg_tensor_read_blocks(const xm_tensor_t *t, size_t n, const xm_dim_t *blks,
    void *const *bufs)
{
	const char *fn = "xmg_tensor_read_blocks";
	struct xmg_block *b;
	size_t i;
	int st = XMG_OK, s2;

	if (t == NULL || (n > 0 && (blks == NULL || bufs == NULL)))
		return xmg_seterr(XMG_EINVAL, "%s: NULL argument", fn);
	for (i = 0; i < n; i++) {
		if ((st = block_of(t, blks[i], fn, &b)) != XMG_OK)
			return st;
		if (b->type == XM_BLOCK_TYPE_ZERO)
			return xmg_seterr(XMG_EINVAL, "%s: cannot read data from "
			    "zero-blocks", fn);
		if (bufs[i] == NULL)
			return xmg_seterr(XMG_EINVAL, "%s: NULL buffer", fn);
	}
	for (i = 0; st == XMG_OK && i < n; i++) {
		uint64_t h = xm_tensor_get_block_data_ptr(t, blks[i]);
		size_t bytes = xm_tensor_get_block_bytes(t, blks[i]);
		st = xmg_alloc_is_device(t->allocator) ?
		    xmgd_d2h_async(bufs[i], h, bytes) :
		    xmg_alloc_io(t->allocator, h, bufs[i], bytes, 0);
	}
	if (xmg_alloc_is_device(t->allocator) && n > 0 &&
	    (s2 = xmgd_sync()) != XMG_OK && st == XMG_OK)
		st = s2;
	return st;
}

/*
 * Iteration space of an unfold: mask_i positions (first fastest) then
 * mask_j positions; matrix side offset i + stride * j; block side offset
 * through the block's (permuted) strides.
 */
static void
unfold_space(const xm_tensor_t *t, xm_dim_t blkidx, xm_dim_t mask_i,
    xm_dim_t mask_j, size_t stride, int64_t *size, int64_t *mat_stride,
    int64_t *blk_stride, int *ndim, size_t *span)
{
	xm_dim_t dims = xm_block_space_get_block_dims(t->bs, blkidx);
	int64_t bs[XM_MAX_DIM], acc;
	size_t k, ni, nj;
	int n = 0;

	xmg_tensor_block_strides(t, blkidx, bs);
	acc = 1;
	for (k = 0; k < mask_i.n; k++, n++) {
		size[n] = (int64_t)dims.i[mask_i.i[k]];
		mat_stride[n] = acc;
		blk_stride[n] = bs[mask_i.i[k]];
		acc *= size[n];
	}
	ni = (size_t)acc;
	acc = (int64_t)stride;
	nj = 1;
	for (k = 0; k < mask_j.n; k++, n++) {
		size[n] = (int64_t)dims.i[mask_j.i[k]];
		mat_stride[n] = acc;
		blk_stride[n] = bs[mask_j.i[k]];
		acc *= size[n];
		nj *= (size_t)size[n];
	}
	*ndim = n;
	*span = (nj - 1) * stride + ni;	/* matrix elements touched */
}

/* Run one unfold (dir = 0) or fold (dir = 1) on the GPU.  Host buffers are
 * staged through engine scratch; device buffers are used in place. */
static void
unfold_fold(const xm_tensor_t *t, xm_dim_t blkidx, xm_dim_t mask_i,
    xm_dim_t mask_j, const void *from, void *to, size_t stride, int dir,
    const char *fn)
{
	int64_t size[XM_MAX_DIM], ms[XM_MAX_DIM], bs[XM_MAX_DIM];
	size_t span, blkbytes, esz = xm_scalar_sizeof(t->type), matbytes;
	uint64_t dfrom, dto;
	int ndim, dev_from, dev_to;
	xmg_ptask_list_t l = {0};
	xmgd_ptask_t *task;

	if (from == NULL || to == NULL || from == to)
		xm_fatal("%s: invalid argument", fn);
	if (mask_i.n + mask_j.n != blkidx.n)
		xm_fatal("%s: invalid mask dimensions", fn);
	if (dir == 1 && xm_tensor_get_block_type(t, blkidx) !=
	    XM_BLOCK_TYPE_CANONICAL)
		xm_fatal("%s: can only fold canonical blocks", fn);
	unfold_space(t, blkidx, mask_i, mask_j, stride, size, ms, bs, &ndim,
	    &span);
	blkbytes = xm_tensor_get_block_size(t, blkidx) * esz;
	matbytes = span * esz;
	xmg_die_on(xmgd_init());
	dev_from = xmgd_is_device_ptr(from);
	dev_to = xmgd_is_device_ptr(to);
	if (dev_from)
		dfrom = (uint64_t)(uintptr_t)from;
	else {
		xmg_die_on(xmgd_scratch(0, dir ? matbytes : blkbytes, &dfrom));
		xmg_die_on(xmgd_h2d(dfrom, from, dir ? matbytes : blkbytes));
	}
	if (dev_to)
		dto = (uint64_t)(uintptr_t)to;
	else {
		xmg_die_on(xmgd_scratch(1, dir ? blkbytes : matbytes, &dto));
		/* elements of the destination outside the written pattern
		 * must come back unchanged */
		xmg_die_on(xmgd_h2d(dto, to, dir ? blkbytes : matbytes));
	}
	task = xmg_ptask_push(&l);
	task->op = XMGD_OP_COPY;
	task->alpha[0] = 1;
	if (dir == 0) {		/* matrix <- block */
		task->dst = dto;
		task->src = dfrom;
		xmg_ptask_shape(task, ndim, size, ms, bs);
	} else {		/* block <- matrix */
		task->dst = dto;
		task->src = dfrom;
		xmg_ptask_shape(task, ndim, size, bs, ms);
	}
	xmg_die_on(xmg_ptask_run(&l, t->type, t->type, NULL));
	xmg_ptask_list_free(&l);
	if (!dev_to)
		xmg_die_on(xmgd_d2h(to, dto, dir ? blkbytes : matbytes));
	xmg_die_on(xmgd_sync());
}

void
xm_tensor_unfold_block(const xm_tensor_t *t, xm_dim_t blkidx, xm_dim_t mask_i,
    xm_dim_t mask_j, const void *from, void *to, size_t stride)
{
	unfold_fold(t, blkidx, mask_i, mask_j, from, to, stride, 0, __func__);
}

void
xm_tensor_fold_block(const xm_tensor_t *t, xm_dim_t blkidx, xm_dim_t mask_i,
    xm_dim_t mask_j, const void *from, void *to, size_t stride)
{
	unfold_fold(t, blkidx, mask_i, mask_j, from, to, stride, 1, __func__);
}

void
xm_tensor_free_block_data(xm_tensor_t *t)
{
	size_t i;

	for (i = 0; i < t->nblocks_total; i++) {
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL)
			xm_allocator_deallocate(t->allocator, t->blocks[i].data);
		t->blocks[i].type = XM_BLOCK_TYPE_ZERO;
		t->blocks[i].perm = xm_dim_identity_permutation(t->blocks[i].perm.n);
		t->blocks[i].scalar = 0;
		t->blocks[i].data = XM_NULL_PTR;
	}
	xmg_tensor_touch(t);
}

void
xm_tensor_free(xm_tensor_t *t)
{
	if (t == NULL)
		return;
	xm_block_space_free(t->bs);
	free(t->blocks);
	free(t);
}
