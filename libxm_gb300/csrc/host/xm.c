/*
 * Element-wise tensor operations of libxm-gb300: set, copy, add, mul,
 * div, dot.  Each walks the canonical blocks of the output (for dot, every
 * nonzero block pair) in the reference's order (xm.c:28-508), maps each
 * block to the matching block of the second tensor through the index
 * strings, and turns the reference's unfold -> scale -> fold -> axpy chain
 * into one permuted, scaled CUDA pass over HBM (xmgd_ptasks).
 */
#include "xmg_host.h"

#define TASK_BATCH 4096

static int
check_pair(const xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb, xm_dim_t *cidxa, xm_dim_t *cidxb, int same_type,
    const char *fn)
{
	size_t k;

	if (a->allocator != b->allocator)
		return xmg_seterr(XMG_EINVAL, "%s: tensors must use same "
		    "allocator", fn);
	if (same_type && a->type != b->type)
		return xmg_seterr(XMG_EINVAL, "%s: tensors must have same "
		    "scalar type", fn);
	if (strlen(idxa) != xm_block_space_get_ndims(a->bs))
		return xmg_seterr(XMG_EINVAL, "%s: idxa does not match tensor "
		    "dimensions", fn);
	if (strlen(idxb) != xm_block_space_get_ndims(b->bs))
		return xmg_seterr(XMG_EINVAL, "%s: idxb does not match tensor "
		    "dimensions", fn);
	xm_make_masks(idxa, idxb, cidxa, cidxb);
	if (cidxa->n != xm_block_space_get_ndims(a->bs) ||
	    cidxb->n != xm_block_space_get_ndims(b->bs))
		return xmg_seterr(XMG_EINVAL, "%s: index spaces do not match",
		    fn);
	for (k = 0; k < cidxa->n; k++)
		if (!xm_block_space_eq1(a->bs, cidxa->i[k], b->bs, cidxb->i[k]))
			return xmg_seterr(XMG_EINVAL, "%s: inconsistent "
			    "block-spaces", fn);
	return XMG_OK;
}

/* Fill t with the iteration space "element of block ia of a (canonical)
 * <- matching element of block ib of b". */
static void
map_task(xmgd_ptask_t *t, const xm_tensor_t *a, xm_dim_t ia,
    const xm_tensor_t *b, xm_dim_t ib, const xm_dim_t *cidxa,
    const xm_dim_t *cidxb, uint64_t dptr_a, uint64_t dptr_b)
{
	xm_dim_t dims = xm_block_space_get_block_dims(a->bs, ia);
	int64_t size[XM_MAX_DIM], ds[XM_MAX_DIM], ss[XM_MAX_DIM];
	int64_t as[XM_MAX_DIM], bst[XM_MAX_DIM];
	size_t k;

	xmg_tensor_block_strides(a, ia, as);
	xmg_tensor_block_strides(b, ib, bst);
	for (k = 0; k < cidxa->n; k++) {
		size[cidxa->i[k]] = (int64_t)dims.i[cidxa->i[k]];
		ds[cidxa->i[k]] = as[cidxa->i[k]];
		ss[cidxa->i[k]] = bst[cidxb->i[k]];
	}
	t->dst = dptr_a;
	t->src = dptr_b;
	xmg_ptask_shape(t, (int)dims.n, size, ds, ss);
}

static uint64_t
dev_ptr(const xm_tensor_t *t, xm_dim_t blk)
{
	uint64_t d;

	xmg_die_on(xmg_alloc_device_view(t->allocator,
	    xm_tensor_get_block_data_ptr(t, blk),
	    xm_tensor_get_block_bytes(t, blk), &d));
	return d;
}

/* Flush a batch; write pagefile-staged outputs back. */
static int
flush(xmg_ptask_list_t *l, const xm_tensor_t *a, int dtype, int stype,
    xm_dim_t *outs, size_t nouts, double *dots)
{
	size_t k;
	int st;

	if ((st = xmg_ptask_run(l, dtype, stype, dots)) != XMG_OK)
		return st;
	l->n = 0;
	if (!xmg_alloc_is_device(a->allocator)) {
		if ((st = xmgd_sync()) != XMG_OK)
			return st;
		for (k = 0; k < nouts; k++)
			if ((st = xmg_alloc_commit_view(a->allocator,
			    xm_tensor_get_block_data_ptr(a, outs[k]),
			    xm_tensor_get_block_bytes(a, outs[k]))) != XMG_OK)
				return st;
		xmg_alloc_release_views(a->allocator, 0);
	}
	return XMG_OK;
}

int
xmg_set(xm_tensor_t *a, xm_scalar_t x)
{
	xm_dim_t *list;
	size_t n, k, first = 0;
	xmg_ptask_list_t l = {0};
	xmgd_ptask_t *t;
	int64_t size;
	int st = XMG_OK;

	xm_tensor_get_canonical_block_list(a, &list, &n);
	for (k = 0; k < n && st == XMG_OK; k++) {
		t = xmg_ptask_push(&l);
		t->op = XMGD_OP_SET;
		xmg_scalar_pack(x, t->alpha);
		t->dst = dev_ptr(a, list[k]);
		size = (int64_t)xm_tensor_get_block_size(a, list[k]);
		xmg_ptask_shape(t, 1, &size, &(int64_t){1}, &(int64_t){0});
		if (l.n == TASK_BATCH || k + 1 == n) {
			st = flush(&l, a, a->type, a->type, list + first,
			    k + 1 - first, NULL);
			first = k + 1;
		}
	}
	if (st == XMG_OK)
		st = xmgd_sync();
	xmg_ptask_list_free(&l);
	free(list);
	return st;
}

void
xm_set(xm_tensor_t *a, xm_scalar_t x)
{
	xmg_die_on(xmg_set(a, x));
}

/* Shared driver for copy / add / mul / div. */
enum { OPK_COPY, OPK_ADD, OPK_MUL, OPK_DIV };

static int
two_tensor(int kind, xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb, const char *fn)
{
	xm_dim_t cidxa, cidxb, *list, ib;
	size_t n, k, first = 0;
	xmg_ptask_list_t l = {0};
	xmgd_ptask_t *t;
	struct xmg_block *bb;
	xm_scalar_t s;
	int64_t size;
	int st;

	if ((st = check_pair(a, b, idxa, idxb, &cidxa, &cidxb,
	    kind != OPK_COPY, fn)) != XMG_OK)
		return st;
	xm_tensor_get_canonical_block_list(a, &list, &n);
	ib = xm_dim_zero(cidxb.n);
	for (k = 0; k < n && st == XMG_OK; k++) {
		xm_dim_set_mask(&ib, &cidxb, &list[k], &cidxa);
		bb = xmg_tensor_block(b, ib);
		t = xmg_ptask_push(&l);
		size = (int64_t)xm_tensor_get_block_size(a, list[k]);
		switch (kind) {
		case OPK_COPY:	/* xm.c:123-146 */
			if (alpha == 0 || bb->type == XM_BLOCK_TYPE_ZERO) {
				t->op = XMGD_OP_SET;
				break;
			}
			t->op = XMGD_OP_COPY;
			s = xm_scalar_mul(alpha, bb->scalar, b->type);
			xmg_scalar_pack(s, t->alpha);
			break;
		case OPK_ADD:	/* xm.c:212-240 */
			if (beta == 0 || bb->type == XM_BLOCK_TYPE_ZERO) {
				t->op = alpha == 0 ? XMGD_OP_SET : XMGD_OP_SCALE;
				xmg_scalar_pack(alpha == 0 ? 0 : alpha, t->alpha);
				break;
			}
			s = xm_scalar_mul(beta, bb->scalar, a->type);
			t->op = alpha == 0 ? XMGD_OP_COPY : XMGD_OP_AXPY;
			xmg_scalar_pack(alpha == 0 ? s : alpha, t->alpha);
			xmg_scalar_pack(s, t->beta);
			break;
		case OPK_MUL:	/* xm.c:304-323 */
			if (bb->type == XM_BLOCK_TYPE_ZERO) {
				t->op = XMGD_OP_SET;
				break;
			}
			t->op = XMGD_OP_MUL;
			xmg_scalar_pack(bb->scalar, t->alpha);
			break;
		case OPK_DIV:	/* xm.c:387-404 */
			if (bb->type == XM_BLOCK_TYPE_ZERO) {
				l.n--;
				st = xmg_seterr(XMG_EINVAL, "%s: division by zero",
				    fn);
				continue;
			}
			t->op = XMGD_OP_DIV;
			xmg_scalar_pack(bb->scalar, t->alpha);
			break;
		}
		if (t->op == XMGD_OP_SET || t->op == XMGD_OP_SCALE) {
			t->dst = dev_ptr(a, list[k]);
			xmg_ptask_shape(t, 1, &size, &(int64_t){1},
			    &(int64_t){0});
		} else {
			map_task(t, a, list[k], b, ib, &cidxa, &cidxb,
			    dev_ptr(a, list[k]), dev_ptr(b, ib));
		}
		if (l.n == TASK_BATCH || k + 1 == n) {
			st = flush(&l, a, a->type, b->type, list + first,
			    k + 1 - first, NULL);
			first = k + 1;
		}
	}
	if (st == XMG_OK)
		st = xmgd_sync();
	if (!xmg_alloc_is_device(b->allocator))
		xmg_alloc_release_views(b->allocator, 0);
	xmg_ptask_list_free(&l);
	free(list);
	return st;
}

void
xm_copy(xm_tensor_t *a, xm_scalar_t s, const xm_tensor_t *b, const char *idxa,
    const char *idxb)
{
	xmg_die_on(two_tensor(OPK_COPY, s, a, 0, b, idxa, idxb, __func__));
}

int
xmg_add(xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb)
{
	return two_tensor(OPK_ADD, alpha, a, beta, b, idxa, idxb, "xm_add");
}

void
xm_add(xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb)
{
	xmg_die_on(xmg_add(alpha, a, beta, b, idxa, idxb));
}

void
xm_mul(xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb)
{
	xmg_die_on(two_tensor(OPK_MUL, 0, a, 0, b, idxa, idxb, __func__));
}

void
xm_div(xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb)
{
	xmg_die_on(two_tensor(OPK_DIV, 0, a, 0, b, idxa, idxb, __func__));
}

/* Sum over every block index of a where both blocks are nonzero of
 * (s_a * s_b) * <perm(a), perm(b)>  (xm.c:472-497). */
xm_scalar_t
xm_dot(const xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb)
{
	xm_dim_t cidxa, cidxb, nb, ia, ib;
	xmg_ptask_list_t l = {0};
	xmgd_ptask_t *t;
	xm_scalar_t *fac = NULL, dot = 0, part;
	double *dots = NULL;
	size_t i, nblk, nt = 0;
	struct xmg_block *ba, *bb;

	xmg_die_on(check_pair(a, b, idxa, idxb, &cidxa, &cidxb, 1, __func__));
	nb = xm_block_space_get_nblocks(a->bs);
	nblk = xm_dim_dot(&nb);
	ia = xm_dim_zero(nb.n);
	ib = xm_dim_zero(cidxb.n);
	for (i = 0; i < nblk; i++, xm_dim_inc(&ia, &nb)) {
		xm_dim_set_mask(&ib, &cidxb, &ia, &cidxa);
		ba = xmg_tensor_block(a, ia);
		bb = xmg_tensor_block(b, ib);
		if (ba->type == XM_BLOCK_TYPE_ZERO ||
		    bb->type == XM_BLOCK_TYPE_ZERO)
			continue;
		if ((fac = realloc(fac, (nt + 1) * sizeof *fac)) == NULL)
			xm_fatal("%s: out of memory", __func__);
		fac[nt++] = xm_scalar_mul(ba->scalar, bb->scalar, a->type);
		t = xmg_ptask_push(&l);
		t->op = XMGD_OP_DOT;
		map_task(t, a, ia, b, ib, &cidxa, &cidxb, dev_ptr(a, ia),
		    dev_ptr(b, ib));
	}
	if (nt > 0) {
		if ((dots = calloc(2 * nt, sizeof *dots)) == NULL)
			xm_fatal("%s: out of memory", __func__);
		xmg_die_on(xmg_ptask_run(&l, a->type, b->type, dots));
		xmg_die_on(xmgd_sync());
		for (i = 0; i < nt; i++) {
			part = dots[2 * i] + dots[2 * i + 1] * I;
			part = xm_scalar_mul(fac[i], part, a->type);
			dot = xm_scalar_add(dot, part, a->type);
		}
	}
	if (!xmg_alloc_is_device(a->allocator))
		xmg_alloc_release_views(a->allocator, 0);
	xmg_ptask_list_free(&l);
	free(fac);
	free(dots);
	return dot;
}

void
xm_print_banner(void)
{
	printf("Libxm Tensor Library (GB300 engine)\n");
	printf("libxm API on hand-written sm_103a CUDA kernels\n");
	printf("Reference algorithm: https://github.com/ilyak/libxm\n");
}
