/*
 * xmg_dot_noalloc: the result of xm_dot computed without allocating any
 * memory (see include/xmg.h and csrc/cuda/noalloc.cu for who needs it).
 * Block tasks are built in a fixed-size array on the stack and run in
 * batches through the engine's static device scratch.
 */
#include "xmg_host.h"

int xmgd_noalloc_begin(void);
int xmgd_noalloc_dot_batch(int dtype, const xmgd_ptask_t *tasks,
    const int64_t *first, int ntasks);
int xmgd_noalloc_result(double out[2]);

int
xmg_dot_noalloc(const xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb, xm_scalar_t *result)
{
	xmgd_ptask_t tasks[XMG_NOALLOC_MAX_TASKS];
	int64_t first[XMG_NOALLOC_MAX_TASKS + 1];
	xm_dim_t cidxa, cidxb, nb, ia, ib, dims;
	int64_t size[XM_MAX_DIM], ds[XM_MAX_DIM], ss[XM_MAX_DIM];
	int64_t as[XM_MAX_DIM], bst[XM_MAX_DIM], nel, nctas;
	struct xmg_block *ba, *bb;
	size_t i, k, nblk;
	double out[2];
	int n = 0, st;

	if (result == NULL)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: result is NULL");
	if (a == NULL || b == NULL || idxa == NULL || idxb == NULL)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: NULL tensor or "
		    "index string");
	if (a->allocator != b->allocator)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: tensors must use "
		    "same allocator");
	if (!xmg_alloc_is_device(a->allocator))
		return xmg_seterr(XMG_ENOTSUP, "xmg_dot_noalloc: tensors must live "
		    "in GPU memory (allocator path NULL)");
	if (a->type != b->type)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: tensors must have "
		    "same scalar type");
	if (strlen(idxa) != xm_block_space_get_ndims(a->bs) ||
	    strlen(idxb) != xm_block_space_get_ndims(b->bs))
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: index strings do "
		    "not match tensor dimensions");
	xm_make_masks(idxa, idxb, &cidxa, &cidxb);
	if (cidxa.n != xm_block_space_get_ndims(a->bs) ||
	    cidxb.n != xm_block_space_get_ndims(b->bs))
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: index spaces do "
		    "not match");
	for (k = 0; k < cidxa.n; k++)
		if (!xm_block_space_eq1(a->bs, cidxa.i[k], b->bs, cidxb.i[k]))
			return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: "
			    "inconsistent block-spaces");
	if ((st = xmgd_noalloc_begin()) != XMG_OK)
		return st;
	nb = xm_block_space_get_nblocks(a->bs);
	nblk = xm_dim_dot(&nb);
	ia = xm_dim_zero(nb.n);
	ib = xm_dim_zero(cidxb.n);
	first[0] = 0;
	for (i = 0; i < nblk; i++, xm_dim_inc(&ia, &nb)) {
		xm_dim_set_mask(&ib, &cidxb, &ia, &cidxa);
		ba = xmg_tensor_block(a, ia);
		bb = xmg_tensor_block(b, ib);
		if (ba->type == XM_BLOCK_TYPE_ZERO || bb->type == XM_BLOCK_TYPE_ZERO)
			continue;
		dims = xm_block_space_get_block_dims(a->bs, ia);
		nel = (int64_t)xm_dim_dot(&dims);
		nctas = (nel + XMG_NOALLOC_ELEMS_PER_CTA - 1) /
		    XMG_NOALLOC_ELEMS_PER_CTA;
		if (nctas > XMG_NOALLOC_MAX_CTAS)
			return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: block of %lld "
			    "elements exceeds the maximum of %lld", (long long)nel,
			    (long long)XMG_NOALLOC_MAX_CTAS *
			    XMG_NOALLOC_ELEMS_PER_CTA);
		if (n == XMG_NOALLOC_MAX_TASKS ||
		    first[n] + nctas > XMG_NOALLOC_MAX_CTAS) {
			if ((st = xmgd_noalloc_dot_batch(a->type, tasks, first, n)))
				return st;
			n = 0;
		}
		/* element of a's block <- matching element of b's block, both
		 * with their block permutations */
		xmg_tensor_block_strides(a, ia, as);
		xmg_tensor_block_strides(b, ib, bst);
		for (k = 0; k < cidxa.n; k++) {
			size[cidxa.i[k]] = (int64_t)dims.i[cidxa.i[k]];
			ds[cidxa.i[k]] = as[cidxa.i[k]];
			ss[cidxa.i[k]] = bst[cidxb.i[k]];
		}
		memset(&tasks[n], 0, sizeof tasks[n]);
		tasks[n].op = XMGD_OP_DOT;
		tasks[n].dst = xm_tensor_get_block_data_ptr(a, ia);
		tasks[n].src = xm_tensor_get_block_data_ptr(b, ib);
		xmg_scalar_pack(xm_scalar_mul(ba->scalar, bb->scalar, a->type),
		    tasks[n].alpha);
		xmg_ptask_shape(&tasks[n], (int)dims.n, size, ds, ss);
		first[n + 1] = first[n] + nctas;
		n++;
	}
	if ((st = xmgd_noalloc_dot_batch(a->type, tasks, first, n)) != XMG_OK ||
	    (st = xmgd_noalloc_result(out)) != XMG_OK)
		return st;
	*result = out[0] + out[1] * I;
	return XMG_OK;
}
