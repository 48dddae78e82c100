/*
 * Building blocks for the permuted element-wise kernels: iteration-space
 * normalisation and batching of per-block tasks.
 */
#include "xmg_host.h"

void
xmg_ptask_shape(xmgd_ptask_t *t, int ndim, const int64_t *size,
    const int64_t *dst_stride, const int64_t *src_stride)
{
	int64_t sz[XM_MAX_DIM], ds[XM_MAX_DIM], ss[XM_MAX_DIM], x;
	int n = 0, k, j, q;

	for (k = 0; k < ndim; k++) {
		if (size[k] == 1)
			continue;
		sz[n] = size[k];
		ds[n] = dst_stride[k];
		ss[n] = src_stride[k];
		n++;
	}
	/* order by destination stride so that dimension 0 is the one with
	 * unit destination stride (coalesced stores) */
	for (k = 1; k < n; k++)
		for (j = k; j > 0 && ds[j] < ds[j - 1]; j--) {
			x = sz[j]; sz[j] = sz[j - 1]; sz[j - 1] = x;
			x = ds[j]; ds[j] = ds[j - 1]; ds[j - 1] = x;
			x = ss[j]; ss[j] = ss[j - 1]; ss[j - 1] = x;
		}
	/* merge neighbours contiguous on both sides */
	for (k = 1, j = 0; k < n; k++) {
		if (ds[k] == ds[j] * sz[j] && ss[k] == ss[j] * sz[j] &&
		    sz[j] * sz[k] < (1LL << 31)) {
			sz[j] *= sz[k];
		} else {
			j++;
			sz[j] = sz[k]; ds[j] = ds[k]; ss[j] = ss[k];
		}
	}
	n = n > 0 ? j + 1 : 0;
	if (n == 0) {
		n = 1;
		sz[0] = 1; ds[0] = 1; ss[0] = 1;
	}
	/* the source's unit-stride dimension goes to position 1: the kernel
	 * then transposes through shared memory between dims 0 and 1 */
	for (q = 1; q < n && ss[q] != 1; q++)
		;
	if (q < n && q != 1 && ss[0] != 1) {
		x = sz[q]; sz[q] = sz[1]; sz[1] = x;
		x = ds[q]; ds[q] = ds[1]; ds[1] = x;
		x = ss[q]; ss[q] = ss[1]; ss[1] = x;
	}
	t->ndim = n;
	for (k = 0; k < 8; k++) {
		t->size[k] = k < n ? (int32_t)sz[k] : 1;
		t->dst_stride[k] = k < n ? ds[k] : 0;
		t->src_stride[k] = k < n ? ss[k] : 0;
	}
}

xmgd_ptask_t *
xmg_ptask_push(xmg_ptask_list_t *l)
{
	xmgd_ptask_t *v;

	if (l->n == l->cap) {
		l->cap = l->cap ? 2 * l->cap : 64;
		if ((v = realloc(l->v, (size_t)l->cap * sizeof *v)) == NULL)
			xm_fatal("%s: out of memory", __func__);
		l->v = v;
	}
	v = &l->v[l->n++];
	memset(v, 0, sizeof *v);
	return v;
}

int
xmg_ptask_run(xmg_ptask_list_t *l, int dtype, int stype, double *dots)
{
	if (l->n == 0)
		return XMG_OK;
	return xmgd_ptasks(dtype, stype, l->v, l->n, dots);
}

void
xmg_ptask_list_free(xmg_ptask_list_t *l)
{
	free(l->v);
	memset(l, 0, sizeof *l);
}
