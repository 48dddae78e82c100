/*
 * Index algebra for libxm-gb300 (host).
 *
 * Semantics follow the reference's src/dim.c: index 0 is the fastest-varying
 * position (dim.c:201-230), increment carries towards higher positions and
 * sets the index to the shape itself once past the end (dim.c:277-291), and
 * permute scatters ret[perm[k]] = idx[k] (dim.c:350-369).
 */
#include "xmg_host.h"

xm_dim_t
xm_dim_same(size_t ndim, size_t dim)
{
	xm_dim_t r;
	size_t k;

	if (ndim > XM_MAX_DIM)
		xm_fatal("%s: too many dimensions", __func__);
	memset(&r, 0, sizeof r);
	r.n = ndim;
	for (k = 0; k < ndim; k++)
		r.i[k] = dim;
	return r;
}

xm_dim_t xm_dim_zero(size_t ndim) { return xm_dim_same(ndim, 0); }

static xm_dim_t
dim_make(size_t n, const size_t *v)
{
	xm_dim_t r;
	size_t k;

	memset(&r, 0, sizeof r);
	r.n = n;
	for (k = 0; k < n; k++)
		r.i[k] = v[k];
	return r;
}

xm_dim_t xm_dim_1(size_t a) { size_t v[] = {a}; return dim_make(1, v); }
xm_dim_t xm_dim_2(size_t a, size_t b) { size_t v[] = {a, b}; return dim_make(2, v); }
xm_dim_t xm_dim_3(size_t a, size_t b, size_t c)
{ size_t v[] = {a, b, c}; return dim_make(3, v); }
xm_dim_t xm_dim_4(size_t a, size_t b, size_t c, size_t d)
{ size_t v[] = {a, b, c, d}; return dim_make(4, v); }
xm_dim_t xm_dim_5(size_t a, size_t b, size_t c, size_t d, size_t e)
{ size_t v[] = {a, b, c, d, e}; return dim_make(5, v); }
xm_dim_t xm_dim_6(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f)
{ size_t v[] = {a, b, c, d, e, f}; return dim_make(6, v); }
xm_dim_t xm_dim_7(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f,
    size_t g)
{ size_t v[] = {a, b, c, d, e, f, g}; return dim_make(7, v); }
xm_dim_t xm_dim_8(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f,
    size_t g, size_t h)
{ size_t v[] = {a, b, c, d, e, f, g, h}; return dim_make(8, v); }

int
xm_dim_eq(const xm_dim_t *a, const xm_dim_t *b)
{
	size_t k;

	if (a->n != b->n)
		return 0;
	for (k = 0; k < a->n; k++)
		if (a->i[k] != b->i[k])
			return 0;
	return 1;
}

int xm_dim_ne(const xm_dim_t *a, const xm_dim_t *b) { return !xm_dim_eq(a, b); }

int
xm_dim_less(const xm_dim_t *idx, const xm_dim_t *dim)
{
	size_t k;

	for (k = 0; k < idx->n; k++)
		if (idx->i[k] >= dim->i[k])
			return 0;
	return 1;
}

size_t
xm_dim_dot(const xm_dim_t *dim)
{
	size_t k, p = 1;

	for (k = 0; k < dim->n; k++)
		p *= dim->i[k];
	return p;
}

size_t
xm_dim_offset(const xm_dim_t *idx, const xm_dim_t *dim)
{
	size_t k, off = 0;

	/* Horner form, highest position first: same value as the reference's
	 * sum of idx[k] * prod(dim[0..k-1]). */
	for (k = idx->n; k-- > 0; )
		off = off * dim->i[k] + idx->i[k];
	return off;
}

xm_dim_t
xm_dim_from_offset(size_t offset, const xm_dim_t *dim)
{
	xm_dim_t r;
	size_t k;

	memset(&r, 0, sizeof r);
	r.n = dim->n;
	for (k = 0; k + 1 < dim->n; k++) {
		r.i[k] = offset % dim->i[k];
		offset /= dim->i[k];
	}
	if (dim->n > 0)
		r.i[dim->n - 1] = offset;
	return r;
}

void
xm_dim_inc(xm_dim_t *idx, const xm_dim_t *dim)
{
	size_t k;

	for (k = 0; k < idx->n; k++) {
		if (++idx->i[k] < dim->i[k])
			return;
		idx->i[k] = 0;
	}
	*idx = *dim;	/* wrapped past the last element */
}

void
xm_dim_zero_mask(xm_dim_t *dim, const xm_dim_t *mask)
{
	size_t k;

	for (k = 0; k < mask->n; k++)
		dim->i[mask->i[k]] = 0;
}

void
xm_dim_set_mask(xm_dim_t *a, const xm_dim_t *maska, const xm_dim_t *b,
    const xm_dim_t *maskb)
{
	size_t k;

	for (k = 0; k < maska->n; k++)
		a->i[maska->i[k]] = b->i[maskb->i[k]];
}

size_t
xm_dim_dot_mask(const xm_dim_t *dim, const xm_dim_t *mask)
{
	size_t k, p = 1;

	for (k = 0; k < mask->n; k++)
		p *= dim->i[mask->i[k]];
	return p;
}

void
xm_dim_inc_mask(xm_dim_t *idx, const xm_dim_t *dim, const xm_dim_t *mask)
{
	size_t k, pos;

	/* No wrap-to-end marker here, matching dim.c:324-336: the masked
	 * positions simply roll over to zero. */
	for (k = 0; k < mask->n; k++) {
		pos = mask->i[k];
		if (++idx->i[pos] < dim->i[pos])
			return;
		idx->i[pos] = 0;
	}
}

xm_dim_t
xm_dim_identity_permutation(size_t ndim)
{
	xm_dim_t r = xm_dim_zero(ndim);
	size_t k;

	for (k = 0; k < ndim; k++)
		r.i[k] = k;
	return r;
}

xm_dim_t
xm_dim_permute(const xm_dim_t *idx, const xm_dim_t *permutation)
{
	xm_dim_t r;
	size_t k;

	memset(&r, 0, sizeof r);
	r.n = idx->n;
	for (k = 0; k < idx->n; k++)
		r.i[permutation->i[k]] = idx->i[k];
	return r;
}
