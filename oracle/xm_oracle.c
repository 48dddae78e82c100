/*
 * ORACLE -- test infrastructure only, never part of the product.
 *
 * A CPU restatement of the reference libxm algorithm for the contraction
 * path, exporting the same C API names as libxm (xm.h) so that one test
 * binding drives the oracle, the reference built from source, and the
 * GB300 engine alike.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it.
 *
 * Each function follows the reference file:line it cites.  GEMMs go to an
 * ILP64 BLAS (the OpenBLAS bundled with numpy, located by the caller via
 * xmo_set_blas) or, when none is available, to a plain C triple loop.
 * Output blocks are processed in parallel with OpenMP, as the reference
 * does (contract.c:288-309).
 */
#include <complex.h>
#include <dlfcn.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- public types (dim.h:30-38, scalar.h:36-53, tensor.h:32-39) ---- */
#define XM_MAX_DIM 8
typedef struct { size_t n; size_t i[XM_MAX_DIM]; } xm_dim_t;
typedef enum { XM_SCALAR_FLOAT = 0, XM_SCALAR_FLOAT_COMPLEX,
    XM_SCALAR_DOUBLE, XM_SCALAR_DOUBLE_COMPLEX } xm_scalar_type_t;
typedef double complex xm_scalar_t;
typedef enum { XM_BLOCK_TYPE_ZERO = 0, XM_BLOCK_TYPE_CANONICAL,
    XM_BLOCK_TYPE_DERIVATIVE } xm_block_type_t;
#define XM_NULL_PTR ((uint64_t)(-1))

__attribute__((noreturn)) void
xm_fatal(const char *fmt, ...)
{
	va_list ap;
	fprintf(stderr, "libxm: ");
	va_start(ap, fmt);
	vfprintf(stderr, fmt, ap);
	va_end(ap);
	fprintf(stderr, "\n");
	exit(1);
}
#define FATAL(msg) xm_fatal("%s: %s", __func__, msg)

/* util.c:37-53 */
void
xm_make_masks(const char *s1, const char *s2, xm_dim_t *m1, xm_dim_t *m2)
{
	size_t a, b, l1 = strlen(s1), l2 = strlen(s2);
	m1->n = m2->n = 0;
	for (a = 0; a < l1; a++)
		for (b = 0; b < l2; b++)
			if (s1[a] == s2[b]) {
				m1->i[m1->n++] = a;
				m2->i[m2->n++] = b;
			}
}

/* ---- dim.c:21-369 ---- */
xm_dim_t xm_dim_same(size_t nd, size_t v)
{ xm_dim_t r; memset(&r, 0, sizeof r); r.n = nd; for (size_t k = 0; k < nd; k++) r.i[k] = v; return r; }
xm_dim_t xm_dim_zero(size_t nd) { return xm_dim_same(nd, 0); }
static xm_dim_t mk(size_t n, size_t a, size_t b, size_t c, size_t d, size_t e,
    size_t f, size_t g, size_t h)
{ xm_dim_t r = {n, {a, b, c, d, e, f, g, h}}; for (size_t k = n; k < 8; k++) r.i[k] = 0; return r; }
xm_dim_t xm_dim_1(size_t a) { return mk(1, a, 0, 0, 0, 0, 0, 0, 0); }
xm_dim_t xm_dim_2(size_t a, size_t b) { return mk(2, a, b, 0, 0, 0, 0, 0, 0); }
xm_dim_t xm_dim_3(size_t a, size_t b, size_t c) { return mk(3, a, b, c, 0, 0, 0, 0, 0); }
xm_dim_t xm_dim_4(size_t a, size_t b, size_t c, size_t d) { return mk(4, a, b, c, d, 0, 0, 0, 0); }
xm_dim_t xm_dim_5(size_t a, size_t b, size_t c, size_t d, size_t e) { return mk(5, a, b, c, d, e, 0, 0, 0); }
xm_dim_t xm_dim_6(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f) { return mk(6, a, b, c, d, e, f, 0, 0); }
xm_dim_t xm_dim_7(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f, size_t g) { return mk(7, a, b, c, d, e, f, g, 0); }
xm_dim_t xm_dim_8(size_t a, size_t b, size_t c, size_t d, size_t e, size_t f, size_t g, size_t h) { return mk(8, a, b, c, d, e, f, g, h); }
int xm_dim_eq(const xm_dim_t *a, const xm_dim_t *b)
{ if (a->n != b->n) return 0; for (size_t k = 0; k < a->n; k++) if (a->i[k] != b->i[k]) return 0; return 1; }
int xm_dim_ne(const xm_dim_t *a, const xm_dim_t *b) { return !xm_dim_eq(a, b); }
int xm_dim_less(const xm_dim_t *x, const xm_dim_t *d)
{ for (size_t k = 0; k < x->n; k++) if (x->i[k] >= d->i[k]) return 0; return 1; }
size_t xm_dim_dot(const xm_dim_t *d) { size_t r = 1; for (size_t k = 0; k < d->n; k++) r *= d->i[k]; return r; }
/* dim.c:201-230: sum_k idx[k] * prod_{q<k} dim[q] */
size_t xm_dim_offset(const xm_dim_t *x, const xm_dim_t *d)
{ size_t r = 0, s = 1; for (size_t k = 0; k < x->n; k++) { r += x->i[k] * s; s *= d->i[k]; } return r; }
xm_dim_t xm_dim_from_offset(size_t off, const xm_dim_t *d)
{ xm_dim_t r = xm_dim_zero(d->n); for (size_t k = 0; k < d->n; k++) { if (k + 1 == d->n) { r.i[k] = off; break; } r.i[k] = off % d->i[k]; off /= d->i[k]; } return r; }
/* dim.c:277-291 */
void xm_dim_inc(xm_dim_t *x, const xm_dim_t *d)
{ size_t carry = 1; for (size_t k = 0; carry && k < x->n; k++) { x->i[k] += carry; carry = x->i[k] / d->i[k]; x->i[k] %= d->i[k]; } if (carry) *x = *d; }
void xm_dim_zero_mask(xm_dim_t *d, const xm_dim_t *m) { for (size_t k = 0; k < m->n; k++) d->i[m->i[k]] = 0; }
void xm_dim_set_mask(xm_dim_t *a, const xm_dim_t *ma, const xm_dim_t *b, const xm_dim_t *mb)
{ for (size_t k = 0; k < ma->n; k++) a->i[ma->i[k]] = b->i[mb->i[k]]; }
size_t xm_dim_dot_mask(const xm_dim_t *d, const xm_dim_t *m)
{ size_t r = 1; for (size_t k = 0; k < m->n; k++) r *= d->i[m->i[k]]; return r; }
/* dim.c:324-336 */
void xm_dim_inc_mask(xm_dim_t *x, const xm_dim_t *d, const xm_dim_t *m)
{ size_t carry = 1; for (size_t k = 0; carry && k < m->n; k++) { size_t p = m->i[k]; x->i[p] += carry; carry = x->i[p] / d->i[p]; x->i[p] %= d->i[p]; } }
xm_dim_t xm_dim_identity_permutation(size_t nd)
{ xm_dim_t r = xm_dim_zero(nd); for (size_t k = 0; k < nd; k++) r.i[k] = k; return r; }
/* dim.c:350-369 */
xm_dim_t xm_dim_permute(const xm_dim_t *x, const xm_dim_t *p)
{ xm_dim_t r = xm_dim_zero(x->n); for (size_t k = 0; k < x->n; k++) r.i[p->i[k]] = x->i[k]; return r; }

/* ---- blockspace.c:25-282 ---- */
typedef struct xm_block_space { xm_dim_t dims, nblocks; size_t *splits[XM_MAX_DIM]; } xm_block_space_t;

xm_block_space_t *
xm_block_space_create(xm_dim_t dims)
{
	xm_block_space_t *bs = calloc(1, sizeof *bs);
	bs->dims = dims;
	bs->nblocks = xm_dim_same(dims.n, 1);
	for (size_t k = 0; k < dims.n; k++) {
		bs->splits[k] = malloc(2 * sizeof(size_t));
		bs->splits[k][0] = 0;
		bs->splits[k][1] = dims.i[k];
	}
	return bs;
}
void xm_block_space_free(xm_block_space_t *bs)
{ if (!bs) return; for (size_t k = 0; k < bs->dims.n; k++) free(bs->splits[k]); free(bs); }
/* blockspace.c:75-97 */
xm_block_space_t *
xm_block_space_permute_clone(const xm_block_space_t *bs, xm_dim_t perm)
{
	xm_block_space_t *r = calloc(1, sizeof *r);
	r->dims = xm_dim_permute(&bs->dims, &perm);
	r->nblocks = xm_dim_permute(&bs->nblocks, &perm);
	for (size_t j = 0; j < bs->dims.n; j++) {
		size_t i = perm.i[j], n = bs->nblocks.i[j] + 1;
		r->splits[i] = malloc(n * sizeof(size_t));
		memcpy(r->splits[i], bs->splits[j], n * sizeof(size_t));
	}
	return r;
}
xm_block_space_t *xm_block_space_clone(const xm_block_space_t *bs)
{ return xm_block_space_permute_clone(bs, xm_dim_identity_permutation(bs->dims.n)); }
size_t xm_block_space_get_ndims(const xm_block_space_t *bs) { return bs->dims.n; }
xm_dim_t xm_block_space_get_abs_dims(const xm_block_space_t *bs) { return bs->dims; }
xm_dim_t xm_block_space_get_nblocks(const xm_block_space_t *bs) { return bs->nblocks; }
/* blockspace.c:117-139 */
void
xm_block_space_split(xm_block_space_t *bs, size_t dim, size_t x)
{
	size_t nb = bs->nblocks.i[dim], i;
	for (i = 0; i <= nb; i++) {
		if (bs->splits[dim][i] == x) return;
		if (bs->splits[dim][i] > x) break;
	}
	bs->splits[dim] = realloc(bs->splits[dim], (nb + 2) * sizeof(size_t));
	memmove(bs->splits[dim] + i + 1, bs->splits[dim] + i, (nb + 1 - i) * sizeof(size_t));
	bs->splits[dim][i] = x;
	bs->nblocks.i[dim]++;
}
/* blockspace.c:141-163 */
void
xm_block_space_autosplit(xm_block_space_t *bs)
{
	for (size_t j = 0; j < bs->dims.n; j++) {
		size_t dim = bs->dims.i[j], nblks = (dim + 31) / 32, pos = 0;
		for (size_t i = 0; i + 1 < nblks; i++) {
			size_t sz = dim / (nblks - i);
			if (sz > 1 && sz % 2 && nblks - i > 1)
				sz += sz < 32 ? 1 : (size_t)-1;
			dim -= sz;
			pos += sz;
			xm_block_space_split(bs, j, pos);
		}
	}
}
size_t xm_block_space_get_split(xm_block_space_t *bs, size_t dim, size_t i) { return bs->splits[dim][i]; }
xm_dim_t
xm_block_space_get_block_dims(const xm_block_space_t *bs, xm_dim_t b)
{
	xm_dim_t r = xm_dim_zero(bs->dims.n);
	for (size_t k = 0; k < r.n; k++)
		r.i[k] = bs->splits[k][b.i[k] + 1] - bs->splits[k][b.i[k]];
	return r;
}
size_t xm_block_space_get_block_size(const xm_block_space_t *bs, xm_dim_t b)
{ xm_dim_t d = xm_block_space_get_block_dims(bs, b); return xm_dim_dot(&d); }
size_t
xm_block_space_get_largest_block_size(const xm_block_space_t *bs)
{
	size_t r = 1;
	for (size_t k = 0; k < bs->dims.n; k++) {
		size_t mx = 0;
		for (size_t j = 0; j < bs->nblocks.i[k]; j++)
			if (bs->splits[k][j + 1] - bs->splits[k][j] > mx)
				mx = bs->splits[k][j + 1] - bs->splits[k][j];
		r *= mx;
	}
	return r;
}
void
xm_block_space_decompose_index(const xm_block_space_t *bs, xm_dim_t idx,
    xm_dim_t *blk, xm_dim_t *el)
{
	*blk = xm_dim_zero(bs->dims.n);
	*el = xm_dim_zero(bs->dims.n);
	for (size_t k = 0; k < bs->dims.n; k++)
		for (size_t j = 0; j < bs->nblocks.i[k]; j++)
			if (bs->splits[k][j + 1] > idx.i[k]) {
				blk->i[k] = j;
				el->i[k] = idx.i[k] - bs->splits[k][j];
				break;
			}
}
int
xm_block_space_eq1(const xm_block_space_t *a, size_t da, const xm_block_space_t *b, size_t db)
{
	if (a->nblocks.i[da] != b->nblocks.i[db]) return 0;
	for (size_t i = 0; i <= a->nblocks.i[da]; i++)
		if (a->splits[da][i] != b->splits[db][i]) return 0;
	return 1;
}
int
xm_block_space_eq(const xm_block_space_t *a, const xm_block_space_t *b)
{
	if (a->dims.n != b->dims.n) return 0;
	for (size_t k = 0; k < a->dims.n; k++)
		if (!xm_block_space_eq1(a, k, b, k)) return 0;
	return 1;
}

/* ---- scalar.c:22-414 (the subset the path uses) ---- */
int xm_scalar_check_type(xm_scalar_type_t t) { return t >= 0 && t <= 3; }
size_t xm_scalar_sizeof(xm_scalar_type_t t)
{ static const size_t s[] = {4, 8, 8, 16}; if (!xm_scalar_check_type(t)) FATAL("unexpected scalar type"); return s[t]; }
xm_scalar_t
xm_scalar_mul(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return (float)a * (float)b;
	case XM_SCALAR_FLOAT_COMPLEX: return (float complex)a * (float complex)b;
	case XM_SCALAR_DOUBLE: return (double)a * (double)b;
	default: return a * b;
	}
}
xm_scalar_t
xm_scalar_add(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return (float)a + (float)b;
	case XM_SCALAR_FLOAT_COMPLEX: return (float complex)a + (float complex)b;
	case XM_SCALAR_DOUBLE: return (double)a + (double)b;
	default: return a + b;
	}
}
static xm_scalar_t
get_el(const void *x, size_t i, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return ((const float *)x)[i];
	case XM_SCALAR_FLOAT_COMPLEX: return ((const float complex *)x)[i];
	case XM_SCALAR_DOUBLE: return ((const double *)x)[i];
	default: return ((const double complex *)x)[i];
	}
}
static void
set_el(void *x, size_t i, xm_scalar_t v, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: ((float *)x)[i] = (float)v; break;
	case XM_SCALAR_FLOAT_COMPLEX: ((float complex *)x)[i] = (float complex)v; break;
	case XM_SCALAR_DOUBLE: ((double *)x)[i] = (double)v; break;
	default: ((double complex *)x)[i] = v; break;
	}
}
xm_scalar_t xm_scalar_get_element(void *x, size_t i, xm_scalar_type_t t) { return get_el(x, i, t); }

/* ---- allocator: RAM only (alloc.c:233-239, 252-263) ---- */
typedef struct xm_allocator { int dummy; } xm_allocator_t;
xm_allocator_t *xm_allocator_create(const char *path) { (void)path; return calloc(1, sizeof(xm_allocator_t)); }
const char *xm_allocator_get_path(xm_allocator_t *a) { (void)a; return NULL; }
uint64_t xm_allocator_allocate(xm_allocator_t *a, size_t n)
{ (void)a; void *p; if (n == 0) return XM_NULL_PTR; p = malloc(n); return p ? (uint64_t)(uintptr_t)p : XM_NULL_PTR; }
void xm_allocator_read(xm_allocator_t *a, uint64_t h, void *m, size_t n)
{ (void)a; if (h == XM_NULL_PTR) FATAL("data pointer is NULL"); memcpy(m, (void *)(uintptr_t)h, n); }
void xm_allocator_write(xm_allocator_t *a, uint64_t h, const void *m, size_t n)
{ (void)a; if (h == XM_NULL_PTR) FATAL("data pointer is NULL"); memcpy((void *)(uintptr_t)h, m, n); }
void xm_allocator_deallocate(xm_allocator_t *a, uint64_t h) { (void)a; if (h != XM_NULL_PTR) free((void *)(uintptr_t)h); }
void xm_allocator_destroy(xm_allocator_t *a) { free(a); }

/* ---- tensor.c:26-669 ---- */
struct blk { xm_block_type_t type; xm_dim_t perm; xm_scalar_t s; uint64_t data; };
typedef struct xm_tensor { xm_scalar_type_t type; xm_block_space_t *bs; xm_allocator_t *al; struct blk *b; } xm_tensor_t;

static struct blk *
tblk(const xm_tensor_t *t, xm_dim_t idx)
{
	xm_dim_t nb = t->bs->nblocks;
	return &t->b[xm_dim_offset(&idx, &nb)];
}
xm_dim_t xm_tensor_get_nblocks(const xm_tensor_t *t) { return t->bs->nblocks; }
xm_dim_t xm_tensor_get_abs_dims(const xm_tensor_t *t) { return t->bs->dims; }
const xm_block_space_t *xm_tensor_get_block_space(const xm_tensor_t *t) { return t->bs; }
xm_scalar_type_t xm_tensor_get_scalar_type(const xm_tensor_t *t) { return t->type; }
xm_allocator_t *xm_tensor_get_allocator(const xm_tensor_t *t) { return t->al; }
xm_block_type_t xm_tensor_get_block_type(const xm_tensor_t *t, xm_dim_t i) { return tblk(t, i)->type; }
xm_dim_t xm_tensor_get_block_dims(const xm_tensor_t *t, xm_dim_t i) { return xm_block_space_get_block_dims(t->bs, i); }
size_t xm_tensor_get_block_size(const xm_tensor_t *t, xm_dim_t i) { return xm_block_space_get_block_size(t->bs, i); }
size_t xm_tensor_get_block_bytes(const xm_tensor_t *t, xm_dim_t i) { return xm_tensor_get_block_size(t, i) * xm_scalar_sizeof(t->type); }
size_t xm_tensor_get_largest_block_size(const xm_tensor_t *t) { return xm_block_space_get_largest_block_size(t->bs); }
size_t xm_tensor_get_largest_block_bytes(const xm_tensor_t *t) { return xm_tensor_get_largest_block_size(t) * xm_scalar_sizeof(t->type); }
xm_dim_t xm_tensor_get_block_permutation(const xm_tensor_t *t, xm_dim_t i) { return tblk(t, i)->perm; }
xm_scalar_t xm_tensor_get_block_scalar(const xm_tensor_t *t, xm_dim_t i) { return tblk(t, i)->s; }
/* tensor.c:218-229 */
uint64_t
xm_tensor_get_block_data_ptr(const xm_tensor_t *t, xm_dim_t i)
{
	struct blk *b = tblk(t, i);
	if (b->type == XM_BLOCK_TYPE_CANONICAL) return b->data;
	if (b->type == XM_BLOCK_TYPE_DERIVATIVE) return t->b[b->data].data;
	return XM_NULL_PTR;
}
/* tensor.c:243-253 */
void
xm_tensor_set_zero_block(xm_tensor_t *t, xm_dim_t i)
{
	struct blk *b = tblk(t, i);
	b->type = XM_BLOCK_TYPE_ZERO;
	b->perm = xm_dim_identity_permutation(i.n);
	b->s = 0;
	b->data = XM_NULL_PTR;
}
/* tensor.c:53-81 */
xm_tensor_t *
xm_tensor_create(const xm_block_space_t *bs, xm_scalar_type_t type, xm_allocator_t *al)
{
	xm_tensor_t *t = calloc(1, sizeof *t);
	xm_dim_t nb = bs->nblocks, idx = xm_dim_zero(nb.n);
	if (!xm_scalar_check_type(type)) FATAL("unexpected scalar type");
	t->type = type;
	t->al = al;
	t->bs = xm_block_space_clone(bs);
	t->b = calloc(xm_dim_dot(&nb), sizeof *t->b);
	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb))
		xm_tensor_set_zero_block(t, idx);
	return t;
}
/* tensor.c:270-285 */
void
xm_tensor_set_canonical_block_raw(xm_tensor_t *t, xm_dim_t i, uint64_t p)
{
	struct blk *b;
	if (p == XM_NULL_PTR) FATAL("unexpected null data pointer");
	if (xm_tensor_get_block_type(t, i) != XM_BLOCK_TYPE_ZERO) FATAL("block must be zero");
	b = tblk(t, i);
	b->type = XM_BLOCK_TYPE_CANONICAL;
	b->perm = xm_dim_identity_permutation(i.n);
	b->s = 1;
	b->data = p;
}
/* tensor.c:255-268 */
void
xm_tensor_set_canonical_block(xm_tensor_t *t, xm_dim_t i)
{
	uint64_t p;
	if (xm_tensor_get_block_type(t, i) != XM_BLOCK_TYPE_ZERO) FATAL("block must be zero");
	p = xm_allocator_allocate(t->al, xm_tensor_get_block_bytes(t, i));
	if (p == XM_NULL_PTR) FATAL("unable to allocate block data");
	xm_tensor_set_canonical_block_raw(t, i, p);
}
xm_tensor_t *
xm_tensor_create_canonical(const xm_block_space_t *bs, xm_scalar_type_t type, xm_allocator_t *al)
{
	xm_tensor_t *t = xm_tensor_create(bs, type, al);
	xm_dim_t nb = bs->nblocks, idx = xm_dim_zero(nb.n);
	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb))
		xm_tensor_set_canonical_block(t, idx);
	return t;
}
/* tensor.c:100-122 */
xm_tensor_t *
xm_tensor_create_structure(const xm_tensor_t *src, xm_scalar_type_t type, xm_allocator_t *al)
{
	xm_tensor_t *t = xm_tensor_create(src->bs, type, al ? al : src->al);
	xm_dim_t nb = src->bs->nblocks, idx = xm_dim_zero(nb.n);
	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb)) {
		size_t o = xm_dim_offset(&idx, &nb);
		t->b[o] = src->b[o];
		if (t->b[o].type == XM_BLOCK_TYPE_CANONICAL) {
			t->b[o].type = XM_BLOCK_TYPE_ZERO;
			xm_tensor_set_canonical_block(t, idx);
		}
	}
	return t;
}
/* tensor.c:287-311 */
void
xm_tensor_set_derivative_block(xm_tensor_t *t, xm_dim_t i, xm_dim_t src,
    xm_dim_t perm, xm_scalar_t s)
{
	xm_dim_t d1, d2, nb = t->bs->nblocks;
	struct blk *b;
	if (xm_tensor_get_block_type(t, i) != XM_BLOCK_TYPE_ZERO) FATAL("block must be zero");
	if (xm_tensor_get_block_type(t, src) != XM_BLOCK_TYPE_CANONICAL)
		FATAL("derivative blocks must have canonical source blocks");
	d1 = xm_block_space_get_block_dims(t->bs, i);
	d1 = xm_dim_permute(&d1, &perm);
	d2 = xm_block_space_get_block_dims(t->bs, src);
	if (xm_dim_ne(&d1, &d2)) FATAL("invalid block permutation");
	b = tblk(t, i);
	b->type = XM_BLOCK_TYPE_DERIVATIVE;
	b->perm = perm;
	b->s = s;
	b->data = xm_dim_offset(&src, &nb);
}
/* tensor.c:313-336 */
void
xm_tensor_get_canonical_block_list(const xm_tensor_t *t, xm_dim_t **list, size_t *n)
{
	xm_dim_t nb = t->bs->nblocks, idx = xm_dim_zero(nb.n), *l = NULL;
	size_t c = 0;
	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb))
		if (xm_tensor_get_block_type(t, idx) == XM_BLOCK_TYPE_CANONICAL) {
			l = realloc(l, (c + 1) * sizeof *l);
			l[c++] = idx;
		}
	*list = l;
	*n = c;
}
/* tensor.c:338-366 */
void
xm_tensor_read_block(const xm_tensor_t *t, xm_dim_t i, void *buf)
{
	if (xm_tensor_get_block_type(t, i) == XM_BLOCK_TYPE_ZERO) FATAL("cannot read data from zero-blocks");
	xm_allocator_read(t->al, xm_tensor_get_block_data_ptr(t, i), buf, xm_tensor_get_block_bytes(t, i));
}
void
xm_tensor_write_block(xm_tensor_t *t, xm_dim_t i, const void *buf)
{
	if (xm_tensor_get_block_type(t, i) != XM_BLOCK_TYPE_CANONICAL) FATAL("can only write to canonical blocks");
	xm_allocator_write(t->al, xm_tensor_get_block_data_ptr(t, i), buf, xm_tensor_get_block_bytes(t, i));
}
/* tensor.c:154-178 */
xm_scalar_t
xm_tensor_get_element(const xm_tensor_t *t, xm_dim_t idx)
{
	xm_dim_t bi, el, d;
	struct blk *b;
	void *buf;
	xm_scalar_t v;
	xm_block_space_decompose_index(t->bs, idx, &bi, &el);
	b = tblk(t, bi);
	if (b->type == XM_BLOCK_TYPE_ZERO) return 0;
	el = xm_dim_permute(&el, &b->perm);
	d = xm_block_space_get_block_dims(t->bs, bi);
	d = xm_dim_permute(&d, &b->perm);
	buf = malloc(xm_tensor_get_block_bytes(t, bi));
	xm_tensor_read_block(t, bi, buf);
	v = get_el(buf, xm_dim_offset(&el, &d), t->type);
	free(buf);
	return xm_scalar_mul(b->s, v, t->type);
}
/*
 * tensor.c:572-639 (unfold) / 436-505 (fold), restated: the first mask_i
 * position is the lead run; each run of lead_n elements is one memcpy when
 * the run is unit-stride in the block data, else a strided element loop.
 * unfold: to[j*stride + i] = from[offset(permute(el, perm), permute(dims, perm))]
 * fold:   to[offset(el, dims)] = from[j*stride + i]    (canonical blocks only)
 */
static void
fold_unfold(const xm_tensor_t *t, xm_dim_t bi, xm_dim_t mi, xm_dim_t mj,
    const void *from, void *to, size_t stride, int unfold)
{
	xm_dim_t d, dp, el, pe, perm;
	size_t ni, nj, esz, inc = 1, lead_n = 1;
	if (from == NULL || to == NULL || from == to) FATAL("invalid argument");
	if (mi.n + mj.n != bi.n) FATAL("invalid mask dimensions");
	if (!unfold && xm_tensor_get_block_type(t, bi) != XM_BLOCK_TYPE_CANONICAL)
		FATAL("can only fold canonical blocks");
	d = xm_block_space_get_block_dims(t->bs, bi);
	perm = unfold ? tblk(t, bi)->perm : xm_dim_identity_permutation(d.n);
	ni = xm_dim_dot_mask(&d, &mi);
	nj = xm_dim_dot_mask(&d, &mj);
	esz = xm_scalar_sizeof(t->type);
	dp = xm_dim_permute(&d, &perm);
	el = xm_dim_zero(d.n);
	if (mi.n > 0) {
		size_t lead = mi.i[0];
		for (size_t q = 0; q < perm.i[lead]; q++)
			inc *= dp.i[q];
		lead_n = d.i[lead];
		for (size_t q = 0; q + 1 < mi.n; q++)
			mi.i[q] = mi.i[q + 1];
		mi.n--;
	}
	for (size_t j = 0; j < nj; j++) {
		xm_dim_zero_mask(&el, &mi);
		for (size_t i = 0; i < ni; i += lead_n) {
			pe = xm_dim_permute(&el, &perm);
			size_t o = xm_dim_offset(&pe, &dp), m = j * stride + i;
			char *dst; const char *src;
			if (inc == 1) {
				if (unfold) { dst = (char *)to + m * esz; src = (const char *)from + o * esz; }
				else { dst = (char *)to + o * esz; src = (const char *)from + m * esz; }
				memcpy(dst, src, lead_n * esz);
			} else if (unfold) {
				for (size_t q = 0; q < lead_n; q++)
					memcpy((char *)to + (m + q) * esz, (const char *)from + (o + q * inc) * esz, esz);
			} else {
				for (size_t q = 0; q < lead_n; q++)
					memcpy((char *)to + (o + q * inc) * esz, (const char *)from + (m + q) * esz, esz);
			}
			xm_dim_inc_mask(&el, &d, &mi);
		}
		xm_dim_inc_mask(&el, &d, &mj);
	}
}
void xm_tensor_unfold_block(const xm_tensor_t *t, xm_dim_t bi, xm_dim_t mi, xm_dim_t mj, const void *from, void *to, size_t stride)
{ fold_unfold(t, bi, mi, mj, from, to, stride, 1); }
void xm_tensor_fold_block(const xm_tensor_t *t, xm_dim_t bi, xm_dim_t mi, xm_dim_t mj, const void *from, void *to, size_t stride)
{ fold_unfold(t, bi, mi, mj, from, to, stride, 0); }
/* tensor.c:641-669 */
void
xm_tensor_free_block_data(xm_tensor_t *t)
{
	xm_dim_t nb = t->bs->nblocks, idx = xm_dim_zero(nb.n);
	for (; xm_dim_ne(&idx, &nb); xm_dim_inc(&idx, &nb)) {
		if (xm_tensor_get_block_type(t, idx) == XM_BLOCK_TYPE_CANONICAL)
			xm_allocator_deallocate(t->al, xm_tensor_get_block_data_ptr(t, idx));
		xm_tensor_set_zero_block(t, idx);
	}
}
void xm_tensor_free(xm_tensor_t *t) { if (!t) return; xm_block_space_free(t->bs); free(t->b); free(t); }

/* ---- scalar.c:123-414 (host vector loops) ---- */
void xm_scalar_set(void *x, xm_scalar_t a, size_t n, xm_scalar_type_t t)
{ for (size_t i = 0; i < n; i++) set_el(x, i, a, t); }
void xm_scalar_scale(void *x, xm_scalar_t a, size_t n, xm_scalar_type_t t)
{ a = xm_scalar_mul(a, 1, t); for (size_t i = 0; i < n; i++) set_el(x, i, xm_scalar_mul(a, get_el(x, i, t), t), t); }
void xm_scalar_axpy(void *x, xm_scalar_t a, const void *y, xm_scalar_t b, size_t n, xm_scalar_type_t t)
{ for (size_t i = 0; i < n; i++) set_el(x, i, xm_scalar_add(xm_scalar_mul(a, get_el(x, i, t), t), xm_scalar_mul(b, get_el(y, i, t), t), t), t); }
void xm_scalar_vec_mul(void *x, xm_scalar_t a, const void *y, size_t n, xm_scalar_type_t t)
{ for (size_t i = 0; i < n; i++) set_el(x, i, xm_scalar_mul(xm_scalar_mul(a, get_el(x, i, t), t), get_el(y, i, t), t), t); }
void xm_scalar_vec_div(void *x, xm_scalar_t a, const void *y, size_t n, xm_scalar_type_t t)
{ for (size_t i = 0; i < n; i++) set_el(x, i, get_el(x, i, t) / xm_scalar_mul(a, get_el(y, i, t), t), t); }
xm_scalar_t xm_scalar_dot(const void *x, const void *y, size_t n, xm_scalar_type_t t)
{ xm_scalar_t s = 0; for (size_t i = 0; i < n; i++) s = xm_scalar_add(s, xm_scalar_mul(get_el(x, i, t), get_el(y, i, t), t), t); return s; }
void xm_scalar_convert(void *x, const void *y, size_t n, xm_scalar_type_t xt, xm_scalar_type_t yt)
{
	if ((xt & 1) != (yt & 1)) FATAL("unsupported scalar conversion");
	for (size_t i = 0; i < n; i++) set_el(x, i, get_el(y, i, yt), xt);
}

/* ---- GEMM back end ------------------------------------------------ */
typedef void (*gemm_fn)(const char *, const char *, const long *, const long *,
    const long *, const void *, const void *, const long *, const void *,
    const long *, const void *, void *, const long *, size_t, size_t);
static gemm_fn blas[4];		/* s, c, d, z by scalar type */
static int blas_tried;

/* Point the oracle at an ILP64 BLAS exporting scipy_?gemm_64_ (numpy's
 * bundled OpenBLAS).  Returns 1 when found, 0 when the C loop is used. */
int
xmo_set_blas(const char *path)
{
	static const char *nm[4] = {"scipy_sgemm_64_", "scipy_cgemm_64_",
	    "scipy_dgemm_64_", "scipy_zgemm_64_"};
	void *h;
	blas_tried = 1;
	if (path == NULL || (h = dlopen(path, RTLD_NOW | RTLD_LOCAL)) == NULL)
		return 0;
	for (int k = 0; k < 4; k++)
		if ((blas[k] = (gemm_fn)dlsym(h, nm[k])) == NULL)
			return 0;
	return 1;
}
int xmo_blas_available(void) { return blas[2] != NULL; }

/* C[m x n] (ld m) += al * A^T B with A k x m (ld k), B k x n (ld k):
 * the reference's xgemm('T','N', ...) call (contract.c:49-84, 207-216). */
static void
xgemm_tn(long m, long n, long k, xm_scalar_t al, const void *A, const void *B,
    void *C, long ldc, xm_scalar_type_t t)
{
	if (blas[t]) {
		float fa = (float)al; float complex ca = (float complex)al;
		double da = (double)al; double complex za = al;
		float f1 = 1; float complex c1 = 1; double d1 = 1; double complex z1 = 1;
		const void *pa = t == 0 ? (void *)&fa : t == 1 ? (void *)&ca : t == 2 ? (void *)&da : (void *)&za;
		const void *p1 = t == 0 ? (void *)&f1 : t == 1 ? (void *)&c1 : t == 2 ? (void *)&d1 : (void *)&z1;
		blas[t]("T", "N", &m, &n, &k, pa, A, &k, B, &k, p1, C, &ldc, 1, 1);
		return;
	}
	for (long j = 0; j < n; j++)
		for (long i = 0; i < m; i++) {
			xm_scalar_t s = 0;
			for (long q = 0; q < k; q++)
				s += get_el(A, (size_t)(q + i * k), t) * get_el(B, (size_t)(q + j * k), t);
			set_el(C, (size_t)(i + j * ldc), xm_scalar_add(get_el(C, (size_t)(i + j * ldc), t),
			    xm_scalar_mul(al, xm_scalar_mul(s, 1, t), t), t), t);
		}
}

/* ---- xm.c: set / copy / add / mul / div / dot --------------------- */
/* xm.c:28-64 */
void
xm_set(xm_tensor_t *a, xm_scalar_t x)
{
	xm_dim_t *l; size_t n;
	void *buf = malloc(xm_tensor_get_largest_block_bytes(a));
	xm_scalar_set(buf, x, xm_tensor_get_largest_block_size(a), a->type);
	xm_tensor_get_canonical_block_list(a, &l, &n);
	for (size_t i = 0; i < n; i++)
		xm_tensor_write_block(a, l[i], buf);
	free(l);
	free(buf);
}

static void
pair_check(const xm_tensor_t *a, const xm_tensor_t *b, const char *ia,
    const char *ib, xm_dim_t *ca, xm_dim_t *cb, int sametype)
{
	if (a->al != b->al) xm_fatal("tensors must use same allocator");
	if (sametype && a->type != b->type) xm_fatal("tensors must have same scalar type");
	if (strlen(ia) != a->bs->dims.n) xm_fatal("idxa does not match tensor dimensions");
	if (strlen(ib) != b->bs->dims.n) xm_fatal("idxb does not match tensor dimensions");
	xm_make_masks(ia, ib, ca, cb);
	if (ca->n != a->bs->dims.n || cb->n != b->bs->dims.n) xm_fatal("index spaces do not match");
	for (size_t k = 0; k < ca->n; k++)
		if (!xm_block_space_eq1(a->bs, ca->i[k], b->bs, cb->i[k]))
			xm_fatal("inconsistent block-spaces");
}

enum { K_COPY, K_ADD, K_MUL, K_DIV };

/* xm.c:66-157, 159-249, 251-332, 334-413 */
static void
two(int kind, xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb)
{
	xm_dim_t ca, cb, *l, zero = xm_dim_zero(0);
	size_t n, mx = xm_tensor_get_largest_block_size(a);
	pair_check(a, b, idxa, idxb, &ca, &cb, kind != K_COPY);
	xm_tensor_get_canonical_block_list(a, &l, &n);
#pragma omp parallel for schedule(dynamic)
	for (size_t q = 0; q < n; q++) {
		xm_dim_t ia = l[q], ib = xm_dim_zero(cb.n);
		size_t bs = 16 * mx + 16;
		void *b1 = malloc(bs), *b2 = malloc(bs), *b3 = malloc(bs);
		size_t sz;
		struct blk *bb;
		xm_dim_set_mask(&ib, &cb, &ia, &ca);
		sz = xm_tensor_get_block_size(b, ib);
		bb = tblk(b, ib);
		switch (kind) {
		case K_COPY:
			if (alpha == 0 || bb->type == XM_BLOCK_TYPE_ZERO)
				memset(b2, 0, bs);
			else {
				xm_scalar_t s = xm_scalar_mul(alpha, bb->s, b->type);
				xm_tensor_read_block(b, ib, b2);
				xm_tensor_unfold_block(b, ib, cb, zero, b2, b1, sz);
				xm_scalar_scale(b1, s, sz, b->type);
				xm_scalar_convert(b3, b1, sz, a->type, b->type);
				xm_tensor_fold_block(a, ia, ca, zero, b3, b2, sz);
			}
			xm_tensor_write_block(a, ia, b2);
			break;
		case K_ADD:
			if (beta == 0 || bb->type == XM_BLOCK_TYPE_ZERO)
				memset(b2, 0, bs);
			else {
				xm_scalar_t s = xm_scalar_mul(beta, bb->s, a->type);
				xm_tensor_read_block(b, ib, b2);
				xm_tensor_unfold_block(b, ib, cb, zero, b2, b1, sz);
				xm_scalar_scale(b1, s, sz, a->type);
				xm_tensor_fold_block(a, ia, ca, zero, b1, b2, sz);
			}
			if (alpha == 0)
				xm_tensor_write_block(a, ia, b2);
			else {
				xm_tensor_read_block(a, ia, b1);
				xm_scalar_axpy(b1, alpha, b2, 1, sz, a->type);
				xm_tensor_write_block(a, ia, b1);
			}
			break;
		case K_MUL:
		case K_DIV:
			if (bb->type == XM_BLOCK_TYPE_ZERO) {
				if (kind == K_DIV) xm_fatal("division by zero");
				memset(b1, 0, bs);
			} else {
				/* b's unfold is in b's index order; fold it into
				 * a's order before the element-wise op */
				xm_tensor_read_block(b, ib, b1);
				xm_tensor_unfold_block(b, ib, cb, zero, b1, b2, sz);
				xm_tensor_fold_block(a, ia, ca, zero, b2, b3, sz);
				xm_tensor_read_block(a, ia, b1);
				if (kind == K_MUL)
					xm_scalar_vec_mul(b1, bb->s, b3, sz, a->type);
				else
					xm_scalar_vec_div(b1, bb->s, b3, sz, a->type);
			}
			xm_tensor_write_block(a, ia, b1);
			break;
		}
		free(b1); free(b2); free(b3);
	}
	free(l);
}
void xm_copy(xm_tensor_t *a, xm_scalar_t s, const xm_tensor_t *b, const char *ia, const char *ib) { two(K_COPY, s, a, 0, b, ia, ib); }
void xm_add(xm_scalar_t al, xm_tensor_t *a, xm_scalar_t be, const xm_tensor_t *b, const char *ia, const char *ib) { two(K_ADD, al, a, be, b, ia, ib); }
void xm_mul(xm_tensor_t *a, const xm_tensor_t *b, const char *ia, const char *ib) { two(K_MUL, 0, a, 0, b, ia, ib); }
void xm_div(xm_tensor_t *a, const xm_tensor_t *b, const char *ia, const char *ib) { two(K_DIV, 0, a, 0, b, ia, ib); }

/* xm.c:415-508: every block index of a, both blocks nonzero */
xm_scalar_t
xm_dot(const xm_tensor_t *a, const xm_tensor_t *b, const char *idxa, const char *idxb)
{
	xm_dim_t ca, cb, nb = a->bs->nblocks, zero = xm_dim_zero(0);
	size_t nblk = xm_dim_dot(&nb), mx = xm_tensor_get_largest_block_bytes(a);
	xm_scalar_t dot = 0;
	pair_check(a, b, idxa, idxb, &ca, &cb, 1);
	void *b1 = malloc(mx), *b2 = malloc(mx), *b3 = malloc(mx);
	for (size_t i = 0; i < nblk; i++) {
		xm_dim_t ia = xm_dim_from_offset(i, &nb), ib = xm_dim_zero(cb.n);
		xm_dim_set_mask(&ib, &cb, &ia, &ca);
		if (tblk(a, ia)->type == XM_BLOCK_TYPE_ZERO || tblk(b, ib)->type == XM_BLOCK_TYPE_ZERO)
			continue;
		size_t sz = xm_tensor_get_block_size(b, ib);
		xm_tensor_read_block(b, ib, b1);
		xm_tensor_unfold_block(b, ib, cb, zero, b1, b2, sz);
		xm_tensor_read_block(a, ia, b1);
		xm_tensor_unfold_block(a, ia, ca, zero, b1, b3, sz);
		xm_scalar_t s = xm_scalar_mul(tblk(a, ia)->s, tblk(b, ib)->s, a->type);
		s = xm_scalar_mul(s, xm_scalar_dot(b2, b3, sz, a->type), a->type);
		dot = xm_scalar_add(dot, s, a->type);
	}
	free(b1); free(b2); free(b3);
	return dot;
}

/* ---- contract.c:86-314 -------------------------------------------- */
struct pair { xm_dim_t ia, ib; xm_scalar_t al; };

/* contract.c:86-115 */
static int
same_contraction(const struct pair *p, size_t i, size_t j, xm_dim_t aa,
    xm_dim_t ab, const xm_tensor_t *a, const xm_tensor_t *b)
{
	if (xm_tensor_get_block_data_ptr(a, p[i].ia) != xm_tensor_get_block_data_ptr(a, p[j].ia) ||
	    xm_tensor_get_block_data_ptr(b, p[i].ib) != xm_tensor_get_block_data_ptr(b, p[j].ib))
		return 0;
	xm_dim_t pia = tblk(a, p[i].ia)->perm, pja = tblk(a, p[j].ia)->perm;
	xm_dim_t pib = tblk(b, p[i].ib)->perm, pjb = tblk(b, p[j].ib)->perm;
	for (size_t k = 0; k < aa.n; k++)
		if (pia.i[aa.i[k]] != pja.i[aa.i[k]]) return 0;
	for (size_t k = 0; k < ab.n; k++)
		if (pib.i[ab.i[k]] != pjb.i[ab.i[k]]) return 0;
	return 1;
}

/* Pair-list hook: when set, every surviving pair of every canonical C
 * block is reported (block list index, pair factor, m, n, k) so tests can
 * compare block structure across implementations. */
typedef void (*xmo_pair_cb)(size_t cblock, double re, double im, long m, long n, long k);
static xmo_pair_cb pair_cb;
static int plan_only;
void xmo_set_pair_callback(xmo_pair_cb cb) { pair_cb = cb; }
/* With plan_only set, xm_contract enumerates and reports pairs but reads,
 * computes and writes nothing (structure comparisons on big grids). */
void xmo_set_plan_only(int on) { plan_only = on; }

/* contract.c:117-225 */
static void
compute_block(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, xm_dim_t cidxa, xm_dim_t aidxa,
    xm_dim_t cidxb, xm_dim_t aidxb, xm_dim_t cidxc, xm_dim_t aidxc,
    xm_dim_t bc, size_t lidx, struct pair *pr, char *buf)
{
	size_t mxa = xm_tensor_get_largest_block_bytes(a), mxb = xm_tensor_get_largest_block_bytes(b);
	size_t mxc = xm_tensor_get_largest_block_bytes(c);
	char *a1 = buf, *a2 = a1 + mxa, *b1 = a2 + mxa, *b2 = b1 + mxb, *c1 = b2 + mxb, *c2 = c1 + mxc;
	xm_scalar_type_t t = c->type;
	xm_dim_t nba = a->bs->nblocks, nbb = b->bs->nblocks, d, ia, ib;
	size_t nk = xm_dim_dot_mask(&nba, &cidxa), m, n, k;
	int ctrans = aidxc.n > 0 && aidxc.i[0] == 0;

	d = xm_tensor_get_block_dims(c, bc);
	m = xm_dim_dot_mask(&d, &cidxc);
	n = xm_dim_dot_mask(&d, &aidxc);
	if (plan_only)
		goto pairs;
	xm_tensor_read_block(c, bc, c2);
	if (ctrans) xm_tensor_unfold_block(c, bc, aidxc, cidxc, c2, c1, n);
	else xm_tensor_unfold_block(c, bc, cidxc, aidxc, c2, c1, m);
	if (beta == 0) xm_scalar_set(c1, 0, m * n, t);
	else xm_scalar_scale(c1, beta, m * n, t);
pairs:
	if (alpha != 0) {
		ia = xm_dim_zero(nba.n);
		ib = xm_dim_zero(nbb.n);
		xm_dim_set_mask(&ia, &aidxa, &bc, &cidxc);
		xm_dim_set_mask(&ib, &aidxb, &bc, &aidxc);
		for (size_t i = 0; i < nk; i++) {
			pr[i].ia = ia; pr[i].ib = ib; pr[i].al = 0;
			if (tblk(a, ia)->type != XM_BLOCK_TYPE_ZERO && tblk(b, ib)->type != XM_BLOCK_TYPE_ZERO)
				pr[i].al = xm_scalar_mul(tblk(a, ia)->s, tblk(b, ib)->s, t);
			xm_dim_inc_mask(&ia, &nba, &cidxa);
			xm_dim_inc_mask(&ib, &nbb, &cidxb);
		}
		for (size_t i = 0; i < nk; i++) {
			if (pr[i].al == 0) continue;
			for (size_t j = i + 1; j < nk; j++) {
				if (pr[j].al == 0) continue;
				if (same_contraction(pr, i, j, aidxa, aidxb, a, b)) {
					pr[i].al = xm_scalar_add(pr[i].al, pr[j].al, t);
					pr[j].al = 0;
				}
			}
		}
		for (size_t i = 0; i < nk; i++) {
			if (pr[i].al == 0) continue;
			d = xm_tensor_get_block_dims(a, pr[i].ia);
			k = xm_dim_dot_mask(&d, &cidxa);
			if (plan_only) {
				if (pair_cb)
					pair_cb(lidx, creal(pr[i].al), cimag(pr[i].al), (long)m, (long)n, (long)k);
				continue;
			}
			xm_tensor_read_block(a, pr[i].ia, a1);
			xm_tensor_unfold_block(a, pr[i].ia, cidxa, aidxa, a1, a2, k);
			xm_tensor_read_block(b, pr[i].ib, b1);
			xm_tensor_unfold_block(b, pr[i].ib, cidxb, aidxb, b1, b2, k);
			xm_scalar_t al = xm_scalar_mul(alpha, pr[i].al, t);
			if (pair_cb)
				pair_cb(lidx, creal(pr[i].al), cimag(pr[i].al), (long)m, (long)n, (long)k);
			if (ctrans) xgemm_tn((long)n, (long)m, (long)k, al, b2, a2, c1, (long)n, t);
			else xgemm_tn((long)m, (long)n, (long)k, al, a2, b2, c1, (long)m, t);
		}
	}
	if (plan_only)
		return;
	if (ctrans) xm_tensor_fold_block(c, bc, aidxc, cidxc, c1, c2, n);
	else xm_tensor_fold_block(c, bc, cidxc, aidxc, c1, c2, m);
	xm_tensor_write_block(c, bc, c2);
}

/* contract.c:227-314 */
void
xm_contract(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc)
{
	xm_dim_t cidxa, aidxa, cidxb, aidxb, cidxc, aidxc, *l, nba;
	size_t nl, nk, bufb;
	if (a->al != c->al || b->al != c->al) xm_fatal("xm_contract: tensors must use same allocator");
	if (a->type != c->type || b->type != c->type) xm_fatal("xm_contract: tensors must have same scalar type");
	if (strlen(idxa) != a->bs->dims.n || strlen(idxb) != b->bs->dims.n || strlen(idxc) != c->bs->dims.n)
		xm_fatal("xm_contract: bad contraction indices");
	xm_make_masks(idxa, idxb, &cidxa, &cidxb);
	xm_make_masks(idxc, idxa, &cidxc, &aidxa);
	xm_make_masks(idxc, idxb, &aidxc, &aidxb);
	if (aidxa.n + cidxa.n != a->bs->dims.n || aidxb.n + cidxb.n != b->bs->dims.n ||
	    aidxc.n + cidxc.n != c->bs->dims.n)
		xm_fatal("xm_contract: bad contraction indices");
	if (!(aidxc.n > 0 && aidxc.i[0] == 0) && !(cidxc.n > 0 && cidxc.i[0] == 0))
		xm_fatal("xm_contract: bad contraction indices");
	for (size_t i = 0; i < cidxa.n; i++)
		if (!xm_block_space_eq1(a->bs, cidxa.i[i], b->bs, cidxb.i[i]))
			xm_fatal("xm_contract: inconsistent a and b tensor block-spaces");
	for (size_t i = 0; i < cidxc.n; i++)
		if (!xm_block_space_eq1(c->bs, cidxc.i[i], a->bs, aidxa.i[i]))
			xm_fatal("xm_contract: inconsistent a and c tensor block-spaces");
	for (size_t i = 0; i < aidxc.n; i++)
		if (!xm_block_space_eq1(c->bs, aidxc.i[i], b->bs, aidxb.i[i]))
			xm_fatal("xm_contract: inconsistent b and c tensor block-spaces");
	nba = a->bs->nblocks;
	nk = xm_dim_dot_mask(&nba, &cidxa);
	bufb = 2 * (xm_tensor_get_largest_block_bytes(a) + xm_tensor_get_largest_block_bytes(b) +
	    xm_tensor_get_largest_block_bytes(c));
	xm_tensor_get_canonical_block_list(c, &l, &nl);
#pragma omp parallel
	{
		struct pair *pr = malloc((nk ? nk : 1) * sizeof *pr);
		char *buf = malloc(bufb);
#pragma omp for schedule(dynamic)
		for (size_t i = 0; i < nl; i++)
			compute_block(alpha, a, b, beta, c, cidxa, aidxa, cidxb, aidxb,
			    cidxc, aidxc, l[i], i, pr, buf);
		free(pr);
		free(buf);
	}
	free(l);
}

void xm_print_banner(void) { printf("libxm oracle (CPU restatement, test use only)\n"); }

/* Run only the canonical output blocks whose list positions are in
 * [first, first+count): a bounded sample of a contraction for CPU-baseline
 * timing.  Same algorithm as xm_contract. */
void
xmo_contract_range(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, size_t first, size_t count)
{
	xm_dim_t cidxa, aidxa, cidxb, aidxb, cidxc, aidxc, *l, nba;
	size_t nl, nk, bufb, end;
	xm_make_masks(idxa, idxb, &cidxa, &cidxb);
	xm_make_masks(idxc, idxa, &cidxc, &aidxa);
	xm_make_masks(idxc, idxb, &aidxc, &aidxb);
	nba = a->bs->nblocks;
	nk = xm_dim_dot_mask(&nba, &cidxa);
	bufb = 2 * (xm_tensor_get_largest_block_bytes(a) + xm_tensor_get_largest_block_bytes(b) +
	    xm_tensor_get_largest_block_bytes(c));
	xm_tensor_get_canonical_block_list(c, &l, &nl);
	end = first + count < nl ? first + count : nl;
#pragma omp parallel
	{
		struct pair *pr = malloc((nk ? nk : 1) * sizeof *pr);
		char *buf = malloc(bufb);
#pragma omp for schedule(dynamic)
		for (size_t i = first; i < end; i++)
			compute_block(alpha, a, b, beta, c, cidxa, aidxa, cidxb, aidxb,
			    cidxc, aidxc, l[i], i, pr, buf);
		free(pr);
		free(buf);
	}
	free(l);
}

int xmo_num_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}
