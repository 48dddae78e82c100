/*
 * libxm-gb300: multidimensional index algebra.
 *
 * Same declarations as the reference's src/dim.h (dim.h:30-199) so that
 * existing C callers compile and link unchanged.  Layout convention: index 0
 * is the fastest-varying one (dim.c:201-230).
 */
#ifndef XM_DIM_H_INCLUDED
#define XM_DIM_H_INCLUDED

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Maximum number of dimensions (dim.h:30). */
#define XM_MAX_DIM 8

/* Multidimensional index or shape: n used entries of i[] (dim.h:33-38).
 * 72 bytes, passed by value across the ABI. */
typedef struct {
	size_t n;
	size_t i[XM_MAX_DIM];
} xm_dim_t;

xm_dim_t xm_dim_zero(size_t ndim);                 /* dim.h:45 */
xm_dim_t xm_dim_same(size_t ndim, size_t dim);     /* dim.h:51 */
xm_dim_t xm_dim_1(size_t dim1);
xm_dim_t xm_dim_2(size_t dim1, size_t dim2);
xm_dim_t xm_dim_3(size_t dim1, size_t dim2, size_t dim3);
xm_dim_t xm_dim_4(size_t dim1, size_t dim2, size_t dim3, size_t dim4);
xm_dim_t xm_dim_5(size_t dim1, size_t dim2, size_t dim3, size_t dim4,
    size_t dim5);
xm_dim_t xm_dim_6(size_t dim1, size_t dim2, size_t dim3, size_t dim4,
    size_t dim5, size_t dim6);
xm_dim_t xm_dim_7(size_t dim1, size_t dim2, size_t dim3, size_t dim4,
    size_t dim5, size_t dim6, size_t dim7);
xm_dim_t xm_dim_8(size_t dim1, size_t dim2, size_t dim3, size_t dim4,
    size_t dim5, size_t dim6, size_t dim7, size_t dim8);
/* Non-zero when equal / not equal (dim.h:119-129). */
int xm_dim_eq(const xm_dim_t *a, const xm_dim_t *b);
int xm_dim_ne(const xm_dim_t *a, const xm_dim_t *b);
/* Non-zero when every idx->i[k] < dim->i[k] (dim.h:135). */
int xm_dim_less(const xm_dim_t *idx, const xm_dim_t *dim);
/* Product of all entries (dim.h:141). */
size_t xm_dim_dot(const xm_dim_t *dim);
/* Linear offset of idx inside dim, index 0 fastest (dim.h:148). */
size_t xm_dim_offset(const xm_dim_t *idx, const xm_dim_t *dim);
/* Inverse of xm_dim_offset (dim.h:155). */
xm_dim_t xm_dim_from_offset(size_t offset, const xm_dim_t *dim);
/* Increment with carry; past the end idx becomes *dim (dim.h:162). */
void xm_dim_inc(xm_dim_t *idx, const xm_dim_t *dim);
/* dim->i[mask->i[k]] = 0 (dim.h:168). */
void xm_dim_zero_mask(xm_dim_t *dim, const xm_dim_t *mask);
/* a->i[maska->i[k]] = b->i[maskb->i[k]] (dim.h:176). */
void xm_dim_set_mask(xm_dim_t *a, const xm_dim_t *maska, const xm_dim_t *b,
    const xm_dim_t *maskb);
/* Product of dim->i[mask->i[k]] (dim.h:183). */
size_t xm_dim_dot_mask(const xm_dim_t *dim, const xm_dim_t *mask);
/* Increment only the masked positions, first mask entry fastest (dim.h:191). */
void xm_dim_inc_mask(xm_dim_t *idx, const xm_dim_t *dim, const xm_dim_t *mask);
xm_dim_t xm_dim_identity_permutation(size_t ndim);  /* dim.h:196 */
/* ret.i[permutation->i[k]] = idx->i[k] (dim.h:202, dim.c:350-369). */
xm_dim_t xm_dim_permute(const xm_dim_t *idx, const xm_dim_t *permutation);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XM_DIM_H_INCLUDED */
