/*
 * libxm-gb300: block spaces (per-dimension sorted split points).
 *
 * Same declarations as the reference's src/blockspace.h:35-126.
 */
#ifndef XM_BLOCKSPACE_H_INCLUDED
#define XM_BLOCKSPACE_H_INCLUDED

#include "dim.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xm_block_space xm_block_space_t;

/* One block per dimension; NULL on out-of-memory (blockspace.h:38). */
xm_block_space_t *xm_block_space_create(xm_dim_t dims);
/* Deep copy; NULL on out-of-memory (blockspace.h:43). */
xm_block_space_t *xm_block_space_clone(const xm_block_space_t *bs);
/* Deep copy with dimensions permuted (blockspace.h:50). */
xm_block_space_t *xm_block_space_permute_clone(const xm_block_space_t *bs,
    xm_dim_t permutation);
size_t xm_block_space_get_ndims(const xm_block_space_t *bs);
xm_dim_t xm_block_space_get_abs_dims(const xm_block_space_t *bs);
xm_dim_t xm_block_space_get_nblocks(const xm_block_space_t *bs);
/* Idempotent sorted insert of split point x on dimension dim (blockspace.h:72). */
void xm_block_space_split(xm_block_space_t *bs, size_t dim, size_t x);
/* Even splits targeting 32 elements per block (blockspace.h:76). */
void xm_block_space_autosplit(xm_block_space_t *bs);
size_t xm_block_space_get_split(xm_block_space_t *bs, size_t dim, size_t i);
xm_dim_t xm_block_space_get_block_dims(const xm_block_space_t *bs,
    xm_dim_t blkidx);
size_t xm_block_space_get_block_size(const xm_block_space_t *bs,
    xm_dim_t blkidx);
/* Product of the per-dimension maximum block sizes (blockspace.h:104). */
size_t xm_block_space_get_largest_block_size(const xm_block_space_t *bs);
void xm_block_space_decompose_index(const xm_block_space_t *bs, xm_dim_t idx,
    xm_dim_t *blkidx, xm_dim_t *elidx);
int xm_block_space_eq(const xm_block_space_t *bsa, const xm_block_space_t *bsb);
int xm_block_space_eq1(const xm_block_space_t *bsa, size_t dima,
    const xm_block_space_t *bsb, size_t dimb);
/* NULL is allowed (blockspace.h:124). */
void xm_block_space_free(xm_block_space_t *bs);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XM_BLOCKSPACE_H_INCLUDED */
