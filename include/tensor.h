/*
 * libxm-gb300: block tensors.
 *
 * Same declarations as the reference's src/tensor.h:32-259.  Every block is
 * zero (no data), canonical (owns data) or derivative (a permuted, scaled view
 * of a canonical block of the same tensor).  Block data buffers passed to
 * read/write/unfold/fold are host memory, as in the reference; unfold/fold
 * also accept device pointers and then run entirely on the GPU.
 */
#ifndef TENSOR_H_INCLUDED
#define TENSOR_H_INCLUDED

#include "alloc.h"
#include "blockspace.h"
#include "scalar.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Enumerator values 0..2 are part of the ABI (tensor.h:32-39). */
typedef enum {
	XM_BLOCK_TYPE_ZERO = 0,
	XM_BLOCK_TYPE_CANONICAL,
	XM_BLOCK_TYPE_DERIVATIVE,
} xm_block_type_t;

typedef struct xm_tensor xm_tensor_t;

/* All blocks zero; the block space is cloned (tensor.c:53-81). */
xm_tensor_t *xm_tensor_create(const xm_block_space_t *bs, xm_scalar_type_t type,
    xm_allocator_t *allocator);
/* All blocks canonical (tensor.c:83-98). */
xm_tensor_t *xm_tensor_create_canonical(const xm_block_space_t *bs,
    xm_scalar_type_t type, xm_allocator_t *allocator);
/* Same block structure, fresh canonical storage; allocator NULL means the
 * source tensor's allocator (tensor.c:100-122). */
xm_tensor_t *xm_tensor_create_structure(const xm_tensor_t *tensor,
    xm_scalar_type_t type, xm_allocator_t *allocator);
const xm_block_space_t *xm_tensor_get_block_space(const xm_tensor_t *tensor);
xm_scalar_type_t xm_tensor_get_scalar_type(const xm_tensor_t *tensor);
xm_allocator_t *xm_tensor_get_allocator(const xm_tensor_t *tensor);
xm_dim_t xm_tensor_get_abs_dims(const xm_tensor_t *tensor);
xm_dim_t xm_tensor_get_nblocks(const xm_tensor_t *tensor);
/* Element at an absolute index, block scalar applied (tensor.c:154-178). */
xm_scalar_t xm_tensor_get_element(const xm_tensor_t *tensor, xm_dim_t idx);
xm_block_type_t xm_tensor_get_block_type(const xm_tensor_t *tensor,
    xm_dim_t blkidx);
xm_dim_t xm_tensor_get_block_dims(const xm_tensor_t *tensor, xm_dim_t blkidx);
size_t xm_tensor_get_block_size(const xm_tensor_t *tensor, xm_dim_t blkidx);
size_t xm_tensor_get_block_bytes(const xm_tensor_t *tensor, xm_dim_t blkidx);
size_t xm_tensor_get_largest_block_size(const xm_tensor_t *tensor);
size_t xm_tensor_get_largest_block_bytes(const xm_tensor_t *tensor);
/* Data handle of the block or of its source; XM_NULL_PTR for zero blocks
 * (tensor.c:218-229). */
uint64_t xm_tensor_get_block_data_ptr(const xm_tensor_t *tensor,
    xm_dim_t blkidx);
xm_dim_t xm_tensor_get_block_permutation(const xm_tensor_t *tensor,
    xm_dim_t blkidx);
xm_scalar_t xm_tensor_get_block_scalar(const xm_tensor_t *tensor,
    xm_dim_t blkidx);
void xm_tensor_set_zero_block(xm_tensor_t *tensor, xm_dim_t blkidx);
/* Block must be zero; allocates its storage (tensor.c:255-268). */
void xm_tensor_set_canonical_block(xm_tensor_t *tensor, xm_dim_t blkidx);
void xm_tensor_set_canonical_block_raw(xm_tensor_t *tensor, xm_dim_t blkidx,
    uint64_t data_ptr);
/* Block must be zero, source canonical, and
 * permute(dims(blkidx), permutation) == dims(source) (tensor.c:287-311). */
void xm_tensor_set_derivative_block(xm_tensor_t *tensor, xm_dim_t blkidx,
    xm_dim_t source_blkidx, xm_dim_t permutation, xm_scalar_t scalar);
/* Canonical blocks in index-0-fastest order; free() the list
 * (tensor.c:313-336). */
void xm_tensor_get_canonical_block_list(const xm_tensor_t *tensor,
    xm_dim_t **blklist, size_t *nblklist);
void xm_tensor_read_block(const xm_tensor_t *tensor, xm_dim_t blkidx,
    void *buf);
/* Only canonical blocks can be written (tensor.c:353-366). */
void xm_tensor_write_block(xm_tensor_t *tensor, xm_dim_t blkidx,
    const void *buf);
/* to[j*stride + i] = from[canonical offset of element (i, j)], with i
 * running over mask_i dimensions and j over mask_j dimensions, the block's
 * permutation applied, and its scalar NOT applied (tensor.c:572-639). */
void xm_tensor_unfold_block(const xm_tensor_t *tensor, xm_dim_t blkidx,
    xm_dim_t mask_i, xm_dim_t mask_j, const void *from, void *to,
    size_t stride);
/* Inverse of unfold, canonical blocks only (tensor.c:436-505). */
void xm_tensor_fold_block(const xm_tensor_t *tensor, xm_dim_t blkidx,
    xm_dim_t mask_i, xm_dim_t mask_j, const void *from, void *to,
    size_t stride);
/* Deallocate all canonical data and reset every block to zero. */
void xm_tensor_free_block_data(xm_tensor_t *tensor);
/* Frees metadata only (tensor.c:661-669). */
void xm_tensor_free(xm_tensor_t *tensor);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* TENSOR_H_INCLUDED */
