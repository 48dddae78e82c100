/*
 * Internal declarations shared by the libxm-gb300 host (C) sources.
 * Not installed; the public interface is include/xm.h and include/xmg.h.
 */
#ifndef XMG_HOST_H
#define XMG_HOST_H

#include <complex.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xm.h"
#include "xmg.h"
#include "xmg_dev.h"

/* Private functions also exported for test drivers (util.h:34-35). */
void xm_fatal(const char *fmt, ...) __attribute__((noreturn, format(printf, 1, 2)));
void xm_make_masks(const char *, const char *, xm_dim_t *, xm_dim_t *);

/* Status-code error channel of the xmg_* C-ABI. */
int xmg_seterr(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
void xmg_die_on(int status);

/* Block table entry (tensor.c:26-32 holds the same information). */
struct xmg_block {
	xm_block_type_t type;
	xm_dim_t perm;          /* identity for canonical blocks */
	xm_scalar_t scalar;     /* 1 for canonical, 0 for zero blocks */
	uint64_t data;          /* canonical: allocator handle;
	                           derivative: linear index of the source */
};

struct xm_tensor {
	xm_scalar_type_t type;
	xm_block_space_t *bs;
	xm_allocator_t *allocator;
	struct xmg_block *blocks;
	size_t nblocks_total;
	uint64_t gen;            /* structure generation, unique per change */
};

/* new structure generation for t (block table changed) */
void xmg_tensor_touch(xm_tensor_t *t);

/* release the adjoint's kept intermediates if they live in `al` */
void xmg_adjoint_forget(const xm_allocator_t *al);

/* allocator internals used by the contraction engine */
int xmg_alloc_is_device(const xm_allocator_t *a);
/* blocks in page-locked host memory (xmg_allocator_create_host) */
int xmg_alloc_is_host(const xm_allocator_t *a);
/* Device address holding the bytes of a data handle.  For pagefile
 * allocators the block is staged into an engine-owned HBM buffer first. */
int xmg_alloc_device_view(xm_allocator_t *a, uint64_t handle, size_t bytes,
    uint64_t *dptr);
int xmg_alloc_release_views(xm_allocator_t *a, int write_back);
/* read-only mapping of a pagefile (NULL base for other allocators) and
 * the file offset of a handle's data */
int xmg_alloc_file_map(xm_allocator_t *a, const unsigned char **base);
uint64_t xmg_alloc_file_offset(uint64_t h);

/* tensor internals */
struct xmg_block *xmg_tensor_block(const xm_tensor_t *t, xm_dim_t blkidx);
size_t xmg_tensor_block_linear(const xm_tensor_t *t, xm_dim_t blkidx);
/* Canonical dims of the source block of blkidx and the per-dimension element
 * stride (in elements) of blkidx's own index space inside that data. */
void xmg_tensor_block_strides(const xm_tensor_t *t, xm_dim_t blkidx,
    int64_t strides[XM_MAX_DIM]);

/* element-type helpers */
static inline int xmg_is_complex(xm_scalar_type_t t)
{ return t == XM_SCALAR_FLOAT_COMPLEX || t == XM_SCALAR_DOUBLE_COMPLEX; }

static inline void xmg_scalar_pack(xm_scalar_t s, double out[2])
{ out[0] = creal(s); out[1] = cimag(s); }

int xmg_alloc_io(xm_allocator_t *a, uint64_t h, void *mem, size_t bytes,
    int wr);
int xmg_alloc_read_range(xm_allocator_t *a, uint64_t h, size_t byte_off,
    void *mem, size_t bytes);
int xmg_alloc_write_range(xm_allocator_t *a, uint64_t h, size_t byte_off,
    const void *mem, size_t bytes);
int xmg_alloc_bulk_views(xm_allocator_t *a, uint64_t bulk, const uint64_t *h,
    const uint64_t *d, size_t n);
uint64_t xmg_alloc_view_addr(const xm_allocator_t *a, uint64_t h);
int xmg_alloc_commit_view(xm_allocator_t *a, uint64_t h, size_t bytes);

/* Permuted-copy task helpers (blockops.c). */
/* Normalise an iteration space: drop extent-1 dimensions and merge
 * neighbours that are contiguous in both source and destination. */
void xmg_ptask_shape(xmgd_ptask_t *t, int ndim, const int64_t *size,
    const int64_t *dst_stride, const int64_t *src_stride);
/* Run a batch of tasks, growing the batch array as needed. */
typedef struct {
	xmgd_ptask_t *v;
	int n, cap;
} xmg_ptask_list_t;
xmgd_ptask_t *xmg_ptask_push(xmg_ptask_list_t *l);
int xmg_ptask_run(xmg_ptask_list_t *l, int dtype, int stype, double *dots);
void xmg_ptask_list_free(xmg_ptask_list_t *l);
/* Strides (elements) of a canonical block of the given dims. */
void xmg_canon_strides(const xm_dim_t *dims, int64_t strides[XM_MAX_DIM]);

#endif /* XMG_HOST_H */
