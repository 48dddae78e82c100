/*
 * libxm-gb300: block-data allocator.
 *
 * Same declarations as the reference's src/alloc.h:31-81.
 *   path == NULL : block data lives in GPU memory (HBM arena).  The returned
 *                  "virtual pointer" is an opaque handle; callers move data
 *                  only through xm_allocator_read/write (host buffers).
 *   path != NULL : block data lives in a host pagefile of 512 KiB pages;
 *                  contractions stage the blocks they need into HBM.
 */
#ifndef XM_ALLOC_H
#define XM_ALLOC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Null data handle (alloc.h:31). */
#define XM_NULL_PTR ((uint64_t)(-1))

typedef struct xm_allocator xm_allocator_t;

/* NULL on failure (alloc.c:147-207). */
xm_allocator_t *xm_allocator_create(const char *path);
const char *xm_allocator_get_path(xm_allocator_t *allocator);
/* XM_NULL_PTR on failure or for size 0 (alloc.c:136-144). */
uint64_t xm_allocator_allocate(xm_allocator_t *allocator, size_t size_bytes);
/* Host buffer <- block data (alloc.h:59). */
void xm_allocator_read(xm_allocator_t *allocator, uint64_t data_ptr,
    void *mem, size_t size_bytes);
/* Block data <- host buffer (alloc.h:68). */
void xm_allocator_write(xm_allocator_t *allocator, uint64_t data_ptr,
    const void *mem, size_t size_bytes);
void xm_allocator_deallocate(xm_allocator_t *allocator, uint64_t data_ptr);
/* NULL is allowed; the pagefile is removed (alloc.c:328-347). */
void xm_allocator_destroy(xm_allocator_t *allocator);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XM_ALLOC_H */
