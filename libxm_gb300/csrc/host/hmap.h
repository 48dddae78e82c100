/* Open-addressing hash map uint64 -> uint64 used by the host planner and
 * the allocator (keys must not be UINT64_MAX). */
#ifndef XMG_HMAP_H
#define XMG_HMAP_H

#include <stddef.h>
#include <stdint.h>

typedef struct {
	uint64_t *keys, *vals;
	size_t cap, len;
} xmg_hmap_t;

void xmg_hmap_init(xmg_hmap_t *m);
void xmg_hmap_free(xmg_hmap_t *m);
/* Remove every entry, keeping the capacity. */
void xmg_hmap_clear(xmg_hmap_t *m);
/* Returns 1 and sets *val when found. */
int xmg_hmap_get(const xmg_hmap_t *m, uint64_t key, uint64_t *val);
/* Insert or overwrite; returns non-zero on out-of-memory. */
int xmg_hmap_put(xmg_hmap_t *m, uint64_t key, uint64_t val);
int xmg_hmap_del(xmg_hmap_t *m, uint64_t key);
/* Iterate: for (i = 0; i < m->cap; i++) if (m->keys[i] != XMG_HMAP_EMPTY) */
#define XMG_HMAP_EMPTY UINT64_MAX
uint64_t xmg_hash64(uint64_t x);

#endif
