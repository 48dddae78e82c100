/* Open-addressing (linear probing) hash map with backward-shift deletion. */
#include <stdlib.h>
#include <string.h>

#include "hmap.h"

uint64_t
xmg_hash64(uint64_t x)
{
	/* splitmix64 finaliser */
	x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
	x ^= x >> 27; x *= 0x94d049bb133111ebULL;
	x ^= x >> 31;
	return x;
}

void
xmg_hmap_init(xmg_hmap_t *m)
{
	memset(m, 0, sizeof *m);
}

void
xmg_hmap_free(xmg_hmap_t *m)
{
	free(m->keys);
	free(m->vals);
	memset(m, 0, sizeof *m);
}

void
xmg_hmap_clear(xmg_hmap_t *m)
{
	if (m->cap)
		memset(m->keys, 0xff, m->cap * sizeof(uint64_t));
	m->len = 0;
}

static int
grow(xmg_hmap_t *m)
{
	xmg_hmap_t n;
	size_t i;

	n.cap = m->cap ? 2 * m->cap : 64;
	n.len = 0;
	n.keys = malloc(n.cap * sizeof(uint64_t));
	n.vals = malloc(n.cap * sizeof(uint64_t));
	if (n.keys == NULL || n.vals == NULL) {
		free(n.keys);
		free(n.vals);
		return 1;
	}
	memset(n.keys, 0xff, n.cap * sizeof(uint64_t));
	for (i = 0; i < m->cap; i++)
		if (m->keys[i] != XMG_HMAP_EMPTY)
			xmg_hmap_put(&n, m->keys[i], m->vals[i]);
	free(m->keys);
	free(m->vals);
	*m = n;
	return 0;
}

int
xmg_hmap_get(const xmg_hmap_t *m, uint64_t key, uint64_t *val)
{
	size_t i;

	if (m->cap == 0)
		return 0;
	for (i = xmg_hash64(key) & (m->cap - 1); m->keys[i] != XMG_HMAP_EMPTY;
	    i = (i + 1) & (m->cap - 1)) {
		if (m->keys[i] == key) {
			if (val)
				*val = m->vals[i];
			return 1;
		}
	}
	return 0;
}

int
xmg_hmap_put(xmg_hmap_t *m, uint64_t key, uint64_t val)
{
	size_t i;

	if ((m->len + 1) * 4 > m->cap * 3 && grow(m))
		return 1;
	for (i = xmg_hash64(key) & (m->cap - 1); m->keys[i] != XMG_HMAP_EMPTY;
	    i = (i + 1) & (m->cap - 1)) {
		if (m->keys[i] == key) {
			m->vals[i] = val;
			return 0;
		}
	}
	m->keys[i] = key;
	m->vals[i] = val;
	m->len++;
	return 0;
}

int
xmg_hmap_del(xmg_hmap_t *m, uint64_t key)
{
	size_t i, j, h, mask;

	if (m->cap == 0)
		return 0;
	mask = m->cap - 1;
	for (i = xmg_hash64(key) & mask; m->keys[i] != key; i = (i + 1) & mask)
		if (m->keys[i] == XMG_HMAP_EMPTY)
			return 0;
	/* backward-shift deletion keeps probe chains intact */
	j = i;
	for (;;) {
		j = (j + 1) & mask;
		if (m->keys[j] == XMG_HMAP_EMPTY)
			break;
		h = xmg_hash64(m->keys[j]) & mask;
		if ((j > i && (h <= i || h > j)) || (j < i && (h <= i && h > j))) {
			m->keys[i] = m->keys[j];
			m->vals[i] = m->vals[j];
			i = j;
		}
	}
	m->keys[i] = XMG_HMAP_EMPTY;
	m->len--;
	return 1;
}
