/*
 * Block-data allocator for libxm-gb300.
 *
 * path == NULL: every allocation is a block of GPU memory from the engine's
 * HBM arena and the handle is its device address.  This replaces the
 * reference's malloc'd RAM storage (alloc.c:233-239); the handle stays an
 * opaque "virtual pointer" and data moves through read/write with host
 * buffers, exactly as the reference API promises (alloc.h:52-68).
 *
 * path != NULL: a pagefile of 512 KiB pages tracked by a first-fit bitmap
 * that grows by doubling (by 256 GiB once past 256 GiB), handle = page
 * offset | page count << 32, I/O in chunks of at most 1 GiB -- the
 * reference's pagefile scheme (alloc.c:40-145, 249-300).  The contraction
 * engine stages the pagefile blocks it touches into HBM (device views).
 *
 * xmg_allocator_create_host(): every allocation is page-locked host memory
 * (the reference's RAM allocator, alloc.c:233-239, kept in host memory)
 * and the handle is its host address.  read/write are memcpy; operations
 * stage the blocks they touch into HBM like pagefile blocks, but copy them
 * straight from the block's own pinned memory.
 */
#include <errno.h>
#include <fcntl.h>
#include <unistd.h>

#include <sys/mman.h>

#include "xmg_host.h"
#include "hmap.h"

#define PAGE_BYTES (512ULL * 1024)
#define GROW_STEP  (256ULL * 1024 * 1024 * 1024)
#define IO_CHUNK   (1ULL << 30)

struct xm_allocator {
	char *path;
	int host;                 /* blocks in page-locked host memory */
	int fd;
	uint64_t file_bytes;
	unsigned char *used;      /* one bit per page */
	xmg_hmap_t live;          /* HBM: live handle -> bytes */
	xmg_hmap_t views;         /* pagefile: handle -> staged device addr */
	xmg_hmap_t bviews;        /* pagefile: handle -> view inside `bulk` */
	uint64_t bulk;            /* one HBM buffer holding the bulk views */
	const unsigned char *map; /* pagefile: read-only mapping of the file */
	uint64_t map_bytes;       /* its length (the file's when mapped) */
};

static int bit_get(const unsigned char *b, uint64_t i) { return (b[i >> 3] >> (i & 7)) & 1; }
static void bit_set(unsigned char *b, uint64_t i) { b[i >> 3] |= (unsigned char)(1u << (i & 7)); }
static void bit_clr(unsigned char *b, uint64_t i) { b[i >> 3] &= (unsigned char)~(1u << (i & 7)); }

int
xmg_alloc_is_device(const xm_allocator_t *a)
{
	return a->path == NULL && !a->host;
}

int
xmg_alloc_is_host(const xm_allocator_t *a)
{
	return a->host;
}

xm_allocator_t *
xmg_allocator_create_host(void)
{
	xm_allocator_t *a;

	if (xmgd_init() != XMG_OK) {
		fprintf(stderr, "libxm: %s\n", xmg_last_error());
		return NULL;
	}
	if ((a = calloc(1, sizeof *a)) == NULL) {
		perror("calloc");
		return NULL;
	}
	xmg_hmap_init(&a->live);
	xmg_hmap_init(&a->views);
	xmg_hmap_init(&a->bviews);
	a->fd = -1;
	a->host = 1;
	return a;
}

xm_allocator_t *
xm_allocator_create(const char *path)
{
	xm_allocator_t *a;

	if ((a = calloc(1, sizeof *a)) == NULL) {
		perror("calloc");
		return NULL;
	}
	xmg_hmap_init(&a->live);
	xmg_hmap_init(&a->views);
	xmg_hmap_init(&a->bviews);
	a->fd = -1;
	if (path == NULL) {
		if (xmgd_init() != XMG_OK) {
			fprintf(stderr, "libxm: %s\n", xmg_last_error());
			free(a);
			return NULL;
		}
		return a;
	}
	a->file_bytes = PAGE_BYTES;
	if ((a->used = calloc(1, 1)) == NULL ||
	    (a->path = strdup(path)) == NULL) {
		perror("calloc");
		free(a->used);
		free(a);
		return NULL;
	}
	if ((a->fd = open(path, O_CREAT | O_RDWR, 0600)) == -1) {
		perror("open");
		goto fail;
	}
	if (ftruncate(a->fd, (off_t)a->file_bytes)) {
		perror("ftruncate");
		close(a->fd);
		goto fail;
	}
	return a;
fail:
	free(a->path);
	free(a->used);
	free(a);
	return NULL;
}

const char *
xm_allocator_get_path(xm_allocator_t *a)
{
	return a->path;
}

static int
grow_file(xm_allocator_t *a)
{
	uint64_t oldmap, newmap, nb;
	unsigned char *u;

	oldmap = (a->file_bytes / PAGE_BYTES + 7) / 8;
	nb = a->file_bytes > GROW_STEP ? a->file_bytes + GROW_STEP :
	    2 * a->file_bytes;
	newmap = (nb / PAGE_BYTES + 7) / 8;
	if (ftruncate(a->fd, (off_t)nb)) {
		perror("ftruncate");
		return 1;
	}
	if ((u = realloc(a->used, newmap)) == NULL) {
		perror("realloc");
		return 1;
	}
	memset(u + oldmap, 0, newmap - oldmap);
	a->used = u;
	a->file_bytes = nb;
	return 0;
}

/* First run of npages free pages starting at or after the first free page
 * (alloc.c:104-128). */
static uint64_t
find_run(xm_allocator_t *a, uint64_t npages)
{
	uint64_t total = a->file_bytes / PAGE_BYTES, p, run = 0, s;

	for (p = 0; p < total && bit_get(a->used, p); p++)
		;
	for (; p < total; p++) {
		run = bit_get(a->used, p) ? 0 : run + 1;
		if (run == npages) {
			s = p + 1 - npages;
			for (p = s; p < s + npages; p++)
				bit_set(a->used, p);
			return s | (npages << 32);
		}
	}
	return XM_NULL_PTR;
}

uint64_t
xm_allocator_allocate(xm_allocator_t *a, size_t bytes)
{
	uint64_t h, npages;

	if (bytes == 0)
		return XM_NULL_PTR;
	if (a->host) {
		void *p;
		if (xmgd_host_alloc(bytes, &p) != XMG_OK) {
			fprintf(stderr, "libxm: %s\n", xmg_last_error());
			return XM_NULL_PTR;
		}
		h = (uint64_t)(uintptr_t)p;
		if (xmg_hmap_put(&a->live, h, bytes)) {
			xmgd_host_free(p);
			return XM_NULL_PTR;
		}
		return h;
	}
	if (a->path == NULL) {
		if (xmgd_alloc(bytes, &h) != XMG_OK) {
			fprintf(stderr, "libxm: %s\n", xmg_last_error());
			return XM_NULL_PTR;
		}
		if (xmg_hmap_put(&a->live, h, bytes)) {
			xmgd_free(h);
			return XM_NULL_PTR;
		}
		return h;
	}
	npages = (bytes + PAGE_BYTES - 1) / PAGE_BYTES;
	while ((h = find_run(a, npages)) == XM_NULL_PTR)
		if (grow_file(a))
			return XM_NULL_PTR;
	return h;
}

static off_t
page_offset(uint64_t h)
{
	return (off_t)((h & 0xffffffffULL) * PAGE_BYTES);
}

static int
file_io(xm_allocator_t *a, uint64_t h, void *mem, size_t bytes, int wr)
{
	off_t off = page_offset(h);
	size_t n;
	ssize_t r;

	while (bytes > 0) {
		n = bytes > IO_CHUNK ? IO_CHUNK : bytes;
		r = wr ? pwrite(a->fd, mem, n, off) : pread(a->fd, mem, n, off);
		if (r != (ssize_t)n)
			return xmg_seterr(XMG_EIO, "%s", wr ? "pwrite" : "pread");
		mem = (char *)mem + n;
		off += (off_t)n;
		bytes -= n;
	}
	return XMG_OK;
}

/* xm_allocator_read (wr = 0) / write (wr = 1) with a status instead of
 * an exit */
int
xmg_alloc_io(xm_allocator_t *a, uint64_t h, void *mem, size_t bytes, int wr)
{
	if (h == XM_NULL_PTR)
		return xmg_seterr(XMG_EINVAL, "data pointer is NULL");
	if (a->host) {
		if (wr)
			memcpy((void *)(uintptr_t)h, mem, bytes);
		else
			memcpy(mem, (const void *)(uintptr_t)h, bytes);
		return XMG_OK;
	}
	if (a->path == NULL)
		return wr ? xmgd_h2d(h, mem, bytes) : xmgd_d2h(mem, h, bytes);
	return file_io(a, h, mem, bytes, wr);
}

void
xm_allocator_read(xm_allocator_t *a, uint64_t h, void *mem, size_t bytes)
{
	if (h == XM_NULL_PTR)
		xm_fatal("%s: data pointer is NULL", __func__);
	if (a->host)
		memcpy(mem, (const void *)(uintptr_t)h, bytes);
	else if (a->path == NULL)
		xmg_die_on(xmgd_d2h(mem, h, bytes));
	else
		xmg_die_on(file_io(a, h, mem, bytes, 0));
}

void
xm_allocator_write(xm_allocator_t *a, uint64_t h, const void *mem, size_t bytes)
{
	if (h == XM_NULL_PTR)
		xm_fatal("%s: data pointer is NULL", __func__);
	if (a->host)
		memcpy((void *)(uintptr_t)h, mem, bytes);
	else if (a->path == NULL)
		xmg_die_on(xmgd_h2d(h, mem, bytes));
	else
		xmg_die_on(file_io(a, h, (void *)mem, bytes, 1));
}

void
xm_allocator_deallocate(xm_allocator_t *a, uint64_t h)
{
	uint64_t p, s, n;

	if (h == XM_NULL_PTR)
		return;
	if (a->host) {
		xmg_hmap_del(&a->live, h);
		xmgd_host_free((void *)(uintptr_t)h);
		return;
	}
	if (a->path == NULL) {
		xmg_hmap_del(&a->live, h);
		xmg_die_on(xmgd_free(h));
		return;
	}
	s = h & 0xffffffffULL;
	n = h >> 32;
	for (p = s; p < s + n; p++)
		bit_clr(a->used, p);
}

int
xmg_alloc_device_view(xm_allocator_t *a, uint64_t h, size_t bytes,
    uint64_t *dptr)
{
	uint64_t d;
	void *pin;
	int st;

	if (xmg_alloc_is_device(a)) {
		*dptr = h;
		return XMG_OK;
	}
	if (xmg_hmap_get(&a->views, h, dptr) ||
	    xmg_hmap_get(&a->bviews, h, dptr))
		return XMG_OK;
	if ((st = xmgd_alloc(bytes, &d)) != XMG_OK)
		return st;
	if (a->host)
		st = xmgd_h2d(d, (const void *)(uintptr_t)h, bytes);
	else if ((st = xmgd_pinned(bytes, &pin)) == XMG_OK &&
	    (st = file_io(a, h, pin, bytes, 0)) == XMG_OK)
		st = xmgd_h2d(d, pin, bytes);
	if (st != XMG_OK) {
		xmgd_free(d);
		return st;
	}
	if (xmg_hmap_put(&a->views, h, d)) {
		xmgd_free(d);
		return xmg_seterr(XMG_ENOMEM, "out of memory");
	}
	*dptr = d;
	return XMG_OK;
}

/* Write a staged view back to the pagefile (or the host block). */
int
xmg_alloc_commit_view(xm_allocator_t *a, uint64_t h, size_t bytes)
{
	uint64_t d;
	void *pin;
	int st;

	if (xmg_alloc_is_device(a))
		return XMG_OK;
	if (!xmg_hmap_get(&a->views, h, &d) && !xmg_hmap_get(&a->bviews, h, &d))
		return xmg_seterr(XMG_EINVAL, "no staged view for handle");
	if (a->host)
		return xmgd_d2h((void *)(uintptr_t)h, d, bytes);
	if ((st = xmgd_pinned(bytes, &pin)) != XMG_OK ||
	    (st = xmgd_d2h(pin, d, bytes)) != XMG_OK)
		return st;
	return file_io(a, h, pin, bytes, 1);
}

int
xmg_alloc_release_views(xm_allocator_t *a, int write_back)
{
	size_t i;

	(void)write_back;
	if (xmg_alloc_is_device(a))
		return XMG_OK;
	for (i = 0; i < a->views.cap; i++)
		if (a->views.keys[i] != XMG_HMAP_EMPTY)
			xmgd_free(a->views.vals[i]);
	xmg_hmap_free(&a->views);
	xmg_hmap_init(&a->views);
	if (a->bulk)
		xmgd_free(a->bulk);
	a->bulk = 0;
	xmg_hmap_free(&a->bviews);
	xmg_hmap_init(&a->bviews);
	return XMG_OK;
}

/* Views staged together: the blocks h[i] live at d[i] inside the HBM
 * buffer `bulk` (filled by the caller), which the allocator takes over in
 * every case (freed here on error, else with the other views). */
int
xmg_alloc_bulk_views(xm_allocator_t *a, uint64_t bulk, const uint64_t *h,
    const uint64_t *d, size_t n)
{
	size_t i;

	if (xmg_alloc_is_device(a) || a->bulk) {
		xmgd_free(bulk);
		return xmg_seterr(XMG_EINVAL, "bulk views: pagefile or host "
		    "allocator without bulk views expected");
	}
	a->bulk = bulk;
	for (i = 0; i < n; i++)
		if (xmg_hmap_put(&a->bviews, h[i], d[i]))
			return xmg_seterr(XMG_ENOMEM, "out of memory");
	return XMG_OK;
}

/* device address of a staged view (either kind), 0 if none */
uint64_t
xmg_alloc_view_addr(const xm_allocator_t *a, uint64_t h)
{
	uint64_t d;

	if (xmg_hmap_get(&a->views, h, &d) || xmg_hmap_get(&a->bviews, h, &d))
		return d;
	return 0;
}

/*
 * A read-only shared mapping of the pagefile up to its last used page, for
 * streaming its blocks to the device with the copy engine straight from
 * the page cache (where the device reads pageable memory through the
 * host's page tables; the file's own writes, pwrite, are visible through
 * the mapping).  Kept until a block lies beyond it or the allocator goes
 * away; its pages are mapped in up front (MAP_POPULATE) -- only the used
 * extent, not the file's sparse tail.  *base receives the mapping, NULL
 * (with XMG_OK) when the allocator has no pagefile or no used page.
 */
int
xmg_alloc_file_map(xm_allocator_t *a, const unsigned char **base)
{
	uint64_t p = a->path ? a->file_bytes / PAGE_BYTES : 0, need;
	void *m;

	*base = NULL;
	while (p > 0 && !bit_get(a->used, p - 1))
		p--;
	need = p * PAGE_BYTES;
	if (need == 0)
		return XMG_OK;
	if (a->map != NULL && a->map_bytes >= need) {
		*base = a->map;
		return XMG_OK;
	}
	if (a->map != NULL)
		munmap((void *)a->map, a->map_bytes);
	a->map = NULL;
	a->map_bytes = 0;
	m = mmap(NULL, need, PROT_READ, MAP_SHARED | MAP_POPULATE, a->fd, 0);
	if (m == MAP_FAILED)
		return xmg_seterr(XMG_EIO, "mmap of the pagefile failed");
	a->map = m;
	a->map_bytes = need;
	*base = a->map;
	return XMG_OK;
}

/* byte offset of a pagefile handle's data in the file */
uint64_t
xmg_alloc_file_offset(uint64_t h)
{
	return (uint64_t)page_offset(h);
}

void
xm_allocator_destroy(xm_allocator_t *a)
{
	size_t i;

	if (a == NULL)
		return;
	xmg_adjoint_forget(a);
	if (a->map != NULL)
		munmap((void *)a->map, a->map_bytes);
	if (a->path != NULL) {
		xmg_alloc_release_views(a, 0);
		if (close(a->fd))
			perror("close");
		if (unlink(a->path))
			perror("unlink");
	} else if (a->host) {
		xmg_alloc_release_views(a, 0);
		for (i = 0; i < a->live.cap; i++)
			if (a->live.keys[i] != XMG_HMAP_EMPTY)
				xmgd_host_free((void *)(uintptr_t)a->live.keys[i]);
	} else {
		/* blocks still allocated when the allocator goes away */
		for (i = 0; i < a->live.cap; i++)
			if (a->live.keys[i] != XMG_HMAP_EMPTY)
				xmgd_free(a->live.keys[i]);
	}
	xmg_hmap_free(&a->live);
	xmg_hmap_free(&a->views);
	xmg_hmap_free(&a->bviews);
	free(a->path);
	free(a->used);
	free(a);
}

/* Read part of a block (byte range) into host memory; used by
 * xm_tensor_get_element so that one element costs one small copy. */
int
xmg_alloc_read_range(xm_allocator_t *a, uint64_t h, size_t byte_off,
    void *mem, size_t bytes)
{
	ssize_t r;

	if (a->host) {
		memcpy(mem, (const char *)(uintptr_t)h + byte_off, bytes);
		return XMG_OK;
	}
	if (a->path == NULL)
		return xmgd_d2h(mem, h + byte_off, bytes);
	r = pread(a->fd, mem, bytes, page_offset(h) + (off_t)byte_off);
	return r == (ssize_t)bytes ? XMG_OK : xmg_seterr(XMG_EIO, "pread");
}

/* Write part of a pagefile block (byte range) from host memory. */
int
xmg_alloc_write_range(xm_allocator_t *a, uint64_t h, size_t byte_off,
    const void *mem, size_t bytes)
{
	ssize_t r;

	if (a->host) {
		memcpy((char *)(uintptr_t)h + byte_off, mem, bytes);
		return XMG_OK;
	}
	if (a->path == NULL)
		return xmg_seterr(XMG_EINVAL, "write_range: pagefile allocator "
		    "expected");
	r = pwrite(a->fd, mem, bytes, page_offset(h) + (off_t)byte_off);
	return r == (ssize_t)bytes ? XMG_OK : xmg_seterr(XMG_EIO, "pwrite");
}
