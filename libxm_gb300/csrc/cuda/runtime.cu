/*
 * libxm-gb300 device runtime: one GPU, one engine stream, a stream-ordered
 * HBM pool for block data, grow-only scratch and pinned staging buffers.
 * All public copies are synchronous with respect to the calling host
 * thread, matching the reference's synchronous API contract.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "common.cuh"

namespace xmg {

static int g_ready = 0;
static int g_dev = 0;
static int g_sms = 0;
static cudaStream_t g_stream = nullptr;
static size_t g_in_use = 0;
static cudaEvent_t g_t0 = nullptr, g_t1 = nullptr;
long long g_launches = 0;

struct buf { void *p; size_t n; };
static buf g_scratch[XMGD_SCRATCH_SLOTS];
static buf g_pinned;

/* staging side stream: host-to-device copies of out-of-core operand
 * blocks from two pinned chunk buffers, overlapping the compute stream */
static cudaStream_t g_side = nullptr;
static cudaEvent_t g_side_ev[XMGD_SIDE_SLOTS];
static bool g_side_rec[XMGD_SIDE_SLOTS];
static buf g_chunk[XMGD_SIDE_SLOTS];

cudaStream_t stream() { return g_stream; }
int device() { return g_dev; }
int num_sms() { return g_sms; }

int
check(cudaError_t e, const char *what)
{
	if (e == cudaSuccess)
		return XMG_OK;
	cudaGetLastError();	/* clear the sticky-free error state */
	if (e == cudaErrorMemoryAllocation)
		return xmg_seterr(XMG_ENOMEM, "out of device memory (%s)", what);
	return xmg_seterr(XMG_ECUDA, "CUDA error %s in %s",
	    cudaGetErrorString(e), what);
}

} /* namespace xmg */

using namespace xmg;

extern "C" int xmgd_noalloc_setup(void);

extern "C" int
xmgd_init(void)
{
	int n = 0;
	cudaMemPool_t pool;
	uint64_t thr = UINT64_MAX;

	const char *dev;

	if (g_ready)
		return XMG_OK;
	if ((dev = getenv("XMG_DEVICE")) != NULL)
		g_dev = atoi(dev);
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
		cudaGetLastError();
		return xmg_seterr(XMG_ECUDA, "no CUDA device available: the "
		    "libxm-gb300 engine runs its kernels on the GPU only");
	}
	if (g_dev < 0 || g_dev >= n)
		return xmg_seterr(XMG_EINVAL, "XMG_DEVICE=%d out of range", g_dev);
	XMG_CK(cudaSetDevice(g_dev));
	XMG_CK(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount,
	    g_dev));
	XMG_CK(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
	XMG_CK(cudaStreamCreateWithFlags(&g_side, cudaStreamNonBlocking));
	for (int i = 0; i < XMGD_SIDE_SLOTS; i++)
		XMG_CK(cudaEventCreateWithFlags(&g_side_ev[i], cudaEventDisableTiming));
	/* keep freed block memory in the pool: tensors are created and freed
	 * often and cudaMalloc/cudaFree would synchronise the device */
	XMG_CK(cudaDeviceGetDefaultMemPool(&pool, g_dev));
	XMG_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold,
	    &thr));
	g_ready = 1;
	/* load the allocation-free dot's module now, so that its static
	 * device array exists before the caller's first xmg_dot_noalloc */
	return xmgd_noalloc_setup();
}

extern "C" int
xmgd_alloc(size_t bytes, uint64_t *dptr)
{
	void *p = nullptr;

	XMG_CK(cudaMallocAsync(&p, bytes, g_stream));
	g_in_use += bytes;
	*dptr = (uint64_t)(uintptr_t)p;
	return XMG_OK;
}

extern "C" int
xmgd_free(uint64_t dptr)
{
	XMG_CK(cudaFreeAsync((void *)(uintptr_t)dptr, g_stream));
	return XMG_OK;
}

extern "C" size_t xmgd_arena_bytes_in_use(void) { return g_in_use; }

extern "C" int
xmgd_h2d(uint64_t dst, const void *src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync((void *)(uintptr_t)dst, src, bytes,
	    cudaMemcpyHostToDevice, g_stream));
	XMG_CK(cudaStreamSynchronize(g_stream));
	return XMG_OK;
}

extern "C" int
xmgd_d2h(void *dst, uint64_t src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync(dst, (const void *)(uintptr_t)src, bytes,
	    cudaMemcpyDeviceToHost, g_stream));
	XMG_CK(cudaStreamSynchronize(g_stream));
	return XMG_OK;
}

extern "C" int
xmgd_h2d_async(uint64_t dst, const void *src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync((void *)(uintptr_t)dst, src, bytes,
	    cudaMemcpyHostToDevice, g_stream));
	return XMG_OK;
}

extern "C" int
xmgd_d2h_async(void *dst, uint64_t src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync(dst, (const void *)(uintptr_t)src, bytes,
	    cudaMemcpyDeviceToHost, g_stream));
	return XMG_OK;
}

extern "C" int
xmgd_d2d(uint64_t dst, uint64_t src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync((void *)(uintptr_t)dst,
	    (const void *)(uintptr_t)src, bytes, cudaMemcpyDeviceToDevice,
	    g_stream));
	return XMG_OK;
}

extern "C" int
xmgd_sync(void)
{
	if (!g_ready)
		return XMG_OK;
	XMG_CK(cudaStreamSynchronize(g_stream));
	XMG_CK(cudaGetLastError());
	return XMG_OK;
}

extern "C" int
xmgd_is_device_ptr(const void *p)
{
	cudaPointerAttributes at;

	if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return at.type == cudaMemoryTypeDevice ||
	    at.type == cudaMemoryTypeManaged;
}

extern "C" int
xmgd_scratch(int slot, size_t bytes, uint64_t *dptr)
{
	buf *b;

	if (slot < 0 || slot >= XMGD_SCRATCH_SLOTS)
		return xmg_seterr(XMG_EINVAL, "bad scratch slot");
	b = &g_scratch[slot];
	if (b->n < bytes) {
		if (b->p) {
			XMG_CK(cudaStreamSynchronize(g_stream));
			XMG_CK(cudaFree(b->p));
			b->p = nullptr;
			b->n = 0;
		}
		size_t n = bytes < 4096 ? 4096 : bytes + bytes / 4;
		XMG_CK(cudaMalloc(&b->p, n));
		b->n = n;
	}
	*dptr = (uint64_t)(uintptr_t)b->p;
	return XMG_OK;
}

extern "C" int
xmgd_pinned(size_t bytes, void **hptr)
{
	if (g_pinned.n < bytes) {
		if (g_pinned.p) {
			XMG_CK(cudaStreamSynchronize(g_stream));
			XMG_CK(cudaFreeHost(g_pinned.p));
			g_pinned.p = nullptr;
			g_pinned.n = 0;
		}
		XMG_CK(cudaMallocHost(&g_pinned.p, bytes));
		g_pinned.n = bytes;
	}
	*hptr = g_pinned.p;
	return XMG_OK;
}

/* 1 when the engine's device reads pageable host memory through the
 * host's page tables (a coherent CPU-GPU link, e.g. Grace): copies from
 * any host mapping then run at the link's rate without staging */
extern "C" int
xmgd_pageable_direct(void)
{
	int v = 0;

	if (cudaDeviceGetAttribute(&v,
	    cudaDevAttrPageableMemoryAccessUsesHostPageTables, g_dev) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return v;
}

/* make the calling host thread use the engine's device */
extern "C" int
xmgd_bind_thread(void)
{
	XMG_CK(cudaSetDevice(g_dev));
	return XMG_OK;
}

extern "C" int
xmgd_side_wait(int slot)
{
	if (g_side_rec[slot]) {
		XMG_CK(cudaEventSynchronize(g_side_ev[slot]));
		g_side_rec[slot] = false;
	}
	return XMG_OK;
}

extern "C" int
xmgd_side_chunk(int slot, size_t bytes, void **hptr)
{
	buf *b = &g_chunk[slot];
	int st;

	if (b->n < bytes) {
		if ((st = xmgd_side_wait(slot)) != XMG_OK)
			return st;
		if (b->p)
			XMG_CK(cudaFreeHost(b->p));
		b->p = nullptr;
		b->n = 0;
		XMG_CK(cudaMallocHost(&b->p, bytes));
		b->n = bytes;
	}
	*hptr = b->p;
	return XMG_OK;
}

extern "C" int
xmgd_side_copy(int slot, uint64_t dst, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync((void *)(uintptr_t)dst, g_chunk[slot].p, bytes,
	    cudaMemcpyHostToDevice, g_side));
	XMG_CK(cudaEventRecord(g_side_ev[slot], g_side));
	g_side_rec[slot] = true;
	return XMG_OK;
}

/* the reverse: device bytes into chunk `slot` (write-back of staged
 * views); side_wait(slot) then makes the chunk readable */
extern "C" int
xmgd_side_fetch(int slot, uint64_t src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync(g_chunk[slot].p, (const void *)(uintptr_t)src, bytes,
	    cudaMemcpyDeviceToHost, g_side));
	XMG_CK(cudaEventRecord(g_side_ev[slot], g_side));
	g_side_rec[slot] = true;
	return XMG_OK;
}

extern "C" int
xmgd_side_put(uint64_t dst, const void *src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync((void *)(uintptr_t)dst, src, bytes,
	    cudaMemcpyHostToDevice, g_side));
	return XMG_OK;
}

extern "C" int
xmgd_side_get(void *dst, uint64_t src, size_t bytes)
{
	XMG_CK(cudaMemcpyAsync(dst, (const void *)(uintptr_t)src, bytes,
	    cudaMemcpyDeviceToHost, g_side));
	return XMG_OK;
}

extern "C" int
xmgd_side_sync(void)
{
	XMG_CK(cudaStreamSynchronize(g_side));
	for (int i = 0; i < XMGD_SIDE_SLOTS; i++)
		g_side_rec[i] = false;
	return XMG_OK;
}

extern "C" int
xmg_timer_start(void)
{
	int st;

	if ((st = xmgd_init()) != XMG_OK)
		return st;
	if (!g_t0) {
		XMG_CK(cudaEventCreate(&g_t0));
		XMG_CK(cudaEventCreate(&g_t1));
	}
	XMG_CK(cudaEventRecord(g_t0, g_stream));
	return XMG_OK;
}

extern "C" double
xmg_timer_stop(void)
{
	float ms = -1;

	if (!g_t0 || cudaEventRecord(g_t1, g_stream) != cudaSuccess ||
	    cudaEventSynchronize(g_t1) != cudaSuccess ||
	    cudaEventElapsedTime(&ms, g_t0, g_t1) != cudaSuccess)
		return -1.0;
	return ms;
}

extern "C" long long xmg_kernel_launches(void) { return g_launches; }

extern "C" int
xmg_device_memory(size_t *free_bytes, size_t *total_bytes)
{
	int st;

	if (free_bytes == NULL || total_bytes == NULL)
		return xmg_seterr(XMG_EINVAL, "xmg_device_memory: NULL argument");
	if ((st = xmgd_init()) != XMG_OK)
		return st;
	XMG_CK(cudaSetDevice(g_dev));
	XMG_CK(cudaMemGetInfo(free_bytes, total_bytes));
	return XMG_OK;
}

/*
 * Page-locked host memory for host-allocator blocks, carved from slabs of
 * at least 1 GiB (one cudaHostAlloc each) with 256-byte aligned bump
 * allocation: the copy engine reads a few large pinned regions much
 * faster than thousands of separately pinned block-sized ones.  A slab
 * keeps a count of its live blocks; when it drops to zero the slab is
 * freed (the newest one is kept and reused from its start).
 */
struct slab { char *p; size_t n, used; long live; };
static std::vector<slab> g_slabs;
static const size_t SLAB_BYTES = (size_t)1 << 30;

extern "C" int
xmgd_host_alloc(size_t bytes, void **hptr)
{
	const size_t need = (bytes + 255) & ~(size_t)255;

	if (g_slabs.empty() || g_slabs.back().n - g_slabs.back().used < need) {
		slab s = {nullptr, need > SLAB_BYTES ? need : SLAB_BYTES, 0, 0};
		XMG_CK(cudaSetDevice(g_dev));
		XMG_CK(cudaHostAlloc((void **)&s.p, s.n, cudaHostAllocDefault));
		g_slabs.push_back(s);
	}
	slab &s = g_slabs.back();
	*hptr = s.p + s.used;
	s.used += need;
	s.live++;
	return XMG_OK;
}

extern "C" void
xmgd_host_free(void *p)
{
	if (!p)
		return;
	for (size_t i = 0; i < g_slabs.size(); i++) {
		slab &s = g_slabs[i];
		if ((char *)p < s.p || (char *)p >= s.p + s.n)
			continue;
		if (--s.live > 0)
			return;
		if (i + 1 == g_slabs.size()) {
			s.used = 0;	/* the newest slab is reused */
			return;
		}
		cudaFreeHost(s.p);
		g_slabs.erase(g_slabs.begin() + (long)i);
		return;
	}
}

extern "C" void *
xmg_host_alloc(size_t bytes)
{
	void *p = nullptr;

	if (xmgd_init() != XMG_OK || cudaMallocHost(&p, bytes) != cudaSuccess)
		return nullptr;
	return p;
}

extern "C" void
xmg_host_free(void *p)
{
	if (p)
		cudaFreeHost(p);
}
