/*
 * Allocation-free dot product (xmg_dot_noalloc, declared in include/xmg.h).
 *
 * Some callers cannot allocate GPU memory when they need a result: a host
 * application whose own pool already holds the HBM it is allowed to use
 * (so a cudaMalloc would fail), or a solver that evaluates a convergence
 * norm inside a latency-critical loop, where the first-use cudaMalloc of
 * the regular xm_dot path would block on the device.  This variant keeps
 * every buffer it needs beyond its inputs and output -- the block task
 * table, one partial sum per CTA and the running result -- in the
 * file-scope array below, sized once at load time.
 *
 * The array's name is only a host-side stand-in for the device object, so
 * its device address is fetched with cudaGetSymbolAddress, with the
 * engine's device current, when the engine initialises on that device
 * (xmgd_init calls xmgd_noalloc_setup).  That lookup also loads this
 * file's module, which is when the driver places the array in device
 * memory: with lazy module loading a lookup deferred to the first
 * xmg_dot_noalloc would allocate at that call.  All calls share the one
 * array and it keeps the previous call's contents: the result is cleared
 * at the start of every call, and calls that overlap on the GPU (several
 * host threads, or several processes' streams on one context) race on it.
 */
#include <stdint.h>

#include "common.cuh"

namespace xmg {

constexpr int NA_MAX_TASKS = XMG_NOALLOC_MAX_TASKS;     /* tasks per batch */
constexpr int NA_MAX_CTAS = XMG_NOALLOC_MAX_CTAS;       /* partials per batch */
constexpr int NA_ELEMS = XMG_NOALLOC_ELEMS_PER_CTA;     /* elements per CTA */
constexpr int NA_THREADS = 256;
constexpr int NA_MAX_DEVICES = 64;

struct noalloc_scratch {
	xmgd_ptask_t tasks[NA_MAX_TASKS];
	int64_t first[NA_MAX_TASKS + 1];
	double partial[2 * NA_MAX_CTAS];
	double result[2];
};

static __device__ __align__(256) noalloc_scratch g_noalloc;

static noalloc_scratch *g_addr[NA_MAX_DEVICES];

template <typename T>
__global__ void __launch_bounds__(NA_THREADS)
noalloc_dot_kernel(noalloc_scratch *sc, int ntasks)
{
	__shared__ double red[2][NA_THREADS / 32];
	const int64_t cta = blockIdx.x;
	int lo = 0, hi = ntasks - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (sc->first[mid] <= cta) lo = mid; else hi = mid - 1;
	}
	const xmgd_ptask_t &t = sc->tasks[lo];
	const T *x = reinterpret_cast<const T *>(t.dst);
	const T *y = reinterpret_cast<const T *>(t.src);
	int64_t n = 1;
	for (int d = 0; d < t.ndim; d++)
		n *= t.size[d];
	const int64_t e0 = (cta - sc->first[lo]) * NA_ELEMS;
	const int64_t e1 = e0 + NA_ELEMS < n ? e0 + NA_ELEMS : n;
	double re = 0, im = 0;
	for (int64_t e = e0 + threadIdx.x; e < e1; e += NA_THREADS) {
		int64_t r = e, ox = 0, oy = 0;
		for (int d = 0; d < t.ndim; d++) {
			int64_t q = r % t.size[d];
			r /= t.size[d];
			ox += q * t.dst_stride[d];
			oy += q * t.src_stride[d];
		}
		T p = num<T>::mul(x[ox], y[oy]);
		re += num<T>::re(p);
		im += num<T>::im(p);
	}
	for (int off = 16; off > 0; off >>= 1) {
		re += __shfl_down_sync(0xffffffffu, re, off);
		im += __shfl_down_sync(0xffffffffu, im, off);
	}
	if ((threadIdx.x & 31) == 0) {
		red[0][threadIdx.x >> 5] = re;
		red[1][threadIdx.x >> 5] = im;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double a = 0, b = 0;
		for (int w = 0; w < NA_THREADS / 32; w++) {
			a += red[0][w];
			b += red[1][w];
		}
		sc->partial[2 * cta] = a;
		sc->partial[2 * cta + 1] = b;
	}
}

/* result += sum over tasks of factor_t * (sum of the task's partials), in
 * task order (deterministic).  For float types the scaled task sum and the
 * running result are rounded to float after every task, as xm_dot rounds
 * each block's contribution and its running sum to the tensor's type. */
__global__ void
noalloc_reduce_kernel(noalloc_scratch *sc, int ntasks, int narrow)
{
	if (threadIdx.x != 0 || blockIdx.x != 0)
		return;
	double rr = sc->result[0], ri = sc->result[1];
	for (int k = 0; k < ntasks; k++) {
		double a = 0, b = 0;
		for (int64_t c = sc->first[k]; c < sc->first[k + 1]; c++) {
			a += sc->partial[2 * c];
			b += sc->partial[2 * c + 1];
		}
		const double *f = sc->tasks[k].alpha;
		double pr = f[0] * a - f[1] * b, pi = f[0] * b + f[1] * a;
		if (narrow) {
			pr = (float)pr;
			pi = (float)pi;
			rr = (float)(rr + pr);
			ri = (float)(ri + pi);
		} else {
			rr += pr;
			ri += pi;
		}
	}
	sc->result[0] = rr;
	sc->result[1] = ri;
}

/* The array's device address on the engine's device (the one every copy
 * and launch below goes to, whichever host thread calls); looked up with
 * that device current. */
static int
scratch_addr(noalloc_scratch **out)
{
	const int dev = device();

	if (dev < 0 || dev >= NA_MAX_DEVICES)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: device %d", dev);
	if (g_addr[dev] == nullptr) {
		void *p = nullptr;
		XMG_CK(cudaSetDevice(dev));
		XMG_CK(cudaGetSymbolAddress(&p, g_noalloc));
		g_addr[dev] = static_cast<noalloc_scratch *>(p);
	}
	*out = g_addr[dev];
	return XMG_OK;
}

} /* namespace xmg */

using namespace xmg;

/* Called once by xmgd_init, after it made the engine's device current. */
extern "C" int
xmgd_noalloc_setup(void)
{
	noalloc_scratch *sc = NULL;

	return scratch_addr(&sc);
}

extern "C" int
xmgd_noalloc_begin(void)
{
	noalloc_scratch *sc = NULL;
	int st;

	if ((st = xmgd_init()) != XMG_OK || (st = scratch_addr(&sc)) != XMG_OK)
		return st;
	XMG_CK(cudaMemsetAsync(sc->result, 0, sizeof sc->result, stream()));
	return XMG_OK;
}

/* Run one batch: tasks (host array, at most NA_MAX_TASKS) with first[] the
 * CTA prefix sums (first[ntasks] = total CTAs <= NA_MAX_CTAS). */
extern "C" int
xmgd_noalloc_dot_batch(int dtype, const xmgd_ptask_t *tasks,
    const int64_t *first, int ntasks)
{
	noalloc_scratch *sc = NULL;
	int st;

	if (ntasks <= 0)
		return XMG_OK;
	if (ntasks > NA_MAX_TASKS || first[ntasks] > NA_MAX_CTAS)
		return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: batch exceeds "
		    "the static scratch");
	if ((st = scratch_addr(&sc)) != XMG_OK)
		return st;
	XMG_CK(cudaMemcpyAsync(sc->tasks, tasks, (size_t)ntasks * sizeof *tasks,
	    cudaMemcpyHostToDevice, stream()));
	XMG_CK(cudaMemcpyAsync(sc->first, first, (size_t)(ntasks + 1) *
	    sizeof *first, cudaMemcpyHostToDevice, stream()));
	const unsigned grid = (unsigned)first[ntasks];
	switch (dtype) {
	case 0: noalloc_dot_kernel<float><<<grid, NA_THREADS, 0, stream()>>>(sc, ntasks); break;
	case 1: noalloc_dot_kernel<cf><<<grid, NA_THREADS, 0, stream()>>>(sc, ntasks); break;
	case 2: noalloc_dot_kernel<double><<<grid, NA_THREADS, 0, stream()>>>(sc, ntasks); break;
	case 3: noalloc_dot_kernel<cd><<<grid, NA_THREADS, 0, stream()>>>(sc, ntasks); break;
	default: return xmg_seterr(XMG_EINVAL, "xmg_dot_noalloc: scalar type");
	}
	XMG_CK(cudaGetLastError());
	noalloc_reduce_kernel<<<1, 32, 0, stream()>>>(sc, ntasks, dtype < 2);
	XMG_CK(cudaGetLastError());
	g_launches += 2;
	/* the host task array may be reused by the caller right away */
	XMG_CK(cudaStreamSynchronize(stream()));
	return XMG_OK;
}

extern "C" int
xmgd_noalloc_result(double out[2])
{
	noalloc_scratch *sc = NULL;
	int st;

	if ((st = scratch_addr(&sc)) != XMG_OK)
		return st;
	XMG_CK(cudaMemcpyAsync(out, sc->result, 2 * sizeof(double),
	    cudaMemcpyDeviceToHost, stream()));
	XMG_CK(cudaStreamSynchronize(stream()));
	return XMG_OK;
}
