/*
 * Failure detection without a fault: one CTA waits on an mbarrier that
 * nothing arrives at, through the same bounded-wait path every pipeline
 * wait of the GEMM kernels takes, gives up after the limit, records the
 * error code and returns.  The host reads the code; the context stays
 * usable.  No counterpart in the reference.
 */
#include "common.cuh"
#include "tc.cuh"

namespace xmg {

__global__ void
selftest_wait_kernel(uint64_t limit_ns, int *flag)
{
	__shared__ __align__(8) uint64_t bar;
	__shared__ volatile int s_err;

	if (threadIdx.x == 0) {
		mbar_init(smem_u32(&bar), 1);
		s_err = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	if (threadIdx.x == 0)
		mbar_wait_for(smem_u32(&bar), 0, &s_err, flag, 11, limit_ns);
	__syncwarp();	/* lane 0 rejoins before the aligned barrier */
	__syncthreads();
}

} /* namespace xmg */

using namespace xmg;

extern "C" int
xmg_selftest_bounded_wait(unsigned timeout_us)
{
	int st, *d = nullptr, h = 0;

	if ((st = xmgd_init()) != XMG_OK)
		return st;
	XMG_CK(cudaMalloc(&d, sizeof(int)));
	st = check(cudaMemsetAsync(d, 0, sizeof(int), stream()), "self-test");
	if (st == XMG_OK) {
		selftest_wait_kernel<<<1, 32, 0, stream()>>>((uint64_t)timeout_us * 1000, d);
		g_launches++;
		st = check(cudaGetLastError(), "self-test launch");
	}
	if (st == XMG_OK)
		st = check(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost,
		    stream()), "self-test");
	if (st == XMG_OK)
		st = check(cudaStreamSynchronize(stream()), "self-test");
	cudaFree(d);
	if (st != XMG_OK)
		return st;
	if (h)
		return xmg_seterr(XMG_ETIMEOUT, "bounded wait %d gave up after %u us",
		    h, timeout_us);
	return XMG_OK;
}
