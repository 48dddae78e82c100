/*
 * Inline-PTX helpers for Blackwell kernels: mbarriers with bounded waits,
 * 1-D bulk copies, tcgen05 MMA / commit / TMEM loads, shared-memory
 * matrix descriptors (no swizzle, K-major).
 */
#ifndef XMG_TC_CUH
#define XMG_TC_CUH

#include <stdint.h>

namespace xmg {

constexpr uint64_t WAIT_NS = 2000000000ull;	/* bounded waits: 2 s */

/* tcgen05 instruction descriptor, kind::f16: D f32 (bits 4-5), A and B
 * bf16 (bits 7-9, 10-12), both K-major, M = 128 (bits 24-28: M >> 4); N
 * (bits 17-22: N >> 3, a multiple of 16 up to 256) is set per tile */
constexpr uint32_t IDESC_M128 = (1u << 4) | (1u << 7) | (1u << 10) |
    ((uint32_t)(128 >> 4) << 24);

__host__ __device__ constexpr uint32_t idesc_n(int n)
{
	return IDESC_M128 | ((uint32_t)(n >> 3) << 17);
}

/* M = 256 over a CTA pair */
__host__ __device__ constexpr uint32_t idesc_pair_n(int n)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(256 >> 4) << 24) |
	    ((uint32_t)(n >> 3) << 17);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gtimer()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
	    :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
	    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
	return ok != 0;
}

/* Bounded wait; false on timeout (after limit_ns, recording `code` in the
 * CTA's and the launch's error flags) or when another role already failed. */
__device__ __forceinline__ bool mbar_wait_for(uint32_t bar, uint32_t parity,
    volatile int *s_err, int *g_err, int code, uint64_t limit_ns)
{
	if (mbar_try(bar, parity))
		return true;
	uint64_t t0 = gtimer();
	for (uint32_t n = 1;; n++) {
		if (mbar_try(bar, parity))
			return true;
		/* the failure flag and the clock only every 16th poll: each
		 * shared-memory read competes with the tensor core's operand
		 * reads */
		if ((n & 15) == 0) {
			if (*s_err)
				return false;
			if (gtimer() - t0 > limit_ns) {
				*s_err = code;
				atomicMax(g_err, code);
				return false;
			}
		}
	}
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
    volatile int *s_err, int *g_err, int code)
{
	return mbar_wait_for(bar, parity, s_err, g_err, code, WAIT_NS);
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src,
    uint32_t bytes, uint32_t bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
	    " [%0], [%1], %2, [%3];" :: "r"(dst), "l"(src), "r"(bytes), "r"(bar)
	    : "memory");
}

/* bring [src, src + bytes) into L2 ahead of its shared-memory copy
 * (address and size multiples of 16 bytes) */
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes)
{
	asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;"
	    :: "l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tc_fence_before()
{
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* shared-memory matrix descriptor: no swizzle, K-major core matrices of
 * 8 rows x 16 bytes; LBO = 128 B between the two K-adjacent core matrices
 * of a 16-wide K step, SBO = byte distance between 8-row groups; bits
 * 46-48 = 0b001 (tcgen05 descriptor version) */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t sbo)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) |
	    ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
	    (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b,
    uint32_t idesc, uint32_t acc)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
	    :: "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

/* the same with each descriptor passed as (low, high) words */
__device__ __forceinline__ void mma_bf16_split(uint32_t d, uint32_t alo,
    uint32_t ahi, uint32_t blo, uint32_t bhi, uint32_t idesc, uint32_t acc)
{
	asm volatile("{\n\t.reg .pred p;\n\t.reg .b64 a, b;\n\t"
	    "mov.b64 a, {%1, %2};\n\tmov.b64 b, {%3, %4};\n\t"
	    "setp.ne.b32 p, %6, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], a, b, %5, p;\n\t}"
	    :: "r"(d), "r"(alo), "r"(ahi), "r"(blo), "r"(bhi), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
	    :: "r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
	uint32_t r[8];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 "
	    "{%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]),
	      "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
	    : "r"(taddr));
#pragma unroll
	for (int i = 0; i < 8; i++)
		v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4])
{
	uint32_t r[4];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(taddr));
#pragma unroll
	for (int i = 0; i < 4; i++)
		v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
	    "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]),
	      "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
	      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
	      "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr));
#pragma unroll
	for (int i = 0; i < 16; i++)
		v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld()
{
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* ---- CTA pairs (cluster of two, cta_group::2) ----------------------- */

__device__ __forceinline__ uint32_t cluster_rank()
{
	uint32_t r;
	asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
	return r;
}

/* the shared::cluster address of `addr` (a shared::cta address of this
 * CTA's layout) in the CTA of cluster rank `rank` */
__device__ __forceinline__ uint32_t map_shared(uint32_t addr, uint32_t rank)
{
	uint32_t r;
	asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
	return r;
}

__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr)
{
	asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];"
	    :: "r"(cluster_addr) : "memory");
}

__device__ __forceinline__ void st_remote_u32(uint32_t cluster_addr, uint32_t v)
{
	asm volatile("st.shared::cluster.u32 [%0], %1;" :: "r"(cluster_addr), "r"(v) : "memory");
}

/* try-wait with cluster-scope acquire: for barriers that peers arrive on */
__device__ __forceinline__ bool mbar_try_cl(uint32_t bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
	    "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
	return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_cl(uint32_t bar, uint32_t parity,
    volatile int *s_err, int *g_err, int code)
{
	if (mbar_try_cl(bar, parity))
		return true;
	uint64_t t0 = gtimer();
	for (uint32_t n = 1;; n++) {
		if (mbar_try_cl(bar, parity))
			return true;
		if ((n & 15) == 0) {
			if (*s_err)
				return false;
			if (gtimer() - t0 > WAIT_NS) {
				*s_err = code;
				atomicMax(g_err, code);
				return false;
			}
		}
	}
}

/* all threads of both CTAs */
__device__ __forceinline__ void cluster_sync()
{
	asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
	    "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

/* tensor-core MMA over the CTA pair: M = 256 (128 rows from each CTA's
 * shared memory at the same offset), the N side split between the CTAs'
 * shared memory, each CTA's TMEM receiving its 128 rows */
__device__ __forceinline__ void mma_bf16_pair(uint32_t d, uint32_t alo,
    uint32_t ahi, uint32_t blo, uint32_t bhi, uint32_t idesc, uint32_t acc)
{
	asm volatile("{\n\t.reg .pred p;\n\t.reg .b64 a, b;\n\t"
	    "mov.b64 a, {%1, %2};\n\tmov.b64 b, {%3, %4};\n\t"
	    "setp.ne.b32 p, %6, 0;\n\t"
	    "tcgen05.mma.cta_group::2.kind::f16 [%0], a, b, %5, p;\n\t}"
	    :: "r"(d), "r"(alo), "r"(ahi), "r"(blo), "r"(bhi), "r"(idesc), "r"(acc));
}

/* arrive on the barrier at this offset in both CTAs once every earlier
 * pair MMA of this thread has completed */
__device__ __forceinline__ void mma_commit_pair(uint32_t bar)
{
	asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster"
	    ".multicast::cluster.b64 [%0], %1;" :: "r"(bar), "h"((uint16_t)3) : "memory");
}


} /* namespace xmg */

#endif
