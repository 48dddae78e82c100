/*
 * Split-precision emulated FP64 contraction on tcgen05 tensor cores.
 *
 * Replaces the reference's per-pair dgemm (contract.c:193-218) for every
 * canonical output block whose merged pair factors are signed powers of
 * two (always the case for (anti)symmetric tensors).  Three kernels:
 *
 *  1. emu_exp_kernel   - per operand view, the largest binary exponent of
 *     every free-index row over all contracted elements, max-reduced into
 *     tables shared by all views with the same free block index, so that
 *     every pair of an output block uses the same row/column scaling.
 *  2. emu_split_kernel - the unfold (permutation gather through the view's
 *     offset tables) fused with the split: each FP64 element becomes a
 *     47-bit fixed-point integer relative to its row exponent, cut into 6
 *     signed base-256 digits d_t in [-128, 128]; digit t is stored as the
 *     bf16 value d_t * 2^(-8t) (exact: at most 8 significant bits).  Only
 *     integer and FP32 arithmetic is used -- GB300's FP64 rate is ~1 TFLOP/s.
 *     Output is pre-tiled in the exact shared-memory image the MMA reads
 *     (no-swizzle K-major core matrices), so the GEMM loads a stage with
 *     two 1-D bulk copies.
 *  3. emu_gemm_kernel  - one CTA per (output block, 128 x 128 tile); warp 0
 *     streams stages with cp.async.bulk, warp 1 issues the 21 triangular
 *     slice products (p + q <= 5) per 16-wide K step with
 *     tcgen05.mma.kind::f16 (bf16 x bf16 -> fp32) into four TMEM
 *     accumulators: weight groups 0, 1, 2 (exact: at most 3*160*2^14 <
 *     2^23 per 160-element chunk) and a rounded low band for groups 3..5.
 *     Warps 2..9 drain the accumulators every chunk into per-thread int64
 *     fixed-point sums (units 2^(-16-F)), applying the pair's sign and
 *     power-of-two factor exactly.  The epilogue is the only FP64 work:
 *     C = alpha * 2^(eA + eB - 2074 - F) * V + beta * C, scattered through
 *     the output block's fold tables.
 *
 * Every mbarrier wait is bounded (2 s of %globaltimer); on timeout the
 * kernel records an error, waits (bounded) for its own copies and MMAs,
 * frees TMEM and returns, and the host reports XMG_ETIMEOUT.
 */
#include <algorithm>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"

namespace xmg {

constexpr int EMU_S = 6;                 /* slices per operand */
constexpr int EMU_TM = 128;              /* rows per tile, both operands */
constexpr int EMU_KS = 16;               /* K per stage = K per MMA */
constexpr int EMU_CHUNK = 10;            /* K steps per exact chunk (160) */
constexpr int EMU_NST = 4;               /* pipeline stages */
constexpr int SLICE_BYTES = EMU_TM * EMU_KS * 2;          /* 4096 */
constexpr int CHUNK_BYTES = EMU_S * SLICE_BYTES;          /* 24576 */
constexpr int STAGE_BYTES = 2 * CHUNK_BYTES;              /* 49152 */
constexpr int GEMM_THREADS = 320;                         /* 10 warps */
constexpr int SMEM_BYTES = EMU_NST * STAGE_BYTES + 1024;
constexpr uint64_t WAIT_NS = 2000000000ull;               /* 2 s */

/* tcgen05 instruction descriptor, kind::f16: D f32, A/B bf16, both
 * K-major, N = 128 (bits 17-22: N >> 3), M = 128 (bits 24-28: M >> 4) */
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) |
    ((uint32_t)(128 >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

struct emu_item {
	int32_t cblock, j0, i0, pad;
};

/* ------------------------------------------------------------------ */
/* PTX wrappers                                                        */

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

/* Bounded wait; false on timeout or when another role already failed. */
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
    volatile int *s_err, int *g_err, int code)
{
	if (mbar_try(bar, parity))
		return true;
	uint64_t t0 = gtimer();
	for (;;) {
		if (mbar_try(bar, parity))
			return true;
		if (*s_err)
			return false;
		if (gtimer() - t0 > WAIT_NS) {
			*s_err = code;
			atomicMax(g_err, code);
			return false;
		}
	}
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src,
    uint32_t bytes, uint32_t bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
	    " [%0], [%1], %2, [%3];" :: "r"(dst), "l"(src), "r"(bytes), "r"(bar)
	    : "memory");
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
 * of a 16-wide K step, SBO = 256 B between 8-row groups; bits 46-48 = 1 */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) |
	    ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
	    (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b,
    uint32_t acc)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
	    :: "r"(d), "l"(a), "l"(b), "r"(IDESC), "r"(acc));
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

/* ------------------------------------------------------------------ */
/* 1. exponent tables                                                  */

struct view_meta {
	int64_t first_cta;
};

__device__ __forceinline__ int find_view(const view_meta *m, int n, int64_t cta)
{
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (m[mid].first_cta <= cta) lo = mid; else hi = mid - 1;
	}
	return lo;
}

/* biased exponent of |x| (0 for zero / subnormal) */
__device__ __forceinline__ int bexp(double x)
{
	return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}

/* CTA = (view, 128-row tile, 256-wide K range); rows are the view's free
 * indices, K its contracted ones. */
__global__ void __launch_bounds__(256)
emu_exp_kernel(const xmgd_view_t *__restrict__ views,
    const view_meta *__restrict__ meta, int nviews,
    const int32_t *__restrict__ tabs, int32_t *__restrict__ E,
    int *__restrict__ flags)
{
	const int v = find_view(meta, nviews, blockIdx.x);
	const xmgd_view_t w = views[v];
	const int64_t local = blockIdx.x - meta[v].first_cta;
	const int nkb = (w.k + 255) / 256;
	const int rt = (int)(local / nkb), kb = (int)(local % nkb);
	const double *X = reinterpret_cast<const double *>(w.ptr);
	const int32_t *rowt = tabs + w.rowtab, *colt = tabs + w.coltab;
	const int k0 = kb * 256, k1 = min(w.k, k0 + 256);
	int bad = 0;

	if (w.kfast) {
		/* K contiguous: a warp walks K for one row at a time */
		const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
		for (int rr = warp; rr < EMU_TM; rr += 8) {
			int r = rt * EMU_TM + rr;
			if (r >= w.mn)
				break;
			int32_t co = colt[r], e = 0;
			for (int k = k0 + lane; k < k1; k += 32) {
				int b = bexp(X[rowt[k] + co]);
				bad |= b == 0x7ff;
				e = max(e, b);
			}
			for (int off = 16; off > 0; off >>= 1)
				e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
			if (lane == 0 && e > 0)
				atomicMax(&E[w.exptab + r], e);
		}
	} else {
		/* free index contiguous: a thread per row, two K halves */
		const int rr = threadIdx.x % EMU_TM, half = threadIdx.x / EMU_TM;
		const int r = rt * EMU_TM + rr;
		if (r < w.mn) {
			int32_t co = colt[r], e = 0;
			for (int k = k0 + half; k < k1; k += 2) {
				int b = bexp(X[rowt[k] + co]);
				bad |= b == 0x7ff;
				e = max(e, b);
			}
			if (e > 0)
				atomicMax(&E[w.exptab + r], e);
		}
	}
	if (bad)
		atomicOr(flags, 1);	/* Inf/NaN: not representable by slices */
}

/* ------------------------------------------------------------------ */
/* 2. unfold + split                                                   */

/* bf16 bits of d * 2^(-8t), exact for |d| <= 256 */
__device__ __forceinline__ uint32_t digit_bf16(int d, float w)
{
	/* exact int -> float for |d| < 2^22 without a conversion unit */
	float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
	return __float_as_uint(f * w) >> 16;
}

/* CTA = (view, 128-row tile, group of 4 K steps); thread = (row, K octet) */
__global__ void __launch_bounds__(256)
emu_split_kernel(const xmgd_view_t *__restrict__ views,
    const view_meta *__restrict__ meta, int nviews,
    const int32_t *__restrict__ tabs, const int32_t *__restrict__ E)
{
	const int v = find_view(meta, nviews, blockIdx.x);
	const xmgd_view_t w = views[v];
	const int64_t local = blockIdx.x - meta[v].first_cta;
	const int ngrp = (w.n_ks + 3) / 4;
	const int rt = (int)(local / ngrp), g = (int)(local % ngrp);
	const int rr = threadIdx.x % EMU_TM, oct = threadIdx.x / EMU_TM;
	const int r = rt * EMU_TM + rr;
	const double *X = reinterpret_cast<const double *>(w.ptr);
	const int32_t *rowt = tabs + w.rowtab, *colt = tabs + w.coltab;
	const bool live = r < w.mn;
	const int32_t co = live ? colt[r] : 0;
	const int er = live ? E[w.exptab + r] : 0;
	uint16_t *out = reinterpret_cast<uint16_t *>(w.slices);

	for (int ks = g * 4; ks < min(w.n_ks, g * 4 + 4); ks++) {
		uint32_t bits[EMU_S][4];
#pragma unroll
		for (int s = 0; s < EMU_S; s++)
#pragma unroll
			for (int q = 0; q < 4; q++)
				bits[s][q] = 0;
#pragma unroll
		for (int e = 0; e < 8; e++) {
			int k = ks * EMU_KS + oct * 8 + e;
			double x = (live && k < w.k) ? X[rowt[k] + co] : 0.0;
			long long xb = __double_as_longlong(x);
			int eb = (int)((xb >> 52) & 0x7ff);
			long long m = xb & 0xFFFFFFFFFFFFFll;
			if (eb == 0)
				eb = 1;		/* subnormal */
			else
				m |= 1ll << 52;
			/* X = round(m * 2^(eb - er - 6)), |X| <= 2^47 */
			int sh = er - eb + 6;
			long long xi = sh >= 63 ? 0 : ((m + (1ll << (sh - 1))) >> sh);
			if (xb < 0)
				xi = -xi;
			int d[EMU_S];
#pragma unroll
			for (int t = EMU_S - 1; t >= 1; t--) {
				d[t] = (int)(((xi + 128) & 255) - 128);
				xi = (xi - d[t]) >> 8;
			}
			d[0] = (int)xi;
#pragma unroll
			for (int t = 0; t < EMU_S; t++) {
				uint32_t h = digit_bf16(d[t], __int_as_float((127 - 8 * t) << 23));
				bits[t][e >> 1] |= h << (16 * (e & 1));
			}
		}
		/* core matrix row: slice t, row r, K octet -> 16 bytes */
		size_t chunk = ((size_t)rt * w.n_ks + ks) * (CHUNK_BYTES / 2);
		size_t within = (size_t)((rr >> 3) * 2 + oct) * 64 + (rr & 7) * 8;
#pragma unroll
		for (int t = 0; t < EMU_S; t++) {
			uint4 val = make_uint4(bits[t][0], bits[t][1], bits[t][2], bits[t][3]);
			*reinterpret_cast<uint4 *>(out + chunk + t * (SLICE_BYTES / 2) + within) = val;
		}
	}
}

/* ------------------------------------------------------------------ */
/* 3. grouped tcgen05 GEMM with exact drains and the fused fold        */

__global__ void __launch_bounds__(GEMM_THREADS, 1)
emu_gemm_kernel(const emu_item *__restrict__ items,
    const xmgd_cblock_t *__restrict__ cbs, const xmgd_pair_t *__restrict__ prs,
    const xmgd_view_t *__restrict__ va, const xmgd_view_t *__restrict__ vb,
    const int32_t *__restrict__ tabs, const int32_t *__restrict__ EA,
    const int32_t *__restrict__ EB, const int32_t *__restrict__ cbF,
    double alpha, double beta, int *__restrict__ g_err)
{
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	uint8_t *stages = reinterpret_cast<uint8_t *>(
	    (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
	__shared__ __align__(8) uint64_t bar_full[EMU_NST], bar_empty[EMU_NST];
	__shared__ __align__(8) uint64_t bar_accfull, bar_accempty, bar_fin;
	__shared__ uint32_t s_tmem;
	__shared__ volatile int s_err;

	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const emu_item it = items[blockIdx.x];
	const xmgd_cblock_t cb = cbs[it.cblock];
	const int F = cbF[it.cblock];

	if (threadIdx.x == 0) {
		for (int s = 0; s < EMU_NST; s++) {
			mbar_init(smem_u32(&bar_full[s]), 1);
			mbar_init(smem_u32(&bar_empty[s]), 1);
		}
		mbar_init(smem_u32(&bar_accfull), 1);
		mbar_init(smem_u32(&bar_accempty), 8);
		mbar_init(smem_u32(&bar_fin), 1);
		s_err = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 1) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;"
		    :: "r"(smem_u32(&s_tmem)));
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = s_tmem;

	if (warp == 0) {
		/* ---------------- producer ---------------- */
		if (lane == 0) {
			int s = 0;
			uint32_t ph = 0;
			int lastp[EMU_NST];
#pragma unroll
			for (int q = 0; q < EMU_NST; q++)
				lastp[q] = -1;
			for (int p = 0; p < cb.npairs && !s_err; p++) {
				const xmgd_pair_t pr = prs[cb.first_pair + p];
				const xmgd_view_t wb = vb[pr.bview], wa = va[pr.aview];
				const uint8_t *gb = reinterpret_cast<const uint8_t *>(wb.slices) +
				    (size_t)(it.j0 / EMU_TM) * wb.n_ks * CHUNK_BYTES;
				const uint8_t *ga = reinterpret_cast<const uint8_t *>(wa.slices) +
				    (size_t)(it.i0 / EMU_TM) * wa.n_ks * CHUNK_BYTES;
				for (int ks = 0; ks < wb.n_ks; ks++) {
					if (!mbar_wait(smem_u32(&bar_empty[s]), ph ^ 1, &s_err, g_err, 1))
						break;
					uint32_t dst = smem_u32(stages + (size_t)s * STAGE_BYTES);
					uint32_t fb = smem_u32(&bar_full[s]);
					mbar_expect_tx(fb, STAGE_BYTES);
					bulk_g2s(dst, gb + (size_t)ks * CHUNK_BYTES, CHUNK_BYTES, fb);
					bulk_g2s(dst + CHUNK_BYTES, ga + (size_t)ks * CHUNK_BYTES, CHUNK_BYTES, fb);
#pragma unroll
					for (int q = 0; q < EMU_NST; q++)
						if (q == s)
							lastp[q] = (int)ph;
					if (++s == EMU_NST) { s = 0; ph ^= 1; }
				}
			}
			/* on failure, let this CTA's copies still in flight land
			 * before it exits (bounded): the last phase issued on each
			 * stage completes when its bytes have arrived */
			if (s_err) {
				uint64_t t0 = gtimer();
#pragma unroll
				for (int q = 0; q < EMU_NST; q++)
					if (lastp[q] >= 0)
						while (!mbar_try(smem_u32(&bar_full[q]), (uint32_t)lastp[q]) &&
						    gtimer() - t0 < WAIT_NS)
							;
			}
		}
	} else if (warp == 1) {
		/* ---------------- MMA issuer ---------------- */
		if (lane == 0) {
			int s = 0, chunk = 0;
			uint32_t ph = 0, eph = 0;
			for (int p = 0; p < cb.npairs && !s_err; p++) {
				const xmgd_pair_t pr = prs[cb.first_pair + p];
				const int nks = vb[pr.bview].n_ks;
				for (int c0 = 0; c0 < nks && !s_err; c0 += EMU_CHUNK) {
					if (chunk > 0) {
						if (!mbar_wait(smem_u32(&bar_accempty), eph, &s_err, g_err, 2))
							break;
						eph ^= 1;
					}
					tc_fence_after();
					/* every accumulator restarts each chunk: the exact
					 * groups for their 2^23 bound, the low band because the
					 * tensor core's fp32 accumulation error grows with the
					 * accumulation length (per-pair accumulation measured
					 * 10x larger error) */
					uint32_t started = 0;
					const int c1 = min(nks, c0 + EMU_CHUNK);
					for (int ks = c0; ks < c1; ks++) {
						if (!mbar_wait(smem_u32(&bar_full[s]), ph, &s_err, g_err, 3))
							break;
						tc_fence_after();
						const uint32_t base = smem_u32(stages + (size_t)s * STAGE_BYTES);
#pragma unroll
						for (int pa = 0; pa < EMU_S; pa++)
#pragma unroll
							for (int qb = 0; qb < EMU_S - pa; qb++) {
								const int acc = min(pa + qb, 3);
								uint64_t ad = sdesc(base + qb * SLICE_BYTES);
								uint64_t bd = sdesc(base + CHUNK_BYTES + pa * SLICE_BYTES);
								mma_bf16(tmem + acc * 128, ad, bd, (started >> acc) & 1u);
								started |= 1u << acc;
							}
						mma_commit(smem_u32(&bar_empty[s]));
						if (++s == EMU_NST) { s = 0; ph ^= 1; }
					}
					mma_commit(smem_u32(&bar_accfull));
					chunk++;
				}
			}
			/* every MMA issued by this CTA has completed once bar_fin
			 * fires; TMEM is released only after that */
			mma_commit(smem_u32(&bar_fin));
			uint64_t t0 = gtimer();
			while (!mbar_try(smem_u32(&bar_fin), 0) && gtimer() - t0 < WAIT_NS)
				;
		}
	} else {
		/* ---------------- drain + epilogue (warps 2..9) ---------------- */
		const int quad = warp & 3, half = (warp - 2) >> 2;
		const uint32_t trow = tmem + ((uint32_t)(quad * 32) << 16) + half * 64;
		long long V[64];
#pragma unroll
		for (int c = 0; c < 64; c++)
			V[c] = 0;
		uint32_t fph = 0;
		bool ok = true;
		for (int p = 0; p < cb.npairs && ok; p++) {
			const xmgd_pair_t pr = prs[cb.first_pair + p];
			const int nks = vb[pr.bview].n_ks;
			/* the pair factor sign * 2^shift (shift 0 or 1, checked by
			 * the planner) rides on the exact fp32 -> int scales */
			const float sg = pr.esign > 0 ? 1.0f : -1.0f;
			const float s0 = sg * __int_as_float((127 + pr.eshift) << 23);
			const float s1 = s0 * 256.0f, s2 = s0 * 65536.0f;
			const float s3 = s0 * __int_as_float((127 + 16 + F) << 23);
			for (int c0 = 0; c0 < nks; c0 += EMU_CHUNK) {
				/* one lane waits, the warp follows its verdict, so the
				 * .sync.aligned TMEM loads below stay convergent */
				int w = 1;
				if (lane == 0)
					w = mbar_wait(smem_u32(&bar_accfull), fph, &s_err, g_err, 4);
				w = __shfl_sync(0xffffffffu, w, 0);
				if (!w) {
					ok = false;
					break;
				}
				fph ^= 1;
				tc_fence_after();
#pragma unroll
				for (int b8 = 0; b8 < 8; b8++) {
					float a0[8], a1[8], a2[8], a3[8];
					tmem_ld8(trow + 0 * 128 + b8 * 8, a0);
					tmem_ld8(trow + 1 * 128 + b8 * 8, a1);
					tmem_ld8(trow + 2 * 128 + b8 * 8, a2);
					tmem_ld8(trow + 3 * 128 + b8 * 8, a3);
					tmem_wait_ld();
#pragma unroll
					for (int c = 0; c < 8; c++) {
						/* exact integers: |i0| <= 2^22.4, |i1| <= 2^23.4,
						 * |i0 * 256 + i1| < 2^31 */
						int i0 = __float2int_rn(a0[c] * s0);
						int i1 = __float2int_rn(a1[c] * s1);
						int i2 = __float2int_rn(a2[c] * s2);
						long long d = ((long long)(i0 * 256 + i1) << 8) + i2;
						V[b8 * 8 + c] += (d << F) + __float2ll_rn(a3[c] * s3);
					}
				}
				tc_fence_before();
				__syncwarp();
				if (lane == 0)
					mbar_arrive(smem_u32(&bar_accempty));
			}
		}
		if (ok && !s_err) {
			const int j = it.j0 + quad * 32 + lane;
			if (j < cb.n) {
				double *C = reinterpret_cast<double *>(cb.c_ptr);
				const int32_t *crow = tabs + cb.crow;
				const int32_t cc = tabs[cb.ccol + j];
				const int ej = EB[cb.eB + j];
				const bool bz = beta == 0.0;
#pragma unroll
				for (int c = 0; c < 64; c++) {
					const int i = it.i0 + half * 64 + c;
					if (i < cb.m) {
						const int e = EA[cb.eA + i] + ej - 2074 - F;
						double v = alpha * ldexp((double)V[c], e);
						double *cp = C + crow[i] + cc;
						*cp = bz ? v : fma(beta, *cp, v);
					}
				}
			}
		}
	}

	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 1)
		asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;"
		    :: "r"(tmem));
}

/* ------------------------------------------------------------------ */
/* host orchestration                                                  */

static int
upload_slot(int slot, const void *h, size_t bytes, uint64_t *d)
{
	int st;

	if ((st = xmgd_scratch(slot, bytes ? bytes : 16, d)) != XMG_OK)
		return st;
	if (bytes)
		return check(cudaMemcpyAsync((void *)*d, h, bytes,
		    cudaMemcpyHostToDevice, stream()), "emu upload");
	return XMG_OK;
}

int
emu_contract(xmgd_contract_t *p, const std::vector<int> &cblocks,
    const xmgd_cblock_t *d_cbs, const xmgd_pair_t *d_prs,
    const int32_t *d_tabs, xmgd_timing_t *tm)
{
	static bool attr_set = false;
	std::vector<xmgd_view_t> VA(p->views_a, p->views_a + p->nviews_a);
	std::vector<xmgd_view_t> VB(p->views_b, p->views_b + p->nviews_b);
	std::vector<char> useA(VA.size(), 0), useB(VB.size(), 0);
	std::vector<int32_t> F(p->ncblocks, 0);
	std::vector<emu_item> items;
	uint64_t d_slices, d_E, d_va, d_vb, d_items, d_F, d_meta, d_err;
	int st;

	if (p->dtype != 2)
		return xmg_seterr(XMG_ENOTSUP, "split-precision path: double only");
	/* operand views used by the emulated blocks, and the fixed-point
	 * scale F of every block (|V| <= K_eff * 2^(30+F) < 2^61) */
	for (int ci : cblocks) {
		const xmgd_cblock_t &cb = p->cblocks[ci];
		double keff = 0;
		for (int q = 0; q < cb.npairs; q++) {
			const xmgd_pair_t &pr = p->pairs[cb.first_pair + q];
			useA[pr.aview] = useB[pr.bview] = 1;
			keff += ldexp(1.0, std::max(pr.eshift, 0)) * pr.k;
		}
		int lg = (int)ceil(log2(std::max(keff, 2.0)));
		if (lg > 31)
			return xmg_seterr(XMG_ENOTSUP, "split-precision path: K too large");
		F[ci] = std::min(24, 31 - lg);
	}
	/* slice storage */
	size_t off = 0;
	auto tile = [&](std::vector<xmgd_view_t> &V, std::vector<char> &use) {
		for (size_t v = 0; v < V.size(); v++) {
			if (!use[v])
				continue;
			V[v].n_rt = (V[v].mn + EMU_TM - 1) / EMU_TM;
			V[v].n_ks = (V[v].k + EMU_KS - 1) / EMU_KS;
			V[v].kfast = V[v].k > 1 && p->tabs[V[v].rowtab + 1] - p->tabs[V[v].rowtab] == 1;
			V[v].slices = off;
			off += (size_t)V[v].n_rt * V[v].n_ks * CHUNK_BYTES;
		}
	};
	tile(VA, useA);
	tile(VB, useB);
	if ((st = xmgd_scratch(8, off, &d_slices)) != XMG_OK)
		return st;
	for (size_t v = 0; v < VA.size(); v++)
		if (useA[v]) VA[v].slices += d_slices;
	for (size_t v = 0; v < VB.size(); v++)
		if (useB[v]) VB[v].slices += d_slices;
	tm->slice_bytes = (int64_t)off;

	size_t nE = (size_t)p->nexp_a + p->nexp_b;
	if ((st = xmgd_scratch(9, (nE + 64) * sizeof(int32_t), &d_E)) != XMG_OK)
		return st;
	XMG_CK(cudaMemsetAsync((void *)d_E, 0, (nE + 64) * sizeof(int32_t), stream()));
	int32_t *EA = (int32_t *)d_E, *EB = EA + p->nexp_a;
	d_err = (uint64_t)(EB + p->nexp_b);	/* flags live after the tables */
	if ((st = upload_slot(10, VA.data(), VA.size() * sizeof(xmgd_view_t), &d_va)) ||
	    (st = upload_slot(11, VB.data(), VB.size() * sizeof(xmgd_view_t), &d_vb)))
		return st;

	cudaEvent_t e0, e1, e2;
	XMG_CK(cudaEventCreate(&e0));
	XMG_CK(cudaEventCreate(&e1));
	XMG_CK(cudaEventCreate(&e2));
	XMG_CK(cudaEventRecord(e0, stream()));

	/* exponent and split launches over the used views of each side */
	for (int side = 0; side < 2; side++) {
		std::vector<xmgd_view_t> &V = side ? VB : VA;
		std::vector<char> &use = side ? useB : useA;
		const xmgd_view_t *dv = (const xmgd_view_t *)(side ? d_vb : d_va);
		int32_t *E = side ? EB : EA;
		for (int kind = 0; kind < 2; kind++) {
			std::vector<view_meta> meta(V.size());
			int64_t n = 0;
			for (size_t v = 0; v < V.size(); v++) {
				meta[v].first_cta = n;
				if (!use[v])
					continue;
				if (kind == 0)
					n += (int64_t)V[v].n_rt * ((V[v].k + 255) / 256);
				else
					n += (int64_t)V[v].n_rt * ((V[v].n_ks + 3) / 4);
			}
			if (n == 0)
				continue;
			if ((st = upload_slot(12 + kind, meta.data(), meta.size() *
			    sizeof(view_meta), &d_meta)))
				return st;
			if (kind == 0)
				emu_exp_kernel<<<(unsigned)n, 256, 0, stream()>>>(dv,
				    (const view_meta *)d_meta, (int)V.size(), d_tabs, E,
				    (int *)d_err);
			else
				emu_split_kernel<<<(unsigned)n, 256, 0, stream()>>>(dv,
				    (const view_meta *)d_meta, (int)V.size(), d_tabs, E);
			g_launches++;
			XMG_CK(cudaGetLastError());
			/* the meta buffer is reused by the next launch */
			XMG_CK(cudaStreamSynchronize(stream()));
		}
	}
	int flags[2] = {0, 0};
	XMG_CK(cudaMemcpy(flags, (void *)d_err, sizeof flags, cudaMemcpyDeviceToHost));
	if (flags[0] & 1)
		return xmg_seterr(XMG_ENOTSUP, "split-precision path: Inf/NaN in operands");
	XMG_CK(cudaEventRecord(e1, stream()));

	/* work list: output blocks by decreasing cost, tiles adjacent */
	std::vector<std::pair<double, int>> order;
	for (int ci : cblocks) {
		const xmgd_cblock_t &cb = p->cblocks[ci];
		double c = 0;
		for (int q = 0; q < cb.npairs; q++)
			c += p->pairs[cb.first_pair + q].k;
		order.push_back({-c * cb.m * (double)cb.n, ci});
	}
	std::stable_sort(order.begin(), order.end());
	for (auto &o : order) {
		const xmgd_cblock_t &cb = p->cblocks[o.second];
		for (int j0 = 0; j0 < cb.n; j0 += EMU_TM)
			for (int i0 = 0; i0 < cb.m; i0 += EMU_TM)
				items.push_back(emu_item{o.second, j0, i0, 0});
	}
	if ((st = upload_slot(14, items.data(), items.size() * sizeof(emu_item), &d_items)) ||
	    (st = upload_slot(15, F.data(), F.size() * sizeof(int32_t), &d_F)))
		return st;
	if (!attr_set) {
		XMG_CK(cudaFuncSetAttribute(emu_gemm_kernel,
		    cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
		attr_set = true;
	}
	emu_gemm_kernel<<<(unsigned)items.size(), GEMM_THREADS, SMEM_BYTES, stream()>>>(
	    (const emu_item *)d_items, d_cbs, d_prs, (const xmgd_view_t *)d_va,
	    (const xmgd_view_t *)d_vb, d_tabs, EA, EB, (const int32_t *)d_F,
	    p->alpha[0], p->beta[0], (int *)d_err + 1);
	g_launches++;
	XMG_CK(cudaGetLastError());
	XMG_CK(cudaEventRecord(e2, stream()));
	XMG_CK(cudaEventSynchronize(e2));
	float ms1 = 0, ms2 = 0;
	cudaEventElapsedTime(&ms1, e0, e1);
	cudaEventElapsedTime(&ms2, e1, e2);
	tm->ms_split += ms1;
	tm->ms_gemm += ms2;
	tm->gemm_launches += 1;
	tm->gemm_items += (int32_t)items.size();
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaEventDestroy(e2);
	XMG_CK(cudaMemcpy(flags, (void *)d_err, sizeof flags, cudaMemcpyDeviceToHost));
	if (flags[1])
		return xmg_seterr(XMG_ETIMEOUT, "split-precision GEMM: bounded "
		    "wait %d timed out", flags[1]);
	return XMG_OK;
}

} /* namespace xmg */
