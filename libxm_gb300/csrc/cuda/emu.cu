/*
 * Split-precision contraction on tcgen05 tensor cores.
 *
 * Replaces the reference's per-pair ?gemm_ calls (contract.c:193-218) for
 * every canonical output block whose merged pair factors are +-1 or +-2
 * (always the case for (anti)symmetric tensors).  Two schemes share the
 * code:
 *
 *   FP64 ("emulated FP64"): 6 signed 8-bit slices per element (47-bit
 *     fixed point), the 21 slice products with p + q <= 5; weight groups
 *     0, 1, 2 accumulate exactly, groups 3..5 form a rounded low band.
 *   FP32 ("compensated bf16 split"): 3 slices (23-bit fixed point), the 6
 *     products with p + q <= 2, all exact -- no FP32 rounding at all.
 *
 * Complex types use the real-GEMM decomposition: each complex operand view
 * is realified along K as [re | im] (each half padded to 16), and the
 * output is computed in two passes over the same slices,
 *     pass 0: re(C) = A_re B_re - A_im B_im   (second half drained negated)
 *     pass 1: im(C) = A_re B_im + A_im B_re   (B halves swapped)
 *
 * Kernels:
 *  1. emu_exp_kernel   - largest binary exponent of every free-index row of
 *     each operand view over all contracted elements (re and im), max-reduced
 *     into tables shared by all views with the same free block index, so
 *     every pair of an output block uses the same row/column scaling.
 *  2. emu_split_kernel - the unfold (permutation gather through the view's
 *     offset tables) fused with the split: each element becomes a fixed-
 *     point integer relative to its row exponent, cut into balanced base-256
 *     digits d_t in [-128, 128]; digit t is stored as bf16 d_t * 2^(-8t)
 *     (exact).  Integer and FP32 arithmetic only -- GB300's FP64 pipe runs at
 *     ~1 TFLOP/s.  The output is pre-tiled in the exact shared-memory image
 *     the MMA reads (no-swizzle K-major core matrices), so the GEMM loads a
 *     pipeline stage with two 1-D bulk copies.
 *  3. emu_gemm_kernel  - one CTA per (output block, 128 x 128 tile, pass);
 *     warp 0 streams stages with cp.async.bulk, warp 1 issues the slice
 *     products per 16-wide K step with tcgen05.mma.kind::f16 (bf16 x bf16 ->
 *     fp32) into TMEM accumulators, warps 2..17 drain them every 256 K
 *     elements for FP64 and every <= 336 for FP32 (the exact groups stay
 *     below 3 * 336 * 2^14 < 2^24, exact in fp32) into
 *     per-thread int64 fixed-point sums in units of 2^(-16-F), applying the
 *     pair factor exactly.  The epilogue is the only FP64 work:
 *     C = alpha * 2^(eA + eB - 2 * EXPOFF - 16 - F) * V + beta * C, scattered
 *     through the output block's fold tables.
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
#include "tc.cuh"

namespace xmg {

constexpr int EMU_TM = 128;              /* rows per tile, both operands */
constexpr int EMU_KS = 16;               /* K per stage = K per MMA */
constexpr int EMU_CHUNK = 16;            /* K steps per chunk, FP64 (256) */
constexpr int EMU_CHUNK32 = 20;          /* K steps per chunk at most, FP32 */
constexpr int SLICE_BYTES = EMU_TM * EMU_KS * 2;          /* 4096 */
#ifndef EMU_DW
#define EMU_DW 16                        /* drain warps: 8 or 16 */
#endif
constexpr int STAGE_BUDGET = 196608;                      /* 192 KiB */

/* input element traits: slices, kept products, fixed-point bits */
template <typename T> struct fin;
template <> struct fin<double> {
	static constexpr int S = 6, KEEP = 5, T1 = 47, MANT = 52, EMAX = 0x7ff;
	static constexpr int EXPOFF = 47 + 1022 - 8 * (6 - 1);    /* 1029 */
	__device__ static inline void parts(double x, long long &m, int &eb, bool &neg)
	{
		long long b = __double_as_longlong(x);
		eb = (int)((b >> 52) & 0x7ff);
		m = b & 0xFFFFFFFFFFFFFll;
		if (eb == 0) eb = 1; else m |= 1ll << 52;
		neg = b < 0;
	}
	__device__ static inline int bexp(double x)
	{ return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }
};
template <> struct fin<float> {
	static constexpr int S = 3, KEEP = 2, T1 = 23, MANT = 23, EMAX = 0xff;
	static constexpr int EXPOFF = 23 + 126 - 8 * (3 - 1);     /* 133 */
	__device__ static inline void parts(float x, long long &m, int &eb, bool &neg)
	{
		unsigned b = __float_as_uint(x);
		eb = (int)((b >> 23) & 0xff);
		m = b & 0x7fffff;
		if (eb == 0) eb = 1; else m |= 1ll << 23;
		neg = (b >> 31) != 0;
	}
	__device__ static inline int bexp(float x)
	{ return (int)((__float_as_uint(x) >> 23) & 0xff); }
};

/* One work item: up to EMU_MAXMEM output blocks (members mfirst ..
 * mfirst + mcount - 1) stacked along one side of a 128 x N tile that share
 * the other side; pr = pass (bit 0) | swap (bit 1) | M-stacked (bit 2) |
 * live N rows in all << 8 (a multiple of 16).  Without swap b's view is
 * the M side (TMEM lanes) and a's the N side (TMEM columns); swap
 * exchanges them.
 *   N-stacked: m0 is the shared M-side tile (rows m0 .. m0 + 127 of the
 *     M-side view); each member is an N-side tile of its block at TMEM
 *     columns off .. off + rows - 1 (rows a multiple of 16).
 *   M-stacked: m0 is the shared N-side tile; each member is an M-side
 *     tile of its block at TMEM lanes off .. off + rows - 1 (off and rows
 *     multiples of 32, so a drain warp's lanes lie in one member).
 * Members share the other side pair by pair: the same view and K at every
 * pair index. */
struct emu_item {
	int32_t m0, mfirst, mcount, pr;
};

/* a member: output block, first row of its tile in that block's view on
 * the stacked side, live rows (rounded up), first TMEM column or lane */
struct emu_member {
	int32_t cblock, n0, rows, off;
};
constexpr int EMU_MAXMEM = 4;

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

/* Element (k', r) of a view: real views directly, complex views realified
 * along K as [re | im] with halves of w.khp (zero padding). */
template <typename T>
__device__ __forceinline__ T fetch(const T *X, const int32_t *rowt, int32_t co,
    const xmgd_view_t &w, int k)
{
	if (!w.cplx) {
		return k < w.k ? X[rowt[k] + co] : T(0);
	}
	const int half = k >= w.khp;
	const int kk = k - half * w.khp;
	return kk < w.k ? X[2 * (rowt[kk] + co) + half] : T(0);
}

/* ------------------------------------------------------------------ */
/* 1. exponent tables                                                  */

/* CTA = (view, 128-row tile, 256-wide K range) */
template <typename T>
__global__ void __launch_bounds__(256)
emu_exp_kernel(const xmgd_view_t *__restrict__ views,
    const view_meta *__restrict__ meta, int nviews,
    const int32_t *__restrict__ tabs, int32_t *__restrict__ E,
    int *__restrict__ flags)
{
	const int v = find_view(meta, nviews, blockIdx.x);
	const xmgd_view_t w = views[v];
	const int64_t local = blockIdx.x - meta[v].first_cta;
	const int kall = w.n_ks * EMU_KS;
	const int nkb = (kall + 255) / 256;
	const int rt = (int)(local / nkb), kb = (int)(local % nkb);
	const T *X = reinterpret_cast<const T *>(w.ptr);
	const int32_t *rowt = tabs + w.rowtab, *colt = tabs + w.coltab;
	const int k0 = kb * 256, k1 = min(kall, k0 + 256);
	int bad = 0;

	if (w.kcontig && !w.cplx) {
		/* K one contiguous run per row: a warp walks it directly (no
		 * offset table), four loads in flight per lane; the padding past
		 * w.k is zero and needs no reading */
		const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
		const T *base = X + rowt[0];
		const int kend = min(k1, w.k);
		for (int rr = warp; rr < EMU_TM; rr += 8) {
			int r = rt * EMU_TM + rr;
			if (r >= w.mn)
				break;
			const T *xr = base + colt[r];
			int e = 0;
#pragma unroll 4
			for (int k = k0 + lane; k < kend; k += 32) {
				int b = fin<T>::bexp(xr[k]);
				bad |= b == fin<T>::EMAX;
				e = max(e, b);
			}
			for (int off = 16; off > 0; off >>= 1)
				e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
			if (lane == 0 && e > 0)
				atomicMax(&E[w.exptab + r], e);
		}
	} else if (w.kfast) {
		/* K unit-stride: a warp walks K for one row at a time */
		const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
		for (int rr = warp; rr < EMU_TM; rr += 8) {
			int r = rt * EMU_TM + rr;
			if (r >= w.mn)
				break;
			int32_t co = colt[r];
			int e = 0;
			for (int k = k0 + lane; k < k1; k += 32) {
				int b = fin<T>::bexp(fetch(X, rowt, co, w, k));
				bad |= b == fin<T>::EMAX;
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
			int32_t co = colt[r];
			int e = 0;
			for (int k = k0 + half; k < k1; k += 2) {
				int b = fin<T>::bexp(fetch(X, rowt, co, w, k));
				bad |= b == fin<T>::EMAX;
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

/* bf16 bits of d * w, exact for |d| <= 256 and w a power of two */
__device__ __forceinline__ uint32_t digit_bf16(int d, float w)
{
	/* exact int -> float for |d| < 2^22 without a conversion unit */
	float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
	return __float_as_uint(f * w) >> 16;
}

/* CTA = (view, 128-row tile, group of 4 K steps); thread = (row, K octet) */
template <typename T>
__global__ void __launch_bounds__(256, 6)
emu_split_kernel(const xmgd_view_t *__restrict__ views,
    const view_meta *__restrict__ meta, int nviews,
    const int32_t *__restrict__ tabs, const int32_t *__restrict__ E)
{
	constexpr int S = fin<T>::S;
	constexpr int CHUNK_ELEMS = S * SLICE_BYTES / 2;
	const int v = find_view(meta, nviews, blockIdx.x);
	const xmgd_view_t w = views[v];
	const int64_t local = blockIdx.x - meta[v].first_cta;
	const int ngrp = (w.n_ks + 3) / 4;
	const int rt = (int)(local / ngrp), g = (int)(local % ngrp);
	const int rr = threadIdx.x % EMU_TM, oct = threadIdx.x / EMU_TM;
	const int r = rt * EMU_TM + rr;
	const T *X = reinterpret_cast<const T *>(w.ptr);
	const int32_t *rowt = tabs + w.rowtab, *colt = tabs + w.coltab;
	const bool live = r < w.mn;
	const int32_t co = live ? colt[r] : 0;
	const int er = live ? E[w.exptab + r] : 0;
	uint16_t *out = reinterpret_cast<uint16_t *>(w.slices);
	/* a contiguous K run: direct loads, no offset table */
	const bool direct = w.kcontig && !w.cplx;
	const T *Xr = X + co + (direct ? rowt[0] : 0);

	for (int ks = g * 4; ks < min(w.n_ks, g * 4 + 4); ks++) {
		uint32_t bits[S][4];
#pragma unroll
		for (int t = 0; t < S; t++)
#pragma unroll
			for (int q = 0; q < 4; q++)
				bits[t][q] = 0;
#pragma unroll
		for (int e = 0; e < 8; e++) {
			const int k = ks * EMU_KS + oct * 8 + e;
			T x = !live ? T(0) : direct ? (k < w.k ? Xr[k] : T(0)) :
			    fetch(X, rowt, co, w, k);
			long long m;
			int eb;
			bool neg;
			fin<T>::parts(x, m, eb, neg);
			/* X = round(m * 2^(eb - er - (MANT + 1 - T1))), |X| <= 2^T1 */
			const int sh = er - eb + (fin<T>::MANT + 1 - fin<T>::T1);
			long long xi = sh >= 63 ? 0 : ((m + (1ll << (sh - 1))) >> sh);
			if (neg)
				xi = -xi;
			int d[S];
#pragma unroll
			for (int t = S - 1; t >= 1; t--) {
				d[t] = (int)(((xi + 128) & 255) - 128);
				xi = (xi - d[t]) >> 8;
			}
			d[0] = (int)xi;
#pragma unroll
			for (int t = 0; t < S; t++) {
				uint32_t h = digit_bf16(d[t], __int_as_float((127 - 8 * t) << 23));
				bits[t][e >> 1] |= h << (16 * (e & 1));
			}
		}
		/* chunk layout [8-row group][slice][2 K core matrices][8 rows x
		 * 16 B]: the first R rows of a tile are a contiguous prefix, and
		 * one slice is K-major with SBO = S * 256 B between row groups */
		const size_t chunk = ((size_t)rt * w.n_ks + ks) * CHUNK_ELEMS;
		const size_t within = (size_t)(rr >> 3) * (S * 128) + oct * 64 + (rr & 7) * 8;
#pragma unroll
		for (int t = 0; t < S; t++) {
			uint4 val = make_uint4(bits[t][0], bits[t][1], bits[t][2], bits[t][3]);
			*reinterpret_cast<uint4 *>(out + chunk + t * 128 + within) = val;
		}
	}
}

/* ------------------------------------------------------------------ */
/* 3. grouped tcgen05 GEMM with exact drains and the fused fold        */

/* V * 2^e (sign flipped by sx) as a double, assembled in integer
 * arithmetic: |V| rounded once to 53 bits (to nearest, ties to even), the
 * exponent field written directly.  Bit-identical to ldexp((double)V, e)
 * whenever the result is a normal number; false otherwise (the caller
 * takes the FP64 path).  GB300's FP64 pipe is ~1/64 of its FP32 rate, so
 * the epilogue keeps the conversion and the scaling off it. */
__device__ __forceinline__ bool pack_f64(long long V, int e, unsigned long long sx,
    double &out)
{
	if (V == 0) {
		out = __longlong_as_double((long long)sx);
		return true;
	}
	const unsigned long long sg = (V < 0 ? 1ull << 63 : 0ull) ^ sx;
	const unsigned long long a = V < 0 ? 0ull - (unsigned long long)V :
	    (unsigned long long)V;
	int msb = 63 - __clzll((long long)a);
	const int sh = msb - 52;
	unsigned long long m;
	if (sh > 0) {
		const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
		m = a >> sh;
		m += (rem > half) || (rem == half && (m & 1));
		if (m >> 53) {
			m >>= 1;
			msb++;
		}
	} else
		m = a << -sh;
	const int be = msb + e + 1023;
	if (be < 1 || be > 2046)
		return false;
	out = __longlong_as_double((long long)(sg | ((unsigned long long)be << 52) |
	    (m & 0xFFFFFFFFFFFFFull)));
	return true;
}

/* A pipeline stage holds KSTEPS consecutive 16-wide K steps (each the
 * M-side chunk then the N-side chunk).  The per-stage synchronisation of
 * the producer and MMA threads (barrier round trips, copy issue, commit)
 * weighs on the stage's MMAs, so both forms take several steps per stage.
 * The 3-slice form (6 MMAs per K step) three, in three stages of 72 KiB
 * (measured on the float32 ring term's GEMM: one step per stage 30.3-32.3
 * ms, two 27.8, three 27.0, four in two stages 26.5 with a one-stage head,
 * 32.6 with two); the 6-slice form (21 MMAs per step) two, in two stages
 * of 96 KiB (FP64 ring term 59.6 -> 56.5 ms, cfg2 ladder 32.4-32.9 ->
 * 32.0 ms, with a head and tail of both stages). */
template <int S>
struct stage_cfg {
#ifndef EMU_KSTEPS32
#define EMU_KSTEPS32 3
#endif
#ifndef EMU_BUDGET32
#define EMU_BUDGET32 221184                   /* 3 stages of 72 KiB */
#endif
#ifndef EMU_KSTEPS64
#define EMU_KSTEPS64 2                        /* 2 stages of 96 KiB */
#endif
	static constexpr int KSTEPS = S == fin<float>::S ? EMU_KSTEPS32 : EMU_KSTEPS64;
	static constexpr int BUDGET = S == fin<float>::S ? EMU_BUDGET32 : STAGE_BUDGET;
	static constexpr int CHUNK_BYTES = S * SLICE_BYTES;
	static constexpr int STEP_BYTES = 2 * CHUNK_BYTES;
	static constexpr int STAGE_BYTES = KSTEPS * STEP_BYTES;
	static constexpr int NST = BUDGET / STAGE_BYTES > 8 ? 8 :
	    BUDGET / STAGE_BYTES;
	static constexpr int SMEM = NST * STAGE_BYTES + 1024;
};

/* the end of the K segment holding step k: the pair, or the re/im half
 * of a realified complex view */
__device__ __forceinline__ int segment_end(int k, int nks, int cplx)
{
	return (cplx && k < nks / 2) ? nks / 2 : nks;
}

/* the stage that starts at step k holds steps [k, super_end): KSTEPS of
 * them, never past the segment's end */
template <int S>
__device__ __forceinline__ int super_end(int k, int nks, int cplx)
{
	return min(segment_end(k, nks, cplx), k + stage_cfg<S>::KSTEPS);
}

/* stages per pair: each segment in stages of KSTEPS steps */
template <int S>
__device__ __forceinline__ int stages_of(int nks, int cplx)
{
	constexpr int KS = stage_cfg<S>::KSTEPS;
	if (!cplx)
		return (nks + KS - 1) / KS;
	const int nh = nks / 2;
	return (nh + KS - 1) / KS + (nks - nh + KS - 1) / KS;
}

/* K steps [c0, c1) of the next chunk: chunks never straddle the re/im
 * boundary of a realified complex view.  An exact group g accumulates at
 * most 3 products of |d_p d_q| <= 2^14 per K element, so its integer sum
 * stays below 2^24 (exact in fp32) for chunks of up to 341 elements.
 * FP64 takes 256 (XMG_EMU_CHUNK steps, at most 20): its rounded low
 * band's error grows with the chunk (cfg2 ladder: 3.1e-13 at 160, 4.4e-13
 * at 224, 6.2e-13 at 320, against GEMM times of 35.8, 34.2 and 33.2 ms);
 * FP32, all exact, takes up to 20 steps, the steps left split into equal
 * chunks rounded up to whole stages (at most 21 steps, 336 elements; 32
 * steps: 18 + 14), so that the stages of a segment, which start at its
 * first step, never straddle a chunk boundary. */
template <int S>
__device__ __forceinline__ int chunk_end(int c0, int nks, int cplx, int kchunk)
{
	const int lim = segment_end(c0, nks, cplx);
	if constexpr (S == fin<float>::S) {
		constexpr int KS = stage_cfg<S>::KSTEPS;
		const int left = lim - c0;
		const int n = (left + EMU_CHUNK32 - 1) / EMU_CHUNK32;
		const int len = ((left + n - 1) / n + KS - 1) / KS * KS;
		return min(lim, c0 + len);
	}
	return min(lim, c0 + kchunk);
}

/* Accumulators: 0, 1, 2 hold the exact weight groups p + q = 0, 1, 2; 3
 * the low band p + q = 3..KEEP.  The top one (3 with a low band, else 2)
 * forms set X, the others set Y.  The drain reads X first and releases it,
 * so at a chunk boundary the MMA warp issues the X products of the next
 * chunk's first (already staged) K steps while the drain still reads Y. */
template <int KEEP>
struct acc_sets {
	static constexpr int XACC = KEEP > 2 ? 3 : 2;
};

/* the slice products of one K step whose accumulator lies in `which`
 * (1: set X, 2: set Y, 3: both).  The two stage descriptors are built once;
 * each product adds its slice offset (>> 4) to the low word, which cannot
 * carry out of the 14-bit address field inside a < 256 KiB stage area. */
template <int S, int KEEP, bool PAIR>
__device__ __forceinline__ void
issue_step(uint32_t tmem, uint32_t base, uint32_t a_off, uint32_t idesc,
    int which, uint32_t &started)
{
	const uint64_t da = sdesc(base, S * 256), db = sdesc(base + a_off, S * 256);
	const uint32_t alo = (uint32_t)da, ahi = (uint32_t)(da >> 32);
	const uint32_t blo = (uint32_t)db, bhi = (uint32_t)(db >> 32);
#pragma unroll
	for (int pa = 0; pa < S; pa++)
#pragma unroll
		for (int qb = 0; qb < S; qb++) {
			if (pa + qb > KEEP)
				continue;
			const int acc = min(pa + qb, 3);
			if (!(which & (acc == acc_sets<KEEP>::XACC ? 1 : 2)))
				continue;
			if constexpr (PAIR)
				mma_bf16_pair(tmem + acc * 128, alo + qb * 16, ahi, blo + pa * 16,
				    bhi, idesc, (started >> acc) & 1u);
			else
				mma_bf16_split(tmem + acc * 128, alo + qb * 16, ahi, blo + pa * 16,
				    bhi, idesc, (started >> acc) & 1u);
			started |= 1u << acc;
		}
}

/* PAIR: a cluster of two CTAs runs each 256-row tile with cta_group::2
 * MMAs issued by rank 0: each CTA stages its own 128 M-side rows and half
 * of the N side, rank 1 forwards its stage completions to rank 0, the
 * drains of both CTAs read their own TMEM and release it to rank 0. */
template <int S, int KEEP, bool LOW, typename TOUT, int DW, bool PAIR>
__global__ void __launch_bounds__(64 + 32 * DW, 1)
emu_gemm_kernel(const emu_item *__restrict__ items, int nitems,
    const emu_member *__restrict__ members,
    const xmgd_cblock_t *__restrict__ cbs, const xmgd_pair_t *__restrict__ prs,
    const xmgd_view_t *__restrict__ va, const xmgd_view_t *__restrict__ vb,
    const int32_t *__restrict__ tabs, const int32_t *__restrict__ EA,
    const int32_t *__restrict__ EB, const int32_t *__restrict__ cbF,
    double alpha, double beta, int expoff2, int cplx, int hmax, int pfd, int kchunk,
    int *__restrict__ flags)
{
	using C = stage_cfg<S>;
	constexpr int NST = C::NST;
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	uint8_t *stages = reinterpret_cast<uint8_t *>(
	    (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
	__shared__ __align__(8) uint64_t bar_full[NST], bar_empty[NST];
	__shared__ __align__(8) uint64_t bar_xfull, bar_yfull, bar_xempty, bar_yempty, bar_fin;
	__shared__ __align__(8) uint64_t bar_ifull[2], bar_iempty[2];
	__shared__ __align__(8) uint64_t bar_pfull[PAIR ? NST : 1];
	__shared__ int s_item[2];
	__shared__ uint32_t s_tmem;
	__shared__ volatile int s_err;
	int *g_err = flags + 1, *g_next = flags + 2;

	/* operands with Inf/NaN (flag set by the exponent kernel): write
	 * nothing, the host recomputes these blocks on the FP64 path */
	if (*(volatile int *)flags & 1)
		return;
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const uint32_t rank = PAIR ? cluster_rank() : 0;
	/* bounded waits; in a pair, with cluster-scope acquire */
	auto wait = [&](uint32_t bar, uint32_t parity, int code) -> bool {
		if constexpr (PAIR)
			return mbar_wait_cl(bar, parity, &s_err, g_err, code);
		else
			return mbar_wait(bar, parity, &s_err, g_err, code);
	};
	/* arrive on a barrier of rank 0 (locally there, remotely from rank 1) */
	auto arrive0 = [&](uint64_t *bar) {
		if (!PAIR || rank == 0)
			mbar_arrive(smem_u32(bar));
		else
			mbar_arrive_remote(map_shared(smem_u32(bar), 0));
	};
	auto commit = [&](uint64_t *bar) {
		if constexpr (PAIR)
			mma_commit_pair(smem_u32(bar));
		else
			mma_commit(smem_u32(bar));
	};

	if (threadIdx.x == 0) {
		for (int s = 0; s < NST; s++) {
			mbar_init(smem_u32(&bar_full[s]), 1);
			mbar_init(smem_u32(&bar_empty[s]), 1);
		}
		mbar_init(smem_u32(&bar_xfull), 1);
		mbar_init(smem_u32(&bar_yfull), 1);
		mbar_init(smem_u32(&bar_xempty), PAIR ? 2 * DW : DW);
		mbar_init(smem_u32(&bar_yempty), PAIR ? 2 * DW : DW);
		mbar_init(smem_u32(&bar_fin), 1);
		for (int q = 0; q < 2; q++) {
			mbar_init(smem_u32(&bar_ifull[q]), 1);
			/* pair: both CTAs' drains, rank 0's MMA warp, rank 1's
			 * producer and forwarder */
			mbar_init(smem_u32(&bar_iempty[q]), PAIR ? 2 * DW + 3 : 1 + DW);
		}
		if (PAIR)
			for (int q = 0; q < NST; q++)
				mbar_init(smem_u32(&bar_pfull[q]), 1);
		s_err = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	if (warp == 1) {
		if constexpr (PAIR) {
			asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;"
			    :: "r"(smem_u32(&s_tmem)));
			asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
		} else {
			asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;"
			    :: "r"(smem_u32(&s_tmem)));
			asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
		}
	}
	tc_fence_before();
	__syncthreads();
	if constexpr (PAIR)
		cluster_sync();	/* peers' barriers exist before any remote arrive */
	tc_fence_after();
	const uint32_t tmem = s_tmem;

	/* persistent: the producer takes the next item of the cost-sorted list
	 * from a global counter and passes its index to the MMA and drain
	 * warps through a two-slot ring (-1 ends); the stage ring and the
	 * accumulator phases carry across items */
	if (warp == 0) {
		/* ---------------- producer ---------------- */
		if (lane == 0) {
			int s = 0;
			uint32_t ph = 0;
			int lastp[NST];
#pragma unroll
			for (int q = 0; q < NST; q++)
				lastp[q] = -1;
			uint32_t iph = 0;
			for (int slot = 0; !s_err; ) {
				int t;
				if (!PAIR || rank == 0) {
					/* fetch the next item and hand it to every role */
					if (!wait(smem_u32(&bar_iempty[slot]), iph ^ 1, 5))
						break;
					t = atomicAdd(g_next, 1);
					t = t < nitems ? t : -1;
					s_item[slot] = t;
					if (PAIR) {
						st_remote_u32(map_shared(smem_u32(&s_item[slot]), 1), (uint32_t)t);
						mbar_arrive_remote(map_shared(smem_u32(&bar_ifull[slot]), 1));
					}
					mbar_arrive(smem_u32(&bar_ifull[slot]));
				} else {
					if (!wait(smem_u32(&bar_ifull[slot]), iph, 5))
						break;
					t = s_item[slot];
					arrive0(&bar_iempty[slot]);
				}
				if (++slot == 2) { slot = 0; iph ^= 1; }
				if (t < 0)
					break;
				const emu_item it = items[t];
				const int nmem = it.mcount;
				const xmgd_cblock_t cb = cbs[members[it.mfirst].cblock];
				const int pass = it.pr & 1, swp = (it.pr >> 1) & 1;
				const int mstk = (it.pr >> 2) & 1;
				/* the shared side: the M side's 128 rows (this CTA's half
				 * of 256 in a pair) or, M-stacked, the N side's live rows;
				 * the members: their live rows at their first column or
				 * lane (a pair: one member, this CTA's half of its rows) */
				const uint32_t ntot = (uint32_t)(it.pr >> 8) * S * 32 / (PAIR ? 2 : 1);
				const uint32_t noff = PAIR ? rank * ntot : 0;
				const uint32_t shb = mstk ? ntot : C::CHUNK_BYTES;
				int mfp[EMU_MAXMEM], mrt[EMU_MAXMEM];
				uint32_t mby[EMU_MAXMEM], mdo[EMU_MAXMEM], stb = 0;
#pragma unroll
				for (int j = 0; j < EMU_MAXMEM; j++) {
					const emu_member mb = members[it.mfirst + (j < nmem ? j : 0)];
					mfp[j] = cbs[mb.cblock].first_pair;
					mrt[j] = mb.n0 / EMU_TM;
					mby[j] = PAIR ? ntot : (uint32_t)mb.rows * S * 32;
					mdo[j] = (mstk ? 0u : C::CHUNK_BYTES) + (uint32_t)mb.off * S * 32;
					stb += j < nmem ? mby[j] : 0;
				}
				/* shared side from a's views when it is a's side */
				const bool sha = (mstk ^ swp) != 0;
				/* a pair's operand chunks: the shared side's tile (live
				 * or past the view) and each member's */
				struct pair_src {
					const uint8_t *gs, *gn[EMU_MAXMEM];
					int nks;
					bool slive;
				};
				auto load_pair = [&](int p, pair_src &o) {
					/* the members' pair lists run in step: pair p of
					 * every member has member 0's view and K on the
					 * shared side */
					const xmgd_pair_t pr = prs[cb.first_pair + p];
					const xmgd_view_t ws = sha ? va[pr.aview] : vb[pr.bview];
					o.nks = vb[pr.bview].n_ks;
					const int stile = it.m0 / EMU_TM + (mstk ? 0 : (int)rank);
					o.slive = stile < ws.n_rt;
					o.gs = reinterpret_cast<const uint8_t *>(ws.slices) +
					    (size_t)stile * o.nks * C::CHUNK_BYTES;
#pragma unroll
					for (int j = 0; j < EMU_MAXMEM; j++) {
						const xmgd_pair_t pj = prs[mfp[j] + p];
						o.gn[j] = reinterpret_cast<const uint8_t *>(sha ?
						    vb[pj.bview].slices : va[pj.aview].slices) +
						    (size_t)mrt[j] * o.nks * C::CHUNK_BYTES + noff;
					}
				};
				/* K step ks of a pair: the shared side reads at its own
				 * K index (the M side's or the N side's), the members at
				 * the other; the imaginary pass swaps B's re/im halves */
				auto kidx = [&](int ks, int nks, int &ksh, int &kst) {
					const int nh = nks / 2;
					const int kb = (cplx && pass) ? (ks < nh ? ks + nh : ks - nh) : ks;
					const int km = swp ? ks : kb, kn = swp ? kb : ks;
					ksh = mstk ? kn : km;
					kst = mstk ? km : kn;
				};
				/* L2 prefetch cursor, pfd steps ahead of the copies within
				 * the item (XMG_EMU_PF; off by default: measured slower,
				 * the ring's copies are not waiting on DRAM misses) */
				pair_src pf;
				int pfp = 0, pfk = 0;
				if (pfd > 0)
					load_pair(0, pf);
				auto pf_step = [&]() {
					if (pfd <= 0 || pfp >= cb.npairs)
						return;
					int ksh, kst;
					kidx(pfk, pf.nks, ksh, kst);
					if (pf.slive)
						bulk_prefetch_l2(pf.gs + (size_t)ksh * C::CHUNK_BYTES, shb);
#pragma unroll
					for (int j = 0; j < EMU_MAXMEM; j++)
						if (j < nmem)
							bulk_prefetch_l2(pf.gn[j] + (size_t)kst * C::CHUNK_BYTES,
							    mby[j]);
					if (++pfk == pf.nks) {
						pfk = 0;
						if (++pfp < cb.npairs)
							load_pair(pfp, pf);
					}
				};
				for (int q = 0; q < pfd; q++)
					pf_step();
				pair_src cur;
				for (int p = 0; p < cb.npairs && !s_err; p++) {
					load_pair(p, cur);
					for (int ks = 0; ks < cur.nks; ) {
						if (!wait(smem_u32(&bar_empty[s]), ph ^ 1, 1))
							break;
						const int ke = super_end<S>(ks, cur.nks, cplx);
						uint32_t dst = smem_u32(stages + (size_t)s * C::STAGE_BYTES);
						uint32_t fb = smem_u32(&bar_full[s]);
						/* a pair's second M tile may lie past the view: its
						 * rows are then never stored */
						mbar_expect_tx(fb, (uint32_t)(ke - ks) *
						    ((cur.slive ? shb : 0) + stb));
						for (int k = ks; k < ke; k++, dst += C::STEP_BYTES) {
							int ksh, kst;
							kidx(k, cur.nks, ksh, kst);
							if (cur.slive)
								bulk_g2s(dst + (mstk ? C::CHUNK_BYTES : 0u),
								    cur.gs + (size_t)ksh * C::CHUNK_BYTES, shb, fb);
#pragma unroll
							for (int j = 0; j < EMU_MAXMEM; j++)
								if (j < nmem)
									bulk_g2s(dst + mdo[j],
									    cur.gn[j] + (size_t)kst * C::CHUNK_BYTES,
									    mby[j], fb);
							pf_step();
						}
#pragma unroll
						for (int q = 0; q < NST; q++)
							if (q == s)
								lastp[q] = (int)ph;
						if (++s == NST) { s = 0; ph ^= 1; }
						ks = ke;
					}
				}
			}
			/* on failure, let this CTA's copies still in flight land
			 * before it exits (bounded): the last phase issued on each
			 * stage completes when its bytes have arrived */
			if (s_err) {
				uint64_t t0 = gtimer();
#pragma unroll
				for (int q = 0; q < NST; q++)
					if (lastp[q] >= 0)
						while (!mbar_try(smem_u32(&bar_full[q]), (uint32_t)lastp[q]) &&
						    gtimer() - t0 < WAIT_NS)
							;
			}
		}
	} else if (warp == 1 && PAIR && rank == 1) {
		/* ---------- rank 1: forward stage completions to rank 0 ---------- */
		if (lane == 0) {
			int s = 0;
			uint32_t ph = 0, iph = 0;
			for (int slot = 0; !s_err; ) {
				if (!wait(smem_u32(&bar_ifull[slot]), iph, 6))
					break;
				const int t = s_item[slot];
				arrive0(&bar_iempty[slot]);
				if (++slot == 2) { slot = 0; iph ^= 1; }
				if (t < 0)
					break;
				const xmgd_cblock_t cb = cbs[members[items[t].mfirst].cblock];
				for (int p = 0; p < cb.npairs && !s_err; p++) {
					const int nst_p = stages_of<S>(vb[prs[cb.first_pair + p].bview].n_ks, cplx);
					for (int q = 0; q < nst_p; q++) {
						if (!wait(smem_u32(&bar_full[s]), ph, 3))
							break;
						mbar_arrive_remote(map_shared(smem_u32(&bar_pfull[s]), 0));
						if (++s == NST) { s = 0; ph ^= 1; }
					}
				}
			}
			/* rank 0's last MMAs (they write this CTA's TMEM) are done
			 * once the final commit lands here */
			uint64_t t0 = gtimer();
			while (!mbar_try_cl(smem_u32(&bar_fin), 0) && gtimer() - t0 < WAIT_NS)
				;
		}
	} else if (warp == 1) {
		/* ---------------- MMA issuer ---------------- */
		if (lane == 0) {
			int s = 0;
			bool first = true;
			uint32_t ph = 0, xph = 0, yph = 0;
			uint32_t iph = 0;
			/* a stage is ready once this CTA's copies (and, in a pair,
			 * the peer's, forwarded) have landed */
			auto ready = [&](int st_, uint32_t par) -> bool {
				if (!wait(smem_u32(&bar_full[st_]), par, 3))
					return false;
				if (PAIR && !wait(smem_u32(&bar_pfull[st_]), par, 10))
					return false;
				return true;
			};
			for (int slot = 0; !s_err; ) {
				if (!wait(smem_u32(&bar_ifull[slot]), iph, 6))
					break;
				const int t = s_item[slot];
				mbar_arrive(smem_u32(&bar_iempty[slot]));
				if (++slot == 2) { slot = 0; iph ^= 1; }
				if (t < 0)
					break;
				const emu_item it = items[t];
				const xmgd_cblock_t cb = cbs[members[it.mfirst].cblock];
				const uint32_t idesc = PAIR ? idesc_pair_n(it.pr >> 8) : idesc_n(it.pr >> 8);
				for (int p = 0; p < cb.npairs && !s_err; p++) {
					const xmgd_pair_t pr = prs[cb.first_pair + p];
					const int nks = vb[pr.bview].n_ks;
					for (int c0 = 0; c0 < nks && !s_err; ) {
						const int c1 = chunk_end<S>(c0, nks, cplx, kchunk);
						/* the chunk's stages: KSTEPS steps each, the last
						 * one shorter at a segment's end */
						constexpr int KS = C::KSTEPS;
						const int nss = (c1 - c0 + KS - 1) / KS;
						/* every accumulator restarts each chunk: the exact
						 * groups for their 2^24 bound, the low band because
						 * the tensor core's fp32 accumulation error grows
						 * with the accumulation length (per-pair
						 * accumulation measured 10x larger error) */
						uint32_t started = 0;
						bool okc = true;
						auto issue_stage = [&](int sj, int j, int which) {
							const uint32_t base = smem_u32(stages + (size_t)sj * C::STAGE_BYTES);
							const int nk = min(KS, c1 - c0 - j * KS);
							for (int u = 0; u < nk; u++)
								issue_step<S, KEEP, PAIR>(tmem, base + u * C::STEP_BYTES,
								    C::CHUNK_BYTES, idesc, which, started);
						};
						/* head: the first H (staged) stages; tail: the last T
						 * stages; middle: the rest.  H, T <= hmax <= NST: the
						 * stages a head or tail holds are released only after
						 * its set-Y products, so hmax < NST leaves stages for
						 * the producer to prefetch the steps after them */
						const int H = min(hmax, nss);
						const int T = min(hmax, nss - H);
						/* head, set X, as soon as the drain has read X of
						 * the previous chunk */
						if (!first) {
							if (!wait(smem_u32(&bar_xempty), xph, 2))
								break;
							xph ^= 1;
						}
						tc_fence_after();
						for (int j = 0; j < H; j++) {
							const int sj = s + j < NST ? s + j : s + j - NST;
							const uint32_t pj = s + j < NST ? ph : ph ^ 1;
							if (!ready(sj, pj)) {
								okc = false;
								break;
							}
							tc_fence_after();
							issue_stage(sj, j, 1);
						}
						if (!okc)
							break;
						if (T == 0)
							commit(&bar_xfull);
						/* head, set Y, once Y is read too */
						if (!first) {
							if (!wait(smem_u32(&bar_yempty), yph, 8))
								break;
							yph ^= 1;
						}
						first = false;
						tc_fence_after();
						for (int j = 0; j < H; j++) {
							const int sj = s + j < NST ? s + j : s + j - NST;
							issue_stage(sj, j, 2);
							commit(&bar_empty[sj]);
						}
						s += H;
						if (s >= NST) { s -= NST; ph ^= 1; }
						/* middle: every product per stage */
						for (int j = H; j < nss - T; j++) {
							if (!ready(s, ph)) {
								okc = false;
								break;
							}
							tc_fence_after();
							issue_stage(s, j, 3);
							commit(&bar_empty[s]);
							if (++s == NST) { s = 0; ph ^= 1; }
						}
						if (!okc)
							break;
						/* tail: set X of the last T stages, then X is
						 * complete and its drain can start while the
						 * tensor core still works on set Y */
						for (int j = 0; j < T; j++) {
							const int sj = s + j < NST ? s + j : s + j - NST;
							const uint32_t pj = s + j < NST ? ph : ph ^ 1;
							if (!ready(sj, pj)) {
								okc = false;
								break;
							}
							tc_fence_after();
							issue_stage(sj, nss - T + j, 1);
						}
						if (!okc)
							break;
						if (T > 0) {
							commit(&bar_xfull);
							for (int j = 0; j < T; j++) {
								const int sj = s + j < NST ? s + j : s + j - NST;
								issue_stage(sj, nss - T + j, 2);
								commit(&bar_empty[sj]);
							}
							s += T;
							if (s >= NST) { s -= NST; ph ^= 1; }
						}
						commit(&bar_yfull);
						c0 = c1;
					}
				}
			}
			/* every MMA issued by this CTA has completed once bar_fin
			 * fires; TMEM is released only after that */
			commit(&bar_fin);
			uint64_t t0 = gtimer();
			while (!(PAIR ? mbar_try_cl(smem_u32(&bar_fin), 0) :
			    mbar_try(smem_u32(&bar_fin), 0)) && gtimer() - t0 < WAIT_NS)
				;
		}
	} else {
		/* ------------- drain + epilogue (warps 2 .. DW+1) -------------
		 * warp w reads TMEM lanes 32 * (w % 4) .. +31 (the tcgen05.ld
		 * lane-quadrant rule) and owns NC of the 128 columns */
		constexpr int NC = 128 / (DW / 4);
		constexpr int NSEG = NC / 16;
		const int quad = warp & 3, half = (warp - 2) >> 2;
		const uint32_t trow = tmem + ((uint32_t)(quad * 32) << 16) + half * NC;
		uint32_t fph = 0;
		bool ok = true;
		uint32_t iph = 0;
		for (int slot = 0; ok; ) {
			int t = -1;
			if (lane == 0) {
				if (wait(smem_u32(&bar_ifull[slot]), iph, 7)) {
					t = s_item[slot];
					arrive0(&bar_iempty[slot]);
				} else
					t = -2;
			}
			t = __shfl_sync(0xffffffffu, t, 0);
			if (++slot == 2) { slot = 0; iph ^= 1; }
			if (t < 0)
				break;
			const emu_item it = items[t];
			const int pass = it.pr & 1, swp = (it.pr >> 1) & 1, rows = it.pr >> 8;
			const int mstk = (it.pr >> 2) & 1;
			/* this warp's NC columns fall into NC / 16 segments of 16, each
			 * inside one member's output block (N-stacked members hold
			 * multiples of 16 columns; M-stacked ones multiples of 32
			 * lanes, so one member holds all of this warp's lanes): per
			 * segment the output block, its first pair, its F and the
			 * N-side row of the segment's first column; and the M-side
			 * row of this warp's first lane */
			int scb[NSEG], sfp[NSEG], sF[NSEG], sq0[NSEG], mrow0;
			if (mstk) {
				const int row0 = quad * 32;
				int j = 0;
				for (int jj = 1; jj < it.mcount; jj++)
					j += row0 >= members[it.mfirst + jj].off;
				const emu_member mb = members[it.mfirst + j];
#pragma unroll
				for (int g = 0; g < NSEG; g++) {
					scb[g] = mb.cblock;
					sfp[g] = cbs[mb.cblock].first_pair;
					sF[g] = cbF[mb.cblock];
					sq0[g] = it.m0 + half * NC + g * 16;
				}
				mrow0 = mb.n0 + row0 - mb.off;
			} else {
#pragma unroll
				for (int g = 0; g < NSEG; g++) {
					const int col = half * NC + g * 16;
					int j = 0;
					for (int jj = 1; jj < it.mcount; jj++)
						j += col >= members[it.mfirst + jj].off;
					const emu_member mb = members[it.mfirst + j];
					scb[g] = mb.cblock;
					sfp[g] = cbs[mb.cblock].first_pair;
					sF[g] = cbF[mb.cblock];
					sq0[g] = mb.n0 + col - mb.off;
				}
				mrow0 = it.m0 + (int)rank * EMU_TM + quad * 32;
			}
			const int npairs = cbs[scb[0]].npairs;
			long long V[NC];
#pragma unroll
			for (int c = 0; c < NC; c++)
				V[c] = 0;
			for (int p = 0; p < npairs && ok; p++) {
				const int nks = vb[prs[sfp[0] + p].bview].n_ks;
				int esg[NSEG], esh[NSEG];
#pragma unroll
				for (int g = 0; g < NSEG; g++) {
					const xmgd_pair_t pg = prs[sfp[g] + p];
					esg[g] = pg.esign;
					esh[g] = pg.eshift;
				}
				for (int c0 = 0; c0 < nks; ) {
					const int c1 = chunk_end<S>(c0, nks, cplx, kchunk);
					/* each segment's pair factor sign * 2^shift (shift 0
					 * or 1, checked by the planner) rides on the exact
					 * fp32 -> int scales; the real pass negates the im * im
					 * half */
					const bool negh = cplx && !pass && c0 >= nks / 2;
					float s0[NSEG];
#pragma unroll
					for (int g = 0; g < NSEG; g++)
						s0[g] = ((esg[g] > 0) != negh ? 1.0f : -1.0f) *
						    __int_as_float((127 + esh[g]) << 23);
					/* one lane waits, the warp follows its verdict, so the
					 * .sync.aligned TMEM loads below stay convergent */
					int w = 1;
					if (lane == 0)
						w = wait(smem_u32(&bar_xfull), fph, 4);
					w = __shfl_sync(0xffffffffu, w, 0);
					if (!w) {
						ok = false;
						break;
					}
					tc_fence_after();
					/* set X first: the low band (or, without one, group 2),
					 * then release it to the MMA warp */
					constexpr int XACC = acc_sets<KEEP>::XACC;
#pragma unroll
					for (int b4 = 0; b4 < NC / 4; b4++) {
						if (half * NC + b4 * 4 >= rows)
							break;	/* warp-uniform: columns past the tile */
						const int g = b4 / 4, F = sF[g];
						const float s2 = s0[g] * 65536.0f;
						const float s3 = s0[g] * __int_as_float((127 + 16 + F) << 23);
						float ax[4];
						tmem_ld4(trow + XACC * 128 + b4 * 4, ax);
						tmem_wait_ld();
#pragma unroll
						for (int c = 0; c < 4; c++) {
							if (LOW) {
								/* low band in units of 2^(-16-F), rounded
								 * to an integer with fp32 adds only (the
								 * conversion pipe runs at 1/8 of the FMA
								 * pipe's rate and bounded this drain):
								 * x = h * 2^22 + l, h = rint(x / 2^22) read
								 * from the bits of x / 2^22 + 1.5 * 2^23,
								 * l = x - h * 2^22 exact (|l| <= 2^21) and
								 * rounded the same way.  |x| < 2^42 (the
								 * band is below 2 units of the leading
								 * group per chunk, scaled by at most
								 * 2^(16 + 24 + 1)), inside the 2^44 the
								 * first add allows; the sum h * 2^22 +
								 * rint(l) equals rint(x), ties to even,
								 * as a direct conversion would give */
								const float M = 12582912.0f;	/* 1.5 * 2^23 */
								const float x = ax[c] * s3;
								const float t = fmaf(x, 2.384185791015625e-7f, M);
								const float l = fmaf(t - M, -4194304.0f, x);
								const int hi = __float_as_int(t) - 0x4B400000;
								const int lo = __float_as_int(l + M) - 0x4B400000;
								V[b4 * 4 + c] += ((long long)hi << 22) + lo;
							} else {
								V[b4 * 4 + c] += (long long)__float2int_rn(ax[c] * s2) << F;
							}
						}
					}
					tc_fence_before();
					__syncwarp();
					if (lane == 0)
						arrive0(&bar_xempty);
					/* set Y: the exact groups below X, once their last
					 * products have landed */
					w = 1;
					if (lane == 0)
						w = wait(smem_u32(&bar_yfull), fph, 9);
					w = __shfl_sync(0xffffffffu, w, 0);
					if (!w) {
						ok = false;
						break;
					}
					fph ^= 1;
					tc_fence_after();
#pragma unroll
					for (int b4 = 0; b4 < NC / 4; b4++) {
						if (half * NC + b4 * 4 >= rows)
							break;
						const int g = b4 / 4, F = sF[g];
						const float sa = s0[g], sb = sa * 256.0f, sc = sa * 65536.0f;
						float a0[4], a1[4], a2[4];
						tmem_ld4(trow + 0 * 128 + b4 * 4, a0);
						tmem_ld4(trow + 1 * 128 + b4 * 4, a1);
						if (LOW)
							tmem_ld4(trow + 2 * 128 + b4 * 4, a2);
						tmem_wait_ld();
#pragma unroll
						for (int c = 0; c < 4; c++) {
							/* exact integers: with the pair factor's 2^1,
							 * |i0| <= 2^14 * 336 * 2 < 2^23.4 and |i1| <
							 * 2^24.4; the packing is 64-bit */
							int i0 = __float2int_rn(a0[c] * sa);
							int i1 = __float2int_rn(a1[c] * sb);
							long long d = ((long long)i0 * 256 + i1) << 8;
							if (LOW)
								d += __float2int_rn(a2[c] * sc);
							V[b4 * 4 + c] += d << F;
						}
					}
					tc_fence_before();
					__syncwarp();
					if (lane == 0)
						arrive0(&bar_yempty);
					c0 = c1;
				}
			}
			if (!ok || s_err)
				break;
			/* epilogue (overlaps the next item's first chunk of MMAs):
			 * this thread's TMEM lane is one M-side row; its columns are
			 * N-side rows of the segments' output blocks.  Without swap
			 * the M side is b's free index (j), with swap a's (i). */
			const int ms = mrow0 + lane;
			const bool bz = beta == 0.0;
			const int cm = cplx ? 2 : 1;
			/* alpha a normal power of two folds into the exponent and
			 * sign; any other alpha costs one multiply */
			const long long ab = __double_as_longlong(alpha);
			const int aex = (int)((ab >> 52) & 0x7ff);
			const bool apow2 = (ab & 0xFFFFFFFFFFFFFll) == 0 && aex > 0 && aex < 0x7ff;
			const int esa = apow2 ? aex - 1023 : 0;
			const unsigned long long asx = apow2 ?
			    (unsigned long long)ab & (1ull << 63) : 0ull;
#pragma unroll
			for (int g = 0; g < NSEG; g++) {
				const xmgd_cblock_t cb = cbs[scb[g]];
				const int flim = swp ? cb.m : cb.n, vlim = swp ? cb.n : cb.m;
				if (ms >= flim)
					continue;
				TOUT *Cp = reinterpret_cast<TOUT *>(cb.c_ptr);
				const int32_t *vtab = tabs + (swp ? cb.ccol : cb.crow);
				const int32_t *vexp = swp ? EB + cb.eB : EA + cb.eA;
				const int32_t fo = tabs[(swp ? cb.crow : cb.ccol) + ms];
				const int fe = (swp ? EA + cb.eA : EB + cb.eB)[ms];
				const int F = sF[g];
#pragma unroll
				for (int c = 0; c < 16; c++) {
					const int q = sq0[g] + c;
					if (q < vlim && half * NC + g * 16 + c < rows) {
						const int e = vexp[q] + fe - expoff2 - 16 - F;
						double v;
						if (!pack_f64(V[g * 16 + c], e + esa, asx, v))
							v = alpha * ldexp((double)V[g * 16 + c], e);
						else if (!apow2)
							v *= alpha;
						TOUT *cp = Cp + (size_t)cm * (vtab[q] + fo) + pass;
						*cp = bz ? (TOUT)v : (TOUT)fma(beta, (double)*cp, v);
					}
				}
			}
		}
	}
	/* the producer, MMA and forwarder roles run on lane 0 alone: their
	 * warps reconverge first, because an aligned barrier counts a whole
	 * warp as arrived when any of its lanes arrives, and TMEM must stay
	 * allocated until the MMA lane has seen its last commit land */
	__syncwarp();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	if (warp == 1) {
		if constexpr (PAIR)
			asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;"
			    :: "r"(tmem));
		else
			asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;"
			    :: "r"(tmem));
	}
	/* neither CTA of a pair leaves while the other may still arrive on
	 * its barriers */
	if constexpr (PAIR)
		cluster_sync();
}

/* ------------------------------------------------------------------ */
/* host side: a reusable plan with an online tile-orientation autotuner  */

/*
 * Work-list policies.  The M side of a tile is always 128 rows (TMEM
 * lanes); the N side is the live rows rounded up to 16, so which operand
 * lies on the N side sets the padded work, and the order of the items
 * sets which tiles run together (L2 reuse: output blocks with the same
 * M-side free block read the same M-side operand rows).  Three policies,
 * each a complete work list:
 *   0  per block the orientation with less padded MMA work; blocks by
 *      decreasing cost, each block's tiles together;
 *   1  the same orientation; blocks grouped by their M-side free block and
 *      the group run M tile by M tile across its blocks;
 *   2  grouped as 1, orientation from a shared-memory model of one K step,
 *      max(N / 2, 32 + N / 4) cycles: the M-side operand (4 KiB) and the
 *      N-side operand (N * 32 B) are read from shared memory at 128 B per
 *      cycle while the tensor core needs N / 2 cycles.
 * (and 6, the stacked form below, which runs first).  The first runs of a
 * plan replay each distinct policy once, timed with events, then keep the
 * fastest; the choice is remembered per block-size histogram so later
 * plans of the same shape start tuned.
 */
enum { EMU_NPOLICY = 3 };

/* policy 6: policy 2's orientation and order, with the N-side tails of the
 * output blocks that share an M side (the same M-side view and K for every
 * pair index) stacked into common 128-column tiles: the MMAs of a K step
 * get wider, the shared-memory operand reads per flop fewer */
enum { EMU_POL_MERGED = 2 * EMU_NPOLICY };

static bool
pair_policy(int pol)
{
	return pol >= EMU_NPOLICY && pol < 2 * EMU_NPOLICY;
}

/* CTA pairs (256-row M tiles, cta_group::2): policies 3..5 repeat 0..2 in
 * that form; offered to the tuner when XMG_CTA_PAIR=1 */
static bool
pairs_enabled()
{
	const char *e = getenv("XMG_CTA_PAIR");
	return e && strcmp(e, "1") == 0;
}

static double
tile_cost(int mside, int nside, int policy, int mrows)
{
	double c = 0;
	const int mt = (mside + mrows - 1) / mrows;
	for (int n0 = 0; n0 < nside; n0 += EMU_TM) {
		const int w = std::min(EMU_TM, (nside - n0 + 15) / 16 * 16);
		c += policy == 2 ? std::max(w / 2.0, 32.0 + w / 4.0) : (double)w;
	}
	return c * mt;
}

static uint64_t
mix64(uint64_t h)
{
	h ^= h >> 33; h *= 0xff51afd7ed558ccdULL;
	h ^= h >> 33; h *= 0xc4ceb93fe53e6ccdULL;
	return h ^ (h >> 33);
}

struct tune_entry {
	uint64_t sig;
	int policy;
};
static std::vector<tune_entry> g_tuned;

struct emu_cand {
	int policy;
	uint64_t d_items, d_members;
	int nitems, grid;
	float ms;
};

struct emu_plan {
	int dtype, cplx;
	double alpha, beta;
	std::vector<xmgd_view_t> VA, VB;     /* slices: offsets in the workspace */
	std::vector<char> useA, useB;
	uint64_t d_va = 0, d_vb = 0, d_meta[2][2] = {{0, 0}, {0, 0}};
	int64_t nctas[2][2] = {{0, 0}, {0, 0}};
	uint64_t d_E = 0, d_F = 0;
	int64_t nE = 0;
	int32_t nexp_a = 0;
	size_t slice_bytes = 0;
	uint64_t ws = 0;                     /* workspace the views point into */
	const xmgd_cblock_t *d_cbs;
	const xmgd_pair_t *d_prs;
	const int32_t *d_tabs;
	std::vector<emu_cand> cand;
	int cur = 0, tuned = 0;
	int hmax = 4;                        /* head/tail steps (<= stages) */
	int pfd = 0;                         /* L2 prefetch distance, steps */
	int a_mode = 0;                      /* shared a side (xmgd_contract_t) */
	uint64_t a_slices = 0, a_E = 0, a_flag = 0;
	int kchunk = EMU_CHUNK;              /* FP64: K steps per chunk */
	uint64_t sig = 0;
	int *h_flags = nullptr;              /* pinned: Inf/NaN, timeout */
	int (*split)(emu_plan *) = nullptr;
	int (*gemm)(emu_plan *) = nullptr;
};

/* exponent tables, then unfold + split of every used view of both sides */
template <typename TIN>
static int
launch_split(emu_plan *e)
{
	int32_t *EA = (int32_t *)e->d_E, *EB = EA + e->nexp_a;
	int *flags = (int *)(EA + e->nE);

	XMG_CK(cudaMemsetAsync((void *)e->d_E, 0, (e->nE + 64) * sizeof(int32_t),
	    stream()));
	/* a shared a side: the preparing plan fills the shared exponent table
	 * and flag, every plan takes the flag's Inf/NaN bit into its own */
	int *aflags = flags;
	if (e->a_mode) {
		EA = (int32_t *)e->a_E;
		aflags = (int *)e->a_flag;
		if (e->a_mode == 1) {
			XMG_CK(cudaMemsetAsync(EA, 0, e->nexp_a * sizeof(int32_t), stream()));
			XMG_CK(cudaMemsetAsync(aflags, 0, sizeof(int), stream()));
		}
	}
	for (int side = 0; side < 2; side++) {
		const xmgd_view_t *dv = (const xmgd_view_t *)(side ? e->d_vb : e->d_va);
		const int nv = (int)(side ? e->VB.size() : e->VA.size());
		int32_t *E = side ? EB : EA;
		if (e->nctas[side][0] > 0 && !(side == 0 && e->a_mode == 2)) {
			emu_exp_kernel<TIN><<<(unsigned)e->nctas[side][0], 256, 0, stream()>>>(
			    dv, (const view_meta *)e->d_meta[side][0], nv, e->d_tabs, E,
			    side ? flags : aflags);
			g_launches++;
			XMG_CK(cudaGetLastError());
		}
		/* every plan of a shared a side, the preparing one and the
		 * ones that use it, takes its Inf/NaN bit */
		if (side == 0 && e->a_mode)
			XMG_CK(cudaMemcpyAsync(flags, aflags, sizeof(int),
			    cudaMemcpyDeviceToDevice, stream()));
	}
	for (int side = 0; side < 2; side++) {
		const xmgd_view_t *dv = (const xmgd_view_t *)(side ? e->d_vb : e->d_va);
		const int nv = (int)(side ? e->VB.size() : e->VA.size());
		const int32_t *E = side ? EB : EA;
		if (side == 0 && e->a_mode == 2)
			continue;
		if (e->nctas[side][1] > 0) {
			emu_split_kernel<TIN><<<(unsigned)e->nctas[side][1], 256, 0, stream()>>>(
			    dv, (const view_meta *)e->d_meta[side][1], nv, e->d_tabs, E);
			g_launches++;
			XMG_CK(cudaGetLastError());
		}
	}
	return XMG_OK;
}

/* the persistent grouped GEMM of the current candidate, then the flags */
template <typename TIN, typename TOUT>
static int
launch_gemm(emu_plan *e)
{
	constexpr int S = fin<TIN>::S, KEEP = fin<TIN>::KEEP;
	constexpr bool LOW = KEEP > 2;
	const emu_cand &c = e->cand[e->cur];
	int32_t *EA = (int32_t *)e->d_E, *EB = EA + e->nexp_a;
	int *flags = (int *)(EA + e->nE);
	if (e->a_mode)
		EA = (int32_t *)e->a_E;	/* the shared a side's table */

	if (pair_policy(c.policy)) {
		/* clusters of two CTAs */
		cudaLaunchConfig_t cfg = {};
		cudaLaunchAttribute at[1];
		at[0].id = cudaLaunchAttributeClusterDimension;
		at[0].val.clusterDim.x = 2;
		at[0].val.clusterDim.y = 1;
		at[0].val.clusterDim.z = 1;
		cfg.gridDim = dim3((unsigned)c.grid);
		cfg.blockDim = dim3(64 + 32 * EMU_DW);
		cfg.dynamicSmemBytes = stage_cfg<S>::SMEM;
		cfg.stream = stream();
		cfg.attrs = at;
		cfg.numAttrs = 1;
		XMG_CK(cudaLaunchKernelEx(&cfg, emu_gemm_kernel<S, KEEP, LOW, TOUT, EMU_DW, true>,
		    (const emu_item *)c.d_items, c.nitems, (const emu_member *)c.d_members,
		    e->d_cbs, e->d_prs,
		    (const xmgd_view_t *)e->d_va, (const xmgd_view_t *)e->d_vb, e->d_tabs,
		    (const int32_t *)EA, (const int32_t *)EB, (const int32_t *)e->d_F,
		    e->alpha, e->beta, 2 * fin<TIN>::EXPOFF, e->cplx, e->hmax, e->pfd, e->kchunk, flags));
	} else {
		emu_gemm_kernel<S, KEEP, LOW, TOUT, EMU_DW, false><<<(unsigned)c.grid,
		    64 + 32 * EMU_DW, stage_cfg<S>::SMEM, stream()>>>(
		    (const emu_item *)c.d_items, c.nitems, (const emu_member *)c.d_members,
		    e->d_cbs, e->d_prs,
		    (const xmgd_view_t *)e->d_va, (const xmgd_view_t *)e->d_vb, e->d_tabs,
		    EA, EB, (const int32_t *)e->d_F, e->alpha, e->beta,
		    2 * fin<TIN>::EXPOFF, e->cplx, e->hmax, e->pfd, e->kchunk, flags);
	}
	g_launches++;
	XMG_CK(cudaGetLastError());
	XMG_CK(cudaMemcpyAsync(e->h_flags, flags, 2 * sizeof(int),
	    cudaMemcpyDeviceToHost, stream()));
	return XMG_OK;
}

template <typename TIN, typename TOUT>
static int
set_attrs()
{
	constexpr int S = fin<TIN>::S, KEEP = fin<TIN>::KEEP;
	static bool done = false;
	if (!done) {
		XMG_CK(cudaFuncSetAttribute(emu_gemm_kernel<S, KEEP, (KEEP > 2), TOUT, EMU_DW, false>,
		    cudaFuncAttributeMaxDynamicSharedMemorySize, stage_cfg<S>::SMEM));
		XMG_CK(cudaFuncSetAttribute(emu_gemm_kernel<S, KEEP, (KEEP > 2), TOUT, EMU_DW, true>,
		    cudaFuncAttributeMaxDynamicSharedMemorySize, stage_cfg<S>::SMEM));
		done = true;
	}
	return XMG_OK;
}

static int
upload_new(const void *h, size_t bytes, uint64_t *d)
{
	int st;

	if ((st = xmgd_alloc(bytes ? bytes : 16, d)) != XMG_OK)
		return st;
	if (bytes)
		XMG_CK(cudaMemcpyAsync((void *)*d, h, bytes, cudaMemcpyHostToDevice,
		    stream()));
	return XMG_OK;
}

void
emu_free(emu_plan *e)
{
	if (!e)
		return;
	uint64_t bufs[] = {e->d_va, e->d_vb, e->d_meta[0][0], e->d_meta[0][1],
	    e->d_meta[1][0], e->d_meta[1][1], e->d_E, e->d_F};
	for (uint64_t b : bufs)
		if (b)
			xmgd_free(b);
	for (emu_cand &c : e->cand) {
		if (c.d_items)
			xmgd_free(c.d_items);
		if (c.d_members)
			xmgd_free(c.d_members);
	}
	if (e->h_flags)
		cudaFreeHost(e->h_flags);
	delete e;
}

/* work list of one policy (see above) */
static void
make_items(const xmgd_contract_t *p, const std::vector<int> &cblocks, int cplx,
    int policy, std::vector<emu_item> &items, std::vector<emu_member> &members)
{
	struct blk {
		int ci, swp, mlen, nlen;
		double cost;
		uint64_t key;
	};
	const bool merged = policy == EMU_POL_MERGED;
	const int base = merged ? 2 : policy % EMU_NPOLICY;
	const int mstep = pair_policy(policy) ? 2 * EMU_TM : EMU_TM;
	const int pol = base == 2 ? 2 : 0;
	std::vector<blk> bl;
	for (int ci : cblocks) {
		const xmgd_cblock_t &cb = p->cblocks[ci];
		double k = 0;
		for (int q = 0; q < cb.npairs; q++)
			k += p->pairs[cb.first_pair + q].k;
		blk b;
		b.ci = ci;
		b.swp = tile_cost(cb.m, cb.n, pol, mstep) < tile_cost(cb.n, cb.m, pol, mstep);
		b.mlen = b.swp ? cb.m : cb.n;
		b.nlen = b.swp ? cb.n : cb.m;
		b.cost = k * cb.m * (double)cb.n;
		/* the M-side free block (its exponent-table slot names it) */
		b.key = ((uint64_t)b.swp << 40) | (uint32_t)(b.swp ? cb.eA : cb.eB);
		bl.push_back(b);
	}
	/* one item per member list (every complex pass); N-stacked: m0 is the
	 * M tile and the members' rows add up to N; M-stacked: m0 is the N tile
	 * and ncols its live rows */
	auto push = [&](int m0, int swp, const std::vector<emu_member> &mem,
	    int mstk = 0, int ncols = 0) {
		int tot = 0;
		for (const emu_member &x : mem)
			tot += x.rows;
		if (mstk)
			tot = ncols;
		for (int ps = 0; ps < (cplx ? 2 : 1); ps++) {
			items.push_back(emu_item{m0, (int)members.size(), (int)mem.size(),
			    ps | (swp ? 2 : 0) | (mstk ? 4 : 0) | (tot << 8)});
			members.insert(members.end(), mem.begin(), mem.end());
		}
	};
	auto emit = [&](const blk &b, int m0) {
		for (int n0 = 0; n0 < b.nlen; n0 += EMU_TM) {
			const int rows = std::min(EMU_TM, (b.nlen - n0 + 15) / 16 * 16);
			push(m0, b.swp, {emu_member{b.ci, n0, rows, 0}});
		}
	};
	items.clear();
	members.clear();
	std::stable_sort(bl.begin(), bl.end(),
	    [](const blk &x, const blk &y) { return x.cost > y.cost; });
	if (base == 0) {
		for (const blk &b : bl)
			for (int m0 = 0; m0 < b.mlen; m0 += mstep)
				emit(b, m0);
		return;
	}
	/* grouped: blocks reading the same M-side rows together, M tile by
	 * M tile, groups by decreasing cost; merged: a group holds only
	 * blocks whose pair lists have the same M-side view and K at every
	 * index, so their tiles can share the M-side stages */
	std::vector<std::vector<int64_t>> gkey;
	std::vector<std::vector<int>> groups;
	std::vector<double> gcost;
	std::vector<int64_t> k;
	for (int i = 0; i < (int)bl.size(); i++) {
		k.assign(1, (int64_t)bl[i].key);
		if (merged) {
			const xmgd_cblock_t &cb = p->cblocks[bl[i].ci];
			k.push_back(bl[i].mlen);
			for (int q = 0; q < cb.npairs; q++) {
				const xmgd_pair_t &pr = p->pairs[cb.first_pair + q];
				k.push_back(((int64_t)(bl[i].swp ? pr.aview : pr.bview) << 32) | pr.k);
			}
		}
		size_t g = 0;
		while (g < groups.size() && gkey[g] != k)
			g++;
		if (g == groups.size()) {
			gkey.push_back(k);
			groups.push_back({});
			gcost.push_back(0);
		}
		groups[g].push_back(i);
		gcost[g] += bl[i].cost;
	}
	std::vector<int> go(groups.size());
	for (size_t g = 0; g < go.size(); g++)
		go[g] = (int)g;
	std::stable_sort(go.begin(), go.end(),
	    [&](int x, int y) { return gcost[x] > gcost[y]; });
	/* merged: partial M tiles wait for the M-stacking pass below */
	struct tail { int i, m0, n0, ncols; };
	std::vector<tail> tails;
	for (int g : go) {
		int mmax = 0;
		for (int i : groups[g])
			mmax = std::max(mmax, bl[i].mlen);
		for (int m0 = 0; m0 < mmax; m0 += mstep) {
			if (!merged) {
				for (int i : groups[g])
					if (m0 < bl[i].mlen)
						emit(bl[i], m0);
				continue;
			}
			if (mmax - m0 < EMU_TM) {
				for (int i : groups[g])
					for (int n0 = 0; n0 < bl[i].nlen; n0 += EMU_TM)
						tails.push_back(tail{i, m0, n0, std::min(EMU_TM,
						    (bl[i].nlen - n0 + 15) / 16 * 16)});
				continue;
			}
			/* full 128-row N tiles alone; the partial ones packed
			 * first-fit decreasing into tiles of <= 128 rows and
			 * <= EMU_MAXMEM members */
			std::vector<emu_member> part;
			for (int i : groups[g]) {
				const blk &b = bl[i];
				for (int n0 = 0; n0 < b.nlen; n0 += EMU_TM) {
					const int rows = std::min(EMU_TM, (b.nlen - n0 + 15) / 16 * 16);
					if (rows == EMU_TM)
						push(m0, b.swp, {emu_member{b.ci, n0, rows, 0}});
					else
						part.push_back(emu_member{b.ci, n0, rows, 0});
				}
			}
			std::stable_sort(part.begin(), part.end(),
			    [](const emu_member &x, const emu_member &y) { return x.rows > y.rows; });
			std::vector<std::vector<emu_member>> bins;
			std::vector<int> fill;
			for (const emu_member &x : part) {
				size_t b = 0;
				while (b < bins.size() && (fill[b] + x.rows > EMU_TM ||
				    (int)bins[b].size() == EMU_MAXMEM))
					b++;
				if (b == bins.size()) {
					bins.push_back({});
					fill.push_back(0);
				}
				emu_member y = x;
				y.off = fill[b];
				bins[b].push_back(y);
				fill[b] += x.rows;
			}
			for (const auto &mem : bins)
				push(m0, bl[groups[g][0]].swp, mem);
		}
	}
	if (!merged)
		return;
	/* M-stacking: the partial M tiles of blocks that share the N side (the
	 * same N-side view and K at every pair index, the same N tile) fill
	 * common 128-lane tiles, 32 lanes at a time; a tile left alone runs
	 * as an ordinary item */
	std::vector<std::vector<int64_t>> tkey;
	std::vector<std::vector<int>> tgrp;
	for (int x = 0; x < (int)tails.size(); x++) {
		const blk &b = bl[tails[x].i];
		const xmgd_cblock_t &cb = p->cblocks[b.ci];
		k.assign({(int64_t)b.swp, tails[x].n0, tails[x].ncols, b.nlen});
		for (int q = 0; q < cb.npairs; q++) {
			const xmgd_pair_t &pr = p->pairs[cb.first_pair + q];
			k.push_back(((int64_t)(b.swp ? pr.bview : pr.aview) << 32) | pr.k);
		}
		size_t g = 0;
		while (g < tkey.size() && tkey[g] != k)
			g++;
		if (g == tkey.size()) {
			tkey.push_back(k);
			tgrp.push_back({});
		}
		tgrp[g].push_back(x);
	}
	for (const std::vector<int> &tg : tgrp) {
		std::vector<emu_member> part;
		for (int x : tg) {
			const tail &tl = tails[x];
			const blk &b = bl[tl.i];
			part.push_back(emu_member{b.ci, tl.m0, (b.mlen - tl.m0 + 31) / 32 * 32, 0});
		}
		std::stable_sort(part.begin(), part.end(),
		    [](const emu_member &x, const emu_member &y) { return x.rows > y.rows; });
		std::vector<std::vector<emu_member>> bins;
		std::vector<int> fill;
		for (const emu_member &x : part) {
			size_t b = 0;
			while (b < bins.size() && (fill[b] + x.rows > EMU_TM ||
			    (int)bins[b].size() == EMU_MAXMEM))
				b++;
			if (b == bins.size()) {
				bins.push_back({});
				fill.push_back(0);
			}
			emu_member y = x;
			y.off = fill[b];
			bins[b].push_back(y);
			fill[b] += x.rows;
		}
		const tail &t0 = tails[tg[0]];
		const int swp = bl[t0.i].swp;
		for (const auto &mem : bins) {
			if (mem.size() == 1)
				push(mem[0].n0, swp, {emu_member{mem[0].cblock, t0.n0, t0.ncols, 0}});
			else
				push(t0.n0, swp, mem, 1, t0.ncols);
		}
	}
}

/* The invariants the kernel's addressing relies on, checked on the host
 * before a work list is uploaded: member tiles inside their views and the
 * stage (rows multiples of 16, stacked without gaps, <= 128 in all), and
 * members that share the M side pair by pair. */
static bool
items_ok(const xmgd_contract_t *p, const std::vector<emu_item> &items,
    const std::vector<emu_member> &mem, bool pair)
{
	for (const emu_item &it : items) {
		if (it.mcount < 1 || it.mcount > (pair ? 1 : EMU_MAXMEM) || it.mfirst < 0 ||
		    (size_t)it.mfirst + it.mcount > mem.size())
			return false;
		const int swp = (it.pr >> 1) & 1, tot = it.pr >> 8;
		const xmgd_cblock_t &c0 = p->cblocks[mem[it.mfirst].cblock];
		if ((it.pr >> 2) & 1) {
			/* M-stacked: the shared N tile, then 32-lane members */
			const int nlen = swp ? c0.n : c0.m;
			if (pair || it.m0 < 0 || it.m0 % EMU_TM || it.m0 >= nlen ||
			    tot != std::min(EMU_TM, (nlen - it.m0 + 15) / 16 * 16))
				return false;
			int off = 0;
			for (int j = 0; j < it.mcount; j++) {
				const emu_member &m = mem[it.mfirst + j];
				if (m.cblock < 0 || m.cblock >= p->ncblocks)
					return false;
				const xmgd_cblock_t &cb = p->cblocks[m.cblock];
				const int ml = swp ? cb.m : cb.n;
				if ((swp ? cb.n : cb.m) != nlen || cb.npairs != c0.npairs ||
				    m.off != off || m.rows < 32 || m.rows % 32 || m.n0 < 0 ||
				    m.n0 % EMU_TM || m.n0 >= ml ||
				    m.rows != std::min(EMU_TM, (ml - m.n0 + 31) / 32 * 32))
					return false;
				for (int q = 0; q < cb.npairs; q++) {
					const xmgd_pair_t &a = p->pairs[c0.first_pair + q];
					const xmgd_pair_t &b = p->pairs[cb.first_pair + q];
					if (a.k != b.k || (swp ? a.bview != b.bview : a.aview != b.aview))
						return false;
				}
				off += m.rows;
			}
			if (off > EMU_TM)
				return false;
			continue;
		}
		const int mlen = swp ? c0.m : c0.n;
		if (it.m0 < 0 || it.m0 % EMU_TM || it.m0 >= mlen)
			return false;
		int off = 0;
		for (int j = 0; j < it.mcount; j++) {
			const emu_member &m = mem[it.mfirst + j];
			if (m.cblock < 0 || m.cblock >= p->ncblocks)
				return false;
			const xmgd_cblock_t &cb = p->cblocks[m.cblock];
			const int nlen = swp ? cb.n : cb.m;
			if ((swp ? cb.m : cb.n) != mlen || cb.npairs != c0.npairs ||
			    m.off != off || m.rows < 16 || m.rows % 16 || m.n0 < 0 ||
			    m.n0 % EMU_TM || m.n0 >= nlen ||
			    m.rows > std::min(EMU_TM, (nlen - m.n0 + 15) / 16 * 16))
				return false;
			for (int q = 0; q < cb.npairs; q++) {
				const xmgd_pair_t &a = p->pairs[c0.first_pair + q];
				const xmgd_pair_t &b = p->pairs[cb.first_pair + q];
				if (a.k != b.k || (swp ? a.aview != b.aview : a.bview != b.bview))
					return false;
			}
			off += m.rows;
		}
		if (off != tot || tot < 16 || tot > EMU_TM)
			return false;
	}
	return true;
}

int
emu_prepare(const xmgd_contract_t *p, const std::vector<int> &cblocks,
    const xmgd_cblock_t *d_cbs, const xmgd_pair_t *d_prs,
    const int32_t *d_tabs, emu_plan **out)
{
	const bool realab = p->alpha[1] == 0 && p->beta[1] == 0;
	int cplx, st;

	*out = nullptr;
	switch (p->dtype) {
	case 0: case 2: cplx = 0; break;
	case 1: case 3:
		/* two real passes need real alpha and beta */
		if (!realab)
			return xmg_seterr(XMG_ENOTSUP, "split-precision path: complex "
			    "alpha/beta");
		cplx = 1;
		break;
	default:
		return xmg_seterr(XMG_ENOTSUP, "split-precision path: scalar type");
	}
	const bool dbl = p->dtype >= 2;
	const int chunk_bytes = (dbl ? fin<double>::S : fin<float>::S) * SLICE_BYTES;
	emu_plan *e = new emu_plan();
	e->dtype = p->dtype;
	e->cplx = cplx;
	{
		const int nst = dbl ? stage_cfg<fin<double>::S>::NST : stage_cfg<fin<float>::S>::NST;
		/* head/tail length in stages: 2 two-step stages (FP64), 1
		 * three-step stage (FP32) */
		const char *h = getenv("XMG_EMU_HEAD");
		e->hmax = h ? atoi(h) : (dbl ? 2 : 1);
		e->hmax = std::max(1, std::min(nst, e->hmax));
		/* FP64 chunks in whole stages (they start at a segment's first
		 * step, as the stages do) */
		const char *kc = getenv("XMG_EMU_CHUNK");
		constexpr int KS64 = stage_cfg<fin<double>::S>::KSTEPS;
		e->kchunk = kc ? std::max(1, std::min(20, atoi(kc))) : EMU_CHUNK;
		e->kchunk = std::max(KS64, e->kchunk / KS64 * KS64);
		const char *f = getenv("XMG_EMU_PF");
		e->pfd = f ? std::max(0, atoi(f)) : 0;
	}
	e->alpha = p->alpha[0];
	e->beta = p->beta[0];
	e->d_cbs = d_cbs;
	e->d_prs = d_prs;
	e->d_tabs = d_tabs;
	e->VA.assign(p->views_a, p->views_a + p->nviews_a);
	e->VB.assign(p->views_b, p->views_b + p->nviews_b);
	/* the plan that prepares a shared a side splits every view of a */
	e->a_mode = p->a_mode;
	e->a_slices = p->a_slices;
	e->a_E = p->a_E;
	e->a_flag = p->a_flag;
	e->useA.assign(e->VA.size(), p->a_mode == 1);
	e->useB.assign(e->VB.size(), 0);
	e->split = dbl ? launch_split<double> : launch_split<float>;
	e->gemm = dbl ? launch_gemm<double, double> : launch_gemm<float, float>;
	if ((st = dbl ? set_attrs<double, double>() : set_attrs<float, float>()))
		goto fail;

	{
	/* operand views used by the emulated blocks, and the fixed-point
	 * scale F of every block (|V| <= K_eff * 2^(30+F) < 2^61) */
	std::vector<int32_t> F(p->ncblocks, 0);
	std::vector<uint64_t> hist;
	for (int ci : cblocks) {
		const xmgd_cblock_t &cb = p->cblocks[ci];
		double keff = 0;
		int64_t ksum = 0;
		for (int q = 0; q < cb.npairs; q++) {
			const xmgd_pair_t &pr = p->pairs[cb.first_pair + q];
			e->useA[pr.aview] = e->useB[pr.bview] = 1;
			double kr = cplx ? 2.0 * 16 * ((pr.k + 15) / 16) : pr.k;
			keff += ldexp(1.0, std::max(pr.eshift, 0)) * kr;
			ksum += pr.k;
		}
		int lg = (int)ceil(log2(std::max(keff, 2.0)));
		if (lg > 31) {
			st = xmg_seterr(XMG_ENOTSUP, "split-precision path: K too large");
			goto fail;
		}
		F[ci] = std::min(24, 31 - lg);
		hist.push_back(mix64(((uint64_t)cb.m << 40) ^ ((uint64_t)cb.n << 20) ^
		    (uint64_t)ksum));
	}
	std::sort(hist.begin(), hist.end());
	uint64_t sig = mix64((uint64_t)p->dtype + 1);
	for (uint64_t h : hist)
		sig = mix64(sig ^ h);
	e->sig = sig;

	/* slice storage: offsets now, rebased onto the workspace at bind */
	size_t off = 0;
	auto tile = [&](std::vector<xmgd_view_t> &V, std::vector<char> &use,
	    const int64_t *ext) {
		for (size_t v = 0; v < V.size(); v++) {
			if (!use[v])
				continue;
			xmgd_view_t &w = V[v];
			w.n_rt = (w.mn + EMU_TM - 1) / EMU_TM;
			w.cplx = cplx;
			w.khp = EMU_KS * ((w.k + EMU_KS - 1) / EMU_KS);
			w.n_ks = (cplx ? 2 : 1) * (w.khp / EMU_KS);
			w.kfast = w.k > 1 && p->tabs[w.rowtab + 1] - p->tabs[w.rowtab] == 1;
			w.kcontig = w.kfast;
			for (int32_t k = 2; w.kcontig && k < w.k; k++)
				w.kcontig = p->tabs[w.rowtab + k] - p->tabs[w.rowtab] == k;
			if (ext) {	/* in the shared a side's buffer */
				w.slices = (uint64_t)ext[v];
				continue;
			}
			w.slices = off;
			off += (size_t)w.n_rt * w.n_ks * chunk_bytes;
		}
	};
	tile(e->VA, e->useA, p->a_mode ? p->a_off : nullptr);
	tile(e->VB, e->useB, nullptr);
	e->slice_bytes = off;

	/* CTA ranges of the exponent and split launches of each side */
	for (int side = 0; side < 2; side++) {
		std::vector<xmgd_view_t> &V = side ? e->VB : e->VA;
		std::vector<char> &use = side ? e->useB : e->useA;
		for (int kind = 0; kind < 2; kind++) {
			std::vector<view_meta> meta(V.size());
			int64_t n = 0;
			for (size_t v = 0; v < V.size(); v++) {
				meta[v].first_cta = n;
				if (!use[v])
					continue;
				if (kind == 0)
					n += (int64_t)V[v].n_rt * ((V[v].n_ks * EMU_KS + 255) / 256);
				else
					n += (int64_t)V[v].n_rt * ((V[v].n_ks + 3) / 4);
			}
			e->nctas[side][kind] = n;
			if ((st = upload_new(meta.data(), meta.size() * sizeof(view_meta),
			    &e->d_meta[side][kind])))
				goto fail;
		}
	}
	e->nexp_a = p->nexp_a;
	e->nE = (int64_t)p->nexp_a + p->nexp_b;
	if ((st = xmgd_alloc((e->nE + 64) * sizeof(int32_t), &e->d_E)) ||
	    (st = upload_new(F.data(), F.size() * sizeof(int32_t), &e->d_F)) ||
	    (st = xmgd_alloc(e->VA.size() * sizeof(xmgd_view_t) + 16, &e->d_va)) ||
	    (st = xmgd_alloc(e->VB.size() * sizeof(xmgd_view_t) + 16, &e->d_vb)))
		goto fail;

	/* work lists: a remembered policy for this histogram, else every
	 * distinct policy once */
	int known = -1;
	for (const tune_entry &t : g_tuned)
		if (t.sig == sig)
			known = t.policy;
	if (getenv("XMG_TUNE") && strcmp(getenv("XMG_TUNE"), "0") == 0)
		known = EMU_POL_MERGED;
	if (getenv("XMG_POLICY"))	/* one fixed work-list policy */
		known = atoi(getenv("XMG_POLICY"));
	/* a plan that runs once has no runs left to tune with: the first
	 * list that passes its checks */
	const bool first_only = p->one_shot && known < 0;
	/* the stacked list first: a plan that runs once (an out-of-core
	 * batch) never finishes tuning and keeps its first candidate */
	std::vector<int> pols = {EMU_POL_MERGED, 0, 1, 2};
	if (pairs_enabled())
		pols.insert(pols.end(), {EMU_NPOLICY, EMU_NPOLICY + 1, EMU_NPOLICY + 2});
	std::vector<std::vector<emu_item>> lists;
	std::vector<std::vector<emu_member>> mlists;
	for (int pol : pols) {
		if (known >= 0 && pol != known)
			continue;
		if (first_only && !e->cand.empty())
			break;
		std::vector<emu_item> items;
		std::vector<emu_member> mem;
		make_items(p, cblocks, cplx, pol, items, mem);
		/* a list that fails its checks is never uploaded; the others
		 * stand in for it */
		if (!items_ok(p, items, mem, pair_policy(pol)))
			continue;
		bool dup = false;
		for (size_t l = 0; l < lists.size(); l++)
			dup |= lists[l].size() == items.size() && mlists[l].size() == mem.size() &&
			    memcmp(lists[l].data(), items.data(), items.size() * sizeof(emu_item)) == 0 &&
			    memcmp(mlists[l].data(), mem.data(), mem.size() * sizeof(emu_member)) == 0;
		if (dup)
			continue;
		emu_cand c;
		c.policy = pol;
		c.nitems = (int)items.size();
		c.grid = pair_policy(pol) ? 2 * std::min(c.nitems, num_sms() / 2) :
		    std::min(c.nitems, num_sms());
		c.ms = -1;
		c.d_items = c.d_members = 0;
		if ((st = upload_new(items.data(), items.size() * sizeof(emu_item),
		    &c.d_items)) || (st = upload_new(mem.data(), mem.size() *
		    sizeof(emu_member), &c.d_members))) {
			e->cand.push_back(c);	/* freed with the plan */
			goto fail;
		}
		e->cand.push_back(c);
		lists.push_back(std::move(items));
		mlists.push_back(std::move(mem));
	}
	if (e->cand.empty()) {
		st = xmg_seterr(XMG_EINVAL, "split-precision path: no work list "
		    "passed its checks");
		goto fail;
	}
	e->tuned = e->cand.size() <= 1;
	if ((st = check(cudaMallocHost(&e->h_flags, 2 * sizeof(int)), "flags")) ||
	    (st = check(cudaStreamSynchronize(stream()), "plan upload")))
		goto fail;
	e->h_flags[0] = e->h_flags[1] = 0;
	}
	*out = e;
	return XMG_OK;
fail:
	emu_free(e);
	return st;
}

/* Slice workspace and absolute view addresses; *moved when the views had
 * to be re-uploaded (a captured graph holding the old ones is stale). */
int
emu_bind(emu_plan *e, bool *moved)
{
	uint64_t ws;
	int st;

	*moved = false;
	if ((st = xmgd_scratch(8, e->slice_bytes + 16, &ws)) != XMG_OK)
		return st;
	if (ws == e->ws)
		return XMG_OK;
	for (int side = 0; side < 2; side++) {
		std::vector<xmgd_view_t> V = side ? e->VB : e->VA;
		std::vector<char> &use = side ? e->useB : e->useA;
		const uint64_t base = side == 0 && e->a_mode ? e->a_slices : ws;
		for (size_t v = 0; v < V.size(); v++)
			if (use[v])
				V[v].slices += base;
		XMG_CK(cudaMemcpyAsync((void *)(side ? e->d_vb : e->d_va), V.data(),
		    V.size() * sizeof(xmgd_view_t), cudaMemcpyHostToDevice, stream()));
		XMG_CK(cudaStreamSynchronize(stream()));
	}
	e->ws = ws;
	*moved = true;
	return XMG_OK;
}

/* the work list of one policy, built and checked on the host (no device) */
extern "C" int
xmgd_work_list_check(const xmgd_contract_t *p, int policy, long long out[4])
{
	int cplx;

	switch (p->dtype) {
	case 0: case 2: cplx = 0; break;
	case 1: case 3: cplx = 1; break;
	default:
		return xmg_seterr(XMG_EINVAL, "work list: scalar type");
	}
	if (policy < 0 || (policy >= EMU_NPOLICY && !pair_policy(policy) &&
	    policy != EMU_POL_MERGED))
		return xmg_seterr(XMG_EINVAL, "work list: no policy %d", policy);
	std::vector<int> cblocks;
	for (int i = 0; i < p->ncblocks; i++)
		if (p->cblocks[i].npairs > 0 && p->emulatable[i])
			cblocks.push_back(i);
	std::vector<emu_item> items;
	std::vector<emu_member> mem;
	make_items(p, cblocks, cplx, policy, items, mem);
	long long stacked = 0;
	for (const emu_item &it : items)
		stacked += it.mcount > 1;
	out[0] = (long long)items.size();
	out[1] = (long long)mem.size();
	out[2] = stacked;
	out[3] = items_ok(p, items, mem, pair_policy(policy)) ? 1 : 0;
	return XMG_OK;
}

int emu_current(const emu_plan *e) { return e->cur; }
int emu_ncand(const emu_plan *e) { return (int)e->cand.size(); }
bool emu_tuned(const emu_plan *e) { return e->tuned != 0; }

int emu_record_split(emu_plan *e) { return e->split(e); }
int emu_record_gemm(emu_plan *e) { return e->gemm(e); }
int64_t emu_slice_bytes(const emu_plan *e) { return (int64_t)e->slice_bytes; }
int emu_a_mode(const emu_plan *e) { return e->a_mode; }

/* the slice bytes tile() gives one view */
extern "C" int64_t
xmgd_emu_view_bytes(const xmgd_view_t *v, int dtype)
{
	if (dtype < 0 || dtype > 3)
		return 0;
	const bool cplx = dtype == 1 || dtype == 3;
	const int chunk_bytes = (dtype >= 2 ? fin<double>::S : fin<float>::S) *
	    SLICE_BYTES;
	const int64_t n_rt = (v->mn + EMU_TM - 1) / EMU_TM;
	const int64_t n_ks = (cplx ? 2 : 1) * ((v->k + EMU_KS - 1) / EMU_KS);
	return n_rt * n_ks * chunk_bytes;
}
int emu_items(const emu_plan *e) { return e->cand[e->cur].nitems; }
int emu_policy(const emu_plan *e) { return e->cand[e->cur].policy; }

/* after the stream has drained: flags, then one tuning step with the
 * measured GEMM time of the candidate that ran */
int
emu_finish(emu_plan *e, float gemm_ms, int *nan)
{
	*nan = e->h_flags[0] & 1;
	if (e->h_flags[1])
		return xmg_seterr(XMG_ETIMEOUT, "split-precision GEMM: bounded "
		    "wait %d timed out", e->h_flags[1]);
	if (!e->tuned && !*nan) {
		e->cand[e->cur].ms = gemm_ms;
		if (e->cur + 1 < (int)e->cand.size())
			e->cur++;
		else {
			int best = 0;
			for (int i = 1; i < (int)e->cand.size(); i++)
				if (e->cand[i].ms < e->cand[best].ms)
					best = i;
			e->cur = best;
			e->tuned = 1;
			g_tuned.push_back(tune_entry{e->sig, e->cand[best].policy});
		}
	}
	return XMG_OK;
}

} /* namespace xmg */
