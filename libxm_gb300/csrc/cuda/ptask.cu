/*
 * Permuted, scaled element-wise block kernels of libxm-gb300.
 *
 * One launch covers a batch of block tasks (xmgd_ptask_t): xm_set,
 * xm_copy, xm_add, xm_mul, xm_div, xm_dot and the standalone
 * xm_tensor_unfold_block / xm_tensor_fold_block all reduce to "for every
 * element of an up-to-8-D box, dst[.] = f(dst[.], src[.])" with independent
 * destination and source strides.  This replaces the reference's per-block
 * unfold -> scale -> fold -> axpy host loops (tensor.c:436-639,
 * scalar.c:123-239, xm.c:28-508) with one HBM pass.
 *
 * Four schedules, chosen per task on the host after xmg_ptask_shape has
 * normalised the iteration space; each schedule is its own kernel
 * instantiation (so the lean ones keep few registers and full occupancy),
 * and a batch launches one kernel per schedule present:
 *  - flat: one contiguous run on both sides (whole canonical blocks);
 *  - row: dimension 0 unit-stride on the destination side; a CTA covers
 *    ROW_ELEMS elements along dim 0 for as many outer rows as fit, with
 *    per-row outer offsets precomputed in shared memory;
 *  - matrix: the source's unit-stride dimension is dim 1 and both extents
 *    fit one tile; a CTA moves whole s0 x s1 slices through padded shared
 *    memory (loads along the source's runs, stores along the
 *    destination's): the gather-transpose of unfold/fold;
 *  - tile: the same for larger extents, TILE x TILE tiles;
 *  - slab: xm_copy's transposes when each s0 x s1 slice lies contiguously
 *    on both sides and consecutive slices follow one another (whole
 *    blocks whose permutation swaps the two leading dimensions): a CTA
 *    brings its slices in with one bulk copy into shared memory,
 *    transposes there and stores along the destination's run.
 */
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "tc.cuh"

namespace xmg {

constexpr int PT_THREADS = 256;
constexpr int ROW_ELEMS = 4096;    /* elements per CTA in row mode */
constexpr int FLAT_ELEMS = 8192;   /* elements per CTA in flat mode */
constexpr int TILE = 32;
/* matrix mode: whole s0 x s1 slices (both <= MT) per CTA; a source and a
 * destination tile of both types fit the 48 KB of static shared memory */
template <typename D, typename S> struct mt_of {
	static constexpr int v = sizeof(S) <= 8 && sizeof(D) <= 8 ? 48 : 32;
};
static inline int mt_host(int dbytes, int sbytes)
{
	return sbytes <= 8 && dbytes <= 8 ? 48 : 32;
}
constexpr int MAT_MAXQ = 64;       /* slices per CTA at most */
/* slab schedule: about SLAB_CHUNK bytes of slices per CTA (one slice at
 * least), at most SLAB_SMEM bytes of shared memory (the source's slices
 * and the padded tile) */
constexpr int64_t SLAB_CHUNK = 16384;
constexpr int64_t SLAB_SMEM = 64 * 1024;


struct task_meta {
	int64_t first_cta;
	int32_t mode;          /* 0 row, 1 tile, 2 flat, 3 matrix, 4 slab */
	int32_t rows_per_cta;  /* row mode: outer rows per CTA */
	int64_t nouter;        /* row: product of dims 1..; tile: dims 2.. */
	int32_t ctas_d0, ctas_d1;
};

template <typename D, typename S>
struct elem_op {
	__device__ static inline void
	apply(int op, D *dp, const S *sp, const D &al, const S &als, const D &be,
	    double &dre, double &dim_)
	{
		switch (op) {
		case XMGD_OP_SET: *dp = al; break;
		case XMGD_OP_COPY: *dp = conv<D, S>(num<S>::mul(als, *sp)); break;
		case XMGD_OP_SCALE: *dp = num<D>::mul(al, *dp); break;
		case XMGD_OP_AXPY: {
			D s = conv<D, S>(*sp);
			*dp = num<D>::add(num<D>::mul(al, *dp), num<D>::mul(be, s));
			break;
		}
		case XMGD_OP_MUL: {
			D s = conv<D, S>(*sp);
			*dp = num<D>::mul(num<D>::mul(al, *dp), s);
			break;
		}
		case XMGD_OP_DIV: {
			D s = conv<D, S>(*sp);
			*dp = num<D>::div(*dp, num<D>::mul(al, s));
			break;
		}
		case XMGD_OP_DOT: {
			D s = conv<D, S>(*sp);
			D pr = num<D>::mul(*dp, s);
			dre += num<D>::re(pr);
			dim_ += num<D>::im(pr);
			break;
		}
		}
	}
};

/*
 * Flat runs with 16-byte accesses.  Each thread issues the loads of U
 * vectors (of both runs) before any of its stores: stores to dst may alias
 * src as far as the compiler knows, so a plain loop keeps one iteration's
 * loads in flight at a time.
 */
template <typename D> struct alignas(16) vec16 { D v[16 / sizeof(D)]; };

template <int OP, typename D>
__device__ inline void
flat_vec(vec16<D> *dv, const vec16<D> *sv, int nv, const D al, const D be,
    double &dre, double &dim_)
{
	constexpr int W = 16 / sizeof(D), U = 4;
	constexpr bool RD = OP != XMGD_OP_COPY && OP != XMGD_OP_SET;
	constexpr bool RS = OP != XMGD_OP_SET && OP != XMGD_OP_SCALE;
	constexpr bool WR = OP != XMGD_OP_DOT;

	for (int e0 = threadIdx.x; e0 < nv; e0 += U * PT_THREADS) {
		vec16<D> x[U], y[U];
#pragma unroll
		for (int u = 0; u < U; u++) {
			const int e = e0 + u * PT_THREADS;
			if (e < nv) {
				if (RD)
					x[u] = dv[e];
				if (RS)
					y[u] = sv[e];
			}
		}
#pragma unroll
		for (int u = 0; u < U; u++) {
			const int e = e0 + u * PT_THREADS;
			if (e >= nv)
				break;
#pragma unroll
			for (int w = 0; w < W; w++) {
				D &xv = x[u].v[w];
				if (OP == XMGD_OP_SET)
					xv = al;
				else if (OP == XMGD_OP_SCALE)
					xv = num<D>::mul(al, xv);
				else if (OP == XMGD_OP_AXPY)
					xv = num<D>::add(num<D>::mul(al, xv),
					    num<D>::mul(be, y[u].v[w]));
				else if (OP == XMGD_OP_COPY)
					xv = num<D>::mul(al, y[u].v[w]);
				else if (OP == XMGD_OP_MUL)
					xv = num<D>::mul(num<D>::mul(al, xv), y[u].v[w]);
				else if (OP == XMGD_OP_DIV)
					xv = num<D>::div(xv, num<D>::mul(al, y[u].v[w]));
				else {
					const D pr = num<D>::mul(xv, y[u].v[w]);
					dre += num<D>::re(pr);
					dim_ += num<D>::im(pr);
				}
			}
			if (WR)
				dv[e] = x[u];
		}
	}
}

static __device__ inline void
outer_offsets(const xmgd_ptask_t &t, int first_dim, int64_t o, int64_t &od,
    int64_t &os)
{
	od = 0;
	os = 0;
	for (int d = first_dim; d < t.ndim; d++) {
		int64_t sz = t.size[d];
		int64_t q = o % sz;
		o /= sz;
		od += q * t.dst_stride[d];
		os += q * t.src_stride[d];
	}
}

template <typename D, typename S, int MODE>
__global__ void __launch_bounds__(PT_THREADS, MODE == 0 ? 6 : MODE == 3 ? 5 : MODE == 2 ? 5 : 1)
ptask_kernel(const xmgd_ptask_t *__restrict__ tasks,
    const task_meta *__restrict__ meta, int ntasks, int64_t cta0,
    double *__restrict__ partial)
{
	__shared__ double s_red[2][PT_THREADS / 32];

	/* locate the task of this CTA (binary search over first_cta) */
	const int64_t cta = cta0 + blockIdx.x;
	int lo = 0, hi = ntasks - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (meta[mid].first_cta <= cta) lo = mid; else hi = mid - 1;
	}
	const xmgd_ptask_t &t = tasks[lo];
	const task_meta &m = meta[lo];
	int64_t local = cta - m.first_cta;
	D *dst = reinterpret_cast<D *>(t.dst);
	const S *src = reinterpret_cast<const S *>(t.src);
	const D al = num<D>::mk(t.alpha), be = num<D>::mk(t.beta);
	const S als = num<S>::mk(t.alpha);
	const int op = t.op;
	double dre = 0, dim_ = 0;

	if constexpr (MODE == 2) {
		/* flat: consecutive threads take consecutive elements, the op
		 * resolved outside the loop */
		const int64_t base = local * FLAT_ELEMS;
		const int n = (int)(t.size[0] - base < FLAT_ELEMS ? t.size[0] - base :
		    FLAT_ELEMS);
		D *dp = dst + base;
		const S *sp = src + base;
		bool done = false;
		if constexpr (std::is_same<D, S>::value && sizeof(D) < 16) {
			/* 16-byte accesses when both runs start on a 16-byte
			 * boundary (whole blocks do), scalar tail */
			constexpr int W = 16 / sizeof(D);
			const bool al16 = ((reinterpret_cast<uintptr_t>(dp) |
			    reinterpret_cast<uintptr_t>(sp)) & 15) == 0;
			const int nv = n / W;
			vec16<D> *dv = reinterpret_cast<vec16<D> *>(dp);
			const vec16<D> *sv = reinterpret_cast<const vec16<D> *>(sp);
			done = al16;
			if (al16) {
				switch (op) {
				case XMGD_OP_SET:
					flat_vec<XMGD_OP_SET>(dv, sv, nv, al, be, dre, dim_);
					break;
				case XMGD_OP_SCALE:
					flat_vec<XMGD_OP_SCALE>(dv, sv, nv, al, be, dre, dim_);
					break;
				case XMGD_OP_AXPY:
					flat_vec<XMGD_OP_AXPY>(dv, sv, nv, al, be, dre, dim_);
					break;
				case XMGD_OP_COPY:
					flat_vec<XMGD_OP_COPY>(dv, sv, nv, als, be, dre, dim_);
					break;
				case XMGD_OP_MUL:
					flat_vec<XMGD_OP_MUL>(dv, sv, nv, al, be, dre, dim_);
					break;
				case XMGD_OP_DIV:
					flat_vec<XMGD_OP_DIV>(dv, sv, nv, al, be, dre, dim_);
					break;
				case XMGD_OP_DOT:
					flat_vec<XMGD_OP_DOT>(dv, sv, nv, al, be, dre, dim_);
					break;
				default:
					done = false;
				}
			}
			if (done)
				for (int e = nv * W + threadIdx.x; e < n; e += PT_THREADS)
					elem_op<D, S>::apply(op, dp + e, sp + e, al, als, be, dre, dim_);
		}
		if (!done)
		switch (op) {
		case XMGD_OP_SET:
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS)
				dp[e] = al;
			break;
		case XMGD_OP_SCALE:
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS)
				dp[e] = num<D>::mul(al, dp[e]);
			break;
		case XMGD_OP_AXPY:
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS) {
				const D x = conv<D, S>(sp[e]);
				dp[e] = num<D>::add(num<D>::mul(al, dp[e]), num<D>::mul(be, x));
			}
			break;
		case XMGD_OP_COPY:
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS)
				dp[e] = conv<D, S>(num<S>::mul(als, sp[e]));
			break;
		default:
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS)
				elem_op<D, S>::apply(op, dp + e, sp + e, al, als, be, dre, dim_);
		}
	} else if constexpr (MODE == 0) {
		/* row */
		__shared__ int64_t s_od[PT_THREADS], s_os[PT_THREADS];
		int64_t s0 = t.size[0];
		int64_t c0 = local % m.ctas_d0;
		int64_t orow = (local / m.ctas_d0) * m.rows_per_cta;
		int64_t i0beg = c0 * ROW_ELEMS;
		int64_t w0 = s0 - i0beg < ROW_ELEMS ? s0 - i0beg : ROW_ELEMS;
		int rows = m.rows_per_cta;
		if (orow + rows > m.nouter)
			rows = (int)(m.nouter - orow);
		for (int r = threadIdx.x; r < rows; r += PT_THREADS)
			outer_offsets(t, 1, orow + r, s_od[r], s_os[r]);
		__syncthreads();
		const int64_t ds0 = t.dst_stride[0], ss0 = t.src_stride[0];
		if (w0 >= 32) {
			/* long rows: wpr warps per row (all eight on one row), lanes
			 * along it */
			const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
			const int wpr = rows >= PT_THREADS / 32 ? 1 : (PT_THREADS / 32) / rows;
			const int step = 32 * wpr;
			for (int r = warp / wpr; r < rows; r += (PT_THREADS / 32) / wpr) {
				D *dr = dst + s_od[r];
				const S *sr = src + s_os[r];
#pragma unroll 4
				for (int64_t i0 = i0beg + (warp % wpr) * 32 + lane;
				    i0 < i0beg + w0; i0 += step)
					elem_op<D, S>::apply(op, dr + i0 * ds0, sr + i0 * ss0, al,
					    als, be, dre, dim_);
			}
		} else {
			/* short rows: flattened, 32-bit index arithmetic */
			const int w0i = (int)w0, n = w0i * rows;
#pragma unroll 4
			for (int e = threadIdx.x; e < n; e += PT_THREADS) {
				const int r = e / w0i;
				const int64_t i0 = i0beg + (e - r * w0i);
				elem_op<D, S>::apply(op, dst + s_od[r] + i0 * ds0,
				    src + s_os[r] + i0 * ss0, al, als, be, dre, dim_);
			}
		}
	} else if constexpr (MODE == 3) {
		/* matrix: whole s0 x s1 slices (dim 0 unit-stride in dst, dim 1
		 * in src); rows_per_cta slices per CTA.  Every load of the CTA is
		 * in flight at once as a cp.async copy: the source transposed
		 * into a padded tile (row pitch s0 + 1), the destination (when
		 * the op reads it) into a second tile in its own order; one wait;
		 * then the op from shared memory and stores along the
		 * destination's runs */
		constexpr int MT = mt_of<D, S>::v;
		__shared__ __align__(16) S mtile[MT * (MT + 1)];
		__shared__ __align__(16) D dtile[MT * MT];
		__shared__ int64_t s_o[2][MAT_MAXQ];
		const int s0 = (int)t.size[0], s1 = (int)t.size[1], n = s0 * s1;
		const int ld = s0 + 1, pitch = s1 * ld;
		const int64_t ss0 = t.src_stride[0], ds1 = t.dst_stride[1];
		const int64_t o0 = local * m.rows_per_cta;
		const int k = (int)(m.nouter - o0 < m.rows_per_cta ? m.nouter - o0 :
		    m.rows_per_cta);
		const bool rd = op != XMGD_OP_COPY;	/* the op reads dst */
		for (int q = threadIdx.x; q < k; q += PT_THREADS)
			outer_offsets(t, 2, o0 + q, s_o[0][q], s_o[1][q]);
		__syncthreads();
		const int kn = k * n;
		/* flattened walks with the mixed-radix digits advanced by the
		 * thread stride (one division per CTA, not per element) */
		{
			/* source: e = q n + i0 s1 + i1 (runs along i1) */
			int q = threadIdx.x / n, r = threadIdx.x - q * n;
			int i0 = r / s1, i1 = r - i0 * s1;
			const int dq = PT_THREADS / n, dr = PT_THREADS - dq * n;
			const int d0 = dr / s1, d1 = dr - d0 * s1;
			for (int e = threadIdx.x; e < kn; e += PT_THREADS) {
				cp_async_elem(&mtile[q * pitch + i1 * ld + i0],
				    &src[s_o[1][q] + i0 * ss0 + i1]);
				i1 += d1;
				if (i1 >= s1) { i1 -= s1; i0++; }
				i0 += d0;
				if (i0 >= s0) { i0 -= s0; q++; }
				q += dq;
			}
		}
		/* destination: e = q n + i1 s0 + i0 (runs along i0); tile slot e */
		int q = threadIdx.x / n, r = threadIdx.x - q * n;
		int i1 = r / s0, i0 = r - i1 * s0;
		const int dq = PT_THREADS / n, dr = PT_THREADS - dq * n;
		const int d1 = dr / s0, d0 = dr - d1 * s0;
		if (rd) {
			int qq = q, j0 = i0, j1 = i1;
			for (int e = threadIdx.x; e < kn; e += PT_THREADS) {
				cp_async_elem(&dtile[e], dst + s_o[0][qq] + j0 + j1 * ds1);
				j0 += d0;
				if (j0 >= s0) { j0 -= s0; j1++; }
				j1 += d1;
				if (j1 >= s1) { j1 -= s1; qq++; }
				qq += dq;
			}
		}
		cp_async_wait_all();
		__syncthreads();
		for (int e = threadIdx.x; e < kn; e += PT_THREADS) {
			D v = rd ? dtile[e] : D();
			elem_op<D, S>::apply(op, &v, &mtile[q * pitch + i1 * ld + i0], al,
			    als, be, dre, dim_);
			if (op != XMGD_OP_DOT)
				dst[s_o[0][q] + i0 + i1 * ds1] = v;
			i0 += d0;
			if (i0 >= s0) { i0 -= s0; i1++; }
			i1 += d1;
			if (i1 >= s1) { i1 -= s1; q++; }
			q += dq;
		}
	} else {
		/* tile: dims 0 (dst unit stride) and 1 (src unit stride) */
		__shared__ S tile[TILE][TILE + 1];
		int64_t c0 = local % m.ctas_d0;
		int64_t rest = local / m.ctas_d0;
		int64_t c1 = rest % m.ctas_d1;
		int64_t o = rest / m.ctas_d1;
		int64_t od, os;
		outer_offsets(t, 2, o, od, os);
		int64_t b0 = c0 * TILE, b1 = c1 * TILE;
		int w0 = (int)(t.size[0] - b0 < TILE ? t.size[0] - b0 : TILE);
		int w1 = (int)(t.size[1] - b1 < TILE ? t.size[1] - b1 : TILE);
		/* load: consecutive threads walk dim 1 (source contiguous) */
		for (int e = threadIdx.x; e < TILE * TILE; e += PT_THREADS) {
			int i1 = e % TILE, i0 = e / TILE;
			if (i0 < w0 && i1 < w1)
				tile[i1][i0] = src[os + (b0 + i0) * t.src_stride[0] +
				    (b1 + i1)];
		}
		__syncthreads();
		/* store: consecutive threads walk dim 0 (destination contiguous) */
		for (int e = threadIdx.x; e < TILE * TILE; e += PT_THREADS) {
			int i0 = e % TILE, i1 = e / TILE;
			if (i0 < w0 && i1 < w1) {
				D *dp = dst + od + (b0 + i0) * t.dst_stride[0] +
				    (b1 + i1) * t.dst_stride[1];
				elem_op<D, S>::apply(op, dp, &tile[i1][i0], al, als, be,
				    dre, dim_);
			}
		}
	}
	if (op == XMGD_OP_DOT) {
		for (int off = 16; off > 0; off >>= 1) {
			dre += __shfl_down_sync(0xffffffffu, dre, off);
			dim_ += __shfl_down_sync(0xffffffffu, dim_, off);
		}
		if ((threadIdx.x & 31) == 0) {
			s_red[0][threadIdx.x >> 5] = dre;
			s_red[1][threadIdx.x >> 5] = dim_;
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			double a = 0, b = 0;
			for (int w = 0; w < PT_THREADS / 32; w++) {
				a += s_red[0][w];
				b += s_red[1][w];
			}
			partial[2 * cta] = a;
			partial[2 * cta + 1] = b;
		}
	}
}

/* a bounded wait of the slab schedule gave up (set on the device, read
 * and cleared by the host after the launches) */
__device__ int g_slab_err;

/*
 * Slab schedule: rows_per_cta consecutive s0 x s1 slices per CTA, each
 * contiguous on both sides (source: dim 1 unit stride, dim 0 stride s1;
 * destination: dim 0 unit stride, dim 1 stride s0; slice q at q * s0 * s1
 * on both), 16-byte aligned.  One bulk copy brings the CTA's slices of the
 * source into shared memory (one instruction, where the matrix schedule
 * issues a copy per element); the source goes into a tile with an odd row
 * pitch, so that both the transposing pass (threads along the source's
 * run) and the storing pass (threads along the destination's run) touch
 * distinct banks; stores follow the destination's run.
 */
template <typename T>
__global__ void __launch_bounds__(PT_THREADS, 6)
slab_kernel(const xmgd_ptask_t *__restrict__ tasks,
    const task_meta *__restrict__ meta, int ntasks, int64_t cta0)
{
	extern __shared__ __align__(16) unsigned char dsm[];
	__shared__ __align__(8) uint64_t bar;
	__shared__ int s_err;

	const int64_t cta = cta0 + blockIdx.x;
	int lo = 0, hi = ntasks - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (meta[mid].first_cta <= cta) lo = mid; else hi = mid - 1;
	}
	const xmgd_ptask_t &t = tasks[lo];
	const task_meta &m = meta[lo];
	const int s0 = (int)t.size[0], s1 = (int)t.size[1], n = s0 * s1;
	const int ld = s0 | 1;
	const int64_t o0 = (cta - m.first_cta) * m.rows_per_cta;
	const int k = (int)(m.nouter - o0 < m.rows_per_cta ? m.nouter - o0 :
	    m.rows_per_cta);
	const int kn = k * n;
	const uint32_t cbytes = (uint32_t)kn * (uint32_t)sizeof(T);
	const T *sb = reinterpret_cast<const T *>(dsm);
	T *tb = reinterpret_cast<T *>(dsm + cbytes);
	T *dst = reinterpret_cast<T *>(t.dst) + o0 * n;
	const T *src = reinterpret_cast<const T *>(t.src) + o0 * n;
	const T al = num<T>::mk(t.alpha);

	const uint32_t b = smem_u32(&bar);
	if (threadIdx.x == 0) {
		s_err = 0;
		mbar_init(b, 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		mbar_expect_tx(b, cbytes);
		bulk_g2s(smem_u32(dsm), src, cbytes, b);
	}
	const bool ok = mbar_wait(b, 0, &s_err, &g_slab_err, 1);
	/* every thread leaves together when the wait gave up */
	if (__syncthreads_or(!ok))
		return;
	/* source order e = q n + i0 s1 + i1 -> tile q s1 ld + i1 ld + i0 */
	{
		int q = threadIdx.x / n, r = threadIdx.x - q * n;
		int i0 = r / s1, i1 = r - i0 * s1;
		const int dq = PT_THREADS / n, dr = PT_THREADS - dq * n;
		const int d0 = dr / s1, d1 = dr - d0 * s1;
		for (int e = threadIdx.x; e < kn; e += PT_THREADS) {
			tb[(q * s1 + i1) * ld + i0] = sb[e];
			i1 += d1;
			if (i1 >= s1) { i1 -= s1; i0++; }
			i0 += d0;
			if (i0 >= s0) { i0 -= s0; q++; }
			q += dq;
		}
	}
	__syncthreads();
	/* destination order e = q n + i1 s0 + i0 */
	int q = threadIdx.x / n, r = threadIdx.x - q * n;
	int i1 = r / s0, i0 = r - i1 * s0;
	const int dq = PT_THREADS / n, dr = PT_THREADS - dq * n;
	const int d1 = dr / s0, d0 = dr - d1 * s0;
	for (int e = threadIdx.x; e < kn; e += PT_THREADS) {
		dst[e] = num<T>::mul(al, tb[(q * s1 + i1) * ld + i0]);
		i0 += d0;
		if (i0 >= s0) { i0 -= s0; i1++; }
		i1 += d1;
		if (i1 >= s1) { i1 -= s1; q++; }
		q += dq;
	}
}

/* the slab schedule for a task: slices per CTA (0 when the schedule does
 * not apply: xm_copy of one scalar type only; an op that reads the
 * destination ran slower with its second bulk copy, 0.69 of HBM against
 * the matrix schedule's 0.71), and the CTA's shared memory */
static int64_t
slab_shape(const xmgd_ptask_t &t, int dbytes, int sbytes, int mt,
    int64_t *smem)
{
	if (dbytes != sbytes || t.op != XMGD_OP_COPY || t.ndim < 2 || t.ndim > 3)
		return 0;
	const int64_t s0 = t.size[0], s1 = t.size[1], n = s0 * s1;
	if (s0 > mt || s1 > mt || s0 < 2 || s1 < 2 ||
	    t.dst_stride[0] != 1 || t.dst_stride[1] != s0 ||
	    t.src_stride[1] != 1 || t.src_stride[0] != s1 ||
	    (t.ndim == 3 && (t.dst_stride[2] != n || t.src_stride[2] != n)) ||
	    (n * sbytes) % 16 != 0 || ((t.dst | t.src) & 15) != 0)
		return 0;
	int64_t k = n * sbytes >= SLAB_CHUNK ? 1 : SLAB_CHUNK / (n * sbytes);
	const int64_t cap = t.ndim == 3 ? t.size[2] : 1;
	if (k > cap)
		k = cap;
	*smem = k * n * sbytes + k * s1 * (s0 | 1) * sbytes;
	return *smem <= SLAB_SMEM ? k : 0;
}

template <typename D, typename S>
static int
launch_slab(const xmgd_ptask_t *dtasks, const task_meta *dmeta, int ntasks,
    int64_t cta0, int64_t n, int64_t smem)
{
	if constexpr (std::is_same<D, S>::value) {
		static bool attr = false;
		if (!attr) {
			XMG_CK(cudaFuncSetAttribute(slab_kernel<D>,
			    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SLAB_SMEM));
			attr = true;
		}
		slab_kernel<D><<<(unsigned)n, PT_THREADS, (size_t)smem, stream()>>>(
		    dtasks, dmeta, ntasks, cta0);
		g_launches++;
		XMG_CK(cudaGetLastError());
		return XMG_OK;
	} else {
		return xmg_seterr(XMG_EINVAL, "slab schedule: scalar conversion");
	}
}

template <typename D, typename S>
static int
launch(const xmgd_ptask_t *dtasks, const task_meta *dmeta, int ntasks,
    const int64_t *begin, int64_t slab_smem, double *dpartial)
{
	if (begin[5] > begin[4]) {
		int st = launch_slab<D, S>(dtasks, dmeta, ntasks, begin[4],
		    begin[5] - begin[4], slab_smem);
		if (st)
			return st;
	}
	/* one launch per schedule, over that schedule's CTA range */
	for (int mode = 0; mode < 4; mode++) {
		const int64_t n = begin[mode + 1] - begin[mode];
		if (n <= 0)
			continue;
		switch (mode) {
		case 0: ptask_kernel<D, S, 0><<<(unsigned)n, PT_THREADS, 0, stream()>>>(
		    dtasks, dmeta, ntasks, begin[mode], dpartial); break;
		case 1: ptask_kernel<D, S, 1><<<(unsigned)n, PT_THREADS, 0, stream()>>>(
		    dtasks, dmeta, ntasks, begin[mode], dpartial); break;
		case 2: ptask_kernel<D, S, 2><<<(unsigned)n, PT_THREADS, 0, stream()>>>(
		    dtasks, dmeta, ntasks, begin[mode], dpartial); break;
		case 3: ptask_kernel<D, S, 3><<<(unsigned)n, PT_THREADS, 0, stream()>>>(
		    dtasks, dmeta, ntasks, begin[mode], dpartial); break;
		}
		g_launches++;
		XMG_CK(cudaGetLastError());
	}
	return XMG_OK;
}

static int
elem_bytes(int type)
{
	return type == 0 ? 4 : type == 3 ? 16 : 8;	/* float, cd; double, cf */
}

/*
 * Schedule of every task of a batch.  Tasks are grouped by schedule (stable
 * within a group, order[] maps group position -> caller's index) so that
 * each schedule owns one contiguous CTA range [begin[m], begin[m+1]); meta
 * and the task copy follow the grouped order.
 */
static void
plan_tasks(const xmgd_ptask_t *tasks, int ntasks, int dtype, int stype,
    std::vector<xmgd_ptask_t> &sorted, std::vector<task_meta> &meta,
    std::vector<int> &order, int64_t begin[6], int64_t *slab_smem)
{
	std::vector<task_meta> m0((size_t)ntasks);
	std::vector<int64_t> cnt((size_t)ntasks);
	const int mt = mt_host(elem_bytes(dtype), elem_bytes(stype));
	const char *e = getenv("XMG_PTASK_SLAB");
	const bool slab_on = !(e && strcmp(e, "0") == 0);

	/* the slab launch's shared memory: the largest of its CTAs' */
	*slab_smem = 0;
	for (int i = 0; i < ntasks; i++) {
		const xmgd_ptask_t &t = tasks[i];
		task_meta &m = m0[i];
		memset(&m, 0, sizeof m);
		int64_t need = 0;
		const int64_t k = slab_on ? slab_shape(t, elem_bytes(dtype),
		    elem_bytes(stype), mt, &need) : 0;
		if (k > 0) {
			m.mode = 4;
			m.nouter = t.ndim == 3 ? t.size[2] : 1;
			m.rows_per_cta = (int32_t)k;
			m.ctas_d0 = 1;
			cnt[i] = (m.nouter + k - 1) / k;
			*slab_smem = std::max(*slab_smem, need);
			continue;
		}
		const bool nosrc = t.op == XMGD_OP_SET || t.op == XMGD_OP_SCALE;
		const bool tile = t.ndim >= 2 && t.src_stride[1] == 1 &&
		    t.src_stride[0] != 1 && !nosrc;
		const bool flat = t.ndim == 1 && t.dst_stride[0] == 1 &&
		    (nosrc || t.src_stride[0] == 1);
		const bool mat = tile && t.dst_stride[0] == 1 && t.size[0] <= mt &&
		    t.size[1] <= mt;
		if (flat) {
			m.mode = 2;
			m.ctas_d0 = (int32_t)((t.size[0] + FLAT_ELEMS - 1) / FLAT_ELEMS);
			m.nouter = 1;
			m.rows_per_cta = 1;
			cnt[i] = m.ctas_d0;
		} else if (mat) {
			m.mode = 3;
			m.nouter = 1;
			for (int d = 2; d < t.ndim; d++)
				m.nouter *= t.size[d];
			/* as many slices as the shared tile holds (pitch s0 + 1) */
			const int64_t per = t.size[1] * (t.size[0] + 1);
			int64_t q = (int64_t)mt * (mt + 1) / per;
			m.rows_per_cta = (int32_t)(q < 1 ? 1 : q > MAT_MAXQ ? MAT_MAXQ : q);
			m.ctas_d0 = 1;
			cnt[i] = (m.nouter + m.rows_per_cta - 1) / m.rows_per_cta;
		} else if (tile) {
			m.mode = 1;
			m.ctas_d0 = (t.size[0] + TILE - 1) / TILE;
			m.ctas_d1 = (t.size[1] + TILE - 1) / TILE;
			m.nouter = 1;
			for (int d = 2; d < t.ndim; d++)
				m.nouter *= t.size[d];
			cnt[i] = (int64_t)m.ctas_d0 * m.ctas_d1 * m.nouter;
		} else {
			m.mode = 0;
			m.ctas_d0 = (t.size[0] + ROW_ELEMS - 1) / ROW_ELEMS;
			m.nouter = 1;
			for (int d = 1; d < t.ndim; d++)
				m.nouter *= t.size[d];
			int64_t rows = t.size[0] >= ROW_ELEMS ? 1 :
			    ROW_ELEMS / t.size[0];
			if (rows > PT_THREADS)
				rows = PT_THREADS;
			m.rows_per_cta = (int32_t)rows;
			cnt[i] = (int64_t)m.ctas_d0 * ((m.nouter + rows - 1) / rows);
		}
	}
	sorted.clear();
	meta.clear();
	order.clear();
	int64_t n = 0;
	for (int mode = 0; mode < 5; mode++) {
		begin[mode] = n;
		for (int i = 0; i < ntasks; i++)
			if (m0[i].mode == mode) {
				task_meta m = m0[i];
				m.first_cta = n;
				n += cnt[i];
				sorted.push_back(tasks[i]);
				meta.push_back(m);
				order.push_back(i);
			}
	}
	begin[5] = n;
}

static int
launch_types(int dtype, int stype, const xmgd_ptask_t *dt, const task_meta *dm,
    int ntasks, const int64_t *begin, int64_t slab_smem, double *dp)
{
	int st;

#define L(D, S) st = launch<D, S>(dt, dm, ntasks, begin, slab_smem, dp)
	if (dtype == stype) {
		switch (dtype) {
		case 0: L(float, float); break;
		case 1: L(cf, cf); break;
		case 2: L(double, double); break;
		case 3: L(cd, cd); break;
		default: st = xmg_seterr(XMG_EINVAL, "bad scalar type");
		}
	} else if (dtype == 2 && stype == 0) L(double, float);
	else if (dtype == 0 && stype == 2) L(float, double);
	else if (dtype == 3 && stype == 1) L(cd, cf);
	else if (dtype == 1 && stype == 3) L(cf, cd);
	else st = xmg_seterr(XMG_EINVAL, "unsupported scalar conversion");
#undef L
	return st;
}

static size_t
task_bytes(int ntasks)
{
	return ((size_t)ntasks * sizeof(xmgd_ptask_t) + 255) & ~(size_t)255;
}

} /* namespace xmg */

using namespace xmg;

extern "C" int
xmgd_ptask_stage(const xmgd_ptask_t *tasks, int ntasks, int stype,
    xmgd_ptask_batch_t *b)
{
	std::vector<xmgd_ptask_t> sorted;
	std::vector<task_meta> meta;
	std::vector<int> order;
	const size_t tb = task_bytes(ntasks);
	int st;

	memset(b, 0, sizeof *b);
	if (ntasks <= 0)
		return XMG_OK;
	/* batches staged for replay carry one type on both sides */
	plan_tasks(tasks, ntasks, stype, stype, sorted, meta, order, b->begin,
	    &b->slab_smem);
	if ((st = xmgd_alloc(tb + meta.size() * sizeof(task_meta), &b->dbuf)))
		return st;
	b->ntasks = ntasks;
	XMG_CK(cudaMemcpyAsync((void *)b->dbuf, sorted.data(), (size_t)ntasks *
	    sizeof(xmgd_ptask_t), cudaMemcpyHostToDevice, stream()));
	XMG_CK(cudaMemcpyAsync((void *)(b->dbuf + tb), meta.data(), meta.size() *
	    sizeof(task_meta), cudaMemcpyHostToDevice, stream()));
	/* the host copies are local: finish before returning */
	XMG_CK(cudaStreamSynchronize(stream()));
	return XMG_OK;
}

extern "C" int
xmgd_ptask_launch(int dtype, int stype, const xmgd_ptask_batch_t *b)
{
	if (b->ntasks <= 0)
		return XMG_OK;
	return launch_types(dtype, stype, (const xmgd_ptask_t *)b->dbuf,
	    (const task_meta *)(b->dbuf + task_bytes(b->ntasks)), b->ntasks,
	    b->begin, b->slab_smem, nullptr);
}

extern "C" int
xmgd_ptasks(int dtype, int stype, const xmgd_ptask_t *tasks, int ntasks,
    double *dots)
{
	std::vector<xmgd_ptask_t> sorted;
	std::vector<task_meta> meta;
	std::vector<int> order;
	int64_t begin[6], nctas, slab_smem;
	uint64_t dbuf, dpart = 0;
	size_t tb, mb;
	int st;

	if (ntasks <= 0)
		return XMG_OK;
	plan_tasks(tasks, ntasks, dtype, stype, sorted, meta, order, begin,
	    &slab_smem);
	nctas = begin[5];
	tb = task_bytes(ntasks);
	mb = (size_t)ntasks * sizeof(task_meta);
	if ((st = xmgd_scratch(2, tb + mb, &dbuf)) != XMG_OK)
		return st;
	XMG_CK(cudaMemcpyAsync((void *)dbuf, sorted.data(), (size_t)ntasks *
	    sizeof(xmgd_ptask_t), cudaMemcpyHostToDevice, stream()));
	XMG_CK(cudaMemcpyAsync((void *)(dbuf + tb), meta.data(), mb,
	    cudaMemcpyHostToDevice, stream()));
	if (dots && (st = xmgd_scratch(3, (size_t)nctas * 2 * sizeof(double),
	    &dpart)) != XMG_OK)
		return st;
	if ((st = launch_types(dtype, stype, (const xmgd_ptask_t *)dbuf,
	    (const task_meta *)(dbuf + tb), ntasks, begin, slab_smem,
	    (double *)dpart)))
		return st;
	/* the task buffers are reused by the next batch: wait here */
	if ((st = check(cudaStreamSynchronize(stream()), "ptask_kernel")))
		return st;
	if (begin[5] > begin[4]) {
		int err = 0;
		XMG_CK(cudaMemcpyFromSymbol(&err, g_slab_err, sizeof err));
		if (err) {
			const int zero = 0;
			XMG_CK(cudaMemcpyToSymbol(g_slab_err, &zero, sizeof zero));
			return xmg_seterr(XMG_ETIMEOUT, "slab schedule: a bulk copy "
			    "did not complete within the bounded wait");
		}
	}
	if (dots) {
		std::vector<double> h((size_t)nctas * 2);
		if ((st = xmgd_d2h(h.data(), dpart, h.size() * sizeof(double))))
			return st;
		for (int j = 0; j < ntasks; j++) {
			const int64_t e = j + 1 < ntasks ? meta[j + 1].first_cta : nctas;
			double a = 0, b = 0;
			for (int64_t c = meta[j].first_cta; c < e; c++) {
				a += h[2 * c];
				b += h[2 * c + 1];
			}
			dots[2 * order[j]] = a;
			dots[2 * order[j] + 1] = b;
		}
	}
	return XMG_OK;
}
