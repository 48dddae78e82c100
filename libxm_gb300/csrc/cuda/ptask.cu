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
 * Two schedules, chosen per task on the host (xmg_ptask_shape):
 *  - row mode: dimension 0 is unit-stride on the destination side; a CTA
 *    covers ROW_ELEMS elements along dim 0 for as many outer rows as fit,
 *    with per-row outer offsets precomputed in shared memory;
 *  - tile mode: the source's unit-stride dimension is dim 1; a CTA moves a
 *    TILE x TILE tile through padded shared memory so that loads are
 *    coalesced along dim 1 and stores along dim 0 (gather-transpose).
 */
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"

namespace xmg {

constexpr int PT_THREADS = 256;
constexpr int ROW_ELEMS = 1024;    /* elements per CTA in row mode */
constexpr int TILE = 32;

struct task_meta {
	int64_t first_cta;
	int32_t mode;          /* 0 row, 1 tile */
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

template <typename D, typename S>
__global__ void __launch_bounds__(PT_THREADS)
ptask_kernel(const xmgd_ptask_t *__restrict__ tasks,
    const task_meta *__restrict__ meta, int ntasks, double *__restrict__ partial)
{
	__shared__ int64_t s_od[PT_THREADS], s_os[PT_THREADS];
	__shared__ __align__(16) char s_tile_raw[TILE * (TILE + 1) * sizeof(S)];
	__shared__ double s_red[2][PT_THREADS / 32];
	S (*tile)[TILE + 1] = reinterpret_cast<S (*)[TILE + 1]>(s_tile_raw);

	/* locate the task of this CTA (binary search over first_cta) */
	int64_t cta = blockIdx.x;
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

	if (m.mode == 0) {
		/* row mode */
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
		int64_t n = w0 * rows;
		int64_t ds0 = t.dst_stride[0], ss0 = t.src_stride[0];
		for (int64_t e = threadIdx.x; e < n; e += PT_THREADS) {
			int r = (int)(e / w0);
			int64_t i0 = i0beg + (e - (int64_t)r * w0);
			D *dp = dst + s_od[r] + i0 * ds0;
			const S *sp = src + s_os[r] + i0 * ss0;
			elem_op<D, S>::apply(op, dp, sp, al, als, be, dre, dim_);
		}
	} else {
		/* tile mode: dims 0 (dst unit stride) and 1 (src unit stride) */
		int64_t c0 = local % m.ctas_d0;
		int64_t rest = local / m.ctas_d0;
		int64_t c1 = rest % m.ctas_d1;
		int64_t o = rest / m.ctas_d1;
		int64_t od, os;
		outer_offsets(t, 2, o, od, os);
		int64_t b0 = c0 * TILE, b1 = c1 * TILE;
		int w0 = (int)(t.size[0] - b0 < TILE ? t.size[0] - b0 : TILE);
		int w1 = (int)(t.size[1] - b1 < TILE ? t.size[1] - b1 : TILE);
		const bool need_src = op != XMGD_OP_SET && op != XMGD_OP_SCALE;
		if (need_src) {
			/* load: consecutive threads walk dim 1 (source contiguous) */
			for (int e = threadIdx.x; e < TILE * TILE; e += PT_THREADS) {
				int i1 = e % TILE, i0 = e / TILE;
				if (i0 < w0 && i1 < w1)
					tile[i1][i0] = src[os + (b0 + i0) * t.src_stride[0] +
					    (b1 + i1)];
			}
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

template <typename D, typename S>
static int
launch(const xmgd_ptask_t *dtasks, const task_meta *dmeta, int ntasks,
    int64_t nctas, double *dpartial)
{
	/* grid.x limit is 2^31-1; batches are far smaller */
	ptask_kernel<D, S><<<(unsigned)nctas, PT_THREADS, 0, stream()>>>(
	    dtasks, dmeta, ntasks, dpartial);
	g_launches++;
	return check(cudaGetLastError(), "ptask_kernel launch");
}

/* CTA schedule of every task of a batch; returns the grid size */
static int64_t
plan_tasks(const xmgd_ptask_t *tasks, int ntasks, task_meta *meta)
{
	int64_t nctas = 0;

	for (int i = 0; i < ntasks; i++) {
		const xmgd_ptask_t &t = tasks[i];
		task_meta &m = meta[i];
		m.first_cta = nctas;
		bool tile = t.ndim >= 2 && t.src_stride[1] == 1 &&
		    t.src_stride[0] != 1 && t.op != XMGD_OP_SET &&
		    t.op != XMGD_OP_SCALE;
		if (tile) {
			m.mode = 1;
			m.ctas_d0 = (t.size[0] + TILE - 1) / TILE;
			m.ctas_d1 = (t.size[1] + TILE - 1) / TILE;
			m.nouter = 1;
			for (int d = 2; d < t.ndim; d++)
				m.nouter *= t.size[d];
			nctas += (int64_t)m.ctas_d0 * m.ctas_d1 * m.nouter;
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
			nctas += (int64_t)m.ctas_d0 *
			    ((m.nouter + rows - 1) / rows);
		}
	}
	return nctas;
}

static int
launch_types(int dtype, int stype, const xmgd_ptask_t *dt, const task_meta *dm,
    int ntasks, int64_t nctas, double *dp)
{
	int st;

#define L(D, S) st = launch<D, S>(dt, dm, ntasks, nctas, dp)
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
xmgd_ptask_stage(const xmgd_ptask_t *tasks, int ntasks, uint64_t *dbuf,
    int64_t *nctas)
{
	std::vector<task_meta> meta((size_t)ntasks);
	const size_t tb = task_bytes(ntasks);
	int st;

	*dbuf = 0;
	*nctas = plan_tasks(tasks, ntasks, meta.data());
	if ((st = xmgd_alloc(tb + meta.size() * sizeof(task_meta), dbuf)))
		return st;
	XMG_CK(cudaMemcpyAsync((void *)*dbuf, tasks, (size_t)ntasks *
	    sizeof(xmgd_ptask_t), cudaMemcpyHostToDevice, stream()));
	XMG_CK(cudaMemcpyAsync((void *)(*dbuf + tb), meta.data(), meta.size() *
	    sizeof(task_meta), cudaMemcpyHostToDevice, stream()));
	/* the host copies are the caller's: finish before returning */
	XMG_CK(cudaStreamSynchronize(stream()));
	return XMG_OK;
}

extern "C" int
xmgd_ptask_launch(int dtype, int stype, uint64_t dbuf, int ntasks,
    int64_t nctas)
{
	if (ntasks <= 0)
		return XMG_OK;
	return launch_types(dtype, stype, (const xmgd_ptask_t *)dbuf,
	    (const task_meta *)(dbuf + task_bytes(ntasks)), ntasks, nctas,
	    nullptr);
}

extern "C" int
xmgd_ptasks(int dtype, int stype, const xmgd_ptask_t *tasks, int ntasks,
    double *dots)
{
	task_meta *meta;
	int64_t nctas = 0;
	uint64_t dbuf, dpart = 0;
	size_t tb, mb, k;
	int st, has_dot = dots != nullptr;

	if (ntasks <= 0)
		return XMG_OK;
	if ((meta = (task_meta *)calloc((size_t)ntasks, sizeof *meta)) == NULL)
		return xmg_seterr(XMG_ENOMEM, "out of memory");
	nctas = plan_tasks(tasks, ntasks, meta);
	tb = (size_t)ntasks * sizeof(xmgd_ptask_t);
	mb = (size_t)ntasks * sizeof(task_meta);
	tb = (tb + 255) & ~(size_t)255;
	if ((st = xmgd_scratch(2, tb + mb, &dbuf)) != XMG_OK)
		goto out;
	if ((st = check(cudaMemcpyAsync((void *)dbuf, tasks, (size_t)ntasks *
	    sizeof(xmgd_ptask_t), cudaMemcpyHostToDevice, stream()),
	    "task upload")) != XMG_OK)
		goto out;
	if ((st = check(cudaMemcpyAsync((void *)(dbuf + tb), meta, mb,
	    cudaMemcpyHostToDevice, stream()), "task upload")) != XMG_OK)
		goto out;
	if (has_dot && (st = xmgd_scratch(3, (size_t)nctas * 2 *
	    sizeof(double), &dpart)) != XMG_OK)
		goto out;
	st = launch_types(dtype, stype, (const xmgd_ptask_t *)dbuf,
	    (const task_meta *)(dbuf + tb), ntasks, nctas, (double *)dpart);
	if (st != XMG_OK)
		goto out;
	/* the task buffers are reused by the next batch: wait here */
	if ((st = check(cudaStreamSynchronize(stream()), "ptask_kernel")) !=
	    XMG_OK)
		goto out;
	if (has_dot) {
		double *h = (double *)malloc((size_t)nctas * 2 * sizeof(double));
		if (h == NULL) {
			st = xmg_seterr(XMG_ENOMEM, "out of memory");
			goto out;
		}
		st = xmgd_d2h(h, dpart, (size_t)nctas * 2 * sizeof(double));
		for (k = 0; st == XMG_OK && k < (size_t)ntasks; k++) {
			int64_t e = k + 1 < (size_t)ntasks ? meta[k + 1].first_cta :
			    nctas;
			double a = 0, b = 0;
			for (int64_t c = meta[k].first_cta; c < e; c++) {
				a += h[2 * c];
				b += h[2 * c + 1];
			}
			dots[2 * k] = a;
			dots[2 * k + 1] = b;
		}
		free(h);
	}
out:
	free(meta);
	return st;
}
