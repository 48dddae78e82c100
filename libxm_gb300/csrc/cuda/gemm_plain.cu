/*
 * Plain grouped block-pair GEMM of libxm-gb300 (the FP64 form, and the
 * float / complex forms on the CUDA cores).
 *
 * One launch computes every canonical output block assigned to it:
 *     C = beta * C + sum_p al_p * A_p^T B_p
 * over the block's merged pairs (contract.c:193-218 issues one host BLAS
 * call per pair instead).  The unfold of A_p, B_p and the fold of C are
 * not separate passes: tile loads gather through the per-operand offset
 * tables (element (k, i) of A_p at a_ptr + arow[k] + acol[i]) and the
 * epilogue scatters C the same way, so operands are read once from their
 * canonical storage and C is written once.
 *
 * Tile 64 x 64, K step 16, 256 threads, 4 x 4 accumulators per thread in
 * registers.  Work items (block, m-tile, n-tile) arrive sorted by cost.
 */
#include "common.cuh"

namespace xmg {

constexpr int PG_BM = 64, PG_BN = 64, PG_BK = 16, PG_THREADS = 256;

struct pg_item {
	int32_t cblock, m0, n0, pad;
};

template <typename T>
__device__ inline void
load_tile(T (*S)[PG_BM + 1], const T *__restrict__ base,
    const int32_t *__restrict__ rowt, const int32_t *__restrict__ colt,
    int k0, int kmax, int c0, int cmax, bool kfast, const T &scale)
{
	int t = threadIdx.x;
	if (kfast) {
		/* consecutive threads walk k: contiguous when rows are unit-stride */
		int kk = t % PG_BK, cc = t / PG_BK;
		int k = k0 + kk;
		int32_t ro = k < kmax ? rowt[k] : 0;
#pragma unroll
		for (int r = 0; r < PG_BM / (PG_THREADS / PG_BK); r++) {
			int c = c0 + cc + r * (PG_THREADS / PG_BK);
			T v = num<T>::zero();
			if (k < kmax && c < cmax)
				v = num<T>::mul(scale, base[ro + colt[c]]);
			S[kk][cc + r * (PG_THREADS / PG_BK)] = v;
		}
	} else {
		int cc = t % PG_BM, kk = t / PG_BM;
		int c = c0 + cc;
		int32_t co = c < cmax ? colt[c] : 0;
#pragma unroll
		for (int r = 0; r < PG_BK / (PG_THREADS / PG_BM); r++) {
			int k = k0 + kk + r * (PG_THREADS / PG_BM);
			T v = num<T>::zero();
			if (k < kmax && c < cmax)
				v = num<T>::mul(scale, base[rowt[k] + co]);
			S[kk + r * (PG_THREADS / PG_BM)][cc] = v;
		}
	}
}

template <typename T>
__global__ void __launch_bounds__(PG_THREADS)
plain_gemm_kernel(const pg_item *__restrict__ items,
    const xmgd_cblock_t *__restrict__ cbs, const xmgd_pair_t *__restrict__ prs,
    const int32_t *__restrict__ tabs, double2 beta2)
{
	__shared__ T As[PG_BK][PG_BM + 1];
	__shared__ T Bs[PG_BK][PG_BN + 1];

	const pg_item it = items[blockIdx.x];
	const xmgd_cblock_t cb = cbs[it.cblock];
	const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
	T acc[4][4];
#pragma unroll
	for (int i = 0; i < 4; i++)
#pragma unroll
		for (int j = 0; j < 4; j++)
			acc[i][j] = num<T>::zero();
	const T one = num<T>::mk((const double[2]){1.0, 0.0});

	for (int p = 0; p < cb.npairs; p++) {
		const xmgd_pair_t pr = prs[cb.first_pair + p];
		const T *A = reinterpret_cast<const T *>(pr.a_ptr);
		const T *B = reinterpret_cast<const T *>(pr.b_ptr);
		const int32_t *arow = tabs + pr.arow, *acol = tabs + pr.acol;
		const int32_t *brow = tabs + pr.brow, *bcol = tabs + pr.bcol;
		const bool akf = pr.k > 1 && arow[1] - arow[0] == 1;
		const bool bkf = pr.k > 1 && brow[1] - brow[0] == 1;
		const T al = num<T>::mk(pr.al);
		for (int k0 = 0; k0 < pr.k; k0 += PG_BK) {
			__syncthreads();
			load_tile<T>(As, A, arow, acol, k0, pr.k, it.m0, cb.m, akf, al);
			load_tile<T>(Bs, B, brow, bcol, k0, pr.k, it.n0, cb.n, bkf, one);
			__syncthreads();
#pragma unroll
			for (int kk = 0; kk < PG_BK; kk++) {
				T a[4], b[4];
#pragma unroll
				for (int i = 0; i < 4; i++)
					a[i] = As[kk][tx + 16 * i];
#pragma unroll
				for (int j = 0; j < 4; j++)
					b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
				for (int i = 0; i < 4; i++)
#pragma unroll
					for (int j = 0; j < 4; j++)
						acc[i][j] = num<T>::fma(a[i], b[j], acc[i][j]);
			}
		}
	}
	/* fused fold: C = beta * C + acc, scattered through the C tables;
	 * beta == 0 never reads C (contract.c:155-156) */
	T *C = reinterpret_cast<T *>(cb.c_ptr);
	const int32_t *crow = tabs + cb.crow, *ccol = tabs + cb.ccol;
	const double bb[2] = {beta2.x, beta2.y};
	const T beta = num<T>::mk(bb);
	const bool bzero = beta2.x == 0 && beta2.y == 0;
#pragma unroll
	for (int j = 0; j < 4; j++) {
		int n = it.n0 + ty + 16 * j;
		if (n >= cb.n)
			continue;
		int32_t co = ccol[n];
#pragma unroll
		for (int i = 0; i < 4; i++) {
			int m = it.m0 + tx + 16 * i;
			if (m >= cb.m)
				continue;
			T *cp = C + crow[m] + co;
			*cp = bzero ? acc[i][j] : num<T>::fma(beta, *cp, acc[i][j]);
		}
	}
}

template <typename T>
int
plain_gemm_launch(const void *items, int nitems, const xmgd_cblock_t *cbs,
    const xmgd_pair_t *prs, const int32_t *tabs, const double *beta)
{
	if (nitems == 0)
		return XMG_OK;
	plain_gemm_kernel<T><<<nitems, PG_THREADS, 0, stream()>>>(
	    (const pg_item *)items, cbs, prs, tabs, make_double2(beta[0], beta[1]));
	g_launches++;
	return check(cudaGetLastError(), "plain_gemm_kernel launch");
}

template int plain_gemm_launch<float>(const void *, int, const xmgd_cblock_t *,
    const xmgd_pair_t *, const int32_t *, const double *);
template int plain_gemm_launch<double>(const void *, int, const xmgd_cblock_t *,
    const xmgd_pair_t *, const int32_t *, const double *);
template int plain_gemm_launch<cf>(const void *, int, const xmgd_cblock_t *,
    const xmgd_pair_t *, const int32_t *, const double *);
template int plain_gemm_launch<cd>(const void *, int, const xmgd_cblock_t *,
    const xmgd_pair_t *, const int32_t *, const double *);

} /* namespace xmg */
