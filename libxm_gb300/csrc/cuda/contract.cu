/*
 * Device side of xm_contract: uploads the host plan, routes each canonical
 * output block to the split-precision tensor-core path or the plain path,
 * and times the phases with events on the engine stream.
 */
#include <algorithm>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"

namespace xmg {

template <typename T>
int plain_gemm_launch(const void *items, int nitems, const xmgd_cblock_t *cbs,
    const xmgd_pair_t *prs, const int32_t *tabs, const double *beta);

/* split-precision path (emu.cu); returns XMG_ENOTSUP when unavailable */
int emu_contract(xmgd_contract_t *plan, const std::vector<int> &cblocks,
    const xmgd_cblock_t *d_cbs, const xmgd_pair_t *d_prs,
    const int32_t *d_tabs, xmgd_timing_t *tm);

static xmgd_timing_t g_timing;

struct pg_item { int32_t cblock, m0, n0, pad; };

static int
upload(int slot, const void *h, size_t bytes, uint64_t *d)
{
	int st;

	if (bytes == 0) {
		*d = 0;
		return XMG_OK;
	}
	if ((st = xmgd_scratch(slot, bytes, d)) != XMG_OK)
		return st;
	return check(cudaMemcpyAsync((void *)*d, h, bytes,
	    cudaMemcpyHostToDevice, stream()), "plan upload");
}

} /* namespace xmg */

using namespace xmg;

extern "C" void
xmgd_last_timing(xmgd_timing_t *t)
{
	*t = g_timing;
}

extern "C" int
xmgd_contract(xmgd_contract_t *p)
{
	uint64_t d_cbs, d_prs, d_tabs, d_items;
	std::vector<int> emu, plain;
	std::vector<pg_item> items;
	std::vector<xmgd_ptask_t> scale;
	cudaEvent_t e0, e1;
	int st;
	float ms = 0;

	memset(&g_timing, 0, sizeof g_timing);
	p->precision_used = XMG_PREC_FP64;
	XMG_CK(cudaEventCreate(&e0));
	XMG_CK(cudaEventCreate(&e1));
	XMG_CK(cudaEventRecord(e0, stream()));

	if ((st = upload(4, p->cblocks, (size_t)p->ncblocks * sizeof(xmgd_cblock_t),
	    &d_cbs)) || (st = upload(5, p->pairs, (size_t)p->npairs *
	    sizeof(xmgd_pair_t), &d_prs)) || (st = upload(6, p->tabs,
	    (size_t)p->ntabs * sizeof(int32_t), &d_tabs)))
		goto out;

	/* route the output blocks */
	for (int i = 0; i < p->ncblocks; i++) {
		const xmgd_cblock_t &cb = p->cblocks[i];
		if (cb.npairs == 0) {
			bool bzero = p->beta[0] == 0 && p->beta[1] == 0;
			bool bone = p->beta[0] == 1 && p->beta[1] == 0;
			if (bone)
				continue;
			xmgd_ptask_t t;
			memset(&t, 0, sizeof t);
			t.op = bzero ? XMGD_OP_SET : XMGD_OP_SCALE;
			t.alpha[0] = bzero ? 0 : p->beta[0];
			t.alpha[1] = bzero ? 0 : p->beta[1];
			t.dst = cb.c_ptr;
			t.ndim = 1;
			t.size[0] = cb.m * cb.n;
			for (int d = 1; d < 8; d++) t.size[d] = 1;
			t.dst_stride[0] = 1;
			scale.push_back(t);
			continue;
		}
		bool want_emu = p->precision != XMG_PREC_FP64 &&
		    p->emulatable[i];
		(want_emu ? emu : plain).push_back(i);
	}
	if (!scale.empty() && (st = xmgd_ptasks(p->dtype, p->dtype,
	    scale.data(), (int)scale.size(), nullptr)))
		goto out;

	if (!emu.empty()) {
		st = emu_contract(p, emu, (const xmgd_cblock_t *)d_cbs,
		    (const xmgd_pair_t *)d_prs, (const int32_t *)d_tabs,
		    &g_timing);
		if (st == XMG_ENOTSUP && p->precision == XMG_PREC_AUTO) {
			plain.insert(plain.end(), emu.begin(), emu.end());
			st = XMG_OK;
		} else if (st != XMG_OK)
			goto out;
		else
			p->precision_used = XMG_PREC_EMU64;
	}

	if (!plain.empty()) {
		for (int ci : plain) {
			const xmgd_cblock_t &cb = p->cblocks[ci];
			for (int m0 = 0; m0 < cb.m; m0 += 64)
				for (int n0 = 0; n0 < cb.n; n0 += 64)
					items.push_back(pg_item{ci, m0, n0, 0});
		}
		/* longest work first: cost ~ total K of the block */
		std::vector<int64_t> cost(p->ncblocks, 0);
		for (int ci : plain) {
			const xmgd_cblock_t &cb = p->cblocks[ci];
			for (int q = 0; q < cb.npairs; q++)
				cost[ci] += p->pairs[cb.first_pair + q].k;
		}
		std::stable_sort(items.begin(), items.end(),
		    [&](const pg_item &x, const pg_item &y) {
			return cost[x.cblock] > cost[y.cblock]; });
		if ((st = upload(7, items.data(), items.size() * sizeof(pg_item),
		    &d_items)))
			goto out;
		cudaEvent_t g0, g1;
		XMG_CK(cudaEventCreate(&g0));
		XMG_CK(cudaEventCreate(&g1));
		XMG_CK(cudaEventRecord(g0, stream()));
		const xmgd_cblock_t *dc = (const xmgd_cblock_t *)d_cbs;
		const xmgd_pair_t *dp = (const xmgd_pair_t *)d_prs;
		const int32_t *dt = (const int32_t *)d_tabs;
		const void *di = (const void *)d_items;
		int n = (int)items.size();
		switch (p->dtype) {
		case 0: st = plain_gemm_launch<float>(di, n, dc, dp, dt, p->beta); break;
		case 1: st = plain_gemm_launch<cf>(di, n, dc, dp, dt, p->beta); break;
		case 2: st = plain_gemm_launch<double>(di, n, dc, dp, dt, p->beta); break;
		case 3: st = plain_gemm_launch<cd>(di, n, dc, dp, dt, p->beta); break;
		}
		XMG_CK(cudaEventRecord(g1, stream()));
		if (st == XMG_OK) {
			XMG_CK(cudaEventSynchronize(g1));
			XMG_CK(cudaEventElapsedTime(&ms, g0, g1));
			g_timing.ms_gemm += ms;
			g_timing.gemm_launches += 1;
			g_timing.gemm_items += n;
		}
		cudaEventDestroy(g0);
		cudaEventDestroy(g1);
		if (st != XMG_OK)
			goto out;
	}
	XMG_CK(cudaEventRecord(e1, stream()));
	XMG_CK(cudaEventSynchronize(e1));
	XMG_CK(cudaEventElapsedTime(&ms, e0, e1));
	g_timing.ms_total = ms;
	st = check(cudaGetLastError(), "contraction kernels");
out:
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (st == XMG_OK)
		st = xmgd_sync();
	return st;
}
