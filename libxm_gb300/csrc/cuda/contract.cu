/*
 * Device side of xm_contract: a reusable device plan per contraction.
 *
 * xmgd_plan_create uploads the host plan once (output blocks, pairs, the
 * offset-table pool), routes every canonical output block to the split-
 * precision tensor-core path or the plain path, and stages the work lists.
 * xmgd_plan_run replays the whole launch sequence -- beta-only blocks,
 * exponent and split kernels, the persistent grouped GEMM, the plain GEMM
 * -- as one CUDA graph captured on first use (one graph per autotuner
 * candidate while tuning), then reads the device flags once.  Operands with
 * Inf/NaN make the split-precision GEMM write nothing; those blocks are then
 * recomputed on the plain FP64 path (AUTO) or reported (EMU64).
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

/* split-precision path (emu.cu) */
struct emu_plan;
int emu_prepare(const xmgd_contract_t *p, const std::vector<int> &cblocks,
    const xmgd_cblock_t *d_cbs, const xmgd_pair_t *d_prs,
    const int32_t *d_tabs, emu_plan **out);
int emu_bind(emu_plan *e, bool *moved);
int emu_record_split(emu_plan *e);
int emu_record_gemm(emu_plan *e);
int emu_finish(emu_plan *e, float gemm_ms, int *nan);
int64_t emu_slice_bytes(const emu_plan *e);
int emu_items(const emu_plan *e);
int emu_policy(const emu_plan *e);
int emu_current(const emu_plan *e);
int emu_ncand(const emu_plan *e);
bool emu_tuned(const emu_plan *e);
int emu_a_mode(const emu_plan *e);
void emu_free(emu_plan *e);

static xmgd_timing_t g_timing;

struct pg_item { int32_t cblock, m0, n0, pad; };

struct segment {
	cudaGraphExec_t x = nullptr;
	long long launches = 0;      /* kernels per replay */
};

static bool
graphs_enabled()
{
	const char *e = getenv("XMG_GRAPHS");
	return !(e && strcmp(e, "0") == 0);
}

} /* namespace xmg */

using namespace xmg;

struct xmgd_plan {
	int dtype, precision;
	bool one_shot;                       /* launched directly, once */
	double alpha[2], beta[2];
	std::vector<xmgd_cblock_t> cbs;      /* host copies, for the fallback */
	std::vector<xmgd_pair_t> prs;
	std::vector<int> emu, plain;
	uint64_t d_cbs = 0, d_prs = 0, d_tabs = 0;
	xmgd_ptask_batch_t scale = {};       /* staged beta-only tasks */
	int n_scale = 0;
	uint64_t d_pg = 0;                   /* plain GEMM work list */
	int n_pg = 0;
	emu_plan *ep = nullptr;
	/* three captured segments, timed by events recorded between their
	 * launches: 0 beta-only blocks + operand split, 1 split-precision
	 * GEMM (one graph per autotuner candidate), 2 plain GEMM */
	segment seg0, seg2;
	std::vector<segment> seg1;
	cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
};

extern "C" void
xmgd_last_timing(xmgd_timing_t *t)
{
	*t = g_timing;
}

/* plain work list of a set of blocks: 64 x 64 tiles, longest K first */
static int
stage_plain(const std::vector<xmgd_cblock_t> &cbs,
    const std::vector<xmgd_pair_t> &prs, const std::vector<int> &blocks,
    uint64_t *d, int *n)
{
	std::vector<pg_item> items;
	std::vector<int64_t> cost(cbs.size(), 0);
	int st;

	*d = 0;
	*n = 0;
	if (blocks.empty())
		return XMG_OK;
	for (int ci : blocks) {
		const xmgd_cblock_t &cb = cbs[ci];
		for (int q = 0; q < cb.npairs; q++)
			cost[ci] += prs[cb.first_pair + q].k;
		for (int m0 = 0; m0 < cb.m; m0 += 64)
			for (int n0 = 0; n0 < cb.n; n0 += 64)
				items.push_back(pg_item{ci, m0, n0, 0});
	}
	std::stable_sort(items.begin(), items.end(),
	    [&](const pg_item &x, const pg_item &y) {
		return cost[x.cblock] > cost[y.cblock]; });
	if ((st = xmgd_alloc(items.size() * sizeof(pg_item), d)) != XMG_OK)
		return st;
	XMG_CK(cudaMemcpyAsync((void *)*d, items.data(), items.size() *
	    sizeof(pg_item), cudaMemcpyHostToDevice, stream()));
	*n = (int)items.size();
	return XMG_OK;
}

static int
launch_plain(xmgd_plan *dp, uint64_t items, int n)
{
	const xmgd_cblock_t *dc = (const xmgd_cblock_t *)dp->d_cbs;
	const xmgd_pair_t *pr = (const xmgd_pair_t *)dp->d_prs;
	const int32_t *dt = (const int32_t *)dp->d_tabs;
	const void *di = (const void *)items;

	switch (dp->dtype) {
	case 0: return plain_gemm_launch<float>(di, n, dc, pr, dt, dp->beta);
	case 1: return plain_gemm_launch<cf>(di, n, dc, pr, dt, dp->beta);
	case 2: return plain_gemm_launch<double>(di, n, dc, pr, dt, dp->beta);
	case 3: return plain_gemm_launch<cd>(di, n, dc, pr, dt, dp->beta);
	}
	return xmg_seterr(XMG_EINVAL, "bad scalar type");
}

/* the launches of one segment, on the engine stream */
static int
record(xmgd_plan *dp, int seg)
{
	int st;

	switch (seg) {
	case 0:
		if (dp->n_scale && (st = xmgd_ptask_launch(dp->dtype, dp->dtype,
		    &dp->scale)))
			return st;
		return dp->ep ? emu_record_split(dp->ep) : XMG_OK;
	case 1:
		return dp->ep ? emu_record_gemm(dp->ep) : XMG_OK;
	default:
		return dp->n_pg ? launch_plain(dp, dp->d_pg, dp->n_pg) : XMG_OK;
	}
}

static bool
seg_empty(const xmgd_plan *dp, int seg)
{
	switch (seg) {
	case 0: return !dp->n_scale && !dp->ep;
	case 1: return !dp->ep;
	default: return !dp->n_pg;
	}
}

static void
drop(segment &g)
{
	if (g.x)
		cudaGraphExecDestroy(g.x);
	g.x = nullptr;
}

static void
drop_graphs(xmgd_plan *dp)
{
	drop(dp->seg0);
	drop(dp->seg2);
	for (segment &g : dp->seg1)
		drop(g);
}

extern "C" void
xmgd_plan_free(xmgd_plan *dp)
{
	if (!dp)
		return;
	cudaStreamSynchronize(stream());
	drop_graphs(dp);
	emu_free(dp->ep);
	uint64_t bufs[] = {dp->d_cbs, dp->d_prs, dp->d_tabs, dp->scale.dbuf, dp->d_pg};
	for (uint64_t b : bufs)
		if (b)
			xmgd_free(b);
	for (cudaEvent_t e : dp->ev)
		if (e)
			cudaEventDestroy(e);
	delete dp;
}

static int
upload(const void *h, size_t bytes, uint64_t *d)
{
	int st;

	if ((st = xmgd_alloc(bytes ? bytes : 16, d)) != XMG_OK)
		return st;
	if (bytes)
		XMG_CK(cudaMemcpyAsync((void *)*d, h, bytes, cudaMemcpyHostToDevice,
		    stream()));
	return XMG_OK;
}

extern "C" int
xmgd_plan_create(const xmgd_contract_t *p, xmgd_plan **out)
{
	xmgd_plan *dp = new xmgd_plan();
	std::vector<xmgd_ptask_t> scale;
	int st;

	*out = nullptr;
	dp->dtype = p->dtype;
	dp->precision = p->precision;
	dp->one_shot = p->one_shot != 0;
	memcpy(dp->alpha, p->alpha, sizeof dp->alpha);
	memcpy(dp->beta, p->beta, sizeof dp->beta);
	dp->cbs.assign(p->cblocks, p->cblocks + p->ncblocks);
	dp->prs.assign(p->pairs, p->pairs + p->npairs);
	for (int i = 0; i < 4; i++)
		if ((st = check(cudaEventCreate(&dp->ev[i]), "event")))
			goto fail;
	if ((st = upload(p->cblocks, (size_t)p->ncblocks * sizeof(xmgd_cblock_t),
	    &dp->d_cbs)) || (st = upload(p->pairs, (size_t)p->npairs *
	    sizeof(xmgd_pair_t), &dp->d_prs)) || (st = upload(p->tabs,
	    (size_t)p->ntabs * sizeof(int32_t), &dp->d_tabs)))
		goto fail;

	/* route the output blocks */
	for (int i = 0; i < p->ncblocks; i++) {
		const xmgd_cblock_t &cb = p->cblocks[i];
		if (cb.npairs == 0) {
			/* no products: c = beta * c (contract.c:155-160) */
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
		bool want_emu = p->precision != XMG_PREC_FP64 && p->emulatable[i];
		(want_emu ? dp->emu : dp->plain).push_back(i);
	}
	if (!scale.empty()) {
		dp->n_scale = (int)scale.size();
		if ((st = xmgd_ptask_stage(scale.data(), dp->n_scale, dp->dtype,
		    &dp->scale)))
			goto fail;
	}
	if (!dp->emu.empty()) {
		st = emu_prepare(p, dp->emu, (const xmgd_cblock_t *)dp->d_cbs,
		    (const xmgd_pair_t *)dp->d_prs, (const int32_t *)dp->d_tabs,
		    &dp->ep);
		if (st == XMG_ENOTSUP && p->precision == XMG_PREC_AUTO) {
			dp->plain.insert(dp->plain.end(), dp->emu.begin(), dp->emu.end());
			dp->emu.clear();
			st = XMG_OK;
		} else if (st != XMG_OK)
			goto fail;
	}
	if ((st = stage_plain(dp->cbs, dp->prs, dp->plain, &dp->d_pg, &dp->n_pg)))
		goto fail;
	dp->seg1.resize(dp->ep ? emu_ncand(dp->ep) : 1);
	if ((st = check(cudaStreamSynchronize(stream()), "plan upload")))
		goto fail;
	*out = dp;
	return XMG_OK;
fail:
	xmgd_plan_free(dp);
	return st;
}

/* capture one segment as a graph */
static int
capture(xmgd_plan *dp, int seg, segment &out)
{
	cudaGraph_t g = nullptr;
	cudaGraphExec_t x = nullptr;
	long long n0 = g_launches;
	int st;

	XMG_CK(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal));
	st = record(dp, seg);
	cudaError_t ce = cudaStreamEndCapture(stream(), &g);
	if (st == XMG_OK)
		st = check(ce, "graph capture");
	if (st == XMG_OK)
		st = check(cudaGraphInstantiate(&x, g, 0), "graph instantiate");
	if (g)
		cudaGraphDestroy(g);
	/* launches are counted when the graph runs, not when captured */
	out.launches = g_launches - n0;
	g_launches = n0;
	if (st != XMG_OK)
		return st;
	out.x = x;
	return XMG_OK;
}

static int
run_segment(xmgd_plan *dp, int seg, segment &g)
{
	int st;

	if (seg_empty(dp, seg))
		return XMG_OK;
	if (!graphs_enabled() || dp->one_shot)
		return record(dp, seg);
	if (!g.x && (st = capture(dp, seg, g)))
		return st;
	XMG_CK(cudaGraphLaunch(g.x, stream()));
	g_launches += g.launches;
	return XMG_OK;
}

extern "C" int
xmgd_plan_run(xmgd_plan *dp, int *precision_used)
{
	int st, nan = 0, cand = 0;
	float ms = 0, ms_split = 0, ms_emu = 0, ms_plain = 0;

	memset(&g_timing, 0, sizeof g_timing);
	g_timing.gemm_policy = -1;
	*precision_used = XMG_PREC_FP64;
	if (dp->ep) {
		bool moved;
		if ((st = emu_bind(dp->ep, &moved)))
			return st;
		if (moved)
			drop_graphs(dp);
		cand = emu_current(dp->ep);
	}
	XMG_CK(cudaEventRecord(dp->ev[0], stream()));
	if ((st = run_segment(dp, 0, dp->seg0)))
		return st;
	XMG_CK(cudaEventRecord(dp->ev[1], stream()));
	if ((st = run_segment(dp, 1, dp->seg1[cand])))
		return st;
	XMG_CK(cudaEventRecord(dp->ev[2], stream()));
	if ((st = run_segment(dp, 2, dp->seg2)))
		return st;
	XMG_CK(cudaEventRecord(dp->ev[3], stream()));
	if ((st = check(cudaEventSynchronize(dp->ev[3]), "contraction kernels")))
		return st;
	XMG_CK(cudaEventElapsedTime(&ms_split, dp->ev[0], dp->ev[1]));
	XMG_CK(cudaEventElapsedTime(&ms_emu, dp->ev[1], dp->ev[2]));
	XMG_CK(cudaEventElapsedTime(&ms_plain, dp->ev[2], dp->ev[3]));
	XMG_CK(cudaEventElapsedTime(&ms, dp->ev[0], dp->ev[3]));
	g_timing.ms_total = ms;
	if (dp->ep) {
		const bool was_tuned = emu_tuned(dp->ep);
		g_timing.ms_split = ms_split;
		g_timing.ms_gemm += ms_emu;
		g_timing.gemm_launches += 1;
		g_timing.gemm_items += emu_items(dp->ep);
		g_timing.gemm_policy = emu_policy(dp->ep);
		g_timing.slice_bytes = emu_slice_bytes(dp->ep);
		if ((st = emu_finish(dp->ep, ms_emu, &nan)))
			return st;
		/* tuning over: keep only the chosen candidate's graph */
		if (!was_tuned && emu_tuned(dp->ep))
			for (size_t i = 0; i < dp->seg1.size(); i++)
				if ((int)i != emu_current(dp->ep))
					drop(dp->seg1[i]);
		if (!nan)
			*precision_used = XMG_PREC_EMU64;
	}
	if (dp->n_pg) {
		g_timing.ms_gemm += ms_plain;
		g_timing.gemm_launches += 1;
		g_timing.gemm_items += dp->n_pg;
	}
	if (nan) {
		/* Inf/NaN in an operand: the split-precision GEMM wrote nothing */
		if (dp->precision == XMG_PREC_EMU64)
			return xmg_seterr(XMG_ENOTSUP, "split-precision path: Inf/NaN "
			    "in operands");
		uint64_t d;
		int n;
		if ((st = stage_plain(dp->cbs, dp->prs, dp->emu, &d, &n)))
			return st;
		st = launch_plain(dp, d, n);
		xmgd_free(d);
		if (st == XMG_OK)
			st = check(cudaStreamSynchronize(stream()), "plain fallback");
		if (st)
			return st;
	}
	return check(cudaGetLastError(), "contraction kernels");
}

extern "C" int
xmgd_plan_a_shared(const xmgd_plan *dp)
{
	return dp->ep && emu_a_mode(dp->ep) == 1;
}

extern "C" int
xmgd_contract(xmgd_contract_t *p)
{
	xmgd_plan *dp;
	int st;

	p->precision_used = XMG_PREC_FP64;
	if ((st = xmgd_plan_create(p, &dp)) != XMG_OK)
		return st;
	st = xmgd_plan_run(dp, &p->precision_used);
	xmgd_plan_free(dp);
	return st;
}
