/*
 * Pagefile and host-memory contractions of libxm-gb300 (host, C): the
 * operands of tensors outside GPU memory are staged into HBM, b in batches
 * streamed through two regions while the previous batch is contracted.
 * The whole plan comes from the planner (contract.c) with data handles in
 * place of device addresses; each batch's plan is cut from it.
 */
#include <math.h>
#include <pthread.h>

#include "xmg_host.h"
#include "hmap.h"
#include "plan.h"

/* ------------------------------------------------------------------ */
/* out-of-core contraction                                             */

/*
 * b's blocks are streamed through two HBM regions: batch i + 1 is copied on
 * the side stream (cudaMemcpyAsync) into the idle region while batch i is
 * contracted on the compute stream.  The copies come straight from the
 * blocks' page-locked memory (host allocator), from a read-only mapping of
 * the pagefile where the GPU reads pageable memory through the host's page
 * tables, or else through reader threads (XMG_STAGE_THREADS, default 12)
 * that read the pagefile into pinned 64 MiB chunks, two per reader used in
 * turn.  Each batch is an ordinary contraction restricted to the merged
 * pairs whose b data lies in the batch (pairs merge only over equal b
 * data, so the restriction commutes with merging); beta is applied by the
 * first batch and the later ones accumulate with beta = 1.  The plan is
 * built once, with data handles for addresses, and each batch's plan cut
 * from it; the batch plans are kept for repeated calls.  a's and c's
 * canonical blocks are staged whole, as views in one HBM buffer, together
 * with batch 0 while batch 0's plan is cut; c's blocks go back once final
 * (pagefile: side-stream fetches into the readers' pinned chunks, pwrite).
 */
#define STAGE_CHUNK ((size_t)64 << 20)
#define STAGE_ALIGN 256

static size_t g_stage_budget, g_stage_region;

static size_t
env_bytes(const char *name, double gb)
{
	const char *e = getenv(name);

	return (size_t)((e ? atof(e) : gb) * 1e9);
}

int
xmg_set_staging(size_t budget, size_t region)
{
	if (budget)
		g_stage_budget = budget;
	if (region)
		g_stage_region = region;
	return XMG_OK;
}

/* a list of pagefile blocks moved by the reader threads: block i is
 * h[i] (sz[i] bytes) in the pagefile and dst[i] in HBM; wr = 0 reads the
 * pagefile into HBM, wr = 1 writes HBM back to the pagefile */
struct io_job {
	xm_allocator_t *al;
	const uint64_t *h, *sz, *dst;
	size_t n;
	int wr;
	int status;
	char err[256];
	pthread_t th;
	int running;
	double ms;               /* wall time of the job (start to drained) */
	/* host blocks: dst[0 .. seg) and dst[seg .. n) each lie in one device
	 * buffer, so runs of blocks inside one part may be copied at once
	 * (0: every block in its own allocation, one copy per block) */
	size_t seg;
	int merge;
};

/* one reader: chunks w, w + nw, w + 2 nw, ... of the list, alternating
 * its two pinned slots */
struct io_worker {
	struct io_job *j;
	int w, nw, status;
	char err[256];
};

static void *
io_worker_main(void *arg)
{
	struct io_worker *r = arg;
	struct io_job *j = r->j;
	size_t i, o, n, k = 0, mine = 0;
	void *buf;
	int st = xmgd_bind_thread();

	/* write-back: the chunk fetched last is written while the next one
	 * is fetched */
	int pslot = -1;
	size_t pi = 0, po = 0, pn = 0;
	void *pbuf = NULL;

	for (i = 0; st == XMG_OK && i < j->n; i++)
		for (o = 0; st == XMG_OK && o < j->sz[i]; o += n, k++) {
			n = j->sz[i] - o < STAGE_CHUNK ? j->sz[i] - o : STAGE_CHUNK;
			if ((int)(k % (size_t)r->nw) != r->w)
				continue;
			const int slot = 2 * r->w + (int)(mine++ & 1);
			if (!j->wr) {
				/* a chunk is refilled only after its previous copy */
				if ((st = xmgd_side_wait(slot)) == XMG_OK &&
				    (st = xmgd_side_chunk(slot, STAGE_CHUNK, &buf)) == XMG_OK &&
				    (st = xmg_alloc_read_range(j->al, j->h[i], o, buf, n)) ==
				    XMG_OK)
					st = xmgd_side_copy(slot, j->dst[i] + o, n);
				continue;
			}
			/* the slot's previous chunk went out one round ago */
			if ((st = xmgd_side_chunk(slot, STAGE_CHUNK, &buf)) != XMG_OK ||
			    (st = xmgd_side_fetch(slot, j->dst[i] + o, n)) != XMG_OK)
				break;
			if (pslot >= 0 && ((st = xmgd_side_wait(pslot)) != XMG_OK ||
			    (st = xmg_alloc_write_range(j->al, j->h[pi], po, pbuf, pn)) !=
			    XMG_OK))
				break;
			pslot = slot; pi = i; po = o; pn = n; pbuf = buf;
		}
	if (st == XMG_OK && pslot >= 0 && (st = xmgd_side_wait(pslot)) == XMG_OK)
		st = xmg_alloc_write_range(j->al, j->h[pi], po, pbuf, pn);
	r->status = st;
	if (st != XMG_OK)
		snprintf(r->err, sizeof r->err, "%s", xmg_last_error());
	return NULL;
}

static int
stage_threads(void)
{
	const char *e = getenv("XMG_STAGE_THREADS");
	int n = e ? atoi(e) : 12;

	return n < 1 ? 1 : n > XMGD_SIDE_SLOTS / 2 ? XMGD_SIDE_SLOTS / 2 : n;
}

/* The end of the run of blocks i, i + 1, ... (below lim) that one copy
 * may move: block r joins when it follows block r - 1 at the same distance
 * in host memory and in HBM with less than one alignment unit between
 * them.  Blocks start 256-byte aligned on both sides, so only padding lies
 * inside a run, never another block (equal end-to-end distances alone
 * would let two equal-sized blocks trade places). */
static size_t
copy_run_end(const uint64_t *h, const uint64_t *sz, const uint64_t *dst,
    size_t i, size_t lim)
{
	uint64_t end = h[i] + sz[i];
	size_t r;

	for (r = i + 1; r < lim && h[r] >= end && h[r] - end < STAGE_ALIGN &&
	    h[r] - h[r - 1] == dst[r] - dst[r - 1]; r++)
		end = h[r] + sz[r];
	return r;
}

/* the runs copy_run_end forms over a list (host-side check): run q starts
 * at block start[q]; returns the number of runs */
size_t
xmg_copy_runs(const uint64_t *h, const uint64_t *sz, const uint64_t *dst,
    size_t n, size_t *start)
{
	size_t i, q = 0;

	for (i = 0; i < n; i = copy_run_end(h, sz, dst, i, n))
		start[q++] = i;
	return q;
}

/* host-allocator blocks: cudaMemcpyAsync straight from (or into) the
 * blocks' own page-locked memory, queued on the side stream.  When the job
 * allows it (its device side lies in one or two buffers), one copy per run
 * of blocks that follow one another in host memory and in HBM (blocks
 * carved one after another from a slab and placed one after another in a
 * staging region: the usual case), since the copy engine moves few large
 * copies faster than many block-sized ones; a run never spans two device
 * buffers (a copy must stay inside one allocation) */
static void
io_host(struct io_job *j)
{
	size_t i, r;
	int st = xmgd_bind_thread();

	for (i = 0; st == XMG_OK && i < j->n; i = r) {
		const size_t lim = !j->merge ? i + 1 : i < j->seg ? j->seg : j->n;
		r = copy_run_end(j->h, j->sz, j->dst, i, lim);
		const uint64_t end = j->h[r - 1] + j->sz[r - 1];
		st = j->wr ? xmgd_side_get((void *)(uintptr_t)j->h[i], j->dst[i],
		    end - j->h[i]) : xmgd_side_put(j->dst[i],
		    (const void *)(uintptr_t)j->h[i], end - j->h[i]);
	}
	if (xmgd_side_sync() != XMG_OK && st == XMG_OK)
		st = XMG_ECUDA;
	if (st != XMG_OK)
		snprintf(j->err, sizeof j->err, "%s", xmg_last_error());
	j->status = st;
}

/* Pagefile blocks read through the file's mapping: where the device reads
 * pageable host memory through the host's page tables, one
 * cudaMemcpyAsync per block straight from the page cache (measured: 212
 * GB/s from a mapped, page-cache-resident file, like page-locked memory,
 * against ~60 GB/s for the reader threads' pread into pinned chunks).
 * XMG_STAGE_MMAP=0 keeps the readers, =1 forces the mapping. */
static int
stage_mapped(void)
{
	const char *e = getenv("XMG_STAGE_MMAP");

	if (e != NULL)
		return atoi(e) != 0;
	return xmgd_pageable_direct();
}

static int
io_mapped(struct io_job *j)
{
	const unsigned char *base;
	size_t i;
	int st = xmgd_bind_thread();

	if (st == XMG_OK && (st = xmg_alloc_file_map(j->al, &base)) == XMG_OK &&
	    base == NULL && j->n > 0)
		st = xmg_seterr(XMG_EINVAL, "staging: pagefile without data");
	for (i = 0; st == XMG_OK && i < j->n; i++)
		st = xmgd_side_put(j->dst[i], base + xmg_alloc_file_offset(j->h[i]),
		    j->sz[i]);
	if (xmgd_side_sync() != XMG_OK && st == XMG_OK)
		st = XMG_ECUDA;
	return st;
}


static void *
io_main(void *arg)
{
	struct io_job *j = arg;
	struct io_worker r[XMGD_SIDE_SLOTS / 2];
	pthread_t th[XMGD_SIDE_SLOTS / 2];
	int nw = stage_threads(), w, started = 0, st = XMG_OK;
	double t0 = xmg_now_ms();

	if (xmg_alloc_is_host(j->al)) {
		io_host(j);
		j->ms = xmg_now_ms() - t0;
		return NULL;
	}
	if (!j->wr && stage_mapped()) {
		if ((st = io_mapped(j)) != XMG_OK)
			snprintf(j->err, sizeof j->err, "%s", xmg_last_error());
		j->status = st;
		j->ms = xmg_now_ms() - t0;
		return NULL;
	}

	for (w = 0; w < nw; w++) {
		r[w].j = j;
		r[w].w = w;
		r[w].nw = nw;
		r[w].status = XMG_OK;
		r[w].err[0] = '\0';
	}
	for (w = 0; w < nw; w++, started++)
		if (pthread_create(&th[w], NULL, io_worker_main, &r[w])) {
			st = XMG_ENOMEM;
			snprintf(j->err, sizeof j->err, "cannot start a reader");
			break;
		}
	for (w = 0; w < started; w++) {
		pthread_join(th[w], NULL);
		if (r[w].status != XMG_OK && st == XMG_OK) {
			st = r[w].status;
			snprintf(j->err, sizeof j->err, "%s", r[w].err);
		}
	}
	xmgd_bind_thread();
	if (xmgd_side_sync() != XMG_OK && st == XMG_OK) {
		st = XMG_ECUDA;
		snprintf(j->err, sizeof j->err, "%s", xmg_last_error());
	}
	j->status = st;
	j->ms = xmg_now_ms() - t0;
	return NULL;
}

static int
io_start(struct io_job *j)
{
	j->status = XMG_OK;
	j->err[0] = '\0';
	if (pthread_create(&j->th, NULL, io_main, j))
		return xmg_seterr(XMG_ENOMEM, "cannot start the staging thread");
	j->running = 1;
	return XMG_OK;
}

static int
io_join(struct io_job *j)
{
	if (!j->running)
		return XMG_OK;
	pthread_join(j->th, NULL);
	j->running = 0;
	if (j->status != XMG_OK)
		return xmg_seterr(j->status, "staging: %s", j->err);
	return XMG_OK;
}

struct hsz {
	uint64_t h, sz;
	int64_t key;             /* ordering key (order_by_output) */
};

static int
cmp_key(const void *x, const void *y)
{
	const struct hsz *p = x, *q = y;

	if (p->key != q->key)
		return p->key < q->key ? -1 : 1;
	return p->h < q->h ? -1 : p->h > q->h;
}

static int
cmp_hsz(const void *x, const void *y)
{
	const struct hsz *p = x, *q = y;

	return p->h < q->h ? -1 : p->h > q->h;
}


/* Write c's staged views back to its pagefile (the reader threads in
 * reverse: side-stream fetches into pinned chunks, pwrite) and drop every
 * view. */
int
xmg_commit_c(xm_tensor_t *c, int st)
{
	xm_dim_t *list;
	size_t n, q, m = 0;
	uint64_t *h = NULL, *sz = NULL, *d = NULL;
	struct io_job j;

	if (xmg_alloc_is_device(c->allocator))
		return st;
	if (st == XMG_OK) {
		xm_tensor_get_canonical_block_list(c, &list, &n);
		h = malloc((n + 1) * sizeof *h);
		sz = malloc((n + 1) * sizeof *sz);
		d = malloc((n + 1) * sizeof *d);
		if (!h || !sz || !d)
			xm_fatal("%s: out of memory", __func__);
		for (q = 0; q < n; q++) {
			h[m] = xm_tensor_get_block_data_ptr(c, list[q]);
			sz[m] = xm_tensor_get_block_bytes(c, list[q]);
			d[m] = xmg_alloc_view_addr(c->allocator, h[m]);
			if (d[m] == 0) {
				st = xmg_seterr(XMG_EINVAL, "xm_contract: output block "
				    "without a staged view");
				break;
			}
			m++;
		}
		free(list);
		if (st == XMG_OK && m > 0) {
			memset(&j, 0, sizeof j);
			j.al = c->allocator;
			j.h = h; j.sz = sz; j.dst = d; j.n = m; j.wr = 1;
			if ((st = io_start(&j)) == XMG_OK)
				st = io_join(&j);
		}
		free(h); free(sz); free(d);
	}
	xmg_alloc_release_views(c->allocator, 0);
	return st;
}

/*
 * Views of a's and c's canonical blocks (one pagefile or host allocator)
 * in one HBM buffer *bulk, each block at a 256-byte aligned offset: vmap
 * maps every block's handle to its address.  Returns the blocks to read
 * into it (c's only when read_c: for beta = 0 the contraction overwrites
 * c, as the reference zeroes it, contract.c:155-158) and c's canonical
 * blocks, the ones to write back.
 */
static int
bulk_views(const xm_tensor_t *a, const xm_tensor_t *c, int read_c,
    uint64_t *bulk, xmg_hmap_t *vmap, uint64_t **rh, uint64_t **rsz,
    uint64_t **rd, size_t *nr, uint64_t **ch, uint64_t **csz, uint64_t **cd,
    size_t *ncw)
{
	const xm_tensor_t *t[2] = {a, c};
	xm_dim_t *list[2] = {NULL, NULL};
	size_t n[2] = {0, 0}, cnt = 0, m = 0, q, s;
	uint64_t *h, *sz, *d, off = 0, v;
	char *rdf;
	int st = XMG_OK;

	*bulk = 0;
	for (s = 0; s < 2; s++) {
		xm_tensor_get_canonical_block_list(t[s], &list[s], &n[s]);
		cnt += n[s];
	}
	h = malloc((cnt + 1) * sizeof *h);
	sz = malloc((cnt + 1) * sizeof *sz);
	d = malloc((cnt + 1) * sizeof *d);
	rdf = malloc(cnt + 1);
	*ch = malloc((n[1] + 1) * sizeof **ch);
	*csz = malloc((n[1] + 1) * sizeof **csz);
	*cd = malloc((n[1] + 1) * sizeof **cd);
	if (!h || !sz || !d || !rdf || !*ch || !*csz || !*cd)
		xm_fatal("%s: out of memory", __func__);
	for (s = 0; s < 2; s++)
		for (q = 0; q < n[s]; q++) {
			uint64_t hq = xm_tensor_get_block_data_ptr(t[s], list[s][q]);
			if (xmg_hmap_get(vmap, hq, &v)) {
				rdf[v] |= s == 0 || read_c;
				continue;
			}
			if (xmg_hmap_put(vmap, hq, m))
				xm_fatal("%s: out of memory", __func__);
			h[m] = hq;
			sz[m] = xm_tensor_get_block_bytes(t[s], list[s][q]);
			d[m] = off;
			rdf[m] = s == 0 || read_c;
			off += (sz[m] + STAGE_ALIGN - 1) / STAGE_ALIGN * STAGE_ALIGN;
			m++;
		}
	if (m > 0 && (st = xmgd_alloc(off, bulk)) == XMG_OK)
		for (q = 0; q < m; q++) {
			d[q] += *bulk;
			/* the map now gives addresses */
			if (xmg_hmap_put(vmap, h[q], d[q]))
				xm_fatal("%s: out of memory", __func__);
		}
	*ncw = 0;
	for (q = 0; st == XMG_OK && q < n[1]; q++) {
		uint64_t hq = xm_tensor_get_block_data_ptr(c, list[1][q]);
		(*ch)[*ncw] = hq;
		(*csz)[*ncw] = xm_tensor_get_block_bytes(c, list[1][q]);
		xmg_hmap_get(vmap, hq, &(*cd)[*ncw]);
		(*ncw)++;
	}
	free(list[0]);
	free(list[1]);
	/* keep the blocks to read, in order */
	*nr = 0;
	for (q = 0; st == XMG_OK && q < m; q++)
		if (rdf[q]) {
			h[*nr] = h[q];
			sz[*nr] = sz[q];
			d[*nr] = d[q];
			(*nr)++;
		}
	free(rdf);
	*rh = h;
	*rsz = sz;
	*rd = d;
	return st;
}

/*
 * Batch k's contraction, derived from the whole plan (built once per call
 * with data handles in place of device addresses): the pairs whose b block
 * is in the batch (dmap: handle -> address in the batch's region), the
 * operand views those pairs use renumbered in order of first use, a's and
 * c's blocks at their bulk views.
 */
struct batch_buf {
	xmgd_cblock_t *cb;
	xmgd_pair_t *pr;
	xmgd_view_t *va, *vb;
	int32_t *vamap, *vbmap;
};

static void
batch_buf_alloc(struct batch_buf *bb, const plan_t *p)
{
	bb->cb = malloc((p->ncb + 1) * sizeof *bb->cb);
	bb->pr = malloc((p->npr + 1) * sizeof *bb->pr);
	bb->va = malloc((p->nva + 1) * sizeof *bb->va);
	bb->vb = malloc((p->nvb + 1) * sizeof *bb->vb);
	bb->vamap = malloc((p->nva + 1) * sizeof *bb->vamap);
	bb->vbmap = malloc((p->nvb + 1) * sizeof *bb->vbmap);
	if (!bb->cb || !bb->pr || !bb->va || !bb->vb || !bb->vamap || !bb->vbmap)
		xm_fatal("%s: out of memory", __func__);
}

static void
batch_buf_free(struct batch_buf *bb)
{
	free(bb->cb); free(bb->pr); free(bb->va); free(bb->vb);
	free(bb->vamap); free(bb->vbmap);
	memset(bb, 0, sizeof *bb);
}

/* a data handle's device address: its staged view in vmap, or the
 * handle itself when there is no map (host-side checks) */
static uint64_t
handle_addr(const xmg_hmap_t *vmap, uint64_t h)
{
	uint64_t d;

	if (vmap == NULL)
		return h;
	return xmg_hmap_get(vmap, h, &d) ? d : 0;
}

/* the distinct b blocks of a collected plan, in handle (file) order */
static size_t
distinct_b(const plan_t *p, struct hsz **out)
{
	struct hsz *u = NULL;
	size_t i, nu = 0;

	if (p->nbh && (u = malloc(p->nbh * sizeof *u)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < p->nbh; i++) {
		u[i].h = p->bh[i];
		u[i].sz = p->bsz[i];
		u[i].key = 0;
	}
	if (p->nbh)
		qsort(u, p->nbh, sizeof *u, cmp_hsz);
	for (i = 0; i < p->nbh; i++)
		if (nu == 0 || u[nu - 1].h != u[i].h)
			u[nu++] = u[i];
	*out = u;
	return nu;
}

/* b's blocks (distinct, in file order) in batches, each block at a
 * STAGE_ALIGN-aligned offset of its batch: batch k holds blocks bstart[k]
 * .. bstart[k + 1] - 1 (bstart[nb] = nu), block i at offset off[i];
 * *rbytes is the largest batch.  Batch k takes at most cap_k bytes, with
 * cap_k = region when first <= 0, else min(region, first * growth^e):
 * e = k, or with tent = n > 0, e = min(k, n - 1 - k) (at least 0), so that
 * the batches grow and then shrink again.  A block larger than cap_k (but
 * within the region) makes a batch of its own.  A block larger than the
 * region is an error. */
static int
form_batches(const struct hsz *u, size_t nu, size_t region, double first,
    double growth, int tent, uint64_t *off, size_t *bstart, size_t *nb,
    uint64_t *rbytes)
{
	uint64_t run = 0;
	double cap = (double)region;
	size_t i;

	*nb = 0;
	*rbytes = 0;
	for (i = 0; i < nu; i++) {
		uint64_t al = (u[i].sz + STAGE_ALIGN - 1) / STAGE_ALIGN * STAGE_ALIGN;
		if (al > region)
			return xmg_seterr(XMG_ENOMEM, "xm_contract: a block of b "
			    "(%llu bytes) exceeds the staging region (%zu bytes)",
			    (unsigned long long)u[i].sz, region);
		if (i == 0 || (run > 0 && (double)(run + al) > cap)) {
			if (first > 0) {
				long e = (long)*nb;
				if (tent > 0) {
					e = tent - 1 - e < e ? tent - 1 - e : e;
					if (e < 0)
						e = 0;
				}
				cap = first * pow(growth, (double)e);
				if (cap > (double)region)
					cap = (double)region;
			}
			bstart[(*nb)++] = i;
			run = 0;
		}
		off[i] = run;
		run += al;
		if (run > *rbytes)
			*rbytes = run;
	}
	bstart[*nb] = nu;
	return XMG_OK;
}

/* b's batches in the output blocks' order (order_by_output) with
 * XMG_STREAM_ORDER=output, else in file order.  Where b's contracted
 * indices lead (the ladders' "cdab"), a batch in output order takes a
 * block from every run of the file: measured on a GB300, host-memory
 * copies no longer merge and the link moved such batches at ~147 GB/s
 * against ~212 for merged ones, with kernels no faster (cfg2 from host
 * memory: 53.8 ms per call against 52.3), and copies from a pagefile's
 * mapping ran 10-20 % slower, about what the early write-back of c won
 * (cfg2 from a pagefile: 107-108 ms against 110-111; cfg5's structure
 * with b = 60 GB: 1151-1266 ms against 1169-1217). */
static int
stream_order_output(const xm_allocator_t *bal)
{
	const char *e = getenv("XMG_STREAM_ORDER");

	(void)bal;
	return e && strcmp(e, "output") == 0;
}

/*
 * b's distinct blocks in the order of the output blocks they feed: by the
 * smallest b-side exponent slot (one per b-side free block index of c)
 * among the pairs that read the block, then by handle.  Batches cut on
 * this order each feed a range of c's blocks, so a block of c is final
 * once the batch holding its last pair has run (and may go back to the
 * host while later batches run), and each batch's kernels read and
 * write only its range of c.  In file order, with b's contracted indices
 * leading, every batch feeds every block of c.
 */
static void
order_by_output(const plan_t *p, struct hsz *u, size_t nu)
{
	xmg_hmap_t ix;
	uint64_t v;
	size_t i;
	int l, q;

	xmg_hmap_init(&ix);
	for (i = 0; i < nu; i++) {
		u[i].key = INT64_MAX;
		if (xmg_hmap_put(&ix, u[i].h, i))
			xm_fatal("%s: out of memory", __func__);
	}
	for (l = 0; l < p->ncb; l++) {
		const xmgd_cblock_t *cb = &p->cb[l];
		for (q = 0; q < cb->npairs; q++)
			if (xmg_hmap_get(&ix, p->pr[cb->first_pair + q].b_ptr, &v) &&
			    cb->eB < u[v].key)
				u[v].key = cb->eB;
	}
	xmg_hmap_free(&ix);
	if (nu)
		qsort(u, nu, sizeof *u, cmp_key);
}

/*
 * c's canonical blocks (ch, csz, cd; n of them) reordered by the batch
 * after which each is final: the batch of its last pair, batch 0 for a
 * block without pairs (only beta applies, in batch 0), the last batch for
 * a block the plan does not list.  cstart[k] .. cstart[k + 1] - 1 are the
 * blocks final after batch k.
 */
static void
c_by_last_batch(const plan_t *p, const uint64_t *H, const size_t *bstart,
    size_t nb, uint64_t *ch, uint64_t *csz, uint64_t *cd, size_t n,
    size_t *cstart)
{
	xmg_hmap_t bk, ck;
	uint64_t v, *t;
	size_t i, k, *last, *pos;
	int l, q;

	xmg_hmap_init(&bk);
	xmg_hmap_init(&ck);
	for (k = 0; k < nb; k++)
		for (i = bstart[k]; i < bstart[k + 1]; i++)
			if (xmg_hmap_put(&bk, H[i], k))
				xm_fatal("%s: out of memory", __func__);
	for (l = 0; l < p->ncb; l++) {
		const xmgd_cblock_t *cb = &p->cb[l];
		uint64_t lb = 0;
		for (q = 0; q < cb->npairs; q++)
			if (xmg_hmap_get(&bk, p->pr[cb->first_pair + q].b_ptr, &v) &&
			    v > lb)
				lb = v;
		if (xmg_hmap_get(&ck, cb->c_ptr, &v) && v > lb)
			lb = v;
		if (xmg_hmap_put(&ck, cb->c_ptr, lb))
			xm_fatal("%s: out of memory", __func__);
	}
	last = malloc((n + 1) * sizeof *last);
	pos = calloc(nb + 1, sizeof *pos);
	t = malloc((n + 1) * sizeof *t);
	if (!last || !pos || !t)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < n; i++) {
		last[i] = xmg_hmap_get(&ck, ch[i], &v) ? (size_t)v : nb - 1;
		pos[last[i] + 1]++;
	}
	for (k = 0; k < nb; k++)
		pos[k + 1] += pos[k];
	memcpy(cstart, pos, (nb + 1) * sizeof *cstart);
	/* a stable counting sort of the three arrays */
	uint64_t *arr[3] = {ch, csz, cd};
	for (int a = 0; a < 3; a++) {
		size_t *at = malloc((nb + 1) * sizeof *at);
		if (!at)
			xm_fatal("%s: out of memory", __func__);
		memcpy(at, cstart, (nb + 1) * sizeof *at);
		for (i = 0; i < n; i++)
			t[at[last[i]]++] = arr[a][i];
		memcpy(arr[a], t, n * sizeof *t);
		free(at);
	}
	free(last); free(pos); free(t);
	xmg_hmap_free(&bk);
	xmg_hmap_free(&ck);
}

static int
batch_plan(const plan_t *pf, const xmg_hmap_t *dmap, const xmg_hmap_t *al,
    struct batch_buf *bb, xm_scalar_t alpha, xm_scalar_t beta, int prec,
    int all_a, xmgd_contract_t *dp)
{
	const double mult = xmg_is_complex(pf->type) ? 8.0 : 2.0;
	double flops = 0;
	int l, q, v, npr = 0, nva = 0, nvb = 0;
	uint64_t d;

	for (v = 0; v < pf->nva; v++)
		bb->vamap[v] = -1;
	for (v = 0; v < pf->nvb; v++)
		bb->vbmap[v] = -1;
	for (l = 0; l < pf->ncb; l++) {
		const xmgd_cblock_t *cs = &pf->cb[l];
		xmgd_cblock_t *cd = &bb->cb[l];
		*cd = *cs;
		if ((cd->c_ptr = handle_addr(al, cs->c_ptr)) == 0)
			return xmg_seterr(XMG_EINVAL, "xm_contract: a block of c "
			    "without a staged view");
		cd->first_pair = npr;
		for (q = 0; q < cs->npairs; q++) {
			const xmgd_pair_t *ps = &pf->pr[cs->first_pair + q];
			if (!xmg_hmap_get(dmap, ps->b_ptr, &d))
				continue;	/* b block outside this batch */
			xmgd_pair_t *pd = &bb->pr[npr++];
			*pd = *ps;
			pd->b_ptr = d;
			if ((pd->a_ptr = handle_addr(al, ps->a_ptr)) == 0)
				return xmg_seterr(XMG_EINVAL, "xm_contract: a block "
				    "of a without a staged view");
			if (bb->vamap[ps->aview] < 0) {
				bb->va[nva] = pf->va[ps->aview];
				bb->va[nva].ptr = pd->a_ptr;
				bb->vamap[ps->aview] = nva++;
			}
			pd->aview = bb->vamap[ps->aview];
			if (bb->vbmap[ps->bview] < 0) {
				bb->vb[nvb] = pf->vb[ps->bview];
				bb->vb[nvb].ptr = d;
				bb->vbmap[ps->bview] = nvb++;
			}
			pd->bview = bb->vbmap[ps->bview];
			flops += mult * cs->m * (double)cs->n * ps->k;
		}
		cd->npairs = npr - cd->first_pair;
	}
	/* all_a: every view of a, the ones no pair of the batch uses last */
	for (v = 0; all_a && v < pf->nva; v++) {
		if (bb->vamap[v] >= 0)
			continue;
		bb->va[nva] = pf->va[v];
		if ((bb->va[nva].ptr = handle_addr(al, pf->va[v].ptr)) == 0)
			return xmg_seterr(XMG_EINVAL, "xm_contract: a block of a "
			    "without a staged view");
		bb->vamap[v] = nva++;
	}
	memset(dp, 0, sizeof *dp);
	dp->dtype = pf->type;
	dp->precision = prec;
	xmg_scalar_pack(alpha, dp->alpha);
	xmg_scalar_pack(beta, dp->beta);
	dp->ncblocks = pf->ncb;
	dp->npairs = npr;
	dp->cblocks = bb->cb;
	dp->pairs = bb->pr;
	dp->views_a = bb->va;
	dp->views_b = bb->vb;
	dp->nviews_a = nva;
	dp->nviews_b = nvb;
	dp->tabs = pf->tabs.v;
	dp->ntabs = pf->tabs.n;
	dp->nexp_a = pf->nexp_a;
	dp->nexp_b = pf->nexp_b;
	dp->flops = flops;
	dp->emulatable = pf->emulatable;
	dp->one_shot = 1;
	return XMG_OK;
}

/* a view of a batch plan against the whole plan's: equal but for the
 * address, which is the pair's (field by field: the structs have padding) */
static int
same_view(const xmgd_view_t *x, const xmgd_view_t *y, uint64_t ptr)
{
	return x->ptr == ptr && x->k == y->k && x->mn == y->mn &&
	    x->rowtab == y->rowtab && x->coltab == y->coltab &&
	    x->exptab == y->exptab && x->n_rt == y->n_rt &&
	    x->n_ks == y->n_ks && x->kfast == y->kfast && x->cplx == y->cplx &&
	    x->khp == y->khp && x->kcontig == y->kcontig &&
	    x->slices == y->slices;
}

/* a pair of a batch plan against the whole plan's, view ids aside */
static int
same_pair(const xmgd_pair_t *x, const xmgd_pair_t *y)
{
	return x->a_ptr == y->a_ptr && x->b_ptr == y->b_ptr && x->k == y->k &&
	    x->arow == y->arow && x->acol == y->acol && x->brow == y->brow &&
	    x->bcol == y->bcol && x->esign == y->esign &&
	    x->eshift == y->eshift && x->al[0] == y->al[0] &&
	    x->al[1] == y->al[1];
}

int
xmg_batch_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int nbatch, long long region, int policy,
    long long out[4])
{
	plan_t p;
	struct batch_buf bb;
	struct hsz *u = NULL;
	xmg_hmap_t dmap;
	xmgd_contract_t dp;
	unsigned char *used = NULL;
	double flops = 0;
	long long wl[4], npairs = 0, items = 0;
	uint64_t *off = NULL, rbytes, *H = NULL, *ch = NULL, *cz = NULL,
	    *cd0 = NULL, fv;
	size_t nu, i, k, *bstart = NULL, nb, *cstart = NULL;
	xmg_hmap_t fin;
	int st, l, j, q, ok = 1;

	memset(out, 0, 4 * sizeof *out);
	if (region <= 0 && nbatch < 1)
		return xmg_seterr(XMG_EINVAL, "xmg_batch_plan_check: nbatch < 1");
	xmg_plan_init(&p);
	p.collect = 1;
	if ((st = xmg_plan_check(a, b, c, idxa, idxb, idxc, &p)) != XMG_OK ||
	    (st = xmg_plan_build(1, a, b, c, &p, 2)) != XMG_OK) {
		xmg_plan_free(&p);
		return st;
	}
	nu = distinct_b(&p, &u);
	if (stream_order_output(b->allocator))
		order_by_output(&p, u, nu);
	batch_buf_alloc(&bb, &p);
	used = calloc(p.npr + 1, 1);
	off = malloc((nu + 1) * sizeof *off);
	bstart = malloc((nu + (size_t)(nbatch > 0 ? nbatch : 0) + 2) *
	    sizeof *bstart);
	if (!used || !off || !bstart)
		xm_fatal("%s: out of memory", __func__);
	if (region > 0) {
		/* the streamed path's batches of at most `region` bytes: each
		 * block inside the region, aligned, after the previous one */
		if ((st = form_batches(u, nu, (size_t)region, 0, 1, 0, off, bstart,
		    &nb, &rbytes)) != XMG_OK)
			goto done;
		if (nu > 0 && (bstart[0] != 0 || bstart[nb] != nu ||
		    rbytes > (uint64_t)region))
			ok = 0;
		for (k = 0; k < nb; k++)
			for (i = bstart[k]; i < bstart[k + 1]; i++)
				if (off[i] % STAGE_ALIGN != 0 ||
				    off[i] + u[i].sz > (uint64_t)region ||
				    (i > bstart[k] && off[i] < off[i - 1] + u[i - 1].sz) ||
				    (i == bstart[k] && off[i] != 0))
					ok = 0;
	} else {
		/* nbatch equal runs of b's blocks */
		nb = (size_t)nbatch;
		for (k = 0; k <= nb; k++)
			bstart[k] = nu * k / nb;
	}
	/* c's blocks by the batch after which they are final */
	xmg_hmap_init(&fin);
	H = malloc((nu + 1) * sizeof *H);
	ch = malloc((p.ncb + 1) * sizeof *ch);
	cz = calloc(p.ncb + 1, sizeof *cz);
	cd0 = calloc(p.ncb + 1, sizeof *cd0);
	cstart = malloc((nb + 1) * sizeof *cstart);
	if (!H || !ch || !cz || !cd0 || !cstart)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < nu; i++)
		H[i] = u[i].h;
	for (l = 0; l < p.ncb; l++)
		ch[l] = p.cb[l].c_ptr;
	c_by_last_batch(&p, H, bstart, nb, ch, cz, cd0, (size_t)p.ncb, cstart);
	for (k = 0; k < nb; k++)
		for (i = cstart[k]; i < cstart[k + 1]; i++)
			if (xmg_hmap_put(&fin, ch[i], k))
				xm_fatal("%s: out of memory", __func__);
	xmg_hmap_init(&dmap);
	for (k = 0; k < nb && st == XMG_OK; k++) {
		xmg_hmap_free(&dmap);
		xmg_hmap_init(&dmap);
		for (i = bstart[k]; i < bstart[k + 1]; i++)
			if (xmg_hmap_put(&dmap, u[i].h, u[i].h))
				xm_fatal("%s: out of memory", __func__);
		if ((st = batch_plan(&p, &dmap, NULL, &bb, 1, k == 0 ? 0 : 1, 0,
		    XMG_PREC_EMU64, &dp)) != XMG_OK)
			break;
		/* each pair of the batch is a later pair of its output block
		 * in the whole plan, with b in the batch, used by no other
		 * batch, with the same views */
		for (l = 0; l < dp.ncblocks; l++) {
			const xmgd_cblock_t *cs = &p.cb[l], *cd = &dp.cblocks[l];
			if (cd->m != cs->m || cd->n != cs->n ||
			    cd->c_ptr != cs->c_ptr || cd->eA != cs->eA ||
			    cd->eB != cs->eB)
				ok = 0;
			/* no block of c goes back before a batch that feeds it */
			if (cd->npairs > 0 && (!xmg_hmap_get(&fin, cs->c_ptr, &fv) ||
			    fv < k))
				ok = 0;
			for (j = 0, q = 0; j < cd->npairs; j++, q++) {
				const xmgd_pair_t *pd = &dp.pairs[cd->first_pair + j];
				const xmgd_pair_t *ps;
				for (; q < cs->npairs; q++)
					if (same_pair(pd, &p.pr[cs->first_pair + q]))
						break;
				if (q == cs->npairs) {
					ok = 0;
					break;
				}
				ps = &p.pr[cs->first_pair + q];
				if (used[cs->first_pair + q]++ ||
				    !xmg_hmap_get(&dmap, ps->b_ptr, NULL) ||
				    pd->aview < 0 || pd->aview >= dp.nviews_a ||
				    pd->bview < 0 || pd->bview >= dp.nviews_b ||
				    !same_view(&dp.views_a[pd->aview], &p.va[ps->aview],
				    pd->a_ptr) ||
				    !same_view(&dp.views_b[pd->bview], &p.vb[ps->bview],
				    pd->b_ptr))
					ok = 0;
			}
		}
		npairs += dp.npairs;
		flops += dp.flops;
		if ((st = xmgd_work_list_check(&dp, policy, wl)) != XMG_OK)
			break;
		items += wl[0];
		ok = ok && wl[3];
	}
	if (st == XMG_OK) {
		for (i = 0; i < (size_t)p.npr; i++)
			if (used[i] != 1)
				ok = 0;
		if (npairs != p.npr || flops != p.flops)
			ok = 0;
		out[0] = (long long)nb;
		out[1] = npairs;
		out[2] = items;
		out[3] = ok;
	}
	xmg_hmap_free(&dmap);
	xmg_hmap_free(&fin);
done:
	free(H); free(ch); free(cz); free(cd0); free(cstart);
	free(off);
	free(bstart);
	free(used);
	free(u);
	batch_buf_free(&bb);
	xmg_plan_free(&p);
	return st;
}

/*
 * A streamed contraction, kept across calls: the whole plan's batches of
 * b (data handles, bytes, device addresses in the two regions), the
 * regions themselves, the HBM buffer holding a's and c's blocks, and one
 * device plan per batch.  A call whose tensors, structure generations,
 * index strings, scalars, precision and staging sizes match the kept one
 * reuses all of it: no planning, no device allocation, the batch plans'
 * captured graphs replayed.  Only the data moves.
 */
struct stream_plan {
	const xm_tensor_t *a, *b, *c;
	uint64_t ga, gb, gc;
	char idx[3][16];
	xm_scalar_t alpha, beta;
	int precision, keep;
	size_t budget, region;
	/* b's distinct blocks in file order, batch k = bstart[k] ..
	 * bstart[k + 1] - 1 */
	size_t nu, nb, *bstart;
	uint64_t *H, *SZ, *D, total, rbytes, reg[2];
	/* a's and c's blocks in one buffer: the ones read before batch 0
	 * (R*) and c's canonical blocks, written back after the last (C*) */
	uint64_t bulk;
	size_t nr, ncw;
	uint64_t *RH, *RSZ, *RD, *CH, *CSZ, *CD;
	size_t *cstart;             /* C* final after batch k: cstart[k] ..
	                               cstart[k + 1] - 1 */
	xmg_hmap_t vmap;            /* a's and c's handles -> addresses */
	/* a's split-precision operands, prepared by batch 0 for the later
	 * batches (a_share 1): slices, exponent table, Inf/NaN flag in abuf */
	uint64_t abuf;
	int a_share;
	xmgd_plan_t **bp;           /* per batch, built on first use */
	double *bflops;
	int *bnpairs;
	double flops;
	int ncb;
};

static struct stream_plan *g_sp;    /* the kept streamed contraction */

static void
sp_free(struct stream_plan *sp)
{
	size_t k;

	if (sp == NULL)
		return;
	if (sp->bp)
		for (k = 0; k < sp->nb; k++)
			if (sp->bp[k])
				xmgd_plan_free(sp->bp[k]);
	xmgd_sync();
	if (sp->reg[0])
		xmgd_free(sp->reg[0]);
	if (sp->reg[1])
		xmgd_free(sp->reg[1]);
	if (sp->bulk)
		xmgd_free(sp->bulk);
	if (sp->abuf)
		xmgd_free(sp->abuf);
	xmg_hmap_free(&sp->vmap);
	free(sp->bstart); free(sp->H); free(sp->SZ); free(sp->D);
	free(sp->RH); free(sp->RSZ); free(sp->RD);
	free(sp->CH); free(sp->CSZ); free(sp->CD); free(sp->cstart);
	free(sp->bp); free(sp->bflops); free(sp->bnpairs);
	free(sp);
}

void
xmg_stream_release(void)
{
	sp_free(g_sp);
	g_sp = NULL;
}

static int
sp_match(const struct stream_plan *sp, xm_scalar_t alpha,
    const xm_tensor_t *a, const xm_tensor_t *b, xm_scalar_t beta,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int prec, size_t budget, size_t region)
{
	return sp != NULL && sp->a == a && sp->b == b && sp->c == c &&
	    sp->ga == a->gen && sp->gb == b->gen && sp->gc == c->gen &&
	    sp->alpha == alpha && sp->beta == beta && sp->precision == prec &&
	    sp->budget == budget && sp->region == region &&
	    strcmp(sp->idx[0], idxa) == 0 && strcmp(sp->idx[1], idxb) == 0 &&
	    strcmp(sp->idx[2], idxc) == 0;
}

/* host-allocator b: about XMG_HOST_BATCHES (default 8) batches that
 * grow by a factor XMG_HOST_GROWTH (default 1.45) per batch up to the
 * middle and shrink again toward the end (XMG_HOST_SHAPE=tent, the
 * default; =geometric keeps growing).  The small first batch is the only
 * copy nothing overlaps; the small last one is the only kernels nothing
 * overlaps where the host link is slower than the kernels consume b (a
 * batch's kernels take about 5.5-6.5 ms per GB of b for the FP64 ladders,
 * its copy 4.7 ms per GB at 212 GB/s, 7-8 ms at the 130-150 GB/s seen on
 * some boxes, where the geometric schedule's last 1.6 GB batch left ~10 ms
 * of kernels after the last copy).  Measured, cfg2 from host memory on a
 * box with a 212 GB/s link (compute-bound): tent 8 at 1.45 51.7 ms per
 * call, 8 at 1.3 52.2, 6 at 1.3 52.2, 8 at 1.2 52.6, 10 at 1.25 52.9;
 * geometric 6 at 1.15 52.1.  Returns the first batch's byte budget;
 * *tent is the batch count of the tent shape, 0 for geometric. */
static double
host_first_batch(uint64_t total, double *growth, int *tent)
{
	const char *e = getenv("XMG_HOST_BATCHES"), *g = getenv("XMG_HOST_GROWTH");
	const char *sh = getenv("XMG_HOST_SHAPE");
	const int geo = sh && strcmp(sh, "geometric") == 0;
	int n = e ? atoi(e) : 8, k;
	double r = g ? atof(g) : 1.45, w = 0;

	if (n < 1)
		n = 1;
	if (!(r >= 1.0))
		r = 1.0;
	*growth = r;
	*tent = geo ? 0 : n;
	for (k = 0; k < n; k++)
		w += pow(r, geo ? k : (k < n - 1 - k ? k : n - 1 - k));
	return (double)total / w;
}

/* pagefile b beyond the staging budget: about XMG_STAGE_BATCHES (default
 * 8) equal batches of at most the region's bytes.  The pagefile readers
 * (page cache, ~40-70 GB/s) are slower than the kernels consume b (about
 * 100 GB/s for the FP64 ladders), so the call takes about the read time
 * plus the last batch's kernels: smaller batches shorten that tail.
 * Returns the batch byte budget. */
static double
file_batch(uint64_t total)
{
	const char *e = getenv("XMG_STAGE_BATCHES");
	double n = e ? atof(e) : 8;

	if (n < 1)
		n = 1;
	return (double)total / n;
}

/* the batches the streamed path cuts for b's distinct blocks of sizes
 * sz[0 .. n - 1] (in that order): host-memory b (host != 0) or a pagefile
 * b beyond the staging budget, batches of at most `region` bytes; batch k
 * is blocks bstart[k] .. bstart[k + 1] - 1 (bstart holds n + 1 entries).
 * Returns the number of batches, 0 on error.  For tests. */
size_t
xmg_stream_batches(const uint64_t *sz, size_t n, size_t region, int host,
    size_t *bstart)
{
	struct hsz *u;
	uint64_t *off, rbytes, total = 0;
	double first, growth = 1;
	size_t i, nb = 0;
	int tent = 0;

	if (n == 0)
		return 0;
	u = malloc(n * sizeof *u);
	off = malloc(n * sizeof *off);
	if (!u || !off)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < n; i++) {
		u[i].h = i + 1;
		u[i].sz = sz[i];
		u[i].key = 0;
		total += sz[i];
	}
	first = host ? host_first_batch(total, &growth, &tent) : file_batch(total);
	if (form_batches(u, n, region, first, growth, tent, off, bstart, &nb,
	    &rbytes) != XMG_OK)
		nb = 0;
	free(u);
	free(off);
	return nb;
}

/*
 * The batches, regions and staged views of a streamed contraction (no
 * device plans yet).  Returns XMG_OK with *sp set, or a status; *incore
 * is set when the in-core path should run instead (no GEMMs, or a
 * structure error the in-core path reports).
 */
static int
sp_build(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int prec, size_t budget, size_t region, plan_t *p0,
    struct stream_plan **out, int *incore)
{
	struct stream_plan *sp;
	struct hsz *u = NULL;
	uint64_t *OFF = NULL;
	size_t i, k;
	int st;

	*out = NULL;
	*incore = 0;
	p0->collect = 1;
	if (xmg_plan_check(a, b, c, idxa, idxb, idxc, p0) != XMG_OK ||
	    xmg_plan_build(alpha, a, b, c, p0, 2) != XMG_OK) {
		*incore = 1;	/* the in-core path reports it */
		return XMG_OK;
	}
	if ((sp = calloc(1, sizeof *sp)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	xmg_hmap_init(&sp->vmap);
	sp->a = a; sp->b = b; sp->c = c;
	sp->ga = a->gen; sp->gb = b->gen; sp->gc = c->gen;
	sp->alpha = alpha; sp->beta = beta; sp->precision = prec;
	sp->budget = budget; sp->region = region;
	sp->keep = strlen(idxa) < 16 && strlen(idxb) < 16 && strlen(idxc) < 16;
	if (sp->keep) {
		strcpy(sp->idx[0], idxa);
		strcpy(sp->idx[1], idxb);
		strcpy(sp->idx[2], idxc);
	}
	sp->flops = p0->flops;
	sp->ncb = p0->ncb;
	/* distinct b blocks in file order */
	sp->nu = distinct_b(p0, &u);
	if (sp->nu == 0) {
		/* no GEMMs (alpha = 0 or no nonzero pair): the in-core path
		 * applies beta to c */
		free(u);
		sp_free(sp);
		*incore = 1;
		return XMG_OK;
	}
	for (i = 0; i < sp->nu; i++)
		sp->total += u[i].sz;
	if (stream_order_output(b->allocator))
		order_by_output(p0, u, sp->nu);
	/* within the budget a pagefile b is staged whole: one batch, still
	 * read by the parallel readers; a host b is always streamed */
	double first = 0, growth = 1;
	int tent = 0;
	if (xmg_alloc_is_host(b->allocator))
		first = host_first_batch(sp->total, &growth, &tent);
	else if (sp->total <= budget)
		region = sp->total + sp->nu * STAGE_ALIGN;
	else
		first = file_batch(sp->total);
	sp->H = malloc(sp->nu * sizeof *sp->H);
	sp->SZ = malloc(sp->nu * sizeof *sp->SZ);
	sp->D = malloc(sp->nu * sizeof *sp->D);
	OFF = malloc(sp->nu * sizeof *OFF);
	sp->bstart = malloc((sp->nu + 1) * sizeof *sp->bstart);
	if (!sp->H || !sp->SZ || !sp->D || !OFF || !sp->bstart)
		xm_fatal("%s: out of memory", __func__);
	for (i = 0; i < sp->nu; i++) {
		sp->H[i] = u[i].h;
		sp->SZ[i] = u[i].sz;
	}
	st = form_batches(u, sp->nu, region, first, growth, tent, OFF, sp->bstart,
	    &sp->nb, &sp->rbytes);
	free(u);
	if (st == XMG_OK) {
		sp->bp = calloc(sp->nb, sizeof *sp->bp);
		sp->bflops = calloc(sp->nb, sizeof *sp->bflops);
		sp->bnpairs = calloc(sp->nb, sizeof *sp->bnpairs);
		if (!sp->bp || !sp->bflops || !sp->bnpairs)
			xm_fatal("%s: out of memory", __func__);
	}
	if (st == XMG_OK)
		st = xmgd_alloc(sp->rbytes, &sp->reg[0]);
	if (st == XMG_OK && sp->nb > 1)
		st = xmgd_alloc(sp->rbytes, &sp->reg[1]);
	/* every b block's address in its batch's region */
	for (k = 0; st == XMG_OK && k < sp->nb; k++)
		for (i = sp->bstart[k]; i < sp->bstart[k + 1]; i++)
			sp->D[i] = sp->reg[k & 1] + OFF[i];
	free(OFF);
	/* a's and c's blocks as views in one buffer */
	if (st == XMG_OK)
		st = bulk_views(a, c, creal(beta) != 0 || cimag(beta) != 0,
		    &sp->bulk, &sp->vmap, &sp->RH, &sp->RSZ, &sp->RD, &sp->nr,
		    &sp->CH, &sp->CSZ, &sp->CD, &sp->ncw);
	/* c's blocks by the batch after which they are final */
	if (st == XMG_OK) {
		if ((sp->cstart = malloc((sp->nb + 1) * sizeof *sp->cstart)) == NULL)
			xm_fatal("%s: out of memory", __func__);
		c_by_last_batch(p0, sp->H, sp->bstart, sp->nb, sp->CH, sp->CSZ,
		    sp->CD, sp->ncw, sp->cstart);
	}
	if (st == XMG_OK)
		st = xmgd_sync();
	if (st != XMG_OK) {
		sp_free(sp);
		return st;
	}
	*out = sp;
	return XMG_OK;
}

/* A job moving c's staged blocks i0 .. i1 - 1 (of C*) back: pagefile
 * through the readers, host blocks straight into their pinned memory. */
static int
c_write_start(struct stream_plan *sp, xm_tensor_t *c, size_t i0, size_t i1,
    struct io_job *j)
{
	memset(j, 0, sizeof *j);
	j->al = c->allocator;
	j->h = sp->CH + i0; j->sz = sp->CSZ + i0; j->dst = sp->CD + i0;
	j->n = i1 - i0; j->wr = 1;
	j->merge = 1; j->seg = j->n;	/* c's views: one bulk buffer */
	return j->n ? io_start(j) : XMG_OK;
}

/*
 * c's blocks go back batch by batch, each block once the batch holding its
 * last pair has run, while the later batches run (XMG_STREAM_CWRITE=0
 * writes all of c after the last batch).  Not with pagefile readers
 * staging b: the write-back's readers would share their pinned slots.
 */
static int
c_write_early(const struct stream_plan *sp)
{
	const char *e = getenv("XMG_STREAM_CWRITE");

	if (e && strcmp(e, "0") == 0)
		return 0;
	return xmg_alloc_is_host(sp->b->allocator) || stage_mapped();
}

/*
 * a's split-precision operands once per call instead of once per batch:
 * batch 0's plan splits every view of a into one buffer of the stream
 * plan, the later batches' plans read them there.  XMG_STREAM_SHARE_A=0
 * splits a in every batch.  *off gets each view's slice offset (whole
 * plan's view ids); returns the slice bytes, 0 when a is not shared.
 */
static uint64_t
a_side_offsets(const struct stream_plan *sp, const plan_t *p0, int64_t *off)
{
	const char *e = getenv("XMG_STREAM_SHARE_A");
	uint64_t tot = 0;
	int v;

	if (sp->nb < 2 || sp->precision == XMG_PREC_FP64 || (int)p0->type < 0 ||
	    (int)p0->type > 3 || (e && strcmp(e, "0") == 0))
		return 0;
	for (v = 0; v < p0->nva; v++) {
		off[v] = (int64_t)tot;
		tot += (uint64_t)xmgd_emu_view_bytes(&p0->va[v], p0->type);
	}
	return tot;
}

/* the shared a side of batch k's plan: batch 0 prepares it (its views
 * are all of a's), the others use it */
static void
a_side_attach(const struct stream_plan *sp, const plan_t *p0,
    const struct batch_buf *bb, const int64_t *offg, uint64_t slice_bytes,
    size_t k, int64_t *offl, xmgd_contract_t *dp)
{
	int v;

	for (v = 0; v < p0->nva; v++)
		if (bb->vamap[v] >= 0)
			offl[bb->vamap[v]] = offg[v];
	dp->a_mode = k == 0 ? 1 : 2;
	dp->a_slices = sp->abuf;
	dp->a_E = sp->abuf + slice_bytes;
	dp->a_flag = dp->a_E + ((uint64_t)p0->nexp_a * 4 + 15) / 16 * 16;
	dp->a_off = offl;
}

/*
 * One call of a streamed contraction: a's (and, for beta != 0, c's)
 * blocks and batch 0 are read while batch 0's plan is built (on the
 * first call), then batch k + 1 streams into the idle region while batch
 * k is contracted, and c is written back.  Batch plans missing from sp
 * are cut from p0 (the whole plan) and kept in sp.
 */
static int
sp_run(struct stream_plan *sp, const plan_t *p0, xm_tensor_t *c)
{
	struct batch_buf bb = {NULL, NULL, NULL, NULL, NULL, NULL};
	struct io_job io[2], cw;
	const int early = c_write_early(sp);
	uint64_t *JH = NULL, *JSZ = NULL, *JD = NULL, abytes = 0;
	int64_t *offg = NULL, *offl = NULL;
	xmg_hmap_t filt;
	xmg_stats_t acc;
	size_t i, k, n0 = sp->bstart[1];
	double tw = 0;
	int st = XMG_OK, used_all = XMG_PREC_EMU64;

	const char *tr = getenv("XMG_STREAM_TRACE");
	const int trace = tr && strcmp(tr, "0") != 0;

	memset(io, 0, sizeof io);
	memset(&cw, 0, sizeof cw);
	memset(&acc, 0, sizeof acc);
	acc.gemm_policy = -1;
	xmg_hmap_init(&filt);
	for (k = 0; k < 2; k++)
		io[k].al = sp->b->allocator;
	JH = malloc((sp->nr + n0 + 1) * sizeof *JH);
	JSZ = malloc((sp->nr + n0 + 1) * sizeof *JSZ);
	JD = malloc((sp->nr + n0 + 1) * sizeof *JD);
	if (!JH || !JSZ || !JD)
		xm_fatal("%s: out of memory", __func__);
	memcpy(JH, sp->RH, sp->nr * sizeof *JH);
	memcpy(JSZ, sp->RSZ, sp->nr * sizeof *JSZ);
	memcpy(JD, sp->RD, sp->nr * sizeof *JD);
	memcpy(JH + sp->nr, sp->H, n0 * sizeof *JH);
	memcpy(JSZ + sp->nr, sp->SZ, n0 * sizeof *JSZ);
	memcpy(JD + sp->nr, sp->D, n0 * sizeof *JD);
	io[0].h = JH; io[0].sz = JSZ; io[0].dst = JD;
	io[0].n = sp->nr + n0;
	/* a's and c's views in the bulk buffer, then batch 0 in its region */
	io[0].merge = 1; io[0].seg = sp->nr;
	if ((st = io_start(&io[0])) != XMG_OK)
		goto out;
	for (k = 0; k < sp->nb && st == XMG_OK; k++) {
		struct io_job *nx = &io[(k + 1) & 1];
		int used = XMG_PREC_FP64;
		double t0 = xmg_now_ms();

		if (sp->bp[k] == NULL) {
			xmgd_contract_t dp;
			if (p0 == NULL) {
				st = xmg_seterr(XMG_EINVAL, "xm_contract: streamed "
				    "plan without its batch plans");
				break;
			}
			if (bb.cb == NULL) {
				batch_buf_alloc(&bb, p0);
				offg = malloc((p0->nva + 1) * sizeof *offg);
				offl = malloc((p0->nva + 1) * sizeof *offl);
				if (!offg || !offl)
					xm_fatal("%s: out of memory", __func__);
			}
			/* a's operands shared: laid out and allocated with
			 * batch 0's plan */
			if (k == 0 && (abytes = a_side_offsets(sp, p0, offg)) > 0) {
				uint64_t eb = ((uint64_t)p0->nexp_a * 4 + 15) / 16 * 16;
				if (sp->abuf == 0 && (st = xmgd_alloc(abytes + eb + 16,
				    &sp->abuf)) != XMG_OK)
					break;
				sp->a_share = 1;
			}
			/* the batch's blocks resolve into its region */
			xmg_hmap_free(&filt);
			xmg_hmap_init(&filt);
			for (i = sp->bstart[k]; i < sp->bstart[k + 1]; i++)
				if (xmg_hmap_put(&filt, sp->H[i], sp->D[i]))
					xm_fatal("%s: out of memory", __func__);
			if ((st = batch_plan(p0, &filt, &sp->vmap, &bb, sp->alpha,
			    k == 0 ? sp->beta : 1, sp->precision,
			    k == 0 && sp->a_share, &dp)) == XMG_OK) {
				if (sp->a_share)
					a_side_attach(sp, p0, &bb, offg, abytes, k,
					    offl, &dp);
				/* a kept plan is replayed: graphs and tuning */
				dp.one_shot = !sp->keep;
				st = xmgd_plan_create(&dp, &sp->bp[k]);
				sp->bflops[k] = dp.flops;
				sp->bnpairs[k] = dp.npairs;
			}
			/* batch 0 without a split-precision part prepares
			 * nothing: the others split a themselves */
			if (st == XMG_OK && k == 0 && sp->a_share &&
			    !xmgd_plan_a_shared(sp->bp[0]))
				sp->a_share = 0;
		}
		acc.ms_plan += xmg_now_ms() - t0;
		/* batch k's data in place (only batch 0 can still be loading:
		 * later batches were joined at the end of the previous round),
		 * then batch k + 1 streams in while batch k is contracted; one
		 * job at a time, as the readers share the pinned slots */
		if (k == 0) {
			t0 = xmg_now_ms();
			int s2 = io_join(&io[0]);
			tw += xmg_now_ms() - t0;
			if (st == XMG_OK)
				st = s2;
			if (trace)
				fprintf(stderr, "xmg stream: a, c and batch 0 staged in "
				    "%.2f ms\n", io[0].ms);
		}
		if (st == XMG_OK && k + 1 < sp->nb) {
			nx->h = sp->H + sp->bstart[k + 1];
			nx->sz = sp->SZ + sp->bstart[k + 1];
			nx->dst = sp->D + sp->bstart[k + 1];
			nx->n = sp->bstart[k + 2] - sp->bstart[k + 1];
			nx->merge = 1; nx->seg = nx->n;	/* one region */
			st = io_start(nx);
		}
		double tr0 = xmg_now_ms(), tw0 = tw;
		if (st == XMG_OK)
			st = xmgd_plan_run(sp->bp[k], &used);
		const double trun = xmg_now_ms() - tr0;
		if (st == XMG_OK) {
			xmgd_timing_t tm;
			xmgd_last_timing(&tm);
			acc.flops += sp->bflops[k];
			acc.ms_device += tm.ms_total;
			acc.ms_split += tm.ms_split;
			acc.ms_gemm += tm.ms_gemm;
			acc.n_pairs += sp->bnpairs[k];
			acc.gemm_launches += tm.gemm_launches;
			acc.gemm_policy = tm.gemm_policy;
			if (tm.slice_bytes > acc.slice_bytes)
				acc.slice_bytes = tm.slice_bytes;
			if (sp->bnpairs[k] > 0 && used != XMG_PREC_EMU64)
				used_all = XMG_PREC_FP64;
		}
		t0 = xmg_now_ms();
		if (k + 1 < sp->nb) {
			int s2 = io_join(nx);
			if (st == XMG_OK)
				st = s2;
		}
		/* c's blocks final after batch k go back (one write-back job
		 * at a time) */
		if (st == XMG_OK && early &&
		    sp->cstart[k + 1] > sp->cstart[k]) {
			st = io_join(&cw);
			if (st == XMG_OK)
				st = c_write_start(sp, c, sp->cstart[k],
				    sp->cstart[k + 1], &cw);
		}
		tw += xmg_now_ms() - t0;
		if (trace) {
			uint64_t bytes = 0;
			for (i = sp->bstart[k]; i < sp->bstart[k + 1]; i++)
				bytes += sp->SZ[i];
			fprintf(stderr, "xmg stream: batch %zu/%zu %.3f GB, run %.2f "
			    "ms, next batch's copy %.2f ms, waits %.2f ms\n", k,
			    sp->nb, bytes / 1e9, trun, k + 1 < sp->nb ? nx->ms : 0.0,
			    tw - tw0);
		}
	}
	for (k = 0; k < 2; k++)
		io_join(&io[k]);	/* never leave a copy in flight */
	double tc = xmg_now_ms();
	{
		int s2 = io_join(&cw);
		if (st == XMG_OK)
			st = s2;
	}
	if (st == XMG_OK && !early && (st = c_write_start(sp, c, 0, sp->ncw,
	    &cw)) == XMG_OK)
		st = io_join(&cw);
	if (trace)
		fprintf(stderr, "xmg stream: c written back in %.2f ms\n",
		    xmg_now_ms() - tc);
	acc.n_cblocks = sp->ncb;
	acc.precision_used = used_all;
	acc.stage_bytes = (long long)sp->total;
	acc.stage_batches = (int)sp->nb;
	acc.ms_stage_wait = tw;
	if (st == XMG_OK)
		xmg_last_stats = acc;
out:
	xmg_hmap_free(&filt);
	batch_buf_free(&bb);
	free(JH); free(JSZ); free(JD);
	free(offg); free(offl);
	return st;
}

/*
 * Pagefile and host-memory path.  Returns 0 when the contraction should
 * run through the in-core path (b in GPU memory or b aliasing a or c, no
 * GEMMs, or a structure error that path reports), else 1 with the status
 * in *st.  A pagefile b is streamed in batches when its blocks exceed the
 * staging budget, else staged whole as a single batch; a host-memory b is
 * always streamed.  The streamed plan of the last such contraction is
 * kept (XMG_STREAM_CACHE=0 disables that) and reused by a matching call.
 */
int
xmg_contract_streamed(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, xm_scalar_t beta, xm_tensor_t *c,
    const char *idxa, const char *idxb, const char *idxc, int prec, int *st)
{
	struct stream_plan *sp = NULL;
	plan_t p0;
	const char *e = getenv("XMG_STREAM_CACHE");
	const int cache = !(e && strcmp(e, "0") == 0);
	double tp = xmg_now_ms();
	int incore = 0;

	if (xmg_alloc_is_device(b->allocator) || b == a || b == c)
		return 0;
	if (!g_stage_budget)
		g_stage_budget = env_bytes("XMG_STAGE_BUDGET_GB", 180);
	if (!g_stage_region)
		g_stage_region = env_bytes("XMG_STAGE_REGION_GB", 32);
	xmg_plan_init(&p0);
	if (cache && sp_match(g_sp, alpha, a, b, beta, c, idxa, idxb, idxc,
	    prec, g_stage_budget, g_stage_region)) {
		sp = g_sp;
		g_sp = NULL;
	} else {
		/* the kept plan's device memory goes before the new one's */
		sp_free(g_sp);
		g_sp = NULL;
		*st = sp_build(alpha, a, b, beta, c, idxa, idxb, idxc, prec,
		    g_stage_budget, g_stage_region, &p0, &sp, &incore);
		if (incore) {
			xmg_plan_free(&p0);
			return 0;
		}
		if (*st != XMG_OK) {
			xmg_plan_free(&p0);
			return 1;
		}
	}
	tp = xmg_now_ms() - tp;
	*st = sp_run(sp, sp->bp[sp->nb - 1] ? NULL : &p0, c);
	xmg_last_stats.ms_plan += tp;
	xmg_plan_free(&p0);
	if (*st == XMG_OK && cache && sp->keep)
		g_sp = sp;
	else
		sp_free(sp);
	return 1;
}
