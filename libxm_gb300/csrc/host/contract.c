/*
 * Block-sparse contraction planner of libxm-gb300 (host, C).
 *
 * For every canonical block of c, in the canonical-list order, the planner
 * enumerates the contraction block pairs, drops pairs with a zero block,
 * forms alpha_pair = s_a * s_b, and merges pairs that read the same
 * canonical data of a and b with the same permutation on the free indices
 * by summing their factors in index order -- the reference's
 * compute_block/same_contraction rules (contract.c:86-115, 161-192),
 * restated with a hash on the pair key instead of the O(nblkk^2) scan so
 * that production-size block grids plan in linear time.  Surviving pairs
 * become one device plan: gather offset tables (the unfold/fold
 * permutations, fused into the GEMM kernels), operand views for the split
 * precision path and a work list for the grouped GEMM.  Tensors outside
 * GPU memory go through stream.c with the same plan.
 */
#include <math.h>
#include <pthread.h>
#include <time.h>

#include "xmg_host.h"
#include "hmap.h"
#include "plan.h"

static int g_precision = -1;
xmg_stats_t xmg_last_stats;

static int
precision_mode(void)
{
	const char *e;

	if (g_precision < 0) {
		g_precision = XMG_PREC_AUTO;
		if ((e = getenv("XMG_PRECISION")) != NULL) {
			if (strcmp(e, "fp64") == 0)
				g_precision = XMG_PREC_FP64;
			else if (strcmp(e, "emu64") == 0)
				g_precision = XMG_PREC_EMU64;
		}
	}
	return g_precision;
}

int
xmg_set_precision(int mode)
{
	if (mode != XMG_PREC_FP64 && mode != XMG_PREC_EMU64 &&
	    mode != XMG_PREC_AUTO)
		return xmg_seterr(XMG_EINVAL, "xmg_set_precision: bad mode");
	g_precision = mode;
	return XMG_OK;
}

int xmg_get_precision(void) { return precision_mode(); }

int
xmg_get_last_stats(xmg_stats_t *out)
{
	*out = xmg_last_stats;
	return XMG_OK;
}

/* ------------------------------------------------------------------ */
/* offset-table pool with interning                                    */


/* Offset table sum_d digit_d(e) * stride[d] (first dimension fastest),
 * interned by its (sizes, strides) descriptor: blocks of equal shape and
 * permutation share one table. */
static int32_t
tab_intern(tabpool_t *p, int nd, const int64_t *size, const int64_t *stride)
{
	uint64_t h = 0x9e3779b97f4a7c15ULL, slot;
	int64_t total = 1, e, r;
	struct tabdesc *t;
	int d;

	for (d = 0; d < nd; d++) {
		h = xmg_hash64(h ^ (uint64_t)size[d] * 0x100000001b3ULL);
		h = xmg_hash64(h ^ (uint64_t)stride[d]);
		total *= size[d];
	}
	h = xmg_hash64(h ^ (uint64_t)nd);
	for (;;) {
		if (h == XMG_HMAP_EMPTY)
			h--;
		if (!xmg_hmap_get(&p->index, h, &slot))
			break;
		t = &p->desc[slot];
		if (t->nd == nd &&
		    memcmp(t->size, size, (size_t)nd * sizeof *size) == 0 &&
		    memcmp(t->stride, stride, (size_t)nd * sizeof *stride) == 0)
			return t->off;
		h = xmg_hash64(h + 1);	/* collision: probe another key */
	}
	if (p->n + total > INT32_MAX) {
		p->overflow = 1;	/* the planner reports it */
		return 0;
	}
	while (p->n + total > p->cap) {
		p->cap = p->cap ? 2 * p->cap : 4096;
		if ((p->v = realloc(p->v, (size_t)p->cap * sizeof *p->v)) == NULL)
			xm_fatal("%s: out of memory", __func__);
	}
	if (p->ndesc == p->capdesc) {
		p->capdesc = p->capdesc ? 2 * p->capdesc : 256;
		if ((p->desc = realloc(p->desc, (size_t)p->capdesc *
		    sizeof *p->desc)) == NULL)
			xm_fatal("%s: out of memory", __func__);
	}
	t = &p->desc[p->ndesc];
	memset(t, 0, sizeof *t);
	t->nd = nd;
	memcpy(t->size, size, (size_t)nd * sizeof *size);
	memcpy(t->stride, stride, (size_t)nd * sizeof *stride);
	t->off = (int32_t)p->n;
	if (nd == 0)
		p->v[p->n++] = 0;
	else {
		/* odometer walk: runs along dimension 0, carries into the
		 * outer digits (no division per element) */
		int64_t dig[XM_MAX_DIM] = {0}, base = 0;
		for (e = 0; e < total; e += size[0]) {
			for (r = 0; r < size[0]; r++)
				p->v[p->n++] = (int32_t)(base + r * stride[0]);
			for (d = 1; d < nd; d++) {
				base += stride[d];
				if (++dig[d] < size[d])
					break;
				base -= stride[d] * size[d];
				dig[d] = 0;
			}
		}
	}
	xmg_hmap_put(&p->index, h, (uint64_t)p->ndesc);
	return p->desc[p->ndesc++].off;
}

/* Table over the masked dimensions of a block with the given strides. */
static int32_t
mask_table(tabpool_t *p, const xm_dim_t *dims, const int64_t *strides,
    const xm_dim_t *mask)
{
	int64_t sz[XM_MAX_DIM], st[XM_MAX_DIM];
	size_t k;

	for (k = 0; k < mask->n; k++) {
		sz[k] = (int64_t)dims->i[mask->i[k]];
		st[k] = strides[mask->i[k]];
	}
	return tab_intern(p, (int)mask->n, sz, st);
}

/* ------------------------------------------------------------------ */
/* the plan                                                            */


#define GROW(arr, n, cap) do {						\
	if ((n) == (cap)) {						\
		(cap) = (cap) ? 2 * (cap) : 256;			\
		if (((arr) = realloc((arr), (size_t)(cap) * sizeof *(arr))) == NULL) \
			xm_fatal("%s: out of memory", __func__);	\
	}								\
} while (0)

void
xmg_plan_free(plan_t *p)
{
	free(p->cb); free(p->pr); free(p->va); free(p->vb); free(p->tabs.v);
	free(p->tabs.desc);
	free(p->emulatable);
	free(p->bh);
	free(p->bsz);
	xmg_hmap_free(&p->tabs.index);
	xmg_hmap_free(&p->va_index); xmg_hmap_free(&p->vb_index);
	xmg_hmap_free(&p->ea_index); xmg_hmap_free(&p->eb_index);
}

/* Exponent-table slot for the free-block index of an operand block. */
static int32_t
exp_slot(xmg_hmap_t *index, int32_t *nexp, const xm_tensor_t *t,
    xm_dim_t blk, const xm_dim_t *freemask, int32_t ncols)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs);
	uint64_t key = 0, v;
	size_t k;

	for (k = 0; k < freemask->n; k++)
		key = key * nb.i[freemask->i[k]] + blk.i[freemask->i[k]];
	if (xmg_hmap_get(index, key, &v))
		return (int32_t)v;
	v = (uint64_t)*nexp;
	*nexp += ncols;
	xmg_hmap_put(index, key, v);
	return (int32_t)v;
}

static int32_t
view_id(xmgd_view_t **arr, int *n, int *cap, xmg_hmap_t *index,
    uint64_t ptr, int32_t k, int32_t mn, int32_t rowtab, int32_t coltab,
    int32_t exptab)
{
	uint64_t key = xmg_hash64(ptr ^ xmg_hash64(((uint64_t)(uint32_t)rowtab
	    << 32) | (uint32_t)coltab)), v;
	xmgd_view_t *w;
	int i;

	if (key == XMG_HMAP_EMPTY)
		key--;
	if (xmg_hmap_get(index, key, &v)) {
		w = &(*arr)[v];
		if (w->ptr == ptr && w->rowtab == rowtab && w->coltab == coltab)
			return (int32_t)v;
		for (i = 0; i < *n; i++) {	/* hash collision: scan */
			w = &(*arr)[i];
			if (w->ptr == ptr && w->rowtab == rowtab &&
			    w->coltab == coltab)
				return i;
		}
	}
	GROW(*arr, *n, *cap);
	w = &(*arr)[*n];
	memset(w, 0, sizeof *w);
	w->ptr = ptr; w->k = k; w->mn = mn;
	w->rowtab = rowtab; w->coltab = coltab; w->exptab = exptab;
	if (!xmg_hmap_get(index, key, NULL))
		xmg_hmap_put(index, key, (uint64_t)*n);
	return (*n)++;
}

/* +-1 or +-2, real: the emulated path folds such pair factors exactly into
 * its integer drains (merged antisymmetric pairs give exactly these). */
static int
pow2_factor(xm_scalar_t s, int *sign, int *shift)
{
	double r = creal(s), m;
	int e;

	if (cimag(s) != 0 || r == 0 || !isfinite(r))
		return 0;
	m = frexp(fabs(r), &e);
	if (m != 0.5 || e - 1 < 0 || e - 1 > 1)
		return 0;
	*sign = r < 0 ? -1 : 1;
	*shift = e - 1;
	return 1;
}

struct cand {
	xm_dim_t ia, ib;
	const struct xmg_block *pa, *pb;    /* the blocks at ia, ib */
	xm_scalar_t al;
	uint64_t da, db;
};

/* xm_dim_inc_mask that also advances the index's linear position in the
 * block grid (st: the grid's strides, index 0 fastest) */
static size_t
inc_mask_linear(xm_dim_t *idx, const xm_dim_t *dim, const xm_dim_t *mask,
    const size_t *st, size_t lin)
{
	size_t k, pos;

	for (k = 0; k < mask->n; k++) {
		pos = mask->i[k];
		if (++idx->i[pos] < dim->i[pos])
			return lin + st[pos];
		lin -= (dim->i[pos] - 1) * st[pos];
		idx->i[pos] = 0;
	}
	return lin;
}

/* data handle of a nonzero block (xm_tensor_get_block_data_ptr) */
static uint64_t
block_data(const xm_tensor_t *t, const struct xmg_block *blk)
{
	return blk->type == XM_BLOCK_TYPE_CANONICAL ? blk->data :
	    t->blocks[blk->data].data;
}

static int
same_key(const struct cand *x, const struct cand *y, const xm_dim_t *aidxa,
    const xm_dim_t *aidxb)
{
	size_t k;

	if (x->da != y->da || x->db != y->db)
		return 0;
	for (k = 0; k < aidxa->n; k++)
		if (x->pa->perm.i[aidxa->i[k]] != y->pa->perm.i[aidxa->i[k]])
			return 0;
	for (k = 0; k < aidxb->n; k++)
		if (x->pb->perm.i[aidxb->i[k]] != y->pb->perm.i[aidxb->i[k]])
			return 0;
	return 1;
}

static uint64_t
cand_hash(const struct cand *x, const xm_dim_t *aidxa, const xm_dim_t *aidxb)
{
	uint64_t h = xmg_hash64(x->da) ^ (xmg_hash64(x->db) * 3);
	size_t k;

	for (k = 0; k < aidxa->n; k++)
		h = xmg_hash64(h + x->pa->perm.i[aidxa->i[k]] + 1);
	for (k = 0; k < aidxb->n; k++)
		h = xmg_hash64(h + 31 * (x->pb->perm.i[aidxb->i[k]] + 1));
	return h == XMG_HMAP_EMPTY ? h - 1 : h;
}

/*
 * Order of the contracted indices inside one pair's K.  Any order gives the
 * same sum as long as both operands of the pair use it, so K follows the
 * memory order of the larger operand block that holds a unit-stride
 * contracted index: its K rows are then contiguous runs, and the unfold
 * gathers of the split kernels read whole sectors.  Without such an index
 * the masks' own order stays.
 */
static void
k_order(const xm_dim_t *cidxa, const xm_dim_t *cidxb, const int64_t *sa,
    const int64_t *sb, int64_t na, int64_t nb, xm_dim_t *ka, xm_dim_t *kb)
{
	const int64_t *st = NULL;
	const xm_dim_t *mk = NULL;
	size_t q, r, n = cidxa->n;
	int hasa = 0, hasb = 0;

	*ka = *cidxa;
	*kb = *cidxb;
	for (q = 0; q < n; q++) {
		hasa |= sa[cidxa->i[q]] == 1;
		hasb |= sb[cidxb->i[q]] == 1;
	}
	if (hasb && (!hasa || nb >= na)) {
		st = sb;
		mk = cidxb;
	} else if (hasa) {
		st = sa;
		mk = cidxa;
	} else
		return;
	/* insertion sort of the positions by the chosen side's strides */
	for (q = 1; q < n; q++) {
		size_t ia = ka->i[q], ib = kb->i[q];
		int64_t key = st[mk == cidxb ? ib : ia];
		for (r = q; r > 0; r--) {
			int64_t prev = st[mk == cidxb ? kb->i[r - 1] : ka->i[r - 1]];
			if (prev <= key)
				break;
			ka->i[r] = ka->i[r - 1];
			kb->i[r] = kb->i[r - 1];
		}
		ka->i[r] = ia;
		kb->i[r] = ib;
	}
}

double
xmg_now_ms(void)
{
	struct timespec ts;

	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

/* Validation and masks: contract.c:237-280, same messages. */
int
xmg_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, plan_t *p)
{
	const char *fn = "xm_contract";
	size_t k;

	if (a->allocator != c->allocator || b->allocator != c->allocator)
		return xmg_seterr(XMG_EINVAL, "%s: tensors must use same "
		    "allocator", fn);
	if (a->type != c->type || b->type != c->type)
		return xmg_seterr(XMG_EINVAL, "%s: tensors must have same "
		    "scalar type", fn);
	if (strlen(idxa) != xm_block_space_get_ndims(a->bs) ||
	    strlen(idxb) != xm_block_space_get_ndims(b->bs) ||
	    strlen(idxc) != xm_block_space_get_ndims(c->bs))
		return xmg_seterr(XMG_EINVAL, "%s: bad contraction indices", fn);
	xm_make_masks(idxa, idxb, &p->cidxa, &p->cidxb);
	xm_make_masks(idxc, idxa, &p->cidxc, &p->aidxa);
	xm_make_masks(idxc, idxb, &p->aidxc, &p->aidxb);
	if (p->aidxa.n + p->cidxa.n != xm_block_space_get_ndims(a->bs) ||
	    p->aidxb.n + p->cidxb.n != xm_block_space_get_ndims(b->bs) ||
	    p->aidxc.n + p->cidxc.n != xm_block_space_get_ndims(c->bs))
		return xmg_seterr(XMG_EINVAL, "%s: bad contraction indices", fn);
	if (!(p->aidxc.n > 0 && p->aidxc.i[0] == 0) &&
	    !(p->cidxc.n > 0 && p->cidxc.i[0] == 0))
		return xmg_seterr(XMG_EINVAL, "%s: bad contraction indices", fn);
	for (k = 0; k < p->cidxa.n; k++)
		if (!xm_block_space_eq1(a->bs, p->cidxa.i[k], b->bs,
		    p->cidxb.i[k]))
			return xmg_seterr(XMG_EINVAL, "%s: inconsistent a and b "
			    "tensor block-spaces", fn);
	for (k = 0; k < p->cidxc.n; k++)
		if (!xm_block_space_eq1(c->bs, p->cidxc.i[k], a->bs,
		    p->aidxa.i[k]))
			return xmg_seterr(XMG_EINVAL, "%s: inconsistent a and c "
			    "tensor block-spaces", fn);
	for (k = 0; k < p->aidxc.n; k++)
		if (!xm_block_space_eq1(c->bs, p->aidxc.i[k], b->bs,
		    p->aidxb.i[k]))
			return xmg_seterr(XMG_EINVAL, "%s: inconsistent b and c "
			    "tensor block-spaces", fn);
	return XMG_OK;
}

/*
 * Build the plan.  With device == 0 only the pair structure and flop count
 * are computed (no data access).
 */
int
xmg_plan_build(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, plan_t *p, int device)
{
	/* device: 0 pairs only; 1 the full device plan (blocks staged);
	 * 2 the full structure with data handles in place of device
	 * addresses (no device needed: work-list checks) */
	xm_dim_t *list, nba, nbb, blkc, ia, ib, dims, dA, dB, ka, kb;
	size_t nlist, nblkk, l, i, la, lb, sta[XM_MAX_DIM], stb[XM_MAX_DIM];
	struct cand *cand = NULL;
	xmg_hmap_t merge;
	int64_t sa[XM_MAX_DIM], sb[XM_MAX_DIM], sc[XM_MAX_DIM];
	int32_t arow, acol, brow, bcol, ea = 0, eb = 0;
	struct xmg_block *ba, *bb;
	uint64_t rep, dptr;
	xmgd_cblock_t *cb;
	xmgd_pair_t *pr;
	int st = XMG_OK, sign, shift, emu;
	double mult = xmg_is_complex(c->type) ? 8.0 : 2.0;

	p->type = c->type;
	nba = xm_block_space_get_nblocks(a->bs);
	nbb = xm_block_space_get_nblocks(b->bs);
	nblkk = xm_dim_dot_mask(&nba, &p->cidxa);
	for (l = 0, sta[0] = stb[0] = 1; l + 1 < XM_MAX_DIM; l++) {
		sta[l + 1] = sta[l] * (l < nba.n ? nba.i[l] : 1);
		stb[l + 1] = stb[l] * (l < nbb.n ? nbb.i[l] : 1);
	}
	xm_tensor_get_canonical_block_list(c, &list, &nlist);
	if (nblkk > 0 && (cand = malloc(nblkk * sizeof *cand)) == NULL)
		xm_fatal("%s: out of memory", __func__);
	xmg_hmap_init(&merge);
	for (l = 0; l < nlist && st == XMG_OK; l++) {
		blkc = list[l];
		dims = xm_block_space_get_block_dims(c->bs, blkc);
		/* offsets inside a block are int32 on the device */
		if (xm_dim_dot(&dims) > INT32_MAX) {
			st = xmg_seterr(XMG_EINVAL, "xm_contract: a block of c has "
			    "more than 2^31 - 1 elements");
			break;
		}
		GROW(p->cb, p->ncb, p->capcb);
		GROW(p->emulatable, p->ncb, p->capem);
		cb = &p->cb[p->ncb];
		memset(cb, 0, sizeof *cb);
		cb->m = (int32_t)xm_dim_dot_mask(&dims, &p->cidxc);
		cb->n = (int32_t)xm_dim_dot_mask(&dims, &p->aidxc);
		cb->first_pair = p->npr;
		emu = 1;
		if (device) {
			xmg_canon_strides(&dims, sc);
			cb->crow = mask_table(&p->tabs, &dims, sc, &p->cidxc);
			cb->ccol = mask_table(&p->tabs, &dims, sc, &p->aidxc);
			dptr = xm_tensor_get_block_data_ptr(c, blkc);
			if (device == 1 && (st = xmg_alloc_device_view(c->allocator,
			    dptr, xm_tensor_get_block_bytes(c, blkc), &dptr)) != XMG_OK)
				break;
			cb->c_ptr = dptr;
		}
		if (alpha == 0)	/* contract.c:159-160: no GEMMs */
			goto next;
		/* enumerate (contract.c:161-179) */
		ia = xm_dim_zero(nba.n);
		ib = xm_dim_zero(nbb.n);
		xm_dim_set_mask(&ia, &p->aidxa, &blkc, &p->cidxc);
		xm_dim_set_mask(&ib, &p->aidxb, &blkc, &p->aidxc);
		la = xmg_tensor_block_linear(a, ia);
		lb = xmg_tensor_block_linear(b, ib);
		for (i = 0; i < nblkk; i++) {
			ba = &a->blocks[la];
			bb = &b->blocks[lb];
			cand[i].ia = ia;
			cand[i].ib = ib;
			cand[i].pa = ba;
			cand[i].pb = bb;
			cand[i].al = 0;
			if (ba->type != XM_BLOCK_TYPE_ZERO &&
			    bb->type != XM_BLOCK_TYPE_ZERO) {
				cand[i].al = xm_scalar_mul(ba->scalar,
				    bb->scalar, c->type);
				cand[i].da = block_data(a, ba);
				cand[i].db = block_data(b, bb);
			}
			la = inc_mask_linear(&ia, &nba, &p->cidxa, sta, la);
			lb = inc_mask_linear(&ib, &nbb, &p->cidxb, stb, lb);
		}
		/* merge (contract.c:180-192): first member of each class
		 * accumulates the others' factors in index order */
		xmg_hmap_clear(&merge);
		for (i = 0; i < nblkk; i++) {
			uint64_t h;
			if (cand[i].al == 0)
				continue;
			h = cand_hash(&cand[i], &p->aidxa, &p->aidxb);
			while (xmg_hmap_get(&merge, h, &rep) &&
			    !same_key(&cand[rep], &cand[i], &p->aidxa, &p->aidxb))
				h = xmg_hash64(h + 1);	/* collision: rehash */
			if (xmg_hmap_get(&merge, h, &rep)) {
				cand[rep].al = xm_scalar_add(cand[rep].al,
				    cand[i].al, c->type);
				cand[i].al = 0;
			} else
				xmg_hmap_put(&merge, h, i);
		}
		/* surviving pairs (contract.c:193-218) */
		for (i = 0; i < nblkk; i++) {
			if (cand[i].al == 0)
				continue;
			if (p->collect) {
				if (p->nbh == p->capbh) {
					p->capbh = p->capbh ? 2 * p->capbh : 256;
					if ((p->bh = realloc(p->bh, p->capbh *
					    sizeof *p->bh)) == NULL || (p->bsz =
					    realloc(p->bsz, p->capbh * sizeof *p->bsz)) == NULL)
						xm_fatal("%s: out of memory", __func__);
				}
				p->bh[p->nbh] = cand[i].db;
				p->bsz[p->nbh++] = xm_tensor_get_block_bytes(b, cand[i].ib);
			}
			dA = xm_block_space_get_block_dims(a->bs, cand[i].ia);
			dB = xm_block_space_get_block_dims(b->bs, cand[i].ib);
			if (xm_dim_dot(&dA) > INT32_MAX || xm_dim_dot(&dB) > INT32_MAX) {
				st = xmg_seterr(XMG_EINVAL, "xm_contract: a block of a "
				    "or b has more than 2^31 - 1 elements");
				break;
			}
			GROW(p->pr, p->npr, p->cappr);
			pr = &p->pr[p->npr++];
			memset(pr, 0, sizeof *pr);
			pr->k = (int32_t)xm_dim_dot_mask(&dA, &p->cidxa);
			xmg_scalar_pack(xm_scalar_mul(alpha, cand[i].al, c->type),
			    pr->al);
			p->flops += mult * cb->m * (double)cb->n * pr->k;
			if (!pow2_factor(cand[i].al, &sign, &shift))
				emu = 0;
			else {
				pr->esign = sign;
				pr->eshift = shift;
			}
			if (!device)
				continue;
			xmg_tensor_block_strides(a, cand[i].ia, sa);
			xmg_tensor_block_strides(b, cand[i].ib, sb);
			k_order(&p->cidxa, &p->cidxb, sa, sb,
			    (int64_t)pr->k * cb->m, (int64_t)pr->k * cb->n, &ka, &kb);
			arow = mask_table(&p->tabs, &dA, sa, &ka);
			acol = mask_table(&p->tabs, &dA, sa, &p->aidxa);
			brow = mask_table(&p->tabs, &dB, sb, &kb);
			bcol = mask_table(&p->tabs, &dB, sb, &p->aidxb);
			pr->arow = arow; pr->acol = acol;
			pr->brow = brow; pr->bcol = bcol;
			dptr = cand[i].da;
			if (device == 1 && (st = xmg_alloc_device_view(a->allocator,
			    cand[i].da, xm_tensor_get_block_bytes(a, cand[i].ia), &dptr)))
				break;
			pr->a_ptr = dptr;
			dptr = cand[i].db;
			if (device == 1 && (st = xmg_alloc_device_view(b->allocator,
			    cand[i].db, xm_tensor_get_block_bytes(b, cand[i].ib), &dptr)))
				break;
			pr->b_ptr = dptr;
			ea = exp_slot(&p->ea_index, &p->nexp_a, a, cand[i].ia,
			    &p->aidxa, cb->m);
			eb = exp_slot(&p->eb_index, &p->nexp_b, b, cand[i].ib,
			    &p->aidxb, cb->n);
			pr->aview = view_id(&p->va, &p->nva, &p->capva,
			    &p->va_index, pr->a_ptr, pr->k, cb->m, arow, acol, ea);
			pr->bview = view_id(&p->vb, &p->nvb, &p->capvb,
			    &p->vb_index, pr->b_ptr, pr->k, cb->n, brow, bcol, eb);
			cb->eA = ea;
			cb->eB = eb;
		}
next:
		cb->npairs = p->npr - cb->first_pair;
		p->emulatable[p->ncb] = (uint8_t)emu;
		p->ncb++;
	}
	xmg_hmap_free(&merge);
	free(cand);
	free(list);
	if (st == XMG_OK && p->tabs.overflow)
		st = xmg_seterr(XMG_EINVAL, "xm_contract: the contraction's "
		    "offset tables exceed 2^31 - 1 entries");
	return st;
}

void
xmg_plan_init(plan_t *p)
{
	memset(p, 0, sizeof *p);
	xmg_hmap_init(&p->tabs.index);
	xmg_hmap_init(&p->va_index);
	xmg_hmap_init(&p->vb_index);
	xmg_hmap_init(&p->ea_index);
	xmg_hmap_init(&p->eb_index);
}

double
xmg_contract_flops(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc)
{
	plan_t p;
	double f = -1;

	xmg_plan_init(&p);
	if (xmg_plan_check(a, b, c, idxa, idxb, idxc, &p) == XMG_OK &&
	    xmg_plan_build(1, a, b, c, &p, 0) == XMG_OK)
		f = p.flops;
	xmg_plan_free(&p);
	return f;
}

int
xmg_contract_pairs(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, xmg_pair_cb cb)
{
	plan_t p;
	int st, l, q;

	xmg_plan_init(&p);
	if ((st = xmg_plan_check(a, b, c, idxa, idxb, idxc, &p)) == XMG_OK &&
	    (st = xmg_plan_build(1, a, b, c, &p, 0)) == XMG_OK) {
		for (l = 0; l < p.ncb; l++)
			for (q = 0; q < p.cb[l].npairs; q++) {
				const xmgd_pair_t *pr = &p.pr[p.cb[l].first_pair + q];
				cb((size_t)l, pr->al[0], pr->al[1], p.cb[l].m,
				    p.cb[l].n, pr->k);
			}
	}
	xmg_plan_free(&p);
	return st;
}

static void
fill_contract(xmgd_contract_t *dp, const plan_t *p, xm_scalar_t alpha,
    xm_scalar_t beta, int prec)
{
	memset(dp, 0, sizeof *dp);
	dp->dtype = p->type;
	dp->precision = prec;
	xmg_scalar_pack(alpha, dp->alpha);
	xmg_scalar_pack(beta, dp->beta);
	dp->ncblocks = p->ncb;
	dp->npairs = p->npr;
	dp->cblocks = p->cb;
	dp->pairs = p->pr;
	dp->views_a = p->va;
	dp->views_b = p->vb;
	dp->nviews_a = p->nva;
	dp->nviews_b = p->nvb;
	dp->tabs = p->tabs.v;
	dp->ntabs = p->tabs.n;
	dp->nexp_a = p->nexp_a;
	dp->nexp_b = p->nexp_b;
	dp->flops = p->flops;
	dp->emulatable = p->emulatable;
}

int
xmg_work_list_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, int policy, long long out[4])
{
	xmgd_contract_t dp;
	plan_t p;
	int st;

	xmg_plan_init(&p);
	if ((st = xmg_plan_check(a, b, c, idxa, idxb, idxc, &p)) == XMG_OK &&
	    (st = xmg_plan_build(1, a, b, c, &p, 2)) == XMG_OK) {
		fill_contract(&dp, &p, 1, 0, XMG_PREC_EMU64);
		st = xmgd_work_list_check(&dp, policy, out);
	}
	xmg_plan_free(&p);
	return st;
}

/* ------------------------------------------------------------------ */
/* plan cache                                                          */

/*
 * Contractions repeat: an iterative solver calls the same xm_contract
 * every iteration on tensors whose block structure never changes.  A
 * device plan (uploaded metadata, work lists, captured CUDA graph) is kept
 * per (a, b, c, their structure generations, index strings, alpha, beta,
 * precision) and replayed; any block-table change draws a new generation,
 * so a stale plan can never match.  Only tensors whose blocks live in GPU
 * memory are cached (pagefile blocks are staged per call).
 */
#define PC_MAX 16

struct pc_entry {
	const xm_tensor_t *a, *b, *c;
	uint64_t ga, gb, gc;
	char idx[3][16];
	xm_scalar_t alpha, beta;
	int precision;
	xmgd_plan_t *dp;
	double flops;
	int ncb, npr;
	uint64_t used;
};
static struct pc_entry g_pc[PC_MAX];
static uint64_t g_pc_tick;
static int g_pc_slots = -1;

static int
pc_slots(void)
{
	const char *e;

	if (g_pc_slots < 0) {
		g_pc_slots = 8;
		if ((e = getenv("XMG_PLAN_CACHE")) != NULL)
			g_pc_slots = atoi(e);
		if (g_pc_slots < 0)
			g_pc_slots = 0;
		if (g_pc_slots > PC_MAX)
			g_pc_slots = PC_MAX;
	}
	return g_pc_slots;
}

static int
pc_match(const struct pc_entry *e, xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, xm_scalar_t beta, const xm_tensor_t *c,
    const char *idxa, const char *idxb, const char *idxc, int prec)
{
	return e->dp != NULL && e->a == a && e->b == b && e->c == c &&
	    e->ga == a->gen && e->gb == b->gen && e->gc == c->gen &&
	    e->alpha == alpha && e->beta == beta && e->precision == prec &&
	    strcmp(e->idx[0], idxa) == 0 && strcmp(e->idx[1], idxb) == 0 &&
	    strcmp(e->idx[2], idxc) == 0;
}

static void
pc_drop(struct pc_entry *e)
{
	if (e->dp)
		xmgd_plan_free(e->dp);
	memset(e, 0, sizeof *e);
}

void
xmg_plan_cache_clear(void)
{
	int i;

	for (i = 0; i < PC_MAX; i++)
		pc_drop(&g_pc[i]);
	xmg_stream_release();
	xmg_adjoint_release();
}

static void
stats_from(double flops, int ncb, int npr, int precision_used, double t0)
{
	xmgd_timing_t tm;

	xmgd_last_timing(&tm);
	xmg_last_stats.flops = flops;
	xmg_last_stats.ms_device = tm.ms_total;
	xmg_last_stats.ms_split = tm.ms_split;
	xmg_last_stats.ms_gemm = tm.ms_gemm;
	xmg_last_stats.n_cblocks = ncb;
	xmg_last_stats.n_pairs = npr;
	xmg_last_stats.slice_bytes = tm.slice_bytes;
	xmg_last_stats.precision_used = precision_used;
	xmg_last_stats.gemm_launches = tm.gemm_launches;
	xmg_last_stats.gemm_policy = tm.gemm_policy;
	(void)t0;
}

int
xmg_contract(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc)
{
	xmgd_contract_t dp;
	xmgd_plan_t *h = NULL;
	struct pc_entry *e = NULL;
	plan_t p;
	double t0 = xmg_now_ms();
	int st, i, prec = precision_mode(), used = XMG_PREC_FP64, cache;

	xmg_plan_init(&p);
	if ((st = xmg_plan_check(a, b, c, idxa, idxb, idxc, &p)) != XMG_OK)
		goto out;
	if ((st = xmgd_init()) != XMG_OK)
		goto out;
	memset(&xmg_last_stats, 0, sizeof xmg_last_stats);
	if (!xmg_alloc_is_device(c->allocator) && xmg_contract_streamed(alpha, a, b,
	    beta, c, idxa, idxb, idxc, prec, &st))
		goto out;
	cache = pc_slots() > 0 && xmg_alloc_is_device(c->allocator) &&
	    strlen(idxa) < 16 && strlen(idxb) < 16 && strlen(idxc) < 16;
	if (cache) {
		for (i = 0; i < pc_slots(); i++)
			if (pc_match(&g_pc[i], alpha, a, b, beta, c, idxa, idxb,
			    idxc, prec))
				e = &g_pc[i];
		if (e) {
			e->used = ++g_pc_tick;
			xmg_last_stats.ms_plan = xmg_now_ms() - t0;
			st = xmgd_plan_run(e->dp, &used);
			stats_from(e->flops, e->ncb, e->npr, used, t0);
			if (st != XMG_OK)
				pc_drop(e);
			goto out;
		}
	}
	if ((st = xmg_plan_build(alpha, a, b, c, &p, 1)) != XMG_OK) {
		st = xmg_commit_c(c, st);
		goto out;
	}
	fill_contract(&dp, &p, alpha, beta, prec);
	if ((st = xmgd_plan_create(&dp, &h)) != XMG_OK) {
		st = xmg_commit_c(c, st);
		goto out;
	}
	xmg_last_stats.ms_plan = xmg_now_ms() - t0;
	st = xmgd_plan_run(h, &used);
	stats_from(p.flops, p.ncb, p.npr, used, t0);
	if (cache && st == XMG_OK) {
		/* keep it: the least recently used slot gives way */
		e = &g_pc[0];
		for (i = 1; i < pc_slots(); i++)
			if (g_pc[i].used < e->used)
				e = &g_pc[i];
		pc_drop(e);
		e->a = a; e->b = b; e->c = c;
		e->ga = a->gen; e->gb = b->gen; e->gc = c->gen;
		strcpy(e->idx[0], idxa);
		strcpy(e->idx[1], idxb);
		strcpy(e->idx[2], idxc);
		e->alpha = alpha;
		e->beta = beta;
		e->precision = prec;
		e->dp = h;
		e->flops = p.flops;
		e->ncb = p.ncb;
		e->npr = p.npr;
		e->used = ++g_pc_tick;
		h = NULL;
	}
	if (h)
		xmgd_plan_free(h);
	st = xmg_commit_c(c, st);
out:
	xmg_plan_free(&p);
	return st;
}

void
xm_contract(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc)
{
	xmg_die_on(xmg_contract(alpha, a, b, beta, c, idxa, idxb, idxc));
}

int
xmg_synchronize(void)
{
	return xmgd_sync();
}
