/*
 * Hand-written adjoint of xm_contract (no counterpart in the reference).
 *
 * Forward: the canonical blocks of c are c = alpha * a * b over the index
 * strings (contract.c:227-314); derivative blocks of c are permuted,
 * scaled views.  With dc of the same block space, the loss is the xm_dot
 * pairing over every block (xm.c:472-497):
 *     L = sum_x s_c(x) s_dc(x) < perm_c(x)(c_src), perm_dc(x)(dc_src) >
 * so dL/d(canonical c block q) = W_q = sum over blocks x whose c-source is
 * q of s_c(x) s_dc(x) * (dc's data of x mapped into q's layout).
 * By bilinearity
 *     G_A = alpha * W * b   (index strings idxc, idxb -> idxa)
 *     G_B = alpha * a * W   (index strings idxa, idxc -> idxb)
 * give the gradient at every nonzero block position x of a (resp. b); the
 * canonical gradient folds them back, dA_q += sum_{x -> q} s_a(x) *
 * (G_A at x mapped into q's layout) -- the derivative blocks' permutations
 * and scalars applied in reverse.  Both contractions run on the engine's
 * own kernels (split-precision or plain, as configured).
 */
#include "xmg_host.h"

/* Scatter-add "dst block q += f * src block x" for every nonzero block x of
 * the structure tensor st, where q = canonical source of x in st.  Element
 * e of x sits at q's data + sum e_d * stride_st(x)[d] and at src's data +
 * sum e_d * stride_src(x)[d].  Blocks sharing a q run in separate rounds. */
static int
fold_onto_canonical(const xm_tensor_t *st, xm_tensor_t *dst,
    const xm_tensor_t *src, int src_scalar)
{
	xm_dim_t nb = xm_block_space_get_nblocks(st->bs), idx, dims;
	size_t nblk = st->nblocks_total, i, round;
	int64_t size[XM_MAX_DIM], ds[XM_MAX_DIM], ss[XM_MAX_DIM];
	unsigned char *done;
	int *taken, st_ = XMG_OK, left = 1;
	xmg_ptask_list_t l = {0};
	struct xmg_block *bx, *bs;
	xm_scalar_t f;
	uint64_t dptr, sptr;
	size_t k;

	if ((done = calloc(nblk, 1)) == NULL ||
	    (taken = calloc(nblk, sizeof *taken)) == NULL) {
		free(done);
		return xmg_seterr(XMG_ENOMEM, "out of memory");
	}
	for (round = 0; left && st_ == XMG_OK; round++) {
		left = 0;
		memset(taken, 0, nblk * sizeof *taken);
		idx = xm_dim_zero(nb.n);
		for (i = 0; i < nblk; i++, xm_dim_inc(&idx, &nb)) {
			size_t q;
			bx = &st->blocks[i];
			if (done[i] || bx->type == XM_BLOCK_TYPE_ZERO) {
				done[i] = 1;
				continue;
			}
			bs = &src->blocks[i];
			if (bs->type == XM_BLOCK_TYPE_ZERO) {
				done[i] = 1;
				continue;
			}
			q = bx->type == XM_BLOCK_TYPE_CANONICAL ? i : (size_t)bx->data;
			if (taken[q]) {
				left = 1;
				continue;
			}
			taken[q] = 1;
			done[i] = 1;
			dims = xm_block_space_get_block_dims(st->bs, idx);
			xmg_tensor_block_strides(st, idx, ds);
			xmg_tensor_block_strides(src, idx, ss);
			for (k = 0; k < dims.n; k++)
				size[k] = (int64_t)dims.i[k];
			f = bx->scalar;
			if (src_scalar)
				f = xm_scalar_mul(f, bs->scalar, st->type);
			if ((st_ = xmg_alloc_device_view(dst->allocator,
			    dst->blocks[q].data, xm_tensor_get_block_bytes(dst, idx),
			    &dptr)) != XMG_OK ||
			    (st_ = xmg_alloc_device_view(src->allocator,
			    xm_tensor_get_block_data_ptr(src, idx),
			    xm_tensor_get_block_bytes(src, idx), &sptr)) != XMG_OK)
				break;
			xmgd_ptask_t *t = xmg_ptask_push(&l);
			t->op = XMGD_OP_AXPY;
			t->dst = dptr;
			t->src = sptr;
			t->alpha[0] = 1;
			xmg_scalar_pack(f, t->beta);
			xmg_ptask_shape(t, (int)dims.n, size, ds, ss);
		}
		if (st_ == XMG_OK)
			st_ = xmg_ptask_run(&l, dst->type, src->type, NULL);
		l.n = 0;
	}
	xmg_ptask_list_free(&l);
	free(done);
	free(taken);
	return st_;
}

/* Tensor on t's block space whose canonical blocks sit at t's canonical
 * positions only (or at every nonzero position of t), zero-filled. */
static xm_tensor_t *
gradient_tensor(const xm_tensor_t *t, int all_nonzero)
{
	xm_tensor_t *g = xm_tensor_create(t->bs, t->type, t->allocator);
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs), idx = xm_dim_zero(nb.n);
	size_t i;

	for (i = 0; i < t->nblocks_total; i++, xm_dim_inc(&idx, &nb)) {
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL ||
		    (all_nonzero && t->blocks[i].type == XM_BLOCK_TYPE_DERIVATIVE))
			xm_tensor_set_canonical_block(g, idx);
	}
	return g;
}

static void
drop(xm_tensor_t *t)
{
	if (t) {
		xm_tensor_free_block_data(t);
		xm_tensor_free(t);
	}
}

static int
same_space(const xm_tensor_t *x, const xm_tensor_t *y)
{
	return x->type == y->type && x->allocator == y->allocator &&
	    xm_block_space_eq(x->bs, y->bs);
}

/*
 * The intermediates of the last adjoint call -- W and the two gradient
 * tensors at every nonzero position -- are kept while a, b and dc keep
 * their block structures (and so are the device plans of the two
 * gradient contractions, which the plan cache keys on these tensors): a
 * training-style loop that calls the adjoint every step plans and
 * allocates once.  xmg_adjoint_release (and xmg_plan_cache_clear) frees
 * them.
 */
static struct {
	const xm_tensor_t *a, *b, *dc;
	uint64_t ga_gen, gb_gen, gdc_gen;
	xm_tensor_t *w, *ga, *gb;
} g_adj;

void
xmg_adjoint_release(void)
{
	drop(g_adj.w);
	drop(g_adj.ga);
	drop(g_adj.gb);
	memset(&g_adj, 0, sizeof g_adj);
}

/* The kept intermediates live in the operands' allocator: its
 * destruction releases them first (xm_allocator_destroy). */
void
xmg_adjoint_forget(const xm_allocator_t *al)
{
	if (g_adj.w != NULL && g_adj.w->allocator == al)
		xmg_adjoint_release();
}

int
xm_contract_adjoint(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, const xm_tensor_t *dc, xm_tensor_t *da,
    xm_tensor_t *db, const char *idxa, const char *idxb, const char *idxc)
{
	xm_tensor_t *w = NULL, *ga = NULL, *gb = NULL;
	int st, kept;

	if (a == NULL || b == NULL || dc == NULL)
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: invalid "
		    "argument");
	if ((da && !same_space(da, a)) || (db && !same_space(db, b)))
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: gradient "
		    "tensors must share the operands' block spaces, types and "
		    "allocator");
	if (a->type != dc->type || a->allocator != dc->allocator)
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: dc must "
		    "match the operands' type and allocator");
	kept = g_adj.w != NULL && g_adj.a == a && g_adj.b == b &&
	    g_adj.dc == dc && g_adj.ga_gen == a->gen && g_adj.gb_gen == b->gen &&
	    g_adj.gdc_gen == dc->gen && xmg_alloc_is_device(a->allocator);
	if (!kept) {
		xmg_adjoint_release();
		/* W: dc folded onto dc's own canonical positions (c and dc
		 * share their block structure; the structure tensor is dc) */
		w = gradient_tensor(dc, 0);
	} else
		w = g_adj.w;
	if ((st = xmg_set(w, 0)) != XMG_OK ||
	    (st = fold_onto_canonical(dc, w, dc, 1)) != XMG_OK)
		goto out;
	if (da) {
		if ((ga = kept ? g_adj.ga : NULL) == NULL)
			ga = gradient_tensor(a, 1);
		if ((st = xmg_contract(alpha, w, b, 0, ga, idxc, idxb, idxa)) !=
		    XMG_OK || (st = fold_onto_canonical(a, da, ga, 0)) != XMG_OK)
			goto out;
	}
	if (db) {
		if ((gb = kept ? g_adj.gb : NULL) == NULL)
			gb = gradient_tensor(b, 1);
		if ((st = xmg_contract(alpha, a, w, 0, gb, idxa, idxc, idxb)) !=
		    XMG_OK || (st = fold_onto_canonical(b, db, gb, 0)) != XMG_OK)
			goto out;
	}
	st = xmgd_sync();
out:
	if (st == XMG_OK && xmg_alloc_is_device(a->allocator)) {
		/* keep the intermediates for the next call */
		g_adj.a = a; g_adj.b = b; g_adj.dc = dc;
		g_adj.ga_gen = a->gen; g_adj.gb_gen = b->gen;
		g_adj.gdc_gen = dc->gen;
		g_adj.w = w;
		if (ga)
			g_adj.ga = ga;
		if (gb)
			g_adj.gb = gb;
		return st;
	}
	if (w != g_adj.w)
		drop(w);
	if (ga != g_adj.ga)
		drop(ga);
	if (gb != g_adj.gb)
		drop(gb);
	if (st != XMG_OK)
		xmg_adjoint_release();
	return st;
}
