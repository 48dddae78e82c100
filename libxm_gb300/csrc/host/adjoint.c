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
 * and scalars applied in reverse (the every-position form, exact for any
 * block structure).  When the structures are consistent with the
 * contraction, the symmetric form below computes each gradient at the
 * canonical positions only.  Both contractions run on the engine's own
 * kernels (split-precision or plain, as configured).
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

/*
 * Symmetric form.  When the block structures are consistent with the
 * contraction, the gradient at a derivative position is the permuted,
 * scaled gradient at its canonical source, so the gradient contractions
 * need only the canonical positions:
 *
 * For a target T = X * Y (T = a: X = dc, Y = b; T = b: X = a, Y = dc;
 * and T = dc: X = a, Y = b for the forward itself) and a derivative block
 * p of T with source q, permutation P and scalar s (element e of p is
 * element f of q with f[P[k]] = e[k], tensor.c:167-171), the letter map
 * phi(it[k]) = it[P[k]] (the identity on summed letters) must send every
 * nonzero term X(z) Y(w) of T at p onto the term X(z') Y(w') at q: same
 * canonical data, element strides related through phi, and scalar ratios
 * whose product sigma is one number for all terms.  Then T*(p) =
 * sigma P T*(q) for the contraction T* = X * Y, whatever the data.
 *
 * The forward check (T = dc) makes the loss the pairing of dc with the
 * contraction at every nonzero position of c, L = sum_x dc(x) (a * b)(x),
 * which holds when sigma equals dc's own scalar at every derivative
 * position.  Then dL/da at position p is G(p) = alpha * (dc * b)(p) (dc
 * taken at every position, derivative blocks included), and for a
 * canonical block q of a
 *     dA_q = sum_{p -> q} s_p P_p^-1 G(p) = m_q G(q),
 *     m_q = 1 + sum over derivative p of q of s_p sigma_p,
 * so one contraction into a's canonical positions and a per-block scale
 * give dA (likewise dB).  For the antisymmetric ladder this is the work of
 * one forward contraction per gradient instead of about 1.5 (every
 * position).  Any failed check keeps the every-position form.
 */

/* position of letter ch in s, -1 if absent */
static int
letter(const char *s, char ch)
{
	const char *p = strchr(s, ch);
	return p != NULL && ch != '\0' ? (int)(p - s) : -1;
}

/* Block of operand o (letters io) at target position v (letters it) and
 * summed block indices u (in o's dims; the target's letters are taken
 * from v). */
static xm_dim_t
operand_block(const char *io, const char *it, xm_dim_t v, xm_dim_t u)
{
	size_t j;

	for (j = 0; j < u.n; j++) {
		int k = letter(it, io[j]);
		if (k >= 0)
			u.i[j] = v.i[k];
	}
	return u;
}

/* canonical source (linear index) and element strides of block z of t;
 * 0 for a zero block */
static int
block_map(const xm_tensor_t *t, xm_dim_t z, size_t *src, int64_t *str,
    xm_scalar_t *sc)
{
	struct xmg_block *b = xmg_tensor_block(t, z);

	if (b->type == XM_BLOCK_TYPE_ZERO)
		return 0;
	*src = b->type == XM_BLOCK_TYPE_CANONICAL ?
	    xmg_tensor_block_linear(t, z) : (size_t)b->data;
	*sc = b->scalar;
	xmg_tensor_block_strides(t, z, str);
	return 1;
}

#define EQV_NO     0	/* not equivariant */
#define EQV_YES    1	/* T*(p) = sigma P T*(q) */
#define EQV_EMPTY  2	/* no nonzero term at p or q */

/* Equivariance of T = X * Y at derivative position p of T (letters it,
 * ix, iy); *sigma on EQV_YES. */
static int
equivariant(const xm_tensor_t *t, const char *it, const xm_tensor_t *x,
    const char *ix, const xm_tensor_t *y, const char *iy, xm_dim_t p,
    xm_scalar_t *sigma)
{
	struct xmg_block *bp = xmg_tensor_block(t, p);
	const xm_tensor_t *op[2] = { x, y };
	const char *io[2] = { ix, iy };
	xm_dim_t nbt = xm_block_space_get_nblocks(t->bs), q, nbx, u[2];
	int sl[XM_MAX_DIM], ns = 0, have = 0;
	size_t cnt[XM_MAX_DIM], cur[XM_MAX_DIM], k, j, lin;
	xm_scalar_t s0 = 0;

	/* q from the linear source index; block indices related like the
	 * element indices; letter classes kept */
	q = xm_dim_zero(nbt.n);
	for (lin = (size_t)bp->data, k = 0; k < nbt.n; k++) {
		q.i[k] = lin % nbt.i[k];
		lin /= nbt.i[k];
	}
	for (k = 0; k < nbt.n; k++) {
		size_t pk = bp->perm.i[k];
		if (p.i[k] != q.i[pk] ||
		    (letter(ix, it[k]) >= 0) != (letter(ix, it[pk]) >= 0))
			return EQV_NO;
	}
	/* summed letters: in x and y, not in t */
	nbx = xm_block_space_get_nblocks(x->bs);
	for (j = 0; j < nbx.n; j++)
		if (letter(it, ix[j]) < 0 && letter(iy, ix[j]) >= 0) {
			sl[ns] = (int)j;
			cnt[ns] = nbx.i[j];
			cur[ns++] = 0;
		}
	for (;;) {
		int zero[2] = { 0, 0 };
		xm_scalar_t ratio[2];
		u[0] = xm_dim_zero(strlen(ix));
		u[1] = xm_dim_zero(strlen(iy));
		for (k = 0; k < (size_t)ns; k++) {
			u[0].i[sl[k]] = cur[k];
			u[1].i[letter(iy, ix[sl[k]])] = cur[k];
		}
		for (int o = 0; o < 2; o++) {
			xm_dim_t z = operand_block(io[o], it, p, u[o]);
			xm_dim_t zq = operand_block(io[o], it, q, u[o]);
			xm_dim_t dz, dq;
			int64_t sz[XM_MAX_DIM], sq[XM_MAX_DIM];
			size_t src, srcq;
			xm_scalar_t cz, cq;
			int nz = block_map(op[o], z, &src, sz, &cz);
			int nq = block_map(op[o], zq, &srcq, sq, &cq);

			if (nz != nq)
				return EQV_NO;
			if (!nz) {
				zero[o] = 1;
				continue;
			}
			if (src != srcq || cq == 0)
				return EQV_NO;
			dz = xm_block_space_get_block_dims(op[o]->bs, z);
			dq = xm_block_space_get_block_dims(op[o]->bs, zq);
			for (j = 0; j < dz.n; j++) {
				int kt = letter(it, io[o][j]);
				int jj = kt < 0 ? (int)j :
				    letter(io[o], it[bp->perm.i[kt]]);
				if (jj < 0 || dz.i[j] != dq.i[jj] ||
				    (dz.i[j] > 1 && sz[j] != sq[jj]))
					return EQV_NO;
			}
			ratio[o] = cz / cq;
		}
		if (!zero[0] && !zero[1]) {
			xm_scalar_t s = ratio[0] * ratio[1];
			if (have && s != s0)
				return EQV_NO;
			s0 = s;
			have = 1;
		}
		for (k = 0; k < (size_t)ns; k++) {
			if (++cur[k] < cnt[k])
				break;
			cur[k] = 0;
		}
		if (k == (size_t)ns)
			break;
	}
	*sigma = s0;
	return have ? EQV_YES : EQV_EMPTY;
}

/* The forward check: the contraction a * b agrees with dc's (= c's)
 * derivative blocks at every derivative position. */
static int
forward_consistent(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *dc, const char *idxa, const char *idxb,
    const char *idxc)
{
	xm_dim_t nb = xm_block_space_get_nblocks(dc->bs), idx;
	size_t i;

	idx = xm_dim_zero(nb.n);
	for (i = 0; i < dc->nblocks_total; i++, xm_dim_inc(&idx, &nb)) {
		xm_scalar_t sig;
		int r;
		if (dc->blocks[i].type != XM_BLOCK_TYPE_DERIVATIVE)
			continue;
		r = equivariant(dc, idxc, a, idxa, b, idxb, idx, &sig);
		if (r == EQV_NO || (r == EQV_YES && sig != dc->blocks[i].scalar))
			return 0;
	}
	return 1;
}

/* Per-block factors m (indexed by t's linear block index; nonzero only
 * at canonical blocks) of the symmetric form for target t = x * y, or 0
 * when some derivative position of t fails the check. */
static int
canonical_factors(const xm_tensor_t *t, const char *it,
    const xm_tensor_t *x, const char *ix, const xm_tensor_t *y,
    const char *iy, xm_scalar_t *m)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs), idx;
	size_t i;

	for (i = 0; i < t->nblocks_total; i++)
		m[i] = t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL ? 1 : 0;
	idx = xm_dim_zero(nb.n);
	for (i = 0; i < t->nblocks_total; i++, xm_dim_inc(&idx, &nb)) {
		struct xmg_block *bp = &t->blocks[i];
		xm_scalar_t sig;
		int r;
		if (bp->type != XM_BLOCK_TYPE_DERIVATIVE)
			continue;
		r = equivariant(t, it, x, ix, y, iy, idx, &sig);
		if (r == EQV_NO)
			return 0;
		/* EQV_EMPTY: the gradient is zero at p and at q, any factor
		 * serves; count the position like a consistent one */
		m[bp->data] += r == EQV_YES ? bp->scalar * sig : 1;
	}
	return 1;
}

/* dst_q += m_q * src_q for every canonical block q of t (dst and src on
 * t's block space; one task per block, no two share a target). */
static int
scale_add_canonical(const xm_tensor_t *t, xm_tensor_t *dst,
    const xm_tensor_t *src, const xm_scalar_t *m)
{
	xm_dim_t nb = xm_block_space_get_nblocks(t->bs), idx, dims;
	xmg_ptask_list_t l = {0};
	int64_t size[XM_MAX_DIM], str[XM_MAX_DIM];
	uint64_t dptr, sptr;
	size_t i, k;
	int st = XMG_OK;

	idx = xm_dim_zero(nb.n);
	for (i = 0; i < t->nblocks_total && st == XMG_OK;
	    i++, xm_dim_inc(&idx, &nb)) {
		if (t->blocks[i].type != XM_BLOCK_TYPE_CANONICAL || m[i] == 0)
			continue;
		dims = xm_block_space_get_block_dims(t->bs, idx);
		xmg_canon_strides(&dims, str);
		for (k = 0; k < dims.n; k++)
			size[k] = (int64_t)dims.i[k];
		if ((st = xmg_alloc_device_view(dst->allocator,
		    dst->blocks[i].data, xm_tensor_get_block_bytes(dst, idx),
		    &dptr)) != XMG_OK ||
		    (st = xmg_alloc_device_view(src->allocator,
		    src->blocks[i].data, xm_tensor_get_block_bytes(src, idx),
		    &sptr)) != XMG_OK)
			break;
		xmgd_ptask_t *tk = xmg_ptask_push(&l);
		tk->op = XMGD_OP_AXPY;
		tk->dst = dptr;
		tk->src = sptr;
		tk->alpha[0] = 1;
		xmg_scalar_pack(m[i], tk->beta);
		xmg_ptask_shape(tk, (int)dims.n, size, str, str);
	}
	if (st == XMG_OK)
		st = xmg_ptask_run(&l, dst->type, src->type, NULL);
	xmg_ptask_list_free(&l);
	return st;
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
 * The intermediates of the last adjoint call -- the checks' outcome, the
 * factors of the symmetric form, W and the gradient tensors -- are kept
 * while a, b and dc keep their block structures (and so are the device
 * plans of the two gradient contractions, which the plan cache keys on
 * these tensors): a training-style loop that calls the adjoint every step
 * checks, plans and allocates once.  xmg_adjoint_release (and
 * xmg_plan_cache_clear) frees them.
 */
#define SIDE_UNSET  0
#define SIDE_SYM    1	/* canonical positions, per-block factors */
#define SIDE_EVERY  2	/* every nonzero position, folded */

struct adj_side {
	int mode;
	xm_scalar_t *m;		/* SIDE_SYM: factors per block of a (b) */
	xm_tensor_t *g;		/* gradient at canonical or every position */
};

static struct {
	const xm_tensor_t *a, *b, *dc;	/* identity only: never dereferenced,
					   they may have been freed since */
	const xm_allocator_t *al_a, *al_b;	/* where the kept tensors live */
	uint64_t ga_gen, gb_gen, gdc_gen;
	char idx[3][XM_MAX_DIM + 1];
	int fwd;		/* forward check: -1 not run, 0 failed, 1 passed */
	xm_tensor_t *w;
	struct adj_side s[2];	/* 0: a, 1: b */
} g_adj = { .fwd = -1 };

void
xmg_adjoint_release(void)
{
	int k;

	drop(g_adj.w);
	for (k = 0; k < 2; k++) {
		drop(g_adj.s[k].g);
		free(g_adj.s[k].m);
	}
	memset(&g_adj, 0, sizeof g_adj);
	g_adj.fwd = -1;
}

/* The kept intermediates live in the operands' allocator: its
 * destruction releases them first (xm_allocator_destroy). */
void
xmg_adjoint_forget(const xm_allocator_t *al)
{
	if (al != NULL && (g_adj.al_a == al || g_adj.al_b == al))
		xmg_adjoint_release();
}

static int
symmetric_form_off(void)
{
	const char *e = getenv("XMG_ADJOINT_EVERY");
	return e != NULL && atoi(e) != 0;
}

/* Which form side k (0: gradient of a, 1: of b) takes; the checks run
 * once per kept structure. */
static int
side_mode(int k, const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *dc, const char *idxa, const char *idxb,
    const char *idxc)
{
	struct adj_side *sd = &g_adj.s[k];
	const xm_tensor_t *t = k ? b : a;

	if (sd->mode != SIDE_UNSET)
		return sd->mode;
	sd->mode = SIDE_EVERY;
	if (symmetric_form_off())
		return sd->mode;
	if (g_adj.fwd < 0)
		g_adj.fwd = forward_consistent(a, b, dc, idxa, idxb, idxc);
	if (!g_adj.fwd)
		return sd->mode;
	if ((sd->m = malloc(t->nblocks_total * sizeof *sd->m)) == NULL)
		return sd->mode;
	if (k == 0 ? canonical_factors(a, idxa, dc, idxc, b, idxb, sd->m) :
	    canonical_factors(b, idxb, a, idxa, dc, idxc, sd->m))
		sd->mode = SIDE_SYM;
	else {
		free(sd->m);
		sd->m = NULL;
	}
	return sd->mode;
}

/* Every canonical block of t is canonical in d too (the gradient's
 * targets). */
static int
same_canonical(const xm_tensor_t *t, const xm_tensor_t *d)
{
	size_t i;

	for (i = 0; i < t->nblocks_total; i++)
		if (t->blocks[i].type == XM_BLOCK_TYPE_CANONICAL &&
		    d->blocks[i].type != XM_BLOCK_TYPE_CANONICAL)
			return 0;
	return 1;
}

int
xm_contract_adjoint(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, const xm_tensor_t *dc, xm_tensor_t *da,
    xm_tensor_t *db, const char *idxa, const char *idxb, const char *idxc)
{
	xm_tensor_t *d[2] = { da, db };
	int st = XMG_OK, k, w_ready = 0;

	if (a == NULL || b == NULL || dc == NULL || idxa == NULL ||
	    idxb == NULL || idxc == NULL)
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: invalid "
		    "argument");
	if ((da && !same_space(da, a)) || (db && !same_space(db, b)))
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: gradient "
		    "tensors must share the operands' block spaces, types and "
		    "allocator");
	if ((da && !same_canonical(a, da)) || (db && !same_canonical(b, db)))
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: every "
		    "canonical block of a (b) must be canonical in da (db)");
	if (a->type != dc->type || a->allocator != dc->allocator)
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: dc must "
		    "match the operands' type and allocator");
	if (strlen(idxa) > XM_MAX_DIM || strlen(idxb) > XM_MAX_DIM ||
	    strlen(idxc) > XM_MAX_DIM)
		return xmg_seterr(XMG_EINVAL, "xm_contract_adjoint: invalid "
		    "index string");
	if (!(g_adj.a == a && g_adj.b == b && g_adj.dc == dc &&
	    g_adj.ga_gen == a->gen && g_adj.gb_gen == b->gen &&
	    g_adj.gdc_gen == dc->gen && strcmp(g_adj.idx[0], idxa) == 0 &&
	    strcmp(g_adj.idx[1], idxb) == 0 && strcmp(g_adj.idx[2], idxc) == 0 &&
	    xmg_alloc_is_device(a->allocator))) {
		xmg_adjoint_release();
		g_adj.a = a; g_adj.b = b; g_adj.dc = dc;
		g_adj.al_a = a->allocator;
		g_adj.al_b = b->allocator;
		g_adj.ga_gen = a->gen; g_adj.gb_gen = b->gen;
		g_adj.gdc_gen = dc->gen;
		strcpy(g_adj.idx[0], idxa);
		strcpy(g_adj.idx[1], idxb);
		strcpy(g_adj.idx[2], idxc);
	}
	for (k = 0; k < 2 && st == XMG_OK; k++) {
		const xm_tensor_t *t = k ? b : a;
		struct adj_side *sd = &g_adj.s[k];
		if (d[k] == NULL)
			continue;
		if (side_mode(k, a, b, dc, idxa, idxb, idxc) == SIDE_SYM) {
			/* G = alpha * (dc * b) or alpha * (a * dc) at t's
			 * canonical positions; d_q += m_q G_q */
			if (sd->g == NULL)
				sd->g = gradient_tensor(t, 0);
			st = k == 0 ?
			    xmg_contract(alpha, dc, b, 0, sd->g, idxc, idxb, idxa) :
			    xmg_contract(alpha, a, dc, 0, sd->g, idxa, idxc, idxb);
			if (st == XMG_OK)
				st = scale_add_canonical(t, d[k], sd->g, sd->m);
			continue;
		}
		/* W: dc folded onto dc's own canonical positions (c and dc
		 * share their block structure; the structure tensor is dc) */
		if (!w_ready) {
			if (g_adj.w == NULL)
				g_adj.w = gradient_tensor(dc, 0);
			if ((st = xmg_set(g_adj.w, 0)) != XMG_OK ||
			    (st = fold_onto_canonical(dc, g_adj.w, dc, 1)) !=
			    XMG_OK)
				break;
			w_ready = 1;
		}
		if (sd->g == NULL)
			sd->g = gradient_tensor(t, 1);
		st = k == 0 ?
		    xmg_contract(alpha, g_adj.w, b, 0, sd->g, idxc, idxb, idxa) :
		    xmg_contract(alpha, a, g_adj.w, 0, sd->g, idxa, idxc, idxb);
		if (st == XMG_OK)
			st = fold_onto_canonical(t, d[k], sd->g, 0);
	}
	if (st == XMG_OK)
		st = xmgd_sync();
	/* tensors outside GPU memory keep nothing; a failed call neither */
	if (st != XMG_OK || !xmg_alloc_is_device(a->allocator))
		xmg_adjoint_release();
	return st;
}

/* Host-only: the form each gradient would take for these tensors (0: a,
 * 1: b; 1 symmetric, 2 every position) and, for the symmetric form, the
 * factor of each block of a (b) (nblocks entries each, re/im pairs);
 * factors may be NULL.  Runs the structural checks only. */
int
xmg_adjoint_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *dc, const char *idxa, const char *idxb,
    const char *idxc, int mode[2], double *fa, double *fb)
{
	double *f[2] = { fa, fb };
	int k;
	size_t i;

	if (a == NULL || b == NULL || dc == NULL || idxa == NULL ||
	    idxb == NULL || idxc == NULL || mode == NULL ||
	    strlen(idxa) > XM_MAX_DIM || strlen(idxb) > XM_MAX_DIM ||
	    strlen(idxc) > XM_MAX_DIM)
		return xmg_seterr(XMG_EINVAL, "xmg_adjoint_plan_check: invalid "
		    "argument");
	xmg_adjoint_release();
	for (k = 0; k < 2; k++) {
		const xm_tensor_t *t = k ? b : a;
		mode[k] = side_mode(k, a, b, dc, idxa, idxb, idxc);
		if (f[k] != NULL)
			for (i = 0; i < t->nblocks_total; i++) {
				xm_scalar_t v = mode[k] == SIDE_SYM ?
				    g_adj.s[k].m[i] : 0;
				f[k][2 * i] = creal(v);
				f[k][2 * i + 1] = cimag(v);
			}
	}
	xmg_adjoint_release();
	return XMG_OK;
}
