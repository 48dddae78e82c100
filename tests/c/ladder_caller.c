/*
 * A C caller of the libxm API, linked against the GB300 engine
 * (libxmgb.so) exactly as a user program links against libxm: the
 * calling pattern of the reference's example.c:30-105 (block spaces,
 * tensors with canonical and derivative blocks, write_block, xm_set,
 * xm_contract, read back), on a small antisymmetric ladder.
 *
 *     ladder_caller EXPECTED_FILE
 *
 * Structure: o = 7 split 4 + 3, v = 11 split 5 + 6; A(i,j,c,d), B(c,d,a,b)
 * and C(i,j,a,b) antisymmetric under i<->j, c<->d and a<->b (derivative
 * blocks with factor -1).  Canonical blocks are chosen by visiting block
 * indices with the last position fastest; the first unassigned block of an
 * orbit becomes canonical and its images derivative.  Canonical blocks of
 * A and B are filled in canonical-list order from one splitmix64-style
 * stream of uniform [-0.5, 0.5) values (element counter running over the
 * blocks).  Steps, each followed by a read of every canonical block of C:
 *
 *   1. C = 0.5 * A B                      xm_contract(.., "ijcd", "cdab", "ijab")
 *   2. C = 2 C - 0.5 perm(A')             xm_add with A' = C's structure,
 *                                         A' = xm_set(0.125), idxb "jiba"
 *   3. C = -1.5 A B + 1.0 C               xm_contract with beta = 1
 *
 * EXPECTED_FILE holds the three results as doubles (canonical blocks of C
 * in list order, step after step), computed by the oracle.  The program
 * prints the largest absolute difference per step and exits 0 when every
 * step is within 1e-10 (the values are O(1)), 1 otherwise, 2 on I/O error.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "xm.h"

static double
uniform(uint64_t seed, uint64_t i)
{
	uint64_t x = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;

	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
	x ^= x >> 31;
	return (double)(x >> 11) * 0x1p-53 - 0.5;
}

/* four dimensions of sizes dims[k], each split once at split[k] */
static xm_block_space_t *
space(const size_t *dims, const size_t *split)
{
	xm_block_space_t *bs = xm_block_space_create(xm_dim_4(dims[0], dims[1],
	    dims[2], dims[3]));
	size_t k;

	for (k = 0; k < 4; k++)
		xm_block_space_split(bs, k, split[k]);
	return bs;
}

/* antisymmetric structure: images of (p, q, r, s) under p<->q and r<->s */
static xm_tensor_t *
antisym(const size_t *dims, const size_t *split, xm_allocator_t *al)
{
	static const size_t perms[3][4] = {{1, 0, 2, 3}, {0, 1, 3, 2}, {1, 0, 3, 2}};
	static const double fac[3] = {-1, -1, 1};
	xm_block_space_t *bs = space(dims, split);
	xm_tensor_t *t = xm_tensor_create(bs, XM_SCALAR_DOUBLE, al);
	xm_dim_t nb = xm_tensor_get_nblocks(t), idx, img, perm;
	size_t b0, b1, b2, b3, g, k;

	xm_block_space_free(bs);
	for (b0 = 0; b0 < nb.i[0]; b0++)
	for (b1 = 0; b1 < nb.i[1]; b1++)
	for (b2 = 0; b2 < nb.i[2]; b2++)
	for (b3 = 0; b3 < nb.i[3]; b3++) {
		idx = xm_dim_4(b0, b1, b2, b3);
		if (xm_tensor_get_block_type(t, idx) != XM_BLOCK_TYPE_ZERO)
			continue;
		xm_tensor_set_canonical_block(t, idx);
		for (g = 0; g < 3; g++) {
			img = xm_dim_zero(4);
			perm = xm_dim_zero(4);
			for (k = 0; k < 4; k++) {
				img.i[k] = idx.i[perms[g][k]];
				perm.i[k] = perms[g][k];
			}
			if (xm_tensor_get_block_type(t, img) == XM_BLOCK_TYPE_ZERO)
				xm_tensor_set_derivative_block(t, img, idx, perm, fac[g]);
		}
	}
	return t;
}

static void
fill(xm_tensor_t *t, uint64_t seed)
{
	xm_dim_t *list;
	size_t n, q, e, cnt = 0;

	xm_tensor_get_canonical_block_list(t, &list, &n);
	for (q = 0; q < n; q++) {
		size_t sz = xm_tensor_get_block_size(t, list[q]);
		double *buf = malloc(sz * sizeof *buf);
		for (e = 0; e < sz; e++)
			buf[e] = uniform(seed, cnt++);
		xm_tensor_write_block(t, list[q], buf);
		free(buf);
	}
	free(list);
}

/* largest |C - expected| over C's canonical blocks; advances *pos */
static double
compare(const xm_tensor_t *c, const double *want, size_t nwant, size_t *pos)
{
	xm_dim_t *list;
	size_t n, q, e;
	double m = 0;

	xm_tensor_get_canonical_block_list(c, &list, &n);
	for (q = 0; q < n; q++) {
		size_t sz = xm_tensor_get_block_size(c, list[q]);
		double *buf = malloc(sz * sizeof *buf);
		xm_tensor_read_block(c, list[q], buf);
		for (e = 0; e < sz; e++, (*pos)++) {
			double d = *pos < nwant ? fabs(buf[e] - want[*pos]) : INFINITY;
			if (!(d <= m))
				m = d;
		}
		free(buf);
	}
	free(list);
	return m;
}

int
main(int argc, char **argv)
{
	static const size_t oovv[4] = {7, 7, 11, 11}, vvvv[4] = {11, 11, 11, 11};
	static const size_t soovv[4] = {4, 4, 5, 5}, svvvv[4] = {5, 5, 5, 5};
	xm_allocator_t *al;
	xm_tensor_t *a, *b, *c, *a2;
	double *want, err[3];
	size_t nwant, pos = 0;
	long sz;
	FILE *f;
	int s, bad = 0;

	if (argc != 2 || (f = fopen(argv[1], "rb")) == NULL) {
		fprintf(stderr, "usage: ladder_caller EXPECTED_FILE\n");
		return 2;
	}
	fseek(f, 0, SEEK_END);
	sz = ftell(f);
	fseek(f, 0, SEEK_SET);
	nwant = (size_t)sz / sizeof(double);
	if ((want = malloc(nwant * sizeof *want + 1)) == NULL ||
	    fread(want, sizeof *want, nwant, f) != nwant) {
		fprintf(stderr, "ladder_caller: cannot read %s\n", argv[1]);
		return 2;
	}
	fclose(f);

	xm_print_banner();
	if ((al = xm_allocator_create(NULL)) == NULL)
		return 2;
	a = antisym(oovv, soovv, al);
	b = antisym(vvvv, svvvv, al);
	c = antisym(oovv, soovv, al);
	a2 = antisym(oovv, soovv, al);
	fill(a, 11);
	fill(b, 12);

	xm_contract(0.5, a, b, 0.0, c, "ijcd", "cdab", "ijab");
	err[0] = compare(c, want, nwant, &pos);
	xm_set(a2, 0.125);
	xm_add(2.0, c, -0.5, a2, "ijab", "jiba");
	err[1] = compare(c, want, nwant, &pos);
	xm_contract(-1.5, a, b, 1.0, c, "ijcd", "cdab", "ijab");
	err[2] = compare(c, want, nwant, &pos);
	for (s = 0; s < 3; s++) {
		printf("step %d: max |C - expected| = %.3e\n", s + 1, err[s]);
		bad |= !(err[s] <= 1e-10);
	}
	if (pos != nwant) {
		printf("expected %zu values, compared %zu\n", nwant, pos);
		bad = 1;
	}
	xm_tensor_free_block_data(a);
	xm_tensor_free_block_data(b);
	xm_tensor_free_block_data(c);
	xm_tensor_free_block_data(a2);
	xm_tensor_free(a);
	xm_tensor_free(b);
	xm_tensor_free(c);
	xm_tensor_free(a2);
	xm_allocator_destroy(al);
	free(want);
	printf(bad ? "FAILED\n" : "ok\n");
	return bad;
}
