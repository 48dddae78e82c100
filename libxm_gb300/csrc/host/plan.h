/*
 * The contraction plan shared by the planner (contract.c) and the staged
 * and streamed paths (stream.c).  Internal to the library.
 */
#ifndef XMG_PLAN_H
#define XMG_PLAN_H

#include "xmg_host.h"
#include "hmap.h"

/* offset-table pool with interning */
typedef struct {
	int32_t *v;
	int64_t n, cap;
	xmg_hmap_t index;        /* descriptor hash -> descriptor slot */
	struct tabdesc {
		int nd;
		int64_t size[XM_MAX_DIM], stride[XM_MAX_DIM];
		int32_t off;
	} *desc;
	int ndesc, capdesc;
	int overflow;            /* the pool outgrew int32 offsets */
} tabpool_t;

/* the plan */
typedef struct {
	xm_scalar_type_t type;
	xm_dim_t cidxa, aidxa, cidxb, aidxb, cidxc, aidxc;
	/* growable arrays */
	xmgd_cblock_t *cb; int ncb, capcb;
	xmgd_pair_t *pr; int npr, cappr;
	xmgd_view_t *va; int nva, capva;
	xmgd_view_t *vb; int nvb, capvb;
	xmg_hmap_t va_index, vb_index, ea_index, eb_index;
	int32_t nexp_a, nexp_b;
	tabpool_t tabs;
	double flops;
	uint8_t *emulatable;     /* per cblock */
	int capem;
	/* out-of-core: collect lists the b data handles (and bytes) of
	 * every surviving pair */
	int collect;
	uint64_t *bh, *bsz;
	size_t nbh, capbh;
} plan_t;

void xmg_plan_init(plan_t *p);
void xmg_plan_free(plan_t *p);
/* validation and masks (the reference's contract.c:237-280 checks) */
int xmg_plan_check(const xm_tensor_t *a, const xm_tensor_t *b,
    const xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc, plan_t *p);
/* the merged pairs, views and tables; device: 0 host checks, 1 addresses
 * of the device views, 2 data handles (staged and streamed paths) */
int xmg_plan_build(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, const xm_tensor_t *c, plan_t *p, int device);
double xmg_now_ms(void);
/* statistics of the last contraction (xmg_get_last_stats) */
extern xmg_stats_t xmg_last_stats;

/* pagefile and host-memory operands (stream.c): 0 when the in-core path
 * runs the contraction, else 1 with the status in *st */
int xmg_contract_streamed(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, xm_scalar_t beta, xm_tensor_t *c,
    const char *idxa, const char *idxb, const char *idxc, int prec, int *st);
/* c's staged views written back and dropped (pagefile c), status st
 * passed through when nonzero */
int xmg_commit_c(xm_tensor_t *c, int st);
/* the kept streamed contraction's plans and HBM regions released */
void xmg_stream_release(void);

#endif /* XMG_PLAN_H */
