/*
 * Hand-written adjoint of xm_contract (placeholder until built).
 */
#include "xmg_host.h"

int
xm_contract_adjoint(xm_scalar_t alpha, const xm_tensor_t *a,
    const xm_tensor_t *b, const xm_tensor_t *dc, xm_tensor_t *da,
    xm_tensor_t *db, const char *idxa, const char *idxb, const char *idxc)
{
	(void)alpha; (void)a; (void)b; (void)dc; (void)da; (void)db;
	(void)idxa; (void)idxb; (void)idxc;
	return xmg_seterr(XMG_ENOTSUP, "xm_contract_adjoint: not built");
}
