/*
 * libxm-gb300: tensor operations.
 *
 * Same declarations as the reference's src/xm.h:29-137.  Every operation is
 * synchronous: when it returns, results are visible through
 * xm_tensor_read_block.  Errors print "libxm: <function>: <message>" and
 * exit(1), as the reference does (util.c:24-35).  GB300-specific controls
 * (precision mode, statistics, the adjoint) are declared in xmg.h.
 */
#ifndef XM_H_INCLUDED
#define XM_H_INCLUDED

#include "tensor.h"

#ifdef __cplusplus
extern "C" {
#endif

void xm_print_banner(void);
/* Every canonical block of a set to x (xm.c:28-64). */
void xm_set(xm_tensor_t *a, xm_scalar_t x);
/* a = s * b with index permutation and type conversion (xm.c:66-157). */
void xm_copy(xm_tensor_t *a, xm_scalar_t s, const xm_tensor_t *b,
    const char *idxa, const char *idxb);
/* a = alpha * a + beta * b (xm.c:159-249). */
void xm_add(xm_scalar_t alpha, xm_tensor_t *a, xm_scalar_t beta,
    const xm_tensor_t *b, const char *idxa, const char *idxb);
/* a = a * b element-wise (xm.c:251-332). */
void xm_mul(xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb);
/* a = a / b element-wise (xm.c:334-413). */
void xm_div(xm_tensor_t *a, const xm_tensor_t *b, const char *idxa,
    const char *idxb);
/* Sum over all blocks of a*b (xm.c:415-508). */
xm_scalar_t xm_dot(const xm_tensor_t *a, const xm_tensor_t *b,
    const char *idxa, const char *idxb);
/* c = alpha * a * b + beta * c over the indices named by the strings
 * (contract.c:227-314). */
void xm_contract(xm_scalar_t alpha, const xm_tensor_t *a, const xm_tensor_t *b,
    xm_scalar_t beta, xm_tensor_t *c, const char *idxa, const char *idxb,
    const char *idxc);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XM_H_INCLUDED */
