/*
 * libxm-gb300: scalar types and host-vector helpers.
 *
 * Same declarations as the reference's src/scalar.h:36-144.  Every scalar
 * argument of the API is a C99 double complex (C++: std::complex<double>),
 * narrowed to the tensor's type where it is used.
 */
#ifndef XM_SCALAR_H_INCLUDED
#define XM_SCALAR_H_INCLUDED

#include <stddef.h>

#ifdef __cplusplus
#include <complex>
#else
#include <complex.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Enumerator values 0..3 are part of the ABI (scalar.h:36-45). */
typedef enum {
	XM_SCALAR_FLOAT = 0,
	XM_SCALAR_FLOAT_COMPLEX,
	XM_SCALAR_DOUBLE,
	XM_SCALAR_DOUBLE_COMPLEX,
} xm_scalar_type_t;

#ifdef __cplusplus
typedef std::complex<double> xm_scalar_t;
#else
typedef double complex xm_scalar_t;
#endif

int xm_scalar_check_type(xm_scalar_type_t type);
size_t xm_scalar_sizeof(xm_scalar_type_t type);
/* a + b and a * b evaluated in the given type (scalar.h:70-81). */
xm_scalar_t xm_scalar_add(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t type);
xm_scalar_t xm_scalar_mul(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t type);
xm_scalar_t xm_scalar_get_element(void *x, size_t idx, xm_scalar_type_t type);
/* Host-vector loops (scalar.h:95-144).  These take host pointers. */
void xm_scalar_set(void *x, xm_scalar_t a, size_t len, xm_scalar_type_t type);
void xm_scalar_scale(void *x, xm_scalar_t a, size_t len, xm_scalar_type_t type);
/* x = a*x + b*y */
void xm_scalar_axpy(void *x, xm_scalar_t a, const void *y, xm_scalar_t b,
    size_t len, xm_scalar_type_t type);
/* x = x * (a*y) */
void xm_scalar_vec_mul(void *x, xm_scalar_t a, const void *y, size_t len,
    xm_scalar_type_t type);
/* x = x / (a*y) */
void xm_scalar_vec_div(void *x, xm_scalar_t a, const void *y, size_t len,
    xm_scalar_type_t type);
xm_scalar_t xm_scalar_dot(const void *x, const void *y, size_t len,
    xm_scalar_type_t type);
void xm_scalar_convert(void *x, const void *y, size_t len,
    xm_scalar_type_t xtype, xm_scalar_type_t ytype);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* XM_SCALAR_H_INCLUDED */
