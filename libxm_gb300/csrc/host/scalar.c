/*
 * Scalar helpers for libxm-gb300.
 *
 * These are the public host-vector routines of the reference's src/scalar.c
 * (scalar.c:22-414).  They operate on caller-owned host memory by contract;
 * the engine's own element-wise work runs in CUDA kernels instead.  Each
 * scalar is narrowed to the vector's type before use, as the reference
 * does, so results agree bit for bit.
 */
#include "xmg_host.h"

int
xm_scalar_check_type(xm_scalar_type_t t)
{
	return t == XM_SCALAR_FLOAT || t == XM_SCALAR_FLOAT_COMPLEX ||
	    t == XM_SCALAR_DOUBLE || t == XM_SCALAR_DOUBLE_COMPLEX;
}

size_t
xm_scalar_sizeof(xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return sizeof(float);
	case XM_SCALAR_FLOAT_COMPLEX: return sizeof(float complex);
	case XM_SCALAR_DOUBLE: return sizeof(double);
	case XM_SCALAR_DOUBLE_COMPLEX: return sizeof(double complex);
	}
	xm_fatal("%s: unexpected scalar type", __func__);
}

xm_scalar_t
xm_scalar_add(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return (float)a + (float)b;
	case XM_SCALAR_FLOAT_COMPLEX: return (float complex)a + (float complex)b;
	case XM_SCALAR_DOUBLE: return (double)a + (double)b;
	case XM_SCALAR_DOUBLE_COMPLEX: return a + b;
	}
	xm_fatal("%s: unexpected scalar type", __func__);
}

xm_scalar_t
xm_scalar_mul(xm_scalar_t a, xm_scalar_t b, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return (float)a * (float)b;
	case XM_SCALAR_FLOAT_COMPLEX: return (float complex)a * (float complex)b;
	case XM_SCALAR_DOUBLE: return (double)a * (double)b;
	case XM_SCALAR_DOUBLE_COMPLEX: return a * b;
	}
	xm_fatal("%s: unexpected scalar type", __func__);
}

xm_scalar_t
xm_scalar_get_element(void *x, size_t i, xm_scalar_type_t t)
{
	switch (t) {
	case XM_SCALAR_FLOAT: return ((float *)x)[i];
	case XM_SCALAR_FLOAT_COMPLEX: return ((float complex *)x)[i];
	case XM_SCALAR_DOUBLE: return ((double *)x)[i];
	case XM_SCALAR_DOUBLE_COMPLEX: return ((double complex *)x)[i];
	}
	xm_fatal("%s: unexpected scalar type", __func__);
}

/* One loop body instantiated for the four element types. */
#define FOR_TYPES(t, ...)						\
	switch (t) {							\
	case XM_SCALAR_FLOAT: { typedef float T; __VA_ARGS__; return; }	\
	case XM_SCALAR_FLOAT_COMPLEX: { typedef float complex T; __VA_ARGS__; return; } \
	case XM_SCALAR_DOUBLE: { typedef double T; __VA_ARGS__; return; }	\
	case XM_SCALAR_DOUBLE_COMPLEX: { typedef double complex T; __VA_ARGS__; return; } \
	}								\
	xm_fatal("%s: unexpected scalar type", __func__)

void
xm_scalar_set(void *x, xm_scalar_t a, size_t len, xm_scalar_type_t t)
{
	size_t i;
	FOR_TYPES(t, { T *v = x; T s = (T)a; for (i = 0; i < len; i++) v[i] = s; });
}

void
xm_scalar_scale(void *x, xm_scalar_t a, size_t len, xm_scalar_type_t t)
{
	size_t i;
	FOR_TYPES(t, { T *v = x; T s = (T)a; for (i = 0; i < len; i++) v[i] *= s; });
}

void
xm_scalar_axpy(void *x, xm_scalar_t a, const void *y, xm_scalar_t b,
    size_t len, xm_scalar_type_t t)
{
	size_t i;
	FOR_TYPES(t, { T *v = x; const T *w = y; T sa = (T)a, sb = (T)b;
	    for (i = 0; i < len; i++) v[i] = sa * v[i] + sb * w[i]; });
}

void
xm_scalar_vec_mul(void *x, xm_scalar_t a, const void *y, size_t len,
    xm_scalar_type_t t)
{
	size_t i;
	FOR_TYPES(t, { T *v = x; const T *w = y; T s = (T)a;
	    for (i = 0; i < len; i++) v[i] = s * v[i] * w[i]; });
}

void
xm_scalar_vec_div(void *x, xm_scalar_t a, const void *y, size_t len,
    xm_scalar_type_t t)
{
	size_t i;
	FOR_TYPES(t, { T *v = x; const T *w = y; T s = (T)a;
	    for (i = 0; i < len; i++) v[i] = v[i] / (s * w[i]); });
}

xm_scalar_t
xm_scalar_dot(const void *x, const void *y, size_t len, xm_scalar_type_t t)
{
	size_t i;

	switch (t) {
	case XM_SCALAR_FLOAT: {
		const float *u = x, *w = y;
		float s = 0;
		for (i = 0; i < len; i++)
			s += u[i] * w[i];
		return s;
	}
	case XM_SCALAR_FLOAT_COMPLEX: {
		const float complex *u = x, *w = y;
		float complex s = 0;
		for (i = 0; i < len; i++)
			s += u[i] * w[i];
		return s;
	}
	case XM_SCALAR_DOUBLE: {
		const double *u = x, *w = y;
		double s = 0;
		for (i = 0; i < len; i++)
			s += u[i] * w[i];
		return s;
	}
	case XM_SCALAR_DOUBLE_COMPLEX: {
		const double complex *u = x, *w = y;
		double complex s = 0;
		for (i = 0; i < len; i++)
			s += u[i] * w[i];
		return s;
	}
	}
	xm_fatal("%s: unexpected scalar type", __func__);
}

void
xm_scalar_convert(void *x, const void *y, size_t len, xm_scalar_type_t xt,
    xm_scalar_type_t yt)
{
	size_t i;

	if (xt == yt) {
		memcpy(x, y, len * xm_scalar_sizeof(xt));
		return;
	}
#define CONV(XT, YT, TX, TY)						\
	if (xt == XT && yt == YT) {					\
		TX *u = x;						\
		const TY *w = y;					\
		for (i = 0; i < len; i++)				\
			u[i] = (TX)w[i];				\
		return;							\
	}
	CONV(XM_SCALAR_DOUBLE, XM_SCALAR_FLOAT, double, float)
	CONV(XM_SCALAR_FLOAT, XM_SCALAR_DOUBLE, float, double)
	CONV(XM_SCALAR_DOUBLE_COMPLEX, XM_SCALAR_FLOAT_COMPLEX, double complex, float complex)
	CONV(XM_SCALAR_FLOAT_COMPLEX, XM_SCALAR_DOUBLE_COMPLEX, float complex, double complex)
#undef CONV
	xm_fatal("%s: unsupported scalar conversion", __func__);
}
