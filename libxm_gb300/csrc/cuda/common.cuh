/* Shared device-side helpers of libxm-gb300. */
#ifndef XMG_COMMON_CUH
#define XMG_COMMON_CUH

#include <cuda_runtime.h>
#include <cuComplex.h>
#include <stdint.h>

#include "xmg_dev.h"
#include "xmg.h"

extern "C" int xmg_seterr(int code, const char *fmt, ...);

namespace xmg {

cudaStream_t stream();          /* engine compute stream */
int device();                   /* engine device ordinal */
int num_sms();
int check(cudaError_t e, const char *what);
extern long long g_launches;     /* kernels launched by the engine */
#define XMG_CK(call) do { int _s = xmg::check((call), #call); if (_s) return _s; } while (0)

/* element types: xm_scalar_type_t order */
struct cf { float x, y; };
struct cd { double x, y; };

template <typename T> struct num;
template <> struct num<float> {
	__host__ __device__ static float mk(const double *s) { return (float)s[0]; }
	__device__ static float mul(float a, float b) { return a * b; }
	__device__ static float fma(float a, float b, float c) { return fmaf(a, b, c); }
	__device__ static float add(float a, float b) { return a + b; }
	__device__ static float div(float a, float b) { return a / b; }
	__device__ static float zero() { return 0.f; }
	__device__ static double re(float a) { return a; }
	__device__ static double im(float) { return 0; }
};
template <> struct num<double> {
	__host__ __device__ static double mk(const double *s) { return s[0]; }
	__device__ static double mul(double a, double b) { return a * b; }
	__device__ static double fma(double a, double b, double c) { return ::fma(a, b, c); }
	__device__ static double add(double a, double b) { return a + b; }
	__device__ static double div(double a, double b) { return a / b; }
	__device__ static double zero() { return 0.0; }
	__device__ static double re(double a) { return a; }
	__device__ static double im(double) { return 0; }
};
template <> struct num<cf> {
	__host__ __device__ static cf mk(const double *s) { return cf{(float)s[0], (float)s[1]}; }
	__device__ static cf mul(cf a, cf b) { return cf{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
	__device__ static cf fma(cf a, cf b, cf c) {
		return cf{fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y))}; }
	__device__ static cf add(cf a, cf b) { return cf{a.x + b.x, a.y + b.y}; }
	__device__ static cf div(cf a, cf b) {
		cuFloatComplex q = cuCdivf(make_cuFloatComplex(a.x, a.y), make_cuFloatComplex(b.x, b.y));
		return cf{cuCrealf(q), cuCimagf(q)}; }
	__device__ static cf zero() { return cf{0.f, 0.f}; }
	__device__ static double re(cf a) { return a.x; }
	__device__ static double im(cf a) { return a.y; }
};
template <> struct num<cd> {
	__host__ __device__ static cd mk(const double *s) { return cd{s[0], s[1]}; }
	__device__ static cd mul(cd a, cd b) { return cd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
	__device__ static cd fma(cd a, cd b, cd c) {
		return cd{::fma(a.x, b.x, ::fma(-a.y, b.y, c.x)), ::fma(a.x, b.y, ::fma(a.y, b.x, c.y))}; }
	__device__ static cd add(cd a, cd b) { return cd{a.x + b.x, a.y + b.y}; }
	__device__ static cd div(cd a, cd b) {
		cuDoubleComplex q = cuCdiv(make_cuDoubleComplex(a.x, a.y), make_cuDoubleComplex(b.x, b.y));
		return cd{cuCreal(q), cuCimag(q)}; }
	__device__ static cd zero() { return cd{0.0, 0.0}; }
	__device__ static double re(cd a) { return a.x; }
	__device__ static double im(cd a) { return a.y; }
};

/* conversions used by xm_copy (float <-> double, cf <-> cd) */
template <typename D, typename S> __device__ inline D conv(S s);
template <> __device__ inline float conv<float, float>(float s) { return s; }
template <> __device__ inline double conv<double, double>(double s) { return s; }
template <> __device__ inline float conv<float, double>(double s) { return (float)s; }
template <> __device__ inline double conv<double, float>(float s) { return s; }
template <> __device__ inline cf conv<cf, cf>(cf s) { return s; }
template <> __device__ inline cd conv<cd, cd>(cd s) { return s; }
template <> __device__ inline cf conv<cf, cd>(cd s) { return cf{(float)s.x, (float)s.y}; }
template <> __device__ inline cd conv<cd, cf>(cf s) { return cd{s.x, s.y}; }

/* asynchronous global -> shared copy of one element (cp.async: no
 * register holds the value while it is in flight) */
template <int B> __device__ __forceinline__ void cp_async_b(void *s, const void *g);
template <> __device__ __forceinline__ void cp_async_b<4>(void *s, const void *g)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 4;"
	    :: "r"((uint32_t)__cvta_generic_to_shared(s)), "l"(g) : "memory");
}
template <> __device__ __forceinline__ void cp_async_b<8>(void *s, const void *g)
{
	asm volatile("cp.async.ca.shared.global [%0], [%1], 8;"
	    :: "r"((uint32_t)__cvta_generic_to_shared(s)), "l"(g) : "memory");
}
template <> __device__ __forceinline__ void cp_async_b<16>(void *s, const void *g)
{
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
	    :: "r"((uint32_t)__cvta_generic_to_shared(s)), "l"(g) : "memory");
}
template <typename T> __device__ __forceinline__ void cp_async_elem(T *s, const T *g)
{
	cp_async_b<sizeof(T)>(s, g);
}
__device__ __forceinline__ void cp_async_wait_all()
{
	asm volatile("cp.async.wait_all;" ::: "memory");
}

} /* namespace xmg */

#endif
