/*
 * ORACLE -- test infrastructure only.
 *
 * BLAS shim linked into the reference libxm built from source: the
 * reference calls Fortran-style sgemm_/dgemm_/cgemm_/zgemm_ with long int
 * arguments (contract.c:32-47); they are forwarded to an ILP64 BLAS found
 * at run time (numpy's bundled OpenBLAS, scipy_?gemm_64_) or, failing
 * that, to a plain C loop.  Every call can be logged (type, m, n, k,
 * alpha) so that tests can read the reference's GEMM sequence -- its
 * merged block-pair structure -- without touching its sources.
 */
#include <complex.h>
#include <dlfcn.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef void (*gemm_fn)(const char *, const char *, const long *, const long *,
    const long *, const void *, const void *, const long *, const void *,
    const long *, const void *, void *, const long *, size_t, size_t);
static gemm_fn fn[4];      /* s c d z */

int
xmref_set_blas(const char *path)
{
	static const char *nm[4] = {"scipy_sgemm_64_", "scipy_cgemm_64_",
	    "scipy_dgemm_64_", "scipy_zgemm_64_"};
	void *h = path ? dlopen(path, RTLD_NOW | RTLD_LOCAL) : NULL;
	if (h == NULL)
		return 0;
	for (int k = 0; k < 4; k++)
		if ((fn[k] = (gemm_fn)dlsym(h, nm[k])) == NULL)
			return 0;
	return 1;
}

struct logent { int type; long m, n, k; double re, im; };
static struct logent *logv;
static size_t logn, logcap;
static int logging;
static pthread_mutex_t logmu = PTHREAD_MUTEX_INITIALIZER;

void xmref_log_enable(int on) { logging = on; if (on) logn = 0; }
size_t xmref_log_count(void) { return logn; }
void
xmref_log_get(size_t i, int *type, long *m, long *n, long *k, double *re, double *im)
{
	*type = logv[i].type; *m = logv[i].m; *n = logv[i].n; *k = logv[i].k;
	*re = logv[i].re; *im = logv[i].im;
}

static void
record(int type, long m, long n, long k, double re, double im)
{
	if (!logging)
		return;
	pthread_mutex_lock(&logmu);
	if (logn == logcap) {
		logcap = logcap ? 2 * logcap : 1024;
		logv = realloc(logv, logcap * sizeof *logv);
	}
	logv[logn++] = (struct logent){type, m, n, k, re, im};
	pthread_mutex_unlock(&logmu);
}

/* C = alpha * op(A) op(B) + beta * C, column-major; only the ('T','N')
 * form the reference issues is needed by the fallback loop. */
#define FALLBACK(T)							\
	for (long j = 0; j < *n; j++)					\
		for (long i = 0; i < *m; i++) {				\
			T s = 0;					\
			for (long q = 0; q < *k; q++)			\
				s += a[q + i * *lda] * b[q + j * *ldb];	\
			c[i + j * *ldc] = *alpha * s + *beta * c[i + j * *ldc]; \
		}

void
sgemm_(char *ta, char *tb, long *m, long *n, long *k, float *alpha, float *a,
    long *lda, float *b, long *ldb, float *beta, float *c, long *ldc)
{
	record(0, *m, *n, *k, *alpha, 0);
	if (fn[0]) { fn[0](ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return; }
	FALLBACK(float)
}

void
cgemm_(char *ta, char *tb, long *m, long *n, long *k, float complex *alpha,
    float complex *a, long *lda, float complex *b, long *ldb,
    float complex *beta, float complex *c, long *ldc)
{
	record(1, *m, *n, *k, crealf(*alpha), cimagf(*alpha));
	if (fn[1]) { fn[1](ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return; }
	FALLBACK(float complex)
}

void
dgemm_(char *ta, char *tb, long *m, long *n, long *k, double *alpha, double *a,
    long *lda, double *b, long *ldb, double *beta, double *c, long *ldc)
{
	record(2, *m, *n, *k, *alpha, 0);
	if (fn[2]) { fn[2](ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return; }
	FALLBACK(double)
}

void
zgemm_(char *ta, char *tb, long *m, long *n, long *k, double complex *alpha,
    double complex *a, long *lda, double complex *b, long *ldb,
    double complex *beta, double complex *c, long *ldc)
{
	record(3, *m, *n, *k, creal(*alpha), cimag(*alpha));
	if (fn[3]) { fn[3](ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, 1); return; }
	FALLBACK(double complex)
}
