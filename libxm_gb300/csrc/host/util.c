/*
 * Error reporting and index-string parsing for libxm-gb300.
 *
 * xm_fatal keeps the reference's message shape "libxm: <text>" followed by
 * exit(1) (util.c:24-35).  xm_make_masks pairs equal letters of two index
 * strings, emitting positions in str1 order (util.c:37-53); test drivers
 * written against the reference call both directly (test.c:147,159).
 */
#include "xmg_host.h"

#include <stdarg.h>

static __thread char last_error[512];

void
xm_fatal(const char *fmt, ...)
{
	va_list ap;

	fputs("libxm: ", stderr);
	va_start(ap, fmt);
	vfprintf(stderr, fmt, ap);
	va_end(ap);
	fputc('\n', stderr);
	fflush(stderr);
	exit(1);
}

int
xmg_seterr(int code, const char *fmt, ...)
{
	va_list ap;

	va_start(ap, fmt);
	vsnprintf(last_error, sizeof last_error, fmt, ap);
	va_end(ap);
	return code;
}

const char *
xmg_last_error(void)
{
	return last_error;
}

void
xmg_die_on(int status)
{
	if (status != XMG_OK)
		xm_fatal("%s", last_error[0] ? last_error : "unknown error");
}

void
xm_make_masks(const char *str1, const char *str2, xm_dim_t *mask1,
    xm_dim_t *mask2)
{
	size_t p, q;

	mask1->n = mask2->n = 0;
	for (p = 0; str1[p] != '\0'; p++) {
		for (q = 0; str2[q] != '\0'; q++) {
			if (str1[p] != str2[q])
				continue;
			if (mask1->n == XM_MAX_DIM)
				xm_fatal("%s: too many matching indices", __func__);
			mask1->i[mask1->n++] = p;
			mask2->i[mask2->n++] = q;
		}
	}
}
