/*
 * libxm-gb300: the two private helpers the reference's own test driver
 * calls, declared as in the reference's src/util.h:32-35 so that its
 * test.c compiles unchanged against this library: xm_fatal prints
 * "libxm: <message>" and exits(1); xm_make_masks pairs equal index letters
 * of two strings (positions in the first and in the second, in the first
 * string's order).  fatal(x) prefixes the calling function's name.
 */
#ifndef UTIL_H_INCLUDED
#define UTIL_H_INCLUDED

#include "dim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define fatal(x) xm_fatal("%s: %s", __func__, (x))

void xm_fatal(const char *, ...) __attribute__((__noreturn__));
void xm_make_masks(const char *, const char *, xm_dim_t *, xm_dim_t *);

#ifdef __cplusplus
}
#endif

#endif /* UTIL_H_INCLUDED */
