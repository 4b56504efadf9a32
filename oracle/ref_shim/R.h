/* Minimal stand-in for R's R.h, only so the reference's CPU loops
 * (src/distance.cpp, src/correlation.cpp) compile outside R.  Part of the
 * oracle's test infrastructure; never shipped. */
#ifndef GT_REF_SHIM_R_H
#define GT_REF_SHIM_R_H
#include <stdlib.h>
#include <stdio.h>
#include <math.h>  /* R.h brings in math.h for its users */
#ifdef __cplusplus
extern "C" {
#endif
void error(const char *fmt, ...);
void warning(const char *fmt, ...);
void Rprintf(const char *fmt, ...);
#ifdef __cplusplus
}
#endif
#define Calloc(n, t) ((t *)calloc((size_t)(n), sizeof(t)))
#define Free(p) (free((void *)(p)), (p) = NULL)
#endif
