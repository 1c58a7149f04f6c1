/*
 * Minimal stand-in for the R headers, used ONLY to compile the reference
 * vectra engine sources (src/*.c of gcol33/vectra) into a host library that
 * serves as a test oracle.  R itself is not installed on the build or GPU
 * machines.
 *
 * The reference engine needs five things from R (src/error.c:4-11,
 * src/agg_ops.c:4,197,218-219,238-239):
 *   Rf_error    -> reported through a longjmp target the driver installs
 *   Rf_warning  -> counted (aggregate warnings on all-NA groups with na.rm)
 *   R_NaN, R_PosInf, R_NegInf
 *
 * Test infrastructure only: nothing in the product links this file.
 */
#ifndef VGPU_ORACLE_RSHIM_R_H
#define VGPU_ORACLE_RSHIM_R_H

/* R.h itself pulls in the C standard I/O and library headers; some
 * reference files rely on that (snprintf in src/join.c:746). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

void Rf_error(const char *fmt, ...);
void Rf_warning(const char *fmt, ...);

#define R_NaN    (NAN)
#define R_PosInf (INFINITY)
#define R_NegInf (-INFINITY)

#ifdef __cplusplus
}
#endif

#endif
