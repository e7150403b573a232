/*
 * TEST INFRASTRUCTURE ONLY.  Minimal FFTW-2.x real-data API (rfftwnd, rank 1)
 * for compiling the reference oracle; see fftw.h.  In-place semantics follow
 * FFTW 2: a real row of length n occupies 2*(n/2+1) reals, so for in-place
 * real-to-complex the complex output uses dist idist/2, and for in-place
 * complex-to-real the real output uses dist 2*idist; strides are unchanged.
 */
#ifndef ORACLE_SHIM_RFFTW_H
#define ORACLE_SHIM_RFFTW_H

#include "fftw.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_REAL_TO_COMPLEX FFTW_FORWARD
#define FFTW_COMPLEX_TO_REAL FFTW_BACKWARD

typedef struct rfftwnd_plan_struct *rfftwnd_plan;

rfftwnd_plan rfftwnd_create_plan(int rank, const int *n, fftw_direction dir,
                                 int flags);
void rfftwnd_real_to_complex(rfftwnd_plan p, int howmany, fftw_real *in,
                             int istride, int idist, fftw_complex *out,
                             int ostride, int odist);
void rfftwnd_complex_to_real(rfftwnd_plan p, int howmany, fftw_complex *in,
                             int istride, int idist, fftw_real *out,
                             int ostride, int odist);
void rfftwnd_destroy_plan(rfftwnd_plan p);

#ifdef __cplusplus
}
#endif
#endif
