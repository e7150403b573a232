/*
 * TEST INFRASTRUCTURE ONLY.  Minimal FFTW-2.x API (complex part) so that the
 * reference's channel/*.c compiles unmodified for use as the CPU oracle.
 * FFTW 2.x itself is not installed; the transforms come from oracle/fft.c
 * (clean-room, written from the DFT definition).  Only the subset the
 * reference calls is provided: fftw_create_plan_specific, fftw, fftw_one,
 * fftw_destroy_plan.  FFTW_FORWARD = -1 (exp(-i...)), FFTW_BACKWARD = +1,
 * both unnormalised, as in FFTW 2.
 */
#ifndef ORACLE_SHIM_FFTW_H
#define ORACLE_SHIM_FFTW_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_real;
typedef struct { fftw_real re, im; } fftw_complex;
typedef enum { FFTW_FORWARD = -1, FFTW_BACKWARD = 1 } fftw_direction;

#define FFTW_ESTIMATE      (0)
#define FFTW_MEASURE       (1)
#define FFTW_OUT_OF_PLACE  (0)
#define FFTW_IN_PLACE      (8)
#define FFTW_USE_WISDOM    (16)

typedef struct fftw_plan_struct *fftw_plan;

fftw_plan fftw_create_plan(int n, fftw_direction dir, int flags);
fftw_plan fftw_create_plan_specific(int n, fftw_direction dir, int flags,
                                    fftw_complex *in, int istride,
                                    fftw_complex *out, int ostride);
void fftw(fftw_plan plan, int howmany, fftw_complex *in, int istride,
          int idist, fftw_complex *out, int ostride, int odist);
void fftw_one(fftw_plan plan, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan plan);

#ifdef __cplusplus
}
#endif
#endif
