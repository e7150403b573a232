/*
 * TEST INFRASTRUCTURE ONLY.  FFTW-2.x API shim over oracle/fft.c; see fftw.h.
 */
#include <stdio.h>
#include <stdlib.h>

#include "fftw.h"
#include "rfftw.h"
#include "../fft.h"

struct fftw_plan_struct {
    offt_plan *p;
    int in_place;
};

struct rfftwnd_plan_struct {
    offt_rplan *p;
    int dir;
    int in_place;
};

fftw_plan fftw_create_plan_specific(int n, fftw_direction dir, int flags,
                                    fftw_complex *in, int istride,
                                    fftw_complex *out, int ostride)
{
    (void)in; (void)istride; (void)out; (void)ostride;
    return fftw_create_plan(n, dir, flags);
}

fftw_plan fftw_create_plan(int n, fftw_direction dir, int flags)
{
    fftw_plan pl = (fftw_plan)calloc(1, sizeof(*pl));
    if (!pl) return NULL;
    pl->p = offt_plan_create(n, (int)dir);
    pl->in_place = (flags & FFTW_IN_PLACE) != 0;
    return pl;
}

void fftw(fftw_plan plan, int howmany, fftw_complex *in, int istride,
          int idist, fftw_complex *out, int ostride, int odist)
{
    for (int t = 0; t < howmany; ++t) {
        offt_cpx *src = (offt_cpx *)(in + (long)t * idist);
        if (plan->in_place || out == NULL) {
            offt_exec(plan->p, src, istride, src, istride);
        } else {
            offt_exec(plan->p, src, istride, (offt_cpx *)(out + (long)t * odist), ostride);
        }
    }
}

void fftw_one(fftw_plan plan, fftw_complex *in, fftw_complex *out)
{
    fftw(plan, 1, in, 1, 0, out, 1, 0);
}

void fftw_destroy_plan(fftw_plan plan)
{
    if (!plan) return;
    offt_plan_destroy(plan->p);
    free(plan);
}

rfftwnd_plan rfftwnd_create_plan(int rank, const int *n, fftw_direction dir,
                                 int flags)
{
    if (rank != 1) {
        fprintf(stderr, "oracle fftw shim: only rank-1 rfftwnd plans are provided\n");
        abort();
    }
    rfftwnd_plan pl = (rfftwnd_plan)calloc(1, sizeof(*pl));
    if (!pl) return NULL;
    pl->p = offt_rplan_create(n[0], (int)dir);
    pl->dir = (int)dir;
    pl->in_place = (flags & FFTW_IN_PLACE) != 0;
    return pl;
}

void rfftwnd_real_to_complex(rfftwnd_plan p, int howmany, fftw_real *in,
                             int istride, int idist, fftw_complex *out,
                             int ostride, int odist)
{
    for (int t = 0; t < howmany; ++t) {
        const double *src = in + (long)t * idist;
        offt_cpx *dst;
        int os;
        if (p->in_place || out == NULL) {
            dst = (offt_cpx *)(in + (long)t * idist); /* complex dist idist/2 */
            os = istride;
        } else {
            dst = (offt_cpx *)(out + (long)t * odist);
            os = ostride;
        }
        offt_r2c(p->p, src, istride, dst, os);
    }
}

void rfftwnd_complex_to_real(rfftwnd_plan p, int howmany, fftw_complex *in,
                             int istride, int idist, fftw_real *out,
                             int ostride, int odist)
{
    for (int t = 0; t < howmany; ++t) {
        const offt_cpx *src = (const offt_cpx *)(in + (long)t * idist);
        double *dst;
        int os;
        if (p->in_place || out == NULL) {
            dst = (double *)(in + (long)t * idist); /* real dist 2*idist */
            os = istride;
        } else {
            dst = out + (long)t * odist;
            os = ostride;
        }
        offt_c2r(p->p, src, istride, dst, os);
    }
}

void rfftwnd_destroy_plan(rfftwnd_plan p)
{
    if (!p) return;
    offt_rplan_destroy(p->p);
    free(p);
}
