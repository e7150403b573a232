/*
 * TEST INFRASTRUCTURE ONLY -- part of the CPU oracle, never linked into the
 * product library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it.
 *
 * Clean-room mixed-radix FFT written from the DFT definition
 *   X[k] = sum_j x[j] * exp(sign * 2*pi*i * j*k / n)     (unnormalised)
 * with specialised radix-2/3/4/5 butterflies and a generic odd-radix DFT for
 * any other prime factor.  It backs two things:
 *   - the FFTW-2.x API shim (oracle/shim) that lets the reference's own
 *     channel/*.c compile here (FFTW 2.x is not installed), and
 *   - the C restatement of the reference path (oracle/chan_port.c).
 * Real transforms follow FFTW-2 "rfftw" semantics: r2c returns bins 0..n/2
 * with exactly-zero imaginary parts at DC (and at n/2 for even n); c2r reads
 * bins 0..n/2 and ignores the imaginary parts of DC and n/2 (halfcomplex
 * storage has no slot for them).
 */
#ifndef ORACLE_FFT_H
#define ORACLE_FFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } offt_cpx;

typedef struct offt_plan_s {
    int n;            /* transform length                                  */
    int sign;         /* -1 forward (exp(-i..)), +1 backward (exp(+i..))    */
    int nfac;         /* number of radix factors                            */
    int fac[32];      /* radix factors, product == n                        */
    offt_cpx *tw;     /* tw[k] = exp(sign*2*pi*i*k/n), k = 0..n-1          */
    offt_cpx *work;   /* 2*n scratch                                        */
} offt_plan;

offt_plan *offt_plan_create(int n, int sign);
void offt_plan_destroy(offt_plan *p);
/* Strided complex transform, in place allowed (in == out). */
void offt_exec(offt_plan *p, const offt_cpx *in, int istride,
               offt_cpx *out, int ostride);

typedef struct offt_rplan_s {
    int n;             /* real length                                       */
    int dir;           /* -1: real -> complex, +1: complex -> real           */
    offt_plan *half;   /* length n/2 complex plan when n is even            */
    offt_plan *full;   /* length n complex plan when n is odd               */
    offt_cpx *tw;      /* exp(dir*2*pi*i*k/n), k = 0..n/2                    */
    offt_cpx *work;    /* scratch, n+2 complex                              */
} offt_rplan;

offt_rplan *offt_rplan_create(int n, int dir);
void offt_rplan_destroy(offt_rplan *p);
/* r2c: in = n reals (stride istride), out = n/2+1 complex (stride ostride). */
void offt_r2c(offt_rplan *p, const double *in, int istride,
              offt_cpx *out, int ostride);
/* c2r: in = n/2+1 complex (stride istride), out = n reals (stride ostride). */
void offt_c2r(offt_rplan *p, const offt_cpx *in, int istride,
              double *out, int ostride);

#ifdef __cplusplus
}
#endif
#endif
