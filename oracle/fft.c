/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle FFT, see fft.h.
 *
 * Recursive decimation-in-time mixed-radix FFT.  A length n = p * m transform
 * is split into p interleaved sub-sequences of length m (x[q + p*j]); each is
 * transformed recursively, then p-point butterflies combine them:
 *     X[k + u*m] = sum_q W_n^{q*k} * W_p^{u*q} * Y_q[k].
 * Twiddles W_n^k = exp(sign*2*pi*i*k/n) are tabulated once per plan in long
 * double and rounded, so every entry is accurate to the last bit of a double.
 */
#include "fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static void unit_root(long n, long k, int sign, offt_cpx *w)
{
    /* exp(sign * 2 pi i k / n) with k reduced to [0, n) */
    long double pi2 = 6.283185307179586476925286766559005768L;
    k %= n;
    if (k < 0) k += n;
    long double a = pi2 * (long double)k / (long double)n;
    w->re = (double)cosl(a);
    w->im = (double)(sign * sinl(a));
    /* exact values where the math gives them */
    if (4 * k == n) { w->re = 0.0; w->im = (double)sign; }
    if (2 * k == n) { w->re = -1.0; w->im = 0.0; }
    if (4 * k == 3 * n) { w->re = 0.0; w->im = -(double)sign; }
    if (k == 0) { w->re = 1.0; w->im = 0.0; }
}

offt_plan *offt_plan_create(int n, int sign)
{
    offt_plan *p = (offt_plan *)calloc(1, sizeof(offt_plan));
    if (!p) return NULL;
    p->n = n;
    p->sign = sign;
    int r = n;
    while (r > 1) {
        int f;
        if (r % 4 == 0) f = 4;
        else if (r % 2 == 0) f = 2;
        else if (r % 3 == 0) f = 3;
        else if (r % 5 == 0) f = 5;
        else {
            f = 7;
            while (r % f) f += 2;
        }
        p->fac[p->nfac++] = f;
        r /= f;
    }
    p->tw = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)(n > 0 ? n : 1));
    p->work = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)(2 * n + 2));
    for (int k = 0; k < n; ++k) unit_root(n, k, sign, &p->tw[k]);
    return p;
}

void offt_plan_destroy(offt_plan *p)
{
    if (!p) return;
    free(p->tw);
    free(p->work);
    free(p);
}

static inline offt_cpx cmul(offt_cpx a, offt_cpx b)
{
    offt_cpx c;
    c.re = a.re * b.re - a.im * b.im;
    c.im = a.re * b.im + a.im * b.re;
    return c;
}

/* Combine p sub-transforms of length m stored at out[q*m + k]. fstride is
   n / (p*m): the twiddle for exponent e of W_{p*m} is tw[e * fstride]. */
static void butterfly(const offt_plan *pl, offt_cpx *out, int fstride, int m,
                      int p)
{
    const offt_cpx *tw = pl->tw;
    const int n = pl->n;
    if (p == 2) {
        for (int k = 0; k < m; ++k) {
            offt_cpx a = out[k];
            offt_cpx b = cmul(out[k + m], tw[k * fstride]);
            out[k].re = a.re + b.re;
            out[k].im = a.im + b.im;
            out[k + m].re = a.re - b.re;
            out[k + m].im = a.im - b.im;
        }
    } else if (p == 4) {
        const double s = (double)pl->sign; /* W_4 = s*i */
        for (int k = 0; k < m; ++k) {
            offt_cpx t0 = out[k];
            offt_cpx t1 = cmul(out[k + m], tw[k * fstride]);
            offt_cpx t2 = cmul(out[k + 2 * m], tw[2 * k * fstride]);
            offt_cpx t3 = cmul(out[k + 3 * m], tw[3 * k * fstride]);
            double a0r = t0.re + t2.re, a0i = t0.im + t2.im;
            double a1r = t0.re - t2.re, a1i = t0.im - t2.im;
            double b0r = t1.re + t3.re, b0i = t1.im + t3.im;
            double b1r = t1.re - t3.re, b1i = t1.im - t3.im;
            /* s*i*(b1) = (-s*b1i, s*b1r) */
            out[k].re = a0r + b0r;
            out[k].im = a0i + b0i;
            out[k + m].re = a1r - s * b1i;
            out[k + m].im = a1i + s * b1r;
            out[k + 2 * m].re = a0r - b0r;
            out[k + 2 * m].im = a0i - b0i;
            out[k + 3 * m].re = a1r + s * b1i;
            out[k + 3 * m].im = a1i - s * b1r;
        }
    } else if (p == 3) {
        /* W_3 = -1/2 + i*h, h = sign*sin(2pi/3) */
        const double h = tw[fstride * m].im;
        for (int k = 0; k < m; ++k) {
            offt_cpx t0 = out[k];
            offt_cpx t1 = cmul(out[k + m], tw[k * fstride]);
            offt_cpx t2 = cmul(out[k + 2 * m], tw[2 * k * fstride]);
            double sr = t1.re + t2.re, si = t1.im + t2.im;
            double dr = t1.re - t2.re, di = t1.im - t2.im;
            double mr = t0.re - 0.5 * sr, mi = t0.im - 0.5 * si;
            out[k].re = t0.re + sr;
            out[k].im = t0.im + si;
            /* i*h*d = (-h*di, h*dr) */
            out[k + m].re = mr - h * di;
            out[k + m].im = mi + h * dr;
            out[k + 2 * m].re = mr + h * di;
            out[k + 2 * m].im = mi - h * dr;
        }
    } else {
        /* generic p-point DFT */
        offt_cpx t[64];
        offt_cpx *tt = p <= 64 ? t : (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)p);
        for (int k = 0; k < m; ++k) {
            for (int q = 0; q < p; ++q) tt[q] = cmul(out[k + q * m], tw[(long)q * k * fstride % n]);
            for (int u = 0; u < p; ++u) {
                double ar = 0.0, ai = 0.0;
                for (int q = 0; q < p; ++q) {
                    offt_cpx w = tw[((long)u * q % p) * fstride * m];
                    ar += tt[q].re * w.re - tt[q].im * w.im;
                    ai += tt[q].re * w.im + tt[q].im * w.re;
                }
                out[k + u * m].re = ar;
                out[k + u * m].im = ai;
            }
        }
        if (tt != t) free(tt);
    }
}

/* Transform the sequence in[0], in[is], ..., in[(len-1)*is] into out[0..len-1]
   where len = product of fac[fi..]. fstride = n / len. */
static void rec(const offt_plan *pl, const offt_cpx *in, long is, offt_cpx *out,
                int fi, int fstride)
{
    const int p = pl->fac[fi];
    int m = 1;
    for (int f = fi + 1; f < pl->nfac; ++f) m *= pl->fac[f];
    if (m == 1) {
        for (int q = 0; q < p; ++q) out[q] = in[q * is];
    } else {
        for (int q = 0; q < p; ++q)
            rec(pl, in + q * is, is * p, out + q * m, fi + 1, fstride * p);
    }
    butterfly(pl, out, fstride, m, p);
}

void offt_exec(offt_plan *p, const offt_cpx *in, int istride, offt_cpx *out,
               int ostride)
{
    const int n = p->n;
    if (n <= 0) return;
    offt_cpx *src = p->work;       /* copy of the input */
    offt_cpx *dst = p->work + n;   /* result */
    for (int j = 0; j < n; ++j) src[j] = in[(long)j * istride];
    if (n == 1) {
        dst[0] = src[0];
    } else {
        rec(p, src, 1, dst, 0, 1);
    }
    for (int j = 0; j < n; ++j) out[(long)j * ostride] = dst[j];
}

offt_rplan *offt_rplan_create(int n, int dir)
{
    offt_rplan *p = (offt_rplan *)calloc(1, sizeof(offt_rplan));
    if (!p) return NULL;
    p->n = n;
    p->dir = dir;
    if (n % 2 == 0) {
        p->half = offt_plan_create(n / 2, dir);
    } else {
        p->full = offt_plan_create(n, dir);
    }
    p->tw = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)(n / 2 + 1));
    for (int k = 0; k <= n / 2; ++k) unit_root(n, k, dir, &p->tw[k]);
    p->work = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)(2 * n + 4));
    return p;
}

void offt_rplan_destroy(offt_rplan *p)
{
    if (!p) return;
    offt_plan_destroy(p->half);
    offt_plan_destroy(p->full);
    free(p->tw);
    free(p->work);
    free(p);
}

void offt_r2c(offt_rplan *p, const double *in, int istride, offt_cpx *out,
              int ostride)
{
    const int n = p->n;
    offt_cpx *z = p->work;
    if (n % 2) {
        for (int j = 0; j < n; ++j) { z[j].re = in[(long)j * istride]; z[j].im = 0.0; }
        offt_exec(p->full, z, 1, z + n, 1);
        for (int k = 0; k <= n / 2; ++k) out[(long)k * ostride] = z[n + k];
        out[0].im = 0.0;
        return;
    }
    const int N = n / 2;
    /* pack even/odd samples into one complex sequence */
    for (int m = 0; m < N; ++m) {
        z[m].re = in[(long)(2 * m) * istride];
        z[m].im = in[(long)(2 * m + 1) * istride];
    }
    offt_cpx *Z = z + N;
    offt_exec(p->half, z, 1, Z, 1);
    Z[N] = Z[0];
    /* X_k = E_k + w^k O_k, E_k = (Z_k + conj Z_{N-k})/2, O_k = (Z_k - conj Z_{N-k})/(2i) */
    offt_cpx X[2];
    for (int k = 0; k <= N; ++k) {
        offt_cpx a = Z[k], b = Z[N - k];
        double er = 0.5 * (a.re + b.re), ei = 0.5 * (a.im - b.im);
        double orr = 0.5 * (a.im + b.im), oi = -0.5 * (a.re - b.re);
        offt_cpx o = { orr, oi };
        offt_cpx wo = cmul(o, p->tw[k]);
        X[0].re = er + wo.re;
        X[0].im = ei + wo.im;
        out[(long)k * ostride] = X[0];
    }
    out[0].im = 0.0;
    out[(long)N * ostride].im = 0.0;
}

void offt_c2r(offt_rplan *p, const offt_cpx *in, int istride, double *out,
              int ostride)
{
    const int n = p->n;
    offt_cpx *z = p->work;
    if (n % 2) {
        /* Hermitian extension, then a full complex transform */
        for (int k = 0; k <= n / 2; ++k) z[k] = in[(long)k * istride];
        z[0].im = 0.0;
        for (int k = n / 2 + 1; k < n; ++k) { z[k].re = z[n - k].re; z[k].im = -z[n - k].im; }
        offt_exec(p->full, z, 1, z + n, 1);
        for (int j = 0; j < n; ++j) out[(long)j * ostride] = z[n + j].re;
        return;
    }
    const int N = n / 2;
    offt_cpx *X = z + 2 * N + 2;   /* local copy of the N+1 input bins */
    for (int k = 0; k <= N; ++k) X[k] = in[(long)k * istride];
    X[0].im = 0.0;
    X[N].im = 0.0;
    /* Z_k = (X_k + conj X_{N-k}) + i w^{k} (X_k - conj X_{N-k}),  w = exp(+2 pi i/n) */
    for (int k = 0; k < N; ++k) {
        offt_cpx a = X[k], b = X[N - k];
        double sr = a.re + b.re, si = a.im - b.im;
        offt_cpx d = { a.re - b.re, a.im + b.im };
        offt_cpx wd = cmul(d, p->tw[k]);
        z[k].re = sr - wd.im;
        z[k].im = si + wd.re;
    }
    offt_cpx *y = z + N;
    offt_exec(p->half, z, 1, y, 1);
    for (int m = 0; m < N; ++m) {
        out[(long)(2 * m) * ostride] = y[m].re;
        out[(long)(2 * m + 1) * ostride] = y[m].im;
    }
}
