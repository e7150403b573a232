/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle restatement; see chan_port.h.
 *
 * Every routine cites the reference file:line it restates.  Expressions keep
 * the reference's association so a no-FMA build matches the compiled
 * reference bit for bit.  Side outputs the reference computes but no entry
 * point can observe (the wall-derivative vectors Uxb/Uzb/HUxb/... and the
 * boundary-lift arrays) are not restated.  The "wasted" halves that do cost
 * time in the reference (pass1's tangent products during a plain primal run,
 * pass2's incremental-adjoint products) are restated, so that timing this
 * port is a fair stand-in for timing the reference.
 */
#include "chan_port.h"
#include "fft.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef offt_cpx cpx;

/* index constants, channel/minChnl.h:44-73 */
enum { XEL = 0, YEL = 1, ZEL = 2, DXEL = 3, DZEL = 4 };
enum { HXEL = 1, HYEL = 2, HZEL = 0 };
enum { WXEL = 4, WYEL = 5, WZEL = 3 };
enum { AXEL = 6, AYEL = 7, AZEL = 8 };
enum { SXEL = 1, SYEL = 2, SZEL = 0 };
enum { TXEL = 5, TYEL = 3, TZEL = 4 };
enum { ALPHA = 0, BETA = 1 };
#define MAXU 5
#define MAXT 6
#define MAXTT 9
#define QSDIAG 5
#define QPSDIAG 4
#define QPPSDIAG 3
#define RSDIAG 3
#define RPSDIAG 2
#define T_QSDIAG 9
#define T_RSDIAG 5
#define CFL_MAX 2.8
#define ITMAX 200
#define TOL 1E-15
#define MAXI(a, b) ((a) > (b) ? (a) : (b))
#define MINI(a, b) ((a) < (b) ? (a) : (b))

/* forward RK3 coefficients, project.c:44-47 */
static const double fa_[3] = { 1. / 3., -1. / 2, 1. / 3. };
static const double fb_[3] = { 1. / 6, 2. / 3, 0. };
static const double fc_[3] = { 1. / 2, 1. / 3., 1., };
static const double fd_[3] = { 0., -1. / 6, -2. / 3 };
/* adjoint RK3 coefficients, adjproject.c:34-37 */
static const double aa_[3] = { 1. / 3., -1. / 2, 1. / 3. };
static const double ab_[3] = { 2. / 3, 1. / 6, 0. };
static const double ac_[3] = { 1., 1. / 3., 1. / 2., };
static const double ad_[3] = { 0., -2. / 3, -1. / 6 };

struct cport {
    int Nx, Ny, Nz, X, qpts, dimR, dimQ, nsteps, pz, px, hx;
    double dt, re, flux, cfl1, cfl3;
    double *Kx, *Kz, *K2, *cfl2;
    double *Qy, *W, *Q, *Qp, *Qpp, *R, *Rp, *Qw, *Qpw, *Qppw, *Rw, *Rpw;
    double *Qs, *Qps, *Qpps, *Rs, *Rps;
    cpx *C, *IC, *AC, *U, *IU, *AU, *IAU, *LU, *MC, *MIC;
    double *MFT;   /* primal flux correction flux_t of each stored substage (not in the reference) */
    cpx *CT, *ICT;
    double *M, *MZ;
    cpx *Fa, *Fb, *TM, *fa, *fb, *tm, *add;
    cpx *ddt_dCdt;
    double *ddt_dudt, *ddt_v;
    offt_plan *pf1, *pf2;
    offt_rplan *pr1, *pr2;
    size_t csz, usz;
};

/* element offsets */
static inline size_t CI(const cport *s, int z, int v, int j, int x)
{
    return (((size_t)z * 2 + v) * s->dimR + j) * s->X + x;
}
static inline size_t UI(const cport *s, int z, int c, int y, int x)
{
    return (((size_t)z * 5 + c) * s->qpts + y) * s->X + x;
}
static inline size_t TI(const cport *s, int i, int z, int x)
{
    return ((size_t)i * s->pz + z) * s->hx + x;
}

/* ------------------------------------------------------------------ */
/* Legendre setup: LegendreSetup.c:25-527, 535-765; RsQs.c:55-174      */
/* ------------------------------------------------------------------ */

/* LegendreSetup.c:535-549 */
static double legendre(int n, double x)
{
    double y, prev = 0., curr = 1.;
    for (int j = 0; j < n; ++j) {
        y = ((double)(2 * j + 1) * x * curr - (double)j * prev) / (double)(j + 1);
        prev = curr;
        curr = y;
    }
    return curr;
}

/* LegendreSetup.c:566-643: Chebyshev bracketing + modified secant */
static int qpoints(int n, double *x)
{
    int k = n, m = 0, r, nd2 = n / 2;
    double p1, p2, p3, x1, x2, x3 = 0.0;
    double *xe = (double *)calloc((size_t)n, sizeof(double));
    if (!xe) return -2;
    while (m < nd2) {
        k = 2 * k;
        x1 = -1.0;
        p1 = legendre(n, x1);
        m = 0;
        for (r = 1; r <= k; ++r) {
            x2 = -cos(0.5 * M_PI * (r - 0.5) / k);
            p2 = legendre(n, x2);
            if (p1 * p2 < 0) {
                x[m] = x1;
                xe[m] = x2;
                m = m + 1;
            }
            p1 = p2;
            x1 = x2;
        }
    }
    for (m = 0; m < nd2; ++m) {
        x1 = x[m];
        x2 = xe[m];
        p1 = legendre(n, x1);
        p2 = legendre(n, x2);
        r = 1;
        while (fabs(x2 - x1) > TOL && r < ITMAX) {
            if (r % 10 == 0) {
                x3 = 0.5 * (x1 + x2);
            } else {
                if (fabs(p1) < fabs(p2)) {
                    x3 = x1 + MAXI(0.05, p1 / (p1 - p2)) * (x2 - x1);
                } else {
                    x3 = x2 + MINI(-0.05, p2 / (p1 - p2)) * (x2 - x1);
                }
            }
            p3 = legendre(n, x3);
            if (p3 * p1 <= 0) {
                x2 = x3;
                p2 = p3;
            } else {
                x1 = x3;
                p1 = p3;
            }
            r = r + 1;
        }
        if (r == ITMAX) {
            free(xe);
            return -3;
        }
        x[m] = x3;
        x[n - 1 - m] = -x3;
    }
    if (n % 2 == 1) x[nd2] = 0.0;
    free(xe);
    return 0;
}

/* LegendreSetup.c:732-745 */
static void qweights(int n, const double *x, double *w)
{
    int lim = (n + 1) / 2;
    for (int k = 0; k < lim; ++k) {
        double v1 = (double)n * (legendre(n - 1, x[k]) - x[k] * legendre(n, x[k]));
        w[k] = 2. * (1. - x[k] * x[k]) / (v1 * v1);
        w[n - 1 - k] = w[k];
    }
}

/* LegendreSetup.c:663-675: P[m][n] = P_n(x_m) */
static void legendre_matrix(double *P, int rows, int cols, const double *x)
{
    for (int m = 0; m < rows; ++m) {
        P[m * cols + 0] = 1.0;
        P[m * cols + 1] = x[m];
        for (int n = 1; n < cols - 1; ++n) {
            P[m * cols + n + 1] = ((2. * n + 1.) * (x[m] * P[m * cols + n]) -
                                   n * P[m * cols + n - 1]) / (double)(n + 1);
        }
    }
}

/* LegendreSetup.c:756-765: Mw[i][j] = w[j] * M[j][i]; M is dim2 x dim1 */
static void weights_to_m(double *Mw, const double *M, int dim1, int dim2, const double *w)
{
    for (int i = 0; i < dim1; ++i)
        for (int j = 0; j < dim2; ++j)
            Mw[i * dim2 + j] = w[j] * M[j * dim1 + i];
}

/* LegendreSetup.c:698-720: banded Gram matrix, every other diagonal */
static void ldiags(double *D, int n, int m, int start, int diags,
                   const double *A, int Adim2, const double *B, int Bcols)
{
    for (int i = 0; i < n * m; ++i) D[i] = 0.0;
    int i, s;
    for (i = start, s = 0; s < diags; ++i, ++s) {
        for (int j = 0; j < n - 2 * s; ++j) {
            for (int k = 0; k < Adim2; ++k) {
                D[j * m + diags - 1 + i] = D[j * m + diags - 1 + i] +
                    A[j * Adim2 + k] * B[k * Bcols + j + 2 * s];
            }
            if (i != start) {
                D[(2 * s + j) * m + diags - 1 + i - 2 * s] = D[j * m + diags - 1 + i];
            }
        }
    }
}

static int legendre_setup(cport *s)
{
    const int q = s->qpts, R = s->dimR, D = s->dimQ;
    double *y = s->Qy, *w = s->W;
    double *P = (double *)malloc(sizeof(double) * (size_t)q * R);
    double *T = (double *)malloc(sizeof(double) * (size_t)R * q);
    if (!P || !T) { free(P); free(T); return -2; }
    int err = qpoints(q, y);
    if (err) { free(P); free(T); return err; }
    qweights(q, y, w);
    legendre_matrix(P, q, R, y);
    /* RsQs.c:55-68 CreateR */
    for (int i = 0; i < q; ++i) {
        double wrk = 1.0 - y[i] * y[i];
        for (int j = 0; j < R; ++j) s->R[i * R + j] = wrk * P[i * R + j];
    }
    /* RsQs.c:91-104 CreateQ */
    for (int i = 0; i < q; ++i) {
        double wrk = 1.0 - y[i] * y[i];
        for (int j = 0; j < D; ++j) s->Q[i * D + j] = wrk * s->R[i * R + j];
    }
    /* RsQs.c:110-126 CreateQp */
    for (int i = 0; i < q; ++i) {
        double wrk = 1.0 - y[i] * y[i];
        s->Qp[i * D + 0] = -4.0 * y[i] * wrk;
        for (int j = 1; j < D; ++j)
            s->Qp[i * D + j] = wrk * (j * P[i * R + j - 1] - (j + 4.0) * (y[i] * P[i * R + j]));
    }
    /* RsQs.c:133-150 CreateQpp */
    for (int i = 0; i < q; ++i) {
        double wrk = y[i] * y[i];
        s->Qpp[i * D + 0] = 12.0 * wrk - 4.0;
        for (int j = 1; j < D; ++j)
            s->Qpp[i * D + j] = (12.0 + 7.0 * j + j * j) * (wrk * P[i * R + j]) -
                (4.0 + j * j + j) * P[i * R + j] - 6.0 * j * (y[i] * P[i * R + j - 1]);
    }
    /* RsQs.c:73-86 CreateRp */
    for (int i = 0; i < q; ++i) {
        s->Rp[i * R + 0] = -2.0 * y[i];
        for (int j = 1; j < R; ++j)
            s->Rp[i * R + j] = j * P[i * R + j - 1] - (j + 2.0) * (y[i] * P[i * R + j]);
    }
    /* LegendreSetup.c:476-490 */
    weights_to_m(s->Qw, s->Q, D, q, w);
    weights_to_m(s->Qpw, s->Qp, D, q, w);
    weights_to_m(s->Qppw, s->Qpp, D, q, w);
    weights_to_m(s->Rw, s->R, R, q, w);
    weights_to_m(s->Rpw, s->Rp, R, q, w);
    ldiags(s->Qs, D, T_QSDIAG, 0, QSDIAG, s->Qw, q, s->Q, D);
    ldiags(s->Qps, D, T_QSDIAG, 1, QPSDIAG, s->Qpw, q, s->Qp, D);
    weights_to_m(T, s->Qpp, D, q, w);
    ldiags(s->Qpps, D, T_QSDIAG, 2, QPPSDIAG, T, q, s->Qpp, D);
    ldiags(s->Rs, R, T_RSDIAG, 0, RSDIAG, s->Rw, q, s->R, R);
    weights_to_m(T, s->Rp, R, q, w);
    ldiags(s->Rps, R, T_RSDIAG, 1, RPSDIAG, T, q, s->Rp, R);
    free(P);
    free(T);
    return 0;
}

/* waveNumsAndCFL.c:22-62 */
static void wave_nums(cport *s, double Lx, double Lz)
{
    const int x = s->X, z = s->Nz;
    for (int i = 0; i < x; ++i) s->Kx[i] = i * (2. * M_PI / Lx);
    for (int i = 0; i < z / 2 + 1; ++i) s->Kz[i] = i * (2. * M_PI / Lz);
    for (int i = z / 2 + 1; i < z; ++i) s->Kz[i] = (i - z) * (2. * M_PI / Lz);
    for (int i = 0; i < z; ++i)
        for (int j = 0; j < x; ++j)
            s->K2[i * x + j] = s->Kz[i] * s->Kz[i] + s->Kx[j] * s->Kx[j];
}

/* waveNumsAndCFL.c:65-96 */
static int cfl_vars(cport *s, double Lx, double Lz)
{
    const int q = s->qpts;
    double *y = (double *)malloc(sizeof(double) * (size_t)q);
    if (!y) return -2;
    int j = qpoints(q, y);
    if (j) { free(y); return j; }
    s->cfl1 = M_PI / (Lx / s->Nx);
    s->cfl3 = M_PI / (Lz / s->Nz);
    for (j = 1; j < q - 1; ++j) s->cfl2[j] = 2. * M_PI / (y[j + 1] - y[j - 1]);
    s->cfl2[0] = s->cfl2[q - 1] = M_PI / (y[0] + 1.0);
    free(y);
    return 0;
}

/* ------------------------------------------------------------------ */
/* banded solves, mvOps.c:29-237.  A is [N][9][X] (pitch 9 per row),  */
/* b is an [N][X] complex block (row pitch X).                        */
/* ------------------------------------------------------------------ */
#define A3(i, j, x) A[((size_t)(i) * 9 + (j)) * X + (x)]

/* mvOps.c:29-91 */
static void bsolve(double *A, cpx *b, int dl, int du, int N, int X, int x0)
{
    int i, j, k, x;
    for (i = 2; i < N; ++i) {
        for (j = MAXI(0, dl - (i / 2)); j < dl; ++j) {
            for (k = 1; k <= j - MAXI(0, dl - (i / 2)); ++k)
                for (x = x0; x < X; ++x)
                    A3(i, j, x) = A3(i, j, x) - A3(i, j - k, x) * A3(i - 2 * (dl - j + k), dl + k, x);
            for (x = x0; x < X; ++x) {
                A3(i, j, x) = A3(i, j, x) / A3(i - 2 * (dl - j), dl, x);
                b[i * X + x].re = b[i * X + x].re - A3(i, j, x) * b[(i - 2 * (dl - j)) * X + x].re;
                b[i * X + x].im = b[i * X + x].im - A3(i, j, x) * b[(i - 2 * (dl - j)) * X + x].im;
            }
        }
        for (j = 0; j < MINI(du, (N - i + 1) / 2); ++j)
            for (k = 1; k <= MINI(i / 2, MINI(dl, du - j)); ++k)
                for (x = x0; x < X; ++x)
                    A3(i, j + dl, x) = A3(i, j + dl, x) - A3(i, dl - k, x) * A3(i - 2 * k, dl + j + k, x);
    }
    for (x = x0; x < X; ++x) {
        b[(N - 1) * X + x].re = b[(N - 1) * X + x].re / A3(N - 1, dl, x);
        b[(N - 1) * X + x].im = b[(N - 1) * X + x].im / A3(N - 1, dl, x);
    }
    for (x = x0; x < X; ++x) {
        b[(N - 2) * X + x].re = b[(N - 2) * X + x].re / A3(N - 2, dl, x);
        b[(N - 2) * X + x].im = b[(N - 2) * X + x].im / A3(N - 2, dl, x);
    }
    for (i = N - 3; i >= 0; --i) {
        for (j = 1; j <= MINI(du, ((N - i + 1) / 2 - 1)); ++j)
            for (x = x0; x < X; ++x) {
                b[i * X + x].re = b[i * X + x].re - A3(i, dl + j, x) * b[(i + 2 * j) * X + x].re;
                b[i * X + x].im = b[i * X + x].im - A3(i, dl + j, x) * b[(i + 2 * j) * X + x].im;
            }
        for (x = x0; x < X; ++x) {
            b[i * X + x].re = b[i * X + x].re / A3(i, dl, x);
            b[i * X + x].im = b[i * X + x].im / A3(i, dl, x);
        }
    }
}

/* mvOps.c:198-220 */
static void smmult(const double *A, const cpx *y, cpx *b, int dl, int du, int N, int X, int x0)
{
    int i, j, x;
    for (i = 0; i < N; ++i)
        for (x = x0; x < X; ++x) { b[i * X + x].re = 0.0; b[i * X + x].im = 0.0; }
    for (i = 0; i < N; ++i)
        for (j = MAXI(0, dl - (i / 2)); j < MINI(dl + du + 1, (N - i + 1) / 2 + dl); ++j)
            for (x = x0; x < X; ++x) {
                b[i * X + x].re = b[i * X + x].re + A3(i, j, x) * y[(i - 2 * (dl - j)) * X + x].re;
                b[i * X + x].im = b[i * X + x].im + A3(i, j, x) * y[(i - 2 * (dl - j)) * X + x].im;
            }
}
#undef A3

/* Single matrix A[N][w] (pitch w).  The right-hand side is element bs*i of b.
   mvOps.c:97-144 (bsolve0, column 0 of a 2D array, bs = X) and
   mvOps.c:149-194 (bsolve_0, a plain vector, bs = 1). */
static void bsolve_single(double *A, int w, cpx *b, int bs, int dl, int du, int N)
{
    int i, j, k;
#define A2(i, j) A[(size_t)(i) * w + (j)]
    for (i = 2; i < N; ++i) {
        for (j = MAXI(0, dl - (i / 2)); j < dl; ++j) {
            for (k = 1; k <= j - MAXI(0, dl - (i / 2)); ++k)
                A2(i, j) = A2(i, j) - A2(i, j - k) * A2(i - 2 * (dl - j + k), dl + k);
            A2(i, j) = A2(i, j) / A2(i - 2 * (dl - j), dl);
            b[i * bs].re = b[i * bs].re - A2(i, j) * b[(i - 2 * (dl - j)) * bs].re;
            b[i * bs].im = b[i * bs].im - A2(i, j) * b[(i - 2 * (dl - j)) * bs].im;
        }
        for (j = 0; j < MINI(du, (N - i + 1) / 2); ++j)
            for (k = 1; k <= MINI(i / 2, MINI(dl, du - j)); ++k)
                A2(i, j + dl) = A2(i, j + dl) - A2(i, dl - k) * A2(i - 2 * k, dl + j + k);
    }
    b[(N - 1) * bs].re = b[(N - 1) * bs].re / A2(N - 1, dl);
    b[(N - 1) * bs].im = b[(N - 1) * bs].im / A2(N - 1, dl);
    b[(N - 2) * bs].re = b[(N - 2) * bs].re / A2(N - 2, dl);
    b[(N - 2) * bs].im = b[(N - 2) * bs].im / A2(N - 2, dl);
    for (i = N - 3; i >= 0; --i) {
        for (j = 1; j <= MINI(du, ((N - i + 1) / 2 - 1)); ++j) {
            b[i * bs].re = b[i * bs].re - A2(i, dl + j) * b[(i + 2 * j) * bs].re;
            b[i * bs].im = b[i * bs].im - A2(i, dl + j) * b[(i + 2 * j) * bs].im;
        }
        b[i * bs].re = b[i * bs].re / A2(i, dl);
        b[i * bs].im = b[i * bs].im / A2(i, dl);
    }
#undef A2
}

/* initAlphaBeta.c:235-266 bsolveI: one matrix, many right-hand sides */
static void bsolve_shared(double *A, int w, cpx *b, int dl, int du, int N, int X, int x0)
{
    int i, j, k, x;
#define A2(i, j) A[(size_t)(i) * w + (j)]
    for (i = 2; i < N; ++i) {
        for (j = MAXI(0, dl - (i / 2)); j < dl; ++j) {
            for (k = 1; k <= j - MAXI(0, dl - (i / 2)); ++k)
                A2(i, j) = A2(i, j) - A2(i, j - k) * A2(i - 2 * (dl - j + k), dl + k);
            A2(i, j) = A2(i, j) / A2(i - 2 * (dl - j), dl);
            for (x = x0; x < X; ++x) {
                b[i * X + x].re = b[i * X + x].re - A2(i, j) * b[(i - 2 * (dl - j)) * X + x].re;
                b[i * X + x].im = b[i * X + x].im - A2(i, j) * b[(i - 2 * (dl - j)) * X + x].im;
            }
        }
        for (j = 0; j < MINI(du, (N - i + 1) / 2); ++j)
            for (k = 1; k <= MINI(i / 2, MINI(dl, du - j)); ++k)
                A2(i, j + dl) = A2(i, j + dl) - A2(i, dl - k) * A2(i - 2 * k, dl + j + k);
    }
    for (x = x0; x < X; ++x) {
        b[(N - 1) * X + x].re = b[(N - 1) * X + x].re / A2(N - 1, dl);
        b[(N - 1) * X + x].im = b[(N - 1) * X + x].im / A2(N - 1, dl);
    }
    for (x = x0; x < X; ++x) {
        b[(N - 2) * X + x].re = b[(N - 2) * X + x].re / A2(N - 2, dl);
        b[(N - 2) * X + x].im = b[(N - 2) * X + x].im / A2(N - 2, dl);
    }
    for (i = N - 3; i >= 0; --i) {
        for (j = 1; j <= MINI(du, ((N - i + 1) / 2 - 1)); ++j)
            for (x = x0; x < X; ++x) {
                b[i * X + x].re = b[i * X + x].re - A2(i, dl + j) * b[(i + 2 * j) * X + x].re;
                b[i * X + x].im = b[i * X + x].im - A2(i, dl + j) * b[(i + 2 * j) * X + x].im;
            }
        for (x = x0; x < X; ++x) {
            b[i * X + x].re = b[i * X + x].re / A2(i, dl);
            b[i * X + x].im = b[i * X + x].im / A2(i, dl);
        }
    }
#undef A2
}

/* mvOps.c:223-237: y element stride ys */
static void smmult_single(const double *A, int w, const cpx *y, int ys, cpx *b, int dl, int du, int N)
{
    for (int i = 0; i < N; ++i) {
        b[i].re = 0.0;
        b[i].im = 0.0;
        for (int j = MAXI(0, dl - (i / 2)); j < MINI(dl + du + 1, (N - i + 1) / 2 + dl); ++j) {
            b[i].re = b[i].re + A[i * w + j] * y[(i - 2 * (dl - j)) * ys].re;
            b[i].im = b[i].im + A[i * w + j] * y[(i - 2 * (dl - j)) * ys].im;
        }
    }
}

/* ------------------------------------------------------------------ */
/* coefficients -> velocity (initAlphaBeta2.c:12-240; the incre_ and  */
/* adj_ copies are the same arithmetic on other arrays)               */
/* ------------------------------------------------------------------ */
static void recon_line(cport *s, const cpx *C, cpx *U, int z, int x0)
{
    const int X = s->X, q = s->qpts, D = s->dimQ, R = s->dimR;
    int i, j, x;
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) { U[UI(s, z, YEL, i, x)].re = 0; U[UI(s, z, YEL, i, x)].im = 0; }
    for (i = 0; i < q; ++i) for (j = 0; j < D; ++j) for (x = x0; x < X; ++x) {
        U[UI(s, z, YEL, i, x)].re += s->Q[i * D + j] * C[CI(s, z, ALPHA, j, x)].re;
        U[UI(s, z, YEL, i, x)].im += s->Q[i * D + j] * C[CI(s, z, ALPHA, j, x)].im;
    }
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) { U[UI(s, z, XEL, i, x)].re = 0; U[UI(s, z, XEL, i, x)].im = 0; }
    for (i = 0; i < q; ++i) for (j = 0; j < D; ++j) for (x = x0; x < X; ++x) {
        U[UI(s, z, XEL, i, x)].re -= s->Qp[i * D + j] * C[CI(s, z, ALPHA, j, x)].re;
        U[UI(s, z, XEL, i, x)].im -= s->Qp[i * D + j] * C[CI(s, z, ALPHA, j, x)].im;
    }
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) { U[UI(s, z, DXEL, i, x)].re = 0; U[UI(s, z, DXEL, i, x)].im = 0; }
    for (i = 0; i < q; ++i) for (j = 0; j < D; ++j) for (x = x0; x < X; ++x) {
        U[UI(s, z, DXEL, i, x)].re += s->Qpp[i * D + j] * C[CI(s, z, ALPHA, j, x)].re;
        U[UI(s, z, DXEL, i, x)].im += s->Qpp[i * D + j] * C[CI(s, z, ALPHA, j, x)].im;
    }
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) { U[UI(s, z, ZEL, i, x)].re = 0; U[UI(s, z, ZEL, i, x)].im = 0; }
    for (i = 0; i < q; ++i) for (j = 0; j < R; ++j) for (x = x0; x < X; ++x) {
        U[UI(s, z, ZEL, i, x)].re += s->R[i * R + j] * C[CI(s, z, BETA, j, x)].re;
        U[UI(s, z, ZEL, i, x)].im += s->R[i * R + j] * C[CI(s, z, BETA, j, x)].im;
    }
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) { U[UI(s, z, DZEL, i, x)].re = 0; U[UI(s, z, DZEL, i, x)].im = 0; }
    for (i = 0; i < q; ++i) for (j = 0; j < R; ++j) for (x = x0; x < X; ++x) {
        U[UI(s, z, DZEL, i, x)].re += s->Rp[i * R + j] * C[CI(s, z, BETA, j, x)].re;
        U[UI(s, z, DZEL, i, x)].im += s->Rp[i * R + j] * C[CI(s, z, BETA, j, x)].im;
    }
    const double kz = s->Kz[z];
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) {
        const double kx = s->Kx[x], k2 = s->K2[z * X + x];
        cpx *ux = &U[UI(s, z, XEL, i, x)], *uz = &U[UI(s, z, ZEL, i, x)];
        double t0 = ux->re, t1 = uz->re;
        ux->re = (kx * ux->im + kz * uz->im) / k2;
        uz->re = (-kx * uz->im + kz * ux->im) / k2;
        ux->im = -(kx * t0 + kz * t1) / k2;
        uz->im = (kx * t1 - kz * t0) / k2;
    }
    for (i = 0; i < q; ++i) for (x = x0; x < X; ++x) {
        const double kx = s->Kx[x], k2 = s->K2[z * X + x];
        cpx *dx = &U[UI(s, z, DXEL, i, x)], *dz = &U[UI(s, z, DZEL, i, x)];
        double t0 = dx->re, t1 = dz->re;
        dx->re = (-kx * dx->im + kz * dz->im) / k2;
        dz->re = -(kx * dz->im + kz * dx->im) / k2;
        dx->im = (kx * t0 - kz * t1) / k2;
        dz->im = (kx * t1 + kz * t0) / k2;
    }
}

/* (0,0) mean-flow column, initAlphaBeta2.c:25-68 / project0.c:178-221 */
static void recon_mean(cport *s, const cpx *C, cpx *U)
{
    const int q = s->qpts, R = s->dimR;
    for (int i = 0; i < q; ++i) {
        cpx *u = &U[UI(s, 0, XEL, i, 0)];
        u->re = 0.0; u->im = 0.0;
        for (int j = 0; j < R; ++j) { u->re += s->R[i * R + j] * C[CI(s, 0, ALPHA, j, 0)].re; u->im += s->R[i * R + j] * C[CI(s, 0, ALPHA, j, 0)].im; }
    }
    for (int i = 0; i < q; ++i) {
        cpx *u = &U[UI(s, 0, DXEL, i, 0)];
        u->re = 0.0; u->im = 0.0;
        for (int j = 0; j < R; ++j) { u->re += s->Rp[i * R + j] * C[CI(s, 0, ALPHA, j, 0)].re; u->im += s->Rp[i * R + j] * C[CI(s, 0, ALPHA, j, 0)].im; }
    }
    for (int i = 0; i < q; ++i) { U[UI(s, 0, YEL, i, 0)].re = 0.0; U[UI(s, 0, YEL, i, 0)].im = 0.0; }
    for (int i = 0; i < q; ++i) {
        cpx *u = &U[UI(s, 0, ZEL, i, 0)];
        u->re = 0.0; u->im = 0.0;
        for (int j = 0; j < R; ++j) { u->re += s->R[i * R + j] * C[CI(s, 0, BETA, j, 0)].re; u->im += s->R[i * R + j] * C[CI(s, 0, BETA, j, 0)].im; }
    }
    for (int i = 0; i < q; ++i) {
        cpx *u = &U[UI(s, 0, DZEL, i, 0)];
        u->re = 0.0; u->im = 0.0;
        for (int j = 0; j < R; ++j) { u->re += s->Rp[i * R + j] * C[CI(s, 0, BETA, j, 0)].re; u->im += s->Rp[i * R + j] * C[CI(s, 0, BETA, j, 0)].im; }
    }
}

static void recon(cport *s, const cpx *C, cpx *U)
{
    recon_mean(s, C, U);
    recon_line(s, C, U, 0, 1);
    for (int z = 1; z < s->Nz; ++z) recon_line(s, C, U, z, 0);
}

/* ------------------------------------------------------------------ */
/* pass1 / pass2 (per y-plane transforms and nonlinear products)       */
/* ------------------------------------------------------------------ */

/* load 5 velocity components of plane y into a padded transform array
   and form the spectral vorticity, pass1.c:42-104 */
static void load_curl(cport *s, cpx *T, const cpx *U, int y)
{
    const int X = s->X, Nz = s->Nz, pz = s->pz;
    for (int i = 0; i < MAXU; ++i)
        for (int z = 0; z < Nz / 2; ++z)
            memcpy(&T[TI(s, i, z, 0)], &U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
    for (int z = 0; z < Nz / 2; ++z)
        for (int x = 0; x < X; ++x) {
            const double kz = s->Kz[z], kx = s->Kx[x];
            T[TI(s, WXEL, z, x)].re = T[TI(s, DZEL, z, x)].re + kz * T[TI(s, YEL, z, x)].im;
            T[TI(s, WXEL, z, x)].im = T[TI(s, DZEL, z, x)].im - kz * T[TI(s, YEL, z, x)].re;
            T[TI(s, WZEL, z, x)].re = -(T[TI(s, DXEL, z, x)].re + kx * T[TI(s, YEL, z, x)].im);
            T[TI(s, WZEL, z, x)].im = -T[TI(s, DXEL, z, x)].im + kx * T[TI(s, YEL, z, x)].re;
            T[TI(s, WYEL, z, x)].re = kx * T[TI(s, ZEL, z, x)].im - kz * T[TI(s, XEL, z, x)].im;
            T[TI(s, WYEL, z, x)].im = kz * T[TI(s, XEL, z, x)].re - kx * T[TI(s, ZEL, z, x)].re;
        }
    for (int i = 0; i < MAXU; ++i)
        for (int z = Nz / 2 + 1; z < Nz; ++z)
            memcpy(&T[TI(s, i, z + Nz / 2, 0)], &U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
    for (int z = Nz + 1; z < pz; ++z)
        for (int x = 0; x < X; ++x) {
            const double kz = s->Kz[z - Nz / 2], kx = s->Kx[x];
            T[TI(s, WXEL, z, x)].re = T[TI(s, DZEL, z, x)].re + kz * T[TI(s, YEL, z, x)].im;
            T[TI(s, WXEL, z, x)].im = T[TI(s, DZEL, z, x)].im - kz * T[TI(s, YEL, z, x)].re;
            T[TI(s, WZEL, z, x)].re = -(T[TI(s, DXEL, z, x)].re + kx * T[TI(s, YEL, z, x)].im);
            T[TI(s, WZEL, z, x)].im = -T[TI(s, DXEL, z, x)].im + kx * T[TI(s, YEL, z, x)].re;
            T[TI(s, WYEL, z, x)].re = kx * T[TI(s, ZEL, z, x)].im - kz * T[TI(s, XEL, z, x)].im;
            T[TI(s, WYEL, z, x)].im = kz * T[TI(s, XEL, z, x)].re - kx * T[TI(s, ZEL, z, x)].re;
        }
}

/* load 3 components (no curl) into fields off..off+2, pass2.c:113-125 */
static void load3(cport *s, cpx *T, const cpx *U, int y, int off)
{
    const int X = s->X, Nz = s->Nz;
    for (int i = 0; i < 3; ++i) {
        for (int z = 0; z < Nz / 2; ++z)
            memcpy(&T[TI(s, i + off, z, 0)], &U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
        for (int z = Nz / 2 + 1; z < Nz; ++z)
            memcpy(&T[TI(s, i + off, z + Nz / 2, 0)], &U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
    }
}

/* inverse transform of field i: z columns (x < Nx/2) then x rows, pass1.c:106-114 */
static void inverse_field(cport *s, cpx *T, int i)
{
    cpx *base = &T[TI(s, i, 0, 0)];
    for (int x = 0; x < s->X; ++x) offt_exec(s->pf1, base + x, s->hx, base + x, s->hx);
    for (int z = 0; z < s->pz; ++z)
        offt_c2r(s->pr1, base + (size_t)z * s->hx, 1, (double *)(base + (size_t)z * s->hx), 1);
}

/* forward transform of field i: x rows then z columns, pass1.c:312-319 */
static void forward_field(cport *s, cpx *T, int i)
{
    cpx *base = &T[TI(s, i, 0, 0)];
    for (int z = 0; z < s->pz; ++z)
        offt_r2c(s->pr2, (double *)(base + (size_t)z * s->hx), 1, base + (size_t)z * s->hx, 1);
    for (int x = 0; x < s->X; ++x) offt_exec(s->pf2, base + x, s->hx, base + x, s->hx);
}

/* scale the kept rows of field i by norm, pass1.c:322-339 */
static void scale_field(cport *s, cpx *T, int i, double norm)
{
    for (int z = 0; z < s->Nz / 2; ++z)
        for (int x = 0; x < s->X; ++x) {
            T[TI(s, i, z, x)].re = norm * T[TI(s, i, z, x)].re;
            T[TI(s, i, z, x)].im = norm * T[TI(s, i, z, x)].im;
        }
    for (int z = s->Nz + 1; z < s->pz; ++z)
        for (int x = 0; x < s->X; ++x) {
            T[TI(s, i, z, x)].re = norm * T[TI(s, i, z, x)].re;
            T[TI(s, i, z, x)].im = norm * T[TI(s, i, z, x)].im;
        }
}

static void store_field(cport *s, cpx *U, const cpx *T, int i, int slot, int y)
{
    for (int z = 0; z < s->Nz / 2; ++z)
        memcpy(&U[UI(s, z, slot, y, 0)], &T[TI(s, i, z, 0)], sizeof(cpx) * s->X);
    for (int z = s->Nz + 1; z < s->pz; ++z)
        memcpy(&U[UI(s, z - s->Nz / 2, slot, y, 0)], &T[TI(s, i, z, 0)], sizeof(cpx) * s->X);
}

/* pass1.c:13-376 */
static int pass1(cport *s, int dctr)
{
    const int pz = s->pz, px = s->px, rp = px + 2;
    const size_t idx = (size_t)pz * rp;
    double *RT = (double *)s->CT, *IRT = (double *)s->ICT;
    const double norm = 1.0 / ((3. * s->Nx / 2.) * (3. * s->Nz / 2.));
    for (int y = 0; y < s->qpts; ++y) {
        memset(s->CT, 0, sizeof(cpx) * (size_t)MAXT * pz * s->hx);
        load_curl(s, s->CT, s->U, y);
        for (int i = 0; i < MAXT; ++i) inverse_field(s, s->CT, i);
        if (dctr == 0) {
            double CFL = 0.0;
            for (int i = 0; i < pz; ++i)
                for (int j = 0; j < px; ++j) {
                    double t = fabs(RT[XEL * idx + (i * rp + j)]) * s->cfl1 +
                               fabs(RT[YEL * idx + (i * rp + j)]) * s->cfl2[y] +
                               fabs(RT[ZEL * idx + (i * rp + j)]) * s->cfl3;
                    if (t > CFL) CFL = t;
                }
            CFL *= s->dt;
            if (CFL >= CFL_MAX) {
                printf("Pass1:  CFL[%d]:%e, Max:%e dt:%e.  CFL condition violated.\n", y, CFL, CFL_MAX, s->dt);
                return -1;
            }
        }
        memset(s->ICT, 0, sizeof(cpx) * (size_t)MAXT * pz * s->hx);
        load_curl(s, s->ICT, s->IU, y);
        for (int i = 0; i < MAXT; ++i) inverse_field(s, s->ICT, i);
        for (int z = 0; z < pz; ++z)
            for (int x = 0; x < px; ++x) {
                const size_t o = (size_t)z * rp + x;
                double Iuy = IRT[YEL * idx + o];
                double uy = RT[YEL * idx + o];
                IRT[HXEL * idx + o] = IRT[YEL * idx + o] * RT[WZEL * idx + o] - IRT[ZEL * idx + o] * RT[WYEL * idx + o] +
                                      RT[YEL * idx + o] * IRT[WZEL * idx + o] - RT[ZEL * idx + o] * IRT[WYEL * idx + o];
                IRT[HYEL * idx + o] = IRT[ZEL * idx + o] * RT[WXEL * idx + o] - IRT[XEL * idx + o] * RT[WZEL * idx + o] +
                                      RT[ZEL * idx + o] * IRT[WXEL * idx + o] - RT[XEL * idx + o] * IRT[WZEL * idx + o];
                IRT[HZEL * idx + o] = IRT[XEL * idx + o] * RT[WYEL * idx + o] - Iuy * RT[WXEL * idx + o] +
                                      RT[XEL * idx + o] * IRT[WYEL * idx + o] - uy * IRT[WXEL * idx + o];
                RT[HXEL * idx + o] = RT[YEL * idx + o] * RT[WZEL * idx + o] - RT[ZEL * idx + o] * RT[WYEL * idx + o];
                RT[HYEL * idx + o] = RT[ZEL * idx + o] * RT[WXEL * idx + o] - RT[XEL * idx + o] * RT[WZEL * idx + o];
                RT[HZEL * idx + o] = RT[XEL * idx + o] * RT[WYEL * idx + o] - uy * RT[WXEL * idx + o];
            }
        for (int i = 0; i < 3; ++i) {
            forward_field(s, s->CT, i);
            scale_field(s, s->CT, i, norm);
            store_field(s, s->U, s->CT, i, i, y);
            forward_field(s, s->ICT, i);
            scale_field(s, s->ICT, i, norm);
            store_field(s, s->IU, s->ICT, i, i, y);
        }
    }
    return 0;
}

/* pass2.c:23-570 */
static void pass2(cport *s)
{
    const int pz = s->pz, px = s->px, rp = px + 2, X = s->X, Nz = s->Nz;
    const size_t idx = (size_t)pz * rp;
    double *RT = (double *)s->CT, *IRT = (double *)s->ICT;
    const double norm = 1.0 / ((3. * s->Nx / 2.) * (3. * s->Nz / 2.));
    for (int y = 0; y < s->qpts; ++y) {
        memset(s->CT, 0, sizeof(cpx) * (size_t)MAXTT * pz * s->hx);
        load_curl(s, s->CT, s->U, y);
        load3(s, s->CT, s->AU, y, MAXT);
        for (int i = 0; i < MAXTT; ++i) inverse_field(s, s->CT, i);
        memset(s->ICT, 0, sizeof(cpx) * (size_t)MAXTT * pz * s->hx);
        load_curl(s, s->ICT, s->IU, y);
        load3(s, s->ICT, s->IAU, y, MAXT);
        for (int i = 0; i < MAXTT; ++i) inverse_field(s, s->ICT, i);
        for (int z = 0; z < pz; ++z)
            for (int x = 0; x < px; ++x) {
                const size_t o = (size_t)z * rp + x;
                double Iuy = IRT[YEL * idx + o];
                double uy = RT[YEL * idx + o];
                double wy = RT[WYEL * idx + o];
                double Iwy = IRT[WYEL * idx + o];
                IRT[SXEL * idx + o] = RT[YEL * idx + o] * IRT[AZEL * idx + o] - RT[ZEL * idx + o] * IRT[AYEL * idx + o] +
                                      IRT[YEL * idx + o] * RT[AZEL * idx + o] - IRT[ZEL * idx + o] * RT[AYEL * idx + o];
                IRT[SYEL * idx + o] = RT[ZEL * idx + o] * IRT[AXEL * idx + o] - RT[XEL * idx + o] * IRT[AZEL * idx + o] +
                                      IRT[ZEL * idx + o] * RT[AXEL * idx + o] - IRT[XEL * idx + o] * RT[AZEL * idx + o];
                IRT[SZEL * idx + o] = RT[XEL * idx + o] * IRT[AYEL * idx + o] - uy * IRT[AXEL * idx + o] +
                                      IRT[XEL * idx + o] * RT[AYEL * idx + o] - Iuy * RT[AXEL * idx + o];
                IRT[TXEL * idx + o] = RT[AYEL * idx + o] * IRT[WZEL * idx + o] - RT[AZEL * idx + o] * IRT[WYEL * idx + o] +
                                      IRT[AYEL * idx + o] * RT[WZEL * idx + o] - IRT[AZEL * idx + o] * RT[WYEL * idx + o];
                IRT[TYEL * idx + o] = RT[AZEL * idx + o] * IRT[WXEL * idx + o] - RT[AXEL * idx + o] * IRT[WZEL * idx + o] +
                                      IRT[AZEL * idx + o] * RT[WXEL * idx + o] - IRT[AXEL * idx + o] * RT[WZEL * idx + o];
                IRT[TZEL * idx + o] = RT[AXEL * idx + o] * Iwy - RT[AYEL * idx + o] * IRT[WXEL * idx + o] +
                                      IRT[AXEL * idx + o] * wy - IRT[AYEL * idx + o] * RT[WXEL * idx + o];
                RT[SXEL * idx + o] = RT[YEL * idx + o] * RT[AZEL * idx + o] - RT[ZEL * idx + o] * RT[AYEL * idx + o];
                RT[SYEL * idx + o] = RT[ZEL * idx + o] * RT[AXEL * idx + o] - RT[XEL * idx + o] * RT[AZEL * idx + o];
                RT[SZEL * idx + o] = RT[XEL * idx + o] * RT[AYEL * idx + o] - uy * RT[AXEL * idx + o];
                RT[TXEL * idx + o] = RT[AYEL * idx + o] * RT[WZEL * idx + o] - RT[AZEL * idx + o] * RT[WYEL * idx + o];
                RT[TYEL * idx + o] = RT[AZEL * idx + o] * RT[WXEL * idx + o] - RT[AXEL * idx + o] * RT[WZEL * idx + o];
                RT[TZEL * idx + o] = RT[AXEL * idx + o] * wy - RT[AYEL * idx + o] * RT[WXEL * idx + o];
            }
        for (int i = 0; i < 6; ++i) {
            forward_field(s, s->CT, i);
            scale_field(s, s->CT, i, norm);
            forward_field(s, s->ICT, i);
            scale_field(s, s->ICT, i, norm);
        }
        /* assemble H = -T + (curl-like terms of S), keep S_x, S_z; pass2.c:474-566 */
        for (int half = 0; half < 2; ++half) {
            const int z0 = half ? Nz + 1 : 0, z1 = half ? pz : Nz / 2, zs = half ? Nz / 2 : 0;
            for (int z = z0; z < z1; ++z) {
                const int zu = z - zs;
                const double kz = s->Kz[zu];
                for (int src = 0; src < 2; ++src) {
                    cpx *Ud = src ? s->IU : s->U;
                    const cpx *T = src ? s->ICT : s->CT;
                    memcpy(&Ud[UI(s, zu, DXEL, y, 0)], &T[TI(s, SXEL, z, 0)], sizeof(cpx) * X);
                    memcpy(&Ud[UI(s, zu, DZEL, y, 0)], &T[TI(s, SZEL, z, 0)], sizeof(cpx) * X);
                    for (int x = 0; x < X; ++x) {
                        const double kx = s->Kx[x];
                        const cpx Tx = T[TI(s, TXEL, z, x)], Ty = T[TI(s, TYEL, z, x)], Tz = T[TI(s, TZEL, z, x)];
                        const cpx Sx = T[TI(s, SXEL, z, x)], Sy = T[TI(s, SYEL, z, x)], Sz = T[TI(s, SZEL, z, x)];
                        Ud[UI(s, zu, HXEL, y, x)].re = -Tx.re - kz * Sy.im;
                        Ud[UI(s, zu, HXEL, y, x)].im = -Tx.im + kz * Sy.re;
                        Ud[UI(s, zu, HYEL, y, x)].re = -Ty.re + kz * Sx.im - kx * Sz.im;
                        Ud[UI(s, zu, HYEL, y, x)].im = -Ty.im - kz * Sx.re + kx * Sz.re;
                        Ud[UI(s, zu, HZEL, y, x)].re = -Tz.re + kx * Sy.im;
                        Ud[UI(s, zu, HZEL, y, x)].im = -Tz.im - kx * Sy.re;
                    }
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Galerkin solves                                                     */
/* ------------------------------------------------------------------ */

static void fill_v_lhs(cport *s, int z, int x0, double coef, int sign_minus)
{
    /* M = -(K2 Qs + Qps) +/- re*coef*dt*(K2^2 Qs + 2 K2 Qps + Qpps), project.c:60-95 */
    const int X = s->X, D = s->dimQ;
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < T_QSDIAG; ++j)
            for (int x = x0; x < X; ++x) {
                const double k2 = s->K2[z * X + x], sq = k2 * k2;
                const double qs = s->Qs[i * 9 + j], qps = s->Qps[i * 9 + j], qpps = s->Qpps[i * 9 + j];
                if (sign_minus)
                    s->M[((size_t)i * 9 + j) * X + x] = -(k2 * qs + qps) - s->re * coef * s->dt * (sq * qs + 2. * k2 * qps + qpps);
                else
                    s->M[((size_t)i * 9 + j) * X + x] = -(k2 * qs + qps) + s->re * coef * s->dt * (sq * qs + 2. * k2 * qps + qpps);
            }
}

static void fill_g_lhs(cport *s, int z, int x0, double coef, int sign_plus)
{
    /* M = Rs -/+ re*coef*dt*(Rps + K2 Rs), project.c:143-174 */
    const int X = s->X, R = s->dimR;
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j)
            for (int x = x0; x < X; ++x) {
                const double k2 = s->K2[z * X + x];
                if (sign_plus)
                    s->M[((size_t)i * 9 + j) * X + x] = s->Rs[i * 5 + j] + s->re * coef * s->dt * (s->Rps[i * 5 + j] + k2 * s->Rs[i * 5 + j]);
                else
                    s->M[((size_t)i * 9 + j) * X + x] = s->Rs[i * 5 + j] - s->re * coef * s->dt * (s->Rps[i * 5 + j] + k2 * s->Rs[i * 5 + j]);
            }
}

/* RHS quadrature for v, project.c:97-115 (+ adjproject.c:113-134 terms when adj) */
static void rhs_fa(cport *s, const cpx *H, int z, int x0, int adj)
{
    const int X = s->X, D = s->dimQ, q = s->qpts;
    memset(s->Fa, 0, sizeof(cpx) * (size_t)s->dimR * X);
    const double kz = s->Kz[z];
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < q; ++j)
            for (int x = x0; x < X; ++x) {
                const double kx = s->Kx[x], k2 = s->K2[z * X + x];
                const cpx hx = H[UI(s, z, HXEL, j, x)], hy = H[UI(s, z, HYEL, j, x)], hz = H[UI(s, z, HZEL, j, x)];
                const double qpw = s->Qpw[i * q + j], qw = s->Qw[i * q + j];
                if (!adj) {
                    s->Fa[i * X + x].re += (qpw * (-kx * hx.im - kz * hz.im) - k2 * (qw * hy.re));
                    s->Fa[i * X + x].im += (qpw * (kx * hx.re + kz * hz.re) - k2 * (qw * hy.im));
                } else {
                    const cpx dx = H[UI(s, z, DXEL, j, x)], dz = H[UI(s, z, DZEL, j, x)];
                    const double qppw = s->Qppw[i * q + j];
                    s->Fa[i * X + x].re += (qpw * (-kx * hx.im - kz * hz.im) - k2 * (qw * hy.re)) +
                                           qppw * (kz * dx.im - kx * dz.im);
                    s->Fa[i * X + x].im += (qpw * (kx * hx.re + kz * hz.re) - k2 * (qw * hy.im)) +
                                           qppw * (-kz * dx.re + kx * dz.re);
                }
            }
}

/* RHS quadrature for g, project.c:177-191 (+ adjproject.c:218-234) */
static void rhs_fb(cport *s, const cpx *H, int z, int x0, int adj)
{
    const int X = s->X, R = s->dimR, q = s->qpts;
    memset(s->Fb, 0, sizeof(cpx) * (size_t)R * X);
    const double kz = s->Kz[z];
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < q; ++j)
            for (int x = x0; x < X; ++x) {
                const double kx = s->Kx[x];
                const cpx hx = H[UI(s, z, HXEL, j, x)], hz = H[UI(s, z, HZEL, j, x)];
                const double rw = s->Rw[i * q + j];
                if (!adj) {
                    s->Fb[i * X + x].re += rw * (-kz * hx.im + kx * hz.im);
                    s->Fb[i * X + x].im += rw * (kz * hx.re - kx * hz.re);
                } else {
                    const cpx dx = H[UI(s, z, DXEL, j, x)], dz = H[UI(s, z, DZEL, j, x)];
                    const double rpw = s->Rpw[i * q + j];
                    s->Fb[i * X + x].re += rw * (-kz * hx.im + kx * hz.im) + rpw * (-kz * dz.im - kx * dx.im);
                    s->Fb[i * X + x].im += rw * (kz * hx.re - kx * hz.re) + rpw * (kz * dz.re + kx * dx.re);
                }
            }
}

/* Re-sensitivity forcing of the tangent.
   kind 2, the reference's own forcing reconnected: at substage 0 only,
     IC += dt * Mass^-1 (F MC[3n+1]) with, per mode,
     F_alpha = -re^2 (K2^2 Qs + 2 K2 Qps + Qpps), Mass_alpha = -(K2 Qs + Qps)
     F_beta  =  re^2 (Rps + K2 Rs),               Mass_beta  = Rs
     (tangent_forcing.c:10-75 and increproject.c:61-104), and for the mean
     mode F = re^2 Rps, Mass = Rs (tangent_forcing0.c:10-44 with the block
     kept commented out in increproject0.c:45-90);
   kind 3, the exact derivative of the discrete step with respect to Re
     (re = 1/Re, dre/dRe = -re^2): every substage k adds
     -re^2 dt (a_k D x_k + b_k D x_{k+1}) to the right-hand side, D the
     viscous operator of the implicit solve and x the primal states MC[3n+k],
     MC[3n+k+1] (from (M - re b_k dt D) x_{k+1} = (M + re a_k dt D) x_k + ...).
   The mean flux is held fixed in both (homogeneous flux correction). */
static void fill_v_visc(cport *s, int z, int x0, double scale)
{
    /* M = scale * (K2^2 Qs + 2 K2 Qps + Qpps), rows < dimQ */
    const int X = s->X, D = s->dimQ;
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < T_QSDIAG; ++j)
            for (int x = x0; x < X; ++x) {
                const double k2 = s->K2[z * X + x], sq = k2 * k2;
                s->M[((size_t)i * 9 + j) * X + x] =
                    scale * (sq * s->Qs[i * 9 + j] + 2. * k2 * s->Qps[i * 9 + j] + s->Qpps[i * 9 + j]);
            }
}

static void fill_g_visc(cport *s, int z, int x0, double scale)
{
    /* M = scale * (Rps + K2 Rs), rows < dimR */
    const int X = s->X, R = s->dimR;
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j)
            for (int x = x0; x < X; ++x) {
                const double k2 = s->K2[z * X + x];
                s->M[((size_t)i * 9 + j) * X + x] = scale * (s->Rps[i * 5 + j] + k2 * s->Rs[i * 5 + j]);
            }
}

/* kind 2 on one line: C += dt Mass^-1 F x (x = MC[3n+1]) */
static void re_force_line_ref(cport *s, int z, int x0, cpx *C, const cpx *x)
{
    const int X = s->X, D = s->dimQ, R = s->dimR;
    const double re2 = s->re * s->re;
    cpx *Ca = &C[CI(s, z, ALPHA, 0, 0)], *Cb = &C[CI(s, z, BETA, 0, 0)];
    memset(s->Fa, 0, sizeof(cpx) * (size_t)D * X);
    memset(s->Fb, 0, sizeof(cpx) * (size_t)R * X);
    fill_v_visc(s, z, x0, -re2);
    smmult(s->M, &x[CI(s, z, ALPHA, 0, 0)], s->Fa, QSDIAG - 1, QSDIAG - 1, D, X, x0);
    fill_g_visc(s, z, x0, re2);
    smmult(s->M, &x[CI(s, z, BETA, 0, 0)], s->Fb, RSDIAG - 1, RSDIAG - 1, R, X, x0);
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < T_QSDIAG; ++j)
            for (int xx = x0; xx < X; ++xx)
                s->M[((size_t)i * 9 + j) * X + xx] = -(s->K2[z * X + xx] * s->Qs[i * 9 + j] + s->Qps[i * 9 + j]);
    bsolve(s->M, s->Fa, QSDIAG - 1, QSDIAG - 1, D, X, x0);
    memset(s->M, 0, sizeof(double) * (size_t)s->dimR * 9 * X);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j)
            for (int xx = x0; xx < X; ++xx) s->M[((size_t)i * 9 + j) * X + xx] = s->Rs[i * 5 + j];
    bsolve(s->M, s->Fb, RSDIAG - 1, RSDIAG - 1, R, X, x0);
    for (int xx = x0; xx < X; ++xx) {
        for (int i = 0; i < D; ++i) {
            Ca[i * X + xx].re += s->dt * s->Fa[i * X + xx].re;
            Ca[i * X + xx].im += s->dt * s->Fa[i * X + xx].im;
        }
        for (int i = 0; i < R; ++i) {
            Cb[i * X + xx].re += s->dt * s->Fb[i * X + xx].re;
            Cb[i * X + xx].im += s->dt * s->Fb[i * X + xx].im;
        }
    }
}

/* kind 3 on one line, alpha (v = ALPHA) or beta: rhs -= re^2 dt (a D xk + b D xk1) */
static void re_force_line_exact(cport *s, int z, int x0, int v, cpx *rhs, const cpx *xk, const cpx *xk1,
                                double ak, double bk)
{
    const int X = s->X, N = v == ALPHA ? s->dimQ : s->dimR;
    const int band = v == ALPHA ? QSDIAG - 1 : RSDIAG - 1;
    const double re2 = s->re * s->re;
    /* alpha: D = K2^2 Qs + 2 K2 Qps + Qpps; beta: D = -(Rps + K2 Rs) */
    if (v == ALPHA) fill_v_visc(s, z, x0, 1.0);
    else fill_g_visc(s, z, x0, -1.0);
    smmult(s->M, &xk[CI(s, z, v, 0, 0)], s->TM, band, band, N, X, x0);
    for (int i = 0; i < N; ++i)
        for (int xx = x0; xx < X; ++xx) {
            rhs[i * X + xx].re -= re2 * s->dt * ak * s->TM[i * X + xx].re;
            rhs[i * X + xx].im -= re2 * s->dt * ak * s->TM[i * X + xx].im;
        }
    smmult(s->M, &xk1[CI(s, z, v, 0, 0)], s->TM, band, band, N, X, x0);
    for (int i = 0; i < N; ++i)
        for (int xx = x0; xx < X; ++xx) {
            rhs[i * X + xx].re -= re2 * s->dt * bk * s->TM[i * X + xx].re;
            rhs[i * X + xx].im -= re2 * s->dt * bk * s->TM[i * X + xx].im;
        }
}

/* One (kz) line of the implicit step for non-(0,0) modes.
   project.c:24-405 (forward, adj == 0) and adjproject.c:10-550 (adj == 1).
   C is the carried coefficient array, H the array holding the nonlinear
   terms (pass1/pass2 output), U the velocity array rebuilt from the solved
   coefficients (the same array as H for primal and tangent, AU for the
   adjoint), store the trajectory slot (NULL: none), LUa the previous-stage
   terms for the adjoint's next-stage right-hand side. */
static void project_line(cport *s, int k, int z, int x0, cpx *C, const cpx *H, cpx *U,
                         cpx *store, const cpx *LUa, int adj, int fkind, const cpx *xk)
{
    const int X = s->X, D = s->dimQ, R = s->dimR;
    const double *a = adj ? aa_ : fa_, *b = adj ? ab_ : fb_, *c = adj ? ac_ : fc_, *d = adj ? ad_ : fd_;
    cpx *Ca = &C[CI(s, z, ALPHA, 0, 0)], *Cb = &C[CI(s, z, BETA, 0, 0)];
    if (fkind == 2 && k == 0) re_force_line_ref(s, z, x0, C, xk + s->csz);  /* MC[3n+1] */
    if (k == 0) {
        fill_v_lhs(s, z, x0, a[0], 0);
        smmult(s->M, Ca, s->TM, QSDIAG - 1, QSDIAG - 1, D, X, x0);
        for (int i = 0; i < D; ++i) memcpy(&Ca[i * X + x0], &s->TM[i * X + x0], sizeof(cpx) * (X - x0));
    }
    fill_v_lhs(s, z, x0, b[k], 1);
    rhs_fa(s, H, z, x0, adj);
    for (int i = 0; i < D; ++i)
        for (int x = x0; x < X; ++x) {
            Ca[i * X + x].re += s->dt * c[k] * s->Fa[i * X + x].re;
            Ca[i * X + x].im += s->dt * c[k] * s->Fa[i * X + x].im;
        }
    if (fkind == 3) {
        re_force_line_exact(s, z, x0, ALPHA, Ca, xk, xk + s->csz, a[k], b[k]);
        fill_v_lhs(s, z, x0, b[k], 1);
    }
    bsolve(s->M, Ca, QSDIAG - 1, QSDIAG - 1, D, X, x0);
    if (k == 0) {
        fill_g_lhs(s, z, x0, a[0], 0);
        smmult(s->M, Cb, s->TM, RSDIAG - 1, RSDIAG - 1, R, X, x0);
        for (int i = 0; i < R; ++i) memcpy(&Cb[i * X + x0], &s->TM[i * X + x0], sizeof(cpx) * (X - x0));
    }
    fill_g_lhs(s, z, x0, b[k], 1);
    rhs_fb(s, H, z, x0, adj);
    for (int i = 0; i < R; ++i)
        for (int x = x0; x < X; ++x) {
            Cb[i * X + x].re += s->dt * c[k] * s->Fb[i * X + x].re;
            Cb[i * X + x].im += s->dt * c[k] * s->Fb[i * X + x].im;
        }
    if (fkind == 3) {
        re_force_line_exact(s, z, x0, BETA, Cb, xk, xk + s->csz, a[k], b[k]);
        fill_g_lhs(s, z, x0, b[k], 1);
    }
    bsolve(s->M, Cb, RSDIAG - 1, RSDIAG - 1, R, X, x0);
    if (store) {
        for (int v = 0; v < 2; ++v)
            for (int i = 0; i < R; ++i)
                for (int x = x0; x < X; ++x) store[CI(s, z, v, i, x)] = C[CI(s, z, v, i, x)];
    }
    recon_line(s, C, U, z, x0);
    if (k != 2) {
        fill_v_lhs(s, z, x0, a[k + 1], 0);
        smmult(s->M, Ca, s->TM, QSDIAG - 1, QSDIAG - 1, D, X, x0);
        if (adj) rhs_fa(s, LUa, z, x0, 1);
        for (int i = 0; i < D; ++i)
            for (int x = x0; x < X; ++x) {
                Ca[i * X + x].re = s->TM[i * X + x].re + s->dt * d[k + 1] * s->Fa[i * X + x].re;
                Ca[i * X + x].im = s->TM[i * X + x].im + s->dt * d[k + 1] * s->Fa[i * X + x].im;
            }
        fill_g_lhs(s, z, x0, a[k + 1], 0);
        smmult(s->M, Cb, s->TM, RSDIAG - 1, RSDIAG - 1, R, X, x0);
        if (adj) rhs_fb(s, LUa, z, x0, 1);
        for (int i = 0; i < R; ++i)
            for (int x = x0; x < X; ++x) {
                Cb[i * X + x].re = s->TM[i * X + x].re + s->dt * d[k + 1] * s->Fb[i * X + x].re;
                Cb[i * X + x].im = s->TM[i * X + x].im + s->dt * d[k + 1] * s->Fb[i * X + x].im;
            }
    }
}

/* (kx,kz) = (0,0) mean-flow step.
   mode 0: primal, project0.c:22-271 (flux_t = flux - sum)
   mode 1: tangent with mean-flux forcing, increproject0.c:209-214 (2.0 - sum)
   mode 2: homogeneous tangent (-sum)
   mode 3: adjoint, adjproject0.c:8-310 */
static void project_mean(cport *s, int k, cpx *C, const cpx *H, cpx *U, cpx *store, const cpx *LUa, int mode,
                         int fkind, const cpx *xk)
{
    const int R = s->dimR, q = s->qpts, X = s->X;
    const int adj = mode == 3;
    const double *a = adj ? aa_ : fa_, *b = adj ? ab_ : fb_, *c = adj ? ac_ : fc_, *d = adj ? ad_ : fd_;
    double *MZ = s->MZ;
    cpx *Ca = &C[CI(s, 0, ALPHA, 0, 0)], *Cb = &C[CI(s, 0, BETA, 0, 0)];
    const double re2 = s->re * s->re;
    if (fkind == 2 && k == 0) {
        /* tangent_forcing0.c:31-41 on MC[3n+1], then Rs^-1 and IC += dt f */
        const cpx *x1 = xk + s->csz;
        for (int v = 0; v < 2; ++v) {
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = re2 * s->Rps[i * 5 + j];
            smmult_single(MZ, 5, &x1[CI(s, 0, v, 0, 0)], X, s->fa, RSDIAG - 1, RSDIAG - 1, R);
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j];
            bsolve_single(MZ, 5, s->fa, 1, RSDIAG - 1, RSDIAG - 1, R);
            cpx *Cv = v == ALPHA ? Ca : Cb;
            for (int i = 0; i < R; ++i) {
                Cv[i * X].re += s->dt * s->fa[i].re;
                Cv[i * X].im += s->dt * s->fa[i].im;
            }
        }
    }
    if (k == 0) {
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] - s->re * a[0] * s->dt * s->Rps[i * 5 + j];
        smmult_single(MZ, 5, Ca, X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) Ca[i * X] = s->tm[i];
        smmult_single(MZ, 5, Cb, X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) Cb[i * X] = s->tm[i];
    }
    /* the flux-correction vector: project0.c:84-98 uses Rs, adjproject0.c:81-95 uses Rs + re b dt Rps */
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j)
            MZ[i * 5 + j] = adj ? s->Rs[i * 5 + j] + s->re * b[k] * s->dt * s->Rps[i * 5 + j] : s->Rs[i * 5 + j];
    memset(s->add, 0, sizeof(cpx) * (size_t)R);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < q; ++j) s->add[i].re += s->Rw[i * q + j];
    bsolve_single(MZ, 5, s->add, 1, RSDIAG - 1, RSDIAG - 1, R);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] + s->re * b[k] * s->dt * s->Rps[i * 5 + j];
    memset(s->fa, 0, sizeof(cpx) * (size_t)R);
    for (int i = 0; i < R; ++i) {
        for (int j = 0; j < q; ++j) {
            if (!adj) s->fa[i].re += s->Rw[i * q + j] * (H[UI(s, 0, HXEL, j, 0)].re);
            else s->fa[i].re += s->Rw[i * q + j] * (H[UI(s, 0, HXEL, j, 0)].re) + s->Rpw[i * q + j] * H[UI(s, 0, DZEL, j, 0)].re;
        }
        Ca[i * X].re += s->dt * c[k] * s->fa[i].re;
    }
    if (fkind == 3) {
        /* D0 = -Rps: rhs += re^2 dt (a Rps xk + b Rps xk1) */
        smmult_single(s->Rps, 5, &xk[CI(s, 0, ALPHA, 0, 0)], X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) {
            Ca[i * X].re += re2 * s->dt * a[k] * s->tm[i].re;
            Ca[i * X].im += re2 * s->dt * a[k] * s->tm[i].im;
        }
        /* the implicit term acts on the primal's solved mean flow, before
           its flux correction: MC[3n+k+1] - 0.5 flux_t add */
        const cpx *x1 = &xk[s->csz + CI(s, 0, ALPHA, 0, 0)];
        const double ft = s->MFT[(x1 - CI(s, 0, ALPHA, 0, 0) - s->MC) / s->csz];
        for (int i = 0; i < R; ++i) {
            s->fb[i].re = x1[i * X].re - ft * s->add[i].re * 0.5;
            s->fb[i].im = x1[i * X].im - ft * s->add[i].im * 0.5;
        }
        smmult_single(s->Rps, 5, s->fb, 1, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) {
            Ca[i * X].re += re2 * s->dt * b[k] * s->tm[i].re;
            Ca[i * X].im += re2 * s->dt * b[k] * s->tm[i].im;
        }
    }
    bsolve_single(MZ, 5, Ca, X, RSDIAG - 1, RSDIAG - 1, R);
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] + s->re * b[k] * s->dt * s->Rps[i * 5 + j];
    memset(s->fb, 0, sizeof(cpx) * (size_t)R);
    for (int i = 0; i < R; ++i) {
        for (int j = 0; j < q; ++j) {
            if (!adj) s->fb[i].re += s->Rw[i * q + j] * H[UI(s, 0, HZEL, j, 0)].re;
            else s->fb[i].re += s->Rw[i * q + j] * H[UI(s, 0, HZEL, j, 0)].re - s->Rpw[i * q + j] * H[UI(s, 0, DXEL, j, 0)].re;
        }
        Cb[i * X].re += s->dt * c[k] * s->fb[i].re;
    }
    if (fkind == 3) {
        smmult_single(s->Rps, 5, &xk[CI(s, 0, BETA, 0, 0)], X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) {
            Cb[i * X].re += re2 * s->dt * a[k] * s->tm[i].re;
            Cb[i * X].im += re2 * s->dt * a[k] * s->tm[i].im;
        }
        smmult_single(s->Rps, 5, &xk[s->csz + CI(s, 0, BETA, 0, 0)], X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        for (int i = 0; i < R; ++i) {
            Cb[i * X].re += re2 * s->dt * b[k] * s->tm[i].re;
            Cb[i * X].im += re2 * s->dt * b[k] * s->tm[i].im;
        }
    }
    bsolve_single(MZ, 5, Cb, X, RSDIAG - 1, RSDIAG - 1, R);
    double flux_t = 0;
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < q; ++j) flux_t += s->Rw[i * q + j] * Ca[i * X].re;
    if (mode == 0) {
        flux_t = s->flux - flux_t;
        if (store && store >= s->MC && store < s->MC + (3 * (size_t)s->nsteps + 1) * s->csz)
            s->MFT[(store - s->MC) / s->csz] = flux_t;
    }
    else if (mode == 1) flux_t = 2.0 - flux_t;
    else flux_t = -flux_t;
    for (int j = 0; j < R; ++j) {
        Ca[j * X].re = Ca[j * X].re + flux_t * s->add[j].re * 0.5;
        Ca[j * X].im = Ca[j * X].im + flux_t * s->add[j].im * 0.5;
    }
    recon_mean(s, C, U);
    if (store) {
        for (int i = 0; i < R; ++i) {
            store[CI(s, 0, ALPHA, i, 0)] = Ca[i * X];
            store[CI(s, 0, BETA, i, 0)] = Cb[i * X];
        }
    }
    if (k != 2) {
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] - s->re * a[k + 1] * s->dt * s->Rps[i * 5 + j];
        smmult_single(MZ, 5, Ca, X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        if (adj) {
            memset(s->fa, 0, sizeof(cpx) * (size_t)R);
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < q; ++j)
                    s->fa[i].re += s->Rw[i * q + j] * (LUa[UI(s, 0, HXEL, j, 0)].re) + s->Rpw[i * q + j] * LUa[UI(s, 0, DZEL, j, 0)].re;
        }
        for (int i = 0; i < R; ++i) {
            Ca[i * X].re = s->tm[i].re + s->dt * d[k + 1] * s->fa[i].re;
            Ca[i * X].im = s->tm[i].im + s->dt * d[k + 1] * s->fa[i].im;
        }
        smmult_single(MZ, 5, Cb, X, s->tm, RSDIAG - 1, RSDIAG - 1, R);
        if (adj) {
            memset(s->fb, 0, sizeof(cpx) * (size_t)R);
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < q; ++j)
                    s->fb[i].re += s->Rw[i * q + j] * LUa[UI(s, 0, HZEL, j, 0)].re - s->Rpw[i * q + j] * LUa[UI(s, 0, DXEL, j, 0)].re;
        }
        for (int i = 0; i < R; ++i) {
            Cb[i * X].re = s->tm[i].re + s->dt * d[k + 1] * s->fb[i].re;
            Cb[i * X].im = s->tm[i].im + s->dt * d[k + 1] * s->fb[i].im;
        }
    }
}

/* one substage of the implicit solve over all modes of one field:
   channel.c:456-470 (primal), 546-573 (tangent), 668-679 (adjoint) */
/* fkind 2 / 3: Re forcing from the primal states xk = MC[3n+k], xk + csz = MC[3n+k+1] */
static void solve_all_forced(cport *s, int k, cpx *C, const cpx *H, cpx *U, cpx *store, const cpx *LUa,
                             int mean_mode, int fkind, const cpx *xk)
{
    const int adj = mean_mode == 3;
    project_mean(s, k, C, H, U, store, LUa, mean_mode, fkind, xk);
    project_line(s, k, 0, 1, C, H, U, store, LUa, adj, fkind, xk);
    for (int z = 1; z < s->Nz; ++z) {
        if (z == s->Nz / 2) {
            memset(&U[UI(s, z, 0, 0, 0)], 0, sizeof(cpx) * 5 * (size_t)s->qpts * s->X);
            memset(&C[CI(s, z, 0, 0, 0)], 0, sizeof(cpx) * 2 * (size_t)s->dimR * s->X);
            continue;
        }
        project_line(s, k, z, 0, C, H, U, store, LUa, adj, fkind, xk);
    }
}

static void solve_all(cport *s, int k, cpx *C, const cpx *H, cpx *U, cpx *store, const cpx *LUa, int mean_mode)
{
    solve_all_forced(s, k, C, H, U, store, LUa, mean_mode, 0, NULL);
}

/* ------------------------------------------------------------------ */
/* laminar start, initAlphaBeta.c:24-205                               */
/* ------------------------------------------------------------------ */
static void init_alpha_beta(cport *s)
{
    const int R = s->dimR, D = s->dimQ, q = s->qpts, X = s->X;
    /* Alpha0 / Beta0 */
    for (int v = 0; v < 2; ++v) {
        const int comp = v == 0 ? XEL : ZEL;
        for (int i = 0; i < R; ++i) {
            cpx *cc = &s->C[CI(s, 0, v, i, 0)];
            cc->re = 0.0; cc->im = 0.0;
            for (int j = 0; j < q; ++j) {
                cc->re += s->Rw[i * q + j] * s->U[UI(s, 0, comp, j, 0)].re;
                cc->im += s->Rw[i * q + j] * s->U[UI(s, 0, comp, j, 0)].im;
            }
        }
        memcpy(s->MZ, s->Rs, sizeof(double) * (size_t)R * 5);
        bsolve_single(s->MZ, 5, &s->C[CI(s, 0, v, 0, 0)], X, RSDIAG - 1, RSDIAG - 1, R);
    }
    double *Mloc = (double *)malloc(sizeof(double) * (size_t)D * 9);
    for (int z = 0; z < s->Nz; ++z) {
        const int x0 = z == 0 ? 1 : 0;
        /* Alpha */
        cpx *Ca = &s->C[CI(s, z, ALPHA, 0, 0)];
        for (int i = 0; i < D; ++i) for (int x = x0; x < X; ++x) { Ca[i * X + x].re = 0.0; Ca[i * X + x].im = 0.0; }
        for (int i = 0; i < D; ++i) for (int j = 0; j < q; ++j) for (int x = x0; x < X; ++x) {
            Ca[i * X + x].re += s->Qw[i * q + j] * s->U[UI(s, z, YEL, j, x)].re;
            Ca[i * X + x].im += s->Qw[i * q + j] * s->U[UI(s, z, YEL, j, x)].im;
        }
        memcpy(Mloc, s->Qs, sizeof(double) * (size_t)D * 9);
        bsolve_shared(Mloc, 9, Ca, QSDIAG - 1, QSDIAG - 1, D, X, x0);
        /* Beta */
        cpx *Cb = &s->C[CI(s, z, BETA, 0, 0)];
        for (int i = 0; i < R; ++i) for (int x = x0; x < X; ++x) { Cb[i * X + x].re = 0.0; Cb[i * X + x].im = 0.0; }
        const double kz = s->Kz[z];
        for (int i = 0; i < R; ++i) for (int j = 0; j < q; ++j) for (int x = x0; x < X; ++x) {
            const double kx = s->Kx[x];
            Cb[i * X + x].re += s->Rw[i * q + j] * (kx * s->U[UI(s, z, ZEL, j, x)].im - kz * s->U[UI(s, z, XEL, j, x)].im);
            Cb[i * X + x].im += s->Rw[i * q + j] * (kz * s->U[UI(s, z, XEL, j, x)].re - kx * s->U[UI(s, z, ZEL, j, x)].re);
        }
        memcpy(s->MZ, s->Rs, sizeof(double) * (size_t)R * 5);
        bsolve_shared(s->MZ, 5, Cb, RSDIAG - 1, RSDIAG - 1, R, X, x0);
    }
    free(Mloc);
}

/* ------------------------------------------------------------------ */
/* entry points, channel.c                                             */
/* ------------------------------------------------------------------ */

cport *cport_init(int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
                  double flux, double dt, int nsteps)
{
    if (Nx % 4 != 0 || Nz % 2 != 0 || Ny - 4 < 0 || nsteps < 0) return NULL;
    cport *s = (cport *)calloc(1, sizeof(cport));
    if (!s) return NULL;
    s->Nx = Nx; s->Ny = Ny; s->Nz = Nz; s->X = Nx / 2;
    s->dt = dt; s->nsteps = nsteps; s->flux = flux;
    s->re = 1. / Re;                       /* channel.c:290 */
    s->qpts = 3 * Ny / 2;
    s->dimR = Ny - 2;
    s->dimQ = Ny - 4;
    s->pz = 3 * Nz / 2;
    s->px = 3 * Nx / 2;
    s->hx = 3 * Nx / 4 + 1;
    const int q = s->qpts, R = s->dimR, D = s->dimQ, X = s->X;
    s->csz = (size_t)Nz * 2 * R * X;
    s->usz = (size_t)Nz * 5 * q * X;
#define DALLOC(p, n) (p = (double *)calloc((size_t)(n), sizeof(double)))
#define CALLOC(p, n) (p = (cpx *)calloc((size_t)(n), sizeof(cpx)))
    DALLOC(s->Kx, X); DALLOC(s->Kz, Nz); DALLOC(s->K2, Nz * X); DALLOC(s->cfl2, q);
    DALLOC(s->Qy, q); DALLOC(s->W, q);
    DALLOC(s->Q, q * D); DALLOC(s->Qp, q * D); DALLOC(s->Qpp, q * D);
    DALLOC(s->R, q * R); DALLOC(s->Rp, q * R);
    DALLOC(s->Qw, D * q); DALLOC(s->Qpw, D * q); DALLOC(s->Qppw, D * q);
    DALLOC(s->Rw, R * q); DALLOC(s->Rpw, R * q);
    DALLOC(s->Qs, D * 9); DALLOC(s->Qps, D * 9); DALLOC(s->Qpps, D * 9);
    DALLOC(s->Rs, R * 5); DALLOC(s->Rps, R * 5);
    CALLOC(s->C, s->csz); CALLOC(s->IC, s->csz); CALLOC(s->AC, s->csz);
    CALLOC(s->U, s->usz); CALLOC(s->IU, s->usz); CALLOC(s->AU, s->usz);
    CALLOC(s->IAU, s->usz); CALLOC(s->LU, s->usz);
    CALLOC(s->MC, s->csz * (3 * (size_t)nsteps + 1));
    DALLOC(s->MFT, 3 * (size_t)nsteps + 1);
    CALLOC(s->MIC, s->csz * (3 * (size_t)nsteps + 1));
    CALLOC(s->CT, (size_t)MAXTT * s->pz * s->hx);
    CALLOC(s->ICT, (size_t)MAXTT * s->pz * s->hx);
    DALLOC(s->M, (size_t)R * 9 * X); DALLOC(s->MZ, R * 5);
    CALLOC(s->Fa, R * X); CALLOC(s->Fb, R * X); CALLOC(s->TM, R * X);
    CALLOC(s->fa, R); CALLOC(s->fb, R); CALLOC(s->tm, R); CALLOC(s->add, R);
    CALLOC(s->ddt_dCdt, s->csz);
    DALLOC(s->ddt_dudt, 3 * (size_t)s->px * q * s->pz);
    DALLOC(s->ddt_v, 3 * (size_t)s->px * q * s->pz);
#undef DALLOC
#undef CALLOC
    if (!s->MC || !s->MIC || !s->ddt_v || !s->CT) { cport_destroy(s); return NULL; }
    if (legendre_setup(s) != 0) { cport_destroy(s); return NULL; }
    wave_nums(s, Lx, Lz);
    s->pf1 = offt_plan_create(s->pz, +1);
    s->pf2 = offt_plan_create(s->pz, -1);
    s->pr1 = offt_rplan_create(s->px, +1);
    s->pr2 = offt_rplan_create(s->px, -1);
    if (cfl_vars(s, Lx, Lz) != 0) { cport_destroy(s); return NULL; }
    return s;
}

void cport_destroy(cport *s)
{
    if (!s) return;
    double *d[] = { s->Kx, s->Kz, s->K2, s->cfl2, s->Qy, s->W, s->Q, s->Qp, s->Qpp, s->R, s->Rp,
                    s->Qw, s->Qpw, s->Qppw, s->Rw, s->Rpw, s->Qs, s->Qps, s->Qpps, s->Rs, s->Rps,
                    s->M, s->MZ, s->ddt_dudt, s->ddt_v, s->MFT };
    for (size_t i = 0; i < sizeof(d) / sizeof(d[0]); ++i) free(d[i]);
    cpx *c[] = { s->C, s->IC, s->AC, s->U, s->IU, s->AU, s->IAU, s->LU, s->MC, s->MIC, s->CT, s->ICT,
                 s->Fa, s->Fb, s->TM, s->fa, s->fb, s->tm, s->add, s->ddt_dCdt };
    for (size_t i = 0; i < sizeof(c) / sizeof(c[0]); ++i) free(c[i]);
    offt_plan_destroy(s->pf1);
    offt_plan_destroy(s->pf2);
    offt_rplan_destroy(s->pr1);
    offt_rplan_destroy(s->pr2);
    free(s);
}

/* channel.c:399-478 */
int cport_primal(cport *s, int ru_steps, double *C_given)
{
    int status = 0;
    if (C_given) {
        memmove(s->C, C_given, sizeof(cpx) * s->csz);
        recon(s, s->C, s->U);
    } else {
        memset(s->U, 0, sizeof(cpx) * s->usz);
        for (int i = 0; i < s->qpts; ++i) {
            s->U[UI(s, 0, XEL, i, 0)].re = (1.0 - s->Qy[i] * s->Qy[i]) * s->flux * 3. / 4;
            s->U[UI(s, 0, XEL, i, 0)].im = 0.0;
        }
        for (int i = 0; i < s->qpts; ++i) {
            s->U[UI(s, 1, XEL, i, 1)].re = (rand() / (double)RAND_MAX - 0.5);
            s->U[UI(s, 1, XEL, i, 1)].im = (rand() / (double)RAND_MAX - 0.5);
        }
        init_alpha_beta(s);
    }
    memset(s->MC, 0, sizeof(cpx) * s->csz * (3 * (size_t)s->nsteps + 1));
    memmove(s->MC, s->C, sizeof(cpx) * s->csz);
    for (int n = 0; n < s->nsteps + ru_steps; ++n) {
        for (int dctr = 0; dctr < 3; ++dctr) {
            if (pass1(s, dctr) != 0) {
                printf("Pass1 failure\n");
                status = -1;
                n = s->nsteps + ru_steps;
                break;
            }
            int count = (n - ru_steps) * 3 + dctr + 1;
            cpx *store = count >= 0 ? s->MC + (size_t)count * s->csz : NULL;
            solve_all(s, dctr, s->C, s->U, s->U, store, NULL, 0);
        }
    }
    if (C_given) memmove(C_given, s->C, sizeof(cpx) * s->csz);
    return status;
}

/* channel.c:486-587 */
int cport_tangent(cport *s, int start_step, int end_step, double *IC_given, int inhomo)
{
    return cport_tangent_forcing(s, start_step, end_step, IC_given, inhomo ? 1 : 0);
}

/* forcing 0: none, 1: mean flux (the reference's inhomo != 0), 2: Re, the
   reference's disconnected forcing reconnected, 3: Re, exact discrete
   derivative (see re_force_line_ref / re_force_line_exact) */
int cport_tangent_forcing(cport *s, int start_step, int end_step, double *IC_given, int forcing)
{
    int status = 0;
    if (!(end_step > start_step && start_step >= 0 && end_step <= s->nsteps && IC_given)) return -2;
    memmove(s->C, s->MC + (size_t)start_step * 3 * s->csz, sizeof(cpx) * s->csz);
    memmove(s->IC, IC_given, sizeof(cpx) * s->csz);
    recon(s, s->C, s->U);
    recon(s, s->IC, s->IU);
    memmove(s->MIC + (size_t)start_step * 3 * s->csz, s->IC, sizeof(cpx) * s->csz);
    for (int n = start_step; n < end_step; ++n) {
        for (int dctr = 0; dctr < 3; ++dctr) {
            if (pass1(s, dctr) != 0) {
                printf("Pass1 failure\n");
                status = -1;
                n = s->nsteps;
                break;
            }
            int count = n * 3 + dctr + 1;
            solve_all_forced(s, dctr, s->IC, s->IU, s->IU, s->MIC + (size_t)count * s->csz, NULL,
                             forcing == 1 ? 1 : 2, forcing >= 2 ? forcing : 0, s->MC + (size_t)(count - 1) * s->csz);
            solve_all(s, dctr, s->C, s->U, s->U, NULL, NULL, 0);
        }
    }
    memmove(IC_given, s->IC, sizeof(cpx) * s->csz);
    return status;
}

/* channel.c:704-780 */
double cport_ddt_project(cport *s, int i_step, double *IC_given)
{
    cpx *IC = (cpx *)IC_given;
    cpx *dCdt = s->ddt_dCdt;
    const size_t plane = (size_t)s->px * s->qpts * s->pz;
    double *dudt = s->ddt_dudt, *v = s->ddt_v;
    int i_plus, i_minus;
    if (i_step == 0) { i_plus = 3 * (i_step + 1); i_minus = 3 * i_step; }
    else { i_plus = 3 * i_step; i_minus = 3 * (i_step - 1); }
    const cpx *Mp = s->MC + (size_t)i_plus * s->csz, *Mm = s->MC + (size_t)i_minus * s->csz;
    for (size_t z = 0; z < s->csz; ++z) {
        dCdt[z].re = (1.0 / s->dt) * (Mp[z].re - Mm[z].re);
        dCdt[z].im = (1.0 / s->dt) * (Mp[z].im - Mm[z].im);
    }
    memset(dudt, 0, sizeof(double) * 3 * plane);
    memset(v, 0, sizeof(double) * 3 * plane);
    cport_spec2phys(s, (double *)dCdt, dudt);
    cport_spec2phys(s, IC_given, v);
    double num = 0.0, den = 0.0;
    const size_t XF = 0, YF = plane, ZF = 2 * plane;
    for (int y = 0; y < s->qpts; ++y)
        for (int z = 0; z < s->pz; ++z)
            for (int x = 0; x < s->px; ++x) {
                size_t i = ((size_t)x * s->qpts + y) * s->pz + z;
                num += dudt[i + XF] * v[i + XF] * s->W[y];
                den += dudt[i + XF] * dudt[i + XF] * s->W[y];
                num += dudt[i + YF] * v[i + YF] * s->W[y];
                den += dudt[i + YF] * dudt[i + YF] * s->W[y];
                num += dudt[i + ZF] * v[i + ZF] * s->W[y];
                den += dudt[i + ZF] * dudt[i + ZF] * s->W[y];
            }
    for (size_t z = 0; z < s->csz; ++z) {
        IC[z].re -= (num / den) * dCdt[z].re;
        IC[z].im -= (num / den) * dCdt[z].im;
    }
    return num / den;
}

/* channel.c:596-696 */
int cport_adjoint(cport *s, int start_step, int end_step, double *AC_given, int inhomo, double strength)
{
    (void)inhomo;
    if (!(end_step < start_step && end_step >= 0 && start_step <= s->nsteps && AC_given)) return -2;
    cpx *ICtmp = (cpx *)malloc(sizeof(cpx) * s->csz);
    memmove(s->C, s->MC + (size_t)start_step * 3 * s->csz, sizeof(cpx) * s->csz);
    memmove(s->AC, AC_given, sizeof(cpx) * s->csz);
    recon(s, s->AC, s->AU);
    strength *= s->dt;
    for (int n = start_step; n > end_step; --n) {
        int count = n * 3;
        memmove(ICtmp, s->MIC + (size_t)count * s->csz, sizeof(cpx) * s->csz);
        cport_ddt_project(s, n, (double *)ICtmp);
        for (size_t z = 0; z < s->csz; ++z) {
            s->AC[z].re -= 0.5 * strength * ICtmp[z].re;
            s->AC[z].im -= 0.5 * strength * ICtmp[z].im;
        }
        for (int dctr = 0; dctr < 3; ++dctr) {
            count = n * 3 - dctr - 1;
            if (dctr < 2) {
                memmove(s->C, s->MC + (size_t)(count - 1) * s->csz, sizeof(cpx) * s->csz);
                recon(s, s->C, s->U);
                pass2(s);
                memmove(s->LU, s->U, sizeof(cpx) * s->usz);
            }
            memmove(s->C, s->MC + (size_t)count * s->csz, sizeof(cpx) * s->csz);
            recon(s, s->C, s->U);
            pass2(s);
            solve_all(s, dctr, s->AC, s->U, s->AU, NULL, s->LU, 3);
        }
        count = (n - 1) * 3;
        memmove(ICtmp, s->MIC + (size_t)count * s->csz, sizeof(cpx) * s->csz);
        cport_ddt_project(s, n - 1, (double *)ICtmp);
        for (size_t z = 0; z < s->csz; ++z) {
            s->AC[z].re -= 0.5 * strength * ICtmp[z].re;
            s->AC[z].im -= 0.5 * strength * ICtmp[z].im;
        }
    }
    memmove(AC_given, s->AC, sizeof(cpx) * s->csz);
    free(ICtmp);
    return 0;
}

/* spec2phys.c:10-90 */
void cport_spec2phys(cport *s, const double *C_ptr, double *flow)
{
    const int pz = s->pz, px = s->px, rp = px + 2, q = s->qpts, X = s->X, Nz = s->Nz;
    const size_t idx = (size_t)pz * rp;
    const size_t plane = (size_t)px * q * pz;
    memcpy(s->C, C_ptr, sizeof(cpx) * s->csz);
    recon(s, s->C, s->U);
    double *RT = (double *)s->CT;
    for (int y = 0; y < q; ++y) {
        memset(s->CT, 0, sizeof(cpx) * (size_t)MAXTT * pz * s->hx);
        for (int i = 0; i < 3; ++i) {
            for (int z = 0; z < Nz / 2; ++z) {
                memcpy(&s->CT[TI(s, i, z, 0)], &s->U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
                memcpy(&s->CT[TI(s, i + 3, z, 0)], &s->IU[UI(s, z, i, y, 0)], sizeof(cpx) * X);
            }
            for (int z = Nz / 2 + 1; z < Nz; ++z) {
                memcpy(&s->CT[TI(s, i, z + Nz / 2, 0)], &s->U[UI(s, z, i, y, 0)], sizeof(cpx) * X);
                memcpy(&s->CT[TI(s, i + 3, z + Nz / 2, 0)], &s->IU[UI(s, z, i, y, 0)], sizeof(cpx) * X);
            }
        }
        for (int i = 0; i < 3; ++i) inverse_field(s, s->CT, i);
        for (int z = 0; z < pz; ++z)
            for (int x = 0; x < px; ++x) {
                size_t i = ((size_t)x * q + y) * pz + z;
                flow[0 * plane + i] = RT[XEL * idx + (size_t)z * rp + x];
                flow[1 * plane + i] = RT[YEL * idx + (size_t)z * rp + x];
                flow[2 * plane + i] = RT[ZEL * idx + (size_t)z * rp + x];
            }
    }
}

double *cport_mc(cport *s, int i_step) { return (double *)(s->MC + (size_t)i_step * 3 * s->csz); }
double *cport_mic(cport *s, int i_step) { return (double *)(s->MIC + (size_t)i_step * 3 * s->csz); }
double *cport_mc_sub(cport *s, int count) { return (double *)(s->MC + (size_t)count * s->csz); }
double *cport_mic_sub(cport *s, int count) { return (double *)(s->MIC + (size_t)count * s->csz); }
const double *cport_qy(cport *s) { return s->Qy; }
const double *cport_w(cport *s) { return s->W; }

int cport_dims(cport *s, int *qpts, int *dimR, int *dimQ, int *Nx, int *Nz, int *nsteps)
{
    if (qpts) *qpts = s->qpts;
    if (dimR) *dimR = s->dimR;
    if (dimQ) *dimQ = s->dimQ;
    if (Nx) *Nx = s->Nx;
    if (Nz) *Nz = s->Nz;
    if (nsteps) *nsteps = s->nsteps;
    return 0;
}

const double *cport_table(cport *s, int which)
{
    const double *t[] = { s->Q, s->Qp, s->Qpp, s->R, s->Rp, s->Qw, s->Qpw, s->Qppw, s->Rw, s->Rpw,
                          s->Qs, s->Qps, s->Qpps, s->Rs, s->Rps };
    if (which < 0 || which >= (int)(sizeof(t) / sizeof(t[0]))) return NULL;
    return t[which];
}

/* ================================================================== */
/* Exact discrete adjoint of the homogeneous tangent step (no reference */
/* counterpart: the reference's adjoint, cport_adjoint, integrates the  */
/* continuous adjoint equations with reversed RK coefficients and is    */
/* not the transpose of its tangent).  Reverse mode by hand of          */
/* cport_tangent_forcing(kind 0): every linear piece of a tangent        */
/* substage is transposed with respect to the Euclidean inner product   */
/* of the real and imaginary parts of all coefficients.                 */
/* ================================================================== */

/* smmult transposed: ybar += A^T bbar */
static void smmult_T(const double *A, const cpx *bbar, cpx *ybar, int dl, int du, int N, int X, int x0)
{
#define A3(i, j, x) A[((size_t)(i) * 9 + (j)) * X + (x)]
    for (int i = 0; i < N; ++i)
        for (int j = MAXI(0, dl - (i / 2)); j < MINI(dl + du + 1, (N - i + 1) / 2 + dl); ++j)
            for (int x = x0; x < X; ++x) {
                ybar[(i - 2 * (dl - j)) * X + x].re += A3(i, j, x) * bbar[i * X + x].re;
                ybar[(i - 2 * (dl - j)) * X + x].im += A3(i, j, x) * bbar[i * X + x].im;
            }
#undef A3
}

/* bsolve transposed: solves A^T y = b in place with the same no-pivot
   every-other-diagonal factorisation A = L U (U^T first, then L^T) */
static void bsolve_T(double *A, cpx *b, int dl, int du, int N, int X, int x0)
{
#define A3(i, j, x) A[((size_t)(i) * 9 + (j)) * X + (x)]
    for (int i = 2; i < N; ++i) {
        for (int j = MAXI(0, dl - (i / 2)); j < dl; ++j) {
            for (int k = 1; k <= j - MAXI(0, dl - (i / 2)); ++k)
                for (int x = x0; x < X; ++x)
                    A3(i, j, x) = A3(i, j, x) - A3(i, j - k, x) * A3(i - 2 * (dl - j + k), dl + k, x);
            for (int x = x0; x < X; ++x) A3(i, j, x) = A3(i, j, x) / A3(i - 2 * (dl - j), dl, x);
        }
        for (int j = 0; j < MINI(du, (N - i + 1) / 2); ++j)
            for (int k = 1; k <= MINI(i / 2, MINI(dl, du - j)); ++k)
                for (int x = x0; x < X; ++x)
                    A3(i, j + dl, x) = A3(i, j + dl, x) - A3(i, dl - k, x) * A3(i - 2 * k, dl + j + k, x);
    }
    /* U^T w = b, U(m, m + 2j) = A[m][dl + j]: ascending */
    for (int i = 0; i < N; ++i) {
        for (int j = 1; j <= du; ++j) {
            const int m = i - 2 * j;
            if (m < 0) break;
            if (j > MINI(du, ((N - m + 1) / 2 - 1))) continue;
            for (int x = x0; x < X; ++x) {
                b[i * X + x].re -= A3(m, dl + j, x) * b[m * X + x].re;
                b[i * X + x].im -= A3(m, dl + j, x) * b[m * X + x].im;
            }
        }
        for (int x = x0; x < X; ++x) {
            b[i * X + x].re /= A3(i, dl, x);
            b[i * X + x].im /= A3(i, dl, x);
        }
    }
    /* L^T y = w, L(m, m - 2(dl - j)) = A[m][j], unit diagonal: descending */
    for (int i = N - 1; i >= 0; --i)
        for (int j = 0; j < dl; ++j) {
            const int m = i + 2 * (dl - j);
            if (m >= N || m < 2 || j < MAXI(0, dl - (m / 2))) continue;
            for (int x = x0; x < X; ++x) {
                b[i * X + x].re -= A3(m, j, x) * b[m * X + x].re;
                b[i * X + x].im -= A3(m, j, x) * b[m * X + x].im;
            }
        }
#undef A3
}

/* single-matrix versions (mean mode), element strides bs / ys */
static void smmult_single_T(const double *A, int w, const cpx *bbar, int bs, cpx *ybar, int ys, int dl, int du, int N)
{
    for (int i = 0; i < N; ++i)
        for (int j = MAXI(0, dl - (i / 2)); j < MINI(dl + du + 1, (N - i + 1) / 2 + dl); ++j) {
            ybar[(i - 2 * (dl - j)) * ys].re += A[i * w + j] * bbar[i * bs].re;
            ybar[(i - 2 * (dl - j)) * ys].im += A[i * w + j] * bbar[i * bs].im;
        }
}

static void bsolve_single_T(double *A, int w, cpx *b, int bs, int dl, int du, int N)
{
#define A2(i, j) A[(size_t)(i) * w + (j)]
    for (int i = 2; i < N; ++i) {
        for (int j = MAXI(0, dl - (i / 2)); j < dl; ++j) {
            for (int k = 1; k <= j - MAXI(0, dl - (i / 2)); ++k)
                A2(i, j) = A2(i, j) - A2(i, j - k) * A2(i - 2 * (dl - j + k), dl + k);
            A2(i, j) = A2(i, j) / A2(i - 2 * (dl - j), dl);
        }
        for (int j = 0; j < MINI(du, (N - i + 1) / 2); ++j)
            for (int k = 1; k <= MINI(i / 2, MINI(dl, du - j)); ++k)
                A2(i, j + dl) = A2(i, j + dl) - A2(i, dl - k) * A2(i - 2 * k, dl + j + k);
    }
    for (int i = 0; i < N; ++i) {
        for (int j = 1; j <= du; ++j) {
            const int m = i - 2 * j;
            if (m < 0) break;
            if (j > MINI(du, ((N - m + 1) / 2 - 1))) continue;
            b[i * bs].re -= A2(m, dl + j) * b[m * bs].re;
            b[i * bs].im -= A2(m, dl + j) * b[m * bs].im;
        }
        b[i * bs].re /= A2(i, dl);
        b[i * bs].im /= A2(i, dl);
    }
    for (int i = N - 1; i >= 0; --i)
        for (int j = 0; j < dl; ++j) {
            const int m = i + 2 * (dl - j);
            if (m >= N || m < 2 || j < MAXI(0, dl - (m / 2))) continue;
            b[i * bs].re -= A2(m, j) * b[m * bs].re;
            b[i * bs].im -= A2(m, j) * b[m * bs].im;
        }
#undef A2
}

/* recon_line transposed: Ub (5 components of line z) -> Cb (accumulate) */
static void recon_line_T(cport *s, const cpx *Ub, cpx *Cb, int z, int x0)
{
    const int X = s->X, q = s->qpts, D = s->dimQ, R = s->dimR;
    const double kz = s->Kz[z];
    for (int i = 0; i < q; ++i)
        for (int x = x0; x < X; ++x) {
            const double kx = s->Kx[x], k2 = s->K2[z * X + x];
            const cpx ux = Ub[UI(s, z, XEL, i, x)], uz = Ub[UI(s, z, ZEL, i, x)];
            const cpx dx = Ub[UI(s, z, DXEL, i, x)], dz = Ub[UI(s, z, DZEL, i, x)];
            /* forward: u = -i (kx Xp + kz Zp)/k2, w = i (kx Zp - kz Xp)/k2 with
               Xp = -Qp a, Zp = R b; du = i (kx dx - kz dz)/k2, dw = i (kx dz + kz dx)/k2
               with dx = Qpp a, dz = Rp b */
            cpx xp, zp, ddx, ddz;
            xp.re = (-kx * ux.im - kz * uz.im) / k2;   /* (i kx u + i kz w)/k2 */
            xp.im = (kx * ux.re + kz * uz.re) / k2;
            zp.re = (-kz * ux.im + kx * uz.im) / k2;   /* (i kz u - i kx w)/k2 */
            zp.im = (kz * ux.re - kx * uz.re) / k2;
            ddx.re = (kx * dx.im + kz * dz.im) / k2;   /* -(i kx du + i kz dw)/k2 */
            ddx.im = (-kx * dx.re - kz * dz.re) / k2;
            ddz.re = (-kz * dx.im + kx * dz.im) / k2;  /* (i kz du - i kx dw)/k2 */
            ddz.im = (kz * dx.re - kx * dz.re) / k2;
            const cpx v = Ub[UI(s, z, YEL, i, x)];
            for (int j = 0; j < D; ++j) {
                cpx *a = &Cb[CI(s, z, ALPHA, j, x)];
                a->re += s->Q[i * D + j] * v.re - s->Qp[i * D + j] * xp.re + s->Qpp[i * D + j] * ddx.re;
                a->im += s->Q[i * D + j] * v.im - s->Qp[i * D + j] * xp.im + s->Qpp[i * D + j] * ddx.im;
            }
            for (int j = 0; j < R; ++j) {
                cpx *b = &Cb[CI(s, z, BETA, j, x)];
                b->re += s->R[i * R + j] * zp.re + s->Rp[i * R + j] * ddz.re;
                b->im += s->R[i * R + j] * zp.im + s->Rp[i * R + j] * ddz.im;
            }
        }
}

static void recon_mean_T(cport *s, const cpx *Ub, cpx *Cb)
{
    const int q = s->qpts, R = s->dimR;
    for (int i = 0; i < q; ++i) {
        const cpx u = Ub[UI(s, 0, XEL, i, 0)], du = Ub[UI(s, 0, DXEL, i, 0)];
        const cpx w = Ub[UI(s, 0, ZEL, i, 0)], dw = Ub[UI(s, 0, DZEL, i, 0)];
        for (int j = 0; j < R; ++j) {
            cpx *a = &Cb[CI(s, 0, ALPHA, j, 0)], *b = &Cb[CI(s, 0, BETA, j, 0)];
            a->re += s->R[i * R + j] * u.re + s->Rp[i * R + j] * du.re;
            a->im += s->R[i * R + j] * u.im + s->Rp[i * R + j] * du.im;
            b->re += s->R[i * R + j] * w.re + s->Rp[i * R + j] * dw.re;
            b->im += s->R[i * R + j] * w.im + s->Rp[i * R + j] * dw.im;
        }
    }
}

static void recon_T(cport *s, const cpx *Ub, cpx *Cb)
{
    recon_mean_T(s, Ub, Cb);
    recon_line_T(s, Ub, Cb, 0, 1);
    for (int z = 1; z < s->Nz; ++z)
        if (z != s->Nz / 2) recon_line_T(s, Ub, Cb, z, 0);
}

/* rhs_fa / rhs_fb transposed: Fa_bar (D rows), Fb_bar (R rows) of line z -> Hbar (accumulate) */
static void quad_line_T(cport *s, const cpx *Fab, const cpx *Fbb, cpx *Hb, int z, int x0)
{
    const int X = s->X, D = s->dimQ, R = s->dimR, q = s->qpts;
    const double kz = s->Kz[z];
    for (int j = 0; j < q; ++j)
        for (int x = x0; x < X; ++x) {
            const double kx = s->Kx[x], k2 = s->K2[z * X + x];
            cpx pa = {0.0, 0.0}, qa = {0.0, 0.0}, rb = {0.0, 0.0};
            for (int i = 0; i < D; ++i) {
                pa.re += s->Qpw[i * q + j] * Fab[i * X + x].re;
                pa.im += s->Qpw[i * q + j] * Fab[i * X + x].im;
                qa.re += s->Qw[i * q + j] * Fab[i * X + x].re;
                qa.im += s->Qw[i * q + j] * Fab[i * X + x].im;
            }
            for (int i = 0; i < R; ++i) {
                rb.re += s->Rw[i * q + j] * Fbb[i * X + x].re;
                rb.im += s->Rw[i * q + j] * Fbb[i * X + x].im;
            }
            /* forward: Fa = Qpw (i kx Hx + i kz Hz) - K2 Qw Hy, Fb = Rw (i kz Hx - i kx Hz) */
            cpx *hx = &Hb[UI(s, z, HXEL, j, x)], *hy = &Hb[UI(s, z, HYEL, j, x)], *hz = &Hb[UI(s, z, HZEL, j, x)];
            hx->re += kx * pa.im + kz * rb.im;      /* -i kx pa - i kz rb */
            hx->im += -kx * pa.re - kz * rb.re;
            hz->re += kz * pa.im - kx * rb.im;      /* -i kz pa + i kx rb */
            hz->im += -kz * pa.re + kx * rb.re;
            hy->re += -k2 * qa.re;
            hy->im += -k2 * qa.im;
        }
}

/* primal real fields of one state on every plane: [Q][MAXT][pz][hx], as pass1 */
static void primal_fields(cport *s, const cpx *C, cpx *out)
{
    recon(s, C, s->U);
    const size_t per = (size_t)MAXT * s->pz * s->hx;
    for (int y = 0; y < s->qpts; ++y) {
        cpx *T = out + (size_t)y * per;
        memset(T, 0, sizeof(cpx) * per);
        load_curl(s, T, s->U, y);
        for (int i = 0; i < MAXT; ++i) inverse_field(s, T, i);
    }
}

/* the tangent half of pass1 transposed: Hbar (slots HZ, HX, HY of the kept
   modes) -> Ubar (5 components, accumulate); RTs the primal real fields */
static void pass1_T(cport *s, const cpx *RTs, const cpx *Hb, cpx *Ub)
{
    const int pz = s->pz, px = s->px, hx = s->hx, rp = px + 2, X = s->X, Nz = s->Nz;
    const size_t idx = (size_t)pz * rp, per = (size_t)MAXT * pz * hx;
    const double norm = 1.0 / ((3. * s->Nx / 2.) * (3. * s->Nz / 2.));
    cpx *NT = s->ICT;  /* product cotangents [3][pz][hx] */
    cpx *FT = s->CT;   /* field cotangents [6][pz][hx] */
    for (int y = 0; y < s->qpts; ++y) {
        const double *RT = (const double *)(RTs + (size_t)y * per);
        memset(NT, 0, sizeof(cpx) * (size_t)3 * pz * hx);
        /* store_field and scale_field transposed: kept rows, x < X */
        for (int c = 0; c < 3; ++c)
            for (int zp = 0; zp < pz; ++zp) {
                int z = -1;
                if (zp < Nz / 2) z = zp;
                else if (zp > Nz) z = zp - Nz / 2;
                if (z < 0) continue;
                for (int x = 0; x < X; ++x) {
                    const cpx h = Hb[UI(s, z, c, y, x)];
                    NT[TI(s, c, zp, x)].re = norm * h.re;
                    NT[TI(s, c, zp, x)].im = norm * h.im;
                }
            }
        for (int c = 0; c < 3; ++c) {
            cpx *base = &NT[TI(s, c, 0, 0)];
            /* the z transform (sign -1) transposed: sign +1, columns x < X */
            for (int x = 0; x < X; ++x) offt_exec(s->pf1, base + x, hx, base + x, hx);
            /* the real-to-complex x transform transposed: halve bins 1..px/2-1, then c2r */
            for (int zp = 0; zp < pz; ++zp) {
                cpx *row = base + (size_t)zp * hx;
                for (int k = 1; k < hx - 1; ++k) { row[k].re *= 0.5; row[k].im *= 0.5; }
                offt_c2r(s->pr1, row, 1, (double *)row, 1);
            }
        }
        const double *NR = (const double *)NT;
        double *FR = (double *)FT;
        memset(FT, 0, sizeof(cpx) * per);
        /* the tangent products (pass1.c:145-170) transposed */
        for (int zp = 0; zp < pz; ++zp)
            for (int x = 0; x < px; ++x) {
                const size_t o = (size_t)zp * rp + x;
                const double nx = NR[HXEL * idx + o], ny = NR[HYEL * idx + o], nz = NR[HZEL * idx + o];
                const double u = RT[XEL * idx + o], v = RT[YEL * idx + o], w = RT[ZEL * idx + o];
                const double wz = RT[WZEL * idx + o], wx = RT[WXEL * idx + o], wy = RT[WYEL * idx + o];
                FR[XEL * idx + o] = -ny * wz + nz * wy;
                FR[YEL * idx + o] = nx * wz - nz * wx;
                FR[ZEL * idx + o] = -nx * wy + ny * wx;
                FR[WZEL * idx + o] = nx * v - ny * u;
                FR[WXEL * idx + o] = ny * w - nz * v;
                FR[WYEL * idx + o] = -nx * w + nz * u;
            }
        for (int f = 0; f < MAXT; ++f) {
            cpx *base = &FT[TI(s, f, 0, 0)];
            /* c2r transposed: r2c, double bins 1..px/2-1 */
            for (int zp = 0; zp < pz; ++zp) {
                cpx *row = base + (size_t)zp * hx;
                offt_r2c(s->pr2, (double *)row, 1, row, 1);
                for (int k = 1; k < hx - 1; ++k) { row[k].re *= 2.0; row[k].im *= 2.0; }
            }
            /* the inverse z transform (sign +1) transposed: sign -1, columns x < X */
            for (int x = 0; x < X; ++x) offt_exec(s->pf2, base + x, hx, base + x, hx);
        }
        /* load_curl transposed: wz = -du + i kx v, wx = dw - i kz v, wy = i kz u - i kx w */
        for (int zp = 0; zp < pz; ++zp) {
            int z = -1;
            if (zp < Nz / 2) z = zp;
            else if (zp > Nz) z = zp - Nz / 2;
            if (z < 0) continue;
            const double kz = s->Kz[z];
            for (int x = 0; x < X; ++x) {
                const double kx = s->Kx[x];
                const cpx t0 = FT[TI(s, XEL, zp, x)], t1 = FT[TI(s, YEL, zp, x)], t2 = FT[TI(s, ZEL, zp, x)];
                const cpx t3 = FT[TI(s, WZEL, zp, x)], t4 = FT[TI(s, WXEL, zp, x)], t5 = FT[TI(s, WYEL, zp, x)];
                cpx *uu = &Ub[UI(s, z, XEL, y, x)], *vv = &Ub[UI(s, z, YEL, y, x)], *ww = &Ub[UI(s, z, ZEL, y, x)];
                cpx *dx = &Ub[UI(s, z, DXEL, y, x)], *dz = &Ub[UI(s, z, DZEL, y, x)];
                /* u += t0 - i kz t5 ; v += t1 - i kx t3 + i kz t4 ; w += t2 + i kx t5 */
                uu->re += t0.re + kz * t5.im;
                uu->im += t0.im - kz * t5.re;
                vv->re += t1.re + kx * t3.im - kz * t4.im;
                vv->im += t1.im - kx * t3.re + kz * t4.re;
                ww->re += t2.re - kx * t5.im;
                ww->im += t2.im + kx * t5.re;
                dx->re -= t3.re;
                dx->im -= t3.im;
                dz->re += t4.re;
                dz->im += t4.im;
            }
        }
    }
}

/* one substage reversed.  In: cb (carried cotangent after the substage) and
   ub (velocity cotangent after it); out: the same before the substage.  Hb
   is scratch of the U size; RTs the primal fields of substage k. */
static void substage_T(cport *s, int k, cpx *cb, cpx *ub, cpx *Hb, cpx *xb, const cpx *RTs)
{
    const int X = s->X, D = s->dimQ, R = s->dimR, q = s->qpts;
    const double *a = fa_, *b = fb_, *c = fc_, *d = fd_;
    memset(Hb, 0, sizeof(cpx) * s->usz);
    memset(xb, 0, sizeof(cpx) * s->csz);
    recon_T(s, ub, xb);
    memset(ub, 0, sizeof(cpx) * s->usz);
    /* ---- mean mode ---- */
    {
        double *MZ = s->MZ;
        cpx *xa = &xb[CI(s, 0, ALPHA, 0, 0)], *xbb = &xb[CI(s, 0, BETA, 0, 0)];
        cpx *ca = &cb[CI(s, 0, ALPHA, 0, 0)], *cbb = &cb[CI(s, 0, BETA, 0, 0)];
        cpx *fab = s->fa, *fbb = s->fb;
        memset(fab, 0, sizeof(cpx) * R);
        memset(fbb, 0, sizeof(cpx) * R);
        if (k != 2) {
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] - s->re * a[k + 1] * s->dt * s->Rps[i * 5 + j];
            smmult_single_T(MZ, 5, ca, X, xa, X, RSDIAG - 1, RSDIAG - 1, R);
            smmult_single_T(MZ, 5, cbb, X, xbb, X, RSDIAG - 1, RSDIAG - 1, R);
            for (int i = 0; i < R; ++i) {
                fab[i].re = s->dt * d[k + 1] * ca[i * X].re;
                fbb[i].re = s->dt * d[k + 1] * cbb[i * X].re;
            }
        } else {
            for (int i = 0; i < R; ++i) {
                xa[i * X].re += ca[i * X].re; xa[i * X].im += ca[i * X].im;
                xbb[i * X].re += cbb[i * X].re; xbb[i * X].im += cbb[i * X].im;
            }
        }
        /* homogeneous flux correction x = xs + 0.5 add (-rwsum . xs.re), transposed */
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j];
        memset(s->add, 0, sizeof(cpx) * (size_t)R);
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < q; ++j) s->add[i].re += s->Rw[i * q + j];
        bsolve_single(MZ, 5, s->add, 1, RSDIAG - 1, RSDIAG - 1, R);
        double ax = 0.0;
        for (int j = 0; j < R; ++j) ax += s->add[j].re * xa[j * X].re;
        for (int i = 0; i < R; ++i) {
            double rws = 0.0;
            for (int j = 0; j < q; ++j) rws += s->Rw[i * q + j];
            xa[i * X].re -= 0.5 * rws * ax;
        }
        for (int v = 0; v < 2; ++v) {
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] + s->re * b[k] * s->dt * s->Rps[i * 5 + j];
            bsolve_single_T(MZ, 5, v == ALPHA ? xa : xbb, X, RSDIAG - 1, RSDIAG - 1, R);
        }
        for (int i = 0; i < R; ++i) {
            fab[i].re += s->dt * c[k] * xa[i * X].re;
            fbb[i].re += s->dt * c[k] * xbb[i * X].re;
        }
        for (int i = 0; i < R; ++i) { ca[i * X].re = 0; ca[i * X].im = 0; cbb[i * X].re = 0; cbb[i * X].im = 0; }
        if (k == 0) {
            for (int i = 0; i < R; ++i)
                for (int j = 0; j < T_RSDIAG; ++j) MZ[i * 5 + j] = s->Rs[i * 5 + j] - s->re * a[0] * s->dt * s->Rps[i * 5 + j];
            smmult_single_T(MZ, 5, xa, X, ca, X, RSDIAG - 1, RSDIAG - 1, R);
            smmult_single_T(MZ, 5, xbb, X, cbb, X, RSDIAG - 1, RSDIAG - 1, R);
        } else {
            for (int i = 0; i < R; ++i) { ca[i * X] = xa[i * X]; cbb[i * X] = xbb[i * X]; }
        }
        /* the mean quadrature fa = Rw Hx.re, fb = Rw Hz.re transposed */
        for (int j = 0; j < q; ++j) {
            double sa = 0.0, sb = 0.0;
            for (int i = 0; i < R; ++i) { sa += s->Rw[i * q + j] * fab[i].re; sb += s->Rw[i * q + j] * fbb[i].re; }
            Hb[UI(s, 0, HXEL, j, 0)].re += sa;
            Hb[UI(s, 0, HZEL, j, 0)].re += sb;
        }
    }
    /* ---- lines ---- */
    for (int z = 0; z < s->Nz; ++z) {
        const int x0 = z == 0 ? 1 : 0;
        cpx *Ca = &cb[CI(s, z, ALPHA, 0, 0)], *Cbt = &cb[CI(s, z, BETA, 0, 0)];
        cpx *Xa = &xb[CI(s, z, ALPHA, 0, 0)], *Xbt = &xb[CI(s, z, BETA, 0, 0)];
        if (z == s->Nz / 2) {
            for (int v = 0; v < 2; ++v)
                for (int i = 0; i < R; ++i)
                    for (int x = 0; x < X; ++x) { cb[CI(s, z, v, i, x)].re = 0; cb[CI(s, z, v, i, x)].im = 0; }
            continue;
        }
        memset(s->Fa, 0, sizeof(cpx) * (size_t)R * X);
        memset(s->Fb, 0, sizeof(cpx) * (size_t)R * X);
        if (k != 2) {
            fill_v_lhs(s, z, x0, a[k + 1], 0);
            smmult_T(s->M, Ca, Xa, QSDIAG - 1, QSDIAG - 1, D, X, x0);
            fill_g_lhs(s, z, x0, a[k + 1], 0);
            smmult_T(s->M, Cbt, Xbt, RSDIAG - 1, RSDIAG - 1, R, X, x0);
            for (int x = x0; x < X; ++x) {
                for (int i = 0; i < D; ++i) {
                    s->Fa[i * X + x].re = s->dt * d[k + 1] * Ca[i * X + x].re;
                    s->Fa[i * X + x].im = s->dt * d[k + 1] * Ca[i * X + x].im;
                }
                for (int i = 0; i < R; ++i) {
                    s->Fb[i * X + x].re = s->dt * d[k + 1] * Cbt[i * X + x].re;
                    s->Fb[i * X + x].im = s->dt * d[k + 1] * Cbt[i * X + x].im;
                }
            }
        } else {
            for (int x = x0; x < X; ++x) {
                for (int i = 0; i < D; ++i) { Xa[i * X + x].re += Ca[i * X + x].re; Xa[i * X + x].im += Ca[i * X + x].im; }
                for (int i = 0; i < R; ++i) { Xbt[i * X + x].re += Cbt[i * X + x].re; Xbt[i * X + x].im += Cbt[i * X + x].im; }
            }
        }
        /* alpha rows >= D ride along unchanged */
        for (int x = x0; x < X; ++x)
            for (int i = D; i < R; ++i) Xa[i * X + x] = Ca[i * X + x];
        fill_v_lhs(s, z, x0, b[k], 1);
        bsolve_T(s->M, Xa, QSDIAG - 1, QSDIAG - 1, D, X, x0);
        fill_g_lhs(s, z, x0, b[k], 1);
        bsolve_T(s->M, Xbt, RSDIAG - 1, RSDIAG - 1, R, X, x0);
        for (int x = x0; x < X; ++x) {
            for (int i = 0; i < D; ++i) {
                s->Fa[i * X + x].re += s->dt * c[k] * Xa[i * X + x].re;
                s->Fa[i * X + x].im += s->dt * c[k] * Xa[i * X + x].im;
            }
            for (int i = 0; i < R; ++i) {
                s->Fb[i * X + x].re += s->dt * c[k] * Xbt[i * X + x].re;
                s->Fb[i * X + x].im += s->dt * c[k] * Xbt[i * X + x].im;
            }
        }
        for (int x = x0; x < X; ++x) {
            for (int i = 0; i < D; ++i) { Ca[i * X + x].re = 0; Ca[i * X + x].im = 0; }
            for (int i = D; i < R; ++i) Ca[i * X + x] = Xa[i * X + x];
            for (int i = 0; i < R; ++i) { Cbt[i * X + x].re = 0; Cbt[i * X + x].im = 0; }
        }
        if (k == 0) {
            fill_v_lhs(s, z, x0, a[0], 0);
            smmult_T(s->M, Xa, Ca, QSDIAG - 1, QSDIAG - 1, D, X, x0);
            fill_g_lhs(s, z, x0, a[0], 0);
            smmult_T(s->M, Xbt, Cbt, RSDIAG - 1, RSDIAG - 1, R, X, x0);
        } else {
            for (int x = x0; x < X; ++x) {
                for (int i = 0; i < D; ++i) Ca[i * X + x] = Xa[i * X + x];
                for (int i = 0; i < R; ++i) Cbt[i * X + x] = Xbt[i * X + x];
            }
        }
        quad_line_T(s, s->Fa, s->Fb, Hb, z, x0);
    }
    pass1_T(s, RTs, Hb, ub);
}

/* the transpose of cport_tangent_forcing(end -> start, kind 0) applied to
   AC_given (the cotangent at start_step > end_step).  The tangent
   linearises about the primal re-advanced from MC[3 end] rebuilt into
   velocity (channel/channel.c:496-514, 557-571), which after a laminar start
   without run-up differs from the stored trajectory, so the primal states
   are re-advanced here the same way. */
int cport_adjoint_exact(cport *s, int start_step, int end_step, double *AC_given)
{
    if (!(start_step > end_step && end_step >= 0 && start_step <= s->nsteps && AC_given)) return -2;
    const int nst = start_step - end_step;
    const size_t per = (size_t)s->qpts * MAXT * s->pz * s->hx;
    cpx *X = (cpx *)malloc(sizeof(cpx) * s->csz * (3 * (size_t)nst + 1));
    cpx *RTs = (cpx *)malloc(sizeof(cpx) * per);
    cpx *cb = (cpx *)calloc(s->csz, sizeof(cpx));
    cpx *xb = (cpx *)calloc(s->csz, sizeof(cpx));
    cpx *ub = (cpx *)calloc(s->usz, sizeof(cpx));
    cpx *Hb = (cpx *)calloc(s->usz, sizeof(cpx));
    int status = 0;
    if (!X || !RTs || !cb || !xb || !ub || !Hb) { status = -3; goto done; }
    /* primal states before every substage, re-advanced as the tangent does */
    memmove(s->C, s->MC + (size_t)end_step * 3 * s->csz, sizeof(cpx) * s->csz);
    memcpy(X, s->C, sizeof(cpx) * s->csz);
    recon(s, s->C, s->U);
    for (int n = 0; n < nst && status == 0; ++n)
        for (int k = 0; k < 3; ++k) {
            if (pass1(s, k) != 0) { status = -1; break; }
            solve_all(s, k, s->C, s->U, s->U, X + (size_t)(3 * n + k + 1) * s->csz, NULL, 0);
        }
    if (status) goto done;
    memcpy(cb, AC_given, sizeof(cpx) * s->csz);
    for (int n = nst - 1; n >= 0; --n)
        for (int k = 2; k >= 0; --k) {
            primal_fields(s, X + (size_t)(3 * n + k) * s->csz, RTs);
            substage_T(s, k, cb, ub, Hb, xb, RTs);
        }
    /* the tangent starts from IU = Recon(IC) */
    recon_T(s, ub, cb);
    memcpy(AC_given, cb, sizeof(cpx) * s->csz);
done:
    free(X); free(RTs); free(cb); free(xb); free(ub); free(Hb);
    return status;
}
