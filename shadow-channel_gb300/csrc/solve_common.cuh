// Banded row operations shared by the implicit solve (recon_solve.cu) and
// its transpose (adjoint_exact.cu): the every-other-diagonal matrices of
// channel/mvOps.c and the viscous operators of the Re forcing.
#pragma once

#include "chn_common.cuh"

namespace chn {

// out[i] = sum_j A[i][j] y[i + 2(j - DL)] over the valid band (channel/mvOps.c:198-220),
// band layout (width W, lower DL, upper DU) known at compile time: the band
// loop unrolls with per-term predicates (the loads issue together), the
// multiply-adds keep the ascending order
template <int W, int DL, int DU>
__device__ __forceinline__ cpx band_matvec_row_t(const double* __restrict__ A, int N, const cpx* y, int ystride,
                                                 int i) {
  int j0 = DL - i / 2;
  if (j0 < 0) j0 = 0;
  int j1 = (N - i + 1) / 2 + DL;
  if (j1 > DL + DU + 1) j1 = DL + DU + 1;
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int j = 0; j < DL + DU + 1; ++j) {
    if (j < j0 || j >= j1) continue;
    const double a = __ldg(A + (size_t)i * W + j);
    const cpx v = y[(i - 2 * (DL - j)) * ystride];
    re = fma(a, v.re, re);
    im = fma(a, v.im, im);
  }
  return cpx{re, im};
}

// the same for the two band layouts in use, chosen by the arguments
__device__ __forceinline__ cpx band_matvec_row(const double* __restrict__ A, int w, int dl, int du, int N,
                                               const cpx* y, int ystride, int i) {
  if (w == 9 && dl == 4 && du == 4) return band_matvec_row_t<9, 4, 4>(A, N, y, ystride, i);
  if (w == 5 && dl == 2 && du == 2) return band_matvec_row_t<5, 2, 2>(A, N, y, ystride, i);
  int j0 = dl - i / 2;
  if (j0 < 0) j0 = 0;
  int j1 = (N - i + 1) / 2 + dl;
  if (j1 > dl + du + 1) j1 = dl + du + 1;
  double re = 0.0, im = 0.0;
  for (int j = j0; j < j1; ++j) {
    const double a = __ldg(A + (size_t)i * w + j);
    const cpx v = y[(i - 2 * (dl - j)) * ystride];
    re = fma(a, v.re, re);
    im = fma(a, v.im, im);
  }
  return cpx{re, im};
}

// row r of (K2^2 Qs + 2 K2 Qps + Qpps) y and of (Rps + K2 Rs) y, the viscous
// operators of the alpha and beta systems (channel/tangent_forcing.c:38-68)
__device__ __forceinline__ cpx visc_v_row(const Grid& g, double k2, const cpx* y, int ystride, int r) {
  const int dl = 4, du = 4, N = g.D;
  int j0 = dl - r / 2;
  if (j0 < 0) j0 = 0;
  int j1 = (N - r + 1) / 2 + dl;
  if (j1 > dl + du + 1) j1 = dl + du + 1;
  const double sq = k2 * k2;
  double re = 0.0, im = 0.0;
  for (int j = j0; j < j1; ++j) {
    const size_t o = (size_t)r * 9 + j;
    const double m = sq * __ldg(g.Qs + o) + 2. * k2 * __ldg(g.Qps + o) + __ldg(g.Qpps + o);
    const cpx v = y[(r - 2 * (dl - j)) * ystride];
    re = fma(m, v.re, re);
    im = fma(m, v.im, im);
  }
  return cpx{re, im};
}

__device__ __forceinline__ cpx visc_g_row(const Grid& g, double k2, const cpx* y, int ystride, int r) {
  const int dl = 2, du = 2, N = g.R;
  int j0 = dl - r / 2;
  if (j0 < 0) j0 = 0;
  int j1 = (N - r + 1) / 2 + dl;
  if (j1 > dl + du + 1) j1 = dl + du + 1;
  double re = 0.0, im = 0.0;
  for (int j = j0; j < j1; ++j) {
    const size_t o = (size_t)r * 5 + j;
    const double m = __ldg(g.Rps + o) + k2 * __ldg(g.Rs + o);
    const cpx v = y[(r - 2 * (dl - j)) * ystride];
    re = fma(m, v.re, re);
    im = fma(m, v.im, im);
  }
  return cpx{re, im};
}

// row r of Rps y for a real vector y (stride 1)
__device__ __forceinline__ double rps_row_real(const Grid& g, const double* y, int r) {
  const int dl = 2, du = 2, N = g.R;
  int j0 = dl - r / 2;
  if (j0 < 0) j0 = 0;
  int j1 = (N - r + 1) / 2 + dl;
  if (j1 > dl + du + 1) j1 = dl + du + 1;
  double acc = 0.0;
  for (int j = j0; j < j1; ++j) acc = fma(__ldg(g.Rps + (size_t)r * 5 + j), y[r - 2 * (dl - j)], acc);
  return acc;
}

}  // namespace chn
