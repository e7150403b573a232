// Exact discrete adjoint of the homogeneous tangent step: the transpose of
// one RK3 substage of the tangent (channel/channel.c:546-573 with
// channel/pass1.c:140-210 and channel/increproject*.c), taken with respect to
// the Euclidean inner product of the real and imaginary parts of every
// coefficient.  The reference's own adjoint (channel/channel.c:596-696) runs
// the continuous adjoint equations with reversed RK coefficients and is not
// this transpose; its dot products <lambda, T v> and <T^T lambda, v> agree
// only to the discretisation error.
//
// A tangent substage k maps (c_in, u_in) -> (c_out, u_out):
//   c1 = E_0 c_in (k == 0) or c_in,  F = Quad(H(u_in)),  c2 = c1 + dt c_k F,
//   x  = L_k^{-1} c2 (plus the homogeneous flux correction of the mean mode),
//   u_out = Recon(x),  c_out = E_{k+1} x + dt d_{k+1} F (k < 2) or x.
// k_solve_T runs the reverse of everything but the products:
//   x_bar = Recon^T(u_out_bar) + E_{k+1}^T c_out_bar (or c_out_bar),
//   F_bar = dt d_{k+1} c_out_bar,  x_bar <- flux^T x_bar,  c2_bar = L^{-T} x_bar,
//   F_bar += dt c_k c2_bar,  c_in_bar = E_0^T c2_bar (or c2_bar),
//   H_bar = Quad^T(F_bar)  (written pre-scaled for the inverse transform),
// and the products kernel (k_products_adj with `exact`) takes H_bar's
// physical fields to u_in_bar.
#include "chn_common.cuh"
#include "kernels.h"
#include "sizes.cuh"
#include "solve_common.cuh"
#include "tc_common.cuh"

namespace chn {

static constexpr int kThreads = 256;
static constexpr int kTile = 16;  // kx columns per block

__device__ __forceinline__ bool blocked_t(const uint32_t* status, int sdiv, int inst) {
  return status != nullptr && (status[inst / sdiv] & ST_CFL) != 0;
}

__device__ __forceinline__ void cfma_t(double w, const cpx& a, double& re, double& im) {
  re = fma(w, a.re, re);
  im = fma(w, a.im, im);
}

// row m of A^T y for a banded every-other-diagonal A (row i holds A[i][j] at
// column i + 2(j - dl), valid j as in channel/mvOps.c:198-220)
__device__ __forceinline__ cpx band_matvecT_row(const double* __restrict__ A, int w, int dl, int du, int N,
                                                const cpx* y, int ystride, int m) {
  double re = 0.0, im = 0.0;
  for (int j = 0; j <= dl + du; ++j) {
    const int i = m + 2 * (dl - j);
    if (i < 0 || i >= N) continue;
    int j0 = dl - i / 2;
    if (j0 < 0) j0 = 0;
    int j1 = (N - i + 1) / 2 + dl;
    if (j1 > dl + du + 1) j1 = dl + du + 1;
    if (j < j0 || j >= j1) continue;
    const double a = __ldg(A + (size_t)i * w + j);
    const cpx v = y[i * ystride];
    re = fma(a, v.re, re);
    im = fma(a, v.im, im);
  }
  return cpx{re, im};
}

// A^T y = b for one parity chain, A = L U the no-pivot factors of
// channel/mvOps.c:29-91 (L unit lower in columns j < dl, U in dl..dl+du):
// U^T w = b ascending, then L^T y = w descending; RD the reciprocal pivots
// (the forward chain multiplies by them too)
template <int W, int DL, int DU>
__device__ void band_solveT_chain(const double* __restrict__ LU, const double* __restrict__ RD, int N, int par,
                                  double* b, int bstride) {
  for (int i = par; i < N; i += 2) {
    double acc = b[i * bstride];
#pragma unroll
    for (int j = 1; j <= DU; ++j) {
      const int m = i - 2 * j;
      // row m of U holds column i when m >= 0 and j <= min(DU, (N - m + 1) / 2 - 1)
      if (m >= 0 && j <= (N - m + 1) / 2 - 1) acc = fma(-__ldg(LU + (size_t)m * W + DL + j), b[m * bstride], acc);
    }
    b[i * bstride] = acc * __ldg(RD + i);
  }
  const int ilast = ((N - 1 - par) % 2 == 0) ? N - 1 : N - 2;
  for (int i = ilast; i >= 0; i -= 2) {
    double acc = b[i * bstride];
#pragma unroll
    for (int t = 1; t <= DL; ++t) {
      const int m = i + 2 * t;
      if (m < N && t <= m / 2) acc = fma(-__ldg(LU + (size_t)m * W + DL - t), b[m * bstride], acc);
    }
    b[i * bstride] = acc;
  }
}

struct SolveTSmem {
  cpx* hc;     // [Qh][kTile][6] parity-combined inputs of Recon^T
  cpx* ra;     // [R][kTile] alpha cotangents (aliases hc)
  cpx* rb;     // [R][kTile]
  cpx* Fa;     // [D][kTile] Recon^T alpha part, then F_bar alpha
  cpx* Fb;     // [R][kTile]
  double* m0;  // mean mode: fa[R], fb[R], ca[R] (cpx), cb[R] (cpx)
};

// bytes of the tensor-core digits: Recon^T's [7][32][Q pad] (+ exponents),
// Quad^T's two [7][32][R pad] (+ exponents)
__host__ __device__ inline size_t solveT_tc_bytes(const Grid& g) {
  const size_t rq = (size_t)kDig * 32 * ((g.Q + 15) / 16 * 16 + 8) * 2 + kTile * sizeof(int);
  const size_t qt = (size_t)2 * kDig * 32 * ((g.R + 15) / 16 * 16 + 8) * 2 + 2 * kTile * sizeof(int);
  return rq > qt ? rq : qt;
}

__host__ __device__ inline size_t solveT_hc_elems(const Grid& g) {
  size_t hc = (size_t)g.Qh * kTile * 6, r = 2 * (size_t)g.R * kTile;
  const size_t tc = (solveT_tc_bytes(g) + sizeof(cpx) - 1) / sizeof(cpx);
  if (tc > hc) hc = tc;
  return hc > r ? hc : r;
}

static size_t solveT_smem_bytes(const Grid& g) {
  size_t n = solveT_hc_elems(g) + (size_t)g.D * kTile + (size_t)g.R * kTile;
  return n * sizeof(cpx) + (size_t)8 * g.R * sizeof(double);
}

__device__ inline SolveTSmem carve_solveT(const Grid& g, unsigned char* base) {
  SolveTSmem s;
  cpx* p = reinterpret_cast<cpx*>(base);
  s.hc = p;
  s.ra = p;
  s.rb = p + (size_t)g.R * kTile;
  p += solveT_hc_elems(g);
  s.Fa = p; p += (size_t)g.D * kTile;
  s.Fb = p; p += (size_t)g.R * kTile;
  s.m0 = reinterpret_cast<double*>(p);
  return s;
}

// Recon^T of the velocity cotangent of columns x0.. (not the mean mode):
//   alpha_bar = Q^T v_bar - Q'^T Xp_bar + Q''^T dx_bar   (rows < D) -> s.Fa
//   beta_bar  = R^T Zp_bar + R'^T dz_bar                 (rows < R) -> s.Fb
// with Xp_bar = (i kx u_bar + i kz w_bar)/K2, Zp_bar = (i kz u_bar - i kx w_bar)/K2,
// dx_bar = -(i kx du_bar + i kz dw_bar)/K2, dz_bar = (i kz du_bar - i kx dw_bar)/K2
// (the transpose of channel/initAlphaBeta2.c:12-240).  The sums over the
// Gauss planes pair y with -y as the quadratures of k_solve do.
__device__ void recon_T_tile(const Grid& g, const cpx* __restrict__ Ub, int z, int x0, int nx, int xfirst,
                             SolveTSmem& s) {
  const int lx = threadIdx.x % kTile, grp = threadIdx.x / kTile, ngrp = blockDim.x / kTile;
  const size_t cs = (size_t)g.Q * g.X;
  const cpx* Uz = Ub + (size_t)z * 5 * cs;
  for (int phase = 0; phase < 2; ++phase) {
    const int nin = phase == 0 ? 3 : 2;
    for (int i = threadIdx.x; i < g.Qh * kTile; i += blockDim.x) {
      const int yp = i / kTile, l = i - yp * kTile;
      cpx* dst = s.hc + (size_t)i * 6;
      if (l >= nx || l < xfirst) continue;
      const int x = x0 + l;
      const double ax = g.kxK2[(size_t)z * g.X + x], az = g.kzK2[(size_t)z * g.X + x];
      const int ya = yp, yb = g.Q - 1 - yp;
      cpx in[2][3];
      for (int side = 0; side < 2; ++side) {
        const int y = side ? yb : ya;
        const cpx u = Uz[0 * cs + (size_t)y * g.X + x], w = Uz[2 * cs + (size_t)y * g.X + x];
        const cpx du = Uz[3 * cs + (size_t)y * g.X + x], dw = Uz[4 * cs + (size_t)y * g.X + x];
        if (phase == 0) {
          in[side][0] = Uz[1 * cs + (size_t)y * g.X + x];
          in[side][1].re = -fma(ax, u.im, az * w.im);  // Xp_bar = i(ax u + az w)
          in[side][1].im = fma(ax, u.re, az * w.re);
          in[side][2].re = fma(ax, du.im, az * dw.im);  // dx_bar = -i(ax du + az dw)
          in[side][2].im = -fma(ax, du.re, az * dw.re);
        } else {
          in[side][0].re = fma(ax, w.im, -az * u.im);  // Zp_bar = i(az u - ax w)
          in[side][0].im = fma(az, u.re, -ax * w.re);
          in[side][1].re = fma(ax, dw.im, -az * du.im);  // dz_bar = i(az du - ax dw)
          in[side][1].im = fma(az, du.re, -ax * dw.re);
        }
      }
      for (int q = 0; q < nin; ++q) {
        if (ya == yb) {  // centre plane of an odd point count
          dst[2 * q] = in[0][q];
          dst[2 * q + 1] = in[0][q];
        } else {
          dst[2 * q].re = in[0][q].re + in[1][q].re;
          dst[2 * q].im = in[0][q].im + in[1][q].im;
          dst[2 * q + 1].re = in[0][q].re - in[1][q].re;
          dst[2 * q + 1].im = in[0][q].im - in[1][q].im;
        }
      }
    }
    __syncthreads();
    if (lx < nx && lx >= xfirst) {
      const int N = phase == 0 ? g.D : g.R;
      constexpr int MAXR = 4;
      for (int ib = grp; ib < N; ib += ngrp * MAXR) {
        double sr[MAXR], si[MAXR];
#pragma unroll
        for (int m = 0; m < MAXR; ++m) { sr[m] = 0.0; si[m] = 0.0; }
        const bool even = (ib & 1) == 0;
        for (int yp = 0; yp < g.Qh; ++yp) {
          const cpx* src = s.hc + ((size_t)yp * kTile + lx) * 6;
          if (phase == 0) {
            // even rows: Q, Q'' (even bases) with "+", Q' (odd basis) with "-"
            const cpx V = src[even ? 0 : 1];
            const cpx Xp = src[even ? 3 : 2];
            const cpx Dx = src[even ? 4 : 5];
#pragma unroll
            for (int m = 0; m < MAXR; ++m) {
              const int i = ib + m * ngrp;
              if (i < N) {
                const size_t o = (size_t)yp * g.D + i;
                cfma_t(__ldg(g.Bq + o), V, sr[m], si[m]);
                cfma_t(-__ldg(g.Bqp + o), Xp, sr[m], si[m]);
                cfma_t(__ldg(g.Bqpp + o), Dx, sr[m], si[m]);
              }
            }
          } else {
            const cpx Zp = src[even ? 0 : 1];
            const cpx Dz = src[even ? 3 : 2];
#pragma unroll
            for (int m = 0; m < MAXR; ++m) {
              const int i = ib + m * ngrp;
              if (i < N) {
                const size_t o = (size_t)yp * g.R + i;
                cfma_t(__ldg(g.Br + o), Zp, sr[m], si[m]);
                cfma_t(__ldg(g.Brp + o), Dz, sr[m], si[m]);
              }
            }
          }
        }
#pragma unroll
        for (int m = 0; m < MAXR; ++m) {
          const int i = ib + m * ngrp;
          if (i >= N) continue;
          (phase == 0 ? s.Fa : s.Fb)[i * kTile + lx] = cpx{sr[m], si[m]};
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// the transposed contractions on the tensor cores (tc_common.cuh), the
// scheme of the forward quadratures (quad_rhs_tc in recon_solve.cu)
// ---------------------------------------------------------------------------

static constexpr int kTRegs = 8;  // plane inputs a thread keeps in registers (Q <= 128)

// comb(row, col, v) for rows < N and columns col < nx of the contraction of
// table b (row-major [rows][Q] digits: [b][ceil(R/16)][KT][7][32][4], row
// exponents TE[b * R + row]) with the per-column plane inputs in(y, col)
// (Re and Im as two GEMM columns sharing the column exponent)
template <class S, typename In, typename Comb>
__device__ void contract_planes_tc(const Grid& g, const S& gsz, const uint4* __restrict__ T, const int* __restrict__ TE,
                                   int b, int N, int nx, In input, Comb comb, uint16_t* dig, int* exc) {
  const int KT = (gsz.Q() + 15) / 16, MTw = (gsz.R() + 15) / 16;
  const size_t KS = (size_t)KT * 16 + 8;
  for (int i = threadIdx.x; i < kTile; i += blockDim.x) exc[i] = 0;
  __syncthreads();
  if (KT <= kTRegs && blockDim.x == 16 * kTile) {
    const int col = threadIdx.x % kTile, y0 = threadIdx.x / kTile;
    cpx vin[kTRegs];
    int emax = 0;
#pragma unroll
    for (int k = 0; k < kTRegs; ++k) {
      const int y = y0 + 16 * k;
      vin[k] = (k < KT && y < gsz.Q() && col < nx) ? input(y, col) : cpx{0.0, 0.0};
      emax = max(emax, max((int)((__double_as_longlong(vin[k].re) >> 52) & 0x7FF),
                           (int)((__double_as_longlong(vin[k].im) >> 52) & 0x7FF)));
    }
    if (emax) atomicMax(&exc[col], emax);
    __syncthreads();
    const int ex = exc[col] - 1022;
#pragma unroll
    for (int k = 0; k < kTRegs; ++k) {
      if (k >= KT) break;
      const int y = y0 + 16 * k;
      digits_bf16(scaled56(vin[k].re, ex), dig + (size_t)(2 * col) * KS + y, 32 * KS);
      digits_bf16(scaled56(vin[k].im, ex), dig + (size_t)(2 * col + 1) * KS + y, 32 * KS);
    }
  } else {
    for (int i = threadIdx.x; i < gsz.Q() * kTile; i += blockDim.x) {
      const int y = i / kTile, col = i - y * kTile;
      if (col >= nx) continue;
      const cpx v = input(y, col);
      const int e = max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                        (int)((__double_as_longlong(v.im) >> 52) & 0x7FF));
      if (e) atomicMax(&exc[col], e);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < KT * 16 * kTile; i += blockDim.x) {
      const int y = i / kTile, col = i - y * kTile;
      const cpx v = (y < gsz.Q() && col < nx) ? input(y, col) : cpx{0.0, 0.0};
      const int ex = exc[col] - 1022;
      digits_bf16(scaled56(v.re, ex), dig + (size_t)(2 * col) * KS + y, 32 * KS);
      digits_bf16(scaled56(v.im, ex), dig + (size_t)(2 * col + 1) * KS + y, 32 * KS);
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  const int NT = (2 * nx + 7) / 8, MTn = (N + 15) / 16;
  for (int item = warp; item < MTn * NT; item += blockDim.x >> 5) {
    const int mt = item / NT, nt = item - mt * NT;
    const int col = nt * 4 + t, n = nt * 8 + gq;
    const int ecol = exc[min(col, kTile - 1)] - 1022;
    long long Hh[4], Ll[4];
    tc_tile(T + (size_t)b * MTw * KT * kDig * 32, mt, KT, dig, KS, (size_t)32 * KS, n, lane, t, Hh, Ll);
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int row = mt * 16 + gq + 8 * rr;
      if (row >= N || col >= nx) continue;
      const int e = TE[(size_t)b * gsz.R() + row] + ecol - 64;
      const cpx val = {round_col(Hh[2 * rr], Ll[2 * rr], e, ecol + 1022),
                       round_col(Hh[2 * rr + 1], Ll[2 * rr + 1], e, ecol + 1022)};
      comb(row, col, val);
    }
  }
  __syncthreads();
}

// Recon^T (as recon_T_tile) with its five contractions on the tensor cores
// (the mean column, col < xfirst, gets zeros: it has its own rows)
template <class S>
__device__ void recon_T_tc(const Grid& g, const S& gsz, const cpx* __restrict__ Ub, int z, int x0, int nx, int xfirst,
                           SolveTSmem& s) {
  const size_t cs = (size_t)gsz.Q() * gsz.X();
  const cpx* Uz = Ub + (size_t)z * 5 * cs;
  uint16_t* dig = reinterpret_cast<uint16_t*>(s.hc);
  int* exc = reinterpret_cast<int*>(dig + (size_t)kDig * 32 * ((size_t)(gsz.Q() + 15) / 16 * 16 + 8));
  const uint4* T = reinterpret_cast<const uint4*>(g.tcBT);
  auto at = [&](int c, int y, int col) { return Uz[(size_t)c * cs + (size_t)y * gsz.X() + x0 + col]; };
  auto axz = [&](int col, double& ax, double& az) {
    ax = g.kxK2[(size_t)z * gsz.X() + x0 + col];
    az = g.kzK2[(size_t)z * gsz.X() + x0 + col];
  };
  // alpha_bar = Q^T v_bar - Q'^T Xp_bar + Q''^T dx_bar -> s.Fa
  contract_planes_tc(
      g, gsz, T, g.tcBTE, 0, gsz.D(), nx,
      [&](int y, int col) { return col < xfirst ? cpx{0.0, 0.0} : at(1, y, col); },
      [&](int row, int col, cpx v) { s.Fa[row * kTile + col] = v; }, dig, exc);
  contract_planes_tc(
      g, gsz, T, g.tcBTE, 1, gsz.D(), nx,
      [&](int y, int col) {
        if (col < xfirst) return cpx{0.0, 0.0};
        double ax, az;
        axz(col, ax, az);
        const cpx u = at(0, y, col), w = at(2, y, col);
        return cpx{-fma(ax, u.im, az * w.im), fma(ax, u.re, az * w.re)};  // Xp_bar = i(ax u + az w)
      },
      [&](int row, int col, cpx v) {
        cpx& f = s.Fa[row * kTile + col];
        f.re -= v.re;
        f.im -= v.im;
      },
      dig, exc);
  contract_planes_tc(
      g, gsz, T, g.tcBTE, 2, gsz.D(), nx,
      [&](int y, int col) {
        if (col < xfirst) return cpx{0.0, 0.0};
        double ax, az;
        axz(col, ax, az);
        const cpx du = at(3, y, col), dw = at(4, y, col);
        return cpx{fma(ax, du.im, az * dw.im), -fma(ax, du.re, az * dw.re)};  // dx_bar = -i(ax du + az dw)
      },
      [&](int row, int col, cpx v) {
        cpx& f = s.Fa[row * kTile + col];
        f.re += v.re;
        f.im += v.im;
      },
      dig, exc);
  // beta_bar = R^T Zp_bar + R'^T dz_bar -> s.Fb
  contract_planes_tc(
      g, gsz, T, g.tcBTE, 3, gsz.R(), nx,
      [&](int y, int col) {
        if (col < xfirst) return cpx{0.0, 0.0};
        double ax, az;
        axz(col, ax, az);
        const cpx u = at(0, y, col), w = at(2, y, col);
        return cpx{fma(ax, w.im, -az * u.im), fma(az, u.re, -ax * w.re)};  // Zp_bar = i(az u - ax w)
      },
      [&](int row, int col, cpx v) { s.Fb[row * kTile + col] = v; }, dig, exc);
  contract_planes_tc(
      g, gsz, T, g.tcBTE, 4, gsz.R(), nx,
      [&](int y, int col) {
        if (col < xfirst) return cpx{0.0, 0.0};
        double ax, az;
        axz(col, ax, az);
        const cpx du = at(3, y, col), dw = at(4, y, col);
        return cpx{fma(ax, dw.im, -az * du.im), fma(az, du.re, -ax * dw.re)};  // dz_bar = i(az du - ax dw)
      },
      [&](int row, int col, cpx v) {
        cpx& f = s.Fb[row * kTile + col];
        f.re += v.re;
        f.im += v.im;
      },
      dig, exc);
}

// Recon^T of the mean mode, row i (transpose of channel/initAlphaBeta2.c:25-68):
// a_bar = R^T u_bar + R'^T du_bar, b_bar = R^T w_bar + R'^T dw_bar
__device__ __forceinline__ void recon_T_mean_row(const Grid& g, const cpx* __restrict__ Ub, int i, cpx& a, cpx& b) {
  const size_t cs = (size_t)g.Q * g.X;
  double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
  for (int y = 0; y < g.Q; ++y) {
    const double r = __ldg(g.Br + (size_t)y * g.R + i), rp = __ldg(g.Brp + (size_t)y * g.R + i);
    const cpx u = Ub[0 * cs + (size_t)y * g.X], w = Ub[2 * cs + (size_t)y * g.X];
    const cpx du = Ub[3 * cs + (size_t)y * g.X], dw = Ub[4 * cs + (size_t)y * g.X];
    ar = fma(r, u.re, fma(rp, du.re, ar));
    ai = fma(r, u.im, fma(rp, du.im, ai));
    br = fma(r, w.re, fma(rp, dw.re, br));
    bi = fma(r, w.im, fma(rp, dw.im, bi));
  }
  a = cpx{ar, ai};
  b = cpx{br, bi};
}

// H_bar = Quad^T(F_bar) on the tensor cores for the columns [xfirst, nx):
// per plane y the contractions over the modes pa = Qpw^T Fa, qa = Qw^T Fa,
// rb = Rw^T Fb as GEMMs (rows: planes), then the combination of the FP64
// loop in k_solve_T (the mean column keeps that loop)
template <class S>
__device__ void quad_T_tc(const Grid& g, const S& gsz, int z, int x0, int nx, int xfirst, SolveTSmem& s, cpx* __restrict__ Hb) {
  const int KTr = (gsz.R() + 15) / 16, MTq = (gsz.Q() + 15) / 16;
  const size_t KS = (size_t)KTr * 16 + 8;
  uint16_t* dA = reinterpret_cast<uint16_t*>(s.hc);             // [7][32][KS] digits of Fa
  uint16_t* dB = dA + (size_t)kDig * 32 * KS;                    // digits of Fb
  int* exa = reinterpret_cast<int*>(dB + (size_t)kDig * 32 * KS);  // [2][kTile] column exponents
  for (int i = threadIdx.x; i < 2 * kTile; i += blockDim.x) exa[i] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < (gsz.D() + gsz.R()) * kTile; i += blockDim.x) {
    const bool fb = i >= gsz.D() * kTile;
    const int j = fb ? i - gsz.D() * kTile : i, row = j / kTile, col = j - row * kTile;
    if (col >= nx || col < xfirst) continue;
    const cpx v = (fb ? s.Fb : s.Fa)[row * kTile + col];
    const int e = max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                      (int)((__double_as_longlong(v.im) >> 52) & 0x7FF));
    if (e) atomicMax(&exa[(fb ? kTile : 0) + col], e);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * KTr * 16 * kTile; i += blockDim.x) {
    const bool fb = i >= KTr * 16 * kTile;
    const int j = fb ? i - KTr * 16 * kTile : i, row = j / kTile, col = j - row * kTile;
    const int N = fb ? gsz.R() : gsz.D();
    const cpx v = (row < N && col < nx && col >= xfirst) ? (fb ? s.Fb : s.Fa)[row * kTile + col] : cpx{0.0, 0.0};
    const int ex = exa[(fb ? kTile : 0) + col] - 1022;
    uint16_t* d = fb ? dB : dA;
    digits_bf16(scaled56(v.re, ex), d + (size_t)(2 * col) * KS + row, 32 * KS);
    digits_bf16(scaled56(v.im, ex), d + (size_t)(2 * col + 1) * KS + row, 32 * KS);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  const int NT = (2 * nx + 7) / 8;
  const uint4* __restrict__ W = reinterpret_cast<const uint4*>(g.tcWT);
  const size_t cs = (size_t)gsz.Q() * gsz.X();
  const double kz = g.Kz[z];
  for (int item = warp; item < MTq * NT; item += blockDim.x >> 5) {
    const int mt = item / NT, nt = item - mt * NT;
    const int col = nt * 4 + t, n = nt * 8 + gq;
    double v[3][4];  // pa, qa, rb at (rows gq, gq + 8) x (Re, Im)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const uint16_t* d = b < 2 ? dA : dB;
      const int ecol = exa[(b < 2 ? 0 : kTile) + min(col, kTile - 1)] - 1022;
      long long Hh[4], Ll[4];
      tc_tile(W + (size_t)b * MTq * KTr * kDig * 32, mt, KTr, d, KS, (size_t)32 * KS, n, lane, t, Hh, Ll);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int y = min(mt * 16 + gq + 8 * (r >> 1), gsz.Q() - 1);
        v[b][r] = round_col(Hh[r], Ll[r], g.tcWTE[(size_t)b * gsz.Q() + y] + ecol - 64, ecol + 1022);
      }
    }
#pragma unroll
    for (int rr = 0; rr < 2; ++rr) {
      const int y = mt * 16 + gq + 8 * rr;
      if (y >= gsz.Q() || col >= nx || col < xfirst) continue;
      const int x = x0 + col;
      const double kx = g.Kx[x], k2 = g.K2[(size_t)z * gsz.X() + x];
      const double scl = x == 0 ? g.norm : 0.5 * g.norm;
      const cpx pa = {v[0][2 * rr], v[0][2 * rr + 1]}, qa = {v[1][2 * rr], v[1][2 * rr + 1]};
      const cpx rb = {v[2][2 * rr], v[2][2 * rr + 1]};
      cpx hx, hy, hz;
      hx.re = scl * (kx * pa.im + kz * rb.im);  // -i kx pa - i kz rb
      hx.im = -scl * (kx * pa.re + kz * rb.re);
      hz.re = scl * (kz * pa.im - kx * rb.im);  // -i kz pa + i kx rb
      hz.im = scl * (kx * rb.re - kz * pa.re);
      hy.re = -scl * k2 * qa.re;
      hy.im = -scl * k2 * qa.im;
      cpx* out = Hb + ((size_t)z * 5 * gsz.Q() + y) * gsz.X() + x;
      out[0] = hz;
      out[cs] = hx;
      out[2 * cs] = hy;
    }
  }
}

// S: the sizes (SizesRT, or SizesCT for a specialised grid)
template <bool MULTI, class S>
__global__ void __launch_bounds__(kThreads, 2) k_solve_T(const __grid_constant__ Grid g0, SolveTArgs a) {
  const int ntx = (g0.X + kTile - 1) / kTile;
  const int z = blockIdx.x / ntx, tx = blockIdx.x - z * ntx;
  const int inst = blockIdx.y;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const S gsz(g);
  if (z >= gsz.Nz() || tx * kTile >= gsz.X()) return;
  if (blocked_t(a.status, a.sdiv, inst)) return;
  const int x0 = tx * kTile;
  const int nx = min(kTile, gsz.X() - x0);
  cpx* __restrict__ Cc = a.Cc.at(inst);
  auto cidx = [&](int v, int r, int x) { return (((size_t)z * 2 + v) * gsz.R() + r) * gsz.X() + x; };
  if (z == gsz.Nz() / 2) {
    // the tangent zeroes this line every substage (channel/channel.c:460-467)
    if (!a.final_only)
      for (int i = threadIdx.x; i < 2 * gsz.R() * nx; i += blockDim.x) {
        const int v = i / (gsz.R() * nx), r = (i / nx) % gsz.R(), x = x0 + i % nx;
        Cc[cidx(v, r, x)] = cpx{0.0, 0.0};
      }
    return;
  }
  extern __shared__ __align__(16) unsigned char smem[];
  SolveTSmem s = carve_solveT(g, smem);
  const cpx* __restrict__ Ub = a.Ub.at(inst);
  const int xfirst = (z == 0 && x0 == 0) ? 1 : 0;
  if (g.tc) recon_T_tc(g, gsz, Ub, z, x0, nx, xfirst, s);
  else recon_T_tile(g, Ub, z, x0, nx, xfirst, s);
  if (a.final_only) {
    // the sweep's start state: IU = Recon(IC), so IC_bar += Recon^T(IU_bar)
    for (int i = threadIdx.x; i < gsz.R() * kTile; i += blockDim.x) {
      const int r = i / kTile, l = i - r * kTile;
      if (l >= nx || l < xfirst) continue;
      const int x = x0 + l;
      if (r < gsz.D()) {
        const cpx f = s.Fa[r * kTile + l];
        Cc[cidx(0, r, x)].re += f.re;
        Cc[cidx(0, r, x)].im += f.im;
      }
      const cpx f = s.Fb[r * kTile + l];
      Cc[cidx(1, r, x)].re += f.re;
      Cc[cidx(1, r, x)].im += f.im;
    }
    if (xfirst == 1)
      for (int i = threadIdx.x; i < gsz.R(); i += blockDim.x) {
        cpx ma, mb;
        recon_T_mean_row(g, Ub, i, ma, mb);
        Cc[cidx(0, i, 0)].re += ma.re;
        Cc[cidx(0, i, 0)].im += ma.im;
        Cc[cidx(1, i, 0)].re += mb.re;
        Cc[cidx(1, i, 0)].im += mb.im;
      }
    return;
  }
  const int k = a.k;
  const double dt = g.dt;
  // forward coefficients c = {1/2, 1/3, 1}, d = {0, -1/6, -2/3}; b[k] is LU index k
  const double ck = k == 0 ? 1. / 2 : (k == 1 ? 1. / 3. : 1.);
  const double dnext = k == 0 ? -1. / 6 : (k == 1 ? -2. / 3 : 0.0);
  const int bidx = k;
  const int aidx_next = (k == 0) ? 1 : 0;  // a[1] = -1/2, a[2] = 1/3
  // x_bar = Recon^T part + E_{k+1}^T c_out_bar (or c_out_bar); F_bar = dt d_{k+1} c_out_bar
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += blockDim.x) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx || l < xfirst) continue;
    const int x = x0 + l;
    const size_t zx = (size_t)z * gsz.X() + x;
    cpx xa, xb;
    if (r < gsz.D()) {
      const cpx rec = s.Fa[r * kTile + l];
      const cpx co = Cc[cidx(0, r, x)];
      if (k < 2) {
        const double* E = g.exA + ((size_t)aidx_next * gsz.Nz() * gsz.X() + zx) * gsz.D() * 9;
        xa = band_matvecT_row(E, 9, 4, 4, gsz.D(), Cc + cidx(0, 0, x), gsz.X(), r);
        s.Fa[r * kTile + l] = cpx{dt * dnext * co.re, dt * dnext * co.im};
      } else {
        xa = co;
        s.Fa[r * kTile + l] = cpx{0.0, 0.0};
      }
      xa.re += rec.re;
      xa.im += rec.im;
    } else {
      xa = Cc[cidx(0, r, x)];  // alpha rows >= Ny-4 ride along unchanged
    }
    {
      const cpx rec = s.Fb[r * kTile + l];
      const cpx co = Cc[cidx(1, r, x)];
      if (k < 2) {
        const double* E = g.exB + ((size_t)aidx_next * gsz.Nz() * gsz.X() + zx) * gsz.R() * 5;
        xb = band_matvecT_row(E, 5, 2, 2, gsz.R(), Cc + cidx(1, 0, x), gsz.X(), r);
        s.Fb[r * kTile + l] = cpx{dt * dnext * co.re, dt * dnext * co.im};
      } else {
        xb = co;
        s.Fb[r * kTile + l] = cpx{0.0, 0.0};
      }
      xb.re += rec.re;
      xb.im += rec.im;
    }
    s.ra[r * kTile + l] = xa;
    s.rb[r * kTile + l] = xb;
  }
  __syncthreads();
  // L^{-T}: per column 4 chains for alpha, 4 for beta (parity x re/im)
  if (threadIdx.x < 8 * kTile) {
    // threads [0, 4 kTile) run the alpha chains, [4 kTile, 8 kTile) the beta
    // ones: a warp holds one system (no divergence between the two bands)
    const int l = (threadIdx.x % (4 * kTile)) / 4, ch = 4 * (threadIdx.x / (4 * kTile)) + threadIdx.x % 4;
    if (l < nx && l >= xfirst) {
      const size_t zx = (size_t)z * gsz.X() + x0 + l;
      const int par = ch & 1, part = (ch >> 1) & 1;
      if (ch < 4)
        band_solveT_chain<9, 4, 4>(g.luA + ((size_t)bidx * gsz.Nz() * gsz.X() + zx) * gsz.D() * 9,
                                   g.rdA + ((size_t)bidx * gsz.Nz() * gsz.X() + zx) * gsz.D(), gsz.D(), par,
                                   reinterpret_cast<double*>(s.ra + l) + part, 2 * kTile);
      else
        band_solveT_chain<5, 2, 2>(g.luB + ((size_t)bidx * gsz.Nz() * gsz.X() + zx) * gsz.R() * 5,
                                   g.rdB + ((size_t)bidx * gsz.Nz() * gsz.X() + zx) * gsz.R(), gsz.R(), par,
                                   reinterpret_cast<double*>(s.rb + l) + part, 2 * kTile);
    }
  }
  __syncthreads();
  // dJ/dRe: <c2_bar, f_Re> of this block's columns (the forcing of
  // recon_solve.cu's kind 3 rebuilt from the stored primal states)
  const bool want_g = a.gacc != nullptr;
  const cpx* xk = nullptr;
  double ft1 = 0.0, gpart = 0.0;
  const double re2 = g.re * g.re;
  const double akf = k == 1 ? -1. / 2 : 1. / 3.;                  // forward a_k
  const double bkf = k == 0 ? 1. / 6 : (k == 1 ? 2. / 3 : 0.0);  // forward b_k
  if (want_g) {
    const int xs = a.xslot.slot();
    xk = a.Xf + (long long)inst * a.xstride + (long long)xs * a.xslot.stride;
    if (a.Ftr) ft1 = a.Ftr[(long long)inst * a.ftr_stride + xs + 1];
    const size_t csz = coef_size(g);
    for (int i = threadIdx.x; i < gsz.R() * kTile; i += blockDim.x) {
      const int r = i / kTile, l = i - r * kTile;
      if (l >= nx || l < xfirst) continue;
      const int x = x0 + l;
      const double k2 = g.K2[(size_t)z * gsz.X() + x];
      if (r < gsz.D()) {
        const cpx d0 = visc_v_row(g, k2, xk + cidx(0, 0, x), gsz.X(), r);
        const cpx d1 = visc_v_row(g, k2, xk + csz + cidx(0, 0, x), gsz.X(), r);
        const cpx c2 = s.ra[r * kTile + l];
        gpart -= re2 * dt * (c2.re * (akf * d0.re + bkf * d1.re) + c2.im * (akf * d0.im + bkf * d1.im));
      }
      const cpx d0 = visc_g_row(g, k2, xk + cidx(1, 0, x), gsz.X(), r);
      const cpx d1 = visc_g_row(g, k2, xk + csz + cidx(1, 0, x), gsz.X(), r);
      const cpx c2 = s.rb[r * kTile + l];
      gpart += re2 * dt * (c2.re * (akf * d0.re + bkf * d1.re) + c2.im * (akf * d0.im + bkf * d1.im));
    }
  }
  // F_bar += dt c_k c2_bar; c_in_bar = E_0^T c2_bar (k == 0) or c2_bar
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += blockDim.x) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx || l < xfirst) continue;
    const int x = x0 + l;
    const size_t zx = (size_t)z * gsz.X() + x;
    if (r < gsz.D()) {
      const cpx c2 = s.ra[r * kTile + l];
      s.Fa[r * kTile + l].re += dt * ck * c2.re;
      s.Fa[r * kTile + l].im += dt * ck * c2.im;
      Cc[cidx(0, r, x)] = k == 0 ? band_matvecT_row(g.exA + zx * gsz.D() * 9, 9, 4, 4, gsz.D(), s.ra + l, kTile, r) : c2;
    } else {
      Cc[cidx(0, r, x)] = s.ra[r * kTile + l];
    }
    const cpx c2 = s.rb[r * kTile + l];
    s.Fb[r * kTile + l].re += dt * ck * c2.re;
    s.Fb[r * kTile + l].im += dt * ck * c2.im;
    Cc[cidx(1, r, x)] = k == 0 ? band_matvecT_row(g.exB + zx * gsz.R() * 5, 5, 2, 2, gsz.R(), s.rb + l, kTile, r) : c2;
  }
  // mean mode (transpose of channel/increproject0.c with the homogeneous
  // flux correction), warp 0
  if (xfirst == 1 && threadIdx.x < 32) {
    double* fa = s.m0;
    double* fb = s.m0 + gsz.R();
    cpx* ca = reinterpret_cast<cpx*>(s.m0 + 2 * gsz.R());
    cpx* cb = ca + gsz.R();
    const int lane = threadIdx.x;
    const double* Enext = g.ex0 + (size_t)aidx_next * gsz.R() * 5;
    for (int i = lane; i < gsz.R(); i += 32) {
      cpx ma, mb;
      recon_T_mean_row(g, Ub, i, ma, mb);
      const cpx coa = Cc[cidx(0, i, 0)], cob = Cc[cidx(1, i, 0)];
      cpx xa, xb;
      if (k < 2) {
        xa = band_matvecT_row(Enext, 5, 2, 2, gsz.R(), Cc + cidx(0, 0, 0), gsz.X(), i);
        xb = band_matvecT_row(Enext, 5, 2, 2, gsz.R(), Cc + cidx(1, 0, 0), gsz.X(), i);
        fa[i] = dt * dnext * coa.re;  // the mean right-hand side is real
        fb[i] = dt * dnext * cob.re;
      } else {
        xa = coa;
        xb = cob;
        fa[i] = 0.0;
        fb[i] = 0.0;
      }
      ca[i] = cpx{xa.re + ma.re, xa.im + ma.im};
      cb[i] = cpx{xb.re + mb.re, xb.im + mb.im};
    }
    __syncwarp();
    // flux correction x = xs - 0.5 add (rwsum . xs.re), transposed:
    // xs_bar.re = x_bar.re - 0.5 rwsum (add . x_bar.re)
    double part = 0.0;
    for (int i = lane; i < gsz.R(); i += 32) part = fma(g.add0[i], ca[i].re, part);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    // the forced tangent adds 0.5 * 2.0 * add to this line's real part
    // (channel/increproject0.c:209-214): its cotangent is <add, x_bar.re>
    if (want_g && lane == 0) a.gacc[(long long)inst * a.gstride] += part;
    __syncwarp();
    for (int i = lane; i < gsz.R(); i += 32) ca[i].re = fma(-0.5 * part, g.rwsum[i], ca[i].re);
    __syncwarp();
    if (lane < 8) {
      const int par = lane & 1, pt = (lane >> 1) & 1;
      band_solveT_chain<5, 2, 2>(g.lu0 + (size_t)bidx * gsz.R() * 5, g.rd0 + (size_t)bidx * gsz.R(), gsz.R(), par,
                                 reinterpret_cast<double*>(lane < 4 ? ca : cb) + pt, 2);
    }
    __syncwarp();
    if (want_g) {
      // the mean lines' Re forcing: D0 = -Rps on the primal's solved mean flow
      // before its flux correction, MC[3n + k + 1] - 0.5 flux_t add
      const size_t csz = coef_size(g);
      double mp = 0.0;
      for (int i = lane; i < gsz.R(); i += 32) {
        const cpx p0 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + cidx(0, 0, 0), gsz.X(), i);
        cpx p1 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + csz + cidx(0, 0, 0), gsz.X(), i);
        p1.re -= 0.5 * ft1 * rps_row_real(g, g.add0, i);
        const cpx q0 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + cidx(1, 0, 0), gsz.X(), i);
        const cpx q1 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + csz + cidx(1, 0, 0), gsz.X(), i);
        mp += re2 * dt * (ca[i].re * (akf * p0.re + bkf * p1.re) + ca[i].im * (akf * p0.im + bkf * p1.im));
        mp += re2 * dt * (cb[i].re * (akf * q0.re + bkf * q1.re) + cb[i].im * (akf * q0.im + bkf * q1.im));
      }
      gpart += mp;  // lane partials; the block reduction below adds every thread's
    }
    for (int i = lane; i < gsz.R(); i += 32) {
      fa[i] = fma(dt * ck, ca[i].re, fa[i]);
      fb[i] = fma(dt * ck, cb[i].re, fb[i]);
      if (k == 0) {
        Cc[cidx(0, i, 0)] = band_matvecT_row(g.ex0, 5, 2, 2, gsz.R(), ca, 1, i);
        Cc[cidx(1, i, 0)] = band_matvecT_row(g.ex0, 5, 2, 2, gsz.R(), cb, 1, i);
      } else {
        Cc[cidx(0, i, 0)] = ca[i];
        Cc[cidx(1, i, 0)] = cb[i];
      }
    }
  }
  __syncthreads();
  if (want_g) {
    // deterministic block sum of the Re parts into this block's slot
    __shared__ double gred[kThreads / 32];
    double v = gpart;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) gred[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += gred[w];
      a.gacc[(long long)inst * a.gstride + 1 + blockIdx.x] += t;
    }
  }
  // H_bar = Quad^T(F_bar) (transpose of channel/project.c:97-115, 177-191):
  //   Hx_bar = -i kx Qpw^T Fa_bar - i kz Rw^T Fb_bar
  //   Hz_bar = -i kz Qpw^T Fa_bar + i kx Rw^T Fb_bar,  Hy_bar = -K2 Qw^T Fa_bar
  // mean mode: Hx_bar.re = Rw^T fa_bar, Hz_bar.re = Rw^T fb_bar.  Scaled for
  // the inverse transform that follows: the forward transform's 1/(px pz),
  // halved off the kx = 0 column (the transpose of the real-to-complex x
  // transform).  Plane pairs (y, -y) share the sums: weights of even type
  // (Qw, Rw) give E + O / E - O, of odd type (Qpw) E + O / O - E.
  if (g.tc) quad_T_tc(g, gsz, z, x0, nx, xfirst, s, a.Hb.at(inst));
  const int lx = threadIdx.x % kTile, grp = threadIdx.x / kTile, ngrp = blockDim.x / kTile;
  if (lx >= nx) return;
  if (g.tc && lx >= xfirst) return;  // the tensor cores took every column but the mean one
  const int x = x0 + lx;
  const bool mean = (z == 0 && x == 0);
  const double kx = g.Kx[x], kz = g.Kz[z], k2 = g.K2[(size_t)z * gsz.X() + x];
  const double scl = x == 0 ? g.norm : 0.5 * g.norm;
  cpx* __restrict__ Hb = a.Hb.at(inst);
  const size_t cs = (size_t)gsz.Q() * gsz.X();
  for (int yp = grp; yp < gsz.Qh(); yp += ngrp) {
    const int y1 = yp, y2 = gsz.Q() - 1 - yp;
    // E/O sums over even/odd rows: [0] Qpw^T Fa, [1] Qw^T Fa, [2] Rw^T Fb
    double er[3] = {0, 0, 0}, ei[3] = {0, 0, 0}, orr[3] = {0, 0, 0}, oi[3] = {0, 0, 0};
    if (!mean) {
      int i = 0;
      for (; i + 1 < gsz.D(); i += 2) {
        const cpx f0 = s.Fa[i * kTile + lx], f1 = s.Fa[(i + 1) * kTile + lx];
        cfma_t(__ldg(g.Wqp + (size_t)i * gsz.Q() + yp), f0, er[0], ei[0]);
        cfma_t(__ldg(g.Wqp + (size_t)(i + 1) * gsz.Q() + yp), f1, orr[0], oi[0]);
        cfma_t(__ldg(g.Wq + (size_t)i * gsz.Q() + yp), f0, er[1], ei[1]);
        cfma_t(__ldg(g.Wq + (size_t)(i + 1) * gsz.Q() + yp), f1, orr[1], oi[1]);
      }
      if (i < gsz.D()) {
        const cpx f0 = s.Fa[i * kTile + lx];
        cfma_t(__ldg(g.Wqp + (size_t)i * gsz.Q() + yp), f0, er[0], ei[0]);
        cfma_t(__ldg(g.Wq + (size_t)i * gsz.Q() + yp), f0, er[1], ei[1]);
      }
      i = 0;
      for (; i + 1 < gsz.R(); i += 2) {
        const cpx f0 = s.Fb[i * kTile + lx], f1 = s.Fb[(i + 1) * kTile + lx];
        cfma_t(__ldg(g.Wr + (size_t)i * gsz.Q() + yp), f0, er[2], ei[2]);
        cfma_t(__ldg(g.Wr + (size_t)(i + 1) * gsz.Q() + yp), f1, orr[2], oi[2]);
      }
      if (i < gsz.R()) cfma_t(__ldg(g.Wr + (size_t)i * gsz.Q() + yp), s.Fb[i * kTile + lx], er[2], ei[2]);
    } else {
      const double* fa = s.m0;
      const double* fb = s.m0 + gsz.R();
      // [0] Rw^T fa, [2] Rw^T fb (real)
      for (int i = 0; i < gsz.R(); ++i) {
        const double w = __ldg(g.Wr + (size_t)i * gsz.Q() + yp);
        if (i & 1) {
          orr[0] = fma(w, fa[i], orr[0]);
          orr[2] = fma(w, fb[i], orr[2]);
        } else {
          er[0] = fma(w, fa[i], er[0]);
          er[2] = fma(w, fb[i], er[2]);
        }
      }
    }
    for (int side = 0; side < 2; ++side) {
      if (side == 1 && y2 == y1) break;
      const int y = side ? y2 : y1;
      auto val = [&](int c, bool odd_basis) {
        cpx r;
        if (!side) { r.re = er[c] + orr[c]; r.im = ei[c] + oi[c]; }
        else if (!odd_basis) { r.re = er[c] - orr[c]; r.im = ei[c] - oi[c]; }
        else { r.re = orr[c] - er[c]; r.im = oi[c] - ei[c]; }
        return r;
      };
      cpx hx, hy, hz;
      if (mean) {
        hx = cpx{val(0, false).re * scl, 0.0};
        hz = cpx{val(2, false).re * scl, 0.0};
        hy = cpx{0.0, 0.0};
      } else {
        const cpx pa = val(0, true), qa = val(1, false), rb = val(2, false);
        hx.re = scl * (kx * pa.im + kz * rb.im);    // -i kx pa - i kz rb
        hx.im = -scl * (kx * pa.re + kz * rb.re);
        hz.re = scl * (kz * pa.im - kx * rb.im);    // -i kz pa + i kx rb
        hz.im = scl * (kx * rb.re - kz * pa.re);
        hy.re = -scl * k2 * qa.re;
        hy.im = -scl * k2 * qa.im;
      }
      cpx* out = Hb + ((size_t)z * 5 * gsz.Q() + y) * gsz.X() + x;
      out[0] = hz;
      out[cs] = hx;
      out[2 * cs] = hy;
    }
  }
}

// Ca[i] += src[i] over each instance's coefficient array (the per-step
// source of a time-summed objective)
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_add_source(const __grid_constant__ Grid g0, Batch<const cpx> src,
                                                         Batch<cpx> ca, const Grid* grids) {
  const int inst = blockIdx.y;
  CHN_INSTANCE_GRID(g0, grids, inst);
  const size_t n = coef_size(g);
  const cpx* __restrict__ s = src.at(inst);
  cpx* __restrict__ c = ca.at(inst);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    c[i].re += s[i].re;
    c[i].im += s[i].im;
  }
}

cudaError_t launch_add_source(const Grid& g, Batch<const cpx> src, Batch<cpx> ca, int ninst, cudaStream_t st,
                              const Grid* grids) {
  if (ninst <= 0) return cudaSuccess;
  const size_t n = coef_size(g);
  int blocks = (int)((n + kThreads - 1) / kThreads);
  if (blocks > 152 * 4) blocks = 152 * 4;
  if (grids) k_add_source<true><<<dim3(blocks, ninst), kThreads, 0, st>>>(g, src, ca, grids);
  else k_add_source<false><<<dim3(blocks, ninst), kThreads, 0, st>>>(g, src, ca, grids);
  return cudaGetLastError();
}

cudaError_t launch_solve_T(const Grid& g, const SolveTArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  const int ntx = (g.X + kTile - 1) / kTile;
  const size_t sm = solveT_smem_bytes(g);
  const bool fx = (g.fixed & FIXED_SOLVE) && !a.grids;  // the solve's fixed-size choice covers its transpose
  if (a.grids) k_solve_T<true, SizesRT><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
  else if (fx && sizes_match<Sizes32>(g)) k_solve_T<false, Sizes32><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
  else if (fx && sizes_match<Sizes16>(g)) k_solve_T<false, Sizes16><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
  else k_solve_T<false, SizesRT><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
  return cudaGetLastError();
}

void prepare_solve_T(int optin) {
  allow_max_smem(k_solve_T<false, SizesRT>, optin);
  allow_max_smem(k_solve_T<true, SizesRT>, optin);
  allow_max_smem(k_solve_T<false, Sizes32>, optin);
  allow_max_smem(k_solve_T<false, Sizes16>, optin);
}

}  // namespace chn
