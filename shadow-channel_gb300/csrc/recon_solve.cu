// Legendre-direction kernels.
//
//   k_recon  coefficients -> velocity at every quadrature plane
//            (channel/initAlphaBeta2.c:12-240, same arithmetic as the
//            reconstruction tail of channel/project.c:231-332)
//   k_solve  one RK3 substage of the implicit Galerkin step for a kz line:
//            quadrature right-hand side, banded solve, trajectory store and
//            next-substage right-hand side (channel/project.c:24-405,
//            project0.c:22-271, increproject*.c, adjproject*.c)
//
// Both exploit the parity of the Legendre bases on the symmetric Gauss
// points: Q_n, Q_n'', R_n are even/odd as (-1)^n and Q_n', R_n' as
// (-1)^(n+1), so for the plane pair (y, -y) a contraction splits into an
// even-index sum E and an odd-index sum O with values E +- O.  This halves
// the FP64 multiply-adds of every quadrature and reconstruction.
#include "chn_common.cuh"
#include "kernels.h"
#include "solve_common.cuh"
#include "sizes.cuh"
#include "tc_common.cuh"

namespace chn {

static constexpr int kThreads = 256;
static constexpr int kTile = 16;   // kx columns per block
static constexpr int kQuadRegs = 8;  // quadrature inputs a thread keeps in registers (Q <= 128)

__device__ __forceinline__ bool blocked(const uint32_t* status, int sdiv, int inst) {
  return status != nullptr && (status[inst / sdiv] & ST_CFL) != 0;
}

__device__ __forceinline__ void cfma(double w, const cpx& a, double& re, double& im) {
  re = fma(w, a.re, re);
  im = fma(w, a.im, im);
}

// ---------------------------------------------------------------------------
// reconstruction
// ---------------------------------------------------------------------------

template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_recon(const __grid_constant__ Grid g0, ReconArgs a) {
  const int ntx = (g0.X + kTile - 1) / kTile;
  const int z = blockIdx.x / ntx, tx = blockIdx.x - z * ntx;
  const int inst = blockIdx.y;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (z >= g.Nz || tx * kTile >= g.X) return;
  if (z == g.Nz / 2) return;  // never read (channel/pass1.c:51-85 skips it)
  if (blocked(a.status, a.sdiv, inst)) return;
  const int x0 = tx * kTile;
  const int nx = min(kTile, g.X - x0);
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* cs = reinterpret_cast<cpx*>(smem);  // [2][R][kTile]
  const cpx* __restrict__ C = a.C.at(inst);
  if (a.slot.stride) C += (long long)a.slot.slot() * a.slot.stride;
  for (int i = threadIdx.x; i < 2 * g.R * kTile; i += blockDim.x) {
    const int v = i / (g.R * kTile), r = (i / kTile) % g.R, x = i % kTile;
    cpx val = {0.0, 0.0};
    if (x < nx) val = C[(((size_t)z * 2 + v) * g.R + r) * g.X + x0 + x];
    cs[i] = val;
  }
  __syncthreads();
  const int lx = threadIdx.x % kTile, grp = threadIdx.x / kTile;
  const int ngrp = blockDim.x / kTile;
  if (lx >= nx) return;
  const int x = x0 + lx;
  cpx* __restrict__ U = a.U.at(inst);
  const cpx* al = cs;                     // alpha_j at al[j*kTile + lx]
  const cpx* be = cs + g.R * kTile;       // beta_j
  const bool mean = (z == 0 && x == 0);
  const double ax = g.kxK2[z * g.X + x], az = g.kzK2[z * g.X + x];
  for (int yp = grp; yp < g.Qh; yp += ngrp) {
    const int y1 = yp, y2 = g.Q - 1 - yp;
    // E/O sums: [0] Q alpha (v), [1] Q' alpha, [2] Q'' alpha, [3] R beta, [4] R' beta
    double er[5] = {0, 0, 0, 0, 0}, ei[5] = {0, 0, 0, 0, 0};
    double orr[5] = {0, 0, 0, 0, 0}, oi[5] = {0, 0, 0, 0, 0};
    if (!mean) {
      const double* bq = g.Bq + (size_t)y1 * g.D;
      const double* bqp = g.Bqp + (size_t)y1 * g.D;
      const double* bqpp = g.Bqpp + (size_t)y1 * g.D;
      int j = 0;
      for (; j + 1 < g.D; j += 2) {
        const cpx c0 = al[j * kTile + lx], c1 = al[(j + 1) * kTile + lx];
        const double q0 = __ldg(bq + j), q1 = __ldg(bq + j + 1);
        const double p0 = __ldg(bqp + j), p1 = __ldg(bqp + j + 1);
        const double s0 = __ldg(bqpp + j), s1 = __ldg(bqpp + j + 1);
        cfma(q0, c0, er[0], ei[0]); cfma(q1, c1, orr[0], oi[0]);
        cfma(p0, c0, er[1], ei[1]); cfma(p1, c1, orr[1], oi[1]);
        cfma(s0, c0, er[2], ei[2]); cfma(s1, c1, orr[2], oi[2]);
      }
      if (j < g.D) {
        const cpx c0 = al[j * kTile + lx];
        cfma(__ldg(bq + j), c0, er[0], ei[0]);
        cfma(__ldg(bqp + j), c0, er[1], ei[1]);
        cfma(__ldg(bqpp + j), c0, er[2], ei[2]);
      }
    }
    {
      const double* br = g.Br + (size_t)y1 * g.R;
      const double* brp = g.Brp + (size_t)y1 * g.R;
      // mean mode: R a and R' a land in slots 1/2 (u, du), R b and R' b in 3/4
      const cpx* src0 = mean ? al : be;
      int j = 0;
      for (; j + 1 < g.R; j += 2) {
        const double r0 = __ldg(br + j), r1 = __ldg(br + j + 1);
        const double p0 = __ldg(brp + j), p1 = __ldg(brp + j + 1);
        const cpx b0 = be[j * kTile + lx], b1 = be[(j + 1) * kTile + lx];
        cfma(r0, b0, er[3], ei[3]); cfma(r1, b1, orr[3], oi[3]);
        cfma(p0, b0, er[4], ei[4]); cfma(p1, b1, orr[4], oi[4]);
        if (mean) {
          const cpx c0 = src0[j * kTile + lx], c1 = src0[(j + 1) * kTile + lx];
          cfma(r0, c0, er[1], ei[1]); cfma(r1, c1, orr[1], oi[1]);
          cfma(p0, c0, er[2], ei[2]); cfma(p1, c1, orr[2], oi[2]);
        }
      }
      if (j < g.R) {
        const double r0 = __ldg(br + j), p0 = __ldg(brp + j);
        const cpx b0 = be[j * kTile + lx];
        cfma(r0, b0, er[3], ei[3]);
        cfma(p0, b0, er[4], ei[4]);
        if (mean) {
          const cpx c0 = src0[j * kTile + lx];
          cfma(r0, c0, er[1], ei[1]);
          cfma(p0, c0, er[2], ei[2]);
        }
      }
    }
    for (int side = 0; side < 2; ++side) {
      if (side == 1 && y2 == y1) break;
      const int y = side ? y2 : y1;
      // even-parity bases: E + O / E - O;  odd-parity (Q', R'): E + O / -(E - O)
      auto val = [&](int c, bool odd_basis) {
        cpx r;
        if (!side) { r.re = er[c] + orr[c]; r.im = ei[c] + oi[c]; }
        else if (!odd_basis) { r.re = er[c] - orr[c]; r.im = ei[c] - oi[c]; }
        else { r.re = orr[c] - er[c]; r.im = oi[c] - ei[c]; }
        return r;
      };
      cpx u, v, w, du, dw;
      if (mean) {
        // (kx,kz) = (0,0): u = R a, du = R' a, v = 0, w = R b, dw = R' b
        u = val(1, false); du = val(2, true); w = val(3, false); dw = val(4, true);
        v.re = 0.0; v.im = 0.0;
      } else {
        v = val(0, false);
        const cpx qp = val(1, true);          // Q' alpha, f = -Q' alpha
        const cpx qpp = val(2, false);
        const cpx g_ = val(3, false);         // g = R beta
        const cpx rp = val(4, true);
        const cpx f = {-qp.re, -qp.im};
        // u = (kx Im f + kz Im g)/K2 - i (kx Re f + kz Re g)/K2, etc.
        u.re = fma(ax, f.im, az * g_.im);
        u.im = -fma(ax, f.re, az * g_.re);
        w.re = fma(-ax, g_.im, az * f.im);
        w.im = fma(ax, g_.re, -az * f.re);
        du.re = fma(-ax, qpp.im, az * rp.im);
        du.im = fma(ax, qpp.re, -az * rp.re);
        dw.re = -fma(ax, rp.im, az * qpp.im);
        dw.im = fma(ax, rp.re, az * qpp.re);
      }
      cpx* out = U + ((size_t)z * 5 * g.Q + y) * g.X + x;
      const size_t cs_ = (size_t)g.Q * g.X;
      out[0] = u;
      out[cs_] = v;
      out[2 * cs_] = w;
      out[3 * cs_] = du;
      out[4 * cs_] = dw;
    }
  }
}

size_t recon_smem_bytes(const Grid& g) { return (size_t)2 * g.R * kTile * sizeof(cpx); }

cudaError_t launch_recon(const Grid& g, const ReconArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.tc) return launch_recon_tc(g, a, st);
  const int ntx = (g.X + kTile - 1) / kTile;
  if (a.grids) k_recon<true><<<dim3(g.Nz * ntx, a.ninst), kThreads, recon_smem_bytes(g), st>>>(g, a);
  else k_recon<false><<<dim3(g.Nz * ntx, a.ninst), kThreads, recon_smem_bytes(g), st>>>(g, a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// implicit solve
// ---------------------------------------------------------------------------

struct RKc {
  double b, c, dnext;
  int bidx, aidx0, aidx_next;
};

__device__ __forceinline__ RKc rk_coeffs(int k, int adjoint) {
  // forward  a = {1/3,-1/2,1/3}, b = {1/6,2/3,0}, c = {1/2,1/3,1}, d = {0,-1/6,-2/3}
  // adjoint  a = {1/3,-1/2,1/3}, b = {2/3,1/6,0}, c = {1,1/3,1/2}, d = {0,-2/3,-1/6}
  RKc r;
  if (!adjoint) {
    r.bidx = k;
    r.c = k == 0 ? 1. / 2 : (k == 1 ? 1. / 3. : 1.);
    r.dnext = k == 0 ? -1. / 6 : (k == 1 ? -2. / 3 : 0.0);
  } else {
    r.bidx = k == 0 ? 1 : (k == 1 ? 0 : 2);
    r.c = k == 0 ? 1. : (k == 1 ? 1. / 3. : 1. / 2.);
    r.dnext = k == 0 ? -2. / 3 : (k == 1 ? -1. / 6 : 0.0);
  }
  r.b = r.bidx == 0 ? 1. / 6 : (r.bidx == 1 ? 2. / 3 : 0.);
  r.aidx0 = 0;                         // a[0] = 1/3
  r.aidx_next = (k == 0) ? 1 : 0;      // a[1] = -1/2, a[2] = 1/3
  return r;
}

struct SolveSmem {
  cpx* hc;    // [Qh][kTile][6] parity-combined inputs (live during a quadrature)
  cpx* ra;    // [R][kTile] alpha right-hand side / solution (aliases hc: live between quadratures)
  cpx* rb;    // [R][kTile]
  cpx* Fa;    // [D][kTile]
  cpx* Fb;    // [R][kTile]
  double* m0; // mean-mode scratch
};

// The solve's functions below take the block's tile width (kx columns per
// block, 16 or 8: the autotuner's choice, Grid::stile) as the template
// parameter kTile, which stands for the file's 16 inside them.

// digits of one quadrature input for the tensor-core quadrature:
// [7][2 kTile columns][KS] bf16 + kTile exponents
__host__ __device__ inline size_t solve_tc_kstride(const Grid& g) { return (size_t)((g.Q + 15) / 16) * 16 + 8; }

// the FP64 quadrature's parity-combined inputs only where it runs (g.tc = 0)
template <int kTile>
__host__ __device__ inline size_t solve_hc_elems(const Grid& g) {
  size_t hc = g.tc ? 0 : (size_t)g.Qh * kTile * 6, r = 2 * (size_t)g.R * kTile;
  const size_t tc =
      ((size_t)kDig * 2 * kTile * solve_tc_kstride(g) * 2 + kTile * sizeof(int) + sizeof(cpx) - 1) / sizeof(cpx);
  if (r > hc) hc = r;
  return tc > hc ? tc : hc;
}

template <int kTile>
size_t solve_smem_bytes_t(const Grid& g) {
  size_t n = solve_hc_elems<kTile>(g) + (size_t)g.D * kTile + (size_t)g.R * kTile;
  return n * sizeof(cpx) + (size_t)8 * g.R * sizeof(double);
}

// the widest tile's (the fit check of a grid)
size_t solve_smem_bytes(const Grid& g) { return solve_smem_bytes_t<16>(g); }

template <int kTile>
__device__ inline SolveSmem carve_solve(const Grid& g, unsigned char* base) {
  SolveSmem s;
  cpx* p = reinterpret_cast<cpx*>(base);
  s.hc = p;
  s.ra = p;
  s.rb = p + (size_t)g.R * kTile;
  p += solve_hc_elems<kTile>(g);
  s.Fa = p; p += (size_t)g.D * kTile;
  s.Fb = p; p += (size_t)g.R * kTile;
  s.m0 = reinterpret_cast<double*>(p);
  return s;
}

// Quadrature right-hand side for columns x0..x0+nx-1 of line z from terms H:
//   Fa = Qpw . i(kx Hx + kz Hz) - K2 Qw . Hy  [+ Qppw . -i(kz Sx - kx Sz)]
//   Fb = Rw . i(kz Hx - kx Hz)                [+ Rpw  .  i(kz Sz + kx Sx)]
// (channel/project.c:97-115, 177-191; channel/adjproject.c:113-134, 218-234)
template <int kTile>
__device__ void quad_rhs(const Grid& g, const cpx* __restrict__ H, int z, int x0, int nx, bool adj,
                         SolveSmem& s) {
  const int lx = threadIdx.x % kTile, grp = threadIdx.x / kTile, ngrp = blockDim.x / kTile;
  const double kz = g.Kz[z];
  const size_t cs = (size_t)g.Q * g.X;
  const cpx* Hz_ = H + (size_t)z * 5 * cs;  // slot c at Hz_ + c*cs + y*X + x
  for (int phase = 0; phase < 2; ++phase) {
    // phase 0: inputs of Fa (P, Hy, Sa); phase 1: inputs of Fb (G, Sb)
    const int nin = phase == 0 ? (adj ? 3 : 2) : (adj ? 2 : 1);
    for (int i = threadIdx.x; i < g.Qh * kTile; i += blockDim.x) {
      const int yp = i / kTile, l = i - yp * kTile;
      cpx* dst = s.hc + (size_t)i * 6;
      if (l >= nx) continue;
      const int x = x0 + l;
      const double kx = g.Kx[x];
      const int ya = yp, yb = g.Q - 1 - yp;
      cpx in[2][3];
      for (int side = 0; side < 2; ++side) {
        const int y = side ? yb : ya;
        const cpx hz = Hz_[0 * cs + (size_t)y * g.X + x];
        const cpx hx = Hz_[1 * cs + (size_t)y * g.X + x];
        if (phase == 0) {
          const cpx hy = Hz_[2 * cs + (size_t)y * g.X + x];
          in[side][0].re = -kx * hx.im - kz * hz.im;   // P = i(kx Hx + kz Hz)
          in[side][0].im = kx * hx.re + kz * hz.re;
          in[side][1] = hy;
          if (adj) {
            const cpx sx = Hz_[3 * cs + (size_t)y * g.X + x], sz = Hz_[4 * cs + (size_t)y * g.X + x];
            in[side][2].re = kz * sx.im - kx * sz.im;  // Sa = -i(kz Sx - kx Sz)
            in[side][2].im = -kz * sx.re + kx * sz.re;
          }
        } else {
          in[side][0].re = -kz * hx.im + kx * hz.im;   // G = i(kz Hx - kx Hz)
          in[side][0].im = kz * hx.re - kx * hz.re;
          if (adj) {
            const cpx sx = Hz_[3 * cs + (size_t)y * g.X + x], sz = Hz_[4 * cs + (size_t)y * g.X + x];
            in[side][1].re = -kz * sz.im - kx * sx.im;  // Sb = i(kz Sz + kx Sx)
            in[side][1].im = kz * sz.re + kx * sx.re;
          }
        }
      }
      for (int q = 0; q < nin; ++q) {
        if (ya == yb) {  // centre plane of an odd point count
          dst[2 * q] = in[0][q];
          dst[2 * q + 1] = in[0][q];
        } else {
          dst[2 * q].re = in[0][q].re + in[1][q].re;      // "+" combination
          dst[2 * q].im = in[0][q].im + in[1][q].im;
          dst[2 * q + 1].re = in[0][q].re - in[1][q].re;  // "-" combination
          dst[2 * q + 1].im = in[0][q].im - in[1][q].im;
        }
      }
    }
    __syncthreads();
    if (lx < nx) {
      const int x = x0 + lx;
      const double k2 = g.K2[z * g.X + x];
      const int N = phase == 0 ? g.D : g.R;
      // rows i = grp, grp + ngrp, ... share the parity of grp (ngrp is even)
      constexpr int MAXR = 4;
      for (int ib = grp; ib < N; ib += ngrp * MAXR) {
        double sr[MAXR][3], si[MAXR][3];
#pragma unroll
        for (int m = 0; m < MAXR; ++m)
#pragma unroll
          for (int q = 0; q < 3; ++q) { sr[m][q] = 0.0; si[m][q] = 0.0; }
        const bool even = (ib & 1) == 0;
        for (int yp = 0; yp < g.Qh; ++yp) {
          const cpx* src = s.hc + ((size_t)yp * kTile + lx) * 6;
          if (phase == 0) {
            // even rows: Qpw (odd basis) pairs with "-", Qw and Qppw with "+"
            const cpx P = src[even ? 1 : 0];
            const cpx Hy = src[even ? 2 : 3];
            const cpx Sa = adj ? src[even ? 4 : 5] : cpx{0.0, 0.0};
#pragma unroll
            for (int m = 0; m < MAXR; ++m) {
              const int i = ib + m * ngrp;
              if (i < N) {
                const size_t o = (size_t)i * g.Q + yp;
                cfma(__ldg(g.Wqp + o), P, sr[m][0], si[m][0]);
                cfma(__ldg(g.Wq + o), Hy, sr[m][1], si[m][1]);
                if (adj) cfma(__ldg(g.Wqpp + o), Sa, sr[m][2], si[m][2]);
              }
            }
          } else {
            // even rows: Rw with "+", Rpw (odd basis) with "-"
            const cpx G = src[even ? 0 : 1];
            const cpx Sb = adj ? src[even ? 3 : 2] : cpx{0.0, 0.0};
#pragma unroll
            for (int m = 0; m < MAXR; ++m) {
              const int i = ib + m * ngrp;
              if (i < N) {
                const size_t o = (size_t)i * g.Q + yp;
                cfma(__ldg(g.Wr + o), G, sr[m][0], si[m][0]);
                if (adj) cfma(__ldg(g.Wrp + o), Sb, sr[m][1], si[m][1]);
              }
            }
          }
        }
#pragma unroll
        for (int m = 0; m < MAXR; ++m) {
          const int i = ib + m * ngrp;
          if (i >= N) continue;
          cpx f;
          if (phase == 0) {
            f.re = fma(-k2, sr[m][1], sr[m][0]) + sr[m][2];
            f.im = fma(-k2, si[m][1], si[m][0]) + si[m][2];
            s.Fa[i * kTile + lx] = f;
          } else {
            f.re = sr[m][0] + sr[m][1];
            f.im = si[m][0] + si[m][1];
            s.Fb[i * kTile + lx] = f;
          }
        }
      }
    }
    __syncthreads();
  }
}

// The same right-hand side on the tensor cores (tc_common.cuh): each input
// vector over the Q planes, per column, as base-256 digits (shared memory
// of the FP64 version's parity-combined inputs), times the digit tables of
// the weighted transposes; one FP64 rounding per contraction.
//   Fa = Qpw P - K2 Qw Hy [+ Qppw Sa],   Fb = Rw G [+ Rpw Sb]
template <int kTile, int NTHR, class S>
__device__ void quad_rhs_tc(const Grid& g, const S& gsz, const cpx* __restrict__ H, int z, int x0, int nx, bool adj,
                            SolveSmem& s) {
  constexpr int NC = 2 * kTile;  // digit columns: Re, Im of each kx column
  const int KT = (gsz.Q() + 15) / 16, MTw = (gsz.R() + 15) / 16;
  const size_t KS = (size_t)((gsz.Q() + 15) / 16) * 16 + 8;  // solve_tc_kstride
  uint16_t* dig = reinterpret_cast<uint16_t*>(s.hc);             // [7][NC][KS]
  int* exc = reinterpret_cast<int*>(dig + (size_t)kDig * NC * KS);  // [kTile]
  const double kz = g.Kz[z];
  const size_t cs = (size_t)gsz.Q() * gsz.X();
  const cpx* Hz_ = H + (size_t)z * 5 * cs;  // slot c at Hz_ + c*cs + y*X + x
  // input q: 0 P = i(kx Hx + kz Hz), 1 Hy, 2 Sa = -i(kz Sx - kx Sz), 3 G = i(kz Hx - kx Hz),
  // 4 Sb = i(kz Sz + kx Sx); weight table: Qpw 1, Qw 0, Qppw 2, Rw 3, Rpw 4
  auto input = [&](int q, int y, int col) -> cpx {
    const int x = x0 + col;
    const double kx = g.Kx[x];
    const cpx* b = Hz_ + (size_t)y * gsz.X() + x;
    switch (q) {
      case 0: { const cpx hx = b[cs], hz = b[0];
                return cpx{-kx * hx.im - kz * hz.im, kx * hx.re + kz * hz.re}; }
      case 1: return b[2 * cs];
      case 2: { const cpx sx = b[3 * cs], sz = b[4 * cs];
                return cpx{kz * sx.im - kx * sz.im, -kz * sx.re + kx * sz.re}; }
      case 3: { const cpx hx = b[cs], hz = b[0];
                return cpx{-kz * hx.im + kx * hz.im, kz * hx.re - kx * hz.re}; }
      default: { const cpx sx = b[3 * cs], sz = b[4 * cs];
                 return cpx{-kz * sz.im - kx * sx.im, kz * sz.re + kx * sx.re}; }
    }
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  const int NT = (2 * nx + 7) / 8;
  const uint4* __restrict__ W = reinterpret_cast<const uint4*>(g.tcW);
  const int qs[5] = {0, 1, 3, 2, 4};
  const int nq = adj ? 5 : 3;
  for (int iq = 0; iq < nq; ++iq) {
    const int q = adj ? iq : qs[iq];
    const int w = q == 0 ? 1 : (q == 1 ? 0 : q);
    const bool toA = q < 3;
    const int N = toA ? gsz.D() : gsz.R();
    cpx* F = toA ? s.Fa : s.Fb;
    const bool first = (q == 0 || q == 3);
    for (int i = threadIdx.x; i < kTile; i += NTHR) exc[i] = 0;
    __syncthreads();
    if (KT <= kQuadRegs && NTHR == 16 * kTile) {
      // thread t holds column t % kTile, planes t / kTile + 16 k (k < KT):
      // its inputs stay in registers from the exponent maximum to the digits
      const int col = threadIdx.x % kTile, y0 = threadIdx.x / kTile;
      cpx vin[kQuadRegs];
      int emax = 0;
#pragma unroll
      for (int k = 0; k < kQuadRegs; ++k) {
        const int y = y0 + 16 * k;
        vin[k] = (k < KT && y < gsz.Q() && col < nx) ? input(q, y, col) : cpx{0.0, 0.0};
        emax = max(emax, max((int)((__double_as_longlong(vin[k].re) >> 52) & 0x7FF),
                             (int)((__double_as_longlong(vin[k].im) >> 52) & 0x7FF)));
      }
      if (emax) atomicMax(&exc[col], emax);
      __syncthreads();
      const int ex = exc[col] - 1022;
#pragma unroll
      for (int k = 0; k < kQuadRegs; ++k) {
        if (k >= KT) break;
        const int y = y0 + 16 * k;
        digits_bf16(scaled56(vin[k].re, ex), dig + (size_t)(2 * col) * KS + y, NC * KS);
        digits_bf16(scaled56(vin[k].im, ex), dig + (size_t)(2 * col + 1) * KS + y, NC * KS);
      }
    } else {
      for (int i = threadIdx.x; i < gsz.Q() * kTile; i += NTHR) {
        const int y = i / kTile, col = i - y * kTile;
        if (col >= nx) continue;
        const cpx v = input(q, y, col);
        const int e = max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                          (int)((__double_as_longlong(v.im) >> 52) & 0x7FF));
        if (e) atomicMax(&exc[col], e);
      }
      __syncthreads();
      for (int i = threadIdx.x; i < KT * 16 * kTile; i += NTHR) {
        const int y = i / kTile, col = i - y * kTile;
        const cpx v = (y < gsz.Q() && col < nx) ? input(q, y, col) : cpx{0.0, 0.0};
        const int ex = exc[col] - 1022;
        digits_bf16(scaled56(v.re, ex), dig + (size_t)(2 * col) * KS + y, NC * KS);
        digits_bf16(scaled56(v.im, ex), dig + (size_t)(2 * col + 1) * KS + y, NC * KS);
      }
    }
    __syncthreads();
    const int MTn = (N + 15) / 16;
    for (int item = warp; item < MTn * NT; item += NTHR >> 5) {
      const int mt = item / NT, nt = item - mt * NT;
      const int col = nt * 4 + t, n = nt * 8 + gq;
      const int ecol = exc[min(col, kTile - 1)] - 1022;
      long long Hh[4], Ll[4];
      tc_tile_pf(W + (size_t)w * MTw * KT * kDig * 32, mt, KT, KT, dig, KS, (size_t)NC * KS, n, lane, t, Hh, Ll);
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        const int row = mt * 16 + gq + 8 * rr;
        if (row >= N || col >= nx) continue;
        const int e = g.tcWE[(size_t)w * gsz.R() + row] + ecol - 64;
        const cpx val = {round_col(Hh[2 * rr], Ll[2 * rr], e, ecol + 1022),
                         round_col(Hh[2 * rr + 1], Ll[2 * rr + 1], e, ecol + 1022)};
        cpx& f = F[row * kTile + col];
        if (first) {
          f = val;
        } else if (q == 1) {
          const double k2 = g.K2[(size_t)z * gsz.X() + x0 + col];
          f.re = fma(-k2, val.re, f.re);
          f.im = fma(-k2, val.im, f.im);
        } else {
          f.re += val.re;
          f.im += val.im;
        }
      }
    }
    __syncthreads();
  }
}


// one elimination chain (fixed parity, real or imaginary part) of the
// no-pivot every-other-diagonal LU solve (channel/mvOps.c:29-91); W, DL, DU
// the band layout (width, lower, upper), RD the reciprocal pivots.  The band
// loops are unrolled with per-row predicates, the multiply-adds in the
// reference's order.
template <int W, int DL, int DU>
__device__ void band_solve_chain(const double* __restrict__ LU, const double* __restrict__ RD, int N, int par,
                                 double* b, int bstride) {
#pragma unroll 4
  for (int i = par; i < N; i += 2) {
    if (i < 2) continue;
    const int j0 = DL - i / 2;
    double acc = b[i * bstride];
#pragma unroll
    for (int j = 0; j < DL; ++j)
      if (j >= j0) acc = fma(-__ldg(LU + (size_t)i * W + j), b[(i - 2 * (DL - j)) * bstride], acc);
    b[i * bstride] = acc;
  }
  // back substitution: the last row of this parity first
  const int ilast = ((N - 1 - par) % 2 == 0) ? N - 1 : N - 2;
#pragma unroll 4
  for (int i = ilast; i >= 0; i -= 2) {
    double acc = b[i * bstride];
    const int jm = min(DU, (N - i + 1) / 2 - 1);  // no terms for i > N - 3
#pragma unroll
    for (int j = 1; j <= DU; ++j)
      if (j <= jm) acc = fma(-__ldg(LU + (size_t)i * W + DL + j), b[(i + 2 * j) * bstride], acc);
    b[i * bstride] = acc * __ldg(RD + i);
  }
}




// S: the sizes (SizesRT, or SizesCT for a specialised grid); NTHR threads
// (256, or 128 with the 8-column tile), MINB blocks per SM
template <bool MULTI, int kTile, class S, int NTHR = kThreads, int MINB = 2>
__global__ void __launch_bounds__(NTHR, MINB) k_solve(const __grid_constant__ Grid g0, SolveArgs a) {
  const int ntx = (g0.X + kTile - 1) / kTile;
  const int z = blockIdx.x / ntx, tx = blockIdx.x - z * ntx;
  const int inst = blockIdx.y;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const S gsz(g);
  if (z >= gsz.Nz() || tx * kTile >= gsz.X()) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  const int x0 = tx * kTile;
  const int nx = min(kTile, gsz.X() - x0);
  const size_t csz = coef_size(g);
  cpx* __restrict__ Cc = a.Cc.at(inst);
  cpx* __restrict__ So = a.Sout.at(inst);
  cpx* Tst = nullptr;
  int tslot = -1;
  if (a.T.base && (inst % a.tdiv) == a.tsel) {
    tslot = a.slot.slot();
    if (tslot >= 0) Tst = a.T.base + (long long)(inst / a.tdiv) * a.T.stride + (long long)tslot * a.slot.stride;
  }
  int mean_mode = a.mean_mode;
  if (mean_mode == MEAN_TAN_HOMOG && ((a.forced_mask >> (inst % a.mdiv)) & 1u)) mean_mode = MEAN_TAN_FORCED;
  auto cidx = [&](int v, int r, int x) { return (((size_t)z * 2 + v) * gsz.R() + r) * gsz.X() + x; };
  if (z == gsz.Nz() / 2) {
    // the Nz/2 line is zeroed every substage and never stored (channel/channel.c:460-467)
    for (int i = threadIdx.x; i < 2 * gsz.R() * nx; i += NTHR) {
      const int v = i / (gsz.R() * nx), r = (i / nx) % gsz.R(), x = x0 + i % nx;
      Cc[cidx(v, r, x)] = cpx{0.0, 0.0};
      So[cidx(v, r, x)] = cpx{0.0, 0.0};
    }
    return;
  }
  extern __shared__ __align__(16) unsigned char smem[];
  SolveSmem s = carve_solve<kTile>(g, smem);
  const RKc rk = rk_coeffs(a.k, a.adjoint);
  const bool adj = a.adjoint != 0;
  const cpx* __restrict__ H = a.H.at(inst);
  if (g.tc) quad_rhs_tc<kTile, NTHR>(g, gsz, H, z, x0, nx, adj, s);
  else quad_rhs<kTile>(g, H, z, x0, nx, adj, s);
  const double dt = g.dt;
  const int xfirst = (z == 0 && x0 == 0) ? 1 : 0;  // the mean mode has its own system
  // Re-sensitivity forcing of this tangent (kind 2: the reference's forcing
  // reconnected, channel/tangent_forcing.c + increproject.c:61-104, at the
  // first substage; kind 3: the exact derivative of the discrete step,
  // -re^2 dt (a_k D x_k + b_k D x_{k+1}) in every substage's right-hand side)
  int fkind = 0;
  const cpx* xk = nullptr;
  double ft1 = 0.0;
  if (a.re2_mask | a.re3_mask) {
    const uint32_t bit = 1u << (inst % a.mdiv);
    fkind = (a.re3_mask & bit) ? 3 : ((a.re2_mask & bit) ? 2 : 0);
    if (fkind) {
      const int xs = a.xslot.slot();
      xk = a.Xf.at(inst / a.xdiv) + (long long)xs * a.xslot.stride;
      if (a.Ftr) ft1 = a.Ftr[(long long)(inst / a.xdiv) * a.ftr_stride + xs + 1];
    }
  }
  const double re2 = g.re * g.re;
  const double ak = a.k == 1 ? -1. / 2 : 1. / 3.;  // forward a_k; b_k is rk.b
  if (fkind == 2 && a.k == 0) {
    // C += dt Mass^-1 F MC[3n+1] with F_alpha = -re^2 Dv, F_beta = re^2 (Rps + K2 Rs)
    __syncthreads();
    const cpx* x1 = xk + csz;
    for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
      const int r = i / kTile, l = i - r * kTile;
      if (l >= nx || l < xfirst) continue;
      const int x = x0 + l;
      const double k2 = g.K2[(size_t)z * gsz.X() + x];
      if (r < gsz.D()) {
        const cpx v = visc_v_row(g, k2, x1 + cidx(0, 0, x), gsz.X(), r);
        s.ra[r * kTile + l] = cpx{-re2 * v.re, -re2 * v.im};
      }
      const cpx w = visc_g_row(g, k2, x1 + cidx(1, 0, x), gsz.X(), r);
      s.rb[r * kTile + l] = cpx{re2 * w.re, re2 * w.im};
    }
    __syncthreads();
    if (threadIdx.x < 8 * kTile) {  // mass matrices: the b = 0 factors
      const int l = (threadIdx.x % (4 * kTile)) / 4, ch = 4 * (threadIdx.x / (4 * kTile)) + threadIdx.x % 4;
      if (l < nx && l >= xfirst) {
        const size_t zx = (size_t)z * gsz.X() + x0 + l;
        const int par = ch & 1, part = (ch >> 1) & 1;
        if (ch < 4)
          band_solve_chain<9, 4, 4>(g.luA + ((size_t)2 * gsz.Nz() * gsz.X() + zx) * gsz.D() * 9,
                                    g.rdA + ((size_t)2 * gsz.Nz() * gsz.X() + zx) * gsz.D(), gsz.D(), par,
                                    reinterpret_cast<double*>(s.ra + l) + part, 2 * kTile);
        else
          band_solve_chain<5, 2, 2>(g.luB + ((size_t)2 * gsz.Nz() * gsz.X() + zx) * gsz.R() * 5,
                                    g.rdB + ((size_t)2 * gsz.Nz() * gsz.X() + zx) * gsz.R(), gsz.R(), par,
                                    reinterpret_cast<double*>(s.rb + l) + part, 2 * kTile);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
      const int r = i / kTile, l = i - r * kTile;
      if (l >= nx || l < xfirst) continue;
      const int x = x0 + l;
      if (r < gsz.D()) {
        const cpx f = s.ra[r * kTile + l];
        Cc[cidx(0, r, x)].re += dt * f.re;
        Cc[cidx(0, r, x)].im += dt * f.im;
      }
      const cpx f = s.rb[r * kTile + l];
      Cc[cidx(1, r, x)].re += dt * f.re;
      Cc[cidx(1, r, x)].im += dt * f.im;
    }
    __syncthreads();
  }
  // right-hand sides (channel/project.c:60-81, 125-130, 143-163, 202-207)
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx || l < xfirst) continue;
    const int x = x0 + l;
    const size_t zx = (size_t)z * gsz.X() + x;
    cpx va, vb;
    if (r < gsz.D()) {
      if (a.k == 0) {
        const double* E = g.exA + ((size_t)rk.aidx0 * gsz.Nz() * gsz.X() + zx) * gsz.D() * 9;
        va = band_matvec_row(E, 9, 4, 4, gsz.D(), Cc + cidx(0, 0, x), gsz.X(), r);
      } else {
        va = Cc[cidx(0, r, x)];
      }
      const cpx f = s.Fa[r * kTile + l];
      va.re += dt * rk.c * f.re;
      va.im += dt * rk.c * f.im;
      if (fkind == 3) {
        const double k2 = g.K2[zx];
        const cpx d0 = visc_v_row(g, k2, xk + cidx(0, 0, x), gsz.X(), r);
        const cpx d1 = visc_v_row(g, k2, xk + csz + cidx(0, 0, x), gsz.X(), r);
        va.re -= re2 * dt * ak * d0.re;
        va.im -= re2 * dt * ak * d0.im;
        va.re -= re2 * dt * rk.b * d1.re;
        va.im -= re2 * dt * rk.b * d1.im;
      }
    } else {
      va = Cc[cidx(0, r, x)];  // alpha rows >= Ny-4 ride along unchanged
    }
    if (a.k == 0) {
      const double* E = g.exB + ((size_t)rk.aidx0 * gsz.Nz() * gsz.X() + zx) * gsz.R() * 5;
      vb = band_matvec_row(E, 5, 2, 2, gsz.R(), Cc + cidx(1, 0, x), gsz.X(), r);
    } else {
      vb = Cc[cidx(1, r, x)];
    }
    const cpx f = s.Fb[r * kTile + l];
    vb.re += dt * rk.c * f.re;
    vb.im += dt * rk.c * f.im;
    if (fkind == 3) {  // beta: D = -(Rps + K2 Rs)
      const double k2 = g.K2[zx];
      const cpx d0 = visc_g_row(g, k2, xk + cidx(1, 0, x), gsz.X(), r);
      const cpx d1 = visc_g_row(g, k2, xk + csz + cidx(1, 0, x), gsz.X(), r);
      vb.re += re2 * dt * ak * d0.re;
      vb.im += re2 * dt * ak * d0.im;
      vb.re += re2 * dt * rk.b * d1.re;
      vb.im += re2 * dt * rk.b * d1.im;
    }
    s.ra[r * kTile + l] = va;
    s.rb[r * kTile + l] = vb;
  }
  __syncthreads();
  // banded solves: per column 4 chains for alpha, 4 for beta (parity x re/im)
  if (threadIdx.x < 8 * kTile) {
    // threads [0, 4 kTile) run the alpha chains, [4 kTile, 8 kTile) the beta
    // ones: a warp holds one system (no divergence between the two bands)
    const int l = (threadIdx.x % (4 * kTile)) / 4, ch = 4 * (threadIdx.x / (4 * kTile)) + threadIdx.x % 4;
    if (l < nx && l >= xfirst) {
      const int x = x0 + l;
      const size_t zx = (size_t)z * gsz.X() + x;
      const int par = ch & 1, part = (ch >> 1) & 1;
      if (ch < 4) {
        const size_t sys = (size_t)rk.bidx * gsz.Nz() * gsz.X() + zx;
        band_solve_chain<9, 4, 4>(g.luA + sys * gsz.D() * 9, g.rdA + sys * gsz.D(), gsz.D(), par,
                                  reinterpret_cast<double*>(s.ra + l) + part, 2 * kTile);
      } else {
        const size_t sys = (size_t)rk.bidx * gsz.Nz() * gsz.X() + zx;
        band_solve_chain<5, 2, 2>(g.luB + sys * gsz.R() * 5, g.rdB + sys * gsz.R(), gsz.R(), par,
                                  reinterpret_cast<double*>(s.rb + l) + part, 2 * kTile);
      }
    }
  }
  __syncthreads();
  // mean mode (channel/project0.c, increproject0.c, adjproject0.c), warp 0
  if (xfirst == 1 && threadIdx.x < 32) {
    double* fa = s.m0;                 // [R]
    double* fb = s.m0 + gsz.R();           // [R]
    cpx* ca = reinterpret_cast<cpx*>(s.m0 + 2 * gsz.R());  // [R]
    cpx* cb = ca + gsz.R();                                // [R]
    const int lane = threadIdx.x;
    const size_t cs = (size_t)gsz.Q() * gsz.X();
    const cpx* H0 = H;  // z = 0, x = 0
    if (fkind == 2 && a.k == 0) {
      // tangent_forcing0.c:31-41 on MC[3n+1], Rs^-1, IC += dt f (increproject0.c:45-90)
      const cpx* x1 = xk + csz;
      for (int i = lane; i < gsz.R(); i += 32) {
        const cpx p = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), x1 + cidx(0, 0, 0), gsz.X(), i);
        const cpx q = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), x1 + cidx(1, 0, 0), gsz.X(), i);
        ca[i] = cpx{re2 * p.re, re2 * p.im};
        cb[i] = cpx{re2 * q.re, re2 * q.im};
      }
      __syncwarp();
      if (lane < 8) {
        const int par = lane & 1, part = (lane >> 1) & 1;
        band_solve_chain<5, 2, 2>(g.lu0 + (size_t)2 * gsz.R() * 5, g.rd0 + (size_t)2 * gsz.R(), gsz.R(), par,
                                  reinterpret_cast<double*>(lane < 4 ? ca : cb) + part, 2);
      }
      __syncwarp();
      for (int i = lane; i < gsz.R(); i += 32) {
        Cc[cidx(0, i, 0)].re += dt * ca[i].re;
        Cc[cidx(0, i, 0)].im += dt * ca[i].im;
        Cc[cidx(1, i, 0)].re += dt * cb[i].re;
        Cc[cidx(1, i, 0)].im += dt * cb[i].im;
      }
      __syncwarp();
    }
    for (int i = lane; i < gsz.R(); i += 32) {
      double sa = 0.0, sb = 0.0;
      for (int y = 0; y < gsz.Q(); ++y) {
        const double rw = __ldg(g.Wr + (size_t)i * gsz.Q() + y);
        sa = fma(rw, H0[1 * cs + (size_t)y * gsz.X()].re, sa);
        sb = fma(rw, H0[0 * cs + (size_t)y * gsz.X()].re, sb);
        if (adj) {
          const double rpw = __ldg(g.Wrp + (size_t)i * gsz.Q() + y);
          sa = fma(rpw, H0[4 * cs + (size_t)y * gsz.X()].re, sa);
          sb = fma(-rpw, H0[3 * cs + (size_t)y * gsz.X()].re, sb);
        }
      }
      fa[i] = sa;
      fb[i] = sb;
      cpx va, vb;
      if (a.k == 0) {
        const double* E = g.ex0 + (size_t)rk.aidx0 * gsz.R() * 5;
        va = band_matvec_row(E, 5, 2, 2, gsz.R(), Cc + cidx(0, 0, 0), gsz.X(), i);
        vb = band_matvec_row(E, 5, 2, 2, gsz.R(), Cc + cidx(1, 0, 0), gsz.X(), i);
      } else {
        va = Cc[cidx(0, i, 0)];
        vb = Cc[cidx(1, i, 0)];
      }
      va.re += dt * rk.c * sa;
      vb.re += dt * rk.c * sb;
      if (fkind == 3) {
        // D0 = -Rps; the implicit term acts on the primal's solved mean flow
        // before its flux correction: MC[3n+k+1] - 0.5 flux_t add
        const cpx p0 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + cidx(0, 0, 0), gsz.X(), i);
        cpx p1 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + csz + cidx(0, 0, 0), gsz.X(), i);
        p1.re -= 0.5 * ft1 * rps_row_real(g, g.add0, i);
        const cpx q0 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + cidx(1, 0, 0), gsz.X(), i);
        const cpx q1 = band_matvec_row(g.Rps, 5, 2, 2, gsz.R(), xk + csz + cidx(1, 0, 0), gsz.X(), i);
        va.re += re2 * dt * ak * p0.re;
        va.im += re2 * dt * ak * p0.im;
        va.re += re2 * dt * rk.b * p1.re;
        va.im += re2 * dt * rk.b * p1.im;
        vb.re += re2 * dt * ak * q0.re;
        vb.im += re2 * dt * ak * q0.im;
        vb.re += re2 * dt * rk.b * q1.re;
        vb.im += re2 * dt * rk.b * q1.im;
      }
      ca[i] = va;
      cb[i] = vb;
    }
    __syncwarp();
    if (lane < 8) {
      const int par = lane & 1, part = (lane >> 1) & 1;
      cpx* vec = (lane < 4) ? ca : cb;
      band_solve_chain<5, 2, 2>(g.lu0 + (size_t)rk.bidx * gsz.R() * 5, g.rd0 + (size_t)rk.bidx * gsz.R(), gsz.R(), par,
                                reinterpret_cast<double*>(vec) + part, 2);
    }
    __syncwarp();
    // constant mass flux: a += 0.5 * flux_t * add (channel/project0.c:153-168)
    double part = 0.0;
    for (int i = lane; i < gsz.R(); i += 32) part = fma(g.rwsum[i], ca[i].re, part);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    double flux_t;
    if (mean_mode == MEAN_PRIMAL) flux_t = g.flux - part;
    else if (mean_mode == MEAN_TAN_FORCED) flux_t = 2.0 - part;
    else flux_t = -part;
    const double* add = g.add0 + (size_t)(adj ? 1 + rk.bidx : 0) * gsz.R();
    if (mean_mode == MEAN_PRIMAL && a.Fts && Tst && lane == 0)
      a.Fts[(long long)(inst / a.tdiv) * a.fts_stride + tslot] = flux_t;
    __syncwarp();
    for (int i = lane; i < gsz.R(); i += 32) ca[i].re = ca[i].re + flux_t * add[i] * 0.5;
    __syncwarp();
    for (int i = lane; i < gsz.R(); i += 32) {
      So[cidx(0, i, 0)] = ca[i];
      So[cidx(1, i, 0)] = cb[i];
      if (Tst) {
        Tst[cidx(0, i, 0)] = ca[i];
        Tst[cidx(1, i, 0)] = cb[i];
      }
    }
  }
  // state rows: alpha from the solve (rows >= Ny-4 carried), beta from the solve
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx || l < xfirst) continue;
    const int x = x0 + l;
    const cpx va = s.ra[r * kTile + l], vb = s.rb[r * kTile + l];
    So[cidx(0, r, x)] = va;
    So[cidx(1, r, x)] = vb;
    if (Tst) {
      Tst[cidx(0, r, x)] = va;
      Tst[cidx(1, r, x)] = vb;
    }
  }
  __syncthreads();
  if (a.k == 2) {
    // the carried array is the state after the last substage
    for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
      const int r = i / kTile, l = i - r * kTile;
      if (l >= nx) continue;
      const int x = x0 + l;
      Cc[cidx(0, r, x)] = So[cidx(0, r, x)];
      Cc[cidx(1, r, x)] = So[cidx(1, r, x)];
    }
    return;
  }
  // next-substage right-hand side: M(a[k+1]) state + dt d[k+1] F
  // (channel/project.c:352-404; adjoint F from the previous-stage terms,
  //  channel/adjproject.c:393-549)
  if (adj) {
    __syncthreads();
    if (g.tc) quad_rhs_tc<kTile, NTHR>(g, gsz, a.Hprev.at(inst), z, x0, nx, true, s);
    else quad_rhs<kTile>(g, a.Hprev.at(inst), z, x0, nx, true, s);
    if (xfirst == 1 && threadIdx.x < 32) {
      // mean mode fa/fb from the previous-stage terms (channel/adjproject0.c:254-294)
      const cpx* H0 = a.Hprev.at(inst);
      const size_t cs = (size_t)gsz.Q() * gsz.X();
      for (int i = threadIdx.x; i < gsz.R(); i += 32) {
        double sa = 0.0, sb = 0.0;
        for (int y = 0; y < gsz.Q(); ++y) {
          const double rw = __ldg(g.Wr + (size_t)i * gsz.Q() + y);
          const double rpw = __ldg(g.Wrp + (size_t)i * gsz.Q() + y);
          sa = fma(rw, H0[1 * cs + (size_t)y * gsz.X()].re, sa);
          sa = fma(rpw, H0[4 * cs + (size_t)y * gsz.X()].re, sa);
          sb = fma(rw, H0[0 * cs + (size_t)y * gsz.X()].re, sb);
          sb = fma(-rpw, H0[3 * cs + (size_t)y * gsz.X()].re, sb);
        }
        s.m0[i] = sa;
        s.m0[gsz.R() + i] = sb;
      }
    }
    __syncthreads();
  }
  // the solved state of this tile (So) is still in ra, rb unless the
  // adjoint's second quadrature overwrote them (they share its digit
  // buffer); the results go to Fa, Fb (each element read and written by one
  // thread)
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx || l < xfirst) continue;
    const int x = x0 + l;
    const size_t zx = (size_t)z * gsz.X() + x;
    const cpx* ya = adj ? So + cidx(0, 0, x) : s.ra + l;
    const cpx* yb = adj ? So + cidx(1, 0, x) : s.rb + l;
    const int ys = adj ? gsz.X() : kTile;
    if (r < gsz.D()) {
      const double* E = g.exA + ((size_t)rk.aidx_next * gsz.Nz() * gsz.X() + zx) * gsz.D() * 9;
      cpx va = band_matvec_row_t<9, 4, 4>(E, gsz.D(), ya, ys, r);
      const cpx f = s.Fa[r * kTile + l];
      va.re += dt * rk.dnext * f.re;
      va.im += dt * rk.dnext * f.im;
      s.Fa[r * kTile + l] = va;
    }
    const double* E = g.exB + ((size_t)rk.aidx_next * gsz.Nz() * gsz.X() + zx) * gsz.R() * 5;
    cpx vb = band_matvec_row_t<5, 2, 2>(E, gsz.R(), yb, ys, r);
    const cpx f = s.Fb[r * kTile + l];
    vb.re += dt * rk.dnext * f.re;
    vb.im += dt * rk.dnext * f.im;
    s.Fb[r * kTile + l] = vb;
  }
  if (xfirst == 1 && threadIdx.x < 32) {
    const double* E = g.ex0 + (size_t)rk.aidx_next * gsz.R() * 5;
    cpx* ca = reinterpret_cast<cpx*>(s.m0 + 2 * gsz.R());
    cpx* cb = ca + gsz.R();
    for (int i = threadIdx.x; i < gsz.R(); i += 32) {
      cpx va = band_matvec_row(E, 5, 2, 2, gsz.R(), So + cidx(0, 0, 0), gsz.X(), i);
      cpx vb = band_matvec_row(E, 5, 2, 2, gsz.R(), So + cidx(1, 0, 0), gsz.X(), i);
      va.re += dt * rk.dnext * s.m0[i];
      vb.re += dt * rk.dnext * s.m0[gsz.R() + i];
      ca[i] = va;
      cb[i] = vb;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < gsz.R() * kTile; i += NTHR) {
    const int r = i / kTile, l = i - r * kTile;
    if (l >= nx) continue;
    const int x = x0 + l;
    if (l < xfirst) {
      const cpx* ca = reinterpret_cast<const cpx*>(s.m0 + 2 * gsz.R());
      Cc[cidx(0, r, x)] = ca[r];
      Cc[cidx(1, r, x)] = ca[gsz.R() + r];
    } else {
      Cc[cidx(0, r, x)] = r < gsz.D() ? s.Fa[r * kTile + l] : So[cidx(0, r, x)];  // rows >= Ny-4 carried
      Cc[cidx(1, r, x)] = s.Fb[r * kTile + l];
    }
  }
}

template <int T, class S, int NTHR = kThreads, int MINB = 2>
static void launch_solve_t(const Grid& g, const SolveArgs& a, cudaStream_t st) {
  const int ntx = (g.X + T - 1) / T;
  const dim3 grid(g.Nz * ntx, a.ninst);
  if (a.grids) k_solve<true, T, SizesRT, NTHR, MINB><<<grid, NTHR, solve_smem_bytes_t<T>(g), st>>>(g, a);
  else k_solve<false, T, S, NTHR, MINB><<<grid, NTHR, solve_smem_bytes_t<T>(g), st>>>(g, a);
}

// Grid::stile 16 or 8 columns in 256-thread blocks, or 8 columns in
// 128-thread blocks at 4 per SM (Grid::sthr 128)
template <class S>
static void launch_solve_s(const Grid& g, const SolveArgs& a, cudaStream_t st) {
  if (g.stile == 8 && g.sthr == 128) launch_solve_t<8, S, 128, 4>(g, a, st);
  else if (g.stile == 8) launch_solve_t<8, S>(g, a, st);
  else launch_solve_t<16, S>(g, a, st);
}

// the block tile of Grid::stile (8 or 16 kx columns; the same results), the
// build compiled for the grid's sizes where Grid::fixed & FIXED_SOLVE
cudaError_t launch_solve(const Grid& g, const SolveArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  const bool fx = (g.fixed & FIXED_SOLVE) && !a.grids;
  if (fx && sizes_match<Sizes32>(g)) launch_solve_s<Sizes32>(g, a, st);
  else if (fx && sizes_match<Sizes16>(g)) launch_solve_s<Sizes16>(g, a, st);
  else launch_solve_s<SizesRT>(g, a, st);
  return cudaGetLastError();
}

void prepare_recon_solve(int optin) {
  allow_max_smem(k_recon<false>, optin);
  allow_max_smem(k_recon<true>, optin);
  allow_max_smem(k_solve<false, 16, SizesRT>, optin);
  allow_max_smem(k_solve<true, 16, SizesRT>, optin);
  allow_max_smem(k_solve<false, 8, SizesRT>, optin);
  allow_max_smem(k_solve<true, 8, SizesRT>, optin);
  allow_max_smem(k_solve<false, 16, Sizes32>, optin);
  allow_max_smem(k_solve<false, 8, Sizes32>, optin);
  allow_max_smem(k_solve<false, 16, Sizes16>, optin);
  allow_max_smem(k_solve<false, 8, Sizes16>, optin);
  allow_max_smem(k_solve<false, 8, SizesRT, 128, 4>, optin);
  allow_max_smem(k_solve<true, 8, SizesRT, 128, 4>, optin);
  allow_max_smem(k_solve<false, 8, Sizes32, 128, 4>, optin);
  allow_max_smem(k_solve<false, 8, Sizes16, 128, 4>, optin);
}

}  // namespace chn
