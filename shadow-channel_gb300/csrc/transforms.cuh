// Split transform passes, templated on the block size NT and the chunk CH.
//
// A plane's 2D transforms run as a z pass (columns) and an x pass (row
// pairs) with the spectral columns in an HBM intermediate
//   T[inst][c][Q][pz][Nx/2]   (c: field or product component).
// A block transforms CH columns (z pass, ordered (x, c)) or CH row pairs (x
// pass, ordered (pair, c)) taken across the components, so the butterflies of
// a radix pass (CH x N/R per pass) can be sized to fill the NT threads: with
// 3Nz/2 = 48, CH = 48 and NT = 192 every pass is an exact multiple of the
// block.  Each 1D transform is the same fft_run sequence on the same data as
// in the one-block-per-plane kernels, so every variant gives identical
// results; the autotuner picks the fastest per grid.  Lengths 3 * 2^i * 3^j
// only (radices 2, 3, 4).
#pragma once

#include <algorithm>

#include "chn_common.cuh"
#include "fft.cuh"
#include "kernels.h"
#include "phys_common.cuh"

namespace chn {

template <int CH>
inline size_t tz_smem(const Grid& g, bool keep) {
  return ((size_t)g.pz + 2 * (size_t)g.pz * CH + (keep ? (size_t)g.Nz * CH : 0)) * sizeof(cpx);
}

template <int CH>
inline size_t tx_smem(const Grid& g) {
  return ((size_t)g.px + 2 * (size_t)CH * g.px) * sizeof(cpx);
}

// intermediate block of (local instance il, component c of nc, plane y), sized by the launch grid
__device__ __forceinline__ size_t tslot(const Grid& g0, int il, int nc, int c, int y) {
  return (((size_t)il * nc + c) * g0.Q + y) * g0.pz * g0.X;
}

// inverse z pass: spectral fields -> T (channel/pass1.c:58-110)
template <bool MULTI, int NT, int CH>
__global__ void __launch_bounds__(NT) k_tz_inv(const __grid_constant__ Grid g0, PhysArgs a, int inst0, int nf,
                                               cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int c0 = blockIdx.z * CH;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int ncol = nf * g.X;
  if (y >= g.Q || c0 >= ncol) return;
  const int nc = min(CH, ncol - c0);
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.pz;
  cpx* b1 = b0 + (size_t)g.pz * CH;
  for (int i = threadIdx.x; i < g.pz; i += NT) tw[i] = g.twz[i];
  const cpx* __restrict__ U = a.U.at(inst);
  for (int i = threadIdx.x; i < g.pz * nc; i += NT) {
    const int zp = i / nc, cl = i - zp * nc;
    const int gc = c0 + cl, x = gc / nf, f = gc - x * nf;
    const int z = zrow_to_kz(g, zp);
    b0[i] = z >= 0 ? field_value(g, U, f, z, y, x) : cpx{0.0, 0.0};
  }
  __syncthreads();
  const FftPlan plan = make_plan(g.pz, true);
  const cpx* zr = fft_run<false>(plan, b0, b1, nc, nc, 1, tw, +1, true);
  for (int i = threadIdx.x; i < g.pz * nc; i += NT) {
    const int zp = i / nc, cl = i - zp * nc;
    const int gc = c0 + cl, x = gc / nf, f = gc - x * nf;
    T[tslot(g0, il, nf, f, y) + (size_t)zp * g.X + x] = zr[i];
  }
}

// inverse x pass: row pairs of T -> physical rows of P; the CFL number of
// the velocity (channel/pass1.c:111-138) over the pairs of the block (CH is a
// multiple of nf, so a block holds u, v and w of each of its pairs)
template <bool MULTI, int NT, int CH>
__global__ void __launch_bounds__(NT) k_tx_inv(const __grid_constant__ Grid g0, PhysArgs a, int inst0, int nf,
                                               const cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int r0 = blockIdx.z * CH;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int npair = (g.pz + 1) / 2, nrow = npair * nf;
  if (y >= g.Q || r0 >= nrow) return;
  const int nr = min(CH, nrow - r0);
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.px;
  cpx* b1 = b0 + (size_t)CH * g.px;
  for (int i = threadIdx.x; i < g.px; i += NT) tw[i] = g.twx[i];
  double* __restrict__ P = a.P.at(inst);
  if (a.pslot.stride) P += (long long)a.pslot.slot() * a.pslot.stride;
  for (int i = threadIdx.x; i < nr * g.px; i += NT) {
    const int rl = i / g.px, k = i - rl * g.px;
    const int gr = r0 + rl, p = gr / nf, f = gr - p * nf;
    const cpx* zr = T + tslot(g0, il, nf, f, y);
    const int ra = 2 * p, rb = ra + 1;
    cpx Z = {0.0, 0.0};
    int kk = -1;
    bool conj = false;
    if (k < g.X) kk = k;
    else if (k > g.px - g.X) { kk = g.px - k; conj = true; }
    if (kk >= 0) {
      const cpx A = zr[(size_t)ra * g.X + kk];
      const cpx B = rb < g.pz ? zr[(size_t)rb * g.X + kk] : cpx{0.0, 0.0};
      if (kk == 0) {  // c2r ignores the imaginary part of the DC bin
        Z.re = A.re; Z.im = B.re;
      } else if (!conj) {
        Z.re = A.re - B.im; Z.im = A.im + B.re;
      } else {
        Z.re = A.re + B.im; Z.im = B.re - A.im;
      }
    }
    b0[i] = Z;
  }
  __syncthreads();
  const FftPlan plan = make_plan(g.px, true);
  const cpx* xr = fft_run<false>(plan, b0, b1, nr, 1, g.px, tw, +1, true);
  const size_t plane = (size_t)g.pz * g.px;
  bool nonfinite = false;
  for (int i = threadIdx.x; i < nr * 2 * g.px; i += NT) {
    const int rl = i / (2 * g.px), rem = i - rl * 2 * g.px, h = rem / g.px, xp = rem - h * g.px;
    const int gr = r0 + rl, p = gr / nf, f = gr - p * nf, row = 2 * p + h;
    if (row >= g.pz) continue;
    const cpx c = xr[(size_t)rl * g.px + xp];
    const double v = h ? c.im : c.re;
    P[((size_t)f * g.Q + y) * plane + (size_t)row * g.px + xp] = v;
    nonfinite |= !isfinite(v);
  }
  if (nonfinite && a.status) atomicOr(&a.status[inst / a.sdiv], ST_NONFINITE);
  if (!a.cfl_check) return;
  __shared__ double red[NT];
  double m = 0.0;
  const int npl = nr / nf;  // whole pairs in this block
  for (int i = threadIdx.x; i < npl * 2 * g.px; i += NT) {
    const int pl = i / (2 * g.px), rem = i - pl * 2 * g.px, h = rem / g.px, xp = rem - h * g.px;
    if (2 * ((r0 / nf) + pl) + h >= g.pz) continue;
    const size_t o = (size_t)pl * nf * g.px + xp;
    const cpx u = xr[o], v = xr[o + g.px], w = xr[o + 2 * g.px];
    const double t = fabs(h ? u.im : u.re) * g.cfl1 + fabs(h ? v.im : v.re) * g.cfl2[y] +
                     fabs(h ? w.im : w.re) * g.cfl3;
    m = fmax(m, t);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double c = red[0] * g.dt;
    if (a.cflmax)
      atomicMax(reinterpret_cast<unsigned long long*>(&a.cflmax[inst / a.sdiv]),
                (unsigned long long)__double_as_longlong(c));
    if (c >= 2.8) atomicOr(&a.status[inst / a.sdiv], ST_CFL);
  }
}

// forward x pass: products of row pairs, x transform, kept bins -> T
// (channel/pass1.c:212-330, pass2.c:352-500)
template <bool MULTI, int NT, int CH>
__global__ void __launch_bounds__(NT) k_tx_fwd(const __grid_constant__ Grid g0, ProdArgs a, int mode, int inst0,
                                               cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int r0 = blockIdx.z * CH;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int ncomp = mode >= 2 ? 6 : 3;
  const int npair = (g.pz + 1) / 2, nrow = npair * ncomp;
  if (y >= g.Q || r0 >= nrow) return;
  const int nr = min(CH, nrow - r0);
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.px;
  cpx* b1 = b0 + (size_t)CH * g.px;
  for (int i = threadIdx.x; i < g.px; i += NT) tw[i] = g.twx[i];
  const size_t plane = (size_t)g.pz * g.px, fs = (size_t)g.Q * plane;
  const double* __restrict__ Pp = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                  (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ Pt = a.Pt.base ? a.Pt.at(inst) + (size_t)y * plane : nullptr;
  for (int i = threadIdx.x; i < nr * g.px; i += NT) {
    const int rl = i / g.px, xp = i - rl * g.px;
    const int gr = r0 + rl, p = gr / ncomp, q = gr - p * ncomp, ra = 2 * p;
    const size_t oa = (size_t)ra * g.px + xp;
    cpx z;
    z.re = split_product(mode, Pp, Pt, fs, oa, q);
    z.im = ra + 1 < g.pz ? split_product(mode, Pp, Pt, fs, oa + g.px, q) : 0.0;
    b0[i] = z;
  }
  __syncthreads();
  const FftPlan plan = make_plan(g.px, false);
  const cpx* xr = fft_run<false>(plan, b0, b1, nr, 1, g.px, tw, -1, true);
  const double hn = mode == 3 ? 0.5 : 0.5 * g.norm;  // the transpose carries no 1/(px pz)
  for (int i = threadIdx.x; i < nr * g.X; i += NT) {
    const int rl = i / g.X, k = i - rl * g.X;
    const int gr = r0 + rl, p = gr / ncomp, q = gr - p * ncomp, ra = 2 * p;
    const cpx Zk = xr[(size_t)rl * g.px + k];
    const cpx Zn = xr[(size_t)rl * g.px + (k == 0 ? 0 : g.px - k)];
    cpx A, B;
    A.re = (Zk.re + Zn.re) * hn;
    A.im = (Zk.im - Zn.im) * hn;
    B.re = (Zk.im + Zn.im) * hn;
    B.im = (Zn.re - Zk.re) * hn;
    cpx* Tq = T + tslot(g0, il, ncomp, q, y);
    Tq[(size_t)ra * g.X + k] = A;
    if (ra + 1 < g.pz) Tq[(size_t)(ra + 1) * g.X + k] = B;
  }
}

// forward z pass: columns of T, z transform, truncation -> H; the adjoint
// (and the exact transpose, mode 3) assembles H from its 6 spectra per
// column (CH is a multiple of 6)
template <bool MULTI, int NT, int CH>
__global__ void __launch_bounds__(NT) k_tz_fwd(const __grid_constant__ Grid g0, ProdArgs a, int mode, int inst0,
                                               const cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int c0 = blockIdx.z * CH;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int ncomp = mode >= 2 ? 6 : 3;
  const int ncol = ncomp * g.X;
  if (y >= g.Q || c0 >= ncol) return;
  const int nc = min(CH, ncol - c0);
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.pz;
  cpx* b1 = b0 + (size_t)g.pz * CH;
  cpx* keep = b1 + (size_t)g.pz * CH;  // adjoint: [column][Nz]
  for (int i = threadIdx.x; i < g.pz; i += NT) tw[i] = g.twz[i];
  for (int i = threadIdx.x; i < g.pz * nc; i += NT) {
    const int zp = i / nc, cl = i - zp * nc;
    const int gc = c0 + cl, x = gc / ncomp, q = gc - x * ncomp;
    b0[i] = T[tslot(g0, il, ncomp, q, y) + (size_t)zp * g.X + x];
  }
  __syncthreads();
  const FftPlan plan = make_plan(g.pz, false);
  const cpx* zr = fft_run<false>(plan, b0, b1, nc, nc, 1, tw, -1, true);
  cpx* __restrict__ H = a.H.at(inst);
  for (int i = threadIdx.x; i < g.pz * nc; i += NT) {
    const int zp = i / nc, cl = i - zp * nc;
    const int z = zrow_to_kz(g, zp);
    if (z < 0) continue;
    const int gc = c0 + cl, x = gc / ncomp, q = gc - x * ncomp;
    if (mode >= 2) keep[(size_t)cl * g.Nz + z] = zr[i];
    else H[(((size_t)z * 5 + q) * g.Q + y) * g.X + x] = zr[i];
  }
  if (mode < 2) return;
  __syncthreads();
  const int nx = nc / 6;
  for (int i = threadIdx.x; i < g.Nz * nx; i += NT) {
    const int xl = i / g.Nz, z = i - xl * g.Nz;
    if (z == g.Nz / 2) continue;
    const cpx* K = keep + (size_t)xl * 6 * g.Nz + z;
    for (int q = 0; q < 6; ++q) assemble_stage(g, mode == 3, H, z, y, c0 / 6 + xl, q, K[q * g.Nz]);
  }
}

// instance chunks that fit the intermediate
template <typename F>
static cudaError_t split_chunks(int ninst, int cap, F&& body) {
  if (cap <= 0) return cudaErrorInvalidValue;
  for (int i0 = 0; i0 < ninst; i0 += cap) {
    const cudaError_t e = body(i0, std::min(cap, ninst - i0));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int NT, int CH>
cudaError_t split_inverse_t(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  if (!a.tmp) return cudaErrorInvalidValue;
  const int nf = a.nfields;
  const int cap = a.tmp_inst * 6 / nf;
  return split_chunks(a.ninst, cap, [&](int i0, int n) {
    const int npair = (g.pz + 1) / 2;
    const dim3 gz(g.Q, n, (nf * g.X + CH - 1) / CH), gx(g.Q, n, (npair * nf + CH - 1) / CH);
    const size_t sz = tz_smem<CH>(g, false), sx = tx_smem<CH>(g);
    if (a.grids) {
      k_tz_inv<true, NT, CH><<<gz, NT, sz, st>>>(g, a, i0, nf, a.tmp);
      k_tx_inv<true, NT, CH><<<gx, NT, sx, st>>>(g, a, i0, nf, a.tmp);
    } else {
      k_tz_inv<false, NT, CH><<<gz, NT, sz, st>>>(g, a, i0, nf, a.tmp);
      k_tx_inv<false, NT, CH><<<gx, NT, sx, st>>>(g, a, i0, nf, a.tmp);
    }
    return cudaGetLastError();
  });
}

template <int NT, int CH>
cudaError_t split_products_t(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {
  if (!a.tmp) return cudaErrorInvalidValue;
  const int ncomp = mode >= 2 ? 6 : 3;
  const int cap = a.tmp_inst * 6 / ncomp;
  return split_chunks(a.ninst, cap, [&](int i0, int n) {
    const int npair = (g.pz + 1) / 2;
    const dim3 gx(g.Q, n, (npair * ncomp + CH - 1) / CH), gz(g.Q, n, (ncomp * g.X + CH - 1) / CH);
    const size_t sx = tx_smem<CH>(g), sz = tz_smem<CH>(g, mode >= 2);
    if (a.grids) {
      k_tx_fwd<true, NT, CH><<<gx, NT, sx, st>>>(g, a, mode, i0, a.tmp);
      k_tz_fwd<true, NT, CH><<<gz, NT, sz, st>>>(g, a, mode, i0, a.tmp);
    } else {
      k_tx_fwd<false, NT, CH><<<gx, NT, sx, st>>>(g, a, mode, i0, a.tmp);
      k_tz_fwd<false, NT, CH><<<gz, NT, sz, st>>>(g, a, mode, i0, a.tmp);
    }
    return cudaGetLastError();
  });
}

template <int NT, int CH>
void prepare_split_t(int optin) {
  allow_max_smem(k_tz_inv<false, NT, CH>, optin);
  allow_max_smem(k_tx_inv<false, NT, CH>, optin);
  allow_max_smem(k_tx_fwd<false, NT, CH>, optin);
  allow_max_smem(k_tz_fwd<false, NT, CH>, optin);
  allow_max_smem(k_tz_inv<true, NT, CH>, optin);
  allow_max_smem(k_tx_inv<true, NT, CH>, optin);
  allow_max_smem(k_tx_fwd<true, NT, CH>, optin);
  allow_max_smem(k_tz_fwd<true, NT, CH>, optin);
}

template <int CH>
bool split_fits_t(const Grid& g, int optin) {
  if (g.general) return false;  // the split passes compile radices 2, 3, 4 only
  const size_t room = (size_t)optin - 4096;
  return tz_smem<CH>(g, true) <= room && tx_smem<CH>(g) <= room;
}

// one translation unit per variant defines these (split_variants_*.cu)
#define CHN_SPLIT_VARIANT(ID, NT, CH)                                                                     \
  cudaError_t split_inverse_##ID(const Grid& g, const PhysArgs& a, cudaStream_t st) {                    \
    return split_inverse_t<NT, CH>(g, a, st);                                                             \
  }                                                                                                        \
  cudaError_t split_products_##ID(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {         \
    return split_products_t<NT, CH>(g, a, mode, st);                                                      \
  }                                                                                                        \
  void prepare_split_##ID(int optin) { prepare_split_t<NT, CH>(optin); }                                  \
  bool split_fits_##ID(const Grid& g, int optin) { return split_fits_t<CH>(g, optin); }

}  // namespace chn
