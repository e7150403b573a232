// The inverse 3/2-padded transforms (channel/pass1.c:42-114,
// channel/spec2phys.c:39-76) as exact digit GEMMs on the tensor cores.
//
// One block per (instance, plane y), two fields per pass:
//   z stage   Z[m][x] = sum_kz F[kz][x] exp(+2 pi i m zp(kz)/pz) over the
//             Nz - 1 kept rows, one column per (field, x);
//   x stage   P[m][xp] = Re Z[m][0] + 2 sum_{0<j<X} Re(Z[m][j] exp(+2 pi i j xp/px))
//             (the complex-to-real transform; the imaginary part of the
//             kx = 0 bin is ignored as by c2r), one column per m.
// Each stage is split radix-2 where its length n is even: with
// exp(2 pi i k (m + n/2)/n) = (-1)^k exp(2 pi i k m/n), the outputs m and
// m + n/2 are E + O and E - O for the sums E, O over the even and odd k, so
// a stage is one GEMM with half the rows (m < n/2) whose K holds the even
// modes and then the odd ones; the two partial sums stay exact 64-bit
// integers (the E and O rows of a table share their row exponent) and their
// sum and difference are rounded once each.  z stage: rows Re, Im of
// Z[m < pz/2] (2 pz/2 rows), K = Re, Im of the even-zp and odd-zp modes;
// x stage: rows xp < px/2, K = Re, Im of the even and odd j.  An odd length
// keeps one class (the full DFT).
// The DFT matrices hold the FFT's own twiddle doubles; operands are base-256
// digits with exact FP32 level sums (tc_common.cuh), so each output is the
// (faithfully) rounded value of the exact sum of the 56-bit operands.  The
// intermediate Z is rounded to FP64 in shared memory between the stages.  Same outputs,
// CFL check and status bits as k_phys_inverse.
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "chn_common.cuh"
#include "kernels.h"
#include "phys_common.cuh"
#include "setup.h"
#include "phys_tc.cuh"
#include "sizes.cuh"
#include "tc_common.cuh"

namespace chn {

static constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// host tables
// ---------------------------------------------------------------------------

// the kept kz modes of one class of the z stage's radix-2 split (padded
// index zp even or odd; the only class for an odd pz)
static void z_class_modes(int Nz, int pz, int cls, std::vector<int>& kk_of) {
  kk_of.clear();
  for (int kk = 0; kk < Nz - 1; ++kk) {
    const int zp = kk < Nz / 2 ? kk : kk + 1 + Nz / 2;  // padded row of kept kz index kk
    if (pz % 2 || (zp & 1) == cls) kk_of.push_back(kk);
  }
}

// the two stages' matrices (rows x K words of Re, Im) and the z stage's
// K-word -> kept kz map, shared by the mma.sync tables below and the
// tcgen05 tables of phys_tc5.cu
bool phys_tc_matrices(const HostTables& h, std::vector<double>& Az, std::vector<double>& Ax,
                      std::vector<int>& zmap, int& zrows, int& Kz, int& xrows, int& Kx) {
  const int pz = h.pz, px = h.px, Nz = h.Nz, X = h.X;
  const int Rz = pz % 2 ? 1 : 2, Rx = px % 2 ? 1 : 2, pzh = pz / Rz, pxh = px / Rx;
  std::vector<int> zE, zO;
  z_class_modes(Nz, pz, 0, zE);
  if (Rz == 2) z_class_modes(Nz, pz, 1, zO);
  int nE = 0, nO = 0;
  z_class_counts(Nz, pz, nE, nO);  // the kernel's closed form
  if (nE != (int)zE.size() || nO != (int)zO.size()) return false;
  const int nxE = (X + Rx - 1) / Rx, nxO = X - nxE;
  const int KTzE = (2 * (int)zE.size() + 15) / 16, KTzO = (2 * (int)zO.size() + 15) / 16;
  const int KTxE = (2 * nxE + 15) / 16, KTxO = (2 * nxO + 15) / 16;
  Kz = (KTzE + KTzO) * 16;
  Kx = (KTxE + KTxO) * 16;
  zrows = 2 * pzh;
  xrows = pxh;
  // z stage: rows Re Z[m], Im Z[m] (m < pzh); K words: even modes, then odd
  Az.assign((size_t)2 * pzh * Kz, 0.0);
  Ax.assign((size_t)pxh * Kx, 0.0);
  zmap.assign((size_t)Kz / 2, -1);
  for (int c = 0; c < 2; ++c) {
    const std::vector<int>& modes = c ? zO : zE;
    const int w0 = c ? KTzE * 8 : 0;
    for (int e = 0; e < (int)modes.size(); ++e) {
      const int kk = modes[e], zp = kk < Nz / 2 ? kk : kk + 1 + Nz / 2, w = w0 + e;
      zmap[w] = kk;
      for (int m = 0; m < pzh; ++m) {
        const int idx = (int)(((long long)m * zp) % pz);
        const double cs = h.twz[2 * idx], sn = -h.twz[2 * idx + 1];  // exp(+i theta) = conj(exp(-i theta))
        Az[(size_t)m * Kz + 2 * w] = cs;
        Az[(size_t)m * Kz + 2 * w + 1] = -sn;
        Az[(size_t)(pzh + m) * Kz + 2 * w] = sn;
        Az[(size_t)(pzh + m) * Kz + 2 * w + 1] = cs;
      }
    }
  }
  // x stage: rows xp < pxh; K words: j = Rx e (even), then j = 2 o + 1 (odd)
  for (int w = 0; w < Kx / 2; ++w) {
    int j;
    if (w < KTxE * 8) {
      if (w >= nxE) continue;
      j = Rx * w;
    } else {
      const int o = w - KTxE * 8;
      if (o >= nxO) continue;
      j = 2 * o + 1;
    }
    for (int xp = 0; xp < pxh; ++xp) {
      if (j == 0) {
        Ax[(size_t)xp * Kx + 2 * w] = 1.0;
        continue;
      }
      const int idx = (int)(((long long)j * xp) % px);
      const double cs = h.twx[2 * idx], sn = -h.twx[2 * idx + 1];
      Ax[(size_t)xp * Kx + 2 * w] = 2.0 * cs;
      Ax[(size_t)xp * Kx + 2 * w + 1] = -2.0 * sn;
    }
  }
  return true;
}

bool build_phys_tc_tables(const HostTables& h, std::vector<uint32_t>& zfrag, std::vector<int>& zex,
                          std::vector<uint32_t>& xfrag, std::vector<int>& xex, std::vector<int>& zmap) {
  std::vector<double> Az, Ax;
  int zrows = 0, Kz = 0, xrows = 0, Kx = 0;
  if (!phys_tc_matrices(h, Az, Ax, zmap, zrows, Kz, xrows, Kx)) return false;
  zfrag.clear(); zex.clear(); xfrag.clear(); xex.clear();
  // one table per stage with both classes in its K: a row's exponent covers
  // its even and odd parts, so their integer sums add exactly
  return append_digit_table(Az.data(), zrows, Kz, (zrows + 15) / 16, Kz / 16, zfrag, zex) &&
         append_digit_table(Ax.data(), xrows, Kx, (xrows + 15) / 16, Kx / 16, xfrag, xex);
}

// forward transforms (channel/pass1.c:312-339): x stage Y[zp][kx] =
// norm sum_xp p[zp][xp] exp(-2 pi i kx xp/px) for kx < X (rows 2kx, 2kx+1 =
// Re, Im; the 1/(px pz) scaling folded in; the exact transpose's products
// take an unscaled copy), z stage F[kz][kx] = sum_zp
// Y[zp][kx] exp(-2 pi i zp(kz) zp/pz) for the Nz - 1 kept rows (rows 2kk,
// 2kk+1; K = 2 pz with Re, Im of Y interleaved)
bool build_fwd_tc_tables(const HostTables& h, std::vector<uint32_t>& xfrag, std::vector<int>& xex,
                         std::vector<uint32_t>& zfrag, std::vector<int>& zex, std::vector<uint32_t>& ufrag,
                         std::vector<int>& uex) {
  const int pz = h.pz, px = h.px, Nz = h.Nz, X = h.X, Kk = Nz - 1;
  const double norm = 1.0 / ((3. * h.Nx / 2.) * (3. * h.Nz / 2.));
  std::vector<double> Ax((size_t)2 * X * px, 0.0), Au((size_t)2 * X * px, 0.0), Az((size_t)2 * Kk * 2 * pz, 0.0);
  for (int kx = 0; kx < X; ++kx)
    for (int xp = 0; xp < px; ++xp) {
      const int idx = (int)(((long long)kx * xp) % px);
      Au[(size_t)(2 * kx) * px + xp] = h.twx[2 * idx];           // cos
      Au[(size_t)(2 * kx + 1) * px + xp] = h.twx[2 * idx + 1];   // -sin
      Ax[(size_t)(2 * kx) * px + xp] = h.twx[2 * idx] * norm;
      Ax[(size_t)(2 * kx + 1) * px + xp] = h.twx[2 * idx + 1] * norm;
    }
  for (int kk = 0; kk < Kk; ++kk) {
    const int zo = kk < Nz / 2 ? kk : kk + 1 + Nz / 2;  // padded output row of kept index kk
    for (int zp = 0; zp < pz; ++zp) {
      const int idx = (int)(((long long)zo * zp) % pz);
      const double c = h.twz[2 * idx], ms = h.twz[2 * idx + 1];  // cos, -sin
      Az[(size_t)(2 * kk) * 2 * pz + 2 * zp] = c;
      Az[(size_t)(2 * kk) * 2 * pz + 2 * zp + 1] = -ms;
      Az[(size_t)(2 * kk + 1) * 2 * pz + 2 * zp] = ms;
      Az[(size_t)(2 * kk + 1) * 2 * pz + 2 * zp + 1] = c;
    }
  }
  xfrag.clear(); xex.clear(); zfrag.clear(); zex.clear(); ufrag.clear(); uex.clear();
  return append_digit_table(Ax.data(), 2 * X, px, (2 * X + 15) / 16, (px + 15) / 16, xfrag, xex) &&
         append_digit_table(Au.data(), 2 * X, px, (2 * X + 15) / 16, (px + 15) / 16, ufrag, uex) &&
         append_digit_table(Az.data(), 2 * Kk, 2 * pz, (2 * Kk + 15) / 16, (2 * pz + 15) / 16, zfrag, zex);
}

// ---------------------------------------------------------------------------
// shared-memory plan
// ---------------------------------------------------------------------------

__host__ __device__ inline size_t phys_tc_dbuf_bytes(const Grid& g, int fb) {
  const PhysTcDims d = phys_tc_dims(g, fb);
  const size_t z = (size_t)kDig * ((d.NZ + 7) / 8 * 8) * d.KSz * 2, x = (size_t)kDig * ((d.NX + 7) / 8 * 8) * d.KSx * 2;
  return (z > x ? z : x + 0);
}

size_t phys_tc_smem_bytes(const Grid& g, bool with_cfl, int fb) {
  const PhysTcDims d = phys_tc_dims(g, fb);
  size_t b = 0;
  b += (size_t)((d.NZ + 3) / 4 * 4) * sizeof(int);            // z-stage column exponents
  b += (size_t)((d.NX + 3) / 4 * 4) * sizeof(int);            // x-stage column exponents
  b += (phys_tc_dbuf_bytes(g, fb) + 15) / 16 * 16;             // digits (z, then x)
  b += (size_t)fb * g.pz * g.X * sizeof(cpx);                  // Z intermediate
  (void)with_cfl;  // the CFL number is read back from the written fields
  return b;
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------

__host__ __device__ constexpr size_t phys_tc_dbuf_of(const PhysTcDims& d) {
  return (size_t)kDig * ((d.NZ + 7) / 8 * 8) * d.KSz * 2 > (size_t)kDig * ((d.NX + 7) / 8 * 8) * d.KSx * 2
             ? (size_t)kDig * ((d.NZ + 7) / 8 * 8) * d.KSz * 2
             : (size_t)kDig * ((d.NX + 7) / 8 * 8) * d.KSx * 2;
}

// FB fields per pass, NTHR threads, MINB blocks per SM (the register
// budget), S the sizes (SizesRT, or SizesCT for a specialised grid)
template <bool MULTI, int MINB, int FB, int NTHR, class S>
__global__ void __launch_bounds__(NTHR, MINB) k_phys_inverse_tc(const __grid_constant__ Grid g0, PhysArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const S gsz(g);
  if (y >= gsz.Q()) return;
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  const PhysTcDims d = phys_tc_dims_n(gsz.Nz(), gsz.pz(), gsz.px(), gsz.X(), FB);
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* p = smem;
  int* exz = reinterpret_cast<int*>(p); p += (size_t)((d.NZ + 3) / 4 * 4) * sizeof(int);
  int* exx = reinterpret_cast<int*>(p); p += (size_t)((d.NX + 3) / 4 * 4) * sizeof(int);
  uint16_t* dig = reinterpret_cast<uint16_t*>(p); p += (phys_tc_dbuf_of(d) + 15) / 16 * 16;
  cpx* Zb = reinterpret_cast<cpx*>(p);  // [fl][m][x]

  const cpx* __restrict__ U = a.U.at(inst);
  double* __restrict__ P = a.P.at(inst);
  if (a.pslot.stride) P += (long long)a.pslot.slot() * a.pslot.stride;
  const size_t plane = (size_t)gsz.pz() * gsz.px();
  const uint4* __restrict__ Az = reinterpret_cast<const uint4*>(g.tcZ);
  const uint4* __restrict__ Ax = reinterpret_cast<const uint4*>(g.tcX);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  constexpr int nwarp = NTHR >> 5;
  const int Kk = gsz.Nz() - 1;  // kept kz rows
  bool nonfinite = false;
  for (int i = threadIdx.x; i < d.NZ; i += NTHR) exz[i] = 0;
  __syncthreads();
  for (int f0 = 0; f0 < a.nfields; f0 += FB) {
    const int nfb = min(FB, a.nfields - f0);
    // ---- z stage: columns n = fl * X + x.  The inputs are staged in the Z
    // buffer (free until the z stage writes it: X (Nz - 1) <= pz X values per
    // field); each thread keeps one column (consecutive threads: consecutive
    // x, coalesced loads) and its exponent maximum.  The x stage's column
    // exponents are cleared here and gathered by the z stage's epilogue.
    cpx* Fin = Zb;  // [n][kk]
    for (int i = threadIdx.x; i < d.NX; i += NTHR) exx[i] = 0;
    {
      const int ncol = nfb * gsz.X(), per = NTHR / ncol;
      if ((int)threadIdx.x < per * ncol) {
        const int n = threadIdx.x % ncol, fl = n / gsz.X(), x = n - fl * gsz.X();
        int emax = 0;
        for (int kk = threadIdx.x / ncol; kk < Kk; kk += per) {
          const int z = kk < gsz.Nz() / 2 ? kk : kk + 1;
          const cpx v = field_value_qx(g, gsz.Q(), gsz.X(), U, f0 + fl, z, y, x);
          Fin[(size_t)n * Kk + kk] = v;
          emax = max(emax, max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                               (int)((__double_as_longlong(v.im) >> 52) & 0x7FF)));
        }
        if (emax) atomicMax(&exz[n], emax);
      }
    }
    __syncthreads();
    {
      // K words (Re, Im of one mode): the even-zp modes, then the odd ones
      const int KW = d.KTz * 8;
      const size_t zstride = (size_t)((d.NZ + 7) / 8 * 8) * d.KSz / 2;  // words between digits
      uint32_t* dw = reinterpret_cast<uint32_t*>(dig);
      FlatRC rc(threadIdx.x, NTHR, KW);
      for (int i = threadIdx.x; i < d.NZ * KW; i += NTHR, rc.next()) {
        const int n = rc.r, w = rc.c;
        const int kk = g.tcZM[w];
        cpx v = {0.0, 0.0};
        if (kk >= 0 && n < nfb * gsz.X()) v = Fin[n * Kk + kk];
        const int ex = exz[n] - 1022;
        digits_pair_bf16(scaled56(v.re, ex), scaled56(v.im, ex), dw + ((size_t)n * d.KSz) / 2 + w, zstride);
      }
    }
    __syncthreads();
    {
      // rows Re Z[m], Im Z[m] for m < pzh; E + O -> Z[m], E - O -> Z[m + pzh];
      // the exponent of each value into its x-stage column (fl, m) (not the
      // imaginary part of the kx = 0 bin, which c2r ignores)
      const int NT = (nfb * gsz.X() + 7) / 8;
      const size_t dstride = (size_t)((d.NZ + 7) / 8 * 8) * d.KSz;  // bf16 between digits
      for (int item = warp; item < d.MTz * NT; item += nwarp) {
        const int mt = item / NT, nt = item - mt * NT;
        const int n = nt * 8 + gq;
        long long HE[4], LE[4], HO[4], LO[4];
        tc_tile_range(Az, mt, d.KTz, 0, d.KTzE, dig, d.KSz, dstride, n, lane, t, HE, LE);
        tc_tile_range(Az, mt, d.KTz, d.KTzE, d.KTz, dig, d.KSz, dstride, n, lane, t, HO, LO);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int row = mt * 16 + gq + 8 * (r >> 1), col = nt * 8 + 2 * t + (r & 1);
          if (row >= 2 * d.pzh || col >= nfb * gsz.X()) continue;
          const int e = g.tcZE[row] + exz[col] - 1022 - 64;
          const bool im = row >= d.pzh;
          const int m = im ? row - d.pzh : row;
          int fl = 0, x = col;  // col = fl X + x, fl < FB
          while (x >= gsz.X()) { x -= gsz.X(); ++fl; }
          const bool counts = !(im && x == 0);
          const double vp = round_col(HE[r] + HO[r], LE[r] + LO[r], e, exz[col]);
          cpx& zp = Zb[((size_t)fl * gsz.pz() + m) * gsz.X() + x];
          if (im) zp.im = vp;
          else zp.re = vp;
          const int ep = (int)((__double_as_longlong(vp) >> 52) & 0x7FF);
          if (counts && ep) atomicMax(&exx[fl * gsz.pz() + m], ep);
          if (d.Rz == 2) {
            const double vm = round_col(HE[r] - HO[r], LE[r] - LO[r], e, exz[col]);
            cpx& zm = Zb[((size_t)fl * gsz.pz() + m + d.pzh) * gsz.X() + x];
            if (im) zm.im = vm;
            else zm.re = vm;
            const int em = (int)((__double_as_longlong(vm) >> 52) & 0x7FF);
            if (counts && em) atomicMax(&exx[fl * gsz.pz() + m + d.pzh], em);
          }
        }
      }
    }
    __syncthreads();
    // ---- x stage, both fields: columns n = fl * pz + m, K words: Re, Im of
    // Z[m][j] for the even j, then the odd j (Im of j = 0 unused).  The z
    // stage's column exponents are cleared for the next pass.
    const int ncx = nfb * gsz.pz();
    const size_t xstride = (size_t)((d.NX + 7) / 8 * 8) * d.KSx;
    for (int i = threadIdx.x; i < d.NZ; i += NTHR) exz[i] = 0;
    {
      uint32_t* dw = reinterpret_cast<uint32_t*>(dig);
      const int npad = (ncx + 7) / 8 * 8, KW = d.KTx * 8, WE = d.KTxE * 8;
      FlatRC rc(threadIdx.x, NTHR, KW);
      for (int i = threadIdx.x; i < npad * KW; i += NTHR, rc.next()) {
        const int n = rc.r, w = rc.c;
        const int j = w < WE ? (w < d.nxE ? d.Rx * w : -1) : (w - WE < d.nxO ? 2 * (w - WE) + 1 : -1);
        cpx v = {0.0, 0.0};
        if (j >= 0 && n < ncx) v = Zb[(size_t)n * gsz.X() + j];
        if (j == 0) v.im = 0.0;
        const int ex = exx[min(n, ncx - 1)] - 1022;
        digits_pair_bf16(scaled56(v.re, ex), scaled56(v.im, ex), dw + ((size_t)n * d.KSx) / 2 + w, xstride / 2);
      }
    }
    __syncthreads();
    {
      // rows xp < pxh; E + O -> P[xp], E - O -> P[xp + pxh]
      const int NT = (ncx + 7) / 8;
      for (int item = warp; item < d.MTx * NT; item += nwarp) {
        const int mt = item / NT, nt = item - mt * NT;
        const int n = nt * 8 + gq;
        long long HE[4], LE[4], HO[4], LO[4];
        tc_tile_range(Ax, mt, d.KTx, 0, d.KTxE, dig, d.KSx, xstride, n, lane, t, HE, LE);
        tc_tile_range(Ax, mt, d.KTx, d.KTxE, d.KTx, dig, d.KSx, xstride, n, lane, t, HO, LO);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int xp = mt * 16 + gq + 8 * (r >> 1), col = nt * 8 + 2 * t + (r & 1);
          if (xp >= d.pxh || col >= ncx) continue;
          int fl = 0, m = col;  // col = fl pz + m, fl < FB
          while (m >= gsz.pz()) { m -= gsz.pz(); ++fl; }
          const int e = g.tcXE[xp] + exx[col] - 1022 - 64;
          double* Pr = P + ((size_t)(f0 + fl) * gsz.Q() + y) * plane + (size_t)m * gsz.px();
          const double vp = round_col(HE[r] + HO[r], LE[r] + LO[r], e, exx[col]);
          Pr[xp] = vp;
          nonfinite |= !finite_bits(vp);
          if (d.Rx == 2) {
            const double vm = round_col(HE[r] - HO[r], LE[r] - LO[r], e, exx[col]);
            Pr[xp + d.pxh] = vm;
            nonfinite |= !finite_bits(vm);
          }
        }
      }
    }
    __syncthreads();
  }
  if (nonfinite && a.status) atomicOr(&a.status[inst / a.sdiv], ST_NONFINITE);
  if (a.cfl_check) {
    // block max of the CFL field (channel/pass1.c:116-138), from the written
    // velocity fields (this block's own stores)
    __shared__ double red[NTHR];
    double mx = 0.0;
    const double* Pu = P + (size_t)y * plane;
    const size_t fs = (size_t)gsz.Q() * plane;
    const double c2 = g.cfl2[y];
    for (int i = threadIdx.x; i < gsz.pz() * gsz.px(); i += NTHR)
      mx = fmax(mx, fabs(Pu[i]) * g.cfl1 + fabs(Pu[fs + i]) * c2 + fabs(Pu[2 * fs + i]) * g.cfl3);
    red[threadIdx.x] = mx;
    __syncthreads();
    constexpr int P2 = NTHR >= 256 ? 256 : (NTHR >= 128 ? 128 : 64);  // largest power of 2 <= NTHR
    if (P2 < NTHR && threadIdx.x < NTHR - P2) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + P2]);
    if (P2 < NTHR) __syncthreads();
    for (int w = P2 / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
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
}

// ---------------------------------------------------------------------------
// products + forward transforms
// ---------------------------------------------------------------------------

static constexpr int kPB = 3;  // products computed per pass over the plane

struct FwdTcDims {
  int KTx, KTz, MTx, MTz, KSx, KSz, pzp, Xp, Kk;
};

__host__ __device__ constexpr FwdTcDims fwd_tc_dims_n(int Nz, int X, int pz, int px) {
  FwdTcDims d{};
  d.Kk = Nz - 1;
  d.KTx = (px + 15) / 16;
  d.KTz = (2 * pz + 15) / 16;
  d.MTx = (2 * X + 15) / 16;
  d.MTz = (2 * d.Kk + 15) / 16;
  d.KSx = d.KTx * 16 + 8;
  d.KSz = d.KTz * 16 + 8;
  d.pzp = (pz + 7) / 8 * 8;
  d.Xp = (X + 7) / 8 * 8;
  return d;
}

__host__ __device__ inline FwdTcDims fwd_tc_dims(const Grid& g) { return fwd_tc_dims_n(g.Nz, g.X, g.pz, g.px); }

// shared memory of a products block: pb product planes, x-stage digits of
// xch columns (a chunk), z-stage digits, exponents, the z-stage outputs
__host__ __device__ constexpr size_t fwd_tc_smem_n(int Nz, int X, int pz, int px, int pb, int xch) {
  const FwdTcDims d = fwd_tc_dims_n(Nz, X, pz, px);
  const size_t dx = (size_t)kDig * xch * d.KSx * 2, dz = (size_t)kDig * d.Xp * d.KSz * 2;
  return (size_t)(pb * ((pz + 3) / 4 * 4) + (X + 3) / 4 * 4) * sizeof(int) + ((dx > dz ? dx : dz) + 15) / 16 * 16 +
         ((size_t)pb * pz * px * sizeof(double) + 15) / 16 * 16 + (size_t)d.Kk * X * sizeof(cpx);
}

// the widest x-stage chunk (a multiple of 8 columns) with which minb blocks
// of pb planes share an SM's 228 KB (1 KB reserved per block); 8 if none
__host__ __device__ constexpr int fwd_tc_xch_n(int Nz, int X, int pz, int px, int pb, int minb) {
  const int pzp = (pz + 7) / 8 * 8;
  for (int c = pzp; c > 8; c -= 8)
    if ((size_t)minb * (fwd_tc_smem_n(Nz, X, pz, px, pb, c) + 1024 + 1024) <= 233472) return c;
  return 8;
}

// pb product planes per pass: kPB for the forward modes (0, 1); for the
// adjoint modes (2, 3, six products) Grid::adjpb: kPB (each field loaded
// once per three products) or one (a smaller footprint leaves L1 to the
// tables), as the autotuner finds faster
inline int products_per_pass(const Grid& g, int mode) {
  if (mode < 2) return g.fwdpb;
  return g.adjpb == kPB && g.fwdpb == kPB ? kPB : 1;
}

// xch: x-stage columns (padded zp rows) digitised per chunk
size_t fwd_tc_smem_bytes(const Grid& g, int pb, int xch) { return fwd_tc_smem_n(g.Nz, g.X, g.pz, g.px, pb, xch); }

// The products of one plane (mode 0 primal, 1 tangent, 2 adjoint S and T,
// 3 the exact transpose; split_product) and their forward transforms as
// digit GEMMs: the products of three components in one pass over the plane
// (each field loaded once), then the transforms one component at a time;
// modes 0/1 write H slots 0..2, modes 2/3 fold each component into the
// output slots (assemble_stage).  Same outputs as k_products_fwd /
// k_products_adj.
// S: the sizes (SizesRT, or SizesCT for a specialised grid); MINB blocks
// per SM (the register budget; with MINB > 2 the x stage runs in the chunks
// that let MINB blocks share an SM)
template <bool MULTI, int PB, class S, int MINB = 2>
__global__ void __launch_bounds__(kThreads, MINB) k_products_tc(const __grid_constant__ Grid g0, ProdArgs a, int mode) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const S gsz(g);
  if (y >= gsz.Q()) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  const FwdTcDims d = fwd_tc_dims_n(gsz.Nz(), gsz.X(), gsz.pz(), gsz.px());
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char* p = smem;
  const int exs = (gsz.pz() + 3) / 4 * 4, pb = PB;
  int* exx3 = reinterpret_cast<int*>(p); p += (size_t)pb * exs * sizeof(int);  // [c][zp]
  int* exz = reinterpret_cast<int*>(p); p += (size_t)((gsz.X() + 3) / 4 * 4) * sizeof(int);
  uint16_t* dig = reinterpret_cast<uint16_t*>(p);
  // x-stage columns per chunk: all of them in the fixed-size builds, else
  // the plan's (Grid::fxch, a multiple of 8)
  int XCH = d.pzp;
  if constexpr (MINB > 2) XCH = fwd_tc_xch_n(gsz.Nz(), gsz.X(), gsz.pz(), gsz.px(), PB, MINB);
  else if constexpr (std::is_same<S, SizesRT>::value) XCH = min(g.fxch, d.pzp);
  {
    const size_t dx = (size_t)kDig * XCH * d.KSx * 2, dz = (size_t)kDig * d.Xp * d.KSz * 2;
    p += ((dx > dz ? dx : dz) + 15) / 16 * 16;
  }
  double* stage3 = reinterpret_cast<double*>(p);  // [c][zp][xp] products; Y [zp][kx] (cpx) over plane c
  p += ((size_t)pb * gsz.pz() * gsz.px() * sizeof(double) + 15) / 16 * 16;
  cpx* Fb = reinterpret_cast<cpx*>(p);  // [kk][kx]
  const size_t plane = (size_t)gsz.pz() * gsz.px(), fs = (size_t)gsz.Q() * plane;
  const double* __restrict__ Pp = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                  (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ Pt = a.Pt.base ? a.Pt.at(inst) + (size_t)y * plane : nullptr;
  cpx* __restrict__ H = a.H.at(inst);
  // the exact transpose's forward transforms carry no 1/(px pz)
  const uint4* __restrict__ Ax = reinterpret_cast<const uint4*>(mode == 3 ? g.tcFXU : g.tcFX);
  const int* __restrict__ AxE = mode == 3 ? g.tcFXUE : g.tcFXE;
  const uint4* __restrict__ Az = reinterpret_cast<const uint4*>(g.tcFZ);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  constexpr int nwarp = kThreads >> 5;
  const int ncomp = mode >= 2 ? 6 : 3;
  const size_t xstride = (size_t)XCH * d.KSx, zstride = (size_t)d.Xp * d.KSz;  // bf16 between digits
  for (int q = 0; q < ncomp; ++q) {
    const int c = q % pb;
    double* stage = stage3 + (size_t)c * plane;
    cpx* Yb = reinterpret_cast<cpx*>(stage);
    int* exx = exx3 + c * exs;
    if (c == 0) {
      // ---- products of components q .. q+2 (each field loaded once per
      // point), row exponents (one column per zp)
      for (int i = threadIdx.x; i < pb * exs; i += kThreads) exx3[i] = 0;
      __syncthreads();
      const int nc = min(pb, ncomp - q);
      FlatRC rc(threadIdx.x, kThreads, gsz.px());
      auto point = [&](int i) {
        double v[PB];
#pragma unroll
        for (int cc = 0; cc < PB; ++cc) v[cc] = cc < nc ? split_product(mode, Pp, Pt, fs, i, q + cc) : 0.0;
        const int row = rc.r;
#pragma unroll
        for (int cc = 0; cc < PB; ++cc) {
          if (cc >= nc) break;
          stage3[(size_t)cc * plane + i] = v[cc];
          const int e = (int)((__double_as_longlong(v[cc]) >> 52) & 0x7FF);
          if (e) atomicMax(&exx3[cc * exs + row], e);
        }
      };
      if constexpr (std::is_same<S, SizesRT>::value) {
        for (int i = threadIdx.x; i < gsz.pz() * gsz.px(); i += kThreads, rc.next()) point(i);
      } else {
#pragma unroll 3
        for (int i = threadIdx.x; i < gsz.pz() * gsz.px(); i += kThreads, rc.next()) point(i);
      }
      __syncthreads();
    }
    // ---- x stage: rows 2kx (+1), columns zp, in chunks of XCH columns; Y
    // into the staging region (Y row zp lies below stage row zp, 16 X < 8 px
    // bytes per row, so a chunk's outputs only cover rows already digitised)
    for (int zc = 0; zc < d.pzp; zc += XCH) {
      const int nch = min(XCH, d.pzp - zc);
      FlatRC rcx(threadIdx.x, kThreads, d.KTx * 16);
      for (int i = threadIdx.x; i < nch * (d.KTx * 16); i += kThreads, rcx.next()) {
        const int n = zc + rcx.r, k = rcx.c;
        const double v = (n < gsz.pz() && k < gsz.px()) ? stage[(size_t)n * gsz.px() + k] : 0.0;
        digits_bf16(scaled56(v, exx[min(n, gsz.pz() - 1)] - 1022), dig + (size_t)rcx.r * d.KSx + k, xstride);
      }
      __syncthreads();
      const int NT = nch / 8;
      for (int item = warp; item < d.MTx * NT; item += nwarp) {
        const int mt = item / NT, nt = item - mt * NT;
        long long Hh[4], Ll[4];
        tc_tile(Ax, mt, d.KTx, dig, d.KSx, xstride, nt * 8 + gq, lane, t, Hh, Ll);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int row = mt * 16 + gq + 8 * (r >> 1), zp = zc + nt * 8 + 2 * t + (r & 1);
          if (row >= 2 * gsz.X() || zp >= gsz.pz()) continue;
          const double v = round_col(Hh[r], Ll[r], AxE[row] + exx[zp] - 1022 - 64, exx[zp]);
          cpx& yv = Yb[(size_t)zp * gsz.X() + (row >> 1)];
          if (row & 1) yv.im = v;
          else yv.re = v;
        }
      }
      __syncthreads();
    }
    // ---- z stage inputs: columns kx, K = 2 pz (Re, Im of Y[zp][kx] interleaved)
    for (int i = threadIdx.x; i < gsz.X(); i += kThreads) exz[i] = 0;
    __syncthreads();
    {
      FlatRC rc(threadIdx.x, kThreads, gsz.X());
      for (int i = threadIdx.x; i < gsz.pz() * gsz.X(); i += kThreads, rc.next()) {
        const cpx v = Yb[i];
        const int e = max((int)((__double_as_longlong(v.re) >> 52) & 0x7FF),
                          (int)((__double_as_longlong(v.im) >> 52) & 0x7FF));
        if (e) atomicMax(&exz[rc.c], e);
      }
    }
    __syncthreads();
    {
      uint32_t* dw = reinterpret_cast<uint32_t*>(dig);
      FlatRC rc(threadIdx.x, kThreads, d.KTz * 8);
      for (int i = threadIdx.x; i < d.Xp * (d.KTz * 8); i += kThreads, rc.next()) {
        const int n = rc.r, zp = rc.c;
        const cpx v = (n < gsz.X() && zp < gsz.pz()) ? Yb[(size_t)zp * gsz.X() + n] : cpx{0.0, 0.0};
        const int ex = exz[min(n, gsz.X() - 1)] - 1022;
        digits_pair_bf16(scaled56(v.re, ex), scaled56(v.im, ex), dw + ((size_t)n * d.KSz) / 2 + zp, zstride / 2);
      }
    }
    __syncthreads();
    // ---- z stage: rows 2kk (+1), columns kx -> Fb
    {
      const int NT = d.Xp / 8;
      for (int item = warp; item < d.MTz * NT; item += nwarp) {
        const int mt = item / NT, nt = item - mt * NT;
        long long Hh[4], Ll[4];
        tc_tile(Az, mt, d.KTz, dig, d.KSz, zstride, nt * 8 + gq, lane, t, Hh, Ll);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int row = mt * 16 + gq + 8 * (r >> 1), kx = nt * 8 + 2 * t + (r & 1);
          if (row >= 2 * d.Kk || kx >= gsz.X()) continue;
          const double v = round_col(Hh[r], Ll[r], g.tcFZE[row] + exz[kx] - 1022 - 64, exz[kx]);
          cpx& fv = Fb[(size_t)(row >> 1) * gsz.X() + kx];
          if (row & 1) fv.im = v;
          else fv.re = v;
        }
      }
    }
    __syncthreads();
    // ---- outputs (the (kk, kx) -> thread map is the same for every q)
    FlatRC rco(threadIdx.x, kThreads, gsz.X());
    for (int i = threadIdx.x; i < d.Kk * gsz.X(); i += kThreads, rco.next()) {
      const int kk = rco.r, x = rco.c;
      const int z = kk < gsz.Nz() / 2 ? kk : kk + 1;
      if (mode < 2) H[(((size_t)z * 5 + q) * gsz.Q() + y) * gsz.X() + x] = Fb[i];
      else assemble_stage(g, mode == 3, H, z, y, x, q, Fb[i]);
    }
    __syncthreads();
  }
}

// The forward products' shared-memory plan: product planes per pass of the
// forward modes (kPB, else one) and x-stage columns per chunk (the widest
// multiple of 8), the first that lets two blocks share an SM; false if none
// does (the FFT kernels then run).  48x97x48: one plane per pass, chunks of
// 24 columns, 111 KB per block.
bool fwd_tc_plan(const Grid& g, int optin, int& pb, int& xch) {
  const FwdTcDims d = fwd_tc_dims(g);
  const int pbs[2] = {kPB, 1};
  for (int p : pbs)
    for (int c = d.pzp; c >= 8; c -= 8)
      if (2 * (fwd_tc_smem_bytes(g, p, c) + 4096) <= (size_t)optin + 4096) {
        pb = p;
        xch = c;
        return true;
      }
  return false;
}

bool fwd_tc_fits(const Grid& g, int optin) {
  int pb = 0, xch = 0;
  return fwd_tc_plan(g, optin, pb, xch);
}

template <class S>
static void launch_products_sizes(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {
  const FwdTcDims d = fwd_tc_dims(g);
  const int xch = std::is_same<S, SizesRT>::value ? (g.fxch < d.pzp ? g.fxch : d.pzp) : d.pzp;
  const size_t sm = fwd_tc_smem_bytes(g, products_per_pass(g, mode), xch);
  const dim3 grid(g.Q, a.ninst);
  constexpr bool M = std::is_same<S, SizesRT>::value;  // only the run-time sizes serve uneven batches
  if (products_per_pass(g, mode) == kPB) {
    if (M && a.grids) k_products_tc<true, kPB, SizesRT><<<grid, kThreads, sm, st>>>(g, a, mode);
    else k_products_tc<false, kPB, S><<<grid, kThreads, sm, st>>>(g, a, mode);
  } else {
    if (M && a.grids) k_products_tc<true, 1, SizesRT><<<grid, kThreads, sm, st>>>(g, a, mode);
    else k_products_tc<false, 1, S><<<grid, kThreads, sm, st>>>(g, a, mode);
  }
}

// Grid::prodb 1 (single-grid batches): two product planes per pass at 3
// blocks per SM (80 registers), the x stage in the chunks that fit
template <class S>
static void launch_products_b3(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {
  const dim3 grid(g.Q, a.ninst);
  const size_t sm = fwd_tc_smem_bytes(g, 2, fwd_tc_xch_n(g.Nz, g.X, g.pz, g.px, 2, 3));
  k_products_tc<false, 2, S, 3><<<grid, kThreads, sm, st>>>(g, a, mode);
}

// Grid::fixed & FIXED_PRODUCTS: the build compiled for the grid's sizes
// (32x65x32, 16x33x16; single-grid batches), else the run-time sizes
cudaError_t launch_products_tc(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {
  if (g.prodb == 1 && !a.grids) {
    const bool fx = (g.fixed & FIXED_PRODUCTS) != 0;
    if (fx && sizes_match<Sizes32>(g)) launch_products_b3<Sizes32>(g, a, mode, st);
    else if (fx && sizes_match<Sizes16>(g)) launch_products_b3<Sizes16>(g, a, mode, st);
    else launch_products_b3<SizesRT>(g, a, mode, st);
    return cudaGetLastError();
  }
  const bool fx = (g.fixed & FIXED_PRODUCTS) && !a.grids && g.fxch >= fwd_tc_dims(g).pzp;
  if (fx && sizes_match<Sizes32>(g)) launch_products_sizes<Sizes32>(g, a, mode, st);
  else if (fx && sizes_match<Sizes16>(g)) launch_products_sizes<Sizes16>(g, a, mode, st);
  else launch_products_sizes<SizesRT>(g, a, mode, st);
  return cudaGetLastError();
}

bool phys_tc_fits(const Grid& g, int optin) {
  // the kernel's static shared memory (reduction, staged grid) is below 4 KB;
  // the input staging keeps one thread per z-stage column (the widest build's
  // plan; the one-field builds need less)
  return kFB * g.X <= kThreads && phys_tc_smem_bytes(g, true, kFB) + 4096 <= (size_t)optin;
}

// Builds of the kernel (Grid::tcminb; the autotuner times them, the results
// are identical): fields per pass, threads, blocks per SM (the register
// budget) and the sizes, run-time (RT) or compiled for the grid (CT):
//   2: 2 fields, 256 threads, 2 blocks, RT   3: the same at 3 blocks
//   4: 1 field, 128 threads, 4 blocks, RT    5: the same at 5 blocks
//   6: build 4, CT                           7: build 2, CT
//   8: 1 field, 192 threads, 3 blocks, RT    9: build 8, CT
//  10: 1 field, 128 threads, 5 blocks, CT   11: 192 threads, 4 blocks, CT
//  12: 1 field, 256 threads, 3 blocks, CT
// One field per pass halves the shared memory; 192 threads give the z
// stage's six output tiles of a field one warp each; the compiled sizes
// need fewer registers (96 at 5 blocks of 128 threads without spills).
template <bool MULTI>
static void launch_inverse_build(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  const dim3 grid(g.Q, a.ninst);
  const bool cfl = a.cfl_check != 0;
  const size_t s2 = phys_tc_smem_bytes(g, cfl, 2), s1 = phys_tc_smem_bytes(g, cfl, 1);
  using RT = SizesRT;
  switch (g.tcminb) {
    case 3: k_phys_inverse_tc<MULTI, 3, 2, 256, RT><<<grid, 256, s2, st>>>(g, a); break;
    case 4: k_phys_inverse_tc<MULTI, 4, 1, 128, RT><<<grid, 128, s1, st>>>(g, a); break;
    case 5: k_phys_inverse_tc<MULTI, 5, 1, 128, RT><<<grid, 128, s1, st>>>(g, a); break;
    case 8: k_phys_inverse_tc<MULTI, 3, 1, 192, RT><<<grid, 192, s1, st>>>(g, a); break;
    default: k_phys_inverse_tc<MULTI, 2, 2, 256, RT><<<grid, 256, s2, st>>>(g, a); break;
  }
}

bool phys_tc_specialised(const Grid& g) { return sizes_match<Sizes32>(g) || sizes_match<Sizes16>(g); }

// the run-time-size build a compile-time one stands for
static int inverse_rt_build(int b) {
  switch (b) {
    case 6: return 4;
    case 7: return 2;
    case 9: case 11: case 12: return 8;
    case 10: return 5;
    default: return b;
  }
}
static bool inverse_ct_build(int b) { return b == 6 || b == 7 || b >= 9; }

template <class S>
static void launch_inverse_ct(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  const dim3 grid(g.Q, a.ninst);
  const bool cfl = a.cfl_check != 0;
  const size_t s1 = phys_tc_smem_bytes(g, cfl, 1);
  switch (g.tcminb) {
    case 6: k_phys_inverse_tc<false, 4, 1, 128, S><<<grid, 128, s1, st>>>(g, a); break;
    case 9: k_phys_inverse_tc<false, 3, 1, 192, S><<<grid, 192, s1, st>>>(g, a); break;
    case 10: k_phys_inverse_tc<false, 5, 1, 128, S><<<grid, 128, s1, st>>>(g, a); break;
    case 11: k_phys_inverse_tc<false, 4, 1, 192, S><<<grid, 192, s1, st>>>(g, a); break;
    case 12: k_phys_inverse_tc<false, 3, 1, 256, S><<<grid, 256, s1, st>>>(g, a); break;
    default: k_phys_inverse_tc<false, 2, 2, 256, S><<<grid, 256, phys_tc_smem_bytes(g, cfl, 2), st>>>(g, a); break;
  }
}

cudaError_t launch_phys_inverse_tc(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  const bool ct = inverse_ct_build(g.tcminb) && !a.grids;
  if (ct && sizes_match<Sizes32>(g)) {
    launch_inverse_ct<Sizes32>(g, a, st);
  } else if (ct && sizes_match<Sizes16>(g)) {
    launch_inverse_ct<Sizes16>(g, a, st);
  } else {
    Grid gr = g;
    gr.tcminb = inverse_rt_build(g.tcminb);
    if (a.grids) launch_inverse_build<true>(gr, a, st);
    else launch_inverse_build<false>(gr, a, st);
  }
  return cudaGetLastError();
}

void prepare_phys_tc(int optin) {
  using RT = SizesRT;
  allow_max_smem(k_phys_inverse_tc<false, 2, 2, 256, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<true, 2, 2, 256, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 2, 256, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<true, 3, 2, 256, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 4, 1, 128, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<true, 4, 1, 128, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 5, 1, 128, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<true, 5, 1, 128, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 4, 1, 128, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 2, 2, 256, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 4, 1, 128, Sizes16>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 1, 192, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<true, 3, 1, 192, RT>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 1, 192, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 1, 192, Sizes16>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 5, 1, 128, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 4, 1, 192, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 1, 256, Sizes32>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 5, 1, 128, Sizes16>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 4, 1, 192, Sizes16>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 3, 1, 256, Sizes16>, optin);
  allow_max_smem(k_phys_inverse_tc<false, 2, 2, 256, Sizes16>, optin);
  allow_max_smem(k_products_tc<false, kPB, RT>, optin);
  allow_max_smem(k_products_tc<true, kPB, RT>, optin);
  allow_max_smem(k_products_tc<false, 1, RT>, optin);
  allow_max_smem(k_products_tc<true, 1, RT>, optin);
  allow_max_smem(k_products_tc<false, kPB, Sizes32>, optin);
  allow_max_smem(k_products_tc<false, 2, SizesRT, 3>, optin);
  allow_max_smem(k_products_tc<false, 2, Sizes32, 3>, optin);
  allow_max_smem(k_products_tc<false, 2, Sizes16, 3>, optin);
  allow_max_smem(k_products_tc<false, 1, Sizes32>, optin);
  allow_max_smem(k_products_tc<false, kPB, Sizes16>, optin);
  allow_max_smem(k_products_tc<false, 1, Sizes16>, optin);
}

}  // namespace chn
