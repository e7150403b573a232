// Coefficients -> velocity (channel/initAlphaBeta2.c:12-240) on the tensor
// cores, exact to the FP64 rounding of its result.
//
// The reconstruction is five real contractions per (kz, kx) column,
//   v = Q alpha, Q' alpha, Q'' alpha, g = R beta, R' beta   (Q planes each),
// followed by the K-algebra that mixes them into u, w, du/dy, dw/dy.  On
// GB300 the FP64 pipe (1.2 TFLOP/s) bounds the direct form; here each
// contraction runs as a bf16 tensor-core GEMM on integer digits:
//   - every basis row (plane y) and every coefficient column is scaled by a
//     power of two into an integer of 56 significant bits, written as seven
//     balanced base-256 digits (the top digit in [-256, 256], the others in
//     [-128, 127]); digits are exact in bf16;
//   - digit products of level l = i + k accumulate in FP32 through
//     mma.sync m16n8k16 (bf16 inputs, FP32 accumulator).  With K <= 112
//     terms a level's partial sums stay below 2^24, so FP32 holds them
//     exactly;
//   - levels l < 7 are kept (the rest lie below 2^-56 of the operands'
//     scale), recombined exactly in 64-bit integers and rounded once to FP64
//     by one fma.
// Only the rounding, the K-algebra and the (kx, kz) = (0, 0) mean mode
// (computed directly) use the FP64 pipe.  Results agree with the FP64
// contraction to its own rounding.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "chn_common.cuh"
#include "kernels.h"
#include "setup.h"
#include "tc_common.cuh"
#include "sizes.cuh"

namespace chn {

static constexpr int kThreads = 256;
static constexpr int kTile = 16;   // kx columns per block (32 real columns: re, im interleaved)
static constexpr int kReconRegs = 8;  // coefficient rows a thread keeps in registers per class (R <= 128)

// ---------------------------------------------------------------------------
// host: basis digit tables in mma A-fragment order
// ---------------------------------------------------------------------------

bool append_digit_table(const double* M, int rows, int K, int MT, int KT, std::vector<uint32_t>& frag,
                        std::vector<int>& ex) {
  const size_t base = frag.size();
  frag.resize(base + (size_t)MT * KT * kDig * 32 * 4, 0u);
  const size_t ebase = ex.size();
  ex.resize(ebase + rows, -1022);
  std::vector<int> dig((size_t)rows * (KT * 16) * kDig, 0);
  for (int y = 0; y < rows; ++y) {
    double mx = 0.0;
    for (int j = 0; j < K; ++j) mx = std::fmax(mx, std::fabs(M[(size_t)y * K + j]));
    if (mx == 0.0) continue;
    int e = 0;
    std::frexp(mx, &e);  // |M[y][j]| < 2^e
    ex[ebase + y] = e;
    for (int j = 0; j < K; ++j) {
      const long long x = std::llround(std::ldexp(M[(size_t)y * K + j], 56 - e));
      digits56(x, &dig[((size_t)y * (KT * 16) + j) * kDig]);
    }
  }
  auto at = [&](int y, int k, int i) -> uint16_t {
    if (y >= rows || k >= K) return 0;
    return bf16_bits_of_int(dig[((size_t)y * (KT * 16) + k) * kDig + i]);
  };
  for (int mt = 0; mt < MT; ++mt)
    for (int kt = 0; kt < KT; ++kt)
      for (int i = 0; i < kDig; ++i)
        for (int lane = 0; lane < 32; ++lane) {
          const int g = lane >> 2, t = lane & 3;
          const int r0 = mt * 16 + g, r1 = r0 + 8, k0 = kt * 16 + 2 * t;
          uint32_t* f = &frag[base + ((((size_t)mt * KT + kt) * kDig + i) * 32 + lane) * 4];
          f[0] = (uint32_t)at(r0, k0, i) | ((uint32_t)at(r0, k0 + 1, i) << 16);
          f[1] = (uint32_t)at(r1, k0, i) | ((uint32_t)at(r1, k0 + 1, i) << 16);
          f[2] = (uint32_t)at(r0, k0 + 8, i) | ((uint32_t)at(r0, k0 + 9, i) << 16);
          f[3] = (uint32_t)at(r1, k0 + 8, i) | ((uint32_t)at(r1, k0 + 9, i) << 16);
        }
  return true;
}

// the five bases [Q][D or R] (rows: planes) and the five weighted
// transposes [D or R][Q] (rows: basis index) as digit tables
bool build_recon_tc_tables(const HostTables& h, std::vector<uint32_t>& frag, std::vector<int>& ex,
                           std::vector<uint32_t>& wfrag, std::vector<int>& wex) {
  const int MT = (h.Q + 15) / 16, KT = (h.R + 15) / 16;
  const std::vector<double>* B[5] = {&h.Bq, &h.Bqp, &h.Bqpp, &h.Br, &h.Brp};
  frag.clear();
  ex.clear();
  for (int b = 0; b < 5; ++b)
    if (!append_digit_table(B[b]->data(), h.Q, b < 3 ? h.D : h.R, MT, KT, frag, ex)) return false;
  const int MTw = (h.R + 15) / 16, KTw = (h.Q + 15) / 16;
  const std::vector<double>* W[5] = {&h.Wq, &h.Wqp, &h.Wqpp, &h.Wr, &h.Wrp};
  wfrag.clear();
  wex.clear();
  for (int b = 0; b < 5; ++b) {
    // rows padded to R so that every table has MTw row tiles and R exponents
    std::vector<double> m((size_t)h.R * h.Q, 0.0);
    const int rows = b < 3 ? h.D : h.R;
    std::copy(W[b]->begin(), W[b]->begin() + (size_t)rows * h.Q, m.begin());
    if (!append_digit_table(m.data(), h.R, h.Q, MTw, KTw, wfrag, wex)) return false;
  }
  return true;
}

// the exact adjoint's tables: the bases transposed ([D or R][Q], rows
// padded to R) for Recon^T, and the weighted transposes of Qpw, Qw, Rw
// turned plane-major ([Q][D or R], columns padded to R) for Quad^T
bool build_adj_tc_tables(const HostTables& h, std::vector<uint32_t>& btfrag, std::vector<int>& btex,
                         std::vector<uint32_t>& wtfrag, std::vector<int>& wtex) {
  const int MTw = (h.R + 15) / 16, KTq = (h.Q + 15) / 16;
  const std::vector<double>* B[5] = {&h.Bq, &h.Bqp, &h.Bqpp, &h.Br, &h.Brp};
  btfrag.clear();
  btex.clear();
  for (int b = 0; b < 5; ++b) {
    const int cols = b < 3 ? h.D : h.R;  // B[b] is [Q][cols]
    std::vector<double> m((size_t)h.R * h.Q, 0.0);
    for (int i = 0; i < cols; ++i)
      for (int y = 0; y < h.Q; ++y) m[(size_t)i * h.Q + y] = (*B[b])[(size_t)y * cols + i];
    if (!append_digit_table(m.data(), h.R, h.Q, MTw, KTq, btfrag, btex)) return false;
  }
  const std::vector<double>* W[3] = {&h.Wqp, &h.Wq, &h.Wr};  // [D or R][Q]
  wtfrag.clear();
  wtex.clear();
  for (int b = 0; b < 3; ++b) {
    const int rows = b < 2 ? h.D : h.R;
    std::vector<double> m((size_t)h.Q * h.R, 0.0);
    for (int y = 0; y < h.Q; ++y)
      for (int i = 0; i < rows; ++i) m[(size_t)y * h.R + i] = (*W[b])[(size_t)i * h.Q + y];
    if (!append_digit_table(m.data(), h.Q, h.R, KTq, MTw, wtfrag, wtex)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// device
// ---------------------------------------------------------------------------

__host__ __device__ inline int recon_tc_kstride(int KT) { return KT * 16 + 8; }  // bf16 per digit row (padded)

// tile: kx columns per block (16 or 8)
size_t recon_tc_smem_bytes(const Grid& g, int tile) {
  const int KT = (g.R + 15) / 16;
  return (size_t)2 * kDig * (2 * tile) * recon_tc_kstride(KT) * sizeof(uint16_t) + 2 * tile * sizeof(int);
}

size_t recon_tc_smem_bytes(const Grid& g) { return recon_tc_smem_bytes(g, kTile); }

// S: the sizes (SizesRT, or SizesCT for a specialised grid); TILE kx
// columns per block (2 TILE real digit columns) in NTHR = 16 TILE threads
template <bool MULTI, class S, int TILE = kTile, int NTHR = kThreads, int MINB = 2>
__global__ void __launch_bounds__(NTHR, MINB) k_recon_tc(const __grid_constant__ Grid g0, ReconArgs a) {
  const int ntx = (g0.X + TILE - 1) / TILE;
  const int z = blockIdx.x / ntx, tx = blockIdx.x - z * ntx;
  const int inst = blockIdx.y;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const S gsz(g);
  if (z >= gsz.Nz() || tx * TILE >= gsz.X()) return;
  if (z == gsz.Nz() / 2) return;  // never read (channel/pass1.c:51-85 skips it)
  if (a.status != nullptr && (a.status[inst / a.sdiv] & ST_CFL) != 0) return;
  const int x0 = tx * TILE;
  const int nx = min(TILE, gsz.X() - x0);
  const int KT = (gsz.R() + 15) / 16, KS = recon_tc_kstride(KT), MT = (gsz.Q() + 15) / 16;
  const bool meancol = (z == 0 && x0 == 0);  // column 0 of this tile is the mean mode
  extern __shared__ __align__(16) unsigned char smem[];
  uint16_t* dig = reinterpret_cast<uint16_t*>(smem);  // [cls][digit][n 2 TILE][KS]
  int* exc = reinterpret_cast<int*>(smem + (size_t)2 * kDig * (2 * TILE) * KS * sizeof(uint16_t));  // [cls][TILE]
  const cpx* __restrict__ C = a.C.at(inst);
  if (a.slot.stride) C += (long long)a.slot.slot() * a.slot.stride;
  auto cval = [&](int cls, int j, int col) -> cpx {
    const int K = cls == 0 ? gsz.D() : gsz.R();
    if (j >= K || col >= nx || (meancol && col == 0)) return cpx{0.0, 0.0};
    return C[(((size_t)z * 2 + cls) * gsz.R() + j) * gsz.X() + x0 + col];
  };
  // column exponents: |c| < 2^exc over the column's real and imaginary parts
  for (int i = threadIdx.x; i < 2 * TILE; i += NTHR) exc[i] = 0;
  __syncthreads();
  const int nent = 2 * (KT * 16) * TILE;
  if (KT <= kReconRegs && NTHR == 16 * TILE) {
    // thread t holds column t % TILE, rows t / TILE + 16 k of both classes:
    // its coefficients stay in registers from the exponent maxima to the digits
    const int col = threadIdx.x % TILE, j0 = threadIdx.x / TILE;
    cpx vin[2][kReconRegs];
    int emax[2] = {0, 0};
#pragma unroll
    for (int cls = 0; cls < 2; ++cls)
#pragma unroll
      for (int k = 0; k < kReconRegs; ++k) {
        vin[cls][k] = k < KT ? cval(cls, j0 + 16 * k, col) : cpx{0.0, 0.0};
        emax[cls] = max(emax[cls], max((int)((__double_as_longlong(vin[cls][k].re) >> 52) & 0x7FF),
                                       (int)((__double_as_longlong(vin[cls][k].im) >> 52) & 0x7FF)));
      }
#pragma unroll
    for (int cls = 0; cls < 2; ++cls)
      if (emax[cls]) atomicMax(&exc[cls * TILE + col], emax[cls]);
    __syncthreads();
#pragma unroll
    for (int cls = 0; cls < 2; ++cls) {
      const int ex = exc[cls * TILE + col] - 1022;
#pragma unroll
      for (int k = 0; k < kReconRegs; ++k) {
        if (k >= KT) break;
        for (int p = 0; p < 2; ++p)  // digit q of column n at dig[((cls * 7 + q) * 2 TILE + n) * KS + j]
          digits_bf16(scaled56(p ? vin[cls][k].im : vin[cls][k].re, ex),
                      dig + ((size_t)cls * kDig * (2 * TILE) + 2 * col + p) * KS + j0 + 16 * k, (size_t)(2 * TILE) * KS);
      }
    }
  } else {
    for (int i = threadIdx.x; i < nent; i += NTHR) {
      const int cls = i / ((KT * 16) * TILE), r = i - cls * (KT * 16) * TILE, j = r / TILE, col = r - j * TILE;
      const cpx v = cval(cls, j, col);
      const int e1 = (int)((__double_as_longlong(v.re) >> 52) & 0x7FF);
      const int e2 = (int)((__double_as_longlong(v.im) >> 52) & 0x7FF);
      const int e = max(e1, e2);
      if (e) atomicMax(&exc[cls * TILE + col], e);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nent; i += NTHR) {
      const int cls = i / ((KT * 16) * TILE), r = i - cls * (KT * 16) * TILE, j = r / TILE, col = r - j * TILE;
      const cpx v = cval(cls, j, col);
      const int ex = exc[cls * TILE + col] - 1022;
      for (int p = 0; p < 2; ++p)  // digit q of column n at dig[((cls * 7 + q) * 2 TILE + n) * KS + j]
        digits_bf16(scaled56(p ? v.im : v.re, ex), dig + ((size_t)cls * kDig * (2 * TILE) + 2 * col + p) * KS + j,
                    (size_t)(2 * TILE) * KS);
    }
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gq = lane >> 2, t = lane & 3;
  const int NT = (2 * nx + 7) / 8;  // n-tiles of 8 real columns (4 complex)
  const uint4* __restrict__ A = reinterpret_cast<const uint4*>(g.tcA);
  cpx* __restrict__ U = a.U.at(inst);
  const size_t cs = (size_t)gsz.Q() * gsz.X();
  const int order[5] = {0, 1, 3, 2, 4};
  for (int item = warp; item < MT * NT; item += NTHR >> 5) {
    const int mt = item / NT, nt = item - mt * NT;
    const int col = nt * 4 + t;  // this thread's complex column
    const int n = nt * 8 + gq;   // the B-fragment column this thread loads
    cpx held[2];                 // Q' alpha, then Q'' alpha, at rows gq and gq + 8
    for (int ob = 0; ob < 5; ++ob) {
      const int b = order[ob], cls = b < 3 ? 0 : 1;
      const int KTb = ((cls == 0 ? gsz.D() : gsz.R()) + 15) / 16;
      const int ecol = exc[cls * TILE + col] - 1022;
      long long H[4], L[4];
      if constexpr (MINB > 2)
        tc_tile_range(A + (size_t)b * MT * KT * kDig * 32, mt, KT, 0, KTb, dig + (size_t)cls * kDig * (2 * TILE) * KS,
                      KS, (size_t)(2 * TILE) * KS, n, lane, t, H, L);
      else
        tc_tile_pf(A + (size_t)b * MT * KT * kDig * 32, mt, KT, KTb, dig + (size_t)cls * kDig * (2 * TILE) * KS, KS,
                   (size_t)(2 * TILE) * KS, n, lane, t, H, L);
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        const int y = mt * 16 + gq + 8 * rr;
        if (y >= gsz.Q() || col >= nx || (meancol && col == 0)) continue;
        const int e = g.tcE[(size_t)b * gsz.Q() + y] + ecol - 64;
        const cpx val = {round_col(H[2 * rr], L[2 * rr], e, ecol + 1022),
                         round_col(H[2 * rr + 1], L[2 * rr + 1], e, ecol + 1022)};
        const int x = x0 + col;
        cpx* out = U + ((size_t)z * 5 * gsz.Q() + y) * gsz.X() + x;
        const double ax = g.kxK2[(size_t)z * gsz.X() + x], az = g.kzK2[(size_t)z * gsz.X() + x];
        if (b == 0) {
          out[cs] = val;  // v = Q alpha
        } else if (b == 1 || b == 2) {
          held[rr] = val;
        } else if (b == 3) {
          // u = (kx Im f + kz Im g)/K2 - i (kx Re f + kz Re g)/K2 etc., f = -Q' alpha
          const cpx f = {-held[rr].re, -held[rr].im}, gg = val;
          out[0] = cpx{fma(ax, f.im, az * gg.im), -fma(ax, f.re, az * gg.re)};
          out[2 * cs] = cpx{fma(-ax, gg.im, az * f.im), fma(ax, gg.re, -az * f.re)};
        } else {
          const cpx qpp = held[rr], rp = val;
          out[3 * cs] = cpx{fma(-ax, qpp.im, az * rp.im), fma(ax, qpp.re, -az * rp.re)};
          out[4 * cs] = cpx{-fma(ax, rp.im, az * qpp.im), fma(ax, rp.re, az * qpp.re)};
        }
      }
    }
  }
  if (meancol) {
    // (kx, kz) = (0, 0): u = R a, du = R' a, v = 0, w = R b, dw = R' b
    // (channel/initAlphaBeta2.c:25-68), direct FP64
    for (int y = threadIdx.x; y < gsz.Q(); y += NTHR) {
      double ur = 0, ui = 0, dur = 0, dui = 0, wr = 0, wi = 0, dwr = 0, dwi = 0;
      for (int j = 0; j < gsz.R(); ++j) {
        const double r = __ldg(g.Br + (size_t)y * gsz.R() + j), rp = __ldg(g.Brp + (size_t)y * gsz.R() + j);
        const cpx al = C[((size_t)0 * gsz.R() + j) * gsz.X()], be = C[((size_t)1 * gsz.R() + j) * gsz.X()];
        ur = fma(r, al.re, ur); ui = fma(r, al.im, ui);
        dur = fma(rp, al.re, dur); dui = fma(rp, al.im, dui);
        wr = fma(r, be.re, wr); wi = fma(r, be.im, wi);
        dwr = fma(rp, be.re, dwr); dwi = fma(rp, be.im, dwi);
      }
      cpx* out = U + (size_t)y * gsz.X();
      out[0] = cpx{ur, ui};
      out[cs] = cpx{0.0, 0.0};
      out[2 * cs] = cpx{wr, wi};
      out[3 * cs] = cpx{dur, dui};
      out[4 * cs] = cpx{dwr, dwi};
    }
  }
}

// Grid::rbuild (single-grid batches) 0: 16-column tiles in 256-thread
// blocks at 2 per SM; 1: 8-column tiles in 128-thread blocks at 4; 2:
// 16-column tiles at 3 per SM, the table fragments loaded without prefetch
// (80 registers)
template <class S>
static void launch_recon_sizes(const Grid& g, const ReconArgs& a, cudaStream_t st) {
  if (g.rbuild == 1 && !a.grids) {
    const int ntx = (g.X + 7) / 8;
    k_recon_tc<false, S, 8, 128, 4><<<dim3(g.Nz * ntx, a.ninst), 128, recon_tc_smem_bytes(g, 8), st>>>(g, a);
    return;
  }
  if (g.rbuild == 2 && !a.grids) {
    const int ntx = (g.X + kTile - 1) / kTile;
    k_recon_tc<false, S, 16, 256, 3><<<dim3(g.Nz * ntx, a.ninst), 256, recon_tc_smem_bytes(g), st>>>(g, a);
    return;
  }
  const int ntx = (g.X + kTile - 1) / kTile;
  const size_t sm = recon_tc_smem_bytes(g);
  if (a.grids) k_recon_tc<true, SizesRT><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
  else k_recon_tc<false, S><<<dim3(g.Nz * ntx, a.ninst), kThreads, sm, st>>>(g, a);
}

// Grid::fixed & FIXED_RECON: the build compiled for the grid's sizes
cudaError_t launch_recon_tc(const Grid& g, const ReconArgs& a, cudaStream_t st) {
  const bool fx = (g.fixed & FIXED_RECON) && !a.grids;
  if (fx && sizes_match<Sizes32>(g)) launch_recon_sizes<Sizes32>(g, a, st);
  else if (fx && sizes_match<Sizes16>(g)) launch_recon_sizes<Sizes16>(g, a, st);
  else launch_recon_sizes<SizesRT>(g, a, st);
  return cudaGetLastError();
}

void prepare_recon_tc(int optin) {
  allow_max_smem(k_recon_tc<false, SizesRT>, optin);
  allow_max_smem(k_recon_tc<true, SizesRT>, optin);
  allow_max_smem(k_recon_tc<false, Sizes32>, optin);
  allow_max_smem(k_recon_tc<false, Sizes16>, optin);
  allow_max_smem(k_recon_tc<false, SizesRT, 16, 256, 3>, optin);
  allow_max_smem(k_recon_tc<false, Sizes32, 16, 256, 3>, optin);
  allow_max_smem(k_recon_tc<false, Sizes16, 16, 256, 3>, optin);
  allow_max_smem(k_recon_tc<false, SizesRT, 8, 128, 4>, optin);
  allow_max_smem(k_recon_tc<false, Sizes32, 8, 128, 4>, optin);
  allow_max_smem(k_recon_tc<false, Sizes16, 8, 128, 4>, optin);
}

}  // namespace chn
