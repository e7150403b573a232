// Physical-space kernels: one thread block per (instance, y-plane).
//
//   k_phys_inverse   velocity (and spectral vorticity) -> physical fields on
//                    the 3/2-padded (pz x px) grid; optional CFL check.
//                    channel/pass1.c:42-138, channel/spec2phys.c:39-76
//   k_products_fwd   u x w (primal) or u x Iw + Iu x w (tangent), then the
//                    forward transform, truncation and 1/(px pz) scaling.
//                    channel/pass1.c:212-371
//   k_products_adj   S = u x lambda, T = lambda x w, forward transforms and
//                    the assembly H = -T + (i k) x S, keeping S_x, S_z.
//                    channel/pass2.c:224-566
//
// Every transform is an FP64 shared-memory Stockham FFT (fft.cuh).  The x
// transforms of two real rows share one complex FFT (row pairs packed as
// a + i b), so no real-to-complex post-processing pass is needed.
#include <algorithm>

#include "chn_common.cuh"
#include "fft.cuh"
#include "kernels.h"

namespace chn {

static constexpr int kThreads = 256;

__device__ __forceinline__ bool blocked(const uint32_t* status, int sdiv, int inst) {
  return status != nullptr && (status[inst / sdiv] & ST_CFL) != 0;
}

// spectral value of physical field f at (z, x) on plane y: f = 0..2 velocity,
// 3 = wz, 4 = wx, 5 = wy (channel/pass1.c:58-104)
__device__ __forceinline__ cpx field_value(const Grid& g, const cpx* __restrict__ U, int f, int z, int y, int x) {
  auto at = [&](int c) { return U[(((size_t)z * 5 + c) * g.Q + y) * g.X + x]; };
  cpx r;
  if (f < 3) return at(f);
  const double kx = g.Kx[x], kz = g.Kz[z];
  if (f == 3) {  // wz = -(du/dy ... ) : -(DX + i kx v)
    cpx dx = at(3), v = at(1);
    r.re = -(dx.re + kx * v.im);
    r.im = -dx.im + kx * v.re;
  } else if (f == 4) {  // wx = DZ - i kz v
    cpx dz = at(4), v = at(1);
    r.re = dz.re + kz * v.im;
    r.im = dz.im - kz * v.re;
  } else {  // wy = i kz u - i kx w
    cpx u = at(0), w = at(2);
    r.re = kx * w.im - kz * u.im;
    r.im = kz * u.re - kx * w.re;
  }
  return r;
}

struct PhysSmem {
  cpx *twz, *twx, *zb0, *zb1, *xb0, *xb1;
  double* cfl;
};

__device__ inline PhysSmem carve(const Grid& g, unsigned char* base, bool with_cfl) {
  PhysSmem s;
  const int npair = (g.pz + 1) / 2;
  cpx* p = reinterpret_cast<cpx*>(base);
  s.twz = p; p += g.pz;
  s.twx = p; p += g.px;
  s.zb0 = p; p += (size_t)g.pz * g.X;
  s.zb1 = p; p += (size_t)g.pz * g.X;
  s.xb0 = p; p += (size_t)npair * g.px;
  s.xb1 = p; p += (size_t)npair * g.px;
  s.cfl = with_cfl ? reinterpret_cast<double*>(p) : nullptr;
  return s;
}

__host__ __device__ inline size_t phys_smem_hd(const Grid& g, bool with_cfl) {
  const int npair = (g.pz + 1) / 2;
  size_t n = (size_t)g.pz + g.px + 2 * (size_t)g.pz * g.X + 2 * (size_t)npair * g.px;
  size_t b = n * sizeof(cpx);
  if (with_cfl) b += (size_t)g.pz * g.px * sizeof(double);
  return b;
}

size_t phys_smem_bytes(const Grid& g, bool with_cfl) { return phys_smem_hd(g, with_cfl); }

__device__ inline void load_tw(const Grid& g, PhysSmem& s) {
  for (int i = threadIdx.x; i < g.pz; i += blockDim.x) s.twz[i] = g.twz[i];
  for (int i = threadIdx.x; i < g.px; i += blockDim.x) s.twx[i] = g.twx[i];
}

// padded spectral row zp -> unpadded kz index, or -1 for the zero band
__device__ __forceinline__ int zrow_to_kz(const Grid& g, int zp) {
  if (zp < g.Nz / 2) return zp;
  if (zp > g.Nz) return zp - g.Nz / 2;
  return -1;
}

template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_phys_inverse(const __grid_constant__ Grid g0, PhysArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, a.cfl_check != 0);
  load_tw(g, s);
  const cpx* __restrict__ U = a.U.at(inst);
  double* __restrict__ P = a.P.at(inst);
  if (a.pslot.stride) P += (long long)a.pslot.slot() * a.pslot.stride;
  const FftPlan pz_plan = make_plan(g.pz, true);
  const FftPlan px_plan = make_plan(g.px, true);
  const int npair = (g.pz + 1) / 2;
  const size_t plane = (size_t)g.pz * g.px;
  bool nonfinite = false;
  for (int f = 0; f < a.nfields; ++f) {
    for (int i = threadIdx.x; i < g.pz * g.X; i += blockDim.x) {
      const int zp = i / g.X, x = i - zp * g.X;
      const int z = zrow_to_kz(g, zp);
      cpx v = {0.0, 0.0};
      if (z >= 0) v = field_value(g, U, f, z, y, x);
      s.zb0[i] = v;
    }
    __syncthreads();
    cpx* zr = fft_run(pz_plan, s.zb0, s.zb1, g.X, g.X, 1, s.twz, +1, true);
    // pack rows (2p, 2p+1) as A + iB with the Hermitian extension in x
    for (int i = threadIdx.x; i < npair * g.px; i += blockDim.x) {
      const int p = i / g.px, k = i - p * g.px;
      const int ra = 2 * p, rb = 2 * p + 1;
      cpx Z = {0.0, 0.0};
      int kk = -1;
      bool conj = false;
      if (k < g.X) kk = k;
      else if (k > g.px - g.X) { kk = g.px - k; conj = true; }
      if (kk >= 0) {
        cpx A = zr[ra * g.X + kk];
        cpx B = rb < g.pz ? zr[rb * g.X + kk] : cpx{0.0, 0.0};
        if (kk == 0) {  // c2r ignores the imaginary part of the DC bin
          Z.re = A.re; Z.im = B.re;
        } else if (!conj) {
          Z.re = A.re - B.im; Z.im = A.im + B.re;
        } else {
          Z.re = A.re + B.im; Z.im = B.re - A.im;
        }
      }
      s.xb0[i] = Z;
    }
    __syncthreads();
    cpx* xr = fft_run(px_plan, s.xb0, s.xb1, npair, 1, g.px, s.twx, +1, true);
    double* Pf = P + ((size_t)f * g.Q + y) * plane;
    for (int i = threadIdx.x; i < g.pz * g.px; i += blockDim.x) {
      const int zp = i / g.px, xp = i - zp * g.px;
      const cpx c = xr[(zp >> 1) * g.px + xp];
      const double v = (zp & 1) ? c.im : c.re;
      Pf[i] = v;
      nonfinite |= !isfinite(v);
      if (a.cfl_check && f < 3) {
        const double t = fabs(v) * (f == 0 ? g.cfl1 : (f == 1 ? g.cfl2[y] : g.cfl3));
        if (f == 0) s.cfl[i] = t;
        else s.cfl[i] = s.cfl[i] + t;
      }
    }
    __syncthreads();
  }
  if (nonfinite && a.status) atomicOr(&a.status[inst / a.sdiv], ST_NONFINITE);
  if (a.cfl_check) {
    // block max of the CFL field (channel/pass1.c:116-138)
    __shared__ double red[kThreads];
    double m = 0.0;
    for (int i = threadIdx.x; i < g.pz * g.px; i += blockDim.x) m = fmax(m, s.cfl[i]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double cfl = red[0] * g.dt;
      if (a.cflmax) atomicMax(reinterpret_cast<unsigned long long*>(&a.cflmax[inst / a.sdiv]),
                              (unsigned long long)__double_as_longlong(cfl));
      if (cfl >= 2.8) atomicOr(&a.status[inst / a.sdiv], ST_CFL);
    }
  }
}

// products: component c in {0: Hz, 1: Hx, 2: Hy} at flat offset o of plane y
__device__ __forceinline__ double prod_primal(const double* __restrict__ P, size_t fs, size_t o, int c) {
  const double u = P[o], v = P[fs + o], w = P[2 * fs + o];
  const double wz = P[3 * fs + o], wx = P[4 * fs + o], wy = P[5 * fs + o];
  if (c == 0) return u * wy - v * wx;
  if (c == 1) return v * wz - w * wy;
  return w * wx - u * wz;
}

__device__ __forceinline__ double prod_tangent(const double* __restrict__ P, const double* __restrict__ I,
                                               size_t fs, size_t o, int c) {
  const double u = P[o], v = P[fs + o], w = P[2 * fs + o];
  const double wz = P[3 * fs + o], wx = P[4 * fs + o], wy = P[5 * fs + o];
  const double iu = I[o], iv = I[fs + o], iw = I[2 * fs + o];
  const double iwz = I[3 * fs + o], iwx = I[4 * fs + o], iwy = I[5 * fs + o];
  if (c == 0) return iu * wy - iv * wx + u * iwy - v * iwx;
  if (c == 1) return iv * wz - iw * wy + v * iwz - w * iwy;
  return iw * wx - iu * wz + w * iwx - u * iwz;
}

// forward transform of the product rows held in xb0; leaves the kept,
// scaled spectral rows in the returned z buffer
__device__ inline cpx* forward_plane(const Grid& g, PhysSmem& s, const FftPlan& pxF, const FftPlan& pzF) {
  const int npair = (g.pz + 1) / 2;
  cpx* xr = fft_run(pxF, s.xb0, s.xb1, npair, 1, g.px, s.twx, -1, true);
  const double hn = 0.5 * g.norm;
  for (int i = threadIdx.x; i < npair * g.X; i += blockDim.x) {
    const int p = i / g.X, k = i - p * g.X;
    const cpx Zk = xr[p * g.px + k];
    const cpx Zn = xr[p * g.px + (k == 0 ? 0 : g.px - k)];
    cpx A, B;
    A.re = (Zk.re + Zn.re) * hn;
    A.im = (Zk.im - Zn.im) * hn;
    B.re = (Zk.im + Zn.im) * hn;
    B.im = (Zn.re - Zk.re) * hn;
    s.zb0[(2 * p) * g.X + k] = A;
    if (2 * p + 1 < g.pz) s.zb0[(2 * p + 1) * g.X + k] = B;
  }
  __syncthreads();
  return fft_run(pzF, s.zb0, s.zb1, g.X, g.X, 1, s.twz, -1, true);
}

template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_products_fwd(const __grid_constant__ Grid g0, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, false);
  load_tw(g, s);
  const size_t plane = (size_t)g.pz * g.px, fs = (size_t)g.Q * plane;
  const double* __restrict__ Pp = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                  (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ Pt = a.Pt.base ? a.Pt.at(inst) + (size_t)y * plane : nullptr;
  cpx* __restrict__ H = a.H.at(inst);
  const FftPlan pxF = make_plan(g.px, false);
  const FftPlan pzF = make_plan(g.pz, false);
  const int npair = (g.pz + 1) / 2;
  __syncthreads();
  for (int c = 0; c < 3; ++c) {
    for (int i = threadIdx.x; i < npair * g.px; i += blockDim.x) {
      const int p = i / g.px, xp = i - p * g.px;
      const size_t oa = (size_t)(2 * p) * g.px + xp, ob = oa + g.px;
      cpx z;
      z.re = Pt ? prod_tangent(Pp, Pt, fs, oa, c) : prod_primal(Pp, fs, oa, c);
      z.im = 0.0;
      if (2 * p + 1 < g.pz) z.im = Pt ? prod_tangent(Pp, Pt, fs, ob, c) : prod_primal(Pp, fs, ob, c);
      s.xb0[i] = z;
    }
    __syncthreads();
    cpx* zr = forward_plane(g, s, pxF, pzF);
    for (int i = threadIdx.x; i < g.pz * g.X; i += blockDim.x) {
      const int zp = i / g.X, x = i - zp * g.X;
      const int z = zrow_to_kz(g, zp);
      if (z >= 0) H[(((size_t)z * 5 + c) * g.Q + y) * g.X + x] = zr[i];
    }
    __syncthreads();
  }
}

size_t prod_adj_smem_bytes(const Grid& g) {
  return phys_smem_bytes(g, false) + (size_t)6 * g.Nz * g.X * sizeof(cpx);
}

template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_products_adj(const __grid_constant__ Grid g0, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, false);
  cpx* keep = reinterpret_cast<cpx*>(smem + phys_smem_hd(g, false));  // [6][Nz][X]
  load_tw(g, s);
  const size_t plane = (size_t)g.pz * g.px, fs = (size_t)g.Q * plane;
  const double* __restrict__ P = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                 (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ L = a.Pt.at(inst) + (size_t)y * plane;  // lambda: 3 fields
  cpx* __restrict__ H = a.H.at(inst);
  const FftPlan pxF = make_plan(g.px, false);
  const FftPlan pzF = make_plan(g.pz, false);
  const int npair = (g.pz + 1) / 2;
  __syncthreads();
  // q = 0..2: S_x, S_y, S_z = u x lambda; q = 3..5: T_x, T_y, T_z = lambda x w
  for (int q = 0; q < 6; ++q) {
    for (int i = threadIdx.x; i < npair * g.px; i += blockDim.x) {
      const int p = i / g.px, xp = i - p * g.px;
      double val[2] = {0.0, 0.0};
      for (int h = 0; h < 2; ++h) {
        if (2 * p + h >= g.pz) break;
        const size_t o = (size_t)(2 * p + h) * g.px + xp;
        const double u = P[o], v = P[fs + o], w = P[2 * fs + o];
        const double wz = P[3 * fs + o], wx = P[4 * fs + o], wy = P[5 * fs + o];
        const double lx = L[o], ly = L[fs + o], lz = L[2 * fs + o];
        double r;
        switch (q) {
          case 0: r = v * lz - w * ly; break;
          case 1: r = w * lx - u * lz; break;
          case 2: r = u * ly - v * lx; break;
          case 3: r = ly * wz - lz * wy; break;
          case 4: r = lz * wx - lx * wz; break;
          default: r = lx * wy - ly * wx; break;
        }
        val[h] = r;
      }
      s.xb0[i] = cpx{val[0], val[1]};
    }
    __syncthreads();
    cpx* zr = forward_plane(g, s, pxF, pzF);
    for (int i = threadIdx.x; i < g.pz * g.X; i += blockDim.x) {
      const int zp = i / g.X, x = i - zp * g.X;
      const int z = zrow_to_kz(g, zp);
      if (z >= 0) keep[((size_t)q * g.Nz + z) * g.X + x] = zr[i];
    }
    __syncthreads();
  }
  // H = -T + (i kz S_y, -i kz S_x + i kx S_z, -i kx S_y); keep S_x, S_z
  for (int i = threadIdx.x; i < g.Nz * g.X; i += blockDim.x) {
    const int z = i / g.X, x = i - z * g.X;
    if (z == g.Nz / 2) continue;
    const double kx = g.Kx[x], kz = g.Kz[z];
    const cpx Sx = keep[(0 * g.Nz + z) * g.X + x], Sy = keep[(1 * g.Nz + z) * g.X + x];
    const cpx Sz = keep[(2 * g.Nz + z) * g.X + x], Tx = keep[(3 * g.Nz + z) * g.X + x];
    const cpx Ty = keep[(4 * g.Nz + z) * g.X + x], Tz = keep[(5 * g.Nz + z) * g.X + x];
    cpx hx, hy, hz;
    hx.re = -Tx.re - kz * Sy.im;
    hx.im = -Tx.im + kz * Sy.re;
    hy.re = -Ty.re + kz * Sx.im - kx * Sz.im;
    hy.im = -Ty.im - kz * Sx.re + kx * Sz.re;
    hz.re = -Tz.re + kx * Sy.im;
    hz.im = -Tz.im - kx * Sy.re;
    auto slot = [&](int c) -> cpx& { return H[(((size_t)z * 5 + c) * g.Q + y) * g.X + x]; };
    slot(0) = hz;
    slot(1) = hx;
    slot(2) = hy;
    slot(3) = Sx;
    slot(4) = Sz;
  }
}

// ---------------------------------------------------------------------------
// split transforms: for grids whose padded plane does not fit one block's
// shared memory (128x129x128: a 192 x 192 plane), every 2D transform runs as
// a z pass over chunks of Nx/2 columns and an x pass over chunks of row
// pairs, with the spectral columns in an HBM intermediate
// T[inst][c][Q][pz][Nx/2].  Each 1D transform is the same fft_run call on the
// same data as in the fused kernels, so results are identical bit for bit.
// ---------------------------------------------------------------------------

static constexpr int kCols = 16;     // z pass: columns per block
static constexpr int kColsAdj = 8;   // adjoint z pass (keeps 6 spectra per column)
static constexpr int kPairs = 16;    // x pass: row pairs per block

size_t split_tmp_elems(const Grid& g) { return (size_t)6 * g.Q * g.pz * g.X; }

static size_t split_z_smem(const Grid& g, int ncol, int nkeep) {
  return ((size_t)g.pz + 2 * (size_t)g.pz * ncol + (size_t)nkeep * g.Nz * ncol) * sizeof(cpx);
}
static size_t split_x_smem(const Grid& g, bool with_cfl) {
  size_t b = ((size_t)g.px + 2 * (size_t)kPairs * g.px) * sizeof(cpx);
  if (with_cfl) b += (size_t)2 * kPairs * g.px * sizeof(double);
  return b;
}

bool fused_transforms_fit(const Grid& g, int smem_optin) {
  const size_t room = (size_t)smem_optin - 4096;  // static shared memory of the kernels (reductions, grid)
  return phys_smem_bytes(g, true) <= room && prod_adj_smem_bytes(g) <= room;
}

// inverse z pass: spectral fields f0..f0+nf-1 -> T (channel/pass1.c:107-110)
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_split_zinv(const __grid_constant__ Grid g0, PhysArgs a, int inst0,
                                                         int nf, cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int nck = (g0.X + kCols - 1) / kCols;
  const int f = blockIdx.z / nck, x0 = (blockIdx.z - f * nck) * kCols;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q || x0 >= g.X) return;
  const int nc = min(kCols, g.X - x0);
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.pz;
  cpx* b1 = b0 + (size_t)g.pz * kCols;
  for (int i = threadIdx.x; i < g.pz; i += blockDim.x) tw[i] = g.twz[i];
  const cpx* __restrict__ U = a.U.at(inst);
  for (int i = threadIdx.x; i < g.pz * nc; i += blockDim.x) {
    const int zp = i / nc, c = i - zp * nc;
    const int z = zrow_to_kz(g, zp);
    b0[i] = z >= 0 ? field_value(g, U, f, z, y, x0 + c) : cpx{0.0, 0.0};
  }
  __syncthreads();
  const FftPlan plan = make_plan(g.pz, true);
  const cpx* zr = fft_run(plan, b0, b1, nc, nc, 1, tw, +1, true);
  cpx* Tf = T + (((size_t)il * nf + f) * g0.Q + y) * g0.pz * g0.X;
  for (int i = threadIdx.x; i < g.pz * nc; i += blockDim.x) {
    const int zp = i / nc, c = i - zp * nc;
    Tf[(size_t)zp * g.X + x0 + c] = zr[i];
  }
}

// inverse x pass: row pairs of T -> physical rows of P, CFL of the velocity
// (channel/pass1.c:111-138)
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_split_xinv(const __grid_constant__ Grid g0, PhysArgs a, int inst0,
                                                         int nf, const cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int npair = (g.pz + 1) / 2;
  const int p0 = blockIdx.z * kPairs;
  if (y >= g.Q || p0 >= npair) return;
  const int np = min(kPairs, npair - p0);
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.px;
  cpx* b1 = b0 + (size_t)kPairs * g.px;
  double* cfl = reinterpret_cast<double*>(b1 + (size_t)kPairs * g.px);
  for (int i = threadIdx.x; i < g.px; i += blockDim.x) tw[i] = g.twx[i];
  double* __restrict__ P = a.P.at(inst);
  if (a.pslot.stride) P += (long long)a.pslot.slot() * a.pslot.stride;
  const FftPlan plan = make_plan(g.px, true);
  const size_t plane = (size_t)g.pz * g.px;
  const int r0 = 2 * p0, nr = min(2 * np, g.pz - r0);
  bool nonfinite = false;
  for (int f = 0; f < nf; ++f) {
    const cpx* zr = T + (((size_t)il * nf + f) * g0.Q + y) * g0.pz * g0.X;
    for (int i = threadIdx.x; i < np * g.px; i += blockDim.x) {
      const int pl = i / g.px, k = i - pl * g.px;
      const int ra = 2 * (p0 + pl), rb = ra + 1;
      cpx Z = {0.0, 0.0};
      int kk = -1;
      bool conj = false;
      if (k < g.X) kk = k;
      else if (k > g.px - g.X) { kk = g.px - k; conj = true; }
      if (kk >= 0) {
        const cpx A = zr[(size_t)ra * g.X + kk];
        const cpx B = rb < g.pz ? zr[(size_t)rb * g.X + kk] : cpx{0.0, 0.0};
        if (kk == 0) {
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
    const cpx* xr = fft_run(plan, b0, b1, np, 1, g.px, tw, +1, true);
    double* Pf = P + ((size_t)f * g.Q + y) * plane;
    for (int i = threadIdx.x; i < nr * g.px; i += blockDim.x) {
      const int rl = i / g.px, xp = i - rl * g.px;
      const cpx c = xr[(rl >> 1) * g.px + xp];
      const double v = (rl & 1) ? c.im : c.re;
      Pf[(size_t)(r0 + rl) * g.px + xp] = v;
      nonfinite |= !isfinite(v);
      if (a.cfl_check && f < 3) {
        const double t = fabs(v) * (f == 0 ? g.cfl1 : (f == 1 ? g.cfl2[y] : g.cfl3));
        cfl[i] = f == 0 ? t : cfl[i] + t;
      }
    }
    __syncthreads();
  }
  if (nonfinite && a.status) atomicOr(&a.status[inst / a.sdiv], ST_NONFINITE);
  if (a.cfl_check) {
    __shared__ double red[kThreads];
    double m = 0.0;
    for (int i = threadIdx.x; i < nr * g.px; i += blockDim.x) m = fmax(m, cfl[i]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double c = red[0] * g.dt;
      if (a.cflmax) atomicMax(reinterpret_cast<unsigned long long*>(&a.cflmax[inst / a.sdiv]),
                              (unsigned long long)__double_as_longlong(c));
      if (c >= 2.8) atomicOr(&a.status[inst / a.sdiv], ST_CFL);
    }
  }
}

// product component q at flat offset o of plane y: mode 0 primal, 1 tangent,
// 2 adjoint (q = 0..2 S = u x lambda, 3..5 T = lambda x w)
__device__ __forceinline__ double split_product(int mode, const double* __restrict__ P,
                                                const double* __restrict__ I, size_t fs, size_t o, int q) {
  if (mode == 0) return prod_primal(P, fs, o, q);
  if (mode == 1) return prod_tangent(P, I, fs, o, q);
  const double u = P[o], v = P[fs + o], w = P[2 * fs + o];
  const double wz = P[3 * fs + o], wx = P[4 * fs + o], wy = P[5 * fs + o];
  const double lx = I[o], ly = I[fs + o], lz = I[2 * fs + o];
  switch (q) {
    case 0: return v * lz - w * ly;
    case 1: return w * lx - u * lz;
    case 2: return u * ly - v * lx;
    case 3: return ly * wz - lz * wy;
    case 4: return lz * wx - lx * wz;
    default: return lx * wy - ly * wx;
  }
}

// forward x pass: products of row pairs, x transform, kept bins -> T
// (channel/pass1.c:312-330, pass2.c:474-500)
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_split_xfwd(const __grid_constant__ Grid g0, ProdArgs a, int mode,
                                                         int inst0, cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  const int npair = (g.pz + 1) / 2;
  const int p0 = blockIdx.z * kPairs;
  if (y >= g.Q || p0 >= npair) return;
  const int np = min(kPairs, npair - p0);
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.px;
  cpx* b1 = b0 + (size_t)kPairs * g.px;
  for (int i = threadIdx.x; i < g.px; i += blockDim.x) tw[i] = g.twx[i];
  const size_t plane = (size_t)g.pz * g.px, fs = (size_t)g.Q * plane;
  const double* __restrict__ Pp = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                  (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ Pt = a.Pt.base ? a.Pt.at(inst) + (size_t)y * plane : nullptr;
  const FftPlan plan = make_plan(g.px, false);
  const int ncomp = mode == 2 ? 6 : 3;
  const double hn = 0.5 * g.norm;
  __syncthreads();
  for (int q = 0; q < ncomp; ++q) {
    for (int i = threadIdx.x; i < np * g.px; i += blockDim.x) {
      const int pl = i / g.px, xp = i - pl * g.px;
      const int ra = 2 * (p0 + pl);
      const size_t oa = (size_t)ra * g.px + xp, ob = oa + g.px;
      cpx z;
      z.re = split_product(mode, Pp, Pt, fs, oa, q);
      z.im = ra + 1 < g.pz ? split_product(mode, Pp, Pt, fs, ob, q) : 0.0;
      b0[i] = z;
    }
    __syncthreads();
    const cpx* xr = fft_run(plan, b0, b1, np, 1, g.px, tw, -1, true);
    cpx* Tq = T + (((size_t)il * ncomp + q) * g0.Q + y) * g0.pz * g0.X;
    for (int i = threadIdx.x; i < np * g.X; i += blockDim.x) {
      const int pl = i / g.X, k = i - pl * g.X;
      const cpx Zk = xr[pl * g.px + k];
      const cpx Zn = xr[pl * g.px + (k == 0 ? 0 : g.px - k)];
      cpx A, B;
      A.re = (Zk.re + Zn.re) * hn;
      A.im = (Zk.im - Zn.im) * hn;
      B.re = (Zk.im + Zn.im) * hn;
      B.im = (Zn.re - Zk.re) * hn;
      const int ra = 2 * (p0 + pl);
      Tq[(size_t)ra * g.X + k] = A;
      if (ra + 1 < g.pz) Tq[(size_t)(ra + 1) * g.X + k] = B;
    }
    __syncthreads();
  }
}

// forward z pass: columns of T, z transform, truncation -> H; the adjoint
// assembles H = -T + (i k) x S and keeps S_x, S_z (channel/pass1.c:331-371,
// pass2.c:501-566)
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_split_zfwd(const __grid_constant__ Grid g0, ProdArgs a, int mode,
                                                         int inst0, const cpx* T) {
  const int y = blockIdx.x, il = blockIdx.y, inst = inst0 + il;
  const int ncol = mode == 2 ? kColsAdj : kCols;
  const int x0 = blockIdx.z * ncol;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q || x0 >= g.X) return;
  const int nc = min(ncol, g.X - x0);
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  cpx* tw = reinterpret_cast<cpx*>(smem);
  cpx* b0 = tw + g.pz;
  cpx* b1 = b0 + (size_t)g.pz * ncol;
  cpx* keep = b1 + (size_t)g.pz * ncol;  // adjoint: [6][Nz][ncol]
  for (int i = threadIdx.x; i < g.pz; i += blockDim.x) tw[i] = g.twz[i];
  cpx* __restrict__ H = a.H.at(inst);
  const FftPlan plan = make_plan(g.pz, false);
  const int ncomp = mode == 2 ? 6 : 3;
  for (int q = 0; q < ncomp; ++q) {
    const cpx* Tq = T + (((size_t)il * ncomp + q) * g0.Q + y) * g0.pz * g0.X;
    for (int i = threadIdx.x; i < g.pz * nc; i += blockDim.x) {
      const int zp = i / nc, c = i - zp * nc;
      b0[i] = Tq[(size_t)zp * g.X + x0 + c];
    }
    __syncthreads();
    const cpx* zr = fft_run(plan, b0, b1, nc, nc, 1, tw, -1, true);
    for (int i = threadIdx.x; i < g.pz * nc; i += blockDim.x) {
      const int zp = i / nc, c = i - zp * nc;
      const int z = zrow_to_kz(g, zp);
      if (z < 0) continue;
      if (mode == 2) keep[((size_t)q * g.Nz + z) * ncol + c] = zr[i];
      else H[(((size_t)z * 5 + q) * g.Q + y) * g.X + x0 + c] = zr[i];
    }
    __syncthreads();
  }
  if (mode != 2) return;
  for (int i = threadIdx.x; i < g.Nz * nc; i += blockDim.x) {
    const int z = i / nc, c = i - z * nc, x = x0 + c;
    if (z == g.Nz / 2) continue;
    const double kx = g.Kx[x], kz = g.Kz[z];
    auto K = [&](int q) { return keep[((size_t)q * g.Nz + z) * ncol + c]; };
    const cpx Sx = K(0), Sy = K(1), Sz = K(2), Tx = K(3), Ty = K(4), Tz = K(5);
    cpx hx, hy, hz;
    hx.re = -Tx.re - kz * Sy.im;
    hx.im = -Tx.im + kz * Sy.re;
    hy.re = -Ty.re + kz * Sx.im - kx * Sz.im;
    hy.im = -Ty.im - kz * Sx.re + kx * Sz.re;
    hz.re = -Tz.re + kx * Sy.im;
    hz.im = -Tz.im - kx * Sy.re;
    auto slot = [&](int s) -> cpx& { return H[(((size_t)z * 5 + s) * g.Q + y) * g.X + x]; };
    slot(0) = hz;
    slot(1) = hx;
    slot(2) = hy;
    slot(3) = Sx;
    slot(4) = Sz;
  }
}

// instance chunks that fit the intermediate
template <typename F>
static cudaError_t split_chunks(int ninst, int cap, F&& body) {
  if (cap <= 0) return cudaErrorInvalidValue;
  for (int i0 = 0; i0 < ninst; i0 += cap) {
    const cudaError_t e = body(i0, min(cap, ninst - i0));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static cudaError_t split_phys_inverse(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  if (!a.tmp) return cudaErrorInvalidValue;
  const int cap = a.tmp_inst * 6 / a.nfields;
  return split_chunks(a.ninst, cap, [&](int i0, int n) {
    const int nck = (g.X + kCols - 1) / kCols, npc = ((g.pz + 1) / 2 + kPairs - 1) / kPairs;
    const dim3 gz(g.Q, n, a.nfields * nck), gx(g.Q, n, npc);
    const size_t sz = split_z_smem(g, kCols, 0), sx = split_x_smem(g, a.cfl_check != 0);
    if (a.grids) {
      k_split_zinv<true><<<gz, kThreads, sz, st>>>(g, a, i0, a.nfields, a.tmp);
      k_split_xinv<true><<<gx, kThreads, sx, st>>>(g, a, i0, a.nfields, a.tmp);
    } else {
      k_split_zinv<false><<<gz, kThreads, sz, st>>>(g, a, i0, a.nfields, a.tmp);
      k_split_xinv<false><<<gx, kThreads, sx, st>>>(g, a, i0, a.nfields, a.tmp);
    }
    return cudaGetLastError();
  });
}

static cudaError_t split_products(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st) {
  if (!a.tmp) return cudaErrorInvalidValue;
  const int ncomp = mode == 2 ? 6 : 3;
  const int cap = a.tmp_inst * 6 / ncomp;
  return split_chunks(a.ninst, cap, [&](int i0, int n) {
    const int npc = ((g.pz + 1) / 2 + kPairs - 1) / kPairs;
    const int ncol = mode == 2 ? kColsAdj : kCols, nck = (g.X + ncol - 1) / ncol;
    const dim3 gx(g.Q, n, npc), gz(g.Q, n, nck);
    const size_t sx = split_x_smem(g, false), sz = split_z_smem(g, ncol, mode == 2 ? 6 : 0);
    if (a.grids) {
      k_split_xfwd<true><<<gx, kThreads, sx, st>>>(g, a, mode, i0, a.tmp);
      k_split_zfwd<true><<<gz, kThreads, sz, st>>>(g, a, mode, i0, a.tmp);
    } else {
      k_split_xfwd<false><<<gx, kThreads, sx, st>>>(g, a, mode, i0, a.tmp);
      k_split_zfwd<false><<<gz, kThreads, sz, st>>>(g, a, mode, i0, a.tmp);
    }
    return cudaGetLastError();
  });
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

cudaError_t launch_phys_inverse(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.split) return split_phys_inverse(g, a, st);
  const size_t sm = phys_smem_bytes(g, a.cfl_check != 0);
  if (a.grids) k_phys_inverse<true><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  else k_phys_inverse<false><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_fwd(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.split) return split_products(g, a, a.Pt.base ? 1 : 0, st);
  const size_t sm = phys_smem_bytes(g, false);
  if (a.grids) k_products_fwd<true><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  else k_products_fwd<false><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_adj(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.split) return split_products(g, a, 2, st);
  const size_t sm = prod_adj_smem_bytes(g);
  if (a.grids) k_products_adj<true><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  else k_products_adj<false><<<dim3(g.Q, a.ninst), kThreads, sm, st>>>(g, a);
  return cudaGetLastError();
}

void prepare_recon_solve(int optin);

// Every kernel may use up to the device's opt-in shared memory per block: the
// single-grid engine and an uneven batch (sized for its largest grid) share
// the kernels, so the limit is not tied to one grid.
template <bool MULTI>
static void prepare_transforms(int optin) {
  allow_max_smem(k_split_zinv<MULTI>, optin);
  allow_max_smem(k_split_xinv<MULTI>, optin);
  allow_max_smem(k_split_xfwd<MULTI>, optin);
  allow_max_smem(k_split_zfwd<MULTI>, optin);
  allow_max_smem(k_phys_inverse<MULTI>, optin);
  allow_max_smem(k_products_fwd<MULTI>, optin);
  allow_max_smem(k_products_adj<MULTI>, optin);
}

void prepare_kernels(const Grid& g) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  (void)g;
  prepare_transforms<false>(optin);
  prepare_transforms<true>(optin);
  prepare_recon_solve(optin);
}

}  // namespace chn
