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

__global__ void __launch_bounds__(kThreads) k_phys_inverse(Grid g, PhysArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
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

__global__ void __launch_bounds__(kThreads) k_products_fwd(Grid g, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
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

__global__ void __launch_bounds__(kThreads) k_products_adj(Grid g, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
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
// launchers
// ---------------------------------------------------------------------------

cudaError_t launch_phys_inverse(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  k_phys_inverse<<<dim3(g.Q, a.ninst), kThreads, phys_smem_bytes(g, a.cfl_check != 0), st>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_fwd(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  k_products_fwd<<<dim3(g.Q, a.ninst), kThreads, phys_smem_bytes(g, false), st>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_adj(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  k_products_adj<<<dim3(g.Q, a.ninst), kThreads, prod_adj_smem_bytes(g), st>>>(g, a);
  return cudaGetLastError();
}

void prepare_recon_solve(const Grid& g);

void prepare_kernels(const Grid& g) {
  cudaFuncSetAttribute(k_phys_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)phys_smem_bytes(g, true));
  cudaFuncSetAttribute(k_products_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)phys_smem_bytes(g, false));
  cudaFuncSetAttribute(k_products_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)prod_adj_smem_bytes(g));
  prepare_recon_solve(g);
}

}  // namespace chn
