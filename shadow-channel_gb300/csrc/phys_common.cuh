// Device helpers shared by the fused and the split transform kernels.
#pragma once

#include "chn_common.cuh"

namespace chn {

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

// padded spectral row zp -> unpadded kz index, or -1 for the zero band
__device__ __forceinline__ int zrow_to_kz(const Grid& g, int zp) {
  if (zp < g.Nz / 2) return zp;
  if (zp > g.Nz) return zp - g.Nz / 2;
  return -1;
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

// the adjoint's assembly H = -T + (i kz S_y, -i kz S_x + i kx S_z, -i kx S_y),
// keeping S_x, S_z (channel/pass2.c:501-566)
__device__ __forceinline__ void adjoint_assemble(const Grid& g, cpx* __restrict__ H, int z, int y, int x,
                                                 cpx Sx, cpx Sy, cpx Sz, cpx Tx, cpx Ty, cpx Tz) {
  const double kx = g.Kx[x], kz = g.Kz[z];
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

}  // namespace chn
