// Device helpers shared by the fused and the split transform kernels.
#pragma once

#include "chn_common.cuh"

namespace chn {

__device__ __forceinline__ bool blocked(const uint32_t* status, int sdiv, int inst) {
  return status != nullptr && (status[inst / sdiv] & ST_CFL) != 0;
}

// spectral value of physical field f at (z, x) on plane y: f = 0..2 velocity,
// 3 = wz, 4 = wx, 5 = wy (channel/pass1.c:58-104)
// (Q, X: the grid's plane count and kx columns, compile-time constants in
// the specialised transform kernels)
__device__ __forceinline__ cpx field_value_qx(const Grid& g, int Q, int X, const cpx* __restrict__ U, int f, int z,
                                              int y, int x) {
  auto at = [&](int c) { return U[(((size_t)z * 5 + c) * Q + y) * X + x]; };
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

__device__ __forceinline__ cpx field_value(const Grid& g, const cpx* __restrict__ U, int f, int z, int y, int x) {
  return field_value_qx(g, g.Q, g.X, U, f, z, y, x);
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

// the transpose of the tangent products (channel/pass1.c:145-170) with
// respect to the tangent fields: n = (nz, nx, ny) the cotangents of the
// products Hz, Hx, Hy (fields 0..2 of N); q = 0..5 the cotangents of
// u, v, w, wz, wx, wy
__device__ __forceinline__ double prod_transpose(const double* __restrict__ P, const double* __restrict__ N,
                                                 size_t fs, size_t o, int q) {
  const double nz = N[o], nx = N[fs + o], ny = N[2 * fs + o];
  switch (q) {
    case 0: return nz * P[5 * fs + o] - ny * P[3 * fs + o];   // u:  nz wy - ny wz
    case 1: return nx * P[3 * fs + o] - nz * P[4 * fs + o];   // v:  nx wz - nz wx
    case 2: return ny * P[4 * fs + o] - nx * P[5 * fs + o];   // w:  ny wx - nx wy
    case 3: return nx * P[fs + o] - ny * P[o];                // wz: nx v - ny u
    case 4: return ny * P[2 * fs + o] - nz * P[fs + o];       // wx: ny w - nz v
    default: return nz * P[o] - nx * P[2 * fs + o];           // wy: nz u - nx w
  }
}

// product component q at flat offset o of plane y: mode 0 primal, 1 tangent,
// 2 adjoint (q = 0..2 S = u x lambda, 3..5 T = lambda x w), 3 the exact
// transpose of the tangent products
__device__ __forceinline__ double split_product(int mode, const double* __restrict__ P,
                                                const double* __restrict__ I, size_t fs, size_t o, int q) {
  if (mode == 0) return prod_primal(P, fs, o, q);
  if (mode == 1) return prod_tangent(P, I, fs, o, q);
  if (mode == 3) return prod_transpose(P, I, fs, o, q);
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

// The adjoint's output slots assembled one forward-transformed product at
// a time, so a kernel needs no buffer for all six: stage q folds product q
// into the slots it feeds, reading the partial sums earlier stages stored
// (the same thread owns an output element through all six stages).
//   reference adjoint (channel/pass2.c:501-566), products S_x, S_y, S_z,
//   T_x, T_y, T_z:  H = -T + (i kz S_y, -i kz S_x + i kx S_z, -i kx S_y)
//   in slots Hx 1, Hy 2, Hz 0, keeping S_x, S_z in slots 3, 4;
//   exact transpose (`exact`), products t0..t5 = the cotangents of
//   u, v, w, wz, wx, wy (the transpose of the vorticity load,
//   channel/pass1.c:58-104), times 2 off the kx = 0 column (the transposed
//   complex-to-real x transform):
//   u = t0 - i kz t5,  v = t1 - i kx t3 + i kz t4,  w = t2 + i kx t5,
//   du/dy = -t3,  dw/dy = t4.
// Explicit roundings (no contraction) make every kernel that uses this
// produce the same bits.
__device__ __forceinline__ void assemble_stage(const Grid& g, bool exact, cpx* __restrict__ H, int z, int y, int x,
                                               int q, cpx t) {
  const double kx = g.Kx[x], kz = g.Kz[z];
  auto slot = [&](int c) -> cpx& { return H[(((size_t)z * 5 + c) * g.Q + y) * g.X + x]; };
  auto scale = [](double a, cpx v) { return cpx{__dmul_rn(a, v.re), __dmul_rn(a, v.im)}; };
  auto add = [](cpx a, cpx b) { return cpx{__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; };
  auto sub = [](cpx a, cpx b) { return cpx{__dsub_rn(a.re, b.re), __dsub_rn(a.im, b.im)}; };
  auto imul = [](double k, cpx v) { return cpx{__dmul_rn(-k, v.im), __dmul_rn(k, v.re)}; };  // i k v
  if (!exact) {
    switch (q) {
      case 0: slot(3) = t; slot(2) = imul(-kz, t); break;                   // S_x
      case 1: slot(1) = imul(kz, t); slot(0) = imul(-kx, t); break;          // S_y
      case 2: slot(4) = t; slot(2) = add(slot(2), imul(kx, t)); break;      // S_z
      case 3: slot(1) = sub(slot(1), t); break;                             // T_x
      case 4: slot(2) = sub(slot(2), t); break;                             // T_y
      default: slot(0) = sub(slot(0), t); break;                            // T_z
    }
    return;
  }
  const double f = x == 0 ? 1.0 : 2.0;
  switch (q) {
    case 0: slot(0) = scale(f, t); break;
    case 1: slot(1) = scale(f, t); break;
    case 2: slot(2) = scale(f, t); break;
    case 3: slot(1) = add(slot(1), scale(f, imul(-kx, t))); slot(3) = scale(-f, t); break;
    case 4: slot(1) = add(slot(1), scale(f, imul(kz, t))); slot(4) = scale(f, t); break;
    default:
      slot(0) = add(slot(0), scale(f, imul(-kz, t)));
      slot(2) = add(slot(2), scale(f, imul(kx, t)));
      break;
  }
}

}  // namespace chn
