// Small kernels: physical-flow layout, the ddt_project pieces, the laminar
// start projection, the device step counter and the FP64 throughput probe.
#include "chn_common.cuh"
#include "kernels.h"

namespace chn {

// flow[d][xp][y][zp] = P[d][y][zp][xp]  (channel/spec2phys.c:78-87)
__global__ void k_flow_out(Grid g, const double* __restrict__ P, double* __restrict__ flow) {
  const int d = blockIdx.z, y = blockIdx.y;
  const size_t plane = (size_t)g.pz * g.px;
  const double* src = P + ((size_t)d * g.Q + y) * plane;
  double* dst = flow + (size_t)d * g.px * g.Q * g.pz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.pz * g.px; i += gridDim.x * blockDim.x) {
    const int xp = i / g.pz, zp = i - xp * g.pz;  // consecutive threads walk zp: coalesced stores
    dst[((size_t)xp * g.Q + y) * g.pz + zp] = src[(size_t)zp * g.px + xp];
  }
}

cudaError_t launch_flow_out(const Grid& g, const double* P, double* flow, cudaStream_t st) {
  const int nb = (g.pz * g.px + 255) / 256;
  k_flow_out<<<dim3(nb, g.Q, 3), 256, 0, st>>>(g, P, flow);
  return cudaGetLastError();
}

// dCdt = (1/dt) (MC[i+] - MC[i-]) per segment (channel/channel.c:728-740)
__global__ void k_ddt_diff(size_t n, double rdt0, DdtArgs d, cpx* __restrict__ dC) {
  const int s = blockIdx.y;
  const double rdt = d.grids ? 1.0 / d.grids[s].dt : rdt0;
  const int i_step = d.step_ptr ? *d.step_ptr + d.step_add : d.step_add;
  const bool cross = i_step == 0 && d.chain > 0 && s > 0;
  const int ip = cross ? 0 : (i_step == 0 ? 3 : 3 * i_step);
  const int im = cross ? 3 * (d.chain - 1) : (i_step == 0 ? 0 : 3 * (i_step - 1));
  const cpx* A = d.MC + (long long)s * d.traj_stride + (long long)ip * n;
  const cpx* B = d.MC + (long long)(cross ? s - 1 : s) * d.traj_stride + (long long)im * n;
  cpx* out = dC + (long long)s * n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    out[i].re = rdt * (A[i].re - B[i].re);
    out[i].im = rdt * (A[i].im - B[i].im);
  }
}

cudaError_t launch_ddt_diff(const Grid& g, const DdtArgs& d, cpx* dC, cudaStream_t st) {
  const size_t n = coef_size(g);
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_ddt_diff<<<dim3(nb < 512 ? nb : 512, d.nseg), 256, 0, st>>>(n, 1.0 / g.dt, d, dC);
  return cudaGetLastError();
}

// per-segment partial sums of the weighted inner products
// (channel/channel.c:746-764); fixed block count and order: deterministic
template <bool MULTI>
__global__ void k_ddt_dots(const __grid_constant__ Grid g0, Batch<const double> Pa, Batch<const double> Pb,
                           double* __restrict__ part, const Grid* grids) {
  const int s = blockIdx.y;
  CHN_INSTANCE_GRID(g0, grids, s);
  const size_t plane = (size_t)g.pz * g.px;
  const size_t n = (size_t)3 * g.Q * plane;
  const double* a_ = Pa.at(s);
  const double* b_ = Pb.at(s);
  double num = 0.0, den = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)((i / plane) % g.Q);
    const double a = a_[i], w = g.W[y];
    num = fma(a * b_[i], w, num);
    den = fma(a * a, w, den);
  }
  __shared__ double sn[256], sd[256];
  sn[threadIdx.x] = num;
  sd[threadIdx.x] = den;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      sn[threadIdx.x] += sn[threadIdx.x + k];
      sd[threadIdx.x] += sd[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[((size_t)s * gridDim.x + blockIdx.x) * 2] = sn[0];
    part[((size_t)s * gridDim.x + blockIdx.x) * 2 + 1] = sd[0];
  }
}

cudaError_t launch_ddt_dots(const Grid& g, Batch<const double> Pa, Batch<const double> Pb, double* part,
                            int nblk, int nseg, cudaStream_t st, const Grid* grids) {
  if (grids) k_ddt_dots<true><<<dim3(nblk, nseg), 256, 0, st>>>(g, Pa, Pb, part, grids);
  else k_ddt_dots<false><<<dim3(nblk, nseg), 256, 0, st>>>(g, Pa, Pb, part, nullptr);
  return cudaGetLastError();
}

// The same partial sums with both fields taken from physical-field caches:
// dudt = (P(MC[i+]) - P(MC[i-])) / dt from the primal cache (the transform is
// linear, so this is spec2phys of the finite difference), v from the cache of
// the coupled tangent's fields at stage 0 of step i (spec2phys(MIC[3i])).
template <bool MULTI>
__global__ void k_ddt_dots_cached(const __grid_constant__ Grid g0, DdtArgs d, const double* __restrict__ Pc,
                                  long long cstride, long long psz, const double* __restrict__ Pv,
                                  long long vstride, long long vslot, double* __restrict__ part) {
  const int s = blockIdx.y;
  CHN_INSTANCE_GRID(g0, d.grids, s);
  const int i_step = d.step_ptr ? *d.step_ptr + d.step_add : d.step_add;
  const bool cross = i_step == 0 && d.chain > 0 && s > 0;
  const int ip = cross ? 0 : (i_step == 0 ? 3 : 3 * i_step);
  const int im = cross ? 3 * (d.chain - 1) : (i_step == 0 ? 0 : 3 * (i_step - 1));
  const double* A = Pc + (long long)s * cstride + (long long)ip * psz;
  const double* B = Pc + (long long)(cross ? s - 1 : s) * cstride + (long long)im * psz;
  const double* V = Pv + (long long)s * vstride + (long long)i_step * vslot;
  const size_t plane = (size_t)g.pz * g.px;
  const size_t n = (size_t)3 * g.Q * plane;
  const double rdt = 1.0 / g.dt;
  double num = 0.0, den = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)((i / plane) % g.Q);
    const double a = rdt * (A[i] - B[i]), w = g.W[y];
    num = fma(a * V[i], w, num);
    den = fma(a * a, w, den);
  }
  __shared__ double sn[256], sd[256];
  sn[threadIdx.x] = num;
  sd[threadIdx.x] = den;
  __syncthreads();
  for (int k = blockDim.x / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) {
      sn[threadIdx.x] += sn[threadIdx.x + k];
      sd[threadIdx.x] += sd[threadIdx.x + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[((size_t)s * gridDim.x + blockIdx.x) * 2] = sn[0];
    part[((size_t)s * gridDim.x + blockIdx.x) * 2 + 1] = sd[0];
  }
}

cudaError_t launch_ddt_dots_cached(const Grid& g, const DdtArgs& d, const double* Pc, long long cstride,
                                   long long psz, const double* Pv, long long vstride, long long vslot,
                                   double* part, int nblk, cudaStream_t st) {
  if (d.grids)
    k_ddt_dots_cached<true><<<dim3(nblk, d.nseg), 256, 0, st>>>(g, d, Pc, cstride, psz, Pv, vstride, vslot, part);
  else
    k_ddt_dots_cached<false><<<dim3(nblk, d.nseg), 256, 0, st>>>(g, d, Pc, cstride, psz, Pv, vstride, vslot, part);
  return cudaGetLastError();
}

// copy the first 3 physical fields (u, v, w) of instance (s * div + sel) of P
// into slot (*step + add) of segment s of a field cache
// (skipped for a segment whose time loop has stopped, like the solve that
// would have stored the matching trajectory slot)
__global__ void k_cache_velocity(size_t n, const double* __restrict__ P, long long pstride, int div, int sel,
                                 double* __restrict__ Pv, long long vstride, long long vslot, const int* step,
                                 int add, const uint32_t* __restrict__ status) {
  const int s = blockIdx.y;
  if (status && (status[s] & ST_CFL)) return;
  const double* src = P + (long long)(s * div + sel) * pstride;
  double* dst = Pv + (long long)s * vstride + (long long)(*step + add) * vslot;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

cudaError_t launch_cache_velocity(const Grid& g, const double* P, long long pstride, int div, int sel, double* Pv,
                                  long long vstride, long long vslot, const int* step, int add,
                                  const uint32_t* status, int nseg, cudaStream_t st) {
  const size_t n = (size_t)3 * g.Q * plane_size(g);
  k_cache_velocity<<<dim3(256, nseg), 256, 0, st>>>(n, P, pstride, div, sel, Pv, vstride, vslot, step, add,
                                                     status);
  return cudaGetLastError();
}

// AC -= coef * IC' for an IC' projected earlier (the same update as k_ddt_apply)
__global__ void k_sub_scaled(size_t n, const cpx* __restrict__ src, long long sstride, cpx* __restrict__ ac,
                             long long astride, double coef0, const Grid* grids) {
  const int s = blockIdx.y;
  const double coef = grids ? coef0 * grids[s].dt : coef0;
  const cpx* v_ = src + (long long)s * sstride;
  cpx* a_ = ac + (long long)s * astride;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const cpx v = v_[i];
    a_[i].re -= coef * v.re;
    a_[i].im -= coef * v.im;
  }
}

cudaError_t launch_sub_scaled(const Grid& g, Batch<const cpx> src, Batch<cpx> ac, double coef, int nseg,
                              cudaStream_t st, const Grid* grids) {
  const size_t n = coef_size(g);
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_sub_scaled<<<dim3(nb < 512 ? nb : 512, nseg), 256, 0, st>>>(n, src.base, src.stride, ac.base, ac.stride, coef,
                                                                 grids);
  return cudaGetLastError();
}

// IC' = IC - (num/den) dCdt (channel/channel.c:769-772), then the adjoint's
// AC -= 0.5*strength*dt*IC' (channel/channel.c:628-631, 686-689)
__global__ void k_ddt_apply(size_t n, const double* __restrict__ part, int nblk, Batch<const cpx> ICsrc,
                            SlotRef icslot, Batch<cpx> ICdst, Batch<const cpx> dC, double* __restrict__ r_out,
                            Batch<cpx> AC, double coef0, const Grid* grids) {
  const int s = blockIdx.y;
  const double coef = grids ? coef0 * grids[s].dt : coef0;
  __shared__ double r_s;
  if (threadIdx.x == 0) {
    double num = 0.0, den = 0.0;
    for (int b = 0; b < nblk; ++b) {
      num += part[((size_t)s * nblk + b) * 2];
      den += part[((size_t)s * nblk + b) * 2 + 1];
    }
    r_s = num / den;
    if (blockIdx.x == 0 && r_out) r_out[s] = r_s;
  }
  __syncthreads();
  const double r = r_s;
  const cpx* src = ICsrc.at(s);
  if (icslot.stride) src += (long long)icslot.slot() * icslot.stride;
  cpx* dst = ICdst.base ? ICdst.at(s) : nullptr;
  cpx* ac = AC.base ? AC.at(s) : nullptr;
  const cpx* dc = dC.at(s);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    cpx v = src[i];
    v.re -= r * dc[i].re;
    v.im -= r * dc[i].im;
    if (dst) dst[i] = v;
    if (ac) {
      ac[i].re -= coef * v.re;
      ac[i].im -= coef * v.im;
    }
  }
}

cudaError_t launch_ddt_apply(const Grid& g, const double* part, int nblk, int nseg, Batch<const cpx> ICsrc,
                             SlotRef icslot, Batch<cpx> ICdst, Batch<const cpx> dC, double* r_out,
                             Batch<cpx> AC, double coef, cudaStream_t st, const Grid* grids) {
  const size_t n = coef_size(g);
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_ddt_apply<<<dim3(nb < 512 ? nb : 512, nseg), 256, 0, st>>>(n, part, nblk, ICsrc, icslot, ICdst, dC, r_out, AC,
                                                                coef, grids);
  return cudaGetLastError();
}

// Laminar start: velocity samples -> Legendre coefficients by Gram projection
// and the mass-matrix solve (channel/initAlphaBeta.c:24-205).  One thread per
// (kz, kx) mode; init only.
__device__ void solve_real_chain(const double* LU, int w, int dl, int du, int N, int par, double* b, int bs) {
  for (int i = par; i < N; i += 2) {
    if (i < 2) continue;
    int j0 = dl - i / 2;
    if (j0 < 0) j0 = 0;
    double acc = b[(size_t)i * bs];
    for (int j = j0; j < dl; ++j) acc -= LU[(size_t)i * w + j] * b[(size_t)(i - 2 * (dl - j)) * bs];
    b[(size_t)i * bs] = acc;
  }
  int ilast = ((N - 1 - par) % 2 == 0) ? N - 1 : N - 2;
  for (int i = ilast; i >= 0; i -= 2) {
    double acc = b[(size_t)i * bs];
    if (i <= N - 3) {
      int jm = (N - i + 1) / 2 - 1;
      if (jm > du) jm = du;
      for (int j = 1; j <= jm; ++j) acc -= LU[(size_t)i * w + dl + j] * b[(size_t)(i + 2 * j) * bs];
    }
    b[(size_t)i * bs] = acc / LU[(size_t)i * w + dl];
  }
}

__global__ void k_project_init(Grid g, const cpx* __restrict__ U, cpx* __restrict__ C, const double* __restrict__ luQs,
                               const double* __restrict__ luRs) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.Nz * g.X) return;
  const int z = m / g.X, x = m - z * g.X;
  auto u = [&](int c, int y) { return U[(((size_t)z * 5 + c) * g.Q + y) * g.X + x]; };
  auto cref = [&](int v, int r) -> cpx& { return C[(((size_t)z * 2 + v) * g.R + r) * g.X + x]; };
  const double kx = g.Kx[x], kz = g.Kz[z];
  if (z == 0 && x == 0) {
    for (int v = 0; v < 2; ++v) {
      for (int i = 0; i < g.R; ++i) {
        double re = 0.0, im = 0.0;
        for (int y = 0; y < g.Q; ++y) {
          const double w = g.Wr[(size_t)i * g.Q + y];
          const cpx s = u(v == 0 ? 0 : 2, y);
          re += w * s.re;
          im += w * s.im;
        }
        cref(v, i) = cpx{re, im};
      }
      for (int ch = 0; ch < 4; ++ch)
        solve_real_chain(luRs, 5, 2, 2, g.R, ch & 1, reinterpret_cast<double*>(&cref(v, 0)) + (ch >> 1), 2 * g.X);
    }
    return;
  }
  for (int i = 0; i < g.D; ++i) {
    double re = 0.0, im = 0.0;
    for (int y = 0; y < g.Q; ++y) {
      const double w = g.Wq[(size_t)i * g.Q + y];
      const cpx s = u(1, y);
      re += w * s.re;
      im += w * s.im;
    }
    cref(0, i) = cpx{re, im};
  }
  for (int ch = 0; ch < 4; ++ch)
    solve_real_chain(luQs, 9, 4, 4, g.D, ch & 1, reinterpret_cast<double*>(&cref(0, 0)) + (ch >> 1), 2 * g.X);
  for (int i = 0; i < g.R; ++i) {
    double re = 0.0, im = 0.0;
    for (int y = 0; y < g.Q; ++y) {
      const double w = g.Wr[(size_t)i * g.Q + y];
      const cpx uu = u(0, y), ww = u(2, y);
      re += w * (kx * ww.im - kz * uu.im);
      im += w * (kz * uu.re - kx * ww.re);
    }
    cref(1, i) = cpx{re, im};
  }
  for (int ch = 0; ch < 4; ++ch)
    solve_real_chain(luRs, 5, 2, 2, g.R, ch & 1, reinterpret_cast<double*>(&cref(1, 0)) + (ch >> 1), 2 * g.X);
}

cudaError_t launch_project_init(const Grid& g, const cpx* Uinit, cpx* C, const double* luQs, const double* luRs,
                                cudaStream_t st) {
  const int n = g.Nz * g.X;
  k_project_init<<<(n + 127) / 128, 128, 0, st>>>(g, Uinit, C, luQs, luRs);
  return cudaGetLastError();
}

__global__ void k_step_advance(int* ctr, int delta) { ctr[0] += delta; }

cudaError_t launch_step_advance(int* ctr, int delta, cudaStream_t st) {
  k_step_advance<<<1, 1, 0, st>>>(ctr, delta);
  return cudaGetLastError();
}

// The device-side loop of a multi-step sweep: the sweep is one graph launch
// whose while-node body is one step followed by k_loop_next, which counts
// the steps left down and keeps the loop running while any are left (the
// condition is the count's positivity, so the loop ends after at most the
// count k_loop_set wrote before the launch).
__global__ void k_loop_set(int* ctr, int n) { ctr[0] = n; }

__global__ void k_loop_next(int* ctr, cudaGraphConditionalHandle h) {
  const int left = --ctr[0];
  cudaGraphSetConditional(h, left > 0 ? 1u : 0u);
}

cudaError_t launch_loop_set(int* ctr, int n, cudaStream_t st) {
  k_loop_set<<<1, 1, 0, st>>>(ctr, n);
  return cudaGetLastError();
}

cudaError_t launch_loop_next(int* ctr, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_loop_next<<<1, 1, 0, st>>>(ctr, h);
  return cudaGetLastError();
}

// A seeded pattern of finite doubles with exponents spread over 2^-6 .. 2^1
// (both signs), written where the autotuner times kernels: zeros would take
// the kernels' zero shortcuts (no exponents to gather, no rounding) and time
// a lighter workload than the real one.
__global__ void k_fill_pattern(double* p, size_t n, uint32_t seed) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const double m = 0.5 + (double)(h & 0xFFFFFu) * (1.0 / 2097152.0);  // [0.5, 1)
    const int k = (int)((h >> 20) & 7u) - 6;
    p[i] = ((h >> 31) ? -m : m) * ldexp(1.0, k);
  }
}

cudaError_t launch_fill_pattern(double* p, size_t n, uint32_t seed, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_fill_pattern<<<1216, 256, 0, st>>>(p, n, seed);
  return cudaGetLastError();
}

// FP64 fused multiply-add throughput probe: 8 independent chains per thread,
// registers only; out gets one value per thread so nothing is optimised away.
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t launch_fp64_probe(double* out, int blocks, int threads, int iters, cudaStream_t st) {
  k_fp64_probe<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
  return cudaGetLastError();
}

// Throughput probes of the other pipes the design choices rest on: FP64 add,
// FP64 warp-level matrix multiply-accumulate (m8n8k4), FP32 FMA.  8
// independent chains per thread (4 accumulator pairs per warp for DMMA).
__global__ void k_dadd_probe(double* out, int iters, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 += b; x1 += b; x2 += b; x3 += b; x4 += b; x5 += b; x6 += b; x7 += b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ffma_probe(double* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-6f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_dmma_probe(double* out, int iters, double a0, double b0) {
  const double a = a0 + threadIdx.x * 1e-12, b = b0 - threadIdx.x * 1e-12;
  double c[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[q][0]), "+d"(c[q][1])
                   : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c[0][0] + c[0][1] + c[1][0] + c[1][1] + c[2][0] + c[2][1] +
                                               c[3][0] + c[3][1];
}

// flop per thread per iteration of each probe kind (0 DFMA, 1 DADD, 2 DMMA, 3 FFMA)
double probe_flop_per_thread_iter(int kind) {
  switch (kind) {
    case 0: return 16.0;          // 8 FMA
    case 1: return 8.0;           // 8 adds
    case 2: return 4 * 512.0 / 32; // 4 mma of 8x8x4 (2 flop per MAC) per warp
    case 3: return 16.0;
    default: return 0.0;
  }
}

cudaError_t launch_pipe_probe(int kind, double* out, int blocks, int threads, int iters, cudaStream_t st) {
  switch (kind) {
    case 0: k_fp64_probe<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7); break;
    case 1: k_dadd_probe<<<blocks, threads, 0, st>>>(out, iters, 1e-7); break;
    case 2: k_dmma_probe<<<blocks, threads, 0, st>>>(out, iters, 0.5, 0.25); break;
    case 3: k_ffma_probe<<<blocks, threads, 0, st>>>(out, iters, 0.999999f, 1e-7f); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace chn
