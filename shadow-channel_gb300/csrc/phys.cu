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
//                    channel/pass2.c:224-566.  With `exact`: the transpose
//                    of the tangent products and of the vorticity load
//                    (the exact discrete adjoint, adjoint_exact.cu).
//
// Every transform is an FP64 shared-memory Stockham FFT (fft.cuh).  The x
// transforms of two real rows share one complex FFT (row pairs packed as
// a + i b), so no real-to-complex post-processing pass is needed.
#include <algorithm>

#include "chn_common.cuh"
#include "fft.cuh"
#include "kernels.h"
#include "phys_common.cuh"

namespace chn {

static constexpr int kThreads = 256;

struct PhysSmem {
  cpx *twz, *twx, *zb0, *zb1, *xb0, *xb1;
  double* cfl;
};

// Three buffer regions: A (the larger of a z block and an x block), B (a z
// block), C (an x block).  The z result is dead once it is packed into the x
// rows (inverse), and the x result once its kept bins are extracted
// (forward), so one region serves both phases:
//   inverse: z ping-pong A <-> B, x ping-pong C <-> A
//   forward: x ping-pong C <-> A, z ping-pong B <-> A
__device__ inline PhysSmem carve(const Grid& g, unsigned char* base, bool with_cfl, bool forward) {
  PhysSmem s;
  const int npair = (g.pz + 1) / 2;
  const size_t zsz = (size_t)g.pz * g.X, xsz = (size_t)npair * g.px;
  cpx* p = reinterpret_cast<cpx*>(base);
  s.twz = p; p += g.pz;
  s.twx = p; p += g.px;
  cpx* A = p; p += zsz > xsz ? zsz : xsz;
  cpx* B = p; p += zsz;
  cpx* C = p; p += xsz;
  s.xb0 = C;
  s.xb1 = A;
  s.zb0 = forward ? B : A;
  s.zb1 = forward ? A : B;
  s.cfl = with_cfl ? reinterpret_cast<double*>(p) : nullptr;
  return s;
}

__host__ __device__ inline size_t phys_smem_hd(const Grid& g, bool with_cfl) {
  const int npair = (g.pz + 1) / 2;
  const size_t zsz = (size_t)g.pz * g.X, xsz = (size_t)npair * g.px;
  size_t n = (size_t)g.pz + g.px + (zsz > xsz ? zsz : xsz) + zsz + xsz;
  size_t b = n * sizeof(cpx);
  if (with_cfl) b += (size_t)g.pz * g.px * sizeof(double);
  return b;
}

size_t phys_smem_bytes(const Grid& g, bool with_cfl) { return phys_smem_hd(g, with_cfl); }

__device__ inline void load_tw(const Grid& g, PhysSmem& s) {
  for (int i = threadIdx.x; i < g.pz; i += blockDim.x) s.twz[i] = g.twz[i];
  for (int i = threadIdx.x; i < g.px; i += blockDim.x) s.twx[i] = g.twx[i];
}

template <bool MULTI, bool GEN>
__global__ void __launch_bounds__(kThreads) k_phys_inverse(const __grid_constant__ Grid g0, PhysArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (a.skip_blocked && blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, a.cfl_check != 0, false);
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
    cpx* zr = fft_run<GEN>(pz_plan, s.zb0, s.zb1, g.X, g.X, 1, s.twz, +1, true);
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
    cpx* xr = fft_run<GEN>(px_plan, s.xb0, s.xb1, npair, 1, g.px, s.twx, +1, true);
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

// forward transform of the product rows held in xb0; leaves the kept,
// scaled spectral rows in the returned z buffer
template <bool GEN>
__device__ inline cpx* forward_plane(const Grid& g, PhysSmem& s, const FftPlan& pxF, const FftPlan& pzF,
                                     double scale) {
  const int npair = (g.pz + 1) / 2;
  cpx* xr = fft_run<GEN>(pxF, s.xb0, s.xb1, npair, 1, g.px, s.twx, -1, true);
  const double hn = 0.5 * scale;
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
  return fft_run<GEN>(pzF, s.zb0, s.zb1, g.X, g.X, 1, s.twz, -1, true);
}

template <bool MULTI, bool GEN>
__global__ void __launch_bounds__(kThreads) k_products_fwd(const __grid_constant__ Grid g0, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, false, true);
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
    cpx* zr = forward_plane<GEN>(g, s, pxF, pzF, g.norm);
    for (int i = threadIdx.x; i < g.pz * g.X; i += blockDim.x) {
      const int zp = i / g.X, x = i - zp * g.X;
      const int z = zrow_to_kz(g, zp);
      if (z >= 0) H[(((size_t)z * 5 + c) * g.Q + y) * g.X + x] = zr[i];
    }
    __syncthreads();
  }
}

size_t prod_adj_smem_bytes(const Grid& g) { return phys_smem_bytes(g, false); }

template <bool MULTI, bool GEN>
__global__ void __launch_bounds__(kThreads) k_products_adj(const __grid_constant__ Grid g0, ProdArgs a) {
  const int inst = blockIdx.y, y = blockIdx.x;
  CHN_INSTANCE_GRID(g0, a.grids, inst);
  if (y >= g.Q) return;
  if (blocked(a.status, a.sdiv, inst)) return;
  extern __shared__ __align__(16) unsigned char smem[];
  PhysSmem s = carve(g, smem, false, true);
  load_tw(g, s);
  const size_t plane = (size_t)g.pz * g.px, fs = (size_t)g.Q * plane;
  const double* __restrict__ P = a.Pp.base + (long long)(inst / a.pdiv) * a.Pp.stride + (size_t)y * plane +
                                 (a.pslot.stride ? (long long)a.pslot.slot() * a.pslot.stride : 0LL);
  const double* __restrict__ L = a.Pt.at(inst) + (size_t)y * plane;  // lambda (exact: N_bar): 3 fields
  cpx* __restrict__ H = a.H.at(inst);
  const FftPlan pxF = make_plan(g.px, false);
  const FftPlan pzF = make_plan(g.pz, false);
  const int npair = (g.pz + 1) / 2;
  const bool exact = a.exact != 0;
  __syncthreads();
  // q = 0..2: S_x, S_y, S_z = u x lambda; q = 3..5: T_x, T_y, T_z = lambda x w
  // (exact: the cotangents of u, v, w, wz, wx, wy)
  for (int q = 0; q < 6; ++q) {
    for (int i = threadIdx.x; i < npair * g.px; i += blockDim.x) {
      const int p = i / g.px, xp = i - p * g.px;
      double val[2] = {0.0, 0.0};
      for (int h = 0; h < 2; ++h) {
        if (2 * p + h >= g.pz) break;
        const size_t o = (size_t)(2 * p + h) * g.px + xp;
        if (exact) {
          val[h] = prod_transpose(P, L, fs, o, q);
          continue;
        }
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
    cpx* zr = forward_plane<GEN>(g, s, pxF, pzF, exact ? 1.0 : g.norm);
    // fold product q into the output slots (the (zp, x) -> thread map is the
    // same for every q, so each thread re-reads only its own partial sums)
    for (int i = threadIdx.x; i < g.pz * g.X; i += blockDim.x) {
      const int zp = i / g.X, x = i - zp * g.X;
      const int z = zrow_to_kz(g, zp);
      if (z >= 0) assemble_stage(g, exact, H, z, y, x, q, zr[i]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// split transforms (transforms.cuh): separate z and x passes through an HBM
// intermediate, for grids whose padded plane does not fit one block's shared
// memory (128x129x128), and, where the autotuner finds them faster, for any
// grid.  Variants differ in block size and chunk only.
// ---------------------------------------------------------------------------

#define CHN_DECLARE_SPLIT(ID)                                                            \
  cudaError_t split_inverse_##ID(const Grid& g, const PhysArgs& a, cudaStream_t st);   \
  cudaError_t split_products_##ID(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st); \
  void prepare_split_##ID(int optin);                                                   \
  bool split_fits_##ID(const Grid& g, int optin);
CHN_DECLARE_SPLIT(0)
CHN_DECLARE_SPLIT(1)
CHN_DECLARE_SPLIT(2)
CHN_DECLARE_SPLIT(3)

struct SplitEntry {
  TransformVariant v;
  cudaError_t (*inverse)(const Grid&, const PhysArgs&, cudaStream_t);
  cudaError_t (*products)(const Grid&, const ProdArgs&, int, cudaStream_t);
  void (*prepare)(int);
  bool (*fits)(const Grid&, int);
};

static const SplitEntry kSplit[] = {
    {{256, 24}, split_inverse_0, split_products_0, prepare_split_0, split_fits_0},
    {{192, 48}, split_inverse_1, split_products_1, prepare_split_1, split_fits_1},
    {{256, 48}, split_inverse_2, split_products_2, prepare_split_2, split_fits_2},
    {{128, 24}, split_inverse_3, split_products_3, prepare_split_3, split_fits_3},
};
static constexpr int kNumSplit = sizeof(kSplit) / sizeof(kSplit[0]);

int split_variant_count() { return kNumSplit; }
TransformVariant split_variant(int v) { return kSplit[v].v; }
bool split_variant_fits(int v, const Grid& g, int optin) { return v >= 0 && v < kNumSplit && kSplit[v].fits(g, optin); }

size_t split_tmp_elems(const Grid& g) { return (size_t)6 * g.Q * g.pz * g.X; }

bool fused_transforms_fit(const Grid& g, int smem_optin) {
  const size_t room = (size_t)smem_optin - 4096;  // static shared memory of the kernels (reductions, grid)
  return phys_smem_bytes(g, true) <= room && prod_adj_smem_bytes(g) <= room;
}

static int split_index(const Grid& g) { return (g.tvar >= 0 && g.tvar < kNumSplit) ? g.tvar : 0; }

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

// the instance of a fused kernel for this launch: uneven batch or not,
// general radices or 2/3/4 only
#define CHN_LAUNCH_FUSED(K, grid, smem, st, g, a)                               \
  do {                                                                            \
    if ((a).grids) {                                                              \
      if ((g).general) K<true, true><<<grid, kThreads, smem, st>>>(g, a);        \
      else K<true, false><<<grid, kThreads, smem, st>>>(g, a);                   \
    } else {                                                                      \
      if ((g).general) K<false, true><<<grid, kThreads, smem, st>>>(g, a);       \
      else K<false, false><<<grid, kThreads, smem, st>>>(g, a);                  \
    }                                                                             \
  } while (0)

cudaError_t launch_phys_inverse(const Grid& g, const PhysArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  // the tensor-core inverse wherever it fits (its results do not depend on
  // the autotuner's choice among the bit-identical FFT variants)
  if (g.tc5 && !a.grids) return launch_phys_inverse_tc5(g, a, st);  // fits every nfields once 6 fit
  if (g.tci) return launch_phys_inverse_tc(g, a, st);
  if (g.split) return kSplit[split_index(g)].inverse(g, a, st);
  const size_t sm = phys_smem_bytes(g, a.cfl_check != 0);
  CHN_LAUNCH_FUSED(k_phys_inverse, dim3(g.Q, a.ninst), sm, st, g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_fwd(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.tcf) return launch_products_tc(g, a, a.Pt.base ? 1 : 0, st);
  if (g.split) return kSplit[split_index(g)].products(g, a, a.Pt.base ? 1 : 0, st);
  const size_t sm = phys_smem_bytes(g, false);
  CHN_LAUNCH_FUSED(k_products_fwd, dim3(g.Q, a.ninst), sm, st, g, a);
  return cudaGetLastError();
}

cudaError_t launch_products_adj(const Grid& g, const ProdArgs& a, cudaStream_t st) {
  if (a.ninst <= 0) return cudaSuccess;
  if (g.tcf) return launch_products_tc(g, a, a.exact ? 3 : 2, st);
  if (g.split) return kSplit[split_index(g)].products(g, a, a.exact ? 3 : 2, st);
  const size_t sm = prod_adj_smem_bytes(g);
  CHN_LAUNCH_FUSED(k_products_adj, dim3(g.Q, a.ninst), sm, st, g, a);
  return cudaGetLastError();
}

void prepare_recon_solve(int optin);
void prepare_solve_T(int optin);
void prepare_recon_tc(int optin);
void prepare_phys_tc(int optin);
void prepare_phys_tc5(int optin);

// Every kernel may use up to the device's opt-in shared memory per block: the
// single-grid engine and an uneven batch (sized for its largest grid) share
// the kernels, so the limit is not tied to one grid.
template <bool MULTI, bool GEN>
static void prepare_transforms(int optin) {
  allow_max_smem(k_phys_inverse<MULTI, GEN>, optin);
  allow_max_smem(k_products_fwd<MULTI, GEN>, optin);
  allow_max_smem(k_products_adj<MULTI, GEN>, optin);
}

void prepare_kernels(const Grid& g) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  (void)g;
  prepare_transforms<false, false>(optin);
  prepare_transforms<false, true>(optin);
  prepare_transforms<true, false>(optin);
  prepare_transforms<true, true>(optin);
  for (const SplitEntry& e : kSplit) e.prepare(optin);
  prepare_recon_solve(optin);
  prepare_solve_T(optin);
  prepare_recon_tc(optin);
  prepare_phys_tc(optin);
  prepare_phys_tc5(optin);
}

}  // namespace chn
