// Shared device-side definitions for the GB300 channel-flow step.
//
// Layouts (all complex numbers are {double re, im}, FP64 throughout):
//   coefficients  C[Nz][2][R][X]            R = Ny-2, X = Nx/2, [..][0] alpha, [..][1] beta
//   velocity      U[Nz][5][Q][X]            Q = 3Ny/2 quadrature planes
//                 slots 0..4 = u, v, w, du/dy, dw/dy (channel/minChnl.h:44-49)
//   nonlinear     H[Nz][5][Q][X]            slot 0 Hz, 1 Hx, 2 Hy; adjoint adds 3 Sx, 4 Sz
//                                           (channel/minChnl.h:50-52, pass2.c:474-566)
//   physical      P[f][Q][pz][px]           pz = 3Nz/2, px = 3Nx/2, reals
//                 f = 0 u, 1 v, 2 w, 3 wz, 4 wx, 5 wy (the reference's CT slot order)
//   flow (spec2phys output) flow[3][px][Q][pz] (channel/spec2phys.c:80-86)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace chn {

struct cpx {
  double re, im;
};

// RK3 coefficient tables, forward (channel/project.c:44-47) and adjoint
// (channel/adjproject.c:34-37).  The implicit-side coefficient b takes three
// distinct values {1/6, 2/3, 0}; LHS factorizations are stored per distinct
// value (index below), explicit matrices per distinct a in {1/3, -1/2}.
struct RK {
  double a[3], b[3], c[3], d[3];
  int bidx[3];       // index of b[k] among {1/6, 2/3, 0}
  int aidx_next[3];  // index of a[k+1] among {1/3, -1/2} (k < 2)
};

// Status bits of the per-instance device status word.
enum : uint32_t {
  ST_CFL = 1u,        // pass1: CFL number >= 2.8, loop stopped (channel/pass1.c:116-138)
  ST_NONFINITE = 2u,  // a non-finite value was seen in a physical field (diagnostic only)
};

// Grid description plus device tables; passed by value to every kernel.
struct Grid {
  int Nx, Ny, Nz, X, Q, R, D, pz, px, Qh;  // Qh = (Q+1)/2 plane pairs
  int split;             // transforms in separate z and x passes (required when a plane exceeds
                         // one block's shared memory; else chosen by the autotuner)
  int tvar;              // split-transform variant (block size and chunk)
  int general;           // 3Nz/2 or 3Nx/2 needs radix 5 or 7 (slower, register-heavy transforms)
  double dt, re, flux, norm, cfl1, cfl3;
  const double* Kx;      // [X]
  const double* Kz;      // [Nz]
  const double* K2;      // [Nz][X]
  const double* kxK2;    // [Nz][X]  kx/K2 (0 for the mean mode)
  const double* kzK2;    // [Nz][X]  kz/K2
  const double* cfl2;    // [Q]
  const double* W;       // [Q] quadrature weights
  // basis values at the quadrature points, row-major [Q][D] / [Q][R]
  const double* Bq;      // Q   (1-y^2)^2 P_j
  const double* Bqp;     // Q'
  const double* Bqpp;    // Q''
  const double* Br;      // R   (1-y^2) P_j
  const double* Brp;     // R'
  // weighted transposes [D][Q] / [R][Q]: Xw[i][j] = w_j X[j][i]
  const double* Wq;      // Qw
  const double* Wqp;     // Qpw
  const double* Wqpp;    // Qppw
  const double* Wr;      // Rw
  const double* Wrp;     // Rpw
  // banded systems, per (z, x): no-pivot LU factors of the LHS, and the
  // explicit right-hand-side matrices; 9 every-other diagonals for the v
  // (alpha) system, 5 for the g (beta) system, centre column 4 / 2.
  const double* luA;     // [3][Nz][X][D][9]
  const double* luB;     // [3][Nz][X][R][5]
  const double* exA;     // [2][Nz][X][D][9]
  const double* exB;     // [2][Nz][X][R][5]
  // mean-flow (kx,kz) = (0,0) systems on the R basis
  const double* lu0;     // [3][R][5]   Rs + re b dt Rps, LU factors
  const double* rdA;     // [3][Nz][X][D] reciprocal pivots of luA (centre column)
  const double* rdB;     // [3][Nz][X][R] of luB
  const double* rd0;     // [3][R]        of lu0
  const double* ex0;     // [2][R][5]   Rs - re a dt Rps
  const double* add0;    // [4][R]      flux-correction vectors: [0] forward, [1+bidx] adjoint
  const double* rwsum;   // [R]         sum_j Rw[i][j]
  const double* Qs;      // [D][9]      banded Gram matrices (every other diagonal)
  const double* Qps;     // [D][9]
  const double* Qpps;    // [D][9]
  const double* Rs;      // [R][5]
  const double* Rps;     // [R][5]
  // FFT twiddles exp(-2 pi i k/N), k < N, for N = pz and N = px
  const cpx* twz;
  const cpx* twx;
  // tensor-core reconstruction (recon_tc.cu): base-256 digits of the five
  // bases in mma A-fragment order [5][ceil(Q/16)][ceil(R/16)][7][32 lanes][4],
  // and the row exponents [5][Q] (|basis row| < 2^tcE); tc = 0: FP64 kernel
  const uint32_t* tcA;
  const int* tcE;
  // the weighted transposes Qw, Qpw, Qppw, Rw, Rpw likewise, rows padded to R:
  // [5][ceil(R/16)][ceil(Q/16)][7][32][4], row exponents [5][R]
  const uint32_t* tcW;
  const int* tcWE;
  // the exact adjoint's transposed contractions (adjoint_exact.cu): the five
  // bases transposed without weights, rows padded to R, in tcW's layout
  // [5][ceil(R/16)][ceil(Q/16)][7][32][4] with exponents [5][R]; and Qpw, Qw,
  // Rw plane-major [3][ceil(Q/16)][ceil(R/16)][7][32][4], exponents [3][Q]
  const uint32_t* tcBT;
  const int* tcBTE;
  const uint32_t* tcWT;
  const int* tcWTE;
  int tc;
  // kx columns per block of the implicit solve (16 or 8) and its threads
  // (256, or 128 with 8 columns: 4 blocks per SM); the autotuner's choice,
  // the same results either way
  int stile;
  int sthr;
  int rbuild;  // tensor-core reconstruction: 0 = 16 columns, 256 threads; 1 = 8 columns, 128 threads;
               // 2 = 16 columns at 3 blocks per SM (autotuned)
  // inverse transforms as DFT GEMMs on the tensor cores (phys_tc.cu), each
  // stage split radix-2 into even and odd modes where its length is even:
  // the z stage's matrix [2 pz / 2][even | odd modes (Re, Im)] and the x
  // stage's [px / 2][even | odd j (Re, Im)] as digit tables with row
  // exponents, and the z stage's K-word -> kept kz index map (-1: padding);
  // tci = 0: the FFT kernels
  const uint32_t* tcZ;
  const int* tcZE;
  const uint32_t* tcX;
  const int* tcXE;
  const int* tcZM;
  int tci;
  int tcminb;  // build of the tensor-core inverse (2..5: fields per pass, threads, blocks per SM; autotuned)
  // the same inverse on the fifth-generation tensor cores (phys_tc5.cu,
  // tcgen05.mma with tensor-memory accumulators): the two stages' digit
  // tables as stacked B operands in the K-major canonical layout; tc5 = 0:
  // the mma.sync kernel above (uneven batches always take it)
  const unsigned char* t5Z;
  const unsigned char* t5X;
  int tc5;
  // forward transforms likewise (phys_tc.cu, k_products_tc): x stage
  // [2X][px] (1/(px pz) folded in), z stage [2 (Nz - 1)][2 pz]; tcf = 0: the FFT kernels
  const uint32_t* tcFX;
  const int* tcFXE;
  const uint32_t* tcFXU;  // the x stage without the 1/(px pz) (exact transpose)
  const int* tcFXUE;
  const uint32_t* tcFZ;
  const int* tcFZE;
  int tcf;
  int fwdpb;  // product planes per pass of the forward modes (3, or 1 where 3 leave no room for two blocks)
  int fxch;   // x-stage columns per chunk of the forward products (a multiple of 8; all where they fit)
  int adjpb;  // product planes per pass of the adjoint product modes (1 or 3; autotuned)
  int prodb;  // products build: 0 = the plan above, 1 = two planes per pass at 3 blocks per SM
              // (single-grid batches; autotuned)
  // kernels that run their build compiled for the grid's sizes (32x65x32,
  // 16x33x16): FIXED_* bits of sizes.cuh (autotuned; the same results)
  int fixed;
};

__host__ __device__ inline size_t coef_size(const Grid& g) { return (size_t)g.Nz * 2 * g.R * g.X; }
__host__ __device__ inline size_t u_size(const Grid& g) { return (size_t)g.Nz * 5 * g.Q * g.X; }
__host__ __device__ inline size_t plane_size(const Grid& g) { return (size_t)g.pz * g.px; }

// One batched array: instance i lives at base + i * stride (elements).
template <typename T>
struct Batch {
  T* base;
  long long stride;
  __host__ __device__ T* at(int i) const { return base + (long long)i * stride; }
};

__device__ __forceinline__ cpx cmul(cpx a, cpx b) {
  cpx r;
  r.re = fma(a.re, b.re, -a.im * b.im);
  r.im = fma(a.re, b.im, a.im * b.re);
  return r;
}

// (row, col) of a flat index i = row * W + col walked in steps of `step`
// without a division per step: one division at the start, then a carry.
struct FlatRC {
  int r, c, dr, dc, W;
  __device__ __forceinline__ FlatRC(int i0, int step, int W_) : W(W_) {
    r = i0 / W;
    c = i0 - r * W;
    dr = step / W;
    dc = step - dr * W;
  }
  __device__ __forceinline__ void next() {
    c += dc;
    r += dr;
    if (c >= W) {
      c -= W;
      ++r;
    }
  }
};

// Uneven batches: a MULTI kernel takes its instance's grid (sizes and
// tables) from a device array, staged once per block in shared memory; the
// launch is sized for the largest grid (kernel argument g0) and blocks beyond
// their own instance's range return.  Non-MULTI kernels use g0 directly.
#define CHN_INSTANCE_GRID(g0, grids, inst)        \
  __shared__ Grid chn_sg_;                        \
  if (MULTI) {                                    \
    if (threadIdx.x == 0) chn_sg_ = (grids)[inst]; \
    __syncthreads();                              \
  }                                               \
  const Grid& g = MULTI ? chn_sg_ : (g0)

// Allow a kernel the device's opt-in shared memory per block, less what it
// declares statically.
template <typename K>
inline cudaError_t allow_max_smem(K kernel, int optin) {
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

}  // namespace chn
