// Grid sizes as a kernel reads them: from the grid at run time, or as
// compile-time constants in the builds specialised for a grid (the same
// arithmetic; loops over known extents unroll and index arithmetic folds).
#pragma once

#include "chn_common.cuh"

namespace chn {

// read from the grid where used
struct SizesRT {
  const Grid& g;
  __device__ explicit SizesRT(const Grid& g_) : g(g_) {}
  __device__ int Nz() const { return g.Nz; }
  __device__ int X() const { return g.X; }
  __device__ int pz() const { return g.pz; }
  __device__ int px() const { return g.px; }
  __device__ int Q() const { return g.Q; }
  __device__ int Qh() const { return g.Qh; }
  __device__ int R() const { return g.R; }
  __device__ int D() const { return g.D; }
};

// the sizes of an NX x NY x NZ grid (Nx, Ny, Nz as in c_init)
template <int NX, int NY, int NZ>
struct SizesCT {
  __device__ explicit SizesCT(const Grid&) {}
  __host__ __device__ static constexpr int Nz() { return NZ; }
  __host__ __device__ static constexpr int X() { return NX / 2; }
  __host__ __device__ static constexpr int pz() { return 3 * NZ / 2; }
  __host__ __device__ static constexpr int px() { return 3 * NX / 2; }
  __host__ __device__ static constexpr int Q() { return 3 * NY / 2; }
  __host__ __device__ static constexpr int Qh() { return (3 * NY / 2 + 1) / 2; }
  __host__ __device__ static constexpr int R() { return NY - 2; }
  __host__ __device__ static constexpr int D() { return NY - 4; }
};

template <class S>
__host__ __device__ inline bool sizes_match(const Grid& g) {
  return g.Nz == S::Nz() && g.X == S::X() && g.pz == S::pz() && g.px == S::px() && g.Q == S::Q() &&
         g.Qh == S::Qh() && g.R == S::R() && g.D == S::D();
}

// the grids with specialised builds
using Sizes32 = SizesCT<32, 65, 32>;
using Sizes16 = SizesCT<16, 33, 16>;

// Grid::fixed bits: the kernels that run their specialised build
enum : int { FIXED_PRODUCTS = 1, FIXED_RECON = 2, FIXED_SOLVE = 4 };

}  // namespace chn
