// Dimensions of the inverse transforms as digit GEMMs (the mma.sync kernel
// of phys_tc.cu and the tcgen05 kernel of phys_tc5.cu share them).
#pragma once

#include <vector>

#include "chn_common.cuh"
#include "setup.h"

namespace chn {

static constexpr int kFB = 2;  // fields per pass of the mma.sync inverse (its widest build)

// kept kz modes of even / odd padded index zp (kk < Nz/2: zp = kk; else
// zp = kk + 1 + Nz/2, which runs over the odd Nz + 1 ... 3Nz/2 - 1); an odd
// pz keeps all modes in one class
__host__ __device__ constexpr void z_class_counts(int Nz, int pz, int& nE, int& nO) {
  if (pz % 2) {
    nE = Nz - 1;
    nO = 0;
    return;
  }
  const int h = Nz / 2;
  nE = (h + 1) / 2 + (h - 1) / 2;
  nO = h / 2 + h / 2;
}

struct PhysTcDims {
  int Rz, Rx, pzh, pxh;           // radix of each stage's split, output rows per half
  int nxE, nxO;                   // x modes of even / odd j
  int KTzE, KTz, KTxE, KTx;       // k-tiles of the even class, and in all
  int MTz, MTx, KSz, KSx, NZ, NX;  // NZ = columns of the z stage, NX = of the x stage
};

// from the sizes (a constant expression for compile-time sizes); fb: fields
// per pass (the x stage has one column per (field, m))
__host__ __device__ constexpr PhysTcDims phys_tc_dims_n(int Nz, int pz, int px, int X, int fb) {
  PhysTcDims d{};
  d.Rz = pz % 2 ? 1 : 2;
  d.Rx = px % 2 ? 1 : 2;
  d.pzh = pz / d.Rz;
  d.pxh = px / d.Rx;
  int nzE = 0, nzO = 0;
  z_class_counts(Nz, pz, nzE, nzO);
  d.nxE = (X + d.Rx - 1) / d.Rx;
  d.nxO = X - d.nxE;
  d.KTzE = (2 * nzE + 15) / 16;
  d.KTz = d.KTzE + (2 * nzO + 15) / 16;
  d.KTxE = (2 * d.nxE + 15) / 16;
  d.KTx = d.KTxE + (2 * d.nxO + 15) / 16;
  d.MTz = (2 * d.pzh + 15) / 16;
  d.MTx = (d.pxh + 15) / 16;
  d.KSz = d.KTz * 16 + 8;
  d.KSx = d.KTx * 16 + 8;
  d.NZ = fb * X;
  d.NX = fb * pz;
  return d;
}

__host__ __device__ inline PhysTcDims phys_tc_dims(const Grid& g, int fb = kFB) {
  return phys_tc_dims_n(g.Nz, g.pz, g.px, g.X, fb);
}

// the two stages' matrices (rows x K words of Re, Im) and the z stage's
// K-word -> kept kz map
bool phys_tc_matrices(const HostTables& h, std::vector<double>& Az, std::vector<double>& Ax,
                      std::vector<int>& zmap, int& zrows, int& Kz, int& xrows, int& Kx);

}  // namespace chn
