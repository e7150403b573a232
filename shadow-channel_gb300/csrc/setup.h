// Host-side construction of the time-invariant tables of the Legendre-Galerkin
// channel discretisation: quadrature, basis values, banded Gram matrices, and
// the LU factors of every implicit operator the RK3 step can ask for.
#pragma once

#include <stdint.h>

#include <vector>

namespace chn {

struct HostTables {
  int Nx, Ny, Nz, X, Q, R, D, pz, px;
  double Lx, Lz, Re, re, flux, dt;
  std::vector<double> y, w;                 // quadrature points (ascending) and weights
  std::vector<double> Bq, Bqp, Bqpp;        // [Q][D]
  std::vector<double> Br, Brp;              // [Q][R]
  std::vector<double> Wq, Wqp, Wqpp;        // [D][Q]
  std::vector<double> Wr, Wrp;              // [R][Q]
  std::vector<double> Qs, Qps, Qpps;        // [D][9]
  std::vector<double> Rs, Rps;              // [R][5]
  std::vector<double> Kx, Kz, K2, kxK2, kzK2, cfl2;
  double cfl1, cfl3;
  std::vector<double> luA, luB, exA, exB;   // see Grid in chn_common.cuh
  std::vector<double> lu0, ex0, add0, rwsum;
  std::vector<double> rdA, rdB, rd0;         // reciprocals of the LU pivots (0 where a pivot is 0)
  std::vector<double> twz, twx;             // interleaved re,im
};

// Returns false (with a message in err) for parameters the reference rejects
// (channel/channel.c:301-312: Nx % 4, Nz % 2, Ny > 4).
bool build_tables(int Nx, int Ny, int Nz, double Lx, double Lz, double Re, double flux,
                  double dt, HostTables& t, const char** err);

// No-pivot LU of a banded matrix whose nonzeros sit on even offsets only, in
// place, rows of pitch w with the diagonal in column dl (the reference's
// elimination order, channel/mvOps.c:35-65): L multipliers left of column
// dl, the pivots in column dl, U to the right.
void band_lu(double* A, int w, int dl, int du, int N);

// base-256 digit tables of the five Legendre bases and of their weighted
// transposes for the tensor-core contractions (recon_tc.cu, tc_common.cuh)
bool build_recon_tc_tables(const HostTables& h, std::vector<uint32_t>& frag, std::vector<int>& ex,
                           std::vector<uint32_t>& wfrag, std::vector<int>& wex);
bool build_adj_tc_tables(const HostTables& h, std::vector<uint32_t>& btfrag, std::vector<int>& btex,
                         std::vector<uint32_t>& wtfrag, std::vector<int>& wtex);
// DFT matrices of the inverse z and x transforms as digit tables (phys_tc.cu)
bool build_phys_tc_tables(const HostTables& h, std::vector<uint32_t>& zfrag, std::vector<int>& zex,
                          std::vector<uint32_t>& xfrag, std::vector<int>& xex, std::vector<int>& zmap);
// the same matrices' digit tables as tcgen05 B operands (phys_tc5.cu)
bool build_phys_tc5_tables(const HostTables& h, std::vector<uint8_t>& zt, std::vector<uint8_t>& xt);
// DFT matrices of the forward x and z transforms as digit tables (phys_tc.cu)
bool build_fwd_tc_tables(const HostTables& h, std::vector<uint32_t>& xfrag, std::vector<int>& xex,
                         std::vector<uint32_t>& zfrag, std::vector<int>& zex, std::vector<uint32_t>& ufrag,
                         std::vector<int>& uex);

}  // namespace chn
