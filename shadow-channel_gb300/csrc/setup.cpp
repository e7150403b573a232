// Host-side table construction; see setup.h.
//
// Discretisation (channel/RsQs.c:30-49, channel/LegendreSetup.c:25-527):
//   Gauss-Legendre points y_j (Q = 3Ny/2 of them) and weights w_j;
//   R_n(y) = (1-y^2) P_n(y),  n < Ny-2   (wall-normal vorticity basis)
//   Q_n(y) = (1-y^2)^2 P_n(y), n < Ny-4  (wall-normal velocity basis)
//   banded Gram matrices <Q_i,Q_j>, <Q_i',Q_j'>, <Q_i'',Q_j''>, <R_i,R_j>,
//   <R_i',R_j'> by quadrature, nonzero only on even offsets (parity).
// The tables are built with the reference's formulas in the same
// floating-point association (this file is compiled without FMA
// contraction), so they agree with the reference's bit for bit;
// tests/test_product_setup.py checks that on the CPU.
#include "setup.h"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace chn {

// Legendre polynomial P_n(x) by the three-term recurrence, evaluated in the
// same association as channel/LegendreSetup.c:535-549.
static double legendre_at(int n, double x) {
  double prev = 0.0, curr = 1.0;
  for (int j = 0; j < n; ++j) {
    const double next = ((double)(2 * j + 1) * x * curr - (double)j * prev) / (double)(j + 1);
    prev = curr;
    curr = next;
  }
  return curr;
}

// Gauss-Legendre nodes.  The nodes are part of the discretisation: every
// basis table, Gram matrix and implicit operator is built on them, and the
// stiff fourth-order operator amplifies a 1e-15 change of a node into a 1e-11
// change of the state after one step.  The reference stops its root search at
// a bracket width of 1e-15 (channel/LegendreSetup.c:566-643), so its nodes
// are not the correctly rounded roots; to reproduce its results the search
// itself is kept alike: sign changes of P_n bracketed on a doubling set of
// Chebyshev points, then a safeguarded secant (steps clamped to at least 5%
// of the bracket, a bisection every tenth iteration) to a 1e-15 bracket.
static bool gauss_nodes(int n, std::vector<double>& x) {
  const int nd2 = n / 2;
  std::vector<double> lo(n, 0.0), hi(n, 0.0);
  int k = n, m = 0;
  while (m < nd2) {
    k *= 2;
    double a = -1.0, pa = legendre_at(n, a);
    m = 0;
    for (int r = 1; r <= k; ++r) {
      const double b = -cos(0.5 * M_PI * (r - 0.5) / k);
      const double pb = legendre_at(n, b);
      if (pa * pb < 0) {
        lo[m] = a;
        hi[m] = b;
        ++m;
      }
      pa = pb;
      a = b;
    }
  }
  x.assign(n, 0.0);
  double x3 = 0.0;
  for (m = 0; m < nd2; ++m) {
    double x1 = lo[m], x2 = hi[m];
    double p1 = legendre_at(n, x1), p2 = legendre_at(n, x2);
    int it = 1;
    while (std::fabs(x2 - x1) > 1e-15 && it < 200) {
      if (it % 10 == 0) {
        x3 = 0.5 * (x1 + x2);
      } else if (std::fabs(p1) < std::fabs(p2)) {
        const double f = p1 / (p1 - p2);
        x3 = x1 + (f > 0.05 ? f : 0.05) * (x2 - x1);
      } else {
        const double f = p2 / (p1 - p2);
        x3 = x2 + (f < -0.05 ? f : -0.05) * (x2 - x1);
      }
      const double p3 = legendre_at(n, x3);
      if (p3 * p1 <= 0) {
        x2 = x3;
        p2 = p3;
      } else {
        x1 = x3;
        p1 = p3;
      }
      ++it;
    }
    if (it == 200) return false;
    x[m] = x3;
    x[n - 1 - m] = -x3;
  }
  if (n % 2 == 1) x[nd2] = 0.0;
  return true;
}

static bool gauss_legendre(int n, std::vector<double>& y, std::vector<double>& w) {
  if (!gauss_nodes(n, y)) return false;
  w.assign(n, 0.0);
  for (int k = 0; k < (n + 1) / 2; ++k) {
    const double v = (double)n * (legendre_at(n - 1, y[k]) - y[k] * legendre_at(n, y[k]));
    w[k] = 2. * (1. - y[k] * y[k]) / (v * v);
    w[n - 1 - k] = w[k];
  }
  return true;
}

// band[i][c + s] = sum_k Wt[i][k] B[k][i+2s] (s < nd), mirrored below the diagonal
static void gram_band(std::vector<double>& band, int N, int width, int centre, int nd,
                      const std::vector<double>& Wt, const std::vector<double>& B, int Bcols, int Q) {
  band.assign((size_t)N * width, 0.0);
  for (int s = 0; s < nd; ++s)
    for (int i = 0; i + 2 * s < N; ++i) {
      double acc = 0.0;
      for (int k = 0; k < Q; ++k) acc += Wt[(size_t)i * Q + k] * B[(size_t)k * Bcols + i + 2 * s];
      band[(size_t)i * width + centre + s] = acc;
      if (s > 0) band[(size_t)(i + 2 * s) * width + centre - s] = acc;
    }
}

void band_lu(double* A, int w, int dl, int du, int N) {
  auto a = [&](int i, int j) -> double& { return A[(size_t)i * w + j]; };
  for (int i = 2; i < N; ++i) {
    const int j0 = dl - i / 2 > 0 ? dl - i / 2 : 0;
    for (int j = j0; j < dl; ++j) {
      for (int k = 1; k <= j - j0; ++k) a(i, j) = a(i, j) - a(i, j - k) * a(i - 2 * (dl - j + k), dl + k);
      a(i, j) = a(i, j) / a(i - 2 * (dl - j), dl);
    }
    const int jm = du < (N - i + 1) / 2 ? du : (N - i + 1) / 2;
    for (int j = 0; j < jm; ++j) {
      int km = i / 2;
      if (dl < km) km = dl;
      if (du - j < km) km = du - j;
      for (int k = 1; k <= km; ++k) a(i, j + dl) = a(i, j + dl) - a(i, dl - k) * a(i - 2 * k, dl + j + k);
    }
  }
}

// solve with factors from band_lu, single real right-hand side
static void band_solve(const double* A, int w, int dl, int du, int N, double* b) {
  auto a = [&](int i, int j) { return A[(size_t)i * w + j]; };
  for (int i = 2; i < N; ++i) {
    const int j0 = dl - i / 2 > 0 ? dl - i / 2 : 0;
    for (int j = j0; j < dl; ++j) b[i] -= a(i, j) * b[i - 2 * (dl - j)];
  }
  b[N - 1] /= a(N - 1, dl);
  b[N - 2] /= a(N - 2, dl);
  for (int i = N - 3; i >= 0; --i) {
    int jm = (N - i + 1) / 2 - 1;
    if (du < jm) jm = du;
    for (int j = 1; j <= jm; ++j) b[i] -= a(i, dl + j) * b[i + 2 * j];
    b[i] /= a(i, dl);
  }
}

static void twiddles(int n, std::vector<double>& tw) {
  tw.assign(2 * (size_t)n, 0.0);
  const long double pi2 = 6.283185307179586476925286766559005768L;
  for (int k = 0; k < n; ++k) {
    long double a = pi2 * k / n;
    double c = (double)cosl(a), s = -(double)sinl(a);
    if (4 * k == n) { c = 0.0; s = -1.0; }
    if (2 * k == n) { c = -1.0; s = 0.0; }
    if (4 * k == 3 * n) { c = 0.0; s = 1.0; }
    if (k == 0) { c = 1.0; s = 0.0; }
    tw[2 * k] = c;
    tw[2 * k + 1] = s;
  }
}

bool build_tables(int Nx, int Ny, int Nz, double Lx, double Lz, double Re, double flux, double dt,
                  HostTables& t, const char** err) {
  if (Nx % 4 != 0 || Nx <= 0) { *err = "Nx must be a positive multiple of 4"; return false; }
  if (Nz % 2 != 0 || Nz <= 0) { *err = "Nz must be a positive even number"; return false; }
  if (Ny - 4 < 1) { *err = "Ny must exceed 4"; return false; }
  t.Nx = Nx; t.Ny = Ny; t.Nz = Nz; t.X = Nx / 2;
  t.Q = 3 * Ny / 2; t.R = Ny - 2; t.D = Ny - 4;
  t.pz = 3 * Nz / 2; t.px = 3 * Nx / 2;
  t.Lx = Lx; t.Lz = Lz; t.Re = Re; t.re = 1.0 / Re; t.flux = flux; t.dt = dt;
  const int Q = t.Q, R = t.R, D = t.D, X = t.X;

  if (!gauss_legendre(Q, t.y, t.w)) { *err = "Gauss-Legendre node search did not converge"; return false; }
  // Legendre values P[k][n], n < R
  std::vector<double> P((size_t)Q * R);
  for (int k = 0; k < Q; ++k) {
    const double x = t.y[k];
    P[(size_t)k * R] = 1.0;
    if (R > 1) P[(size_t)k * R + 1] = x;
    for (int n = 1; n + 1 < R; ++n)
      P[(size_t)k * R + n + 1] = ((2.0 * n + 1.0) * (x * P[(size_t)k * R + n]) - n * P[(size_t)k * R + n - 1]) / (n + 1.0);
  }
  t.Bq.assign((size_t)Q * D, 0); t.Bqp.assign((size_t)Q * D, 0); t.Bqpp.assign((size_t)Q * D, 0);
  t.Br.assign((size_t)Q * R, 0); t.Brp.assign((size_t)Q * R, 0);
  for (int k = 0; k < Q; ++k) {
    const double x = t.y[k], s = 1.0 - x * x, x2 = x * x;
    const double* p = &P[(size_t)k * R];
    for (int n = 0; n < R; ++n) {
      t.Br[(size_t)k * R + n] = s * p[n];
      // d/dy [(1-y^2) P_n] = n P_{n-1} - (n+2) y P_n   (from (1-y^2)P_n' = n(P_{n-1} - y P_n))
      t.Brp[(size_t)k * R + n] = n == 0 ? -2.0 * x : n * p[n - 1] - (n + 2.0) * (x * p[n]);
    }
    for (int n = 0; n < D; ++n) {
      t.Bq[(size_t)k * D + n] = s * (s * p[n]);
      // d/dy [(1-y^2)^2 P_n] = (1-y^2) [n P_{n-1} - (n+4) y P_n]
      t.Bqp[(size_t)k * D + n] = n == 0 ? -4.0 * x * s : s * (n * p[n - 1] - (n + 4.0) * (x * p[n]));
      // second derivative, using Legendre's equation to remove P_n''
      t.Bqpp[(size_t)k * D + n] = n == 0 ? 12.0 * x2 - 4.0
          : (12.0 + 7.0 * n + (double)n * n) * (x2 * p[n]) - (4.0 + (double)n * n + n) * p[n] - 6.0 * n * (x * p[n - 1]);
    }
  }
  auto weighted = [&](const std::vector<double>& B, int cols, std::vector<double>& Wt) {
    Wt.assign((size_t)cols * Q, 0.0);
    for (int i = 0; i < cols; ++i)
      for (int k = 0; k < Q; ++k) Wt[(size_t)i * Q + k] = t.w[k] * B[(size_t)k * cols + i];
  };
  weighted(t.Bq, D, t.Wq); weighted(t.Bqp, D, t.Wqp); weighted(t.Bqpp, D, t.Wqpp);
  weighted(t.Br, R, t.Wr); weighted(t.Brp, R, t.Wrp);
  gram_band(t.Qs, D, 9, 4, 5, t.Wq, t.Bq, D, Q);
  gram_band(t.Qps, D, 9, 4, 4, t.Wqp, t.Bqp, D, Q);
  gram_band(t.Qpps, D, 9, 4, 3, t.Wqpp, t.Bqpp, D, Q);
  gram_band(t.Rs, R, 5, 2, 3, t.Wr, t.Br, R, Q);
  gram_band(t.Rps, R, 5, 2, 2, t.Wrp, t.Brp, R, Q);

  // wavenumbers in FFT order (channel/waveNumsAndCFL.c:22-62)
  t.Kx.assign(X, 0); t.Kz.assign(Nz, 0);
  for (int i = 0; i < X; ++i) t.Kx[i] = i * (2.0 * M_PI / Lx);
  for (int i = 0; i < Nz / 2 + 1; ++i) t.Kz[i] = i * (2.0 * M_PI / Lz);
  for (int i = Nz / 2 + 1; i < Nz; ++i) t.Kz[i] = (i - Nz) * (2.0 * M_PI / Lz);
  t.K2.assign((size_t)Nz * X, 0); t.kxK2.assign((size_t)Nz * X, 0); t.kzK2.assign((size_t)Nz * X, 0);
  for (int z = 0; z < Nz; ++z)
    for (int x = 0; x < X; ++x) {
      const double k2 = t.Kz[z] * t.Kz[z] + t.Kx[x] * t.Kx[x];
      t.K2[(size_t)z * X + x] = k2;
      if (k2 > 0) {
        t.kxK2[(size_t)z * X + x] = t.Kx[x] / k2;
        t.kzK2[(size_t)z * X + x] = t.Kz[z] / k2;
      }
    }
  // CFL constants (channel/waveNumsAndCFL.c:65-96)
  t.cfl1 = M_PI / (Lx / Nx);
  t.cfl3 = M_PI / (Lz / Nz);
  t.cfl2.assign(Q, 0);
  for (int j = 1; j < Q - 1; ++j) t.cfl2[j] = 2.0 * M_PI / (t.y[j + 1] - t.y[j - 1]);
  t.cfl2[0] = t.cfl2[Q - 1] = M_PI / (t.y[0] + 1.0);

  // implicit / explicit operators (channel/project.c:60-95, 143-174, 354-390)
  const double bval[3] = {1.0 / 6, 2.0 / 3, 0.0};
  const double aval[2] = {1.0 / 3, -1.0 / 2};
  const size_t nA = (size_t)D * 9, nB = (size_t)R * 5;
  t.luA.assign(3 * (size_t)Nz * X * nA, 0); t.luB.assign(3 * (size_t)Nz * X * nB, 0);
  t.exA.assign(2 * (size_t)Nz * X * nA, 0); t.exB.assign(2 * (size_t)Nz * X * nB, 0);
  const double re = t.re;
  for (int z = 0; z < Nz; ++z)
    for (int x = 0; x < X; ++x) {
      const double k2 = t.K2[(size_t)z * X + x], sq = k2 * k2;
      const size_t zx = (size_t)z * X + x;
      if (k2 == 0.0) continue;  // the mean mode uses the R-basis systems below
      for (int bi = 0; bi < 3; ++bi) {
        double* A = &t.luA[((size_t)bi * Nz * X + zx) * nA];
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < 9; ++j) {
            const double qs = t.Qs[(size_t)i * 9 + j], qps = t.Qps[(size_t)i * 9 + j], qpps = t.Qpps[(size_t)i * 9 + j];
            A[(size_t)i * 9 + j] = -(k2 * qs + qps) - re * bval[bi] * dt * (sq * qs + 2. * k2 * qps + qpps);
          }
        band_lu(A, 9, 4, 4, D);
        double* B = &t.luB[((size_t)bi * Nz * X + zx) * nB];
        for (int i = 0; i < R; ++i)
          for (int j = 0; j < 5; ++j)
            B[(size_t)i * 5 + j] = t.Rs[(size_t)i * 5 + j] + re * bval[bi] * dt * (t.Rps[(size_t)i * 5 + j] + k2 * t.Rs[(size_t)i * 5 + j]);
        band_lu(B, 5, 2, 2, R);
      }
      for (int ai = 0; ai < 2; ++ai) {
        double* A = &t.exA[((size_t)ai * Nz * X + zx) * nA];
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < 9; ++j) {
            const double qs = t.Qs[(size_t)i * 9 + j], qps = t.Qps[(size_t)i * 9 + j], qpps = t.Qpps[(size_t)i * 9 + j];
            A[(size_t)i * 9 + j] = -(k2 * qs + qps) + re * aval[ai] * dt * (sq * qs + 2. * k2 * qps + qpps);
          }
        double* B = &t.exB[((size_t)ai * Nz * X + zx) * nB];
        for (int i = 0; i < R; ++i)
          for (int j = 0; j < 5; ++j)
            B[(size_t)i * 5 + j] = t.Rs[(size_t)i * 5 + j] - re * aval[ai] * dt * (t.Rps[(size_t)i * 5 + j] + k2 * t.Rs[(size_t)i * 5 + j]);
      }
    }
  // mean mode (channel/project0.c:61-149, channel/adjproject0.c:47-151)
  t.lu0.assign(3 * nB, 0); t.ex0.assign(2 * nB, 0); t.add0.assign(4 * (size_t)R, 0); t.rwsum.assign(R, 0);
  for (int i = 0; i < R; ++i) {
    double acc = 0.0;
    for (int k = 0; k < Q; ++k) acc += t.Wr[(size_t)i * Q + k];
    t.rwsum[i] = acc;
  }
  for (int bi = 0; bi < 3; ++bi) {
    double* A = &t.lu0[(size_t)bi * nB];
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < 5; ++j) A[(size_t)i * 5 + j] = t.Rs[(size_t)i * 5 + j] + re * bval[bi] * dt * t.Rps[(size_t)i * 5 + j];
    band_lu(A, 5, 2, 2, R);
    std::vector<double> v(t.rwsum);
    band_solve(A, 5, 2, 2, R, v.data());
    std::memcpy(&t.add0[(size_t)(1 + bi) * R], v.data(), sizeof(double) * R);
  }
  // the back substitution multiplies by the pivot's reciprocal (one FP64
  // rounding more than the reference's division, channel/mvOps.c:80-90)
  auto recip = [](const std::vector<double>& lu, int w, int dl, std::vector<double>& rd) {
    rd.assign(lu.size() / w, 0.0);
    for (size_t r = 0; r < rd.size(); ++r) {
      const double p = lu[r * w + dl];
      rd[r] = p != 0.0 ? 1.0 / p : 0.0;
    }
  };
  recip(t.luA, 9, 4, t.rdA);
  recip(t.luB, 5, 2, t.rdB);
  recip(t.lu0, 5, 2, t.rd0);
  {
    std::vector<double> A(t.Rs);
    band_lu(A.data(), 5, 2, 2, R);
    std::vector<double> v(t.rwsum);
    band_solve(A.data(), 5, 2, 2, R, v.data());
    std::memcpy(&t.add0[0], v.data(), sizeof(double) * R);
  }
  for (int ai = 0; ai < 2; ++ai)
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < 5; ++j)
        t.ex0[(size_t)ai * nB + (size_t)i * 5 + j] = t.Rs[(size_t)i * 5 + j] - re * aval[ai] * dt * t.Rps[(size_t)i * 5 + j];
  twiddles(t.pz, t.twz);
  twiddles(t.px, t.twx);
  return true;
}

}  // namespace chn

// Host-only access to the setup tables (no GPU needed), for tests.
extern "C" int c_setup_table(int Nx, int Ny, int Nz, double Lx, double Lz, double Re, double flux, double dt,
                             int which, double* out, int n) {
  chn::HostTables t;
  const char* err = nullptr;
  if (!chn::build_tables(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, t, &err)) return -1;
  const std::vector<double>* v[] = {&t.Bq, &t.Bqp, &t.Bqpp, &t.Br, &t.Brp, &t.Wq, &t.Wqp, &t.Wqpp, &t.Wr,
                                    &t.Wrp, &t.Qs, &t.Qps, &t.Qpps, &t.Rs, &t.Rps, &t.y, &t.w};
  if (which < 0 || which >= (int)(sizeof(v) / sizeof(v[0]))) return -1;
  const std::vector<double>& a = *v[which];
  if (out && n >= (int)a.size()) std::memcpy(out, a.data(), sizeof(double) * a.size());
  return (int)a.size();
}

extern "C" int c_setup_tc_table(int Nx, int Ny, int Nz, double Lx, double Lz, double Re, double flux, double dt,
                                int which, uint32_t* frag, long long nfrag, int* ex, long long nex,
                                long long* sizes) {
  chn::HostTables t;
  const char* err = nullptr;
  if (!sizes || !chn::build_tables(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, t, &err)) return -1;
  std::vector<uint32_t> f[3];
  std::vector<int> e[3], m;
  bool ok = false;
  int sel = 0;
  switch (which) {
    case 0: case 1: ok = chn::build_recon_tc_tables(t, f[0], e[0], f[1], e[1]); sel = which; break;
    case 2: case 3: ok = chn::build_phys_tc_tables(t, f[0], e[0], f[1], e[1], m); sel = which - 2; break;
    case 4: case 5: case 6: ok = chn::build_fwd_tc_tables(t, f[0], e[0], f[1], e[1], f[2], e[2]); sel = which - 4; break;
    case 7: case 8: ok = chn::build_adj_tc_tables(t, f[0], e[0], f[1], e[1]); sel = which - 7; break;
    case 9: case 10: {
      // the tcgen05 inverse's stacked tables (bytes as 32-bit words) with the
      // row exponents of the mma.sync tables they share
      std::vector<uint8_t> zt, xt;
      ok = chn::build_phys_tc5_tables(t, zt, xt) && chn::build_phys_tc_tables(t, f[2], e[0], f[2], e[1], m);
      const std::vector<uint8_t>& b = which == 9 ? zt : xt;
      f[which - 9].assign(b.size() / 4, 0u);
      if (!b.empty()) std::memcpy(f[which - 9].data(), b.data(), b.size());
      sel = which - 9;
      break;
    }
    default: return -1;
  }
  if (!ok) return -1;
  sizes[0] = (long long)f[sel].size();
  sizes[1] = (long long)e[sel].size();
  // null buffers: a size query; a buffer shorter than its table: an error
  if ((frag && nfrag < sizes[0]) || (ex && nex < sizes[1])) return -2;
  if (frag) std::memcpy(frag, f[sel].data(), sizeof(uint32_t) * f[sel].size());
  if (ex) std::memcpy(ex, e[sel].data(), sizeof(int) * e[sel].size());
  return 0;
}
