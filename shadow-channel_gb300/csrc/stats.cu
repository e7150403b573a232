// Objectives and statistics straight from the stored trajectories, on the
// device, without going through physical space step by step.
//
// The reference's statistics (channel/__init__.py:217-299,
// drivers/sensitivities.py) call spec2phys for every step and average the
// physical field over x and z.  That average is the (kx, kz) = (0, 0) Fourier
// mode, which the Legendre coefficients give directly:
//   <u>(y) = sum_r R_r(y) a_r,  <w>(y) = sum_r R_r(y) b_r,  <v> = 0
// with (a, b) = C[0][alpha | beta][:, 0] (channel/project0.c:180-220).  Means
// of products use Parseval on the reconstructed velocity at the quadrature
// planes: <f g>(y) = sum over modes of w_kx Re(f^ conj(g^)), w_kx = 1 for
// kx = 0 and 2 otherwise (the real fields' kx < 0 half).  The wall shear is
// the reference's Uxb = Rp0 . a, Uzb = Rp0 . b (channel/project0.c:224-234)
// with Rp0 = R'(-1) (channel/RsQs.c:158-186).
#include <cstdio>
#include <vector>

#include "../../include/c_channel.h"
#include "chn_common.cuh"
#include "kernels.h"

namespace chn {

bool engine_grid_stream(const Grid** g, cudaStream_t* st);
void engine_set_error(int code, const char* msg);
void engine_count_launches(int n);
bool engine_traj(int batch, int inc, const cpx** base, long long* traj_stride, int* nseg, int* nsteps);

// out[s][j][y] = sum_r Br[y][r] Re(C_{s, start + j}[0][v][r][0])
__global__ void k_mean_mode_profile(Grid g, const cpx* __restrict__ traj, long long traj_stride, int start, int v,
                                    double* __restrict__ out) {
  const int j = blockIdx.x, s = blockIdx.y, count = gridDim.x;
  const size_t csz = coef_size(g);
  const cpx* C = traj + (long long)s * traj_stride + (size_t)3 * (start + j) * csz;
  for (int y = threadIdx.x; y < g.Q; y += blockDim.x) {
    const double* br = g.Br + (size_t)y * g.R;
    double acc = 0.0;
    for (int r = 0; r < g.R; ++r) acc += br[r] * C[((size_t)v * g.R + r) * g.X].re;
    out[((size_t)s * count + j) * g.Q + y] = acc;
  }
}

// out[s][j][0 | 1] = sum_r Rp0[r] Re(C[0][alpha | beta][r][0])
__global__ void k_wall_shear(Grid g, const cpx* __restrict__ traj, long long traj_stride, int start,
                             const double* __restrict__ rp0, double* __restrict__ out) {
  const int j = blockIdx.x, s = blockIdx.y, count = gridDim.x;
  const int v = threadIdx.x;  // 2 threads
  if (v > 1) return;
  const size_t csz = coef_size(g);
  const cpx* C = traj + (long long)s * traj_stride + (size_t)3 * (start + j) * csz;
  double acc = 0.0;
  for (int r = 0; r < g.R; ++r) acc += rp0[r] * C[((size_t)v * g.R + r) * g.X].re;
  out[((size_t)s * count + j) * 2 + v] = acc;
}

// out[i][y] = sum_{z != Nz/2, x} w_x Re(Ua_i[z][ca][y][x] conj(Ub_i[z][cb][y][x])), one block per (y, i)
__global__ void k_mean_product(Grid g, const cpx* __restrict__ Ua, const cpx* __restrict__ Ub, long long usz, int ca,
                               int cb, double* __restrict__ out) {
  const int y = blockIdx.x, i = blockIdx.y;
  const cpx* a = Ua + (long long)i * usz;
  const cpx* b = Ub + (long long)i * usz;
  double acc = 0.0;
  for (int t = threadIdx.x; t < g.Nz * g.X; t += blockDim.x) {
    const int z = t / g.X, x = t - z * g.X;
    if (z == g.Nz / 2) continue;
    const cpx p = a[(((size_t)z * 5 + ca) * g.Q + y) * g.X + x];
    const cpx q = b[(((size_t)z * 5 + cb) * g.Q + y) * g.X + x];
    acc += (x == 0 ? 1.0 : 2.0) * fma(p.re, q.re, p.im * q.im);
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(size_t)i * g.Q + y] = sh[0];
}

// R'_n(-1) for n < R: R_n = (1 - y^2) P_n, so R'_n = -2y P_n + (1 - y^2) P_n'
// = n P_{n-1} - (n + 2) y P_n (Legendre derivative identity), at y = -1
static std::vector<double> rp_at(int R, double y) {
  std::vector<double> P(R > 1 ? R : 2), out(R);
  P[0] = 1.0;
  P[1] = y;
  for (int n = 1; n + 1 < R; ++n) P[n + 1] = ((2. * n + 1.) * (y * P[n]) - n * P[n - 1]) / (double)(n + 1);
  out[0] = -2.0 * y;
  for (int n = 1; n < R; ++n) out[n] = n * P[n - 1] - (n + 2.0) * (y * P[n]);
  return out;
}

static bool trajectory(const char* fn, int batch, int inc, int start, int end, const Grid** g, cudaStream_t* st,
                       const cpx** base, long long* stride, int* nseg) {
  int nsteps = 0;
  char msg[256];
  if (!engine_grid_stream(g, st) || !engine_traj(batch, inc, base, stride, nseg, &nsteps)) {
    snprintf(msg, sizeof(msg), "%s: needs c_init%s first", fn, batch ? " and c_batch_init" : "");
    engine_set_error(-2, msg);
    return false;
  }
  if (!(0 <= start && start < end && end <= nsteps + 1)) {
    snprintf(msg, sizeof(msg), "%s: need 0 <= start < end <= nsteps + 1", fn);
    engine_set_error(-4, msg);
    return false;
  }
  return true;
}

static int finish(cudaStream_t st, int launches) {
  engine_count_launches(launches);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "statistics launch failed: %s", cudaGetErrorString(e));
    engine_set_error(-1, msg);
    return -1;
  }
  (void)st;
  return 0;
}

static int mean_profile(int batch, int inc, int comp, int start, int end, double* out_dev) {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  const cpx* base = nullptr;
  long long stride = 0;
  int nseg = 0;
  if (!trajectory("mean profile", batch, inc, start, end, &g, &st, &base, &stride, &nseg)) return -4;
  if (comp < 0 || comp > 2) {
    engine_set_error(-4, "mean profile: comp must be 0 (u), 1 (v) or 2 (w)");
    return -4;
  }
  const int count = end - start;
  if (comp == 1) {  // <v> = 0: the mean mode carries no wall-normal velocity
    return cudaMemsetAsync(out_dev, 0, sizeof(double) * (size_t)nseg * count * g->Q, st) == cudaSuccess ? 0 : -1;
  }
  k_mean_mode_profile<<<dim3(count, nseg), 128, 0, st>>>(*g, base, stride, start, comp == 0 ? 0 : 1, out_dev);
  return finish(st, 1);
}

static int wall_shear(int batch, int inc, int start, int end, double* out_dev) {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  const cpx* base = nullptr;
  long long stride = 0;
  int nseg = 0;
  if (!trajectory("wall shear", batch, inc, start, end, &g, &st, &base, &stride, &nseg)) return -4;
  const std::vector<double> rp0 = rp_at(g->R, -1.0);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * rp0.size()) != cudaSuccess) return -1;
  cudaMemcpyAsync(d, rp0.data(), sizeof(double) * rp0.size(), cudaMemcpyHostToDevice, st);
  k_wall_shear<<<dim3(end - start, nseg), 32, 0, st>>>(*g, base, stride, start, d, out_dev);
  const int rc = finish(st, 1);
  cudaStreamSynchronize(st);
  cudaFree(d);
  return rc;
}

// <f g>(y) for f = component ca of trajectory inc_a, g = component cb of inc_b
static int mean_product(int batch, int inc_a, int ca, int inc_b, int cb, int start, int end, double* out_dev) {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  const cpx *ba = nullptr, *bb = nullptr;
  long long sa = 0, sb = 0;
  int nseg = 0;
  if (!trajectory("mean product", batch, inc_a, start, end, &g, &st, &ba, &sa, &nseg) ||
      !trajectory("mean product", batch, inc_b, start, end, &g, &st, &bb, &sb, &nseg))
    return -4;
  if (ca < 0 || ca > 2 || cb < 0 || cb > 2) {
    engine_set_error(-4, "mean product: components must be 0 (u), 1 (v) or 2 (w)");
    return -4;
  }
  const int count = end - start;
  const size_t csz = coef_size(*g), usz = u_size(*g);
  const int chunk = count < 32 ? count : 32;
  cpx *Ua = nullptr, *Ub = nullptr;
  if (cudaMalloc(&Ua, sizeof(cpx) * usz * chunk) != cudaSuccess ||
      cudaMalloc(&Ub, sizeof(cpx) * usz * chunk) != cudaSuccess) {
    cudaFree(Ua);
    cudaGetLastError();
    engine_set_error(-1, "mean product: device allocation failed");
    return -1;
  }
  int launches = 0;
  for (int s = 0; s < nseg; ++s)
    for (int j0 = 0; j0 < count; j0 += chunk) {
      const int n = (count - j0) < chunk ? (count - j0) : chunk;
      ReconArgs r{};
      r.slot = SlotRef{nullptr, 0, 0, 0};
      r.ninst = n;
      r.status = nullptr;
      r.sdiv = 1;
      r.C = Batch<const cpx>{ba + (long long)s * sa + (long long)(3 * (start + j0) * csz), (long long)(3 * csz)};
      r.U = Batch<cpx>{Ua, (long long)usz};
      launch_recon(*g, r, st);
      r.C = Batch<const cpx>{bb + (long long)s * sb + (long long)(3 * (start + j0) * csz), (long long)(3 * csz)};
      r.U = Batch<cpx>{Ub, (long long)usz};
      launch_recon(*g, r, st);
      k_mean_product<<<dim3(g->Q, n), 256, 0, st>>>(*g, Ua, Ub, (long long)usz, ca, cb,
                                                     out_dev + ((size_t)s * count + j0) * g->Q);
      launches += 3;
    }
  const int rc = finish(st, launches);
  cudaStreamSynchronize(st);
  cudaFree(Ua);
  cudaFree(Ub);
  return rc;
}

// host-array variants: one device staging buffer per call
template <typename F>
static int to_host(size_t n, double* out, F&& f) {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  if (!engine_grid_stream(&g, &st)) {
    engine_set_error(-2, "statistics: needs c_init first");
    return -2;
  }
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (n > 0 ? n : 1)) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  int rc = f(d);
  if (rc == 0 && (cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                  cudaStreamSynchronize(st) != cudaSuccess))
    rc = -1;
  cudaFree(d);
  return rc;
}

static int qpts_now() {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  return engine_grid_stream(&g, &st) ? g->Q : 0;
}

static int batch_nseg() {
  const cpx* b = nullptr;
  long long s = 0;
  int nseg = 0, nsteps = 0;
  return engine_traj(1, 0, &b, &s, &nseg, &nsteps) ? nseg : 0;
}

}  // namespace chn

using namespace chn;

extern "C" {

int c_mean_profile(int inc, int comp, int start_step, int end_step, double* out) {
  const size_t n = (size_t)(end_step > start_step ? end_step - start_step : 0) * qpts_now();
  return to_host(n, out, [&](double* d) { return mean_profile(0, inc, comp, start_step, end_step, d); });
}

int c_wall_shear_weights(double* out) {
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  if (!out || !engine_grid_stream(&g, &st)) {
    engine_set_error(-2, "c_wall_shear_weights: needs c_init first and an output array");
    return -2;
  }
  const std::vector<double> rp0 = rp_at(g->R, -1.0);
  for (size_t i = 0; i < rp0.size(); ++i) out[i] = rp0[i];
  return 0;
}

int c_wall_shear(int inc, int start_step, int end_step, double* out) {
  const size_t n = (size_t)(end_step > start_step ? end_step - start_step : 0) * 2;
  return to_host(n, out, [&](double* d) { return wall_shear(0, inc, start_step, end_step, d); });
}

int c_mean_product(int inc_a, int comp_a, int inc_b, int comp_b, int start_step, int end_step, double* out) {
  const size_t n = (size_t)(end_step > start_step ? end_step - start_step : 0) * qpts_now();
  return to_host(n, out,
                 [&](double* d) { return mean_product(0, inc_a, comp_a, inc_b, comp_b, start_step, end_step, d); });
}

int c_batch_mean_profile_dev(int inc, int comp, int start_step, int end_step, double* out) {
  return mean_profile(1, inc, comp, start_step, end_step, out);
}

int c_batch_wall_shear_dev(int inc, int start_step, int end_step, double* out) {
  return wall_shear(1, inc, start_step, end_step, out);
}

int c_batch_mean_product_dev(int inc_a, int comp_a, int inc_b, int comp_b, int start_step, int end_step,
                             double* out) {
  return mean_product(1, inc_a, comp_a, inc_b, comp_b, start_step, end_step, out);
}

int c_batch_mean_profile(int inc, int comp, int start_step, int end_step, double* out) {
  const size_t n = (size_t)batch_nseg() * (end_step > start_step ? end_step - start_step : 0) * qpts_now();
  return to_host(n, out, [&](double* d) { return mean_profile(1, inc, comp, start_step, end_step, d); });
}

}  // extern "C"
