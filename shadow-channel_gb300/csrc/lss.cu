// Least-squares shadowing (LSS) on the device: the KKT matrix-vector product
// of drivers/wrapper.py:5-54 and the MINRES iteration of drivers/pariter.py:63-125,
// over a batch whose segments are the consecutive time windows of one
// trajectory (c_batch_init_steps + c_batch_set_chain + c_batch_primal_dev).
//
// Unknowns x = [v_0 .. v_{n-1}, w_0 .. w_{n-2}], each a coefficient array
// [Nz][2][dimR][Nx/2] of complex doubles (the reference's float view x[::2] +
// 1j x[1::2] is the same memory).  Per segment i:
//   forward:  v' = P_end T(P_start v_i)       (tangent, no forcing or mean-flux forcing)
//   backward: w' = P_start A(P_end w_i)       (adjoint with ddt coupling, strength 1)
// with P the ddt_project of channel/channel.c:704-780, and the residual
//   R_v[i] = w_{i-1} - w'_i  (w_{-1} = 0),   R_w[i] = v_{i+1} - v'_i.
// zeta[i] = -(projection coefficient of v' at the window end).
#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/c_channel.h"
#include "chn_common.cuh"
#include "kernels.h"

namespace chn {

bool engine_batch_shape(int* nseg, int* ntan, int* chain, size_t* csz, int* nsteps);
bool engine_grid_stream(const Grid** g, cudaStream_t* st);
void engine_set_error(int code, const char* msg);
void engine_count_launches(int n);
int engine_status();

__global__ void k_kkt_residual(size_t m, int nseg, const cpx* __restrict__ x, const cpx* __restrict__ V,
                               const cpx* __restrict__ W, cpx* __restrict__ y) {
  const size_t nv = (size_t)nseg * m;
  const size_t n = nv + (size_t)(nseg - 1) * m;
  const cpx* xw = x + nv;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    cpx out;
    if (i < nv) {
      const size_t seg = i / m;
      const cpx a = seg > 0 ? xw[i - m] : cpx{0.0, 0.0};
      out.re = a.re - W[i].re;
      out.im = a.im - W[i].im;
    } else {
      const size_t j = i - nv;  // R_w[seg] = v_{seg+1} - V[seg]
      out.re = x[j + m].re - V[j].re;
      out.im = x[j + m].im - V[j].im;
    }
    y[i] = out;
  }
}

__global__ void k_negate(int n, const double* __restrict__ a, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = -a[i];
}

// deterministic dot product: a fixed grid of partial sums, then one block
constexpr int kDotGrid = 304;  // 2 x 152 SMs
constexpr int kDotThreads = 256;

__global__ void k_dot_partial(size_t n, const double* __restrict__ a, const double* __restrict__ b,
                              double* __restrict__ part) {
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    acc = fma(a[i], b[i], acc);
  __shared__ double sh[kDotThreads];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int k = kDotThreads / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_dot_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sh[kDotThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) acc += part[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int k = kDotThreads / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) sh[threadIdx.x] += sh[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// MINRES vector updates, in the reference's operation order
__global__ void k_sub_scaled_pair(size_t n, double* __restrict__ out, const double* __restrict__ av, double alpha,
                                  const double* __restrict__ v, double beta, const double* __restrict__ vm) {
  // out = (av - alpha v) - beta vm
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (av[i] - alpha * v[i]) - beta * vm[i];
}

__global__ void k_direction(size_t n, double* __restrict__ out, const double* __restrict__ v, double p3,
                            const double* __restrict__ wm, double p2, const double* __restrict__ w, double p1) {
  // out = ((v - p3 wm) - p2 w) / p1
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = ((v[i] - p3 * wm[i]) - p2 * w[i]) / p1;
}

__global__ void k_axpy(size_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

__global__ void k_div(size_t n, double* __restrict__ x, double d) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    x[i] /= d;
}

__global__ void k_sub(size_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] - b[i];
}

static unsigned vec_blocks(size_t n) {
  const size_t nb = (n + 255) / 256;
  return (unsigned)(nb < 1216 ? (nb > 0 ? nb : 1) : 1216);  // 8 x 152 SMs
}

// device buffers of the LSS operator, sized for the current batch
struct LssBuffers {
  int nseg = 0;
  size_t csz = 0;
  cpx *V = nullptr, *W = nullptr;
  double *r = nullptr, *part = nullptr, *dot = nullptr;
  double* vec[7] = {};  // MINRES: vi, vim, vip, Avi, wi, wim, wip
  size_t nvec = 0;      // doubles per MINRES vector
  void release() {
    cudaFree(V);
    cudaFree(W);
    cudaFree(r);
    cudaFree(part);
    cudaFree(dot);
    for (double*& p : vec) {
      cudaFree(p);
      p = nullptr;
    }
    *this = LssBuffers();
  }
};
static LssBuffers B;

static bool lss_ready(const char* fn, int* nseg, size_t* csz, int* L, const Grid** g, cudaStream_t* st) {
  int ntan = 0, chain = 0, nsteps = 0;
  char msg[256];
  if (!engine_grid_stream(g, st) || !engine_batch_shape(nseg, &ntan, &chain, csz, &nsteps)) {
    snprintf(msg, sizeof(msg), "%s: needs c_init and c_batch_init_steps first", fn);
    engine_set_error(-2, msg);
    return false;
  }
  if (ntan != 1 || chain <= 0 || *nseg < 1) {
    snprintf(msg, sizeof(msg), "%s: the batch must hold one tangent per segment (ntan 1) and be chained "
             "(c_batch_set_chain)", fn);
    engine_set_error(-4, msg);
    return false;
  }
  *L = chain;
  if (B.nseg != *nseg || B.csz != *csz) {
    B.release();
    const size_t bytes = sizeof(cpx) * (size_t)(*nseg) * (*csz);
    if (cudaMalloc(&B.V, bytes) != cudaSuccess || cudaMalloc(&B.W, bytes) != cudaSuccess ||
        cudaMalloc(&B.r, sizeof(double) * (*nseg)) != cudaSuccess ||
        cudaMalloc(&B.part, sizeof(double) * kDotGrid) != cudaSuccess ||
        cudaMalloc(&B.dot, sizeof(double) * 2) != cudaSuccess) {
      B.release();
      cudaGetLastError();
      engine_set_error(-1, "LSS: device allocation failed");
      return false;
    }
    B.nseg = *nseg;
    B.csz = *csz;
  }
  return true;
}

static int lss_matvec(const cpx* x, cpx* y, int inhomo, double* zeta) {
  int nseg = 0, L = 0;
  size_t m = 0;
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  if (!lss_ready("c_lss_matvec_dev", &nseg, &m, &L, &g, &st)) return engine_status();
  const size_t seg_bytes = sizeof(cpx) * m;
  const int inh[1] = {inhomo ? 1 : 0};
  int rc = 0;
  // forward sweep of every window: v' = P_L T P_0 v
  if (cudaMemcpyAsync(B.V, x, seg_bytes * nseg, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return -1;
  if ((rc = c_batch_ddt_project_dev(0, reinterpret_cast<chn_complex*>(B.V), nullptr)) != 0) return rc;
  if ((rc = c_batch_tangent_dev(0, L, reinterpret_cast<chn_complex*>(B.V), inh)) != 0) return rc;
  if ((rc = c_batch_ddt_project_dev(L, reinterpret_cast<chn_complex*>(B.V), B.r)) != 0) return rc;
  if (zeta) {
    k_negate<<<(nseg + 127) / 128, 128, 0, st>>>(nseg, B.r, zeta);
    engine_count_launches(1);
  }
  // backward sweep: w' = P_0 A P_L w, with w_{n-1} = 0
  if (nseg > 1 &&
      cudaMemcpyAsync(B.W, x + (size_t)nseg * m, seg_bytes * (nseg - 1), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return -1;
  if (cudaMemsetAsync(B.W + (size_t)(nseg - 1) * m, 0, seg_bytes, st) != cudaSuccess) return -1;
  if ((rc = c_batch_ddt_project_dev(L, reinterpret_cast<chn_complex*>(B.W), nullptr)) != 0) return rc;
  if ((rc = c_batch_adjoint_dev(L, 0, reinterpret_cast<chn_complex*>(B.W), 1.0)) != 0) return rc;
  if ((rc = c_batch_ddt_project_dev(0, reinterpret_cast<chn_complex*>(B.W), nullptr)) != 0) return rc;
  const size_t n = (size_t)(2 * nseg - 1) * m;
  k_kkt_residual<<<vec_blocks(n), 256, 0, st>>>(m, nseg, x, B.V, B.W, y);
  engine_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

static bool dot(size_t n, const double* a, const double* b, double* out, cudaStream_t st) {
  k_dot_partial<<<kDotGrid, kDotThreads, 0, st>>>(n, a, b, B.part);
  k_dot_final<<<1, kDotThreads, 0, st>>>(kDotGrid, B.part, B.dot);
  engine_count_launches(2);
  if (cudaMemcpyAsync(out, B.dot, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
  return cudaStreamSynchronize(st) == cudaSuccess;
}

}  // namespace chn

using namespace chn;

extern "C" int c_lss_matvec_dev(const chn_complex* x, chn_complex* y, int inhomo, double* zeta) {
  if (!x || !y) {
    engine_set_error(-4, "c_lss_matvec_dev: null array");
    return -4;
  }
  return lss_matvec(reinterpret_cast<const cpx*>(x), reinterpret_cast<cpx*>(y), inhomo, zeta);
}

extern "C" int c_lss_dot_dev(long long n, const double* a, const double* b, double* out) {
  int nseg = 0, L = 0;
  size_t m = 0;
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  if (!lss_ready("c_lss_dot_dev", &nseg, &m, &L, &g, &st)) return engine_status();
  if (n < 0 || !a || !b || !out) return -4;
  return dot((size_t)n, a, b, out, st) ? 0 : -1;
}

// Unpreconditioned MINRES on the KKT operator (inhomo 0), the recurrences of
// drivers/pariter.py:63-125 with the Euclidean inner product of the float
// view.  Stops when |eta| / |b - A x0| < tol or after maxiter iterations.
// Returns 0 converged, 1 not converged, < 0 error.
extern "C" int c_lss_minres_dev(const chn_complex* b, chn_complex* x, double tol, int maxiter, int* iters,
                                double* rel_residual) {
  int nseg = 0, L = 0;
  size_t m = 0;
  const Grid* g = nullptr;
  cudaStream_t st = nullptr;
  if (!lss_ready("c_lss_minres_dev", &nseg, &m, &L, &g, &st)) return engine_status();
  if (!b || !x || maxiter < 0) {
    engine_set_error(-4, "c_lss_minres_dev: null array or negative maxiter");
    return -4;
  }
  const size_t nd = (size_t)(2 * nseg - 1) * m * 2;  // doubles
  if (B.nvec != nd) {
    for (double*& p : B.vec) {
      cudaFree(p);
      p = nullptr;
    }
    for (double*& p : B.vec)
      if (cudaMalloc(&p, sizeof(double) * nd) != cudaSuccess) {
        cudaGetLastError();
        engine_set_error(-1, "c_lss_minres_dev: device allocation failed");
        B.nvec = 0;
        return -1;
      }
    B.nvec = nd;
  }
  double *vi = B.vec[0], *vim = B.vec[1], *vip = B.vec[2], *Avi = B.vec[3];
  double *wi = B.vec[4], *wim = B.vec[5], *wip = B.vec[6];
  double* X = reinterpret_cast<double*>(x);
  const unsigned nb = vec_blocks(nd);
  int rc = 0;
  // vi = b - A x
  if ((rc = lss_matvec(reinterpret_cast<const cpx*>(x), reinterpret_cast<cpx*>(Avi), 0, nullptr)) != 0) return rc;
  k_sub<<<nb, 256, 0, st>>>(nd, reinterpret_cast<const double*>(b), Avi, vi);
  cudaMemsetAsync(vim, 0, sizeof(double) * nd, st);
  cudaMemsetAsync(wi, 0, sizeof(double) * nd, st);
  cudaMemsetAsync(wim, 0, sizeof(double) * nd, st);
  engine_count_launches(1);
  double bb = 0.0;
  if (!dot(nd, vi, vi, &bb, st)) return -1;
  double betai = std::sqrt(bb);
  const double r0 = betai;
  double eta = betai;
  double gammai = 1.0, gammaim = 1.0, sigmai = 0.0, sigmaim = 0.0;
  if (iters) *iters = 0;
  if (rel_residual) *rel_residual = r0 > 0.0 ? 1.0 : 0.0;
  if (r0 == 0.0) return 0;
  for (int k = 0; k < maxiter; ++k) {
    k_div<<<nb, 256, 0, st>>>(nd, vi, betai);
    engine_count_launches(1);
    if ((rc = lss_matvec(reinterpret_cast<const cpx*>(vi), reinterpret_cast<cpx*>(Avi), 0, nullptr)) != 0)
      return rc;
    double alphai = 0.0;
    if (!dot(nd, vi, Avi, &alphai, st)) return -1;
    k_sub_scaled_pair<<<nb, 256, 0, st>>>(nd, vip, Avi, alphai, vi, betai, vim);
    engine_count_launches(1);
    double vv = 0.0;
    if (!dot(nd, vip, vip, &vv, st)) return -1;
    const double betaip = std::sqrt(vv);
    // QR factor and Givens rotation
    const double delta = gammai * alphai - gammaim * sigmai * betai;
    const double p1 = std::sqrt(delta * delta + betaip * betaip);
    const double p2 = sigmai * alphai + gammaim * gammai * betai;
    const double p3 = sigmaim * betai;
    const double gammaip = delta / p1, sigmaip = betaip / p1;
    k_direction<<<nb, 256, 0, st>>>(nd, wip, vi, p3, wim, p2, wi, p1);
    k_axpy<<<nb, 256, 0, st>>>(nd, gammaip * eta, wip, X);
    engine_count_launches(2);
    eta *= -sigmaip;
    betai = betaip;
    sigmaim = sigmai;
    sigmai = sigmaip;
    gammaim = gammai;
    gammai = gammaip;
    // roll the vectors: wim <- wi <- wip, vim <- vi <- vip
    double* t = wim;
    wim = wi;
    wi = wip;
    wip = t;
    t = vim;
    vim = vi;
    vi = vip;
    vip = t;
    if (iters) *iters = k + 1;
    if (rel_residual) *rel_residual = std::fabs(eta) / r0;
    if (std::fabs(eta) / r0 < tol) return cudaStreamSynchronize(st) == cudaSuccess ? 0 : -1;
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? 1 : -1;
}
