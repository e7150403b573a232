// spec2phys for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc at the moment they need a physical
// field: code that runs while a CUDA stream is being captured into a graph
// (allocation is not a capturable operation), real-time loops that must not
// hit the allocator, and hosts embedding this library under a fixed memory
// budget.  c_spec2phys_noalloc serves them: the caller passes device arrays
// for the input coefficients and the output flow, and the two intermediate
// arrays (velocity at the quadrature planes, physical fields on the padded
// grid) live in file-scope __device__ arrays of fixed size instead of
// library allocations.  Every GPU that loads the library holds these 16 MiB
// until the process exits.
#include <cstdio>

#include "../../include/c_channel.h"
#include "chn_common.cuh"
#include "kernels.h"

namespace chn {

bool engine_grid_stream(const Grid** g, cudaStream_t* st);
void engine_set_error(int code, const char* msg);
void engine_count_launches(int n);

// Capacities: one field's velocity U[Nz][5][qpts][Nx/2] and three physical
// fields [3][qpts][3Nz/2][3Nx/2].  32x65x32 needs 248,320 and 670,464.
static constexpr size_t kNoAllocU = (size_t)1 << 19;  // complex elements (8 MiB)
static constexpr size_t kNoAllocP = (size_t)1 << 20;  // doubles (8 MiB)

static __device__ __align__(256) cpx g_noalloc_u[kNoAllocU];
static __device__ __align__(256) double g_noalloc_p[kNoAllocP];

static constexpr int kMaxDevices = 64;
static cpx* s_u[kMaxDevices];
static double* s_p[kMaxDevices];

// Device addresses of the scratch arrays on the current device, looked up
// once per device (the host-side names are stand-ins, not device addresses).
static bool scratch_addresses(cpx** u, double** p) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    engine_set_error(-1, "c_spec2phys_noalloc: no usable current device");
    return false;
  }
  if (!s_u[dev]) {
    void* a = nullptr;
    void* b = nullptr;
    cudaError_t e1 = cudaGetSymbolAddress(&a, g_noalloc_u);
    cudaError_t e2 = cudaGetSymbolAddress(&b, g_noalloc_p);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      char msg[256];
      snprintf(msg, sizeof(msg), "c_spec2phys_noalloc: cudaGetSymbolAddress failed: %s",
               cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
      engine_set_error(-1, msg);
      return false;
    }
    s_u[dev] = static_cast<cpx*>(a);
    s_p[dev] = static_cast<double*>(b);
  }
  *u = s_u[dev];
  *p = s_p[dev];
  return true;
}

}  // namespace chn

using namespace chn;

extern "C" int c_spec2phys_noalloc(const chn_complex* C_dev, double* flow_dev) {
  const Grid* gp = nullptr;
  cudaStream_t st = nullptr;
  if (!engine_grid_stream(&gp, &st)) {
    engine_set_error(-2, "c_spec2phys_noalloc called before c_init");
    return -2;
  }
  // the one-block-per-plane transforms: they need no intermediate array.
  // The tensor-core inverse (the default) fits every grid within the
  // capacity below; the FP64 one (CHN_TRANSFORMS_FP64=1, or where the
  // tensor-core inverse did not fit at c_init) is checked against the
  // device's shared memory per block.
  Grid g = *gp;
  g.split = 0;
  if (!g.tci) {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
      engine_set_error(-1, "c_spec2phys_noalloc: no usable current device");
      return -1;
    }
    if (!fused_transforms_fit(g, optin)) {
      char msg[256];
      snprintf(msg, sizeof(msg),
               "c_spec2phys_noalloc: grid %dx%dx%d: the one-block-per-plane FP64 transforms need %zu bytes of "
               "shared memory per block, the device allows %d",
               g.Nx, g.Ny, g.Nz, phys_smem_bytes(g, true), optin);
      engine_set_error(-5, msg);
      return -5;
    }
  }
  const size_t need_u = u_size(g);
  const size_t need_p = (size_t)3 * g.Q * plane_size(g);
  if (need_u > kNoAllocU || need_p > kNoAllocP) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "c_spec2phys_noalloc: grid %dx%dx%d needs %zu velocity and %zu physical scratch elements; "
             "the fixed capacity is %zu and %zu",
             g.Nx, g.Ny, g.Nz, need_u, need_p, kNoAllocU, kNoAllocP);
    engine_set_error(-5, msg);
    return -5;
  }
  if (!C_dev || !flow_dev) {
    engine_set_error(-4, "c_spec2phys_noalloc: null array");
    return -4;
  }
  cpx* U = nullptr;
  double* P = nullptr;
  if (!scratch_addresses(&U, &P)) return -1;
  // No scratch needs clearing: the reconstruction writes every plane of every
  // line the transforms read (the kz = Nz/2 line is read by neither), and the
  // transforms and the layout pass overwrite P and flow entirely.
  ReconArgs ra{};
  ra.C = Batch<const cpx>{reinterpret_cast<const cpx*>(C_dev), 0};
  ra.slot = SlotRef{nullptr, 0, 0, 0};
  ra.U = Batch<cpx>{U, 0};
  ra.ninst = 1;
  ra.status = nullptr;
  ra.sdiv = 1;
  PhysArgs pa{};
  pa.U = Batch<const cpx>{U, 0};
  pa.P = Batch<double>{P, 0};
  pa.nfields = 3;
  pa.ninst = 1;
  pa.status = nullptr;
  pa.sdiv = 1;
  cudaError_t e = launch_recon(g, ra, st);
  if (e == cudaSuccess) e = launch_phys_inverse(g, pa, st);
  if (e == cudaSuccess) e = launch_flow_out(g, P, flow_dev, st);
  engine_count_launches(3);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "c_spec2phys_noalloc: launch failed: %s", cudaGetErrorString(e));
    engine_set_error(-1, msg);
    return -1;
  }
  return 0;
}
