// Host orchestration and the C ABI (include/c_channel.h).
//
// One substage of every solver is a short fixed pipeline of batched kernels
// (reconstruct -> physical transforms -> products -> implicit solve); one
// time step is three substages.  The trajectory slot each kernel touches is
// derived on the device from a step counter that the last kernel of the step
// advances, so a step is captured once into a CUDA graph and replayed for
// every time step of a call.
//
// The reference keeps one solver per process in globals (channel/main.h:81-201)
// and the Python layer enforces a single init (channel/__init__.py:80-82);
// this library keeps one Engine per process likewise.
#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c_channel.h"
#include "chn_common.cuh"
#include "fft.cuh"
#include "kernels.h"
#include "sizes.cuh"
#include "setup.h"

namespace chn {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static int g_status = 0;
static std::string g_msg;
static double g_cfl = 0.0;
static long long g_launches = 0;

static void set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_status = code;
  g_msg = buf;
}

#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      set_error(-1, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return false;                                                                \
    }                                                                              \
  } while (0)

// an NVTX range around each kernel launch (named by the launch call) and
// each entry-point operation: profilers that attach an NVTX tool see which
// sweep and substage a kernel was enqueued from; without a tool the calls
// return at once
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

#define LK(call)                    \
  do {                              \
    ++g_launches;                   \
    NvtxRange nvtx_launch_(#call);  \
    CK(call);                       \
  } while (0)

// the reference asserts shapes and aborts (channel/channel.i:45-48)
static void shape_assert(bool ok, const char* what) {
  if (!ok) {
    fprintf(stderr, "c_channel: assertion failed: %s\n", what);
    fflush(stderr);
    abort();
  }
}

// ---------------------------------------------------------------------------
// device tables
// ---------------------------------------------------------------------------

struct DevTables {
  HostTables ht;
  Grid g{};
  std::vector<void*> ptrs;
  double* luQs = nullptr;
  double* luRs = nullptr;

  template <typename T>
  bool up(const std::vector<T>& v, const T** out) {
    void* p = nullptr;
    size_t n = v.size() * sizeof(T);
    if (n == 0) n = sizeof(T);
    CK(cudaMalloc(&p, n));
    ptrs.push_back(p);
    if (!v.empty()) CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    *out = reinterpret_cast<const T*>(p);
    return true;
  }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

static bool fft_length_ok(int n) {
  if (n % 3) return false;
  int m = n / 3;
  for (int f : {4, 2, 3, 5, 7})
    while (m % f == 0) m /= f;
  return m == 1;
}

static bool build_device_tables(DevTables& T, int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
                                double flux, double dt) {
  const char* err = nullptr;
  if (!build_tables(Nx, Ny, Nz, Lx, Lz, Re, flux, dt, T.ht, &err)) {
    set_error(1, "%s", err);
    return false;
  }
  HostTables& h = T.ht;
  if (!fft_length_ok(h.pz) || !fft_length_ok(h.px)) {
    set_error(1, "unsupported transform length (3Nx/2 = %d, 3Nz/2 = %d): Nx/2 and Nz/2 must factor into 2, 3, 5, 7",
              h.px, h.pz);
    return false;
  }
  Grid& g = T.g;
  g.Nx = h.Nx; g.Ny = h.Ny; g.Nz = h.Nz; g.X = h.X; g.Q = h.Q; g.R = h.R; g.D = h.D;
  g.pz = h.pz; g.px = h.px; g.Qh = (h.Q + 1) / 2;
  g.dt = dt; g.re = h.re; g.flux = flux;
  g.norm = 1.0 / ((3. * Nx / 2.) * (3. * Nz / 2.));
  g.cfl1 = h.cfl1; g.cfl3 = h.cfl3;
  bool ok = T.up(h.Kx, &g.Kx) && T.up(h.Kz, &g.Kz) && T.up(h.K2, &g.K2) && T.up(h.kxK2, &g.kxK2) &&
            T.up(h.kzK2, &g.kzK2) && T.up(h.cfl2, &g.cfl2) && T.up(h.w, &g.W) && T.up(h.Bq, &g.Bq) &&
            T.up(h.Bqp, &g.Bqp) && T.up(h.Bqpp, &g.Bqpp) && T.up(h.Br, &g.Br) && T.up(h.Brp, &g.Brp) &&
            T.up(h.Wq, &g.Wq) && T.up(h.Wqp, &g.Wqp) && T.up(h.Wqpp, &g.Wqpp) && T.up(h.Wr, &g.Wr) &&
            T.up(h.Wrp, &g.Wrp) && T.up(h.luA, &g.luA) && T.up(h.luB, &g.luB) && T.up(h.exA, &g.exA) &&
            T.up(h.exB, &g.exB) && T.up(h.lu0, &g.lu0) && T.up(h.ex0, &g.ex0) && T.up(h.add0, &g.add0) &&
            T.up(h.rwsum, &g.rwsum) && T.up(h.Qs, &g.Qs) && T.up(h.Qps, &g.Qps) && T.up(h.Qpps, &g.Qpps) &&
            T.up(h.Rs, &g.Rs) && T.up(h.Rps, &g.Rps) && T.up(h.rdA, &g.rdA) && T.up(h.rdB, &g.rdB) &&
            T.up(h.rd0, &g.rd0);
  if (!ok) return false;
  const double* tz;
  const double* tx;
  if (!T.up(h.twz, &tz) || !T.up(h.twx, &tx)) return false;
  g.twz = reinterpret_cast<const cpx*>(tz);
  g.twx = reinterpret_cast<const cpx*>(tx);
  std::vector<double> qs(h.Qs), rs(h.Rs);
  band_lu(qs.data(), 9, 4, 4, h.D);
  band_lu(rs.data(), 5, 2, 2, h.R);
  const double *a, *b;
  if (!T.up(qs, &a) || !T.up(rs, &b)) return false;
  T.luQs = const_cast<double*>(a);
  T.luRs = const_cast<double*>(b);
  {
    std::vector<uint32_t> frag, wfrag;
    std::vector<int> ex, wex;
    std::vector<uint32_t> btf, wtf;
    std::vector<int> bte, wte;
    if (!build_adj_tc_tables(h, btf, bte, wtf, wte) || !T.up(btf, &g.tcBT) || !T.up(bte, &g.tcBTE) ||
        !T.up(wtf, &g.tcWT) || !T.up(wte, &g.tcWTE))
      return false;
    if (!build_recon_tc_tables(h, frag, ex, wfrag, wex) || !T.up(frag, &g.tcA) || !T.up(ex, &g.tcE) ||
        !T.up(wfrag, &g.tcW) || !T.up(wex, &g.tcWE))
      return false;
    std::vector<uint32_t> zf, xf;
    std::vector<int> ze, xe, zm;
    if (!build_phys_tc_tables(h, zf, ze, xf, xe, zm) || !T.up(zf, &g.tcZ) || !T.up(ze, &g.tcZE) ||
        !T.up(xf, &g.tcX) || !T.up(xe, &g.tcXE) || !T.up(zm, &g.tcZM))
      return false;
    std::vector<uint32_t> fxf, fzf, fuf;
    std::vector<int> fxe, fze, fue;
    if (!build_fwd_tc_tables(h, fxf, fxe, fzf, fze, fuf, fue) || !T.up(fxf, &g.tcFX) || !T.up(fxe, &g.tcFXE) ||
        !T.up(fzf, &g.tcFZ) || !T.up(fze, &g.tcFZE) || !T.up(fuf, &g.tcFXU) || !T.up(fue, &g.tcFXUE))
      return false;
  }
  // transforms: one block per plane where the plane fits the shared memory,
  // else separate z / x passes (CHN_SPLIT_TRANSFORMS=1 forces them)
  int dev = 0, optin = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const char* force = getenv("CHN_SPLIT_TRANSFORMS");
  g.general = (radix234_only(g.pz) && radix234_only(g.px)) ? 0 : 1;
  g.split = (!fused_transforms_fit(g, optin) || (force && force[0] == '1')) ? 1 : 0;
  g.tvar = 0;
  const char* var = getenv("CHN_SPLIT_VARIANT");  // with CHN_SPLIT_TRANSFORMS=1: this variant
  if (force && force[0] == '1' && var) g.tvar = atoi(var);
  if (g.split && !split_variant_fits(g.tvar, g, optin)) {
    set_error(1, "grid %dx%dx%d: the split transforms need more shared memory than the device has", Nx, Ny, Nz);
    return false;
  }
  // reconstruction and quadratures on the tensor cores unless CHN_RECON_FP64=1 (or it does not fit)
  const char* fp64 = getenv("CHN_RECON_FP64");
  g.tc = (!(fp64 && fp64[0] == '1') && recon_tc_smem_bytes(g) + 4096 <= (size_t)optin) ? 1 : 0;
  // inverse transforms on the tensor cores unless CHN_TRANSFORMS_FP64=1 (or they do not fit)
  const char* tfp64 = getenv("CHN_TRANSFORMS_FP64");
  g.tci = (!(tfp64 && tfp64[0] == '1') && phys_tc_fits(g, optin)) ? 1 : 0;
  g.fwdpb = 3;
  g.fxch = 8;
  g.tcf = (!(tfp64 && tfp64[0] == '1') && fwd_tc_plan(g, optin, g.fwdpb, g.fxch)) ? 1 : 0;
  // the kernels' builds compiled for the grid's sizes where it has them
  // (a batch's autotuner then times both); CHN_FIXED_SIZES=0 / 1 fixes it
  const bool spec = phys_tc_specialised(g);
  const char* fx = getenv("CHN_FIXED_SIZES");
  const bool fixed_on = (fx && fx[0]) ? fx[0] == '1' : spec;
  g.fixed = fixed_on ? (FIXED_PRODUCTS | FIXED_RECON | FIXED_SOLVE) : 0;
  // the inverse's build (phys_tc.cu) until a batch's autotuner has timed
  // them: two fields per pass (the single trajectory's plane count gives a
  // block per plane), compiled for the grid's sizes where it has them;
  // CHN_INVERSE_BUILD=2..7 fixes it (and skips that timing)
  const char* ib = getenv("CHN_INVERSE_BUILD");
  const int ibv = ib ? atoi(ib) : 0;
  g.tcminb = (ibv >= 2 && ibv <= 12) ? ibv : (spec ? 7 : 2);
  // the adjoint products' planes per pass: 1 until the autotuner has timed
  // 1 and 3; CHN_ADJ_PRODUCTS_PER_PASS=1 or 3 fixes it
  const char* apb = getenv("CHN_ADJ_PRODUCTS_PER_PASS");
  g.adjpb = (apb && apb[0] == '3') ? 3 : 1;
  // the products' build (phys_tc.cu): 0 until the autotuner has timed 0 and
  // 1 (two planes per pass at 3 blocks per SM); CHN_PRODUCTS_BUILD fixes it
  const char* pbe = getenv("CHN_PRODUCTS_BUILD");
  g.prodb = (pbe && pbe[0] == '1' && pbe[1] == 0) ? 1 : 0;
  // the solve's block tile: 16 until the autotuner has timed both;
  // CHN_SOLVE_TILE=8 or 16 fixes it (and skips that timing)
  const char* stl = getenv("CHN_SOLVE_TILE");  // 16, 8 or 8/128 (8 columns, 128 threads)
  g.stile = (stl && atoi(stl) == 8) ? 8 : 16;
  g.sthr = (g.stile == 8 && stl && strstr(stl, "/128")) ? 128 : 256;
  // the tensor-core reconstruction's build (recon_tc.cu): 0 until the
  // autotuner has timed 0, 1, 2; CHN_RECON_BUILD fixes it
  const char* rbe = getenv("CHN_RECON_BUILD");
  g.rbuild = (rbe && rbe[0] >= '0' && rbe[0] <= '2' && rbe[1] == 0) ? rbe[0] - '0' : 0;
  // the inverse on tcgen05 where it fits: a candidate of the autotuner
  // (bit-identical results); CHN_INVERSE_TC5=1 forces it, =0 leaves it out
  const char* t5 = getenv("CHN_INVERSE_TC5");
  g.tc5 = 0;
  g.t5Z = g.t5X = nullptr;
  if (g.tci && !(t5 && t5[0] == '0') && phys_tc5_fits(g, 6, optin)) {
    std::vector<uint8_t> zt, xt;
    if (!build_phys_tc5_tables(h, zt, xt) || !T.up(zt, &g.t5Z) || !T.up(xt, &g.t5X)) return false;
    g.tc5 = (t5 && t5[0] == '1') ? 1 : 0;
  }
  if (solve_smem_bytes(g) > (size_t)optin || recon_smem_bytes(g) > (size_t)optin) {
    set_error(1, "grid %dx%dx%d: the implicit solve needs %zu bytes of shared memory per block, the device has %d",
              Nx, Ny, Nz, solve_smem_bytes(g), optin);
    return false;
  }
  prepare_kernels(g);
  CK(cudaGetLastError());
  return true;
}

// ---------------------------------------------------------------------------
// per-run working set: nseg segments, ntan tangents each
// ---------------------------------------------------------------------------

struct Work {
  int nseg = 0, ntan = 0, nsteps = 0, couple = 0;
  size_t csz = 0, usz = 0, psz = 0;   // coefficient, velocity, physical (6 fields) sizes
  long long traj = 0;                 // elements per stored trajectory
  cpx *MC = nullptr, *MIC = nullptr;
  cpx *Cp = nullptr, *Sp = nullptr, *Ct = nullptr, *St = nullptr, *Ca = nullptr, *Sa = nullptr;
  cpx *Up = nullptr, *Ut = nullptr, *Uprev = nullptr, *Ul = nullptr, *dC = nullptr, *io = nullptr;
  double *Pp = nullptr, *Pt = nullptr, *Pprev = nullptr, *Pl = nullptr, *flow = nullptr;
  double *part = nullptr, *r = nullptr, *cflmax = nullptr;
  double* Ft = nullptr;   // primal flux correction of each stored substage, [seg][3 nsteps + 1]
  uint32_t* status = nullptr;
  int* step = nullptr;
  int* loopctr = nullptr;      // steps left in the device-side loop of a sweep graph
  // Primal physical-field cache: the six physical fields of the primal state
  // before every substage of the stored trajectory, [seg][3 nsteps][6][Q][pz][px].
  // Tangent and adjoint sweeps read them instead of rebuilding them from MC.
  // Allocated only when it fits in half of the free device memory.
  double* Pc = nullptr;
  long long cstride = 0;       // elements per segment in Pc
  std::vector<char> slot_ok;   // slot c of Pc holds the fields of MC[c]
  // Velocity cache of the coupled tangent: u, v, w of MIC[3i] for every step
  // i, [seg][nsteps][3][Q][pz][px], written by the forward sweep at substage
  // 0; the adjoint coupling (ddt_project) reads it with the primal cache.
  double* Pv = nullptr;
  long long vslot = 0, vstride = 0;
  std::vector<char> vel_ok;    // slot i of Pv holds the fields of MIC[3i]
  cpx* icp = nullptr;          // projected IC' of the last coupling, per segment
  cpx* src = nullptr;          // per-step source of the exact adjoint (host-array entry point), per segment
  // parameter gradients of the exact adjoint, per segment: [0] dJ/dmeanU,
  // [1 + block] the solve blocks' parts of dJ/dRe (summed on the host)
  double* gacc = nullptr;
  int gstride = 0;
  std::vector<double> grad;    // [nseg][2] after the last gradient sweep: dJ/dmeanU, dJ/dRe
  const Grid* gdev = nullptr;  // uneven batch: grid of each segment (device array); null: one grid
  cpx* Zt = nullptr;           // split transforms: spectral-column intermediate for zt_inst instances
  int zt_inst = 0;
  bool raw_start = false;      // MC came from a laminar start without run-up
  int chain = 0;               // > 0: segments are consecutive windows of one trajectory (DdtArgs::chain)
  std::vector<void*> ptrs;
  void mark(int c0, int c1, bool ok) {
    for (int c = c0; c < c1 && c < (int)slot_ok.size(); ++c)
      if (c >= 0) slot_ok[c] = ok;
  }
  bool cached(int c0, int c1) const {
    if (!Pc || c0 < 0 || c1 > (int)slot_ok.size()) return false;
    for (int c = c0; c < c1; ++c)
      if (!slot_ok[c]) return false;
    return true;
  }
  // the coupling at step i can take its fields from the caches
  bool coupling_cached(int i) const {
    if (!Pv || i < 0 || i >= (int)vel_ok.size() || !vel_ok[i]) return false;
    const int ip = i == 0 ? 3 : 3 * i, im = i == 0 ? 0 : 3 * (i - 1);
    if (i == 0 && chain > 0 && !cached(3 * (chain - 1), 3 * (chain - 1) + 1)) return false;
    return cached(ip, ip + 1) && cached(im, im + 1);
  }
  void mark_vel(int i0, int i1, bool ok) {
    for (int i = i0; i < i1 && i < (int)vel_ok.size(); ++i)
      if (i >= 0) vel_ok[i] = ok;
  }
  static constexpr int kDotBlocks = 64;

  template <typename T>
  bool alloc(T** p, size_t n) {
    void* q = nullptr;
    CK(cudaMalloc(&q, n * sizeof(T) + 16));
    CK(cudaMemset(q, 0, n * sizeof(T) + 16));
    ptrs.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return true;
  }
  // Instantiated one-step graphs, kept across calls: the key holds every
  // value the captured launches read (sweep kind, options, the arrays they
  // address, the grid's kernel variants), so a matching entry replays the
  // same launches.  At most kMaxGraphs, the oldest dropped first.
  struct StepGraph {
    std::string key;
    cudaGraphExec_t exec;
    long long per_step;
  };
  std::vector<StepGraph> graphs;
  static constexpr size_t kMaxGraphs = 32;
  void release() {
    for (StepGraph& sg : graphs) cudaGraphExecDestroy(sg.exec);
    graphs.clear();
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
    *this = Work();
  }
  bool create(const Grid& g, int nseg_, int ntan_, int nsteps_, int couple_) {
    nseg = nseg_; ntan = ntan_; nsteps = nsteps_; couple = couple_;
    csz = coef_size(g);
    usz = u_size(g);
    psz = (size_t)6 * g.Q * plane_size(g);
    traj = (long long)(3 * (long long)nsteps + 1) * (long long)csz;
    const size_t nt = (size_t)nseg * (ntan > 0 ? ntan : 1);
    return alloc(&MC, (size_t)nseg * traj) && alloc(&MIC, (size_t)nseg * traj) && alloc(&Cp, nseg * csz) &&
           alloc(&Sp, nseg * csz) && alloc(&Ct, nt * csz) && alloc(&St, nt * csz) && alloc(&Ca, nseg * csz) &&
           alloc(&Sa, nseg * csz) && alloc(&Up, nseg * usz) && alloc(&Ut, nt * usz) &&
           alloc(&Uprev, nseg * usz) && alloc(&Ul, nseg * usz) && alloc(&dC, nseg * csz) &&
           alloc(&io, nt * csz) && alloc(&Pp, nseg * psz) && alloc(&Pt, nt * psz) &&
           alloc(&Pprev, nseg * psz) && alloc(&Pl, nseg * psz) && alloc(&flow, (size_t)3 * g.Q * plane_size(g)) &&
           alloc(&part, (size_t)nseg * kDotBlocks * 2) && alloc(&r, nseg) && alloc(&cflmax, nseg) &&
           alloc(&status, nseg) && alloc(&step, 4) && alloc(&loopctr, 1) && alloc(&icp, nseg * csz) &&
           alloc(&src, nseg * csz) &&
           alloc(&Ft, (size_t)nseg * (3 * (size_t)nsteps + 1)) && alloc_split(g, nt) && alloc_cache(g) &&
           alloc_grad(g);
  }
  bool alloc_grad(const Grid& g) {
    gstride = 1 + g.Nz * ((g.X + 15) / 16);  // the solve's blocks: kz lines x 16-column tiles
    return alloc(&gacc, (size_t)nseg * gstride);
  }
  // split transforms (required where a plane exceeds a block's shared
  // memory, else an autotuner candidate): room for up to 2 GiB of
  // intermediate, at least one instance
  bool alloc_split(const Grid& g, size_t nt) {
    const size_t per = split_tmp_elems(g);
    size_t n = ((size_t)2 << 30) / (per * sizeof(cpx));
    if (n < 1) n = 1;
    if (n > nt) n = nt;
    zt_inst = (int)n;
    return alloc(&Zt, n * per);
  }
  bool alloc_cache(const Grid& g) {
    Pc = nullptr;
    Pv = nullptr;
    slot_ok.assign(3 * (size_t)(nsteps > 0 ? nsteps : 0), 0);
    vel_ok.assign((size_t)(nsteps > 0 ? nsteps : 0), 0);
    const char* off = getenv("CHN_NO_FIELD_CACHE");
    if ((off && off[0] == '1') || nsteps <= 0) return true;
    cstride = (long long)3 * nsteps * (long long)psz;
    vslot = (long long)3 * g.Q * (long long)plane_size(g);
    vstride = (ntan > 0) ? (long long)nsteps * vslot : 0;
    const size_t need_c = (size_t)nseg * (size_t)cstride * sizeof(double);
    const size_t need_v = (size_t)nseg * (size_t)vstride * sizeof(double);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || need_c + need_v > free_b / 2) return true;
    void* q = nullptr;
    if (cudaMalloc(&q, need_c) != cudaSuccess) {
      cudaGetLastError();
      return true;
    }
    ptrs.push_back(q);
    Pc = reinterpret_cast<double*>(q);
    if (need_v) {
      q = nullptr;
      if (cudaMalloc(&q, need_v) != cudaSuccess) {
        cudaGetLastError();
        return true;
      }
      ptrs.push_back(q);
      Pv = reinterpret_cast<double*>(q);
    }
    return true;
  }
};

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------

struct Engine {
  DevTables T;
  Work single;     // the reference API: one segment, one tangent
  Work batch;      // c_batch_*
  bool have_batch = false;
  cudaStream_t st = nullptr;
  // a second stream and the events that fork and join the concurrent
  // branches of a substage (chains_concurrent)
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool conc = true;  // CHN_CONCURRENT_CHAINS at creation
  int nsteps = 0;
  std::vector<double> qy, qw;
  cpx* host_mc = nullptr;   // pinned mirrors for c_getsoln / c_getincresoln
  cpx* host_mic = nullptr;
  std::vector<cpx> last_ic;  // the reference's global IC after the last tangent call
};

static Engine* E = nullptr;

static bool engine_streams_create(Engine& e) {
  const char* v = getenv("CHN_CONCURRENT_CHAINS");
  e.conc = !(v && v[0] == '0');
  if (cudaStreamCreateWithFlags(&e.st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e.st2, cudaStreamNonBlocking) != cudaSuccess)
    return false;
  for (cudaEvent_t& v : e.ev)
    if (cudaEventCreateWithFlags(&v, cudaEventDisableTiming) != cudaSuccess) return false;
  return true;
}

static void engine_streams_destroy(Engine& e) {
  for (cudaEvent_t& v : e.ev)
    if (v) cudaEventDestroy(v);
  for (cudaEvent_t& v : e.ev) v = nullptr;
  if (e.st2) cudaStreamDestroy(e.st2);
  if (e.st) cudaStreamDestroy(e.st);
  e.st2 = e.st = nullptr;
}

// Independent chains of a substage (the primal's and the tangents' kernels
// of a forward substage, the reference adjoint's two product passes) run as
// concurrent branches: on st and st2 outside a graph, as parallel branches
// of the captured step inside one, joined by events where one reads what
// the other writes and at the end of the substage, so each fills the other's
// last waves.  Only where the kernels share no scratch (the one-block-per-
// plane tensor-core transforms; the split and FFT passes share Work::Zt).
// The arithmetic is the same either way.  CHN_CONCURRENT_CHAINS=0 (read at
// c_init / c_multi_init) keeps one stream.
static bool chains_concurrent(const Engine& e) {
  const Grid& g = e.T.g;
  return e.conc && e.st2 && g.tci && g.tcf && !g.split && !g.tc5;
}

// both streams drained: before the engine's arrays are released (a failed
// enqueue can leave a branch on st2 that never joined st)
static void engine_sync(Engine& e) {
  if (e.st) cudaStreamSynchronize(e.st);
  if (e.st2) cudaStreamSynchronize(e.st2);
}

// st2 waits for what st has enqueued so far (fork), or the reverse (join)
static bool fork_to(Engine& e, cudaStream_t from, cudaStream_t to, int ev) {
  CK(cudaEventRecord(e.ev[ev], from));
  CK(cudaStreamWaitEvent(to, e.ev[ev], 0));
  return true;
}

// sizes and shorthands
static inline Batch<const cpx> cb(const cpx* p, long long s) { return Batch<const cpx>{p, s}; }
static inline Batch<cpx> mb(cpx* p, long long s) { return Batch<cpx>{p, s}; }
static inline Batch<const double> cbd(const double* p, long long s) { return Batch<const double>{p, s}; }
static inline Batch<double> mbd(double* p, long long s) { return Batch<double>{p, s}; }
static inline SlotRef noslot() { return SlotRef{nullptr, 0, 0, 0}; }

// ---------------------------------------------------------------------------
// stage pipelines
// ---------------------------------------------------------------------------

struct FwdOpts {
  bool adv_primal;      // advance the primal (and store MC) or read it from MC
  bool tangents;        // advance the tangents (store MIC of tangent `couple`)
  int ru;               // run-up steps of the primal (MC slot offset)
  uint32_t forced_mask; // tangents with the mean-flux forcing
  bool raw_u_first;     // the primal velocity of substage 0 is already in Up
  bool cache;           // adv_primal: write the primal fields to the cache;
                        // otherwise: read them from the (valid) cache
  bool store = true;    // adv_primal: store the primal states in MC
  uint32_t re2_mask = 0, re3_mask = 0;  // tangents with Re forcing (reference / exact)
};

static bool enqueue_forward_step(Engine& e, Work& w, const FwdOpts& o) {
  const Grid& g = e.T.g;
  cudaStream_t st = e.st;
  const int nt = w.nseg * w.ntan;
  const bool use_cache = o.cache && w.Pc != nullptr;
  // the tangents' chain on its own branch where the primal advances beside it
  const bool conc = o.tangents && o.adv_primal && chains_concurrent(e);
  cudaStream_t stt = conc ? e.st2 : st;
  for (int k = 0; k < 3; ++k) {
    if (conc && !fork_to(e, st, stt, 0)) return false;
    // where this substage's primal physical fields live
    Batch<const double> Pprim = cbd(w.Pp, w.psz);
    SlotRef pslot = noslot();
    if (use_cache) {
      Pprim = cbd(w.Pc, w.cstride);
      // state before substage k: 3(n - ru) + k when advancing, 3n + k otherwise
      pslot = SlotRef{w.step, 3, k - (o.adv_primal ? 3 * o.ru : 0), (long long)w.psz};
    }
    const bool need_primal_fields = o.adv_primal || !use_cache;
    if (need_primal_fields) {
      ReconArgs rp{};
      rp.grids = w.gdev;
      rp.ninst = w.nseg;
      rp.U = mb(w.Up, w.usz);
      rp.status = w.status;
      rp.sdiv = 1;
      if (o.adv_primal) {
        rp.C = cb(w.Sp, w.csz);
        rp.slot = noslot();
      } else {
        rp.C = cb(w.MC, w.traj);
        rp.slot = SlotRef{w.step, 3, k, (long long)w.csz};  // state before substage k: MC[3n + k]
      }
      if (!(o.raw_u_first && k == 0)) LK(launch_recon(g, rp, st));
    }
    if (o.tangents) {
      ReconArgs rt{};
      rt.grids = w.gdev;
      rt.ninst = nt;
      rt.C = cb(w.St, w.csz);
      rt.slot = noslot();
      rt.U = mb(w.Ut, w.usz);
      rt.status = w.status;
      rt.sdiv = w.ntan;
      LK(launch_recon(g, rt, stt));
    }
    if (need_primal_fields) {
      PhysArgs pp{};
      pp.grids = w.gdev;
      pp.tmp = w.Zt;
      pp.tmp_inst = w.zt_inst;
      pp.U = cb(w.Up, w.usz);
      pp.P = Batch<double>{const_cast<double*>(Pprim.base), Pprim.stride};
      pp.pslot = pslot;
      pp.nfields = 6;
      pp.ninst = w.nseg;
      pp.status = w.status;
      pp.sdiv = 1;
      pp.cflmax = w.cflmax;
      pp.cfl_check = k == 0;  // channel/pass1.c:117
      pp.skip_blocked = 1;
      LK(launch_phys_inverse(g, pp, st));
      if (conc) CK(cudaEventRecord(e.ev[1], st));  // the tangents' products read these fields
    }
    if (o.tangents) {
      PhysArgs pt{};
      pt.grids = w.gdev;
      pt.tmp = w.Zt;
      pt.tmp_inst = w.zt_inst;
      pt.U = cb(w.Ut, w.usz);
      pt.P = mbd(w.Pt, w.psz);
      pt.pslot = noslot();
      pt.nfields = 6;
      pt.ninst = nt;
      pt.status = w.status;
      pt.sdiv = w.ntan;
      pt.skip_blocked = 1;
      LK(launch_phys_inverse(g, pt, stt));
      if (k == 0 && w.Pv)
        LK(launch_cache_velocity(g, w.Pt, w.psz, w.ntan, w.couple, w.Pv, w.vstride, w.vslot, w.step, 0, w.status,
                                 w.nseg, stt));
      ProdArgs ap{};
      ap.grids = w.gdev;
      ap.tmp = w.Zt;
      ap.tmp_inst = w.zt_inst;
      ap.Pp = Pprim;
      ap.pdiv = w.ntan;
      ap.pslot = pslot;
      ap.Pt = cbd(w.Pt, w.psz);
      ap.H = mb(w.Ut, w.usz);
      ap.ninst = nt;
      ap.status = w.status;
      ap.sdiv = w.ntan;
      if (conc) CK(cudaStreamWaitEvent(stt, e.ev[1], 0));
      LK(launch_products_fwd(g, ap, stt));
    }
    if (o.adv_primal) {
      ProdArgs ap{};
      ap.grids = w.gdev;
      ap.tmp = w.Zt;
      ap.tmp_inst = w.zt_inst;
      ap.Pp = Pprim;
      ap.pdiv = 1;
      ap.pslot = pslot;
      ap.Pt = cbd(nullptr, 0);
      ap.H = mb(w.Up, w.usz);
      ap.ninst = w.nseg;
      ap.status = w.status;
      ap.sdiv = 1;
      LK(launch_products_fwd(g, ap, st));
    }
    // the primal solve first: tangent Re forcing reads the state it stores
    if (o.adv_primal) {
      SolveArgs sa{};
      sa.grids = w.gdev;
      sa.H = cb(w.Up, w.usz);
      sa.Hprev = cb(nullptr, 0);
      sa.Cc = mb(w.Cp, w.csz);
      sa.Sout = mb(w.Sp, w.csz);
      sa.T = o.store ? mb(w.MC, w.traj) : mb(nullptr, 0);
      sa.tdiv = 1;
      sa.tsel = 0;
      sa.slot = SlotRef{w.step, 3, k + 1 - 3 * o.ru, (long long)w.csz};  // MC[3(n - ru) + k + 1]
      sa.k = k;
      sa.adjoint = 0;
      sa.mean_mode = MEAN_PRIMAL;
      sa.forced_mask = 0;
      sa.mdiv = 1;
      sa.ninst = w.nseg;
      sa.status = w.status;
      sa.sdiv = 1;
      sa.Fts = w.Ft;
      sa.fts_stride = 3 * (long long)w.nsteps + 1;
      LK(launch_solve(g, sa, st));
      // a tangent Re forcing reads the primal states and fluxes this solve stores
      if (conc && (o.re2_mask | o.re3_mask) && !fork_to(e, st, stt, 2)) return false;
    }
    if (o.tangents) {
      SolveArgs sa{};
      sa.grids = w.gdev;
      sa.H = cb(w.Ut, w.usz);
      sa.Hprev = cb(nullptr, 0);
      sa.Cc = mb(w.Ct, w.csz);
      sa.Sout = mb(w.St, w.csz);
      sa.T = mb(w.MIC, w.traj);
      sa.tdiv = w.ntan;
      sa.tsel = w.couple;
      sa.slot = SlotRef{w.step, 3, k + 1, (long long)w.csz};  // MIC[3n + k + 1]
      sa.k = k;
      sa.adjoint = 0;
      sa.mean_mode = MEAN_TAN_HOMOG;
      sa.forced_mask = o.forced_mask;
      sa.mdiv = w.ntan;
      sa.ninst = nt;
      sa.status = w.status;
      sa.sdiv = w.ntan;
      sa.re2_mask = o.re2_mask;
      sa.re3_mask = o.re3_mask;
      if (o.re2_mask | o.re3_mask) {
        // primal states MC[3n + k], MC[3n + k + 1] (stored before this solve) and their flux corrections
        sa.Xf = cb(w.MC, w.traj);
        sa.xslot = SlotRef{w.step, 3, k - (o.adv_primal ? 3 * o.ru : 0), (long long)w.csz};
        sa.xdiv = w.ntan;
        sa.Ftr = w.Ft;
        sa.ftr_stride = 3 * (long long)w.nsteps + 1;
      }
      LK(launch_solve(g, sa, stt));
    }
    if (conc && !fork_to(e, stt, st, 3)) return false;  // join
  }
  LK(launch_step_advance(w.step, +1, st));
  return true;
}

// spec2phys of nseg coefficient arrays (optionally at a trajectory slot) into P (3 fields)
static bool enqueue_spec2phys(Engine& e, Work& w, Batch<const cpx> C, SlotRef slot, cpx* U, double* P, int nseg) {
  const Grid& g = e.T.g;
  ReconArgs ra{};
  ra.grids = w.gdev;
  ra.C = C;
  ra.slot = slot;
  ra.U = mb(U, w.usz);
  ra.ninst = nseg;
  ra.status = nullptr;
  ra.sdiv = 1;
  LK(launch_recon(g, ra, e.st));
  PhysArgs pa{};
  pa.grids = w.gdev;
  pa.tmp = w.Zt;
  pa.tmp_inst = w.zt_inst;
  pa.U = cb(U, w.usz);
  pa.P = mbd(P, w.psz);
  pa.nfields = 3;
  pa.ninst = nseg;
  pa.status = nullptr;
  pa.sdiv = 1;
  LK(launch_phys_inverse(g, pa, e.st));
  return true;
}

// Adjoint coupling to the stored tangent at i_step = *step + add
// (channel/channel.c:624-631 and 682-689 with ddt_project, channel.c:704-780):
// IC' = ddt_project(i_step, MIC[3 i_step]) into w.icp, then AC -= coef * IC'
// (coef == 0: projection only).  With `cached` the inner products read the
// primal and velocity caches instead of transforming dCdt and MIC[3 i_step].
static bool enqueue_coupling(Engine& e, Work& w, int add, double coef, bool cached) {
  const Grid& g = e.T.g;
  DdtArgs d{w.MC, w.traj, w.step, add, w.nseg, w.chain, w.gdev};
  LK(launch_ddt_diff(g, d, w.dC, e.st));
  const SlotRef icslot{w.step, 3, 3 * add, (long long)w.csz};
  if (cached) {
    LK(launch_ddt_dots_cached(g, d, w.Pc, w.cstride, w.psz, w.Pv, w.vstride, w.vslot, w.part, Work::kDotBlocks,
                              e.st));
  } else {
    if (!enqueue_spec2phys(e, w, cb(w.dC, w.csz), noslot(), w.Uprev, w.Pprev, w.nseg)) return false;
    if (!enqueue_spec2phys(e, w, cb(w.MIC, w.traj), icslot, w.Ul, w.Pl, w.nseg)) return false;
    LK(launch_ddt_dots(g, cbd(w.Pprev, w.psz), cbd(w.Pl, w.psz), w.part, Work::kDotBlocks, w.nseg, e.st, w.gdev));
  }
  LK(launch_ddt_apply(g, w.part, Work::kDotBlocks, w.nseg, cb(w.MIC, w.traj), icslot, mb(w.icp, w.csz),
                      cb(w.dC, w.csz), w.r, coef != 0.0 ? mb(w.Ca, w.csz) : mb(nullptr, 0), coef, e.st, w.gdev));
  return true;
}

// One adjoint step n = *step.  The reference couples to step n at the start
// and to step n - 1 at the end of every step, so each interior projection is
// applied twice with nothing in between; it is computed once, at the end of
// step n + 1 (or before the first step), and carried in w.icp.
static bool enqueue_adjoint_step(Engine& e, Work& w, double strength_dt, bool cached, bool cpl_cached) {
  const Grid& g = e.T.g;
  cudaStream_t st = e.st;
  const double coef = 0.5 * strength_dt;
  if (strength_dt != 0.0) LK(launch_sub_scaled(g, cb(w.icp, w.csz), mb(w.Ca, w.csz), coef, w.nseg, st, w.gdev));
  // Without the cache the primal fields of substage k's previous state are the
  // current state of substage k + 1, so they are computed once: buffers A/B
  // alternate (cur: A, B, A; prev: B, A).
  double* PA = w.Pp;
  double* PB = w.Pprev;
  for (int k = 0; k < 3; ++k) {
    Batch<const double> Pcur, Pprv;
    SlotRef scur = noslot(), sprv = noslot();
    if (cached) {
      Pcur = Pprv = cbd(w.Pc, w.cstride);
      scur = SlotRef{w.step, 3, -k - 1, (long long)w.psz};  // MC[3n - k - 1]
      sprv = SlotRef{w.step, 3, -k - 2, (long long)w.psz};  // MC[3n - k - 2]
    } else {
      double* cur = (k == 1) ? PB : PA;
      double* prv = (k == 1) ? PA : PB;
      Pcur = cbd(cur, w.psz);
      Pprv = cbd(prv, w.psz);
      ReconArgs r{};
      r.grids = w.gdev;
      r.ninst = w.nseg;
      r.status = nullptr;
      r.sdiv = 1;
      r.C = cb(w.MC, w.traj);
      PhysArgs p{};
      p.grids = w.gdev;
      p.tmp = w.Zt;
      p.tmp_inst = w.zt_inst;
      p.nfields = 6;
      p.ninst = w.nseg;
      p.status = nullptr;
      p.sdiv = 1;
      p.pslot = noslot();
      if (k == 0) {
        r.slot = SlotRef{w.step, 3, -1, (long long)w.csz};
        r.U = mb(w.Up, w.usz);
        LK(launch_recon(g, r, st));
        p.U = cb(w.Up, w.usz);
        p.P = mbd(cur, w.psz);
        LK(launch_phys_inverse(g, p, st));
      }
      if (k < 2) {
        r.slot = SlotRef{w.step, 3, -k - 2, (long long)w.csz};
        r.U = mb(w.Uprev, w.usz);
        LK(launch_recon(g, r, st));
        p.U = cb(w.Uprev, w.usz);
        p.P = mbd(prv, w.psz);
        LK(launch_phys_inverse(g, p, st));
      }
    }
    ReconArgs rl{};
    rl.grids = w.gdev;
    rl.ninst = w.nseg;
    rl.status = nullptr;
    rl.sdiv = 1;
    rl.C = cb(w.Sa, w.csz);
    rl.slot = noslot();
    rl.U = mb(w.Ul, w.usz);
    LK(launch_recon(g, rl, st));
    PhysArgs pl{};
    pl.grids = w.gdev;
    pl.tmp = w.Zt;
    pl.tmp_inst = w.zt_inst;
    pl.nfields = 3;
    pl.ninst = w.nseg;
    pl.status = nullptr;
    pl.sdiv = 1;
    pl.pslot = noslot();
    pl.U = cb(w.Ul, w.usz);
    pl.P = mbd(w.Pl, w.psz);
    LK(launch_phys_inverse(g, pl, st));
    ProdArgs a{};
    a.grids = w.gdev;
    a.tmp = w.Zt;
    a.tmp_inst = w.zt_inst;
    a.pdiv = 1;
    a.ninst = w.nseg;
    a.status = nullptr;
    a.sdiv = 1;
    a.Pt = cbd(w.Pl, w.psz);
    a.Pp = Pcur;
    a.pslot = scur;
    a.H = mb(w.Up, w.usz);
    // the two passes read the same adjoint fields and write apart: branches
    const bool conc = k < 2 && chains_concurrent(e);
    if (conc && !fork_to(e, st, e.st2, 0)) return false;
    LK(launch_products_adj(g, a, st));
    if (k < 2) {
      a.Pp = Pprv;
      a.pslot = sprv;
      a.H = mb(w.Uprev, w.usz);
      LK(launch_products_adj(g, a, conc ? e.st2 : st));
      if (conc && !fork_to(e, e.st2, st, 3)) return false;  // join
    }
    SolveArgs s{};
    s.grids = w.gdev;
    s.H = cb(w.Up, w.usz);
    s.Hprev = cb(w.Uprev, w.usz);
    s.Cc = mb(w.Ca, w.csz);
    s.Sout = mb(w.Sa, w.csz);
    s.T = mb(nullptr, 0);
    s.tdiv = 1;
    s.tsel = 0;
    s.slot = noslot();
    s.k = k;
    s.adjoint = 1;
    s.mean_mode = MEAN_ADJOINT;
    s.mdiv = 1;
    s.ninst = w.nseg;
    s.status = nullptr;
    s.sdiv = 1;
    LK(launch_solve(g, s, st));
  }
  if (strength_dt != 0.0 && !enqueue_coupling(e, w, -1, coef, cpl_cached)) return false;
  LK(launch_step_advance(w.step, -1, st));
  return true;
}

// One step of the exact discrete adjoint of the homogeneous tangent, for
// step n = *step - 1 (the counter then moves down by one): substages 2, 1, 0
// transposed.  w.Ca carries the state cotangent, w.Ul the velocity
// cotangent, w.Uprev H_bar, w.Pl its physical fields; the primal fields of
// the state before substage k, slot 3n + k of `traj` (segment stride
// `tstride`), come from the field cache or are rebuilt into w.Pp.
static bool enqueue_adjoint_exact_step(Engine& e, Work& w, bool cached, const cpx* traj, long long tstride,
                                       const cpx* src, const double* ftr = nullptr, bool grad = false) {
  const Grid& g = e.T.g;
  cudaStream_t st = e.st;
  for (int k = 2; k >= 0; --k) {
    SolveTArgs t{};
    t.grids = w.gdev;
    t.Ub = cb(w.Ul, w.usz);
    t.Cc = mb(w.Ca, w.csz);
    t.Hb = mb(w.Uprev, w.usz);
    t.k = k;
    t.final_only = 0;
    t.ninst = w.nseg;
    t.status = nullptr;
    t.sdiv = 1;
    if (grad) {
      t.gacc = w.gacc;
      t.gstride = w.gstride;
      t.Xf = traj;
      t.xstride = tstride;
      t.xslot = SlotRef{w.step, 3, k - 3, (long long)w.csz};  // MC[3n + k]: slot 3(*step - 1) + k
      t.Ftr = ftr;
      t.ftr_stride = 3 * (long long)w.nsteps + 1;
    }
    LK(launch_solve_T(g, t, st));
    PhysArgs ph{};
    ph.grids = w.gdev;
    ph.tmp = w.Zt;
    ph.tmp_inst = w.zt_inst;
    ph.U = cb(w.Uprev, w.usz);
    ph.P = mbd(w.Pl, w.psz);
    ph.pslot = noslot();
    ph.nfields = 3;
    ph.ninst = w.nseg;
    ph.status = nullptr;
    ph.sdiv = 1;
    LK(launch_phys_inverse(g, ph, st));
    Batch<const double> Pprim = cbd(w.Pp, w.psz);
    SlotRef pslot = noslot();
    if (cached) {
      Pprim = cbd(w.Pc, w.cstride);
      pslot = SlotRef{w.step, 3, k - 3, (long long)w.psz};  // slot 3(*step - 1) + k
    } else {
      ReconArgs r{};
      r.grids = w.gdev;
      r.C = cb(traj, tstride);
      r.slot = SlotRef{w.step, 3, k - 3, (long long)w.csz};
      r.U = mb(w.Up, w.usz);
      r.ninst = w.nseg;
      r.status = nullptr;
      r.sdiv = 1;
      LK(launch_recon(g, r, st));
      PhysArgs pp{};
      pp.grids = w.gdev;
      pp.tmp = w.Zt;
      pp.tmp_inst = w.zt_inst;
      pp.U = cb(w.Up, w.usz);
      pp.P = mbd(w.Pp, w.psz);
      pp.pslot = noslot();
      pp.nfields = 6;
      pp.ninst = w.nseg;
      pp.status = nullptr;
      pp.sdiv = 1;
      LK(launch_phys_inverse(g, pp, st));
    }
    ProdArgs a{};
    a.grids = w.gdev;
    a.tmp = w.Zt;
    a.tmp_inst = w.zt_inst;
    a.Pp = Pprim;
    a.pdiv = 1;
    a.pslot = pslot;
    a.Pt = cbd(w.Pl, w.psz);
    a.H = mb(w.Ul, w.usz);
    a.ninst = w.nseg;
    a.status = nullptr;
    a.sdiv = 1;
    a.exact = 1;
    LK(launch_products_adj(g, a, st));
  }
  // the source of the state this step started from: lambda_n += src
  if (src) LK(launch_add_source(g, cb(src, w.csz), mb(w.Ca, w.csz), w.nseg, st, w.gdev));
  LK(launch_step_advance(w.step, -1, st));
  return true;
}

// the key of a step graph: raw bytes of the values its launches read
struct GraphKey {
  std::string s;
  template <typename T>
  GraphKey& add(const T& v) {
    s.append(reinterpret_cast<const char*>(&v), sizeof(T));
    return *this;
  }
};

// what every step graph of a working set reads besides its own options:
// the grid (sizes, tables, kernel variants) and the arrays that a sweep may
// point elsewhere for its duration, and the LSS window chaining of the
// coupling's time derivative
static GraphKey step_key(const Engine& e, const Work& w, char kind) {
  GraphKey k;
  k.add(kind).add(e.T.g).add(w.MC).add(w.Ft).add(w.gdev).add(w.nseg).add(w.ntan).add(w.chain);
  return k;
}

static GraphKey& add_opts(GraphKey& k, const FwdOpts& o) {
  return k.add(o.adv_primal).add(o.tangents).add(o.ru).add(o.forced_mask).add(o.raw_u_first).add(o.cache)
      .add(o.store).add(o.re2_mask).add(o.re3_mask);
}

// A multi-step sweep as ONE graph launch: a graph whose while node runs one
// captured step followed by k_loop_next, which counts the device-side
// steps-left counter down and ends the loop after the last step.  The graph
// is built once per working set and key (or taken from the working set's
// graphs when the key matches); each sweep sets the counter and launches it.
// CHN_SWEEP_GRAPHS=0 launches every step's kernels on the stream instead
// (the same kernels and results; profilers that skip the kernel nodes of
// graphs with conditional nodes then see every launch).
static bool sweep_graphs_on() {
  static const bool on = [] {
    const char* v = getenv("CHN_SWEEP_GRAPHS");
    return !(v && v[0] == '0');
  }();
  return on;
}

template <typename F>
static bool run_steps(Engine& e, Work& w, const GraphKey& key, int nsteps, F&& enqueue) {
  if (nsteps <= 0) return true;
  if (nsteps == 1) return enqueue();
  if (!sweep_graphs_on()) {
    for (int i = 0; i < nsteps; ++i)
      if (!enqueue()) return false;
    return true;
  }
  Work::StepGraph* sg = nullptr;
  for (Work::StepGraph& x : w.graphs)
    if (x.key == key.s) sg = &x;
  if (!sg) {
    cudaGraph_t graph = nullptr;
    CK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h{};
    cudaGraphNodeParams p{};
    cudaGraphNode_t node = nullptr;
    cudaError_t ge = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
    if (ge == cudaSuccess) {
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = h;
      p.conditional.type = cudaGraphCondTypeWhile;
      p.conditional.size = 1;
      ge = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &p);
    }
    if (ge == cudaSuccess)
      ge = cudaStreamBeginCaptureToGraph(e.st, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal);
    if (ge != cudaSuccess) {
      cudaGraphDestroy(graph);
      set_error(-1, "sweep graph: %s", cudaGetErrorString(ge));
      return false;
    }
    const long long before = g_launches;
    bool ok = enqueue();
    ok = ok && launch_loop_next(w.loopctr, h, e.st) == cudaSuccess;
    cudaGraph_t body = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e.st, &body);
    const long long per_step = g_launches - before;
    g_launches = before;  // counted for every step the launch below runs
    if (!ok || ce != cudaSuccess) {
      cudaGraphDestroy(graph);
      if (ok) set_error(-1, "sweep graph capture: %s", cudaGetErrorString(ce));
      return false;
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie);
    if (w.graphs.size() >= Work::kMaxGraphs) {
      cudaGraphExecDestroy(w.graphs.front().exec);
      w.graphs.erase(w.graphs.begin());
    }
    w.graphs.push_back(Work::StepGraph{key.s, exec, per_step});
    sg = &w.graphs.back();
  }
  LK(launch_loop_set(w.loopctr, nsteps, e.st));
  const cudaError_t le = cudaGraphLaunch(sg->exec, e.st);
  if (le != cudaSuccess) {
    set_error(-1, "cudaGraphLaunch: %s", cudaGetErrorString(le));
    return false;
  }
  g_launches += sg->per_step * nsteps;
  return true;
}

static bool set_step(Engine& e, Work& w, int n) {
  CK(cudaMemcpyAsync(w.step, &n, sizeof(int), cudaMemcpyHostToDevice, e.st));
  return true;
}

static bool reset_status(Engine& e, Work& w) {
  CK(cudaMemsetAsync(w.status, 0, sizeof(uint32_t) * w.nseg, e.st));
  CK(cudaMemsetAsync(w.cflmax, 0, sizeof(double) * w.nseg, e.st));
  return true;
}

static bool collect_status(Engine& e, Work& w) {
  std::vector<uint32_t> s(w.nseg);
  std::vector<double> c(w.nseg);
  CK(cudaMemcpyAsync(s.data(), w.status, sizeof(uint32_t) * w.nseg, cudaMemcpyDeviceToHost, e.st));
  CK(cudaMemcpyAsync(c.data(), w.cflmax, sizeof(double) * w.nseg, cudaMemcpyDeviceToHost, e.st));
  CK(cudaStreamSynchronize(e.st));
  uint32_t any = 0;
  double cm = 0.0;
  for (int i = 0; i < w.nseg; ++i) {
    any |= s[i];
    cm = std::fmax(cm, c[i]);
  }
  g_cfl = cm;
  g_status = (int)any;
  if (any & ST_CFL) g_msg = "CFL condition violated: time loop stopped (channel/pass1.c:133-137)";
  else if (any & ST_NONFINITE) g_msg = "non-finite values in the physical fields";
  else g_msg.clear();
  if (tc5_take_error()) {
    set_error(-3, "a tensor-core wait of the inverse transform expired; its results are not valid");
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// autotuner: the transform kernels (inverse of six fields, tangent products,
// adjoint products) of one batched substage, timed on the working set's
// buffers for the one-block-per-plane kernels (where a plane fits) and every
// split variant that fits; the fastest is kept in the engine's grid.  All
// candidates compute identical results.  CHN_AUTOTUNE=0 skips it.
// ---------------------------------------------------------------------------

static std::string g_tune_report;

// the builds of the tensor-core inverse (Grid::tcminb): fields per pass,
// blocks per SM, compile-time sizes
static const char* inverse_build_name(int b) {
  switch (b) {
    case 3: return "f2_b3";
    case 4: return "f1_b4";
    case 5: return "f1_b5";
    case 6: return "f1_b4_fixed";
    case 7: return "f2_b2_fixed";
    case 8: return "f1_t192_b3";
    case 9: return "f1_t192_b3_fixed";
    case 10: return "f1_b5_fixed";
    case 11: return "f1_t192_b4_fixed";
    case 12: return "f1_t256_b3_fixed";
    default: return "f2_b2";
  }
}

static bool autotune_transforms(Engine& e, Work& w) {
  const char* off = getenv("CHN_AUTOTUNE");
  if (off && off[0] == '0') return true;
  const char* force = getenv("CHN_SPLIT_TRANSFORMS");
  if (force && force[0] == '1') return true;
  Grid& g = e.T.g;
  int dev = 0, optin = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  struct Cand {
    int split, tvar, minb, tc5;
    float ms;
  };
  std::vector<Cand> cands;
  const char* t5env = getenv("CHN_INVERSE_TC5");
  const bool t5forced = t5env && (t5env[0] == '0' || t5env[0] == '1');
  const char* ibenv = getenv("CHN_INVERSE_BUILD");
  const bool ibforced = ibenv && ibenv[0];
  if (g.tci && g.tcf) {
    // both transforms on the tensor cores: the FFT variants are unused; time
    // the builds of the mma.sync inverse and the tcgen05 one
    if (!(t5forced && g.tc5)) {
      if (ibforced) {
        cands.push_back({g.split, g.tvar, g.tcminb, 0, 0.f});
      } else {
        const int rt[5] = {2, 3, 4, 5, 8}, ct[6] = {6, 7, 9, 10, 11, 12};
        for (int b : rt) cands.push_back({g.split, g.tvar, b, 0, 0.f});
        if (!w.gdev && phys_tc_specialised(g))
          for (int b : ct) cands.push_back({g.split, g.tvar, b, 0, 0.f});
      }
    }
    if (g.t5Z && !(t5forced && !g.tc5) && !(ibforced && !t5forced) && !w.gdev)
      cands.push_back({g.split, g.tvar, 2, 1, 0.f});
  } else {
    if (fused_transforms_fit(g, optin)) cands.push_back({0, 0, g.tcminb, 0, 0.f});
    for (int v = 0; v < split_variant_count(); ++v)
      if (split_variant_fits(v, g, optin)) cands.push_back({1, v, g.tcminb, 0, 0.f});
  }
  if (cands.size() < 2 || !w.Zt) return true;
  const int nt = w.nseg * (w.ntan > 0 ? w.ntan : 1);
  auto enqueue = [&]() -> bool {
    PhysArgs p{};
    p.U = cb(w.Ut, w.usz);
    p.P = mbd(w.Pt, w.psz);
    p.nfields = 6;
    p.ninst = nt;
    p.sdiv = 1;
    p.tmp = w.Zt;
    p.tmp_inst = w.zt_inst;
    p.grids = w.gdev;
    LK(launch_phys_inverse(g, p, e.st));
    ProdArgs f{};
    f.Pp = cbd(w.Pp, w.psz);
    f.pdiv = w.ntan > 0 ? w.ntan : 1;
    f.Pt = cbd(w.Pt, w.psz);
    f.H = mb(w.Ut, w.usz);
    f.ninst = nt;
    f.sdiv = 1;
    f.tmp = w.Zt;
    f.tmp_inst = w.zt_inst;
    f.grids = w.gdev;
    LK(launch_products_fwd(g, f, e.st));
    ProdArgs b = f;
    b.pdiv = 1;
    b.Pt = cbd(w.Pl, w.psz);
    b.H = mb(w.Up, w.usz);
    b.ninst = w.nseg;
    LK(launch_products_adj(g, b, e.st));
    return true;
  };
  cudaEvent_t t0, t1;
  CK(cudaEventCreate(&t0));
  CK(cudaEventCreate(&t1));
  const int saved_split = g.split, saved_tvar = g.tvar, saved_minb = g.tcminb, saved_tc5 = g.tc5;
  bool ok = true;
  for (Cand& c : cands) {
    g.split = c.split;
    g.tvar = c.tvar;
    g.tcminb = c.minb;
    g.tc5 = c.tc5;
    ok = ok && enqueue();  // warm-up
    ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
    for (int r = 0; r < 3; ++r) ok = ok && enqueue();
    ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
    if (!ok) break;
    cudaEventElapsedTime(&c.ms, t0, t1);
    c.ms /= 3;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (!ok) {
    g.split = saved_split;
    g.tvar = saved_tvar;
    g.tcminb = saved_minb;
    g.tc5 = saved_tc5;
    return false;
  }
  const Cand* best = &cands[0];
  for (const Cand& c : cands)
    if (c.ms < best->ms) best = &c;
  g.split = best->split;
  g.tvar = best->tvar;
  g.tcminb = best->minb;
  g.tc5 = best->tc5;
  char buf[160];
  g_tune_report = "{";
  const bool tcv = g.tci && g.tcf;
  for (const Cand& c : cands) {
    if (tcv && c.tc5) {
      snprintf(buf, sizeof(buf), "\"tc_inverse_tcgen05\": %.4f, ", c.ms);
    } else if (tcv) {
      snprintf(buf, sizeof(buf), "\"tc_inverse_%s\": %.4f, ", inverse_build_name(c.minb), c.ms);
    } else if (c.split) {
      const TransformVariant v = split_variant(c.tvar);
      snprintf(buf, sizeof(buf), "\"split_nt%d_ch%d\": %.4f, ", v.nt, v.ch, c.ms);
    } else {
      snprintf(buf, sizeof(buf), "\"fused\": %.4f, ", c.ms);
    }
    g_tune_report += buf;
  }
  if (tcv && best->tc5) {
    snprintf(buf, sizeof(buf), "\"chosen\": \"tc_inverse_tcgen05\", \"instances\": %d}", nt);
  } else if (tcv) {
    snprintf(buf, sizeof(buf), "\"chosen\": \"tc_inverse_%s\", \"instances\": %d}", inverse_build_name(best->minb),
             nt);
  } else if (best->split) {
    const TransformVariant v = split_variant(best->tvar);
    snprintf(buf, sizeof(buf), "\"chosen\": \"split_nt%d_ch%d\", \"instances\": %d}", v.nt, v.ch, nt);
  } else {
    snprintf(buf, sizeof(buf), "\"chosen\": \"fused\", \"instances\": %d}", nt);
  }
  g_tune_report += buf;
  return true;
}

// ---------------------------------------------------------------------------
// operations shared by the single and batched APIs (device pointers in/out)
// ---------------------------------------------------------------------------

// primal from C (device, nseg arrays) or, when C == nullptr, the laminar start
// autotuner, the implicit solve: the block tile (kx columns per block, 16
// or 8) timed on one batched tangent solve of the working set; both compute
// the same results.  The choice and the times join c_autotune_report.
static bool autotune_solve(Engine& e, Work& w) {
  const char* off = getenv("CHN_AUTOTUNE");
  const char* fixed = getenv("CHN_SOLVE_TILE");
  if ((off && off[0] == '0') || (fixed && fixed[0])) return true;
  Grid& g = e.T.g;
  const int nt = w.nseg * (w.ntan > 0 ? w.ntan : 1);
  SolveArgs sa{};
  sa.grids = w.gdev;
  sa.H = cb(w.Ut, w.usz);
  sa.Hprev = cb(nullptr, 0);
  sa.Cc = mb(w.io, w.csz);  // scratch: no state of the working set is touched
  sa.Sout = mb(w.io, w.csz);
  sa.T = mb(nullptr, 0);
  sa.tdiv = 1;
  sa.slot = noslot();
  sa.k = 1;
  sa.mean_mode = MEAN_TAN_HOMOG;
  sa.mdiv = w.ntan > 0 ? w.ntan : 1;
  sa.ninst = nt;
  sa.sdiv = w.ntan > 0 ? w.ntan : 1;
  const int tiles[3] = {16, 8, 8}, thr[3] = {256, 256, 128};
  float ms[3] = {0.f, 0.f, 0.f};
  cudaEvent_t t0, t1;
  CK(cudaEventCreate(&t0));
  CK(cudaEventCreate(&t1));
  const int saved = g.stile, saved_thr = g.sthr;
  bool ok = true;
  for (int c = 0; c < 3 && ok; ++c) {
    g.stile = tiles[c];
    g.sthr = thr[c];
    ok = launch_solve(g, sa, e.st) == cudaSuccess;  // warm-up
    ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
    for (int r = 0; r < 3 && ok; ++r) ok = launch_solve(g, sa, e.st) == cudaSuccess;
    ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
    if (ok) cudaEventElapsedTime(&ms[c], t0, t1);
    ms[c] /= 3;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  g_launches += ok ? 12 : 0;
  if (!ok) {
    g.stile = saved;
    g.sthr = saved_thr;
    set_error(-1, "solve autotuner: %s", cudaGetErrorString(cudaGetLastError()));
    return false;
  }
  int best = 0;
  for (int c = 1; c < 3; ++c)
    if (ms[c] < ms[best]) best = c;
  g.stile = tiles[best];
  g.sthr = thr[best];
  char buf[200];
  snprintf(buf, sizeof(buf),
           "\"solve_tile16\": %.4f, \"solve_tile8\": %.4f, \"solve_tile8_t128\": %.4f, \"solve_chosen\": \"%s\"",
           ms[0], ms[1], ms[2], best == 0 ? "tile16" : (best == 1 ? "tile8" : "tile8_t128"));
  if (g_tune_report.size() > 1 && g_tune_report.back() == '}') {
    g_tune_report.pop_back();
    g_tune_report += ", ";
  } else {
    g_tune_report = "{";
  }
  g_tune_report += buf;
  g_tune_report += "}";
  return true;
}

// autotuner, the builds compiled for the grid's sizes (sizes.cuh; the
// same results): for the product kernels (one batched substage's tangent
// and adjoint products), the reconstruction (tangents) and the implicit
// solve (a tangent solve into scratch), each timed against its run-time-
// size build and kept where faster (Grid::fixed).  CHN_FIXED_SIZES=0 / 1
// fixes all three off / on.  Then the adjoint products' planes per pass,
// 1 or 3 (Grid::adjpb; CHN_ADJ_PRODUCTS_PER_PASS fixes it), and the
// reconstruction's build, tile and blocks per SM (Grid::rbuild; CHN_RECON_BUILD).
static bool autotune_fixed(Engine& e, Work& w) {
  const char* off = getenv("CHN_AUTOTUNE");
  const char* forced = getenv("CHN_FIXED_SIZES");
  Grid& g = e.T.g;
  const char* apb = getenv("CHN_ADJ_PRODUCTS_PER_PASS");
  const bool do_fixed = !(forced && forced[0]) && !w.gdev && phys_tc_specialised(g);
  const bool do_pb = g.tcf && !w.gdev;  // the adjoint planes per pass, the products' build
  const char* rbe = getenv("CHN_RECON_BUILD");
  const bool do_rt = g.tc && !(rbe && rbe[0]) && !w.gdev;
  if ((off && off[0] == '0') || !(do_fixed || do_pb || do_rt)) return true;
  const int nt = w.nseg * (w.ntan > 0 ? w.ntan : 1);
  ProdArgs f{};
  f.Pp = cbd(w.Pp, w.psz);
  f.pdiv = w.ntan > 0 ? w.ntan : 1;
  f.Pt = cbd(w.Pt, w.psz);
  f.H = mb(w.Ut, w.usz);
  f.ninst = nt;
  f.sdiv = 1;
  f.tmp = w.Zt;
  f.tmp_inst = w.zt_inst;
  ProdArgs b = f;
  b.pdiv = 1;
  b.Pt = cbd(w.Pl, w.psz);
  b.H = mb(w.Up, w.usz);
  b.ninst = w.nseg;
  ReconArgs r{};
  r.ninst = nt;
  r.C = cb(w.St, w.csz);
  r.slot = noslot();
  r.U = mb(w.Ut, w.usz);
  r.sdiv = 1;
  SolveArgs sa{};
  sa.H = cb(w.Ut, w.usz);
  sa.Hprev = cb(nullptr, 0);
  sa.Cc = mb(w.io, w.csz);  // scratch: no state of the working set is touched
  sa.Sout = mb(w.io, w.csz);
  sa.T = mb(nullptr, 0);
  sa.tdiv = 1;
  sa.slot = noslot();
  sa.k = 1;
  sa.mean_mode = MEAN_TAN_HOMOG;
  sa.mdiv = w.ntan > 0 ? w.ntan : 1;
  sa.ninst = nt;
  sa.sdiv = w.ntan > 0 ? w.ntan : 1;
  struct Part {
    int bit;
    const char* name;
    int launches;
  };
  const Part parts[3] = {{FIXED_PRODUCTS, "products", 2}, {FIXED_RECON, "recon", 1}, {FIXED_SOLVE, "solve", 1}};
  auto enqueue = [&](int bit) -> bool {
    if (bit == FIXED_PRODUCTS)
      return launch_products_fwd(g, f, e.st) == cudaSuccess && launch_products_adj(g, b, e.st) == cudaSuccess;
    if (bit == FIXED_RECON) return launch_recon(g, r, e.st) == cudaSuccess;
    return launch_solve(g, sa, e.st) == cudaSuccess;
  };
  cudaEvent_t t0, t1;
  CK(cudaEventCreate(&t0));
  CK(cudaEventCreate(&t1));
  const int saved = g.fixed;
  bool ok = true;
  std::string rep;
  char buf[160];
  for (const Part& pt : parts) {
    if (!do_fixed) break;
    float ms[2] = {0.f, 0.f};
    for (int c = 0; c < 2 && ok; ++c) {
      g.fixed = c ? (g.fixed | pt.bit) : (g.fixed & ~pt.bit);
      ok = enqueue(pt.bit);  // warm-up
      ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
      for (int k = 0; k < 3 && ok; ++k) ok = enqueue(pt.bit);
      ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
      if (ok) cudaEventElapsedTime(&ms[c], t0, t1);
      ms[c] /= 3;
    }
    if (!ok) break;
    g_launches += 8 * pt.launches;
    g.fixed = ms[1] < ms[0] ? (g.fixed | pt.bit) : (g.fixed & ~pt.bit);
    snprintf(buf, sizeof(buf), "\"%s_runtime_sizes\": %.4f, \"%s_fixed_sizes\": %.4f, \"%s_sizes\": \"%s\"", pt.name,
             ms[0], pt.name, ms[1], pt.name, (g.fixed & pt.bit) ? "fixed" : "runtime");
    if (!rep.empty()) rep += ", ";
    rep += buf;
  }
  // the adjoint products' planes per pass (its own switch)
  if (ok && do_pb && !(apb && apb[0])) {
    const int saved_pb = g.adjpb;
    float ms[2] = {0.f, 0.f};
    const int pbs[2] = {1, 3};
    for (int c = 0; c < 2 && ok; ++c) {
      g.adjpb = pbs[c];
      ok = launch_products_adj(g, b, e.st) == cudaSuccess;  // warm-up
      ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
      for (int k = 0; k < 3 && ok; ++k) ok = launch_products_adj(g, b, e.st) == cudaSuccess;
      ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
      if (ok) cudaEventElapsedTime(&ms[c], t0, t1);
      ms[c] /= 3;
    }
    if (ok) {
      g_launches += 8;
      g.adjpb = ms[1] < ms[0] ? 3 : 1;
      snprintf(buf, sizeof(buf), "\"adjoint_products_pb1\": %.4f, \"adjoint_products_pb3\": %.4f, "
               "\"adjoint_products_per_pass\": %d", ms[0], ms[1], g.adjpb);
      if (!rep.empty()) rep += ", ";
      rep += buf;
    } else {
      g.adjpb = saved_pb;
    }
  }
  // the products' build: three planes per pass at 2 blocks per SM (the
  // plan) against two planes at 3 blocks
  const char* pbe = getenv("CHN_PRODUCTS_BUILD");
  if (ok && g.tcf && !w.gdev && !(pbe && pbe[0])) {
    const int saved_b = g.prodb;
    float ms[2] = {0.f, 0.f};
    for (int c = 0; c < 2 && ok; ++c) {
      g.prodb = c;
      ok = enqueue(FIXED_PRODUCTS);  // warm-up
      ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
      for (int k = 0; k < 3 && ok; ++k) ok = enqueue(FIXED_PRODUCTS);
      ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
      if (ok) cudaEventElapsedTime(&ms[c], t0, t1);
      ms[c] /= 3;
    }
    if (ok) {
      g_launches += 16;
      g.prodb = ms[1] < ms[0] ? 1 : 0;
      snprintf(buf, sizeof(buf), "\"products_b0\": %.4f, \"products_b1\": %.4f, \"products_build\": %d", ms[0], ms[1],
               g.prodb);
      if (!rep.empty()) rep += ", ";
      rep += buf;
    } else {
      g.prodb = saved_b;
    }
  }
  // the reconstruction's build (tile, threads, blocks per SM)
  if (ok && do_rt) {
    const int saved_t = g.rbuild;
    float ms[3] = {0.f, 0.f, 0.f};
    for (int c = 0; c < 3 && ok; ++c) {
      g.rbuild = c;
      ok = enqueue(FIXED_RECON);  // warm-up
      ok = ok && cudaEventRecord(t0, e.st) == cudaSuccess;
      for (int k = 0; k < 3 && ok; ++k) ok = enqueue(FIXED_RECON);
      ok = ok && cudaEventRecord(t1, e.st) == cudaSuccess && cudaEventSynchronize(t1) == cudaSuccess;
      if (ok) cudaEventElapsedTime(&ms[c], t0, t1);
      ms[c] /= 3;
    }
    if (ok) {
      g_launches += 12;
      int best = 0;
      for (int c = 1; c < 3; ++c)
        if (ms[c] < ms[best]) best = c;
      g.rbuild = best;
      snprintf(buf, sizeof(buf), "\"recon_b0\": %.4f, \"recon_b1\": %.4f, \"recon_b2\": %.4f, \"recon_build\": %d",
               ms[0], ms[1], ms[2], g.rbuild);
      if (!rep.empty()) rep += ", ";
      rep += buf;
    } else {
      g.rbuild = saved_t;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (!ok) {
    g.fixed = saved;
    set_error(-1, "fixed-size autotuner: %s", cudaGetErrorString(cudaGetLastError()));
    return false;
  }
  if (g_tune_report.size() > 1 && g_tune_report.back() == '}') {
    g_tune_report.pop_back();
    g_tune_report += ", ";
  } else {
    g_tune_report = "{";
  }
  g_tune_report += rep;
  g_tune_report += "}";
  return true;
}

// The autotuners' timing inputs: the working set's spectral planes,
// physical fields and tangent coefficients filled with a seeded pattern
// before the timings (fill) and cleared again after them, so a batch starts
// from the zeroed buffers it would have had without tuning.
static bool tune_inputs(Engine& e, Work& w, bool fill) {
  const size_t nt = (size_t)w.nseg * (w.ntan > 0 ? w.ntan : 1);
  struct Buf {
    double* p;
    size_t n;
  };
  const Buf bufs[6] = {{reinterpret_cast<double*>(w.Ut), 2 * nt * w.usz},
                       {reinterpret_cast<double*>(w.Up), 2 * (size_t)w.nseg * w.usz},
                       {reinterpret_cast<double*>(w.St), 2 * nt * w.csz},
                       {w.Pp, (size_t)w.nseg * w.psz},
                       {w.Pt, nt * w.psz},
                       {w.Pl, (size_t)w.nseg * w.psz}};
  uint32_t seed = 0x9E3779B9u;
  for (const Buf& b : bufs) {
    if (!b.p) continue;
    if (fill) LK(launch_fill_pattern(b.p, b.n, seed++, e.st));
    else CK(cudaMemsetAsync(b.p, 0, b.n * sizeof(double), e.st));
  }
  return true;
}

static bool op_primal(Engine& e, Work& w, int ru, const cpx* C) {
  NvtxRange nvtx_op("op_primal");
  const size_t csz = w.csz;
  CK(cudaMemsetAsync(w.MC, 0, sizeof(cpx) * (size_t)w.nseg * w.traj, e.st));
  if (C) {
    CK(cudaMemcpy2DAsync(w.Cp, csz * sizeof(cpx), C, csz * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                         cudaMemcpyDeviceToDevice, e.st));
  } else {
    // channel/channel.c:409-422: laminar (1 - y^2) flux 3/4 plus rand() noise on
    // (kz, kx) = (1, 1), then the Gram projection of initAlphaBeta()
    const Grid& g = e.T.g;
    std::vector<cpx> U(w.usz, cpx{0.0, 0.0});
    for (int i = 0; i < g.Q; ++i)
      U[((size_t)0 * 5 + 0) * g.Q * g.X + (size_t)i * g.X + 0] =
          cpx{(1.0 - e.qy[i] * e.qy[i]) * g.flux * 3. / 4, 0.0};
    for (int i = 0; i < g.Q; ++i) {
      const double re = (rand() / (double)RAND_MAX - 0.5);
      const double im = (rand() / (double)RAND_MAX - 0.5);
      U[((size_t)1 * 5 + 0) * g.Q * g.X + (size_t)i * g.X + 1] = cpx{re, im};
    }
    CK(cudaMemcpyAsync(w.Ul, U.data(), sizeof(cpx) * w.usz, cudaMemcpyHostToDevice, e.st));
    // the projection overwrites alpha rows < Ny-4 and beta; other rows keep the carried array
    for (int s = 0; s < w.nseg; ++s) {
      LK(launch_project_init(g, w.Ul, w.Cp + (size_t)s * csz, e.T.luQs, e.T.luRs, e.st));
      // the first substage runs on these samples, not on their projection:
      // the reference never rebuilds U after initAlphaBeta() (channel/channel.c:409-422)
      CK(cudaMemcpyAsync(w.Up + (size_t)s * w.usz, w.Ul, sizeof(cpx) * w.usz, cudaMemcpyDeviceToDevice, e.st));
    }
  }
  CK(cudaMemcpyAsync(w.Sp, w.Cp, sizeof(cpx) * csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
  CK(cudaMemcpy2DAsync(w.MC, w.traj * sizeof(cpx), w.Cp, csz * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                       cudaMemcpyDeviceToDevice, e.st));
  if (!reset_status(e, w) || !set_step(e, w, 0)) return false;
  w.mark(0, 3 * w.nsteps, false);
  w.raw_start = !C && ru == 0;
  // run-up steps are not stored, so their fields are not cached
  FwdOpts o{true, false, ru, 0u, false, false};
  int n = 0;
  auto run_range = [&](int n1, bool cache) -> bool {
    FwdOpts oo = o;
    oo.cache = cache;
    if (n == 0 && !C && n < n1) {
      FwdOpts first = oo;
      first.raw_u_first = true;
      if (!enqueue_forward_step(e, w, first)) return false;
      ++n;
    }
    const int cnt = n1 - n;
    n = n1;
    GraphKey key = step_key(e, w, 'p');
    return run_steps(e, w, add_opts(key, oo), cnt, [&] { return enqueue_forward_step(e, w, oo); });
  };
  if (!run_range(ru, false) || !run_range(ru + w.nsteps, true)) return false;
  if (!C && ru == 0 && w.Pc && w.nsteps > 0) {
    // cache slot 0 holds the fields of the raw laminar samples that the first
    // substage ran on; the tangent and adjoint sweeps rebuild MC[0] instead
    // (channel/channel.c:496-514), so slot 0 gets the fields of MC[0]
    ReconArgs r{};
    r.grids = w.gdev;
    r.C = cb(w.MC, w.traj);
    r.slot = noslot();
    r.U = mb(w.Up, w.usz);
    r.ninst = w.nseg;
    r.status = nullptr;
    r.sdiv = 1;
    LK(launch_recon(e.T.g, r, e.st));
    PhysArgs p{};
    p.grids = w.gdev;
    p.tmp = w.Zt;
    p.tmp_inst = w.zt_inst;
    p.U = cb(w.Up, w.usz);
    p.P = mbd(w.Pc, w.cstride);
    p.pslot = noslot();
    p.nfields = 6;
    p.ninst = w.nseg;
    p.status = nullptr;
    p.sdiv = 1;
    LK(launch_phys_inverse(e.T.g, p, e.st));
  }
  if (!collect_status(e, w)) return false;
  w.mark(0, 3 * w.nsteps, w.Pc != nullptr && (g_status & ST_CFL) == 0);
  return true;
}

// tangents (and optionally the primal) from start to end; IC device [nseg*ntan]
// Tangent forcings per tangent t: bit t of forced (mean flux, the reference's
// inhomo != 0), re2 (Re, the reference's disconnected forcing reconnected),
// re3 (Re, exact derivative of the discrete step).
struct Forcing {
  uint32_t forced = 0, re2 = 0, re3 = 0;
};

static bool op_forward(Engine& e, Work& w, int start, int end, const cpx* C, const cpx* IC, Forcing f,
                       bool adv_primal) {
  NvtxRange nvtx_op(adv_primal ? "op_forward" : "op_tangent");
  const size_t csz = w.csz;
  const int nt = w.nseg * w.ntan;
  if (adv_primal) {
    if (C) {
      CK(cudaMemcpy2DAsync(w.Cp, csz * sizeof(cpx), C, csz * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                           cudaMemcpyDeviceToDevice, e.st));
    } else {
      CK(cudaMemcpy2DAsync(w.Cp, csz * sizeof(cpx), w.MC + (size_t)3 * start * csz, w.traj * sizeof(cpx),
                           csz * sizeof(cpx), w.nseg, cudaMemcpyDeviceToDevice, e.st));
    }
    CK(cudaMemcpyAsync(w.Sp, w.Cp, sizeof(cpx) * csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
    CK(cudaMemcpy2DAsync(w.MC + (size_t)3 * start * csz, w.traj * sizeof(cpx), w.Cp, csz * sizeof(cpx),
                         csz * sizeof(cpx), w.nseg, cudaMemcpyDeviceToDevice, e.st));
  }
  if (w.ntan > 0) {
    CK(cudaMemcpyAsync(w.Ct, IC, sizeof(cpx) * csz * nt, cudaMemcpyDeviceToDevice, e.st));
    CK(cudaMemcpyAsync(w.St, IC, sizeof(cpx) * csz * nt, cudaMemcpyDeviceToDevice, e.st));
    // MIC[3 start] = IC of the coupled tangent (channel/channel.c:525-527)
    CK(cudaMemcpy2DAsync(w.MIC + (size_t)3 * start * csz, w.traj * sizeof(cpx), IC + (size_t)w.couple * csz,
                         (size_t)w.ntan * csz * sizeof(cpx), csz * sizeof(cpx), w.nseg, cudaMemcpyDeviceToDevice,
                         e.st));
  }
  // The reference's tangent re-advances the primal from MC[3 start] rebuilt
  // into velocity (channel/channel.c:496-514, 557-571).  That reproduces the
  // stored trajectory except after a laminar start without run-up, whose
  // first substage ran on the raw samples: then the primal is re-advanced
  // here too, without storing it.
  const bool readvance = !adv_primal && w.raw_start && start == 0;
  if (readvance) {
    CK(cudaMemcpy2DAsync(w.Cp, csz * sizeof(cpx), w.MC, w.traj * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                         cudaMemcpyDeviceToDevice, e.st));
    CK(cudaMemcpyAsync(w.Sp, w.Cp, sizeof(cpx) * csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
  }
  if (!reset_status(e, w) || !set_step(e, w, start)) return false;
  const bool cache = adv_primal ? true : (!readvance && w.cached(3 * start, 3 * end));
  if (adv_primal) w.mark(3 * start, 3 * end + 1, false);
  FwdOpts o{adv_primal || readvance, w.ntan > 0, 0, f.forced, false, cache && !readvance, !readvance};
  o.re2_mask = f.re2;
  o.re3_mask = f.re3;
  GraphKey key = step_key(e, w, 'f');
  if (!run_steps(e, w, add_opts(key, o), end - start, [&] { return enqueue_forward_step(e, w, o); })) return false;
  const bool with_vel = w.ntan > 0 && w.Pv != nullptr;
  if (adv_primal || with_vel) {
    if (!collect_status(e, w)) return false;
  }
  const bool clean = (g_status & ST_CFL) == 0;
  // the fused sweep rewrote MC[3 start + 1 .. 3 end] and cache slots [3 start, 3 end)
  if (adv_primal) w.mark(3 * start, 3 * end, w.Pc != nullptr && clean);
  if (w.ntan > 0) {
    // MIC[3 start .. 3 end] were rewritten and velocity slots [start, end) with them
    w.mark_vel(start, end, with_vel && clean);
    w.mark_vel(end, end + 1, false);
  }
  return true;
}

static bool op_adjoint(Engine& e, Work& w, int start, int end, const cpx* AC, double strength) {
  NvtxRange nvtx_op("op_adjoint");
  CK(cudaMemcpyAsync(w.Ca, AC, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
  CK(cudaMemcpyAsync(w.Sa, AC, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
  if (!reset_status(e, w) || !set_step(e, w, start)) return false;
  // channel/channel.c:619; an uneven batch scales by each segment's dt on the device
  const double sdt = w.gdev ? strength : strength * e.T.g.dt;
  const bool cached = w.cached(3 * end, 3 * start);
  bool cpl_cached = true;
  for (int i = end; i < start; ++i) cpl_cached = cpl_cached && w.coupling_cached(i);
  if (sdt != 0.0 && start > end && !enqueue_coupling(e, w, 0, 0.0, w.coupling_cached(start))) return false;
  GraphKey key = step_key(e, w, 'a');
  key.add(sdt).add(cached).add(cpl_cached);
  return run_steps(e, w, key, start - end, [&] { return enqueue_adjoint_step(e, w, sdt, cached, cpl_cached); });
}

// The transpose of the homogeneous tangent from `end` to `start` applied to
// AC (device, nseg arrays) at step `start`; the result (the cotangent at
// step `end`) is left in w.Ca.  The tangent linearises about the primal
// re-advanced from MC[3 end] rebuilt into velocity (channel/channel.c:496-514),
// which is the stored trajectory except after a laminar start without
// run-up with end == 0: then the primal is re-advanced here into a
// temporary trajectory, as op_forward does.  With `src` (device, nseg
// arrays) every step adds it after its transposition:
//   lambda_n = T_n^T lambda_{n+1} + src,  n = start - 1 .. end,
// the cotangent of a sum over steps end .. start - 1 of a linear functional.
static bool op_adjoint_exact(Engine& e, Work& w, int start, int end, const cpx* AC, const cpx* src = nullptr,
                             bool grad = false) {
  NvtxRange nvtx_op("op_adjoint_exact");
  const size_t csz = w.csz;
  const bool readvance = w.raw_start && end == 0;
  cpx* scratch = nullptr;
  double* scratch_ft = nullptr;
  if (!reset_status(e, w)) return false;
  if (readvance) {
    const size_t tbytes = sizeof(cpx) * (size_t)w.nseg * (size_t)w.traj;
    const size_t fbytes = sizeof(double) * (size_t)w.nseg * (3 * (size_t)w.nsteps + 1);
    if (cudaMalloc(&scratch, tbytes) != cudaSuccess || cudaMalloc(&scratch_ft, fbytes) != cudaSuccess) {
      cudaGetLastError();
      if (scratch) cudaFree(scratch);
      set_error(-1, "c_adjoint_exact: no device memory for the re-advanced primal trajectory");
      return false;
    }
    CK(cudaMemcpy2DAsync(w.Cp, csz * sizeof(cpx), w.MC, w.traj * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                         cudaMemcpyDeviceToDevice, e.st));
    CK(cudaMemcpyAsync(w.Sp, w.Cp, sizeof(cpx) * csz * w.nseg, cudaMemcpyDeviceToDevice, e.st));
    CK(cudaMemcpy2DAsync(scratch, w.traj * sizeof(cpx), w.Cp, csz * sizeof(cpx), csz * sizeof(cpx), w.nseg,
                         cudaMemcpyDeviceToDevice, e.st));
    // the forward sweep stores into w.MC / w.Ft: point them at the scratch
    // trajectory while its steps are enqueued
    cpx* keep_mc = w.MC;
    double* keep_ft = w.Ft;
    w.MC = scratch;
    w.Ft = scratch_ft;
    bool ok = set_step(e, w, 0);
    FwdOpts o{true, false, 0, 0u, false, false, true};
    GraphKey key = step_key(e, w, 'r');
    ok = ok && run_steps(e, w, add_opts(key, o), start, [&] { return enqueue_forward_step(e, w, o); });
    w.MC = keep_mc;
    w.Ft = keep_ft;
    if (!ok) {
      cudaStreamSynchronize(e.st);
      cudaFree(scratch);
      cudaFree(scratch_ft);
      return false;
    }
  }
  bool ok = true;
  const cpx* traj = readvance ? scratch : w.MC;
  const double* ftr = readvance ? scratch_ft : w.Ft;
  const bool cached = !readvance && w.cached(3 * end, 3 * start);
  if (grad && cudaMemsetAsync(w.gacc, 0, sizeof(double) * (size_t)w.nseg * w.gstride, e.st) != cudaSuccess) {
    set_error(-1, "c_adjoint_exact: gradient accumulator reset failed");
    ok = false;
  }
  if (cudaMemcpyAsync(w.Ca, AC, sizeof(cpx) * csz * w.nseg, cudaMemcpyDeviceToDevice, e.st) != cudaSuccess ||
      cudaMemsetAsync(w.Ul, 0, sizeof(cpx) * w.usz * w.nseg, e.st) != cudaSuccess) {
    set_error(-1, "c_adjoint_exact: copy failed");
    ok = false;
  }
  ok = ok && set_step(e, w, start);
  GraphKey key = step_key(e, w, 'x');
  key.add(cached).add(traj).add(w.traj).add(src).add(grad).add(ftr);
  ok = ok && run_steps(e, w, key, start - end,
                       [&] { return enqueue_adjoint_exact_step(e, w, cached, traj, w.traj, src, ftr, grad); });
  if (ok && grad) {
    // per segment: dJ/dmeanU, and dJ/dRe as the blocks' parts summed in order
    std::vector<double> h((size_t)w.nseg * w.gstride);
    if (cudaMemcpyAsync(h.data(), w.gacc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, e.st) != cudaSuccess ||
        cudaStreamSynchronize(e.st) != cudaSuccess) {
      set_error(-1, "c_adjoint_exact: gradient read-back failed");
      ok = false;
    } else {
      w.grad.assign((size_t)2 * w.nseg, 0.0);
      for (int s = 0; s < w.nseg; ++s) {
        const double* r = h.data() + (size_t)s * w.gstride;
        double re = 0.0;
        for (int b = 1; b < w.gstride; ++b) re += r[b];
        w.grad[2 * s] = r[0];
        w.grad[2 * s + 1] = re;
      }
    }
  }
  if (ok) {
    // the tangent starts from IU = Recon(IC)
    SolveTArgs t{};
    t.grids = w.gdev;
    t.Ub = cb(w.Ul, w.usz);
    t.Cc = mb(w.Ca, w.csz);
    t.Hb = mb(nullptr, 0);
    t.k = 0;
    t.final_only = 1;
    t.ninst = w.nseg;
    t.status = nullptr;
    t.sdiv = 1;
    const cudaError_t le = launch_solve_T(e.T.g, t, e.st);
    if (le != cudaSuccess) {
      set_error(-1, "launch_solve_T: %s", cudaGetErrorString(le));
      ok = false;
    }
  }
  if (readvance) {
    cudaStreamSynchronize(e.st);
    cudaFree(scratch);
    cudaFree(scratch_ft);
  }
  return ok;
}

// ---------------------------------------------------------------------------
// helpers for the host-array API
// ---------------------------------------------------------------------------

static bool need_init(const char* fn) {
  if (!E) {
    set_error(-2, "%s called before c_init", fn);
    fprintf(stderr, "c_channel: %s called before c_init\n", fn);
    return false;
  }
  return true;
}

static void check_coef_dims(const Grid& g, int Nz_, int Nvar, int Ny_, int Nx_) {
  shape_assert(Nx_ == g.Nx / 2, "Nx_dup == Nx / 2");
  shape_assert(Ny_ == g.R, "Ny_dup == dimR");
  shape_assert(Nz_ == g.Nz, "Nz_dup == Nz");
  shape_assert(Nvar == 2, "Nvar_dup == 2");
}

static bool h2d(Engine& e, void* d, const void* h, size_t bytes) {
  CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, e.st));
  return true;
}

static bool d2h(Engine& e, void* h, const void* d, size_t bytes) {
  CK(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, e.st));
  CK(cudaStreamSynchronize(e.st));
  return true;
}

static double ddt_project_single(Engine& e, int i_step, cpx* IC_host) {
  Work& w = e.single;
  const Grid& g = e.T.g;
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, IC_host, bytes)) return NAN;
  DdtArgs d{w.MC, w.traj, nullptr, i_step, 1, 0, nullptr};
  ++g_launches;
  if (launch_ddt_diff(g, d, w.dC, e.st) != cudaSuccess) return NAN;
  if (!enqueue_spec2phys(e, w, cb(w.dC, w.csz), noslot(), w.Uprev, w.Pprev, 1)) return NAN;
  if (!enqueue_spec2phys(e, w, cb(w.io, w.csz), noslot(), w.Ul, w.Pl, 1)) return NAN;
  ++g_launches;
  if (launch_ddt_dots(g, cbd(w.Pprev, w.psz), cbd(w.Pl, w.psz), w.part, Work::kDotBlocks, 1, e.st) != cudaSuccess)
    return NAN;
  ++g_launches;
  if (launch_ddt_apply(g, w.part, Work::kDotBlocks, 1, cb(w.io, w.csz), noslot(), mb(w.io, w.csz), cb(w.dC, w.csz),
                       w.r, mb(nullptr, 0), 0.0, e.st) != cudaSuccess)
    return NAN;
  double r = NAN;
  if (!d2h(e, IC_host, w.io, bytes)) return NAN;
  if (!d2h(e, &r, w.r, sizeof(double))) return NAN;
  g_status = 0;
  g_msg.clear();
  return r;
}

// access for the allocation-free entry point (noalloc.cu)
bool engine_grid_stream(const Grid** g, cudaStream_t* st) {
  if (!E) return false;
  *g = &E->T.g;
  *st = E->st;
  return true;
}
void engine_set_error(int code, const char* msg) { set_error(code, "%s", msg); }
void engine_count_launches(int n) { g_launches += n; }
// the batch working set's shape (lss.cu)
bool engine_batch_shape(int* nseg, int* ntan, int* chain, size_t* csz, int* nsteps) {
  if (!E || !E->have_batch) return false;
  *nseg = E->batch.nseg;
  *ntan = E->batch.ntan;
  *chain = E->batch.chain;
  *csz = E->batch.csz;
  *nsteps = E->batch.nsteps;
  return true;
}
int engine_status() { return g_status; }
// stored trajectories for the statistics (stats.cu): MC (inc 0) or MIC (inc 1)
// of the single-trajectory working set (batch 0) or of the batch (batch 1)
bool engine_traj(int batch, int inc, const cpx** base, long long* traj_stride, int* nseg, int* nsteps) {
  if (!E || (batch && !E->have_batch)) return false;
  const Work& w = batch ? E->batch : E->single;
  *base = inc ? w.MIC : w.MC;
  *traj_stride = w.traj;
  *nseg = w.nseg;
  *nsteps = w.nsteps;
  return true;
}

// ddt_project of one vector per segment against the segment's own stored
// primal (channel/channel.c:704-780), in place; r[s] = num/den
static bool batch_ddt_project(Engine& e, Work& w, int i_step, cpx* V, double* r) {
  const Grid& g = e.T.g;
  DdtArgs d{w.MC, w.traj, nullptr, i_step, w.nseg, w.chain, w.gdev};
  LK(launch_ddt_diff(g, d, w.dC, e.st));
  if (!enqueue_spec2phys(e, w, cb(w.dC, w.csz), noslot(), w.Uprev, w.Pprev, w.nseg)) return false;
  if (!enqueue_spec2phys(e, w, cb(V, w.csz), noslot(), w.Ul, w.Pl, w.nseg)) return false;
  LK(launch_ddt_dots(g, cbd(w.Pprev, w.psz), cbd(w.Pl, w.psz), w.part, Work::kDotBlocks, w.nseg, e.st, w.gdev));
  LK(launch_ddt_apply(g, w.part, Work::kDotBlocks, w.nseg, cb(V, w.csz), noslot(), mb(V, w.csz), cb(w.dC, w.csz),
                      r ? r : w.r, mb(nullptr, 0), 0.0, e.st));
  return true;
}

}  // namespace chn

using namespace chn;

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int c_init(int Nx, int Ny, int Nz, double Lx, double Lz, double Re, double flux, double dt, int nsteps) {
  printf("Nx,Ny,Nz,Lx  |  Lz,dt,nsteps  |  flux,Re\n%d %d %d %f  |  %f %f %d |  %f %f\n", Nx, Ny, Nz, Lx, Lz, dt,
         nsteps, flux, Re);
  if (E) c_destroy();
  if (nsteps < 0) {
    set_error(1, "nsteps must be >= 0");
    return 1;
  }
  Engine* e = new Engine();
  if (!engine_streams_create(*e)) {
    set_error(-1, "no CUDA device available");
    engine_streams_destroy(*e);
    delete e;
    return 1;
  }
  if (!build_device_tables(e->T, Nx, Ny, Nz, Lx, Lz, Re, flux, dt)) {
    e->T.release();
    engine_streams_destroy(*e);
    delete e;
    return 1;
  }
  e->nsteps = nsteps;
  e->qy = e->T.ht.y;
  e->qw = e->T.ht.w;
  if (!e->single.create(e->T.g, 1, 1, nsteps, 0)) {
    e->single.release();
    e->T.release();
    engine_streams_destroy(*e);
    delete e;
    return 1;
  }
  e->last_ic.assign(e->single.csz, cpx{0.0, 0.0});
  E = e;
  g_status = 0;
  g_msg.clear();
  return 0;
}

void c_destroy(void) {
  if (!E) return;
  engine_sync(*E);
  E->single.release();
  if (E->have_batch) E->batch.release();
  if (E->host_mc) cudaFreeHost(E->host_mc);
  if (E->host_mic) cudaFreeHost(E->host_mic);
  E->T.release();
  engine_streams_destroy(*E);
  delete E;
  E = nullptr;
}

void c_primal(int ru_steps, chn_complex* C_given, int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup) {
  if (!need_init("c_primal")) return;
  Engine& e = *E;
  Work& w = e.single;
  const bool empty = (Nx_dup == 0 && Ny_dup == 0 && Nz_dup == 0 && Nvar_dup == 0);
  if (!empty) check_coef_dims(e.T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!empty && !h2d(e, w.io, C_given, bytes)) return;
  if (!op_primal(e, w, ru_steps, empty ? nullptr : w.io)) return;
  if (!collect_status(e, w)) return;
  if (g_status & ST_CFL) printf("Pass1 failure\n");
  if (!empty) d2h(e, C_given, w.Cp, bytes);
}

void c_tangent(int start_step, int end_step, chn_complex* IC_given, int Nz_dup, int Nvar_dup, int Ny_dup,
               int Nx_dup, int inhomo) {
  c_tangent_forcing(start_step, end_step, IC_given, Nz_dup, Nvar_dup, Ny_dup, Nx_dup, inhomo ? 1 : 0);
}

void c_tangent_forcing(int start_step, int end_step, chn_complex* IC_given, int Nz_dup, int Nvar_dup, int Ny_dup,
                       int Nx_dup, int forcing) {
  if (!need_init("c_tangent")) return;
  Engine& e = *E;
  Work& w = e.single;
  check_coef_dims(e.T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  shape_assert(end_step > start_step, "end_step > start_step");
  shape_assert(start_step >= 0, "start_step >= 0");
  shape_assert(end_step <= e.nsteps, "end_step <= nsteps");
  shape_assert(IC_given != nullptr, "IC_given != 0");
  shape_assert(forcing >= 0 && forcing <= 3, "0 <= forcing <= 3");
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, IC_given, bytes)) return;
  Forcing f;
  f.forced = forcing == 1 ? 1u : 0u;
  f.re2 = forcing == 2 ? 1u : 0u;
  f.re3 = forcing == 3 ? 1u : 0u;
  if (!op_forward(e, w, start_step, end_step, nullptr, w.io, f, false)) return;
  if (!collect_status(e, w)) return;
  if (g_status & ST_CFL) printf("Pass1 failure\n");
  d2h(e, IC_given, w.Ct, bytes);
  memcpy(e.last_ic.data(), IC_given, bytes);
}

void c_adjoint(int start_step, int end_step, chn_complex* AC_given, int Nz_dup, int Nvar_dup, int Ny_dup,
               int Nx_dup, int inhomo, double strength) {
  (void)inhomo;  // unused by the reference too (channel/channel.c:596-696)
  if (!need_init("c_adjoint")) return;
  Engine& e = *E;
  Work& w = e.single;
  check_coef_dims(e.T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  shape_assert(end_step < start_step, "end_step < start_step");
  shape_assert(end_step >= 0, "end_step >= 0");
  shape_assert(start_step <= e.nsteps, "start_step <= nsteps");
  shape_assert(AC_given != nullptr, "AC_given != 0");
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, AC_given, bytes)) return;
  if (!op_adjoint(e, w, start_step, end_step, w.io, strength)) return;
  if (!collect_status(e, w)) return;
  d2h(e, AC_given, w.Ca, bytes);
}

void c_adjoint_exact(int start_step, int end_step, chn_complex* AC_given, int Nz_dup, int Nvar_dup, int Ny_dup,
                     int Nx_dup) {
  if (!need_init("c_adjoint_exact")) return;
  Engine& e = *E;
  Work& w = e.single;
  check_coef_dims(e.T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  shape_assert(end_step < start_step, "end_step < start_step");
  shape_assert(end_step >= 0, "end_step >= 0");
  shape_assert(start_step <= e.nsteps, "start_step <= nsteps");
  shape_assert(AC_given != nullptr, "AC_given != 0");
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, AC_given, bytes)) return;
  if (!op_adjoint_exact(e, w, start_step, end_step, w.io)) return;
  if (!collect_status(e, w)) return;
  d2h(e, AC_given, w.Ca, bytes);
}

void c_adjoint_exact_source(int start_step, int end_step, chn_complex* AC_given, const chn_complex* src,
                            int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup) {
  if (!need_init("c_adjoint_exact_source")) return;
  Engine& e = *E;
  Work& w = e.single;
  check_coef_dims(e.T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  shape_assert(end_step < start_step, "end_step < start_step");
  shape_assert(end_step >= 0, "end_step >= 0");
  shape_assert(start_step <= e.nsteps, "start_step <= nsteps");
  shape_assert(AC_given != nullptr && src != nullptr, "AC_given != 0 && src != 0");
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, AC_given, bytes) || !h2d(e, w.src, src, bytes)) return;
  if (!op_adjoint_exact(e, w, start_step, end_step, w.io, w.src)) return;
  if (!collect_status(e, w)) return;
  d2h(e, AC_given, w.Ca, bytes);
}

int c_adjoint_exact_grad(int start_step, int end_step, chn_complex* AC_given, const chn_complex* src,
                         double* grad) {
  if (!need_init("c_adjoint_exact_grad")) return g_status;
  Engine& e = *E;
  Work& w = e.single;
  if (!(end_step < start_step && end_step >= 0 && start_step <= e.nsteps) || !AC_given || !grad) {
    set_error(-4, "c_adjoint_exact_grad: need 0 <= end < start <= nsteps, the state array and grad[2]");
    return -4;
  }
  const size_t bytes = sizeof(cpx) * w.csz;
  if (!h2d(e, w.io, AC_given, bytes)) return -1;
  if (src && !h2d(e, w.src, src, bytes)) return -1;
  if (!op_adjoint_exact(e, w, start_step, end_step, w.io, src ? w.src : nullptr, true)) return g_status;
  if (!collect_status(e, w)) return g_status;
  if (!d2h(e, AC_given, w.Ca, bytes)) return -1;
  grad[0] = w.grad[0];
  grad[1] = w.grad[1];
  return g_status;
}

double c_ddt_project(int i_step, chn_complex* IC_given, int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup) {
  if (!need_init("c_ddt_project")) return NAN;
  check_coef_dims(E->T.g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  return ddt_project_single(*E, i_step, reinterpret_cast<cpx*>(IC_given));
}

static void get_traj(bool inc, int i_step, chn_complex** ptr, int* Nz_ptr, int* Nvar_ptr, int* Ny_ptr, int* Nx_ptr) {
  Engine& e = *E;
  Work& w = e.single;
  shape_assert(i_step >= 0 && i_step <= e.nsteps, "i_step >= 0 && i_step <= nsteps");
  cpx*& mirror = inc ? e.host_mic : e.host_mc;
  if (!mirror) {
    if (cudaMallocHost(&mirror, sizeof(cpx) * w.csz * (size_t)(e.nsteps + 1)) != cudaSuccess) {
      set_error(-1, "cudaMallocHost failed for the trajectory mirror");
      *ptr = nullptr;
      return;
    }
  }
  cpx* dst = mirror + (size_t)i_step * w.csz;
  const cpx* src = (inc ? w.MIC : w.MC) + (size_t)3 * i_step * w.csz;
  d2h(e, dst, src, sizeof(cpx) * w.csz);
  *ptr = reinterpret_cast<chn_complex*>(dst);
  *Nz_ptr = e.T.g.Nz;
  *Nvar_ptr = 2;
  *Ny_ptr = e.T.g.R;
  *Nx_ptr = e.T.g.Nx / 2;
}

void c_getsoln(int i_step, chn_complex** MC_ptr, int* Nz_ptr, int* Nvar_ptr, int* Ny_ptr, int* Nx_ptr) {
  if (!need_init("c_getsoln")) return;
  get_traj(false, i_step, MC_ptr, Nz_ptr, Nvar_ptr, Ny_ptr, Nx_ptr);
}

void c_getincresoln(int i_step, chn_complex** MIC_ptr, int* Nz_ptr, int* Nvar_ptr, int* Ny_ptr, int* Nx_ptr) {
  if (!need_init("c_getincresoln")) return;
  get_traj(true, i_step, MIC_ptr, Nz_ptr, Nvar_ptr, Ny_ptr, Nx_ptr);
}

void c_spec2phys(chn_complex* C_ptr, int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup, double* flow_ptr, int Nd_flow,
                 int Nx_flow, int Ny_flow, int Nz_flow) {
  if (!need_init("c_spec2phys")) return;
  Engine& e = *E;
  Work& w = e.single;
  const Grid& g = e.T.g;
  check_coef_dims(g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  shape_assert(Nd_flow == 3, "Nd_flow == 3");
  shape_assert(Nx_flow == 3 * g.Nx / 2, "Nx_flow == 3 * Nx / 2");
  shape_assert(Ny_flow == g.Q, "Ny_flow == qpts");
  shape_assert(Nz_flow == 3 * g.Nz / 2, "Nz_flow == 3 * Nz / 2");
  if (!h2d(e, w.io, C_ptr, sizeof(cpx) * w.csz)) return;
  if (!enqueue_spec2phys(e, w, cb(w.io, w.csz), noslot(), w.Ul, w.Pl, 1)) return;
  ++g_launches;
  if (launch_flow_out(g, w.Pl, w.flow, e.st) != cudaSuccess) return;
  d2h(e, flow_ptr, w.flow, sizeof(double) * 3 * (size_t)g.Q * plane_size(g));
  g_status = 0;
  g_msg.clear();
}

// Raw solution container: "SCHNRAW1", int32 Nx, Ny, Nz, 0, double dt, 1/Re,
// mpg, then alpha, beta, ialpha, ibeta as [dimR][Nz][Nx/2] {re, im} doubles
// (the datasets of channel/channel.c:889-1028).
void c_save_solution(char* filename, chn_complex* C_ptr, int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup) {
  if (!need_init("c_save_solution")) return;
  Engine& e = *E;
  const Grid& g = e.T.g;
  check_coef_dims(g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  FILE* f = fopen(filename, "wb");
  if (!f) {
    set_error(-3, "cannot open %s for writing", filename);
    return;
  }
  const char magic[8] = {'S', 'C', 'H', 'N', 'R', 'A', 'W', '1'};
  const int dims[4] = {g.Nx, g.Ny, g.Nz, 0};
  const double sc[3] = {g.dt, g.re, 0.0};
  fwrite(magic, 1, 8, f);
  fwrite(dims, sizeof(int), 4, f);
  fwrite(sc, sizeof(double), 3, f);
  const cpx* C = reinterpret_cast<const cpx*>(C_ptr);
  const cpx* IC = e.last_ic.data();
  for (int src = 0; src < 2; ++src)
    for (int v = 0; v < 2; ++v)
      for (int r = 0; r < g.R; ++r)
        for (int z = 0; z < g.Nz; ++z)
          for (int x = 0; x < g.X; ++x) {
            const cpx* A = src ? IC : C;
            fwrite(&A[(((size_t)z * 2 + v) * g.R + r) * g.X + x], sizeof(cpx), 1, f);
          }
  fclose(f);
  g_status = 0;
  g_msg.clear();
}

void c_read_solution(char* filename, chn_complex* C_ptr, int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup) {
  if (!need_init("c_read_solution")) return;
  Engine& e = *E;
  const Grid& g = e.T.g;
  check_coef_dims(g, Nz_dup, Nvar_dup, Ny_dup, Nx_dup);
  FILE* f = fopen(filename, "rb");
  shape_assert(f != nullptr, "solution file opens");
  char magic[8];
  int dims[4];
  double sc[3];
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "SCHNRAW1", 8) == 0 && fread(dims, sizeof(int), 4, f) == 4 &&
            fread(sc, sizeof(double), 3, f) == 3 && dims[0] == g.Nx && dims[1] == g.Ny && dims[2] == g.Nz;
  shape_assert(ok, "solution file header matches the grid");
  cpx* C = reinterpret_cast<cpx*>(C_ptr);
  for (int src = 0; src < 2; ++src)
    for (int v = 0; v < 2; ++v)
      for (int r = 0; r < g.R; ++r)
        for (int z = 0; z < g.Nz; ++z)
          for (int x = 0; x < g.X; ++x) {
            cpx* A = src ? e.last_ic.data() : C;
            ok = ok && fread(&A[(((size_t)z * 2 + v) * g.R + r) * g.X + x], sizeof(cpx), 1, f) == 1;
          }
  fclose(f);
  shape_assert(ok, "solution file complete");
  g_status = 0;
  g_msg.clear();
}

void c_quad(double** y_ptr, int* qpts_ptr1, double** w_ptr, int* qpts_ptr2) {
  if (!need_init("c_quad")) return;
  *y_ptr = E->qy.data();
  *w_ptr = E->qw.data();
  *qpts_ptr1 = *qpts_ptr2 = E->T.g.Q;
}

int c_qpts(void) { return E ? E->T.g.Q : 0; }
int c_dimR(void) { return E ? E->T.g.R : 0; }
int c_dimQ(void) { return E ? E->T.g.D : 0; }
int c_Nx(void) { return E ? E->T.g.Nx : 0; }
int c_Nz(void) { return E ? E->T.g.Nz : 0; }
int c_nsteps(void) { return E ? E->nsteps : 0; }

int c_last_error(void) { return g_status; }
const char* c_last_error_message(void) { return g_msg.c_str(); }
double c_last_cfl(void) { return g_cfl; }

int c_batch_init(int nseg, int ntan, int couple) {
  if (!need_init("c_batch_init")) return -2;
  return c_batch_init_steps(nseg, ntan, couple, E->nsteps);
}

int c_batch_init_steps(int nseg, int ntan, int couple, int nsteps) {
  if (!need_init("c_batch_init_steps")) return -2;
  if (nseg <= 0 || ntan < 0 || ntan > 32 || (ntan > 0 && (couple < 0 || couple >= ntan)) || nsteps < 0) {
    set_error(-4, "c_batch_init: need nseg > 0, 0 <= ntan <= 32, 0 <= couple < ntan, nsteps >= 0");
    return -4;
  }
  Engine& e = *E;
  if (e.have_batch) {
    engine_sync(e);
    e.batch.release();
    e.have_batch = false;
  }
  if (!e.batch.create(e.T.g, nseg, ntan, nsteps, couple)) {
    e.batch.release();
    return g_status;
  }
  e.have_batch = true;
  g_tune_report.clear();
  if (!tune_inputs(e, e.batch, true) || !autotune_transforms(e, e.batch) || !autotune_solve(e, e.batch) ||
      !autotune_fixed(e, e.batch) || !tune_inputs(e, e.batch, false))
    return g_status;
  g_status = 0;
  return 0;
}

int c_batch_destroy(void) {
  if (!E || !E->have_batch) return 0;
  engine_sync(*E);
  E->batch.release();
  E->have_batch = false;
  return 0;
}

static bool batch_ready(const char* fn) {
  if (!need_init(fn)) return false;
  if (!E->have_batch) {
    set_error(-4, "%s: call c_batch_init first", fn);
    return false;
  }
  return true;
}

// batched tangents: inhomo[t] 0 none, 1 mean flux, 2 Re (reference forcing), 3 Re (exact)
static Forcing mask_of(const int* inhomo, int ntan) {
  Forcing f;
  for (int t = 0; t < ntan; ++t) {
    const int v = inhomo ? inhomo[t] : 0;
    if (v == 2) f.re2 |= 1u << t;
    else if (v == 3) f.re3 |= 1u << t;
    else if (v) f.forced |= 1u << t;
  }
  return f;
}

int c_batch_primal_dev(int ru_steps, chn_complex* C) {
  if (!batch_ready("c_batch_primal_dev")) return g_status;
  Work& w = E->batch;
  if (!op_primal(*E, w, ru_steps, reinterpret_cast<cpx*>(C))) return g_status;
  if (C && cudaMemcpyAsync(C, w.Cp, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  return collect_status(*E, w) ? g_status : -1;
}

int c_batch_tangent_dev(int start_step, int end_step, chn_complex* IC, const int* inhomo) {
  if (!batch_ready("c_batch_tangent_dev")) return g_status;
  Work& w = E->batch;
  if (!(end_step > start_step && start_step >= 0 && end_step <= E->batch.nsteps) || w.ntan == 0) {
    set_error(-4, "c_batch_tangent: need 0 <= start < end <= nsteps and ntan > 0");
    return -4;
  }
  if (!op_forward(*E, w, start_step, end_step, nullptr, reinterpret_cast<cpx*>(IC), mask_of(inhomo, w.ntan), false))
    return g_status;
  if (cudaMemcpyAsync(IC, w.Ct, sizeof(cpx) * w.csz * w.nseg * w.ntan, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  return collect_status(*E, w) ? g_status : -1;
}

int c_batch_forward_dev(int start_step, int end_step, chn_complex* C, chn_complex* IC, const int* inhomo) {
  if (!batch_ready("c_batch_forward_dev")) return g_status;
  Work& w = E->batch;
  if (!(end_step > start_step && start_step >= 0 && end_step <= E->batch.nsteps)) {
    set_error(-4, "c_batch_forward: need 0 <= start < end <= nsteps");
    return -4;
  }
  if (!op_forward(*E, w, start_step, end_step, reinterpret_cast<cpx*>(C), reinterpret_cast<cpx*>(IC),
                  mask_of(inhomo, w.ntan), true))
    return g_status;
  if (C && cudaMemcpyAsync(C, w.Cp, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  if (w.ntan > 0 &&
      cudaMemcpyAsync(IC, w.Ct, sizeof(cpx) * w.csz * w.nseg * w.ntan, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  return collect_status(*E, w) ? g_status : -1;
}

int c_batch_adjoint_dev(int start_step, int end_step, chn_complex* AC, double strength) {
  if (!batch_ready("c_batch_adjoint_dev")) return g_status;
  Work& w = E->batch;
  if (!(end_step < start_step && end_step >= 0 && start_step <= E->batch.nsteps)) {
    set_error(-4, "c_batch_adjoint: need 0 <= end < start <= nsteps");
    return -4;
  }
  if (!op_adjoint(*E, w, start_step, end_step, reinterpret_cast<cpx*>(AC), strength)) return g_status;
  if (cudaMemcpyAsync(AC, w.Ca, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  return collect_status(*E, w) ? g_status : -1;
}

int c_batch_adjoint_exact_source_dev(int start_step, int end_step, chn_complex* AC, const chn_complex* src) {
  if (!batch_ready("c_batch_adjoint_exact_dev")) return g_status;
  Work& w = E->batch;
  if (!(end_step < start_step && end_step >= 0 && start_step <= E->batch.nsteps) || !AC) {
    set_error(-4, "c_batch_adjoint_exact: need 0 <= end < start <= nsteps and the state array");
    return -4;
  }
  if (!op_adjoint_exact(*E, w, start_step, end_step, reinterpret_cast<cpx*>(AC),
                        reinterpret_cast<const cpx*>(src)))
    return g_status;
  if (cudaMemcpyAsync(AC, w.Ca, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  return collect_status(*E, w) ? g_status : -1;
}

int c_batch_adjoint_exact_dev(int start_step, int end_step, chn_complex* AC) {
  return c_batch_adjoint_exact_source_dev(start_step, end_step, AC, nullptr);
}

int c_batch_adjoint_exact_grad_dev(int start_step, int end_step, chn_complex* AC, const chn_complex* src,
                                   double* grad) {
  if (!batch_ready("c_batch_adjoint_exact_grad_dev")) return g_status;
  Work& w = E->batch;
  if (!(end_step < start_step && end_step >= 0 && start_step <= w.nsteps) || !AC || !grad) {
    set_error(-4, "c_batch_adjoint_exact_grad_dev: need 0 <= end < start <= nsteps, the state array and grad");
    return -4;
  }
  if (!op_adjoint_exact(*E, w, start_step, end_step, reinterpret_cast<cpx*>(AC), reinterpret_cast<const cpx*>(src),
                        true))
    return g_status;
  if (cudaMemcpyAsync(AC, w.Ca, sizeof(cpx) * w.csz * w.nseg, cudaMemcpyDeviceToDevice, E->st) != cudaSuccess)
    return -1;
  if (!collect_status(*E, w)) return -1;
  std::copy(w.grad.begin(), w.grad.end(), grad);
  return g_status;
}

// host-array variants: staged through the working set's own device buffers
// (dC holds the primal states, io the tangent / adjoint states)
int c_batch_primal(int ru_steps, chn_complex* C) {
  if (!batch_ready("c_batch_primal")) return g_status;
  Work& w = E->batch;
  const size_t bytes = sizeof(cpx) * w.csz * w.nseg;
  if (C && !h2d(*E, w.dC, C, bytes)) return -1;
  const int rc = c_batch_primal_dev(ru_steps, C ? reinterpret_cast<chn_complex*>(w.dC) : nullptr);
  if (C && !d2h(*E, C, w.dC, bytes)) return -1;
  return rc;
}

int c_batch_tangent(int start_step, int end_step, chn_complex* IC, const int* inhomo) {
  if (!batch_ready("c_batch_tangent")) return g_status;
  Work& w = E->batch;
  const size_t bytes = sizeof(cpx) * w.csz * w.nseg * (w.ntan > 0 ? w.ntan : 1);
  if (!h2d(*E, w.io, IC, bytes)) return -1;
  const int rc = c_batch_tangent_dev(start_step, end_step, reinterpret_cast<chn_complex*>(w.io), inhomo);
  if (!d2h(*E, IC, w.io, bytes)) return -1;
  return rc;
}

int c_batch_forward(int start_step, int end_step, chn_complex* C, chn_complex* IC, const int* inhomo) {
  if (!batch_ready("c_batch_forward")) return g_status;
  Work& w = E->batch;
  const size_t bc = sizeof(cpx) * w.csz * w.nseg;
  const size_t bt = sizeof(cpx) * w.csz * w.nseg * w.ntan;
  if (!h2d(*E, w.dC, C, bc)) return -1;
  if (bt && !h2d(*E, w.io, IC, bt)) return -1;
  const int rc = c_batch_forward_dev(start_step, end_step, reinterpret_cast<chn_complex*>(w.dC),
                                     reinterpret_cast<chn_complex*>(w.io), inhomo);
  if (!d2h(*E, C, w.dC, bc)) return -1;
  if (bt && !d2h(*E, IC, w.io, bt)) return -1;
  return rc;
}

int c_batch_adjoint(int start_step, int end_step, chn_complex* AC, double strength) {
  if (!batch_ready("c_batch_adjoint")) return g_status;
  Work& w = E->batch;
  const size_t bytes = sizeof(cpx) * w.csz * w.nseg;
  if (!h2d(*E, w.io, AC, bytes)) return -1;
  const int rc = c_batch_adjoint_dev(start_step, end_step, reinterpret_cast<chn_complex*>(w.io), strength);
  if (!d2h(*E, AC, w.io, bytes)) return -1;
  return rc;
}

int c_batch_adjoint_exact(int start_step, int end_step, chn_complex* AC) {
  if (!batch_ready("c_batch_adjoint_exact")) return g_status;
  Work& w = E->batch;
  if (!AC) {
    set_error(-4, "c_batch_adjoint_exact: null state array");
    return -4;
  }
  const size_t bytes = sizeof(cpx) * w.csz * w.nseg;
  if (!h2d(*E, w.io, AC, bytes)) return -1;
  const int rc = c_batch_adjoint_exact_dev(start_step, end_step, reinterpret_cast<chn_complex*>(w.io));
  if (!d2h(*E, AC, w.io, bytes)) return -1;
  return rc;
}

int c_batch_set_chain(int window_steps) {
  if (!batch_ready("c_batch_set_chain")) return g_status;
  if (window_steps < 0 || window_steps > E->batch.nsteps) {
    set_error(-4, "c_batch_set_chain: need 0 <= window_steps <= nsteps");
    return -4;
  }
  E->batch.chain = window_steps;
  g_status = 0;
  return 0;
}

int c_batch_ddt_project_dev(int i_step, chn_complex* V, double* r) {
  if (!batch_ready("c_batch_ddt_project_dev")) return g_status;
  if (i_step < 0 || i_step > E->batch.nsteps || !V) {
    set_error(-4, "c_batch_ddt_project: need 0 <= i_step <= nsteps and a vector array");
    return -4;
  }
  g_status = 0;
  return batch_ddt_project(*E, E->batch, i_step, reinterpret_cast<cpx*>(V), r) ? 0 : g_status;
}

int c_batch_ddt_project(int i_step, chn_complex* V, double* r) {
  if (!batch_ready("c_batch_ddt_project")) return g_status;
  Work& w = E->batch;
  const size_t bytes = sizeof(cpx) * w.csz * w.nseg;
  if (!V || !h2d(*E, w.io, V, bytes)) return -4;
  const int rc = c_batch_ddt_project_dev(i_step, reinterpret_cast<chn_complex*>(w.io), nullptr);
  if (rc != 0) return rc;
  if (!d2h(*E, V, w.io, bytes)) return -1;
  if (r && !d2h(*E, r, w.r, sizeof(double) * w.nseg)) return -1;
  return 0;
}

int c_batch_getsoln(int seg, int i_step, chn_complex* out) {
  if (!batch_ready("c_batch_getsoln")) return g_status;
  Work& w = E->batch;
  if (seg < 0 || seg >= w.nseg || i_step < 0 || i_step > E->batch.nsteps) return -4;
  return d2h(*E, out, w.MC + (size_t)seg * w.traj + (size_t)3 * i_step * w.csz, sizeof(cpx) * w.csz) ? 0 : -1;
}

int c_batch_getincresoln(int seg, int i_step, chn_complex* out) {
  if (!batch_ready("c_batch_getincresoln")) return g_status;
  Work& w = E->batch;
  if (seg < 0 || seg >= w.nseg || i_step < 0 || i_step > E->batch.nsteps) return -4;
  return d2h(*E, out, w.MIC + (size_t)seg * w.traj + (size_t)3 * i_step * w.csz, sizeof(cpx) * w.csz) ? 0 : -1;
}

// ---------------------------------------------------------------------------
// Uneven batches: n instances, each with its own grid, Re, flux and dt, all
// advanced by the same launches (kernels in their MULTI form read their
// instance's grid from a device array; buffers are padded to the largest
// grid).  Host arrays are packed: instance after instance, each in the
// reference layout [Nz][2][Ny-2][Nx/2] of its own grid (tangents: the ntan
// arrays of an instance one after another).
// ---------------------------------------------------------------------------
}  // extern "C"

namespace chn {
struct Multi {
  Engine e;                    // e.T.g: launch sizes of the largest grid; e.batch: the working set
  std::vector<DevTables> tabs; // per instance
  std::vector<size_t> csz;     // per-instance coefficient elements
  std::vector<size_t> off;     // packed offsets
  Grid* gdev = nullptr;
  void release() {
    engine_sync(e);
    if (e.have_batch) e.batch.release();
    for (DevTables& t : tabs) t.release();
    tabs.clear();
    if (gdev) cudaFree(gdev);
    gdev = nullptr;
    engine_streams_destroy(e);
  }
};
static Multi* MX = nullptr;

static bool multi_ready(const char* fn) {
  if (!MX) {
    set_error(-2, "%s called before c_multi_init", fn);
    return false;
  }
  return true;
}

// packed host <-> padded device, one copy per instance
static bool multi_h2d(cpx* dev, const chn_complex* host, int per) {
  Multi& m = *MX;
  Work& w = m.e.batch;
  CK(cudaMemsetAsync(dev, 0, sizeof(cpx) * w.csz * (size_t)w.nseg * per, m.e.st));
  for (int i = 0; i < w.nseg; ++i)
    for (int t = 0; t < per; ++t)
      CK(cudaMemcpyAsync(dev + ((size_t)i * per + t) * w.csz,
                         reinterpret_cast<const cpx*>(host) + m.off[i] * per + (size_t)t * m.csz[i],
                         sizeof(cpx) * m.csz[i], cudaMemcpyHostToDevice, m.e.st));
  return true;
}

static bool multi_d2h(chn_complex* host, const cpx* dev, int per) {
  Multi& m = *MX;
  Work& w = m.e.batch;
  for (int i = 0; i < w.nseg; ++i)
    for (int t = 0; t < per; ++t)
      CK(cudaMemcpyAsync(reinterpret_cast<cpx*>(host) + m.off[i] * per + (size_t)t * m.csz[i],
                         dev + ((size_t)i * per + t) * w.csz, sizeof(cpx) * m.csz[i], cudaMemcpyDeviceToHost,
                         m.e.st));
  CK(cudaStreamSynchronize(m.e.st));
  return true;
}
}  // namespace chn

extern "C" {

int c_multi_destroy(void) {
  if (!MX) return 0;
  MX->release();
  delete MX;
  MX = nullptr;
  return 0;
}

int c_multi_init(int n, const int* Nx, const int* Ny, const int* Nz, const double* Lx, const double* Lz,
                 const double* Re, const double* flux, const double* dt, int nsteps, int ntan, int couple) {
  c_multi_destroy();
  if (n <= 0 || nsteps < 0 || ntan < 0 || ntan > 32 || (ntan > 0 && (couple < 0 || couple >= ntan)) || !Nx ||
      !Ny || !Nz || !Lx || !Lz || !Re || !flux || !dt) {
    set_error(-4, "c_multi_init: need n > 0, nsteps >= 0, 0 <= ntan <= 32, 0 <= couple < ntan and all arrays");
    return -4;
  }
  Multi* m = new Multi();
  MX = m;
  if (!engine_streams_create(m->e)) {
    set_error(-1, "no CUDA device available");
    c_multi_destroy();
    return -1;
  }
  m->tabs.resize(n);
  size_t acc = 0;
  int big = 0;
  for (int i = 0; i < n; ++i) {
    if (!build_device_tables(m->tabs[i], Nx[i], Ny[i], Nz[i], Lx[i], Lz[i], Re[i], flux[i], dt[i])) {
      const int rc = g_status ? g_status : -1;
      c_multi_destroy();
      return rc;
    }
    const size_t c = coef_size(m->tabs[i].g);
    if (c > coef_size(m->tabs[big].g)) big = i;
    m->csz.push_back(c);
    m->off.push_back(acc);
    acc += c;
  }
  // launch sizes: the maxima over the instances (tables of the largest one)
  Grid gmax = m->tabs[big].g;
  for (int i = 0; i < n; ++i) {
    const Grid& g = m->tabs[i].g;
    gmax.Nx = std::max(gmax.Nx, g.Nx); gmax.Ny = std::max(gmax.Ny, g.Ny); gmax.Nz = std::max(gmax.Nz, g.Nz);
    gmax.X = std::max(gmax.X, g.X); gmax.Q = std::max(gmax.Q, g.Q); gmax.R = std::max(gmax.R, g.R);
    gmax.D = std::max(gmax.D, g.D); gmax.pz = std::max(gmax.pz, g.pz); gmax.px = std::max(gmax.px, g.px);
    gmax.Qh = std::max(gmax.Qh, g.Qh);
    gmax.general = std::max(gmax.general, g.general);
    gmax.tc = std::min(gmax.tc, g.tc);
    gmax.tci = std::min(gmax.tci, g.tci);
    gmax.tcf = std::min(gmax.tcf, g.tcf);
  }
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const char* force = getenv("CHN_SPLIT_TRANSFORMS");
  gmax.split = (!fused_transforms_fit(gmax, optin) || (force && force[0] == '1')) ? 1 : 0;
  if (!phys_tc_fits(gmax, optin)) gmax.tci = 0;
  if (!fwd_tc_plan(gmax, optin, gmax.fwdpb, gmax.fxch)) gmax.tcf = 0;
  if (solve_smem_bytes(gmax) > (size_t)optin) {
    set_error(1, "c_multi_init: the largest grid needs more shared memory than the device has");
    c_multi_destroy();
    return 1;
  }
  std::vector<Grid> gs(n);
  for (int i = 0; i < n; ++i) {
    gs[i] = m->tabs[i].g;
    gs[i].split = gmax.split;
    gs[i].tc = gmax.tc;
    gs[i].tci = gmax.tci;
    gs[i].tcf = gmax.tcf;
    gs[i].tcminb = gmax.tcminb;
    gs[i].stile = gmax.stile;
    gs[i].sthr = gmax.sthr;
    gs[i].adjpb = gmax.adjpb;
    gs[i].fwdpb = gmax.fwdpb;
    gs[i].fxch = gmax.fxch;
    gs[i].prodb = 0;  // uneven batches keep the plan's build
  }
  if (cudaMalloc(&m->gdev, sizeof(Grid) * n) != cudaSuccess ||
      cudaMemcpy(m->gdev, gs.data(), sizeof(Grid) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error(-1, "c_multi_init: device allocation failed");
    c_multi_destroy();
    return -1;
  }
  m->e.T.g = gmax;
  m->e.nsteps = nsteps;
  if (!m->e.batch.create(gmax, n, ntan, nsteps, couple)) {
    const int rc = g_status ? g_status : -1;
    c_multi_destroy();
    return rc;
  }
  m->e.batch.gdev = m->gdev;
  m->e.have_batch = true;
  g_tune_report.clear();
  if (!tune_inputs(m->e, m->e.batch, true) || !autotune_transforms(m->e, m->e.batch) ||
      !autotune_solve(m->e, m->e.batch) || !autotune_fixed(m->e, m->e.batch) || !tune_inputs(m->e, m->e.batch, false)) {
    const int rc = g_status ? g_status : -1;
    c_multi_destroy();
    return rc;
  }
  g_status = 0;
  g_msg.clear();
  return 0;
}

long long c_multi_coef_elems(int i) {
  if (!MX || i < 0 || i >= (int)MX->csz.size()) return -1;
  return (long long)MX->csz[i];
}

int c_multi_primal(int ru_steps, chn_complex* C) {
  if (!multi_ready("c_multi_primal")) return g_status;
  if (!C) {
    set_error(-4, "c_multi_primal: an uneven batch starts from given states");
    return -4;
  }
  Work& w = MX->e.batch;
  if (!multi_h2d(w.dC, C, 1)) return -1;
  if (!op_primal(MX->e, w, ru_steps, w.dC)) return g_status;
  if (!multi_d2h(C, w.Cp, 1)) return -1;
  return collect_status(MX->e, w) ? g_status : -1;
}

int c_multi_forward(int start_step, int end_step, chn_complex* C, chn_complex* IC, const int* inhomo) {
  if (!multi_ready("c_multi_forward")) return g_status;
  Work& w = MX->e.batch;
  if (!(end_step > start_step && start_step >= 0 && end_step <= w.nsteps) || !C || (w.ntan > 0 && !IC)) {
    set_error(-4, "c_multi_forward: need 0 <= start < end <= nsteps and the state arrays");
    return -4;
  }
  if (!multi_h2d(w.dC, C, 1)) return -1;
  if (w.ntan > 0 && !multi_h2d(w.io, IC, w.ntan)) return -1;
  if (!op_forward(MX->e, w, start_step, end_step, w.dC, w.io, mask_of(inhomo, w.ntan), true)) return g_status;
  if (!multi_d2h(C, w.Cp, 1)) return -1;
  if (w.ntan > 0 && !multi_d2h(IC, w.Ct, w.ntan)) return -1;
  return collect_status(MX->e, w) ? g_status : -1;
}

int c_multi_adjoint(int start_step, int end_step, chn_complex* AC, double strength) {
  if (!multi_ready("c_multi_adjoint")) return g_status;
  Work& w = MX->e.batch;
  if (!(end_step < start_step && end_step >= 0 && start_step <= w.nsteps) || !AC) {
    set_error(-4, "c_multi_adjoint: need 0 <= end < start <= nsteps and the state array");
    return -4;
  }
  if (!multi_h2d(w.io, AC, 1)) return -1;
  if (!op_adjoint(MX->e, w, start_step, end_step, w.io, strength)) return g_status;
  if (!multi_d2h(AC, w.Ca, 1)) return -1;
  return collect_status(MX->e, w) ? g_status : -1;
}

int c_multi_adjoint_exact(int start_step, int end_step, chn_complex* AC) {
  if (!multi_ready("c_multi_adjoint_exact")) return g_status;
  Work& w = MX->e.batch;
  if (!(end_step < start_step && end_step >= 0 && start_step <= w.nsteps) || !AC) {
    set_error(-4, "c_multi_adjoint_exact: need 0 <= end < start <= nsteps and the state array");
    return -4;
  }
  if (!multi_h2d(w.io, AC, 1)) return -1;
  if (!op_adjoint_exact(MX->e, w, start_step, end_step, w.io)) return g_status;
  if (!multi_d2h(AC, w.Ca, 1)) return -1;
  return collect_status(MX->e, w) ? g_status : -1;
}

int c_multi_getsoln(int i, int i_step, chn_complex* out) {
  if (!multi_ready("c_multi_getsoln")) return g_status;
  Work& w = MX->e.batch;
  if (i < 0 || i >= w.nseg || i_step < 0 || i_step > w.nsteps || !out) return -4;
  return d2h(MX->e, out, w.MC + (size_t)i * w.traj + (size_t)3 * i_step * w.csz, sizeof(cpx) * MX->csz[i]) ? 0
                                                                                                            : -1;
}

void* c_stream(void) { return E ? (void*)E->st : nullptr; }

// Average device time (ms, CUDA events on the library stream) of one launch
// of one kernel of the batched forward substage 0, on the current batch
// buffers (run c_batch_forward first so they hold a real state).
// which: 0 reconstruct (primal + tangents), 1 physical transforms (primal +
// tangents), 2 tangent products, 3 tangent solve, 4 adjoint products.
double c_batch_kernel_ms(int which, int reps) {
  if (!E || !E->have_batch || reps <= 0) return -1.0;
  Engine& e = *E;
  Work& w = e.batch;
  const Grid& g = e.T.g;
  const int nt = w.nseg * w.ntan;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int zero = 0;
  cudaMemcpyAsync(w.step, &zero, sizeof(int), cudaMemcpyHostToDevice, e.st);
  cudaMemsetAsync(w.status, 0, sizeof(uint32_t) * w.nseg, e.st);
  auto launch = [&]() -> cudaError_t {
    switch (which) {
      case 0: {
        ReconArgs r{};
        r.grids = w.gdev;
        r.ninst = nt;
        r.C = cb(w.St, w.csz);
        r.slot = noslot();
        r.U = mb(w.Ut, w.usz);
        r.sdiv = w.ntan;
        return launch_recon(g, r, e.st);
      }
      case 1: {
        PhysArgs p{};
        p.grids = w.gdev;
        p.tmp = w.Zt;
        p.tmp_inst = w.zt_inst;
        p.U = cb(w.Ut, w.usz);
        p.P = mbd(w.Pt, w.psz);
        p.nfields = 6;
        p.ninst = nt;
        p.sdiv = w.ntan;
        return launch_phys_inverse(g, p, e.st);
      }
      case 2: {
        ProdArgs ap{};
        ap.grids = w.gdev;
        ap.tmp = w.Zt;
        ap.tmp_inst = w.zt_inst;
        ap.Pp = cbd(w.Pp, w.psz);
        ap.pdiv = w.ntan;
        ap.Pt = cbd(w.Pt, w.psz);
        ap.H = mb(w.Ut, w.usz);
        ap.ninst = nt;
        ap.sdiv = w.ntan;
        return launch_products_fwd(g, ap, e.st);
      }
      case 3: {
        SolveArgs sa{};
        sa.grids = w.gdev;
        sa.H = cb(w.Ut, w.usz);
        sa.Hprev = cb(nullptr, 0);
        sa.Cc = mb(w.io, w.csz);   // scratch copy: the carried state is left alone
        sa.Sout = mb(w.io, w.csz);
        sa.T = mb(nullptr, 0);
        sa.tdiv = 1;
        sa.slot = noslot();
        sa.k = 1;
        sa.mean_mode = MEAN_TAN_HOMOG;
        sa.mdiv = w.ntan;
        sa.ninst = nt;
        sa.sdiv = w.ntan;
        return launch_solve(g, sa, e.st);
      }
      case 4: {
        ProdArgs ap{};
        ap.grids = w.gdev;
        ap.tmp = w.Zt;
        ap.tmp_inst = w.zt_inst;
        ap.Pp = cbd(w.Pp, w.psz);
        ap.pdiv = 1;
        ap.Pt = cbd(w.Pl, w.psz);
        ap.H = mb(w.Up, w.usz);
        ap.ninst = w.nseg;
        ap.sdiv = 1;
        return launch_products_adj(g, ap, e.st);
      }
      default:
        return cudaErrorInvalidValue;
    }
  };
  if (which == 3) cudaMemcpyAsync(w.io, w.Ct, sizeof(cpx) * w.csz * nt, cudaMemcpyDeviceToDevice, e.st);
  if (launch() != cudaSuccess) return -1.0;  // warm-up
  cudaEventRecord(a, e.st);
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(b, e.st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  g_launches += reps + 1;
  return ms / reps;
}

int c_synchronize(void) {
  if (!E) return 0;
  return cudaStreamSynchronize(E->st) == cudaSuccess ? 0 : -1;
}

long long c_launch_count(void) { return g_launches; }

const char* c_autotune_report(void) { return g_tune_report.c_str(); }

double c_pipe_peak_tflops(int kind) {
  const double fpi = probe_flop_per_thread_iter(kind);
  if (fpi <= 0.0) return NAN;
  cudaStream_t st = E ? E->st : nullptr;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8, iters = kind == 3 ? 16384 : 4096;
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * threads * blocks) != cudaSuccess) return NAN;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch_pipe_probe(kind, buf, blocks, threads, iters, st);  // warm-up
  cudaEventRecord(a, st);
  for (int r = 0; r < 3; ++r) launch_pipe_probe(kind, buf, blocks, threads, iters, st);
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  g_launches += 4;
  const double flop = 3.0 * blocks * threads * (double)iters * fpi;
  return flop / (ms * 1e-3) / 1e12;
}

double c_fp64_peak_tflops(void) { return c_pipe_peak_tflops(0); }

}  // extern "C"
