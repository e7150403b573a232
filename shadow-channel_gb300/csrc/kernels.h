// Kernel argument blocks and launchers (host-callable).
#pragma once

#include "chn_common.cuh"

namespace chn {

// A trajectory slot chosen on the device: slot = mul * (*ptr) + add (ptr may
// be null: slot = add).  Lets one captured CUDA graph serve every time step.
struct SlotRef {
  const int* ptr;
  int mul, add;
  long long stride;  // elements between consecutive slots
  __device__ __forceinline__ int slot() const { return ptr ? mul * (*ptr) + add : add; }
};

// coefficients -> velocity U (channel/initAlphaBeta2.c:12-240)
struct ReconArgs {
  Batch<const cpx> C;   // [inst] -> coefficient array (plus slot offset when slot.stride != 0)
  SlotRef slot;
  Batch<cpx> U;         // [inst] -> U[Nz][5][Q][X]
  int ninst;
  const uint32_t* status;
  int sdiv;
  const Grid* grids;    // uneven batch: grid of each instance (device array), else null
};

struct PhysArgs {
  Batch<const cpx> U;
  Batch<double> P;      // [inst] -> P[nf][Q][pz][px] (plus a slot offset when pslot.stride != 0)
  SlotRef pslot;
  int nfields;          // 3: u, v, w;  6: plus wz, wx, wy
  int ninst;
  uint32_t* status;     // per-segment status word (instance i -> status[i / sdiv])
  int sdiv;
  double* cflmax;       // per-segment largest CFL number seen (nullable)
  int cfl_check;
  int skip_blocked;
  cpx* tmp;             // split transforms: intermediate for tmp_inst instances of 6
  int tmp_inst;         //   spectral columns [6][Q][pz][Nx/2] each
  const Grid* grids;    // uneven batch: grid of each instance
};

struct ProdArgs {
  Batch<const double> Pp;  // primal physical fields, instance i -> Pp.base + (i / pdiv) * Pp.stride
  int pdiv;                //   (plus a slot offset when pslot.stride != 0)
  SlotRef pslot;
  Batch<const double> Pt;  // tangent fields (forward) / lambda (adjoint); base == nullptr: primal H
  Batch<cpx> H;            // [inst] -> H[Nz][5][Q][X]
  int ninst;
  const uint32_t* status;
  int sdiv;
  cpx* tmp;                // split transforms: as PhysArgs::tmp
  int tmp_inst;
  const Grid* grids;       // uneven batch: grid of each instance
  // adjoint products only: 1 = the exact transpose of the tangent products
  // (Pt holds the physical fields of the scaled H_bar, slots Hz, Hx, Hy; H
  // receives the velocity cotangent u, v, w, du/dy, dw/dy)
  int exact;
};

// mean-mode variants (channel/project0.c:153-168, increproject0.c:209-214, adjproject0.c:153-167)
enum MeanMode : int { MEAN_PRIMAL = 0, MEAN_TAN_FORCED = 1, MEAN_TAN_HOMOG = 2, MEAN_ADJOINT = 3 };

// One RK3 substage of the implicit Galerkin solve, one block per (instance, kz line, kx tile).
// channel/project.c:24-405, project0.c:22-271, increproject*.c, adjproject*.c:10-550
struct SolveArgs {
  Batch<const cpx> H;       // nonlinear terms of this stage
  Batch<const cpx> Hprev;   // adjoint: previous-stage terms for the next right-hand side
  Batch<cpx> Cc;            // carried right-hand side / state (in place)
  Batch<cpx> Sout;          // solved state output (scratch for the next reconstruction)
  // trajectory store of instance i (only when i % tdiv == tsel):
  //   T.base + (i / tdiv) * T.stride + slot * slot.stride, skipped for slot < 0
  Batch<cpx> T;
  int tdiv, tsel;
  SlotRef slot;
  int k;                    // RK substage 0..2
  int adjoint;              // 0 forward coefficients, 1 adjoint coefficients
  int mean_mode;            // for tangents: MEAN_TAN_HOMOG, or MEAN_TAN_FORCED where
  uint32_t forced_mask;     //   bit (i % mdiv) of forced_mask is set
  int mdiv;
  int ninst;
  const uint32_t* status;
  int sdiv;
  // Re-sensitivity forcing of tangents: bit (i % mdiv) of re2_mask selects the
  // reference's forcing reconnected, of re3_mask the exact derivative.  The
  // primal state before this substage of instance i is
  //   Xf.base + (i / xdiv) * Xf.stride + xslot.slot() * xslot.stride
  // (the state after it follows one slot later), its flux correction after
  // this substage Ftr[(i / xdiv) * ftr_stride + xslot.slot() + 1].
  uint32_t re2_mask, re3_mask;
  Batch<const cpx> Xf;
  SlotRef xslot;
  int xdiv;
  const double* Ftr;
  long long ftr_stride;
  // primal only: store flux_t of each stored substage at
  // Fts[(i / tdiv) * fts_stride + slot] (nullable)
  double* Fts;
  long long fts_stride;
  const Grid* grids;        // uneven batch: grid of each instance
};

// One substage of the exact discrete adjoint of the homogeneous tangent
// (adjoint_exact.cu), one block per (instance, kz line, kx tile): the
// transpose of the quadrature, banded solve and reconstruction of a tangent
// substage.  final_only: Cc += Recon^T(Ub) (the sweep's start state) only.
struct SolveTArgs {
  Batch<const cpx> Ub;      // velocity cotangent after the substage, U layout
  Batch<cpx> Cc;            // carried cotangent: after the substage in, before it out (in place)
  Batch<cpx> Hb;            // H_bar out, slots 0..2 (Hz, Hx, Hy), scaled for the inverse transform
  int k;                    // RK substage 0..2
  int final_only;
  int ninst;
  const uint32_t* status;
  int sdiv;
  const Grid* grids;        // uneven batch: grid of each instance
  // Parameter gradients (gacc null: none).  Per instance, gacc[i * gstride]
  // accumulates <x_bar, add> of the mean line over the substages (the
  // cotangent of the mean-flux forcing of the tangent: dJ/dmeanU), and
  // gacc[i * gstride + 1 + block] this block's <c2_bar, f_Re> (the cotangent
  // of the exact Re forcing, f_Re = -re^2 dt (a_k D x_k + b_k D x_{k+1}):
  // dJ/dRe), from the primal states x_k = MC[3n + k] at Xf + i * xstride,
  // slot xslot, and the flux corrections Ftr[i * ftr_stride + slot].
  double* gacc;
  int gstride;
  const cpx* Xf;
  long long xstride;
  SlotRef xslot;
  const double* Ftr;
  long long ftr_stride;
};

// one ddt_project / adjoint coupling for nseg segments (channel/channel.c:704-780)
struct DdtArgs {
  const cpx* MC;            // segment s trajectory: MC + s * traj_stride
  long long traj_stride;
  const int* step_ptr;      // i_step = *step_ptr + step_add (or step_add when null)
  int step_add;
  int nseg;
  // > 0: the segments are consecutive windows of one trajectory, each chain
  // steps long; at i_step 0 segment s > 0 takes its earlier state from
  // segment s - 1, step chain - 1 (the reference's global step before the window)
  int chain;
  const Grid* grids;        // uneven batch: grid of each segment (its sizes, weights and dt)
};

void prepare_kernels(const Grid& g);  // function attributes; call once, outside graph capture

cudaError_t launch_recon(const Grid& g, const ReconArgs& a, cudaStream_t st);
// the reconstruction on the tensor cores (exact digit products, one FP64 rounding)
cudaError_t launch_recon_tc(const Grid& g, const ReconArgs& a, cudaStream_t st);
size_t recon_tc_smem_bytes(const Grid& g);
cudaError_t launch_phys_inverse(const Grid& g, const PhysArgs& a, cudaStream_t st);
// the inverse transforms as exact digit GEMMs on the tensor cores (fused, one block per plane)
cudaError_t launch_phys_inverse_tc(const Grid& g, const PhysArgs& a, cudaStream_t st);
bool phys_tc_fits(const Grid& g, int optin);
// the grid has compile-time-size builds of the tensor-core inverse (Grid::tcminb 6, 7)
bool phys_tc_specialised(const Grid& g);
// the inverse on tcgen05 (phys_tc5.cu): fits for nf fields; the error word
// of its bounded waits (returned and cleared)
cudaError_t launch_phys_inverse_tc5(const Grid& g, const PhysArgs& a, cudaStream_t st);
bool phys_tc5_fits(const Grid& g, int nf, int optin);
int tc5_take_error();
// products + forward transforms as digit GEMMs (mode 0 primal, 1 tangent, 2 adjoint, 3 exact transpose)
cudaError_t launch_products_tc(const Grid& g, const ProdArgs& a, int mode, cudaStream_t st);
bool fwd_tc_fits(const Grid& g, int optin);
// the forward products' shared-memory plan (planes per pass, x-stage columns per chunk)
bool fwd_tc_plan(const Grid& g, int optin, int& pb, int& xch);
cudaError_t launch_products_fwd(const Grid& g, const ProdArgs& a, cudaStream_t st);
cudaError_t launch_products_adj(const Grid& g, const ProdArgs& a, cudaStream_t st);
cudaError_t launch_solve(const Grid& g, const SolveArgs& a, cudaStream_t st);
cudaError_t launch_solve_T(const Grid& g, const SolveTArgs& a, cudaStream_t st);
// ca[i] += src[i] per instance (grids: each instance's own coefficient size)
cudaError_t launch_add_source(const Grid& g, Batch<const cpx> src, Batch<cpx> ca, int ninst, cudaStream_t st,
                              const Grid* grids = nullptr);

// split-transform intermediate per instance, in complex elements
size_t split_tmp_elems(const Grid& g);
// whether the fused one-block-per-plane transforms fit this device's shared memory
bool fused_transforms_fit(const Grid& g, int smem_optin);
// split-transform variants (block size, chunk) the autotuner chooses from
struct TransformVariant {
  int nt, ch;
};
int split_variant_count();
TransformVariant split_variant(int v);
bool split_variant_fits(int v, const Grid& g, int optin);
size_t recon_smem_bytes(const Grid& g);
size_t phys_smem_bytes(const Grid& g, bool with_cfl);
size_t prod_adj_smem_bytes(const Grid& g);
size_t solve_smem_bytes(const Grid& g);

// flow[d][xp][y][zp] <- P[d][y][zp][xp]
cudaError_t launch_flow_out(const Grid& g, const double* P, double* flow, cudaStream_t st);
// dC[s] = (MC[s][i+] - MC[s][i-]) / dt
cudaError_t launch_ddt_diff(const Grid& g, const DdtArgs& d, cpx* dC, cudaStream_t st);
// per-segment partial sums of sum a*b*W[y], sum a*a*W[y] over 3 fields: part[s][nblk][2]
cudaError_t launch_ddt_dots(const Grid& g, Batch<const double> Pa, Batch<const double> Pb, double* part,
                            int nblk, int nseg, cudaStream_t st, const Grid* grids = nullptr);
// r = num/den; IC' = IC - r dC (written to ICdst when non-null); AC -= coef * IC'
// (grids non-null: the coefficient is coef * dt of each segment's grid)
cudaError_t launch_ddt_apply(const Grid& g, const double* part, int nblk, int nseg, Batch<const cpx> ICsrc,
                             SlotRef icslot, Batch<cpx> ICdst, Batch<const cpx> dC, double* r_out,
                             Batch<cpx> AC, double coef, cudaStream_t st, const Grid* grids = nullptr);
// the same partial sums from field caches: dCdt's fields from primal cache
// slots i+ and i- ([seg][slot][6][Q][pz][px]), the tangent's from velocity
// cache slot i ([seg][step][3][Q][pz][px])
cudaError_t launch_ddt_dots_cached(const Grid& g, const DdtArgs& d, const double* Pc, long long cstride,
                                   long long psz, const double* Pv, long long vstride, long long vslot,
                                   double* part, int nblk, cudaStream_t st);
// velocity cache slot (*step + add) of segment s <- fields 0..2 of P instance s * div + sel
cudaError_t launch_cache_velocity(const Grid& g, const double* P, long long pstride, int div, int sel, double* Pv,
                                  long long vstride, long long vslot, const int* step, int add,
                                  const uint32_t* status, int nseg, cudaStream_t st);
// AC[s] -= coef * src[s]
cudaError_t launch_sub_scaled(const Grid& g, Batch<const cpx> src, Batch<cpx> ac, double coef, int nseg,
                              cudaStream_t st, const Grid* grids = nullptr);
cudaError_t launch_project_init(const Grid& g, const cpx* Uinit, cpx* C, const double* luQs,
                                const double* luRs, cudaStream_t st);
cudaError_t launch_step_advance(int* ctr, int delta, cudaStream_t st);
// a multi-step sweep as one graph launch: the steps-left counter, and the
// while node's per-iteration kernel that counts it down and sets its condition
cudaError_t launch_loop_set(int* ctr, int n, cudaStream_t st);
// a seeded pattern of finite doubles (the autotuner's timing inputs)
cudaError_t launch_fill_pattern(double* p, size_t n, uint32_t seed, cudaStream_t st);
cudaError_t launch_loop_next(int* ctr, cudaGraphConditionalHandle h, cudaStream_t st);
cudaError_t launch_fp64_probe(double* out, int blocks, int threads, int iters, cudaStream_t st);
// pipe throughput probes: kind 0 DFMA, 1 DADD, 2 DMMA (m8n8k4 f64), 3 FFMA
cudaError_t launch_pipe_probe(int kind, double* out, int blocks, int threads, int iters, cudaStream_t st);
double probe_flop_per_thread_iter(int kind);

}  // namespace chn
