/*
 * c_channel -- GB300 drop-in for the C entry points of the shadow-channel
 * SWIG module (channel/channel.i) plus batched additions.
 *
 * Plain C ABI: complex numbers are {double re, im} (the layout of FFTW-2's
 * fftw_complex, channel/mcomplex.h:19-22), arrays are caller-owned,
 * C-contiguous and updated in place exactly as the SWIG INPLACE_ARRAY4
 * typemaps do.  The dimension arguments that follow each array are the ones
 * SWIG passes; a mismatch aborts the process like the reference's assert().
 *
 * Shapes: coefficients [Nz][2][Ny-2][Nx/2]; flow [3][3Nx/2][qpts][3Nz/2],
 * qpts = 3Ny/2.  All arithmetic is FP64 on the GPU; the host only moves data.
 *
 * One global instance per process, as in the reference (channel/main.h
 * keeps all state in globals; channel/__init__.py:80-82 enforces one init).
 */
#ifndef SHADOW_CHANNEL_GB300_C_CHANNEL_H
#define SHADOW_CHANNEL_GB300_C_CHANNEL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double re, im;
} chn_complex;

/* ---- reference entry points (channel/channel.i) ---------------------- */

/* channel.i:18-22 -> channel.c:207 init().  Returns 0, or 1 (EXIT_FAILURE)
   for Nx % 4 != 0, Nz % 2 != 0, Ny <= 4, an unsupported FFT length or an
   allocation failure.  flux is 2*meanU as the Python layer passes it. */
int c_init(int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
           double flux, double dt, int nsteps);

/* channel.i:27-30 -> channel.c:52 destroy() */
void c_destroy(void);

/* channel.i:38-52 -> channel.c:399 primal().  A zero-sized array (all four
   dims 0) starts from the laminar profile plus a rand() perturbation. */
void c_primal(int ru_steps, chn_complex *C_given, int Nz_dup, int Nvar_dup,
              int Ny_dup, int Nx_dup);

/* channel.i:60-70 -> channel.c:486 tangent() */
void c_tangent(int start_step, int end_step, chn_complex *IC_given,
               int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup, int inhomo);

/* channel.i:78-88 -> channel.c:596 adjoint() */
/* c_tangent with a choice of forcing (no reference entry point; the
   reference's c_tangent is forcing = inhomo != 0): 0 none, 1 mean flux
   (meanU sensitivity, channel/increproject0.c:209-214), 2 Re sensitivity
   with the reference's forcing reconnected (channel/tangent_forcing.c,
   tangent_forcing0.c, increproject.c:61-104, disconnected at
   channel/channel.c:521; first order in dt), 3 Re sensitivity, exact
   derivative of the discrete RK3 step.  The mean flux is held fixed for 2, 3. */
void c_tangent_forcing(int start_step, int end_step, chn_complex *IC_given,
                       int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup,
                       int forcing);
void c_adjoint(int start_step, int end_step, chn_complex *AC_given,
               int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup, int inhomo,
               double strength);
/* The exact discrete adjoint: the transpose of the homogeneous tangent
   (c_tangent with inhomo 0, c_tangent_forcing with forcing 0) from end_step
   to start_step, applied in place to AC_given, the cotangent at
   start_step > end_step: <AC, T v> = <T^T AC, v> in the Euclidean inner
   product of the real and imaginary parts.  No reference counterpart: the
   reference's adjoint (channel/channel.c:596-696) integrates the continuous
   adjoint equations with reversed RK coefficients.  No ddt coupling. */
void c_adjoint_exact(int start_step, int end_step, chn_complex *AC_given,
                     int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup);
/* c_adjoint_exact with a source added after every step:
     lambda_n = T_n^T lambda_{n+1} + src,  n = start_step - 1 .. end_step,
   lambda_{start_step} = AC_given, the result lambda_{end_step} in AC_given:
   the gradient with respect to the state at end_step of a sum over steps
   end_step .. start_step - 1 of <src, C_n> (src the gradient of a linear
   per-step functional, e.g. the wall shear).  No reference counterpart. */
void c_adjoint_exact_source(int start_step, int end_step,
                            chn_complex *AC_given, const chn_complex *src,
                            int Nz_dup, int Nvar_dup, int Ny_dup, int Nx_dup);
/* c_adjoint_exact_source (src may be null: no source) that also returns the
   two parameter gradients of the same functional in grad[2]:
     grad[0] = dJ/dmeanU, the cotangents of the mean-flux forcing the
               reference's inhomogeneous tangent adds to every substage
               (channel/increproject0.c:209-214; c_tangent_forcing kind 1);
     grad[1] = dJ/dRe, of the exact Re forcing -re^2 dt (a_k D x_k +
               b_k D x_{k+1}) of every substage (c_tangent_forcing kind 3),
   where J = <AC_given, C_start_step> + sum_n <src, C_n>: one reverse sweep
   gives what one forced tangent sweep per parameter gives.  The Re parts
   are summed in a fixed order (bit-reproducible).  Returns the status
   (c_last_error).  No reference counterpart. */
int c_adjoint_exact_grad(int start_step, int end_step, chn_complex *AC_given,
                         const chn_complex *src, double *grad);

/* channel.i:96-105 -> channel.c:704 ddt_project() */
double c_ddt_project(int i_step, chn_complex *IC_given, int Nz_dup,
                     int Nvar_dup, int Ny_dup, int Nx_dup);

/* channel.i:115-125 / 133-142: pointer to the stored (incremental) solution
   at step i_step.  The pointer refers to a library-owned host mirror that
   is refreshed by every call; it stays valid until c_destroy(). */
void c_getsoln(int i_step, chn_complex **MC_ptr, int *Nz_ptr, int *Nvar_ptr,
               int *Ny_ptr, int *Nx_ptr);
void c_getincresoln(int i_step, chn_complex **MIC_ptr, int *Nz_ptr,
                    int *Nvar_ptr, int *Ny_ptr, int *Nx_ptr);

/* channel.i:152-170 -> spec2phys.c:10 spec2phys() */
void c_spec2phys(chn_complex *C_ptr, int Nz_dup, int Nvar_dup, int Ny_dup,
                 int Nx_dup, double *flow_ptr, int Nd_flow, int Nx_flow,
                 int Ny_flow, int Nz_flow);

/* channel.i:178-205 -> channel.c:791/889.  HDF5 is not part of this build;
   these write / read the same datasets (alpha, beta as [dimR][Nz][Nx/2]
   {real, imaginary} records, Nx, Ny, Nz, dt, 1/Re, mpg) in a raw
   little-endian container: 8 bytes "SCHNRAW1", int32 Nx, Ny, Nz, 0,
   double dt, 1/Re, mpg, then alpha, beta, ialpha, ibeta. */
void c_read_solution(char *filename, chn_complex *C_ptr, int Nz_dup,
                     int Nvar_dup, int Ny_dup, int Nx_dup);
void c_save_solution(char *filename, chn_complex *C_ptr, int Nz_dup,
                     int Nvar_dup, int Ny_dup, int Nx_dup);

/* channel.i:212-219: quadrature points and weights (library-owned) */
void c_quad(double **y_ptr, int *qpts_ptr1, double **w_ptr, int *qpts_ptr2);

/* channel.i:222-229 */
int c_qpts(void);
int c_dimR(void);
int c_dimQ(void);
int c_Nx(void);
int c_Nz(void);
int c_nsteps(void);

/* ---- additions (no counterpart in the reference) --------------------- */

/* Status of the last call: 0 ok; bit 0 = the CFL limit stopped the time loop
   (the reference prints and returns silently, channel/pass1.c:133-137);
   bit 1 = non-finite values seen; negative = CUDA or argument error. */
int c_last_error(void);
const char *c_last_error_message(void);
/* largest CFL number seen by the last primal/tangent call */
double c_last_cfl(void);

/* Batched segments: nseg independent trajectories on the c_init grid, each
   with ntan tangents; the adjoint couples (strength != 0) to the stored
   trajectory of tangent `couple`.  Host arrays, segment-major.  The sweep
   calls return the call's status, the value c_last_error() returns after
   it: a segment stopped by the CFL limit or holding non-finite values
   gives bits 0 / 1 and leaves the other segments' results as they would
   be without it. */
int c_batch_init(int nseg, int ntan, int couple);
/* the same with a trajectory length of the batch's own (<= any length; the
   reference's nsteps of c_init is not used by the batch) */
int c_batch_init_steps(int nseg, int ntan, int couple, int nsteps);
int c_batch_destroy(void);
/* primal trajectories for all segments; C [nseg][Nz][2][dimR][Nx/2] in/out */
int c_batch_primal(int ru_steps, chn_complex *C);
/* tangents on stored primal trajectories; IC [nseg][ntan][...] in/out;
   inhomo[ntan] selects the forcing per tangent (the values of
   c_tangent_forcing: 0 none, 1 mean flux, 2 / 3 Re) */
int c_batch_tangent(int start_step, int end_step, chn_complex *IC,
                    const int *inhomo);
/* primal and tangents advanced together from C (fused forward sweep) */
int c_batch_forward(int start_step, int end_step, chn_complex *C,
                    chn_complex *IC, const int *inhomo);
/* adjoints; AC [nseg][...] in/out */
int c_batch_adjoint(int start_step, int end_step, chn_complex *AC,
                    double strength);
/* exact discrete adjoints (as c_adjoint_exact) on the stored primal
   trajectories; AC [nseg][...] in/out */
int c_batch_adjoint_exact(int start_step, int end_step, chn_complex *AC);
/* MC / MIC of one segment at step i_step into out [Nz][2][dimR][Nx/2] */
int c_batch_getsoln(int seg, int i_step, chn_complex *out);
int c_batch_getincresoln(int seg, int i_step, chn_complex *out);

/* Segments as consecutive windows of one trajectory, each window_steps long
   (LSS time segments, drivers/wrapper.py): ddt_project at a window start
   takes dC/dt across the boundary from the previous segment, as the
   reference does on its single global trajectory (channel/channel.c:729-740).
   0 turns it off. */
int c_batch_set_chain(int window_steps);
/* ddt_project (channel.i:96-105 -> channel/channel.c:704-780) of one vector
   per segment at the segment's step i_step, in place; r[nseg] receives the
   projection coefficients (nullable).  Host arrays / device arrays. */
int c_batch_ddt_project(int i_step, chn_complex *V, double *r);
int c_batch_ddt_project_dev(int i_step, chn_complex *V, double *r);

/* The same batched calls on device-resident arrays (CUDA device pointers,
   same layouts); no host copies.  stream 0 = the library's stream. */
int c_batch_forward_dev(int start_step, int end_step, chn_complex *C,
                        chn_complex *IC, const int *inhomo);
int c_batch_adjoint_dev(int start_step, int end_step, chn_complex *AC,
                        double strength);
int c_batch_adjoint_exact_dev(int start_step, int end_step, chn_complex *AC);
int c_batch_adjoint_exact_source_dev(int start_step, int end_step,
                                     chn_complex *AC, const chn_complex *src);
/* the same with the parameter gradients of c_adjoint_exact_grad per segment:
   grad (host) [nseg][2] = dJ/dmeanU, dJ/dRe; src device, may be null */
int c_batch_adjoint_exact_grad_dev(int start_step, int end_step,
                                   chn_complex *AC, const chn_complex *src,
                                   double *grad);
int c_batch_primal_dev(int ru_steps, chn_complex *C);
int c_batch_tangent_dev(int start_step, int end_step, chn_complex *IC,
                        const int *inhomo);

/* the library's CUDA stream (cudaStream_t), for recording events on it */
void *c_stream(void);
/* average device time in ms of one launch of one kernel of a batched forward
   substage on the current batch buffers: 0 reconstruct, 1 physical
   transforms, 2 tangent products, 3 tangent solve, 4 adjoint products */
double c_batch_kernel_ms(int which, int reps);

/* wait for all queued device work of the library */
int c_synchronize(void);
/* kernel launches issued by the library since c_init (for bookkeeping) */
long long c_launch_count(void);
/* FP64 fused-multiply-add throughput of this GPU in TFLOP/s (2 flop/FMA),
   measured with a register-only kernel; used as the roofline peak. */
double c_fp64_peak_tflops(void);
/* throughput of one pipe in TFLOP/s (counting an FMA as 2): kind 0 FP64
   FMA, 1 FP64 add, 2 FP64 warp matrix multiply-accumulate (m8n8k4), 3 FP32
   FMA; NaN for other kinds */
double c_pipe_peak_tflops(int kind);
/* the transform autotuner's timings (ms per batched substage) and choice
   for the last c_batch_init / c_multi_init, as a JSON object ("" before) */
const char *c_autotune_report(void);

/* spec2phys without allocating: no counterpart in the reference.  For
   callers that cannot call cudaMalloc when they need a physical field (code
   running while a stream is captured into a graph, real-time loops that must
   not touch the allocator).  C_dev (complex [Nz][2][dimR][Nx/2]) and flow_dev
   (double [3][3Nx/2][qpts][3Nz/2]) are CUDA device arrays owned by the
   caller; the intermediate arrays live in fixed device arrays of the library
   (16 MiB on every GPU that loads it, kept until exit), so grids needing more
   than 2^19 complex velocity or 2^20 physical scratch elements (beyond
   32x65x32) are rejected with -5 and a message.  Requires c_init.  The first
   call on a device looks up the scratch addresses; make that first call
   before any stream capture.  The work is queued on the library stream
   (c_stream); c_synchronize before reading flow_dev.  All calls share the
   scratch, so calls that overlap on the GPU race.  Returns 0 or a negative
   error (c_last_error_message). */
int c_spec2phys_noalloc(const chn_complex *C_dev, double *flow_dev);

/* Uneven batches (no reference counterpart): n instances, each with its own
   grid, Re, flux and dt, advanced together by the same kernel launches.
   Host arrays are packed instance after instance, each in the reference
   layout of its own grid (c_multi_coef_elems(i) complex elements; tangents:
   the ntan arrays of an instance one after another).  Same semantics as the
   c_batch_* calls per instance; the adjoint's coupling strength is scaled by
   each instance's own dt. */
int c_multi_init(int n, const int *Nx, const int *Ny, const int *Nz,
                 const double *Lx, const double *Lz, const double *Re,
                 const double *flux, const double *dt, int nsteps, int ntan,
                 int couple);
int c_multi_destroy(void);
long long c_multi_coef_elems(int i);
int c_multi_primal(int ru_steps, chn_complex *C);
int c_multi_forward(int start_step, int end_step, chn_complex *C,
                    chn_complex *IC, const int *inhomo);
int c_multi_adjoint(int start_step, int end_step, chn_complex *AC,
                    double strength);
int c_multi_adjoint_exact(int start_step, int end_step, chn_complex *AC);
int c_multi_getsoln(int i, int i_step, chn_complex *out);

/* Objectives and statistics of the stored trajectories, computed on the
   device from the coefficients (no reference C counterpart: the reference
   averages spec2phys output in Python, channel/__init__.py:217-299 and
   drivers/sensitivities.py).  inc 0: primal MC, 1: tangent MIC; comp 0 u,
   1 v, 2 w; steps start..end-1.
   c_mean_profile: x-z mean of the component at each quadrature point,
     out [end-start][qpts];
   c_wall_shear: dU/dy and dW/dy of the mean flow at y = -1 (the reference's
     Uxb, Uzb of channel/project0.c:224-234), out [end-start][2];
   c_mean_product: x-z mean of comp_a (of inc_a) times comp_b (of inc_b) at
     each quadrature point, out [end-start][qpts].
   Batch variants: the same for every segment, out [nseg][end-start][...]. */
int c_mean_profile(int inc, int comp, int start_step, int end_step, double *out);
/* the weights Rp0 = R'(-1) of the wall shear, out[dimR]: c_wall_shear's
   dU/dy = sum_r Rp0[r] Re(C[0][0][r][0]) (dW/dy likewise on beta), i.e. the
   gradient of the wall shear with respect to the mean-mode coefficients */
int c_wall_shear_weights(double *out);
int c_wall_shear(int inc, int start_step, int end_step, double *out);
int c_mean_product(int inc_a, int comp_a, int inc_b, int comp_b, int start_step,
                   int end_step, double *out);
int c_batch_mean_profile(int inc, int comp, int start_step, int end_step, double *out);
int c_batch_mean_profile_dev(int inc, int comp, int start_step, int end_step, double *out);
int c_batch_wall_shear_dev(int inc, int start_step, int end_step, double *out);
int c_batch_mean_product_dev(int inc_a, int comp_a, int inc_b, int comp_b,
                             int start_step, int end_step, double *out);

/* Least-squares shadowing on the device (no reference C counterpart: the
   reference does this in Python, drivers/wrapper.py:5-54 and
   drivers/pariter.py:63-125).  Needs a chained batch with ntan = 1.
   x, y: device arrays of 2*nseg - 1 coefficient arrays [v_0..v_{n-1},
   w_0..w_{n-2}]; y = KKT x (the reference's Wrapper.matvec); zeta[nseg]
   (device, nullable) = minus the window-end projection coefficients. */
int c_lss_matvec_dev(const chn_complex *x, chn_complex *y, int inhomo, double *zeta);
/* Euclidean dot product of two device arrays of n doubles (deterministic) */
int c_lss_dot_dev(long long n, const double *a, const double *b, double *out);
/* MINRES (pariter.par_minres) for KKT x = b from the x given; returns 0 when
   |eta|/|b - A x0| < tol, 1 after maxiter iterations, < 0 on error */
int c_lss_minres_dev(const chn_complex *b, chn_complex *x, double tol, int maxiter, int *iters,
                     double *rel_residual);

/* The time-invariant setup tables on the host (no GPU needed): which =
   0 Q, 1 Q', 2 Q'', 3 R, 4 R' (values at the quadrature points, [qpts][n]),
   5..9 the same weighted and transposed ([n][qpts]), 10 <Q,Q>, 11 <Q',Q'>,
   12 <Q'',Q''> ([Ny-4][9] bands), 13 <R,R>, 14 <R',R'> ([Ny-2][5] bands),
   15 quadrature points, 16 weights.  Writes when n is large enough; returns
   the table size, or -1 for bad arguments. */
int c_setup_table(int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
                  double flux, double dt, int which, double *out, int n);

/* Host-only, no device: the digit tables of the tensor-core contractions
   for a grid (base-256 digits of 56-bit scaled rows in mma fragment order,
   and the row exponents).  which: 0 the five bases [5][Q/16][R/16] tiles,
   1 their weighted transposes, 2 the inverse transform's z stage, 3 its x
   stage, 4 the forward x stage, 5 the forward z stage, 6 the unscaled
   forward x stage, 7 the bases transposed, 8 Qpw, Qw, Rw plane-major,
   9 / 10 the inverse's z / x stage as the tcgen05 kernel's B operands
   (the seven digit planes stacked along N, K-major core matrices; bytes
   as 32-bit words), with the exponents of tables 2 / 3.
   sizes[0] = uint32 words, sizes[1] = exponents.  With frag and ex null the
   call is a size query; a non-null buffer shorter than its table
   (nfrag < sizes[0] or nex < sizes[1]) is refused with -2 and nothing is
   written.  Returns 0, -1 for bad arguments, -2 for a short buffer. */
int c_setup_tc_table(int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
                     double flux, double dt, int which, uint32_t *frag,
                     long long nfrag, int *ex, long long nex, long long *sizes);

#ifdef __cplusplus
}
#endif
#endif
