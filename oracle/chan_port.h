/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle.  Never linked into the product
 * library; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it, and only as the checker or the timed CPU baseline.
 *
 * A reentrant C restatement of the reference channel-flow time step
 * (channel/channel.c and the per-substage routines it calls).  All solver
 * state lives in one struct, so several independent instances (LSS segments)
 * can run in parallel threads, which the single-global-instance reference
 * cannot.  The arithmetic follows the reference statement by statement (same
 * loop order, same association of every floating-point expression), so on a
 * build without FMA contraction it reproduces the compiled reference bit for
 * bit; tests/test_oracle_pin.py checks that against oracle/_ref.
 *
 * Array layouts are the reference's (channel/getMem.c):
 *   coefficients  C[Nz][2][dimR][Nx/2]          complex (ALPHA=0, BETA=1)
 *   trajectories  MC[3*nsteps+1][Nz][2][dimR][Nx/2]
 *   velocity      U[Nz][5][qpts][Nx/2]           complex (XEL..DZEL)
 *   physical flow flow[3][3Nx/2][qpts][3Nz/2]    double
 */
#ifndef ORACLE_CHAN_PORT_H
#define ORACLE_CHAN_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cport cport;

/* channel.c:207 init(); returns NULL on the reference's EXIT_FAILURE cases. */
cport *cport_init(int Nx, int Ny, int Nz, double Lx, double Lz, double Re,
                  double flux, double dt, int nsteps);
void cport_destroy(cport *s);

/* channel.c:399 primal(); C_given may be NULL (laminar + rand() start).
   Returns 0, or -1 when pass1 stopped the loop on a CFL violation. */
int cport_primal(cport *s, int ru_steps, double *C_given);
/* channel.c:486 tangent() */
int cport_tangent(cport *s, int start_step, int end_step, double *IC_given,
                  int inhomo);
/* channel.c:596 adjoint() */
/* forcing 0 none, 1 mean flux, 2 Re (reference forcing reconnected), 3 Re (exact) */
int cport_tangent_forcing(cport *s, int start_step, int end_step, double *IC_given,
                          int forcing);
/* the transpose of the homogeneous tangent (cport_tangent_forcing kind 0)
   from end_step to start_step (start > end) applied to AC_given in place;
   no reference counterpart */
int cport_adjoint_exact(cport *s, int start_step, int end_step, double *AC_given);
int cport_adjoint(cport *s, int start_step, int end_step, double *AC_given,
                  int inhomo, double strength);
/* channel.c:704 ddt_project() */
double cport_ddt_project(cport *s, int i_step, double *IC_given);
/* spec2phys.c:10 spec2phys() */
void cport_spec2phys(cport *s, const double *C_ptr, double *flow);

/* views of library-owned arrays (channel.i:115-142, 212-219) */
double *cport_mc(cport *s, int i_step);   /* MC[3*i_step]  */
double *cport_mic(cport *s, int i_step);  /* MIC[3*i_step] */
double *cport_mc_sub(cport *s, int count);   /* MC[count]  (any substage) */
double *cport_mic_sub(cport *s, int count);  /* MIC[count] */
const double *cport_qy(cport *s);
const double *cport_w(cport *s);
int cport_dims(cport *s, int *qpts, int *dimR, int *dimQ, int *Nx, int *Nz,
               int *nsteps);
/* Legendre tables for cross-checking the product's setup:
   which = 0 Q, 1 Qp, 2 Qpp, 3 R, 4 Rp, 5 Qw, 6 Qpw, 7 Qppw, 8 Rw, 9 Rpw,
           10 Qs, 11 Qps, 12 Qpps, 13 Rs, 14 Rps */
const double *cport_table(cport *s, int which);

#ifdef __cplusplus
}
#endif
#endif
