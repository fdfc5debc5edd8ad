/*
 * oracle.h -- CPU FP64 restatement of the ImmerseFlow++ hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle for the CUDA path:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it;
 * the product library never links or calls it.
 *
 * Parity is pinned against the reference's own result files
 * (results/uc.dat, results/vc.dat, results/p.dat, results/final_results.dat),
 * converted to tests/golden/ by tests/golden/make_golden.py.
 *
 * Two parts:
 *  - REFERENCE primitives (orc_ref_*): the reference's buildable algorithm,
 *    restated operation for operation (src/include/ADSolver.cu,
 *    src/include/PPESolver.cu, src/include/preSim.cu).
 *  - METHOD solver (orc_create/orc_step/...): the full fractional step with
 *    ghost-cell IBM, written from the published method because the reference
 *    leaves it unimplemented (src/include/AD_PPE_Correction.cu:1-12 is empty,
 *    src/include/PPESolver.cu does not compile).  The CUDA path implements the
 *    same algorithm, sweep for sweep.
 */
#ifndef IFX_ORACLE_H
#define IFX_ORACLE_H

#include <stdint.h>
#include "../include/immerseflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* readGridData (src/include/preSim.cu:293-355): faces -> centres with the
 * reference's ghost rule, and dx/dy as full nx*ny arrays. nx = NX+2. */
void orc_grid(int nx, int ny, const double* xf, const double* yf, double* xc,
              double* yc, double* dx, double* dy);

/* initializeKernel (src/include/preSim.cu:53-97): vortex in uniform flow. */
void orc_ref_init(int nx, int ny, const double* xc, const double* yc, double* u,
                  double* v, double* p);

/* nsteps x ImmerseFlow::ADsolver (src/include/ADSolver.cu:268-395) with the
 * reference's buffer swaps.  u,v hold the state; ut,vt are the second
 * buffers (their content on entry is used exactly as the reference would).
 * On return the state is in u,v.  uf: (nx-1)*(ny-2), vf: (nx-2)*(ny-1).
 * iters[s] receives the Jacobi iterations of step s. */
int orc_ref_ad_steps(int nx, int ny, const double* dx, const double* dy,
                     const double* iblank, double dt, double re, int itermax,
                     double tol, int nsteps, double* u, double* v, double* ut,
                     double* vt, double* uf, double* vf, int* iters);

/* ImmerseFlow::PPESolver (src/include/PPESolver.cu:137-205) with the
 * coefficients it intends: Jacobi on Laplace, p=100 on the i=0/j=0 ghosts,
 * stopped when the signed residual sum over the interior drops below tol. */
int orc_ref_ppe(int nx, int ny, const double* dx, const double* dy, int itermax,
                double tol, double* p, int* iters);
/* The same with the solver inputs/inputs.txt:14 advertises: method 0 Jacobi,
 * 1 red-black point Gauss-Seidel / SOR, 2 zebra x-line SOR; w = relaxation. */
int orc_ref_ppe_opt(int nx, int ny, const double* dx, const double* dy, int itermax,
                    double tol, int method, double w, double* p, int* iters);
/* orc_ref_ad_steps with the Jacobi update relaxed by w_ad (1: none), the
 * reference's commented-out lines src/include/ADSolver.cu:95,116. */
int orc_ref_ad_steps_w(int nx, int ny, const double* dx, const double* dy,
                       const double* iblank, double dt, double re, int itermax,
                       double tol, double w_ad, int nsteps, double* u, double* v, double* ut,
                       double* vt, double* uf, double* vf, int* iters);

/* Bit-exact body predicate used for iBlank tagging: 1 = inside the ellipse. */
int orc_inside(double x, double y, double cx, double cy, double c, double s,
               double ia2, double ib2);

/* ------------------------------------------------------ method solver */
typedef struct orc_solver orc_solver;

orc_solver* orc_create(const ifx_config* cfg, const double* xf, const double* yf,
                       int nthreads);
int  orc_step(orc_solver* s, int nsteps);
/* fields as IFX_FIELD_*; n must match */
int  orc_get(orc_solver* s, int field, double* out, long n);
int  orc_set(orc_solver* s, int field, const double* in, long n);
int  orc_stats(orc_solver* s, ifx_stats* out);
/* IBM ghost list: cells[n], nb[4n], wu[4n], wp[4n]; returns count (arrays may be NULL) */
int  orc_ghosts(orc_solver* s, int* cells, int* nb, double* wu, double* wp,
                double* bi, double* ip);
int  orc_mg_levels(orc_solver* s);
void orc_destroy(orc_solver* s);
/* Prescribed body motion: sin, cos of 2 pi x (x in turns), and the current
 * pose (x, y, cos, sin, u, v, rotation rate). */
void orc_sincos_turns(double x, double* s, double* c);
void orc_body(orc_solver* s, double* out);

#ifdef __cplusplus
}
#endif
#endif
