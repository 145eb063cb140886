/*
 * CPU oracle for the ScaFES explicit update path -- TEST INFRASTRUCTURE ONLY.
 *
 * This header declares a plain-C restatement of the reference's per-node
 * update sweeps.  It exists so that tests, the smoke check and the CPU
 * baseline leg of the benchmark can check the CUDA path against the
 * reference arithmetic.  Nothing in the product library links or calls it.
 *
 * Layout of every field array: the nodes of the global grid in Fortran order
 * (x fastest), idx = i + nx*(j + ny*k), without ghost layers and without the
 * trailing "time" slot the reference appends
 * (src/ScaFES_DataField.hpp:948-953).
 *
 * Parity: pinned bit-for-bit against the reference itself, compiled from the
 * untouched reference headers by oracle/Makefile into oracle/_ref/, on the
 * system-test problems (tests/golden/ holds the vectors and the script).
 */
#ifndef SCAFES_ORACLE_H
#define SCAFES_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Discrete domain + time axis (src/ScaFES_Grid.hpp:538-556,
 * src/ScaFES_Parameters.hpp tau/timeIntervalStart). */
typedef struct orc_grid {
    int dim;            /* 1..3; unused axes have n = 1 */
    int n[3];           /* nodes per axis */
    double first[3];    /* coordinate of node 0 */
    double last[3];     /* coordinate of node n-1 */
    double h[3];        /* (last-first)/(n-1), filled by orc_grid_init */
    double tau;         /* time step size */
    double t_start;     /* timeIntervalStart */
    int n_layers;       /* nLayersAtBorder (reference default 1) */
} orc_grid;

void orc_grid_init(orc_grid* g, int dim, const int* n, const double* first,
                   const double* last, double tau, double t_start,
                   int n_layers);
double orc_time(const orc_grid* g, int timestep);
int orc_is_border(const orc_grid* g, int i, int j, int k);
void orc_coords(const orc_grid* g, int i, int j, int k, double* x);

/* A known field evaluated at time(t); base may be NULL (=> 0).
 *   form 0: base * (a + b*time)          (HeatEqnFDM TimeLinSpaceLin g, f)
 *   form 1: base*a + b*(base*(1 + time)) (PennesBioheatEqnFDM/Dirichlet/
 *           TimeLinSpaceLin/TimeLinSpaceLin.hpp:82-91 f, with
 *           a = RHO*C and b = RHO_BLOOD*C_BLOOD*W) */
/*   form 2: base*(a*(1 + time)) + b*(1 + time)  (Cauchy flux field)   */
/*   form 3: (base*(1 + time))^4 * a + b*(1 + time)  (Radiation field)  */
typedef struct orc_known {
    const double* base;
    int form;
    double a, b;
} orc_known;

/* Heat / Pennes (constant coefficients) with Dirichlet border.
 * Inner nodes: tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218 (perf_q1 == 0)
 *   or tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168.
 * Border nodes: u = knownDf(1) at time(t)  (Dirichlet/Dirichlet.hpp:125-131).
 * u holds the t = 0 iterate on entry and the t = nsteps iterate on exit.
 * Returns 0 or a negative status. */
int orc_heat_dirichlet(const orc_grid* g, double coeff_a, double rho_c,
                       double perf_q1, double perf_w, int nsteps, double* u,
                       orc_known f_src, orc_known g_bdry, int nthreads);

/* The same sweeps on caller-owned fields, allocating nothing: u holds the
 * t = 0 iterate on entry, w is a second field of the same size; on exit the
 * t = nsteps iterate is in u when nsteps is even and in w when it is odd
 * (the other field holds iterate nsteps - 1).  For timing the sweeps alone. */
int orc_heat_dirichlet_ws(const orc_grid* g, double coeff_a, double rho_c,
                          double perf_q1, double perf_w, int nsteps, double* u,
                          double* w, orc_known f_src, orc_known g_bdry, int nthreads);

/* Writes zeros into a[0..n) from the threads of a static OpenMP schedule,
 * so that the pages are mapped before a timed region. */
void orc_first_touch(double* a, size_t n, int nthreads);

/* Heat / Pennes with the flux-condition border of the reference's system
 * tests (kind 0: tests/system/HeatEqnFDM/Neumann/Neumann.hpp and
 * tests/system/PennesBioheatEqnFDM/Neumann/Neumann.hpp; kind 1: the
 * Cauchy.hpp files beside them): a border node with an index 0 takes
 * Dirichlet g_dir at time(t); the others take the inner update where, in
 * each direction of a max face, the missing neighbour is the inner one and
 * the flux of g_flux at time(t-1) enters (- (2h/lambda) G for Neumann,
 * - (2h/lambda) alpha u + (2h/lambda) G for Cauchy), in the reference's
 * operation order.  Known-field form 2 (base*(a*(1+t)) + b*(1+t)) is the
 * Cauchy flux field of Cauchy/TimeLinSpaceLin. */
int orc_heat_flux(const orc_grid* g, double coeff_a, double rho_c, double perf_q1,
                  double perf_w, double lambda, double alpha, int kind, int nsteps,
                  double* u, orc_known f_src, orc_known g_dir, orc_known g_flux,
                  int nthreads);

/* Pennes with the radiation border of tests/system/PennesBioheatEqnFDM/
 * Radiation/Radiation.hpp:126-174: as orc_heat_flux, with the max-face
 * flux - (2h/lambda) epsilon sigma u^4 + (2h/lambda) G in the reference's
 * operation order.  Known-field form 3 is the radiation field of
 * Radiation/TimeLinSpaceLin. */
int orc_heat_radiation(const orc_grid* g, double coeff_a, double rho_c, double perf_q1,
                       double perf_w, double lambda, double epsilon, double sigma, int nsteps,
                       double* u, orc_known f_src, orc_known g_dir, orc_known g_flux,
                       int nthreads);

/* Variable-coefficient Pennes bioheat (examples/MRIDataPBHEqnFDM/
 * MRIDataPBHEqnFDM.hpp:143-169) with scalar rho, c, k, rho_b, c_b, omega,
 * T_b and a stored heat-source field q; Dirichlet border value g_bdry. */
int orc_pennes_mri(const orc_grid* g, double rho, double c, double k,
                   double rho_b, double c_b, double omega, double t_blood,
                   const double* q, const double* g_bdry, int nsteps,
                   double* u, int nthreads);

/* Pennes bioheat with every coefficient a field over the nodes -- the
 * updateInner/updateBorder of the reference's tissue examples,
 * examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:143-275 (known fields
 * rho, c, lambda, rho_blood, c_blood, omega, T_blood, q, surface) and
 * examples/TumorHeatEqnFDM/TumorHeatEqnFDM.hpp:234-353 (constants, with
 * omega and Q chosen per node by the tumour sphere), in the reference's
 * operation order.  border 0: the examples' flux border -- Neumann with
 * q_bc at the min faces and the x, y max faces; at the z max face
 * Neumann with q_skull (MRI, surface 0 or NULL), Cauchy and radiation with
 * h_conv, t_amb, epsilon, sigma (MRI, surface 1; the radiated temperature
 * is the partially updated node value, as in the reference), or Cauchy
 * with h_conv, t_amb (zmax_kind 1, the tumour); border 1: Dirichlet from
 * g_bdry. */
typedef struct orc_tissue {
    const double *rho, *c, *k, *rho_b, *c_b, *omega, *t_blood, *q;
    const double* surface;
    int zmax_kind;
    double q_bc, q_skull, h_conv, t_amb, epsilon, sigma;
    int border;
    const double* g_bdry;
} orc_tissue;
int orc_pennes_tissue(const orc_grid* g, const orc_tissue* ts, int nsteps, double* u,
                      int nthreads);

/* HeatEqnFdmStencilWidthOne (tests/system/HeatEqnFdmStencilWidthOne/
 * HeatEqnFdmStencilWidthOne.hpp:120-163). */
int orc_stencil_width_one(const orc_grid* g, int nsteps, double* u,
                          int nthreads);

/* HeatEqnFdmStencilWidthVar (tests/system/HeatEqnFdmStencilWidthVar/
 * HeatEqnFdmStencilWidthVar.hpp:120-165) for one field of width bw. */
int orc_stencil_width_var(const orc_grid* g, int bw, int nsteps, double* u,
                          int nthreads);

/* L-infinity norm of (u - exact) over all nodes, and max |exact|
 * (src/ScaFES_DataField.hpp:1440-1530 computes the former). */
void orc_err_linf(const double* u, const double* exact, size_t n,
                  double* err, double* max_exact);

/* Flux-form heat with conductivity field k (adjoint workload).
 *   u'_i = u_i + sum_p (tau/h_p^2) [ kp (u_{i+p} - u_i) - km (u_i - u_{i-p}) ]
 *   kp = 0.5 (k_i + k_{i+p}),  km = 0.5 (k_i + k_{i-p});  border nodes fixed.
 * orc_kheat_forward advances u by nsteps; if traj != NULL it receives the
 * nsteps+1 iterates (t = 0..nsteps) back to back. */
int orc_kheat_forward(const orc_grid* g, const double* k, int nsteps,
                      double* u, double* traj, int nthreads);

/* Forward-mode AD (dual numbers) of orc_kheat_forward along one direction:
 * on entry u = u0, du = the u0 direction, dk = the k direction; on exit
 * u = u_T and du = its derivative.  The same mode as the reference's ADOL-C
 * gradient (fov_forward, src/ScaFES_Problem.hpp:6633-6747), so
 * <u_T - target, du> checks the adjoint's <dJ/dk, dk> + <dJ/du0, du0>. */
int orc_kheat_tangent(const orc_grid* g, const double* k, const double* dk, int nsteps,
                      double* u, double* du, int nthreads);

/* Adjoint of orc_kheat_forward for J = 0.5 ||u_T - target||^2.
 * traj holds the nsteps+1 forward iterates. Outputs dJ/dk and dJ/du0 and
 * returns J in *j_out. */
int orc_kheat_adjoint(const orc_grid* g, const double* k, int nsteps,
                      const double* traj, const double* target,
                      double* grad_k, double* grad_u0, double* j_out,
                      int nthreads);

/* The same adjoint for a border that is reset to a fixed value every step
 * (the Dirichlet border of the plain heat problem, Dirichlet.hpp:125-131)
 * instead of held at u0's values: u0's border values enter only the first
 * step, so dJ/du0 on border nodes is that step's part alone; inner nodes
 * and dJ/dk are unchanged (the border values themselves are the same). */
int orc_kheat_adjoint_reset(const orc_grid* g, const double* k, int nsteps,
                            const double* traj, const double* target,
                            double* grad_k, double* grad_u0, double* j_out,
                            int nthreads);

/* Lame-Navier elastic wave, leapfrog in time (no reference counterpart that
 * runs: examples/LameNavierEqnFDM/LameNavierEqnFDM.hpp:23-25 states the
 * reference cannot advance it).  u and uprev hold 3 components of n nodes
 * each (component-major); inner nodes:
 *   u_new_c = 2 u_c - uprev_c + tau^2/rho [ (lambda+2mu) d_cc u_c
 *             + mu sum_{p!=c} d_pp u_c + (lambda+mu) sum_{q!=c} d_cq u_q ]
 * with central second differences and the 4-point mixed difference
 * d_pq f = (f(+p+q) - f(+p-q) - f(-p+q) + f(-p-q)) / (4 h_p h_q);
 * border nodes are held at 0.  On exit u is step nsteps, uprev step
 * nsteps-1. */
int orc_lame(const orc_grid* g, double lambda, double mu, double rho, int nsteps,
             double* u, double* uprev, int nthreads);

/* Yee FDTD in a PEC box, eps = mu = 1 scaled (see orc_yee in the .c file
 * for the staggering).  f holds Ex, Ey, Ez, Hx, Hy, Hz (n nodes each).
 * Each step: H half step, E step, then the soft current source
 * Ez[src] -= tau * J(time), J(t) = amp * exp(-((t - t0)/w)^2) sin(2 pi freq t). */
int orc_yee(const orc_grid* g, int nsteps, double* f, int src_i, int src_j, int src_k,
            double amp, double t0, double w, double freq, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
