/*
 * CPU oracle for the ScaFES explicit update path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-node update sweeps, written
 * operation for operation in the order the reference's callbacks evaluate
 * them, so that the result is bit-identical to the reference built with the
 * same compiler flags (-ffp-contract=off).  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py use it, as the checker; the product
 * library never links it.
 *
 * Step semantics (src/ScaFES_Problem.hpp:2582-2638, 5078-5082, 5419-5466):
 *   - t = 0 is the initial iterate (given by the caller);
 *   - for t = 1..nsteps every node of the new iterate starts as a copy of
 *     the old one, global-inner nodes run updateInner, global-border nodes
 *     (within nLayersAtBorder of a face, :3952-3971) run updateBorder;
 *   - knownDf(i, n) is the known field at time(t), knownDfOld(i, n) the one
 *     at time(t-1), time(t) = t_start + t*tau (:2483-2486, :2519-2541);
 *   - old/new are swapped after each step (:3273-3316).
 */
#include "scafes_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, k, nx, ny) ((size_t)(i) + (size_t)(nx) * ((size_t)(j) + (size_t)(ny) * (size_t)(k)))

static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* src/ScaFES_Grid.hpp:551-553: h_p = (last_p - first_p)/(n_p - 1). */
void orc_grid_init(orc_grid* g, int dim, const int* n, const double* first,
                   const double* last, double tau, double t_start,
                   int n_layers)
{
    memset(g, 0, sizeof(*g));
    g->dim = dim;
    for (int p = 0; p < 3; ++p) {
        g->n[p] = (p < dim) ? n[p] : 1;
        g->first[p] = (p < dim) ? first[p] : 0.0;
        g->last[p] = (p < dim) ? last[p] : 0.0;
        g->h[p] = (p < dim && g->n[p] > 1)
                      ? (g->last[p] - g->first[p]) / (g->n[p] - 1)
                      : 0.0;
    }
    g->tau = tau;
    g->t_start = t_start;
    g->n_layers = n_layers;
}

/* src/ScaFES_Problem.hpp:2483-2486. */
double orc_time(const orc_grid* g, int timestep)
{
    return g->t_start + timestep * g->tau;
}

/* src/ScaFES_Problem.hpp:3952-3971 (global border: within nLayers of a face). */
int orc_is_border(const orc_grid* g, int i, int j, int k)
{
    const int idx[3] = {i, j, k};
    for (int p = 0; p < g->dim; ++p) {
        if (idx[p] < g->n_layers || idx[p] > g->n[p] - 1 - g->n_layers)
            return 1;
    }
    return 0;
}

/* src/ScaFES_Grid.hpp:721-733. */
void orc_coords(const orc_grid* g, int i, int j, int k, double* x)
{
    const int idx[3] = {i, j, k};
    for (int p = 0; p < 3; ++p) x[p] = g->first[p] + g->h[p] * idx[p];
}

static double known_at(orc_known kf, size_t m, double time)
{
    if (!kf.base) return 0.0;
    if (kf.form == 1) {
        double v = kf.base[m];
        v *= kf.a;
        double tmp = kf.base[m];
        tmp *= (1.0 + time);
        v += kf.b * tmp;
        return v;
    }
    if (kf.form == 3) {
        /* tests/system/PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin/
         * TimeLinSpaceLin.hpp evalBorder, radiation nodes:
         * G = ((1 + sum x)(1 + t))^4 * (SIGMA*EPSILON) + LAMBDA*(1+t)
         * with base = 1 + sum x, a = SIGMA*EPSILON, b = LAMBDA. */
        double v = kf.base[m];
        v *= (1.0 + time);
        v = v * v * v * v;
        v *= kf.a;
        v += kf.b * (1.0 + time);
        return v;
    }
    if (kf.form == 2) {
        /* tests/system/HeatEqnFDM/Cauchy/TimeLinSpaceLin/TimeLinSpaceLin.hpp
         * evalBorder, flux nodes: G = (1 + sum x) * (ALPHA*(1+t))
         * + LAMBDA*(1+t) with base = 1 + sum x, a = ALPHA, b = LAMBDA. */
        double v = kf.base[m];
        v *= kf.a * (1.0 + time);
        v += kf.b * (1.0 + time);
        return v;
    }
    return kf.base[m] * (kf.a + kf.b * time);
}

static size_t n_total(const orc_grid* g)
{
    return (size_t)g->n[0] * g->n[1] * g->n[2];
}

/* The sweeps of orc_heat_dirichlet on the caller's two fields: iterate t
 * is in u for even t and in w for odd t. */
static void heat_dirichlet_pp(const orc_grid* g, double coeff_a, double rho_c,
                              double perf_q1, double perf_w, int nsteps, double* u,
                              double* w, orc_known f_src, orc_known g_bdry, int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const int use_perf = (perf_q1 != 0.0 || perf_w != 0.0);
    const long sx = 1, sy = nx, sz = (long)nx * ny;
    const long stride[3] = {sx, sy, sz};
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
        const double t_new = orc_time(g, t);
        const double t_old = orc_time(g, t - 1);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, k, nx, ny);
                    if (orc_is_border(g, i, j, k)) {
                        /* Dirichlet.hpp:125-131: vNew = knownDf(1) (time t). */
                        un[m] = known_at(g_bdry, m, t_new);
                        continue;
                    }
                    /* HeatEqnFDM.hpp:207-217 / PennesBioheatEqnFDM.hpp:155-167 */
                    double v = uo[m];
                    for (int p = 0; p < g->dim; ++p) {
                        const double s = uo[m - stride[p]] + uo[m + stride[p]] - 2.0 * uo[m];
                        v += g->tau * coeff_a * s / (g->h[p] * g->h[p]);
                    }
                    if (use_perf) v -= g->tau * perf_q1 * perf_w * uo[m];
                    v += g->tau * (1.0 / rho_c) * known_at(f_src, m, t_old);
                    un[m] = v;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
}

int orc_heat_dirichlet(const orc_grid* g, double coeff_a, double rho_c,
                       double perf_q1, double perf_w, int nsteps, double* u,
                       orc_known f_src, orc_known g_bdry, int nthreads)
{
    const size_t nn = n_total(g);
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    heat_dirichlet_pp(g, coeff_a, rho_c, perf_q1, perf_w, nsteps, u, w, f_src, g_bdry, nthreads);
    if (nsteps % 2 == 1) memcpy(u, w, nn * sizeof(double));
    free(w);
    return 0;
}

int orc_heat_dirichlet_ws(const orc_grid* g, double coeff_a, double rho_c,
                          double perf_q1, double perf_w, int nsteps, double* u,
                          double* w, orc_known f_src, orc_known g_bdry, int nthreads)
{
    if (!u || !w || nsteps < 0) return -2;
    heat_dirichlet_pp(g, coeff_a, rho_c, perf_q1, perf_w, nsteps, u, w, f_src, g_bdry, nthreads);
    return 0;
}

void orc_first_touch(double* a, size_t n, int nthreads)
{
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)((n + 4095) / 4096); ++k) {
        const size_t lo = (size_t)k * 4096, hi = lo + 4096 < n ? lo + 4096 : n;
        for (size_t m = lo; m < hi; ++m) a[m] = 0.0;
    }
}

/* kind 0 Neumann, 1 Cauchy (alpha), 2 Radiation (epsilon, sigma). */
static int heat_flux_impl(const orc_grid* g, double coeff_a, double rho_c, double perf_q1,
                          double perf_w, double lambda, double alpha, double epsilon,
                          double sigma, int kind, int nsteps, double* u, orc_known f_src,
                          orc_known g_dir, orc_known g_flux, int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const int nn3[3] = {nx, ny, nz};
    const size_t nn = n_total(g);
    if (kind < 0 || kind > 2) return -2;
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    const int use_perf = (perf_q1 != 0.0 || perf_w != 0.0);
    const long stride[3] = {1, nx, (long)nx * ny};
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
        const double t_new = orc_time(g, t);
        const double t_old = orc_time(g, t - 1);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, k, nx, ny);
                    const int idx[3] = {i, j, k};
                    if (!orc_is_border(g, i, j, k)) {
                        /* HeatEqnFDM.hpp:207-217 / PennesBioheatEqnFDM.hpp:155-167 */
                        double v = uo[m];
                        for (int p = 0; p < g->dim; ++p) {
                            const double s = uo[m - stride[p]] + uo[m + stride[p]] - 2.0 * uo[m];
                            v += g->tau * coeff_a * s / (g->h[p] * g->h[p]);
                        }
                        if (use_perf) v -= g->tau * perf_q1 * perf_w * uo[m];
                        v += g->tau * (1.0 / rho_c) * known_at(f_src, m, t_old);
                        un[m] = v;
                        continue;
                    }
                    /* Neumann.hpp / Cauchy.hpp / Radiation.hpp updateBorder: an
                     * index 0 in any direction -> Dirichlet knownDf(1) (time t). */
                    int at_min = 0;
                    for (int p = 0; p < g->dim; ++p)
                        if (idx[p] == 0) at_min = 1;
                    if (at_min) {
                        un[m] = known_at(g_dir, m, t_new);
                        continue;
                    }
                    /* Otherwise the inner update with, in each direction of a
                     * max face, the missing neighbour replaced by the inner one
                     * and the flux term of knownDfOld(1). */
                    const double gold = known_at(g_flux, m, t_old);
                    double v = uo[m];
                    for (int p = 0; p < g->dim; ++p) {
                        const double hp = g->h[p];
                        double s;
                        if (idx[p] == nn3[p] - 1) {
                            const double um = uo[m];
                            if (kind == 0)
                                s = uo[m - stride[p]] + uo[m - stride[p]] - ((2.0 * hp / lambda) * gold)
                                    - 2.0 * uo[m];
                            else if (kind == 2)
                                /* Radiation.hpp:146-159 */
                                s = uo[m - stride[p]] + uo[m - stride[p]]
                                    - ((2.0 * hp / lambda) * epsilon * sigma * um * um * um * um)
                                    + ((2.0 * hp / lambda) * gold) - 2.0 * um;
                            else
                                s = uo[m - stride[p]] + uo[m - stride[p]]
                                    - ((2.0 * hp / lambda) * alpha * uo[m])
                                    + ((2.0 * hp / lambda) * gold) - 2.0 * uo[m];
                        } else {
                            s = uo[m - stride[p]] + uo[m + stride[p]] - 2.0 * uo[m];
                        }
                        v += g->tau * coeff_a * s / (hp * hp);
                    }
                    if (use_perf) v -= g->tau * perf_q1 * perf_w * uo[m];
                    v += g->tau * (1.0 / rho_c) * known_at(f_src, m, t_old);
                    un[m] = v;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

int orc_heat_flux(const orc_grid* g, double coeff_a, double rho_c, double perf_q1,
                  double perf_w, double lambda, double alpha, int kind, int nsteps,
                  double* u, orc_known f_src, orc_known g_dir, orc_known g_flux,
                  int nthreads)
{
    if (kind != 0 && kind != 1) return -2;
    return heat_flux_impl(g, coeff_a, rho_c, perf_q1, perf_w, lambda, alpha, 0.0, 0.0, kind,
                          nsteps, u, f_src, g_dir, g_flux, nthreads);
}

int orc_heat_radiation(const orc_grid* g, double coeff_a, double rho_c, double perf_q1,
                       double perf_w, double lambda, double epsilon, double sigma, int nsteps,
                       double* u, orc_known f_src, orc_known g_dir, orc_known g_flux,
                       int nthreads)
{
    return heat_flux_impl(g, coeff_a, rho_c, perf_q1, perf_w, lambda, 0.0, epsilon, sigma, 2,
                          nsteps, u, f_src, g_dir, g_flux, nthreads);
}

int orc_pennes_mri(const orc_grid* g, double rho, double c, double k,
                   double rho_b, double c_b, double omega, double t_blood,
                   const double* q, const double* g_bdry, int nsteps,
                   double* u, int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t nn = n_total(g);
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    const long stride[3] = {1, nx, (long)nx * ny};
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int kk = 0; kk < nz; ++kk) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, kk, nx, ny);
                    if (orc_is_border(g, i, j, kk)) {
                        un[m] = g_bdry ? g_bdry[m] : 0.0;
                        continue;
                    }
                    /* MRIDataPBHEqnFDM.hpp:156-168 */
                    double v = uo[m];
                    for (int p = 0; p < g->dim; ++p) {
                        v += g->tau * (k / (rho * c))
                             * (uo[m - stride[p]] + uo[m + stride[p]] - 2.0 * uo[m])
                             / (g->h[p] * g->h[p]);
                    }
                    v += g->tau * ((rho_b * c_b) / (rho * c)) * omega * (t_blood - uo[m]);
                    v += g->tau * (1.0 / (rho * c)) * (q ? q[m] : 0.0);
                    un[m] = v;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

/* One flux term of the reference's tissue examples in direction p at a
 * border node: the bracket (...) / (h*h) of MRIDataPBHEqnFDM.hpp:189-262
 * and TumorHeatEqnFDM.hpp:303-346, with the missing neighbour replaced. */
static double tissue_bracket(const orc_grid* g, const orc_tissue* ts, const double* uo, size_t m,
                             long sp, int p, int at_min, int at_max, double k, double v_partial)
{
    const double h = g->h[p];
    const double u = uo[m];
    if (at_max) {
        const double a = uo[m - sp];
        if (p == g->dim - 1) {
            if (ts->zmax_kind == 1) {
                /* TumorHeatEqnFDM.hpp:307-317: Cauchy. */
                return ((a + a) - ((2.0 * h / k) * ts->h_conv * (u - ts->t_amb))) - 2.0 * u;
            }
            if (ts->surface && (int)ts->surface[m] == 1) {
                /* MRIDataPBHEqnFDM.hpp:197-217: open skull, Cauchy and
                 * radiation; the radiated temperature is the partially
                 * updated vNew of this node. */
                const double tempOld = v_partial + 273.15;
                const double tempOldPow4 = tempOld * tempOld * tempOld * tempOld;
                const double tempAmb = ts->t_amb + 273.15;
                const double tempAmbPow4 = tempAmb * tempAmb * tempAmb * tempAmb;
                return (((a + a) - ((2.0 * h / k) * ts->h_conv * (u - ts->t_amb)))
                        - ((2.0 * h / k) * ts->epsilon * ts->sigma * (tempOldPow4 - tempAmbPow4)))
                       - 2.0 * u;
            }
            /* MRIDataPBHEqnFDM.hpp:219-229: closed skull, Neumann. */
            return ((a + a) - ((2.0 * h / k) * (-1.0 * ts->q_skull))) - 2.0 * u;
        }
        /* Neumann at the other max faces. */
        return ((a + a) - ((2.0 * h / k) * (-1.0 * ts->q_bc))) - 2.0 * u;
    }
    if (at_min) {
        /* Neumann at the min faces (MRIDataPBHEqnFDM.hpp:244-253). */
        const double b = uo[m + sp];
        return ((b + ((2.0 * h / k) * ts->q_bc)) + b) - 2.0 * u;
    }
    return (uo[m - sp] + uo[m + sp]) - 2.0 * u;
}

int orc_pennes_tissue(const orc_grid* g, const orc_tissue* ts, int nsteps, double* u,
                      int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const int nn3[3] = {nx, ny, nz};
    const size_t nn = n_total(g);
    if (!ts || !ts->rho || !ts->c || !ts->k || !ts->rho_b || !ts->c_b || !ts->omega || !ts->t_blood)
        return -2;
    if (ts->border == 1 && !ts->g_bdry) return -2;
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    const long stride[3] = {1, nx, (long)nx * ny};
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int kk = 0; kk < nz; ++kk) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, kk, nx, ny);
                    const int idx[3] = {i, j, kk};
                    const int border = orc_is_border(g, i, j, kk);
                    if (border && ts->border == 1) {
                        un[m] = ts->g_bdry[m];
                        continue;
                    }
                    /* MRIDataPBHEqnFDM.hpp:147-154 (TumorHeatEqnFDM.hpp:
                     * 234-252 with the tissue constants in every node). */
                    const double rho = ts->rho[m], c = ts->c[m], k = ts->k[m];
                    const double rho_blood = ts->rho_b[m], c_blood = ts->c_b[m];
                    const double omega = ts->omega[m], T_blood = ts->t_blood[m];
                    const double q = ts->q ? ts->q[m] : 0.0;
                    double v = uo[m];
                    for (int p = 0; p < g->dim; ++p) {
                        double br;
                        if (!border) {
                            br = uo[m - stride[p]] + uo[m + stride[p]] - 2.0 * uo[m];
                        } else {
                            br = tissue_bracket(g, ts, uo, m, stride[p], p, idx[p] == 0,
                                                idx[p] == nn3[p] - 1, k, v);
                        }
                        v += g->tau * (k / (rho * c)) * br / (g->h[p] * g->h[p]);
                    }
                    v += g->tau * ((rho_blood * c_blood) / (rho * c)) * omega * (T_blood - uo[m]);
                    v += g->tau * (1.0 / (rho * c)) * q;
                    un[m] = v;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

int orc_stencil_width_one(const orc_grid* g, int nsteps, double* u,
                          int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t nn = n_total(g);
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    const long stride[3] = {1, nx, (long)nx * ny};
    const int ndir = 2 * g->dim;
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const int idx[3] = {i, j, k};
                    const size_t m = IDX(i, j, k, nx, ny);
                    double v = uo[m]; /* copy-before-update */
                    if (!orc_is_border(g, i, j, k)) {
                        /* HeatEqnFdmStencilWidthOne.hpp:124-131 */
                        for (int pp = 0; pp < ndir; ++pp) {
                            const long off = (pp % 2 == 0) ? -stride[pp / 2] : stride[pp / 2];
                            v += uo[m + off];
                        }
                        v *= (2.0 / (2 * g->dim + 1));
                    } else {
                        /* HeatEqnFdmStencilWidthOne.hpp:140-162: at a face in
                         * direction pp, mirror from the opposite neighbour. */
                        const double correction = pow(2.0, t - 1);
                        for (int pp = 0; pp < ndir; ++pp) {
                            const int p = pp / 2;
                            const int at_edge = (pp % 2 == 0) ? (idx[p] == 0) : (idx[p] == g->n[p] - 1);
                            if (at_edge) {
                                const long off = (pp % 2 == 0) ? stride[p] : -stride[p];
                                const double sgn = pow(-1.0, pp);
                                v = uo[m] + uo[m + off] - sgn * correction;
                            }
                        }
                    }
                    un[m] = v;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

int orc_stencil_width_var(const orc_grid* g, int bw, int nsteps, double* u,
                          int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t nn = n_total(g);
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    const long stride[3] = {1, nx, (long)nx * ny};
    set_threads(nthreads);
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const int idx[3] = {i, j, k};
                    const size_t m = IDX(i, j, k, nx, ny);
                    /* HeatEqnFdmStencilWidthVar.hpp:127-163 (inner and border) */
                    double sum = 0.0;
                    int cc = 0;
                    int nadd = 1;
                    for (int p = 0; p < g->dim; ++p) {
                        const int d_start = idx[p];
                        const int d_end = g->n[p] - 1 - idx[p];
                        const int min_s = d_start < bw ? d_start : bw;
                        for (int rr = 1; rr <= min_s; ++rr) {
                            sum += uo[m - rr * stride[p]];
                            cc -= rr;
                        }
                        const int min_e = d_end < bw ? d_end : bw;
                        for (int rr = 1; rr <= min_e; ++rr) {
                            sum += uo[m + rr * stride[p]];
                            cc += rr;
                        }
                        nadd += min_s + min_e;
                    }
                    un[m] = 2.0 + (sum + uo[m] - cc) / nadd;
                }
            }
        }
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

void orc_err_linf(const double* u, const double* exact, size_t n,
                  double* err, double* max_exact)
{
    double e = 0.0, mx = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double d = fabs(u[i] - exact[i]);
        if (d > e || d != d) e = (d != d) ? INFINITY : d;
        const double a = fabs(exact[i]);
        if (a > mx) mx = a;
    }
    *err = e;
    *max_exact = mx;
}

/* ---- Flux-form variable-conductivity heat and its adjoint. ------------- */

static void kheat_step(const orc_grid* g, const double* k, const double* uo,
                       double* un)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const long stride[3] = {1, nx, (long)nx * ny};
#pragma omp parallel for schedule(static)
    for (int kk = 0; kk < nz; ++kk) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const size_t m = IDX(i, j, kk, nx, ny);
                if (orc_is_border(g, i, j, kk)) { un[m] = uo[m]; continue; }
                double v = uo[m];
                for (int p = 0; p < g->dim; ++p) {
                    const double c = g->tau / (g->h[p] * g->h[p]);
                    const double kp = 0.5 * (k[m] + k[m + stride[p]]);
                    const double km = 0.5 * (k[m] + k[m - stride[p]]);
                    v += c * (kp * (uo[m + stride[p]] - uo[m]) - km * (uo[m] - uo[m - stride[p]]));
                }
                un[m] = v;
            }
        }
    }
}

int orc_kheat_forward(const orc_grid* g, const double* k, int nsteps,
                      double* u, double* traj, int nthreads)
{
    const size_t nn = n_total(g);
    double* w = (double*)malloc(nn * sizeof(double));
    if (!w) return -1;
    set_threads(nthreads);
    if (traj) memcpy(traj, u, nn * sizeof(double));
    double* uo = u;
    double* un = w;
    for (int t = 1; t <= nsteps; ++t) {
        kheat_step(g, k, uo, un);
        if (traj) memcpy(traj + (size_t)t * nn, un, nn * sizeof(double));
        double* tmp = uo; uo = un; un = tmp;
    }
    if (uo != u) memcpy(u, uo, nn * sizeof(double));
    free(w);
    return 0;
}

/* Forward-mode automatic differentiation of orc_kheat_forward: every
 * value is a dual number (value, derivative along one direction) and every
 * operation of kheat_step is applied to duals -- the forward vector mode
 * the reference runs through ADOL-C (fov_forward, src/ScaFES_Problem.hpp:
 * 6633-6747), here with one direction and a project-written dual type. */
typedef struct { double v, d; } orc_dual;

static orc_dual dadd(orc_dual a, orc_dual b) { orc_dual r = {a.v + b.v, a.d + b.d}; return r; }
static orc_dual dsub(orc_dual a, orc_dual b) { orc_dual r = {a.v - b.v, a.d - b.d}; return r; }
static orc_dual dmul(orc_dual a, orc_dual b) { orc_dual r = {a.v * b.v, a.d * b.v + a.v * b.d}; return r; }
static orc_dual dconst(double c) { orc_dual r = {c, 0.0}; return r; }

static void kheat_step_dual(const orc_grid* g, const orc_dual* k, const orc_dual* uo, orc_dual* un)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const long stride[3] = {1, nx, (long)nx * ny};
#pragma omp parallel for schedule(static)
    for (int kk = 0; kk < nz; ++kk) {
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const size_t m = IDX(i, j, kk, nx, ny);
                if (orc_is_border(g, i, j, kk)) { un[m] = uo[m]; continue; }
                orc_dual v = uo[m];
                for (int p = 0; p < g->dim; ++p) {
                    const orc_dual c = dconst(g->tau / (g->h[p] * g->h[p]));
                    const orc_dual kp = dmul(dconst(0.5), dadd(k[m], k[m + stride[p]]));
                    const orc_dual km = dmul(dconst(0.5), dadd(k[m], k[m - stride[p]]));
                    v = dadd(v, dmul(c, dsub(dmul(kp, dsub(uo[m + stride[p]], uo[m])),
                                             dmul(km, dsub(uo[m], uo[m - stride[p]])))));
                }
                un[m] = v;
            }
        }
    }
}

int orc_kheat_tangent(const orc_grid* g, const double* k, const double* dk, int nsteps,
                      double* u, double* du, int nthreads)
{
    const size_t nn = n_total(g);
    orc_dual* kd = (orc_dual*)malloc(nn * sizeof(orc_dual));
    orc_dual* a = (orc_dual*)malloc(nn * sizeof(orc_dual));
    orc_dual* b = (orc_dual*)malloc(nn * sizeof(orc_dual));
    if (!kd || !a || !b) { free(kd); free(a); free(b); return -1; }
    set_threads(nthreads);
    for (size_t m = 0; m < nn; ++m) {
        kd[m].v = k[m];
        kd[m].d = dk[m];
        a[m].v = u[m];
        a[m].d = du[m];
    }
    for (int t = 1; t <= nsteps; ++t) {
        kheat_step_dual(g, kd, a, b);
        orc_dual* tmp = a; a = b; b = tmp;
    }
    for (size_t m = 0; m < nn; ++m) {
        u[m] = a[m].v;
        du[m] = a[m].d;
    }
    free(kd); free(a); free(b);
    return 0;
}

static int kheat_adjoint_impl(const orc_grid* g, const double* k, int nsteps,
                              const double* traj, const double* target,
                              double* grad_k, double* grad_u0, double* j_out,
                              int reset_border, int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t nn = n_total(g);
    const long stride[3] = {1, nx, (long)nx * ny};
    double* lam = (double*)malloc(nn * sizeof(double));
    double* lam2 = (double*)malloc(nn * sizeof(double));
    double* lt = (double*)malloc(nn * sizeof(double)); /* lambda masked to inner */
    if (!lam || !lam2 || !lt) { free(lam); free(lam2); free(lt); return -1; }
    set_threads(nthreads);
    const double* uT = traj + (size_t)nsteps * nn;
    double jsum = 0.0;
    for (size_t m = 0; m < nn; ++m) {
        lam[m] = uT[m] - target[m];
        jsum += 0.5 * lam[m] * lam[m];
        grad_k[m] = 0.0;
    }
    for (int t = nsteps - 1; t >= 0; --t) {
        const double* un = traj + (size_t)t * nn; /* state the step t -> t+1 read */
#pragma omp parallel for schedule(static)
        for (int kk = 0; kk < nz; ++kk)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, kk, nx, ny);
                    lt[m] = orc_is_border(g, i, j, kk) ? 0.0 : lam[m];
                }
#pragma omp parallel for schedule(static)
        for (int kk = 0; kk < nz; ++kk) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const int idx[3] = {i, j, kk};
                    const size_t m = IDX(i, j, kk, nx, ny);
                    const int border = orc_is_border(g, i, j, kk);
                    /* lambda_t = M^T lambda_{t+1} */
                    double v = lam[m];
                    double gk = 0.0;
                    for (int p = 0; p < g->dim; ++p) {
                        const double c = g->tau / (g->h[p] * g->h[p]);
                        const int has_m = idx[p] > 0;
                        const int has_p = idx[p] < g->n[p] - 1;
                        const double lm = has_m ? lt[m - stride[p]] : 0.0;
                        const double lp = has_p ? lt[m + stride[p]] : 0.0;
                        const double kpv = has_p ? 0.5 * (k[m] + k[m + stride[p]]) : 0.0;
                        const double kmv = has_m ? 0.5 * (k[m] + k[m - stride[p]]) : 0.0;
                        const double dup = has_p ? un[m + stride[p]] - un[m] : 0.0;
                        const double dum = has_m ? un[m - stride[p]] - un[m] : 0.0;
                        if (border) {
                            /* Held border: its lambda accumulates over all
                             * steps.  Reset border (Dirichlet): the next
                             * border value does not depend on this one, so
                             * only this step's inner neighbours count. */
                            if (reset_border && p == 0) v = 0.0;
                            v += c * (kmv * lm + kpv * lp);
                        } else {
                            v += c * (kpv * (lp - lt[m]) + kmv * (lm - lt[m]));
                        }
                        gk += 0.5 * c * (dup * (lt[m] - lp) + dum * (lt[m] - lm));
                    }
                    lam2[m] = v;
                    grad_k[m] += gk;
                }
            }
        }
        double* tmp = lam; lam = lam2; lam2 = tmp;
    }
    memcpy(grad_u0, lam, nn * sizeof(double));
    *j_out = jsum;
    free(lam); free(lam2); free(lt);
    return 0;
}

int orc_kheat_adjoint(const orc_grid* g, const double* k, int nsteps,
                      const double* traj, const double* target,
                      double* grad_k, double* grad_u0, double* j_out,
                      int nthreads)
{
    return kheat_adjoint_impl(g, k, nsteps, traj, target, grad_k, grad_u0, j_out, 0, nthreads);
}

int orc_kheat_adjoint_reset(const orc_grid* g, const double* k, int nsteps,
                            const double* traj, const double* target,
                            double* grad_k, double* grad_u0, double* j_out,
                            int nthreads)
{
    return kheat_adjoint_impl(g, k, nsteps, traj, target, grad_k, grad_u0, j_out, 1, nthreads);
}

/* ---- Lame-Navier (leapfrog) ------------------------------------------- */

int orc_lame(const orc_grid* g, double lambda, double mu, double rho, int nsteps,
             double* u, double* uprev, int nthreads)
{
    const int nx = g->n[0], ny = g->n[1], nz = g->n[2];
    const size_t nn = n_total(g);
    const long stride[3] = {1, nx, (long)nx * ny};
    double* un = (double*)malloc(3 * nn * sizeof(double));
    if (!un) return -1;
    set_threads(nthreads);
    const double c = g->tau * g->tau / rho;
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k) {
            for (int j = 0; j < ny; ++j) {
                for (int i = 0; i < nx; ++i) {
                    const size_t m = IDX(i, j, k, nx, ny);
                    if (orc_is_border(g, i, j, k)) {
                        for (int cc = 0; cc < 3; ++cc) un[cc * nn + m] = 0.0;
                        continue;
                    }
                    for (int cc = 0; cc < 3; ++cc) {
                        const double* uc = u + cc * nn;
                        double L = 0.0;
                        for (int p = 0; p < 3; ++p) {
                            const double d2 = (uc[m + stride[p]] - 2.0 * uc[m] + uc[m - stride[p]]) / (g->h[p] * g->h[p]);
                            L += (p == cc ? lambda + 2.0 * mu : mu) * d2;
                        }
                        for (int q = 0; q < 3; ++q) {
                            if (q == cc) continue;
                            const double* uq = u + q * nn;
                            const long sp = stride[cc], sq = stride[q];
                            const double dm = (uq[m + sp + sq] - uq[m + sp - sq] - uq[m - sp + sq] + uq[m - sp - sq])
                                              / (4.0 * g->h[cc] * g->h[q]);
                            L += (lambda + mu) * dm;
                        }
                        un[cc * nn + m] = 2.0 * uc[m] - uprev[cc * nn + m] + c * L;
                    }
                }
            }
        }
        memcpy(uprev, u, 3 * nn * sizeof(double));
        memcpy(u, un, 3 * nn * sizeof(double));
    }
    free(un);
    return 0;
}

/* ---- Yee FDTD ----------------------------------------------------------
 * Staggering on an n^3 index grid with spacing h (the grid's h[0]):
 *   Ex(i,j,k) at (i+1/2, j, k)   Hx(i,j,k) at (i, j+1/2, k+1/2)
 *   Ey(i,j,k) at (i, j+1/2, k)   Hy(i,j,k) at (i+1/2, j, k+1/2)
 *   Ez(i,j,k) at (i, j, k+1/2)   Hz(i,j,k) at (i+1/2, j+1/2, k)
 * H update for all cells with the forward neighbours inside; E update for
 * all edges with the backward neighbours inside; tangential E on the
 * boundary faces (and components past the last node) held at 0 (PEC). */
int orc_yee(const orc_grid* g, int nsteps, double* f, int si, int sj, int sk,
            double amp, double t0, double w, double freq, int nthreads)
{
    const int n0 = g->n[0], n1 = g->n[1], n2 = g->n[2];
    const size_t nn = n_total(g);
    double *ex = f, *ey = f + nn, *ez = f + 2 * nn, *hx = f + 3 * nn, *hy = f + 4 * nn, *hz = f + 5 * nn;
    const long sy = n0, sz = (long)n0 * n1;
    const double ch = g->tau / g->h[0];
    set_threads(nthreads);
    for (int t = 1; t <= nsteps; ++t) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n2; ++k)
            for (int j = 0; j < n1; ++j)
                for (int i = 0; i < n0; ++i) {
                    const size_t m = IDX(i, j, k, n0, n1);
                    if (j + 1 < n1 && k + 1 < n2)
                        hx[m] -= ch * ((ez[m + sy] - ez[m]) - (ey[m + sz] - ey[m]));
                    if (i + 1 < n0 && k + 1 < n2)
                        hy[m] -= ch * ((ex[m + sz] - ex[m]) - (ez[m + 1] - ez[m]));
                    if (i + 1 < n0 && j + 1 < n1)
                        hz[m] -= ch * ((ey[m + 1] - ey[m]) - (ex[m + sy] - ex[m]));
                }
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n2; ++k)
            for (int j = 0; j < n1; ++j)
                for (int i = 0; i < n0; ++i) {
                    const size_t m = IDX(i, j, k, n0, n1);
                    if (i + 1 < n0 && j > 0 && j + 1 < n1 && k > 0 && k + 1 < n2)
                        ex[m] += ch * ((hz[m] - hz[m - sy]) - (hy[m] - hy[m - sz]));
                    if (j + 1 < n1 && i > 0 && i + 1 < n0 && k > 0 && k + 1 < n2)
                        ey[m] += ch * ((hx[m] - hx[m - sz]) - (hz[m] - hz[m - 1]));
                    if (k + 1 < n2 && i > 0 && i + 1 < n0 && j > 0 && j + 1 < n1)
                        ez[m] += ch * ((hy[m] - hy[m - 1]) - (hx[m] - hx[m - sy]));
                }
        const double time = orc_time(g, t);
        const double a = (time - t0) / w;
        const double J = amp * exp(-a * a) * sin(2.0 * 3.14159265358979323846 * freq * time);
        ez[IDX(si, sj, sk, n0, n1)] -= g->tau * J;
    }
    return 0;
}
