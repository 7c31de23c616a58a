/*
 * CPU oracle: an FP64 restatement of MOCC's 2-D MoC eigenvalue path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the GPU
 * library (tests/, the smoke check and the benchmark's CPU baseline use
 * it); no product code path links, loads or calls it.
 *
 * It restates these MOCC routines on a flat problem (tracks, quadrature,
 * cross sections) that it builds itself from the input text (tracer.cpp:
 * XML and .xsl reading, core mesh, quadrature, modular ray tracing) or,
 * for unit checks, takes from the library it checks:
 *   sweep1g                    src/sweepers/moc/moc_sweeper_kernel.inc.hpp:36-180
 *   moc::Current               src/sweepers/moc/moc_current_worker.hpp:137-330
 *   BoundaryCondition          src/core/boundary_condition.cpp:87-191
 *   Exponential_Linear<10000>  src/core/exponential.hpp:56-112
 *   MoCSweeper::sweep, initialize, get/set_pin_flux_1g
 *                              src/sweepers/moc/moc_sweeper.cpp:189-433
 *   Source, SourceIsotropic    src/core/source.cpp:41-112, source_isotropic.cpp:21-57
 *   TransportSweeper reductions src/core/transport_sweeper.cpp:104-223
 *   XSMeshHomogenized::update  src/core/xs_mesh_homogenized.cpp:176-363
 *   CMFD                       src/core/cmfd.cpp:171-666 (Eigen's BiCGSTAB restated
 *                              as preconditioned BiCGSTAB with a diagonal
 *                              preconditioner, see oracle.cpp)
 *   EigenSolver, FixedSourceSolver
 *                              src/solvers/eigen_solver.cpp:131-291,
 *                              src/solvers/fixed_source_solver.cpp:102-117
 */
#ifndef MOCC_ORACLE_H
#define MOCC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem {
    int ng, n_fsr, n_mat, ndir_oct, n_ang, n_sets, pol_per_set;
    int nx, ny, n_pin, n_surf, n_fuel_2d, n_tracks;
    int64_t n_seg;
    double hz;
    int bc[6];
    const double *xstr, *xsnf, *xsf, *xsch, *scat;
    const int *fsr_mat;
    const double *fsr_vol, *fsr_area;
    const double *ang_ox, *ang_oy, *ang_oz, *ang_alpha, *ang_theta, *ang_weight, *ang_rsintheta;
    const int *set_nx, *set_ny, *set_first_track;
    const double *set_spacing;
    const int *trk_bc0, *trk_bc1, *trk_set;
    const int64_t *trk_seg_begin;
    const int *trk_cm_cell_fw, *trk_cm_cell_bw, *trk_cm_surf_fw, *trk_cm_surf_bw, *trk_cm_begin;
    const int *cm_fw, *cm_bw, *cm_nseg_fw, *cm_nseg_bw;
    const double *seg_len;
    const int *seg_fsr;
    const double *dx, *dy;
    const int *pin_first_reg, *pin_cell, *pin_fuel;
    const double *pin_area;
} orc_problem;

typedef struct orc_options {
    double k_tol, psi_tol;
    int max_iter, min_iter;
    int cmfd, cmfd_enabled;
    double cmfd_k_tol, cmfd_psi_tol, cmfd_resid_reduction;
    int cmfd_max_iter, cmfd_negative_fixup;
    int n_inner, gs_boundary, precision;
    int incoming_update; /* 0 off, 1 MoCSweeper::update_incoming_flux as written, 2 entry-surface variant */
    int tl_splitting;    /* MoCSweeper's allow_splitting_ (<sweeper tl_splitting>) */
} orc_options;

typedef struct orc_result {
    double k;
    int iterations;
    int converged;
    double error_k, error_psi;
    double seconds;
    int64_t sweeps;
    int64_t cmfd_iterations;
} orc_result;

typedef struct orc_solver orc_solver;

const char *orc_last_error(void);
/* n_threads <= 0: all available OpenMP threads */
int orc_create(const orc_problem *p, const orc_options *o, int n_threads, orc_solver **out);
void orc_destroy(orc_solver *s);
int orc_threads(orc_solver *s);
int orc_initialize(orc_solver *s);
int orc_set_coarse_data(orc_solver *s, int enabled);
int orc_calc_fission_source(orc_solver *s, double k, double *fs);
int orc_set_fission_source(orc_solver *s, const double *fs);
int orc_store_old_flux(orc_solver *s);
int orc_source_group(orc_solver *s, int g);
int orc_sweep_group(orc_solver *s, int g);
int orc_total_fission(orc_solver *s, int old, double *out);
int orc_flux_residual(orc_solver *s, double *out);
int orc_get_flux(orc_solver *s, double *flux);
int orc_set_flux(orc_solver *s, const double *flux);
int orc_get_pin_flux_1g(orc_solver *s, int g, double *out);
int orc_set_pin_flux_1g(orc_solver *s, int g, const double *in, double *resid);
int orc_pin_powers(orc_solver *s, double *out);
int orc_get_coarse_currents(orc_solver *s, double *cur, double *sflux);
/* incoming boundary flux of group g (bc_per_group entries; the count alone
 * when out is NULL) */
int orc_get_boundary(orc_solver *s, int g, double *out, int64_t *n);
/* update_incoming_flux from given 2 (J+ + J-) sums, [G][n_surf] (part_old
 * read when has_old), mode 1 (MOCC's lookup) or 2 (entry surface) */
int orc_update_incoming(orc_solver *s, const double *part, const double *part_old, int has_old, int mode);
/* XSMeshHomogenized::update (xs_mesh_homogenized.cpp:176-363) of the current
 * flux; writes the pins' nu-Sigma_f, [n_pin, in FSR order][G] */
int orc_homogenized_nu_fission(orc_solver *s, double *out);
/* The CMFD system of the current state (coarse flux from the pin flux,
 * homogenisation, CMFD::setup_solve, cmfd.cpp:333-553), unsolved: op
 * [G][5][n_cell] (diagonal, west, east, south, north couplings), the
 * homogenised nu-Sigma_f and chi [n_cell][G], scattering [n_cell][G][G]
 * (to, from) and cell volumes [n_cell]. */
int orc_cmfd_system(orc_solver *s, double *op, double *xsnf, double *xsch, double *scat, double *vol);
int orc_cmfd_solve(orc_solver *s, double *k);
int orc_eigen_solve(orc_solver *s, int max_outer, orc_result *out);
/* the last eigen_solve's outer iterations: [n][4] = k, error_k, error_psi,
 * seconds since the solve began (EigenSolver's convergence_ and
 * iteration_times_, eigen_solver.cpp:185-190) */
int orc_history(orc_solver *s, const double **data, int64_t *n);
/* MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472): tl [nreg] */
int orc_apply_transverse_leakage(orc_solver *s, int g, const double *tl);
/* exponential table check: value of MOCC's table exponential at x */
double orc_table_exp(double x);

/* The oracle's own path from input text to the flat problem (tracer.cpp):
 * MOCC's XML input and .xsl library read, the core mesh built, the
 * quadrature modularised and the rays traced. The orc_traced object owns
 * every array the returned orc_problem points to. */
typedef struct orc_traced orc_traced;
const char *orc_trace_error(void);
/* mocc_literal != 0: MOCC's own corner handling of the coarse walk (see
 * tracer.cpp) instead of the rule the checked library follows */
int orc_trace(const char *xml, const char *xsl, int mocc_literal, orc_traced **out);
void orc_traced_destroy(orc_traced *t);
const orc_problem *orc_traced_problem(const orc_traced *t);
const orc_options *orc_traced_options(const orc_traced *t);
/* one named array of the traced problem (the orc_problem field names):
 * *kind 0 int32, 1 double, 2 int64 */
int orc_traced_array(const orc_traced *t, const char *name, const void **data, int64_t *n, int *kind);

#ifdef __cplusplus
}
#endif

#endif
