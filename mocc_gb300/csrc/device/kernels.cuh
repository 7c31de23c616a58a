// Device data views and kernel launchers for one 2-D eigenvalue solve.
//
// Layout in HBM (per solve):
//   segments      seg_len[n_seg] (Real) + seg_fsr[n_seg] (int32), tracks
//                 contiguous, tracks grouped by track set (azimuth)
//   flux          phi[G][n_fsr] (FP64), group-major so a group sweep touches
//                 one contiguous slice
//   boundary psi  psi_in[G][bc_per_group] (Real); one angle's entries are the
//                 x-face then y-face boundary indices of its tracks
//   coarse data   current/surface flux [G][n_surf] (FP64), pin flux [G][n_pin]
#pragma once

#include <cstdint>

#include "common.cuh"

namespace mocgpu {

constexpr int kExpN = 10000;       // table intervals on [-10, 0]
constexpr int kMaxPolar = 4;

struct SetPolar {
    int ang_fwd, ang_bwd; // angle indices (octants 1-4) swept forward/backward
    double rsin;          // 1 / sin(theta)
    double wt;            // weight * spacing * plane height * sin(theta) * pi
    double cw[2], fw[2];  // current and surface-flux weights for X/Y crossings
};

struct GeomView {
    int G, n_fsr, n_mat, n_tracks, n_sets, pol, n_ang, ndir_oct;
    int nx, ny, n_pin, n_surf, bc_per_group;
    double hz;
    const int64_t *seg_begin; // n_tracks + 1
    const int *trk_bc0, *trk_bc1, *trk_set;
    const void *seg_len; // Real
    const int *seg_fsr;
    const int *fsr_mat;
    const double *fsr_vol, *fsr_area;
    const double *xstr, *xsnf, *xsf, *xsch, *scat; // per material
    const SetPolar *sp;                             // [n_sets * pol]
    const int *bc_off;                              // [n_ang]
    const int *set_ny;                              // [n_sets]
    const int *wt_tgt; // [n_ang*2] reflect targets (-1 vacuum), [n_ang] x-face sizes, [n_ang*2] target bases
    const int *ev_fw_begin, *ev_fw_pt, *ev_fw_code; // forward crossing events
    const int *ev_bw_begin, *ev_bw_pt, *ev_bw_code; // backward crossing events
    const double *exp_tab;                          // kExpN + 1 entries
    const int *pin_first_reg, *pin_cell;            // pins in FSR order
    const double *pin_area;
    const int *pin_fuel;
};

struct StateView {
    double *phi, *phi_old, *fs, *src1g;
    void *qbar, *sigt, *tally; // Real
    void *psi_in, *psi_out;    // Real
    double *cur, *sflux;       // [G][n_surf]
    double *red;               // reduction scratch (64 doubles)
    unsigned *status;
};

// CMFD (coarse mesh finite difference) working set, all FP64.
struct CmfdView {
    int G, nx, ny, n_cell, n_surf;
    double hz;
    const double *dx, *dy;
    int bc[6];
    double *flux;                                 // [G][n_cell]
    double *xstr, *xsnf, *xsf, *xsch, *xsrm;      // [cell][G]
    double *scat;                                 // [cell][G][G] (to, from)
    double *d_tilde, *d_hat, *s_tilde, *s_hat;    // [G][n_surf]
    double *mat;                                  // [G][6][n_cell]: diag, W, E, S, N, 1/diag
    double *fs, *fs_old, *vec;                    // vec: 10 * n_cell work vectors
    const double *cur, *sflux;                    // [G][n_surf] from the sweep
    int has_radial;
    double k_tol, psi_tol, resid_reduction;
    int max_iter, fixup;
    double *k;      // in/out
    double *stats;  // [0]=iterations, [1]=r0, [2]=ri/r0, [3]=psi_err, [4]=bicgstab its
    unsigned *status;
};

// Bundled work-unit layout of the fast sweep (see host/layout.hpp).
struct WorkUnitDev {
    int set, bundle_begin, n_bundles, fsr_begin, n_local;
};
struct FastView {
    const WorkUnitDev *wu;
    const int64_t *bundle_row;
    const int *bundle_nrows, *bundle_track;
    const void *len; // Real [rows][32]
    const uint16_t *lfsr;
    const int *local_fsr;
    int bundles_per_unit; // warps per CTA = bundles_per_unit * (split ? 2 : 1)
    int split;            // forward and backward on separate warps
    int max_local;
};

// ---- launchers (stream-ordered) ----
template <typename Real>
void launch_sweep_fast(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       bool gs, bool currents, cudaStream_t s);
template <typename Real> size_t fast_sweep_smem(const FastView &fv);
void launch_fill(double *p, double v, int64_t n, cudaStream_t s);
template <typename Real> void launch_fill_real(Real *p, double v, int64_t n, cudaStream_t s);
void launch_fission_source(const GeomView &g, const StateView &st, double k, cudaStream_t s);
void launch_total_fission(const GeomView &g, const double *phi, double *out, cudaStream_t s);
template <typename Real> void launch_group_source(const GeomView &g, const StateView &st, int group, cudaStream_t s);
template <typename Real>
void launch_sweep(const GeomView &g, const StateView &st, int group, int t0, int t1, bool gs, bool currents,
                  cudaStream_t s);
template <typename Real> void launch_jacobi_update(const GeomView &g, const StateView &st, int group, cudaStream_t s);
template <typename Real>
void launch_sweep_epilogue(const GeomView &g, const StateView &st, int group, bool update_q, cudaStream_t s);
void launch_zero_radial_currents(const GeomView &g, const StateView &st, int group, cudaStream_t s);
void launch_normalize_currents(const GeomView &g, const StateView &st, int group, const double *surf_area,
                               cudaStream_t s);
void launch_pin_flux(const GeomView &g, const double *phi, double *cflux, cudaStream_t s);
void launch_set_pin_flux(const GeomView &g, double *phi, const double *cflux, double *resid, unsigned *status,
                         cudaStream_t s);
void launch_homogenize(const GeomView &g, const double *phi, const CmfdView &c, cudaStream_t s);
void launch_cmfd_solve(const CmfdView &c, cudaStream_t s);
void launch_psi_error(const GeomView &g, const double *fs, const double *fs_prev, double *red, cudaStream_t s);
void launch_flux_residual(const GeomView &g, const StateView &st, double *out, cudaStream_t s);
void launch_pin_power(const GeomView &g, const double *phi, double *pow, cudaStream_t s);
void set_exp_constants(double min, double space, double rspace);
int64_t launch_count();

} // namespace mocgpu
