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
// Cap on the adds one FSR tally of a work unit takes in a group sweep: the
// low words of the FP32 path's fixed-point tally take up to 2^20 per add and
// must not wrap (2048 * 2^20 = 2^31).
constexpr int kMaxTallyHits = 2048;

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
    const int4 *trk_entry; // per track: coarse cell and core-boundary surface where each direction starts (fw cell, bw cell, fw surface, bw surface)
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
    const int2 *ev_fw, *ev_bw;                      // the same events packed as (row, code)
    const double *exp_tab;                          // kExpN + 1 entries
    const int *pin_first_reg, *pin_cell;            // pins in FSR order
    const double *pin_area;
    const int *pin_fuel;
};

// Copies of the FP32 crossing-current tallies. On a small lattice the
// reductions of all concurrent CTAs land on a few hundred surfaces (every
// track starts and ends on the boundary ones) and queue up behind each
// other; spread over copies they queue a copy's share. Measured on the
// 17x17 assembly (FP32): the five inner sweeps of a group, the last one
// tallying currents, took 0.51 ms with one copy and 0.40 ms with eight
// (0.35 ms without the tally). The normalisation folds the copies in a
// fixed order.
constexpr int kCurCopies = 8;

struct StateView {
    double *phi, *phi_old, *fs, *fs_prev, *src1g;
    void *qbar, *sigt, *tally; // Real
    void *psi_in, *psi_out;    // Real
    double *cur, *sflux;       // [G][n_surf]
    // FP32 sweep: the crossing currents and surface fluxes of the group being
    // tallied, [kCurCopies][n_surf] each (native float reductions, CTA b
    // adding into copy b % kCurCopies), folded into cur and sflux by the
    // normalisation and cleared
    float *cur32, *sfl32;
    double *part;              // [2][G][n_surf]: 2 (J+ + J-) of the last CMFD solve and the one before
    // [n_fsr]: Sigma_t added by transverse-leakage splitting (MoCSweeper::
    // split_), nullptr when <sweeper tl_splitting> is off
    double *split;
    double *cflux;             // coarse (pin) flux [G][n_pin]
    double *red;               // per-solve scalars and reduction scratch (64 doubles)
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
    double *red;    // the solve's scalars (batched path reads RED_HAS_RADIAL here)
};

// Bundled work-unit layout of the fast sweep (see host/layout.hpp).
struct WorkUnitDev {
    int set, bundle_begin, n_bundles, win_begin, n_win; // row windows [win_begin, win_begin + n_win)
};
struct FastView {
    const WorkUnitDev *wu;
    const int64_t *bundle_row;
    const int *bundle_nrows, *bundle_track;
    const int2 *bundle_bc; // [bundle][32]: both boundary indices of each lane's track (0 for padding lanes)
    // [bundle][32]: each lane's crossing events, forward [x, y) and backward
    // [z, w) in GeomView::ev_fw / ev_bw (empty for padding lanes), so a warp
    // starting a bundle reaches its first events in one load less
    const int4 *bundle_ev;
    const void *len; // Real [rows][32]
    const uint16_t *lfsr;      // window-local FSR id of every row entry
    const int *local_fsr;      // window tables: window-local -> plane FSR ids
    const int2 *win;           // per row window: (first entry in local_fsr, FSRs)
    int window_rows;           // rows per window of units with several windows
    int table_slots;           // FSR slots of one window table (the largest + its padding slot)
    int bundles_per_unit; // warps per CTA = 2 * bundles_per_unit (forward and backward on separate warps)
    int max_local;             // FSR slots a CTA stages: one table, or two when a unit has several windows
    int max_hits; // most tally adds on one unit FSR in one group sweep (bounds the fixed-point tally)
};

// Per-solve scalars kept in device memory (StateView::red) so that batched
// solves advance without host round trips.
enum RedSlot {
    RED_TFIS = 8,        // total fission scratch
    RED_FLUXRES = 9,     // flux residual scratch
    RED_PINRES = 10,     // set_pin_flux residual scratch
    RED_K = 16,          // k
    RED_K_PREV = 17,     // k of the previous outer
    RED_TF_NEW = 18,     // total fission of the new flux
    RED_TF_OLD = 19,     // total fission of the old flux
    RED_PSI = 20,        // 20..24: fission-source change sums
    RED_ERR_K = 25,      // |k - k_prev|
    RED_ERR_PSI = 26,    // fission-source L2 change
    RED_N_FISSILE = 27,  // fissile FSR count
    RED_HAS_RADIAL = 28, // 1 once the sweep has tallied coarse currents
    RED_CMFD_ITS = 29,   // CMFD iterations accumulated
    // batched solves: the convergence test runs on the device, so the host
    // can keep replays in flight and a finished solve is frozen at once
    RED_DONE = 30,       // 0 while the solve runs, else how it ended (BatchDone)
    RED_ITERS = 31,      // outer iterations done
    RED_K_TOL = 32,      // the solve's <solver k_tol>, psi_tol, min_iter, max_iter
    RED_PSI_TOL = 33,
    RED_MIN_ITER = 34,
    RED_MAX_ITER = 35,
    RED_CMFD_SOLVES = 36 // CMFD solves since admission (the incoming-flux update's "previous currents" test)
};
// How a batched solve ended (RED_DONE and the summary row).
enum BatchDone { DONE_RUNNING = 0, DONE_CONVERGED = 1, DONE_NONPOSITIVE = 2, DONE_NAN = 3, DONE_MAX_ITER = 4,
                 DONE_CANCELLED = 5 };
// Summary row per slot written by the last kernel of a replay: k, error_k,
// error_psi, status, CMFD iterations, coarse-current flag, BatchDone, outer
// iterations.
constexpr int kSummaryStride = 8;

// Arrays of per-solve views for the batched kernels (device memory), and the
// list of active solve slots. The active list and its length live in device
// memory so that one captured graph serves every mix of active solves; grids
// span `cap` solves and blocks past the active count return at once.
struct BatchViews {
    const GeomView *gv;
    const StateView *sv;
    const CmfdView *cv;
    const FastView *fv;
    const double *const *surf_area; // per slot: coarse surface areas
    const int *act;                 // active slots
    const int *n_act;               // number of active slots
    int cap;                        // grid extent over solves
    int max_fsr, max_pin, max_surf, max_cell, max_g;
};

// ---- batched launchers (one solve per blockIdx.y unless noted) ----
void launch_b_fission_source(const BatchViews &b, cudaStream_t s);
void launch_b_copy_old(const BatchViews &b, cudaStream_t s); // fs_prev = fs, phi_old = phi
template <typename Real> void launch_b_group_source(const BatchViews &b, int group, cudaStream_t s);
template <typename Real> void launch_b_epilogue(const BatchViews &b, int group, bool update_q, cudaStream_t s);
void launch_b_zero_currents(const BatchViews &b, int group, cudaStream_t s);
void launch_b_normalize_currents(const BatchViews &b, int group, cudaStream_t s);
void launch_b_pin_flux(const BatchViews &b, cudaStream_t s);
void launch_b_homogenize(const BatchViews &b, cudaStream_t s);
void launch_b_set_pin_flux(const BatchViews &b, cudaStream_t s);
void launch_b_k_update(const BatchViews &b, cudaStream_t s); // total fission ratio, k, then fs(k)
void launch_b_errors(const BatchViews &b, cudaStream_t s);   // error_k, error_psi per solve
// Convergence test of every running solve (eigen_solver.cpp:213: k_tol,
// psi_tol, min_iter; max_iter; non-positive pin flux and NaN end a solve with
// an error) and its summary row out[slot * kSummaryStride + ...]. Solves that
// end are frozen: every batched kernel skips them from the next replay on.
void launch_b_retire(const BatchViews &b, double *out, cudaStream_t s);
void launch_b_cmfd(const BatchViews &b, cudaStream_t s);
// MoCSweeper::update_incoming_flux after each solve's CMFD (mode 1 or 2 as
// for launch_incoming_update); counts the CMFD solves of each solve.
void launch_b_incoming_update(const BatchViews &b, int precision, int mode, cudaStream_t s);
// MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472): adds the
// transverse leakage tl [n_fsr] to the group source, with splitting when
// st.split is set; then the group's qbar and Sigma_t as the next sweep uses
// them.
template <typename Real>
void launch_apply_transverse_leakage(const GeomView &g, const StateView &st, int group, const double *tl,
                                     cudaStream_t s);
// pin powers of every active solve: out[slot * stride + cell], total at n_pin
void launch_b_pin_powers(const BatchViews &b, double *out, int stride, cudaStream_t s);
// Batched sweep (Gauss-Seidel boundary update) in streaming shape `shape`:
// rows per chunk and chunks in flight of each warp's segment ring, one of
// kSweepShapeCount built shapes (FP64: shape 0 only). cur: 0 no coarse
// tallies, 1 net currents and surface fluxes (the incoming-flux update reads
// the surface fluxes), 2 net currents only.
template <typename Real>
void launch_b_sweep(const BatchViews &b, const int2 *items, const int *n_items, int max_items, int group, int cur,
                    int pol, int bundles_per_unit, int max_local, int shape, int *counter, cudaStream_t s);
// Sets the shared-memory limit of the batched sweep ahead of graph capture.
template <typename Real> void prepare_b_sweep(int pol, int bundles_per_unit, int max_local, int shape);
constexpr int kSweepShapeCount = 5;
void sweep_shape_info(int shape, int *rows, int *stages); // throws for a shape that is not built
void note_launches(int64_t n); // adds replayed launches to launch_count()

// ---- launchers (stream-ordered) ----
// currents: 0 none, 1 net currents and surface fluxes, 2 net currents only
// (Gauss-Seidel; a Jacobi sweep tallies both)
template <typename Real>
void launch_sweep_fast(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       bool gs, int currents, cudaStream_t s);
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
// Same solve with the work vectors in a fixed module-scope array (no
// allocation); meshes up to static_cmfd_max_cells() cells, calls must not
// overlap in time on one device.
void launch_cmfd_solve_static(const CmfdView &c, cudaStream_t s);
int static_cmfd_max_cells();
// MoCSweeper::update_incoming_flux from the CMFD solution in c: stores the
// partial currents of every surface (part[G][n_surf], the previous ones to
// part + G * n_surf), then rewrites every track's starting boundary entries
// of psi_in (Real of the precision). mode 1: MOCC's surface lookup, mode 2:
// the track's entry surface; has_old: a previous solve's currents exist.
void launch_incoming_update(const GeomView &gv, const CmfdView &c, void *psi_in, int precision, double *part,
                            int mode, int has_old, cudaStream_t s);
// The second half alone: psi_in rescaled from given partial-current sums.
void launch_apply_incoming(const GeomView &gv, const CmfdView &c, void *psi_in, int precision, const double *part,
                           int mode, int has_old, cudaStream_t s);
void launch_psi_error(const GeomView &g, const double *fs, const double *fs_prev, double *red, cudaStream_t s);
void launch_flux_residual(const GeomView &g, const StateView &st, double *out, cudaStream_t s);
void launch_pin_power(const GeomView &g, const double *phi, double *pow, cudaStream_t s);
void set_exp_constants(double min, double space, double rspace);
int64_t launch_count();
// Kernel attributes are set per device; these set them on the current device
// once per (kernel, attribute) and value, safely from several host threads.
void raise_func_attr(const void *kernel, cudaFuncAttribute attr, int value);
void ensure_smem_limit(const void *kernel, size_t bytes); // dynamic shared memory above 48 KB
void copy_bytes(int64_t *h2d, int64_t *d2h); // host<->device bytes moved so far

} // namespace mocgpu
