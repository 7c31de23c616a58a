// A fully set-up 2-D eigenvalue problem: solver options from the XML input,
// the core mesh, the modularised quadrature, the traced tracks, and a flat
// (structure-of-arrays) view of all of it that both the device upload and
// the CPU oracle consume.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "mesh.hpp"
#include "quadrature.hpp"
#include "rays.hpp"

namespace mocgpu {

// Options of <solver type="eigenvalue">, its <cmfd> and <sweeper type="moc">
// (MOCC: eigen_solver.cpp:31-107, cmfd.cpp:34-150, moc_sweeper.cpp:54-116).
struct SolverOptions {
    double k_tol = 1e-6, psi_tol = 1e-5;
    int max_iter = 100, min_iter = 0;
    bool cmfd = false;
    bool cmfd_enabled = true;
    double cmfd_k_tol = 1e-6, cmfd_psi_tol = 1e-5, cmfd_resid_reduction = 1e-3;
    int cmfd_max_iter = 100;
    bool cmfd_negative_fixup = false;
    int n_inner = 1;
    bool gs_boundary = true; // Gauss-Seidel (default) or Jacobi boundary update
    int precision = 0;       // 0: FP64 sweep, 1: FP32 sweep + FP64 reductions/CMFD
    int sweep_kernel = 1;    // 0: one thread per track (plain), 1: bundled work units
    int bundles_per_unit = 0; // bundled sweep work-unit shape (1..4 bundles of 32 tracks), 0: chosen from the size
    int window_rows = -1;     // bundled sweep: rows staged per window (a multiple of 16), 0 whole units, -1 automatic
    // boundary angular flux update after each CMFD solve
    // (MoCSweeper::update_incoming_flux): 0 off (MOCC's behaviour, its call
    // is disabled), 1 as MOCC's code reads the partial currents, 2 from the
    // partial currents of each track's entry surface
    int incoming_update = 0;
    // MoCSweeper's allow_splitting_ (<sweeper tl_splitting>, moc_sweeper.cpp:
    // 119): a transverse-leakage source that would go negative in an FSR is
    // moved into that FSR's Sigma_t instead (apply_transverse_leakage)
    bool tl_splitting = false;
    // <sweeper dump_fsr_flux> (moc_sweeper.cpp:103): MoCSweeper::output also
    // writes the FSR flux of every group
    bool dump_fsr_flux = false;
};

// Flat problem description. Angles cover octants 1-4 (2-D); tracks are
// grouped by track set (octants 1-2); segment FSR indices are plane-global.
struct FlatProblem {
    int ng = 0, n_fsr = 0, n_mat = 0;
    int ndir_oct = 0, n_ang = 0; // n_ang = 4 * ndir_oct
    int n_sets = 0, pol_per_set = 1;
    int nx = 0, ny = 0, n_pin = 0, n_surf = 0, n_fuel_2d = 0;
    double hz = 1.0;
    int bc[6] = {0, 0, 0, 0, 0, 0};
    int n_tracks = 0;
    int64_t n_seg = 0;
    int max_seg = 0;

    // materials, dense order [mat][g] and [mat][to][from]
    std::vector<double> xstr, xsnf, xsf, xsch, scat;
    // FSRs
    std::vector<int> fsr_mat;
    std::vector<double> fsr_vol, fsr_area;
    // angles (octants 1-4)
    std::vector<double> ang_ox, ang_oy, ang_oz, ang_alpha, ang_theta, ang_weight, ang_rsintheta;
    // track sets
    std::vector<int> set_nx, set_ny, set_first_track;
    std::vector<double> set_spacing;
    // tracks
    std::vector<int> trk_bc0, trk_bc1, trk_set;
    std::vector<int64_t> trk_seg_begin; // n_tracks + 1
    std::vector<int> trk_cm_cell_fw, trk_cm_cell_bw, trk_cm_surf_fw, trk_cm_surf_bw;
    std::vector<int> trk_cm_begin; // n_tracks + 1
    std::vector<int> cm_fw, cm_bw, cm_nseg_fw, cm_nseg_bw;
    // segments
    std::vector<double> seg_len;
    std::vector<int> seg_fsr;
    // coarse mesh
    std::vector<double> dx, dy;
    std::vector<int> pin_first_reg; // n_pin + 1, pins in FSR order
    std::vector<int> pin_cell, pin_fuel;
    std::vector<double> pin_area;
};

struct Problem {
    SolverOptions opts;
    std::unique_ptr<CoreMesh> mesh;
    std::unique_ptr<RayData> rays;
    FlatProblem flat;

    // xsl_text, when non-empty, replaces the file named by <material_lib path>.
    static std::unique_ptr<Problem> from_xml(const std::string &xml_text, const std::string &xsl_text,
                                             const std::string &base_dir);
};

// Macroscopic cross sections of every assigned material, dense order
// [mat][g] and [mat][to][from] as in FlatProblem.
struct CrossSections {
    int ng = 0;
    std::vector<double> xstr, xsnf, xsf, xsch, scat;
};

CrossSections cross_sections_of(const FlatProblem &f);

// Cross sections for `base`'s material assignment (the <material id name>
// list of its input) read from another .xsl library. The library must have
// the same group count and leave every material's fissile flag unchanged,
// since the fuel-pin map of the traced geometry depends on it.
CrossSections cross_sections_from_xsl(const Problem &base, const std::string &xsl_text);

// Copy of f without the per-track and per-segment arrays (what a solve keeps
// once its geometry lives on the device).
FlatProblem flat_without_tracks(const FlatProblem &f);

} // namespace mocgpu
