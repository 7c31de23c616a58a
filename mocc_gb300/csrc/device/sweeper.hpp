// Device-resident 2-D MoC sweeper with the CMFD-accelerated power iteration.
//
// Mirrors the duties of MOCC's MoCSweeper + FixedSourceSolver + EigenSolver
// + CMFD (src/sweepers/moc/moc_sweeper.cpp, src/solvers/eigen_solver.cpp,
// src/solvers/fixed_source_solver.cpp, src/core/cmfd.cpp) with all arrays in
// HBM and every per-iteration loop a device kernel. The host only sequences
// launches and reads back a handful of scalars per outer iteration.
//
// A Sweeper owns the per-solve state (cross sections, scalar and angular
// flux, sources, coarse data, CMFD working set) and shares a DeviceGeometry
// with every other solve of the same traced lattice shape.
#pragma once

#include <memory>
#include <vector>

#include "../host/problem.hpp"
#include "geometry.hpp"
#include "kernels.cuh"

namespace mocgpu {

struct EigenResult {
    double k = 1.0;
    int iterations = 0;
    int converged = 0;
    double error_k = 0.0, error_psi = 0.0;
    double seconds = 0.0;
    int64_t sweeps = 0; // one-group sweeps (inner iterations) performed
    int64_t cmfd_iterations = 0;
};

class Sweeper {
  public:
    // xs, when given, replaces the problem's own cross sections (same
    // material assignment, see cross_sections_from_xsl).
    Sweeper(const Problem &P, int precision, cudaStream_t stream = 0,
            std::shared_ptr<const DeviceGeometry> geo = nullptr, const CrossSections *xs = nullptr);
    ~Sweeper();
    Sweeper(const Sweeper &) = delete;
    Sweeper &operator=(const Sweeper &) = delete;

    // Re-targets this handle (same traced geometry, same materials) at
    // another solve: new options and cross sections, no device allocation.
    void rebind(const Problem &P, const CrossSections *xs = nullptr);

    int precision() const { return precision_; }
    const FlatProblem &flat() const { return f_; }
    const SolverOptions &options() const { return opts_; }
    SolverOptions &options() { return opts_; }
    cudaStream_t stream() const { return stream_; }
    const std::shared_ptr<const DeviceGeometry> &geometry() const { return geo_; }

    // MoCSweeper / TransportSweeper duties
    void initialize();
    void calc_fission_source(double k); // device fission source
    void set_fission_source(const double *host_fs);
    void get_fission_source(double *host_fs);
    void store_old_flux();
    void group_source(int g); // initialize_group + fission + in_scatter
    void sweep(int g);        // n_inner inner iterations of group g
    double total_fission(bool old);
    double flux_residual();
    void get_flux(double *host_flux) const; // [n_fsr][G]
    void set_flux(const double *host_flux);
    void get_pin_flux(int g, double *out) const; // [n_pin] (coarse cell order)
    double set_pin_flux(int g, const double *in);
    void pin_powers(double *out) const; // [ny][nx], normalised to n_fuel
    void get_currents(double *cur, double *sflux) const;
    std::vector<double> get_boundary(int g) const; // incoming boundary psi of group g, as double
    // pin-homogenised cross sections of the current flux, [n_pin][G] and [n_pin][G][G]
    void homogenized_xs(double *xstr, double *xsnf, double *xsf, double *xsch, double *xsrm, double *scat);
    void set_coarse_enabled(bool on) { coarse_enabled_ = on; }
    bool coarse_enabled() const { return coarse_enabled_; }
    bool has_radial() const { return has_radial_; }
    void set_has_radial(bool v) { has_radial_ = v; }

    // CMFD + eigen solver
    void cmfd_solve(double &k); // EigenSolver::do_cmfd
    // cmfd_solve with the CMFD work vectors in the library's fixed scratch
    // array instead of this handle's buffer
    void cmfd_solve_static(double &k);
    // MoCSweeper::update_incoming_flux from partial-current sums computed
    // elsewhere (2 (J+ + J-) per [G][n_surf], this and the previous CMFD solve)
    void update_incoming_flux(const double *part, const double *part_old, int has_old, int mode);
    // MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472), after
    // group_source(g): tl [n_fsr] (host) added to the group source, split
    // into Sigma_t where the sum goes negative when <sweeper tl_splitting>
    void apply_transverse_leakage(int g, const double *tl);
    EigenResult eigen_solve(int max_outer = -1);
    // the last eigen_solve's outer iterations, 4 values each: k, error_k,
    // error_psi, seconds since the solve began (EigenSolver's convergence_
    // and iteration_times_, eigen_solver.cpp:185-190)
    const std::vector<double> &history() const { return history_; }
    void eigen_step(double &k, double &k_prev);
    double psi_error();

    // last CMFD statistics
    double cmfd_stats[5] = {0, 0, 0, 0, 0};
    int64_t sweeps_done = 0;
    int64_t cmfd_iters = 0;

    // Runs `reps` single-inner sweeps of group g; returns the summed device
    // time (ms, CUDA events on the handle's stream) of the sweep kernels only
    // and the number of sweep-kernel launches they took.
    double time_sweep(int g, int reps, int *launches);

    // device memory footprint (bytes): per-solve state plus the geometry
    size_t device_bytes() const { return dev_bytes_ + geo_->bytes(); }
    size_t state_bytes() const { return dev_bytes_; }
    // per-solve device bytes of a solve of f on a geometry with the given
    // boundary-flux entries per group (what the constructor allocates)
    static size_t state_bytes_for(const FlatProblem &f, int precision, int bc_per_group);
    double sweep_bytes() const { return geo_->sweep_bytes(); }
    int n_fissile() const { return n_fissile_; }

    const GeomView &geom() const { return gv_; }
    const StateView &state() const { return sv_; }
    const CmfdView &cmfd_view() const { return cv_; }
    const FastView &fast_view() const { return geo_->fv; }

  private:
    void check_status();
    void launch_phase(int g, int phase, bool gs, int cur); // cur as launch_sweep_fast's currents
    void launch_epilogue(int g, bool update_q);
    void after_cmfd();

    FlatProblem f_;
    SolverOptions opts_;
    int precision_;
    cudaStream_t stream_;
    std::shared_ptr<const DeviceGeometry> geo_;
    bool coarse_enabled_ = false;
    // the last inner sweep tallies surface fluxes with the net currents (as
    // MOCC's current worker does); the library's own eigenvalue iteration
    // clears it unless the incoming-flux update reads them
    bool tally_sflux_ = true;
    std::vector<double> history_;
    bool has_radial_ = false;
    int n_fissile_ = 0;
    int cmfd_solves_ = 0; // CMFD solves since initialize (the first has no previous partial currents)
    size_t dev_bytes_ = 0;

    // cross sections of this solve
    DevBuf<double> xstr_, xsnf_, xsf_, xsch_, scat_;
    // state
    DevBuf<double> phi_, phi_old_, fs_, fs_prev_, src1g_, cur_, sflux_, red_;
    DevBuf<float> cur32_; // FP32 sweep: [2][kCurCopies][n_surf] crossing currents and surface fluxes of one group
    DevBuf<unsigned char> qbar_, sigt_, tally_, psi_in_, psi_out_;
    DevBuf<unsigned> status_;
    // CMFD
    DevBuf<double> cflux_, hxs_, hscat_, dtil_, dhat_, stil_, shat_, cmat_, cfs_, cfs_old_, cvec_, cstats_;
    DevBuf<double> part_; // [2][G][n_surf]: 2 (J+ + J-) of the last CMFD solve, then of the one before
    DevBuf<double> split_, tl_; // [n_fsr]: split Sigma_t (zero until a leakage is applied), leakage staging
    DevBuf<double> pinbuf_;

    GeomView gv_{};
    StateView sv_{};
    CmfdView cv_{};
};

} // namespace mocgpu
