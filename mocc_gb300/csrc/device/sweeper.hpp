// Device-resident 2-D MoC sweeper with the CMFD-accelerated power iteration.
//
// Mirrors the duties of MOCC's MoCSweeper + FixedSourceSolver + EigenSolver
// + CMFD (src/sweepers/moc/moc_sweeper.cpp, src/solvers/eigen_solver.cpp,
// src/solvers/fixed_source_solver.cpp, src/core/cmfd.cpp) with all arrays in
// HBM and every per-iteration loop a device kernel. The host only sequences
// launches and reads back a handful of scalars per outer iteration.
#pragma once

#include <memory>
#include <vector>

#include "../host/layout.hpp"
#include "../host/problem.hpp"
#include "kernels.cuh"

namespace mocgpu {

struct EigenResult {
    double k = 1.0;
    int iterations = 0;
    int converged = 0;
    double error_k = 0.0, error_psi = 0.0;
    double seconds = 0.0;
    int64_t sweeps = 0;        // one-group sweeps (inner iterations) performed
    int64_t cmfd_iterations = 0;
};

class Sweeper {
  public:
    Sweeper(const Problem &P, int precision, cudaStream_t stream = 0);
    ~Sweeper();
    Sweeper(const Sweeper &) = delete;
    Sweeper &operator=(const Sweeper &) = delete;

    int precision() const { return precision_; }
    const FlatProblem &flat() const { return f_; }
    const SolverOptions &options() const { return opts_; }
    SolverOptions &options() { return opts_; }
    cudaStream_t stream() const { return stream_; }

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
    void set_coarse_enabled(bool on) { coarse_enabled_ = on; }

    // CMFD + eigen solver
    void cmfd_solve(double &k); // EigenSolver::do_cmfd
    EigenResult eigen_solve(int max_outer = -1);
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

    // device memory footprint (bytes)
    size_t device_bytes() const { return dev_bytes_; }
    // sweep-only algorithmic traffic per group sweep (bytes)
    double sweep_bytes() const;

    const GeomView &geom() const { return gv_; }
    const StateView &state() const { return sv_; }

  private:
    template <typename Real> void sweep_impl(int g);
    void check_status();
    void launch_phase(int g, int phase, bool gs, bool cur);
    void launch_epilogue(int g, bool update_q);

    FlatProblem f_;
    SolverOptions opts_;
    int precision_;
    cudaStream_t stream_;
    bool coarse_enabled_ = false;
    bool has_radial_ = false;
    int n_fissile_ = 0;
    int phaseA_end_ = 0; // first track of octant-2 sets
    size_t dev_bytes_ = 0;

    // geometry
    DevBuf<int64_t> seg_begin_;
    DevBuf<int> trk_bc0_, trk_bc1_, trk_set_, seg_fsr_, fsr_mat_, bc_off_, set_ny_, wt_tgt_;
    DevBuf<double> seg_len_d_;
    DevBuf<float> seg_len_f_;
    DevBuf<double> fsr_vol_, fsr_area_, xstr_, xsnf_, xsf_, xsch_, scat_, exp_tab_;
    DevBuf<SetPolar> sp_;
    DevBuf<int> ev_fw_begin_, ev_fw_pt_, ev_fw_code_, ev_bw_begin_, ev_bw_pt_, ev_bw_code_;
    DevBuf<int> pin_first_reg_, pin_cell_, pin_fuel_;
    DevBuf<double> pin_area_, surf_area_, dx_, dy_;
    // state
    DevBuf<double> phi_, phi_old_, fs_, fs_prev_, src1g_, cur_, sflux_, red_;
    DevBuf<unsigned char> qbar_, sigt_, tally_, psi_in_, psi_out_;
    DevBuf<unsigned> status_;
    // CMFD
    DevBuf<double> cflux_, hxs_, hscat_, dtil_, dhat_, stil_, shat_, cmat_, cfs_, cfs_old_, cvec_, ck_, cstats_;
    DevBuf<double> pinbuf_;
    std::vector<double> psi_init_;
    // bundled work-unit layout
    DevBuf<WorkUnitDev> wu_;
    DevBuf<int64_t> bundle_row_;
    DevBuf<int> bundle_nrows_, bundle_track_, local_fsr_;
    DevBuf<float> blen_f_;
    DevBuf<double> blen_d_;
    DevBuf<uint16_t> blfsr_;
    std::vector<int> phase_wu_;
    FastView fv_{};

  public:
    double layout_padding = 0.0;
    int layout_units = 0, layout_max_local = 0, layout_tracks_per_unit = 0;

  private:

    GeomView gv_{};
    StateView sv_{};
    CmfdView cv_{};
};

} // namespace mocgpu
