// Device-resident geometry of one traced lattice shape: segment streams (per
// track and in the bundled work-unit layout), track boundary indices, coarse
// crossing events, per-(set, polar) sweep constants, boundary-flux maps,
// pin/FSR maps and the exponential table. Solves whose inputs differ only in
// cross sections share one DeviceGeometry.
#pragma once

#include <memory>
#include <vector>

#include "../host/layout.hpp"
#include "../host/problem.hpp"
#include "kernels.cuh"

namespace mocgpu {

class DeviceGeometry {
  public:
    // bundles_per_unit: bundles of 32 tracks per work unit (CTA); 0 picks it
    // from the number of tracks so that one phase fills the GPU.
    // window_rows: rows of a unit staged at a time by the single-solve kernel
    // (a multiple of 16); 0 whole units (the batched kernel takes only
    // those); -1 automatic: windows of MOCGPU_WINDOW_ROWS rows where they
    // shrink a unit's shared memory well.
    DeviceGeometry(const FlatProblem &f, int precision, int bundles_per_unit = 0, int window_rows = -1);
    DeviceGeometry(const DeviceGeometry &) = delete;
    DeviceGeometry &operator=(const DeviceGeometry &) = delete;

    int precision;
    int G, n_fsr, n_pin, n_surf, n_tracks, n_sets, pol, n_ang, ndir_oct, nx, ny, bc_per_group;
    int64_t n_seg;
    double hz;
    int bc[6];
    int phaseA_end = 0;        // first track of the octant-2 sets
    std::vector<int> phase_wu; // work-unit ranges of the two Gauss-Seidel phases
    std::vector<int> wu_rows;  // segment rows (of 32 lanes) per work unit
    std::vector<double> psi_init;
    FastView fv{};
    double layout_padding = 0.0;
    int layout_units = 0, layout_max_local = 0, layout_tracks_per_unit = 0, layout_window_rows = 0;
    std::vector<int> set_nx, set_ny;

    // view with geometry pointers filled and cross-section pointers null
    GeomView view() const { return gv_; }
    const double *surf_area() const { return surf_area_.p; }
    // initial incoming boundary flux of one group, in the sweep precision
    const void *psi_init_device() const { return psi_init_dev_.p; }
    const double *dx() const { return dx_.p; }
    const double *dy() const { return dy_.p; }
    size_t bytes() const { return bytes_; }
    // algorithmic bytes of one group sweep (segment stream, FSR data, boundary psi)
    double sweep_bytes() const;

  private:
    GeomView gv_{};
    size_t bytes_ = 0;
    DevBuf<int64_t> seg_begin_;
    DevBuf<int> trk_bc0_, trk_bc1_, trk_set_, seg_fsr_, fsr_mat_, bc_off_, set_ny_, wt_tgt_;
    DevBuf<double> seg_len_d_;
    DevBuf<float> seg_len_f_;
    DevBuf<double> fsr_vol_, fsr_area_, exp_tab_;
    DevBuf<SetPolar> sp_;
    DevBuf<int> ev_fw_begin_, ev_fw_pt_, ev_fw_code_, ev_bw_begin_, ev_bw_pt_, ev_bw_code_;
    DevBuf<int2> ev_fw_, ev_bw_, bundle_bc_;
    DevBuf<int4> bundle_ev_;
    DevBuf<int4> trk_entry_;
    DevBuf<unsigned char> psi_init_dev_;
    DevBuf<int> pin_first_reg_, pin_cell_, pin_fuel_;
    DevBuf<double> pin_area_, surf_area_, dx_, dy_;
    DevBuf<WorkUnitDev> wu_;
    DevBuf<int64_t> bundle_row_;
    DevBuf<int> bundle_nrows_, bundle_track_, local_fsr_;
    DevBuf<int2> win_;
    DevBuf<float> blen_f_;
    DevBuf<double> blen_d_;
    DevBuf<uint16_t> blfsr_;
};

} // namespace mocgpu
