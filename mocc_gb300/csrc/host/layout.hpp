// Sweep work-unit layout for the bundled GPU sweep kernel.
//
// Tracks of one sweep phase are cut into work units (one CTA each): runs of
// spatially adjacent tracks of one azimuthal set, capped so that the FSRs a
// unit touches fit the unit's shared-memory tally. Inside a unit the tracks
// are sorted by length and grouped into bundles of 32 (one warp-row each);
// a bundle's segments are stored row-interleaved ([row][lane]) and padded
// with zero-length segments to the bundle's longest track, so that both the
// forward and the backward pass read 32 consecutive entries per row.
// Segment FSR indices are stored window-local (16-bit) with a table per row
// window mapping them back to plane FSR indices. A row window is rows
// [w * window_rows, (w + 1) * window_rows) of every bundle of the unit (one
// window covering the whole unit when window_rows is 0 or the unit is
// shorter): the kernel stages the FSRs of one window at a time, so the
// shared memory a unit needs follows the window's band of FSRs rather than
// its tracks' whole length.
#pragma once

#include <cstdint>
#include <vector>

#include "problem.hpp"

namespace mocgpu {

struct WorkUnitHost {
    int set;          // azimuthal track set
    int bundle_begin; // first bundle
    int n_bundles;
    int win_begin;    // first row window (into SweepLayout::win)
    int n_win;        // row windows
    int n_local;      // FSRs the whole unit touches
};

struct RowWindowHost {
    int fsr_begin; // into local_fsr
    int n_local;   // FSRs its rows touch (its table's padding slot is n_local)
};

struct SweepLayout {
    static constexpr int kLanes = 32;
    int n_phases = 0;
    std::vector<int> phase_wu_begin;   // n_phases + 1
    std::vector<WorkUnitHost> wu;
    std::vector<int64_t> bundle_row;   // first row of each bundle (row = kLanes entries)
    std::vector<int> bundle_nrows;
    std::vector<int> bundle_track;     // [n_bundles * kLanes], -1 for empty lanes
    std::vector<double> len;           // [rows * kLanes]
    std::vector<uint16_t> lfsr;        // [rows * kLanes]
    std::vector<RowWindowHost> win;
    std::vector<int> local_fsr;        // concatenated window maps
    int64_t n_rows = 0;
    int window_rows = 0;               // rows per window (0: one window per unit)
    int max_local = 0;                 // FSR slots of the largest window table (its FSRs + the padding slot)
    int max_windows = 0;               // most windows of one unit
    int max_hits = 0;                  // most tally adds (segment entries x 2 directions) on one table slot
    double padding = 0.0;              // padded / real segments - 1
};

// gs: two phases (octant-1 sets, then octant-2 sets); otherwise one phase.
// tracks_per_unit: target tracks per unit (a multiple of 32); max_local: cap
// on FSRs per unit; window_rows: rows per staged window (a multiple of 16, 0
// for whole units).
SweepLayout build_sweep_layout(const FlatProblem &f, bool gs, int tracks_per_unit, int max_local,
                               bool interleave = false, int window_rows = 0);

} // namespace mocgpu
