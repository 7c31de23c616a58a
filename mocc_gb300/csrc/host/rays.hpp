// Modular ray tracing for the 2-D MoC sweep.
//
// Follows MOCC's RayData/Ray (src/sweepers/moc/ray_data.cpp:67-527,
// src/sweepers/moc/ray.cpp:52-175): rational-fraction modularisation of each
// octant-1 angle, ray laydown from the x- and y-normal faces at half-spacing
// offsets, boundary-condition indices by position, per-pin segment tracing,
// coarse-surface crossing data for the CMFD current tally, and the "flat"
// (per angle) segment-length volume correction.
//
// Unlike MOCC, which stores the tracks of every (azimuth, polar) pair
// separately, the tracks of one azimuth are stored once and shared by all
// polar angles of a product quadrature: the tracks depend on the azimuth only.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

#include "mesh.hpp"
#include "quadrature.hpp"

namespace mocgpu {

// One coarse-mesh crossing record (MOCC's RayCoarseData).
struct CoarseCrossing {
    Surface fw = INVALID, bw = INVALID;
    int nseg_fw = 0, nseg_bw = 0;
};

struct Ray {
    std::array<int, 2> bc{};
    Point2 p1, p2;
    std::vector<double> seg_len;
    std::vector<int> seg_fsr;
    int cm_cell_fw = 0, cm_cell_bw = 0, cm_surf_fw = 0, cm_surf_bw = 0;
    std::vector<CoarseCrossing> cm_data;
    Ray() = default;
    Ray(Point2 p1, Point2 p2, std::array<int, 2> bc, const CoreMesh &mesh);
    int nseg() const { return (int)seg_len.size(); }
};

enum class VolumeCorrection { FLAT, ANGLE, NONE };

struct RaySpec {
    double spacing = -1.0;
    VolumeCorrection correction = VolumeCorrection::FLAT;
    bool core_modular = true;
    bool rational = true;
};

struct RayData {
    AngularQuadrature quad;   // modularised copy
    int n_sets = 0;           // track sets in octants 1-2
    int pol_per_set = 1;      // polar angles sharing a track set
    std::vector<int> nx, ny;  // per track set (octants 1-2)
    std::vector<double> spacing;
    std::vector<std::vector<Ray>> rays; // per track set
    int max_seg = 0;

    RayData(const RaySpec &spec, const AngularQuadrature &q, const CoreMesh &mesh);
    // Track set used by angle iang in octants 1-2 (and its polar slot).
    int set_of(int iang) const { return (iang % quad.ndir_oct) / pol_per_set + (iang / quad.ndir_oct) * (n_sets / 2); }
    int polar_of(int iang) const { return (iang % quad.ndir_oct) % pol_per_set; }
};

std::pair<int, int> rational_approximation(double target, double tol, int max_d);

} // namespace mocgpu
