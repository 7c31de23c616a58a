// 2-D structured core geometry: pin meshes, pins, lattices, assemblies, the
// core, and the coarse (pin-cell) mesh with MOCC's cell/surface numbering.
//
// Follows:
//   PinMesh_Cyl  src/core/pin_mesh_cyl.cpp:36-219 (mesh radii, sector lines,
//                region numbering: ring-major, counter-clockwise from +x)
//   PinMesh_Rect src/core/pin_mesh_rect.cpp:29-160
//   Lattice      src/core/lattice.cpp (rows listed top-down in the input)
//   Plane        src/core/plane.cpp (lattice-major FSR numbering)
//   Core         src/core/core.cpp
//   CoreMesh     src/core/core_mesh.cpp:36-260
//   Mesh         src/core/mesh.cpp:88-671 (coarse surfaces, corner conventions)
//
// Only single-plane (2-D) cores are supported: assemblies must have np="1".
#pragma once

#include <array>
#include <map>
#include <memory>
#include <vector>

#include "geom.hpp"
#include "materials.hpp"

namespace mocgpu {

struct XmlNode;

struct PinMesh {
    int id = 0;
    double pitch_x = 0, pitch_y = 0;
    int n_reg = 0, n_xsreg = 0;
    std::vector<double> areas;
    virtual ~PinMesh() = default;
    // Traces the segment p1->p2 (pin-local coordinates); appends lengths and
    // region indices (offset by first_reg); returns the number of segments.
    virtual int trace(Point2 p1, Point2 p2, int first_reg, std::vector<double> &s, std::vector<int> &reg) const = 0;
    virtual int find_reg(Point2 p) const = 0;
    virtual int n_fsrs(int xsreg) const = 0;
};

struct PinMeshCyl : PinMesh {
    std::vector<double> xs_radii, radii;
    std::vector<int> sub_rad;
    int sub_azi = 0;
    std::vector<Circle> circles;
    std::vector<Line> lines;
    explicit PinMeshCyl(const XmlNode &node);
    int trace(Point2 p1, Point2 p2, int first_reg, std::vector<double> &s, std::vector<int> &reg) const override;
    int find_reg(Point2 p) const override;
    int n_fsrs(int xsreg) const override
    {
        return (xsreg < (int)xs_radii.size()) ? sub_rad[xsreg] * sub_azi : sub_azi;
    }
};

struct PinMeshRect : PinMesh {
    int nx = 0, ny = 0;
    std::vector<double> hx, hy;
    std::vector<Line> lines;
    explicit PinMeshRect(const XmlNode &node);
    int trace(Point2 p1, Point2 p2, int first_reg, std::vector<double> &s, std::vector<int> &reg) const override;
    int find_reg(Point2 p) const override;
    int n_fsrs(int) const override { return 1; }
};

struct Pin {
    int id = 0;
    const PinMesh *mesh = nullptr;
    std::vector<int> mat_ids;
    bool is_fuel = false;
};

struct Lattice {
    int id = 0;
    int nx = 0, ny = 0;
    std::vector<const Pin *> pins; // row-major, bottom row first
    std::vector<double> hx_vec, hy_vec, x_vec, y_vec;
    double hx = 0, hy = 0;
    int n_reg = 0, n_xsreg = 0;
    std::vector<int> first_reg_pin;
    const Pin &at(int ix, int iy) const { return *pins[iy * nx + ix]; }
    const PinMesh *get_pinmesh(Point2 &p, int &first_reg) const;
};

struct CoreMesh {
    // input objects
    std::map<int, std::unique_ptr<PinMesh>> pin_meshes;
    MaterialLib mat_lib;
    std::map<int, Pin> pins;
    std::map<int, Lattice> lattices;
    std::map<int, const Lattice *> assemblies; // assembly id -> its single lattice
    std::map<int, double> assembly_hz;

    // core layout
    int nasy_x = 0, nasy_y = 0;
    std::vector<const Lattice *> plane_lattices; // row-major, bottom first
    std::vector<double> plane_hx, plane_hy;      // cumulative lattice boundaries
    std::vector<int> first_reg_lattice;
    std::array<BoundaryType, 6> bc{};
    double hz = 1.0;

    // pin-level mesh
    int nx = 0, ny = 0;
    double hx = 0, hy = 0;
    std::vector<double> x_vec, y_vec, dx_vec, dy_vec;
    std::vector<Line> lines;
    std::vector<const Pin *> core_pins; // FSR order (lattice-major)
    std::vector<int> pin_first_reg;     // first FSR of each pin in core_pins
    std::vector<int> pin_cell;          // coarse cell of each pin in core_pins
    int n_reg = 0;
    int n_fuel_2d = 0;

    static std::unique_ptr<CoreMesh> from_xml(const XmlNode &doc, const std::string &base_dir,
                                              const std::string &xsl_override);

    // coarse mesh numbering (single plane)
    int n_pin() const { return nx * ny; }
    int n_surf_plane() const { return (nx + 1) * ny + (ny + 1) * nx + nx * ny; }
    int n_surf() const { return (nx + 1) * ny + (ny + 1) * nx + 2 * nx * ny; }
    int coarse_cell(int ix, int iy) const { return iy * nx + ix; }
    // Coarse cell containing an interior point (no boundary disambiguation).
    int point_cell(Point2 p) const;
    int coarse_surf(int cell, Surface s) const { return coarse_surf_[cell * 6 + (int)s]; }
    int coarse_neighbor(int cell, Surface s) const;
    Normal surface_normal(int surf) const;
    std::pair<int, int> coarse_neigh_cells(int surf) const;
    double coarse_area(int surf) const;
    double coarse_area(int cell, Surface s) const;
    int coarse_norm_point(Point2 p, int octant, Surface (&s)[2]) const;
    int coarse_boundary_cell(Point2 p, int octant) const;
    void trace(std::vector<Point2> &ps) const; // adds pin-boundary crossings, sorts
    const PinMesh *get_pinmesh(Point2 &p, int &first_reg) const;
    std::vector<double> volumes() const; // FSR areas * plane height
    std::vector<double> areas() const;   // FSR areas

  private:
    std::vector<int> coarse_surf_;
    void prepare_surfaces();
};

} // namespace mocgpu
