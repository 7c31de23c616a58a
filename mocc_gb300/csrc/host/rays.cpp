#include "rays.hpp"

#include <algorithm>
#include <cmath>
#include <limits>

namespace mocgpu {

// Farey-sequence binary search for the closest fraction a/b to target in
// [0, 1], returning early once within tol (MOCC
// src/util/rational_approximation.hpp:39-80).
std::pair<int, int> rational_approximation(double target, double tol, int max_d)
{
    if (max_d == 0) max_d = std::numeric_limits<int>::max();
    int a = 0, b = 1, c = 1, d = 1;
    if (std::fabs((double)a / b - target) < tol) return {a, b};
    if (std::fabs((double)c / d - target) < tol) return {c, d};
    while (b <= max_d && d <= max_d) {
        double med = (double)(a + c) / (double)(b + d);
        if (std::fabs(target - med) < tol) {
            if (b + d <= max_d) return {a + c, b + d};
            if (d > b) return {c, d};
            return {a, b};
        } else if (target > med) {
            a += c;
            b += d;
        } else {
            c += a;
            d += b;
        }
    }
    if (b > max_d) return {c, d};
    return {a, b};
}

namespace {

// One pin crossing of the fine trace: its coarse cell, segment count and
// chord length.
struct PinCrossing {
    int cell, nseg;
    double len;
};

// Crossings shorter than this (a ray grazing a pin-cell corner) are slivers:
// the fuzzy point comparisons of the trace can leave them as pin crossings of
// their own, sometimes assigned to a pin off the ray's path.
constexpr double kSliver = 1e-9;

int cell_x(const CoreMesh &m, int c) { return c % m.nx; }
int cell_y(const CoreMesh &m, int c) { return c / m.nx; }

// Coarse crossings of one direction of a ray (moc::Current's walk data,
// ray.cpp:52-166): the entry cell and surface, then for every crossing the
// surface and the number of segments before it. The surfaces between two
// pins follow the cells of the traced segments (adjacent cells: one face;
// diagonal cells: the corner pair in MOCC's order for the octant, the second
// after zero segments), so the walk always visits the cells the segments lie
// in. Slivers are folded into the neighbouring crossing in traversal order.
void coarse_walk(const CoreMesh &m, const std::vector<PinCrossing> &px, int octant, Point2 start, Point2 end,
                 int &cell0, int &surf0, std::vector<Surface> &surfs, std::vector<int> &nsegs)
{
    std::vector<int> cells, counts;
    int pending = 0;
    for (const PinCrossing &c : px) {
        const bool sliver = c.len < kSliver && px.size() > 1;
        if (sliver) {
            if (counts.empty()) pending += c.nseg;
            else counts.back() += c.nseg;
            continue;
        }
        if (!cells.empty() && cells.back() == c.cell) {
            counts.back() += c.nseg + pending; // a split of one pin crossing
        } else {
            cells.push_back(c.cell);
            counts.push_back(c.nseg + pending);
        }
        pending = 0;
    }
    if (cells.empty()) MOCGPU_THROW(6, "ray crosses no pin");
    if (pending) counts.back() += pending;

    Surface s[2];
    cell0 = cells.front();
    if (m.coarse_norm_point(start, octant, s) != 1) MOCGPU_THROW(6, "ray starts on more than one coarse surface");
    surf0 = m.coarse_surf(cell0, s[0]);
    for (size_t k = 0; k + 1 < cells.size(); k++) {
        const int dx = cell_x(m, cells[k + 1]) - cell_x(m, cells[k]);
        const int dy = cell_y(m, cells[k + 1]) - cell_y(m, cells[k]);
        Surface fx = dx > 0 ? EAST : WEST, fy = dy > 0 ? NORTH : SOUTH;
        if (std::abs(dx) + std::abs(dy) == 1) {
            surfs.push_back(dx != 0 ? fx : fy);
            nsegs.push_back(counts[k]);
        } else if (std::abs(dx) == 1 && std::abs(dy) == 1) {
            // corner: x face first, then y face (mesh.cpp:471-493)
            surfs.push_back(fx);
            surfs.push_back(fy);
            nsegs.push_back(counts[k]);
            nsegs.push_back(0);
        } else {
            MOCGPU_THROW(6, "consecutive pin crossings of a ray are not neighbouring cells");
        }
    }
    const int ns = m.coarse_norm_point(end, octant, s);
    if (ns < 1) MOCGPU_THROW(6, "ray does not end on a coarse surface");
    for (int j = 0; j < ns; j++) surfs.push_back(s[j]);
    nsegs.push_back(counts.back());
    if (ns > 1) nsegs.push_back(0);
}

} // namespace

Ray::Ray(Point2 a, Point2 b, std::array<int, 2> bc_, const CoreMesh &mesh) : bc(bc_), p1(a), p2(b)
{
    std::vector<Point2> ps{a, b};
    mesh.trace(ps);
    const std::vector<Point2> &cps = ps;

    // Fine trace, pin crossing by pin crossing (ray.cpp:62-83).
    std::vector<PinCrossing> px;
    Point2 prev = cps.front();
    for (size_t i = 1; i < ps.size(); i++) {
        Point2 pin_p = midpoint(ps[i], prev);
        const Point2 mid = pin_p;
        int first_reg = 0;
        const PinMesh *pm = mesh.get_pinmesh(pin_p, first_reg);
        int n = pm->trace(prev - pin_p, ps[i] - pin_p, first_reg, seg_len, seg_fsr);
        px.push_back(PinCrossing{mesh.point_cell(mid), n, std::hypot(ps[i].x - prev.x, ps[i].y - prev.y)});
        prev = ps[i];
    }

    // Coarse crossings, forward then backward.
    const int octant = (b.x > a.x) ? 1 : 2;
    std::vector<Surface> surfs_fw, surfs_bw;
    std::vector<int> nsegs_fw, nsegs_bw;
    coarse_walk(mesh, px, octant, cps.front(), cps.back(), cm_cell_fw, cm_surf_fw, surfs_fw, nsegs_fw);
    std::reverse(px.begin(), px.end());
    coarse_walk(mesh, px, octant == 1 ? 3 : 4, cps.back(), cps.front(), cm_cell_bw, cm_surf_bw, surfs_bw, nsegs_bw);

    size_t stp = std::min(nsegs_fw.size(), nsegs_bw.size());
    for (size_t i = 0; i < stp; i++) {
        CoarseCrossing c;
        c.fw = surfs_fw[i];
        c.bw = surfs_bw[i];
        c.nseg_fw = nsegs_fw[i];
        c.nseg_bw = nsegs_bw[i];
        cm_data.push_back(c);
    }
    // A corner double-crossing at one end only: extra record, no-op on the
    // other direction (ray.cpp:147-166).
    if (nsegs_fw.size() > nsegs_bw.size()) {
        CoarseCrossing c;
        c.fw = surfs_fw.back();
        c.bw = INVALID;
        cm_data.push_back(c);
    }
    if (nsegs_bw.size() > nsegs_fw.size()) {
        CoarseCrossing c;
        c.fw = INVALID;
        c.bw = surfs_bw.back();
        cm_data.push_back(c);
    }
}

static std::pair<int, int> modularize(const Angle &ang, double hx, double hy, double spacing, bool rational)
{
    int Nx, Ny;
    if (rational) {
        double m = (ang.alpha < kPi / 4.0) ? std::tan(ang.alpha) : std::tan(kPi / 2.0 - ang.alpha);
        auto f = rational_approximation(m, 0.002, 0);
        Nx = f.first;
        Ny = f.second;
        if (Nx == 0) MOCGPU_THROW(6, "azimuthal angle too shallow for rational modularisation");
        double alpha = std::atan((Nx * hy) / (Ny * hx));
        int scale = (int)std::ceil((hx / Nx * std::fabs(std::sin(alpha))) / spacing);
        Nx *= scale;
        Ny *= scale;
        if (ang.alpha > kPi / 4.0) std::swap(Nx, Ny);
    } else {
        Nx = (int)std::ceil(hx / spacing * std::fabs(std::sin(ang.alpha)));
        Ny = (int)std::ceil(hy / spacing * std::fabs(std::cos(ang.alpha)));
        Nx += Nx % 2;
        Ny += Ny % 2;
    }
    return {Nx, Ny};
}

RayData::RayData(const RaySpec &spec, const AngularQuadrature &q, const CoreMesh &mesh) : quad(q)
{
    if (spec.spacing <= 0.0) MOCGPU_THROW(6, "Failed to read valid ray spacing.");
    pol_per_set = quad.polars_per_set();
    if (quad.ndir_oct % pol_per_set != 0) MOCGPU_THROW(6, "quadrature layout mismatch");
    const int sets_oct = quad.ndir_oct / pol_per_set;
    n_sets = 2 * sets_oct;
    const double hx = mesh.hx, hy = mesh.hy;
    double hx_mod = hx, hy_mod = hy;
    if (!spec.core_modular) {
        hx_mod = mesh.core_pins.front()->mesh->pitch_x;
        hy_mod = mesh.core_pins.front()->mesh->pitch_y;
        for (const Pin *p : mesh.core_pins)
            if (p->mesh->pitch_x != hx_mod || p->mesh->pitch_y != hy_mod)
                MOCGPU_THROW(6, "Core Mesh does not support pin modular ray tracing.");
    }

    // Modularise octant-1 angles; each polar of a set gets the same alpha.
    std::vector<int> nx1(quad.ndir_oct), ny1(quad.ndir_oct);
    std::vector<double> sp1(quad.ndir_oct);
    for (int iang = 0; iang < quad.ndir_oct; iang++) {
        Angle ang = quad.angles[iang];
        auto N = modularize(ang, hx_mod, hy_mod, spec.spacing, spec.rational);
        int Nx = N.first, Ny = N.second;
        if (!spec.core_modular) {
            Nx *= mesh.nx;
            Ny *= mesh.ny;
        }
        double new_alpha = std::atan(hy * Nx / (hx * Ny));
        ang.modify_alpha(new_alpha);
        quad.modify_angle(iang, ang);
        nx1[iang] = Nx;
        ny1[iang] = Ny;
        sp1[iang] = std::cos(quad.angles[iang].alpha) * hy / Ny;
    }
    quad.update_weights();
    nx.resize(n_sets);
    ny.resize(n_sets);
    spacing.resize(n_sets);
    for (int s = 0; s < sets_oct; s++) {
        int iang = s * pol_per_set;
        for (int p = 1; p < pol_per_set; p++)
            if (nx1[iang + p] != nx1[iang] || ny1[iang + p] != ny1[iang])
                MOCGPU_THROW(6, "polar angles of one azimuth modularised differently");
        nx[s] = nx[s + sets_oct] = nx1[iang];
        ny[s] = ny[s + sets_oct] = ny1[iang];
        spacing[s] = spacing[s + sets_oct] = sp1[iang];
    }

    // Lay down and trace the tracks of every set in octants 1 and 2.
    Box core_box(Point2(0.0, 0.0), Point2(hx, hy));
    rays.resize(n_sets);
    max_seg = 0;
    for (int set = 0; set < n_sets; set++) {
        const Angle &ang = quad.angles[(set / sets_oct) * quad.ndir_oct + (set % sets_oct) * pol_per_set];
        int Nx = nx[set], Ny = ny[set];
        double space = spacing[set];
        double space_x = std::fabs(space / std::sin(ang.alpha));
        double space_y = std::fabs(space / std::cos(ang.alpha));
        auto exit_bc = [&](const Point2 &p2) -> int {
            if (fp_equiv(p2.x, hx)) return (int)(p2.y / space_y);
            if (fp_equiv(p2.y, hy)) return (int)(p2.x / space_x) + Ny;
            if (fp_equiv(p2.x, 0.0)) return (int)(p2.y / space_y);
            MOCGPU_THROW(6, "ray trace failed to find an exit face");
        };
        std::vector<Ray> rs;
        rs.reserve(Nx + Ny);
        for (int i = 0; i < Ny; i++) {
            Point2 p1((ang.ox > 0.0) ? 0.0 : hx, (0.5 + i) * space_y);
            Point2 p2 = core_box.intersect(p1, ang.alpha);
            if (!p2.ok) MOCGPU_THROW(6, "ray exit point not found");
            std::array<int, 2> bc{i, exit_bc(p2)};
            rs.emplace_back(p1, p2, bc, mesh);
            max_seg = std::max(max_seg, rs.back().nseg());
        }
        for (int i = 0; i < Nx; i++) {
            Point2 p1((0.5 + i) * space_x, 0.0);
            Point2 p2 = core_box.intersect(p1, ang.alpha);
            if (!p2.ok) MOCGPU_THROW(6, "ray exit point not found");
            std::array<int, 2> bc{i + Ny, exit_bc(p2)};
            rs.emplace_back(p1, p2, bc, mesh);
            max_seg = std::max(max_seg, rs.back().nseg());
        }
        for (const Ray &r : rs)
            if (r.bc[1] < 0 || r.bc[1] >= Nx + Ny) MOCGPU_THROW(6, "ray boundary index out of range");
        rays[set] = std::move(rs);
    }

    // Volume correction.
    const std::vector<double> true_vol = mesh.areas();
    const int nreg = (int)true_vol.size();
    if (spec.correction == VolumeCorrection::FLAT) {
        for (int set = 0; set < n_sets; set++) {
            std::vector<double> fsr_vol(nreg, 0.0);
            for (const Ray &r : rays[set])
                for (int s = 0; s < r.nseg(); s++) fsr_vol[r.seg_fsr[s]] += r.seg_len[s] * spacing[set];
            std::vector<double> cf(nreg);
            for (int i = 0; i < nreg; i++) cf[i] = true_vol[i] / fsr_vol[i];
            for (Ray &r : rays[set])
                for (int s = 0; s < r.nseg(); s++) r.seg_len[s] = r.seg_len[s] * cf[r.seg_fsr[s]];
        }
    } else if (spec.correction == VolumeCorrection::ANGLE) {
        std::vector<double> fsr_vol(nreg, 0.0);
        for (int iang = 0; iang < 2 * quad.ndir_oct; iang++) {
            int set = set_of(iang);
            double wgt = quad.angles[iang].weight * 0.5;
            for (const Ray &r : rays[set])
                for (int s = 0; s < r.nseg(); s++) fsr_vol[r.seg_fsr[s]] += r.seg_len[s] * spacing[set] * wgt;
        }
        for (int i = 0; i < nreg; i++) fsr_vol[i] = true_vol[i] / fsr_vol[i];
        for (int set = 0; set < n_sets; set++)
            for (Ray &r : rays[set])
                for (int s = 0; s < r.nseg(); s++) r.seg_len[s] = r.seg_len[s] * fsr_vol[r.seg_fsr[s]];
    }
}

} // namespace mocgpu
