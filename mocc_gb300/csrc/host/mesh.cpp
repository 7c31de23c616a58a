#include "mesh.hpp"

#include <algorithm>
#include <cmath>
#include <sstream>

#include "xml.hpp"

namespace mocgpu {

// ---------------------------------------------------------------------------
// Pin meshes
static void read_pin_mesh_common(PinMesh &pm, const XmlNode &node)
{
    pm.id = node.attr_int("id", -1);
    if (pm.id < 0) MOCGPU_THROW(5, "Failed to read pin ID.");
    pm.pitch_x = node.attr_double("pitch", -1.0);
    pm.pitch_y = pm.pitch_x;
    if (pm.pitch_x <= 0.0) MOCGPU_THROW(5, "Failed to read valid pin pitch.");
}

PinMeshCyl::PinMeshCyl(const XmlNode &node)
{
    read_pin_mesh_common(*this, node);
    const XmlNode *r = node.child("radii");
    if (!r) MOCGPU_THROW(5, "cylindrical pin mesh without <radii>");
    xs_radii = explode<double>(r->text);
    if (xs_radii.empty()) MOCGPU_THROW(5, "Ran into a problem reading radii");
    for (size_t i = 0; i + 1 < xs_radii.size(); i++)
        if (xs_radii[i] > xs_radii[i + 1]) MOCGPU_THROW(5, "Pin radii do not appear to be ordered");
    if (xs_radii.back() > pitch_x * 0.5) MOCGPU_THROW(5, "Largest radius is too big!");
    n_xsreg = (int)xs_radii.size() + 1;
    const XmlNode *sa = node.child("sub_azi");
    if (!sa) MOCGPU_THROW(5, "Improper input to azimuthal subdivisions!");
    auto azi = explode<int>(sa->text);
    if (azi.size() != 1) MOCGPU_THROW(5, "Only supporting one azimuthal subdivision entry.");
    sub_azi = azi[0];
    if ((sub_azi % 2 != 0) || sub_azi > 8 || sub_azi <= 0)
        MOCGPU_THROW(5, "Only supporting even azimuthal subdivisions <=8.");
    const XmlNode *sr = node.child("sub_radii");
    sub_rad = sr ? explode<int>(sr->text) : std::vector<int>();
    if ((int)sub_rad.size() != n_xsreg - 1) MOCGPU_THROW(5, "Wrong number of radial subdivisions specified.");

    // Equal-area mesh rings inside each material ring.
    double rxsi = 0.0, ri = 0.0;
    for (int ixs = 0; ixs < n_xsreg - 1; ixs++) {
        double vn = (xs_radii[ixs] * xs_radii[ixs] - rxsi * rxsi) / sub_rad[ixs];
        for (int ir = 0; ir < sub_rad[ixs]; ir++) {
            double rr = std::sqrt(vn + ri * ri);
            radii.push_back(rr);
            ri = rr;
        }
        rxsi = xs_radii[ixs];
    }
    Point2 origin(0.0, 0.0);
    for (double rr : radii) circles.emplace_back(origin, rr);
    double hpx = 0.5 * pitch_x, hpy = 0.5 * pitch_y;
    Box pin_box(Point2(-hpx, -hpy), Point2(hpx, hpy));
    double sep = kTwoPi / sub_azi;
    for (int i = 0; i < sub_azi; i++) lines.emplace_back(origin, pin_box.intersect(origin, i * sep));
    n_reg = ((int)radii.size() + 1) * sub_azi;
    double prev = 0.0;
    for (double rr : radii) {
        double a = kPi * (rr * rr - prev * prev) / sub_azi;
        for (int i = 0; i < sub_azi; i++) areas.push_back(a);
        prev = rr;
    }
    double big = radii.back();
    double outer = (pitch_x * pitch_y - kPi * big * big) / sub_azi;
    for (int i = 0; i < sub_azi; i++) areas.push_back(outer);
}

int PinMeshCyl::find_reg(Point2 p) const
{
    if (std::fabs(p.x) > 0.5 * pitch_x || std::fabs(p.y) > 0.5 * pitch_y) return -1;
    double r = std::sqrt(p.x * p.x + p.y * p.y);
    size_t ir = 0;
    for (ir = 0; ir < radii.size(); ir++)
        if (r < radii[ir]) break;
    int ia = (int)(p.alpha() / (kTwoPi / sub_azi));
    return (int)ir * sub_azi + ia;
}

int PinMeshCyl::trace(Point2 p1, Point2 p2, int first_reg, std::vector<double> &s, std::vector<int> &reg) const
{
    Line l(p1, p2);
    std::vector<Point2> ps{p1, p2};
    for (const auto &c : circles) {
        Point2 a, b;
        if (intersect(l, c, a, b) == 2) {
            ps.push_back(a);
            ps.push_back(b);
        }
    }
    for (const auto &li : lines) {
        Point2 p;
        if (intersect(li, l, p) == 1) ps.push_back(p);
    }
    std::sort(ps.begin(), ps.end());
    ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
    for (size_t i = 1; i < ps.size(); i++) {
        s.push_back(ps[i].distance(ps[i - 1]));
        reg.push_back(find_reg(midpoint(ps[i], ps[i - 1])) + first_reg);
    }
    return (int)ps.size() - 1;
}

PinMeshRect::PinMeshRect(const XmlNode &node)
{
    read_pin_mesh_common(*this, node);
    const XmlNode *sx = node.child("sub_x");
    const XmlNode *sy = node.child("sub_y");
    nx = sx ? std::atoi(sx->text.c_str()) : 0;
    ny = sy ? std::atoi(sy->text.c_str()) : 0;
    if (nx < 1) MOCGPU_THROW(5, "Failed to read valid number of X divisions in rect pin mesh.");
    if (ny < 1) MOCGPU_THROW(5, "Failed to read valid number of Y divisions in rect pin mesh.");
    n_xsreg = n_reg = nx * ny;
    double dx = pitch_x / nx, dy = pitch_y / ny;
    double hpx = 0.5 * pitch_x, hpy = 0.5 * pitch_y;
    for (int i = 0; i <= nx; i++) hx.push_back(i * dx - hpx);
    for (int i = 0; i <= ny; i++) hy.push_back(i * dy - hpy);
    for (size_t i = 1; i + 1 < hx.size(); i++) lines.emplace_back(Point2(hx[i], -hpy), Point2(hx[i], hpy));
    for (size_t i = 1; i + 1 < hy.size(); i++) lines.emplace_back(Point2(-hpx, hy[i]), Point2(hpx, hy[i]));
    areas.assign(n_reg, dx * dy);
}

int PinMeshRect::find_reg(Point2 p) const
{
    if (std::fabs(p.x) > 0.5 * pitch_x || std::fabs(p.y) > 0.5 * pitch_y) return -1;
    int ix = (int)(std::lower_bound(hx.begin(), hx.end(), p.x) - hx.begin()) - 1;
    int iy = (int)(std::lower_bound(hy.begin(), hy.end(), p.y) - hy.begin()) - 1;
    return nx * iy + ix;
}

int PinMeshRect::trace(Point2 p1, Point2 p2, int first_reg, std::vector<double> &s, std::vector<int> &reg) const
{
    std::vector<Point2> ps{p1, p2};
    Line l(p1, p2);
    for (const auto &li : lines) {
        Point2 p;
        if (intersect(li, l, p) == 1) ps.push_back(p);
    }
    std::sort(ps.begin(), ps.end());
    ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
    for (size_t i = 1; i < ps.size(); i++) {
        s.push_back(ps[i].distance(ps[i - 1]));
        reg.push_back(find_reg(midpoint(ps[i], ps[i - 1])) + first_reg);
    }
    return (int)ps.size() - 1;
}

// ---------------------------------------------------------------------------
// Lattice lookup with the default (+x, +y) tie-break direction.
const PinMesh *Lattice::get_pinmesh(Point2 &p, int &first_reg) const
{
    long ix = std::lower_bound(x_vec.begin(), x_vec.end(), p.x, fuzzy_lt) - x_vec.begin();
    if (ix < (long)x_vec.size() && fp_equiv_abs(p.x, x_vec[ix])) ix++;
    ix--;
    ix = std::min<long>(nx - 1, std::max<long>(0, ix));
    p.x = 0.5 * (x_vec[ix + 1] + x_vec[ix]);
    long iy = std::lower_bound(y_vec.begin(), y_vec.end(), p.y, fuzzy_lt) - y_vec.begin();
    if (iy < (long)y_vec.size() && fp_equiv_abs(p.y, y_vec[iy])) iy++;
    iy--;
    iy = std::min<long>(ny - 1, std::max<long>(0, iy));
    p.y = 0.5 * (y_vec[iy + 1] + y_vec[iy]);
    int i = (int)(iy * nx + ix);
    first_reg += first_reg_pin[i];
    return at((int)ix, (int)iy).mesh;
}

// ---------------------------------------------------------------------------
static BoundaryType parse_bc(const XmlNode &n, const char *attr)
{
    std::string v = n.attr(attr);
    if (v == "vacuum") return BoundaryType::VACUUM;
    if (v == "reflect") return BoundaryType::REFLECT;
    if (v == "prescribed") return BoundaryType::PRESCRIBED;
    return BoundaryType::INVALID;
}

std::unique_ptr<CoreMesh> CoreMesh::from_xml(const XmlNode &doc, const std::string &base_dir,
                                             const std::string &xsl_override)
{
    auto cm = std::make_unique<CoreMesh>();
    // pin meshes
    for (const XmlNode *m : doc.children_named("mesh")) {
        std::string t = sanitize(m->attr("type"));
        std::unique_ptr<PinMesh> pm;
        if (t == "cyl") pm = std::make_unique<PinMeshCyl>(*m);
        else if (t == "rect") pm = std::make_unique<PinMeshRect>(*m);
        else MOCGPU_THROW(5, "Unrecognized mesh type: " + t);
        int id = pm->id;
        if (cm->pin_meshes.count(id)) MOCGPU_THROW(5, "Duplicate pin mesh ID");
        cm->pin_meshes[id] = std::move(pm);
    }
    // materials
    const XmlNode *ml = doc.child("material_lib");
    if (!ml) MOCGPU_THROW(4, "No material library specified.");
    std::string xsl_text = xsl_override;
    if (xsl_text.empty()) {
        std::string path = ml->attr("path");
        if (!path.empty() && path[0] != '/' && !base_dir.empty()) path = base_dir + "/" + path;
        xsl_text = read_file(path);
    }
    cm->mat_lib = MaterialLib::from_xsl_text(xsl_text);
    for (const XmlNode *m : ml->children_named("material")) cm->mat_lib.assign(m->attr_int("id", 0), m->attr("name"));
    // pins
    for (const XmlNode *pn : doc.children_named("pin")) {
        Pin pin;
        pin.id = pn->attr_int("id", 0);
        if (pin.id == 0) MOCGPU_THROW(5, "Failed to read pin ID.");
        int mid = pn->attr_int("mesh", 0);
        if (!cm->pin_meshes.count(mid)) MOCGPU_THROW(5, "Invalid pin mesh ID.");
        pin.mesh = cm->pin_meshes[mid].get();
        pin.mat_ids = explode<int>(pn->text);
        if ((int)pin.mat_ids.size() != pin.mesh->n_xsreg)
            MOCGPU_THROW(5, "Wrong number of materials specified in pin definition");
        for (int m : pin.mat_ids) {
            if (!cm->mat_lib.has(m)) MOCGPU_THROW(5, "Invalid material specified in pin");
            if (cm->mat_lib.by_id(m).fissile) {
                pin.is_fuel = true;
                break;
            }
        }
        if (pn->has_attr("fuel")) pin.is_fuel = pn->attr_bool("fuel", pin.is_fuel);
        if (cm->pins.count(pin.id)) MOCGPU_THROW(5, "Duplicate pin ID");
        cm->pins[pin.id] = pin;
    }
    // lattices
    for (const XmlNode *ln : doc.children_named("lattice")) {
        Lattice lat;
        lat.id = ln->attr_int("id", 0);
        if (lat.id == 0) MOCGPU_THROW(5, "Trouble reading lattice ID.");
        lat.nx = ln->attr_int("nx", 0);
        lat.ny = ln->attr_int("ny", 0);
        if (lat.nx <= 0 || lat.ny <= 0) MOCGPU_THROW(5, "Trouble reading lattice dimensions.");
        auto ids = explode<int>(ln->text);
        if ((int)ids.size() != lat.nx * lat.ny) MOCGPU_THROW(5, "Incorrect number of pin IDs specified for lattice.");
        lat.pins.resize(lat.nx * lat.ny);
        for (int iy = 0; iy < lat.ny; iy++) {
            int row = lat.ny - iy - 1;
            for (int ix = 0; ix < lat.nx; ix++) {
                auto it = cm->pins.find(ids[iy * lat.nx + ix]);
                if (it == cm->pins.end()) MOCGPU_THROW(5, "Unknown pin ID in lattice");
                lat.pins[row * lat.nx + ix] = &it->second;
            }
        }
        for (int ix = 0; ix < lat.nx; ix++) {
            double dx = lat.at(ix, 0).mesh->pitch_x;
            lat.hx += dx;
            lat.hx_vec.push_back(dx);
        }
        for (int iy = 0; iy < lat.ny; iy++) {
            double dy = lat.at(0, iy).mesh->pitch_y;
            lat.hy += dy;
            lat.hy_vec.push_back(dy);
        }
        lat.x_vec.push_back(0.0);
        for (int ix = 0; ix < lat.nx; ix++) lat.x_vec.push_back(lat.x_vec[ix] + lat.hx_vec[ix]);
        lat.y_vec.push_back(0.0);
        for (int iy = 0; iy < lat.ny; iy++) lat.y_vec.push_back(lat.y_vec[iy] + lat.hy_vec[iy]);
        for (int iy = 0; iy < lat.ny; iy++)
            for (int ix = 0; ix < lat.nx; ix++)
                if (lat.at(ix, iy).mesh->pitch_x != lat.hx_vec[ix] || lat.at(ix, iy).mesh->pitch_y != lat.hy_vec[iy])
                    MOCGPU_THROW(5, "Incongruent pin pitches found in lattice.");
        int prev = 0;
        for (size_t i = 0; i < lat.pins.size(); i++) {
            lat.first_reg_pin.push_back(prev);
            prev += lat.pins[i]->mesh->n_reg;
            lat.n_xsreg += lat.pins[i]->mesh->n_xsreg;
        }
        lat.n_reg = prev;
        if (cm->lattices.count(lat.id)) MOCGPU_THROW(5, "Duplicate lattice ID");
        cm->lattices[lat.id] = lat;
    }
    // assemblies (single plane)
    for (const XmlNode *an : doc.children_named("assembly")) {
        int id = an->attr_int("id", 0);
        if (id == 0) MOCGPU_THROW(5, "Invalid assembly ID.");
        int np = an->attr_int("np", 0);
        if (np != 1) MOCGPU_THROW(5, "only single-plane (np=\"1\") assemblies are supported by the 2-D MoC path");
        double hz = an->attr_double("hz", 0.0);
        if (const XmlNode *h = an->child("hz")) {
            auto v = explode<double>(h->text);
            if (v.size() != 1) MOCGPU_THROW(5, "Wrong number of plane heights provided for assembly");
            hz = v[0];
        }
        if (hz <= 0.0) MOCGPU_THROW(5, "Plane heights improperly specified for assembly");
        const XmlNode *ls = an->child("lattices");
        if (!ls) MOCGPU_THROW(5, "No lattices specified!");
        std::string t = ls->text;
        std::replace(t.begin(), t.end(), '{', ' ');
        std::replace(t.begin(), t.end(), '}', ' ');
        auto ids = explode<int>(t);
        if (ids.size() != 1) MOCGPU_THROW(5, "Incorrect number of lattices specified for assembly.");
        auto it = cm->lattices.find(ids[0]);
        if (it == cm->lattices.end()) MOCGPU_THROW(5, "Unrecognized lattice ID in assembly.");
        cm->assemblies[id] = &it->second;
        cm->assembly_hz[id] = hz;
    }
    // core
    const XmlNode *core = nullptr;
    int n_enabled = 0;
    for (const XmlNode *c : doc.children_named("core")) {
        if (c->attr_bool("enabled", true)) {
            core = c;
            n_enabled++;
        }
    }
    if (n_enabled == 0) MOCGPU_THROW(5, "No enabled core specifications.");
    if (n_enabled > 1) MOCGPU_THROW(5, "More than one enabled core specification found.");
    cm->nasy_x = core->attr_int("nx", 0);
    cm->nasy_y = core->attr_int("ny", 0);
    if (cm->nasy_x < 1 || cm->nasy_y < 1) MOCGPU_THROW(5, "Invalid core dimensions.");
    cm->bc[EAST] = parse_bc(*core, "east");
    cm->bc[NORTH] = parse_bc(*core, "north");
    cm->bc[WEST] = parse_bc(*core, "west");
    cm->bc[SOUTH] = parse_bc(*core, "south");
    cm->bc[TOP] = parse_bc(*core, "top");
    cm->bc[BOTTOM] = parse_bc(*core, "bottom");
    for (auto b : cm->bc)
        if (b == BoundaryType::INVALID) MOCGPU_THROW(5, "Not all boundary conditions properly specified.");
    auto asy_ids = explode<int>(core->text);
    if ((int)asy_ids.size() != cm->nasy_x * cm->nasy_y) MOCGPU_THROW(5, "Wrong number of assemblies specified for core.");
    std::vector<int> asy_grid(asy_ids.size());
    int k = 0;
    for (int iy = 0; iy < cm->nasy_y; iy++) {
        int row = cm->nasy_y - iy - 1;
        for (int ix = 0; ix < cm->nasy_x; ix++) asy_grid[row * cm->nasy_x + ix] = asy_ids[k++];
    }
    for (int id : asy_grid) {
        auto it = cm->assemblies.find(id);
        if (it == cm->assemblies.end()) MOCGPU_THROW(5, "Failed to locate assembly in core specification.");
        cm->plane_lattices.push_back(it->second);
    }
    cm->hz = cm->assembly_hz[asy_grid[0]];
    for (int id : asy_grid)
        if (cm->assembly_hz[id] != cm->hz) MOCGPU_THROW(5, "Assemblies in the core are not compatible.");
    auto lat_at = [&](int ix, int iy) -> const Lattice & { return *cm->plane_lattices[iy * cm->nasy_x + ix]; };

    // plane-level lattice boundaries and FSR offsets
    cm->plane_hx.push_back(0.0);
    double prev = 0.0;
    for (int ix = 0; ix < cm->nasy_x; ix++) {
        cm->plane_hx.push_back(prev + lat_at(ix, 0).hx);
        prev += lat_at(ix, 0).hx;
        cm->nx += lat_at(ix, 0).nx;
    }
    cm->plane_hy.push_back(0.0);
    prev = 0.0;
    for (int iy = 0; iy < cm->nasy_y; iy++) {
        cm->plane_hy.push_back(prev + lat_at(0, iy).hy);
        prev += lat_at(0, iy).hy;
        cm->ny += lat_at(0, iy).ny;
    }
    for (int iy = 0; iy < cm->nasy_y; iy++)
        for (int ix = 0; ix < cm->nasy_x; ix++)
            if (!fp_equiv_ulp(lat_at(ix, iy).hx, lat_at(ix, 0).hx) || !fp_equiv_ulp(lat_at(ix, iy).hy, lat_at(0, iy).hy))
                MOCGPU_THROW(5, "Lattices do not have compatible dimensions.");
    int reg = 0;
    for (const Lattice *l : cm->plane_lattices) {
        cm->first_reg_lattice.push_back(reg);
        reg += l->n_reg;
    }
    cm->n_reg = reg;

    // pin-level mesh boundaries (cumulative per pin, as the core mesh does)
    cm->hx = 0.0;
    for (int ix = 0; ix < cm->nasy_x; ix++) cm->hx += lat_at(ix, 0).hx;
    cm->hy = 0.0;
    for (int iy = 0; iy < cm->nasy_y; iy++) cm->hy += lat_at(0, iy).hy;
    cm->x_vec.push_back(0.0);
    double hprev = 0.0;
    for (int ix = 0; ix < cm->nasy_x; ix++)
        for (double h : lat_at(ix, 0).hx_vec) {
            cm->dx_vec.push_back(h);
            cm->x_vec.push_back(h + hprev);
            hprev += h;
        }
    cm->y_vec.push_back(0.0);
    hprev = 0.0;
    for (int iy = 0; iy < cm->nasy_y; iy++)
        for (double h : lat_at(0, iy).hy_vec) {
            cm->dy_vec.push_back(h);
            cm->y_vec.push_back(h + hprev);
            hprev += h;
        }
    // Internal pin-boundary lines. (MOCC sizes the vertical lines with the core
    // width; the core height is used here so non-square cores trace fully.
    // Both agree for square cores.)
    for (size_t i = 1; i + 1 < cm->x_vec.size(); i++)
        cm->lines.emplace_back(Point2(cm->x_vec[i], 0.0), Point2(cm->x_vec[i], std::max(cm->hx, cm->hy)));
    for (size_t i = 1; i + 1 < cm->y_vec.size(); i++)
        cm->lines.emplace_back(Point2(0.0, cm->y_vec[i]), Point2(cm->hx, cm->y_vec[i]));

    // pins in FSR order, with coarse-cell positions
    int fr = 0;
    for (int ilat = 0; ilat < (int)cm->plane_lattices.size(); ilat++) {
        const Lattice &l = *cm->plane_lattices[ilat];
        int lat_x = ilat % cm->nasy_x, lat_y = ilat / cm->nasy_x;
        int px0 = 0, py0 = 0;
        for (int ix = 0; ix < lat_x; ix++) px0 += lat_at(ix, 0).nx;
        for (int iy = 0; iy < lat_y; iy++) py0 += lat_at(0, iy).ny;
        for (int ip = 0; ip < (int)l.pins.size(); ip++) {
            cm->core_pins.push_back(l.pins[ip]);
            cm->pin_first_reg.push_back(fr);
            fr += l.pins[ip]->mesh->n_reg;
            cm->pin_cell.push_back(cm->coarse_cell(px0 + ip % l.nx, py0 + ip / l.nx));
            if (l.pins[ip]->is_fuel) cm->n_fuel_2d++;
        }
    }
    cm->prepare_surfaces();
    return cm;
}

const PinMesh *CoreMesh::get_pinmesh(Point2 &p, int &first_reg) const
{
    long ix = std::lower_bound(plane_hx.begin(), plane_hx.end(), p.x, fuzzy_lt) - plane_hx.begin();
    if (ix < (long)plane_hx.size() && fp_equiv(p.x, plane_hx[ix])) ix++;
    ix--;
    long iy = std::lower_bound(plane_hy.begin(), plane_hy.end(), p.y, fuzzy_lt) - plane_hy.begin();
    if (iy < (long)plane_hy.size() && fp_equiv(p.y, plane_hy[iy])) iy++;
    iy--;
    ix = std::min<long>(nasy_x - 1, std::max<long>(0, ix));
    iy = std::min<long>(nasy_y - 1, std::max<long>(0, iy));
    int ilat = (int)(nasy_x * iy + ix);
    p.x -= plane_hx[ix];
    p.y -= plane_hy[iy];
    first_reg += first_reg_lattice[ilat];
    const PinMesh *pm = plane_lattices[ilat]->get_pinmesh(p, first_reg);
    p.x += plane_hx[ix];
    p.y += plane_hy[iy];
    return pm;
}

int CoreMesh::point_cell(Point2 p) const
{
    long ix = std::upper_bound(x_vec.begin(), x_vec.end(), p.x) - x_vec.begin() - 1;
    long iy = std::upper_bound(y_vec.begin(), y_vec.end(), p.y) - y_vec.begin() - 1;
    ix = std::min<long>(nx - 1, std::max<long>(0, ix));
    iy = std::min<long>(ny - 1, std::max<long>(0, iy));
    return coarse_cell((int)ix, (int)iy);
}

void CoreMesh::trace(std::vector<Point2> &ps) const
{
    Line l(ps[0], ps[1]);
    for (const auto &li : lines) {
        Point2 p;
        if (intersect(li, l, p) == 1) ps.push_back(p);
    }
    std::sort(ps.begin(), ps.end());
    ps.erase(std::unique(ps.begin(), ps.end()), ps.end());
    // A ray that starts or ends (to within rounding) on a pin-cell corner
    // picks up a pin-line crossing a few 1e-13 cm from its end point that the
    // fuzzy comparison does not merge. MOCC keeps that sliver as a pin
    // crossing of its own, which adds a spurious coarse-surface crossing and
    // shifts the coarse-current walk of the whole ray by one cell (breaking
    // the CMFD balance on cores with vacuum faces). Crossings closer than
    // kSliver to either end point are dropped here; the end point's cell is
    // already chosen by the corner convention of coarse_boundary_cell().
    constexpr double kSliver = 1e-10;
    if (ps.size() > 2) {
        const Point2 a = ps.front(), b = ps.back();
        auto near_end = [&](const Point2 &p) {
            return std::hypot(p.x - a.x, p.y - a.y) < kSliver || std::hypot(p.x - b.x, p.y - b.y) < kSliver;
        };
        ps.erase(std::remove_if(ps.begin() + 1, ps.end() - 1, near_end), ps.end() - 1);
    }
}

std::vector<double> CoreMesh::areas() const
{
    std::vector<double> a;
    for (const Pin *p : core_pins)
        for (double v : p->mesh->areas) a.push_back(v);
    return a;
}

std::vector<double> CoreMesh::volumes() const
{
    std::vector<double> a = areas();
    for (double &v : a) v *= hz;
    return a;
}

// ---------------------------------------------------------------------------
// Coarse mesh numbering: per plane, the bottom z-surfaces (nx*ny), then the
// x-normal surfaces row by row, then the y-normal surfaces column by column,
// then the top z-surfaces.
void CoreMesh::prepare_surfaces()
{
    int nxsurf = nx + 1, nysurf = ny + 1;
    int nxysurf = (nx + 1) * ny + (ny + 1) * nx;
    coarse_surf_.assign(6 * nx * ny, 0);
    int i = 0;
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++) {
            int o = i * 6;
            coarse_surf_[o + EAST] = nxsurf * iy + ix + 1 + nx * ny;
            coarse_surf_[o + WEST] = nxsurf * iy + ix + nx * ny;
            coarse_surf_[o + NORTH] = nx * ny + (nx + 1) * ny + (ny + 1) * ix + iy + 1;
            coarse_surf_[o + SOUTH] = nxsurf * ny + nysurf * ix + iy + nx * ny;
            coarse_surf_[o + BOTTOM] = nx * iy + ix;
            coarse_surf_[o + TOP] = nx * ny + nxysurf + nx * iy + ix;
            i++;
        }
}

int CoreMesh::coarse_neighbor(int cell, Surface s) const
{
    int px = cell % nx, py = cell / nx;
    switch (s) {
    case NORTH: return (py < ny - 1) ? cell + nx : -1;
    case SOUTH: return (py > 0) ? cell - nx : -1;
    case EAST: return (px < nx - 1) ? cell + 1 : -1;
    case WEST: return (px > 0) ? cell - 1 : -1;
    case TOP:
    case BOTTOM: return -1;
    default: return -5;
    }
}

Normal CoreMesh::surface_normal(int surf) const
{
    int nsurfz = nx * ny + (nx + 1) * ny + (ny + 1) * nx;
    int s = surf % nsurfz;
    if (s < nx * ny) return Z_NORM;
    if (s < nx * ny + (nx + 1) * ny) return X_NORM;
    return Y_NORM;
}

std::pair<int, int> CoreMesh::coarse_neigh_cells(int surf) const
{
    int nsp = n_surf_plane();
    std::pair<int, int> c{-1, -1};
    switch (surface_normal(surf)) {
    case X_NORM: {
        int iz = surf / nsp;
        int s = surf - iz * nsp;
        int iy = (s - nx * ny) / (nx + 1);
        int ix = (s - nx * ny) % (nx + 1);
        c.first = (ix > 0) ? coarse_cell(ix - 1, iy) : -1;
        c.second = (ix < nx) ? coarse_cell(ix, iy) : -1;
    } break;
    case Y_NORM: {
        int iz = surf / nsp;
        int s = surf - iz * nsp - (nx * ny + (nx + 1) * ny);
        int iy = s % (ny + 1);
        int ix = s / (ny + 1);
        c.first = (iy > 0) ? coarse_cell(ix, iy - 1) : -1;
        c.second = (iy < ny) ? coarse_cell(ix, iy) : -1;
    } break;
    case Z_NORM: {
        int iz = surf / nsp;
        int s = surf - iz * nsp;
        int iy = s / nx, ix = s % nx;
        c.first = (iz > 0) ? coarse_cell(ix, iy) : -1;
        c.second = (iz < 1) ? coarse_cell(ix, iy) : -1;
    } break;
    }
    return c;
}

double CoreMesh::coarse_area(int surf) const
{
    int nsp = n_surf_plane();
    switch (surface_normal(surf)) {
    case X_NORM: {
        int s = surf % nsp;
        int iy = (s - nx * ny) / (nx + 1);
        return dy_vec[iy] * hz;
    }
    case Y_NORM: {
        int s = surf % nsp - (nx * ny + (nx + 1) * ny);
        int ix = s / (ny + 1);
        return dx_vec[ix] * hz;
    }
    case Z_NORM: {
        int s = (surf >= nsp) ? surf - nsp : surf;
        int iy = s / nx, ix = s % nx;
        return dx_vec[ix] * dy_vec[iy];
    }
    }
    return -1.0;
}

double CoreMesh::coarse_area(int cell, Surface s) const
{
    int px = cell % nx, py = cell / nx;
    switch (s) {
    case EAST:
    case WEST: return dy_vec[py] * hz;
    case NORTH:
    case SOUTH: return dx_vec[px] * hz;
    case TOP:
    case BOTTOM: return dx_vec[px] * dy_vec[py];
    default: return -1.0;
    }
}

namespace {
// Locates a point against the pin boundaries the way the coarse-mesh
// routines do: a coordinate "on" a boundary stops at that boundary index,
// otherwise the index is that of the cell below.
void locate(const std::vector<double> &v, double c, int &idx, bool &on)
{
    idx = 0;
    on = false;
    for (double vi : v) {
        if (fp_equiv(c, vi)) {
            on = true;
            return;
        }
        if (vi > c) {
            idx--;
            return;
        }
        idx++;
    }
}
} // namespace

int CoreMesh::coarse_norm_point(Point2 p, int octant, Surface (&s)[2]) const
{
    int ix, iy;
    bool on_x, on_y;
    locate(x_vec, p.x, ix, on_x);
    locate(y_vec, p.y, iy, on_y);
    if (!on_x && !on_y) return 0;
    if (on_x != on_y) {
        if (on_x) {
            if (ix == 0 && (octant == 1 || octant == 4)) { s[0] = WEST; return 1; }
            if (ix == nx && (octant == 2 || octant == 3)) { s[0] = EAST; return 1; }
        }
        if (on_y) {
            if (iy == 0 && (octant == 1 || octant == 2)) { s[0] = SOUTH; return 1; }
            if (iy == ny && (octant == 3 || octant == 4)) { s[0] = NORTH; return 1; }
        }
        if (on_x) {
            if (octant == 1 || octant == 4) s[0] = EAST;
            if (octant == 2 || octant == 3) s[0] = WEST;
        } else {
            if (octant == 1 || octant == 2) s[0] = NORTH;
            if (octant == 3 || octant == 4) s[0] = SOUTH;
        }
        return 1;
    }
    // corner
    if (ix > 0 && ix < nx && iy > 0 && iy < ny) {
        switch (octant) {
        case 1: s[0] = EAST; s[1] = NORTH; break;
        case 2: s[0] = WEST; s[1] = NORTH; break;
        case 3: s[0] = WEST; s[1] = SOUTH; break;
        case 4: s[0] = EAST; s[1] = SOUTH; break;
        }
        return 2;
    }
    if (ix == 0) {
        switch (octant) {
        case 1: s[0] = WEST; return 1;
        case 2: s[0] = NORTH; s[1] = WEST; return 2;
        case 3: s[0] = SOUTH; s[1] = WEST; return 2;
        case 4: s[0] = WEST; return 1;
        }
    }
    if (ix == nx) {
        switch (octant) {
        case 1: s[0] = NORTH; s[1] = EAST; return 2;
        case 2: s[0] = EAST; return 1;
        case 3: s[0] = EAST; return 1;
        case 4: s[0] = SOUTH; s[1] = EAST; return 2;
        }
    }
    if (iy == 0) {
        switch (octant) {
        case 1: s[0] = SOUTH; return 1;
        case 2: s[0] = SOUTH; return 1;
        case 3: s[0] = WEST; s[1] = SOUTH; return 2;
        case 4: s[0] = EAST; s[1] = SOUTH; return 2;
        }
    }
    if (iy == ny) {
        switch (octant) {
        case 1: s[0] = EAST; s[1] = NORTH; return 2;
        case 2: s[0] = WEST; s[1] = NORTH; return 2;
        case 3: s[0] = NORTH; return 1;
        case 4: s[0] = NORTH; return 1;
        }
    }
    return 0;
}

int CoreMesh::coarse_boundary_cell(Point2 p, int octant) const
{
    int ix, iy;
    bool on_x, on_y;
    locate(x_vec, p.x, ix, on_x);
    locate(y_vec, p.y, iy, on_y);
    if (fp_equiv_abs(p.x, 0.0)) {
        if (octant != 1 && on_y) iy--;
    } else if (fp_equiv(p.x, hx)) {
        ix--;
        if (octant != 2 && on_y) iy--;
    } else if (fp_equiv_abs(p.y, 0.0)) {
        if (octant != 1 && on_x) ix--;
    } else if (fp_equiv(p.y, hy)) {
        iy--;
        if (octant == 3 && on_x) ix--;
    } else {
        MOCGPU_THROW(6, "coarse_boundary_cell: point is not on the core boundary");
    }
    int cell = coarse_cell(ix, iy);
    if (ix < 0 || iy < 0 || ix >= nx || iy >= ny) MOCGPU_THROW(6, "coarse_boundary_cell: cell out of range");
    return cell;
}

} // namespace mocgpu
