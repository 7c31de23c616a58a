#include "problem.hpp"

#include <cmath>

#include "xml.hpp"

namespace mocgpu {

static void read_options(const XmlNode &doc, SolverOptions &o, const XmlNode *&sweeper)
{
    const XmlNode *solver = doc.child("solver");
    if (!solver) MOCGPU_THROW(7, "No <solver> specified.");
    std::string t = sanitize(solver->attr("type"));
    if (t != "eigenvalue") MOCGPU_THROW(7, "only <solver type=\"eigenvalue\"> is supported");
    o.k_tol = solver->attr_double("k_tol", -1.0);
    if (o.k_tol <= 0.0) MOCGPU_THROW(7, "Invalid k tolerance.");
    o.psi_tol = solver->attr_double("psi_tol", -1.0);
    if (o.psi_tol <= 0.0) MOCGPU_THROW(7, "Invalid psi tolerance.");
    o.max_iter = solver->attr_int("max_iter", -1);
    if (o.max_iter < 0) MOCGPU_THROW(7, "Invalid number of maximum iterations.");
    if (solver->has_attr("min_iter")) {
        o.min_iter = solver->attr_int("min_iter", -1);
        if (o.min_iter < 0 || o.min_iter > o.max_iter) MOCGPU_THROW(7, "Invalid number of minimum iterations.");
    }
    o.cmfd = solver->attr_bool("cmfd", false);
    if (const XmlNode *c = solver->child("cmfd")) {
        if (c->has_attr("k_tol")) {
            o.cmfd_k_tol = c->attr_double("k_tol", -1.0);
            if (o.cmfd_k_tol <= 0.0) MOCGPU_THROW(7, "K tolerance is invalid.");
        }
        if (c->has_attr("psi_tol")) {
            o.cmfd_psi_tol = c->attr_double("psi_tol", -1.0);
            if (o.cmfd_psi_tol <= 0.0) MOCGPU_THROW(7, "Psi tolerance is invalid.");
        }
        if (c->has_attr("residual_reduction")) {
            o.cmfd_resid_reduction = c->attr_double("residual_reduction", -1.0);
            if (o.cmfd_resid_reduction <= 0.0) MOCGPU_THROW(7, "Residual reduction is invalid.");
        }
        if (c->has_attr("max_iter")) {
            o.cmfd_max_iter = c->attr_int("max_iter", -1);
            if (o.cmfd_max_iter < 0) MOCGPU_THROW(7, "Max iterations invalid.");
        }
        o.cmfd_negative_fixup = c->attr_bool("negative_fixup", false);
        o.cmfd_enabled = c->attr_bool("enabled", true);
    }
    sweeper = solver->child("sweeper");
    if (!sweeper) MOCGPU_THROW(7, "No <sweeper> specified.");
    std::string st = sanitize(sweeper->attr("type"));
    if (st != "moc") MOCGPU_THROW(7, "only <sweeper type=\"moc\"> is supported");
    o.n_inner = sweeper->attr_int("n_inner", -1);
    if (o.n_inner < 0) MOCGPU_THROW(7, "Invalid number of inner iterations specified (n_inner).");
    if (sweeper->has_attr("boundary_update")) {
        std::string b = sanitize(sweeper->attr("boundary_update"));
        if (b == "jacobi" || b == "j") o.gs_boundary = false;
        else if (b == "gs") o.gs_boundary = true;
        else MOCGPU_THROW(7, "Unrecognized boundary update option.");
    }
    if (sweeper->has_attr("precision")) {
        std::string p = sanitize(sweeper->attr("precision"));
        if (p == "double" || p == "fp64") o.precision = 0;
        else if (p == "mixed" || p == "single" || p == "fp32") o.precision = 1;
        else MOCGPU_THROW(7, "Unrecognized precision option (double|mixed).");
    }
    if (sweeper->has_attr("bundles_per_unit")) {
        o.bundles_per_unit = sweeper->attr_int("bundles_per_unit", -1);
        if (o.bundles_per_unit < 0 || o.bundles_per_unit > 4)
            MOCGPU_THROW(7, "bundles_per_unit must be 0 (automatic) or 1..4.");
    }
    if (sweeper->has_attr("window_rows")) {
        o.window_rows = sweeper->attr_int("window_rows", -2);
        if (o.window_rows < -1 || (o.window_rows > 0 && o.window_rows % 16 != 0))
            MOCGPU_THROW(7, "window_rows must be -1 (automatic), 0 or a positive multiple of 16.");
    }
    o.tl_splitting = sweeper->attr_bool("tl_splitting", false);
    o.dump_fsr_flux = sweeper->attr_bool("dump_fsr_flux", false);
    if (sweeper->has_attr("incoming_update")) {
        std::string u = sanitize(sweeper->attr("incoming_update"));
        if (u == "off") o.incoming_update = 0;
        else if (u == "mocc") o.incoming_update = 1;
        else if (u == "surface") o.incoming_update = 2;
        else MOCGPU_THROW(7, "Unrecognized incoming_update option (off|mocc|surface).");
    }
    if (sweeper->has_attr("kernel")) {
        std::string k = sanitize(sweeper->attr("kernel"));
        if (k == "plain") o.sweep_kernel = 0;
        else if (k == "bundled") o.sweep_kernel = 1;
        else MOCGPU_THROW(7, "Unrecognized sweep kernel option (plain|bundled).");
    }
}

static RaySpec read_rays(const XmlNode &rn)
{
    RaySpec r;
    r.spacing = rn.attr_double("spacing", -1.0);
    if (r.spacing <= 0.0) MOCGPU_THROW(6, "Failed to read valid ray spacing.");
    if (rn.has_attr("volume_correction")) {
        std::string t = sanitize(rn.attr("volume_correction"));
        if (t == "flat") r.correction = VolumeCorrection::FLAT;
        else if (t == "angle") r.correction = VolumeCorrection::ANGLE;
        else if (t == "none") r.correction = VolumeCorrection::NONE;
        else MOCGPU_THROW(6, "Unrecognized volume correction option in <rays>");
    }
    if (rn.has_attr("modularity")) {
        std::string t = sanitize(rn.attr("modularity"));
        if (t == "pin") r.core_modular = false;
        else if (t == "core") r.core_modular = true;
        else MOCGPU_THROW(6, "Unrecognized modularity option.");
    }
    if (rn.has_attr("modularization")) {
        std::string t = sanitize(rn.attr("modularization"));
        if (t == "trig") r.rational = false;
        else if (t == "rational_fraction") r.rational = true;
        else MOCGPU_THROW(6, "Unrecognized modularization method specified.");
    }
    return r;
}

// <ang_quad> may sit on the sweeper or any ancestor (MOCC
// transport_sweeper.cpp:30-55); the search goes sweeper -> solver -> document.
static const XmlNode *find_angquad(const XmlNode &doc, const XmlNode &sweeper)
{
    if (const XmlNode *a = sweeper.child("ang_quad")) return a;
    if (const XmlNode *s = doc.child("solver"))
        if (const XmlNode *a = s->child("ang_quad")) return a;
    if (const XmlNode *a = doc.child("ang_quad")) return a;
    MOCGPU_THROW(7, "No angular quadrature (<ang_quad>) found.");
}

std::unique_ptr<Problem> Problem::from_xml(const std::string &xml_text, const std::string &xsl_text,
                                           const std::string &base_dir)
{
    auto doc = parse_xml(xml_text);
    auto P = std::make_unique<Problem>();
    const XmlNode *sweeper = nullptr;
    read_options(*doc, P->opts, sweeper);
    P->mesh = CoreMesh::from_xml(*doc, base_dir, xsl_text);
    const XmlNode *rn = sweeper->child("rays");
    if (!rn) MOCGPU_THROW(6, "No input privided for ray spacing.");
    RaySpec rs = read_rays(*rn);
    AngularQuadrature q = AngularQuadrature::from_xml(*find_angquad(*doc, *sweeper));
    P->rays = std::make_unique<RayData>(rs, q, *P->mesh);

    // ---- flatten ----
    const CoreMesh &m = *P->mesh;
    const RayData &rd = *P->rays;
    FlatProblem &f = P->flat;
    f.ng = m.mat_lib.ng;
    f.n_mat = (int)m.mat_lib.assigned.size();
    const int G = f.ng;
    for (const Material &mat : m.mat_lib.assigned) {
        for (int g = 0; g < G; g++) {
            f.xstr.push_back(mat.xstr[g]);
            f.xsnf.push_back(mat.xsnf[g]);
            f.xsf.push_back(mat.xsf[g]);
            f.xsch.push_back(mat.xsch[g]);
        }
        f.scat.insert(f.scat.end(), mat.scat.begin(), mat.scat.end());
    }
    for (const Pin *p : m.core_pins) {
        int xsreg = 0;
        for (int mid : p->mat_ids) {
            int dense = m.mat_lib.id_to_dense.at(mid);
            for (int k = 0; k < p->mesh->n_fsrs(xsreg); k++) f.fsr_mat.push_back(dense);
            xsreg++;
        }
    }
    f.fsr_vol = m.volumes();
    f.fsr_area = m.areas();
    f.n_fsr = (int)f.fsr_vol.size();
    if ((int)f.fsr_mat.size() != f.n_fsr) MOCGPU_THROW(5, "FSR/material count mismatch");

    const AngularQuadrature &aq = rd.quad;
    f.ndir_oct = aq.ndir_oct;
    f.n_ang = 4 * aq.ndir_oct;
    for (int i = 0; i < f.n_ang; i++) {
        const Angle &a = aq.angles[i];
        f.ang_ox.push_back(a.ox);
        f.ang_oy.push_back(a.oy);
        f.ang_oz.push_back(a.oz);
        f.ang_alpha.push_back(a.alpha);
        f.ang_theta.push_back(a.theta);
        f.ang_weight.push_back(a.weight);
        f.ang_rsintheta.push_back(a.rsintheta);
    }
    f.n_sets = rd.n_sets;
    f.pol_per_set = rd.pol_per_set;
    f.set_nx = rd.nx;
    f.set_ny = rd.ny;
    f.set_spacing = rd.spacing;
    f.max_seg = rd.max_seg;
    f.trk_seg_begin.push_back(0);
    f.trk_cm_begin.push_back(0);
    for (int s = 0; s < rd.n_sets; s++) {
        f.set_first_track.push_back(f.n_tracks);
        for (const Ray &r : rd.rays[s]) {
            f.trk_bc0.push_back(r.bc[0]);
            f.trk_bc1.push_back(r.bc[1]);
            f.trk_set.push_back(s);
            f.seg_len.insert(f.seg_len.end(), r.seg_len.begin(), r.seg_len.end());
            f.seg_fsr.insert(f.seg_fsr.end(), r.seg_fsr.begin(), r.seg_fsr.end());
            f.trk_seg_begin.push_back((int64_t)f.seg_len.size());
            f.trk_cm_cell_fw.push_back(r.cm_cell_fw);
            f.trk_cm_cell_bw.push_back(r.cm_cell_bw);
            f.trk_cm_surf_fw.push_back(r.cm_surf_fw);
            f.trk_cm_surf_bw.push_back(r.cm_surf_bw);
            for (const CoarseCrossing &c : r.cm_data) {
                f.cm_fw.push_back((int)c.fw);
                f.cm_bw.push_back((int)c.bw);
                f.cm_nseg_fw.push_back(c.nseg_fw);
                f.cm_nseg_bw.push_back(c.nseg_bw);
            }
            f.trk_cm_begin.push_back((int)f.cm_fw.size());
            f.n_tracks++;
        }
    }
    f.set_first_track.push_back(f.n_tracks);
    f.n_seg = (int64_t)f.seg_len.size();
    for (int64_t i = 0; i < f.n_seg; i++)
        if (f.seg_fsr[i] < 0 || f.seg_fsr[i] >= f.n_fsr) MOCGPU_THROW(6, "segment FSR index out of range");

    f.nx = m.nx;
    f.ny = m.ny;
    f.n_pin = m.nx * m.ny;
    f.n_surf = m.n_surf();
    f.n_fuel_2d = m.n_fuel_2d;
    f.hz = m.hz;
    for (int i = 0; i < 6; i++) f.bc[i] = (int)m.bc[i];
    f.dx = m.dx_vec;
    f.dy = m.dy_vec;
    for (size_t i = 0; i < m.core_pins.size(); i++) {
        f.pin_first_reg.push_back(m.pin_first_reg[i]);
        f.pin_cell.push_back(m.pin_cell[i]);
        f.pin_fuel.push_back(m.core_pins[i]->is_fuel ? 1 : 0);
        f.pin_area.push_back(m.core_pins[i]->mesh->pitch_x * m.core_pins[i]->mesh->pitch_y);
    }
    f.pin_first_reg.push_back(f.n_fsr);
    return P;
}

CrossSections cross_sections_of(const FlatProblem &f)
{
    CrossSections x;
    x.ng = f.ng;
    x.xstr = f.xstr;
    x.xsnf = f.xsnf;
    x.xsf = f.xsf;
    x.xsch = f.xsch;
    x.scat = f.scat;
    return x;
}

CrossSections cross_sections_from_xsl(const Problem &base, const std::string &xsl_text)
{
    MaterialLib lib = MaterialLib::from_xsl_text(xsl_text);
    const MaterialLib &ref = base.mesh->mat_lib;
    if (lib.ng != ref.ng) MOCGPU_THROW(4, "cross-section library has a different number of groups");
    CrossSections x;
    x.ng = lib.ng;
    const int G = lib.ng;
    for (const Material &old : ref.assigned) {
        auto it = lib.by_name.find(old.name);
        if (it == lib.by_name.end()) MOCGPU_THROW(4, "material not in library: " + old.name);
        const Material &m = lib.lib[it->second];
        if (m.fissile != old.fissile) MOCGPU_THROW(4, "library changes whether material " + old.name + " is fissile");
        for (int g = 0; g < G; g++) {
            x.xstr.push_back(m.xstr[g]);
            x.xsnf.push_back(m.xsnf[g]);
            x.xsf.push_back(m.xsf[g]);
            x.xsch.push_back(m.xsch[g]);
        }
        x.scat.insert(x.scat.end(), m.scat.begin(), m.scat.end());
    }
    return x;
}

FlatProblem flat_without_tracks(const FlatProblem &f)
{
    FlatProblem c;
    c.ng = f.ng;
    c.n_fsr = f.n_fsr;
    c.n_mat = f.n_mat;
    c.ndir_oct = f.ndir_oct;
    c.n_ang = f.n_ang;
    c.n_sets = f.n_sets;
    c.pol_per_set = f.pol_per_set;
    c.nx = f.nx;
    c.ny = f.ny;
    c.n_pin = f.n_pin;
    c.n_surf = f.n_surf;
    c.n_fuel_2d = f.n_fuel_2d;
    c.hz = f.hz;
    for (int i = 0; i < 6; i++) c.bc[i] = f.bc[i];
    c.n_tracks = f.n_tracks;
    c.n_seg = f.n_seg;
    c.max_seg = f.max_seg;
    c.xstr = f.xstr;
    c.xsnf = f.xsnf;
    c.xsf = f.xsf;
    c.xsch = f.xsch;
    c.scat = f.scat;
    c.fsr_mat = f.fsr_mat;
    c.fsr_vol = f.fsr_vol;
    c.fsr_area = f.fsr_area;
    c.ang_ox = f.ang_ox;
    c.ang_oy = f.ang_oy;
    c.ang_oz = f.ang_oz;
    c.ang_alpha = f.ang_alpha;
    c.ang_theta = f.ang_theta;
    c.ang_weight = f.ang_weight;
    c.ang_rsintheta = f.ang_rsintheta;
    c.set_nx = f.set_nx;
    c.set_ny = f.set_ny;
    c.set_first_track = f.set_first_track;
    c.set_spacing = f.set_spacing;
    c.dx = f.dx;
    c.dy = f.dy;
    c.pin_first_reg = f.pin_first_reg;
    c.pin_cell = f.pin_cell;
    c.pin_fuel = f.pin_fuel;
    c.pin_area = f.pin_area;
    return c;
}

} // namespace mocgpu
