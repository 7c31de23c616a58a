// extern "C" boundary of the library (declarations in include/mocgpu.h).
#include "../../include/mocgpu.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "device/batch.hpp"
#include "device/sweeper.hpp"
#include "host/materials.hpp"
#include "host/problem.hpp"
#include "host/xml.hpp"

struct mocgpu_problem {
    std::shared_ptr<mocgpu::Problem> P;
};
struct mocgpu_sweeper {
    std::unique_ptr<mocgpu::Sweeper> S;
    cudaStream_t stream = nullptr;
};
struct mocgpu_batch {
    std::unique_ptr<mocgpu::BatchEngine> E;
    cudaStream_t stream = nullptr;
};

namespace {
thread_local std::string g_err;

template <typename F> int guarded(F &&f)
{
    try {
        f();
        return MOCGPU_OK;
    } catch (const mocgpu::Error &e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_err = "host out of memory";
        return MOCGPU_ERR_INTERNAL;
    } catch (const std::exception &e) {
        g_err = e.what();
        return MOCGPU_ERR_INTERNAL;
    }
}

#define REQUIRE(cond, msg)                                                                                           \
    do {                                                                                                             \
        if (!(cond)) throw mocgpu::Error(MOCGPU_ERR_ARG, msg);                                                       \
    } while (0)

struct Field {
    const void *p;
    int64_t bytes;
};

template <typename T> Field fld(const std::vector<T> &v) { return Field{v.data(), (int64_t)(v.size() * sizeof(T))}; }

Field find_field(const mocgpu::FlatProblem &f, const std::string &name)
{
    static const char *names[] = {nullptr};
    (void)names;
    if (name == "xstr") return fld(f.xstr);
    if (name == "xsnf") return fld(f.xsnf);
    if (name == "xsf") return fld(f.xsf);
    if (name == "xsch") return fld(f.xsch);
    if (name == "scat") return fld(f.scat);
    if (name == "fsr_mat") return fld(f.fsr_mat);
    if (name == "fsr_vol") return fld(f.fsr_vol);
    if (name == "fsr_area") return fld(f.fsr_area);
    if (name == "ang_ox") return fld(f.ang_ox);
    if (name == "ang_oy") return fld(f.ang_oy);
    if (name == "ang_oz") return fld(f.ang_oz);
    if (name == "ang_alpha") return fld(f.ang_alpha);
    if (name == "ang_theta") return fld(f.ang_theta);
    if (name == "ang_weight") return fld(f.ang_weight);
    if (name == "ang_rsintheta") return fld(f.ang_rsintheta);
    if (name == "set_nx") return fld(f.set_nx);
    if (name == "set_ny") return fld(f.set_ny);
    if (name == "set_first_track") return fld(f.set_first_track);
    if (name == "set_spacing") return fld(f.set_spacing);
    if (name == "trk_bc0") return fld(f.trk_bc0);
    if (name == "trk_bc1") return fld(f.trk_bc1);
    if (name == "trk_set") return fld(f.trk_set);
    if (name == "trk_seg_begin") return fld(f.trk_seg_begin);
    if (name == "trk_cm_cell_fw") return fld(f.trk_cm_cell_fw);
    if (name == "trk_cm_cell_bw") return fld(f.trk_cm_cell_bw);
    if (name == "trk_cm_surf_fw") return fld(f.trk_cm_surf_fw);
    if (name == "trk_cm_surf_bw") return fld(f.trk_cm_surf_bw);
    if (name == "trk_cm_begin") return fld(f.trk_cm_begin);
    if (name == "cm_fw") return fld(f.cm_fw);
    if (name == "cm_bw") return fld(f.cm_bw);
    if (name == "cm_nseg_fw") return fld(f.cm_nseg_fw);
    if (name == "cm_nseg_bw") return fld(f.cm_nseg_bw);
    if (name == "seg_len") return fld(f.seg_len);
    if (name == "seg_fsr") return fld(f.seg_fsr);
    if (name == "dx") return fld(f.dx);
    if (name == "dy") return fld(f.dy);
    if (name == "pin_first_reg") return fld(f.pin_first_reg);
    if (name == "pin_cell") return fld(f.pin_cell);
    if (name == "pin_fuel") return fld(f.pin_fuel);
    if (name == "pin_area") return fld(f.pin_area);
    if (name == "bc") return Field{f.bc, (int64_t)sizeof(f.bc)};
    if (name == "hz") return Field{&f.hz, (int64_t)sizeof(double)};
    throw mocgpu::Error(MOCGPU_ERR_ARG, "unknown problem field: " + name);
}

void opts_to_c(const mocgpu::SolverOptions &o, mocgpu_options *c)
{
    c->k_tol = o.k_tol;
    c->psi_tol = o.psi_tol;
    c->max_iter = o.max_iter;
    c->min_iter = o.min_iter;
    c->cmfd = o.cmfd;
    c->cmfd_enabled = o.cmfd_enabled;
    c->cmfd_k_tol = o.cmfd_k_tol;
    c->cmfd_psi_tol = o.cmfd_psi_tol;
    c->cmfd_resid_reduction = o.cmfd_resid_reduction;
    c->cmfd_max_iter = o.cmfd_max_iter;
    c->cmfd_negative_fixup = o.cmfd_negative_fixup;
    c->n_inner = o.n_inner;
    c->gs_boundary = o.gs_boundary;
    c->precision = o.precision;
    c->sweep_kernel = o.sweep_kernel;
    c->bundles_per_unit = o.bundles_per_unit;
    c->window_rows = o.window_rows;
    c->incoming_update = o.incoming_update;
    c->tl_splitting = o.tl_splitting ? 1 : 0;
    c->dump_fsr_flux = o.dump_fsr_flux ? 1 : 0;
}
void opts_from_c(const mocgpu_options *c, mocgpu::SolverOptions &o)
{
    REQUIRE(c->k_tol > 0 && c->psi_tol > 0, "tolerances must be positive");
    REQUIRE(c->max_iter >= 0 && c->min_iter >= 0 && c->n_inner >= 0, "iteration counts must be non-negative");
    o.k_tol = c->k_tol;
    o.psi_tol = c->psi_tol;
    o.max_iter = c->max_iter;
    o.min_iter = c->min_iter;
    o.cmfd = c->cmfd != 0;
    o.cmfd_enabled = c->cmfd_enabled != 0;
    o.cmfd_k_tol = c->cmfd_k_tol;
    o.cmfd_psi_tol = c->cmfd_psi_tol;
    o.cmfd_resid_reduction = c->cmfd_resid_reduction;
    o.cmfd_max_iter = c->cmfd_max_iter;
    o.cmfd_negative_fixup = c->cmfd_negative_fixup != 0;
    o.n_inner = c->n_inner;
    o.gs_boundary = c->gs_boundary != 0;
    o.precision = c->precision;
    REQUIRE(c->sweep_kernel == 0 || c->sweep_kernel == 1, "sweep_kernel must be 0 or 1");
    o.sweep_kernel = c->sweep_kernel;
    REQUIRE(c->bundles_per_unit >= 0 && c->bundles_per_unit <= 4, "bundles_per_unit must be 0..4");
    o.bundles_per_unit = c->bundles_per_unit;
    REQUIRE(c->window_rows >= -1 && (c->window_rows <= 0 || c->window_rows % 16 == 0),
            "window_rows must be -1, 0 or a positive multiple of 16");
    o.window_rows = c->window_rows;
    REQUIRE(c->incoming_update >= 0 && c->incoming_update <= 2, "incoming_update must be 0, 1 or 2");
    o.incoming_update = c->incoming_update;
    o.tl_splitting = c->tl_splitting != 0;
    o.dump_fsr_flux = c->dump_fsr_flux != 0;
}
} // namespace

extern "C" {

const char *mocgpu_last_error(void) { return g_err.c_str(); }
int mocgpu_version(void) { return 100; }

int mocgpu_device_count(int *n)
{
    return guarded([&] {
        REQUIRE(n, "null output");
        int c = 0;
        cudaError_t e = cudaGetDeviceCount(&c);
        *n = (e == cudaSuccess) ? c : 0;
    });
}

int mocgpu_problem_create(const char *xml_text, const char *xsl_text, const char *base_dir, mocgpu_problem **out)
{
    return guarded([&] {
        REQUIRE(xml_text && out, "null argument");
        auto h = std::make_unique<mocgpu_problem>();
        h->P = mocgpu::Problem::from_xml(xml_text, xsl_text ? xsl_text : "", base_dir ? base_dir : "");
        *out = h.release();
    });
}

void mocgpu_problem_destroy(mocgpu_problem *p) { delete p; }

int mocgpu_problem_quadrature(const mocgpu_problem *p, int *n_polar, int *n_azimuthal, double *out, int64_t cap,
                              int64_t *ndir)
{
    return guarded([&] {
        REQUIRE(p && n_polar && n_azimuthal && ndir && cap >= 0 && (out || cap == 0), "null argument");
        const mocgpu::AngularQuadrature &q = p->P->rays->quad;
        *n_polar = q.n_polar;
        *n_azimuthal = q.n_azimuthal;
        *ndir = q.ndir();
        for (int i = 0; i < q.ndir() && i < cap; i++) {
            const mocgpu::Angle &a = q[i];
            const double v[6] = {a.alpha, a.theta, a.ox, a.oy, a.oz, a.weight};
            std::copy(v, v + 6, out + (size_t)6 * i);
        }
    });
}
int mocgpu_problem_group_bounds(const mocgpu_problem *p, double *out, int cap, int *n)
{
    return guarded([&] {
        REQUIRE(p && n && cap >= 0 && (out || cap == 0), "null argument");
        const std::vector<double> &b = p->P->mesh->mat_lib.group_bounds;
        *n = (int)b.size();
        std::copy(b.begin(), b.begin() + std::min<size_t>((size_t)cap, b.size()), out);
    });
}
int mocgpu_problem_sizes(const mocgpu_problem *p, int64_t *s)
{
    return guarded([&] {
        REQUIRE(p && s, "null argument");
        const auto &f = p->P->flat;
        s[MOCGPU_SZ_NGROUP] = f.ng;
        s[MOCGPU_SZ_NFSR] = f.n_fsr;
        s[MOCGPU_SZ_NMAT] = f.n_mat;
        s[MOCGPU_SZ_NDIR_OCT] = f.ndir_oct;
        s[MOCGPU_SZ_NANG] = f.n_ang;
        s[MOCGPU_SZ_NSETS] = f.n_sets;
        s[MOCGPU_SZ_POL_PER_SET] = f.pol_per_set;
        s[MOCGPU_SZ_NX] = f.nx;
        s[MOCGPU_SZ_NY] = f.ny;
        s[MOCGPU_SZ_NPIN] = f.n_pin;
        s[MOCGPU_SZ_NSURF] = f.n_surf;
        s[MOCGPU_SZ_NFUEL] = f.n_fuel_2d;
        s[MOCGPU_SZ_NTRACKS] = f.n_tracks;
        s[MOCGPU_SZ_NSEG] = f.n_seg;
        s[MOCGPU_SZ_NCM] = (int64_t)f.cm_fw.size();
        s[MOCGPU_SZ_MAXSEG] = f.max_seg;
    });
}

int mocgpu_problem_options(const mocgpu_problem *p, mocgpu_options *out)
{
    return guarded([&] {
        REQUIRE(p && out, "null argument");
        opts_to_c(p->P->opts, out);
    });
}

int mocgpu_problem_set_options(mocgpu_problem *p, const mocgpu_options *in)
{
    return guarded([&] {
        REQUIRE(p && in, "null argument");
        opts_from_c(in, p->P->opts);
    });
}

int mocgpu_problem_field_bytes(const mocgpu_problem *p, const char *field, int64_t *nbytes)
{
    return guarded([&] {
        REQUIRE(p && field && nbytes, "null argument");
        *nbytes = find_field(p->P->flat, field).bytes;
    });
}

int mocgpu_problem_export(const mocgpu_problem *p, const char *field, void *dst, int64_t nbytes)
{
    return guarded([&] {
        REQUIRE(p && field && dst, "null argument");
        Field f = find_field(p->P->flat, field);
        REQUIRE(f.bytes == nbytes, std::string("size mismatch for field ") + field);
        if (nbytes) std::memcpy(dst, f.p, (size_t)nbytes);
    });
}

int mocgpu_synthetic_xsl(uint64_t seed, int n_group, int n_fuel, const double *fuel_nf_scale, double mod_factor,
                         double fuel_nf_factor, char *buf, int64_t buflen, int64_t *needed)
{
    return guarded([&] {
        REQUIRE(n_group >= 3 && n_fuel >= 1, "need n_group >= 3 and n_fuel >= 1");
        mocgpu::SyntheticXsSpec spec;
        spec.ng = n_group;
        spec.seed = seed;
        spec.n_fuel = n_fuel;
        if (fuel_nf_scale) spec.fuel_nf_scale.assign(fuel_nf_scale, fuel_nf_scale + n_fuel);
        spec.mod_factor = mod_factor;
        spec.fuel_nf_factor = fuel_nf_factor;
        std::string t = mocgpu::synthetic_xsl(spec);
        if (needed) *needed = (int64_t)t.size() + 1;
        if (buf && buflen > 0) {
            size_t n = std::min<size_t>((size_t)buflen - 1, t.size());
            std::memcpy(buf, t.data(), n);
            buf[n] = '\0';
        }
    });
}

int mocgpu_trace_ray(const char *xml_text, const char *xsl_text, double x1, double y1, double x2, double y2,
                     int *nseg, double *seg_len, int *seg_fsr, int cap, int *coarse, int *ncm, int *cm, int cm_cap)
{
    return guarded([&] {
        REQUIRE(xml_text && nseg && ncm, "null argument");
        auto doc = mocgpu::parse_xml(xml_text);
        auto mesh = mocgpu::CoreMesh::from_xml(*doc, "", xsl_text ? xsl_text : "");
        mocgpu::Ray r(mocgpu::Point2(x1, y1), mocgpu::Point2(x2, y2), {0, 0}, *mesh);
        *nseg = r.nseg();
        for (int i = 0; i < r.nseg() && i < cap; i++) {
            if (seg_len) seg_len[i] = r.seg_len[i];
            if (seg_fsr) seg_fsr[i] = r.seg_fsr[i];
        }
        if (coarse) {
            coarse[0] = r.cm_cell_fw;
            coarse[1] = r.cm_cell_bw;
            coarse[2] = r.cm_surf_fw;
            coarse[3] = r.cm_surf_bw;
        }
        *ncm = (int)r.cm_data.size();
        for (int i = 0; i < (int)r.cm_data.size() && i < cm_cap; i++) {
            if (!cm) break;
            cm[4 * i + 0] = (int)r.cm_data[i].fw;
            cm[4 * i + 1] = (int)r.cm_data[i].bw;
            cm[4 * i + 2] = r.cm_data[i].nseg_fw;
            cm[4 * i + 3] = r.cm_data[i].nseg_bw;
        }
    });
}

// ---------------------------------------------------------------------------
int mocgpu_sweeper_create(const mocgpu_problem *p, int precision, mocgpu_sweeper **out)
{
    return guarded([&] {
        REQUIRE(p && out, "null argument");
        REQUIRE(precision >= -1 && precision <= 1, "precision must be -1, 0 or 1");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
            throw mocgpu::Error(MOCGPU_ERR_CUDA, "no CUDA device available: the sweeper runs on the GPU only");
        auto h = std::make_unique<mocgpu_sweeper>();
        MOCGPU_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        try {
            h->S = std::make_unique<mocgpu::Sweeper>(*p->P, precision, h->stream);
        } catch (...) {
            cudaStreamDestroy(h->stream);
            throw;
        }
        *out = h.release();
    });
}

int mocgpu_sweeper_create_xsl(const mocgpu_problem *p, int precision, const char *xsl_text, mocgpu_sweeper **out)
{
    return guarded([&] {
        REQUIRE(p && out, "null argument");
        REQUIRE(precision >= -1 && precision <= 1, "precision must be -1, 0 or 1");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
            throw mocgpu::Error(MOCGPU_ERR_CUDA, "no CUDA device available: the sweeper runs on the GPU only");
        std::unique_ptr<mocgpu::CrossSections> xs;
        if (xsl_text && *xsl_text)
            xs = std::make_unique<mocgpu::CrossSections>(mocgpu::cross_sections_from_xsl(*p->P, xsl_text));
        auto h = std::make_unique<mocgpu_sweeper>();
        MOCGPU_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        try {
            h->S = std::make_unique<mocgpu::Sweeper>(*p->P, precision, h->stream, nullptr, xs.get());
        } catch (...) {
            cudaStreamDestroy(h->stream);
            throw;
        }
        *out = h.release();
    });
}

void mocgpu_sweeper_destroy(mocgpu_sweeper *s)
{
    if (!s) return;
    cudaStream_t st = s->stream;
    s->S.reset();
    if (st) cudaStreamDestroy(st);
    delete s;
}

static mocgpu::Sweeper &sw(mocgpu_sweeper *s)
{
    if (!s || !s->S) throw mocgpu::Error(MOCGPU_ERR_ARG, "null sweeper");
    return *s->S;
}

int mocgpu_sweeper_set_options(mocgpu_sweeper *s, const mocgpu_options *in)
{
    return guarded([&] {
        REQUIRE(in, "null argument");
        auto &S = sw(s);
        int prec = S.precision();
        opts_from_c(in, S.options());
        S.options().precision = prec;
    });
}
int mocgpu_initialize(mocgpu_sweeper *s)
{
    return guarded([&] { sw(s).initialize(); });
}
int mocgpu_calc_fission_source(mocgpu_sweeper *s, double k, double *fs)
{
    return guarded([&] {
        REQUIRE(k != 0.0, "k must be non-zero");
        auto &S = sw(s);
        S.calc_fission_source(k);
        if (fs) S.get_fission_source(fs);
    });
}
int mocgpu_set_fission_source(mocgpu_sweeper *s, const double *fs)
{
    return guarded([&] {
        REQUIRE(fs, "null argument");
        sw(s).set_fission_source(fs);
    });
}
int mocgpu_store_old_flux(mocgpu_sweeper *s)
{
    return guarded([&] { sw(s).store_old_flux(); });
}
int mocgpu_source_group(mocgpu_sweeper *s, int group)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(group >= 0 && group < S.flat().ng, "group out of range");
        S.group_source(group);
    });
}
int mocgpu_sweep_group(mocgpu_sweeper *s, int group)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(group >= 0 && group < S.flat().ng, "group out of range");
        S.sweep(group);
        MOCGPU_CUDA(cudaStreamSynchronize(S.stream()));
        MOCGPU_CUDA(cudaGetLastError());
    });
}
int mocgpu_set_coarse_data(mocgpu_sweeper *s, int enabled)
{
    return guarded([&] { sw(s).set_coarse_enabled(enabled != 0); });
}
int mocgpu_total_fission(mocgpu_sweeper *s, int old, double *out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        *out = sw(s).total_fission(old != 0);
    });
}
int mocgpu_flux_residual(mocgpu_sweeper *s, double *out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        *out = sw(s).flux_residual();
    });
}
int mocgpu_get_flux(mocgpu_sweeper *s, double *flux)
{
    return guarded([&] {
        REQUIRE(flux, "null argument");
        sw(s).get_flux(flux);
    });
}
int mocgpu_set_flux(mocgpu_sweeper *s, const double *flux)
{
    return guarded([&] {
        REQUIRE(flux, "null argument");
        sw(s).set_flux(flux);
    });
}
int mocgpu_eigen_history(mocgpu_sweeper *s, double *out, int64_t cap, int64_t *n)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(n && cap >= 0 && (out || cap == 0), "bad argument");
        const std::vector<double> &h = S.history();
        *n = (int64_t)h.size() / 4;
        std::copy(h.begin(), h.begin() + std::min<int64_t>(4 * cap, (int64_t)h.size()), out);
    });
}
int mocgpu_get_boundary_flux(mocgpu_sweeper *s, int group, double *out, int64_t cap, int64_t *n)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(n && group >= 0 && group < S.flat().ng && cap >= 0 && (out || cap == 0), "bad argument");
        std::vector<double> v = S.get_boundary(group);
        *n = (int64_t)v.size();
        std::copy(v.begin(), v.begin() + std::min<int64_t>(cap, (int64_t)v.size()), out);
    });
}
int mocgpu_get_pin_flux_1g(mocgpu_sweeper *s, int group, double *out)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(out && group >= 0 && group < S.flat().ng, "bad argument");
        S.get_pin_flux(group, out);
    });
}
int mocgpu_set_pin_flux_1g(mocgpu_sweeper *s, int group, const double *in, double *resid)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(in && group >= 0 && group < S.flat().ng, "bad argument");
        double r = S.set_pin_flux(group, in);
        if (resid) *resid = r;
    });
}
int mocgpu_pin_powers(mocgpu_sweeper *s, double *out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        sw(s).pin_powers(out);
    });
}
int mocgpu_get_coarse_currents(mocgpu_sweeper *s, double *current, double *surface_flux)
{
    return guarded([&] {
        REQUIRE(current && surface_flux, "null argument");
        sw(s).get_currents(current, surface_flux);
    });
}
int mocgpu_homogenized_xs(mocgpu_sweeper *s, double *xstr, double *xsnf, double *xsf, double *xsch, double *xsrm,
                          double *scat)
{
    return guarded([&] { sw(s).homogenized_xs(xstr, xsnf, xsf, xsch, xsrm, scat); });
}
int mocgpu_cmfd_solve(mocgpu_sweeper *s, double *k)
{
    return guarded([&] {
        REQUIRE(k, "null argument");
        sw(s).cmfd_solve(*k);
    });
}
int mocgpu_update_incoming_flux(mocgpu_sweeper *s, const double *part, const double *part_old, int has_old, int mode)
{
    return guarded([&] {
        REQUIRE(part && (part_old || !has_old), "null argument");
        REQUIRE(mode == 1 || mode == 2, "mode must be 1 (MOCC's lookup) or 2 (entry surface)");
        sw(s).update_incoming_flux(part, part_old, has_old, mode);
    });
}
int mocgpu_apply_transverse_leakage(mocgpu_sweeper *s, int group, const double *tl)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(tl && group >= 0 && group < S.flat().ng, "bad argument");
        S.apply_transverse_leakage(group, tl);
    });
}
int mocgpu_cmfd_solve_static(mocgpu_sweeper *s, double *k)
{
    return guarded([&] {
        REQUIRE(k, "null argument");
        sw(s).cmfd_solve_static(*k);
    });
}
int mocgpu_eigen_solve(mocgpu_sweeper *s, int max_outer, mocgpu_result *out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        mocgpu::EigenResult r = sw(s).eigen_solve(max_outer);
        out->k = r.k;
        out->iterations = r.iterations;
        out->converged = r.converged;
        out->error_k = r.error_k;
        out->error_psi = r.error_psi;
        out->seconds = r.seconds;
        out->sweeps = r.sweeps;
        out->cmfd_iterations = r.cmfd_iterations;
    });
}
int mocgpu_sweeper_bytes(mocgpu_sweeper *s, int64_t *device_bytes, double *sweep_bytes)
{
    return guarded([&] {
        auto &S = sw(s);
        if (device_bytes) *device_bytes = (int64_t)S.device_bytes();
        if (sweep_bytes) *sweep_bytes = S.sweep_bytes();
    });
}

int mocgpu_layout_stats(const mocgpu_problem *p, int gs, int tracks_per_unit, int max_local, int window_rows,
                        int64_t *stats, double *stats_d)
{
    return guarded([&] {
        REQUIRE(p && stats && stats_d, "null argument");
        mocgpu::SweepLayout L =
            mocgpu::build_sweep_layout(p->P->flat, gs != 0, tracks_per_unit, max_local, true, window_rows);
        int64_t real = 0;
        double sum = 0.0;
        std::vector<int> unit_of(L.bundle_row.size(), -1);
        for (size_t u = 0; u < L.wu.size(); u++)
            for (int b = L.wu[u].bundle_begin; b < L.wu[u].bundle_begin + L.wu[u].n_bundles; b++) unit_of[b] = (int)u;
        const auto &f = p->P->flat;
        for (size_t b = 0; b < L.bundle_row.size(); b++) {
            const int wu = unit_of[b];
            if (wu < 0) throw mocgpu::Error(MOCGPU_ERR_INTERNAL, "bundle outside every work unit");
            for (int lane = 0; lane < 32; lane++) {
                int t = L.bundle_track[b * 32 + lane];
                int n = t < 0 ? 0 : (int)(f.trk_seg_begin[t + 1] - f.trk_seg_begin[t]);
                for (int r = 0; r < L.bundle_nrows[b]; r++) {
                    size_t i = (size_t)(L.bundle_row[b] + r) * 32 + lane;
                    // the row's window
                    const int wr = L.wu[wu].n_win > 1 ? L.window_rows : (1 << 30);
                    const int w = r / wr;
                    if (w >= L.wu[wu].n_win) throw mocgpu::Error(MOCGPU_ERR_INTERNAL, "row outside its unit's windows");
                    const mocgpu::RowWindowHost &W = L.win[L.wu[wu].win_begin + w];
                    if (r < n) {
                        real++;
                        sum += L.len[i];
                        // the window-local index must map back to the segment's FSR
                        if (L.lfsr[i] >= W.n_local || L.local_fsr[W.fsr_begin + L.lfsr[i]] != f.seg_fsr[f.trk_seg_begin[t] + r] ||
                            L.len[i] != f.seg_len[f.trk_seg_begin[t] + r])
                            throw mocgpu::Error(MOCGPU_ERR_INTERNAL, "layout maps a segment to the wrong FSR or length");
                    } else if (L.len[i] != 0.0 || L.lfsr[i] != W.n_local) {
                        throw mocgpu::Error(MOCGPU_ERR_INTERNAL, "padding entry not zero-length or not on the padding slot");
                    }
                }
            }
        }
        stats[0] = (int64_t)L.wu.size();
        stats[1] = (int64_t)L.bundle_row.size();
        stats[2] = L.n_rows;
        stats[3] = real;
        stats[4] = L.max_local;
        stats[5] = L.n_phases;
        stats[6] = L.max_windows;
        stats[7] = (int64_t)L.win.size();
        stats_d[0] = sum;
        stats_d[1] = L.padding;
    });
}

int mocgpu_sweeper_layout(mocgpu_sweeper *s, int *units, int *tracks_per_unit, int *window_rows, int *table_slots)
{
    return guarded([&] {
        REQUIRE(units && tracks_per_unit && window_rows && table_slots, "null argument");
        const auto &G = *sw(s).geometry();
        *units = G.layout_units;
        *tracks_per_unit = G.layout_tracks_per_unit;
        *window_rows = G.layout_window_rows;
        *table_slots = G.layout_max_local;
    });
}
int mocgpu_sweeper_stream(mocgpu_sweeper *s, void **stream)
{
    return guarded([&] {
        REQUIRE(s && stream, "null argument");
        *stream = (void *)s->stream;
    });
}
int mocgpu_time_sweep(mocgpu_sweeper *s, int group, int reps, double *ms, int *launches)
{
    return guarded([&] {
        auto &S = sw(s);
        REQUIRE(ms && reps > 0 && group >= 0 && group < S.flat().ng, "bad argument");
        *ms = S.time_sweep(group, reps, launches);
    });
}
int mocgpu_launch_count(int64_t *n)
{
    return guarded([&] {
        REQUIRE(n, "null argument");
        *n = mocgpu::launch_count();
    });
}

/* ---- batched solves ------------------------------------------------------ */
static mocgpu::BatchEngine &eng(mocgpu_batch *b)
{
    if (!b || !b->E) throw mocgpu::Error(MOCGPU_ERR_ARG, "null batch handle");
    return *b->E;
}

int mocgpu_batch_create(int precision, int capacity, double mem_budget_bytes, int bundles_per_unit,
                        mocgpu_batch **out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        REQUIRE(precision == 0 || precision == 1, "precision must be 0 or 1");
        REQUIRE(capacity >= 1 && capacity <= 65535, "capacity must be in [1, 65535]");
        REQUIRE(bundles_per_unit >= 1 && bundles_per_unit <= 4, "bundles_per_unit must be in [1, 4]");
        REQUIRE(mem_budget_bytes >= 0.0, "negative memory budget");
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
            throw mocgpu::Error(MOCGPU_ERR_CUDA, "no CUDA device available: the batch engine runs on the GPU only");
        auto h = std::make_unique<mocgpu_batch>();
        MOCGPU_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        try {
            h->E = std::make_unique<mocgpu::BatchEngine>(precision, capacity, (size_t)mem_budget_bytes,
                                                         bundles_per_unit, h->stream);
        } catch (...) {
            cudaStreamDestroy(h->stream);
            throw;
        }
        *out = h.release();
    });
}

void mocgpu_batch_destroy(mocgpu_batch *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->E.reset();
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int mocgpu_batch_submit(mocgpu_batch *b, const mocgpu_problem *p, const char *xsl_text, int64_t *id)
{
    return guarded([&] {
        REQUIRE(p && p->P && id, "null argument");
        auto &E = eng(b);
        if (xsl_text && *xsl_text) {
            mocgpu::CrossSections xs = mocgpu::cross_sections_from_xsl(*p->P, xsl_text);
            *id = E.submit(p->P, &xs);
        } else {
            *id = E.submit(p->P, nullptr);
        }
    });
}

int mocgpu_batch_submit_xml(mocgpu_batch *b, const char *xml_text, const char *xsl_text, const char *base_dir,
                            int64_t *id)
{
    return guarded([&] {
        REQUIRE(xml_text && id, "null argument");
        *id = eng(b).submit_xml(xml_text, xsl_text ? xsl_text : "", base_dir ? base_dir : "");
    });
}

int mocgpu_batch_cancel(mocgpu_batch *b, int64_t id, int *found)
{
    return guarded([&] {
        REQUIRE(found, "null argument");
        *found = eng(b).cancel(id) ? 1 : 0;
    });
}

int mocgpu_debug_fail_allocations(int64_t after)
{
    return guarded([&] { mocgpu::set_alloc_fault(after); });
}

int mocgpu_batch_step(mocgpu_batch *b, int *n_active)
{
    return guarded([&] {
        int n = eng(b).step();
        if (n_active) *n_active = n;
    });
}

int mocgpu_batch_launch(mocgpu_batch *b, int *n_active)
{
    return guarded([&] {
        int n = eng(b).launch();
        if (n_active) *n_active = n;
    });
}

int mocgpu_batch_finish(mocgpu_batch *b, int *n_active)
{
    return guarded([&] {
        int n = eng(b).finish();
        if (n_active) *n_active = n;
    });
}

int mocgpu_batch_set_pipeline_depth(mocgpu_batch *b, int depth)
{
    return guarded([&] { eng(b).set_pipeline_depth(depth); });
}
int mocgpu_batch_set_sweep_shape(mocgpu_batch *b, int shape)
{
    return guarded([&] { eng(b).set_sweep_shape(shape); });
}
int mocgpu_sweep_shape_info(int shape, int *rows, int *stages)
{
    return guarded([&] {
        REQUIRE(rows && stages, "null argument");
        static_assert(MOCGPU_SWEEP_SHAPES == mocgpu::kSweepShapeCount, "shape count");
        mocgpu::sweep_shape_info(shape, rows, stages);
    });
}
int mocgpu_batch_in_flight(mocgpu_batch *b, int *n)
{
    return guarded([&] {
        REQUIRE(n, "null argument");
        *n = eng(b).in_flight();
    });
}
int mocgpu_batch_poll(mocgpu_batch *b, int *done)
{
    return guarded([&] {
        REQUIRE(done, "null argument");
        *done = eng(b).poll() ? 1 : 0;
    });
}

int mocgpu_batch_run(mocgpu_batch *b)
{
    return guarded([&] { eng(b).run(); });
}

int mocgpu_batch_take(mocgpu_batch *b, int64_t id, int *ready, mocgpu_batch_result *res, double *pin_powers,
                        int n_pin_capacity)
{
    return guarded([&] {
        REQUIRE(ready && res, "null argument");
        auto &E = eng(b);
        mocgpu::BatchResult r;
        *ready = E.take_result(id, r) ? 1 : 0;
        if (!*ready) return;
        std::memset(res, 0, sizeof(*res));
        res->id = r.id;
        res->error = r.error;
        std::strncpy(res->message, r.message.c_str(), sizeof(res->message) - 1);
        res->k = r.k;
        res->iterations = r.iterations;
        res->converged = r.converged;
        res->error_k = r.error_k;
        res->error_psi = r.error_psi;
        res->cmfd_iterations = r.cmfd_iterations;
        res->t_submit = r.t_submit;
        res->t_admit = r.t_admit;
        res->t_done = r.t_done;
        res->n_pin = (int)r.pin_powers.size();
        if (pin_powers && res->n_pin) {
            REQUIRE(n_pin_capacity >= res->n_pin, "pin_powers buffer too small");
            std::memcpy(pin_powers, r.pin_powers.data(), sizeof(double) * r.pin_powers.size());
        }
    });
}

int mocgpu_batch_ready(mocgpu_batch *b, int64_t *ids, int capacity, int *n)
{
    return guarded([&] {
        REQUIRE(n && (ids || capacity == 0), "null argument");
        std::vector<int64_t> v = eng(b).ready_ids();
        *n = (int)v.size();
        for (int i = 0; i < (int)v.size() && i < capacity; i++) ids[i] = v[i];
    });
}

int mocgpu_batch_get_stats(mocgpu_batch *b, mocgpu_batch_stats *out)
{
    return guarded([&] {
        REQUIRE(out, "null argument");
        auto &E = eng(b);
        mocgpu::BatchStats s = E.stats();
        out->submitted = s.submitted;
        out->completed = s.completed;
        out->outer_iterations = s.outer_iterations;
        out->graph_replays = s.graph_replays;
        out->captures = s.captures;
        out->active = s.active;
        out->queued = s.queued;
        out->capacity = s.capacity;
        out->geometries = s.geometries;
        out->bundles_per_unit = s.bundles_per_unit;
        out->bytes_in_use = (double)s.bytes_in_use;
        out->bytes_budget = (double)s.bytes_budget;
        out->geometry_bytes = (double)s.geometry_bytes;
        out->now = E.now();
        out->replay_ms = s.replay_ms;
        out->sweep_ms = s.sweep_ms;
        out->sweep_launches = s.sweep_launches;
        out->sweep_bytes = s.sweep_bytes;
        out->sweep_sgu = s.sweep_sgu;
        out->trace_hits = s.trace_hits;
        out->trace_misses = s.trace_misses;
        out->trace_ms = s.trace_ms;
        out->xs_ms = s.xs_ms;
    });
}

int mocgpu_batch_set_timing(mocgpu_batch *b, int on)
{
    return guarded([&] { eng(b).set_timing(on != 0); });
}

int mocgpu_copy_bytes(int64_t *h2d, int64_t *d2h)
{
    return guarded([&] {
        REQUIRE(h2d && d2h, "null argument");
        mocgpu::copy_bytes(h2d, d2h);
    });
}

int mocgpu_batch_stream(mocgpu_batch *b, void **stream)
{
    return guarded([&] {
        REQUIRE(stream, "null argument");
        eng(b);
        *stream = (void *)b->stream;
    });
}

} // extern "C"
