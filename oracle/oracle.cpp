// CPU oracle (FP64, OpenMP): restatement of MOCC's 2-D MoC eigenvalue path.
// TEST INFRASTRUCTURE ONLY -- see oracle.h. Each routine names the MOCC
// source it follows. Arrays use MOCC's layouts: scalar flux [n_fsr][G],
// coarse data [n_surf][G] and [n_cell][G].
#include "oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.1415926535897932;
constexpr double FPI = 4.0 * PI;
enum { EAST = 0, NORTH = 1, WEST = 2, SOUTH = 3, TOP = 4, BOTTOM = 5, INVALID = 7 };
enum { X_NORM = 0, Y_NORM = 1, Z_NORM = 2 };
enum { VACUUM = 0, REFLECT = 1 };

thread_local std::string g_err;

// Exponential_Linear<10000> on [-10, 0] (exponential.hpp:56-112); outside
// the table the library exponential is used (without MOCC's stdout notice).
struct ExpTable {
    static constexpr int N = 10000;
    double min_ = -10.0, max_ = 0.0, space_, rspace_;
    std::vector<double> d_;
    ExpTable() : space_((max_ - min_) / (double)N), rspace_(1.0 / space_), d_(N + 1)
    {
        for (int i = 0; i <= N; i++) d_[i] = std::exp(min_ + i * space_);
    }
    double exp(double v) const
    {
        if (v < min_ || v > max_) return std::exp(v);
        int i = (int)((v - min_) * rspace_);
        if (i >= N) i = N - 1; // v == max_ exactly
        v -= space_ * i + min_;
        return d_[i] + (d_[i + 1] - d_[i]) * v * rspace_;
    }
};
const ExpTable &table()
{
    static ExpTable t;
    return t;
}

} // namespace

struct orc_solver {
    orc_problem p;
    orc_options o;
    int nthreads = 1;
    int G = 0, nreg = 0, ncell = 0, nsurf = 0, nsp = 0;
    // boundary layout
    std::vector<int> bc_off, ang_nx, ang_ny;
    int bcpg = 0;
    // sweeper state
    std::vector<double> flux, flux_old, fs, src, q, xstr_exp, bc_in, bc_out;
    std::vector<double> current, surface_flux; // [n_surf][G]
    bool coarse = false, has_radial = false;
    int max_seg = 0;
    // CMFD state ([n_cell][G])
    std::vector<double> cflux, hxstr, hxsnf, hxsf, hxsch, hxsrm, hscat;
    std::vector<double> d_tilde, d_hat, s_tilde, s_hat; // [n_surf][G]
    // CoarseData::partial_current and partial_current_old, [n_surf][G] pairs
    std::vector<std::array<double, 2>> partial, partial_old;
    bool has_old_partial = false;
    int n_cmfd_solve = 0;
    std::vector<double> mdiag, mW, mE, mS, mN;          // [G][n_cell]
    int64_t sweeps = 0, cmfd_its = 0;
    std::vector<double> history; // per outer iteration of eigen_solve: k, error_k, error_psi, seconds
    std::vector<double> split;   // MoCSweeper::split_ (with tl_splitting; zero until a leakage is applied)
    int n_fissile = 0;

    // ---- indexing helpers (mesh.hpp / mesh.cpp) ----
    int ndo() const { return p.ndir_oct; }
    int reverse(int iang) const { return (iang + ndo() * 2) % (ndo() * 4); }
    int reflect(int iang, int n) const
    {
        static const int t[3][8] = {{1, 0, 3, 2, 5, 4, 7, 6}, {3, 2, 1, 0, 7, 6, 5, 4}, {4, 5, 6, 7, 0, 1, 2, 3}};
        int oct = iang / ndo();
        return iang + (t[n][oct] - oct) * ndo();
    }
    int set_of(int iang) const
    {
        int a = (iang / ndo() >= 2) ? reverse(iang) : iang;
        return (a % ndo()) / p.pol_per_set + (a / ndo()) * (p.n_sets / 2);
    }
    int upwind(int iang, int n) const
    {
        if (n == X_NORM) return p.ang_ox[iang] > 0.0 ? WEST : EAST;
        return p.ang_oy[iang] > 0.0 ? SOUTH : NORTH;
    }
    int coarse_surf(int cell, int s) const
    {
        const int nx = p.nx, ny = p.ny;
        int ix = cell % nx, iy = cell / nx;
        int nxy = (nx + 1) * ny + (ny + 1) * nx;
        switch (s) {
        case EAST: return (nx + 1) * iy + ix + 1 + nx * ny;
        case WEST: return (nx + 1) * iy + ix + nx * ny;
        case NORTH: return nx * ny + (nx + 1) * ny + (ny + 1) * ix + iy + 1;
        case SOUTH: return (nx + 1) * ny + (ny + 1) * ix + iy + nx * ny;
        case BOTTOM: return nx * iy + ix;
        default: return nx * ny + nxy + nx * iy + ix;
        }
    }
    int coarse_neighbor(int cell, int s) const
    {
        int ix = cell % p.nx, iy = cell / p.nx;
        switch (s) {
        case NORTH: return iy < p.ny - 1 ? cell + p.nx : -1;
        case SOUTH: return iy > 0 ? cell - p.nx : -1;
        case EAST: return ix < p.nx - 1 ? cell + 1 : -1;
        case WEST: return ix > 0 ? cell - 1 : -1;
        case TOP:
        case BOTTOM: return -1;
        default: return -5;
        }
    }
    int surface_normal(int surf) const
    {
        int s = surf % nsp;
        if (s < p.nx * p.ny) return Z_NORM;
        if (s < p.nx * p.ny + (p.nx + 1) * p.ny) return X_NORM;
        return Y_NORM;
    }
    static int surface_to_normal(int s) { return (s == EAST || s == WEST) ? X_NORM : (s == NORTH || s == SOUTH) ? Y_NORM : Z_NORM; }
    void neigh_cells(int surf, int &c1, int &c2) const
    {
        const int nx = p.nx, ny = p.ny;
        int iz = surf / nsp, s = surf % nsp;
        int nrm = surface_normal(surf);
        if (nrm == X_NORM) {
            int t = s - nx * ny;
            int iy = t / (nx + 1), ix = t % (nx + 1);
            c1 = ix > 0 ? iy * nx + ix - 1 : -1;
            c2 = ix < nx ? iy * nx + ix : -1;
        } else if (nrm == Y_NORM) {
            int t = s - nx * ny - (nx + 1) * ny;
            int iy = t % (ny + 1), ix = t / (ny + 1);
            c1 = iy > 0 ? (iy - 1) * nx + ix : -1;
            c2 = iy < ny ? iy * nx + ix : -1;
        } else {
            c1 = iz > 0 ? s : -1;
            c2 = iz < 1 ? s : -1;
        }
    }
    double coarse_area_surf(int surf) const
    {
        int s = surf % nsp, nrm = surface_normal(surf);
        if (nrm == X_NORM) return p.dy[(s - p.nx * p.ny) / (p.nx + 1)] * p.hz;
        if (nrm == Y_NORM) return p.dx[(s - p.nx * p.ny - (p.nx + 1) * p.ny) / (p.ny + 1)] * p.hz;
        return p.dx[s % p.nx] * p.dy[s / p.nx];
    }
    double coarse_area(int cell, int s) const
    {
        int ix = cell % p.nx, iy = cell / p.nx;
        if (s == EAST || s == WEST) return p.dy[iy] * p.hz;
        if (s == NORTH || s == SOUTH) return p.dx[ix] * p.hz;
        return p.dx[ix] * p.dy[iy];
    }
    double cell_volume(int cell) const { return p.dx[cell % p.nx] * p.dy[cell / p.nx] * p.hz; }
    double xs(const double *a, int r, int g) const { return a[(size_t)p.fsr_mat[r] * G + g]; }
    double sc(int r, int to, int from) const { return p.scat[((size_t)p.fsr_mat[r] * G + to) * G + from]; }

    // ---- set-up ----
    void setup()
    {
        G = p.ng;
        nreg = p.n_fsr;
        ncell = p.n_pin;
        nsurf = p.n_surf;
        nsp = p.nx * p.ny + (p.nx + 1) * p.ny + (p.ny + 1) * p.nx;
        for (int s : {EAST, NORTH, WEST, SOUTH})
            if (p.bc[s] != VACUUM && p.bc[s] != REFLECT) throw std::runtime_error("unsupported radial boundary");
        const int nang = 4 * ndo();
        bc_off.resize(nang);
        ang_nx.resize(nang);
        ang_ny.resize(nang);
        int off = 0;
        for (int a = 0; a < nang; a++) {
            int s = set_of(a);
            bc_off[a] = off;
            ang_nx[a] = p.set_nx[s];
            ang_ny[a] = p.set_ny[s];
            off += p.set_nx[s] + p.set_ny[s];
        }
        bcpg = off;
        flux.assign((size_t)nreg * G, 0.0);
        flux_old = flux;
        fs.assign(nreg, 0.0);
        src.assign(nreg, 0.0);
        q.assign(nreg, 0.0);
        xstr_exp.assign(nreg, 0.0);
        if (o.tl_splitting) split.assign(nreg, 0.0);
        bc_in.assign((size_t)G * bcpg, 0.0);
        bc_out.assign(bcpg, 0.0);
        current.assign((size_t)nsurf * G, 0.0);
        surface_flux = current;
        for (int t = 0; t < p.n_tracks; t++)
            max_seg = std::max<int>(max_seg, (int)(p.trk_seg_begin[t + 1] - p.trk_seg_begin[t]));
        cflux.assign((size_t)ncell * G, 1.0);
        hxstr.assign((size_t)ncell * G, 0.0);
        hxsnf = hxsf = hxsch = hxsrm = hxstr;
        hscat.assign((size_t)ncell * G * G, 0.0);
        d_tilde.assign((size_t)nsurf * G, 0.0);
        d_hat = s_tilde = s_hat = d_tilde;
        partial.assign((size_t)nsurf * G, {0.0, 0.0});
        partial_old = partial;
        mdiag.assign((size_t)G * ncell, 0.0);
        mW = mE = mS = mN = mdiag;
        for (int r = 0; r < nreg; r++) {
            bool fis = false;
            for (int g = 0; g < G; g++)
                if (xs(p.xsnf, r, g) > 0.0) fis = true;
            if (fis) n_fissile++;
        }
    }

    // MoCSweeper::initialize (moc_sweeper.cpp:234-253) and
    // BoundaryCondition::initialize_scalar (boundary_condition.cpp:87-131)
    void initialize()
    {
        std::fill(flux.begin(), flux.end(), 1.0);
        std::fill(flux_old.begin(), flux_old.end(), 1.0);
        std::fill(cflux.begin(), cflux.end(), 1.0);
        std::fill(bc_in.begin(), bc_in.end(), 0.0);
        const double val = 1.0 / FPI;
        for (int g = 0; g < G; g++)
            for (int a = 0; a < 4 * ndo(); a++)
                for (int n = 0; n < 2; n++) {
                    int surf = upwind(a, n);
                    int lo = bc_off[a] + (n == 0 ? 0 : ang_ny[a]);
                    int cnt = (n == 0) ? ang_ny[a] : ang_nx[a];
                    if (p.bc[surf] == REFLECT)
                        for (int i = 0; i < cnt; i++) bc_in[(size_t)g * bcpg + lo + i] = val;
                }
        std::fill(current.begin(), current.end(), 0.0);
        std::fill(surface_flux.begin(), surface_flux.end(), 0.0);
        has_radial = false;
        sweeps = 0;
        cmfd_its = 0;
        std::fill(partial.begin(), partial.end(), std::array<double, 2>{0.0, 0.0});
        partial_old = partial;
        has_old_partial = false;
        n_cmfd_solve = 0;
    }

    // BoundaryCondition::update(group, angle, out) (boundary_condition.cpp:155-191)
    void bc_update(int group, int angle)
    {
        for (int n = 0; n < 2; n++) {
            int size = (n == 0) ? ang_ny[angle] : ang_nx[angle];
            int iin = reflect(angle, n);
            int off_in = group * bcpg + bc_off[iin] + (n == 0 ? 0 : ang_ny[iin]);
            int off_out = bc_off[angle] + (n == 0 ? 0 : ang_ny[angle]);
            int bt = p.bc[upwind(iin, n)];
            for (int i = 0; i < size; i++) bc_in[off_in + i] = (bt == VACUUM) ? 0.0 : bc_out[off_out + i];
        }
    }

    // Source::initialize_group + fission + in_scatter (source.cpp:41-112)
    void source_group(int g)
    {
        for (int r = 0; r < nreg; r++) {
            double s = 0.0;
            s += xs(p.xsch, r, g) * fs[r];
            for (int gg = 0; gg < G; gg++)
                if (gg != g) s += sc(r, g, gg) * flux[(size_t)r * G + gg];
            src[r] = s;
        }
    }
    // MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472)
    void apply_transverse_leakage(int g, const double *tl)
    {
        if (!split.empty()) {
            std::fill(split.begin(), split.end(), 0.0);
            for (int r = 0; r < nreg; r++) {
                double s = src[r] + tl[r];
                if (s < 0.0) {
                    const double f = flux[(size_t)r * G + g];
                    if (f < 0.0) throw std::runtime_error("Negative flux when splitting");
                    split[r] = -s / f;
                    src[r] = 0.0;
                } else {
                    src[r] = s;
                }
            }
        } else {
            for (int r = 0; r < nreg; r++) src[r] += tl[r];
        }
    }
    // SourceIsotropic::self_scatter (source_isotropic.cpp:21-57)
    void self_scatter(int g)
    {
        for (int r = 0; r < nreg; r++) {
            double rft = 1.0 / (xs(p.xstr, r, g) * FPI);
            q[r] = (src[r] + flux[(size_t)r * G + g] * sc(r, g, g)) * rft;
        }
    }

    // sweep1g (moc_sweeper_kernel.inc.hpp:36-180) with moc::Current
    // (moc_current_worker.hpp:182-318) when tally_currents is set.
    void sweep1g(int group, bool tally_currents)
    {
        const ExpTable &ex = table();
        for (int r = 0; r < nreg; r++) flux[(size_t)r * G + group] = 0.0;
        std::vector<double> t_all;
        double *in_g = &bc_in[(size_t)group * bcpg];
        const int nang_half = 2 * ndo();
#pragma omp parallel num_threads(nthreads)
        {
            std::vector<double> e_tau(max_seg), psi1(max_seg + 1), psi2(max_seg + 1), t_flux(nreg, 0.0);
            double cw[2], fw[2];
            for (int iang = 0; iang < nang_half; iang++) {
                const int iang1 = iang, iang2 = reverse(iang);
                const int set = set_of(iang);
                const double spacing = p.set_spacing[set];
                const double *bc_in_1 = in_g + bc_off[iang1];
                double *bc_out_1 = &bc_out[bc_off[iang1]];
                const double *bc_in_2 = in_g + bc_off[iang2];
                double *bc_out_2 = &bc_out[bc_off[iang2]];
                if (tally_currents) {
                    double w = p.ang_weight[iang] * PI;
                    double ca = std::fabs(std::cos(p.ang_alpha[iang])), sa = std::fabs(std::sin(p.ang_alpha[iang]));
                    cw[0] = w * p.ang_ox[iang] * spacing / ca * p.hz;
                    cw[1] = w * p.ang_oy[iang] * spacing / sa * p.hz;
                    fw[0] = w * spacing / ca * p.hz;
                    fw[1] = w * spacing / sa * p.hz;
                }
                const double stheta = std::sin(p.ang_theta[iang]);
                const double rstheta = p.ang_rsintheta[iang];
                const double wt_v_st = p.ang_weight[iang] * spacing * p.hz * stheta * PI;
                const int t0 = p.set_first_track[set], t1 = p.set_first_track[set + 1];
#pragma omp for schedule(static, 1)
                for (int t = t0; t < t1; t++) {
                    const int64_t b = p.trk_seg_begin[t];
                    const int n = (int)(p.trk_seg_begin[t + 1] - b);
                    const int bc1 = p.trk_bc0[t], bc2 = p.trk_bc1[t];
                    for (int s = 0; s < n; s++) {
                        int r = p.seg_fsr[b + s];
                        e_tau[s] = 1.0 - ex.exp(-xstr_exp[r] * p.seg_len[b + s] * rstheta);
                    }
                    psi1[0] = bc_in_1[bc1];
                    for (int s = 0; s < n; s++) {
                        int r = p.seg_fsr[b + s];
                        double d = (psi1[s] - q[r]) * e_tau[s];
                        psi1[s + 1] = psi1[s] - d;
                        t_flux[r] += d * wt_v_st;
                    }
                    bc_out_1[bc2] = psi1[n];
                    psi2[n] = bc_in_2[bc2];
                    for (int s = n - 1; s >= 0; s--) {
                        int r = p.seg_fsr[b + s];
                        double d = (psi2[s + 1] - q[r]) * e_tau[s];
                        psi2[s] = psi2[s + 1] - d;
                        t_flux[r] += d * wt_v_st;
                    }
                    bc_out_2[bc1] = psi2[0];
                    if (tally_currents) {
#pragma omp critical
                        post_ray(t, group, n, psi1.data(), psi2.data(), cw, fw);
                    }
                }
                if (o.gs_boundary) {
#pragma omp single
                    {
                        bc_update(group, iang1);
                        bc_update(group, iang2);
                    }
                }
            }
            if (!o.gs_boundary) {
#pragma omp single
                for (int a = 0; a < 4 * ndo(); a++) bc_update(group, a);
            }
#pragma omp barrier
#pragma omp critical
            {
                for (int r = 0; r < nreg; r++) flux[(size_t)r * G + group] += t_flux[r];
            }
#pragma omp barrier
#pragma omp single
            {
                for (int r = 0; r < nreg; r++) {
                    double &f = flux[(size_t)r * G + group];
                    f = f / (xstr_exp[r] * p.fsr_vol[r]) + q[r] * FPI;
                }
                if (tally_currents) {
                    // post_sweep: per-unit-area currents on x/y-normal surfaces
                    for (int s = p.nx * p.ny; s < nsp; s++) {
                        double a = coarse_area_surf(s);
                        current[(size_t)s * G + group] /= a;
                        surface_flux[(size_t)s * G + group] /= a;
                    }
                }
            }
        }
        sweeps++;
    }

    // moc::Current::post_ray (moc_current_worker.hpp:202-264)
    void post_ray(int t, int group, int n, const double *psi1, const double *psi2, const double *cw, const double *fw)
    {
        int cell_fw = p.trk_cm_cell_fw[t], cell_bw = p.trk_cm_cell_bw[t];
        int surf_fw = p.trk_cm_surf_fw[t], surf_bw = p.trk_cm_surf_bw[t];
        int iseg_fw = 0, iseg_bw = n;
        int norm_fw = surface_normal(surf_fw), norm_bw = surface_normal(surf_bw);
        current[(size_t)surf_fw * G + group] += psi1[iseg_fw] * cw[norm_fw];
        current[(size_t)surf_bw * G + group] -= psi2[iseg_bw] * cw[norm_bw];
        surface_flux[(size_t)surf_fw * G + group] += psi1[iseg_fw] * fw[norm_fw];
        surface_flux[(size_t)surf_bw * G + group] += psi2[iseg_bw] * fw[norm_bw];
        // A crossing recorded after the walk stepped out of the core (a track
        // leaving through a pin-cell corner on the core boundary,
        // ray.cpp:147-166) lies outside the core and is dropped; MOCC indexes
        // a surface from the out-of-core cell there, which is undefined.
        for (int c = p.trk_cm_begin[t]; c < p.trk_cm_begin[t + 1]; c++) {
            int fws = p.cm_fw[c], bws = p.cm_bw[c];
            if (fws != INVALID) iseg_fw += p.cm_nseg_fw[c];
            if (fws != INVALID && cell_fw >= 0) {
                norm_fw = surface_to_normal(fws);
                surf_fw = coarse_surf(cell_fw, fws);
                current[(size_t)surf_fw * G + group] += psi1[iseg_fw] * cw[norm_fw];
                surface_flux[(size_t)surf_fw * G + group] += psi1[iseg_fw] * fw[norm_fw];
            }
            if (bws != INVALID) iseg_bw -= p.cm_nseg_bw[c];
            if (bws != INVALID && cell_bw >= 0) {
                norm_bw = surface_to_normal(bws);
                surf_bw = coarse_surf(cell_bw, bws);
                current[(size_t)surf_bw * G + group] -= psi2[iseg_bw] * cw[norm_bw];
                surface_flux[(size_t)surf_bw * G + group] += psi2[iseg_bw] * fw[norm_bw];
            }
            if (cell_fw >= 0) cell_fw = coarse_neighbor(cell_fw, fws);
            if (cell_bw >= 0) cell_bw = coarse_neighbor(cell_bw, bws);
        }
    }

    // MoCSweeper::sweep (moc_sweeper.cpp:189-225)
    void sweep(int g)
    {
        // XSMesh::expand(group, split_) (xs_mesh.hpp:282-296)
        for (int r = 0; r < nreg; r++) xstr_exp[r] = xs(p.xstr, r, g) + (split.empty() ? 0.0 : split[r]);
        for (int inner = 0; inner < o.n_inner; inner++) {
            self_scatter(g);
            if (inner == o.n_inner - 1 && coarse) {
                for (int s = 0; s < nsurf; s++) {
                    current[(size_t)s * G + g] = 0.0;
                    surface_flux[(size_t)s * G + g] = 0.0;
                }
                sweep1g(g, true);
                has_radial = true;
            } else {
                sweep1g(g, false);
            }
        }
    }

    // TransportSweeper::calc_fission_source (transport_sweeper.cpp:119-134)
    void calc_fission_source(double k)
    {
        double rk = 1.0 / k;
        for (int r = 0; r < nreg; r++) {
            double f = 0.0;
            for (int g = 0; g < G; g++) f += rk * xs(p.xsnf, r, g) * flux[(size_t)r * G + g];
            fs[r] = f;
        }
    }
    // TransportSweeper::total_fission (transport_sweeper.cpp:104-117)
    double total_fission(bool old) const
    {
        const std::vector<double> &f = old ? flux_old : flux;
        double t = 0.0;
        for (int r = 0; r < nreg; r++)
            for (int g = 0; g < G; g++) t += f[(size_t)r * G + g] * p.fsr_vol[r] * xs(p.xsnf, r, g);
        return t;
    }

    // MoCSweeper::get_pin_flux_1g, PIN_PLANE (moc_sweeper.cpp:293-326)
    void get_pin_flux_1g(int g, double *out) const
    {
        for (int i = 0; i < ncell; i++) out[i] = 0.0;
        for (int ip = 0; ip < p.n_pin; ip++) {
            double v = 0.0, pf = 0.0;
            for (int r = p.pin_first_reg[ip]; r < p.pin_first_reg[ip + 1]; r++) {
                v += p.fsr_vol[r];
                pf += flux[(size_t)r * G + g] * p.fsr_vol[r];
            }
            out[p.pin_cell[ip]] += pf / v;
        }
    }
    // MoCSweeper::set_pin_flux_1g, PIN_PLANE (moc_sweeper.cpp:360-433)
    double set_pin_flux_1g(int g, const double *in)
    {
        for (int i = 0; i < ncell; i++)
            if (in[i] <= 0.0) throw std::runtime_error("Negative or zero input flux");
        double resid = 0.0;
        for (int ip = 0; ip < p.n_pin; ip++) {
            int c = p.pin_cell[ip];
            double fm = 0.0;
            for (int r = p.pin_first_reg[ip]; r < p.pin_first_reg[ip + 1]; r++)
                fm += flux[(size_t)r * G + g] * p.fsr_area[r];
            fm /= p.pin_area[ip];
            double e = in[c] - fm, f = in[c] / fm;
            for (int r = p.pin_first_reg[ip]; r < p.pin_first_reg[ip + 1]; r++) flux[(size_t)r * G + g] *= f;
            resid += e * e;
        }
        return std::sqrt(resid) / ncell;
    }

    // XSMeshHomogenized::homogenize_region_flux (xs_mesh_homogenized.cpp:261-363)
    void homogenize()
    {
        for (int ip = 0; ip < p.n_pin; ip++) {
            const int cell = p.pin_cell[ip];
            const int r0 = p.pin_first_reg[ip], r1 = p.pin_first_reg[ip + 1];
            std::vector<double> fsl(r1 - r0, 0.0);
            for (int g = 0; g < G; g++)
                for (int r = r0; r < r1; r++) fsl[r - r0] += xs(p.xsnf, r, g) * flux[(size_t)r * G + g] * p.fsr_area[r];
            double fs_sum = 0.0;
            for (double v : fsl) fs_sum += v;
            for (int g = 0; g < G; g++) {
                double fvs = 0.0, xt = 0.0, xnf = 0.0, xf = 0.0, xch = 0.0;
                std::vector<double> scatsum(G, 0.0), scg(G, 0.0);
                for (int r = r0; r < r1; r++) {
                    double v = p.fsr_area[r], fl = flux[(size_t)r * G + g];
                    fvs += v * fl;
                    xt += v * fl * xs(p.xstr, r, g);
                    xnf += v * fl * xs(p.xsnf, r, g);
                    xf += v * fl * xs(p.xsf, r, g);
                    xch += fsl[r - r0] * xs(p.xsch, r, g);
                    for (int gg = 0; gg < G; gg++) {
                        double fgg = flux[(size_t)r * G + gg];
                        scatsum[gg] += fgg * v;
                        scg[gg] += sc(r, g, gg) * v * fgg;
                    }
                }
                for (int gg = 0; gg < G; gg++) {
                    if (scg[gg] > 0.0) scg[gg] /= scatsum[gg];
                    hscat[((size_t)cell * G + g) * G + gg] = scg[gg];
                }
                hxstr[(size_t)cell * G + g] = xt / fvs;
                hxsnf[(size_t)cell * G + g] = xnf / fvs;
                hxsf[(size_t)cell * G + g] = xf / fvs;
                hxsch[(size_t)cell * G + g] = (fs_sum > 0.0) ? xch / fs_sum : xch;
            }
            for (int g = 0; g < G; g++)
                hxsrm[(size_t)cell * G + g] = hxstr[(size_t)cell * G + g] - hscat[((size_t)cell * G + g) * G + g];
        }
    }

    // ---- CMFD (cmfd.cpp) ----
    // CMFD::setup_solve (cmfd.cpp:333-553)
    void cmfd_setup()
    {
        for (int g = 0; g < G; g++) {
            for (int is = 0; is < nsurf; is++) {
                int c1, c2;
                neigh_cells(is, c1, c2);
                int nrm = surface_normal(is);
                auto thick = [&](int cell) {
                    if (nrm == X_NORM) return p.dx[cell % p.nx];
                    if (nrm == Y_NORM) return p.dy[cell / p.nx];
                    return p.hz;
                };
                int lo = nrm == X_NORM ? WEST : nrm == Y_NORM ? SOUTH : BOTTOM;
                int hi = nrm == X_NORM ? EAST : nrm == Y_NORM ? NORTH : TOP;
                double d1, d2;
                if (c1 > -1) d1 = (1.0 / (3.0 * hxstr[(size_t)c1 * G + g])) / thick(c1);
                else if (p.bc[lo] == REFLECT) d1 = 0.0 / 2.0;
                else if (p.bc[lo] == VACUUM) d1 = 0.5 / 2.0;
                else throw std::runtime_error("Unsupported boundary type");
                if (c2 > -1) d2 = (1.0 / (3.0 * hxstr[(size_t)c2 * G + g])) / thick(c2);
                else if (p.bc[hi] == REFLECT) d2 = 0.0 / 2.0;
                else if (p.bc[hi] == VACUUM) d2 = 0.5 / 2.0;
                else throw std::runtime_error("Unsupported boundary type");
                double dt = 2.0 * d1 * d2 / (d1 + d2);
                double st = (d1 > 0.0) ? d1 / (d1 + d2) : d2 / (d1 + d2);
                d_tilde[(size_t)is * G + g] = dt;
                s_tilde[(size_t)is * G + g] = st;
                bool have = (nrm == Z_NORM) ? false : has_radial;
                double dh = 0.0, sh = 0.0;
                if (have) {
                    double j = current[(size_t)is * G + g];
                    double sfc = surface_flux[(size_t)is * G + g];
                    double fl = c1 >= 0 ? cflux[(size_t)c1 * G + g] : 0.0;
                    double fr = c2 >= 0 ? cflux[(size_t)c2 * G + g] : 0.0;
                    dh = (j + dt * (fr - fl)) / (fl + fr);
                    if (!std::isfinite(dh)) dh = 0.0;
                    sh = (c1 >= 0) ? (sfc - st * fl - (1.0 - st) * fr) / (fl + fr) : (sfc - st * fr) / fr;
                }
                d_hat[(size_t)is * G + g] = dh;
                s_hat[(size_t)is * G + g] = sh;
            }
            for (int i = 0; i < ncell; i++) {
                double v = cell_volume(i) * hxsrm[(size_t)i * G + g];
                for (int s : {EAST, NORTH, WEST, SOUTH, TOP, BOTTOM}) {
                    int surf = coarse_surf(i, s);
                    double a = coarse_area(i, s);
                    double dh = d_hat[(size_t)surf * G + g];
                    if (s == WEST || s == SOUTH || s == BOTTOM) dh = -dh;
                    v += a * (d_tilde[(size_t)surf * G + g] + dh);
                }
                mdiag[(size_t)g * ncell + i] = v;
                auto off = [&](int s) {
                    if (coarse_neighbor(i, s) < 0) return 0.0;
                    int surf = coarse_surf(i, s);
                    double a = coarse_area(i, s);
                    double dh = d_hat[(size_t)surf * G + g];
                    if (s == WEST || s == SOUTH || s == BOTTOM) dh = -dh;
                    return a * (dh - d_tilde[(size_t)surf * G + g]);
                };
                mW[(size_t)g * ncell + i] = off(WEST);
                mE[(size_t)g * ncell + i] = off(EAST);
                mS[(size_t)g * ncell + i] = off(SOUTH);
                mN[(size_t)g * ncell + i] = off(NORTH);
            }
        }
    }
    void spmv(int g, const double *x, double *y) const
    {
        const int n = ncell, nx = p.nx;
        const double *d = &mdiag[(size_t)g * n], *w = &mW[(size_t)g * n], *e = &mE[(size_t)g * n],
                     *s = &mS[(size_t)g * n], *no = &mN[(size_t)g * n];
        for (int i = 0; i < n; i++) {
            double v = d[i] * x[i];
            int ix = i % nx;
            if (ix > 0) v += w[i] * x[i - 1];
            if (ix < nx - 1) v += e[i] * x[i + 1];
            if (i >= nx) v += s[i] * x[i - nx];
            if (i + nx < n) v += no[i] * x[i + nx];
            y[i] = v;
        }
    }
    // Preconditioned BiCGSTAB with a diagonal preconditioner: MOCC calls
    // Eigen::BiCGSTAB (default DiagonalPreconditioner) with a relative
    // tolerance and 150 iterations (cmfd.cpp:202-204, 546-547, 291). Eigen is
    // an unvendored submodule of unknown revision; this is the published
    // algorithm (van der Vorst 1992) with Eigen's stopping test
    // ||r||^2 <= tol^2 ||b||^2 and a shadow-residual restart.
    int bicgstab(int g, const std::vector<double> &b, double *x, double tol, int max_it) const
    {
        const int n = ncell;
        std::vector<double> r(n), r0(n), pv(n, 0.0), v(n, 0.0), y(n), z(n), s(n), t(n), dinv(n);
        // diagonal preconditioner: multiply by the stored inverse diagonal
        for (int i = 0; i < n; i++) {
            double dd = mdiag[(size_t)g * n + i];
            dinv[i] = (dd != 0.0) ? 1.0 / dd : 1.0;
        }
        spmv(g, x, r.data());
        double rr = 0.0, bb = 0.0;
        for (int i = 0; i < n; i++) {
            r[i] = b[i] - r[i];
            r0[i] = r[i];
            rr += r[i] * r[i];
            bb += b[i] * b[i];
        }
        if (bb == 0.0) {
            for (int i = 0; i < n; i++) x[i] = 0.0;
            return 0;
        }
        double r0_sq = rr, rho = 1.0, alpha = 1.0, w = 1.0;
        const double tol2 = tol * tol * bb, eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
        int it = 0, restarts = 0;
        while (rr > tol2 && it < max_it) {
            double rho_old = rho;
            rho = 0.0;
            for (int i = 0; i < n; i++) rho += r0[i] * r[i];
            if (std::fabs(rho) < eps2 * r0_sq) {
                spmv(g, x, r.data());
                double acc = 0.0;
                for (int i = 0; i < n; i++) {
                    r[i] = b[i] - r[i];
                    r0[i] = r[i];
                    acc += r[i] * r[i];
                }
                rho = r0_sq = acc;
                if (restarts++ == 0) it = 0;
            }
            double beta = (rho / rho_old) * (alpha / w);
            for (int i = 0; i < n; i++) {
                pv[i] = r[i] + beta * (pv[i] - w * v[i]);
                y[i] = pv[i] * dinv[i];
            }
            spmv(g, y.data(), v.data());
            double r0v = 0.0;
            for (int i = 0; i < n; i++) r0v += r0[i] * v[i];
            alpha = rho / r0v;
            for (int i = 0; i < n; i++) {
                s[i] = r[i] - alpha * v[i];
                z[i] = s[i] * dinv[i];
            }
            spmv(g, z.data(), t.data());
            double tt = 0.0, ts = 0.0;
            for (int i = 0; i < n; i++) {
                tt += t[i] * t[i];
                ts += t[i] * s[i];
            }
            w = (tt > 0.0) ? ts / tt : 0.0;
            rr = 0.0;
            for (int i = 0; i < n; i++) {
                x[i] += alpha * y[i] + w * z[i];
                r[i] = s[i] - w * t[i];
                rr += r[i] * r[i];
            }
            it++;
        }
        return it;
    }
    void cmfd_source(int g, const std::vector<double> &cfs, std::vector<double> &b) const
    {
        for (int i = 0; i < ncell; i++) {
            double s = hxsch[(size_t)i * G + g] * cfs[i];
            for (int gg = 0; gg < G; gg++)
                if (gg != g) s += hscat[((size_t)i * G + g) * G + gg] * cflux[(size_t)i * G + gg];
            b[i] = s * cell_volume(i);
        }
    }
    double cmfd_residual_g(int g, const std::vector<double> &b) const
    {
        std::vector<double> x(ncell), y(ncell);
        for (int i = 0; i < ncell; i++) x[i] = cflux[(size_t)i * G + g];
        spmv(g, x.data(), y.data());
        double r = 0.0;
        for (int i = 0; i < ncell; i++) r += (y[i] - b[i]) * (y[i] - b[i]);
        return r;
    }
    void cmfd_fission_source(double k, std::vector<double> &cfs) const
    {
        for (int i = 0; i < ncell; i++) {
            double f = 0.0;
            for (int g = 0; g < G; g++) f += hxsnf[(size_t)i * G + g] * cflux[(size_t)i * G + g];
            cfs[i] = f * (1.0 / k);
        }
    }
    double cmfd_total_fission() const
    {
        double f = 0.0;
        for (int i = 0; i < ncell; i++)
            for (int g = 0; g < G; g++) f += hxsnf[(size_t)i * G + g] * cflux[(size_t)i * G + g];
        return f;
    }
    // CMFD::solve (cmfd.cpp:171-279)
    void cmfd_solve(double &k)
    {
        if (o.cmfd_negative_fixup)
            for (double &v : cflux) v = std::max(v, 0.0);
        homogenize();
        cmfd_setup();
        std::vector<double> cfs(ncell), cfs_old(ncell), b(ncell), x(ncell);
        cmfd_fission_source(k, cfs);
        double tfis = cmfd_total_fission();
        double r0 = 0.0;
        for (int g = 0; g < G; g++) {
            cmfd_source(g, cfs, b);
            r0 += cmfd_residual_g(g, b);
        }
        r0 = std::sqrt(r0) / (ncell * G);
        const double tol = o.cmfd_resid_reduction * r0;
        int iter = 0;
        while (true) {
            iter++;
            cfs_old = cfs;
            cmfd_fission_source(k, cfs);
            double tfis_old = tfis;
            double ri = 0.0;
            for (int g = 0; g < G; g++) {
                cmfd_source(g, cfs, b);
                ri += cmfd_residual_g(g, b);
                for (int i = 0; i < ncell; i++) x[i] = cflux[(size_t)i * G + g];
                bicgstab(g, b, x.data(), tol, 150);
                for (int i = 0; i < ncell; i++) cflux[(size_t)i * G + g] = x[i];
            }
            ri = std::sqrt(ri) / (ncell * G);
            tfis = cmfd_total_fission();
            double k_old = k;
            k = k * tfis / tfis_old;
            double pe = 0.0;
            for (int i = 0; i < ncell; i++) pe += (cfs[i] - cfs_old[i]) * (cfs[i] - cfs_old[i]);
            pe = std::sqrt(pe);
            if ((std::fabs(k - k_old) < o.cmfd_k_tol && pe < o.cmfd_psi_tol && ri / r0 < o.cmfd_resid_reduction) ||
                iter > o.cmfd_max_iter)
                break;
        }
        for (double &v : cflux)
            if (v < 0.0) v = -v;
        if (o.incoming_update) store_currents();
        n_cmfd_solve++;
        cmfd_its += iter;
    }
    // CMFD::store_currents (cmfd.cpp:555-638), the partial currents only
    // (the net currents it also writes back are not read again in 2-D)
    void store_currents()
    {
        for (int g = 0; g < G; g++) {
            for (int is = 0; is < nsurf; is++) partial_old[(size_t)is * G + g] = partial[(size_t)is * G + g];
            has_old_partial = n_cmfd_solve > 0;
            for (int is = 0; is < nsurf; is++) {
                int c1, c2;
                neigh_cells(is, c1, c2);
                double fr = c2 >= 0 ? cflux[(size_t)c2 * G + g] : 0.0;
                double fl = c1 >= 0 ? cflux[(size_t)c1 * G + g] : 0.0;
                double dh = d_hat[(size_t)is * G + g], dt = d_tilde[(size_t)is * G + g];
                double cur = -dt * (fr - fl) + dh * (fr + fl);
                double sh = s_hat[(size_t)is * G + g], st = s_tilde[(size_t)is * G + g];
                double sf = (c1 >= 0) ? st * fl + (1.0 - st) * fr + sh * (fl + fr) : st * fr + sh * (fl + fr);
                partial[(size_t)is * G + g] = {0.25 * sf + 0.5 * cur, 0.25 * sf - 0.5 * cur};
            }
        }
    }
    // MoCSweeper::update_incoming_flux (moc_sweeper.cpp:255-291) through
    // update_incoming_generic (moc_sweeper.hpp:198-233). Mode 1 keeps MOCC's
    // lookup, which passes the ray's starting coarse cell (cm_cell_fw/bw)
    // where partial_current takes a surface index, so it reads the cell's
    // bottom z-face. Mode 2 reads the surface the ray enters through
    // (cm_surf_fw/bw) and leaves vacuum faces at zero.
    void update_incoming_flux()
    {
        auto f = [&](double in, int is, int g) {
            const auto &pc = partial[(size_t)is * G + g];
            if (has_old_partial) {
                const auto &po = partial_old[(size_t)is * G + g];
                double part = 2.0 * (pc[0] + pc[1]);
                double part_old = 2.0 * (po[0] + po[1]);
                if (part_old > 0.0) {
                    double r = part / part_old;
                    return in * r;
                }
                return in;
            }
            return 2.0 * (1.0 / FPI) * (pc[0] + pc[1]);
        };
        auto surface = [&](int cell, int surf) {
            if (o.incoming_update == 1) return cell;
            int c1, c2;
            neigh_cells(surf, c1, c2);
            int nrm = surface_normal(surf);
            int face = nrm == X_NORM ? (c1 < 0 ? WEST : EAST) : (c1 < 0 ? SOUTH : NORTH);
            return p.bc[face] == VACUUM ? -1 : surf;
        };
        for (int g = 0; g < G; g++) {
            for (int iang = 0; iang < 2 * ndo(); iang++) {
                int iang1 = iang, iang2 = reverse(iang);
                double *bc_fw = &bc_in[(size_t)g * bcpg + bc_off[iang1]];
                double *bc_bw = &bc_in[(size_t)g * bcpg + bc_off[iang2]];
                int set = set_of(iang);
                for (int t = p.set_first_track[set]; t < p.set_first_track[set + 1]; t++) {
                    int is1 = surface(p.trk_cm_cell_fw[t], p.trk_cm_surf_fw[t]);
                    int is2 = surface(p.trk_cm_cell_bw[t], p.trk_cm_surf_bw[t]);
                    int bc1 = p.trk_bc0[t], bc2 = p.trk_bc1[t];
                    if (is1 >= 0) bc_fw[bc1] = f(bc_fw[bc1], is1, g);
                    if (is2 >= 0) bc_bw[bc2] = f(bc_bw[bc2], is2, g);
                }
            }
        }
    }
    // EigenSolver::do_cmfd (eigen_solver.cpp:263-291)
    void do_cmfd(double &k)
    {
        std::vector<double> pf(ncell);
        for (int g = 0; g < G; g++) {
            get_pin_flux_1g(g, pf.data());
            for (int i = 0; i < ncell; i++) cflux[(size_t)i * G + g] = pf[i];
        }
        cmfd_solve(k);
        for (int g = 0; g < G; g++) {
            for (int i = 0; i < ncell; i++) pf[i] = cflux[(size_t)i * G + g];
            set_pin_flux_1g(g, pf.data());
        }
        // the call MOCC leaves commented out, when the options ask for it
        if (o.incoming_update) update_incoming_flux();
    }
    // Normalize() (util/utils.hpp:29-51)
    static void normalize(std::vector<double> &v)
    {
        int n = 0;
        double sum = 0.0;
        for (double x : v) {
            if (x > 0.0) n++;
            sum += x;
        }
        double f = (double)n / sum;
        for (double &x : v) x *= f;
    }
    // EigenSolver::solve / step (eigen_solver.cpp:131-253)
    orc_result eigen_solve(int max_outer)
    {
        auto t0 = std::chrono::steady_clock::now();
        orc_result res{};
        coarse = o.cmfd && o.cmfd_enabled;
        initialize();
        history.clear();
        double k = 1.0, k_prev = 1.0;
        calc_fission_source(k);
        int max_it = max_outer >= 0 ? max_outer : o.max_iter;
        std::vector<double> fs_prev;
        for (int it = 0; it < max_it; it++) {
            if (o.cmfd && o.cmfd_enabled) do_cmfd(k);
            calc_fission_source(k);
            fs_prev = fs;
            flux_old = flux;
            for (int g = 0; g < G; g++) {
                source_group(g);
                sweep(g);
            }
            double t1 = total_fission(false), t2 = total_fission(true);
            k_prev = k;
            k = k * t1 / t2;
            calc_fission_source(k);
            res.error_k = std::fabs(k - k_prev);
            std::vector<double> a = fs, b = fs_prev;
            normalize(a);
            normalize(b);
            double e = 0.0;
            for (int r = 0; r < nreg; r++) e += (a[r] - b[r]) * (a[r] - b[r]);
            res.error_psi = std::sqrt(e / n_fissile);
            res.iterations = it + 1;
            // EigenSolver::solve's convergence_ and iteration_times_
            // (eigen_solver.cpp:185-190), the time since the solve began
            history.insert(history.end(), {k, res.error_k, res.error_psi,
                                           std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count()});
            if (k != k) throw std::runtime_error("Eigenvalue is not a number. Giving up.");
            if (res.error_k < o.k_tol && res.error_psi < o.psi_tol && it >= o.min_iter) {
                res.converged = 1;
                break;
            }
        }
        res.k = k;
        res.sweeps = sweeps;
        res.cmfd_iterations = cmfd_its;
        res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return res;
    }
};

namespace {
template <typename F> int guard(F &&f)
{
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 1;
    }
}
} // namespace

extern "C" {
const char *orc_last_error(void) { return g_err.c_str(); }

int orc_create(const orc_problem *p, const orc_options *o, int n_threads, orc_solver **out)
{
    return guard([&] {
        auto *s = new orc_solver();
        s->p = *p;
        s->o = *o;
#ifdef _OPENMP
        s->nthreads = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
        s->nthreads = 1;
        (void)n_threads;
#endif
        try {
            s->setup();
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}
void orc_destroy(orc_solver *s) { delete s; }
int orc_threads(orc_solver *s) { return s->nthreads; }
int orc_initialize(orc_solver *s)
{
    return guard([&] { s->initialize(); });
}
int orc_set_coarse_data(orc_solver *s, int enabled)
{
    return guard([&] { s->coarse = enabled != 0; });
}
int orc_calc_fission_source(orc_solver *s, double k, double *fs)
{
    return guard([&] {
        s->calc_fission_source(k);
        if (fs) std::memcpy(fs, s->fs.data(), sizeof(double) * s->nreg);
    });
}
int orc_set_fission_source(orc_solver *s, const double *fs)
{
    return guard([&] { std::memcpy(s->fs.data(), fs, sizeof(double) * s->nreg); });
}
int orc_store_old_flux(orc_solver *s)
{
    return guard([&] { s->flux_old = s->flux; });
}
int orc_source_group(orc_solver *s, int g)
{
    return guard([&] { s->source_group(g); });
}
int orc_sweep_group(orc_solver *s, int g)
{
    return guard([&] { s->sweep(g); });
}
int orc_total_fission(orc_solver *s, int old, double *out)
{
    return guard([&] { *out = s->total_fission(old != 0); });
}
int orc_flux_residual(orc_solver *s, double *out)
{
    return guard([&] {
        double r = 0.0;
        for (size_t i = 0; i < s->flux.size(); i++) r += (s->flux[i] - s->flux_old[i]) * (s->flux[i] - s->flux_old[i]);
        *out = std::sqrt(r);
    });
}
int orc_get_flux(orc_solver *s, double *flux)
{
    return guard([&] { std::memcpy(flux, s->flux.data(), sizeof(double) * s->flux.size()); });
}
int orc_set_flux(orc_solver *s, const double *flux)
{
    return guard([&] { std::memcpy(s->flux.data(), flux, sizeof(double) * s->flux.size()); });
}
int orc_get_pin_flux_1g(orc_solver *s, int g, double *out)
{
    return guard([&] { s->get_pin_flux_1g(g, out); });
}
int orc_set_pin_flux_1g(orc_solver *s, int g, const double *in, double *resid)
{
    return guard([&] {
        double r = s->set_pin_flux_1g(g, in);
        if (resid) *resid = r;
    });
}
int orc_pin_powers(orc_solver *s, double *out)
{
    return guard([&] {
        const int G = s->G;
        std::vector<double> pw(s->ncell, 0.0);
        double tot = 0.0;
        for (int ip = 0; ip < s->p.n_pin; ip++)
            for (int r = s->p.pin_first_reg[ip]; r < s->p.pin_first_reg[ip + 1]; r++) {
                double f = 0.0;
                for (int g = 0; g < G; g++) f += s->flux[(size_t)r * G + g] * s->xs(s->p.xsf, r, g) * s->p.fsr_vol[r];
                tot += f;
                pw[s->p.pin_cell[ip]] += f;
            }
        double sc = s->p.n_fuel_2d / tot;
        for (int i = 0; i < s->ncell; i++) out[i] = pw[i] * sc;
    });
}
int orc_get_coarse_currents(orc_solver *s, double *cur, double *sflux)
{
    return guard([&] {
        // [n_surf][G] -> [G][n_surf] to match the GPU library's export
        for (int is = 0; is < s->nsurf; is++)
            for (int g = 0; g < s->G; g++) {
                cur[(size_t)g * s->nsurf + is] = s->current[(size_t)is * s->G + g];
                sflux[(size_t)g * s->nsurf + is] = s->surface_flux[(size_t)is * s->G + g];
            }
    });
}
int orc_get_boundary(orc_solver *s, int g, double *out, int64_t *n)
{
    return guard([&] {
        if (g < 0 || g >= s->G) throw std::runtime_error("bad group");
        *n = s->bcpg;
        if (out) std::copy(s->bc_in.begin() + (size_t)g * s->bcpg, s->bc_in.begin() + (size_t)(g + 1) * s->bcpg, out);
    });
}
int orc_update_incoming(orc_solver *s, const double *part, const double *part_old, int has_old, int mode)
{
    return guard([&] {
        if (mode != 1 && mode != 2) throw std::runtime_error("bad mode");
        for (int g = 0; g < s->G; g++)
            for (int is = 0; is < s->nsurf; is++) {
                // a pair whose 2 (J+ + J-) is the given sum exactly
                s->partial[(size_t)is * s->G + g] = {0.5 * part[(size_t)g * s->nsurf + is], 0.0};
                if (has_old) s->partial_old[(size_t)is * s->G + g] = {0.5 * part_old[(size_t)g * s->nsurf + is], 0.0};
            }
        s->has_old_partial = has_old != 0;
        const int keep = s->o.incoming_update;
        s->o.incoming_update = mode;
        s->update_incoming_flux();
        s->o.incoming_update = keep;
    });
}
int orc_homogenized_nu_fission(orc_solver *s, double *out)
{
    return guard([&] {
        // pin-homogenised nu-Sigma_f of the current flux, [n_pin in FSR order][G]
        s->homogenize();
        for (int ip = 0; ip < s->p.n_pin; ip++)
            for (int g = 0; g < s->G; g++)
                out[(size_t)ip * s->G + g] = s->hxsnf[(size_t)s->p.pin_cell[ip] * s->G + g];
    });
}
int orc_cmfd_system(orc_solver *s, double *op, double *xsnf, double *xsch, double *scat, double *vol)
{
    return guard([&] {
        // the CMFD system CMFD::solve would iterate on from the current state
        // (EigenSolver::do_cmfd's coarse flux, homogenisation, setup_solve)
        const int n = s->ncell, G = s->G;
        std::vector<double> pf(n);
        for (int g = 0; g < G; g++) {
            s->get_pin_flux_1g(g, pf.data());
            for (int i = 0; i < n; i++) s->cflux[(size_t)i * G + g] = pf[i];
        }
        if (s->o.cmfd_negative_fixup)
            for (double &v : s->cflux) v = std::max(v, 0.0);
        s->homogenize();
        s->cmfd_setup();
        const std::vector<double> *rows[5] = {&s->mdiag, &s->mW, &s->mE, &s->mS, &s->mN};
        for (int g = 0; g < G; g++)
            for (int q = 0; q < 5; q++)
                for (int i = 0; i < n; i++) op[((size_t)g * 5 + q) * n + i] = (*rows[q])[(size_t)g * n + i];
        std::copy(s->hxsnf.begin(), s->hxsnf.end(), xsnf);
        std::copy(s->hxsch.begin(), s->hxsch.end(), xsch);
        std::copy(s->hscat.begin(), s->hscat.end(), scat);
        for (int i = 0; i < n; i++) vol[i] = s->cell_volume(i);
    });
}
int orc_cmfd_solve(orc_solver *s, double *k)
{
    return guard([&] { s->do_cmfd(*k); });
}
int orc_eigen_solve(orc_solver *s, int max_outer, orc_result *out)
{
    return guard([&] { *out = s->eigen_solve(max_outer); });
}
int orc_apply_transverse_leakage(orc_solver *s, int g, const double *tl)
{
    return guard([&] { s->apply_transverse_leakage(g, tl); });
}
int orc_history(orc_solver *s, const double **data, int64_t *n)
{
    *data = s->history.data();
    *n = (int64_t)s->history.size() / 4;
    return 0;
}
double orc_table_exp(double x) { return table().exp(x); }
}
