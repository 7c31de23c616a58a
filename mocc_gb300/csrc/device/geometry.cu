#include "geometry.hpp"

#include <algorithm>
#include <cmath>

namespace mocgpu {

namespace {
constexpr double kPiD = 3.1415926535897932;

// Row windows of the bundled sweep: rows per window, and the FSRs of a whole
// unit above which the unit is staged a window at a time (build-time knobs).
// Measured on the 68x68 mini-core (one group sweep, 2 bundles per unit):
// whole units 618 us (3 CTAs per SM), windows of 128 rows 589 us (5 CTAs),
// 64 rows 635 us and 32 rows 674 us: the restaging and the per-window tally
// flushes grow as the windows shrink and eat the occupancy they buy.
#ifndef MOCGPU_WINDOW_ROWS
#define MOCGPU_WINDOW_ROWS 128
#endif
#ifndef MOCGPU_WINDOW_MIN_FSRS
#define MOCGPU_WINDOW_MIN_FSRS 1024
#endif

int reflect_angle(int iang, int normal, int ndir_oct)
{
    static const int table[3][8] = {{1, 0, 3, 2, 5, 4, 7, 6}, {3, 2, 1, 0, 7, 6, 5, 4}, {4, 5, 6, 7, 0, 1, 2, 3}};
    int oct = iang / ndir_oct;
    return iang + (table[normal][oct] - oct) * ndir_oct;
}
int reverse_angle(int iang, int ndir_oct) { return (iang + ndir_oct * 2) % (ndir_oct * 4); }
Surface upwind(double ox, double oy, int normal)
{
    if (normal == X_NORM) return ox > 0.0 ? WEST : EAST;
    return oy > 0.0 ? SOUTH : NORTH;
}
} // namespace

DeviceGeometry::DeviceGeometry(const FlatProblem &f, int prec, int bundles_per_unit, int window_rows) : precision(prec)
{
    for (int s : {EAST, NORTH, WEST, SOUTH})
        if (f.bc[s] != (int)BoundaryType::VACUUM && f.bc[s] != (int)BoundaryType::REFLECT)
            MOCGPU_THROW(5, "radial boundaries must be vacuum or reflect for the eigenvalue path");
    if (f.pol_per_set > kMaxPolar) MOCGPU_THROW(1, "too many polar angles per track set");
    G = f.ng;
    n_fsr = f.n_fsr;
    n_pin = f.n_pin;
    n_surf = f.n_surf;
    n_tracks = f.n_tracks;
    n_sets = f.n_sets;
    pol = f.pol_per_set;
    n_ang = f.n_ang;
    ndir_oct = f.ndir_oct;
    nx = f.nx;
    ny = f.ny;
    n_seg = f.n_seg;
    hz = f.hz;
    for (int i = 0; i < 6; i++) bc[i] = f.bc[i];
    set_nx = f.set_nx;
    set_ny = f.set_ny;

    // --- angle -> track set, boundary offsets (boundary_condition.cpp:33-78) --
    const int nd = f.ndir_oct, sets_oct = f.n_sets / 2;
    auto set_of = [&](int iang) {
        int a = (iang / nd >= 2) ? reverse_angle(iang, nd) : iang;
        return (a % nd) / f.pol_per_set + (a / nd) * sets_oct;
    };
    std::vector<int> bc_off(n_ang), ang_ny(n_ang);
    int off = 0;
    for (int a = 0; a < n_ang; a++) {
        int s = set_of(a);
        bc_off[a] = off;
        ang_ny[a] = f.set_ny[s];
        off += f.set_nx[s] + f.set_ny[s];
    }
    bc_per_group = off;
    // Write-through targets of outgoing flux (the reflected angle's incoming
    // slot, or -1 on vacuum faces) and the initial incoming flux
    // (boundary_condition.cpp:87-191).
    std::vector<int> wt(5 * n_ang, -1);
    psi_init.assign(bc_per_group, 0.0);
    for (int a = 0; a < n_ang; a++) {
        int s = set_of(a);
        for (int n = 0; n < 2; n++) {
            int tgt = reflect_angle(a, n, nd);
            Surface up = upwind(f.ang_ox[tgt], f.ang_oy[tgt], n);
            wt[a * 2 + n] = (f.bc[up] == (int)BoundaryType::REFLECT) ? bc_off[tgt] : -1;
            wt[3 * n_ang + a * 2 + n] = bc_off[tgt];
            Surface own = upwind(f.ang_ox[a], f.ang_oy[a], n);
            int lo = bc_off[a] + (n == 0 ? 0 : f.set_ny[s]);
            int cnt = (n == 0) ? f.set_ny[s] : f.set_nx[s];
            double v = (f.bc[own] == (int)BoundaryType::REFLECT) ? 1.0 / (4.0 * kPiD) : 0.0;
            for (int i = 0; i < cnt; i++) psi_init[lo + i] = v;
        }
        wt[2 * n_ang + a] = ang_ny[a];
    }

    // --- per (set, polar) sweep constants (moc_sweeper_kernel.inc.hpp:76-82,
    //     moc_current_worker.hpp:182-200) -------------------------------------
    std::vector<SetPolar> sp(f.n_sets * f.pol_per_set);
    for (int s = 0; s < f.n_sets; s++)
        for (int p = 0; p < f.pol_per_set; p++) {
            int iang = (s / sets_oct) * nd + (s % sets_oct) * f.pol_per_set + p;
            SetPolar &x = sp[s * f.pol_per_set + p];
            x.ang_fwd = iang;
            x.ang_bwd = reverse_angle(iang, nd);
            double spc = f.set_spacing[s];
            x.rsin = f.ang_rsintheta[iang];
            x.wt = f.ang_weight[iang] * spc * f.hz * std::sin(f.ang_theta[iang]) * kPiD;
            double w = f.ang_weight[iang] * kPiD;
            double ca = std::fabs(std::cos(f.ang_alpha[iang])), sa = std::fabs(std::sin(f.ang_alpha[iang]));
            x.cw[0] = w * f.ang_ox[iang] * spc / ca * f.hz;
            x.cw[1] = w * f.ang_oy[iang] * spc / sa * f.hz;
            x.fw[0] = w * spc / ca * f.hz;
            x.fw[1] = w * spc / sa * f.hz;
        }

    // --- coarse crossing events: the walk of moc::Current::post_ray
    //     (moc_current_worker.hpp:202-264) precomputed per track ----------------
    auto coarse_surf = [&](int cell, int s) {
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
    };
    auto neighbor = [&](int cell, int s) {
        int ix = cell % nx, iy = cell / nx;
        switch (s) {
        case NORTH: return iy < ny - 1 ? cell + nx : -1;
        case SOUTH: return iy > 0 ? cell - nx : -1;
        case EAST: return ix < nx - 1 ? cell + 1 : -1;
        case WEST: return ix > 0 ? cell - 1 : -1;
        default: return -5;
        }
    };
    auto surf_code = [&](int surf) {
        int nsz = nx * ny + (nx + 1) * ny + (ny + 1) * nx;
        int s = surf % nsz;
        int nrm = (s < nx * ny) ? 2 : (s < nx * ny + (nx + 1) * ny) ? 0 : 1;
        if (nrm == 2) MOCGPU_THROW(6, "track crosses a z-normal surface");
        return surf * 2 + nrm;
    };
    // A track that leaves the core exactly through a pin-cell corner on the
    // core boundary has its second corner surface recorded after the walk
    // has stepped out of the core (the extra record of ray.cpp:147-166).
    // MOCC then indexes a surface from the out-of-core cell, which is
    // undefined; that second crossing lies outside the core, so it is
    // dropped here.
    std::vector<int> efb{0}, efp, efc, ebb{0}, ebp, ebc;
    for (int t = 0; t < f.n_tracks; t++) {
        int n = (int)(f.trk_seg_begin[t + 1] - f.trk_seg_begin[t]);
        int c0 = f.trk_cm_begin[t], c1 = f.trk_cm_begin[t + 1];
        int cell = f.trk_cm_cell_fw[t], k = 0;
        efp.push_back(0);
        efc.push_back(surf_code(f.trk_cm_surf_fw[t]));
        for (int c = c0; c < c1; c++) {
            int s = f.cm_fw[c];
            if (s != INVALID) {
                k += f.cm_nseg_fw[c];
                if (cell >= 0) {
                    efp.push_back(k);
                    efc.push_back(coarse_surf(cell, s) * 2 + (s == NORTH || s == SOUTH ? 1 : 0));
                } else if (f.cm_nseg_fw[c] != 0) {
                    MOCGPU_THROW(6, "coarse walk left the core before the track ends (forward)");
                }
            }
            if (cell >= 0) cell = neighbor(cell, s);
        }
        if (k != n) MOCGPU_THROW(6, "coarse forward walk does not end at the last segment");
        efb.push_back((int)efp.size());
        cell = f.trk_cm_cell_bw[t];
        k = n;
        ebp.push_back(n);
        ebc.push_back(surf_code(f.trk_cm_surf_bw[t]));
        for (int c = c0; c < c1; c++) {
            int s = f.cm_bw[c];
            if (s != INVALID) {
                k -= f.cm_nseg_bw[c];
                if (cell >= 0) {
                    ebp.push_back(k);
                    ebc.push_back(coarse_surf(cell, s) * 2 + (s == NORTH || s == SOUTH ? 1 : 0));
                } else if (f.cm_nseg_bw[c] != 0) {
                    MOCGPU_THROW(6, "coarse walk left the core before the track ends (backward)");
                }
            }
            if (cell >= 0) cell = neighbor(cell, s);
        }
        if (k != 0) MOCGPU_THROW(6, "coarse backward walk does not end at the first segment");
        ebb.push_back((int)ebp.size());
    }

    // --- exponential table (exponential.hpp:56-112 with N = 10000) --------
    const double emin = -10.0, emax = 0.0;
    const double espace = (emax - emin) / (double)kExpN, erspace = 1.0 / espace;
    std::vector<double> tab(kExpN + 1);
    for (int i = 0; i <= kExpN; i++) tab[i] = std::exp(emin + i * espace);
    set_exp_constants(emin, espace, erspace);

    // --- coarse surface areas --------------------------------------------------
    std::vector<double> surf_area(f.n_surf, 1.0);
    {
        int nsz = nx * ny + (nx + 1) * ny + (ny + 1) * nx;
        for (int is = 0; is < f.n_surf; is++) {
            int s = is % nsz;
            if (s < nx * ny) surf_area[is] = f.dx[s % nx] * f.dy[s / nx];
            else if (s < nx * ny + (nx + 1) * ny) surf_area[is] = f.dy[(s - nx * ny) / (nx + 1)] * f.hz;
            else surf_area[is] = f.dx[(s - nx * ny - (nx + 1) * ny) / (ny + 1)] * f.hz;
        }
    }
    phaseA_end = f.set_first_track[sets_oct];

    // --- bundled work-unit layout (two Gauss-Seidel phases) -----------------
    {
        int tracks_phase = f.set_first_track[sets_oct];
        // 1-2 bundles per unit when chosen automatically (measured best on
        // the 68x68 mini-core; the batch engine passes its own); unit FSR
        // sets sized so the staged pairs, the tallies and the warps' segment
        // rings fit in 227 KB; bundles dealt round-robin from the
        // length-sorted tracks
        int tpu = 32 * std::max(1, std::min(2, tracks_phase / (2 * 152 * 32)));
        if (bundles_per_unit > 0) tpu = 32 * std::min(bundles_per_unit, 4);
        int max_local = (precision == 0) ? 4096 : 8192;
        SweepLayout L = build_sweep_layout(f, true, tpu, max_local, true);
        // Units whose FSRs would take more than a few KB of shared memory
        // are staged a window of rows at a time (two tables: the forward
        // warps' window and the backward warps'), so that more CTAs fit on
        // an SM; kept where the two tables come to well under the one.
        if (window_rows > 0) {
            L = build_sweep_layout(f, true, tpu, max_local, true, window_rows);
        } else if (window_rows < 0 && MOCGPU_WINDOW_ROWS > 0 && L.max_local > MOCGPU_WINDOW_MIN_FSRS) {
            SweepLayout Lw = build_sweep_layout(f, true, tpu, max_local, true, MOCGPU_WINDOW_ROWS);
            if (10 * 2 * Lw.max_local <= 6 * L.max_local) L = std::move(Lw);
        }
        std::vector<WorkUnitDev> wud(L.wu.size());
        for (const WorkUnitHost &w : L.wu)
            if (w.n_bundles > tpu / 32) // the kernel gives each bundle direction one warp of the CTA
                MOCGPU_THROW(99, "a work unit has more bundles than its CTA has warp pairs");
        for (size_t i = 0; i < L.wu.size(); i++)
            wud[i] = WorkUnitDev{L.wu[i].set, L.wu[i].bundle_begin, L.wu[i].n_bundles, L.wu[i].win_begin,
                                 L.wu[i].n_win};
        wu_.upload(wud);
        {
            std::vector<int2> wi(L.win.size());
            for (size_t i = 0; i < L.win.size(); i++) wi[i] = make_int2(L.win[i].fsr_begin, L.win[i].n_local);
            win_.upload(wi);
        }
        bundle_row_.upload(L.bundle_row);
        bundle_nrows_.upload(L.bundle_nrows);
        bundle_track_.upload(L.bundle_track);
        {
            std::vector<int2> bbc(L.bundle_track.size(), make_int2(0, 0));
            for (size_t i = 0; i < L.bundle_track.size(); i++)
                if (L.bundle_track[i] >= 0) bbc[i] = make_int2(f.trk_bc0[L.bundle_track[i]], f.trk_bc1[L.bundle_track[i]]);
            bundle_bc_.upload(bbc);
            std::vector<int4> bev(L.bundle_track.size(), make_int4(0, 0, 0, 0));
            for (size_t i = 0; i < L.bundle_track.size(); i++) {
                const int t = L.bundle_track[i];
                if (t >= 0) bev[i] = make_int4(efb[t], efb[t + 1], ebb[t], ebb[t + 1]);
            }
            bundle_ev_.upload(bev);
        }
        local_fsr_.upload(L.local_fsr);
        blfsr_.upload(L.lfsr);
        if (precision == 0) blen_d_.upload(L.len);
        else {
            std::vector<float> lf(L.len.begin(), L.len.end());
            blen_f_.upload(lf);
        }
        phase_wu = L.phase_wu_begin;
        wu_rows.assign(L.wu.size(), 0);
        for (size_t i = 0; i < L.wu.size(); i++)
            for (int b = 0; b < L.wu[i].n_bundles; b++) wu_rows[i] += L.bundle_nrows[L.wu[i].bundle_begin + b];
        fv.wu = wu_.p;
        fv.bundle_row = bundle_row_.p;
        fv.bundle_nrows = bundle_nrows_.p;
        fv.bundle_track = bundle_track_.p;
        fv.bundle_bc = bundle_bc_.p;
        fv.bundle_ev = bundle_ev_.p;
        fv.len = precision == 0 ? (const void *)blen_d_.p : (const void *)blen_f_.p;
        fv.lfsr = blfsr_.p;
        fv.local_fsr = local_fsr_.p;
        fv.win = win_.p;
        fv.window_rows = L.window_rows;
        fv.table_slots = L.max_local;
        fv.bundles_per_unit = tpu / 32;
        fv.max_local = L.max_local * (L.max_windows > 1 ? 2 : 1);
        fv.max_hits = L.max_hits;
        if (precision != 0 && L.max_hits > kMaxTallyHits)
            MOCGPU_THROW(6, "a work unit adds more often to one FSR tally than the fixed-point tally allows");
        layout_padding = L.padding;
        layout_units = (int)L.wu.size();
        layout_max_local = L.max_local;
        layout_window_rows = L.max_windows > 1 ? L.window_rows : 0;
        layout_tracks_per_unit = tpu;
    }

    // --- upload ---------------------------------------------------------------
    seg_begin_.upload(f.trk_seg_begin);
    trk_bc0_.upload(f.trk_bc0);
    trk_bc1_.upload(f.trk_bc1);
    trk_set_.upload(f.trk_set);
    {
        std::vector<int4> te(f.n_tracks);
        for (int t = 0; t < f.n_tracks; t++)
            te[t] = make_int4(f.trk_cm_cell_fw[t], f.trk_cm_cell_bw[t], f.trk_cm_surf_fw[t], f.trk_cm_surf_bw[t]);
        trk_entry_.upload(te);
    }
    seg_fsr_.upload(f.seg_fsr);
    if (precision == 0) {
        seg_len_d_.upload(f.seg_len);
    } else {
        std::vector<float> lf(f.seg_len.begin(), f.seg_len.end());
        seg_len_f_.upload(lf);
    }
    fsr_mat_.upload(f.fsr_mat);
    fsr_vol_.upload(f.fsr_vol);
    fsr_area_.upload(f.fsr_area);
    exp_tab_.upload(tab);
    sp_.upload(sp);
    bc_off_.upload(bc_off);
    set_ny_.upload(f.set_ny);
    wt_tgt_.upload(wt);
    ev_fw_begin_.upload(efb);
    ev_fw_pt_.upload(efp);
    ev_fw_code_.upload(efc);
    ev_bw_begin_.upload(ebb);
    ev_bw_pt_.upload(ebp);
    ev_bw_code_.upload(ebc);
    if (precision == 0) {
        psi_init_dev_.upload(reinterpret_cast<const unsigned char *>(psi_init.data()), psi_init.size() * 8);
    } else {
        std::vector<float> pf(psi_init.begin(), psi_init.end());
        psi_init_dev_.upload(reinterpret_cast<const unsigned char *>(pf.data()), pf.size() * 4);
    }
    {
        std::vector<int2> pf(efp.size()), pb(ebp.size());
        for (size_t i = 0; i < efp.size(); i++) pf[i] = make_int2(efp[i], efc[i]);
        for (size_t i = 0; i < ebp.size(); i++) pb[i] = make_int2(ebp[i], ebc[i]);
        ev_fw_.upload(pf);
        ev_bw_.upload(pb);
    }
    std::vector<int> pfr(f.pin_first_reg.begin(), f.pin_first_reg.end());
    pin_first_reg_.upload(pfr);
    pin_cell_.upload(f.pin_cell);
    pin_fuel_.upload(f.pin_fuel);
    pin_area_.upload(f.pin_area);
    surf_area_.upload(surf_area);
    dx_.upload(f.dx);
    dy_.upload(f.dy);

    GeomView &g = gv_;
    g.G = G;
    g.n_fsr = f.n_fsr;
    g.n_mat = f.n_mat;
    g.n_tracks = f.n_tracks;
    g.n_sets = f.n_sets;
    g.pol = f.pol_per_set;
    g.n_ang = n_ang;
    g.ndir_oct = nd;
    g.nx = nx;
    g.ny = ny;
    g.n_pin = f.n_pin;
    g.n_surf = f.n_surf;
    g.bc_per_group = bc_per_group;
    g.hz = f.hz;
    g.seg_begin = seg_begin_.p;
    g.trk_bc0 = trk_bc0_.p;
    g.trk_bc1 = trk_bc1_.p;
    g.trk_set = trk_set_.p;
    g.trk_entry = trk_entry_.p;
    g.seg_len = precision == 0 ? (const void *)seg_len_d_.p : (const void *)seg_len_f_.p;
    g.seg_fsr = seg_fsr_.p;
    g.fsr_mat = fsr_mat_.p;
    g.fsr_vol = fsr_vol_.p;
    g.fsr_area = fsr_area_.p;
    g.xstr = g.xsnf = g.xsf = g.xsch = g.scat = nullptr;
    g.sp = sp_.p;
    g.bc_off = bc_off_.p;
    g.set_ny = set_ny_.p;
    g.wt_tgt = wt_tgt_.p;
    g.ev_fw_begin = ev_fw_begin_.p;
    g.ev_fw_pt = ev_fw_pt_.p;
    g.ev_fw_code = ev_fw_code_.p;
    g.ev_bw_begin = ev_bw_begin_.p;
    g.ev_bw_pt = ev_bw_pt_.p;
    g.ev_bw_code = ev_bw_code_.p;
    g.ev_fw = ev_fw_.p;
    g.ev_bw = ev_bw_.p;
    g.exp_tab = exp_tab_.p;
    g.pin_first_reg = pin_first_reg_.p;
    g.pin_cell = pin_cell_.p;
    g.pin_area = pin_area_.p;
    g.pin_fuel = pin_fuel_.p;

    bytes_ = seg_begin_.bytes() + trk_bc0_.bytes() * 3 + seg_fsr_.bytes() + seg_len_d_.bytes() + seg_len_f_.bytes() +
             fsr_mat_.bytes() + fsr_vol_.bytes() * 2 + sp_.bytes() + bc_off_.bytes() + wt_tgt_.bytes() +
             ev_fw_pt_.bytes() * 2 + ev_bw_pt_.bytes() * 2 + ev_fw_begin_.bytes() * 2 + wu_.bytes() +
             ev_fw_.bytes() + ev_bw_.bytes() + bundle_bc_.bytes() + bundle_ev_.bytes() + psi_init_dev_.bytes() +
             bundle_row_.bytes() + bundle_nrows_.bytes() + bundle_track_.bytes() + local_fsr_.bytes() +
             blen_f_.bytes() + blen_d_.bytes() + blfsr_.bytes() + exp_tab_.bytes() + trk_entry_.bytes() +
             win_.bytes();
    MOCGPU_CUDA(cudaDeviceSynchronize());
}

double DeviceGeometry::sweep_bytes() const
{
    // one group sweep, algorithmic: the segment stream read once (length +
    // int32 FSR id), Sigma_t/qbar read and phi written per FSR, boundary psi
    // in and out for every polar angle of every track. (The bundled layout
    // stores a 16-bit unit-local FSR id, so it moves fewer bytes per segment
    // but adds padding rows.)
    const double rb = precision == 0 ? 8.0 : 4.0;
    double psi = 0.0;
    for (int s = 0; s < n_sets; s++) psi += (double)(set_nx[s] + set_ny[s]) * pol * 2;
    return (rb + 4.0) * (double)n_seg + 3.0 * rb * n_fsr + 2.0 * rb * psi;
}

} // namespace mocgpu
