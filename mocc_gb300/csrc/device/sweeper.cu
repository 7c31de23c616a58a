#include "sweeper.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace mocgpu {

namespace {
constexpr double kPiD = 3.1415926535897932;

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

Sweeper::Sweeper(const Problem &P, int precision, cudaStream_t stream)
    : f_(P.flat), opts_(P.opts), precision_(precision < 0 ? P.opts.precision : precision), stream_(stream)
{
    const FlatProblem &f = f_;
    const int G = f.ng;
    for (int s : {EAST, NORTH, WEST, SOUTH})
        if (f.bc[s] != (int)BoundaryType::VACUUM && f.bc[s] != (int)BoundaryType::REFLECT)
            MOCGPU_THROW(5, "radial boundaries must be vacuum or reflect for the eigenvalue path");
    if (f.pol_per_set > kMaxPolar) MOCGPU_THROW(1, "too many polar angles per track set");

    // --- angle -> track set, boundary offsets -----------------------------
    const int nd = f.ndir_oct, n_ang = f.n_ang, sets_oct = f.n_sets / 2;
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
    const int bcpg = off;
    // write-through targets and initial incoming flux
    std::vector<int> wt(4 * n_ang + n_ang, -1);
    psi_init_.assign(bcpg, 0.0);
    for (int a = 0; a < n_ang; a++) {
        int s = set_of(a);
        for (int n = 0; n < 2; n++) {
            int tgt = reflect_angle(a, n, nd);
            Surface up = upwind(f.ang_ox[tgt], f.ang_oy[tgt], n);
            wt[a * 2 + n] = (f.bc[up] == (int)BoundaryType::REFLECT) ? bc_off[tgt] : -1;
            wt[3 * n_ang + a * 2 + n] = bc_off[tgt];
            // initial value of this angle's own incoming face n
            Surface own = upwind(f.ang_ox[a], f.ang_oy[a], n);
            int lo = bc_off[a] + (n == 0 ? 0 : f.set_ny[s]);
            int cnt = (n == 0) ? f.set_ny[s] : f.set_nx[s];
            double v = (f.bc[own] == (int)BoundaryType::REFLECT) ? 1.0 / (4.0 * kPiD) : 0.0;
            for (int i = 0; i < cnt; i++) psi_init_[lo + i] = v;
        }
        wt[2 * n_ang + a] = ang_ny[a];
    }

    // --- per (set, polar) sweep parameters ----------------------------------
    std::vector<SetPolar> sp(f.n_sets * f.pol_per_set);
    for (int s = 0; s < f.n_sets; s++)
        for (int p = 0; p < f.pol_per_set; p++) {
            int iang = (s / sets_oct) * nd + (s % sets_oct) * f.pol_per_set + p;
            SetPolar &x = sp[s * f.pol_per_set + p];
            x.ang_fwd = iang;
            x.ang_bwd = reverse_angle(iang, nd);
            double sp_ = f.set_spacing[s];
            x.rsin = f.ang_rsintheta[iang];
            x.wt = f.ang_weight[iang] * sp_ * f.hz * std::sin(f.ang_theta[iang]) * kPiD;
            double w = f.ang_weight[iang] * kPiD;
            double ca = std::fabs(std::cos(f.ang_alpha[iang])), sa = std::fabs(std::sin(f.ang_alpha[iang]));
            x.cw[0] = w * f.ang_ox[iang] * sp_ / ca * f.hz;
            x.cw[1] = w * f.ang_oy[iang] * sp_ / sa * f.hz;
            x.fw[0] = w * sp_ / ca * f.hz;
            x.fw[1] = w * sp_ / sa * f.hz;
        }

    // --- coarse crossing events (moc_current_worker.hpp:202-264 walk) -----
    const int nx = f.nx, ny = f.ny;
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
    std::vector<int> efb{0}, efp, efc, ebb{0}, ebp, ebc;
    for (int t = 0; t < f.n_tracks; t++) {
        int n = (int)(f.trk_seg_begin[t + 1] - f.trk_seg_begin[t]);
        int c0 = f.trk_cm_begin[t], c1 = f.trk_cm_begin[t + 1];
        // forward
        int cell = f.trk_cm_cell_fw[t], k = 0;
        efp.push_back(0);
        efc.push_back(surf_code(f.trk_cm_surf_fw[t]));
        for (int c = c0; c < c1; c++) {
            int s = f.cm_fw[c];
            if (s != INVALID) {
                if (cell < 0) MOCGPU_THROW(6, "coarse walk left the core (forward)");
                k += f.cm_nseg_fw[c];
                efp.push_back(k);
                efc.push_back(coarse_surf(cell, s) * 2 + (s == NORTH || s == SOUTH ? 1 : 0));
            }
            cell = (cell >= 0) ? neighbor(cell, s) : cell;
        }
        if (k != n) MOCGPU_THROW(6, "coarse forward walk does not end at the last segment");
        efb.push_back((int)efp.size());
        // backward
        cell = f.trk_cm_cell_bw[t];
        k = n;
        ebp.push_back(n);
        ebc.push_back(surf_code(f.trk_cm_surf_bw[t]));
        for (int c = c0; c < c1; c++) {
            int s = f.cm_bw[c];
            if (s != INVALID) {
                if (cell < 0) MOCGPU_THROW(6, "coarse walk left the core (backward)");
                k -= f.cm_nseg_bw[c];
                ebp.push_back(k);
                ebc.push_back(coarse_surf(cell, s) * 2 + (s == NORTH || s == SOUTH ? 1 : 0));
            }
            cell = (cell >= 0) ? neighbor(cell, s) : cell;
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

    // --- areas ---------------------------------------------------------------
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
    // fissile FSR count (materials with any nu-fission)
    for (int r = 0; r < f.n_fsr; r++) {
        bool fis = false;
        for (int g = 0; g < G; g++)
            if (f.xsnf[(size_t)f.fsr_mat[r] * G + g] > 0.0) fis = true;
        if (fis) n_fissile_++;
    }
    phaseA_end_ = f.set_first_track[sets_oct];

    // --- bundled work-unit layout (two Gauss-Seidel phases) -----------------
    {
        int tracks_phase = f.set_first_track[sets_oct];
        // up to 4 bundles (8 warps) per unit; unit FSR sets sized so the
        // staged pairs, the tally and the warps' segment rings fit in 227 KB
        int tpu = 32 * std::max(1, std::min(4, tracks_phase / (2 * 152 * 32)));
        int max_local = (precision_ == 0) ? 4096 : 8192;
        SweepLayout L = build_sweep_layout(f, true, tpu, max_local);
        std::vector<WorkUnitDev> wud(L.wu.size());
        for (size_t i = 0; i < L.wu.size(); i++)
            wud[i] = WorkUnitDev{L.wu[i].set, L.wu[i].bundle_begin, L.wu[i].n_bundles, L.wu[i].fsr_begin,
                                 L.wu[i].n_local};
        wu_.upload(wud);
        bundle_row_.upload(L.bundle_row);
        bundle_nrows_.upload(L.bundle_nrows);
        bundle_track_.upload(L.bundle_track);
        local_fsr_.upload(L.local_fsr);
        blfsr_.upload(L.lfsr);
        if (precision_ == 0) blen_d_.upload(L.len);
        else {
            std::vector<float> lf(L.len.begin(), L.len.end());
            blen_f_.upload(lf);
        }
        phase_wu_ = L.phase_wu_begin;
        fv_.wu = wu_.p;
        fv_.bundle_row = bundle_row_.p;
        fv_.bundle_nrows = bundle_nrows_.p;
        fv_.bundle_track = bundle_track_.p;
        fv_.len = precision_ == 0 ? (const void *)blen_d_.p : (const void *)blen_f_.p;
        fv_.lfsr = blfsr_.p;
        fv_.local_fsr = local_fsr_.p;
        fv_.bundles_per_unit = tpu / 32;
        fv_.split = 1;
        fv_.max_local = L.max_local;
        layout_padding = L.padding;
        layout_units = (int)L.wu.size();
        layout_max_local = L.max_local;
        layout_tracks_per_unit = tpu;
    }

    // --- upload ---------------------------------------------------------------
    seg_begin_.upload(f.trk_seg_begin);
    trk_bc0_.upload(f.trk_bc0);
    trk_bc1_.upload(f.trk_bc1);
    trk_set_.upload(f.trk_set);
    seg_fsr_.upload(f.seg_fsr);
    if (precision_ == 0) {
        seg_len_d_.upload(f.seg_len);
    } else {
        std::vector<float> lf(f.seg_len.begin(), f.seg_len.end());
        seg_len_f_.upload(lf);
    }
    fsr_mat_.upload(f.fsr_mat);
    fsr_vol_.upload(f.fsr_vol);
    fsr_area_.upload(f.fsr_area);
    xstr_.upload(f.xstr);
    xsnf_.upload(f.xsnf);
    xsf_.upload(f.xsf);
    xsch_.upload(f.xsch);
    scat_.upload(f.scat);
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
    std::vector<int> pfr(f.pin_first_reg.begin(), f.pin_first_reg.end());
    pin_first_reg_.upload(pfr);
    pin_cell_.upload(f.pin_cell);
    pin_fuel_.upload(f.pin_fuel);
    pin_area_.upload(f.pin_area);
    surf_area_.upload(surf_area);
    dx_.upload(f.dx);
    dy_.upload(f.dy);

    const size_t rb = precision_ == 0 ? sizeof(double) : sizeof(float);
    phi_.alloc((size_t)G * f.n_fsr);
    phi_old_.alloc((size_t)G * f.n_fsr);
    fs_.alloc(f.n_fsr);
    fs_prev_.alloc(f.n_fsr);
    src1g_.alloc(f.n_fsr);
    qbar_.alloc(rb * f.n_fsr);
    sigt_.alloc(rb * f.n_fsr);
    tally_.alloc(rb * f.n_fsr);
    tally_.zero(stream_);
    psi_in_.alloc(rb * (size_t)G * bcpg);
    psi_out_.alloc(rb * (size_t)bcpg);
    psi_out_.zero(stream_);
    cur_.alloc((size_t)G * f.n_surf);
    sflux_.alloc((size_t)G * f.n_surf);
    cur_.zero(stream_);
    sflux_.zero(stream_);
    red_.alloc(64);
    status_.alloc(1);
    status_.zero(stream_);
    const int nc = f.n_pin;
    cflux_.alloc((size_t)G * nc);
    hxs_.alloc((size_t)5 * nc * G);
    hscat_.alloc((size_t)nc * G * G);
    dtil_.alloc((size_t)G * f.n_surf);
    dhat_.alloc((size_t)G * f.n_surf);
    stil_.alloc((size_t)G * f.n_surf);
    shat_.alloc((size_t)G * f.n_surf);
    cmat_.alloc((size_t)G * 6 * nc);
    cfs_.alloc(nc);
    cfs_old_.alloc(nc);
    cvec_.alloc((size_t)12 * nc);
    ck_.alloc(1);
    cstats_.alloc(8);
    pinbuf_.alloc((size_t)nc + 1);

    // --- views --------------------------------------------------------------
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
    g.bc_per_group = bcpg;
    g.hz = f.hz;
    g.seg_begin = seg_begin_.p;
    g.trk_bc0 = trk_bc0_.p;
    g.trk_bc1 = trk_bc1_.p;
    g.trk_set = trk_set_.p;
    g.seg_len = precision_ == 0 ? (const void *)seg_len_d_.p : (const void *)seg_len_f_.p;
    g.seg_fsr = seg_fsr_.p;
    g.fsr_mat = fsr_mat_.p;
    g.fsr_vol = fsr_vol_.p;
    g.fsr_area = fsr_area_.p;
    g.xstr = xstr_.p;
    g.xsnf = xsnf_.p;
    g.xsf = xsf_.p;
    g.xsch = xsch_.p;
    g.scat = scat_.p;
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
    g.exp_tab = exp_tab_.p;
    g.pin_first_reg = pin_first_reg_.p;
    g.pin_cell = pin_cell_.p;
    g.pin_area = pin_area_.p;
    g.pin_fuel = pin_fuel_.p;

    StateView &s = sv_;
    s.phi = phi_.p;
    s.phi_old = phi_old_.p;
    s.fs = fs_.p;
    s.src1g = src1g_.p;
    s.qbar = qbar_.p;
    s.sigt = sigt_.p;
    s.tally = tally_.p;
    s.psi_in = psi_in_.p;
    s.psi_out = psi_out_.p;
    s.cur = cur_.p;
    s.sflux = sflux_.p;
    s.red = red_.p;
    s.status = status_.p;

    CmfdView &c = cv_;
    c.G = G;
    c.nx = nx;
    c.ny = ny;
    c.n_cell = nc;
    c.n_surf = f.n_surf;
    c.hz = f.hz;
    c.dx = dx_.p;
    c.dy = dy_.p;
    for (int i = 0; i < 6; i++) c.bc[i] = f.bc[i];
    c.flux = cflux_.p;
    c.xstr = hxs_.p;
    c.xsnf = hxs_.p + (size_t)nc * G;
    c.xsf = hxs_.p + (size_t)2 * nc * G;
    c.xsch = hxs_.p + (size_t)3 * nc * G;
    c.xsrm = hxs_.p + (size_t)4 * nc * G;
    c.scat = hscat_.p;
    c.d_tilde = dtil_.p;
    c.d_hat = dhat_.p;
    c.s_tilde = stil_.p;
    c.s_hat = shat_.p;
    c.mat = cmat_.p;
    c.fs = cfs_.p;
    c.fs_old = cfs_old_.p;
    c.vec = cvec_.p;
    c.cur = cur_.p;
    c.sflux = sflux_.p;
    c.k = ck_.p;
    c.stats = cstats_.p;
    c.status = status_.p;

    dev_bytes_ = seg_begin_.bytes() + trk_bc0_.bytes() * 3 + seg_fsr_.bytes() + seg_len_d_.bytes() + seg_len_f_.bytes() +
                  phi_.bytes() * 2 + psi_in_.bytes() + psi_out_.bytes() + cur_.bytes() * 2 + cvec_.bytes() +
                  cmat_.bytes() + hscat_.bytes() + ev_fw_pt_.bytes() * 2 + ev_bw_pt_.bytes() * 2;
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

Sweeper::~Sweeper() = default;

double Sweeper::sweep_bytes() const
{
    // algorithmic bytes of one group sweep: segment stream read once,
    // Sigma_t/qbar read and phi written per FSR, boundary psi in and out.
    const double rb = precision_ == 0 ? 8.0 : 4.0;
    double psi = 0.0;
    for (int s = 0; s < f_.n_sets; s++) psi += (double)(f_.set_nx[s] + f_.set_ny[s]) * f_.pol_per_set * 2;
    return (rb + 4.0) * (double)f_.n_seg + 3.0 * rb * f_.n_fsr + 2.0 * rb * psi;
}

void Sweeper::check_status()
{
    unsigned st = 0;
    MOCGPU_CUDA(cudaMemcpyAsync(&st, status_.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    if (st & DEV_NONPOSITIVE_PIN_FLUX) {
        status_.zero(stream_);
        MOCGPU_THROW(11, "Negative or zero input flux in set_pin_flux");
    }
    if (st & DEV_NAN) {
        status_.zero(stream_);
        MOCGPU_THROW(12, "Eigenvalue is not a number. Giving up.");
    }
}

void Sweeper::initialize()
{
    const int G = f_.ng;
    launch_fill(phi_.p, 1.0, (int64_t)G * f_.n_fsr, stream_);
    launch_fill(phi_old_.p, 1.0, (int64_t)G * f_.n_fsr, stream_);
    launch_fill(cflux_.p, 1.0, (int64_t)G * f_.n_pin, stream_);
    // psi_in = 1/4pi on reflective upwind faces, 0 on vacuum faces
    std::vector<double> init((size_t)G * gv_.bc_per_group);
    for (int g = 0; g < G; g++) std::copy(psi_init_.begin(), psi_init_.end(), init.begin() + (size_t)g * gv_.bc_per_group);
    if (precision_ == 0) {
        MOCGPU_CUDA(cudaMemcpyAsync(psi_in_.p, init.data(), init.size() * 8, cudaMemcpyHostToDevice, stream_));
        MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    } else {
        std::vector<float> fi(init.begin(), init.end());
        MOCGPU_CUDA(cudaMemcpyAsync(psi_in_.p, fi.data(), fi.size() * 4, cudaMemcpyHostToDevice, stream_));
        MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    }
    tally_.zero(stream_);
    cur_.zero(stream_);
    sflux_.zero(stream_);
    status_.zero(stream_);
    has_radial_ = false;
    sweeps_done = 0;
    cmfd_iters = 0;
}

void Sweeper::calc_fission_source(double k) { launch_fission_source(gv_, sv_, k, stream_); }

void Sweeper::set_fission_source(const double *h)
{
    MOCGPU_CUDA(cudaMemcpyAsync(fs_.p, h, sizeof(double) * f_.n_fsr, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}
void Sweeper::get_fission_source(double *h)
{
    MOCGPU_CUDA(cudaMemcpyAsync(h, fs_.p, sizeof(double) * f_.n_fsr, cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::store_old_flux()
{
    MOCGPU_CUDA(cudaMemcpyAsync(phi_old_.p, phi_.p, phi_.bytes(), cudaMemcpyDeviceToDevice, stream_));
}

void Sweeper::group_source(int g)
{
    if (precision_ == 0) launch_group_source<double>(gv_, sv_, g, stream_);
    else launch_group_source<float>(gv_, sv_, g, stream_);
}

// phase 0: octant-1 track sets, 1: octant-2 track sets, -1: all (Jacobi)
void Sweeper::launch_phase(int g, int phase, bool gs, bool cur)
{
    if (opts_.sweep_kernel == 0) {
        int t0 = (phase == 1) ? phaseA_end_ : 0;
        int t1 = (phase == 0) ? phaseA_end_ : f_.n_tracks;
        if (precision_ == 0) launch_sweep<double>(gv_, sv_, g, t0, t1, gs, cur, stream_);
        else launch_sweep<float>(gv_, sv_, g, t0, t1, gs, cur, stream_);
    } else {
        int w0 = (phase == 1) ? phase_wu_[1] : 0;
        int w1 = (phase == 0) ? phase_wu_[1] : phase_wu_[2];
        if (precision_ == 0) launch_sweep_fast<double>(gv_, fv_, sv_, g, w0, w1, gs, cur, stream_);
        else launch_sweep_fast<float>(gv_, fv_, sv_, g, w0, w1, gs, cur, stream_);
    }
}

void Sweeper::launch_epilogue(int g, bool update_q)
{
    if (precision_ == 0) launch_sweep_epilogue<double>(gv_, sv_, g, update_q, stream_);
    else launch_sweep_epilogue<float>(gv_, sv_, g, update_q, stream_);
}

// MoCSweeper::sweep (moc_sweeper.cpp:189-225): the group source is already
// built; each inner iteration sweeps all tracks (Gauss-Seidel: octant-1 then
// octant-2 track sets, Jacobi: all at once plus the boundary update) and
// finishes with the flux scaling and the self-scatter source update.
void Sweeper::sweep(int g)
{
    for (int inner = 0; inner < opts_.n_inner; inner++) {
        bool last = (inner == opts_.n_inner - 1);
        bool cur = last && coarse_enabled_;
        if (cur) launch_zero_radial_currents(gv_, sv_, g, stream_);
        if (opts_.gs_boundary) {
            launch_phase(g, 0, true, cur);
            launch_phase(g, 1, true, cur);
        } else {
            launch_phase(g, -1, false, cur);
            if (precision_ == 0) launch_jacobi_update<double>(gv_, sv_, g, stream_);
            else launch_jacobi_update<float>(gv_, sv_, g, stream_);
        }
        launch_epilogue(g, !last);
        if (cur) {
            launch_normalize_currents(gv_, sv_, g, surf_area_.p, stream_);
            has_radial_ = true;
        }
        sweeps_done++;
    }
}

double Sweeper::time_sweep(int g, int reps, int *launches)
{
    cudaEvent_t e0, e1;
    MOCGPU_CUDA(cudaEventCreate(&e0));
    MOCGPU_CUDA(cudaEventCreate(&e1));
    double total = 0.0;
    int nl = 0;
    for (int r = 0; r < reps; r++) {
        MOCGPU_CUDA(cudaEventRecord(e0, stream_));
        if (opts_.gs_boundary) {
            launch_phase(g, 0, true, false);
            launch_phase(g, 1, true, false);
            nl += 2;
        } else {
            launch_phase(g, -1, false, false);
            nl += 1;
        }
        MOCGPU_CUDA(cudaEventRecord(e1, stream_));
        if (!opts_.gs_boundary) {
            if (precision_ == 0) launch_jacobi_update<double>(gv_, sv_, g, stream_);
            else launch_jacobi_update<float>(gv_, sv_, g, stream_);
        }
        launch_epilogue(g, true);
        MOCGPU_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        MOCGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        total += ms;
    }
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (launches) *launches = nl;
    return total;
}

double Sweeper::total_fission(bool old)
{
    launch_total_fission(gv_, old ? phi_old_.p : phi_.p, red_.p + 8, stream_);
    double v = 0.0;
    MOCGPU_CUDA(cudaMemcpyAsync(&v, red_.p + 8, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return v;
}

double Sweeper::flux_residual()
{
    launch_flux_residual(gv_, sv_, red_.p + 9, stream_);
    double v = 0.0;
    MOCGPU_CUDA(cudaMemcpyAsync(&v, red_.p + 9, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return std::sqrt(v);
}

void Sweeper::get_flux(double *h) const
{
    const int G = f_.ng, n = f_.n_fsr;
    std::vector<double> tmp((size_t)G * n);
    MOCGPU_CUDA(cudaMemcpyAsync(tmp.data(), phi_.p, phi_.bytes(), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    for (int r = 0; r < n; r++)
        for (int g = 0; g < G; g++) h[(size_t)r * G + g] = tmp[(size_t)g * n + r];
}

void Sweeper::set_flux(const double *h)
{
    const int G = f_.ng, n = f_.n_fsr;
    std::vector<double> tmp((size_t)G * n);
    for (int r = 0; r < n; r++)
        for (int g = 0; g < G; g++) tmp[(size_t)g * n + r] = h[(size_t)r * G + g];
    MOCGPU_CUDA(cudaMemcpyAsync(phi_.p, tmp.data(), phi_.bytes(), cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::get_pin_flux(int g, double *out) const
{
    launch_pin_flux(gv_, phi_.p, cflux_.p, stream_);
    MOCGPU_CUDA(cudaMemcpyAsync(out, cflux_.p + (size_t)g * f_.n_pin, sizeof(double) * f_.n_pin,
                                cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

double Sweeper::set_pin_flux(int g, const double *in)
{
    for (int i = 0; i < f_.n_pin; i++)
        if (!(in[i] > 0.0)) MOCGPU_THROW(11, "Negative or zero input flux: " + std::to_string(in[i]));
    // Rescale only group g: run the kernel on a one-group view of the state.
    GeomView one = gv_;
    one.G = 1;
    double *phig = phi_.p + (size_t)g * f_.n_fsr;
    MOCGPU_CUDA(cudaMemcpyAsync(pinbuf_.p, in, sizeof(double) * f_.n_pin, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaMemsetAsync(red_.p + 10, 0, sizeof(double), stream_));
    launch_set_pin_flux(one, phig, pinbuf_.p, red_.p + 10, status_.p, stream_);
    double e2 = 0.0;
    MOCGPU_CUDA(cudaMemcpyAsync(&e2, red_.p + 10, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    check_status();
    return std::sqrt(e2) / f_.n_pin;
}

void Sweeper::pin_powers(double *out) const
{
    launch_pin_power(gv_, phi_.p, pinbuf_.p, stream_);
    std::vector<double> p(f_.n_pin + 1);
    MOCGPU_CUDA(cudaMemcpyAsync(p.data(), pinbuf_.p, sizeof(double) * (f_.n_pin + 1), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    double scale = f_.n_fuel_2d / p[f_.n_pin];
    for (int i = 0; i < f_.n_pin; i++) out[i] = p[i] * scale;
}

void Sweeper::get_currents(double *cur, double *sfl) const
{
    MOCGPU_CUDA(cudaMemcpyAsync(cur, cur_.p, cur_.bytes(), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaMemcpyAsync(sfl, sflux_.p, sflux_.bytes(), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

// EigenSolver::do_cmfd (eigen_solver.cpp:263-291): coarse flux from the
// fine flux, homogenise, CMFD solve, then rescale the fine flux.
void Sweeper::cmfd_solve(double &k)
{
    launch_pin_flux(gv_, phi_.p, cflux_.p, stream_);
    launch_homogenize(gv_, phi_.p, cv_, stream_);
    cv_.has_radial = has_radial_ ? 1 : 0;
    cv_.k_tol = opts_.cmfd_k_tol;
    cv_.psi_tol = opts_.cmfd_psi_tol;
    cv_.resid_reduction = opts_.cmfd_resid_reduction;
    cv_.max_iter = opts_.cmfd_max_iter;
    cv_.fixup = opts_.cmfd_negative_fixup ? 1 : 0;
    MOCGPU_CUDA(cudaMemcpyAsync(ck_.p, &k, sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_cmfd_solve(cv_, stream_);
    launch_set_pin_flux(gv_, phi_.p, cflux_.p, nullptr, status_.p, stream_);
    MOCGPU_CUDA(cudaMemcpyAsync(&k, ck_.p, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaMemcpyAsync(cmfd_stats, cstats_.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, stream_));
    check_status();
    cmfd_iters += (int64_t)cmfd_stats[0];
}

double Sweeper::psi_error()
{
    launch_psi_error(gv_, fs_.p, fs_prev_.p, red_.p, stream_);
    double r[5];
    MOCGPU_CUDA(cudaMemcpyAsync(r, red_.p, sizeof(r), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return std::sqrt(r[4] / n_fissile_);
}

// EigenSolver::step (eigen_solver.cpp:225-253)
void Sweeper::eigen_step(double &k, double &k_prev)
{
    if (opts_.cmfd && opts_.cmfd_enabled) cmfd_solve(k);
    calc_fission_source(k);
    MOCGPU_CUDA(cudaMemcpyAsync(fs_prev_.p, fs_.p, fs_.bytes(), cudaMemcpyDeviceToDevice, stream_));
    store_old_flux();
    for (int g = 0; g < f_.ng; g++) {
        group_source(g);
        sweep(g);
    }
    double t1 = total_fission(false);
    double t2 = total_fission(true);
    k_prev = k;
    k = k * t1 / t2;
    calc_fission_source(k);
}

// EigenSolver::solve (eigen_solver.cpp:131-223)
EigenResult Sweeper::eigen_solve(int max_outer)
{
    auto t0 = std::chrono::steady_clock::now();
    EigenResult res;
    set_coarse_enabled(opts_.cmfd && opts_.cmfd_enabled);
    initialize();
    double k = 1.0, k_prev = 1.0;
    calc_fission_source(k);
    int max_it = (max_outer >= 0) ? max_outer : opts_.max_iter;
    for (int it = 0; it < max_it; it++) {
        eigen_step(k, k_prev);
        res.error_k = std::fabs(k - k_prev);
        res.error_psi = psi_error();
        res.iterations = it + 1;
        if (!std::isfinite(k)) MOCGPU_THROW(12, "Eigenvalue is not a number. Giving up.");
        if (res.error_k < opts_.k_tol && res.error_psi < opts_.psi_tol && it >= opts_.min_iter) {
            res.converged = 1;
            break;
        }
    }
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    res.k = k;
    res.sweeps = sweeps_done;
    res.cmfd_iterations = cmfd_iters;
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return res;
}

} // namespace mocgpu
