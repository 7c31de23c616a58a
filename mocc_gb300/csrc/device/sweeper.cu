#include "sweeper.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace mocgpu {

size_t Sweeper::state_bytes_for(const FlatProblem &f, int precision, int bcpg)
{
    const size_t G = f.ng, n = f.n_fsr, nc = f.n_pin, ns = f.n_surf, nm = f.n_mat;
    const size_t rb = precision == 0 ? sizeof(double) : sizeof(float);
    size_t d = 4 * nm * G + nm * G * G;                   // cross sections
    d += 2 * G * n + 3 * n;                               // phi, phi_old, fs, fs_prev, src1g
    d += 2 * G * ns;                                      // currents, surface flux
    d += G * nc + 5 * nc * G + nc * G * G + 4 * G * ns;   // coarse flux, homogenised data, coupling
    d += 2 * G * ns;                                      // partial-current sums, this and the previous CMFD solve
    d += G * 6 * nc + 2 * nc + 12 * nc + 8 + nc + 1 + 64; // CMFD operator, sources, vectors, stats, pins, red
    return d * sizeof(double) + rb * (3 * n + (G + 1) * (size_t)bcpg) + 2 * ns * sizeof(float) + sizeof(unsigned);
}

Sweeper::Sweeper(const Problem &P, int precision, cudaStream_t stream, std::shared_ptr<const DeviceGeometry> geo,
                 const CrossSections *xs)
    : f_(flat_without_tracks(P.flat)), opts_(P.opts), precision_(precision < 0 ? P.opts.precision : precision),
      stream_(stream), geo_(std::move(geo))
{
    if (xs) {
        if (xs->ng != f_.ng || xs->xstr.size() != f_.xstr.size() || xs->scat.size() != f_.scat.size())
            MOCGPU_THROW(4, "cross sections do not match the problem's materials and groups");
        f_.xstr = xs->xstr;
        f_.xsnf = xs->xsnf;
        f_.xsf = xs->xsf;
        f_.xsch = xs->xsch;
        f_.scat = xs->scat;
    }
    const FlatProblem &f = f_;
    if (!geo_)
        geo_ = std::make_shared<const DeviceGeometry>(P.flat, precision_, P.opts.bundles_per_unit, P.opts.window_rows);
    if (geo_->precision != precision_) MOCGPU_THROW(1, "shared geometry has a different precision");
    if (geo_->n_fsr != f.n_fsr || geo_->n_tracks != f.n_tracks || geo_->G != f.ng)
        MOCGPU_THROW(1, "shared geometry does not match this problem");
    const int G = f.ng;
    for (int r = 0; r < f.n_fsr; r++) {
        bool fis = false;
        for (int g = 0; g < G; g++)
            if (f.xsnf[(size_t)f.fsr_mat[r] * G + g] > 0.0) fis = true;
        if (fis) n_fissile_++;
    }

    // cross sections of this solve
    xstr_.upload(f.xstr);
    xsnf_.upload(f.xsnf);
    xsf_.upload(f.xsf);
    xsch_.upload(f.xsch);
    scat_.upload(f.scat);

    const int bcpg = geo_->bc_per_group;
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
    cur32_.alloc((size_t)2 * kCurCopies * f.n_surf);
    cur32_.zero(stream_);
    red_.alloc(64);
    red_.zero(stream_);
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
    part_.alloc((size_t)2 * G * f.n_surf);
    part_.zero(stream_);
    if (P.opts.tl_splitting) {
        split_.alloc(f.n_fsr);
        split_.zero(stream_);
    }
    cmat_.alloc((size_t)G * 6 * nc);
    cfs_.alloc(nc);
    cfs_old_.alloc(nc);
    cvec_.alloc((size_t)12 * nc);
    cstats_.alloc(8);
    pinbuf_.alloc((size_t)nc + 1);

    GeomView &g = gv_;
    g = geo_->view();
    g.n_mat = f.n_mat;
    g.xstr = xstr_.p;
    g.xsnf = xsnf_.p;
    g.xsf = xsf_.p;
    g.xsch = xsch_.p;
    g.scat = scat_.p;

    StateView &s = sv_;
    s.phi = phi_.p;
    s.phi_old = phi_old_.p;
    s.fs = fs_.p;
    s.fs_prev = fs_prev_.p;
    s.src1g = src1g_.p;
    s.qbar = qbar_.p;
    s.sigt = sigt_.p;
    s.tally = tally_.p;
    s.psi_in = psi_in_.p;
    s.psi_out = psi_out_.p;
    s.cur = cur_.p;
    s.sflux = sflux_.p;
    s.cur32 = cur32_.p;
    s.sfl32 = cur32_.p + (size_t)kCurCopies * f.n_surf;
    s.part = part_.p;
    s.split = P.opts.tl_splitting ? split_.p : nullptr;
    s.cflux = cflux_.p;
    s.red = red_.p;
    s.status = status_.p;

    CmfdView &c = cv_;
    c.G = G;
    c.nx = f.nx;
    c.ny = f.ny;
    c.n_cell = nc;
    c.n_surf = f.n_surf;
    c.hz = f.hz;
    c.dx = geo_->dx();
    c.dy = geo_->dy();
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
    c.k = red_.p + RED_K;
    c.stats = cstats_.p;
    c.status = status_.p;
    c.red = red_.p;
    c.k_tol = opts_.cmfd_k_tol;
    c.psi_tol = opts_.cmfd_psi_tol;
    c.resid_reduction = opts_.cmfd_resid_reduction;
    c.max_iter = opts_.cmfd_max_iter;
    c.fixup = opts_.cmfd_negative_fixup ? 1 : 0;
    c.has_radial = 0;

    dev_bytes_ = state_bytes_for(f, precision_, bcpg);
    double nfis = n_fissile_;
    MOCGPU_CUDA(copy_async(red_.p + RED_N_FISSILE, &nfis, sizeof(double), cudaMemcpyHostToDevice, stream_));
}

Sweeper::~Sweeper() = default;

void Sweeper::rebind(const Problem &P, const CrossSections *xs)
{
    const FlatProblem &pf = P.flat;
    if (pf.n_fsr != f_.n_fsr || pf.ng != f_.ng || pf.n_mat != f_.n_mat || pf.n_pin != f_.n_pin ||
        pf.n_tracks != f_.n_tracks || pf.n_seg != f_.n_seg)
        MOCGPU_THROW(1, "rebind needs a problem with the same traced geometry and materials");
    FlatProblem f = flat_without_tracks(pf);
    if (xs) {
        if (xs->ng != f.ng || xs->xstr.size() != f.xstr.size() || xs->scat.size() != f.scat.size())
            MOCGPU_THROW(4, "cross sections do not match the problem's materials and groups");
        f.xstr = xs->xstr;
        f.xsnf = xs->xsnf;
        f.xsf = xs->xsf;
        f.xsch = xs->xsch;
        f.scat = xs->scat;
    }
    f_ = std::move(f);
    opts_ = P.opts;
    // stream-ordered uploads into the existing buffers (the sizes match: same
    // materials and groups); f_ keeps the host arrays alive
    auto put = [&](DevBuf<double> &d, const std::vector<double> &h) {
        if (h.size() != d.n) MOCGPU_THROW(1, "rebind: cross-section array size changed");
        MOCGPU_CUDA(copy_async(d.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
    };
    put(xstr_, f_.xstr);
    put(xsnf_, f_.xsnf);
    put(xsf_, f_.xsf);
    put(xsch_, f_.xsch);
    put(scat_, f_.scat);
    gv_.xstr = xstr_.p;
    gv_.xsnf = xsnf_.p;
    gv_.xsf = xsf_.p;
    gv_.xsch = xsch_.p;
    gv_.scat = scat_.p;
    n_fissile_ = 0;
    const int G = f_.ng;
    for (int r = 0; r < f_.n_fsr; r++) {
        bool fis = false;
        for (int g = 0; g < G; g++)
            if (f_.xsnf[(size_t)f_.fsr_mat[r] * G + g] > 0.0) fis = true;
        if (fis) n_fissile_++;
    }
    cv_.k_tol = opts_.cmfd_k_tol;
    cv_.psi_tol = opts_.cmfd_psi_tol;
    cv_.resid_reduction = opts_.cmfd_resid_reduction;
    cv_.max_iter = opts_.cmfd_max_iter;
    cv_.fixup = opts_.cmfd_negative_fixup ? 1 : 0;
    double nfis = n_fissile_;
    MOCGPU_CUDA(copy_async(red_.p + RED_N_FISSILE, &nfis, sizeof(double), cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::check_status()
{
    unsigned st = 0;
    MOCGPU_CUDA(copy_async(&st, status_.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    if (st & DEV_NONPOSITIVE_PIN_FLUX) {
        status_.zero(stream_);
        MOCGPU_THROW(11, "Negative or zero input flux in set_pin_flux");
    }
    if (st & DEV_NAN) {
        status_.zero(stream_);
        MOCGPU_THROW(12, "Eigenvalue is not a number. Giving up.");
    }
    if (st & DEV_NEGATIVE_SPLIT_FLUX) {
        status_.zero(stream_);
        MOCGPU_THROW(15, "Negative flux when splitting");
    }
}

void Sweeper::apply_transverse_leakage(int g, const double *tl)
{
    // the option may have been switched on since the handle was made
    if (opts_.tl_splitting && !split_.p) {
        split_.alloc(f_.n_fsr);
        split_.zero(stream_);
    }
    sv_.split = opts_.tl_splitting ? split_.p : nullptr;
    if (!tl_.p) tl_.alloc(f_.n_fsr);
    MOCGPU_CUDA(copy_async(tl_.p, tl, sizeof(double) * f_.n_fsr, cudaMemcpyHostToDevice, stream_));
    if (precision_ == 0) launch_apply_transverse_leakage<double>(gv_, sv_, g, tl_.p, stream_);
    else launch_apply_transverse_leakage<float>(gv_, sv_, g, tl_.p, stream_);
    check_status();
}

// MoCSweeper::initialize (moc_sweeper.cpp:234-253): phi = 1, psi = 1/4pi on
// reflective upwind faces (0 on vacuum faces), coarse flux = 1.
void Sweeper::initialize()
{
    const int G = f_.ng;
    launch_fill(phi_.p, 1.0, (int64_t)G * f_.n_fsr, stream_);
    launch_fill(phi_old_.p, 1.0, (int64_t)G * f_.n_fsr, stream_);
    launch_fill(cflux_.p, 1.0, (int64_t)G * f_.n_pin, stream_);
    // incoming boundary flux of every group from the geometry's device copy
    // (stream-ordered, no host round trip)
    const size_t rb = precision_ == 0 ? sizeof(double) : sizeof(float);
    const size_t gbytes = rb * (size_t)geo_->bc_per_group;
    for (int g = 0; g < G; g++)
        MOCGPU_CUDA(cudaMemcpyAsync(psi_in_.p + g * gbytes, geo_->psi_init_device(), gbytes, cudaMemcpyDeviceToDevice,
                                    stream_));
    tally_.zero(stream_);
    cur_.zero(stream_);
    sflux_.zero(stream_);
    cur32_.zero(stream_);
    status_.zero(stream_);
    part_.zero(stream_);
    cmfd_solves_ = 0;
    has_radial_ = false;
    sweeps_done = 0;
    cmfd_iters = 0;
}

// MoCSweeper::update_incoming_flux after a CMFD solve, when the options ask
// for it (MOCC's EigenSolver::do_cmfd has the call commented out,
// eigen_solver.cpp:289, so the default leaves the boundary flux alone).
void Sweeper::update_incoming_flux(const double *part, const double *part_old, int has_old, int mode)
{
    const size_t n = (size_t)f_.ng * f_.n_surf;
    MOCGPU_CUDA(copy_async(part_.p, part, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    if (has_old) MOCGPU_CUDA(copy_async(part_.p + n, part_old, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_apply_incoming(gv_, cv_, psi_in_.p, precision_, part_.p, mode, has_old ? 1 : 0, stream_);
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::after_cmfd()
{
    if (opts_.incoming_update)
        launch_incoming_update(gv_, cv_, psi_in_.p, precision_, part_.p, opts_.incoming_update, cmfd_solves_ > 0 ? 1 : 0,
                               stream_);
    cmfd_solves_++;
}

void Sweeper::calc_fission_source(double k) { launch_fission_source(gv_, sv_, k, stream_); }

void Sweeper::set_fission_source(const double *h)
{
    MOCGPU_CUDA(copy_async(fs_.p, h, sizeof(double) * f_.n_fsr, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}
void Sweeper::get_fission_source(double *h)
{
    MOCGPU_CUDA(copy_async(h, fs_.p, sizeof(double) * f_.n_fsr, cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::store_old_flux()
{
    MOCGPU_CUDA(copy_async(phi_old_.p, phi_.p, phi_.bytes(), cudaMemcpyDeviceToDevice, stream_));
}

void Sweeper::group_source(int g)
{
    if (precision_ == 0) launch_group_source<double>(gv_, sv_, g, stream_);
    else launch_group_source<float>(gv_, sv_, g, stream_);
}

// phase 0: octant-1 track sets, 1: octant-2 track sets, -1: all (Jacobi)
void Sweeper::launch_phase(int g, int phase, bool gs, int cur)
{
    if (opts_.sweep_kernel == 0) {
        int t0 = (phase == 1) ? geo_->phaseA_end : 0;
        int t1 = (phase == 0) ? geo_->phaseA_end : f_.n_tracks;
        if (precision_ == 0) launch_sweep<double>(gv_, sv_, g, t0, t1, gs, cur != 0, stream_);
        else launch_sweep<float>(gv_, sv_, g, t0, t1, gs, cur != 0, stream_);
    } else {
        int w0 = (phase == 1) ? geo_->phase_wu[1] : 0;
        int w1 = (phase == 0) ? geo_->phase_wu[1] : geo_->phase_wu[2];
        if (precision_ == 0) launch_sweep_fast<double>(gv_, geo_->fv, sv_, g, w0, w1, gs, cur, stream_);
        else launch_sweep_fast<float>(gv_, geo_->fv, sv_, g, w0, w1, gs, cur, stream_);
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
        const int mode = cur ? (tally_sflux_ ? 1 : 2) : 0;
        if (cur) launch_zero_radial_currents(gv_, sv_, g, stream_);
        if (opts_.gs_boundary) {
            launch_phase(g, 0, true, mode);
            launch_phase(g, 1, true, mode);
        } else {
            launch_phase(g, -1, false, cur ? 1 : 0);
            if (precision_ == 0) launch_jacobi_update<double>(gv_, sv_, g, stream_);
            else launch_jacobi_update<float>(gv_, sv_, g, stream_);
        }
        launch_epilogue(g, !last);
        if (cur) {
            launch_normalize_currents(gv_, sv_, g, geo_->surf_area(), stream_);
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
    launch_total_fission(gv_, old ? phi_old_.p : phi_.p, red_.p + RED_TFIS, stream_);
    double v = 0.0;
    MOCGPU_CUDA(copy_async(&v, red_.p + RED_TFIS, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return v;
}

double Sweeper::flux_residual()
{
    launch_flux_residual(gv_, sv_, red_.p + RED_FLUXRES, stream_);
    double v = 0.0;
    MOCGPU_CUDA(copy_async(&v, red_.p + RED_FLUXRES, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return std::sqrt(v);
}

void Sweeper::get_flux(double *h) const
{
    const int G = f_.ng, n = f_.n_fsr;
    std::vector<double> tmp((size_t)G * n);
    MOCGPU_CUDA(copy_async(tmp.data(), phi_.p, phi_.bytes(), cudaMemcpyDeviceToHost, stream_));
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
    MOCGPU_CUDA(copy_async(phi_.p, tmp.data(), phi_.bytes(), cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Sweeper::get_pin_flux(int g, double *out) const
{
    launch_pin_flux(gv_, phi_.p, cflux_.p, stream_);
    MOCGPU_CUDA(copy_async(out, cflux_.p + (size_t)g * f_.n_pin, sizeof(double) * f_.n_pin,
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
    MOCGPU_CUDA(copy_async(pinbuf_.p, in, sizeof(double) * f_.n_pin, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(cudaMemsetAsync(red_.p + RED_PINRES, 0, sizeof(double), stream_));
    launch_set_pin_flux(one, phig, pinbuf_.p, red_.p + RED_PINRES, status_.p, stream_);
    double e2 = 0.0;
    MOCGPU_CUDA(copy_async(&e2, red_.p + RED_PINRES, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    check_status();
    return std::sqrt(e2) / f_.n_pin;
}

void Sweeper::pin_powers(double *out) const
{
    launch_pin_power(gv_, phi_.p, pinbuf_.p, stream_);
    std::vector<double> p(f_.n_pin + 1);
    MOCGPU_CUDA(copy_async(p.data(), pinbuf_.p, sizeof(double) * (f_.n_pin + 1), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    double scale = f_.n_fuel_2d / p[f_.n_pin];
    for (int i = 0; i < f_.n_pin; i++) out[i] = p[i] * scale;
}

std::vector<double> Sweeper::get_boundary(int g) const
{
    const size_t n = (size_t)geo_->bc_per_group;
    std::vector<double> out(n);
    if (precision_ == 0) {
        MOCGPU_CUDA(copy_async(out.data(), psi_in_.p + (size_t)g * n * sizeof(double), n * sizeof(double),
                               cudaMemcpyDeviceToHost, stream_));
        MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    } else {
        std::vector<float> f(n);
        MOCGPU_CUDA(copy_async(f.data(), psi_in_.p + (size_t)g * n * sizeof(float), n * sizeof(float),
                               cudaMemcpyDeviceToHost, stream_));
        MOCGPU_CUDA(cudaStreamSynchronize(stream_));
        std::copy(f.begin(), f.end(), out.begin());
    }
    return out;
}

void Sweeper::get_currents(double *cur, double *sfl) const
{
    MOCGPU_CUDA(copy_async(cur, cur_.p, cur_.bytes(), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(copy_async(sfl, sflux_.p, sflux_.bytes(), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

// XSMeshHomogenized::update (xs_mesh_homogenized.cpp:176-363) of the current
// flux, copied out per pin (coarse-cell order)
void Sweeper::homogenized_xs(double *xstr, double *xsnf, double *xsf, double *xsch, double *xsrm, double *scat)
{
    launch_homogenize(gv_, phi_.p, cv_, stream_);
    const size_t n = (size_t)cv_.n_cell * cv_.G * sizeof(double);
    const double *src[5] = {cv_.xstr, cv_.xsnf, cv_.xsf, cv_.xsch, cv_.xsrm};
    double *dst[5] = {xstr, xsnf, xsf, xsch, xsrm};
    for (int i = 0; i < 5; i++)
        if (dst[i]) MOCGPU_CUDA(copy_async(dst[i], src[i], n, cudaMemcpyDeviceToHost, stream_));
    if (scat) MOCGPU_CUDA(copy_async(scat, cv_.scat, n * cv_.G, cudaMemcpyDeviceToHost, stream_));
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
    MOCGPU_CUDA(copy_async(red_.p + RED_K, &k, sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_cmfd_solve(cv_, stream_);
    launch_set_pin_flux(gv_, phi_.p, cflux_.p, nullptr, status_.p, stream_);
    after_cmfd();
    MOCGPU_CUDA(copy_async(&k, red_.p + RED_K, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(copy_async(cmfd_stats, cstats_.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, stream_));
    check_status();
    cmfd_iters += (int64_t)cmfd_stats[0];
}

void Sweeper::cmfd_solve_static(double &k)
{
    // refuse an oversized mesh before any work is queued, so that a refused
    // call leaves the handle's coarse flux and homogenised data untouched
    if (cv_.n_cell > static_cmfd_max_cells())
        throw Error(21, "coarse mesh has " + std::to_string(cv_.n_cell) + " cells; the static CMFD scratch holds " +
                            std::to_string(static_cmfd_max_cells()));
    launch_pin_flux(gv_, phi_.p, cflux_.p, stream_);
    launch_homogenize(gv_, phi_.p, cv_, stream_);
    cv_.has_radial = has_radial_ ? 1 : 0;
    cv_.k_tol = opts_.cmfd_k_tol;
    cv_.psi_tol = opts_.cmfd_psi_tol;
    cv_.resid_reduction = opts_.cmfd_resid_reduction;
    cv_.max_iter = opts_.cmfd_max_iter;
    cv_.fixup = opts_.cmfd_negative_fixup ? 1 : 0;
    MOCGPU_CUDA(copy_async(red_.p + RED_K, &k, sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_cmfd_solve_static(cv_, stream_);
    launch_set_pin_flux(gv_, phi_.p, cflux_.p, nullptr, status_.p, stream_);
    after_cmfd();
    MOCGPU_CUDA(copy_async(&k, red_.p + RED_K, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(copy_async(cmfd_stats, cstats_.p, sizeof(double) * 5, cudaMemcpyDeviceToHost, stream_));
    check_status();
    cmfd_iters += (int64_t)cmfd_stats[0];
}

double Sweeper::psi_error()
{
    launch_psi_error(gv_, fs_.p, fs_prev_.p, red_.p + RED_PSI, stream_);
    double r[5];
    MOCGPU_CUDA(copy_async(r, red_.p + RED_PSI, sizeof(r), cudaMemcpyDeviceToHost, stream_));
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
    return std::sqrt(r[4] / n_fissile_);
}

// EigenSolver::step (eigen_solver.cpp:225-253)
void Sweeper::eigen_step(double &k, double &k_prev)
{
    if (opts_.cmfd && opts_.cmfd_enabled) cmfd_solve(k);
    calc_fission_source(k);
    MOCGPU_CUDA(copy_async(fs_prev_.p, fs_.p, fs_.bytes(), cudaMemcpyDeviceToDevice, stream_));
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
    // the CMFD operator reads the net currents only; the surface fluxes feed
    // the partial currents of the incoming-flux update
    struct Restore {
        bool &f, v;
        ~Restore() { f = v; }
    } restore{tally_sflux_, tally_sflux_};
    tally_sflux_ = opts_.incoming_update != 0;
    initialize();
    history_.clear();
    double k = 1.0, k_prev = 1.0;
    calc_fission_source(k);
    int max_it = (max_outer >= 0) ? max_outer : opts_.max_iter;
    for (int it = 0; it < max_it; it++) {
        eigen_step(k, k_prev);
        res.error_k = std::fabs(k - k_prev);
        res.error_psi = psi_error();
        res.iterations = it + 1;
        history_.insert(history_.end(),
                        {k, res.error_k, res.error_psi,
                         std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count()});
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
