#include "batch.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>

namespace mocgpu {

static double wall_seconds()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

BatchEngine::BatchEngine(int precision, int capacity, size_t mem_budget, int bundles_per_unit, cudaStream_t stream)
    : precision_(precision), cap_(capacity), bpu_(bundles_per_unit), stream_(stream), t0_(wall_seconds())
{
    if (precision != 0 && precision != 1) MOCGPU_THROW(1, "precision must be 0 (double) or 1 (mixed)");
    if (capacity < 1 || capacity > 65535) MOCGPU_THROW(1, "batch capacity must be in [1, 65535]");
    if (bpu_ < 1 || bpu_ > 4) MOCGPU_THROW(1, "bundles per work unit must be in [1, 4]");
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) MOCGPU_THROW(20, "no CUDA device");
    if (mem_budget == 0) {
        size_t fr = 0, tot = 0;
        MOCGPU_CUDA(cudaMemGetInfo(&fr, &tot));
        mem_budget = (size_t)(0.8 * (double)fr);
    }
    budget_ = mem_budget;
    slots_.resize(cap_);
    d_gv_.alloc(cap_);
    d_sv_.alloc(cap_);
    d_cv_.alloc(cap_);
    d_fv_.alloc(cap_);
    d_area_.alloc(cap_);
    d_act_.alloc(cap_);
    d_nact_.alloc(1);
    d_nact_.zero(stream_);
    d_sum_.alloc((size_t)cap_ * kSummaryStride);
    ring_.resize(4);
    captured_.resize(4);
    for (Ring &r : ring_) {
        MOCGPU_CUDA(cudaEventCreate(&r.e0));
        MOCGPU_CUDA(cudaEventCreate(&r.e1));
        MOCGPU_CUDA(cudaEventCreateWithFlags(&r.e2, cudaEventDisableTiming));
        MOCGPU_CUDA(cudaMallocHost((void **)&r.h_sum, sizeof(double) * kSummaryStride * (size_t)cap_));
    }
    MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

// Waits for every replay in flight (they stay queued for finish()); needed
// before freeing or moving device memory those replays may read.
void BatchEngine::drain()
{
    if (!flights_.empty()) MOCGPU_CUDA(cudaStreamSynchronize(stream_));
}

void BatchEngine::set_pipeline_depth(int d)
{
    if (d < 1 || d > (int)ring_.size()) MOCGPU_THROW(1, "pipeline depth must be in [1, 4]");
    if (!flights_.empty()) MOCGPU_THROW(1, "change the pipeline depth with no replay in flight");
    depth_ = d;
}

void BatchEngine::set_sweep_shape(int shape)
{
    int rows = 0, stages = 0;
    sweep_shape_info(shape, &rows, &stages); // throws for a shape that is not built
    if (precision_ == 0 && shape != 0) MOCGPU_THROW(1, "the FP64 batched sweep is built in shape 0 only");
    if (!flights_.empty()) MOCGPU_THROW(1, "change the sweep shape with no replay in flight");
    if (shape == sweep_shape_) return;
    sweep_shape_ = shape;
    for (Shape &c : captured_) c = Shape{}; // force new captures
}

void BatchEngine::set_timing(bool on)
{
    if (on == timing_) return;
    if (!flights_.empty()) MOCGPU_THROW(1, "change timing with no replay in flight");
    timing_ = on;
    for (Shape &c : captured_) c = Shape{}; // force new captures
}

BatchEngine::~BatchEngine()
{
    cudaStreamSynchronize(stream_);
    for (Ring &r : ring_) {
        if (r.exec) cudaGraphExecDestroy(r.exec);
        if (r.graph) cudaGraphDestroy(r.graph);
        if (r.h_sum) cudaFreeHost(r.h_sum);
        if (r.h_pins) cudaFreeHost(r.h_pins);
        for (cudaEvent_t e : r.tev) cudaEventDestroy(e);
        if (r.e0) cudaEventDestroy(r.e0);
        if (r.e1) cudaEventDestroy(r.e1);
        if (r.e2) cudaEventDestroy(r.e2);
    }
}

double BatchEngine::now() const { return wall_seconds() - t0_; }

// All solves of one batch share the launch sequence: polar angles per track
// set (a kernel template parameter), inner iterations, Gauss-Seidel boundary
// update and whether CMFD runs.
void BatchEngine::check_config(const Problem &P)
{
    const SolverOptions &o = P.opts;
    if (!o.gs_boundary) MOCGPU_THROW(1, "the batched engine runs the Gauss-Seidel boundary update only");
    const bool cm = o.cmfd && o.cmfd_enabled;
    const int inc = cm ? o.incoming_update : 0; // the update follows a CMFD solve
    if (!configured_) {
        pol_ = P.flat.pol_per_set;
        n_inner_ = o.n_inner;
        cmfd_ = cm;
        incoming_mode_ = inc;
        configured_ = true;
        return;
    }
    if (P.flat.pol_per_set != pol_ || o.n_inner != n_inner_ || cm != cmfd_ || inc != incoming_mode_)
        MOCGPU_THROW(1, "solve does not share the batch's sweep configuration (polar angles per set, inner "
                        "iterations, CMFD, incoming flux update)");
}

size_t BatchEngine::geometry_estimate(const FlatProblem &f) const
{
    // plain and bundled segment streams (bundles padded to 32 lanes), crossing
    // events and per-track data; the measured size replaces this once built
    const size_t rb = precision_ == 0 ? 8 : 4;
    return (size_t)((double)f.n_seg * ((rb + 4) + 1.5 * (rb + 2))) + (size_t)f.n_tracks * 64 +
           (size_t)f.n_fsr * 64 + (size_t)f.cm_fw.size() * 24 + (1 << 20);
}

std::shared_ptr<const DeviceGeometry> BatchEngine::geometry_for(const Problem &P)
{
    for (auto &kv : geos_)
        if (kv.first == &P) return kv.second.geo;
    return nullptr;
}

int64_t BatchEngine::submit(std::shared_ptr<const Problem> P, const CrossSections *xs)
{
    if (!P) MOCGPU_THROW(1, "null problem");
    check_config(*P);
    if (xs && (xs->ng != P->flat.ng || xs->xstr.size() != P->flat.xstr.size()))
        MOCGPU_THROW(4, "cross sections do not match the problem's materials and groups");
    for (int s : {EAST, NORTH, WEST, SOUTH})
        if (P->flat.bc[s] != (int)BoundaryType::VACUUM && P->flat.bc[s] != (int)BoundaryType::REFLECT)
            MOCGPU_THROW(5, "radial boundaries must be vacuum or reflect for the eigenvalue path");
    Pending p;
    p.id = next_id_++;
    p.t_submit = now();
    if (xs) p.xs = std::make_unique<CrossSections>(*xs);
    p.P = std::move(P);
    queue_.push_back(std::move(p));
    st_.submitted++;
    return queue_.back().id;
}

int64_t BatchEngine::submit_xml(const std::string &xml_text, const std::string &xsl_text,
                                const std::string &base_dir)
{
    std::shared_ptr<const Problem> P;
    auto it = traced_.find(xml_text);
    if (it != traced_.end()) {
        P = it->second;
        st_.trace_hits++;
    } else {
        const double t = now();
        std::shared_ptr<const Problem> np(Problem::from_xml(xml_text, xsl_text, base_dir).release());
        st_.trace_ms += 1e3 * (now() - t);
        st_.trace_misses++;
        traced_[xml_text] = np;
        P = np;
        if (!xsl_text.empty()) return submit(P, nullptr); // traced with these cross sections
    }
    if (xsl_text.empty()) return submit(P, nullptr);
    const double t = now();
    CrossSections xs = cross_sections_from_xsl(*P, xsl_text);
    st_.xs_ms += 1e3 * (now() - t);
    return submit(P, &xs);
}

bool BatchEngine::try_admit(Pending &p)
{
    int slot = -1;
    for (int i = 0; i < cap_; i++)
        if (slots_[i].id < 0) {
            slot = i;
            break;
        }
    if (slot < 0) return false;
    const FlatProblem &f = p.P->flat;
    std::shared_ptr<const DeviceGeometry> geo = geometry_for(*p.P);
    size_t need_geo = geo ? 0 : geometry_estimate(f);
    // boundary-flux entries per group: both faces of every angle's set
    size_t bcpg = 0;
    {
        const int nd = f.ndir_oct, sets_oct = f.n_sets / 2;
        for (int a = 0; a < f.n_ang; a++) {
            int r = (a / nd >= 2) ? (a + 2 * nd) % (4 * nd) : a;
            int s = (r % nd) / f.pol_per_set + (r / nd) * sets_oct;
            bcpg += f.set_nx[s] + f.set_ny[s];
        }
    }
    size_t need_state = Sweeper::state_bytes_for(f, precision_, (int)bcpg);
    auto pit = pool_.find(p.P.get());
    const bool reuse = pit != pool_.end() && !pit->second.empty();
    if (reuse) need_state = 0;
    if (in_use_ + need_geo + need_state > budget_) {
        // release pooled handles of other geometries, then resident
        // geometries that no solve uses (replays in flight may still read a
        // retired solve's flags: let them end first)
        drain();
        for (auto it = pool_.begin(); it != pool_.end() && in_use_ + need_geo + need_state > budget_; ++it) {
            if (it->first == p.P.get()) continue;
            while (!it->second.empty() && in_use_ + need_geo + need_state > budget_) {
                const size_t b = it->second.back()->state_bytes();
                it->second.pop_back();
                in_use_ -= b;
                pooled_bytes_ -= b;
            }
        }
        for (auto it = geos_.begin(); it != geos_.end() && in_use_ + need_geo + need_state > budget_;) {
            auto pl = pool_.find(it->first);
            const bool pooled = pl != pool_.end() && !pl->second.empty();
            if (it->second.users == 0 && !pooled && it->first != p.P.get()) {
                in_use_ -= it->second.geo->bytes();
                it = geos_.erase(it);
            } else {
                ++it;
            }
        }
        if (in_use_ + need_geo + need_state > budget_) return false;
    }
    if (!geo) {
        geo = std::make_shared<const DeviceGeometry>(f, precision_, bpu_, 0); // whole units: the batched kernel
        GeoEntry e;
        e.P = p.P;
        e.geo = geo;
        geos_[p.P.get()] = e;
        in_use_ += geo->bytes();
    }
    GeoEntry &ge = geos_[p.P.get()];

    Slot &S = slots_[slot];
    if (reuse) {
        S.sw = std::move(pit->second.back());
        pit->second.pop_back();
        pooled_bytes_ -= S.sw->state_bytes();
        in_use_ -= S.sw->state_bytes(); // counted again below
        try {
            S.sw->rebind(*p.P, p.xs.get());
        } catch (...) {
            S.sw.reset(); // the handle's memory is released with it
            throw;
        }
    } else {
        // an allocation failure here leaves the engine as it was: the
        // request stays at the head of the queue
        S.sw = std::make_unique<Sweeper>(*p.P, precision_, stream_, geo, p.xs.get());
    }
    in_use_ += S.sw->state_bytes();
    ge.users++;
    S.geo = geo;
    S.key = p.P.get();
    S.id = p.id;
    S.iterations = 0;
    S.t_submit = p.t_submit;
    S.t_admit = now();
    S.bytes = S.sw->state_bytes();

    // EigenSolver::solve start (eigen_solver.cpp:131-160): flat flux, k = 1,
    // fission source at k = 1.
    Sweeper &sw = *S.sw;
    sw.set_coarse_enabled(cmfd_);
    sw.initialize();
    // per-solve scalars RED_K .. RED_CMFD_SOLVES, with the convergence test's
    // parameters (<solver k_tol psi_tol min_iter max_iter>) for kb_retire
    double init[RED_CMFD_SOLVES - RED_K + 1] = {0};
    init[RED_K - RED_K] = 1.0;
    init[RED_K_PREV - RED_K] = 1.0;
    init[RED_N_FISSILE - RED_K] = (double)sw.n_fissile();
    init[RED_K_TOL - RED_K] = p.P->opts.k_tol;
    init[RED_PSI_TOL - RED_K] = p.P->opts.psi_tol;
    init[RED_MIN_ITER - RED_K] = (double)p.P->opts.min_iter;
    init[RED_MAX_ITER - RED_K] = (double)p.P->opts.max_iter;
    MOCGPU_CUDA(copy_async(sw.state().red + RED_K, init, sizeof(init), cudaMemcpyHostToDevice, stream_));
    sw.calc_fission_source(1.0);

    // shape of the captured graph
    shape_.max_fsr = std::max(shape_.max_fsr, f.n_fsr);
    shape_.max_pin = std::max(shape_.max_pin, f.n_pin);
    shape_.max_surf = std::max(shape_.max_surf, f.n_surf);
    shape_.max_cell = std::max(shape_.max_cell, f.n_pin);
    shape_.max_g = std::max(shape_.max_g, f.ng);
    shape_.max_local = std::max(shape_.max_local, geo->fv.max_local);
    int wmax = std::max(geo->phase_wu[1] - geo->phase_wu[0], geo->phase_wu[2] - geo->phase_wu[1]);
    max_items_phase_ = std::max(max_items_phase_, wmax);
    lists_dirty_ = true;
    return true;
}

void BatchEngine::retire(int slot, int error, const std::string &msg, bool converged, const double *row,
                         const double *pins, int pins_stride)
{
    Slot &S = slots_[slot];
    BatchResult r;
    r.id = S.id;
    r.error = error;
    r.message = msg;
    r.k = row[0];
    r.iterations = (int)row[7];
    r.converged = converged ? 1 : 0;
    r.error_k = row[1];
    r.error_psi = row[2];
    r.cmfd_iterations = (int64_t)row[4];
    r.t_submit = S.t_submit;
    r.t_admit = S.t_admit;
    st_.outer_iterations += r.iterations;
    if (!error) {
        // fission-rate pin powers normalised to the fuel pin count, from the
        // read-back of the replay that ended the solve (transport_sweeper.cpp:
        // 140-193; later replays leave the row as it is)
        const FlatProblem &f = S.sw->flat();
        const double *pr = pins + (size_t)slot * pins_stride;
        const double scale = f.n_fuel_2d / pr[f.n_pin];
        r.pin_powers.resize(f.n_pin);
        for (int i = 0; i < f.n_pin; i++) r.pin_powers[i] = pr[i] * scale;
    }
    r.t_done = now();
    done_[r.id] = std::move(r);
    // the handle (and its device memory) waits in the pool for the next solve
    // of the same geometry: admission then allocates nothing
    pool_[S.key].push_back(std::move(S.sw));
    pooled_bytes_ += S.bytes;
    auto it = geos_.find(S.key);
    if (it != geos_.end()) it->second.users--;
    S.geo.reset();
    S.key = nullptr;
    S.id = -1;
    st_.completed++;
    lists_dirty_ = true;
}

// Device copies of every slot's views, the active list and the sweep work
// lists. One list per Gauss-Seidel phase holds (slot, work unit) items sorted
// by the slot's group count (descending) and then by unit size (descending),
// so the items of group g are a prefix of the list.
void BatchEngine::rebuild_lists()
{
    act_.clear();
    std::vector<GeomView> gv(cap_);
    std::vector<StateView> sv(cap_);
    std::vector<CmfdView> cv(cap_);
    std::vector<FastView> fv(cap_);
    std::vector<const double *> area(cap_, nullptr);
    for (int i = 0; i < cap_; i++) {
        const Slot &S = slots_[i];
        if (S.id < 0) continue;
        act_.push_back(i);
        gv[i] = S.sw->geom();
        sv[i] = S.sw->state();
        cv[i] = S.sw->cmfd_view();
        fv[i] = S.geo->fv;
        area[i] = S.geo->surf_area();
    }
    const int items_cap = std::max(1, max_items_phase_ * cap_);
    if (items_cap > shape_.items_cap) shape_.items_cap = items_cap;
    if ((size_t)shape_.items_cap * 2 > d_items_.n || (size_t)shape_.max_g * 2 > d_nitems_.n) drain();
    if ((size_t)shape_.items_cap * 2 > d_items_.n) d_items_.alloc((size_t)shape_.items_cap * 2);
    if ((size_t)shape_.max_g * 2 > d_nitems_.n) d_nitems_.alloc((size_t)std::max(shape_.max_g, 1) * 2);

    std::vector<int2> items[2];
    std::vector<int> nitems((size_t)shape_.max_g * 2, 0);
    for (int ph = 0; ph < 2; ph++) {
        struct It {
            int g, rows, slot, wu;
        };
        std::vector<It> v;
        for (int s : act_) {
            const DeviceGeometry &geo = *slots_[s].geo;
            for (int w = geo.phase_wu[ph]; w < geo.phase_wu[ph + 1]; w++) v.push_back({geo.G, geo.wu_rows[w], s, w});
        }
        std::stable_sort(v.begin(), v.end(), [](const It &a, const It &b) {
            if (a.g != b.g) return a.g > b.g;
            return a.rows > b.rows;
        });
        for (const It &x : v) items[ph].push_back(make_int2(x.slot, x.wu));
        for (int g = 0; g < shape_.max_g; g++) {
            int n = 0;
            for (const It &x : v) n += (x.g > g) ? 1 : 0;
            nitems[(size_t)g * 2 + ph] = n;
        }
    }
    MOCGPU_CUDA(copy_async(d_gv_.p, gv.data(), sizeof(GeomView) * cap_, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(copy_async(d_sv_.p, sv.data(), sizeof(StateView) * cap_, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(copy_async(d_cv_.p, cv.data(), sizeof(CmfdView) * cap_, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(copy_async(d_fv_.p, fv.data(), sizeof(FastView) * cap_, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(
        copy_async(d_area_.p, area.data(), sizeof(const double *) * cap_, cudaMemcpyHostToDevice, stream_));
    int nact = (int)act_.size();
    if (nact)
        MOCGPU_CUDA(copy_async(d_act_.p, act_.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(copy_async(d_nact_.p, &nact, sizeof(int), cudaMemcpyHostToDevice, stream_));
    for (int ph = 0; ph < 2; ph++)
        if (!items[ph].empty())
            MOCGPU_CUDA(copy_async(d_items_.p + (size_t)ph * shape_.items_cap, items[ph].data(),
                                        sizeof(int2) * items[ph].size(), cudaMemcpyHostToDevice, stream_));
    MOCGPU_CUDA(copy_async(d_nitems_.p, nitems.data(), sizeof(int) * nitems.size(), cudaMemcpyHostToDevice,
                                stream_));
    // (pageable sources are staged before each call returns: no wait needed)
    lists_dirty_ = false;
}

// One outer iteration of every active solve (EigenSolver::step,
// eigen_solver.cpp:225-253), captured once per batch shape into ring r's
// graph (timed graphs carry events of their own).
void BatchEngine::capture(int r)
{
    Ring &R = ring_[r];
    if (R.exec) {
        cudaGraphExecDestroy(R.exec);
        R.exec = nullptr;
    }
    if (R.graph) {
        cudaGraphDestroy(R.graph);
        R.graph = nullptr;
    }
    BatchViews b{};
    b.gv = d_gv_.p;
    b.sv = d_sv_.p;
    b.cv = d_cv_.p;
    b.fv = d_fv_.p;
    b.surf_area = d_area_.p;
    b.act = d_act_.p;
    b.n_act = d_nact_.p;
    b.cap = cap_;
    b.max_fsr = shape_.max_fsr;
    b.max_pin = shape_.max_pin;
    b.max_surf = shape_.max_surf;
    b.max_cell = shape_.max_cell;
    b.max_g = shape_.max_g;
    if (precision_ == 0) prepare_b_sweep<double>(pol_, bpu_, shape_.max_local, sweep_shape_);
    else prepare_b_sweep<float>(pol_, bpu_, shape_.max_local, sweep_shape_);
    // pin powers of every active solve, read back with the summary
    if (shape_.max_pin + 1 > pins_stride_ || (size_t)cap_ * (shape_.max_pin + 1) > d_pins_.n) {
        drain();
        pins_stride_ = shape_.max_pin + 1;
        d_pins_.alloc((size_t)cap_ * pins_stride_);
    }

    const int n_sweeps = shape_.max_g * n_inner_ * 2;
    R.timed = timing_;
    if (timing_)
        while ((int)R.tev.size() < 2 * n_sweeps) {
            cudaEvent_t e;
            MOCGPU_CUDA(cudaEventCreate(&e));
            R.tev.push_back(e);
        }
    R.tev_used = 0;
    const int64_t l0 = launch_count();
    const size_t n_ctr = (size_t)std::max(shape_.max_g, 1) * n_inner_ * 2;
    if (d_ctr_.n < n_ctr) {
        drain();
        d_ctr_.alloc(n_ctr);
    }
    MOCGPU_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed));
    try {
        MOCGPU_CUDA(cudaMemsetAsync(d_ctr_.p, 0, n_ctr * sizeof(int), stream_));
        if (cmfd_) {
            launch_b_pin_flux(b, stream_);
            launch_b_homogenize(b, stream_);
            launch_b_cmfd(b, stream_);
            launch_b_set_pin_flux(b, stream_);
            if (incoming_mode_) launch_b_incoming_update(b, precision_, incoming_mode_, stream_);
        }
        launch_b_fission_source(b, stream_);
        launch_b_copy_old(b, stream_);
        for (int g = 0; g < shape_.max_g; g++) {
            if (precision_ == 0) launch_b_group_source<double>(b, g, stream_);
            else launch_b_group_source<float>(b, g, stream_);
            for (int inner = 0; inner < n_inner_; inner++) {
                const bool last = inner == n_inner_ - 1;
                const bool tally = last && cmfd_;
                // the CMFD operator reads the net currents; the incoming-flux
                // update's partial currents read the surface fluxes too
                const int cur = tally ? (incoming_mode_ ? 1 : 2) : 0;
                if (tally) launch_b_zero_currents(b, g, stream_);
                for (int ph = 0; ph < 2; ph++) {
                    const int2 *items = d_items_.p + (size_t)ph * shape_.items_cap;
                    const int *nit = d_nitems_.p + (size_t)g * 2 + ph;
                    int *ctr = d_ctr_.p + ((size_t)g * n_inner_ + inner) * 2 + ph;
                    if (timing_)
                        MOCGPU_CUDA(cudaEventRecordWithFlags(R.tev[2 * R.tev_used], stream_, cudaEventRecordExternal));
                    if (precision_ == 0)
                        launch_b_sweep<double>(b, items, nit, shape_.items_cap, g, cur, pol_, bpu_,
                                               shape_.max_local, sweep_shape_, ctr, stream_);
                    else
                        launch_b_sweep<float>(b, items, nit, shape_.items_cap, g, cur, pol_, bpu_, shape_.max_local,
                                              sweep_shape_, ctr, stream_);
                    if (timing_) {
                        MOCGPU_CUDA(
                            cudaEventRecordWithFlags(R.tev[2 * R.tev_used + 1], stream_, cudaEventRecordExternal));
                        R.tev_used++;
                    }
                }
                if (precision_ == 0) launch_b_epilogue<double>(b, g, !last, stream_);
                else launch_b_epilogue<float>(b, g, !last, stream_);
                if (cur) launch_b_normalize_currents(b, g, stream_);
            }
        }
        launch_b_k_update(b, stream_);
        launch_b_errors(b, stream_);
        // pin powers before the convergence test: a solve that ends in this
        // replay still gets its final row
        launch_b_pin_powers(b, d_pins_.p, pins_stride_, stream_);
        launch_b_retire(b, d_sum_.p, stream_);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    MOCGPU_CUDA(cudaStreamEndCapture(stream_, &R.graph));
    MOCGPU_CUDA(cudaGraphInstantiate(&R.exec, R.graph, 0));
    R.nodes = launch_count() - l0;
    note_launches(-R.nodes); // capture records launches; replays count them
    captured_[r] = shape_;
    st_.captures++;
}

int BatchEngine::launch()
{
    if ((int)flights_.size() >= depth_)
        MOCGPU_THROW(1, "the pipeline is full: finish() the oldest outer iteration first");
    // continuous batching: fill free slots from the queue, in order
    while (!queue_.empty()) {
        if (try_admit(queue_.front())) {
            queue_.pop_front();
            continue;
        }
        bool any = false;
        for (const Slot &S : slots_) any |= S.id >= 0;
        if (any) break;
        // the head does not fit an empty engine: it never will
        Pending p = std::move(queue_.front());
        queue_.pop_front();
        BatchResult r;
        r.id = p.id;
        r.error = 21;
        r.message = "solve does not fit the engine's device-memory budget";
        r.t_submit = p.t_submit;
        r.t_done = now();
        done_[r.id] = std::move(r);
        st_.completed++;
    }
    if (lists_dirty_) rebuild_lists();
    if (act_.empty()) return 0;
    // host buffers rotate over the ring; untimed replays share one graph
    const int r = (int)(seq_ % ring_.size());
    const int gr = timing_ ? r : 0;
    if (!ring_[gr].exec || shape_ != captured_[gr] || ring_[gr].timed != timing_) capture(gr);
    Ring &R = ring_[r], &GR = ring_[gr];
    if (R.h_pins_n < (size_t)cap_ * pins_stride_) {
        if (R.h_pins) cudaFreeHost(R.h_pins);
        R.h_pins = nullptr;
        R.h_pins_n = (size_t)cap_ * pins_stride_;
        MOCGPU_CUDA(cudaMallocHost((void **)&R.h_pins, sizeof(double) * R.h_pins_n));
    }
    R.pins_stride = pins_stride_;
    MOCGPU_CUDA(cudaEventRecord(R.e0, stream_));
    MOCGPU_CUDA(cudaGraphLaunch(GR.exec, stream_));
    MOCGPU_CUDA(cudaEventRecord(R.e1, stream_));
    note_launches(GR.nodes);
    MOCGPU_CUDA(copy_async(R.h_sum, d_sum_.p, sizeof(double) * kSummaryStride * (size_t)cap_, cudaMemcpyDeviceToHost,
                           stream_));
    MOCGPU_CUDA(copy_async(R.h_pins, d_pins_.p, sizeof(double) * (size_t)cap_ * pins_stride_, cudaMemcpyDeviceToHost,
                           stream_));
    MOCGPU_CUDA(cudaEventRecord(R.e2, stream_));
    Flight F;
    F.ring = r;
    F.timed = timing_;
    F.graph_ring = gr;
    for (int s : act_) F.solves.emplace_back(s, slots_[s].id);
    flights_.push_back(std::move(F));
    seq_++;
    return (int)act_.size();
}

int BatchEngine::finish()
{
    if (flights_.empty()) {
        int n = 0;
        for (const Slot &S : slots_) n += S.id >= 0;
        return n;
    }
    const Flight F = std::move(flights_.front());
    flights_.pop_front();
    Ring &R = ring_[F.ring];
    // e2 follows the replay's read-back copies (later replays may still run)
    MOCGPU_CUDA(cudaEventSynchronize(R.e2));
    st_.graph_replays++;
    {
        float ms = 0.f;
        MOCGPU_CUDA(cudaEventElapsedTime(&ms, R.e0, R.e1));
        st_.replay_ms += ms;
    }
    if (F.timed) {
        const Ring &GR = ring_[F.graph_ring];
        for (int i = 0; i < GR.tev_used; i++) {
            float ms = 0.f;
            MOCGPU_CUDA(cudaEventElapsedTime(&ms, GR.tev[2 * i], GR.tev[2 * i + 1]));
            st_.sweep_ms += ms;
        }
        st_.sweep_launches += GR.tev_used;
    }
    for (const auto &sv : F.solves) {
        const int s = sv.first;
        Slot &S = slots_[s];
        if (S.id != sv.second) continue; // retired from an earlier replay's summary
        const double *o = R.h_sum + (size_t)s * kSummaryStride;
        const int iters = (int)o[7];
        if (iters > S.iterations && F.timed) {
            // the solve ran in this replay (a frozen one keeps its count)
            const DeviceGeometry &geo = *S.geo;
            st_.sweep_bytes += (double)geo.G * n_inner_ * geo.sweep_bytes();
            st_.sweep_sgu += (int64_t)geo.G * n_inner_ * geo.n_seg;
        }
        S.iterations = std::max(S.iterations, iters);
        switch ((int)o[6]) {
        case DONE_NONPOSITIVE:
            retire(s, 11, "Negative or zero input flux in set_pin_flux", false, o, R.h_pins, R.pins_stride);
            break;
        case DONE_NAN: retire(s, 12, "Eigenvalue is not a number. Giving up.", false, o, R.h_pins, R.pins_stride); break;
        case DONE_CONVERGED: retire(s, 0, "", true, o, R.h_pins, R.pins_stride); break;
        case DONE_MAX_ITER: retire(s, 0, "", false, o, R.h_pins, R.pins_stride); break;
        default: break;
        }
    }
    int n = 0;
    for (const Slot &S : slots_) n += S.id >= 0;
    return n;
}

bool BatchEngine::poll() const
{
    if (flights_.empty()) return true;
    cudaError_t e = cudaEventQuery(ring_[flights_.front().ring].e2);
    if (e == cudaSuccess) return true;
    if (e == cudaErrorNotReady) return false;
    MOCGPU_CUDA(e);
    return false;
}

int BatchEngine::step()
{
    launch();
    return finish();
}

void BatchEngine::run()
{
    // the pipeline stays full: the next replays are on the GPU while the
    // host reads the oldest one's summary and retires and admits solves
    while (true) {
        while ((int)flights_.size() < depth_) {
            if (launch() == 0) break;
        }
        if (flights_.empty()) {
            if (queue_.empty()) break;
            continue; // the queue head was refused; launch() went on to the next
        }
        finish();
    }
}

bool BatchEngine::cancel(int64_t id)
{
    auto done = [&](int64_t sid, double t_submit) {
        BatchResult r;
        r.id = sid;
        r.error = 14;
        r.message = "solve cancelled";
        r.t_submit = t_submit;
        r.t_done = now();
        done_[sid] = std::move(r);
        st_.completed++;
    };
    for (auto it = queue_.begin(); it != queue_.end(); ++it)
        if (it->id == id) {
            done(id, it->t_submit);
            queue_.erase(it);
            return true;
        }
    for (int s = 0; s < cap_; s++) {
        Slot &S = slots_[s];
        if (S.id != id) continue;
        // frozen on the device for replays launched from now on; the slot is
        // free for the next admission (stream order keeps the new solve's
        // initialisation after the replays in flight)
        static const double flag = (double)DONE_CANCELLED;
        MOCGPU_CUDA(copy_async(S.sw->state().red + RED_DONE, &flag, sizeof(double), cudaMemcpyHostToDevice, stream_));
        done(id, S.t_submit);
        pool_[S.key].push_back(std::move(S.sw));
        pooled_bytes_ += S.bytes;
        auto g = geos_.find(S.key);
        if (g != geos_.end()) g->second.users--;
        S.geo.reset();
        S.key = nullptr;
        S.id = -1;
        lists_dirty_ = true;
        return true;
    }
    return false;
}

bool BatchEngine::take_result(int64_t id, BatchResult &out)
{
    auto it = done_.find(id);
    if (it == done_.end()) return false;
    out = std::move(it->second);
    done_.erase(it);
    return true;
}

std::vector<int64_t> BatchEngine::ready_ids() const
{
    std::vector<int64_t> v;
    v.reserve(done_.size());
    for (const auto &kv : done_) v.push_back(kv.first);
    return v;
}

BatchStats BatchEngine::stats() const
{
    BatchStats s = st_;
    s.active = 0;
    for (const Slot &S : slots_) s.active += S.id >= 0;
    s.queued = (int)queue_.size();
    s.capacity = cap_;
    s.bytes_in_use = in_use_;
    s.bytes_budget = budget_;
    s.geometry_bytes = 0;
    for (const auto &kv : geos_) s.geometry_bytes += kv.second.geo->bytes();
    s.geometries = (int)geos_.size();
    s.bundles_per_unit = bpu_;
    return s;
}

} // namespace mocgpu
