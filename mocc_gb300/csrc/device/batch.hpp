// Batched k-eigenvalue engine: many independent 2-D solves (different cross
// sections, lattice sizes and group counts) advance together, one power
// iteration of every active solve per replay of a captured CUDA graph.
//
// Each solve follows MOCC's EigenSolver::step sequence
// (src/solvers/eigen_solver.cpp:225-253) with its own k, sources and
// convergence test; only the launches are shared. Per-solve scalars stay in
// device memory (StateView::red), and the convergence test itself runs on
// the device at the end of every replay: a solve that ends is frozen (every
// later replay skips it), so the host may keep several replays in flight and
// read each replay's small summary while the next runs. Solves retire as the
// host reads that they ended, and queued solves take their slots before the
// next launch (continuous batching); admission is gated by a device-memory
// budget against the solve's segment and state sizes.
#pragma once

#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "sweeper.hpp"

namespace mocgpu {

struct BatchResult {
    int64_t id = -1;
    int error = 0; // 0, or the status code that ended the solve
    std::string message;
    double k = 1.0;
    int iterations = 0;
    int converged = 0;
    double error_k = 0.0, error_psi = 0.0;
    int64_t cmfd_iterations = 0;
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0; // seconds on the engine clock
    std::vector<double> pin_powers;                      // [ny][nx], normalised to the fuel pin count
};

struct BatchStats {
    int64_t submitted = 0, completed = 0, outer_iterations = 0, graph_replays = 0, captures = 0;
    int64_t trace_hits = 0, trace_misses = 0; // submit_xml: traced problems reused / traced anew
    double trace_ms = 0.0;                    // host time spent tracing in submit_xml
    double xs_ms = 0.0;                       // host time spent reading cross sections in submit_xml
    int active = 0, queued = 0, capacity = 0;
    size_t bytes_in_use = 0, bytes_budget = 0, geometry_bytes = 0;
    int geometries = 0, bundles_per_unit = 0;
    double replay_ms = 0.0;      // device time of all graph replays (CUDA events on the engine stream)
    double sweep_ms = 0.0;       // device time of the sweep launches inside them (timing on)
    int64_t sweep_launches = 0;  // sweep launches timed
    double sweep_bytes = 0.0;    // algorithmic bytes of the timed sweep launches
    int64_t sweep_sgu = 0;       // segment-group updates of the timed sweep launches
};

class BatchEngine {
  public:
    // capacity: solves advanced together; mem_budget: device bytes the
    // engine may hold for geometry + solve state (0: 80% of free memory);
    // bundles_per_unit: sweep work-unit shape (1..4 bundles of 32 tracks).
    BatchEngine(int precision, int capacity, size_t mem_budget, int bundles_per_unit, cudaStream_t stream = 0);
    ~BatchEngine();
    BatchEngine(const BatchEngine &) = delete;
    BatchEngine &operator=(const BatchEngine &) = delete;

    // Queues one solve of `P` (optionally with other cross sections for the
    // same materials). `P` stays referenced until the solve is admitted.
    int64_t submit(std::shared_ptr<const Problem> P, const CrossSections *xs = nullptr);
    // Queues one solve given as MOCC input text. Solves whose XML text is
    // the same share one traced problem (and so one device geometry): the
    // first such request traces it, later ones read only their cross
    // sections from `xsl_text` (ray_data.cpp:67-343 runs once per lattice
    // shape, not once per request).
    int64_t submit_xml(const std::string &xml_text, const std::string &xsl_text, const std::string &base_dir);
    // Admits queued solves that fit, runs one outer iteration of every active
    // solve and retires the finished ones. Returns the number still active.
    int step();
    // step() in two halves: launch() admits, (re)captures and enqueues one
    // replay and returns at once (up to pipeline_depth() replays may be in
    // flight); finish() waits for the oldest replay in flight and retires the
    // solves it ended. Both return the number of active solves. Several
    // engines on their own streams overlap on the GPU the same way.
    int launch();
    int finish();
    // true when nothing is in flight or the oldest replay in flight has
    // completed (finish() would not block)
    bool poll() const;
    int in_flight() const { return (int)flights_.size(); }
    // replays that launch() may have in flight (1..4, default 2)
    void set_pipeline_depth(int d);
    // streaming shape of the batched sweep (see kSweepShapeCount); the next
    // replay re-captures the graphs
    void set_sweep_shape(int shape);
    int sweep_shape() const { return sweep_shape_; }
    int pipeline_depth() const { return depth_; }
    // Runs with the pipeline full until nothing is queued or active.
    void run();
    // Cancels solve `id`: a queued solve leaves the queue, an active one its
    // slot (replays already launched may still advance it; their results
    // are dropped). Its result reports error 14. False if `id` is unknown or
    // already finished.
    bool cancel(int64_t id);
    // Finished result of solve `id` (removed from the engine); false if the
    // solve has not finished.
    bool take_result(int64_t id, BatchResult &out);
    // ids of the finished solves whose results have not been taken yet
    std::vector<int64_t> ready_ids() const;
    BatchStats stats() const;
    double now() const; // engine clock (s)
    // Records CUDA events around every sweep launch of the captured graph so
    // that stats() reports the sweep kernels' own device time.
    void set_timing(bool on);
    cudaStream_t stream() const { return stream_; }

  private:
    struct Pending {
        int64_t id;
        std::shared_ptr<const Problem> P;
        std::unique_ptr<CrossSections> xs;
        double t_submit;
        size_t bytes; // state bytes (+ geometry bytes when not yet resident)
    };
    struct Slot {
        int64_t id = -1;
        std::unique_ptr<Sweeper> sw;
        std::shared_ptr<const DeviceGeometry> geo;
        const Problem *key = nullptr;
        int iterations = 0; // outer iterations seen in the summaries read so far
        double t_submit = 0.0, t_admit = 0.0;
        size_t bytes = 0;
    };
    // Resources of one replay in flight: its graph (its own when the sweep
    // launches are timed, whose events must not be re-recorded before they
    // are read), events around it and pinned copies of its summary and pin
    // powers.
    struct Ring {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int64_t nodes = 0;
        bool timed = false;
        std::vector<cudaEvent_t> tev; // before/after pairs around sweep launches
        int tev_used = 0;
        cudaEvent_t e0 = nullptr, e1 = nullptr; // around the replay
        cudaEvent_t e2 = nullptr;                // after its read-back copies
        double *h_sum = nullptr, *h_pins = nullptr;
        size_t h_pins_n = 0;
        int pins_stride = 0;
    };
    struct Flight {
        int ring;
        bool timed;
        int graph_ring;
        std::vector<std::pair<int, int64_t>> solves; // (slot, solve id) active at launch
    };

    std::shared_ptr<const DeviceGeometry> geometry_for(const Problem &P);
    size_t geometry_estimate(const FlatProblem &f) const;
    bool try_admit(Pending &p);
    void retire(int slot, int error, const std::string &msg, bool converged, const double *row, const double *pins,
                int pins_stride);
    void rebuild_lists();
    void capture(int r);
    void drain();
    void check_config(const Problem &P);

    int precision_, cap_, bpu_;
    int sweep_shape_ = 0;
    size_t budget_ = 0, in_use_ = 0;
    cudaStream_t stream_;
    double t0_;
    int64_t next_id_ = 0;
    std::deque<Pending> queue_;
    std::vector<Slot> slots_;
    std::map<int64_t, BatchResult> done_;
    // Resident geometries, keyed by the problem that was traced; the entry
    // keeps that problem alive so the key is never reused while cached.
    struct GeoEntry {
        std::shared_ptr<const Problem> P;
        std::shared_ptr<const DeviceGeometry> geo;
        int users = 0;
    };
    std::map<const Problem *, GeoEntry> geos_;
    // traced problems of submit_xml, by their XML text
    std::map<std::string, std::shared_ptr<const Problem>> traced_;
    // retired solve handles kept for reuse, by geometry
    std::map<const Problem *, std::vector<std::unique_ptr<Sweeper>>> pool_;
    size_t pooled_bytes_ = 0;
    int depth_ = 2;
    int64_t seq_ = 0;
    std::deque<Flight> flights_;
    BatchStats st_{};

    // batch configuration fixed by the first solve
    bool configured_ = false;
    int pol_ = 0, n_inner_ = 1;
    bool cmfd_ = false;
    int incoming_mode_ = 0; // <solver incoming_update>, shared by every solve of the batch

    // device-side views and lists
    DevBuf<GeomView> d_gv_;
    DevBuf<StateView> d_sv_;
    DevBuf<CmfdView> d_cv_;
    DevBuf<FastView> d_fv_;
    DevBuf<const double *> d_area_;
    DevBuf<int> d_act_, d_nact_;
    DevBuf<int2> d_items_;
    DevBuf<int> d_nitems_;
    DevBuf<int> d_ctr_; // per sweep launch of a replay: next-item counter of the persistent sweep
    DevBuf<double> d_sum_;  // [cap][kSummaryStride] summary rows of the last replay
    DevBuf<double> d_pins_; // [cap][pins_stride_] pin powers of the last replay
    int pins_stride_ = 0;
    std::vector<int> act_;
    bool lists_dirty_ = true;

    // graphs and the sizes they were captured for
    bool timing_ = false;
    std::vector<Ring> ring_;
    struct Shape {
        int max_fsr = 0, max_pin = 0, max_surf = 0, max_cell = 0, max_g = 0, max_local = 0, items_cap = 0;
        bool operator!=(const Shape &o) const
        {
            return max_fsr != o.max_fsr || max_pin != o.max_pin || max_surf != o.max_surf ||
                   max_cell != o.max_cell || max_g != o.max_g || max_local != o.max_local || items_cap != o.items_cap;
        }
    } shape_;
    std::vector<Shape> captured_; // per ring
    int max_items_phase_ = 0; // capacity of one (group, phase) item list
};

} // namespace mocgpu
