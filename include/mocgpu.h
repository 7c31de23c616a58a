/*
 * mocgpu: C ABI of the GB300 2-D MoC sweep and CMFD power iteration.
 *
 * Every entry point returns an int status (MOCGPU_OK on success). On failure
 * mocgpu_last_error() returns a message for the calling thread. Pointer
 * arguments are HOST pointers unless the name ends in _dev. Arrays follow
 * MOCC's conventions: scalar flux is [n_fsr][n_group] row-major (MOCC's
 * ArrayB2 flux_(n_reg, n_group)), pin-mesh arrays are in coarse-cell order
 * (cell = iy * nx + ix, iy = 0 at the south face).
 *
 * Threading: a mocgpu_sweeper is bound to one CUDA stream and is not
 * re-entrant; distinct handles may be driven from distinct host threads.
 */
#ifndef MOCGPU_H
#define MOCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MOCGPU_OK 0
#define MOCGPU_ERR_ARG 1            /* invalid argument / unsupported option */
#define MOCGPU_ERR_XML 2            /* malformed XML input */
#define MOCGPU_ERR_IO 3             /* file could not be read */
#define MOCGPU_ERR_XS 4             /* cross-section library problem */
#define MOCGPU_ERR_GEOMETRY 5       /* invalid core geometry */
#define MOCGPU_ERR_RAYS 6           /* ray tracing failure */
#define MOCGPU_ERR_SOLVER 7         /* invalid solver options */
#define MOCGPU_ERR_NONPOSITIVE 11   /* non-positive pin flux in set_pin_flux */
#define MOCGPU_ERR_NAN 12           /* eigenvalue became NaN */
#define MOCGPU_ERR_NOT_CONVERGED 13 /* iteration limit reached (result still valid) */
#define MOCGPU_ERR_CANCELLED 14     /* batched solve cancelled by the caller */
#define MOCGPU_ERR_NEGATIVE_FLUX 15 /* negative scalar flux met by transverse-leakage splitting */
#define MOCGPU_ERR_CUDA 20          /* CUDA runtime error (out of memory included) */
#define MOCGPU_ERR_CAPACITY 21      /* over a memory budget or a fixed scratch size */
#define MOCGPU_ERR_INTERNAL 99

typedef struct mocgpu_problem mocgpu_problem; /* traced problem (host) */
typedef struct mocgpu_sweeper mocgpu_sweeper; /* device-resident solve */
typedef struct mocgpu_batch mocgpu_batch;     /* batched solve engine */

/* sizes reported by mocgpu_problem_sizes(), in this order */
enum {
    MOCGPU_SZ_NGROUP = 0,
    MOCGPU_SZ_NFSR,
    MOCGPU_SZ_NMAT,
    MOCGPU_SZ_NDIR_OCT,
    MOCGPU_SZ_NANG,
    MOCGPU_SZ_NSETS,
    MOCGPU_SZ_POL_PER_SET,
    MOCGPU_SZ_NX,
    MOCGPU_SZ_NY,
    MOCGPU_SZ_NPIN,
    MOCGPU_SZ_NSURF,
    MOCGPU_SZ_NFUEL,
    MOCGPU_SZ_NTRACKS,
    MOCGPU_SZ_NSEG,
    MOCGPU_SZ_NCM,
    MOCGPU_SZ_MAXSEG,
    MOCGPU_SZ_COUNT
};

typedef struct mocgpu_options {
    double k_tol, psi_tol;
    int max_iter, min_iter;
    int cmfd, cmfd_enabled;
    double cmfd_k_tol, cmfd_psi_tol, cmfd_resid_reduction;
    int cmfd_max_iter, cmfd_negative_fixup;
    int n_inner, gs_boundary, precision;
    int sweep_kernel; /* 0: one thread per track, 1: bundled work units (default) */
    int bundles_per_unit; /* bundled sweep: bundles of 32 tracks per work unit, 1..4; 0 chosen from the size */
    int window_rows;      /* bundled sweep: rows of a unit staged at a time (multiple of 16); 0 whole units; -1
                           * automatic (windows where they shrink a unit's shared memory well) */
    /* boundary angular flux update after each CMFD solve, MoCSweeper::
     * update_incoming_flux (src/sweepers/moc/moc_sweeper.cpp:255-291):
     * 0 off (default; MOCC's EigenSolver::do_cmfd has the call commented out,
     * src/solvers/eigen_solver.cpp:289), 1 as MOCC's code reads the partial
     * currents (at the index of the track's starting coarse cell), 2 from the
     * partial currents of the surface each track enters through, vacuum
     * faces left at zero. XML: <sweeper incoming_update="off|mocc|surface">.
     * Every solve of one batch engine must ask for the same value. */
    int incoming_update;
    /* MoCSweeper's allow_splitting_ (<sweeper tl_splitting>,
     * src/sweepers/moc/moc_sweeper.cpp:119): see
     * mocgpu_apply_transverse_leakage. Off by default. */
    int tl_splitting;
    /* <sweeper dump_fsr_flux> (src/sweepers/moc/moc_sweeper.cpp:103): the
     * output datasets include fsr_flux/NNN. Off by default. */
    int dump_fsr_flux;
} mocgpu_options;

typedef struct mocgpu_result {
    double k;
    int iterations;
    int converged;
    double error_k, error_psi;
    double seconds;
    int64_t sweeps;          /* one-group inner sweeps performed */
    int64_t cmfd_iterations; /* CMFD power iterations performed */
} mocgpu_result;

/* ---- library ---------------------------------------------------------- */
const char *mocgpu_last_error(void);
int mocgpu_version(void);
int mocgpu_device_count(int *n);

/* ---- problem set-up (host only; replaces MOCC's input processing,
 *      src/input_proc.cpp:164-213, CoreMesh + RayData construction,
 *      src/core/core_mesh.cpp:36-260, src/sweepers/moc/ray_data.cpp:67-343)
 * xsl_text, when non-NULL, replaces the file named by <material_lib path>.
 * base_dir resolves a relative <material_lib path>. ------------------------ */
int mocgpu_problem_create(const char *xml_text, const char *xsl_text, const char *base_dir, mocgpu_problem **out);
void mocgpu_problem_destroy(mocgpu_problem *p);
int mocgpu_problem_sizes(const mocgpu_problem *p, int64_t *sizes /* [MOCGPU_SZ_COUNT] */);
/* What AngularQuadrature::output writes (src/core/angular_quadrature.cpp:
 * 213-248) for the traced (modularised) quadrature: polar and azimuthal
 * angles per octant, and per angle of all 8 octants alpha, theta, omega_x,
 * omega_y, omega_z, weight (out: [ndir][6]; min(cap, ndir) angles written,
 * ndir reported). */
int mocgpu_problem_quadrature(const mocgpu_problem *p, int *n_polar, int *n_azimuthal, double *out, int64_t cap,
                              int64_t *ndir);
/* The cross-section library's group upper energy bounds (MaterialLib::
 * g_bounds, src/core/material_lib.cpp:80-90; written as eubounds by
 * FixedSourceSolver::output, src/solvers/fixed_source_solver.cpp:119-129). */
int mocgpu_problem_group_bounds(const mocgpu_problem *p, double *out, int cap, int *n);
int mocgpu_problem_options(const mocgpu_problem *p, mocgpu_options *out);
int mocgpu_problem_set_options(mocgpu_problem *p, const mocgpu_options *in);
/* Copies a named flat array (see FlatProblem: "seg_len", "seg_fsr", ...)
 * into dst; nbytes must equal the array's size in bytes. */
int mocgpu_problem_export(const mocgpu_problem *p, const char *field, void *dst, int64_t nbytes);
int mocgpu_problem_field_bytes(const mocgpu_problem *p, const char *field, int64_t *nbytes);

/* Seeded synthetic cross-section library in .xsl text form (materials
 * fuel1..fuelN and moderator). Writes at most buflen bytes (NUL included)
 * and reports the size needed. */
int mocgpu_synthetic_xsl(uint64_t seed, int n_group, int n_fuel, const double *fuel_nf_scale, double mod_factor,
                         double fuel_nf_factor, char *buf, int64_t buflen, int64_t *needed);

/* Traces one ray through the geometry of xml_text (which needs only the
 * geometry and material sections) as MOCC's Ray(p1, p2, bc, plane, mesh)
 * does (src/sweepers/moc/ray.cpp:52-175). Arrays receive up to cap entries.
 * coarse[] receives cm_cell_fw, cm_cell_bw, cm_surf_fw, cm_surf_bw; cm[]
 * receives (fw, bw, nseg_fw, nseg_bw) per coarse crossing. */
int mocgpu_trace_ray(const char *xml_text, const char *xsl_text, double x1, double y1, double x2, double y2,
                     int *nseg, double *seg_len, int *seg_fsr, int cap, int *coarse, int *ncm, int *cm, int cm_cap);

/* ---- sweeper: MOCC's TransportSweeper / MoCSweeper API
 *      (src/core/transport_sweeper.hpp:41-351, src/sweepers/moc/moc_sweeper.cpp)
 * precision: 0 = FP64 sweep, 1 = FP32 sweep with FP64 reductions and CMFD,
 *            -1 = the <sweeper precision> of the input (default FP64). ---- */
int mocgpu_sweeper_create(const mocgpu_problem *p, int precision, mocgpu_sweeper **out);
/* mocgpu_sweeper_create with the cross sections of another .xsl library
 * for p's materials (same names, groups and fissile flags); NULL or empty
 * xsl_text uses p's own. No MOCC counterpart (MOCC reads one library per
 * input). */
int mocgpu_sweeper_create_xsl(const mocgpu_problem *p, int precision, const char *xsl_text, mocgpu_sweeper **out);
void mocgpu_sweeper_destroy(mocgpu_sweeper *s);
int mocgpu_sweeper_set_options(mocgpu_sweeper *s, const mocgpu_options *in);
/* MoCSweeper::initialize (moc_sweeper.cpp:234-253): phi = 1, psi = 1/4pi */
int mocgpu_initialize(mocgpu_sweeper *s);
/* TransportSweeper::calc_fission_source (transport_sweeper.cpp:119-134);
 * fs may be NULL (device copy only) */
int mocgpu_calc_fission_source(mocgpu_sweeper *s, double k, double *fs);
/* FixedSourceSolver::set_fission_source: device copy of a host fs[n_fsr] */
int mocgpu_set_fission_source(mocgpu_sweeper *s, const double *fs);
/* TransportSweeper::store_old_flux */
int mocgpu_store_old_flux(mocgpu_sweeper *s);
/* Source::initialize_group + fission + in_scatter (source.cpp:41-112) */
int mocgpu_source_group(mocgpu_sweeper *s, int group);
/* MoCSweeper::sweep(group) (moc_sweeper.cpp:189-225): n_inner inner sweeps;
 * coarse currents on the last inner when coarse data is attached */
int mocgpu_sweep_group(mocgpu_sweeper *s, int group);
/* TransportSweeper::set_coarse_data: attach (1) or detach (0) the current tally */
int mocgpu_set_coarse_data(mocgpu_sweeper *s, int enabled);
/* TransportSweeper::total_fission(old) (transport_sweeper.cpp:104-117) */
int mocgpu_total_fission(mocgpu_sweeper *s, int old, double *out);
/* TransportSweeper::flux_residual (transport_sweeper.cpp:210-223) */
int mocgpu_flux_residual(mocgpu_sweeper *s, double *out);
int mocgpu_get_flux(mocgpu_sweeper *s, double *flux /* [n_fsr][G] */);
int mocgpu_set_flux(mocgpu_sweeper *s, const double *flux /* [n_fsr][G] */);
/* MoCSweeper::get_pin_flux_1g / set_pin_flux_1g, PIN_PLANE treatment
 * (moc_sweeper.cpp:293-433); resid may be NULL */
int mocgpu_get_pin_flux_1g(mocgpu_sweeper *s, int group, double *out /* [n_pin] */);
int mocgpu_set_pin_flux_1g(mocgpu_sweeper *s, int group, const double *in /* [n_pin] */, double *resid);
/* TransportSweeper::pin_powers (transport_sweeper.cpp:140-193), [ny][nx] */
int mocgpu_pin_powers(mocgpu_sweeper *s, double *out);
/* CoarseData current and surface flux after the last current sweep, [G][n_surf].
 * mocgpu_sweep_group tallies both, as MOCC's current worker does; the sweeps inside
 * mocgpu_eigen_solve tally surface fluxes only when the incoming_update
 * option reads them (CMFD itself reads the net currents), so after an eigen
 * solve without it the surface fluxes are those of the last mocgpu_sweep_group. */
int mocgpu_get_coarse_currents(mocgpu_sweeper *s, double *current, double *surface_flux);
/* BoundaryCondition::get_boundary (src/core/boundary_condition.hpp:144-164):
 * the incoming angular flux entries of one group, every angle of octants
 * 1-4 in turn, each angle's x-face entries then its y-face entries (MOCC's
 * layout). Writes min(cap, n) values converted to double and reports n in
 * *n (out may be NULL with cap 0 to ask for the size). */
int mocgpu_get_boundary_flux(mocgpu_sweeper *s, int group, double *out, int64_t cap, int64_t *n);
/* TransportSweeper::get_homogenized_xsmesh (transport_sweeper.hpp:184) with
 * XSMeshHomogenized::update (xs_mesh_homogenized.cpp:176-363): homogenises
 * the current flux on the device, one region per pin, and copies out the
 * transport, nu-fission, fission, chi and removal cross sections
 * [n_pin][G] and the scattering matrix [n_pin][G (to)][G (from)], pins in
 * coarse-cell order (x fastest). Any output pointer may be NULL. */
int mocgpu_homogenized_xs(mocgpu_sweeper *s, double *xstr, double *xsnf, double *xsf, double *xsch, double *xsrm,
                          double *scat);
/* EigenSolver::do_cmfd (eigen_solver.cpp:263-291) incl. CMFD::solve
 * (cmfd.cpp:171-279); k is read and updated. With the incoming_update
 * option on, MoCSweeper::update_incoming_flux (moc_sweeper.cpp:255-291)
 * follows, from the partial currents of CMFD::store_currents
 * (cmfd.cpp:555-638). */
int mocgpu_cmfd_solve(mocgpu_sweeper *s, double *k);
/* MoCSweeper::update_incoming_flux (moc_sweeper.cpp:255-291) from partial
 * currents that MOCC's own CMFD stored (CMFD::store_currents,
 * cmfd.cpp:555-638): part and part_old hold 2 (J+ + J-) of every coarse
 * surface, [G][n_surf], for the last and (has_old != 0) the previous CMFD
 * solve; part_old may be NULL when has_old is 0. mode 1 reads them as MOCC's
 * update_incoming_generic does (at the index of each ray's starting coarse
 * cell), mode 2 at the surface each ray enters through, leaving vacuum
 * faces at zero. For a MOCC build that keeps its CPU CMFD and calls the
 * sweeper's update_incoming_flux. */
int mocgpu_update_incoming_flux(mocgpu_sweeper *s, const double *part, const double *part_old, int has_old, int mode);
/* MoCSweeper::apply_transverse_leakage (src/sweepers/moc/moc_sweeper.cpp:
 * 435-472), the hook through which MOCC's 2-D/3-D sweeper feeds the axial
 * transverse leakage tl [n_fsr] of one group into the MoC source. Call it
 * after the group's source is built and before mocgpu_sweep_group: tl is
 * added to the group source; with the tl_splitting option, an FSR whose sum
 * would be negative gets a zero source and Sigma_t raised by -sum / phi
 * (phi its scalar flux of the group) for the sweeps that follow, the split
 * staying until the next call (a negative phi there fails with
 * MOCGPU_ERR_NEGATIVE_FLUX, as MOCC's "Negative flux when splitting"). */
int mocgpu_apply_transverse_leakage(mocgpu_sweeper *s, int group, const double *tl);
/* mocgpu_cmfd_solve without allocation (no MOCC counterpart). The CMFD work
 * vectors live in a fixed array inside the library (10 x 8192 doubles, 640
 * KiB per device) instead of a buffer of the handle, so no call allocates
 * device memory. The first call on each device looks up the array's address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. Meshes over 8192 coarse cells fail with
 * MOCGPU_ERR_CAPACITY. Nothing in the array needs to start at zero. The
 * array is shared by every handle in the process: calls that overlap in time
 * on one device race on it and must be serialised by the caller. This entry
 * point always runs the single-CTA solver; mocgpu_cmfd_solve moves meshes
 * above 1024 cells to a thread-block cluster, so between 1025 and 8192
 * cells this one is several times slower (about 3.4x on a 68x68 mesh). A
 * refused call queues no work and leaves the handle unchanged. */
int mocgpu_cmfd_solve_static(mocgpu_sweeper *s, double *k);
/* EigenSolver::solve (eigen_solver.cpp:131-223): the whole power iteration.
 * max_outer < 0 uses <solver max_iter>. Its sweeps tally net currents only,
 * unless the incoming_update option needs the surface fluxes. */
int mocgpu_eigen_solve(mocgpu_sweeper *s, int max_outer, mocgpu_result *out);
/* The last mocgpu_eigen_solve's outer iterations (EigenSolver's
 * convergence_ and iteration_times_, src/solvers/eigen_solver.cpp:185-190):
 * out [n][4] = k, error_k, error_psi, seconds since the solve began;
 * min(cap, n) rows written, n reported. */
int mocgpu_eigen_history(mocgpu_sweeper *s, double *out, int64_t cap, int64_t *n);
/* device bytes held by the handle; algorithmic bytes of one group sweep */
int mocgpu_sweeper_bytes(mocgpu_sweeper *s, int64_t *device_bytes, double *sweep_bytes);

/* ---- layout inspection (no MOCC counterpart) ---------------------------
 * Builds the bundled work-unit layout of the GPU sweep on the host (rows
 * staged window_rows at a time, a multiple of 16; 0: whole units), checks
 * that every segment maps back to its FSR and length, and reports:
 * [0] units, [1] bundles, [2] rows, [3] real segment entries, [4] FSR slots
 * of the largest window table (its FSRs + 1 padding slot), [5] phases,
 * [6] most windows of one unit, [7] windows; stats_d: [0] sum of real
 * segment lengths, [1] padding fraction. */
int mocgpu_layout_stats(const mocgpu_problem *p, int gs, int tracks_per_unit, int max_local, int window_rows,
                        int64_t *stats, double *stats_d);

/* ---- measurement helpers (no MOCC counterpart) ------------------------- */
/* The bundled sweep layout of the handle's geometry: work units, tracks per
 * unit, rows per staged window (0: whole units) and FSR slots per table. */
int mocgpu_sweeper_layout(mocgpu_sweeper *s, int *units, int *tracks_per_unit, int *window_rows, int *table_slots);
/* The CUDA stream (cudaStream_t) every launch of this handle is ordered on. */
int mocgpu_sweeper_stream(mocgpu_sweeper *s, void **stream);
/* Runs reps single-inner sweeps of a group and returns the summed device
 * time of the sweep kernels (CUDA events on the handle's stream) and the
 * number of sweep-kernel launches. Leaves the flux of that group updated. */
int mocgpu_time_sweep(mocgpu_sweeper *s, int group, int reps, double *ms, int *launches);
/* Total kernels launched by the library in this process so far. */
int mocgpu_launch_count(int64_t *n);

/* ---- batched solves (no MOCC counterpart) -------------------------------
 * MOCC runs one EigenSolver::solve (eigen_solver.cpp:131-223) per input.
 * The batch engine runs many independent solves (different cross sections,
 * lattice sizes and group counts) at once: every active solve advances one
 * power iteration per replay of one captured CUDA graph, with its own k,
 * sources and convergence test (k_tol, psi_tol, min_iter, max_iter of its
 * problem). Converged solves retire between iterations and queued ones take
 * their slots (continuous batching); admission waits until the device bytes
 * of the solve's geometry and state fit the memory budget. Retired handles
 * are kept and re-used by later solves of the same geometry, so steady-state
 * admission allocates no device memory. All solves of one
 * engine must share polar angles per track set, inner iterations and the
 * CMFD switch; the Gauss-Seidel boundary update is the only one batched.
 * The engine keeps what it needs of a submitted problem, so the problem
 * handle may be destroyed after submission; its options must not change
 * while its solves are queued. */
typedef struct mocgpu_batch_result {
    int64_t id;
    int error;          /* 0, or the MOCGPU_ERR_* code that ended this solve */
    char message[128];  /* error text */
    double k;
    int iterations;
    int converged;
    double error_k, error_psi;
    int64_t cmfd_iterations;
    double t_submit, t_admit, t_done; /* engine clock, seconds */
    int n_pin;                        /* entries of the pin-power map */
} mocgpu_batch_result;

typedef struct mocgpu_batch_stats {
    int64_t submitted, completed, outer_iterations, graph_replays, captures;
    int active, queued, capacity, geometries, bundles_per_unit;
    double bytes_in_use, bytes_budget, geometry_bytes;
    double now;           /* engine clock, seconds */
    double replay_ms;     /* device time of all graph replays */
    double sweep_ms;      /* device time of the sweep launches in them (timing on) */
    int64_t sweep_launches;
    double sweep_bytes;   /* algorithmic bytes of the timed sweep launches */
    int64_t sweep_sgu;    /* segment-group updates of the timed sweep launches */
    int64_t trace_hits, trace_misses; /* mocgpu_batch_submit_xml: traces reused / made */
    double trace_ms, xs_ms;           /* host time tracing / reading cross sections there */
} mocgpu_batch_stats;

/* precision: 0 FP64 sweep, 1 FP32 sweep (mixed); capacity: solves advanced
 * together; mem_budget_bytes: device bytes for geometry + state (0: 80% of
 * the free memory); bundles_per_unit: sweep work-unit shape, 1..4 bundles
 * of 32 tracks per CTA. Fails with MOCGPU_ERR_CUDA without a GPU. */
int mocgpu_batch_create(int precision, int capacity, double mem_budget_bytes, int bundles_per_unit,
                        mocgpu_batch **out);
void mocgpu_batch_destroy(mocgpu_batch *b);
/* Queues a solve of p; xsl_text, when not NULL, gives other cross sections
 * for p's materials (same names, groups and fissile flags) and the traced
 * geometry of p is shared. *id names the solve in mocgpu_batch_take. */
int mocgpu_batch_submit(mocgpu_batch *b, const mocgpu_problem *p, const char *xsl_text, int64_t *id);
/* Queues one solve given as MOCC input text (the XML of MOCC's input
 * processing, src/input_proc.cpp; xsl_text replaces the library file named
 * by <material_lib path> when not NULL). Requests with the same XML text
 * share one traced problem and device geometry: RayData
 * (src/sweepers/moc/ray_data.cpp:67-343) runs for the first of them only,
 * later ones read just their cross sections. */
int mocgpu_batch_submit_xml(mocgpu_batch *b, const char *xml_text, const char *xsl_text, const char *base_dir,
                            int64_t *id);
/* Admits what fits, runs one outer iteration of every active solve, retires
 * finished ones; *n_active = solves still active. */
int mocgpu_batch_step(mocgpu_batch *b, int *n_active);
/* mocgpu_batch_step in two halves: launch admits and enqueues one replay
 * (one outer iteration of every active solve) and returns at once; finish
 * waits for the oldest replay in flight and retires the solves it ended.
 * The convergence test runs on the device and a solve that ends is frozen,
 * so up to the pipeline depth (default 2) replays may be in flight: the
 * host reads one replay's summary while the next runs. Several engines,
 * each on its own stream, overlap on the GPU the same way. A launch beyond
 * the depth fails with MOCGPU_ERR_ARG. */
int mocgpu_batch_launch(mocgpu_batch *b, int *n_active);
int mocgpu_batch_finish(mocgpu_batch *b, int *n_active);
/* replays launch may have in flight, 1..4 (set with none in flight) */
int mocgpu_batch_set_pipeline_depth(mocgpu_batch *b, int depth);
/* Streaming shape of the batched sweep kernel, 0..MOCGPU_SWEEP_SHAPES-1
 * (set with none in flight; the next replay re-captures its graph): each
 * shape is a (rows per chunk, chunks in flight) pair of the warps' segment
 * rings, reported by mocgpu_sweep_shape_info. The FP64 engine has shape 0
 * only. Chosen per engine by the autotuner (mocc_gb300.tune). */
#define MOCGPU_SWEEP_SHAPES 5
int mocgpu_batch_set_sweep_shape(mocgpu_batch *b, int shape);
int mocgpu_sweep_shape_info(int shape, int *rows, int *stages);
/* replays launched and not yet finished */
int mocgpu_batch_in_flight(mocgpu_batch *b, int *n);
/* *done = 1 when nothing is in flight or the oldest replay in flight has
 * completed, so that mocgpu_batch_finish would not block. */
int mocgpu_batch_poll(mocgpu_batch *b, int *done);
/* Runs with the pipeline full until nothing is queued or active. */
int mocgpu_batch_run(mocgpu_batch *b);
/* Cancels solve id (no MOCC counterpart): a queued solve leaves the queue,
 * an active one its slot; its result then reports MOCGPU_ERR_CANCELLED.
 * Replays already launched may still advance it (their results are
 * dropped); the other solves are not disturbed. *found = 0 when id is
 * unknown or already finished. */
int mocgpu_batch_cancel(mocgpu_batch *b, int64_t id, int *found);
/* Test hook (no MOCC counterpart): after `after` more device allocations
 * the next one fails as out of memory (MOCGPU_ERR_CUDA), once; negative
 * switches it off. */
int mocgpu_debug_fail_allocations(int64_t after);
/* *ready = 1 and the result (removed from the engine) once solve id is done;
 * pin_powers (may be NULL) receives res->n_pin values. */
int mocgpu_batch_take(mocgpu_batch *b, int64_t id, int *ready, mocgpu_batch_result *res, double *pin_powers,
                        int n_pin_capacity);
/* Ids of finished solves not taken yet: up to `capacity` into ids, the
 * total in *n. */
int mocgpu_batch_ready(mocgpu_batch *b, int64_t *ids, int capacity, int *n);
int mocgpu_batch_get_stats(mocgpu_batch *b, mocgpu_batch_stats *out);
/* The CUDA stream (cudaStream_t) of the engine's launches. */
int mocgpu_batch_stream(mocgpu_batch *b, void **stream);
/* on != 0: CUDA events around every sweep launch of the graph (re-captured),
 * so the stats report the sweep kernels' device time and bytes. */
int mocgpu_batch_set_timing(mocgpu_batch *b, int on);
/* Host<->device bytes the library has copied in this process so far. */
int mocgpu_copy_bytes(int64_t *h2d, int64_t *d2h);

#ifdef __cplusplus
}
#endif

#endif /* MOCGPU_H */
