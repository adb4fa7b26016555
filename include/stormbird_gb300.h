/*
 * stormbird_gb300 — C ABI of the GB300 (sm_103a) lifting-line hot path.
 *
 * This library is a drop-in for the path behind the reference's `Simulation`
 * (stormbird/src/lifting_line/simulation.rs:20-217): JSON setup in, one `do_step`
 * per time step with the freestream at the points `get_freestream_velocity_points`
 * returns, per-step circulation and forces out. Conventions follow the reference's
 * C interface `cstormbird` (interfaces/cstormbird/src/lifting_line/complete_sail_model.rs:18-110):
 * an opaque handle built from a JSON string (NULL on error), caller-owned buffers,
 * negative integer status codes, `#[repr(C)]`-style POD results in f64.
 *
 * Numbers are f64 at the boundary ([x, y, z] triples, i.e. `[f64; 3]` arrays as the
 * PyO3 binding passes them, interfaces/pystormbird/src/lifting_line/simulation.rs:117-164).
 * Inside, the Biot-Savart sweeps run in FP32 with compensated accumulation; wake
 * positions, the circulation solve and the residual reductions run in FP64.
 *
 * Threading: one handle owns one CUDA stream and its device memory. A handle is not
 * thread-safe; different handles may be driven from different host threads.
 * Device pointers passed in: the call reads them after the work enqueued before it on the
 * legacy default stream (stream 0, PyTorch's default stream) has finished, and is done
 * with them (and has written device outputs) when it returns. A caller producing device
 * inputs on another stream synchronises that stream first. (sb_panel_sweep_no_alloc takes
 * the stream to work on and follows that stream's order instead.)
 * Errors: every entry point returns SB_OK (0) or a negative SB_ERR_* code; the
 * message of the last error on the calling thread is available from sb_last_error().
 */
#ifndef STORMBIRD_GB300_H
#define STORMBIRD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SB_OK 0
#define SB_ERR_NULL_ARG (-1)    /* a required pointer was NULL (cstormbird: -1)                  */
#define SB_ERR_SIZE (-2)        /* a buffer length does not match the model (cstormbird: -2)     */
#define SB_ERR_BAD_JSON (-3)    /* setup JSON malformed or violates the SimulationBuilder schema  */
#define SB_ERR_CUDA (-4)        /* a CUDA call failed; the handle should be freed                 */
#define SB_ERR_NONFINITE (-5)   /* NaN/Inf in an input array                                      */
#define SB_ERR_TIMEOUT (-6)     /* a bounded device-side wait ran out                             */
#define SB_ERR_UNSUPPORTED (-7) /* valid reference setup outside this path (e.g. rotor sections)  */
#define SB_ERR_STATE (-8)       /* call not valid in this state (e.g. induced velocities in QS)   */

typedef struct sb_sim sb_sim; /* opaque simulation handle */

/*
 * Per-step output, mirroring the reference's SimulationResult
 * (stormbird/src/common_utils/results/simulation.rs:27-40) and SolverResult
 * (common_utils/results/solver.rs:12-18). N = span lines, S = wings.
 * Array members are caller-owned and may be NULL (not written). The six force
 * components are ordered circulatory, viscous_lift, sectional_drag, added_mass,
 * gyroscopic, total (common_utils/forces_and_moments.rs:108-160).
 */
typedef struct sb_step_output {
    double* circulation_strength;       /* [N]        SolverResult.circulation_strength            */
    double* ctrl_points_velocity;       /* [N*3]      SolverResult.output_ctrl_points_velocity      */
    double* solver_input_velocity;      /* [N*3]      felt freestream at the control points         */
    double* angles_of_attack;           /* [N]        force_input.angles_of_attack                  */
    double* force_input_velocity;       /* [N*3]      force_input.velocity (output frame)           */
    double* acceleration;               /* [N*3]      force_input.acceleration (output frame)       */
    double* ctrl_points;                /* [N*3]      ctrl points (global)                          */
    double* sectional_forces;           /* [6*N*3]    component-major                               */
    double* integrated_forces;          /* [S*6*3]    wing-major                                    */
    double* integrated_moments;         /* [S*6*3]    wing-major                                    */
    /* always written */
    double force_sum[3];                /* SimulationResult::integrated_forces_sum  (simulation.rs:61-69) */
    double moment_sum[3];               /* SimulationResult::integrated_moments_sum (simulation.rs:71-79) */
    double residual;                    /* SolverResult.residual                                     */
    int64_t iterations;                 /* SolverResult.iterations                                   */
    int32_t converged;                  /* 1 if a tolerance was met before the iteration cap         */
    int32_t reserved;
} sb_step_output;

/* Message of the last failed call on this thread ("" if none). */
const char* sb_last_error(void);

/* Status code of the last call on this thread that reports one (e.g. why sb_sim_new gave NULL). */
int sb_last_status(void);

/* Library version string. */
const char* sb_version(void);

/*
 * Builds a simulation from a SimulationBuilder JSON string.
 * Replaces Simulation::new_from_string (stormbird/src/lifting_line/simulation.rs:33-39)
 * and cstormbird's new_from_string constructor (complete_sail_model.rs:29-45).
 * Returns NULL on error (sb_last_error() says why). device = CUDA ordinal.
 */
sb_sim* sb_sim_new(const char* setup_json, int device);

/* Frees the handle and all device memory it owns. NULL is accepted. */
void sb_sim_free(sb_sim* sim);

/* Model sizes: span lines N, wings S, freestream points (N + wake points; N in quasi-steady). */
int sb_sim_sizes(const sb_sim* sim, size_t* nr_span_lines, size_t* nr_wings, size_t* nr_freestream_points);

/*
 * Writes the points where do_step needs the freestream: control points, then all wake
 * points (row-major along the span, streamwise-major). Replaces
 * Simulation::get_freestream_velocity_points (simulation.rs:45-63). n = number of points.
 */
int sb_sim_get_freestream_points(const sb_sim* sim, double* points_xyz, size_t n);

/*
 * One time step. freestream_xyz holds n = nr_freestream_points velocities (host memory).
 * Replaces Simulation::do_step (simulation.rs:107-203) and pystormbird's
 * Simulation.do_step (interfaces/pystormbird/src/lifting_line/simulation.rs:131-149).
 */
int sb_sim_do_step(sb_sim* sim, double time, double time_step, const double* freestream_xyz, size_t n,
                   sb_step_output* out);

/*
 * Same as sb_sim_do_step with the freestream already in device memory (n*3 doubles) and
 * no host copy of the output: results stay on the device until sb_sim_read_output.
 * Used by callers that generate the freestream on the GPU.
 */
int sb_sim_do_step_device(sb_sim* sim, double time, double time_step, const double* freestream_xyz_device, size_t n);

/* Copies the output of the last step to host buffers (same layout as sb_sim_do_step). */
int sb_sim_read_output(sb_sim* sim, sb_step_output* out);

/*
 * Induced velocity of the whole dynamic wake at arbitrary points (host arrays, n points).
 * Replaces Simulation::induced_velocities (simulation.rs:207-216); SB_ERR_STATE in
 * quasi-steady mode where the reference panics.
 */
int sb_sim_induced_velocities(sb_sim* sim, const double* points_xyz, size_t n, double* velocities_xyz);

/* Rigid-body motion and wing-angle setters (line_force_model/data_update.rs:171-234). */
int sb_sim_set_translation_and_rotation_with_finite_difference(sb_sim* sim, double time_step,
                                                                const double translation[3], const double rotation[3]);
int sb_sim_set_translation_only(sb_sim* sim, const double translation[3]);
int sb_sim_set_rotation_only(sb_sim* sim, const double rotation[3]);
int sb_sim_set_velocity_linear(sb_sim* sim, const double velocity[3]);
int sb_sim_set_velocity_angular(sb_sim* sim, const double velocity[3]);
int sb_sim_set_local_wing_angles(sb_sim* sim, const double* angles, size_t nr_wings);
/* LineForceModel::local_wing_angles (line_force_model/mod.rs), read back. */
int sb_sim_get_local_wing_angles(const sb_sim* sim, double* angles, size_t nr_wings);

/* previous_circulation_strength (simulation.rs:26): reset to zero, set (warm start) or read. */
int sb_sim_reset_previous_circulation(sb_sim* sim);
int sb_sim_set_previous_circulation(sb_sim* sim, const double* circulation, size_t n);
int sb_sim_get_previous_circulation(const sb_sim* sim, double* circulation, size_t n);

/*
 * Wake state for inspection and tests: points [nr_wake_points*3], strengths [nr_panels],
 * velocity at points [nr_wake_points*3]. Any pointer may be NULL. Sizes come from
 * sb_sim_wake_sizes. SB_ERR_STATE in quasi-steady mode.
 */
int sb_sim_wake_sizes(const sb_sim* sim, size_t* nr_wake_points, size_t* nr_wake_panels, size_t* nr_points_along_span,
                      size_t* nr_panels_per_line_element);
int sb_sim_get_wake_state(sb_sim* sim, double* points_xyz, double* strengths, double* velocities_xyz);

/*
 * The state a step reads from the steps before it, as one f64 array: what the public fields
 * of the reference's Simulation (simulation.rs:20-28: previous_circulation_strength,
 * flow_derivatives, first_time_step_completed) and DynamicWake (wake/dynamic_wake/mod.rs:41-64:
 * points, velocity_at_points, strengths, number_of_time_steps_completed) hold, which Rust code
 * reads and assigns directly (Simulation derives Clone). Layout: [0] wake time steps
 * completed, [1] first time step completed (0/1), [2] flow-derivative updates, then for a
 * dynamic wake the points [nr_wake_points*3], the velocity at the points [nr_wake_points*3]
 * and the panel strengths [nr_wake_panels], then the previous circulation [N] and the two
 * stored control-point velocities of the flow derivatives [2*N*3]. Rigid-body motion and wing
 * angles are not included (their setters above set them). n must equal sb_sim_state_size.
 * A state taken from one simulation and set on another built from the same setup makes its
 * next step compute what the first one's next step would.
 */
int sb_sim_state_size(const sb_sim* sim, size_t* n);
int sb_sim_get_state(sb_sim* sim, double* state, size_t n);
int sb_sim_set_state(sb_sim* sim, const double* state, size_t n);

/*
 * Biot-Savart precision variant used by the Biot-Savart sweeps of this handle:
 * 0 = FP32 with compensated (Kahan) accumulation (default), 1 = plain FP32,
 * 2 = FP64. Kept as a switch for the precision study.
 */
int sb_sim_set_precision(sb_sim* sim, int precision_mode);

/*
 * Timing of the device work of the last step (CUDA events on the handle's stream, ms):
 * [0] whole step, [1] wake update, [2] free-wake sweep at control points (with its
 * reduction), [3] unit-strength matrix, [4] circulation solve, [5] wake roll-up sweep
 * (with its reduction), [6] forces, [7] roll-up sweep kernel alone, [8] control-point
 * sweep kernel alone, [9] wake-point advection kernel, [10] wake panel-record kernel,
 * [11] chain-record kernel (shared-segment roll-up; 0 when the step built none); n <= 12.
 * Only filled when enabled with sb_sim_enable_timing(sim, 1).
 */
int sb_sim_enable_timing(sb_sim* sim, int enable);
int sb_sim_last_step_timing(const sb_sim* sim, double* ms, size_t n);

/*
 * Sizes of the last step's Biot-Savart sweeps: [0] roll-up target points, [1] panels
 * swept for the roll-up, [2] control points, [3] free-wake panels swept at the control
 * points, [4] steps completed, [5] kernels launched by the step, [6] vortex segments
 * evaluated per roll-up target (4 per panel, or fewer with shared segments). Zero-strength
 * panels are included in the panel counts (the sweeps skip them).
 */
int sb_sim_last_step_counters(const sb_sim* sim, double* counters, size_t n);

/*
 * Shared-segment roll-up (default on). In a wake where every panel pair is near-field
 * (far_field_ratio >= 1e15) and all panels have one core length, each wake segment lies on
 * two adjacent vortex rings with opposite directions; as the segment velocity of
 * vortex_line.rs:18-106 is antisymmetric in its end points, the roll-up sweep evaluates each
 * segment once with the difference of the two strengths (about half the evaluations of
 * four segments per ring). The sum is the reference's, rounded differently. Active only in
 * the FP32 modes; the control-point sweep and sb_sim_induced_velocities keep the rings.
 */
int sb_sim_set_segment_sharing(sb_sim* sim, int enable);

/*
 * Freestream from a wind model, generated on the GPU: the reference's
 * CompleteSailModel::freestream_velocity (complete_sail_model/mod.rs:213-257) with a
 * WindEnvironment (wind/environment.rs:21-55) and a WindCondition
 * (wind/wind_condition/mod.rs:19-39) given as JSON, the ship moving at `ship_velocity`
 * along the environment's zero direction. sb_sim_do_step_wind is sb_sim_do_step with that
 * freestream, so no freestream crosses the host boundary; sb_sim_wind_freestream writes it
 * (all freestream points, host buffer of n = nr_freestream_points) for inspection.
 */
int sb_sim_set_wind(sb_sim* sim, const char* environment_json, const char* condition_json);
int sb_sim_wind_freestream(sb_sim* sim, double time, double ship_velocity, double* freestream_xyz, size_t n);
int sb_sim_do_step_wind(sb_sim* sim, double time, double time_step, double ship_velocity, sb_step_output* out);

/*
 * Result output in the reference's formats (stormbird/src/common_utils/results/simulation.rs).
 * sb_sim_result_json: the last step's SimulationResult as serde writes it (write_to_file,
 * simulation.rs:91-98); *length = bytes needed including the terminating NUL (SB_ERR_SIZE
 * when capacity is smaller). sb_sim_result_csv: the reduced flattened header and data row
 * (as_reduced_flatten_csv_string, simulation.rs:168-205). "Last step" = the last
 * sb_sim_do_step / sb_sim_do_step_wind, or the step sb_sim_read_output copied.
 * sb_sim_set_result_file: from the next step on, every sb_sim_do_step / sb_sim_do_step_wind
 * result goes to `path`, formatted and written on a background thread from a host copy:
 * SB_RESULTS_JSON_HISTORY writes a JSON array of SimulationResult (the file
 * result_history_from_file reads, simulation.rs:37-45), closed when the writer is replaced
 * or the handle freed; SB_RESULTS_CSV appends one reduced row per step, with the header first
 * when the file is new (io_utils/csv_data.rs:11-33). NULL or SB_RESULTS_OFF stops writing.
 * sb_sim_flush_results waits until every queued step is written, including the wake files
 * a dynamic setup asks for with write_wake_data_to_file (one VTK PolyData file
 * `{wake_files_folder_path}/wake_{time / time_step}.vtp` per step, as
 * lifting_line/wake/dynamic_wake/export.rs:75-163 writes it, also on a background thread).
 */
#define SB_RESULTS_OFF 0
#define SB_RESULTS_JSON_HISTORY 1
#define SB_RESULTS_CSV 2
int sb_sim_result_json(const sb_sim* sim, char* buffer, size_t capacity, size_t* length);
int sb_sim_result_csv(const sb_sim* sim, char* header, size_t header_capacity, char* data, size_t data_capacity);
int sb_sim_set_result_file(sb_sim* sim, const char* path, int format);
int sb_sim_flush_results(sb_sim* sim);
/* 1 if the roll-up sweep of this simulation uses shared segments in its current mode. */
int sb_sim_segment_sharing_active(const sb_sim* sim, int* active);

/*
 * Standalone Biot-Savart sweep over caller-given vortex-ring panels: the velocity that
 * n_panels unit rings (corners [n_panels*12], four corners in ring order), scaled by their
 * strengths [n_panels], with viscous core lengths [n_panels] and the far-field ratio of the
 * point-doublet approximation, induce at n_targets points [n_targets*3], written to
 * velocities [n_targets*3]. It is the computation DynamicWake::induced_velocities runs over
 * its own panels (stormbird/src/lifting_line/wake/dynamic_wake/induced_velocity_calc.rs:18-26,
 * singularity_elements/panel.rs:26-118, symmetry_condition.rs:27-43), offered on caller data.
 * symmetry: 0 none, 1 X, 2 Y, 3 Z. precision as in sb_sim_set_precision. Host arrays; the
 * device work space is allocated (stream-ordered) and freed on every call.
 */
int sb_panel_sweep(int device, const double* corners, const double* strengths, const double* core_lengths,
                   size_t n_panels, double far_field_ratio, int symmetry, const double* targets, size_t n_targets,
                   int precision, double* velocities);

/*
 * The standalone sweep without any device allocation, for callers that may not allocate
 * device memory while they run: a co-simulation master stepping the lifting line in real
 * time (as the FMU's do_step is called), where allocating after initialisation is
 * forbidden, or a host framework whose memory pool owns the whole GPU. Not a counterpart
 * of any reference function: it is sb_panel_sweep (FP32, compensated) with every pointer
 * in device memory the caller owns — corners [n_panels*12], strengths and core lengths
 * [n_panels], targets and velocities [n_targets*3], f64 — and the sweep's scratch (panel
 * records, partial sums, work counter, error word: 7 MiB + 256 B) in one fixed device array
 * that each GPU loading the library holds until the process exits. At most
 * SB_NO_ALLOC_MAX_PANELS panels and SB_NO_ALLOC_MAX_TARGETS targets per call (larger
 * sizes: SB_ERR_SIZE). Work is enqueued on `stream` (a cudaStream_t, NULL = the legacy
 * default stream) and the call returns when it has finished; the caller's current device is
 * the same after the call as before it. The first call on a device (and the first after
 * that device's context has been reset) resolves the array's device address. No call may
 * be made while a stream is being captured: every call reads the error word back into host
 * memory and synchronises `stream` before it returns. Every call shares the array: calls
 * that overlap on the GPU race and must be serialised.
 */
#define SB_NO_ALLOC_MAX_PANELS 16384
#define SB_NO_ALLOC_MAX_TARGETS 65536
int sb_panel_sweep_no_alloc(int device, const double* corners, const double* strengths, const double* core_lengths,
                            size_t n_panels, double far_field_ratio, int symmetry, const double* targets,
                            size_t n_targets, double* velocities, void* stream);

/*
 * Measured FP32 FMA throughput of a device in TFLOP/s (best of `reps` timed launches of
 * an FMA-chain kernel): the denominator of the Biot-Savart sweep's roofline. Diagnostic
 * entry point with no counterpart in the reference.
 */
int sb_measure_fp32_peak(int device, int reps, double* tflops);
/* The same for FP64 FMAs (the denominator of the FP64 sweep of the precision study). */
int sb_measure_fp64_peak(int device, int reps, double* tflops);

/*
 * Failure path of the bounded device-side waits (diagnostics with no counterpart in the
 * reference, whose CPU loops have no waits). Every wait of a kernel on an asynchronous copy
 * polls a bounded number of times; when it runs out the kernel records the timeout, waits
 * (bounded again) for its copies still in flight, leaves, and the call returns
 * SB_ERR_TIMEOUT with the device context still usable.
 * sb_set_sweep_wait_polls: polls of each tile wait of the Biot-Savart sweeps launched after
 * it, process-wide (0: every sweep's first wait runs out at once; < 0 restores the default,
 * 2^22). sb_wait_timeout_self_test: one CTA waits, with `polls` polls, on an mbarrier armed
 * for bytes no copy delivers; returns SB_ERR_TIMEOUT when the wait ran out and the kernel
 * returned (the expected outcome).
 */
int sb_set_sweep_wait_polls(int polls);
int sb_wait_timeout_self_test(int device, int polls);

/* ===================================================================================
 * Batched cases. The reference runs independent cases (apparent-wind sweeps, differing
 * sail counts and wake lengths) as separate `Simulation`s, one `do_step` each
 * (simulation.rs:107-203; CompleteSailModel loops over them,
 * complete_sail_model/mod.rs:187-191). A batch steps many such cases together: each case
 * is built from its own setup JSON exactly as by sb_sim_new and computes what its own
 * Simulation::do_step would, but the Biot-Savart sweeps of all cases run as one persistent
 * launch per sweep kind and the steady step is replayed as a CUDA graph.
 * =================================================================================== */
typedef struct sb_batch sb_batch;

/* Per-case summary after a step: force sum [3], moment sum [3], residual, iterations,
 * converged (0/1), device status word (0 = ok), start of the solve (0 = the plain start,
 * 1 = the solution extrapolated in time, 2 = extrapolation plus the network's correction:
 * the one with the lowest residual; -1 = no warm start). */
#define SB_BATCH_SUMMARY 11
/* sb_batch_info fields: last step ms, panel-target pairs swept in the last step, tuning
 * waves, tuning CTAs per SM (0 = occupancy limit), roll-up grid, roll-up work items,
 * tuned (0/1), candidates timed, best tuned roll-up ms, graph in use (0/1), steps done,
 * panels per shared-memory stage of the compensated panel sweeps, item schedule (0 the
 * costliest case's items first, 1 case order). */
#define SB_BATCH_INFO 13

/* n_cases setup JSON strings (as sb_sim_new). NULL on error (sb_last_error names the case). */
sb_batch* sb_batch_new(const char* const* setup_jsons, size_t n_cases, int device);
void sb_batch_free(sb_batch* batch);
/* Number of cases, total span lines (sum of N) and total freestream points (sum of nfs). */
int sb_batch_sizes(const sb_batch* batch, size_t* n_cases, size_t* total_lines, size_t* total_freestream);
/* Sizes of case i and the offsets of its lines / freestream points in the batch's arrays. */
int sb_batch_case_sizes(const sb_batch* batch, size_t i, size_t* n_lines, size_t* n_wings, size_t* n_freestream,
                        size_t* line_offset, size_t* freestream_offset);
/* Freestream points of all cases, case after case (each as sb_sim_get_freestream_points). */
int sb_batch_get_freestream_points(sb_batch* batch, double* points_xyz, size_t n_total);
/* One step of every case: freestream [total_freestream*3], case after case. */
int sb_batch_do_step(sb_batch* batch, double time, double time_step, const double* freestream_xyz, size_t n_total);
int sb_batch_do_step_device(sb_batch* batch, double time, double time_step, const double* freestream_dev,
                            size_t n_total);
/* Wind models for all cases (one environment, one WindCondition JSON per case; see
 * sb_sim_set_wind) and a step with every case's freestream generated on the GPU: the
 * batched form of CompleteSailModel::do_step (complete_sail_model/mod.rs:187-199) over a
 * sweep of wind conditions, ship_velocities [n_cases]. */
int sb_batch_set_wind(sb_batch* batch, const char* environment_json, const char* const* condition_jsons);
int sb_batch_do_step_wind(sb_batch* batch, double time, double time_step, const double* ship_velocities);
/* Results of the last step: circulation [total_lines] and summaries [n_cases*SB_BATCH_SUMMARY]. */
int sb_batch_get_circulation(const sb_batch* batch, double* circulation, size_t n_total);
int sb_batch_get_summary(const sb_batch* batch, double* summary, size_t n);
/* Full output block of case i for the last step (as sb_sim_read_output). */
int sb_batch_read_case_output(sb_batch* batch, size_t i, sb_step_output* out);
/* State of case i after the last step, in the layout of sb_sim_get_state (n = its size), and
 * the same to load a state into case i (a batch of the same setups can so start where
 * another stopped; the cases of a batch step together, so load every case's state). A loaded
 * case's warm-start history (previous freestream and solution) starts empty: its candidates
 * wait for two steps of this batch. */
int sb_batch_case_state_size(const sb_batch* batch, size_t i, size_t* n);
int sb_batch_get_case_state(sb_batch* batch, size_t i, double* state, size_t n);
int sb_batch_set_case_state(sb_batch* batch, size_t i, const double* state, size_t n);
/* Initial solution of the next step's solve for every case (the reference's
 * previous_circulation_strength, simulation.rs:165,189): the warm-start hook. */
int sb_batch_set_initial_circulation(sb_batch* batch, const double* circulation, size_t n_total);
int sb_batch_set_initial_circulation_device(sb_batch* batch, const double* circulation_dev, size_t n_total);
/* Device address of the batch's previous-circulation array [total_lines] (read/write). */
int sb_batch_previous_circulation_device(sb_batch* batch, double** circulation_dev);
/* Sweep precision of every case: 0 FP32 compensated (default), 1 FP32, 2 FP64. */
int sb_batch_set_precision(sb_batch* batch, int mode);
/* CUDA-graph replay of the steady step (default on). */
int sb_batch_use_graph(sb_batch* batch, int enable);
/* Times the roll-up sweep of the current state for each candidate within about
 * budget_seconds and keeps the fastest for this batch and for later batches of the same
 * workload bucket in this process: first the tile shape (panels per shared-memory stage of
 * the compensated panel sweeps: 64, 32, 96), then items per persistent CTA x CTAs per SM,
 * then the item schedule (costliest case first, or case order). Needs a batch whose
 * roll-up has started. */
int sb_batch_autotune(sb_batch* batch, double budget_seconds);
int sb_batch_info(const sb_batch* batch, double* info, size_t n);

/* ===================================================================================
 * Learned warm start. No counterpart in the reference, which starts every solve from the
 * previous step's circulation (simulation.rs:165,189; simple_iterative.rs:86-101). A network
 * (4 hidden layers of 256, GELU, BF16 weights on the tensor cores with FP32 accumulation)
 * predicts, per panel, a correction to the solution extrapolated linearly in time, from
 * per-panel features the batch builds on the GPU. The SimpleIterative solve evaluates the
 * residual of the plain start, of the extrapolation and of extrapolation plus correction
 * and starts from the lowest, so the solver alone decides the result; the batch
 * reports per case which start was taken.
 * =================================================================================== */
typedef struct sb_mlp sb_mlp;
/* Number of per-panel features the batch builds (the network's input size for mode 1). */
#define SB_WARM_START_FEATURES 16
/* A network with n_inputs (1..64) inputs, He-uniform weights from `seed`. */
sb_mlp* sb_mlp_new(int device, int n_inputs, unsigned long long seed);
void sb_mlp_free(sb_mlp* network);
int sb_mlp_num_params(const sb_mlp* network, size_t* n);
/* Parameters (FP32 master copy) in the order W1 [256][64], b1, W2 [256][256], b2, W3, b3,
 * W4, b4, w_out [256], b_out. */
int sb_mlp_get_params(sb_mlp* network, float* params, size_t n);
int sb_mlp_set_params(sb_mlp* network, const float* params, size_t n);
/* y [rows] = network(x [rows][n_inputs]); device pointers. */
int sb_mlp_forward(sb_mlp* network, const float* x_dev, size_t rows, float* y_dev);
/* Mean-squared-error loss and its gradient (host buffer [num_params]) on device data. */
int sb_mlp_gradients(sb_mlp* network, const float* x_dev, const float* target_dev, size_t rows, float* grads,
                     double* loss);
/* One Adam step (beta 0.9 / 0.999) on device data; `loss` (may be NULL) gets the batch's
 * loss before the update. */
int sb_mlp_train_step(sb_mlp* network, const float* x_dev, const float* target_dev, size_t rows, float learning_rate,
                      double* loss);
/* Warm start of a batch: mode 0 off, 1 the network's candidates (SimpleIterative cases),
 * 2 features and targets recorded each step without a candidate (training data). */
int sb_batch_set_warm_start(sb_batch* batch, sb_mlp* network, int mode);
/* Guard on the network's start (mode 1): each case's solve starts from the plain start, the
 * extrapolation in time if its mean and largest per-line residual are both lower, and the
 * network's candidate only if both of its residuals are below `margin` times the best start's
 * (0 < margin <= 1; default 0.5). */
int sb_batch_set_warm_start_guard(sb_batch* batch, double margin);
/* The last step's features [total_lines][SB_WARM_START_FEATURES] and targets [total_lines]
 * (device or host pointers; either may be NULL). */
int sb_batch_copy_warm_start_data(sb_batch* batch, float* features, float* targets, size_t rows);

/* ---------------------------------------------------------------------------------------
 * CompleteSailModel: a lifting-line simulation with a wind environment and a sail
 * controller (stormbird/src/lifting_line/complete_sail_model/mod.rs), JSON schema
 * CompleteSailModelBuilder {lifting_line_simulation, wind_environment, controller}
 * (complete_sail_model/builder.rs:19-24). The C functions replace cstormbird's
 * complete_sail_model_* (interfaces/cstormbird/src/lifting_line/complete_sail_model.rs).
 * ------------------------------------------------------------------------------------- */
typedef struct sb_csm sb_csm;

/* cstormbird WindCondition (interfaces/cstormbird/src/wind.rs:9-13): a power-law profile
 * with this velocity at 10 m and factor 1/9, coming from this direction (radians). */
typedef struct sb_wind_condition {
    double velocity;
    double direction_coming_from;
} sb_wind_condition;

/* cstormbird SingleSailResult (interfaces/cstormbird/src/results.rs:5-10): per sail the
 * total integrated force and moment and the input power. */
typedef struct sb_single_sail_result {
    double force[3];
    double moment[3];
    double input_power;
} sb_single_sail_result;

/* complete_sail_model_new (complete_sail_model.rs:26-43): NULL on error (sb_last_error). */
sb_csm* sb_csm_new(const char* setup_json, int device);
/* complete_sail_model_drop (complete_sail_model.rs:61-67) */
void sb_csm_free(sb_csm* model);
/* complete_sail_model_get_number_of_sails (complete_sail_model.rs:46-58): -1 on NULL. */
int sb_csm_get_number_of_sails(const sb_csm* model);
/* complete_sail_model_simulate_steady_state_condition (complete_sail_model.rs:69-110): the
 * controller applied for the condition, then one step at time 0 with time step 1; writes
 * min(sails, results_out_length) results and returns that count; -1 NULL, -2 zero length. */
int sb_csm_simulate_steady_state_condition(sb_csm* model, sb_wind_condition wind_condition, double ship_velocity,
                                           double controller_loading, sb_single_sail_result* results_out,
                                           size_t results_out_length);
/* CompleteSailModel::apply_controller_based_on_wind_condition (mod.rs:190-212) and ::do_step
 * (mod.rs:170-188) with a WindCondition JSON document (wind_condition/mod.rs:19-39). */
int sb_csm_apply_controller(sb_csm* model, double time, double time_step, const char* condition_json,
                            double ship_velocity, double controller_loading);
int sb_csm_do_step(sb_csm* model, double time, double time_step, const char* condition_json, double ship_velocity,
                   sb_step_output* out);
/* The model's lifting-line simulation (owned by the model): wing angles, motion, sizes. */
int sb_csm_sim(sb_csm* model, sb_sim** sim);
/* n steady-state conditions in one batched pass, each on its own replica of the model that
 * starts from the model's current wing angles and motion (the model itself is unchanged);
 * results_out [n_conditions][sails], results_out_length = n_conditions x sails. A replica
 * keeps its own previous solution and velocity history between sweeps of the same size. */
int sb_csm_sweep_steady_state(sb_csm* model, const sb_wind_condition* wind_conditions, const double* ship_velocities,
                              const double* controller_loadings, size_t n_conditions, sb_single_sail_result* results_out,
                              size_t results_out_length);
/* CompleteSailModel::simulate_condition_optimal_controller_loading (mod.rs:60-101): the
 * loadings linspace(0.1, 1, n) as one sweep; the sails' results of the loading with the
 * largest -F_x * ship_velocity - input power (first maximum), and that loading. */
int sb_csm_simulate_condition_optimal_controller_loading(sb_csm* model, sb_wind_condition wind_condition,
                                                         double ship_velocity, size_t nr_loadings_to_test,
                                                         sb_single_sail_result* results_out, size_t results_out_length,
                                                         double* best_loading);

#ifdef __cplusplus
}
#endif

#endif /* STORMBIRD_GB300_H */
