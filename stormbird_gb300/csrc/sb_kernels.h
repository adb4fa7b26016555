// Launch interfaces of the lifting-line kernels (host side). Each .cu file holds its
// kernels and the host launchers declared here, so no relocatable device code is needed.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "sb_device.cuh"

namespace sbgpu {

constexpr int kBsThreads = 128;  // threads per Biot-Savart CTA
constexpr int kMaxTargetGroups = 8;  // wings of a sweep's target order (BsJob::group_off)

// One Biot-Savart sweep: velocities at M targets induced by panels [p_begin, p_end).
// Its work items are (source chunk, target tile) pairs, chunk-major.
struct BsJob {
    const void* panels = nullptr;      // PanelRec<float> or PanelRec<double>
    long long p_begin = 0, p_end = 0;
    const d3* targets = nullptr;       // [M] f64 positions
    const int* target_wing = nullptr;  // [M] wing index (neglect-self variant only)
    long long M = 0;
    int chunk_panels = 0;              // panels per source chunk (multiple of the tile)
    int n_chunks = 1;
    long long n_ttiles = 0;            // target tiles of kBsThreads * T targets
    double* partial = nullptr;         // [n_chunks][M][3]
    long long item_begin = 0;          // first item of this sweep in a batched launch
    // reduction (batched launches): out[i] = base[i] + sum over chunks, base only for i >= M
    long long M_total = 0;
    const d3* base = nullptr;
    d3* out = nullptr;
    long long block_begin = 0;         // first block of this sweep in the batched reduce
    // Order in which the FP32 far-field sweeps take their targets (sweeps over wake points):
    // rows of row_pts points, each row made of n_groups groups (one wing's span points)
    // starting at point group_off[g] (group_off[n_groups] = row_pts). Target slot s runs
    // through the groups one after another and within a group through the rows, so that a
    // warp's 64 targets are one wing's points on adjacent rows (a compact box) rather than a
    // stretch of a row across two wings. slots = rows x row_pts >= M (a slot whose point is
    // M or beyond is empty). n_groups == 0: slot s is target s; slots == 0: M slots.
    long long slots = 0;
    int row_pts = 0, n_groups = 0;
    int group_off[kMaxTargetGroups + 1] = {};
};

// Target index of slot s (see BsJob::slots).
__host__ __device__ inline long long bs_slot_target(const BsJob& J, long long s) {
    if (J.n_groups == 0) return s;
    const long long R = J.slots / J.row_pts;
    int g = 0;
    while (g + 1 < J.n_groups && s >= R * J.group_off[g + 1]) ++g;
    const int off = J.group_off[g], n = J.group_off[g + 1] - off;
    const long long t = s - R * off;
    const long long r = t / n;
    return r * J.row_pts + off + (t - r * n);
}
__host__ __device__ inline long long bs_slots(const BsJob& J) { return J.slots > 0 ? J.slots : J.M; }

// A sweep launch: one job (job0, jobs == nullptr) or a list of jobs in device memory
// whose items are handed out in list order (the batch puts the costliest items first).
// The list ends with a sentinel entry whose item_begin is the number of items of all jobs.
struct BsArgs {
    BsJob job0;
    const BsJob* jobs = nullptr;       // [n_jobs + 1] device memory
    int n_jobs = 0;
    unsigned long long* work_counter = nullptr;  // zero before launch
    int* err = nullptr;
    int symmetry = 0;
    int neglect = 0;
    int chain = 0;  // the sources are chain records (FP32 only, no neglect-self)
    int wait_polls = kWaitPolls;  // polls of each bounded wait on a tile copy
    int tile = 0;  // panels per shared-memory stage (0: the precision's default; see bs_tile_panels)
};

// Polls of the bounded tile waits of later sweep launches (launch_bs_sweep overrides
// BsArgs::wait_polls with it when >= 0; < 0 = each launch's own value). Process-wide;
// exists so that a test can make the waits run out.
void set_sweep_wait_polls(int polls);
// One CTA waiting, with `polls` polls, on an mbarrier that expects bytes no copy delivers:
// the wait runs out, *err gets kDevTimeout and the kernel returns (k_probe.cu).
cudaError_t launch_wait_probe(int polls, int* err, cudaStream_t s);

constexpr int kBsReduceThreads = 256;

int bs_targets_per_thread(int symmetry);
int bs_tile_panels(int precision);
// Panels per stage a launch with BsArgs::tile = `tile` uses: the tuned shape where a variant
// exists (compensated FP32, no symmetry, panel records), else the default.
int bs_tile_panels(int precision, int symmetry, int chain, int tile);
// The tile shapes the autotuner may try (the default first); returns how many were written.
int bs_tile_choices(int* tiles, int n);
int bs_occupancy_blocks_per_sm(int precision, int symmetry, int neglect, int tile = 0);
cudaError_t launch_bs_sweep(const BsArgs& a, int precision, int grid, cudaStream_t s);
cudaError_t launch_bs_reduce(const double* partial, int n_chunks, long long M, long long M_total, const d3* base, d3* out,
                             cudaStream_t s);
// Reduction of every job of a batched sweep; blocks = sum over jobs of
// ceil(M_total / kBsReduceThreads), job k starting at its block_begin.
cudaError_t launch_bs_reduce_jobs(const BsJob* jobs, int n_jobs, long long blocks, cudaStream_t s);
// The influence matrices are written in f64 (`factors`, [N][N] d3, for the Linearized
// solver) and/or as f32 (hi, lo) pairs (`split`: the hi plane [N][3][si_matrix_stride(N)]
// floats, row c, component, column, then the lo plane; hi = the nearest float, lo = the
// nearest float of the remainder, for the SimpleIterative solver's matrix-vector products;
// the padding columns are left untouched). Either pointer may be null.
// Frozen-wake unit matrix of the first wake row: from the FP32 row-0 records when row0_32 is
// given (k_unit_matrix_f32; the control point's own panel in FP64), else all in FP64.
// basis: the rows' in-plane bases (DevModel::solve_basis) for a two-component split matrix,
// or nullptr for three components.
cudaError_t launch_unit_matrix(const PanelRec<double>* row0, const PanelRec<float>* row0_32, const d3* ctrl, int N,
                               int sym, int neglect, const int* wing_of_line, d3* factors, float* split, const d3* basis,
                               cudaStream_t s);
// Quasi-steady horseshoe matrix; core_kind 0 relative, 1 absolute, 2 none.
cudaError_t launch_horseshoe_matrix(const DevModel& m, int core_kind, double core_value, double wake_length, d3* wake_vec,
                                    double* rc_dev, int sym, d3* factors, float* split, const d3* basis,
                                    cudaStream_t s);

// ---- wake and geometry (k_wake.cu) ------------------------------------------------------
struct WakeBuffers {
    d3* pts_old = nullptr;   // [Wp][Np]
    d3* pts_new = nullptr;   // [Wp][Np]
    d3* vel = nullptr;       // [Wp][Np] velocity at the (old) points
    double* str_old = nullptr;  // [W][N]
    double* str_new = nullptr;  // [W][N]
    PanelRec<float>* rec32 = nullptr;    // [W][N]
    PanelRec<double>* rec64 = nullptr;   // [W][N] (FP64 precision mode) or nullptr
    PanelRec<double>* row0_64 = nullptr; // [N]
};

// Global geometry and felt velocities of the line force model for one step
// (line_force_model/data_update.rs:13-90, force_calculations.rs:50-69, value_mapping.rs:87-137).
// When mean_out is not null, also writes the mean control-point freestream (simulation.rs:74-75).
cudaError_t launch_prep_geometry(const DevModel& m, const StepParams& p, const d3* freestream_ctrl, d3* mean_out,
                                 cudaStream_t s);

// Wake initialisation with a uniform velocity (dynamic_wake/initialization.rs:12-41).
// `velocity` is read from device memory (mean_dev) when not null, else `velocity_host`.
// fill_rows = 1 first puts every row on the span points (the builder's state).
cudaError_t launch_wake_init(const DevModel& m, const WakeBuffers& w, const d3* mean_dev, d3 velocity_host, double dt,
                             int fill_rows, cudaStream_t s);

// Wake points before solving (update_data.rs:65-82, 90-99, 152-316) into pts_new.
cudaError_t launch_wake_advect(const DevModel& m, const WakeBuffers& w, double dt, int steps_completed, cudaStream_t s);

// Panels of the new points and downstream strength shift (update_data.rs:102-115, 319-328).
// `shift_strengths` = 0 rebuilds the panels without moving strengths (initialisation).
cudaError_t launch_wake_panels(const DevModel& m, const WakeBuffers& w, int shift_strengths, cudaStream_t s);

// Chain records of a wake whose panels all share one core length (kChain* layout in
// sb_device.cuh), ordered in quads of point rows: quad q holds the spanwise chains of point
// rows 4q..4q+3 (SP chains per row, up to 4 lines of one wing each), then the streamwise
// chains of panel rows 4q..4q+3 (one per point column). Records past the wake's last row are
// written empty. Only the first n_build records are written.
struct ChainArgs {
    const d3* pts = nullptr;        // [W+1][Np] wake points
    const double* str = nullptr;    // [W][N] strengths (row 0: this step's solution)
    const int* span_tab = nullptr;  // [SP][3]: wing, first line, number of lines (<= 4)
    const int* col_tab = nullptr;   // [Np][2]: wing, point number j (column = j + wing)
    const int* wing_start = nullptr;
    const int* wing_end = nullptr;
    int W = 0, N = 0, Np = 0, SP = 0;
    long long Bq = 0;               // records per quad: 4 SP + Np
    double rc = 0.0;                // the common core length
    PanelRec<float>* out = nullptr;
};
cudaError_t launch_chain_records(const ChainArgs& a, long long n_build, cudaStream_t s);

// One dynamic case of a batched step, for the per-case kernels that a batch runs as ONE
// launch per kind for all its cases (geometry, wake advection, panel records, unit-strength
// matrix, chain records): the case's model, step parameters and wake buffers of the step,
// and the first block of each kind that belongs to it (ascending over the job list).
struct CaseStepJob {
    DevModel m;
    StepParams p;                             // p.dt: the step's time step
    WakeBuffers w;                            // old -> new buffers of the step
    const d3* fs_ctrl = nullptr;              // freestream at the control points
    int steps_done = 0;                       // wake steps completed before the step
    const PanelRec<float>* row0_32 = nullptr; // unit matrix from FP32 row-0 records (null: FP64)
    d3* factors = nullptr;
    float* split = nullptr;
    const d3* basis = nullptr;                // two-component split matrix (nullptr: three)
    ChainArgs chain;                          // chain records (chain_n = 0: none)
    long long chain_n = 0;
    long long blk_advect = 0, blk_panels = 0, blk_matrix = 0, blk_chain = 0;
};
// Blocks a job needs per kind.
long long wake_advect_blocks(const DevModel& m);
long long wake_panels_blocks(const DevModel& m);
long long chain_records_blocks(long long n_build);
long long unit_matrix_blocks(int N, bool fp32);
// One CTA per job: the geometry of every case (k_prep_geometry).
cudaError_t launch_prep_geometry_jobs(const CaseStepJob* jobs, int n, cudaStream_t s);
// Wake advection (with the last row) of every case, then its panel records with the strength
// shift (k_wake_advect, k_wake_panels).
cudaError_t launch_wake_jobs(const CaseStepJob* jobs, int n, long long advect_blocks, long long panel_blocks,
                             cudaStream_t s);
cudaError_t launch_unit_matrix_jobs(const CaseStepJob* jobs, int n, long long blocks, cudaStream_t s);
cudaError_t launch_chain_records_jobs(const CaseStepJob* jobs, int n, long long blocks, cudaStream_t s);

// Records of caller-given panels for the standalone sweep (corners [P][4][3] in ring order).
cudaError_t launch_panels_from_corners(const double* corners, const double* strengths, const double* cores, long long P,
                                       double far_field_ratio, PanelRec<float>* r32, PanelRec<double>* r64,
                                       cudaStream_t s);

// ---- solver and forces (k_solve.cu) ----------------------------------------------------
struct SolveSettings {
    int max_iterations = 40;
    double damping = 0.05;
    double residual_tolerance = 1e-4;
    double strength_tolerance = 1e-6;
    int velocity_correction = 0;  // 0 none, 1 max induced ratio, 2 fixed magnitude
    double velocity_correction_ratio = 0.0;
    double correction_factor_initial = 1.0;
    int start_with_linearized = 0;
    // Linearized
    int disable_viscous_corrections = 0;
    int full_induced_correction = 1;
};

// Row length of the SimpleIterative matrix planes: N rounded up to a multiple of 4, so that a
// row's entries load as 16-byte vectors (the padding entries are zero).
__host__ __device__ inline int si_matrix_stride(int N) { return (N + 3) & ~3; }

struct SolveBuffers {
    const d3* fixed = nullptr;      // [N]
    const d3* factors = nullptr;    // [N][N] (Linearized)
    // SimpleIterative matrix as floats: hi plane [N][split_comps][stride] (row, component, column;
    // stride = si_matrix_stride(N)), then the lo plane (the nearest float of the remainder);
    // split_full = 0 when only the diagonal carries lo parts (the FP32 unit matrix: every
    // other entry is an FP32 value, lo = 0)
    const float* factors_split = nullptr;
    int split_full = 1;
    // components per entry: 2 in the rows' in-plane bases (basis, [2N]: the velocity's span
    // component is projected out anyway; no velocity correction), else 3 (x, y, z)
    int split_comps = 3;
    const d3* basis = nullptr;
    double* gamma_prev = nullptr;   // [N] in: initial solution, out: solution
    d3* vel_out = nullptr;          // [N] output control-point velocity
    double* scalars = nullptr;      // [8]: residual, iterations, converged, singular, start (below)
    double* lin_work = nullptr;     // [N*(N+1)] Gaussian elimination scratch (linearized)
    double* wake_str_row0 = nullptr;        // strengths row 0 (dynamic) or nullptr
    PanelRec<float>* rec32_row0 = nullptr;  // FP32 record row 0 (dynamic) or nullptr
    PanelRec<double>* rec64_row0 = nullptr; // FP64 record row 0 in the FP64 sweep mode
    // Optional further initial solutions (predicted warm starts). The solve evaluates the
    // residual of the plain start and of each candidate and starts from the lowest one;
    // scalars[4] = k + 1 when candidate k was taken, 0 when the plain start was (fallback),
    // -1 without candidates.
    const double* candidate[2] = {nullptr, nullptr};  // [N] each, or nullptr
    // factor the second candidate's mean and largest residual must stay under, times the
    // best start's before it (the warm-start guard, see si_solve)
    double second_margin = 0.5;
    int* err = nullptr;
};

int solve_cluster_size(int N);
cudaError_t launch_solve_simple_iterative(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, cudaStream_t s);
cudaError_t launch_solve_linearized(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, cudaStream_t s);

// One solve of a batch (k_solve_lin_jobs, k_solve_lin_cluster_jobs, k_solve_si_jobs).
struct SolveJob {
    DevModel m;
    SolveSettings st;
    SolveBuffers b;
};
// How a linearized solve of N span lines runs. cluster == 1: one CTA, its matrix in shared
// memory when matrix and vectors fit under kLinSmemLimit, else in SolveBuffers::lin_work;
// cluster > 1: a thread-block cluster of that many CTAs with the rows spread over their
// shared memory. smem = dynamic shared memory per CTA.
constexpr size_t kLinSmemLimit = 227 * 1024 - 1024;
struct LinPlan {
    int cluster = 1;
    size_t smem = 0;
};
LinPlan linearized_plan(int N);
// n solves of one plan shape in one launch (smem: the largest of the jobs' plans).
cudaError_t launch_solve_linearized_jobs(const SolveJob* jobs, int n, const LinPlan& plan, cudaStream_t s);
// SimpleIterative solves of a batch: n cases of one cluster size (solve_cluster_size of
// their N) in one launch, a cluster per case; smem = the largest si_smem_bytes of the jobs.
// full: the matrix's lo plane is read (SolveBuffers::split_full); comps: SolveBuffers::split_comps
size_t si_smem_bytes(int N, int full, int comps);
int si_rows_per_thread(int N);  // 1 or 4: a launch holds one kind (rows_per_thread below)
cudaError_t launch_solve_simple_iterative_jobs(const SolveJob* jobs, int n, int cluster, int rows_per_thread,
                                               size_t smem, cudaStream_t s);

struct ForceArgs {
    const double* gamma = nullptr;  // [N]
    const d3* vel = nullptr;        // [N] solver output velocity
    d3* hist0 = nullptr;            // [N] flow derivative history
    d3* hist1 = nullptr;
    int fd_count = 0;               // updates done so far
    double* out = nullptr;          // output block
    const double* scalars = nullptr;
};

// Output block layout (doubles), N span lines, S wings.
struct OutLayout {
    long long gamma, vel, felt, aoa, fvel, acc, ctrl, sect, intf, intm, fsum, msum, residual, iterations, converged,
        total;
    __host__ __device__ static OutLayout make(int N, int S) {
        OutLayout o{};
        long long at = 0;
        o.gamma = at; at += N;
        o.vel = at; at += 3LL * N;
        o.felt = at; at += 3LL * N;
        o.aoa = at; at += N;
        o.fvel = at; at += 3LL * N;
        o.acc = at; at += 3LL * N;
        o.ctrl = at; at += 3LL * N;
        o.sect = at; at += 18LL * N;
        o.intf = at; at += 18LL * S;
        o.intm = at; at += 18LL * S;
        o.fsum = at; at += 3;
        o.msum = at; at += 3;
        o.residual = at; at += 1;
        o.iterations = at; at += 1;
        o.converged = at; at += 1;
        o.total = at;
        return o;
    }
};

// ---- freestream from a wind model (k_wind.cu) -----------------------------------------
// A WindEnvironment + WindCondition in device form. Spectra: for gust k (parallel,
// perpendicular, vertical) spectra[spec_off[k] ...] holds frequencies, amplitudes and
// phases (spec_n[k] each; spec_n[k] < 0: no gust). Inflow corrections: for direction d,
// corr[corr_off[d] ...] holds heights, magnitudes and angles (corr_len[d] each) and
// ranges[(d * S + wing) * 2 ...] the wing's [start, end). step[0] = time, step[1] = ship
// velocity (device memory, so a captured step reads the current values).
struct WindDevice {
    d3 up{0, 0, 1}, axis{0, 0, 1}, zero{1, 0, 0};
    double water_plane_height = 0.0, direction_coming_from = 0.0;
    int vv_kind = 0;  // 0 constant, 1 power model, 2 logarithmic model
    double vv_constant = 0.0, reference_velocity = 0.0, reference_height = 10.0, power_factor = 1.0 / 9.0;
    double friction_velocity = 0.0, surface_roughness = 0.0, obukhov_length = 0.0;
    double von_karman = 0.41, stable_coefficient = 6.0, unstable_coefficient = 19.3;
    int has_obukhov = 0;
    const double* spectra = nullptr;
    int spec_off[3] = {0, 0, 0}, spec_n[3] = {-1, -1, -1};
    int n_dirs = 0, S = 0;
    const double* dirs = nullptr;
    const double* corr = nullptr;
    const int* corr_off = nullptr;
    const int* corr_len = nullptr;
    const long long* ranges = nullptr;
    const double* step = nullptr;
};
// Freestream at the control points [N] then the wake points [n_wake] into out.
cudaError_t launch_wind_freestream(const WindDevice& w, const d3* ctrl, const int* wing_of_line, int N, const d3* wake,
                                   long long n_wake, d3* out, cudaStream_t s);
// Controller flow measurements per line from the control-point velocities v [N]:
// out [3][N] = |v|, angle of attack, apparent wind direction (geometry from k_prep_geometry).
cudaError_t launch_controller_input(const DevModel& m, const StepParams& p, const d3* v, double* out, cudaStream_t s);

// Sets the calling thread's sb_last_error / sb_last_status (sim_host.cu).
void report_error(int code, const std::string& message);

// FP32 / FP64 FMA throughput of `device` in TFLOP/s (k_probe.cu); negative on error.
double measure_fp32_peak(int device, int reps);
double measure_fp64_peak(int device, int reps);

// Sectional and integrated forces (force_calculations.rs:322-452, 669-698;
// forces_and_moments.rs:163-245; flow_derivatives.rs:31-63).
cudaError_t launch_forces(const DevModel& m, const StepParams& p, const ForceArgs& f, cudaStream_t s);
// The forces of every case of a batch in one launch (one CTA per case).
struct ForceJob {
    DevModel m;
    StepParams p;
    ForceArgs f;
};
cudaError_t launch_forces_jobs(const ForceJob* jobs, int n, cudaStream_t s);

}  // namespace sbgpu
