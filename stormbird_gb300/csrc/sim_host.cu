// Single-case C ABI of the GB300 lifting-line library (include/stormbird_gb300.h): the
// `sb_sim_*` functions over the simulation handle of sim_core.hpp, the standalone sweep and
// the thread's last-error state shared by every entry point of the library.
#include "sim_core.hpp"

namespace {

thread_local std::string g_last_error;
thread_local int g_last_status = SB_OK;

}  // namespace

namespace sbgpu {
void report_error(int code, const std::string& message) {
    g_last_status = code;
    g_last_error = message;
}
}  // namespace sbgpu

// =======================================================================================
// C ABI
// =======================================================================================
namespace {
d3 v3(const double* p) { return mk(p[0], p[1], p[2]); }
}  // namespace

extern "C" {

const char* sb_last_error(void) { return g_last_error.c_str(); }
int sb_last_status(void) { return g_last_status; }
const char* sb_version(void) { return "stormbird_gb300 0.1 (sm_103a)"; }

sb_sim* sb_sim_new(const char* setup_json, int device) {
    if (!setup_json) {
        g_last_error = "setup_json is NULL";
        g_last_status = SB_ERR_NULL_ARG;
        return nullptr;
    }
    std::unique_ptr<sb_sim> s(new sb_sim());
    int rc = guard([&] { s->build(setup_json, device); });
    if (rc != SB_OK) return nullptr;
    return s.release();
}

void sb_sim_free(sb_sim* sim) {
    if (!sim) return;
    cudaSetDevice(sim->device);
    if (sim->stream) cudaStreamSynchronize(sim->stream);
    delete sim;
}

int sb_sim_sizes(const sb_sim* sim, size_t* n, size_t* s, size_t* nfs) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    if (n) *n = static_cast<size_t>(sim->N);
    if (s) *s = static_cast<size_t>(sim->S);
    if (nfs) *nfs = static_cast<size_t>(sim->nfs);
    return SB_OK;
}

int sb_sim_get_freestream_points(const sb_sim* sim, double* points, size_t n) {
    if (!sim || !points) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { const_cast<sb_sim*>(sim)->freestream_points(points, n); });
}

int sb_sim_do_step(sb_sim* sim, double time, double dt, const double* fs, size_t n, sb_step_output* out) {
    if (!sim || !fs) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->do_step(time, dt, fs, n, out); });
}

int sb_sim_do_step_device(sb_sim* sim, double time, double dt, const double* fs_dev, size_t n) {
    if (!sim || !fs_dev) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->do_step_device(time, dt, fs_dev, n); });
}

int sb_sim_read_output(sb_sim* sim, sb_step_output* out) {
    if (!sim || !out) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->read_output(out); });
}

int sb_sim_induced_velocities(sb_sim* sim, const double* p, size_t n, double* o) {
    if (!sim || (n && (!p || !o))) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->induced_velocities(p, n, o); });
}

// data_update.rs:188-205 and rigid_body_motion.rs:68-103
int sb_sim_set_translation_and_rotation_with_finite_difference(sb_sim* sim, double dt, const double t[3], const double r[3]) {
    if (!sim || !t || !r) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    auto& p = sim->params;
    d3 old_t = p.translation;
    p.translation = v3(t);
    p.velocity_linear = (p.translation - old_t) / dt;
    d3 old_r = p.rotation;
    p.rotation = v3(r);
    d3 d = p.rotation - old_r;
    double* dd[3] = {&d.x, &d.y, &d.z};
    for (auto* c : dd) {
        if (*c > kPi) *c = *c + kTau;
        else if (*c < -kPi) *c = *c + kTau;
    }
    p.velocity_angular = d / dt;
    return SB_OK;
}

int sb_sim_set_translation_only(sb_sim* sim, const double t[3]) {
    if (!sim || !t) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    sim->params.translation = v3(t);
    return SB_OK;
}

int sb_sim_set_rotation_only(sb_sim* sim, const double r[3]) {
    if (!sim || !r) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    sim->params.rotation = v3(r);
    return SB_OK;
}

int sb_sim_set_velocity_linear(sb_sim* sim, const double v[3]) {
    if (!sim || !v) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    sim->params.velocity_linear = v3(v);
    return SB_OK;
}

int sb_sim_set_velocity_angular(sb_sim* sim, const double v[3]) {
    if (!sim || !v) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    sim->params.velocity_angular = v3(v);
    return SB_OK;
}

int sb_sim_set_local_wing_angles(sb_sim* sim, const double* a, size_t n) {
    if (!sim || !a) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    if (n != static_cast<size_t>(sim->S)) {
        g_last_error = "The number of wing angles must match the number of wings in the simulation.";
        return SB_ERR_SIZE;
    }
    for (size_t i = 0; i < n; ++i) sim->params.local_wing_angles[i] = a[i];
    return SB_OK;
}

int sb_sim_get_local_wing_angles(const sb_sim* sim, double* a, size_t n) {
    if (!sim || !a) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    if (n != static_cast<size_t>(sim->S)) {
        g_last_error = "The number of wing angles must match the number of wings in the simulation.";
        return SB_ERR_SIZE;
    }
    for (size_t i = 0; i < n; ++i) a[i] = sim->params.local_wing_angles[i];
    return SB_OK;
}

int sb_sim_reset_previous_circulation(sb_sim* sim) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    return guard([&] {
        ck(cudaMemsetAsync(sim->gamma_p, 0, sim->N * sizeof(double), sim->stream), "memset");
        ck(cudaStreamSynchronize(sim->stream), "sync");
    });
}

int sb_sim_set_previous_circulation(sb_sim* sim, const double* g, size_t n) {
    if (!sim || !g) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    if (n != static_cast<size_t>(sim->N)) { g_last_error = "size mismatch"; return SB_ERR_SIZE; }
    return guard([&] {
        ck(cudaMemcpyAsync(sim->gamma_p, g, n * sizeof(double), cudaMemcpyHostToDevice, sim->stream), "H2D");
        ck(cudaStreamSynchronize(sim->stream), "sync");
    });
}

int sb_sim_get_previous_circulation(const sb_sim* sim, double* g, size_t n) {
    if (!sim || !g) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    if (n != static_cast<size_t>(sim->N)) { g_last_error = "size mismatch"; return SB_ERR_SIZE; }
    return guard([&] {
        ck(cudaMemcpyAsync(g, sim->gamma_p, n * sizeof(double), cudaMemcpyDeviceToHost, sim->stream), "D2H");
        ck(cudaStreamSynchronize(sim->stream), "sync");
    });
}

int sb_sim_wake_sizes(const sb_sim* sim, size_t* npts, size_t* npan, size_t* nspan, size_t* W) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    if (!sim->dynamic) { g_last_error = "quasi-steady simulation has no dynamic wake"; return SB_ERR_STATE; }
    if (npts) *npts = static_cast<size_t>(sim->P_pts);
    if (npan) *npan = static_cast<size_t>(sim->P_pan);
    if (nspan) *nspan = static_cast<size_t>(sim->Np);
    if (W) *W = static_cast<size_t>(sim->W);
    return SB_OK;
}

int sb_sim_get_wake_state(sb_sim* sim, double* pts, double* str, double* vel) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    if (!sim->dynamic) { g_last_error = "quasi-steady simulation has no dynamic wake"; return SB_ERR_STATE; }
    return guard([&] {
        auto s = sim->stream;
        if (pts) ck(cudaMemcpyAsync(pts, sim->pts[sim->cur].p, sim->P_pts * sizeof(d3), cudaMemcpyDeviceToHost, s), "D2H");
        if (str) ck(cudaMemcpyAsync(str, sim->str[sim->cur].p, sim->P_pan * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
        if (vel) ck(cudaMemcpyAsync(vel, sim->vel.p, sim->P_pts * sizeof(d3), cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "sync");
    });
}

int sb_sim_state_size(const sb_sim* sim, size_t* n) {
    if (!sim || !n) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    *n = sim->state_size();
    return SB_OK;
}

int sb_sim_get_state(sb_sim* sim, double* state, size_t n) {
    if (!sim || !state) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->get_state(state, n); });
}

int sb_sim_set_state(sb_sim* sim, const double* state, size_t n) {
    if (!sim || !state) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->set_state(state, n); });
}

int sb_sim_set_precision(sb_sim* sim, int mode) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    if (mode < 0 || mode > 2) { g_last_error = "precision mode must be 0, 1 or 2"; return SB_ERR_SIZE; }
    sim->precision = mode;
    return SB_OK;
}

int sb_sim_enable_timing(sb_sim* sim, int enable) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    sim->timing = enable != 0;
    return SB_OK;
}

int sb_sim_last_step_timing(const sb_sim* sim, double* ms, size_t n) {
    if (!sim || !ms) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    for (size_t i = 0; i < n && i < 12; ++i) ms[i] = sim->last_ms[i];
    return SB_OK;
}

int sb_sim_last_step_counters(const sb_sim* sim, double* c, size_t n) {
    if (!sim || !c) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    for (size_t i = 0; i < n && i < 7; ++i) c[i] = sim->last_counters[i];
    return SB_OK;
}

int sb_sim_set_wind(sb_sim* sim, const char* environment_json, const char* condition_json) {
    if (!sim || !environment_json || !condition_json) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->set_wind(environment_json, condition_json); });
}

int sb_sim_wind_freestream(sb_sim* sim, double time, double ship_velocity, double* freestream, size_t n) {
    if (!sim || !freestream) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->wind_freestream(time, ship_velocity, freestream, n); });
}

int sb_sim_do_step_wind(sb_sim* sim, double time, double time_step, double ship_velocity, sb_step_output* out) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    return guard([&] { sim->do_step_wind(time, time_step, ship_velocity, out); });
}

int sb_sim_set_result_file(sb_sim* sim, const char* path, int format) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    if (format < SB_RESULTS_OFF || format > SB_RESULTS_CSV) { g_last_error = "unknown result format"; return SB_ERR_SIZE; }
    return guard([&] { sim->set_result_file(path, format); });
}

int sb_sim_flush_results(sb_sim* sim) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    return guard([&] {
        if (sim->writer && !sim->writer->flush()) raise(SB_ERR_STATE, "writing the result file failed");
        if (sim->wake_writer && !sim->wake_writer->flush()) raise(SB_ERR_STATE, "writing a wake file failed");
    });
}

int sb_sim_result_json(const sb_sim* sim, char* buf, size_t capacity, size_t* length) {
    if (!sim || !length) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] {
        const std::string s = sbhost::result_json(sim->result_record());
        *length = s.size() + 1;
        if (!buf || capacity < s.size() + 1) raise(SB_ERR_SIZE, "buffer too small: " + std::to_string(s.size() + 1) + " bytes needed");
        std::memcpy(buf, s.c_str(), s.size() + 1);
    });
}

int sb_sim_result_csv(const sb_sim* sim, char* header, size_t header_capacity, char* data, size_t data_capacity) {
    if (!sim || !header || !data) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    return guard([&] {
        std::string h, d;
        sbhost::result_csv(sim->result_record(), h, d);
        if (header_capacity < h.size() + 1 || data_capacity < d.size() + 1) raise(SB_ERR_SIZE, "buffer too small");
        std::memcpy(header, h.c_str(), h.size() + 1);
        std::memcpy(data, d.c_str(), d.size() + 1);
    });
}

int sb_sim_set_segment_sharing(sb_sim* sim, int enable) {
    if (!sim) { g_last_error = "null handle"; return SB_ERR_NULL_ARG; }
    sim->share_segments = enable != 0;
    return SB_OK;
}

int sb_sim_segment_sharing_active(const sb_sim* sim, int* active) {
    if (!sim || !active) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    *active = sim->use_chains() ? 1 : 0;
    return SB_OK;
}

// Standalone sweep over caller-given panels (see include/stormbird_gb300.h).
int sb_panel_sweep(int device, const double* corners, const double* strengths, const double* core_lengths,
                   size_t n_panels, double far_field_ratio, int symmetry, const double* targets, size_t n_targets,
                   int precision, double* velocities) {
    if ((n_panels && (!corners || !strengths || !core_lengths)) || (n_targets && (!targets || !velocities))) {
        g_last_error = "null argument";
        g_last_status = SB_ERR_NULL_ARG;
        return SB_ERR_NULL_ARG;
    }
    if (symmetry < 0 || symmetry > 3 || precision < 0 || precision > 2) {
        g_last_error = "symmetry must be 0..3 and precision 0..2";
        g_last_status = SB_ERR_SIZE;
        return SB_ERR_SIZE;
    }
    if (n_targets == 0) {
        report_error(SB_OK, "");
        return SB_OK;
    }
    return guard([&] {
        panel_sweep_impl(device, corners, strengths, core_lengths, static_cast<long long>(n_panels), far_field_ratio,
                         symmetry, targets, static_cast<long long>(n_targets), precision, velocities);
    });
}

int sb_measure_fp32_peak(int device, int reps, double* tflops) {
    if (!tflops) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    double v = measure_fp32_peak(device, reps < 1 ? 1 : reps);
    if (v < 0.0) { g_last_error = "FP32 probe failed"; return SB_ERR_CUDA; }
    *tflops = v;
    return SB_OK;
}

int sb_measure_fp64_peak(int device, int reps, double* tflops) {
    if (!tflops) { g_last_error = "null argument"; return SB_ERR_NULL_ARG; }
    double v = measure_fp64_peak(device, reps < 1 ? 1 : reps);
    if (v < 0.0) { g_last_error = "FP64 probe failed"; return SB_ERR_CUDA; }
    *tflops = v;
    return SB_OK;
}

// Bounded-wait diagnostics (see include/stormbird_gb300.h).
int sb_set_sweep_wait_polls(int polls) {
    set_sweep_wait_polls(polls);
    report_error(SB_OK, "");
    return SB_OK;
}

int sb_wait_timeout_self_test(int device, int polls) {
    if (polls < 0) {
        report_error(SB_ERR_SIZE, "polls must be >= 0");
        return SB_ERR_SIZE;
    }
    return guard([&] {
        ck(cudaSetDevice(device), "cudaSetDevice");
        cudaStream_t st;
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
        StreamBufs B(st);
        int* derr = B.get<int>(1);
        int herr = 0;
        ck(cudaMemsetAsync(derr, 0, sizeof(int), st), "memset");
        ck(launch_wait_probe(polls, derr, st), "wait probe");
        ck(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "wait probe");
        if (herr == kDevTimeout) raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out");
        if (herr != kDevOk) raise(SB_ERR_CUDA, "device error word " + std::to_string(herr));
    });
}

}  // extern "C"
