// ORACLE — TEST INFRASTRUCTURE ONLY (see sb_oracle.hpp).
//
// C ABI over the f64 restatement, shaped like the library's own C ABI
// (include/stormbird_gb300.h) so that tests drive both through the same calls.
// Prefix `sbo_`. Status codes are the library's SB_* codes.
#include <cstring>
#include <string>

#include "../include/stormbird_gb300.h"
#include "sb_oracle.hpp"
#include "sb_oracle_wind.hpp"
#include "sb_oracle_controller.hpp"

namespace {
thread_local std::string g_err;
int fail(int code, const std::string& m) { g_err = m; return code; }

struct OracleSim {
    sbo::Simulation sim;
    sbo::StepResult last;
    OracleSim(const std::string& j, int t) : sim(j, t) {}
};

void write_output(const OracleSim& h, sb_step_output* out) {
    const auto& R = h.last;
    size_t n = R.circulation.size(), S = R.integrated_forces.size() / 6;
    auto v3 = [](double* dst, const std::vector<sbo::V3>& src) {
        if (!dst) return;
        for (size_t i = 0; i < src.size(); ++i) { dst[3 * i] = src[i].x; dst[3 * i + 1] = src[i].y; dst[3 * i + 2] = src[i].z; }
    };
    if (out->circulation_strength) std::memcpy(out->circulation_strength, R.circulation.data(), n * sizeof(double));
    if (out->angles_of_attack) std::memcpy(out->angles_of_attack, R.aoa.data(), n * sizeof(double));
    v3(out->ctrl_points_velocity, R.output_velocity);
    v3(out->solver_input_velocity, R.solver_input_velocity);
    v3(out->force_input_velocity, R.force_velocity);
    v3(out->acceleration, R.acceleration);
    v3(out->ctrl_points, R.ctrl_points);
    if (out->sectional_forces)
        for (int c = 0; c < 6; ++c) v3(out->sectional_forces + static_cast<size_t>(c) * n * 3, R.sectional[c]);
    v3(out->integrated_forces, R.integrated_forces);
    v3(out->integrated_moments, R.integrated_moments);
    (void)S;
    out->force_sum[0] = R.force_sum.x; out->force_sum[1] = R.force_sum.y; out->force_sum[2] = R.force_sum.z;
    out->moment_sum[0] = R.moment_sum.x; out->moment_sum[1] = R.moment_sum.y; out->moment_sum[2] = R.moment_sum.z;
    out->residual = R.residual;
    out->iterations = R.iterations;
    out->converged = R.converged ? 1 : 0;
}
}  // namespace

extern "C" {

const char* sbo_last_error(void) { return g_err.c_str(); }

void* sbo_sim_new(const char* json, int nthreads) {
    if (!json) { fail(SB_ERR_NULL_ARG, "setup_json is NULL"); return nullptr; }
    try {
        return new OracleSim(json, nthreads < 1 ? 1 : nthreads);
    } catch (const std::exception& e) {
        fail(SB_ERR_BAD_JSON, e.what());
        return nullptr;
    }
}

void sbo_sim_free(void* h) { delete static_cast<OracleSim*>(h); }

int sbo_sim_set_threads(void* h, int t) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    static_cast<OracleSim*>(h)->sim.set_threads(t < 1 ? 1 : t);
    return SB_OK;
}

int sbo_sim_sizes(void* h, size_t* n, size_t* s, size_t* nfs) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    if (n) *n = sim.lfm.nr_span_lines();
    if (s) *s = sim.lfm.nr_wings();
    if (nfs) *nfs = sim.nr_freestream_points();
    return SB_OK;
}

int sbo_sim_get_freestream_points(void* h, double* out, size_t n) {
    if (!h || !out) return fail(SB_ERR_NULL_ARG, "null argument");
    auto p = static_cast<OracleSim*>(h)->sim.freestream_points();
    if (n != p.size()) return fail(SB_ERR_SIZE, "size mismatch");
    for (size_t i = 0; i < n; ++i) { out[3 * i] = p[i].x; out[3 * i + 1] = p[i].y; out[3 * i + 2] = p[i].z; }
    return SB_OK;
}

int sbo_sim_do_step(void* h, double time, double dt, const double* fs, size_t n, sb_step_output* out) {
    if (!h || !fs) return fail(SB_ERR_NULL_ARG, "null argument");
    auto* o = static_cast<OracleSim*>(h);
    if (n != o->sim.nr_freestream_points()) return fail(SB_ERR_SIZE, "freestream length mismatch");
    try {
        std::vector<sbo::V3> v(n);
        for (size_t i = 0; i < n; ++i) v[i] = {fs[3 * i], fs[3 * i + 1], fs[3 * i + 2]};
        o->last = o->sim.do_step(time, dt, v.data(), n);
    } catch (const std::exception& e) {
        return fail(SB_ERR_STATE, e.what());
    }
    if (out) write_output(*o, out);
    return SB_OK;
}

int sbo_sim_induced_velocities(void* h, const double* pts, size_t n, double* out) {
    if (!h || !pts || !out) return fail(SB_ERR_NULL_ARG, "null argument");
    auto* o = static_cast<OracleSim*>(h);
    if (!o->sim.dynamic) return fail(SB_ERR_STATE, "Induced velocities not implemented for pure quasi-steady simulations");
    std::vector<sbo::V3> p(n);
    for (size_t i = 0; i < n; ++i) p[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    auto u = o->sim.induced_velocities(p.data(), n);
    for (size_t i = 0; i < n; ++i) { out[3 * i] = u[i].x; out[3 * i + 1] = u[i].y; out[3 * i + 2] = u[i].z; }
    return SB_OK;
}

int sbo_sim_set_translation_and_rotation_with_finite_difference(void* h, double dt, const double* t, const double* r) {
    if (!h || !t || !r) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& lfm = static_cast<OracleSim*>(h)->sim.lfm;
    lfm.rbm.update_translation_fd({t[0], t[1], t[2]}, dt);  // data_update.rs:188-205
    lfm.rbm.update_rotation_fd({r[0], r[1], r[2]}, dt);
    lfm.update_global_data_representations();
    return SB_OK;
}

int sbo_sim_set_translation_only(void* h, const double* t) {
    if (!h || !t) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& lfm = static_cast<OracleSim*>(h)->sim.lfm;
    lfm.rbm.translation = {t[0], t[1], t[2]};
    lfm.update_global_data_representations();
    return SB_OK;
}

int sbo_sim_set_rotation_only(void* h, const double* r) {
    if (!h || !r) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& lfm = static_cast<OracleSim*>(h)->sim.lfm;
    lfm.rbm.rotation = {r[0], r[1], r[2]};
    lfm.update_global_data_representations();
    return SB_OK;
}

int sbo_sim_set_velocity_linear(void* h, const double* v) {
    if (!h || !v) return fail(SB_ERR_NULL_ARG, "null argument");
    static_cast<OracleSim*>(h)->sim.lfm.rbm.velocity_linear = {v[0], v[1], v[2]};
    return SB_OK;
}

int sbo_sim_set_velocity_angular(void* h, const double* v) {
    if (!h || !v) return fail(SB_ERR_NULL_ARG, "null argument");
    static_cast<OracleSim*>(h)->sim.lfm.rbm.velocity_angular = {v[0], v[1], v[2]};
    return SB_OK;
}

int sbo_sim_set_local_wing_angles(void* h, const double* a, size_t n) {
    if (!h || !a) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& lfm = static_cast<OracleSim*>(h)->sim.lfm;
    if (n != lfm.nr_wings()) return fail(SB_ERR_SIZE, "The number of wing angles must match the number of wings in the simulation.");
    for (size_t i = 0; i < n; ++i) lfm.local_wing_angles[i] = a[i];
    lfm.update_global_data_representations();
    return SB_OK;
}

int sbo_sim_reset_previous_circulation(void* h) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    sim.previous_circulation.assign(sim.lfm.nr_span_lines(), 0.0);
    return SB_OK;
}

int sbo_sim_set_previous_circulation(void* h, const double* g, size_t n) {
    if (!h || !g) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    if (n != sim.lfm.nr_span_lines()) return fail(SB_ERR_SIZE, "size mismatch");
    sim.previous_circulation.assign(g, g + n);
    return SB_OK;
}

// State between steps, in the layout of the library's sb_sim_get_state: [0] wake steps
// completed, [1] first step completed, [2] flow-derivative updates, then (dynamic) wake points,
// velocity at the points, strengths, then previous circulation and the flow-derivative
// history h0, h1 (the public fields of simulation.rs:20-28 and dynamic_wake/mod.rs:41-64).
int sbo_sim_state_size(void* h, size_t* n) {
    if (!h || !n) return fail(SB_ERR_NULL_ARG, "null argument");
    const auto& sim = static_cast<OracleSim*>(h)->sim;
    const size_t N = sim.lfm.nr_span_lines();
    *n = 3 + (sim.dynamic ? sim.wake.points.size() * 6 + sim.wake.strengths.size() : 0) + 7 * N;
    return SB_OK;
}

int sbo_sim_get_state(void* h, double* o, size_t n) {
    size_t need = 0;
    if (sbo_sim_state_size(h, &need) != SB_OK || !o) return fail(SB_ERR_NULL_ARG, "null argument");
    if (n != need) return fail(SB_ERR_SIZE, "state size mismatch");
    const auto& sim = static_cast<OracleSim*>(h)->sim;
    o[0] = sim.dynamic ? static_cast<double>(sim.wake.steps_completed) : 0.0;
    o[1] = sim.first_step_completed ? 1.0 : 0.0;
    o[2] = static_cast<double>(sim.fd.count);
    double* p = o + 3;
    auto put = [&](const std::vector<sbo::V3>& v) {
        for (const auto& x : v) { p[0] = x.x; p[1] = x.y; p[2] = x.z; p += 3; }
    };
    if (sim.dynamic) {
        put(sim.wake.points);
        put(sim.wake.velocity_at_points);
        for (double g : sim.wake.strengths) *p++ = g;
    }
    for (double g : sim.previous_circulation) *p++ = g;
    put(sim.fd.h0);
    put(sim.fd.h1);
    return SB_OK;
}

int sbo_sim_set_state(void* h, const double* s, size_t n) {
    size_t need = 0;
    if (sbo_sim_state_size(h, &need) != SB_OK || !s) return fail(SB_ERR_NULL_ARG, "null argument");
    if (n != need) return fail(SB_ERR_SIZE, "state size mismatch");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    const double* p = s + 3;
    auto get = [&](std::vector<sbo::V3>& v) {
        for (auto& x : v) { x = {p[0], p[1], p[2]}; p += 3; }
    };
    sim.first_step_completed = s[1] != 0.0;
    sim.fd.count = static_cast<size_t>(s[2]);
    if (sim.dynamic) {
        sim.wake.steps_completed = static_cast<size_t>(s[0]);
        get(sim.wake.points);
        get(sim.wake.velocity_at_points);
        for (double& g : sim.wake.strengths) g = *p++;
        sim.wake.update_panel_data();
    }
    for (double& g : sim.previous_circulation) g = *p++;
    get(sim.fd.h0);
    get(sim.fd.h1);
    return SB_OK;
}

// Harness option: the next step's wake-velocity update keeps the freestream only.
int sbo_sim_skip_next_rollup(void* h) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    static_cast<OracleSim*>(h)->sim.wake.skip_induced_once = true;
    return SB_OK;
}

int sbo_sim_wake_sizes(void* h, size_t* npts, size_t* npan, size_t* nspan, size_t* W) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    if (!sim.dynamic) return fail(SB_ERR_STATE, "quasi-steady simulation has no dynamic wake");
    if (npts) *npts = sim.wake.points.size();
    if (npan) *npan = sim.wake.strengths.size();
    if (nspan) *nspan = sim.wake.nr_points_along_span;
    if (W) *W = sim.wake.nr_panels_per_line;
    return SB_OK;
}

int sbo_sim_get_wake_state(void* h, double* pts, double* str, double* vel) {
    if (!h) return fail(SB_ERR_NULL_ARG, "null handle");
    auto& sim = static_cast<OracleSim*>(h)->sim;
    if (!sim.dynamic) return fail(SB_ERR_STATE, "quasi-steady simulation has no dynamic wake");
    const auto& w = sim.wake;
    for (size_t i = 0; i < w.points.size(); ++i) {
        if (pts) { pts[3 * i] = w.points[i].x; pts[3 * i + 1] = w.points[i].y; pts[3 * i + 2] = w.points[i].z; }
        if (vel) { vel[3 * i] = w.velocity_at_points[i].x; vel[3 * i + 1] = w.velocity_at_points[i].y; vel[3 * i + 2] = w.velocity_at_points[i].z; }
    }
    if (str) std::memcpy(str, w.strengths.data(), w.strengths.size() * sizeof(double));
    return SB_OK;
}

// --- element-level helpers for the ported reference unit tests --------------------------

// Unit-strength velocity of a vortex panel. mode 0: near/far rule, 1: vortex ring, 2: doublet.
int sbo_panel_unit_velocity(const double* corners12, double far_field_ratio, double rc, const double* x, int mode, double* out) {
    sbo::V3 p[4];
    for (int i = 0; i < 4; ++i) p[i] = {corners12[3 * i], corners12[3 * i + 1], corners12[3 * i + 2]};
    sbo::Panel pan(p, far_field_ratio, rc);
    sbo::V3 X{x[0], x[1], x[2]};
    sbo::V3 u = mode == 1 ? pan.ring(X) : (mode == 2 ? pan.doublet(X) : pan.unit(X));
    out[0] = u.x; out[1] = u.y; out[2] = u.z;
    return SB_OK;
}

int sbo_line_unit_velocity(const double* a, const double* b, const double* x, double rc, double* out) {
    sbo::V3 u = sbo::line_unit_velocity({a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {x[0], x[1], x[2]}, rc);
    out[0] = u.x; out[1] = u.y; out[2] = u.z;
    return SB_OK;
}

double sbo_quad_area(const double* corners12) {
    sbo::V3 p[4];
    for (int i = 0; i < 4; ++i) p[i] = {corners12[3 * i], corners12[3 * i + 1], corners12[3 * i + 2]};
    return sbo::area_of_quadrilateral(p);
}

int sbo_rotate(const double* v, const double* r, int type, double* out) {
    sbo::V3 o = sbo::rotate({v[0], v[1], v[2]}, {r[0], r[1], r[2]},
                            type == 0 ? sbsetup::RotationType::XYZ : sbsetup::RotationType::YawPitchRoll);
    out[0] = o.x; out[1] = o.y; out[2] = o.z;
    return SB_OK;
}

double sbo_sigmoid(double x, double x0, double r) { return sbo::sigmoid_zero_to_one(x, x0, r); }

// Foil evaluation from the Foil JSON object body (e.g. "{}" for defaults).
// out: [cl, cl_pre_stall_with_drop_off, cl_post_stall_with_weight, cd, amount_of_stall, cl_linear]
int sbo_foil_eval(const char* foil_json, double alpha, double* out) {
    try {
        sbjson::Value v = sbjson::parse(foil_json);
        sbo::Foil f;
        f.p = sbsetup::detail::foil(v, "Foil");
        out[0] = f.cl(alpha);
        out[1] = f.cl_pre_stall_with_drop_off(alpha);
        out[2] = f.cl_post_stall_with_weight(alpha);
        out[3] = f.cd(alpha);
        out[4] = f.amount_of_stall(alpha);
        out[5] = f.cl_linear(alpha);
    } catch (const std::exception& e) {
        return fail(SB_ERR_BAD_JSON, e.what());
    }
    return SB_OK;
}

// Raw Biot-Savart sweep for the CPU baseline: u_i = sum_j gamma_j * unit(panel_j, x_i) over
// Freestream of CompleteSailModel::freestream_velocity (complete_sail_model/mod.rs:213-257)
// at the simulation's freestream points for a WindEnvironment / WindCondition JSON pair.
int sbo_sim_wind_freestream(void* h, const char* env_json, const char* cond_json, double time, double ship_velocity,
                            double* out, size_t n) {
    if (!h || !env_json || !cond_json || !out) return fail(SB_ERR_NULL_ARG, "null argument");
    try {
        sbo::WindModel w;
        w.env = sbsetup::parse_wind_environment(env_json);
        w.cond = sbsetup::parse_wind_condition(cond_json);
        const auto& sim = static_cast<OracleSim*>(h)->sim;
        if (n != sim.nr_freestream_points()) return fail(SB_ERR_SIZE, "size mismatch");
        const auto fs = sbo::complete_sail_freestream(sim, w, ship_velocity, time);
        for (size_t i = 0; i < n; ++i) { out[3 * i] = fs[i].x; out[3 * i + 1] = fs[i].y; out[3 * i + 2] = fs[i].z; }
    } catch (const std::exception& e) {
        return fail(SB_ERR_BAD_JSON, e.what());
    }
    return SB_OK;
}

// Unsteady apparent wind (environment.rs:175-188) at arbitrary locations [n*3], no
// inflow corrections.
int sbo_wind_velocity_at(const char* env_json, const char* cond_json, const double* points, size_t n, double time,
                         double ship_velocity, double* out) {
    if (!env_json || !cond_json || (n && (!points || !out))) return fail(SB_ERR_NULL_ARG, "null argument");
    try {
        sbo::WindModel w;
        w.env = sbsetup::parse_wind_environment(env_json);
        w.cond = sbsetup::parse_wind_condition(cond_json);
        const sbo::V3 linear = ship_velocity * sbo::to_v3(w.env.zero_direction_vector);
        for (size_t i = 0; i < n; ++i) {
            const sbo::V3 u = w.unsteady_apparent_wind({points[3 * i], points[3 * i + 1], points[3 * i + 2]}, linear, time);
            out[3 * i] = u.x; out[3 * i + 1] = u.y; out[3 * i + 2] = u.z;
        }
    } catch (const std::exception& e) {
        return fail(SB_ERR_BAD_JSON, e.what());
    }
    return SB_OK;
}

// panels given by corners [P*12], far-field ratio, cores [P], strengths [P]; targets [M*3].
// Runs the reference's per-target loop (induced_velocity_calc.rs:111-126) on nthreads threads.
int sbo_bs_sweep(const double* corners, const double* cores, const double* strengths, size_t P, double far_field_ratio,
                 const double* targets, size_t M, double* out, int nthreads) {
    std::vector<sbo::Panel> pans(P);
    for (size_t j = 0; j < P; ++j) {
        sbo::V3 p[4];
        for (int i = 0; i < 4; ++i) p[i] = {corners[12 * j + 3 * i], corners[12 * j + 3 * i + 1], corners[12 * j + 3 * i + 2]};
        pans[j] = sbo::Panel(p, far_field_ratio, cores[j]);
    }
    const long long mm = static_cast<long long>(M);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads < 1 ? 1 : nthreads)
    for (long long i = 0; i < mm; ++i) {
        sbo::V3 x{targets[3 * i], targets[3 * i + 1], targets[3 * i + 2]};
        sbo::V3 acc;
        for (size_t j = 0; j < P; ++j) {
            if (strengths[j] == 0.0) continue;
            acc = acc + strengths[j] * pans[j].unit(x);
        }
        out[3 * i] = acc.x; out[3 * i + 1] = acc.y; out[3 * i + 2] = acc.z;
    }
    return SB_OK;
}

// The same sweep with a symmetry condition (0 none, 1 X, 2 Y, 3 Z): each panel's unit velocity
// at x is corrected by its velocity at the mirrored point (induced_velocity_calc.rs:182-198,
// symmetry_condition.rs:27-43).
int sbo_bs_sweep_sym(const double* corners, const double* cores, const double* strengths, size_t P,
                     double far_field_ratio, int symmetry, const double* targets, size_t M, double* out, int nthreads) {
    if (symmetry < 0 || symmetry > 3) return fail(SB_ERR_SIZE, "symmetry must be 0..3");
    const auto sym = static_cast<sbsetup::Symmetry>(symmetry);
    std::vector<sbo::Panel> pans(P);
    for (size_t j = 0; j < P; ++j) {
        sbo::V3 p[4];
        for (int i = 0; i < 4; ++i) p[i] = {corners[12 * j + 3 * i], corners[12 * j + 3 * i + 1], corners[12 * j + 3 * i + 2]};
        pans[j] = sbo::Panel(p, far_field_ratio, cores[j]);
    }
    const long long mm = static_cast<long long>(M);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads < 1 ? 1 : nthreads)
    for (long long i = 0; i < mm; ++i) {
        sbo::V3 x{targets[3 * i], targets[3 * i + 1], targets[3 * i + 2]};
        sbo::V3 acc, m;
        const bool mirrored = sbo::mirrored_point(sym, x, &m);
        for (size_t j = 0; j < P; ++j) {
            if (strengths[j] == 0.0) continue;
            sbo::V3 u = pans[j].unit(x);
            if (mirrored) u = sbo::corrected_velocity(sym, u, pans[j].unit(m));
            acc = acc + strengths[j] * u;
        }
        out[3 * i] = acc.x; out[3 * i + 1] = acc.y; out[3 * i + 2] = acc.z;
    }
    return SB_OK;
}

// CompleteSailModel steady-state conditions (sb_oracle_controller.hpp)
void* sbo_csm_new(const char* json) {
    if (!json) { fail(SB_ERR_NULL_ARG, "setup_json is NULL"); return nullptr; }
    try {
        return new sbo::CompleteSailModel(json);
    } catch (const std::exception& e) {
        fail(SB_ERR_BAD_JSON, e.what());
        return nullptr;
    }
}

void sbo_csm_free(void* h) { delete static_cast<sbo::CompleteSailModel*>(h); }

// per sail: total force [3], total moment [3], input power (0: NoPower) -> out [sails][7]
int sbo_csm_steady_state(void* h, double velocity, double direction, double ship_velocity, double loading, double* out,
                         size_t n_sails) {
    if (!h || !out) return fail(SB_ERR_NULL_ARG, "null argument");
    auto* m = static_cast<sbo::CompleteSailModel*>(h);
    if (n_sails != m->sim.lfm.nr_wings()) return fail(SB_ERR_SIZE, "size mismatch");
    try {
        const sbo::StepResult r = m->steady_state(sbo::power_model_condition(velocity, direction), ship_velocity, loading);
        for (size_t w = 0; w < n_sails; ++w) {
            const sbo::V3 f = r.integrated_forces[w * 6 + 5], mo = r.integrated_moments[w * 6 + 5];
            double* o = out + 7 * w;
            o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = mo.x; o[4] = mo.y; o[5] = mo.z; o[6] = 0.0;
        }
    } catch (const std::exception& e) {
        return fail(SB_ERR_STATE, e.what());
    }
    return SB_OK;
}

int sbo_csm_local_wing_angles(void* h, double* out, size_t n) {
    if (!h || !out) return fail(SB_ERR_NULL_ARG, "null argument");
    const auto& lfm = static_cast<sbo::CompleteSailModel*>(h)->sim.lfm;
    if (n != lfm.nr_wings()) return fail(SB_ERR_SIZE, "size mismatch");
    for (size_t i = 0; i < n; ++i) out[i] = lfm.local_wing_angles[i];
    return SB_OK;
}

int sbo_csm_set_local_wing_angles(void* h, const double* a, size_t n) {
    if (!h || !a) return fail(SB_ERR_NULL_ARG, "null argument");
    auto& lfm = static_cast<sbo::CompleteSailModel*>(h)->sim.lfm;
    if (n != lfm.nr_wings()) return fail(SB_ERR_SIZE, "size mismatch");
    for (size_t i = 0; i < n; ++i) lfm.local_wing_angles[i] = a[i];
    lfm.update_global_data_representations();
    return SB_OK;
}

}  // extern "C"
