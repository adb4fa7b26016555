// CompleteSailModel: a lifting-line simulation with a wind model and a sail controller, the
// sb_csm_* functions of the C ABI (the operator cstormbird exposes as complete_sail_model_*,
// interfaces/cstormbird/src/lifting_line/complete_sail_model.rs:18-110, over
// stormbird/src/lifting_line/complete_sail_model/mod.rs).
//
// A steady-state condition (mod.rs:103-139) is: the wind freestream at the control points
// of the current geometry (generated on the GPU, k_wind_freestream), the controller's flow
// measurements per line (k_controller_input: |u|, angle of attack, apparent wind
// direction), the controller on the host (O(sails): measurement per wing, set points
// interpolated over the apparent wind direction and scaled by the loading, new local wing
// angles), then one step at time 0 with time step 1 with the freestream generated again.
// A sweep of conditions (wind speeds / directions / ship speeds / loadings) runs every
// condition on its own replica of the model in one batch (sb_batch): one batched
// measurement pass, one batched step; the optimal-loading search (mod.rs:60-101) is such a
// sweep over its loadings.
//
// The section model here is Foil, which has no internal state
// (line_force_model/data_update.rs:145-158 ignores the controller's state output for it) and
// the input power model NoPower (input_power.rs:33-35), so the controller's internal-state
// output is not computed and every input power is 0.
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "batch_access.hpp"
#include "sb_controller_setup.hpp"
#include "sim_core.hpp"

namespace {

// stormath/src/interpolation.rs:17-100 for scalars
double interpolate(double x, const std::vector<double>& xd, const std::vector<double>& yd) {
    auto two = [x](double x0, double x1, double y0, double y1) {
        if (x <= x0) return y0;
        if (x >= x1) return y1;
        return y0 + (y1 - y0) * ((x - x0) / (x1 - x0));
    };
    const size_t n = xd.size();
    if (n == 1) return yd[0];
    if (n == 2) return two(xd[0], xd[1], yd[0], yd[1]);
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        if (xd[mid] > x) hi = mid;
        else lo = mid;
    }
    if (lo == n - 1) return yd[lo];
    return two(xd[lo], xd[lo + 1], yd[lo], yd[lo + 1]);
}

// controller/set_points.rs:43-56
double limit_value(double old_value, double raw_new_value, double max_change) {
    const double d = raw_new_value - old_value;
    // f64::signum: -1 for negative numbers and -0, +1 otherwise
    if (std::fabs(d) > max_change) return old_value + max_change * (std::signbit(d) ? -1.0 : 1.0);
    return raw_new_value;
}

// set_points.rs:188-199
double wrap_pi(double a) {
    const double pi = 3.14159265358979323846, tau = 2.0 * pi;
    while (a > pi) a -= tau;
    while (a < -pi) a += tau;
    return a;
}

// measurements.rs:50-81 over the lines [start, end) of one wing
double measure(const double* values, int start, int end, const sbsetup::MeasurementSettings& ms) {
    const long long strips = end - start;
    const long long s = static_cast<long long>(ms.start_index);
    // (strips - end_offset - 1).max(start + 1).min(strips - 1) on unsigned integers: a
    // negative first term wraps to a huge value, which the min turns into strips - 1
    long long e = strips - static_cast<long long>(ms.end_offset) - 1;
    if (e < 0) e = strips - 1;
    else e = std::min(std::max(e, s + 1), strips - 1);
    if (s >= e) raise(SB_ERR_SIZE, "the controller's flow measurement range of a wing is empty");
    const double* v = values + start;
    double out = v[s];
    switch (ms.type) {
        case sbsetup::MeasurementType::Mean:  // stormath/src/statistics.rs:11-24
            for (long long i = s + 1; i < e; ++i) out += v[i];
            return out / static_cast<double>(e - s);
        case sbsetup::MeasurementType::Max:
            for (long long i = s + 1; i < e; ++i) if (v[i] > out) out = v[i];
            return out;
        case sbsetup::MeasurementType::Min:
            for (long long i = s + 1; i < e; ++i) if (v[i] < out) out = v[i];
            return out;
    }
    return out;
}

// Controller::update (controller/mod.rs:39-64) with ControllerInput::new_from_velocity
// (controller/input.rs:99-157) and ControllerSetPoints::get_new_output (set_points.rs:77-161)
// for one model: new local wing angles from the per-line measurements `meas` [3][N] (|u|,
// angle of attack, apparent wind direction). False when the controller does not update
// (time before start_time); the index it tests is never advanced by the reference, so every
// call at or after start_time updates.
bool controller_update(const sbsetup::ControllerSettings& c, double time, double time_step, double loading,
                       const double* meas, int N, const std::vector<std::pair<int, int>>& wings,
                       const double* current_angles, double* new_angles) {
    const bool initialization_done = time >= c.start_time;
    const bool time_to_update = (0 % c.time_steps_between_updates) == 0;
    const bool first_time_step = false;
    if (!(first_time_step || (time_to_update && initialization_done))) return false;
    // one output per set point (the model checks there are no more set points than wings);
    // wings without a set point keep their angle (data_update.rs:171-177)
    for (size_t w = 0; w < wings.size(); ++w) new_angles[w] = current_angles[w];
    for (size_t w = 0; w < c.set_points.size(); ++w) {
        const sbsetup::ControllerSetPoints& sp = c.set_points[w];
        const int a = wings[w].first, b = wings[w].second;
        const double aoa = measure(meas + N, a, b, c.flow_measurement.angle_of_attack);
        (void)measure(meas, a, b, c.flow_measurement.wind_velocity);  // feeds only the internal state
        const double direction = measure(meas + 2 * N, a, b, c.flow_measurement.wind_direction);
        double angle = 0.0;
        if (sp.has_angle_of_attack) {
            const double set_point = loading * interpolate(direction, sp.apparent_wind_directions, sp.angle_of_attack);
            if (sp.use_effective_angle_of_attack) {  // set_points.rs:122-140
                angle = wrap_pi(current_angles[w] + wrap_pi(aoa - set_point));
            } else {  // set_points.rs:108-120
                angle = direction - set_point;
            }
        }
        if (sp.has_max_local_wing_angle_change_rate)
            angle = limit_value(current_angles[w], angle, sp.max_local_wing_angle_change_rate * time_step);
        new_angles[w] = angle;
    }
    return true;
}

// WindCondition of the C interface (interfaces/cstormbird/src/wind.rs:15-33): a power-law
// profile with the reference velocity at the default height (10 m) and factor (1/9).
std::string condition_json(const sb_wind_condition& wc) {
    char buf[256];
    std::snprintf(buf, sizeof(buf),
                  "{\"direction_coming_from\": %.17g, \"velocity_variation\": {\"PowerModel\": "
                  "{\"reference_velocity\": %.17g}}}",
                  wc.direction_coming_from, wc.velocity);
    return buf;
}

void check_condition(const sb_wind_condition& wc, double ship_velocity, double loading) {
    if (!std::isfinite(wc.velocity) || !std::isfinite(wc.direction_coming_from) || !std::isfinite(ship_velocity) ||
        !std::isfinite(loading))
        raise(SB_ERR_NONFINITE, "non-finite wind condition, ship velocity or loading");
}

}  // namespace

struct sb_csm {
    int device = 0;
    sbsetup::CompleteSailModelSetup setup;
    std::unique_ptr<sb_sim> sim;
    std::vector<std::pair<int, int>> wings;  // line range of each wing
    DevBuf<double> meas;                     // [3][N] controller measurements
    PinnedBuf<double> h_meas;
    std::string condition;                   // WindCondition JSON the model's wind was set from
    // replicas for sweeps of conditions
    sb_batch* sweep = nullptr;
    size_t sweep_cases = 0;

    ~sb_csm() {
        if (sweep) sb_batch_free(sweep);
    }

    void build(const char* json, int dev) {
        device = dev;
        try {
            setup = sbsetup::parse_complete_sail_model(json);
        } catch (const sbsetup::SetupError& e) {
            raise(SB_ERR_BAD_JSON, e.what());
        }
        sim.reset(new sb_sim());
        sim->build(setup.lifting_line_json.c_str(), dev);
        if (setup.controller.set_points.size() > static_cast<size_t>(sim->S))
            raise(SB_ERR_SIZE, "the controller has " + std::to_string(setup.controller.set_points.size()) +
                                   " set points for " + std::to_string(sim->S) + " wings");
        std::vector<int> ws(sim->S), we(sim->S);
        ck(cudaMemcpy(ws.data(), sim->wing_start.p, sim->S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
        ck(cudaMemcpy(we.data(), sim->wing_end.p, sim->S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
        for (int w = 0; w < sim->S; ++w) wings.emplace_back(ws[w], we[w]);
        meas.alloc(static_cast<size_t>(sim->N) * 3);
        h_meas.alloc(static_cast<size_t>(sim->N) * 3);
    }

    void set_condition(const std::string& cond) {
        if (cond != condition || !sim->has_wind) {
            sim->set_wind(setup.wind_environment_json.c_str(), cond.c_str());
            condition = cond;
        }
    }

    // CompleteSailModel::apply_controller_based_on_wind_condition (mod.rs:190-212) and
    // apply_controller_based_on_freestream (mod.rs:259-288).
    void apply_controller(double time, double time_step, const std::string& cond, double ship_velocity, double loading) {
        set_condition(cond);
        ck(cudaSetDevice(device), "cudaSetDevice");
        sim->set_wind_step(time, ship_velocity);
        sim->enqueue_wind_freestream();
        ck(launch_controller_input(sim->dm, sim->params, sim->fs_p, meas.p, sim->stream), "controller input");
        ck(cudaMemcpyAsync(h_meas.p, meas.p, 3 * sim->N * sizeof(double), cudaMemcpyDeviceToHost, sim->stream),
           "D2H controller input");
        ck(cudaStreamSynchronize(sim->stream), "controller input");
        double angles[kMaxWings];
        if (controller_update(setup.controller, time, time_step, loading, h_meas.p, sim->N, wings,
                              sim->params.local_wing_angles, angles))
            for (int w = 0; w < sim->S; ++w) sim->params.local_wing_angles[w] = angles[w];
    }

    // CompleteSailModel::do_step (mod.rs:170-188)
    void do_step(double time, double time_step, const std::string& cond, double ship_velocity, sb_step_output* out) {
        set_condition(cond);
        ck(cudaSetDevice(device), "cudaSetDevice");
        sim->do_step_wind(time, time_step, ship_velocity, out);
    }

    // simulate_steady_state_condition (mod.rs:103-122) with the simplified output
    // (mod.rs:124-136): per sail the total force, total moment and input power.
    size_t steady_state(const sb_wind_condition& wc, double ship_velocity, double loading, sb_single_sail_result* out,
                        size_t n) {
        check_condition(wc, ship_velocity, loading);
        const std::string cond = condition_json(wc);
        apply_controller(0.0, 1.0, cond, ship_velocity, loading);
        do_step(0.0, 1.0, cond, ship_velocity, nullptr);
        const size_t count = std::min(n, static_cast<size_t>(sim->S));
        for (size_t w = 0; w < count; ++w) write_sail(sim->h_out.p + sim->L.intf, sim->h_out.p + sim->L.intm, w, out[w]);
        return count;
    }

    static void write_sail(const double* forces, const double* moments, size_t w, sb_single_sail_result& r) {
        for (int k = 0; k < 3; ++k) {
            r.force[k] = forces[(w * 6 + 5) * 3 + k];
            r.moment[k] = moments[(w * 6 + 5) * 3 + k];
        }
        r.input_power = 0.0;  // NoPower (input_power.rs:33-35)
    }

    sb_batch* replicas(size_t n) {
        if (sweep && sweep_cases == n) return sweep;
        if (sweep) {
            sb_batch_free(sweep);
            sweep = nullptr;
            sweep_cases = 0;
        }
        std::vector<const char*> jsons(n, setup.lifting_line_json.c_str());
        sweep = sb_batch_new(jsons.data(), n, device);
        if (!sweep) raise(SB_ERR_STATE, std::string("replica batch: ") + sb_last_error());
        // every sweep changes the replicas' wing angles, which a captured graph would hold fixed
        if (sb_batch_use_graph(sweep, 0) != SB_OK) raise(SB_ERR_STATE, sb_last_error());
        sweep_cases = n;
        return sweep;
    }

    // Steady-state conditions i = 0..n-1, each on its own replica of the model starting from
    // the model's current wing angles and motion: one batched measurement pass, the
    // controllers on the host, one batched step. out [n][sails].
    void sweep_steady_state(const sb_wind_condition* wcs, const double* ship_velocities, const double* loadings,
                            size_t n, sb_single_sail_result* out) {
        if (n == 0) raise(SB_ERR_SIZE, "no conditions");
        for (size_t i = 0; i < n; ++i) check_condition(wcs[i], ship_velocities[i], loadings[i]);
        sb_batch* b = replicas(n);
        std::vector<std::string> conds(n);
        std::vector<const char*> cj(n);
        for (size_t i = 0; i < n; ++i) {
            conds[i] = condition_json(wcs[i]);
            cj[i] = conds[i].c_str();
        }
        if (sb_batch_set_wind(b, setup.wind_environment_json.c_str(), cj.data()) != SB_OK)
            raise(sb_last_status(), sb_last_error());
        for (size_t i = 0; i < n; ++i) sbhost::batch_case(b, i)->params = sim->params;
        const double* m = sbhost::batch_controller_inputs(b, 0.0, ship_velocities);
        for (size_t i = 0; i < n; ++i) {
            sb_sim* c = sbhost::batch_case(b, i);
            double angles[kMaxWings];
            if (controller_update(setup.controller, 0.0, 1.0, loadings[i], m + 3 * sbhost::batch_line_offset(b, i), c->N,
                                  wings, c->params.local_wing_angles, angles))
                for (int w = 0; w < c->S; ++w) c->params.local_wing_angles[w] = angles[w];
        }
        if (sb_batch_do_step_wind(b, 0.0, 1.0, ship_velocities) != SB_OK) raise(sb_last_status(), sb_last_error());
        const double* t = sbhost::batch_wing_totals(b);
        const size_t S = static_cast<size_t>(sim->S);
        for (size_t i = 0; i < n; ++i) {
            const double* f = t + i * S * 36;
            for (size_t w = 0; w < S; ++w) write_sail(f, f + S * 18, w, out[i * S + w]);
        }
    }

    // simulate_condition_optimal_controller_loading (mod.rs:60-101): loadings linspace(0.1,
    // 1.0, n) (stormath/src/array_generation.rs:16-30, accumulated steps), effective power =
    // -F_x * ship velocity - input power, the first maximum wins. The loadings run as one sweep.
    double optimal_loading(const sb_wind_condition& wc, double ship_velocity, size_t nr_loadings,
                           sb_single_sail_result* out) {
        if (nr_loadings == 0) raise(SB_ERR_SIZE, "nr_loadings must be at least 1");
        std::vector<double> loadings(nr_loadings);
        const double dx = (1.0 - 0.1) / static_cast<double>(nr_loadings - 1);
        double x = 0.1;
        for (size_t i = 0; i < nr_loadings; ++i) {
            loadings[i] = x;
            x += dx;
        }
        const size_t S = static_cast<size_t>(sim->S);
        std::vector<sb_single_sail_result> all(nr_loadings * S);
        std::vector<sb_wind_condition> wcs(nr_loadings, wc);
        std::vector<double> ships(nr_loadings, ship_velocity);
        sweep_steady_state(wcs.data(), ships.data(), loadings.data(), nr_loadings, all.data());
        double best = -INFINITY;
        size_t best_i = 0;
        for (size_t i = 0; i < nr_loadings; ++i) {
            double fx = 0.0, power = 0.0;  // integrated_forces_sum / input_power_sum (results/simulation.rs:61-89)
            for (size_t w = 0; w < S; ++w) {
                fx += all[i * S + w].force[0];
                power += all[i * S + w].input_power;
            }
            const double effective = -fx * ship_velocity - power;
            if (effective > best) {
                best = effective;
                best_i = i;
            }
        }
        for (size_t w = 0; w < S; ++w) out[w] = all[best_i * S + w];
        return loadings[best_i];
    }
};

extern "C" {

sb_csm* sb_csm_new(const char* setup_json, int device) {
    if (!setup_json) {
        report_error(SB_ERR_NULL_ARG, "setup_json is NULL");
        return nullptr;
    }
    std::unique_ptr<sb_csm> m(new sb_csm());
    if (guard([&] { m->build(setup_json, device); }) != SB_OK) return nullptr;
    return m.release();
}

void sb_csm_free(sb_csm* m) { delete m; }

int sb_csm_get_number_of_sails(const sb_csm* m) {
    if (!m) return SB_ERR_NULL_ARG;
    return m->sim->S;
}

int sb_csm_simulate_steady_state_condition(sb_csm* m, sb_wind_condition wind_condition, double ship_velocity,
                                           double controller_loading, sb_single_sail_result* results_out,
                                           size_t results_out_length) {
    if (!m || !results_out) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    if (results_out_length == 0) {
        report_error(SB_ERR_SIZE, "results_out_length is 0");
        return SB_ERR_SIZE;
    }
    size_t count = 0;
    const int rc = guard([&] {
        count = m->steady_state(wind_condition, ship_velocity, controller_loading, results_out, results_out_length);
    });
    return rc != SB_OK ? rc : static_cast<int>(count);
}

int sb_csm_apply_controller(sb_csm* m, double time, double time_step, const char* condition_json, double ship_velocity,
                            double controller_loading) {
    if (!m || !condition_json) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    return guard([&] { m->apply_controller(time, time_step, condition_json, ship_velocity, controller_loading); });
}

int sb_csm_do_step(sb_csm* m, double time, double time_step, const char* condition_json, double ship_velocity,
                   sb_step_output* out) {
    if (!m || !condition_json) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    return guard([&] { m->do_step(time, time_step, condition_json, ship_velocity, out); });
}

int sb_csm_sim(sb_csm* m, sb_sim** sim) {
    if (!m || !sim) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    *sim = m->sim.get();
    return SB_OK;
}

int sb_csm_sweep_steady_state(sb_csm* m, const sb_wind_condition* wind_conditions, const double* ship_velocities,
                              const double* controller_loadings, size_t n_conditions, sb_single_sail_result* results_out,
                              size_t results_out_length) {
    if (!m || !wind_conditions || !ship_velocities || !controller_loadings || !results_out) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    return guard([&] {
        if (results_out_length != n_conditions * static_cast<size_t>(m->sim->S))
            raise(SB_ERR_SIZE, "results_out_length must be n_conditions x sails");
        m->sweep_steady_state(wind_conditions, ship_velocities, controller_loadings, n_conditions, results_out);
    });
}

int sb_csm_simulate_condition_optimal_controller_loading(sb_csm* m, sb_wind_condition wind_condition,
                                                         double ship_velocity, size_t nr_loadings_to_test,
                                                         sb_single_sail_result* results_out, size_t results_out_length,
                                                         double* best_loading) {
    if (!m || !results_out) {
        report_error(SB_ERR_NULL_ARG, "null argument");
        return SB_ERR_NULL_ARG;
    }
    return guard([&] {
        if (results_out_length != static_cast<size_t>(m->sim->S)) raise(SB_ERR_SIZE, "results_out_length must be sails");
        const double l = m->optimal_loading(wind_condition, ship_velocity, nr_loadings_to_test, results_out);
        if (best_loading) *best_loading = l;
    });
}

}  // extern "C"
