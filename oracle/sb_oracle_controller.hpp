// ORACLE — TEST INFRASTRUCTURE ONLY (see sb_oracle.hpp).
//
// f64 restatement of the reference's CompleteSailModel steady-state condition: the sail
// controller (stormbird/src/controller/: set_points.rs, measurements.rs, input.rs, mod.rs)
// acting on the freestream of the wind model (sb_oracle_wind.hpp), then one step of the
// lifting-line simulation (complete_sail_model/mod.rs:103-139).
#pragma once

#include <cmath>
#include <stdexcept>
#include <vector>

#include "../stormbird_gb300/csrc/sb_controller_setup.hpp"
#include "sb_oracle.hpp"
#include "sb_oracle_wind.hpp"

namespace sbo {

// controller/measurements.rs:50-81; the usize arithmetic of the end index as in a release
// build (a negative difference wraps, and min() then gives nr_strips - 1)
inline double measure_float_values_wing(const std::vector<double>& all, Range r, const sbsetup::MeasurementSettings& ms) {
    const std::vector<double> wing(all.begin() + r.start, all.begin() + r.end);
    const size_t nr_strips = wing.size();
    const size_t start = ms.start_index;
    size_t end;
    if (ms.end_offset + 1 > nr_strips) end = nr_strips - 1;
    else end = std::min(std::max(nr_strips - ms.end_offset - 1, start + 1), nr_strips - 1);
    if (start >= end) throw std::runtime_error("empty measurement range");
    const std::vector<double> v(wing.begin() + start, wing.begin() + end);
    switch (ms.type) {
        case sbsetup::MeasurementType::Mean: {  // stormath/src/statistics.rs:11-24
            double s = v[0];
            for (size_t i = 1; i < v.size(); ++i) s = s + v[i];
            return s / static_cast<double>(v.size());
        }
        case sbsetup::MeasurementType::Max: {
            double m = v[0];
            for (size_t i = 1; i < v.size(); ++i) if (v[i] > m) m = v[i];
            return m;
        }
        case sbsetup::MeasurementType::Min: {
            double m = v[0];
            for (size_t i = 1; i < v.size(); ++i) if (v[i] < m) m = v[i];
            return m;
        }
    }
    return 0.0;
}

// controller/input.rs:29-37
struct ControllerInput {
    double loading = 0.0, current_local_wing_angle = 0.0, current_section_model_internal_state = 0.0;
    double angle_of_attack = 0.0, velocity = 0.0, apparent_wind_direction = 0.0;
};

// environment.rs:315-345
inline std::vector<double> apparent_wind_direction_from_velocity(const std::vector<V3>& velocity, const LineForceModel& lfm) {
    std::vector<double> out;
    for (size_t i = 0; i < lfm.nr_span_lines(); ++i) {
        const size_t w = lfm.wing_index(i);
        const size_t first = lfm.wing_indices[w].start;
        const V3 axis = normalize(lfm.span_lines_global[first].rel());
        const V3 chord = lfm.rbm.transform_vector(lfm.chord_not_rotated[first]);
        out.push_back(signed_angle_between(chord, velocity[i], axis));
    }
    return out;
}

// input.rs:99-157 (section internal states are 0: Foil sections, data_access.rs:101-117)
inline std::vector<ControllerInput> controller_input_from_velocity(double loading, const LineForceModel& lfm,
                                                                   const std::vector<V3>& velocity,
                                                                   const sbsetup::FlowMeasurementSettings& s) {
    std::vector<double> speeds;
    for (const auto& v : velocity) speeds.push_back(length(v));
    const std::vector<double> aoa = lfm.angles_of_attack(velocity);
    const std::vector<double> dirs = apparent_wind_direction_from_velocity(velocity, lfm);
    std::vector<ControllerInput> out;
    for (size_t w = 0; w < lfm.nr_wings(); ++w) {
        ControllerInput in;
        in.loading = loading;
        in.current_local_wing_angle = lfm.local_wing_angles[w];
        in.angle_of_attack = measure_float_values_wing(aoa, lfm.wing_indices[w], s.angle_of_attack);
        in.velocity = measure_float_values_wing(speeds, lfm.wing_indices[w], s.wind_velocity);
        in.apparent_wind_direction = measure_float_values_wing(dirs, lfm.wing_indices[w], s.wind_direction);
        out.push_back(in);
    }
    return out;
}

// set_points.rs:43-56 (f64::signum)
inline double limit_value(double old_value, double raw_new_value, double max_change) {
    const double diff = raw_new_value - old_value;
    if (std::fabs(diff) > max_change) return old_value + max_change * std::copysign(1.0, diff);
    return raw_new_value;
}

// set_points.rs:188-199
inline double correct_angle(double a) {
    double c = a;
    while (c > PI) c -= TAU;
    while (c < -PI) c += TAU;
    return c;
}

// set_points.rs:77-106, 108-140, 163-173 (local wing angle)
inline double new_local_wing_angle(const sbsetup::ControllerSetPoints& sp, const ControllerInput& in, double time_step) {
    double angle = 0.0;
    if (sp.has_angle_of_attack) {
        const double set_point = in.loading * linear_interpolation(in.apparent_wind_direction, sp.apparent_wind_directions,
                                                                   sp.angle_of_attack);
        if (sp.use_effective_angle_of_attack) {
            const double error = correct_angle(in.angle_of_attack - set_point);
            angle = correct_angle(in.current_local_wing_angle + error);
        } else {
            angle = in.apparent_wind_direction - set_point;
        }
    }
    if (sp.has_max_local_wing_angle_change_rate)
        angle = limit_value(in.current_local_wing_angle, angle, sp.max_local_wing_angle_change_rate * time_step);
    return angle;
}

struct CompleteSailModel {
    sbsetup::CompleteSailModelSetup setup;
    Simulation sim;
    WindModel wind;

    explicit CompleteSailModel(const std::string& json)
        : setup(sbsetup::parse_complete_sail_model(json)), sim(setup.lifting_line_json, 1) {
        wind.env = setup.wind_environment;
    }

    // mod.rs:190-212 and 259-288; Controller::update (controller/mod.rs:39-64) with its
    // step index at 0: updates whenever time >= start_time
    void apply_controller(double time, double time_step, const sbsetup::WindCondition& cond, double ship_velocity,
                          double loading) {
        wind.cond = cond;
        const std::vector<V3> fs = complete_sail_freestream(sim, wind, ship_velocity, time);
        const size_t n = sim.lfm.nr_span_lines();
        const std::vector<V3> ctrl(fs.begin(), fs.begin() + n);
        const auto inputs = controller_input_from_velocity(loading, sim.lfm, ctrl, setup.controller.flow_measurement);
        const auto& c = setup.controller;
        const bool initialization_done = time >= c.start_time;
        const bool time_to_update = 0 % c.time_steps_between_updates == 0;
        if (!(time_to_update && initialization_done)) return;
        for (size_t w = 0; w < c.set_points.size(); ++w)
            sim.lfm.local_wing_angles[w] = new_local_wing_angle(c.set_points[w], inputs[w], time_step);
        sim.lfm.update_global_data_representations();
    }

    // mod.rs:170-188
    StepResult do_step(double time, double time_step, const sbsetup::WindCondition& cond, double ship_velocity) {
        wind.cond = cond;
        const std::vector<V3> fs = complete_sail_freestream(sim, wind, ship_velocity, time);
        return sim.do_step(time, time_step, fs.data(), fs.size());
    }

    // mod.rs:103-122
    StepResult steady_state(const sbsetup::WindCondition& cond, double ship_velocity, double loading) {
        apply_controller(0.0, 1.0, cond, ship_velocity, loading);
        return do_step(0.0, 1.0, cond, ship_velocity);
    }
};

// cstormbird WindCondition -> WindCondition (interfaces/cstormbird/src/wind.rs:15-33)
inline sbsetup::WindCondition power_model_condition(double velocity, double direction) {
    sbsetup::WindCondition c;
    c.direction_coming_from = direction;
    c.velocity_variation.kind = sbsetup::VelocityVariationKind::PowerModel;
    c.velocity_variation.reference_velocity = velocity;
    c.velocity_variation.reference_height = 10.0;
    c.velocity_variation.power_factor = 1.0 / 9.0;
    return c;
}

}  // namespace sbo
