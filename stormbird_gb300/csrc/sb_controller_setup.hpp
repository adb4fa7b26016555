// Stormbird controller and CompleteSailModel schema: JSON -> plain settings structs.
//
// Follows the reference's serde definitions and defaults:
//   CompleteSailModelBuilder  stormbird/src/lifting_line/complete_sail_model/builder.rs:19-24
//                             (deny_unknown_fields; lifting_line_simulation, wind_environment
//                             and controller all required)
//   ControllerBuilder         controller/builder.rs:17-30 (deny_unknown_fields;
//                             time_steps_between_updates 1, start_time 0,
//                             moving_average_window_size accepted and unused, as in build())
//   ControllerSetPoints       controller/set_points.rs:58-75 (deny_unknown_fields)
//   InternalStateType         set_points.rs:34-39 (Generic | {"SpinRatio": {diameter, max_rps}})
//   FlowMeasurementSettings   controller/measurements.rs:39-48 (deny_unknown_fields)
//   MeasurementSettings       measurements.rs:28-37 (Mean | Max | Min, start_index, end_offset)
#pragma once

#include <string>
#include <vector>

#include "sb_wind_setup.hpp"

namespace sbsetup {

enum class MeasurementType : int { Mean = 0, Max = 1, Min = 2 };

struct MeasurementSettings {
    MeasurementType type = MeasurementType::Mean;
    uint64_t start_index = 0;
    uint64_t end_offset = 0;
};

struct FlowMeasurementSettings {
    MeasurementSettings angle_of_attack, wind_direction, wind_velocity;
};

struct ControllerSetPoints {
    std::vector<double> apparent_wind_directions;
    bool has_angle_of_attack = false;
    std::vector<double> angle_of_attack;
    bool has_internal_state = false;
    std::vector<double> internal_state;
    bool spin_ratio = false;  // InternalStateType::SpinRatio
    double spin_diameter = 0.0, spin_max_rps = 0.0;
    bool use_effective_angle_of_attack = false;
    bool has_max_local_wing_angle_change_rate = false;
    double max_local_wing_angle_change_rate = 0.0;
    bool has_max_internal_section_state_change_rate = false;
    double max_internal_section_state_change_rate = 0.0;
};

struct ControllerSettings {
    std::vector<ControllerSetPoints> set_points;
    FlowMeasurementSettings flow_measurement;
    uint64_t time_steps_between_updates = 1;
    double start_time = 0.0;
    bool use_input_velocity_for_apparent_wind_direction = false;
};

struct CompleteSailModelSetup {
    std::string lifting_line_json;  // the SimulationBuilder document, re-serialised
    std::string wind_environment_json;
    WindEnvironment wind_environment;
    ControllerSettings controller;
};

namespace detail {

inline MeasurementSettings measurement_settings(const Value& v, const std::string& path) {
    MeasurementSettings m;
    fields(v, path, {"measurement_type", "start_index", "end_offset"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "measurement_type") {
                   const Value* payload;
                   const std::string name = variant(f, p, &payload);
                   if (name == "Mean") m.type = MeasurementType::Mean;
                   else if (name == "Max") m.type = MeasurementType::Max;
                   else if (name == "Min") m.type = MeasurementType::Min;
                   else bad(p, "unknown MeasurementType `" + name + "`");
               } else if (k == "start_index") {
                   m.start_index = uint_(f, p);
               } else {
                   m.end_offset = uint_(f, p);
               }
           }, /*deny_unknown=*/false);
    return m;
}

inline ControllerSetPoints controller_set_points(const Value& v, const std::string& path) {
    ControllerSetPoints s;
    require(v, path, {"apparent_wind_directions_data"});
    fields(v, path,
           {"apparent_wind_directions_data", "angle_of_attack_data", "section_model_internal_state_data",
            "internal_state_type", "use_effective_angle_of_attack", "max_local_wing_angle_change_rate",
            "max_internal_section_state_change_rate"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "apparent_wind_directions_data") {
                   s.apparent_wind_directions = numbers(f, p);
               } else if (k == "angle_of_attack_data") {
                   s.has_angle_of_attack = !f.is_null();
                   if (s.has_angle_of_attack) s.angle_of_attack = numbers(f, p);
               } else if (k == "section_model_internal_state_data") {
                   s.has_internal_state = !f.is_null();
                   if (s.has_internal_state) s.internal_state = numbers(f, p);
               } else if (k == "internal_state_type") {
                   const Value* payload;
                   const std::string name = variant(f, p, &payload);
                   if (name == "Generic") {
                       s.spin_ratio = false;
                   } else if (name == "SpinRatio") {
                       if (!payload) bad(p, "SpinRatio needs diameter and max_rps");
                       s.spin_ratio = true;
                       require(*payload, p + ".SpinRatio", {"diameter", "max_rps"});
                       fields(*payload, p + ".SpinRatio", {"diameter", "max_rps"},
                              [&](const std::string& kk, const Value& g, const std::string& q) {
                                  if (kk == "diameter") s.spin_diameter = num(g, q);
                                  else s.spin_max_rps = num(g, q);
                              }, /*deny_unknown=*/false);
                   } else {
                       bad(p, "unknown InternalStateType `" + name + "`");
                   }
               } else if (k == "use_effective_angle_of_attack") {
                   s.use_effective_angle_of_attack = boolean(f, p);
               } else if (k == "max_local_wing_angle_change_rate") {
                   s.has_max_local_wing_angle_change_rate = !f.is_null();
                   if (s.has_max_local_wing_angle_change_rate) s.max_local_wing_angle_change_rate = num(f, p);
               } else {
                   s.has_max_internal_section_state_change_rate = !f.is_null();
                   if (s.has_max_internal_section_state_change_rate)
                       s.max_internal_section_state_change_rate = num(f, p);
               }
           });
    // linear_interpolation (stormath/src/interpolation.rs:24-27) needs equal, non-empty data
    if (s.apparent_wind_directions.empty()) bad(path, "apparent_wind_directions_data is empty");
    if (s.has_angle_of_attack && s.angle_of_attack.size() != s.apparent_wind_directions.size())
        bad(path, "angle_of_attack_data and apparent_wind_directions_data differ in length");
    if (s.has_internal_state && s.internal_state.size() != s.apparent_wind_directions.size())
        bad(path, "section_model_internal_state_data and apparent_wind_directions_data differ in length");
    return s;
}

inline ControllerSettings controller_settings(const Value& v, const std::string& path) {
    ControllerSettings c;
    require(v, path, {"set_points"});
    fields(v, path,
           {"set_points", "flow_measurement_settings", "time_steps_between_updates", "start_time",
            "moving_average_window_size", "use_input_velocity_for_apparent_wind_direction"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "set_points") {
                   const auto& a = array(f, p);
                   for (size_t i = 0; i < a.size(); ++i)
                       c.set_points.push_back(controller_set_points(a[i], p + "[" + std::to_string(i) + "]"));
               } else if (k == "flow_measurement_settings") {
                   fields(f, p, {"angle_of_attack", "wind_direction", "wind_velocity"},
                          [&](const std::string& kk, const Value& g, const std::string& q) {
                              if (kk == "angle_of_attack") c.flow_measurement.angle_of_attack = measurement_settings(g, q);
                              else if (kk == "wind_direction") c.flow_measurement.wind_direction = measurement_settings(g, q);
                              else c.flow_measurement.wind_velocity = measurement_settings(g, q);
                          });
               } else if (k == "time_steps_between_updates") {
                   c.time_steps_between_updates = uint_(f, p);
                   // Controller::update takes the index modulo this value (controller/mod.rs:46)
                   if (c.time_steps_between_updates == 0) bad(p, "must be at least 1");
               } else if (k == "start_time") {
                   c.start_time = num(f, p);
               } else if (k == "moving_average_window_size") {
                   if (!f.is_null()) (void)uint_(f, p);
               } else {
                   c.use_input_velocity_for_apparent_wind_direction = boolean(f, p);
               }
           });
    return c;
}

}  // namespace detail

// Parses a `CompleteSailModelBuilder` JSON document.
inline CompleteSailModelSetup parse_complete_sail_model(const std::string& text) {
    using namespace detail;
    const Value root = parse_document(text);
    CompleteSailModelSetup s;
    require(root, "CompleteSailModelBuilder", {"lifting_line_simulation", "wind_environment", "controller"});
    fields(root, "CompleteSailModelBuilder", {"lifting_line_simulation", "wind_environment", "controller"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "lifting_line_simulation") {
                   if (!f.is_obj()) bad(p, "expected an object");
                   s.lifting_line_json = sbjson::dump(f);
               } else if (k == "wind_environment") {
                   if (!f.is_obj()) bad(p, "expected an object");
                   s.wind_environment_json = sbjson::dump(f);
                   s.wind_environment = parse_wind_environment(s.wind_environment_json);
               } else {
                   s.controller = controller_settings(f, p);
               }
           });
    return s;
}

}  // namespace sbsetup
