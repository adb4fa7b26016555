// Stormbird wind schema: `WindEnvironment` and `WindCondition` JSON -> plain settings structs.
//
// Follows the reference's serde definitions and defaults:
//   WindEnvironment      stormbird/src/wind/environment.rs:21-55 (deny_unknown_fields; every
//                        field defaulted: up (0,0,1), rotation axis (0,0,1), zero direction
//                        (1,0,0), water plane 0, no inflow corrections)
//   InflowCorrections    wind/inflow_corrections.rs:13-19, 47-51
//   WindCondition        wind/wind_condition/mod.rs:19-39 (gusts optional)
//   VelocityVariation    wind/wind_condition/velocity_variation/mod.rs:13-23 (externally tagged)
//   PowerModel           velocity_variation/power_model.rs:8-29 (height 10, factor 1/9)
//   LogarithmicModel     velocity_variation/logarithmic_model.rs:8-46 (kappa 0.41, 6.0, 19.3)
//   DiscretizedSpectrum  wind/wind_condition/discretized_spectrum.rs:11-20
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "sb_setup.hpp"

namespace sbsetup {

struct Spectrum {
    bool present = false;
    std::vector<double> frequencies, amplitudes, phases;
};

enum class VelocityVariationKind : int { Constant = 0, PowerModel = 1, LogarithmicModel = 2 };

struct VelocityVariation {
    VelocityVariationKind kind = VelocityVariationKind::Constant;
    double constant = 0.0;
    // PowerModel
    double reference_velocity = 0.0, reference_height = 10.0, power_factor = 1.0 / 9.0;
    // LogarithmicModel
    double friction_velocity = 0.0, surface_roughness = 0.0;
    bool has_obukhov_length = false;
    double obukhov_length = 0.0;
    double von_karman_constant = 0.41, stable_coefficient = 6.0, unstable_coefficient = 19.3;
};

struct WindCondition {
    double direction_coming_from = 0.0;
    VelocityVariation velocity_variation;
    Spectrum parallel_gust, perpendicular_gust, vertical_gust;
};

struct InflowCorrectionsSingleDirection {
    std::vector<double> height_values, magnitude_corrections, angle_corrections;
    std::vector<std::pair<int64_t, int64_t>> wing_indices;  // [start, end) into the three arrays
};

struct InflowCorrections {
    bool present = false;
    std::vector<double> apparent_wind_directions;
    std::vector<InflowCorrectionsSingleDirection> corrections;
};

struct WindEnvironment {
    Vec3 up_direction{0.0, 0.0, 1.0};
    Vec3 wind_rotation_axis{0.0, 0.0, 1.0};
    Vec3 zero_direction_vector{1.0, 0.0, 0.0};
    double water_plane_height = 0.0;
    InflowCorrections inflow_corrections;
};

namespace detail {

inline std::vector<double> numbers(const Value& v, const std::string& path) {
    std::vector<double> out;
    const auto& a = array(v, path);
    for (size_t i = 0; i < a.size(); ++i) out.push_back(num(a[i], path + "[" + std::to_string(i) + "]"));
    return out;
}

inline Spectrum spectrum(const Value& v, const std::string& path) {
    Spectrum s;
    if (v.kind == Value::Null) return s;  // Option::None
    s.present = true;
    require(v, path, {"frequencies", "amplitudes", "phases"});
    fields(v, path, {"frequencies", "amplitudes", "phases"}, [&](const std::string& k, const Value& f, const std::string& p) {
        if (k == "frequencies") s.frequencies = numbers(f, p);
        else if (k == "amplitudes") s.amplitudes = numbers(f, p);
        else s.phases = numbers(f, p);
    }, /*deny_unknown=*/false);
    if (s.amplitudes.size() != s.frequencies.size() || s.phases.size() != s.frequencies.size())
        bad(path, "frequencies, amplitudes and phases must have the same length");
    return s;
}

inline VelocityVariation velocity_variation(const Value& v, const std::string& path) {
    const Value* payload;
    std::string name = variant(v, path, &payload);
    VelocityVariation w;
    if (!payload) bad(path, "VelocityVariation `" + name + "` needs a value");
    if (name == "Constant") {
        w.kind = VelocityVariationKind::Constant;
        w.constant = num(*payload, path + ".Constant");
    } else if (name == "PowerModel") {
        w.kind = VelocityVariationKind::PowerModel;
        const std::string p = path + ".PowerModel";
        require(*payload, p, {"reference_velocity"});
        fields(*payload, p, {"reference_velocity", "reference_height", "power_factor"},
               [&](const std::string& k, const Value& f, const std::string& q) {
                   if (k == "reference_velocity") w.reference_velocity = num(f, q);
                   else if (k == "reference_height") w.reference_height = num(f, q);
                   else w.power_factor = num(f, q);
               }, /*deny_unknown=*/false);
    } else if (name == "LogarithmicModel") {
        w.kind = VelocityVariationKind::LogarithmicModel;
        const std::string p = path + ".LogarithmicModel";
        require(*payload, p, {"friction_velocity", "surface_roughness"});
        fields(*payload, p,
               {"friction_velocity", "surface_roughness", "obukhov_length", "von_karman_constant", "stable_coefficient",
                "unstable_coefficient"},
               [&](const std::string& k, const Value& f, const std::string& q) {
                   if (k == "friction_velocity") w.friction_velocity = num(f, q);
                   else if (k == "surface_roughness") w.surface_roughness = num(f, q);
                   else if (k == "obukhov_length") {
                       w.has_obukhov_length = f.kind != Value::Null;
                       if (w.has_obukhov_length) w.obukhov_length = num(f, q);
                   } else if (k == "von_karman_constant") w.von_karman_constant = num(f, q);
                   else if (k == "stable_coefficient") w.stable_coefficient = num(f, q);
                   else w.unstable_coefficient = num(f, q);
               }, /*deny_unknown=*/false);
    } else {
        bad(path, "unknown VelocityVariation variant `" + name + "`");
    }
    return w;
}

inline InflowCorrections inflow_corrections(const Value& v, const std::string& path) {
    InflowCorrections c;
    if (v.kind == Value::Null) return c;
    c.present = true;
    require(v, path, {"apparent_wind_directions", "corrections"});
    fields(v, path, {"apparent_wind_directions", "corrections"}, [&](const std::string& k, const Value& f, const std::string& p) {
        if (k == "apparent_wind_directions") {
            c.apparent_wind_directions = numbers(f, p);
            return;
        }
        const auto& a = array(f, p);
        for (size_t i = 0; i < a.size(); ++i) {
            const std::string q = p + "[" + std::to_string(i) + "]";
            InflowCorrectionsSingleDirection d;
            require(a[i], q, {"height_values", "magnitude_corrections", "angle_corrections", "wing_indices"});
            fields(a[i], q, {"height_values", "magnitude_corrections", "angle_corrections", "wing_indices"},
                   [&](const std::string& kk, const Value& g, const std::string& r) {
                       if (kk == "height_values") d.height_values = numbers(g, r);
                       else if (kk == "magnitude_corrections") d.magnitude_corrections = numbers(g, r);
                       else if (kk == "angle_corrections") d.angle_corrections = numbers(g, r);
                       else {
                           const auto& ranges = array(g, r);
                           for (size_t j = 0; j < ranges.size(); ++j) {
                               const std::string rr = r + "[" + std::to_string(j) + "]";
                               require(ranges[j], rr, {"start", "end"});
                               int64_t s = 0, e = 0;
                               fields(ranges[j], rr, {"start", "end"}, [&](const std::string& kr, const Value& h, const std::string& pr) {
                                   if (kr == "start") s = uint_(h, pr);
                                   else e = uint_(h, pr);
                               });
                               d.wing_indices.push_back({s, e});
                           }
                       }
                   }, /*deny_unknown=*/false);
            const size_t n = d.height_values.size();
            if (d.magnitude_corrections.size() != n || d.angle_corrections.size() != n)
                bad(q, "height, magnitude and angle arrays must have the same length");
            for (const auto& r : d.wing_indices)
                if (r.first >= r.second || static_cast<size_t>(r.second) > n) bad(q, "wing index range outside the arrays");
            c.corrections.push_back(d);
        }
    }, /*deny_unknown=*/false);
    if (c.corrections.size() != c.apparent_wind_directions.size())
        bad(path, "one set of corrections per apparent wind direction is needed");
    if (c.apparent_wind_directions.empty()) bad(path, "no apparent wind directions");
    return c;
}

inline sbjson::Value parse_document(const std::string& text) {
    try {
        return sbjson::parse(text);
    } catch (const sbjson::ParseError& e) {
        throw SetupError(e.what());
    }
}

}  // namespace detail

inline WindEnvironment parse_wind_environment(const std::string& text) {
    using namespace detail;
    const Value root = parse_document(text);
    WindEnvironment w;
    fields(root, "WindEnvironment",
           {"up_direction", "wind_rotation_axis", "zero_direction_vector", "water_plane_height", "inflow_corrections"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "up_direction") w.up_direction = vec3(f, p);
               else if (k == "wind_rotation_axis") w.wind_rotation_axis = vec3(f, p);
               else if (k == "zero_direction_vector") w.zero_direction_vector = vec3(f, p);
               else if (k == "water_plane_height") w.water_plane_height = num(f, p);
               else w.inflow_corrections = inflow_corrections(f, p);
           });
    return w;
}

inline WindCondition parse_wind_condition(const std::string& text) {
    using namespace detail;
    const Value root = parse_document(text);
    WindCondition c;
    require(root, "WindCondition", {"direction_coming_from", "velocity_variation"});
    fields(root, "WindCondition",
           {"direction_coming_from", "velocity_variation", "parallel_gust", "perpendicular_gust", "vertical_gust"},
           [&](const std::string& k, const Value& f, const std::string& p) {
               if (k == "direction_coming_from") c.direction_coming_from = num(f, p);
               else if (k == "velocity_variation") c.velocity_variation = velocity_variation(f, p);
               else if (k == "parallel_gust") c.parallel_gust = spectrum(f, p);
               else if (k == "perpendicular_gust") c.perpendicular_gust = spectrum(f, p);
               else c.vertical_gust = spectrum(f, p);
           }, /*deny_unknown=*/false);
    return c;
}

}  // namespace sbsetup
