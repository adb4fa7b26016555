// ORACLE — TEST INFRASTRUCTURE ONLY (see sb_oracle.hpp).
//
// f64 restatement of the reference's wind model as CompleteSailModel uses it to make the
// freestream of a lifting-line simulation (stormbird/src/lifting_line/complete_sail_model/
// mod.rs:213-257): true wind from a WindCondition (direction, height profile, gust spectra)
// in a WindEnvironment (directions, water plane, inflow corrections), plus the ship's
// linear velocity, at every freestream point; inflow corrections at the control points.
#pragma once

#include <cmath>
#include <vector>

#include "../stormbird_gb300/csrc/sb_wind_setup.hpp"
#include "sb_oracle.hpp"

namespace sbo {

inline V3 to_v3(const sbsetup::Vec3& v) { return {v.x, v.y, v.z}; }

// discretized_spectrum.rs:38-46
inline double spectrum_value(const sbsetup::Spectrum& s, double time) {
    double out = 0.0;
    for (size_t i = 0; i < s.frequencies.size(); ++i)
        out += s.amplitudes[i] * std::sin(TAU * s.frequencies[i] * time + s.phases[i]);
    return out;
}

// logarithmic_model.rs:56-110
inline double log_model_velocity(const sbsetup::VelocityVariation& m, double height) {
    const double scale = m.friction_velocity / m.von_karman_constant;
    double neutral = 0.0;
    if (!(m.surface_roughness <= 0.0 || height <= 0.0)) neutral = scale * std::log(height / m.surface_roughness);
    double unscaled = 0.0;
    if (m.has_obukhov_length) {
        const double length = m.obukhov_length;
        const double zeta = height / length;
        if (length > 0.0) {
            unscaled = -m.stable_coefficient * zeta;
        } else {
            const double x = std::pow(1.0 - m.unstable_coefficient * zeta, 0.25);
            const double first = 2.0 * std::log((1.0 + x) / 2.0);
            const double second = std::log((1.0 + x * x) / 2.0);
            const double third = -2.0 * std::atan(x) + PI / 2.0;
            unscaled = first + second + third;
        }
    }
    return neutral - unscaled * scale;
}

// velocity_variation/mod.rs:27-33, power_model.rs:31-47
inline double velocity_at_height(const sbsetup::VelocityVariation& v, double height) {
    switch (v.kind) {
        case sbsetup::VelocityVariationKind::Constant: return v.constant;
        case sbsetup::VelocityVariationKind::PowerModel: {
            const double f = v.power_factor > 0.0 ? std::pow(height / v.reference_height, v.power_factor) : 1.0;
            return v.reference_velocity * f;
        }
        case sbsetup::VelocityVariationKind::LogarithmicModel: return log_model_velocity(v, height);
    }
    return 0.0;
}

struct WindModel {
    sbsetup::WindEnvironment env;
    sbsetup::WindCondition cond;

    V3 up() const { return to_v3(env.up_direction); }

    // environment.rs:91-96
    double height_from_location(V3 p) const { return std::max(dot(p, up()) - env.water_plane_height, 0.0); }

    // environment.rs:99-105
    V3 true_wind_direction_vector() const {
        return rotate_around_axis(to_v3(env.zero_direction_vector), cond.direction_coming_from, to_v3(env.wind_rotation_axis));
    }

    // environment.rs:131-155 + 175-188 (wind_condition/mod.rs:58-87)
    V3 unsteady_apparent_wind(V3 location, V3 linear_velocity, double time) const {
        const double h = height_from_location(location);
        double parallel = velocity_at_height(cond.velocity_variation, h);
        if (cond.parallel_gust.present) parallel += spectrum_value(cond.parallel_gust, time);
        const V3 pdir = true_wind_direction_vector();
        const double perpendicular = cond.perpendicular_gust.present ? spectrum_value(cond.perpendicular_gust, time) : 0.0;
        const V3 perp_dir = cross(up(), pdir);
        const double vertical = cond.vertical_gust.present ? spectrum_value(cond.vertical_gust, time) : 0.0;
        const V3 true_wind = parallel * pdir + perpendicular * perp_dir + vertical * up();
        return true_wind + linear_velocity;
    }

    // environment.rs:273-292 (steady true wind, environment.rs:158-166)
    double apparent_wind_direction(V3 linear_velocity, double height) const {
        const V3 location = height * up();
        const double v = velocity_at_height(cond.velocity_variation, height_from_location(location));
        const V3 true_wind = v * true_wind_direction_vector();
        return signed_angle_between(to_v3(env.zero_direction_vector), true_wind + linear_velocity,
                                    to_v3(env.wind_rotation_axis));
    }

    // inflow_corrections.rs:21-44, 54-95
    V3 corrected_velocity(size_t wing, double direction, double height, V3 velocity) const {
        const auto& ic = env.inflow_corrections;
        std::vector<V3> corrected;
        for (size_t d = 0; d < ic.apparent_wind_directions.size(); ++d) {
            const auto& c = ic.corrections[d];
            const auto r = c.wing_indices.at(wing);
            const std::vector<double> hs(c.height_values.begin() + r.first, c.height_values.begin() + r.second);
            const std::vector<double> ms(c.magnitude_corrections.begin() + r.first, c.magnitude_corrections.begin() + r.second);
            const std::vector<double> as(c.angle_corrections.begin() + r.first, c.angle_corrections.begin() + r.second);
            const double mag = linear_interpolation(height, hs, ms);
            const double ang = linear_interpolation(height, hs, as);
            corrected.push_back(mag * rotate_around_axis(velocity, ang, up()));
        }
        return linear_interpolation(direction, ic.apparent_wind_directions, corrected);
    }
};

// complete_sail_model/mod.rs:213-257: the freestream at every freestream point of `sim`
// (control points, then wake points) for the ship moving at `ship_velocity` along the
// zero direction, with the inflow corrections applied at the control points.
inline std::vector<V3> complete_sail_freestream(const Simulation& sim, const WindModel& w, double ship_velocity,
                                                double time) {
    const std::vector<V3> points = sim.freestream_points();
    const V3 linear = ship_velocity * to_v3(w.env.zero_direction_vector);
    std::vector<V3> out(points.size());
    for (size_t i = 0; i < points.size(); ++i) out[i] = w.unsteady_apparent_wind(points[i], linear, time);
    if (w.env.inflow_corrections.present) {
        const double direction = w.apparent_wind_direction(linear, 10.0);
        const auto& lfm = sim.lfm;
        for (size_t wing = 0; wing < lfm.wing_indices.size(); ++wing)
            for (size_t i = lfm.wing_indices[wing].start; i < lfm.wing_indices[wing].end; ++i) {
                const double h = dot(lfm.ctrl_points_global[i], w.up());
                out[i] = w.corrected_velocity(wing, direction, h, out[i]);
            }
    }
    return out;
}

}  // namespace sbo
