// Stormbird simulation-setup schema: JSON document -> plain settings structs.
//
// This is the drop-in boundary's input format. It mirrors the serde schema of the
// reference's `SimulationBuilder` (stormbird/src/lifting_line/simulation_builder.rs:21-63),
// including the per-field `default = ...` functions and `deny_unknown_fields`:
//   - LineForceModelBuilder   stormbird/src/line_force_model/builder/mod.rs:21-46
//   - WingBuilder             stormbird/src/line_force_model/builder/single_wing.rs:26-44
//   - Foil                    stormbird/src/section_models/foil.rs:43-117, defaults :279-302
//   - SimpleIterative         stormbird/src/lifting_line/solvers/simple_iterative.rs:59-84
//   - QuasiSteadySimpleIterativeBuilder  simple_iterative.rs:21-55 (1000 iterations, d=0.04)
//   - Linearized              stormbird/src/lifting_line/solvers/linearized.rs:18-47
//   - VelocityCorrections     stormbird/src/lifting_line/solvers/velocity_corrections.rs:18-27
//   - DynamicWakeBuilder      stormbird/src/lifting_line/wake/dynamic_wake/builder.rs:37-119
//   - QuasiSteadyWakeSettings stormbird/src/lifting_line/wake/settings.rs:10-45
// Externally tagged enums are accepted in serde's forms: "Variant" for unit variants and
// {"Variant": payload} otherwise. Rust defaults are applied (not the Python builder's).
// Section models other than Foil, and circulation / angle-of-attack corrections other
// than "None", are outside the lifting-line hot path and are rejected with a clear error.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "json_min.hpp"

namespace sbsetup {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTau = 2.0 * kPi;

struct SetupError : std::runtime_error {
    explicit SetupError(const std::string& m) : std::runtime_error(m) {}
};

struct Vec3 { double x = 0.0, y = 0.0, z = 0.0; };

enum class CoreKind : int { Relative = 0, Absolute = 1, NoViscousCore = 2 };
struct CoreLength { CoreKind kind = CoreKind::Relative; double value = 0.1; };

struct Foil {
    double cl_zero_angle = 0.0;
    double cl_initial_slope = kTau;
    double cl_high_order_factor_positive = 0.0;
    double cl_high_order_factor_negative = 0.0;
    double cl_high_order_power = 0.0;
    double cl_max_after_stall = 1.0;
    double cd_min = 0.0;
    double angle_cd_min = 0.0;
    double cd_second_order_factor = 0.0;
    double cd_max_after_stall = 1.0;
    double cd_power_after_stall = 1.6;
    double cdi_correction_factor = 0.0;
    double mean_positive_stall_angle = 20.0 * kPi / 180.0;
    double mean_negative_stall_angle = 20.0 * kPi / 180.0;
    double stall_range = 6.0 * kPi / 180.0;
    double cd_bump_during_stall = 0.0;
    double cd_stall_angle_offset = 0.0;
    double added_mass_factor = 0.0;
};

// RotatingCylinder (section_models/rotating_cylinder.rs:10-61): lift and drag coefficients
// tabulated over the spin ratio. Read for the oracle's rotor test only; the GPU path rejects
// it (parse_setup without allow_rotating_cylinder).
struct RotatingCylinder {
    double revolutions_per_second = 0.0;
    std::vector<double> spin_ratio_data = {0.0, 0.5, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0, 8.0};
    std::vector<double> cl_data = {0.0, 1.22, 2.56, 5.93, 9.10, 10.77, 12.80, 13.71, 16.90};
    std::vector<double> cd_data = {0.457, 0.411, 0.296, 0.093, 0.066, 0.042, 0.064, 0.05, 0.076};
    bool has_wake_angle_data = false;
    std::vector<double> wake_angle_data;
    double added_mass_factor = 0.0;
    double moment_of_inertia_2d = 0.0;
};

struct WingBuilder {
    std::vector<Vec3> section_points;
    std::vector<Vec3> chord_vectors;
    Foil foil;
    bool rotating_cylinder = false;  // the section model is `cylinder`, not `foil`
    RotatingCylinder cylinder;
    bool has_virtual = false;
    std::vector<bool> line_segment_is_virtual;
    bool non_zero_circulation_at_ends[2] = {false, false};
    int64_t nr_sections = -1;  // -1: use the line force model's value
};

enum class RotationType : int { XYZ = 0, YawPitchRoll = 1 };
enum class CoordinateSystem : int { Global = 0, Body = 1 };

struct LineForceModelBuilder {
    std::vector<WingBuilder> wing_builders;
    int64_t nr_sections = 0;
    double density = 1.225;
    RotationType rotation_type = RotationType::XYZ;
    std::vector<double> local_wing_angles;
    Vec3 rotation;
    Vec3 translation;
    CoordinateSystem output_coordinate_system = CoordinateSystem::Global;
    bool include_viscous_lift_in_the_circulation = false;
};

enum class VelocityCorrectionKind : int { NoCorrection = 0, MaxInducedVelocityMagnitudeRatio = 1, FixedMagnitudeEqualToFreestream = 2 };
struct VelocityCorrections { VelocityCorrectionKind kind = VelocityCorrectionKind::NoCorrection; double ratio = 0.0; };

struct SimpleIterative {
    int64_t max_iterations_per_time_step = 40;
    double damping_factor = 0.05;
    double residual_tolerance_absolute = 1e-4;
    double strength_difference_tolerance = 1e-6;
    VelocityCorrections velocity_corrections;
    bool use_raw_circulation_during_iterations = false;
    bool start_with_linearized_solution = false;
    double correction_factor_initial_solution = 1.0;
};

struct Linearized {
    VelocityCorrections velocity_corrections;
    bool disable_viscous_corrections = false;
    bool full_induced_velocity_correction = true;  // FullCorrection (default) vs NoCorrection
};

enum class SolverKind : int { SimpleIterative = 0, Linearized = 1 };
struct Solver { SolverKind kind = SolverKind::SimpleIterative; SimpleIterative si; Linearized lin; };

enum class Symmetry : int { NoSymmetry = 0, X = 1, Y = 2, Z = 3 };
enum class FirstWakePointsDirection : int { Chord = 0, Freestream = 1, ActualVelocity = 2 };

struct DynamicWakeBuilder {
    int64_t nr_panels_per_line_element = 100;
    CoreLength viscous_core_length;
    bool core_sin_increase = false;
    CoreLength sin_last_panel_value;
    double sin_evolution_length_factor = 1.0;
    double first_panel_relative_length = 0.75;
    double last_panel_relative_length = 0.25;
    FirstWakePointsDirection first_wake_points_direction = FirstWakePointsDirection::Chord;
    Symmetry symmetry_condition = Symmetry::NoSymmetry;
    double ratio_of_wake_affected_by_induced_velocities = 0.0;
    double far_field_ratio = 5.0;
    double shape_damping_factor = 0.0;
    bool neglect_self_induced_velocities = false;
    double initial_relative_wake_length = 50.0;
    bool write_wake_data_to_file = false;
    std::string wake_files_folder_path;
};

struct QuasiSteadyWakeSettings {
    double wake_length_factor = 100.0;
    Symmetry symmetry_condition = Symmetry::NoSymmetry;
    CoreLength viscous_core_length;
};

struct Setup {
    LineForceModelBuilder line_force_model;
    bool dynamic = false;
    Solver solver;                   // the built solver (QS builder already applied)
    DynamicWakeBuilder dynamic_wake; // used when dynamic
    QuasiSteadyWakeSettings quasi_steady_wake;  // used when !dynamic
};

namespace detail {

using sbjson::Value;

inline const char* kind_name(const Value& v) {
    switch (v.kind) {
        case Value::Null: return "null";
        case Value::Bool: return "bool";
        case Value::Number: return "number";
        case Value::String: return "string";
        case Value::Arr: return "array";
        case Value::Obj: return "object";
    }
    return "?";
}

[[noreturn]] inline void bad(const std::string& path, const std::string& what) {
    throw SetupError(path + ": " + what);
}

inline double num(const Value& v, const std::string& path) {
    if (!v.is_num()) bad(path, std::string("expected a number, got ") + kind_name(v));
    return v.num;
}

inline int64_t uint_(const Value& v, const std::string& path) {
    double d = num(v, path);
    if (d < 0 || d != std::floor(d) || d > 9.0e15) bad(path, "expected a non-negative integer");
    return static_cast<int64_t>(d);
}

inline bool boolean(const Value& v, const std::string& path) {
    if (!v.is_bool()) bad(path, std::string("expected a bool, got ") + kind_name(v));
    return v.b;
}

inline std::string string_(const Value& v, const std::string& path) {
    if (!v.is_str()) bad(path, std::string("expected a string, got ") + kind_name(v));
    return v.str;
}

inline const sbjson::Object& object(const Value& v, const std::string& path) {
    if (!v.is_obj()) bad(path, std::string("expected an object, got ") + kind_name(v));
    return *v.obj;
}

inline const sbjson::Array& array(const Value& v, const std::string& path) {
    if (!v.is_arr()) bad(path, std::string("expected an array, got ") + kind_name(v));
    return *v.arr;
}

// Walks an object's fields, rejecting unknown and duplicate keys (serde deny_unknown_fields).
template <class F>
inline void fields(const Value& v, const std::string& path, std::initializer_list<const char*> known, F&& on_field,
                   bool deny_unknown = true) {
    const auto& o = object(v, path);
    std::vector<std::string> seen;
    for (const auto& kv : o) {
        bool ok = false;
        for (const char* k : known) if (kv.first == k) { ok = true; break; }
        if (!ok) {
            if (deny_unknown) bad(path, "unknown field `" + kv.first + "`");
            continue;
        }
        for (const auto& s : seen) if (s == kv.first) bad(path, "duplicate field `" + kv.first + "`");
        seen.push_back(kv.first);
        on_field(kv.first, kv.second, path + "." + kv.first);
    }
}

inline void require(const Value& v, const std::string& path, std::initializer_list<const char*> req) {
    const auto& o = object(v, path);
    for (const char* k : req) {
        bool found = false;
        for (const auto& kv : o) if (kv.first == k) { found = true; break; }
        if (!found) bad(path, std::string("missing field `") + k + "`");
    }
}

// Externally tagged enum: returns the variant name and a pointer to the payload (or null).
inline std::string variant(const Value& v, const std::string& path, const Value** payload) {
    *payload = nullptr;
    if (v.is_str()) return v.str;
    const auto& o = object(v, path);
    if (o.size() != 1) bad(path, "expected an externally tagged enum with exactly one variant");
    *payload = &o[0].second;
    return o[0].first;
}

inline Vec3 vec3(const Value& v, const std::string& path) {
    Vec3 r;
    require(v, path, {"x", "y", "z"});
    fields(v, path, {"x", "y", "z"}, [&](const std::string& k, const Value& f, const std::string& p) {
        if (k == "x") r.x = num(f, p);
        else if (k == "y") r.y = num(f, p);
        else r.z = num(f, p);
    }, /*deny_unknown=*/false);
    return r;
}

inline CoreLength core_length(const Value& v, const std::string& path) {
    const Value* payload;
    std::string name = variant(v, path, &payload);
    CoreLength c;
    if (name == "Relative") { if (!payload) bad(path, "Relative needs a value"); c.kind = CoreKind::Relative; c.value = num(*payload, path + ".Relative"); }
    else if (name == "Absolute") { if (!payload) bad(path, "Absolute needs a value"); c.kind = CoreKind::Absolute; c.value = num(*payload, path + ".Absolute"); }
    else if (name == "NoViscousCore") { if (payload) bad(path, "NoViscousCore takes no value"); c.kind = CoreKind::NoViscousCore; c.value = 0.0; }
    else bad(path, "unknown ViscousCoreLength variant `" + name + "`");
    return c;
}

inline Symmetry symmetry(const Value& v, const std::string& path) {
    std::string s = string_(v, path);
    if (s == "NoSymmetry") return Symmetry::NoSymmetry;
    if (s == "X") return Symmetry::X;
    if (s == "Y") return Symmetry::Y;
    if (s == "Z") return Symmetry::Z;
    bad(path, "unknown SymmetryCondition `" + s + "`");
}

inline VelocityCorrections velocity_corrections(const Value& v, const std::string& path) {
    const Value* payload;
    std::string name = variant(v, path, &payload);
    VelocityCorrections c;
    if (name == "NoCorrection") c.kind = VelocityCorrectionKind::NoCorrection;
    else if (name == "MaxInducedVelocityMagnitudeRatio") {
        if (!payload) bad(path, "MaxInducedVelocityMagnitudeRatio needs a value");
        c.kind = VelocityCorrectionKind::MaxInducedVelocityMagnitudeRatio;
        c.ratio = num(*payload, path);
    } else if (name == "FixedMagnitudeEqualToFreestream") c.kind = VelocityCorrectionKind::FixedMagnitudeEqualToFreestream;
    else bad(path, "unknown VelocityCorrections variant `" + name + "`");
    return c;
}

inline Foil foil(const Value& v, const std::string& path) {
    Foil f;
    fields(v, path, {"cl_zero_angle", "cl_initial_slope", "cl_high_order_factor_positive", "cl_high_order_factor_negative",
                     "cl_high_order_power", "cl_max_after_stall", "cd_min", "angle_cd_min", "cd_second_order_factor",
                     "cd_max_after_stall", "cd_power_after_stall", "cdi_correction_factor", "mean_positive_stall_angle",
                     "mean_negative_stall_angle", "stall_range", "cd_bump_during_stall", "cd_stall_angle_offset",
                     "added_mass_factor"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               double d = num(x, p);
               if (k == "cl_zero_angle") f.cl_zero_angle = d;
               else if (k == "cl_initial_slope") f.cl_initial_slope = d;
               else if (k == "cl_high_order_factor_positive") f.cl_high_order_factor_positive = d;
               else if (k == "cl_high_order_factor_negative") f.cl_high_order_factor_negative = d;
               else if (k == "cl_high_order_power") f.cl_high_order_power = d;
               else if (k == "cl_max_after_stall") f.cl_max_after_stall = d;
               else if (k == "cd_min") f.cd_min = d;
               else if (k == "angle_cd_min") f.angle_cd_min = d;
               else if (k == "cd_second_order_factor") f.cd_second_order_factor = d;
               else if (k == "cd_max_after_stall") f.cd_max_after_stall = d;
               else if (k == "cd_power_after_stall") f.cd_power_after_stall = d;
               else if (k == "cdi_correction_factor") f.cdi_correction_factor = d;
               else if (k == "mean_positive_stall_angle") f.mean_positive_stall_angle = d;
               else if (k == "mean_negative_stall_angle") f.mean_negative_stall_angle = d;
               else if (k == "stall_range") f.stall_range = d;
               else if (k == "cd_bump_during_stall") f.cd_bump_during_stall = d;
               else if (k == "cd_stall_angle_offset") f.cd_stall_angle_offset = d;
               else f.added_mass_factor = d;
           });
    return f;
}

inline RotatingCylinder rotating_cylinder(const Value& v, const std::string& path) {
    RotatingCylinder c;
    auto nums = [](const Value& x, const std::string& p) {
        std::vector<double> o;
        const auto& a = array(x, p);
        for (size_t i = 0; i < a.size(); ++i) o.push_back(num(a[i], p + "[" + std::to_string(i) + "]"));
        return o;
    };
    fields(v, path, {"revolutions_per_second", "spin_ratio_data", "cl_data", "cd_data", "wake_angle_data",
                     "added_mass_factor", "moment_of_inertia_2d"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "revolutions_per_second") c.revolutions_per_second = num(x, p);
               else if (k == "spin_ratio_data") c.spin_ratio_data = nums(x, p);
               else if (k == "cl_data") c.cl_data = nums(x, p);
               else if (k == "cd_data") c.cd_data = nums(x, p);
               else if (k == "wake_angle_data") {
                   if (x.is_null()) return;
                   c.has_wake_angle_data = true;
                   c.wake_angle_data = nums(x, p);
               } else if (k == "added_mass_factor") c.added_mass_factor = num(x, p);
               else c.moment_of_inertia_2d = num(x, p);
           });
    if (c.spin_ratio_data.empty() || c.cl_data.size() != c.spin_ratio_data.size() ||
        c.cd_data.size() != c.spin_ratio_data.size())
        bad(path, "spin_ratio_data, cl_data and cd_data must be non-empty and of one length");
    return c;
}

inline WingBuilder wing_builder(const Value& v, const std::string& path, bool allow_rotating_cylinder) {
    WingBuilder w;
    require(v, path, {"section_points", "chord_vectors", "section_model"});
    fields(v, path, {"section_points", "chord_vectors", "section_model", "line_segment_is_virtual",
                     "non_zero_circulation_at_ends", "nr_sections", "input_power_model"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "section_points" || k == "chord_vectors") {
                   auto& dst = (k == "section_points") ? w.section_points : w.chord_vectors;
                   const auto& a = array(x, p);
                   for (size_t i = 0; i < a.size(); ++i) dst.push_back(vec3(a[i], p + "[" + std::to_string(i) + "]"));
               } else if (k == "section_model") {
                   const Value* payload;
                   std::string name = variant(x, p, &payload);
                   if (name == "RotatingCylinder" && allow_rotating_cylinder) {
                       w.rotating_cylinder = true;
                       if (payload) w.cylinder = rotating_cylinder(*payload, p + ".RotatingCylinder");
                       return;
                   }
                   if (name != "Foil")
                       bad(p, "section model `" + name + "` is not supported by the GPU lifting-line path (Foil only)");
                   if (!payload) bad(p, "Foil needs an object");
                   w.foil = foil(*payload, p + ".Foil");
               } else if (k == "line_segment_is_virtual") {
                   if (x.is_null()) return;
                   w.has_virtual = true;
                   for (const auto& e : array(x, p)) w.line_segment_is_virtual.push_back(boolean(e, p));
               } else if (k == "non_zero_circulation_at_ends") {
                   const auto& a = array(x, p);
                   if (a.size() != 2) bad(p, "expected two bools");
                   w.non_zero_circulation_at_ends[0] = boolean(a[0], p);
                   w.non_zero_circulation_at_ends[1] = boolean(a[1], p);
               } else if (k == "nr_sections") {
                   if (!x.is_null()) w.nr_sections = uint_(x, p);
               } else {  // input_power_model
                   const Value* payload;
                   std::string name = variant(x, p, &payload);
                   if (name != "NoPower") bad(p, "input power model `" + name + "` is not supported (NoPower only)");
               }
           });
    if (w.section_points.size() < 2) bad(path, "a wing needs at least two section points");
    if (w.chord_vectors.size() != w.section_points.size()) bad(path, "chord_vectors and section_points differ in length");
    if (w.has_virtual && w.line_segment_is_virtual.size() != w.section_points.size() - 1)
        bad(path, "line_segment_is_virtual needs one entry per segment between section points");
    return w;
}

inline LineForceModelBuilder line_force_model(const Value& v, const std::string& path,
                                              bool allow_rotating_cylinder = false) {
    LineForceModelBuilder b;
    require(v, path, {"wing_builders", "nr_sections"});
    fields(v, path, {"wing_builders", "nr_sections", "density", "circulation_correction", "angle_of_attack_correction",
                     "output_coordinate_system", "rotation_type", "local_wing_angles", "rotation", "translation",
                     "force_calculation_settings"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "wing_builders") {
                   const auto& a = array(x, p);
                   for (size_t i = 0; i < a.size(); ++i) b.wing_builders.push_back(
                       wing_builder(a[i], p + "[" + std::to_string(i) + "]", allow_rotating_cylinder));
               } else if (k == "nr_sections") b.nr_sections = uint_(x, p);
               else if (k == "density") b.density = num(x, p);
               else if (k == "circulation_correction") {
                   const Value* payload;
                   std::string name = variant(x, p, &payload);
                   if (name != "None") bad(p, "circulation correction `" + name + "` is not supported (None only)");
               } else if (k == "angle_of_attack_correction") {
                   const Value* payload;
                   std::string name = variant(x, p, &payload);
                   if (name != "None") bad(p, "angle of attack correction `" + name + "` is not supported (None only)");
               } else if (k == "output_coordinate_system") {
                   std::string s = string_(x, p);
                   if (s == "Global") b.output_coordinate_system = CoordinateSystem::Global;
                   else if (s == "Body") b.output_coordinate_system = CoordinateSystem::Body;
                   else bad(p, "unknown CoordinateSystem `" + s + "`");
               } else if (k == "rotation_type") {
                   std::string s = string_(x, p);
                   if (s == "XYZ") b.rotation_type = RotationType::XYZ;
                   else if (s == "YawPitchRoll") b.rotation_type = RotationType::YawPitchRoll;
                   else bad(p, "unknown RotationType `" + s + "`");
               } else if (k == "local_wing_angles") {
                   for (const auto& e : array(x, p)) b.local_wing_angles.push_back(num(e, p));
               } else if (k == "rotation") b.rotation = vec3(x, p);
               else if (k == "translation") b.translation = vec3(x, p);
               else {  // force_calculation_settings (no deny_unknown_fields in the reference)
                   fields(x, p, {"include_viscous_lift_in_the_circulation"},
                          [&](const std::string&, const Value& y, const std::string& q) {
                              b.include_viscous_lift_in_the_circulation = boolean(y, q);
                          }, /*deny_unknown=*/false);
               }
           });
    if (b.wing_builders.empty()) bad(path, "at least one wing builder is required");
    if (!b.local_wing_angles.empty() && b.local_wing_angles.size() != b.wing_builders.size())
        bad(path, "The number of local wing angles does not match the number of wings.");
    return b;
}

inline SimpleIterative simple_iterative(const Value& v, const std::string& path, bool quasi_steady_builder) {
    SimpleIterative s;
    if (quasi_steady_builder) {
        s.max_iterations_per_time_step = 1000;
        s.damping_factor = 0.04;
        fields(v, path, {"max_iterations_per_time_step", "damping_factor", "residual_tolerance_absolute",
                         "strength_difference_tolerance", "velocity_corrections", "start_with_linearized_solution",
                         "correction_factor_initial_solution"},
               [&](const std::string& k, const Value& x, const std::string& p) {
                   if (k == "max_iterations_per_time_step") s.max_iterations_per_time_step = uint_(x, p);
                   else if (k == "damping_factor") s.damping_factor = num(x, p);
                   else if (k == "residual_tolerance_absolute") s.residual_tolerance_absolute = num(x, p);
                   else if (k == "strength_difference_tolerance") s.strength_difference_tolerance = num(x, p);
                   else if (k == "velocity_corrections") s.velocity_corrections = velocity_corrections(x, p);
                   else if (k == "start_with_linearized_solution") s.start_with_linearized_solution = boolean(x, p);
                   else s.correction_factor_initial_solution = num(x, p);
               });
    } else {
        fields(v, path, {"max_iterations_per_time_step", "damping_factor", "residual_tolerance_absolute",
                         "strength_difference_tolerance", "velocity_corrections", "use_raw_circulation_during_iterations",
                         "start_with_linearized_solution", "correction_factor_initial_solution"},
               [&](const std::string& k, const Value& x, const std::string& p) {
                   if (k == "max_iterations_per_time_step") s.max_iterations_per_time_step = uint_(x, p);
                   else if (k == "damping_factor") s.damping_factor = num(x, p);
                   else if (k == "residual_tolerance_absolute") s.residual_tolerance_absolute = num(x, p);
                   else if (k == "strength_difference_tolerance") s.strength_difference_tolerance = num(x, p);
                   else if (k == "velocity_corrections") s.velocity_corrections = velocity_corrections(x, p);
                   else if (k == "use_raw_circulation_during_iterations") s.use_raw_circulation_during_iterations = boolean(x, p);
                   else if (k == "start_with_linearized_solution") s.start_with_linearized_solution = boolean(x, p);
                   else s.correction_factor_initial_solution = num(x, p);
               });
    }
    return s;
}

inline Linearized linearized(const Value& v, const std::string& path) {
    Linearized l;
    fields(v, path, {"velocity_corrections", "disable_viscous_corrections", "induced_velocity_correction_method"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "velocity_corrections") l.velocity_corrections = velocity_corrections(x, p);
               else if (k == "disable_viscous_corrections") l.disable_viscous_corrections = boolean(x, p);
               else {
                   std::string s = string_(x, p);
                   if (s == "FullCorrection") l.full_induced_velocity_correction = true;
                   else if (s == "NoCorrection") l.full_induced_velocity_correction = false;
                   else bad(p, "unknown InducedVelocityCorrectionMethod `" + s + "`");
               }
           });
    return l;
}

inline Solver solver(const Value& v, const std::string& path, bool quasi_steady) {
    const Value* payload;
    std::string name = variant(v, path, &payload);
    Solver s;
    static const Value empty_obj = [] { Value e; e.kind = Value::Obj; e.obj = std::make_shared<sbjson::Object>(); return e; }();
    const Value& body = payload ? *payload : empty_obj;
    if (name == "SimpleIterative") {
        s.kind = SolverKind::SimpleIterative;
        s.si = simple_iterative(body, path + ".SimpleIterative", quasi_steady);
    } else if (name == "Linearized") {
        s.kind = SolverKind::Linearized;
        s.lin = linearized(body, path + ".Linearized");
    } else bad(path, "unknown solver `" + name + "`");
    return s;
}

inline DynamicWakeBuilder dynamic_wake(const Value& v, const std::string& path) {
    DynamicWakeBuilder w;
    fields(v, path, {"nr_panels_per_line_element", "viscous_core_length", "viscous_core_length_evolution",
                     "first_panel_relative_length", "last_panel_relative_length", "first_wake_points_direction",
                     "symmetry_condition", "ratio_of_wake_affected_by_induced_velocities", "far_field_ratio",
                     "shape_damping_factor", "neglect_self_induced_velocities", "initial_relative_wake_length",
                     "write_wake_data_to_file", "wake_files_folder_path"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "nr_panels_per_line_element") w.nr_panels_per_line_element = uint_(x, p);
               else if (k == "viscous_core_length") w.viscous_core_length = core_length(x, p);
               else if (k == "viscous_core_length_evolution") {
                   const Value* payload;
                   std::string name = variant(x, p, &payload);
                   if (name == "Constant") w.core_sin_increase = false;
                   else if (name == "SinIncrease") {
                       if (!payload) bad(p, "SinIncrease needs an object");
                       w.core_sin_increase = true;
                       require(*payload, p + ".SinIncrease", {"last_panel_value"});
                       fields(*payload, p + ".SinIncrease", {"last_panel_value", "evolution_length_factor"},
                              [&](const std::string& kk, const Value& y, const std::string& q) {
                                  if (kk == "last_panel_value") w.sin_last_panel_value = core_length(y, q);
                                  else w.sin_evolution_length_factor = num(y, q);
                              });
                   } else bad(p, "unknown ViscousCoreLengthEvolution `" + name + "`");
               } else if (k == "first_panel_relative_length") w.first_panel_relative_length = num(x, p);
               else if (k == "last_panel_relative_length") w.last_panel_relative_length = num(x, p);
               else if (k == "first_wake_points_direction") {
                   std::string s = string_(x, p);
                   if (s == "Chord") w.first_wake_points_direction = FirstWakePointsDirection::Chord;
                   else if (s == "Freestream") w.first_wake_points_direction = FirstWakePointsDirection::Freestream;
                   else if (s == "ActualVelocity") w.first_wake_points_direction = FirstWakePointsDirection::ActualVelocity;
                   else bad(p, "unknown FirstWakePointsDirection `" + s + "`");
               } else if (k == "symmetry_condition") w.symmetry_condition = symmetry(x, p);
               else if (k == "ratio_of_wake_affected_by_induced_velocities") w.ratio_of_wake_affected_by_induced_velocities = num(x, p);
               else if (k == "far_field_ratio") w.far_field_ratio = num(x, p);
               else if (k == "shape_damping_factor") w.shape_damping_factor = num(x, p);
               else if (k == "neglect_self_induced_velocities") w.neglect_self_induced_velocities = boolean(x, p);
               else if (k == "initial_relative_wake_length") w.initial_relative_wake_length = num(x, p);
               else if (k == "write_wake_data_to_file") w.write_wake_data_to_file = boolean(x, p);
               else w.wake_files_folder_path = string_(x, p);
           });
    if (w.nr_panels_per_line_element < 1) bad(path + ".nr_panels_per_line_element", "must be at least 1");
    return w;
}

inline QuasiSteadyWakeSettings quasi_steady_wake(const Value& v, const std::string& path) {
    QuasiSteadyWakeSettings w;
    fields(v, path, {"wake_length_factor", "symmetry_condition", "viscous_core_length"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "wake_length_factor") w.wake_length_factor = num(x, p);
               else if (k == "symmetry_condition") w.symmetry_condition = symmetry(x, p);
               else w.viscous_core_length = core_length(x, p);
           });
    return w;
}

}  // namespace detail

// Parses a `SimulationBuilder` JSON document (simulation_builder.rs:62-88). Rotating-cylinder
// section models are accepted only with allow_rotating_cylinder (the oracle's rotor test).
inline Setup parse_setup(const std::string& text, bool allow_rotating_cylinder = false) {
    using namespace detail;
    sbjson::Value root;
    try {
        root = sbjson::parse(text);
    } catch (const sbjson::ParseError& e) {
        throw SetupError(e.what());
    }
    Setup s;
    bool have_settings = false;
    require(root, "SimulationBuilder", {"line_force_model"});
    fields(root, "SimulationBuilder", {"line_force_model", "simulation_settings"},
           [&](const std::string& k, const Value& x, const std::string& p) {
               if (k == "line_force_model") {
                   s.line_force_model = line_force_model(x, p, allow_rotating_cylinder);
                   return;
               }
               have_settings = true;
               const Value* payload;
               std::string name = variant(x, p, &payload);
               static const Value empty_obj = [] { Value e; e.kind = Value::Obj; e.obj = std::make_shared<sbjson::Object>(); return e; }();
               const Value& body = payload ? *payload : empty_obj;
               if (name == "QuasiSteady") {
                   s.dynamic = false;
                   s.solver.kind = SolverKind::Linearized;  // QuasiSteadySolverBuilder default (solvers/mod.rs:38-42)
                   fields(body, p + ".QuasiSteady", {"solver", "wake"},
                          [&](const std::string& kk, const Value& y, const std::string& q) {
                              if (kk == "solver") s.solver = solver(y, q, /*quasi_steady=*/true);
                              else s.quasi_steady_wake = quasi_steady_wake(y, q);
                          });
               } else if (name == "Dynamic") {
                   s.dynamic = true;
                   s.solver.kind = SolverKind::SimpleIterative;  // Solver default (solvers/mod.rs:26-30)
                   fields(body, p + ".Dynamic", {"solver", "wake"},
                          [&](const std::string& kk, const Value& y, const std::string& q) {
                              if (kk == "solver") s.solver = solver(y, q, /*quasi_steady=*/false);
                              else s.dynamic_wake = dynamic_wake(y, q);
                          });
               } else bad(p, "unknown SimulationSettings variant `" + name + "`");
           });
    if (!have_settings) {  // SimulationSettings default: QuasiSteady with default settings
        s.dynamic = false;
        s.solver.kind = SolverKind::Linearized;
    }
    return s;
}

}  // namespace sbsetup
