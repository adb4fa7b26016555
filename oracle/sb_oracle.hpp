// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A CPU, f64 restatement of the reference's lifting-line hot path, used as the checker
// for the GPU library and as the timed CPU baseline. Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load it. The product library never links it.
//
// The reference (NTNU-IMT/stormbird, Rust) cannot be compiled in this environment (no
// Rust toolchain), so this file restates its algorithm function by function, in the same
// floating-point operation order, each citing the reference file:line it follows.
// Compiled with -ffp-contract=off so that no multiply-add is fused, as in the Rust build.
// Parity of this restatement with the Rust binary itself is pinned by the reference's
// own unit and integration tests (ported in tests/test_oracle_reference_tests.py); no
// stored golden vectors exist in the reference.
//
// The JSON setup is decoded by the library's schema reader (stormbird_gb300/csrc/
// sb_setup.hpp); only parsing is shared — every computation below is restated here.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../stormbird_gb300/csrc/sb_setup.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace sbo {

constexpr double PI = 3.14159265358979323846;
constexpr double TAU = 2.0 * PI;
constexpr double MIN_POSITIVE = 2.2250738585072014e-308;  // f64::MIN_POSITIVE

// ---------------------------------------------------------------------------------------
// SpatialVector (stormath/src/spatial_vector/*.rs)
// ---------------------------------------------------------------------------------------
struct V3 {
    double x = 0.0, y = 0.0, z = 0.0;
    V3() = default;
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3& operator-=(V3& a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }

// vector_math.rs:11-13
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// vector_math.rs:18-20
inline double length_squared(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// vector_math.rs:24-26
inline double length(V3 a) { return std::sqrt(length_squared(a)); }
// vector_math.rs:30-45
inline V3 normalize(V3 a) {
    double l = length(a);
    if (l > 0.0) return {a.x / l, a.y / l, a.z / l};
    return {};
}
// vector_math.rs:55-61
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// vector_math.rs:65-79
inline double absolute_angle_between(V3 a, V3 b) {
    double al = length_squared(a), bl = length_squared(b);
    if (al == 0.0 || bl == 0.0) return 0.0;
    double c = dot(a, b) / std::sqrt(al * bl);
    c = std::min(std::max(c, -1.0), 1.0);
    return std::acos(c);
}
// vector_math.rs:85-95
inline double signed_angle_between(V3 a, V3 b, V3 axis) {
    double triple = dot(a, cross(b, axis));
    double ang = absolute_angle_between(a, b);
    return triple > 0.0 ? ang : -ang;
}
// vector_math.rs:99-103
inline V3 project(V3 a, V3 onto) {
    V3 n = normalize(onto);
    return n * dot(a, n);
}
// Rust f64::signum (+0.0 -> 1, -0.0 -> -1)
inline double signum(double v) { return std::isnan(v) ? v : std::copysign(1.0, v); }

// transformations.rs:139-150 (Rodrigues)
inline V3 rotate_around_axis(V3 v, double angle, V3 axis) {
    V3 n = normalize(axis);
    double c = std::cos(angle), s = std::sin(angle);
    V3 t1 = v * c;
    V3 t2 = cross(n, v) * s;
    V3 t3 = n * dot(n, v) * (1.0 - c);
    return t1 + t2 + t3;
}
// transformations.rs:182-207
inline V3 rotate_xyz(V3 v, V3 r) {
    V3 n = v;
    if (r.x != 0.0) {
        double ty = n.y, tz = n.z;
        n.y = ty * std::cos(r.x) - tz * std::sin(r.x);
        n.z = ty * std::sin(r.x) + tz * std::cos(r.x);
    }
    if (r.y != 0.0) {
        double tx = n.x, tz = n.z;
        n.x = tx * std::cos(r.y) + tz * std::sin(r.y);
        n.z = -tx * std::sin(r.y) + tz * std::cos(r.y);
    }
    if (r.z != 0.0) {
        double tx = n.x, ty = n.y;
        n.x = tx * std::cos(r.z) - ty * std::sin(r.z);
        n.y = tx * std::sin(r.z) + ty * std::cos(r.z);
    }
    return n;
}
// transformations.rs:211-224
inline V3 rotate_yaw_pitch_roll(V3 v, V3 r) {
    V3 yaw{0, 0, 1};
    V3 pitch = rotate_around_axis(V3{0, 1, 0}, r.z, yaw);
    V3 roll = rotate_around_axis(rotate_around_axis(V3{1, 0, 0}, r.z, yaw), r.y, pitch);
    return rotate_around_axis(rotate_around_axis(rotate_around_axis(v, r.z, yaw), r.y, pitch), r.x, roll);
}
// transformations.rs:152-157
inline V3 rotate(V3 v, V3 r, sbsetup::RotationType t) {
    return t == sbsetup::RotationType::XYZ ? rotate_xyz(v, r) : rotate_yaw_pitch_roll(v, r);
}
// transformations.rs:233-265
inline V3 in_rotated_coordinate_system(V3 v, V3 r, sbsetup::RotationType t) {
    V3 ax = rotate(V3{1, 0, 0}, r, t), ay = rotate(V3{0, 1, 0}, r, t), az = rotate(V3{0, 0, 1}, r, t);
    return {dot(v, ax), dot(v, ay), dot(v, az)};
}

// ---------------------------------------------------------------------------------------
// Vortex line (stormbird/src/lifting_line/singularity_elements/vortex_line.rs)
// ---------------------------------------------------------------------------------------
constexpr double FOUR_PI_INVERSE = 1.0 / (4.0 * PI);  // vortex_line.rs:11
constexpr double CLOSENESS_ERROR = 1.0e-10;           // vortex_line.rs:13

// vortex_line.rs:59-84
inline double normal_distance_squared(V3 a, V3 b, V3 x, double r1sq, double r2sq) {
    V3 rel_line = b - a;
    V3 rel_point = x - a;
    double len_sq = length_squared(rel_line);
    double len = std::sqrt(len_sq);
    V3 dir = rel_line / len;
    double t = dot(rel_point, dir);
    if (t < 0.0) return r1sq;
    if (t > len) return r2sq;
    return length_squared(rel_point) - t * t;
}
// vortex_line.rs:90-106
inline double viscous_core_term(V3 a, V3 b, V3 x, double rc, double r1sq, double r2sq) {
    double d2 = normal_distance_squared(a, b, x, r1sq, r2sq);
    double rc2 = rc * rc;
    double den = std::sqrt(rc2 * rc2 + d2 * d2);  // powi(4) as repeated squaring
    return den > 0.0 ? d2 / den : 0.0;
}
// vortex_line.rs:18-55
inline V3 line_unit_velocity(V3 a, V3 b, V3 x, double rc) {
    V3 r1 = x - a, r2 = x - b;
    double r1sq = length_squared(r1), r2sq = length_squared(r2);
    double l1 = std::sqrt(r1sq), l2 = std::sqrt(r2sq);
    double r1r2 = l1 * l2;
    double den = r1r2 * (r1r2 + dot(r1, r2));
    if (std::fabs(den) > CLOSENESS_ERROR) {
        double core = (rc == 0.0) ? 1.0 : viscous_core_term(a, b, x, rc, r1sq, r2sq);
        double k = (l1 + l2) / den;
        return (core * cross(r1, r2)) * (k * FOUR_PI_INVERSE);
    }
    return {};
}

// ---------------------------------------------------------------------------------------
// Vortex panel (singularity_elements/panel.rs) and quadrilateral geometry
// (stormath/src/spatial_vector/geometry_functions.rs)
// ---------------------------------------------------------------------------------------
// geometry_functions.rs:11-21
inline double area_of_quadrilateral(const V3 p[4]) {
    double a = length(p[1] - p[0]), b = length(p[2] - p[1]), c = length(p[3] - p[2]), d = length(p[0] - p[3]);
    double s = (a + b + c + d) * 0.5;
    return std::sqrt((s - a) * (s - b) * (s - c) * (s - d));
}
// geometry_functions.rs:25-30
inline V3 normal_of_quadrilateral(const V3 p[4]) { return normalize(cross(p[2] - p[0], p[3] - p[1])); }

struct Panel {
    V3 points[4];
    V3 center;
    V3 normal;
    double far_field_length_squared = 0.0;
    double viscous_core_length = 0.0;
    double point_doublet_area_term = 0.0;

    Panel() = default;
    // panel.rs:26-50
    Panel(const V3 p[4], double far_field_ratio, double rc) {
        for (int i = 0; i < 4; ++i) points[i] = p[i];
        center = 0.25 * (((p[0] + p[1]) + p[2]) + p[3]);
        double area = area_of_quadrilateral(p);
        normal = normal_of_quadrilateral(p);
        double bound = length(p[1] - p[0]);
        double stream = length(p[2] - p[1]);
        double rep = std::max(bound, stream);
        double t = rep * far_field_ratio;
        far_field_length_squared = t * t;
        viscous_core_length = rc;
        point_doublet_area_term = area * FOUR_PI_INVERSE;
    }
    // panel.rs:53-57
    bool near(V3 x) const { return length_squared(x - center) <= far_field_length_squared; }
    // panel.rs:82-96
    V3 doublet(V3 x) const {
        V3 t = x - center;
        double d2 = length_squared(t);
        double d5 = d2 * d2 * std::sqrt(d2);
        double h = dot(t, normal);
        return (point_doublet_area_term * ((3.0 * h) * t - d2 * normal)) / d5;
    }
    // panel.rs:99-118
    V3 ring(V3 x) const {
        V3 u;
        for (int i = 0; i < 4; ++i) u += line_unit_velocity(points[i], points[(i + 1) & 3], x, viscous_core_length);
        return u;
    }
    // panel.rs:61-76
    V3 unit(V3 x) const { return near(x) ? ring(x) : doublet(x); }
};

// symmetry_condition.rs:27-43
inline bool mirrored_point(sbsetup::Symmetry s, V3 p, V3* m) {
    switch (s) {
        case sbsetup::Symmetry::NoSymmetry: return false;
        case sbsetup::Symmetry::X: *m = {-p.x, p.y, p.z}; return true;
        case sbsetup::Symmetry::Y: *m = {p.x, -p.y, p.z}; return true;
        case sbsetup::Symmetry::Z: *m = {p.x, p.y, -p.z}; return true;
    }
    return false;
}
inline V3 corrected_velocity(sbsetup::Symmetry s, V3 u, V3 um) {
    switch (s) {
        case sbsetup::Symmetry::NoSymmetry: return u;
        case sbsetup::Symmetry::X: return {u.x - um.x, u.y + um.y, u.z + um.z};
        case sbsetup::Symmetry::Y: return {u.x + um.x, u.y - um.y, u.z + um.z};
        case sbsetup::Symmetry::Z: return {u.x + um.x, u.y + um.y, u.z - um.z};
    }
    return u;
}

// horseshoe_vortex.rs:15-51
struct Horseshoe {
    V3 bound[2], start_trailing[2], end_trailing[2];
    double rc = 0.0;
    V3 unit(V3 x) const {
        V3 u;
        u += line_unit_velocity(bound[0], bound[1], x, rc);
        u += line_unit_velocity(start_trailing[0], start_trailing[1], x, rc);
        u += line_unit_velocity(end_trailing[0], end_trailing[1], x, rc);
        return u;
    }
};

// ---------------------------------------------------------------------------------------
// Foil section model (stormbird/src/section_models/foil.rs) and sigmoid
// (stormath/src/transition_functions.rs:20-27)
// ---------------------------------------------------------------------------------------
inline double sigmoid_zero_to_one(double x, double x0, double range) {
    double slope = 4.5951212 / range;
    double xp = slope * (x - x0);
    return 1.0 / (1.0 + std::exp(-xp));
}
// foil.rs:119-129
inline double get_stall_angle(double a) {
    double e = std::fabs(a);
    while (e > PI) e -= PI;
    e *= signum(a);
    return e;
}
struct Foil {
    sbsetup::Foil p;
    // foil.rs:256-270
    double amount_of_stall(double a) const {
        double e = a + p.angle_cd_min;
        double mean = e >= 0.0 ? std::fabs(p.mean_positive_stall_angle) : std::fabs(p.mean_negative_stall_angle);
        return sigmoid_zero_to_one(std::fabs(e), mean, p.stall_range);
    }
    // foil.rs:161-163
    double cl_linear(double a) const { return p.cl_zero_angle + p.cl_initial_slope * std::sin(a); }
    // foil.rs:166-181
    double cl_pre_stall_raw(double a) const {
        double hp = p.cl_high_order_power > 0.0 ? std::pow(std::fabs(a), p.cl_high_order_power) * signum(a) : 0.0;
        double f = a >= 0.0 ? p.cl_high_order_factor_positive : p.cl_high_order_factor_negative;
        return cl_linear(a) + f * hp;
    }
    // foil.rs:184-190
    double cl_pre_stall_with_drop_off(double a) const {
        double s = amount_of_stall(a);
        return cl_pre_stall_raw(a) * (1.0 - s);
    }
    // foil.rs:193-206
    double cl_post_stall_with_weight(double a) const {
        double raw = p.cl_max_after_stall * std::sin(2.0 * get_stall_angle(a));
        return raw * amount_of_stall(a);
    }
    // foil.rs:152-158
    double cl(double a) const { return cl_post_stall_with_weight(a) + cl_pre_stall_with_drop_off(a); }
    // foil.rs:272-276
    double combine(double a, double pre, double post) const {
        double s = amount_of_stall(a);
        return pre * (1.0 - s) + s * post;
    }
    // foil.rs:237-243
    double additional_cd_during_stall(double a) const {
        double s = amount_of_stall(a);
        return p.cd_bump_during_stall * ((1.0 - std::cos(s * TAU)) * 0.5);
    }
    // foil.rs:212-235
    double cd(double a) const {
        double sa = get_stall_angle(a);
        double eff = std::fabs(a + p.angle_cd_min);
        double pre = p.cd_min + p.cd_second_order_factor * (eff * eff);
        double post = p.cd_max_after_stall * std::pow(std::fabs(std::sin(sa)), p.cd_power_after_stall);
        double at = a + p.cd_stall_angle_offset * signum(a);
        double raw = combine(at, pre, post);
        double during = additional_cd_during_stall(at);
        if (p.cdi_correction_factor != 0.0) {
            double c = std::fabs(cl(a));
            return raw + p.cdi_correction_factor * (c * c) + during;
        }
        return raw + during;
    }
    // foil.rs:250-252
    double added_mass_coefficient(double acc) const { return p.added_mass_factor * acc; }
};

template <class T>
inline T linear_interpolation(double xt, const std::vector<double>& xd, const std::vector<T>& yd);

// section_models/rotating_cylinder.rs: coefficients tabulated over the spin ratio (the
// surface speed over the flow speed), with the cylinder diameter = the chord length
struct Cylinder {
    sbsetup::RotatingCylinder p;
    // rotating_cylinder.rs:76-83
    double spin_ratio(double diameter, double velocity) const {
        double circumference = PI * diameter;
        double tangential_velocity = circumference * p.revolutions_per_second;
        return -tangential_velocity / velocity;
    }
    // rotating_cylinder.rs:85-93
    double lift_coefficient_from_spin_ratio(double sr) const {
        return linear_interpolation(std::fabs(sr), p.spin_ratio_data, p.cl_data) * signum(sr);
    }
    // rotating_cylinder.rs:95-101
    double drag_coefficient_from_spin_ratio(double sr) const {
        return linear_interpolation(std::fabs(sr), p.spin_ratio_data, p.cd_data);
    }
    // rotating_cylinder.rs:103-113
    double lift_coefficient(double diameter, double velocity) const {
        return lift_coefficient_from_spin_ratio(spin_ratio(diameter, velocity));
    }
    double drag_coefficient(double diameter, double velocity) const {
        return drag_coefficient_from_spin_ratio(spin_ratio(diameter, velocity));
    }
    // rotating_cylinder.rs:127-129
    double added_mass_coefficient(double acc) const { return p.added_mass_factor * acc; }
};

// ---------------------------------------------------------------------------------------
// Rigid body motion (stormath/src/rigid_body_motion.rs)
// ---------------------------------------------------------------------------------------
struct RigidBodyMotion {
    V3 translation, rotation, velocity_linear, velocity_angular;
    sbsetup::RotationType rotation_type = sbsetup::RotationType::XYZ;
    V3 transform_point(V3 p) const { return rotate(p, rotation, rotation_type) + translation; }   // :32-34
    V3 transform_vector(V3 v) const { return rotate(v, rotation, rotation_type); }                // :37-39
    V3 to_body(V3 v) const { return in_rotated_coordinate_system(v, rotation, rotation_type); }    // :43-45
    V3 velocity_at_point(V3 p) const { return velocity_linear + cross(velocity_angular, p - translation); }  // :53-60
    void update_translation_fd(V3 t, double dt) {  // :68-78
        V3 old = translation;
        translation = t;
        velocity_linear = (translation - old) / dt;
    }
    void update_rotation_fd(V3 r, double dt) {  // :80-103
        V3 old = rotation;
        rotation = r;
        V3 d = rotation - old;
        for (int i = 0; i < 3; ++i) {
            if (d[i] > PI) d[i] = d[i] + TAU;
            else if (d[i] < -PI) d[i] = d[i] + TAU;
        }
        velocity_angular = d / dt;
    }
};

// stormath/src/interpolation.rs:17-100 (binary search + two-point interpolation)
template <class T>
inline T linear_interpolation(double xt, const std::vector<double>& xd, const std::vector<T>& yd) {
    auto two = [](double x, double x0, double x1, const T& y0, const T& y1) -> T {
        if (x <= x0) return y0;
        if (x >= x1) return y1;
        T dy = y1 - y0;
        double dx = x1 - x0;
        return y0 + dy * ((x - x0) / dx);
    };
    size_t n = xd.size();
    if (n == 0) throw std::runtime_error("x_data is empty");
    if (n == 1) return yd[0];
    if (n == 2) return two(xt, xd[0], xd[1], yd[0], yd[1]);
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        size_t mid = (lo + hi) / 2;
        if (xd[mid] > xt) hi = mid; else lo = mid;
    }
    if (lo == n - 1) return yd[lo];
    return two(xt, xd[lo], xd[lo + 1], yd[lo], yd[lo + 1]);
}

// ---------------------------------------------------------------------------------------
// Line force model (stormbird/src/line_force_model/*)
// ---------------------------------------------------------------------------------------
struct SpanLine {
    V3 s, e;
    V3 rel() const { return e - s; }                  // span_line.rs:27-29
    double len() const { return length(rel()); }     // :31-33
    V3 dir() const { return normalize(rel()); }       // :35-37
    V3 ctrl() const { return 0.5 * (s + e); }         // :44-46
};

struct Range { size_t start = 0, end = 0; bool contains(size_t i) const { return i >= start && i < end; } };

struct LineForceModel {
    std::vector<SpanLine> span_lines_local;
    std::vector<V3> chord_not_rotated;
    std::vector<double> chord_lengths;
    std::vector<bool> is_virtual;
    std::vector<Foil> foils;
    std::vector<Cylinder> cylinders;  // per wing; used where is_cylinder
    std::vector<char> is_cylinder;
    std::vector<Range> wing_indices;
    double density = 1.225;
    sbsetup::CoordinateSystem output_cs = sbsetup::CoordinateSystem::Global;
    bool include_viscous_lift = false;
    RigidBodyMotion rbm;
    std::vector<double> local_wing_angles;
    std::vector<V3> chord_local, chord_global, chord_global_at_span_points;
    std::vector<SpanLine> span_lines_global;
    std::vector<V3> span_points_global, ctrl_points_global;

    size_t nr_span_lines() const { return span_lines_local.size(); }
    size_t nr_wings() const { return wing_indices.size(); }
    size_t wing_index(size_t i) const {  // mod.rs:210-218
        for (size_t w = 0; w < wing_indices.size(); ++w) if (wing_indices[w].contains(i)) return w;
        throw std::runtime_error("Wing index not found");
    }
    const std::vector<SpanLine>& span_lines_out() const {
        return output_cs == sbsetup::CoordinateSystem::Global ? span_lines_global : span_lines_local;
    }

    // value_mapping.rs:87-137 (extrapolate_ends = false in every call on the path)
    template <class T>
    std::vector<T> span_point_values_from_ctrl_point_values(const std::vector<T>& c) const {
        std::vector<T> out;
        out.reserve(c.size() + wing_indices.size());
        for (const auto& r : wing_indices) {
            out.push_back(c[r.start]);
            size_t last = r.end - 1;
            for (size_t i = r.start; i < r.end; ++i) {
                if (i == last) out.push_back(c[last]);
                else out.push_back((c[i] + c[i + 1]) * 0.5);
            }
        }
        return out;
    }

    // data_update.rs:57-80
    void update_chord_vectors() {
        chord_local.resize(chord_not_rotated.size());
        chord_global.resize(chord_not_rotated.size());
        for (size_t i = 0; i < chord_not_rotated.size(); ++i) {
            size_t w = wing_index(i);
            V3 axis = span_lines_local[wing_indices[w].start].rel();  // data_access.rs:256-258
            chord_local[i] = rotate_around_axis(chord_not_rotated[i], local_wing_angles[w], axis);
            chord_global[i] = rbm.transform_vector(chord_local[i]);
        }
        chord_global_at_span_points = span_point_values_from_ctrl_point_values(chord_global);
    }
    // data_update.rs:25-39
    void update_global_span_lines() {
        span_lines_global.resize(span_lines_local.size());
        for (size_t i = 0; i < span_lines_local.size(); ++i) {
            span_lines_global[i].s = rbm.transform_point(span_lines_local[i].s);
            span_lines_global[i].e = rbm.transform_point(span_lines_local[i].e);
        }
    }
    // data_update.rs:41-55
    void update_global_span_points() {
        span_points_global.clear();
        for (const auto& r : wing_indices) {
            for (size_t i = r.start; i < r.end; ++i) span_points_global.push_back(span_lines_global[i].s);
            span_points_global.push_back(span_lines_global[r.end - 1].e);
        }
    }
    // data_update.rs:82-90
    void update_ctrl_points() {
        ctrl_points_global.resize(span_lines_global.size());
        for (size_t i = 0; i < span_lines_global.size(); ++i) ctrl_points_global[i] = span_lines_global[i].ctrl();
    }
    // data_update.rs:13-18
    void update_global_data_representations() {
        update_chord_vectors();
        update_global_span_lines();
        update_global_span_points();
        update_ctrl_points();
    }

    // force_calculations.rs:50-69
    std::vector<V3> felt_ctrl_points_velocity(const V3* u) const {
        std::vector<V3> out(ctrl_points_global.size());
        for (size_t i = 0; i < out.size(); ++i) out[i] = u[i] - rbm.velocity_at_point(ctrl_points_global[i]);
        return out;
    }
    // mod.rs:235-254 (Global input frame)
    std::vector<V3> remove_span_velocity(const std::vector<V3>& v) const {
        std::vector<V3> out(v.size());
        for (size_t i = 0; i < v.size(); ++i) out[i] = v[i] - project(v[i], span_lines_global[i].rel());
        return out;
    }
    // force_calculations.rs:79-107 (Global frame, no angle correction)
    std::vector<double> angles_of_attack(const std::vector<V3>& v) const {
        std::vector<double> a(v.size());
        for (size_t i = 0; i < v.size(); ++i)
            a[i] = length(v[i]) > MIN_POSITIVE ? signed_angle_between(chord_global[i], v[i], span_lines_global[i].dir()) : 0.0;
        return a;
    }
    const Foil& foil(size_t i) const { return foils[wing_index(i)]; }
    // section model of line i: a rotating cylinder (else the foil)
    const Cylinder* cylinder(size_t i) const {
        size_t w = wing_index(i);
        return is_cylinder[w] ? &cylinders[w] : nullptr;
    }
    // force_calculations.rs:138-160 (a rotating cylinder's lift depends on the speed, not the angle)
    std::vector<double> cl_pre_stall_drop(const std::vector<double>& a, const std::vector<V3>& v) const {
        std::vector<double> o(a.size());
        for (size_t i = 0; i < a.size(); ++i) {
            const Cylinder* c = cylinder(i);
            o[i] = c ? c->lift_coefficient(chord_lengths[i], length(v[i])) : foil(i).cl_pre_stall_with_drop_off(a[i]);
        }
        return o;
    }
    // force_calculations.rs:162-183 (zero for a rotating cylinder)
    double cl_post_stall(size_t i, double a) const { return cylinder(i) ? 0.0 : foil(i).cl_post_stall_with_weight(a); }
    // force_calculations.rs:188-210
    std::vector<double> cl_linear(const std::vector<double>& a, const std::vector<V3>& v) const {
        std::vector<double> o(a.size());
        for (size_t i = 0; i < a.size(); ++i) {
            const Cylinder* c = cylinder(i);
            o[i] = c ? c->lift_coefficient(chord_lengths[i], length(v[i])) : foil(i).cl_linear(a[i]);
        }
        return o;
    }
    // force_calculations.rs:212-229
    double cl_derivative(size_t i) const { return cylinder(i) ? 0.0 : foil(i).p.cl_initial_slope; }
    // force_calculations.rs:271-292 (circulation_strength with CirculationCorrection::None, :237-261)
    std::vector<double> circulation_strength(const std::vector<double>& a, const std::vector<V3>& v) const {
        std::vector<double> cl = cl_pre_stall_drop(a, v);
        if (include_viscous_lift)
            for (size_t i = 0; i < cl.size(); ++i) cl[i] += cl_post_stall(i, a[i]);
        std::vector<double> g(v.size());
        for (size_t i = 0; i < v.size(); ++i) g[i] = -0.5 * chord_lengths[i] * length(v[i]) * cl[i];
        return g;
    }
    // force_calculations.rs:390-411
    std::vector<V3> sectional_circulatory_forces(const std::vector<double>& g, const std::vector<V3>& v) const {
        const auto& sl = span_lines_out();
        std::vector<V3> f(nr_span_lines());
        for (size_t i = 0; i < f.size(); ++i)
            f[i] = length(v[i]) == 0.0 ? V3{} : (g[i] * cross(v[i], sl[i].rel())) * density;
        return f;
    }
    // force_calculations.rs:552-573
    std::vector<double> lift_coefficient_from_circulation(const std::vector<double>& g, const std::vector<V3>& v) const {
        std::vector<V3> f = sectional_circulatory_forces(g, v);
        std::vector<double> o(nr_span_lines());
        for (size_t i = 0; i < o.size(); ++i) {
            double sign = -1.0 * signum(g[i]);
            double area = chord_lengths[i] * span_lines_local[i].len();
            double ff = 0.5 * area * density * length_squared(v[i]);
            o[i] = ff == 0.0 ? 0.0 : length(f[i]) * sign / ff;
        }
        return o;
    }
    // force_calculations.rs:591-627
    double average_residual_absolute(const std::vector<double>& g, const std::vector<double>& a, const std::vector<V3>& v) const {
        std::vector<double> cg = lift_coefficient_from_circulation(g, v);
        std::vector<double> cd = cl_pre_stall_drop(a, v);
        double s = 0.0;
        for (size_t i = 0; i < cg.size(); ++i) s += std::fabs(cg[i] - cd[i]);
        return s / static_cast<double>(cg.size());
    }
};

// builder/single_wing.rs:73-150 and builder/mod.rs:79-113, mod.rs:164-205
inline LineForceModel build_line_force_model(const sbsetup::LineForceModelBuilder& b) {
    LineForceModel m;
    m.density = b.density;
    for (const auto& wb : b.wing_builders) {
        std::vector<V3> sp, cv;
        for (auto& p : wb.section_points) sp.push_back({p.x, p.y, p.z});
        for (auto& c : wb.chord_vectors) cv.push_back({c.x, c.y, c.z});
        // single_wing.rs:52-68
        std::vector<double> dist;
        for (size_t i = 0; i < sp.size(); ++i) dist.push_back(i == 0 ? 0.0 : dist.back() + length(sp[i] - sp[i - 1]));
        size_t nseg = sp.size() - 1;
        int64_t nsec = wb.nr_sections >= 0 ? wb.nr_sections : b.nr_sections;
        if (nsec <= 0) throw sbsetup::SetupError("nr_sections must be positive");
        double total = dist.back();
        double ds_avg = total / static_cast<double>(nsec);
        std::vector<double> ds_loc;
        std::vector<size_t> n_loc;
        for (size_t i = 0; i < nseg; ++i) {
            double sd = dist[i + 1] - dist[i];
            n_loc.push_back(static_cast<size_t>(std::ceil(sd / ds_avg)));
            ds_loc.push_back(sd / static_cast<double>(n_loc[i]));
        }
        size_t start = m.span_lines_local.size();
        for (size_t s = 0; s < nseg; ++s) {
            double ds = ds_loc[s];
            double s0 = dist[s];
            bool virt = wb.has_virtual ? wb.line_segment_is_virtual[s] : false;
            for (size_t i = 0; i < n_loc[s]; ++i) {
                double a = s0 + static_cast<double>(i) * ds;
                double e = a + ds;
                double c = 0.5 * (a + e);
                SpanLine l{linear_interpolation(a, dist, sp), linear_interpolation(e, dist, sp)};
                m.span_lines_local.push_back(l);
                V3 ch = linear_interpolation(c, dist, cv);
                m.chord_not_rotated.push_back(ch);
                m.chord_lengths.push_back(length(ch));
                m.is_virtual.push_back(virt);
            }
        }
        m.wing_indices.push_back({start, m.span_lines_local.size()});
        Foil f;
        f.p = wb.foil;
        m.foils.push_back(f);
        Cylinder cy;
        cy.p = wb.cylinder;
        m.cylinders.push_back(cy);
        m.is_cylinder.push_back(wb.rotating_cylinder ? 1 : 0);
        m.local_wing_angles.push_back(0.0);
    }
    if (!b.local_wing_angles.empty()) m.local_wing_angles = b.local_wing_angles;
    m.output_cs = b.output_coordinate_system;
    m.include_viscous_lift = b.include_viscous_lift_in_the_circulation;
    // builder/mod.rs:107-108: translation and rotation are copied; the rotation type stays XYZ
    m.rbm.translation = {b.translation.x, b.translation.y, b.translation.z};
    m.rbm.rotation = {b.rotation.x, b.rotation.y, b.rotation.z};
    m.update_global_data_representations();
    return m;
}

// ---------------------------------------------------------------------------------------
// Dynamic wake (stormbird/src/lifting_line/wake/dynamic_wake/*)
// ---------------------------------------------------------------------------------------
struct DynamicWake {
    size_t nr_points_along_span = 0, nr_panels_along_span = 0, nr_panels_per_line = 0, nr_points_per_line = 0;
    std::vector<V3> points, velocity_at_points;
    std::vector<double> strengths, panel_core;
    std::vector<Panel> panels;
    std::vector<Range> wing_indices;
    double first_rel = 0.75, last_rel = 0.25, damping = 0.0, far_field_ratio = 5.0, representative_chord = 0.0;
    sbsetup::FirstWakePointsDirection first_dir = sbsetup::FirstWakePointsDirection::Chord;
    sbsetup::Symmetry symmetry = sbsetup::Symmetry::NoSymmetry;
    size_t end_index = 0;
    bool neglect_self = false;
    size_t steps_completed = 0;
    int nthreads = 1;
    // Harness option, not in the reference: the next update_velocity_at_points keeps the
    // freestream only (no induced velocity), for checks of one step's circulation and forces,
    // which do not depend on the O(points x panels) roll-up sweep at the end of that step.
    bool skip_induced_once = false;

    size_t nr_points() const { return nr_points_along_span * nr_points_per_line; }
    size_t nr_panels() const { return nr_panels_along_span * nr_panels_per_line; }
    size_t point_index(size_t s, size_t j) const { return s * nr_points_along_span + j; }  // settings.rs:35-37
    size_t panel_index(size_t s, size_t j) const { return s * nr_panels_along_span + j; }  // settings.rs:18-20
    size_t wing_index(size_t j) const {  // mod.rs:68-76
        for (size_t w = 0; w < wing_indices.size(); ++w) if (wing_indices[w].contains(j)) return w;
        throw std::runtime_error("Span index not found in any wing");
    }
    // mod.rs:82-103
    void panel_points(size_t s, size_t j, V3 out[4]) const {
        size_t w = wing_index(j);
        out[0] = points[point_index(s, j + w)];
        out[1] = points[point_index(s, j + 1 + w)];
        out[2] = points[point_index(s + 1, j + 1 + w)];
        out[3] = points[point_index(s + 1, j + w)];
    }

    // induced_velocity_calc.rs:182-198
    V3 unit_velocity(size_t pi, V3 x) const {
        V3 u = panels[pi].unit(x);
        V3 m;
        if (mirrored_point(symmetry, x, &m)) return corrected_velocity(symmetry, u, panels[pi].unit(m));
        return u;
    }
    // induced_velocity_calc.rs:202-210
    V3 from_panel(size_t pi, V3 x) const {
        if (strengths[pi] == 0.0) return {};
        return strengths[pi] * unit_velocity(pi, x);
    }
    // induced_velocity_calc.rs:111-126 (the `parallel` build: per point, panels in order)
    std::vector<V3> local_include_self(const V3* pts, size_t n, size_t start, size_t end) const {
        std::vector<V3> out(n);
        const long long nn = static_cast<long long>(n);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
        for (long long i = 0; i < nn; ++i) {
            V3 acc;
            for (size_t p = start; p < end; ++p) acc = acc + from_panel(p, pts[i]);
            out[static_cast<size_t>(i)] = acc;
        }
        return out;
    }
    // induced_velocity_calc.rs:128-150
    std::vector<V3> local_neglect_self(const V3* pts, size_t n, size_t start, size_t end) const {
        std::vector<V3> out(n);
        for (size_t p = start; p < end; ++p) {
            size_t wp = wing_index(p % nr_panels_along_span);
            for (size_t i = 0; i < n; ++i) {
                size_t wi = wing_index(i);
                if (wp != wi) out[i] += from_panel(p, pts[i]);
            }
        }
        return out;
    }
    // induced_velocity_calc.rs:153-165
    std::vector<V3> local(const V3* pts, size_t n, size_t start, size_t end, bool neglect) const {
        return neglect ? local_neglect_self(pts, n, start, end) : local_include_self(pts, n, start, end);
    }
    // induced_velocity_calc.rs:18-26
    std::vector<V3> induced_velocities(const V3* pts, size_t n) const { return local(pts, n, 0, strengths.size(), false); }
    // induced_velocity_calc.rs:52-62
    std::vector<V3> induced_velocities_from_free_wake(const std::vector<V3>& pts) const {
        return local(pts.data(), pts.size(), nr_panels_along_span, strengths.size(), neglect_self);
    }

    // update_data.rs:90-99
    void synchronize_first_points(const LineForceModel& lfm) {
        for (size_t i = 0; i < lfm.span_points_global.size(); ++i) points[i] = lfm.span_points_global[i];
    }
    // update_data.rs:102-115
    void update_panel_data() {
        for (size_t i = 0; i < nr_panels(); ++i) {
            size_t s = i / nr_panels_along_span, j = i % nr_panels_along_span;
            V3 pp[4];
            panel_points(s, j, pp);
            panels[i] = Panel(pp, far_field_ratio, panel_core[i]);
        }
    }
    // update_data.rs:125-141
    void update_velocity_at_points(const V3* fs) {
        for (size_t i = 0; i < points.size(); ++i) velocity_at_points[i] = fs[i];
        size_t e = std::min(end_index, points.size());
        const bool skip = skip_induced_once;
        skip_induced_once = false;
        if (e > 0 && steps_completed > 2 && !skip) {
            std::vector<V3> u = induced_velocities(points.data(), e);
            for (size_t i = 0; i < e; ++i) velocity_at_points[i] += u[i];
        }
    }
    // update_data.rs:146-150
    void update_wing_strength(const std::vector<double>& g) {
        for (size_t i = 0; i < g.size(); ++i) strengths[i] = g[i];
    }
    // update_data.rs:152-199
    std::vector<V3> first_free_wake_points_direction(const LineForceModel& lfm, const V3* felt_span) const {
        size_t n = nr_points_along_span;
        std::vector<V3> d;
        d.reserve(n);
        switch (first_dir) {
            case sbsetup::FirstWakePointsDirection::Chord:
                for (size_t i = 0; i < n; ++i) d.push_back(normalize(lfm.chord_global_at_span_points[i]));
                break;
            case sbsetup::FirstWakePointsDirection::Freestream:
                for (size_t i = 0; i < n; ++i) d.push_back(normalize(felt_span[i]));
                break;
            case sbsetup::FirstWakePointsDirection::ActualVelocity:
                if (steps_completed > 2) {
                    for (size_t i = 0; i < n; ++i) d.push_back(normalize(0.5 * (velocity_at_points[i] + velocity_at_points[n + i])));
                } else {
                    for (size_t i = 0; i < n; ++i) d.push_back(normalize(felt_span[i]));
                }
                break;
        }
        return d;
    }
    // update_data.rs:205-252
    void move_first_free_wake_points(const LineForceModel& lfm, const V3* felt_span) {
        size_t n = nr_points_along_span;
        std::vector<V3> old(points.begin() + n, points.begin() + 2 * n);
        std::vector<V3> d = first_free_wake_points_direction(lfm, felt_span);
        double fl = representative_chord * first_rel;
        for (size_t i = 0; i < n; ++i) {
            V3 est = points[i] + d[i] * fl;
            if (damping > 0.0) points[i + n] = old[i] * damping + est * (1.0 - damping);
            else points[i + n] = est;
        }
    }
    // update_data.rs:262-292
    void move_last_wake_points(const V3* felt_span) {
        size_t np = points.size(), n = nr_points_along_span;
        bool multi = nr_panels_per_line > 1;
        size_t last = np - n, prev = last - n;
        std::vector<V3> dirs(n);
        for (size_t i = 0; i < n; ++i)
            dirs[i] = multi ? normalize(points[prev + i] - points[prev - n + i]) : normalize(felt_span[i]);
        for (size_t i = 0; i < n; ++i) {
            V3 c = last_rel * representative_chord * dirs[i];
            points[last + i] = points[prev + i] + c;
        }
    }
    // update_data.rs:295-316
    void stream_free_wake_points(double dt) {
        for (size_t s = nr_points_per_line - 1; s >= 2; --s) {
            for (size_t j = 0; j < nr_points_along_span; ++j) {
                size_t pi = point_index(s - 1, j), ci = point_index(s, j);
                V3 integ = points[pi] + dt * velocity_at_points[pi];
                if (damping > 0.0) points[ci] = points[ci] * damping + integ * (1.0 - damping);
                else points[ci] = integ;
            }
        }
    }
    // update_data.rs:319-328
    void stream_strength_values_downstream() {
        for (size_t s = nr_panels_per_line - 1; s >= 1; --s)
            for (size_t j = 0; j < nr_panels_along_span; ++j) strengths[panel_index(s, j)] = strengths[panel_index(s - 1, j)];
    }
    // update_data.rs:65-82
    void update_wake_points_before_solving(double dt, const LineForceModel& lfm, const V3* felt_span) {
        synchronize_first_points(lfm);
        stream_free_wake_points(dt);
        move_first_free_wake_points(lfm, felt_span);
        move_last_wake_points(felt_span);
    }
    // update_data.rs:28-42
    void update_before_solving(double dt, const LineForceModel& lfm, const V3* felt_span) {
        update_wake_points_before_solving(dt, lfm, felt_span);
        update_panel_data();
        stream_strength_values_downstream();
    }
    // update_data.rs:49-59
    void update_after_solving(const std::vector<double>& g, const V3* wake_fs) {
        update_wing_strength(g);
        update_velocity_at_points(wake_fs);
        steps_completed += 1;
    }
    // initialization.rs:12-41
    void initialize_with_velocity_and_time_step(const LineForceModel& lfm, V3 vel, double dt) {
        std::fill(strengths.begin(), strengths.end(), 0.0);
        std::fill(velocity_at_points.begin(), velocity_at_points.end(), vel);
        std::vector<V3> fs(points.size(), vel);
        synchronize_first_points(lfm);
        for (size_t k = 0; k < nr_points_per_line; ++k) update_wake_points_before_solving(dt, lfm, fs.data());
        update_panel_data();
    }
    // initialization.rs:46-71
    void initialize_based_on_chord_length(const LineForceModel& lfm, double factor) {
        const auto& cv = lfm.chord_global_at_span_points;
        V3 sum;
        for (const auto& c : cv) sum = sum + c;
        V3 avg = sum / static_cast<double>(cv.size());
        double wl = factor * length(avg);
        V3 v = (wl / static_cast<double>(nr_panels_per_line)) * avg;
        initialize_with_velocity_and_time_step(lfm, v, 1.0);
    }
};

// builder.rs:121-198 and :201-255
inline DynamicWake build_dynamic_wake(const LineForceModel& lfm, const sbsetup::DynamicWakeBuilder& b) {
    DynamicWake w;
    w.nr_panels_along_span = lfm.nr_span_lines();
    w.nr_points_along_span = lfm.span_points_global.size();
    w.nr_panels_per_line = static_cast<size_t>(b.nr_panels_per_line_element);
    w.nr_points_per_line = w.nr_panels_per_line + 1;
    w.points.assign(w.nr_points(), V3{});
    for (size_t s = 0; s < w.nr_points_per_line; ++s)
        for (size_t j = 0; j < lfm.span_points_global.size(); ++j) w.points[w.point_index(s, j)] = lfm.span_points_global[j];
    w.end_index = static_cast<size_t>(std::ceil(b.ratio_of_wake_affected_by_induced_velocities * static_cast<double>(w.nr_points() - 1)));
    w.first_rel = b.first_panel_relative_length;
    w.last_rel = b.last_panel_relative_length;
    w.first_dir = b.first_wake_points_direction;
    w.damping = b.shape_damping_factor;
    w.neglect_self = b.neglect_self_induced_velocities;
    w.symmetry = b.symmetry_condition;
    w.far_field_ratio = b.far_field_ratio;
    w.strengths.assign(w.nr_panels(), 0.0);
    // builder.rs:201-255
    auto raw_core = [&](const sbsetup::CoreLength& c, double span_len) {
        switch (c.kind) {
            case sbsetup::CoreKind::Relative: return c.value * span_len;
            case sbsetup::CoreKind::Absolute: return c.value;
            case sbsetup::CoreKind::NoViscousCore: return MIN_POSITIVE;
        }
        return 0.0;
    };
    w.panel_core.assign(w.nr_panels(), 0.0);
    for (size_t s = 0; s < w.nr_panels_per_line; ++s) {
        for (size_t j = 0; j < w.nr_panels_along_span; ++j) {
            double sl = lfm.span_lines_global[j].len();
            double raw = raw_core(b.viscous_core_length, sl);
            double v = raw;
            if (b.core_sin_increase) {
                double fin = raw_core(b.sin_last_panel_value, sl);
                double before = static_cast<double>(w.nr_panels_per_line - 1) * b.sin_evolution_length_factor;
                double rel = std::max(std::min(static_cast<double>(s) / before, 1.0), 0.0);
                double sf = std::sin(0.5 * rel * PI);
                v = raw * (1.0 - sf) + fin * sf;
            }
            w.panel_core[w.panel_index(s, j)] = v;
        }
    }
    w.panels.assign(w.nr_panels(), Panel{});
    w.velocity_at_points.assign(w.nr_points(), V3{});
    double csum = 0.0;
    for (double c : lfm.chord_lengths) csum += c;
    w.representative_chord = csum / static_cast<double>(lfm.chord_lengths.size());
    w.wing_indices = lfm.wing_indices;
    w.initialize_based_on_chord_length(lfm, b.initial_relative_wake_length);
    return w;
}

// ---------------------------------------------------------------------------------------
// Frozen wake (stormbird/src/lifting_line/wake/frozen_wake.rs)
// ---------------------------------------------------------------------------------------
struct FrozenWake {
    size_t n = 0;
    std::vector<V3> fixed, factors, induced;  // factors: row-major [n x n]
    void initialize(size_t nr) { n = nr; fixed.assign(n, V3{}); factors.assign(n * n, V3{}); induced.assign(n, V3{}); }

    // frozen_wake.rs:68-129 with horseshoe_vortex.rs:54-103
    void update_as_steady(const LineForceModel& lfm, const std::vector<V3>& span_vel, const sbsetup::QuasiSteadyWakeSettings& s) {
        const auto& sl = lfm.span_lines_global;
        double csum = 0.0;
        for (double c : lfm.chord_lengths) csum += c;
        double avg_c = csum / static_cast<double>(n);
        double wl = s.wake_length_factor * avg_c;
        std::vector<V3> wv;
        for (const auto& v : span_vel) wv.push_back(normalize(v) * wl);
        double rc = 0.0;
        switch (s.viscous_core_length.kind) {
            case sbsetup::CoreKind::Relative: {
                double ls = 0.0;
                for (const auto& l : sl) ls += l.len();
                rc = s.viscous_core_length.value * (ls / static_cast<double>(n));
                break;
            }
            case sbsetup::CoreKind::Absolute: rc = s.viscous_core_length.value; break;
            case sbsetup::CoreKind::NoViscousCore: rc = 0.0; break;
        }
        std::vector<Horseshoe> hs;
        size_t k = 0;
        for (const auto& r : lfm.wing_indices) {
            for (size_t i = r.start; i < r.end; ++i) {
                Horseshoe h;
                h.bound[0] = sl[i].s; h.bound[1] = sl[i].e;
                h.start_trailing[0] = sl[i].s + wv[k]; h.start_trailing[1] = sl[i].s;
                h.end_trailing[0] = sl[i].e; h.end_trailing[1] = sl[i].e + wv[k + 1];
                h.rc = rc;
                hs.push_back(h);
                k += 1;
            }
            k += 1;
        }
        for (size_t r = 0; r < n; ++r) {
            V3 cp = lfm.ctrl_points_global[r];
            for (size_t c = 0; c < n; ++c) {
                V3 u = hs[c].unit(cp);
                V3 m;
                if (mirrored_point(s.symmetry_condition, cp, &m)) u = corrected_velocity(s.symmetry_condition, u, hs[c].unit(m));
                factors[r * n + c] = u;
            }
        }
    }
    // frozen_wake.rs:189-261
    void update_from_full_wake(const std::vector<V3>& ctrl, const DynamicWake& w) {
        fixed = w.induced_velocities_from_free_wake(ctrl);
        for (size_t p = 0; p < n; ++p) {
            for (size_t c = 0; c < n; ++c) {
                if (w.neglect_self && w.wing_index(c) == w.wing_index(p)) factors[c * n + p] = V3{};
                else factors[c * n + p] = w.unit_velocity(w.panel_index(0, p), ctrl[c]);
            }
        }
    }
    // frozen_wake.rs:268-301
    void update_induced_velocities_at_control_points(const std::vector<double>& g) {
        induced = fixed;
        for (size_t r = 0; r < n; ++r) {
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (size_t c = 0; c < n; ++c) {
                const V3& f = factors[r * n + c];
                sx += f.x * g[c];
                sy += f.y * g[c];
                sz += f.z * g[c];
            }
            induced[r].x += sx;
            induced[r].y += sy;
            induced[r].z += sz;
        }
    }
};

// ---------------------------------------------------------------------------------------
// Solvers (stormbird/src/lifting_line/solvers/*)
// ---------------------------------------------------------------------------------------
struct SolverResult {
    std::vector<V3> input_velocity;
    std::vector<double> circulation;
    std::vector<V3> output_velocity;
    int64_t iterations = 0;
    double residual = 0.0;
    bool converged = false;
};

// velocity_corrections.rs:28-100; returns false for NoCorrection
inline bool corrected_velocity(const sbsetup::VelocityCorrections& vc, const std::vector<V3>& fs, const std::vector<V3>& ind,
                               std::vector<V3>* out) {
    switch (vc.kind) {
        case sbsetup::VelocityCorrectionKind::NoCorrection: return false;
        case sbsetup::VelocityCorrectionKind::MaxInducedVelocityMagnitudeRatio: {
            out->resize(fs.size());
            for (size_t i = 0; i < fs.size(); ++i) {
                double im = length(ind[i]);
                double fm = length(fs[i]);
                double mx = vc.ratio * fm;
                V3 c = im > mx ? normalize(ind[i]) * mx : ind[i];
                (*out)[i] = fs[i] + c;
            }
            return true;
        }
        case sbsetup::VelocityCorrectionKind::FixedMagnitudeEqualToFreestream: {
            out->resize(fs.size());
            for (size_t i = 0; i < fs.size(); ++i) (*out)[i] = normalize(fs[i] + ind[i]) * length(fs[i]);
            return true;
        }
    }
    return false;
}

// stormath/src/matrix/linalg.rs:41-103
inline std::vector<double> solve_gaussian_elimination(const std::vector<double>& A, const std::vector<double>& b, size_t n) {
    std::vector<double> aug(n * (n + 1));
    const size_t w = n + 1;
    for (size_t i = 0; i < n; ++i) {
        for (size_t j = 0; j < n; ++j) aug[i * w + j] = A[i * n + j];
        aug[i * w + n] = b[i];
    }
    for (size_t k = 0; k < n; ++k) {
        size_t mr = k;
        for (size_t i = k + 1; i < n; ++i) if (std::fabs(aug[i * w + k]) > std::fabs(aug[mr * w + k])) mr = i;
        if (mr != k) for (size_t j = 0; j <= n; ++j) std::swap(aug[k * w + j], aug[mr * w + j]);
        if (std::fabs(aug[k * w + k]) < 1e-12) throw std::runtime_error("Matrix is singular or nearly singular");
        for (size_t i = k + 1; i < n; ++i) {
            double f = aug[i * w + k] / aug[k * w + k];
            for (size_t j = k; j <= n; ++j) aug[i * w + j] -= f * aug[k * w + j];
        }
    }
    std::vector<double> x(n, 0.0);
    for (size_t ii = n; ii-- > 0;) {
        double s = 0.0;
        for (size_t j = ii + 1; j < n; ++j) s += aug[ii * w + j] * x[j];
        x[ii] = (aug[ii * w + n] - s) / aug[ii * w + ii];
    }
    return x;
}

// linearized.rs:54-222
inline SolverResult solve_linearized(const sbsetup::Linearized& st, const LineForceModel& lfm, const std::vector<V3>& felt,
                                     FrozenWake& fw) {
    size_t n = lfm.nr_span_lines();
    std::vector<V3> vel = felt;
    // check_for_zero_linear_lift (:226-265) never returns early: its flag starts as true.
    for (size_t i = 0; i < n; ++i) vel[i] += fw.fixed[i];
    vel = lfm.remove_span_velocity(vel);
    std::vector<V3> vdir(n), ndir(n);
    for (size_t i = 0; i < n; ++i) {
        V3 un = normalize(vel[i]);
        V3 sd = normalize(lfm.span_lines_global[i].rel());
        vdir[i] = un;
        ndir[i] = cross(un, sd);
    }
    std::vector<double> aoa = lfm.angles_of_attack(vel);
    std::vector<double> cll = lfm.cl_linear(aoa, vel);
    std::vector<double> A(n * n), rhs(n);
    for (size_t r = 0; r < n; ++r) {
        double ut = dot(vel[r], vdir[r]);
        double dcl = lfm.cl_derivative(r);  // force_calculations.rs:212-229
        for (size_t c = 0; c < n; ++c) {
            double uin = dot(fw.factors[r * n + c], ndir[r]);
            A[r * n + c] = -dcl * uin / ut;
            if (r == c) A[r * n + c] += 2.0 / (lfm.chord_lengths[r] * ut);
        }
        rhs[r] = -cll[r];
    }
    std::vector<double> g = solve_gaussian_elimination(A, rhs, n);
    fw.update_induced_velocities_at_control_points(g);
    std::vector<V3> cv;
    auto total_velocity = [&](std::vector<V3>& out) {
        if (corrected_velocity(st.velocity_corrections, felt, fw.induced, &cv)) out = cv;
        else for (size_t i = 0; i < n; ++i) out[i] = felt[i] + fw.induced[i];
    };
    total_velocity(vel);
    if (!st.disable_viscous_corrections) {
        std::vector<double> a2 = lfm.angles_of_attack(vel);
        std::vector<double> cl_lin = lfm.cl_linear(a2, vel);
        std::vector<double> cl_full = lfm.cl_pre_stall_drop(a2, vel);
        for (size_t i = 0; i < n; ++i) if (std::fabs(cl_lin[i]) > MIN_POSITIVE) g[i] *= cl_full[i] / cl_lin[i];
        if (st.full_induced_velocity_correction) fw.update_induced_velocities_at_control_points(g);
        total_velocity(vel);
    }
    std::vector<double> a3 = lfm.angles_of_attack(vel);
    SolverResult r;
    r.residual = lfm.average_residual_absolute(g, a3, vel);
    r.input_velocity = felt;
    r.circulation = g;
    r.output_velocity = vel;
    r.iterations = 1;
    r.converged = true;
    return r;
}

// simple_iterative.rs:86-212
inline SolverResult solve_simple_iterative(const sbsetup::SimpleIterative& st, const LineForceModel& lfm,
                                           const std::vector<V3>& felt, FrozenWake& fw, const std::vector<double>& init) {
    size_t n = lfm.nr_span_lines();
    std::vector<double> g = init;
    if (std::fabs(st.correction_factor_initial_solution - 1.0) > MIN_POSITIVE)
        for (auto& x : g) x *= st.correction_factor_initial_solution;
    if (st.start_with_linearized_solution) {
        sbsetup::Linearized def;
        g = solve_linearized(def, lfm, felt, fw).circulation;
    }
    std::vector<V3> vel(n);
    std::vector<double> aoa(n, 0.0);
    double residual = lfm.average_residual_absolute(g, aoa, vel);
    int64_t it = 0;
    bool conv = false;
    std::vector<V3> cv;
    while (it < st.max_iterations_per_time_step && !conv) {
        it += 1;
        fw.update_induced_velocities_at_control_points(g);
        if (corrected_velocity(st.velocity_corrections, felt, fw.induced, &cv)) vel = cv;
        else for (size_t i = 0; i < n; ++i) vel[i] = felt[i] + fw.induced[i];
        vel = lfm.remove_span_velocity(vel);
        aoa = lfm.angles_of_attack(vel);
        std::vector<double> est;
        if (st.use_raw_circulation_during_iterations) est = lfm.circulation_strength(aoa, vel);  // raw == corrected without correction
        else est = lfm.circulation_strength(aoa, vel);
        residual = lfm.average_residual_absolute(g, aoa, vel);
        if (residual < st.residual_tolerance_absolute) conv = true;
        double mx = 0.0;
        for (size_t i = 0; i < n; ++i) {
            double d = est[i] - g[i];
            double ad = std::fabs(d);
            if (ad > mx) mx = ad;
            g[i] += st.damping_factor * d;
        }
        if (mx < st.strength_difference_tolerance) conv = true;
    }
    SolverResult r;
    r.circulation = lfm.circulation_strength(aoa, vel);
    r.input_velocity = felt;
    r.output_velocity = vel;
    r.iterations = it;
    r.residual = residual;
    r.converged = conv;
    return r;
}

// ---------------------------------------------------------------------------------------
// Results (common_utils/forces_and_moments.rs, results/simulation.rs, flow_derivatives.rs)
// ---------------------------------------------------------------------------------------
struct FlowDerivatives {  // flow_derivatives.rs:16-63
    std::vector<V3> h0, h1;
    size_t count = 0;
    void reset(const std::vector<V3>& v) { h0 = v; h1 = v; count = 0; }
    std::vector<V3> acceleration(const std::vector<V3>& cur, double dt) const {
        if (count < 2) return std::vector<V3>(cur.size());
        std::vector<V3> a(cur.size());
        // stormath/src/finite_difference.rs:33-42
        for (size_t i = 0; i < cur.size(); ++i) a[i] = (cur[i] * 3.0 - h1[i] * 4.0 + h0[i]) / (2.0 * dt);
        return a;
    }
    void update(const std::vector<V3>& cur) { h0 = h1; h1 = cur; count += 1; }
};

struct StepResult {
    double time = 0.0;
    std::vector<V3> ctrl_points, solver_input_velocity;
    std::vector<double> circulation, aoa;
    std::vector<V3> output_velocity, force_velocity, acceleration;
    std::vector<V3> sectional[6];                   // circulatory, viscous_lift, drag, added_mass, gyroscopic, total
    std::vector<V3> integrated_forces, integrated_moments;  // [S*6]
    V3 force_sum, moment_sum;
    int64_t iterations = 0;
    double residual = 0.0;
    bool converged = false;
};

// force_calculations.rs:322-452, 669-698; forces_and_moments.rs:163-245
inline StepResult calculate_simulation_result(const LineForceModel& lfm, const SolverResult& sr, const std::vector<V3>& acc_in, double time) {
    size_t n = lfm.nr_span_lines(), S = lfm.nr_wings();
    bool body = lfm.output_cs == sbsetup::CoordinateSystem::Body;
    StepResult R;
    R.time = time;
    R.aoa = lfm.angles_of_attack(sr.output_velocity);
    R.acceleration = acc_in;
    R.force_velocity = sr.output_velocity;
    V3 rot_vel = lfm.rbm.velocity_angular;
    if (body) {
        for (size_t i = 0; i < n; ++i) {
            R.force_velocity[i] = lfm.rbm.to_body(R.force_velocity[i]);
            R.acceleration[i] = lfm.rbm.to_body(R.acceleration[i]);
        }
        rot_vel = lfm.rbm.to_body(rot_vel);
    }
    const auto& v = R.force_velocity;
    const auto& sl = lfm.span_lines_out();
    const auto& cv = body ? lfm.chord_local : lfm.chord_global;
    for (auto& s : R.sectional) s.assign(n, V3{});
    R.sectional[0] = lfm.sectional_circulatory_forces(sr.circulation, v);
    for (size_t i = 0; i < n; ++i) {
        const Foil& f = lfm.foil(i);
        const Cylinder* cyl = lfm.cylinder(i);
        double area = lfm.chord_lengths[i] * lfm.span_lines_local[i].len();
        double ff = 0.5 * area * lfm.density * length_squared(v[i]);
        // viscous lift :413-433
        if (!lfm.include_viscous_lift) {
            double clv = lfm.cl_post_stall(i, R.aoa[i]);
            V3 ld = normalize(cross(lfm.span_lines_local[i].rel(), v[i]));
            R.sectional[1][i] = ld * clv * ff;
        }
        // drag :438-452 (viscous_drag_coefficients :301-320)
        double cd = cyl ? cyl->drag_coefficient(lfm.chord_lengths[i], length(v[i])) : f.cd(R.aoa[i]);
        R.sectional[2][i] = normalize(v[i]) * cd * ff;
        // added mass :467-513 (a foil's acceleration along its chord is left out, a cylinder's not)
        double strip = lfm.chord_lengths[i] * sl[i].len();
        V3 ra = R.acceleration[i];
        ra -= project(ra, sl[i].dir());
        if (!cyl) ra -= project(ra, cv[i]);
        if (length(ra) != 0.0) {
            double cam = cyl ? cyl->added_mass_coefficient(length(ra)) : f.added_mass_coefficient(length(ra));
            R.sectional[3][i] = cam * lfm.density * strip * normalize(ra);
        }
        // gyroscopic :520-548: zero for a foil; a cylinder's spin angular momentum crossed with
        // the body's rotation velocity
        if (cyl) {
            double i_zz = cyl->p.moment_of_inertia_2d * sl[i].len();
            double radial_velocity = 2.0 * PI * cyl->p.revolutions_per_second;
            V3 angular_momentum = i_zz * radial_velocity * sl[i].rel();
            R.sectional[4][i] = cross(angular_momentum, rot_vel);
        }
        V3 t = R.sectional[0][i];  // compute_total :163-172
        t += R.sectional[1][i];
        t += R.sectional[2][i];
        t += R.sectional[3][i];
        t += R.sectional[4][i];
        R.sectional[5][i] = t;
    }
    R.integrated_forces.assign(S * 6, V3{});
    R.integrated_moments.assign(S * 6, V3{});
    for (size_t w = 0; w < S; ++w) {
        for (size_t i = lfm.wing_indices[w].start; i < lfm.wing_indices[w].end; ++i) {
            if (lfm.is_virtual[i]) continue;
            V3 cp = sl[i].ctrl();
            for (int c = 0; c < 6; ++c) {
                R.integrated_forces[w * 6 + c] += R.sectional[c][i];
                R.integrated_moments[w * 6 + c] += cross(cp, R.sectional[c][i]);
            }
        }
        R.force_sum += R.integrated_forces[w * 6 + 5];
        R.moment_sum += R.integrated_moments[w * 6 + 5];
    }
    R.ctrl_points = lfm.ctrl_points_global;
    R.solver_input_velocity = sr.input_velocity;
    R.circulation = sr.circulation;
    R.output_velocity = sr.output_velocity;
    R.iterations = sr.iterations;
    R.residual = sr.residual;
    R.converged = sr.converged;
    return R;
}

// ---------------------------------------------------------------------------------------
// Simulation (stormbird/src/lifting_line/simulation.rs, simulation_builder.rs:97-143)
// ---------------------------------------------------------------------------------------
struct Simulation {
    sbsetup::Setup setup;
    LineForceModel lfm;
    FlowDerivatives fd;
    bool dynamic = false;
    DynamicWake wake;
    FrozenWake frozen;
    std::vector<double> previous_circulation;
    bool first_step_completed = false;

    explicit Simulation(const std::string& json, int nthreads = 1) {
        setup = sbsetup::parse_setup(json, /*allow_rotating_cylinder=*/true);
        lfm = build_line_force_model(setup.line_force_model);
        size_t n = lfm.nr_span_lines();
        dynamic = setup.dynamic;
        if (dynamic) {
            wake = build_dynamic_wake(lfm, setup.dynamic_wake);
            wake.nthreads = nthreads;
        }
        frozen.initialize(n);
        previous_circulation.assign(n, 0.0);
        fd.reset(std::vector<V3>(n));
    }

    void set_threads(int t) { wake.nthreads = t; }

    // simulation.rs:45-63
    std::vector<V3> freestream_points() const {
        std::vector<V3> p = lfm.ctrl_points_global;
        if (dynamic) p.insert(p.end(), wake.points.begin(), wake.points.end());
        return p;
    }
    size_t nr_freestream_points() const { return lfm.nr_span_lines() + (dynamic ? wake.points.size() : 0); }

    // simulation.rs:65-94
    void initialize(const V3* ctrl_fs, double dt) {
        size_t n = lfm.nr_span_lines();
        if (dynamic) {
            V3 s;
            for (size_t i = 0; i < n; ++i) s = s + ctrl_fs[i];
            V3 avg = s / static_cast<double>(n);
            std::fill(wake.velocity_at_points.begin(), wake.velocity_at_points.end(), avg);
            wake.initialize_with_velocity_and_time_step(lfm, avg, dt);
        }
        fd.reset(std::vector<V3>(ctrl_fs, ctrl_fs + n));
        first_step_completed = true;
        previous_circulation.assign(n, 0.0);
    }

    // simulation.rs:107-203
    StepResult do_step(double time, double dt, const V3* fs, size_t nfs) {
        size_t n = lfm.nr_span_lines();
        if (nfs != nr_freestream_points()) throw std::runtime_error("freestream length mismatch");
        lfm.update_global_data_representations();
        std::vector<V3> felt = lfm.felt_ctrl_points_velocity(fs);
        std::vector<V3> felt_span = lfm.span_point_values_from_ctrl_point_values(felt);
        if (!first_step_completed) initialize(fs, dt);
        if (dynamic) {
            wake.update_before_solving(dt, lfm, felt_span.data());
            frozen.update_from_full_wake(lfm.ctrl_points_global, wake);
        } else {
            frozen.update_as_steady(lfm, felt_span, setup.quasi_steady_wake);
        }
        SolverResult sr = setup.solver.kind == sbsetup::SolverKind::SimpleIterative
                              ? solve_simple_iterative(setup.solver.si, lfm, felt, frozen, previous_circulation)
                              : solve_linearized(setup.solver.lin, lfm, felt, frozen);
        if (dynamic) wake.update_after_solving(sr.circulation, fs + n);
        previous_circulation = sr.circulation;
        std::vector<V3> acc = fd.acceleration(sr.output_velocity, dt);
        fd.update(sr.output_velocity);
        return calculate_simulation_result(lfm, sr, acc, time);
    }

    // simulation.rs:207-216
    std::vector<V3> induced_velocities(const V3* pts, size_t n) const {
        if (!dynamic) throw std::runtime_error("Induced velocities not implemented for pure quasi-steady simulations yet");
        return wake.induced_velocities(pts, n);
    }
};

}  // namespace sbo
