// Device-side data layout and math shared by the lifting-line kernels (sm_103a).
//
// Layout in HBM (one simulation handle):
//   * line force model, constant: local span lines, chord vectors, chord lengths, wing of
//     each line, Foil parameters per wing                       (SoA, f64)
//   * per-step geometry written by k_prep_geometry: global span lines, span points,
//     control points, chord vectors, felt velocities            (SoA, f64)
//   * wake points, two buffers (old/new) of [W+1][Np] double3, streamwise-major, and the
//     velocity at the points [W+1][Np] double3                   (f64: position integration)
//   * wake strengths, two buffers of [W][N] f64
//   * wake panel records [W][N], 48 floats each (192 B, 16-B aligned) for the FP32
//     Biot-Savart sweep, plus f64 records for the first row (unit-strength matrix) and,
//     in the FP64 precision mode, for every panel
//   * frozen wake: fixed velocities [N] double3, unit matrix [N][N] double3
//   * solver state: previous circulation [N], flow-derivative history [2][N] double3
//   * output block: every per-step result in one contiguous f64 array, copied to the host
//     with a single D2H per step.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sbgpu {

constexpr int kMaxWings = 64;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTau = 2.0 * kPi;
constexpr double kMinPositive = 2.2250738585072014e-308;
constexpr double kFourPiInv = 1.0 / (4.0 * kPi);

// ---------------------------------------------------------------------------------------
// f64 3-vector
// ---------------------------------------------------------------------------------------
struct d3 {
    double x, y, z;
};
__host__ __device__ inline d3 mk(double x, double y, double z) { return d3{x, y, z}; }
__host__ __device__ inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline d3 operator-(d3 a) { return {-a.x, -a.y, -a.z}; }
__host__ __device__ inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ inline d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ inline d3 operator/(d3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline double len2(d3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__host__ __device__ inline double len(d3 a) { return sqrt(len2(a)); }
__host__ __device__ inline d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ inline d3 normalize(d3 a) {
    double l = len(a);
    if (l > 0.0) return {a.x / l, a.y / l, a.z / l};
    return {0.0, 0.0, 0.0};
}
__host__ __device__ inline d3 project(d3 a, d3 onto) {
    d3 n = normalize(onto);
    return n * dot(a, n);
}
__host__ __device__ inline double signum(double v) { return copysign(1.0, v); }

// f64 value as a pair of floats: hi = the nearest float, lo = the nearest float of v - hi
// (hi + lo carries about 48 significant bits)
__device__ inline float2 split_f64(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - static_cast<double>(h)));
}

// Angle between two vectors, signed by the right-hand rule about `axis`
// (stormath/src/spatial_vector/vector_math.rs:65-95).
__device__ inline double signed_angle_between(d3 a, d3 b, d3 axis) {
    double triple = dot(a, cross(b, axis));
    double al = len2(a), bl = len2(b);
    double ang = 0.0;
    if (!(al == 0.0 || bl == 0.0)) {
        double c = dot(a, b) / sqrt(al * bl);
        c = fmin(fmax(c, -1.0), 1.0);
        ang = acos(c);
    }
    return triple > 0.0 ? ang : -ang;
}

// Rodrigues rotation (stormath/src/spatial_vector/transformations.rs:139-150).
__device__ inline d3 rotate_around_axis(d3 v, double angle, d3 axis) {
    d3 n = normalize(axis);
    double c = cos(angle), s = sin(angle);
    d3 t1 = v * c;
    d3 t2 = cross(n, v) * s;
    d3 t3 = n * dot(n, v) * (1.0 - c);
    return t1 + t2 + t3;
}

// Euler XYZ rotation (transformations.rs:182-207). The line force model's rigid-body
// motion always uses this form: the builder never copies its rotation_type into the
// motion (line_force_model/builder/mod.rs:107-108).
__host__ __device__ inline d3 rotate_xyz(d3 v, d3 r) {
    d3 n = v;
    if (r.x != 0.0) {
        double ty = n.y, tz = n.z, c = cos(r.x), s = sin(r.x);
        n.y = ty * c - tz * s;
        n.z = ty * s + tz * c;
    }
    if (r.y != 0.0) {
        double tx = n.x, tz = n.z, c = cos(r.y), s = sin(r.y);
        n.x = tx * c + tz * s;
        n.z = -tx * s + tz * c;
    }
    if (r.z != 0.0) {
        double tx = n.x, ty = n.y, c = cos(r.z), s = sin(r.z);
        n.x = tx * c - ty * s;
        n.y = tx * s + ty * c;
    }
    return n;
}

// Vector expressed in the body frame (transformations.rs:233-265, XYZ).
__host__ __device__ inline d3 to_body(d3 v, d3 r) {
    d3 ax = rotate_xyz(mk(1, 0, 0), r), ay = rotate_xyz(mk(0, 1, 0), r), az = rotate_xyz(mk(0, 0, 1), r);
    return {dot(v, ax), dot(v, ay), dot(v, az)};
}

// ---------------------------------------------------------------------------------------
// Foil section model (stormbird/src/section_models/foil.rs), f64
// ---------------------------------------------------------------------------------------
struct FoilP {
    double cl_zero_angle, cl_initial_slope, cl_high_order_factor_positive, cl_high_order_factor_negative,
        cl_high_order_power, cl_max_after_stall, cd_min, angle_cd_min, cd_second_order_factor, cd_max_after_stall,
        cd_power_after_stall, cdi_correction_factor, mean_positive_stall_angle, mean_negative_stall_angle, stall_range,
        cd_bump_during_stall, cd_stall_angle_offset, added_mass_factor;
    // 4.5951212 / stall_range, the stall sigmoid's slope (transition_functions.rs:20-27),
    // divided once on the host (both sides round the f64 quotient correctly: same bits)
    double stall_slope;
};

// stormath/src/transition_functions.rs:20-27, with slope = 4.5951212 / range
__device__ inline double sigmoid_zero_to_one_slope(double x, double x0, double slope) {
    return 1.0 / (1.0 + exp(-(slope * (x - x0))));
}
// foil.rs:119-129
__device__ inline double stall_angle(double a) {
    double e = fabs(a);
    while (e > kPi) e -= kPi;
    return e * signum(a);
}
// foil.rs:256-270
__device__ inline double foil_amount_of_stall(const FoilP& f, double a) {
    double e = a + f.angle_cd_min;
    double mean = e >= 0.0 ? fabs(f.mean_positive_stall_angle) : fabs(f.mean_negative_stall_angle);
    return sigmoid_zero_to_one_slope(fabs(e), mean, f.stall_slope);
}
// foil.rs:161-163
__device__ inline double foil_cl_linear(const FoilP& f, double a) { return f.cl_zero_angle + f.cl_initial_slope * sin(a); }
// foil.rs:166-190
__device__ inline double foil_cl_pre_stall(const FoilP& f, double a) {
    double hp = f.cl_high_order_power > 0.0 ? pow(fabs(a), f.cl_high_order_power) * signum(a) : 0.0;
    double hf = a >= 0.0 ? f.cl_high_order_factor_positive : f.cl_high_order_factor_negative;
    double raw = foil_cl_linear(f, a) + hf * hp;
    return raw * (1.0 - foil_amount_of_stall(f, a));
}
// foil.rs:193-206
__device__ inline double foil_cl_post_stall(const FoilP& f, double a) {
    double raw = f.cl_max_after_stall * sin(2.0 * stall_angle(a));
    return raw * foil_amount_of_stall(f, a);
}
// foil.rs:212-243
__device__ inline double foil_cd(const FoilP& f, double a) {
    double sa = stall_angle(a);
    double eff = fabs(a + f.angle_cd_min);
    double pre = f.cd_min + f.cd_second_order_factor * (eff * eff);
    double post = f.cd_max_after_stall * pow(fabs(sin(sa)), f.cd_power_after_stall);
    double at = a + f.cd_stall_angle_offset * signum(a);
    double s = foil_amount_of_stall(f, at);
    double raw = pre * (1.0 - s) + s * post;
    double during = f.cd_bump_during_stall * ((1.0 - cos(s * kTau)) * 0.5);
    if (f.cdi_correction_factor != 0.0) {
        double cl = fabs(foil_cl_post_stall(f, a) + foil_cl_pre_stall(f, a));
        return raw + f.cdi_correction_factor * (cl * cl) + during;
    }
    return raw + during;
}

// ---------------------------------------------------------------------------------------
// Panel records
// ---------------------------------------------------------------------------------------
// Records of one vortex-ring panel for the Biot-Savart sweeps.
//
// FP32 record (PanelRec<float>, 48 floats = 192 B). The centre is a float-float pair
// (hi = fl32(c), lo = fl32(c - hi)) and the corners are FP32 offsets from it, so a sweep
// forms e = x - c = (x_hi - c_hi) + (x_lo - c_lo) once per panel (the hi difference is exact
// for nearby points, Sterbenz) and r_k = e - o_k per corner: accurate to ~ulp(|r|) + ulp(|o|)
// wherever the geometry sits in space.
//   [0..11]  corner offsets o_k = p_k - centre (rounded from f64)
//   [12..23] segment vectors d_k = p_{k+1} - p_k (rounded from f64)
//   [24..27] 1/|d_k|^2 per ring segment k (0 for a degenerate segment)
//   [28..30] centre hi, [31] far-field length squared (hi)
//   [32..34] centre lo, [35] area / (4 pi) / (3 sqrt 3) (the doublet's factor, see doublet2)
//   [36..38] unit normal, [39] strength Gamma
//   [40] core length^4, [41] wing index, [42..45] |d_k|^2,
//   [46] far-field length squared lo (fl32(ff2 - hi), 0 when hi is infinite),
//   [47] near/far band: a bound on |fl32 |x_hi - c_hi|^2 - |x - c|^2| for targets x at the
//        far-field radius (0 when hi is infinite)
// FP64 record (PanelRec<double>, 28 doubles = 224 B):
//   [0..11] corners, [16..18] centre, [19] far-field length squared, [20..22] normal,
//   [23] area / (4 pi), [24] Gamma, [25] core length, [26] wing index.
template <class R>
struct PanelRecSize;
template <>
struct PanelRecSize<float> { static constexpr int value = 48; };
template <>
struct PanelRecSize<double> { static constexpr int value = 28; };

template <class R>
struct __align__(16) PanelRec {
    R v[PanelRecSize<R>::value];
};
static_assert(sizeof(PanelRec<float>) == 192, "FP32 panel record is 192 bytes");
static_assert(sizeof(PanelRec<double>) == 224, "FP64 panel record is 224 bytes");

constexpr int kRec32Gamma = 39;  // strength slot of the FP32 record
constexpr double kInv3Sqrt3 = 0.19245008972987526;  // 1 / (3 sqrt 3), folded into slot 35
constexpr int kRec32DD = 42;     // |d_k|^2 of the FP32 record's four segments (slots 42..45)
constexpr int kRec32FF2Lo = 46;    // lo part of the far-field length squared
constexpr int kRec32FF2Band = 47;  // band of the hi-part near/far test (above)
// Near/far decisions (panel.rs:53-57) that FP32 cannot make: the squared distance from the
// float-float difference carries a relative error of a few 2^-24, so within this relative
// band of the far-field length squared the f64 distance of the float-float points decides.
constexpr float kNearFarBand = 4.0e-6f;
constexpr int kRec64Gamma = 24;  // strength slot of the FP64 record

// Chain record (FP32, same 48-float size): an open chain of up to 4 wake segments that
// each belong to two adjacent vortex rings (or one at the wake's edge), with the
// difference of the two rings' strengths. Slots: [0..2] anchor hi, [3..5] anchor lo
// (float-float point 2), [6..20] offsets of points 0..4 from the anchor, [21..32] segment
// vectors, [33..36] 1/|d|^2, [37..40] strength difference / 4 pi, [41] rc^4, [42] wing,
// [43] sum of |strength differences| (0: nothing to evaluate), [44..47] |d|^2.
constexpr int kChainOff = 6, kChainD = 21, kChainIl = 33, kChainG = 37, kChainRc4 = 41, kChainWing = 42, kChainAny = 43,
              kChainDD = 44;
constexpr int kChainSegs = 4;

// ---------------------------------------------------------------------------------------
// Model and step parameters
// ---------------------------------------------------------------------------------------
struct DevModel {
    int N = 0;        // span lines
    int S = 0;        // wings
    int Np = 0;       // span points (N + S)
    int W = 0;        // panels per line element (wake rows of panels)
    int Wp = 0;       // points per line element (W + 1)
    long long P_pan = 0, P_pts = 0;
    double density = 1.225;
    double rep_chord = 0.0;          // representative chord (mean chord length)
    double first_rel = 0.75, last_rel = 0.25, damping = 0.0, far_field_ratio = 5.0;
    int first_dir = 0;               // 0 chord, 1 freestream, 2 actual velocity
    int symmetry = 0;                // 0 none, 1 X, 2 Y, 3 Z
    int neglect_self = 0;
    int output_body = 0;             // output coordinate system 0 global, 1 body
    int include_viscous_lift = 0;
    long long end_index = 0;         // wake points that get induced velocities
    // constant line force model
    const d3* span_s_local = nullptr;
    const d3* span_e_local = nullptr;
    const d3* chord_not_rotated = nullptr;
    const double* chord_len = nullptr;
    const double* span_len_local = nullptr;
    const int* wing_of_line = nullptr;
    const int* wing_start = nullptr;
    const int* wing_end = nullptr;
    const unsigned char* is_virtual = nullptr;
    const FoilP* foils = nullptr;
    const int* sp_line = nullptr;    // [Np] line whose start (or end, sp_end) is span point k
    const unsigned char* sp_end = nullptr;
    const int* sp_val_a = nullptr;   // [Np] value mapping control -> span points
    const int* sp_val_b = nullptr;   //       value = (c[a] + c[b]) * 0.5, or c[a] if a == b
    const double* panel_core = nullptr;  // [W*N]
    // per-step geometry
    d3* chord_local = nullptr;
    d3* chord_global = nullptr;
    d3* chord_span_pts = nullptr;
    d3* span_s = nullptr;
    d3* span_e = nullptr;
    d3* span_pts = nullptr;
    d3* ctrl = nullptr;
    d3* felt_ctrl = nullptr;
    d3* felt_span = nullptr;
    // [2N] per line, the plane perpendicular to its span: e1 = the chord made perpendicular
    // to the span, unit; e2 = span direction x e1 (line_basis)
    d3* solve_basis = nullptr;
};

// In-plane basis of a line (the plane perpendicular to its span direction): the solver only
// uses the velocity's components in that plane (the span component is projected out before
// the angle of attack), so its influence matrix can hold two components per entry. A chord
// along the span (degenerate) takes the in-plane axis closest to x or y instead.
__device__ inline void line_basis(d3 chord, d3 span_s, d3 span_e, d3& e1, d3& e2) {
    const d3 sd = normalize(span_e - span_s);
    d3 c = chord - sd * dot(chord, sd);
    if (!(len2(c) > 1e-300)) {
        c = mk(1, 0, 0) - sd * sd.x;
        if (!(len2(c) > 1e-300)) c = mk(0, 1, 0) - sd * sd.y;
    }
    e1 = normalize(c);
    e2 = cross(sd, e1);
}

struct StepParams {
    double time = 0.0, dt = 0.0;
    d3 translation{0, 0, 0}, rotation{0, 0, 0}, velocity_linear{0, 0, 0}, velocity_angular{0, 0, 0};
    double local_wing_angles[kMaxWings] = {0};
};

// Error word written by kernels whose bounded waits ran out (0 = none).
enum DeviceError : int { kDevOk = 0, kDevTimeout = 1, kDevSingular = 2 };

// Polls a bounded device-side wait makes before it gives up and records kDevTimeout.
constexpr int kWaitPolls = 1 << 22;

}  // namespace sbgpu
