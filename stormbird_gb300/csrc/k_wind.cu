// Freestream generator (sm_103a): the reference's CompleteSailModel::freestream_velocity
// (stormbird/src/lifting_line/complete_sail_model/mod.rs:213-257) evaluated on the GPU at
// every freestream point of a simulation, so a step needs no host freestream.
//
// Per point: height above the water plane (environment.rs:91-96), steady velocity from the
// height profile (Constant, PowerModel power_model.rs:31-47, LogarithmicModel with the
// Businger-Dyer correction logarithmic_model.rs:56-110), plus the parallel gust; the
// perpendicular (up x wind direction) and vertical gusts (discretized_spectrum.rs:38-46;
// wind_condition/mod.rs:58-87; environment.rs:131-155), plus the ship's linear velocity
// along the zero direction. Control points then get the inflow corrections
// (environment.rs:242-271, inflow_corrections.rs:21-95) at the apparent wind direction of
// the steady wind at 10 m (environment.rs:273-292). f64 throughout.
//
// k_controller_input: the flow measurements a CompleteSailModel's controller reads from
// that freestream before each steady-state step.
#include "sb_kernels.h"

namespace sbgpu {

namespace {

__device__ double spectrum_value(const double* s, int n, double time) {
    double out = 0.0;
    for (int i = 0; i < n; ++i) out += s[n + i] * sin(kTau * s[i] * time + s[2 * n + i]);
    return out;
}

__device__ double velocity_at_height(const WindDevice& w, double h) {
    if (w.vv_kind == 0) return w.vv_constant;
    if (w.vv_kind == 1) {
        const double f = w.power_factor > 0.0 ? pow(h / w.reference_height, w.power_factor) : 1.0;
        return w.reference_velocity * f;
    }
    const double scale = w.friction_velocity / w.von_karman;
    double neutral = 0.0;
    if (!(w.surface_roughness <= 0.0 || h <= 0.0)) neutral = scale * log(h / w.surface_roughness);
    double unscaled = 0.0;
    if (w.has_obukhov) {
        const double zeta = h / w.obukhov_length;
        if (w.obukhov_length > 0.0) {
            unscaled = -w.stable_coefficient * zeta;
        } else {
            const double x = pow(1.0 - w.unstable_coefficient * zeta, 0.25);
            unscaled = 2.0 * log((1.0 + x) / 2.0) + log((1.0 + x * x) / 2.0) + (-2.0 * atan(x) + kPi / 2.0);
        }
    }
    return neutral - unscaled * scale;
}

// stormath/src/interpolation.rs:17-100 on values produced on demand by y(i)
template <class T, class Y>
__device__ T interpolate(double x, const double* xd, int n, Y&& y) {
    auto two = [&](double x0, double x1, T y0, T y1) -> T {
        if (x <= x0) return y0;
        if (x >= x1) return y1;
        return y0 + (y1 - y0) * ((x - x0) / (x1 - x0));
    };
    if (n == 1) return y(0);
    if (n == 2) return two(xd[0], xd[1], y(0), y(1));
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (xd[mid] > x) hi = mid;
        else lo = mid;
    }
    if (lo == n - 1) return y(lo);
    return two(xd[lo], xd[lo + 1], y(lo), y(lo + 1));
}

__device__ d3 true_wind_direction(const WindDevice& w) {
    return rotate_around_axis(w.zero, w.direction_coming_from, w.axis);
}

__global__ void k_wind_freestream(WindDevice w, const d3* ctrl, const int* wing_of_line, int N, const d3* wake,
                                  long long n_wake, d3* out) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= N + n_wake) return;
    const double time = w.step[0];
    const d3 linear = w.zero * w.step[1];
    const d3 p = i < N ? ctrl[i] : wake[i - N];
    const double h = fmax(dot(p, w.up) - w.water_plane_height, 0.0);
    double parallel = velocity_at_height(w, h);
    if (w.spec_n[0] >= 0) parallel += spectrum_value(w.spectra + w.spec_off[0], w.spec_n[0], time);
    const d3 pdir = true_wind_direction(w);
    const double perpendicular = w.spec_n[1] >= 0 ? spectrum_value(w.spectra + w.spec_off[1], w.spec_n[1], time) : 0.0;
    const d3 perp_dir = cross(w.up, pdir);
    const double vertical = w.spec_n[2] >= 0 ? spectrum_value(w.spectra + w.spec_off[2], w.spec_n[2], time) : 0.0;
    d3 u = (parallel * pdir + perpendicular * perp_dir + vertical * w.up) + linear;
    if (i < N && w.n_dirs > 0) {
        // apparent wind direction of the steady wind at 10 m
        const d3 location = 10.0 * w.up;
        const double vh = velocity_at_height(w, fmax(dot(location, w.up) - w.water_plane_height, 0.0));
        const double direction = signed_angle_between(w.zero, vh * pdir + linear, w.axis);
        const int wing = wing_of_line[i];
        const double hc = dot(p, w.up);
        const d3 vel = u;
        auto corrected = [&](int d) -> d3 {
            const double* c = w.corr + w.corr_off[d];
            const int len = w.corr_len[d];
            const long long r0 = w.ranges[2 * (static_cast<long long>(d) * w.S + wing)];
            const long long r1 = w.ranges[2 * (static_cast<long long>(d) * w.S + wing) + 1];
            const double* hs = c + r0;
            const double* ms = c + len + r0;
            const double* as = c + 2 * len + r0;
            const int m = static_cast<int>(r1 - r0);
            const double mag = interpolate<double>(hc, hs, m, [&](int k) { return ms[k]; });
            const double ang = interpolate<double>(hc, hs, m, [&](int k) { return as[k]; });
            return mag * rotate_around_axis(vel, ang, w.up);
        };
        u = interpolate<d3>(direction, w.dirs, w.n_dirs, corrected);
    }
    out[i] = u;
}

// ControllerInput::new_from_velocity (controller/input.rs:99-157) per line, on the geometry
// k_prep_geometry left for the current wing angles and motion: out[i] = |v_i|,
// out[N + i] = the angle of attack (force_calculations.rs:79-107: signed angle from the global
// chord to v about the span line's direction, 0 when |v| <= MIN_POSITIVE), out[2N + i] = the
// apparent wind direction (environment.rs:315-345: signed angle from the unrotated chord of
// the wing's first strip, moved by the rigid body's rotation, to v about that strip's global
// span direction).
__global__ void k_controller_input(DevModel m, StepParams p, const d3* v, double* out) {
    const int N = m.N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const d3 u = v[i];
        const d3 span_dir = normalize(m.span_e[i] - m.span_s[i]);
        out[i] = len(u);
        out[N + i] = len(u) > kMinPositive ? signed_angle_between(m.chord_global[i], u, span_dir) : 0.0;
        const int ws = m.wing_start[m.wing_of_line[i]];
        const d3 axis = normalize(m.span_e[ws] - m.span_s[ws]);
        const d3 chord_first = rotate_xyz(m.chord_not_rotated[ws], p.rotation);
        out[2 * N + i] = signed_angle_between(chord_first, u, axis);
    }
}

}  // namespace

cudaError_t launch_controller_input(const DevModel& m, const StepParams& p, const d3* v, double* out, cudaStream_t s) {
    if (m.N <= 0) return cudaSuccess;
    k_controller_input<<<(m.N + 127) / 128, 128, 0, s>>>(m, p, v, out);
    return cudaGetLastError();
}

cudaError_t launch_wind_freestream(const WindDevice& w, const d3* ctrl, const int* wing_of_line, int N, const d3* wake,
                                   long long n_wake, d3* out, cudaStream_t s) {
    const long long n = N + n_wake;
    if (n <= 0) return cudaSuccess;
    k_wind_freestream<<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(w, ctrl, wing_of_line, N, wake, n_wake, out);
    return cudaGetLastError();
}

}  // namespace sbgpu
