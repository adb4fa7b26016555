// Line-force-model geometry and dynamic-wake update kernels (sm_103a). HBM-bound.
//
// Reference: stormbird/src/line_force_model/data_update.rs:13-90 (global geometry),
// force_calculations.rs:50-69 (felt velocity), value_mapping.rs:87-137 (control point ->
// span point values), lifting_line/wake/dynamic_wake/update_data.rs:28-328 (wake points
// before solving, panels, strength shift) and initialization.rs:12-71.
//
// The wake points live in two buffers (current / next). A step reads the current points
// and velocities and writes the next points, so the reference's in-place reverse sweep
// (new row i = old row i-1 + dt * velocity) becomes one independent update per point.
// Positions are integrated in f64; the panel records for the sweep are written in FP32
// (and f64 for the first row and in the FP64 precision mode).
#include "sb_device.cuh"
#include "sb_kernels.h"

namespace sbgpu {

// ---------------------------------------------------------------------------------------
// Geometry of the line force model for one step. One CTA: O(N) work.
// ---------------------------------------------------------------------------------------
__device__ void prep_geometry_block(const DevModel& m, const StepParams& p, const d3* fs_ctrl, d3* mean_out) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < m.N; i += nt) {
        int w = m.wing_of_line[i];
        int ws = m.wing_start[w];
        d3 axis = m.span_e_local[ws] - m.span_s_local[ws];  // data_access.rs:256-258
        d3 cl = rotate_around_axis(m.chord_not_rotated[i], p.local_wing_angles[w], axis);
        m.chord_local[i] = cl;
        m.chord_global[i] = rotate_xyz(cl, p.rotation);
        d3 s = rotate_xyz(m.span_s_local[i], p.rotation) + p.translation;
        d3 e = rotate_xyz(m.span_e_local[i], p.rotation) + p.translation;
        m.span_s[i] = s;
        m.span_e[i] = e;
        d3 c = 0.5 * (s + e);
        m.ctrl[i] = c;
        if (m.solve_basis) line_basis(m.chord_global[i], s, e, m.solve_basis[2 * i], m.solve_basis[2 * i + 1]);
        if (fs_ctrl) {
            // rigid_body_motion.rs:53-60
            d3 mv = p.velocity_linear + cross(p.velocity_angular, c - p.translation);
            m.felt_ctrl[i] = fs_ctrl[i] - mv;
        }
    }
    __syncthreads();
    for (int k = tid; k < m.Np; k += nt) {
        int l = m.sp_line[k];
        m.span_pts[k] = m.sp_end[k] ? m.span_e[l] : m.span_s[l];
        int a = m.sp_val_a[k], b = m.sp_val_b[k];
        m.chord_span_pts[k] = (a == b) ? m.chord_global[a] : (m.chord_global[a] + m.chord_global[b]) * 0.5;
        if (fs_ctrl) m.felt_span[k] = (a == b) ? m.felt_ctrl[a] : (m.felt_ctrl[a] + m.felt_ctrl[b]) * 0.5;
    }
    if (mean_out && tid == 0) {
        // simulation.rs:74-75: sum in order, then divide
        d3 s = mk(0, 0, 0);
        for (int i = 0; i < m.N; ++i) s = s + fs_ctrl[i];
        *mean_out = s / static_cast<double>(m.N);
    }
}

__global__ void k_prep_geometry(DevModel m, StepParams p, const d3* fs_ctrl, d3* mean_out) {
    prep_geometry_block(m, p, fs_ctrl, mean_out);
}

// The geometry of every case of a batch: one CTA per case.
__global__ void k_prep_geometry_jobs(const CaseStepJob* jobs) {
    const CaseStepJob& J = jobs[blockIdx.x];
    prep_geometry_block(J.m, J.p, J.fs_ctrl, nullptr);
}

cudaError_t launch_prep_geometry(const DevModel& m, const StepParams& p, const d3* fs_ctrl, d3* mean_out, cudaStream_t s) {
    k_prep_geometry<<<1, 512, 0, s>>>(m, p, fs_ctrl, mean_out);
    return cudaGetLastError();
}

cudaError_t launch_prep_geometry_jobs(const CaseStepJob* jobs, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_prep_geometry_jobs<<<n, 512, 0, s>>>(jobs);
    return cudaGetLastError();
}

// Direction of the first free wake row (update_data.rs:152-199).
__device__ inline d3 first_row_direction(const DevModel& m, int j, const d3* vel_row0, const d3* vel_row1, int steps_done,
                                         d3 felt_span_j) {
    if (m.first_dir == 0) return normalize(m.chord_span_pts[j]);
    if (m.first_dir == 2 && steps_done > 2) return normalize(0.5 * (vel_row0[j] + vel_row1[j]));
    return normalize(felt_span_j);
}

// ---------------------------------------------------------------------------------------
// Initialisation (initialization.rs:12-41): W+1 passes of update_wake_points_before_solving
// with a uniform velocity U. One thread per spanwise column, in place on the current buffer.
// Without shape damping the passes collapse to rows 0, 1, then rows 2..W-1 reached by
// repeated addition of dt*U along the column (the same additions, in the same order, as
// the reference's passes), and the last row. With damping the passes are run literally.
// ---------------------------------------------------------------------------------------
__global__ void k_wake_init(DevModel m, WakeBuffers w, const d3* mean_dev, d3 U_host, double dt, int fill_rows) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    const d3 U = mean_dev ? *mean_dev : U_host;
    // strengths and velocities (both strength buffers hold zeros afterwards)
    for (long long id = j; id < m.P_pan; id += static_cast<long long>(gridDim.x) * blockDim.x) {
        w.str_old[id] = 0.0;
        w.str_new[id] = 0.0;
    }
    for (long long id = j; id < m.P_pts; id += static_cast<long long>(gridDim.x) * blockDim.x) w.vel[id] = U;
    if (j >= m.Np) return;
    const int Np = m.Np, W = m.W;
    d3* P = w.pts_old;
    const d3 S = m.span_pts[j];
    const d3 dir1 = first_row_direction(m, j, nullptr, nullptr, 0, U);
    const double L1 = m.rep_chord * m.first_rel;
    const double Ll = m.last_rel * m.rep_chord;
    const d3 dU = dt * U;
    if (fill_rows)  // builder state: every row on the span points (builder.rs:128-135)
        for (int s = 0; s <= W; ++s) P[static_cast<long long>(s) * Np + j] = S;
    if (m.damping <= 0.0) {
        P[j] = S;
        if (W == 1) {
            P[Np + j] = S + Ll * normalize(U);
            return;
        }
        d3 r1 = S + dir1 * L1;
        P[Np + j] = r1;
        d3 prev2 = S, prev = r1;
        for (int s = 2; s <= W - 1; ++s) {
            d3 r = prev + dU;
            P[static_cast<long long>(s) * Np + j] = r;
            prev2 = prev;
            prev = r;
        }
        P[static_cast<long long>(W) * Np + j] = prev + Ll * normalize(prev - prev2);
        return;
    }
    const double D = m.damping;
    for (int pass = 0; pass <= W; ++pass) {
        P[j] = S;
        for (int s = W; s >= 2; --s) {
            d3 integ = P[static_cast<long long>(s - 1) * Np + j] + dU;
            long long ci = static_cast<long long>(s) * Np + j;
            P[ci] = P[ci] * D + integ * (1.0 - D);
        }
        d3 est = P[j] + dir1 * L1;
        P[Np + j] = P[Np + j] * D + est * (1.0 - D);
        if (W > 1) {
            d3 a = P[static_cast<long long>(W - 1) * Np + j], b = P[static_cast<long long>(W - 2) * Np + j];
            P[static_cast<long long>(W) * Np + j] = a + Ll * normalize(a - b);
        } else {
            P[Np + j] = P[j] + Ll * normalize(U);
        }
    }
}

cudaError_t launch_wake_init(const DevModel& m, const WakeBuffers& w, const d3* mean_dev, d3 U, double dt, int fill_rows,
                             cudaStream_t s) {
    int threads = 128;
    int blocks = (m.Np + threads - 1) / threads;
    if (blocks < 64) blocks = 64;  // the zero-fill loops are grid-strided
    k_wake_init<<<blocks, threads, 0, s>>>(m, w, mean_dev, U, dt, fill_rows);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// The next wake points (update_data.rs:65-82, 90-99, 205-252, 262-316): rows 0..W-1 one per
// thread, and the last row by the thread of row W-1, from rows W-1 and W-2 (row W-2
// evaluated again there by the same expression, so it equals what its own thread writes).
// ---------------------------------------------------------------------------------------
// Row s < W of column j of the next points.
__device__ inline d3 advected_point(const DevModel& m, const WakeBuffers& w, double dt, int steps_done, int s, int j) {
    const long long Np = m.Np;
    const double D = m.damping;
    if (s == 0) return m.span_pts[j];
    if (s == 1) {
        d3 dir = first_row_direction(m, j, w.vel, w.vel + Np, steps_done, m.felt_span[j]);
        d3 est = m.span_pts[j] + dir * (m.rep_chord * m.first_rel);
        return D > 0.0 ? w.pts_old[Np + j] * D + est * (1.0 - D) : est;
    }
    const long long id = static_cast<long long>(s) * Np + j, pi = id - Np;
    d3 integ = w.pts_old[pi] + dt * w.vel[pi];
    return D > 0.0 ? w.pts_old[id] * D + integ * (1.0 - D) : integ;
}

__device__ inline void wake_advect_elem(const DevModel& m, const WakeBuffers& w, double dt, int steps_done, long long id) {
    const long long Np = m.Np;
    if (id >= static_cast<long long>(m.W) * Np) return;
    const int s = static_cast<int>(id / Np), j = static_cast<int>(id % Np);
    const d3 out = advected_point(m, w, dt, steps_done, s, j);
    w.pts_new[id] = out;
    if (s == m.W - 1) {  // last row (update_data.rs:262-292)
        const d3 dir = m.W > 1 ? normalize(out - advected_point(m, w, dt, steps_done, s - 1, j)) : normalize(m.felt_span[j]);
        w.pts_new[static_cast<long long>(m.W) * Np + j] = out + (m.last_rel * m.rep_chord) * dir;
    }
}

__global__ void k_wake_advect(DevModel m, WakeBuffers w, double dt, int steps_done) {
    wake_advect_elem(m, w, dt, steps_done, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

constexpr int kAdvectThreads = 256;

cudaError_t launch_wake_advect(const DevModel& m, const WakeBuffers& w, double dt, int steps_done, cudaStream_t s) {
    const long long tot = static_cast<long long>(m.W) * m.Np;
    k_wake_advect<<<static_cast<unsigned>((tot + kAdvectThreads - 1) / kAdvectThreads), kAdvectThreads, 0, s>>>(
        m, w, dt, steps_done);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Panel records from the new points (panel.rs:26-50, geometry_functions.rs:11-30,
// dynamic_wake/mod.rs:82-103) and the strength shift (update_data.rs:319-328).
// ---------------------------------------------------------------------------------------
// Panel::new (panel.rs:26-50, geometry_functions.rs:11-30) for corners p[0..3], written as
// the FP32 sweep record (float-float positions) and, when r64 is not null, the FP64 record.
// With an FP64 record (row 0, the FP64 mode) every field is evaluated in f64 as the reference
// does and the FP32 record is its rounding. Without one, the fields that are only stored in
// FP32 (edge reciprocals, area, normal) are evaluated in FP32 from the f64 edge vectors, and
// the far-field radius^2 is max(|p1-p0|^2, |p2-p1|^2) * ratio^2, the reference's
// (ratio * max(|p1-p0|, |p2-p1|))^2 without its square roots: this part's FP64 rate is 1/64 of
// its FP32 rate, and the f64 square roots and divisions made the record kernel compute-bound.
// Far-field length squared as hi + lo (the f64 near/far decision of the sweeps reads both),
// and the band of the sweeps' FP32 test from hi parts alone (panel.rs:53-57). A target x at
// the far-field radius r from the centre c has |x_k| <= |c|_inf + r; the hi parts of x and c
// are within 2^-24 of each coordinate and their FP32 difference within 2^-24 of itself, so
// |e_hi - e| <= d = sqrt(3) 2^-24 (2 |c|_inf + 2 r) and ||e_hi|^2 - r^2| <= 2 r d + d^2, plus
// the FP32 rounding of |e_hi|^2 and of ff2 (below 2^-21 ff2). The band is twice that sum.
__device__ inline void far_field_fields(double ff2, d3 c, float* hi, float* lo, float* band) {
    const float h = static_cast<float>(ff2);
    *hi = h;
    if (isinf(h)) {
        *lo = 0.f;
        *band = 0.f;
        return;
    }
    *lo = static_cast<float>(ff2 - static_cast<double>(h));
    const float r = __fsqrt_ru(h);
    const float cm = fmaxf(fmaxf(fabsf(static_cast<float>(c.x)), fabsf(static_cast<float>(c.y))),
                           fabsf(static_cast<float>(c.z)));
    const float d = 1.7320509f * 0x1p-24f * (2.f * cm + 2.f * r);
    *band = 2.f * ((2.f * r * d + d * d) + 0x1p-21f * h);
}

__device__ void write_panel_records(const d3 (&pp)[4], double rc, double g, double far_field_ratio, int wing,
                                    PanelRec<float>* r32, PanelRec<double>* r64) {
    const d3 c = 0.25 * (((pp[0] + pp[1]) + pp[2]) + pp[3]);
    PanelRec<float> r;
    auto split = [](double x, float* hi, float* lo) {
        float h = static_cast<float>(x);
        *hi = h;
        *lo = static_cast<float>(x - static_cast<double>(h));
    };
    double l2[4];
    for (int k = 0; k < 4; ++k) {
        const d3 ok = pp[k] - c;
        r.v[3 * k] = static_cast<float>(ok.x);
        r.v[3 * k + 1] = static_cast<float>(ok.y);
        r.v[3 * k + 2] = static_cast<float>(ok.z);
        const d3 dk = pp[(k + 1) & 3] - pp[k];
        r.v[12 + 3 * k] = static_cast<float>(dk.x);
        r.v[12 + 3 * k + 1] = static_cast<float>(dk.y);
        r.v[12 + 3 * k + 2] = static_cast<float>(dk.z);
        l2[k] = len2(dk);
        r.v[kRec32DD + k] = static_cast<float>(l2[k]);
    }
    split(c.x, &r.v[28], &r.v[32]);
    split(c.y, &r.v[29], &r.v[33]);
    split(c.z, &r.v[30], &r.v[34]);
    r.v[kRec32Gamma] = static_cast<float>(g);
    // core length^4; a zero core (reference: factor 1) only occurs in the horseshoe path, which
    // runs in FP64, so the FP32 sweep always evaluates d^2 / sqrt(d^4 + rc^4)
    const double rc2 = rc * rc;
    r.v[40] = static_cast<float>(rc2 * rc2);
    r.v[41] = static_cast<float>(wing);
    for (int k = kRec32DD + 4; k < 48; ++k) r.v[k] = 0.f;
    if (r64) {
        const double la = sqrt(l2[0]), lb = sqrt(l2[1]), lc = sqrt(l2[2]), ld = sqrt(l2[3]);
        const double sp = (la + lb + lc + ld) * 0.5;
        const double area = sqrt((sp - la) * (sp - lb) * (sp - lc) * (sp - ld));
        const d3 n = normalize(cross(pp[2] - pp[0], pp[3] - pp[1]));
        const double t = fmax(la, lb) * far_field_ratio;
        const double ff2 = t * t;
        for (int k = 0; k < 4; ++k) r.v[24 + k] = l2[k] > 0.0 ? static_cast<float>(1.0 / l2[k]) : 0.f;
        far_field_fields(ff2, c, &r.v[31], &r.v[kRec32FF2Lo], &r.v[kRec32FF2Band]);
        r.v[35] = static_cast<float>(area * kFourPiInv * kInv3Sqrt3);
        r.v[36] = static_cast<float>(n.x);
        r.v[37] = static_cast<float>(n.y);
        r.v[38] = static_cast<float>(n.z);
        PanelRec<double> q;
        for (int k = 0; k < 4; ++k) {
            q.v[3 * k] = pp[k].x;
            q.v[3 * k + 1] = pp[k].y;
            q.v[3 * k + 2] = pp[k].z;
            q.v[12 + k] = 0.0;
        }
        q.v[16] = c.x;
        q.v[17] = c.y;
        q.v[18] = c.z;
        q.v[19] = ff2;
        q.v[20] = n.x;
        q.v[21] = n.y;
        q.v[22] = n.z;
        q.v[23] = area * kFourPiInv;
        q.v[kRec64Gamma] = g;
        q.v[25] = rc;
        q.v[26] = static_cast<double>(wing);
        q.v[27] = 0.0;
        *r64 = q;
    } else {
        float lf[4];
        for (int k = 0; k < 4; ++k) {
            const float q = static_cast<float>(l2[k]);
            r.v[24 + k] = q > 0.f ? __frcp_rn(q) : 0.f;
            lf[k] = __fsqrt_rn(q);
        }
        const float sp = (lf[0] + lf[1] + lf[2] + lf[3]) * 0.5f;
        // a degenerate quadrilateral can round the product below zero: area 0
        const float prod = fmaxf((sp - lf[0]) * (sp - lf[1]) * (sp - lf[2]) * (sp - lf[3]), 0.f);
        r.v[35] = __fsqrt_rn(prod) * static_cast<float>(kFourPiInv * kInv3Sqrt3);
        const d3 a = pp[2] - pp[0], b = pp[3] - pp[1];
        const float ax = static_cast<float>(a.x), ay = static_cast<float>(a.y), az = static_cast<float>(a.z);
        const float bx = static_cast<float>(b.x), by = static_cast<float>(b.y), bz = static_cast<float>(b.z);
        const float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
        const float nl = __fsqrt_rn(nx * nx + ny * ny + nz * nz);
        const float inl = nl > 0.f ? __frcp_rn(nl) : 0.f;
        r.v[36] = nx * inl;
        r.v[37] = ny * inl;
        r.v[38] = nz * inl;
        far_field_fields(fmax(l2[0], l2[1]) * (far_field_ratio * far_field_ratio), c, &r.v[31], &r.v[kRec32FF2Lo],
                         &r.v[kRec32FF2Band]);
    }
    *r32 = r;
}

__device__ inline void wake_panel_elem(const DevModel& m, const WakeBuffers& w, int shift, long long id) {
    if (id >= m.P_pan) return;
    const int N = m.N;
    const long long Np = m.Np;
    const int s = static_cast<int>(id / N), j = static_cast<int>(id % N);
    const int wg = m.wing_of_line[j];
    const d3* P = w.pts_new;
    const d3 pp[4] = {P[s * Np + j + wg], P[s * Np + j + 1 + wg], P[(s + 1) * Np + j + 1 + wg], P[(s + 1) * Np + j + wg]};
    double g;
    if (shift) g = (s == 0) ? w.str_old[j] : w.str_old[id - N];
    else g = w.str_old[id];
    w.str_new[id] = g;
    // A panel of zero strength is skipped by every sweep (induced_velocity_calc.rs:203): only
    // its strength slot matters, so its record is not rebuilt. While a wake fills (the first
    // W steps) that is every row past the newest strengths; row 0 (the frozen-wake matrix)
    // and the FP64 records are always built.
    if (g == 0.0 && s != 0 && !w.rec64) {
        w.rec32[id].v[kRec32Gamma] = 0.f;
        return;
    }
    PanelRec<double> q;
    const bool need64 = (s == 0) || w.rec64;
    write_panel_records(pp, m.panel_core[id], g, m.far_field_ratio, wg, &w.rec32[id], need64 ? &q : nullptr);
    if (s == 0) w.row0_64[j] = q;
    if (w.rec64) w.rec64[id] = q;
}

__global__ void k_wake_panels(DevModel m, WakeBuffers w, int shift) {
    wake_panel_elem(m, w, shift, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

// ---------------------------------------------------------------------------------------
// Chain records. Panel (s, j) of wing w has corners p0 = P[s][j+w], p1 = P[s][j+1+w],
// p2 = P[s+1][j+1+w], p3 = P[s+1][j+w] and segments p0->p1, p1->p2, p2->p3, p3->p0
// (mod.rs:82-103 indexing, panel.rs:99-118 ring). The spanwise segment P[r][j+w] ->
// P[r][j+1+w] is segment 0 of panel (r, j) and, reversed, segment 2 of panel (r-1, j);
// the streamwise segment P[s][c] -> P[s+1][c] on column c = j + w is segment 1 of panel
// (s, j-1) and, reversed, segment 3 of panel (s, j). The unit-strength velocity of a
// segment changes sign with its direction (vortex_line.rs:18-106 is antisymmetric in the
// two end points, the core factor symmetric), so with one core length for all panels the
// two rings' contributions are one evaluation with the strength difference.
// ---------------------------------------------------------------------------------------
__device__ inline double chain_strength(const ChainArgs& a, int s, int j) {
    return (s >= 0 && s < a.W) ? a.str[static_cast<long long>(s) * a.N + j] : 0.0;
}

__device__ inline void chain_record_elem(const ChainArgs& a, long long n_build, long long id) {
    if (id >= n_build) return;
    const long long q = id / a.Bq, local = id % a.Bq;
    const long long Np = a.Np;
    d3 pt[kChainSegs + 1];
    double g[kChainSegs] = {0.0, 0.0, 0.0, 0.0};
    int npts = 0, wing = 0;
    if (local < 4LL * a.SP) {  // spanwise chain
        const int r = static_cast<int>(4 * q + local / a.SP);
        const int piece = static_cast<int>(local % a.SP);
        wing = a.span_tab[3 * piece];
        const int j0 = a.span_tab[3 * piece + 1], n = a.span_tab[3 * piece + 2];
        if (r <= a.W) {
            npts = n + 1;
            for (int k = 0; k <= n; ++k) pt[k] = a.pts[r * Np + j0 + k + wing];
            for (int k = 0; k < n; ++k) g[k] = chain_strength(a, r, j0 + k) - chain_strength(a, r - 1, j0 + k);
        }
    } else {  // streamwise chain of panel rows 4q..4q+3 on one point column
        const int col = static_cast<int>(local - 4LL * a.SP);
        wing = a.col_tab[2 * col];
        const int j = a.col_tab[2 * col + 1];
        const int ws = a.wing_start[wing], we = a.wing_end[wing];
        const int s0 = static_cast<int>(4 * q);
        if (s0 < a.W) {
            const int n = min(kChainSegs, a.W - s0);
            npts = n + 1;
            for (int k = 0; k <= n; ++k) pt[k] = a.pts[static_cast<long long>(s0 + k) * Np + col];
            for (int k = 0; k < n; ++k) {
                const double left = j - 1 >= ws ? chain_strength(a, s0 + k, j - 1) : 0.0;
                const double right = j < we ? chain_strength(a, s0 + k, j) : 0.0;
                g[k] = left - right;
            }
        }
    }
    PanelRec<float> rec;
    for (int k = 0; k < 48; ++k) rec.v[k] = 0.f;
    if (npts > 1) {
        for (int k = npts; k <= kChainSegs; ++k) pt[k] = pt[npts - 1];  // empty segments
        const d3 anchor = pt[2 < npts ? 2 : npts - 1];
        auto split = [](double x, float* hi, float* lo) {
            const float h = static_cast<float>(x);
            *hi = h;
            *lo = static_cast<float>(x - static_cast<double>(h));
        };
        split(anchor.x, &rec.v[0], &rec.v[3]);
        split(anchor.y, &rec.v[1], &rec.v[4]);
        split(anchor.z, &rec.v[2], &rec.v[5]);
        for (int k = 0; k <= kChainSegs; ++k) {
            const d3 o = pt[k] - anchor;
            rec.v[kChainOff + 3 * k] = static_cast<float>(o.x);
            rec.v[kChainOff + 3 * k + 1] = static_cast<float>(o.y);
            rec.v[kChainOff + 3 * k + 2] = static_cast<float>(o.z);
        }
        double any = 0.0;
        for (int k = 0; k < kChainSegs; ++k) {
            const d3 dk = pt[k + 1] - pt[k];
            rec.v[kChainD + 3 * k] = static_cast<float>(dk.x);
            rec.v[kChainD + 3 * k + 1] = static_cast<float>(dk.y);
            rec.v[kChainD + 3 * k + 2] = static_cast<float>(dk.z);
            const float l2 = static_cast<float>(len2(dk));
            rec.v[kChainIl + k] = l2 > 0.f ? __frcp_rn(l2) : 0.f;  // FP32: an f64 division costs ~10 FP64 instructions here
            rec.v[kChainDD + k] = l2;
            rec.v[kChainG + k] = static_cast<float>(g[k] * kFourPiInv);
            any += fabs(g[k]);
        }
        const double rc2 = a.rc * a.rc;
        rec.v[kChainRc4] = static_cast<float>(rc2 * rc2);
        rec.v[kChainWing] = static_cast<float>(wing);
        rec.v[kChainAny] = static_cast<float>(any);
    }
    a.out[id] = rec;
}

__global__ void k_chain_records(ChainArgs a, long long n_build) {
    chain_record_elem(a, n_build, blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

cudaError_t launch_chain_records(const ChainArgs& a, long long n_build, cudaStream_t s) {
    if (n_build <= 0) return cudaSuccess;
    k_chain_records<<<static_cast<unsigned>((n_build + 127) / 128), 128, 0, s>>>(a, n_build);
    return cudaGetLastError();
}

// Records of caller-given panels (corners [P][4][3], strengths, core lengths) for the
// standalone sweep sb_panel_sweep.
__global__ void k_panels_from_corners(const double* corners, const double* strengths, const double* cores, long long P,
                                      double far_field_ratio, PanelRec<float>* r32, PanelRec<double>* r64) {
    long long id = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (id >= P) return;
    const double* c = corners + id * 12;
    const d3 pp[4] = {mk(c[0], c[1], c[2]), mk(c[3], c[4], c[5]), mk(c[6], c[7], c[8]), mk(c[9], c[10], c[11])};
    write_panel_records(pp, cores[id], strengths[id], far_field_ratio, 0, &r32[id], r64 ? &r64[id] : nullptr);
}

cudaError_t launch_panels_from_corners(const double* corners, const double* strengths, const double* cores, long long P,
                                       double far_field_ratio, PanelRec<float>* r32, PanelRec<double>* r64,
                                       cudaStream_t s) {
    if (P <= 0) return cudaSuccess;
    k_panels_from_corners<<<static_cast<unsigned>((P + 127) / 128), 128, 0, s>>>(corners, strengths, cores, P,
                                                                                 far_field_ratio, r32, r64);
    return cudaGetLastError();
}

constexpr int kPanelThreads = 128;
constexpr int kChainThreads = 128;

cudaError_t launch_wake_panels(const DevModel& m, const WakeBuffers& w, int shift, cudaStream_t s) {
    const long long blocks = (m.P_pan + kPanelThreads - 1) / kPanelThreads;
    k_wake_panels<<<static_cast<unsigned>(blocks), kPanelThreads, 0, s>>>(m, w, shift);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// The same per-case kernels for every case of a batch, one launch per kind: block b belongs
// to the last job whose first block of that kind is at or before b (jobs [n] ascending in
// each kind's first block), and runs that job's element at b's offset within it.
// ---------------------------------------------------------------------------------------
template <long long CaseStepJob::*First>
__device__ inline int job_of_block(const CaseStepJob* jobs, int n, long long b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].*First <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_wake_advect_jobs(const CaseStepJob* jobs, int n) {
    const CaseStepJob& J = jobs[job_of_block<&CaseStepJob::blk_advect>(jobs, n, blockIdx.x)];
    const long long id = (blockIdx.x - J.blk_advect) * static_cast<long long>(kAdvectThreads) + threadIdx.x;
    wake_advect_elem(J.m, J.w, J.p.dt, J.steps_done, id);
}

__global__ void k_wake_panels_jobs(const CaseStepJob* jobs, int n) {
    const CaseStepJob& J = jobs[job_of_block<&CaseStepJob::blk_panels>(jobs, n, blockIdx.x)];
    const long long id = (blockIdx.x - J.blk_panels) * static_cast<long long>(kPanelThreads) + threadIdx.x;
    wake_panel_elem(J.m, J.w, 1, id);
}

__global__ void k_chain_records_jobs(const CaseStepJob* jobs, int n) {
    const CaseStepJob& J = jobs[job_of_block<&CaseStepJob::blk_chain>(jobs, n, blockIdx.x)];
    const long long id = (blockIdx.x - J.blk_chain) * static_cast<long long>(kChainThreads) + threadIdx.x;
    chain_record_elem(J.chain, J.chain_n, id);
}

long long wake_advect_blocks(const DevModel& m) {
    return (static_cast<long long>(m.W) * m.Np + kAdvectThreads - 1) / kAdvectThreads;
}
long long wake_panels_blocks(const DevModel& m) { return (m.P_pan + kPanelThreads - 1) / kPanelThreads; }
long long chain_records_blocks(long long n_build) { return (n_build + kChainThreads - 1) / kChainThreads; }

cudaError_t launch_wake_jobs(const CaseStepJob* jobs, int n, long long advect_blocks, long long panel_blocks,
                             cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (advect_blocks > 0) {
        k_wake_advect_jobs<<<static_cast<unsigned>(advect_blocks), kAdvectThreads, 0, s>>>(jobs, n);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (panel_blocks > 0) k_wake_panels_jobs<<<static_cast<unsigned>(panel_blocks), kPanelThreads, 0, s>>>(jobs, n);
    return cudaGetLastError();
}

cudaError_t launch_chain_records_jobs(const CaseStepJob* jobs, int n, long long blocks, cudaStream_t s) {
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    k_chain_records_jobs<<<static_cast<unsigned>(blocks), kChainThreads, 0, s>>>(jobs, n);
    return cudaGetLastError();
}

}  // namespace sbgpu
