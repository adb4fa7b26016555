// Simulation handle shared by the single-case C ABI (sim_host.cu) and the batched C ABI
// (batch_host.cu).
//
// Mirrors the reference's `Simulation` (stormbird/src/lifting_line/simulation.rs:20-217)
// and its builder (simulation_builder.rs:97-143): the JSON setup is decoded on the host,
// the wing discretisation (line_force_model/builder/single_wing.rs:73-150) is built once,
// and every per-step computation runs as CUDA kernels on the handle's stream. The host
// only enqueues work, copies the freestream in and the output block out (one copy each
// way per step), and keeps the step counters that select which kernels run.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/stormbird_gb300.h"
#include "sb_device.cuh"
#include "sb_kernels.h"
#include "sb_setup.hpp"
#include "sb_wind_setup.hpp"
#include "result_io.hpp"

namespace sbhost {

using namespace sbgpu;

struct SbFail {
    int code;
    std::string msg;
};

[[noreturn]] inline void raise(int code, const std::string& msg) { throw SbFail{code, msg}; }

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        // a failed call (e.g. cudaMalloc out of memory) also leaves its code in the runtime's
        // last-error slot, where the next launch check of any handle would find it: clear it
        // (a sticky error stays in the context regardless)
        cudaGetLastError();
        raise(SB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Runs f, turning a thrown SbFail into its status code and the thread's last error.
template <class F>
int guard(F&& f) {
    try {
        f();
        report_error(SB_OK, "");
        return SB_OK;
    } catch (const SbFail& e) {
        report_error(e.code, e.msg);
        return e.code;
    } catch (const std::exception& e) {
        report_error(SB_ERR_STATE, e.what());
        return SB_ERR_STATE;
    }
}

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { if (p) cudaFree(p); }
    void alloc(size_t count) {
        if (p) { cudaFree(p); p = nullptr; }
        n = count;
        if (count) ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    }
    void upload(const std::vector<T>& h) {
        alloc(h.size());
        if (!h.empty()) ck(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    }
};

// Device memory a caller passes in is read after the work the caller enqueued before the
// call on the legacy default stream (where PyTorch's default stream and the runtime's
// stream 0 both put their work): `s` waits on an event recorded there, without blocking the
// host. Without it a handle's own (non-blocking) stream could read an input that a kernel
// of the caller is still writing.
inline void order_after_caller(cudaStream_t s) {
    cudaEvent_t ev = nullptr;
    ck(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    cudaError_t e = cudaEventRecord(ev, cudaStreamLegacy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    cudaEventDestroy(ev);
    ck(e, "order after the caller's stream");
}

template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
    void alloc(size_t count) {
        if (p) { cudaFreeHost(p); p = nullptr; }
        n = count;
        if (count) ck(cudaMallocHost(&p, count * sizeof(T)), "cudaMallocHost");
    }
};

inline FoilP to_dev(const sbsetup::Foil& f) {
    FoilP o;
    o.stall_slope = 4.5951212 / f.stall_range;
    o.cl_zero_angle = f.cl_zero_angle;
    o.cl_initial_slope = f.cl_initial_slope;
    o.cl_high_order_factor_positive = f.cl_high_order_factor_positive;
    o.cl_high_order_factor_negative = f.cl_high_order_factor_negative;
    o.cl_high_order_power = f.cl_high_order_power;
    o.cl_max_after_stall = f.cl_max_after_stall;
    o.cd_min = f.cd_min;
    o.angle_cd_min = f.angle_cd_min;
    o.cd_second_order_factor = f.cd_second_order_factor;
    o.cd_max_after_stall = f.cd_max_after_stall;
    o.cd_power_after_stall = f.cd_power_after_stall;
    o.cdi_correction_factor = f.cdi_correction_factor;
    o.mean_positive_stall_angle = f.mean_positive_stall_angle;
    o.mean_negative_stall_angle = f.mean_negative_stall_angle;
    o.stall_range = f.stall_range;
    o.cd_bump_during_stall = f.cd_bump_during_stall;
    o.cd_stall_angle_offset = f.cd_stall_angle_offset;
    o.added_mass_factor = f.added_mass_factor;
    return o;
}

// Linear interpolation on a distance table (stormath/src/interpolation.rs:17-100).
inline d3 interp(double x, const std::vector<double>& xd, const std::vector<d3>& yd) {
    auto two = [](double t, double x0, double x1, d3 y0, d3 y1) {
        if (t <= x0) return y0;
        if (t >= x1) return y1;
        return y0 + (y1 - y0) * ((t - x0) / (x1 - x0));
    };
    size_t n = xd.size();
    if (n == 1) return yd[0];
    if (n == 2) return two(x, xd[0], xd[1], yd[0], yd[1]);
    size_t lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        size_t mid = (lo + hi) / 2;
        if (xd[mid] > x) hi = mid; else lo = mid;
    }
    if (lo == n - 1) return yd[lo];
    return two(x, xd[lo], xd[lo + 1], yd[lo], yd[lo + 1]);
}

// Copies n values into the staging buffer and returns the index of the first non-finite
// one (n when all are finite; the copy is then complete). Large inputs are split over
// host threads, each checking and copying its own contiguous part in one pass.
inline size_t copy_finite(const double* src, double* dst, size_t n) {
    auto part = [](const double* s, double* d, size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            if (!std::isfinite(s[i])) return i;
            d[i] = s[i];
        }
        return e;
    };
    constexpr size_t kSerial = size_t(1) << 20;
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::min<size_t>(hw ? hw : 1, 16);
    if (n < kSerial || T < 2) {
        const size_t r = part(src, dst, 0, n);
        return r;
    }
    std::vector<size_t> first(T, n);
    std::vector<std::thread> th;
    const size_t chunk = (n + T - 1) / T;
    for (size_t t = 0; t < T; ++t) {
        const size_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
        th.emplace_back([&, t, b, e] {
            const size_t r = part(src, dst, b, e);
            first[t] = r < e ? r : n;
        });
    }
    for (auto& x : th) x.join();
    size_t bad = n;
    for (size_t r : first) bad = std::min(bad, r);
    return bad;
}

inline int num_sms(int device) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    return v > 0 ? v : 1;
}


// Work decomposition of one sweep: target tiles x source chunks, with enough work items
// for ~16 waves of the persistent grid (sweep kernels in k_biot_savart.cu).
struct SweepPlan {
    int grid = 1, n_chunks = 1, chunk = 0;
    long long n_ttiles = 0;
};

inline SweepPlan make_sweep_plan(long long M, long long P, int precision, int sym, int neglect, int sms) {
    SweepPlan sp;
    int T = bs_targets_per_thread(sym);
    long long TM = static_cast<long long>(kBsThreads) * T;
    sp.n_ttiles = (M + TM - 1) / TM;
    int tile = bs_tile_panels(precision);
    int occ = bs_occupancy_blocks_per_sm(precision, sym, neglect);
    long long slots = static_cast<long long>(sms) * occ;
    // ~16 items per persistent CTA: a roll-up item (256 targets x a source chunk) runs for
    // milliseconds, and with 4 the last wave left SMs idle (4-wave plan 17.42 ms, 16 waves
    // 16.71 ms, 32 and 64 no better for the 4 x 64 panel, 300-row roll-up)
    long long want = 16 * slots;
    long long max_chunks = std::max<long long>(1, (P + tile - 1) / tile);
    long long nc = (want + sp.n_ttiles - 1) / std::max<long long>(1, sp.n_ttiles);
    nc = std::min(std::max<long long>(nc, 1), max_chunks);
    long long chunk = (P + nc - 1) / nc;
    chunk = ((chunk + tile - 1) / tile) * tile;
    sp.chunk = static_cast<int>(std::max<long long>(chunk, tile));
    sp.n_chunks = static_cast<int>((P + sp.chunk - 1) / sp.chunk);
    if (sp.n_chunks < 1) sp.n_chunks = 1;
    sp.grid = static_cast<int>(std::min<long long>(slots, sp.n_ttiles * sp.n_chunks));
    if (sp.grid < 1) sp.grid = 1;
    return sp;
}

// Device work space of one standalone call: stream-ordered allocations freed on exit.
struct StreamBufs {
    cudaStream_t s = nullptr;
    std::vector<void*> ptrs;
    explicit StreamBufs(cudaStream_t st) : s(st) {}
    ~StreamBufs() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        ck(cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), s), "cudaMallocAsync");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

inline void panel_sweep_impl(int device, const double* corners, const double* strengths, const double* core_lengths,
                      long long P, double far_field_ratio, int symmetry, const double* targets, long long M,
                      int precision, double* velocities) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    cudaStream_t st;
    ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    StreamBufs B(st);
    double* dc = B.get<double>(static_cast<size_t>(P) * 12);
    double* ds = B.get<double>(static_cast<size_t>(P));
    double* dr = B.get<double>(static_cast<size_t>(P));
    PanelRec<float>* r32 = B.get<PanelRec<float>>(static_cast<size_t>(P));
    PanelRec<double>* r64 = precision == 2 ? B.get<PanelRec<double>>(static_cast<size_t>(P)) : nullptr;
    d3* dt = B.get<d3>(static_cast<size_t>(M));
    d3* dout = B.get<d3>(static_cast<size_t>(M));
    unsigned long long* ctr = B.get<unsigned long long>(1);
    int* derr = B.get<int>(1);
    ck(cudaMemsetAsync(derr, 0, sizeof(int), st), "memset");
    if (P > 0) {
        ck(cudaMemcpyAsync(dc, corners, P * 12 * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
        ck(cudaMemcpyAsync(ds, strengths, P * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
        ck(cudaMemcpyAsync(dr, core_lengths, P * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
    }
    ck(cudaMemcpyAsync(dt, targets, M * sizeof(d3), cudaMemcpyHostToDevice, st), "H2D");
    ck(launch_panels_from_corners(dc, ds, dr, P, far_field_ratio, r32, r64, st), "panel records");
    if (P > 0) {
        SweepPlan sp = make_sweep_plan(M, P, precision, symmetry, 0, num_sms(device));
        double* partial = B.get<double>(static_cast<size_t>(sp.n_chunks) * static_cast<size_t>(M) * 3);
        BsArgs a;
        a.job0.panels = precision == 2 ? static_cast<const void*>(r64) : static_cast<const void*>(r32);
        a.job0.p_begin = 0;
        a.job0.p_end = P;
        a.job0.targets = dt;
        a.job0.M = M;
        a.job0.chunk_panels = sp.chunk;
        a.job0.n_chunks = sp.n_chunks;
        a.job0.n_ttiles = sp.n_ttiles;
        a.job0.partial = partial;
        a.work_counter = ctr;
        a.err = derr;
        a.symmetry = symmetry;
        ck(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st), "memset");
        ck(launch_bs_sweep(a, precision, sp.grid, st), "Biot-Savart sweep");
        ck(launch_bs_reduce(partial, sp.n_chunks, M, M, nullptr, dout, st), "sweep reduce");
    } else {
        ck(launch_bs_reduce(nullptr, 0, 0, M, nullptr, dout, st), "sweep reduce");
    }
    int herr = 0;
    ck(cudaMemcpyAsync(velocities, dout, M * sizeof(d3), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "panel sweep");
    if (herr == kDevTimeout) raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out");
}

}  // namespace sbhost

using namespace sbhost;

struct sb_sim {
    int device = 0;
    cudaStream_t stream = nullptr;
    sbsetup::Setup setup;
    bool dynamic = false;
    int solver_kind = 0;
    SolveSettings solve;
    DevModel dm;
    StepParams params;
    int N = 0, S = 0, Np = 0, W = 0;
    long long P_pan = 0, P_pts = 0, nfs = 0;
    int precision = 0;
    int sms = 1;
    bool first_step_completed = false;
    int steps_completed = 0;
    int fd_count = 0;
    OutLayout L{};
    std::vector<double> chord_lengths_h;
    bool timing = false;
    double last_ms[12] = {0};
    bool chains_built = false;  // the step built chain records (timing slot 11)
    double last_counters[7] = {0};
    int launches = 0;
    bool swept[2] = {false, false};

    // constants
    DevBuf<d3> span_s_local, span_e_local, chord_nr;
    DevBuf<double> chord_len, span_len_local, panel_core;
    DevBuf<int> wing_of_line, wing_start, wing_end, sp_line, sp_a, sp_b;
    DevBuf<unsigned char> is_virtual, sp_end;
    DevBuf<FoilP> foils;
    // geometry
    DevBuf<d3> chord_local, chord_global, chord_span_pts, span_s, span_e, span_pts, ctrl, felt_ctrl, felt_span, mean;
    DevBuf<d3> solve_basis;  // [2N] in-plane basis of each line (line_basis)
    // wake
    DevBuf<d3> pts[2], vel;
    DevBuf<double> str[2];
    DevBuf<PanelRec<float>> rec32;
    DevBuf<PanelRec<double>> rec64, row0_64;
    int cur = 0;
    // frozen wake and sweeps
    DevBuf<d3> fixed, factors, qs_wake_vec;
    DevBuf<float> factors_split;  // the SimpleIterative solver's matrix: hi plane, then lo plane
    DevBuf<double> qs_rc, partial;
    DevBuf<unsigned long long> counters;
    DevBuf<int> err;
    // solver, forces, io
    DevBuf<double> gamma_prev, gamma_tmp, scalars, lin_work, out;
    DevBuf<d3> vel_out, hist0, hist1, fs, aux_targets, aux_out;
    PinnedBuf<double> h_out, h_fs;
    PinnedBuf<int> h_err;
    cudaEvent_t ev[15] = {nullptr};
    // The handle's own stream; `stream` is the one its work is enqueued on, which a batch
    // points at one of its streams.
    cudaStream_t home_stream = nullptr;
    // Freestream [nfs] and previous circulation [N]: the handle's buffers, or slices of a
    // batch's contiguous buffers.
    d3* fs_p = nullptr;
    double* gamma_p = nullptr;
    // Predicted initial solutions [N] offered to the SimpleIterative solve, or nullptr.
    const double* candidate_p[2] = {nullptr, nullptr};
    // Shared-segment roll-up (chain records, launch_chain_records): possible when every pair
    // is near-field and all panels share one core length; on unless switched off.
    bool chain_ok = false, share_segments = true;
    DevBuf<PanelRec<float>> chains;
    DevBuf<int> chain_span_tab, chain_col_tab;
    // Freestream from a wind model (set_wind): device form, its tables, and the step's
    // time and ship velocity (device memory; a batch points `wind.step` at its own array).
    bool has_wind = false;
    WindDevice wind;
    DevBuf<double> wind_data, wind_step_own;
    DevBuf<int> wind_ints;
    DevBuf<long long> wind_ranges;
    PinnedBuf<double> h_wind_step;
    int chain_SP = 0;
    long long chain_Bq = 0, chain_Q = 0;
    double chain_rc = 0.0;

    ~sb_sim() {
        for (auto& e : ev) if (e) cudaEventDestroy(e);
        if (home_stream) cudaStreamDestroy(home_stream);
    }

    WakeBuffers wake(bool step) const {
        WakeBuffers w;
        w.pts_old = pts[cur].p;
        w.pts_new = step ? pts[cur ^ 1].p : pts[cur].p;
        w.vel = vel.p;
        w.str_old = str[cur].p;
        w.str_new = step ? str[cur ^ 1].p : str[cur].p;
        w.rec32 = rec32.p;
        w.rec64 = precision == 2 ? rec64.p : nullptr;
        w.row0_64 = row0_64.p;
        return w;
    }

    // ---------------------------------------------------------------- construction
    void build(const char* json, int dev) {
        device = dev;
        try {  // the setup is validated before any CUDA call
            setup = sbsetup::parse_setup(json);
        } catch (const sbsetup::SetupError& e) {
            std::string m = e.what();
            raise(m.find("not supported") != std::string::npos ? SB_ERR_UNSUPPORTED : SB_ERR_BAD_JSON, m);
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        sms = num_sms(device);
        dynamic = setup.dynamic;
        build_line_force_model();
        ck(cudaStreamCreateWithFlags(&home_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        stream = home_stream;
        for (auto& e : ev) ck(cudaEventCreate(&e), "cudaEventCreate");
        solver_settings();
        allocate();
        // global geometry at build time (data_update.rs:20-23)
        ck(launch_prep_geometry(dm, params, nullptr, nullptr, stream), "prep geometry");
        if (dynamic) build_wake();
        ck(cudaStreamSynchronize(stream), "build");
    }

    void build_line_force_model() {
        const auto& b = setup.line_force_model;
        std::vector<d3> ss, se, cn;
        std::vector<double> cl, sl;
        std::vector<int> wol, ws, we;
        std::vector<unsigned char> virt;
        std::vector<FoilP> fo;
        for (size_t w = 0; w < b.wing_builders.size(); ++w) {
            const auto& wb = b.wing_builders[w];
            std::vector<d3> sp, cv;
            for (auto& p : wb.section_points) sp.push_back(mk(p.x, p.y, p.z));
            for (auto& c : wb.chord_vectors) cv.push_back(mk(c.x, c.y, c.z));
            std::vector<double> dist;
            for (size_t i = 0; i < sp.size(); ++i) dist.push_back(i == 0 ? 0.0 : dist.back() + len(sp[i] - sp[i - 1]));
            int64_t nsec = wb.nr_sections >= 0 ? wb.nr_sections : b.nr_sections;
            if (nsec <= 0) raise(SB_ERR_BAD_JSON, "nr_sections must be positive");
            double ds_avg = dist.back() / static_cast<double>(nsec);
            ws.push_back(static_cast<int>(ss.size()));
            for (size_t sg = 0; sg + 1 < sp.size(); ++sg) {
                double sd = dist[sg + 1] - dist[sg];
                size_t nl = static_cast<size_t>(std::ceil(sd / ds_avg));
                double ds = sd / static_cast<double>(nl);
                for (size_t i = 0; i < nl; ++i) {
                    double a = dist[sg] + static_cast<double>(i) * ds;
                    double e = a + ds;
                    ss.push_back(interp(a, dist, sp));
                    se.push_back(interp(e, dist, sp));
                    d3 ch = interp(0.5 * (a + e), dist, cv);
                    cn.push_back(ch);
                    cl.push_back(len(ch));
                    sl.push_back(len(se.back() - ss.back()));
                    wol.push_back(static_cast<int>(w));
                    virt.push_back(wb.has_virtual && wb.line_segment_is_virtual[sg] ? 1 : 0);
                }
            }
            we.push_back(static_cast<int>(ss.size()));
            if (we.back() == ws.back()) raise(SB_ERR_BAD_JSON, "a wing has no span lines");
            fo.push_back(to_dev(wb.foil));
        }
        N = static_cast<int>(ss.size());
        S = static_cast<int>(ws.size());
        if (S > kMaxWings) raise(SB_ERR_UNSUPPORTED, "more than 64 wings");
        Np = N + S;
        chord_lengths_h = cl;
        // span points and control -> span value mapping (data_update.rs:41-55, value_mapping.rs:87-137)
        std::vector<int> spl, spa, spb;
        std::vector<unsigned char> spe;
        for (int w = 0; w < S; ++w) {
            spl.push_back(ws[w]); spe.push_back(0); spa.push_back(ws[w]); spb.push_back(ws[w]);
            for (int i = ws[w]; i < we[w]; ++i) {
                if (i == we[w] - 1) { spl.push_back(i); spe.push_back(1); spa.push_back(i); spb.push_back(i); }
                else { spl.push_back(i + 1); spe.push_back(0); spa.push_back(i); spb.push_back(i + 1); }
            }
        }
        span_s_local.upload(ss); span_e_local.upload(se); chord_nr.upload(cn);
        chord_len.upload(cl); span_len_local.upload(sl);
        wing_of_line.upload(wol); wing_start.upload(ws); wing_end.upload(we);
        wing_of_line_h = wol;
        wing_start_h = ws;
        is_virtual.upload(virt); foils.upload(fo);
        sp_line.upload(spl); sp_end.upload(spe); sp_a.upload(spa); sp_b.upload(spb);

        // step parameters from the builder (builder/mod.rs:97-108)
        for (int w = 0; w < S; ++w) params.local_wing_angles[w] = b.local_wing_angles.empty() ? 0.0 : b.local_wing_angles[w];
        params.translation = mk(b.translation.x, b.translation.y, b.translation.z);
        params.rotation = mk(b.rotation.x, b.rotation.y, b.rotation.z);

        dm.N = N; dm.S = S; dm.Np = Np;
        dm.density = b.density;
        double csum = 0.0;
        for (double c : cl) csum += c;
        dm.rep_chord = csum / static_cast<double>(N);
        dm.output_body = b.output_coordinate_system == sbsetup::CoordinateSystem::Body ? 1 : 0;
        dm.include_viscous_lift = b.include_viscous_lift_in_the_circulation ? 1 : 0;
        dm.span_s_local = span_s_local.p; dm.span_e_local = span_e_local.p; dm.chord_not_rotated = chord_nr.p;
        dm.chord_len = chord_len.p; dm.span_len_local = span_len_local.p; dm.wing_of_line = wing_of_line.p;
        dm.wing_start = wing_start.p; dm.wing_end = wing_end.p; dm.is_virtual = is_virtual.p; dm.foils = foils.p;
        dm.sp_line = sp_line.p; dm.sp_end = sp_end.p; dm.sp_val_a = sp_a.p; dm.sp_val_b = sp_b.p;
        if (dynamic) {
            const auto& w = setup.dynamic_wake;
            W = static_cast<int>(w.nr_panels_per_line_element);
            dm.W = W; dm.Wp = W + 1;
            P_pan = static_cast<long long>(W) * N;
            P_pts = static_cast<long long>(W + 1) * Np;
            dm.P_pan = P_pan; dm.P_pts = P_pts;
            dm.first_rel = w.first_panel_relative_length;
            dm.last_rel = w.last_panel_relative_length;
            dm.damping = w.shape_damping_factor;
            dm.far_field_ratio = w.far_field_ratio;
            dm.first_dir = static_cast<int>(w.first_wake_points_direction);
            dm.symmetry = static_cast<int>(w.symmetry_condition);
            dm.neglect_self = w.neglect_self_induced_velocities ? 1 : 0;
            dm.end_index = static_cast<long long>(std::ceil(w.ratio_of_wake_affected_by_induced_velocities * static_cast<double>(P_pts - 1)));
            if (dm.end_index < 0) dm.end_index = 0;
        }
        nfs = N + (dynamic ? P_pts : 0);
    }

    void solver_settings() {
        solver_kind = setup.solver.kind == sbsetup::SolverKind::SimpleIterative ? 0 : 1;
        const auto& si = setup.solver.si;
        const auto& li = setup.solver.lin;
        if (solver_kind == 0) {
            solve.max_iterations = static_cast<int>(si.max_iterations_per_time_step);
            solve.damping = si.damping_factor;
            solve.residual_tolerance = si.residual_tolerance_absolute;
            solve.strength_tolerance = si.strength_difference_tolerance;
            solve.velocity_correction = static_cast<int>(si.velocity_corrections.kind);
            solve.velocity_correction_ratio = si.velocity_corrections.ratio;
            solve.correction_factor_initial = si.correction_factor_initial_solution;
            solve.start_with_linearized = si.start_with_linearized_solution ? 1 : 0;
        } else {
            solve.velocity_correction = static_cast<int>(li.velocity_corrections.kind);
            solve.velocity_correction_ratio = li.velocity_corrections.ratio;
            solve.disable_viscous_corrections = li.disable_viscous_corrections ? 1 : 0;
            solve.full_induced_correction = li.full_induced_velocity_correction ? 1 : 0;
        }
    }

    void allocate() {
        chord_local.alloc(N); chord_global.alloc(N); chord_span_pts.alloc(Np); span_s.alloc(N); span_e.alloc(N);
        solve_basis.alloc(2 * static_cast<size_t>(N));
        dm.solve_basis = solve_basis.p;
        span_pts.alloc(Np); ctrl.alloc(N); felt_ctrl.alloc(N); felt_span.alloc(Np); mean.alloc(1);
        dm.chord_local = chord_local.p; dm.chord_global = chord_global.p; dm.chord_span_pts = chord_span_pts.p;
        dm.span_s = span_s.p; dm.span_e = span_e.p; dm.span_pts = span_pts.p; dm.ctrl = ctrl.p;
        dm.felt_ctrl = felt_ctrl.p; dm.felt_span = felt_span.p;
        fixed.alloc(N);
        // f64 matrix for the Linearized solve (also the start of a SimpleIterative one),
        // split matrix for the SimpleIterative iterations
        if (solver_kind == 1 || solve.start_with_linearized) factors.alloc(static_cast<size_t>(N) * N);
        if (solver_kind == 0) {  // two planes of N rows x 3 x stride; the padding columns stay 0
            factors_split.alloc(static_cast<size_t>(N) * si_matrix_stride(N) * 6);
            ck(cudaMemset(factors_split.p, 0, factors_split.n * sizeof(float)), "memset");
        }
        ck(cudaMemset(fixed.p, 0, N * sizeof(d3)), "memset");
        counters.alloc(4); err.alloc(4);
        ck(cudaMemset(err.p, 0, 4 * sizeof(int)), "memset");
        gamma_prev.alloc(N); gamma_tmp.alloc(N); scalars.alloc(8);
        ck(cudaMemset(gamma_prev.p, 0, N * sizeof(double)), "memset");
        gamma_p = gamma_prev.p;
        ck(cudaMemset(scalars.p, 0, 8 * sizeof(double)), "memset");
        if (solver_kind == 1 || solve.start_with_linearized) lin_work.alloc(static_cast<size_t>(N) * (N + 1));
        vel_out.alloc(N); hist0.alloc(N); hist1.alloc(N);
        ck(cudaMemset(hist0.p, 0, N * sizeof(d3)), "memset");
        ck(cudaMemset(hist1.p, 0, N * sizeof(d3)), "memset");
        L = OutLayout::make(N, S);
        out.alloc(L.total);
        ck(cudaMemset(out.p, 0, L.total * sizeof(double)), "memset");
        h_out.alloc(L.total);
        h_err.alloc(4);
        fs.alloc(nfs);
        fs_p = fs.p;
        h_fs.alloc(static_cast<size_t>(nfs) * 3);
        if (dynamic) {
            for (int b = 0; b < 2; ++b) { pts[b].alloc(P_pts); str[b].alloc(P_pan); }
            vel.alloc(P_pts);
            rec32.alloc(P_pan);
            row0_64.alloc(N);
        } else {
            qs_wake_vec.alloc(Np);
            qs_rc.alloc(1);
        }
    }

    // DynamicWakeBuilder::build (builder.rs:121-198): panel cores, then the chord-based
    // initialisation (initialization.rs:46-71).
    void build_wake() {
        std::vector<d3> hs(N), he(N), hc(Np);
        ck(cudaMemcpyAsync(hs.data(), span_s.p, N * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaMemcpyAsync(he.data(), span_e.p, N * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaMemcpyAsync(hc.data(), chord_span_pts.p, Np * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "build wake");
        const auto& w = setup.dynamic_wake;
        auto raw = [&](const sbsetup::CoreLength& c, double span_len) {
            switch (c.kind) {
                case sbsetup::CoreKind::Relative: return c.value * span_len;
                case sbsetup::CoreKind::Absolute: return c.value;
                case sbsetup::CoreKind::NoViscousCore: return kMinPositive;
            }
            return 0.0;
        };
        std::vector<double> core(static_cast<size_t>(P_pan));
        for (int s = 0; s < W; ++s) {
            for (int j = 0; j < N; ++j) {
                double sl = len(he[j] - hs[j]);
                double r = raw(w.viscous_core_length, sl);
                double v = r;
                if (w.core_sin_increase) {
                    double fin = raw(w.sin_last_panel_value, sl);
                    double before = static_cast<double>(W - 1) * w.sin_evolution_length_factor;
                    double rel = std::max(std::min(static_cast<double>(s) / before, 1.0), 0.0);
                    double sf = std::sin(0.5 * rel * kPi);
                    v = r * (1.0 - sf) + fin * sf;
                }
                core[static_cast<size_t>(s) * N + j] = v;
            }
        }
        panel_core.upload(core);
        panel_core_h = core;
        dm.panel_core = panel_core.p;
        setup_chains(core);
        d3 sum = mk(0, 0, 0);
        for (const auto& c : hc) sum = sum + c;
        d3 avg = sum / static_cast<double>(Np);
        double wl = w.initial_relative_wake_length * len(avg);
        d3 U = (wl / static_cast<double>(W)) * avg;
        ck(launch_wake_init(dm, wake(false), nullptr, U, 1.0, 1, stream), "wake init");
        ck(launch_wake_panels(dm, wake(false), 0, stream), "wake panels");
    }

    // Every pair is near-field when far_field_ratio >= 1e15: the near-field radius is then at
    // least 1e6 m for any panel longer than 1e-9 m (panel.rs:53-57), beyond any target
    // distance; shorter (degenerate) panels contribute nothing either way.
    static constexpr double kAllNearRatio = 1e15;

    void setup_chains(const std::vector<double>& core) {
        chain_ok = dm.far_field_ratio >= kAllNearRatio && !core.empty() &&
                   std::all_of(core.begin(), core.end(), [&](double c) { return c == core[0]; });
        if (!chain_ok) return;
        chain_rc = core[0];
        std::vector<int> st, ct;
        std::vector<int> ws(S), we(S);
        ck(cudaMemcpy(ws.data(), wing_start.p, S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
        ck(cudaMemcpy(we.data(), wing_end.p, S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
        for (int w = 0; w < S; ++w) {
            for (int j0 = ws[w]; j0 < we[w]; j0 += kChainSegs) {
                st.push_back(w);
                st.push_back(j0);
                st.push_back(std::min(kChainSegs, we[w] - j0));
            }
            for (int j = ws[w]; j <= we[w]; ++j) {  // point column j + w
                ct.push_back(w);
                ct.push_back(j);
            }
        }
        chain_SP = static_cast<int>(st.size() / 3);
        chain_span_tab.upload(st);
        chain_col_tab.upload(ct);
        chain_Bq = 4LL * chain_SP + Np;
        chain_Q = (W + 1 + 3) / 4;
        chains.alloc(static_cast<size_t>(chain_Q * chain_Bq));
    }

    bool use_chains() const { return chain_ok && share_segments && precision != 2; }

    // Panel rows that can hold a nonzero strength (see active_panels); row_extra covers the
    // rows of a loaded state (set_state) that lie beyond what its age could have filled.
    int row_extra = 0;
    int active_rows() const { return std::min<long long>(W, static_cast<long long>(steps_completed) + 2 + row_extra); }

    // Chain records covering the active rows: the quads up to the one holding point row R
    // (its spanwise segments carry -strength of row R - 1).
    long long active_chain_records() const {
        return std::min<long long>(chain_Q, active_rows() / 4 + 1) * chain_Bq;
    }

    // Chain records from wake buffer `buf` (after the step's begin: the current one).
    ChainArgs chain_args(int buf) const {
        ChainArgs c;
        c.pts = pts[buf].p;
        c.str = str[buf].p;
        c.span_tab = chain_span_tab.p;
        c.col_tab = chain_col_tab.p;
        c.wing_start = wing_start.p;
        c.wing_end = wing_end.p;
        c.W = W;
        c.N = N;
        c.Np = Np;
        c.SP = chain_SP;
        c.Bq = chain_Bq;
        c.rc = chain_rc;
        c.out = chains.p;
        return c;
    }

    void build_chains() {
        // all records, also the empty ones past the active rows: a captured step replays
        // this launch with its arguments unchanged while the wake grows
        record(13);
        ck(launch_chain_records(chain_args(cur), chain_Q * chain_Bq, stream), "chain records");
        record(14);
        chains_built = true;
        launches += 1;
    }

    // ---------------------------------------------------------------- one step
    void ensure_rec64() {
        if (precision == 2 && dynamic && rec64.n != static_cast<size_t>(P_pan)) {
            rec64.alloc(P_pan);
            // records for the current wake
            ck(launch_wake_panels(dm, wake(false), 0, stream), "wake panels");
        }
    }

    SweepPlan plan_sweep(long long M, long long P, int sym, int neglect) {
        return make_sweep_plan(M, P, precision, sym, neglect, sms);
    }

    // One Biot-Savart sweep of a step: targets [0, M) against panels [p0, p1), written to
    // dst with `base` added; dst rows [M, M_total) get `base` only.
    struct SweepDesc {
        const d3* targets;
        long long M, p0, p1;
        const int* twing;
        const d3* base;
        long long M_total;
        d3* dst;
        const void* src = nullptr;  // chain records, or nullptr for the panel records
        bool chain = false;
        double segments = 0.0;      // segment evaluations per target
        bool wake_targets = false;  // the targets are the wake points (rows of Np points)
    };

    // Target order of a sweep over the wake points (BsJob::slots): wing by wing, rows within a
    // wing, so that the far-field fast path sees compact warp boxes. Other sweeps, and one wing
    // (whose natural order is that already), keep the index order.
    void target_layout(const SweepDesc& d, BsJob& J) const {
        J.slots = d.M;
        J.row_pts = 0;
        J.n_groups = 0;
        if (!d.wake_targets || d.chain || S < 2 || S > kMaxTargetGroups || d.M <= 0) return;
        J.slots = (d.M + Np - 1) / Np * static_cast<long long>(Np);
        J.row_pts = Np;
        J.n_groups = S;
        for (int w = 0; w < S; ++w) J.group_off[w] = wing_start_h[w] + w;  // a wing's first point
        J.group_off[S] = Np;
    }

    // Biot-Savart sweep into out[0..M) (+ base), base only for [M, M_total).
    void sweep(const SweepDesc& d, int counter_slot) {
        const d3* targets = d.targets;
        const long long M = d.M, p0 = d.p0, p1 = d.p1, M_total = d.M_total;
        const int* twing = d.twing;
        const d3* base = d.base;
        d3* dst = d.dst;
        int sym = dm.symmetry;
        int neglect = twing ? 1 : 0;
        long long P = p1 - p0;
        if (M > 0 && P > 0) {
            BsArgs a;
            target_layout(d, a.job0);
            SweepPlan sp = plan_sweep(bs_slots(a.job0), P, sym, neglect);
            size_t need = static_cast<size_t>(sp.n_chunks) * static_cast<size_t>(M) * 3;
            if (partial.n < need) partial.alloc(need);
            a.job0.panels = d.src ? d.src : precision == 2 ? static_cast<const void*>(rec64.p) : static_cast<const void*>(rec32.p);
            a.chain = d.chain ? 1 : 0;
            a.job0.p_begin = p0;
            a.job0.p_end = p1;
            a.job0.targets = targets;
            a.job0.target_wing = twing;
            a.job0.M = M;
            a.job0.chunk_panels = sp.chunk;
            a.job0.n_chunks = sp.n_chunks;
            a.job0.n_ttiles = sp.n_ttiles;
            a.job0.partial = partial.p;
            a.work_counter = counters.p + counter_slot;
            a.err = err.p;
            a.symmetry = sym;
            a.neglect = neglect;
            ck(cudaMemsetAsync(a.work_counter, 0, sizeof(unsigned long long), stream), "memset counter");
            if (timing && counter_slot < 2) ck(cudaEventRecord(ev[8 + 2 * counter_slot], stream), "event");
            ck(launch_bs_sweep(a, precision, sp.grid, stream), "Biot-Savart sweep");
            if (timing && counter_slot < 2) ck(cudaEventRecord(ev[9 + 2 * counter_slot], stream), "event");
            ck(launch_bs_reduce(partial.p, sp.n_chunks, M, M_total, base, dst, stream), "sweep reduce");
            launches += 2;
            if (counter_slot < 2) swept[counter_slot] = true;
        } else {
            ck(launch_bs_reduce(nullptr, 0, 0, M_total, base, dst, stream), "sweep reduce");
            launches += 1;
        }
    }

    void record(int i) { if (timing) ck(cudaEventRecord(ev[i], stream), "event"); }

    // Simulation::do_step (simulation.rs:107-203) with the freestream already in fs_p: the
    // geometry and the wake before solving, the frozen wake, the solve, the wake roll-up
    // and the forces. A batch runs the same phases for all of its cases, with the two
    // sweeps of every case in one launch each.
    void enqueue_step(double time, double dt) {
        step_begin(time, dt);
        if (dynamic) {
            sweep(fixed_desc(), 0);
            after_fixed_sweep();
        }
        step_matrix_and_solve();
        if (dynamic) {
            sweep(rollup_desc(), 1);
            after_rollup_sweep();
        }
        step_end();
    }

    // Panels that can hold a nonzero strength in this step's sweeps. Strength rows move one
    // row downstream per step and row 0 takes the new solution (update_data.rs:146-150,
    // 319-328), from all-zero rows at initialisation: with k steps completed, rows 0..k
    // (rows 1..k before the solve) are the only nonzero ones. Panels beyond contribute
    // nothing (zero strengths are skipped, induced_velocity_calc.rs:203), so the sweeps
    // stop there (one row of margin).
    long long active_panels() const { return std::min<long long>(P_pan, static_cast<long long>(active_rows()) * N); }

    // frozen wake (frozen_wake.rs:189-261): the free wake at the control points
    SweepDesc fixed_desc() const {
        const long long p1 = std::max<long long>(N, active_panels());
        return {ctrl.p, N, N, p1, dm.neglect_self ? wing_of_line.p : nullptr, nullptr, N, fixed.p, nullptr, false,
                4.0 * static_cast<double>(p1 - N)};
    }

    // DynamicWake::update_after_solving (update_data.rs:49-59, 125-141)
    bool rollup_active() const { return dm.end_index > 0 && steps_completed > 2; }
    SweepDesc rollup_desc() const {
        const d3* wake_fs = fs_p + N;
        if (!rollup_active()) return {nullptr, 0, 0, 0, nullptr, wake_fs, P_pts, vel.p};
        long long e = std::min<long long>(dm.end_index, P_pts);
        if (use_chains()) {
            // segments of rows < R: spanwise on point rows 0..R, streamwise on panel rows 0..R-1
            const double R = static_cast<double>(active_rows());
            return {pts[cur].p, e, 0, active_chain_records(), nullptr, wake_fs, P_pts, vel.p, chains.p, true,
                    (R + 1.0) * N + R * Np};
        }
        return {pts[cur].p, e, 0, active_panels(), nullptr, wake_fs, P_pts, vel.p, nullptr, false,
                4.0 * static_cast<double>(active_panels()), true};
    }

    void after_fixed_sweep() {
        last_counters[2] = static_cast<double>(N);
        last_counters[3] = static_cast<double>(P_pan - N);
        record(3);
    }

    void after_rollup_sweep() {
        SweepDesc d = rollup_desc();
        last_counters[0] = static_cast<double>(d.M);
        last_counters[1] = static_cast<double>(d.chain ? active_panels() : d.p1 - d.p0);
        last_counters[6] = d.M > 0 ? d.segments : 0.0;
        steps_completed += 1;
        last_counters[4] = static_cast<double>(steps_completed);
        record(6);
    }

    // Geometry, first-step initialisation and the wake before solving.
    void step_begin(double time, double dt) {
        params.time = time;
        params.dt = dt;
        ensure_rec64();
        record(0);
        const bool first = !first_step_completed;
        launches = 0;
        swept[0] = swept[1] = false;
        chains_built = false;
        ck(launch_prep_geometry(dm, params, fs_p, first ? mean.p : nullptr, stream), "prep geometry");
        launches += 1;
        if (first) {
            // Simulation::initialize (simulation.rs:65-94)
            if (dynamic) {
                ck(launch_wake_init(dm, wake(false), mean.p, mk(0, 0, 0), dt, 0, stream), "wake init");
                ck(launch_wake_panels(dm, wake(false), 0, stream), "wake panels");
                launches += 2;
            }
            ck(cudaMemcpyAsync(hist0.p, fs_p, N * sizeof(d3), cudaMemcpyDeviceToDevice, stream), "fd init");
            ck(cudaMemcpyAsync(hist1.p, fs_p, N * sizeof(d3), cudaMemcpyDeviceToDevice, stream), "fd init");
            fd_count = 0;
            ck(cudaMemsetAsync(gamma_p, 0, N * sizeof(double), stream), "memset");
            first_step_completed = true;
        }
        record(1);
        if (dynamic) {
            ck(launch_wake_advect(dm, wake(true), dt, steps_completed, stream), "wake advect");
            record(12);
            ck(launch_wake_panels(dm, wake(true), 1, stream), "wake panels");
            launches += 3;
            cur ^= 1;
        }
        record(2);
    }

    // ---- a step whose per-case kernels a batch launches for all its cases at once
    // A dynamic case past its first step: its geometry, wake update, unit-strength matrix and
    // chain records come from the batch's job-list launches (CaseStepJob).
    bool batch_kernels_ok() const { return dynamic && first_step_completed; }

    // The case's job for a step, from the state before the step.
    CaseStepJob step_job(double time, double dt) const {
        CaseStepJob j;
        j.m = dm;
        j.p = params;
        j.p.time = time;
        j.p.dt = dt;
        j.w = wake(true);
        j.fs_ctrl = fs_p;
        j.steps_done = steps_completed;
        j.row0_32 = precision == 2 ? nullptr : rec32.p;
        j.factors = factors.p;
        j.split = factors_split.p;
        j.basis = split_basis();
        if (use_chains() && rollup_active()) {
            j.chain = chain_args(cur ^ 1);  // the buffer the step writes
            j.chain_n = chain_Q * chain_Bq;
        }
        return j;
    }

    // step_begin's host side for such a case (its kernels come from the batch).
    void step_begin_host(double time, double dt) {
        params.time = time;
        params.dt = dt;
        launches = 0;
        swept[0] = swept[1] = false;
        cur ^= 1;
    }

    // Influence matrix (unit matrix of the first wake row, or horseshoes) and the solve.
    // The frozen wake's matrix: unit first-row panels (dynamic) or horseshoes (quasi-steady).
    // In-plane bases for a two-component SimpleIterative matrix (no velocity correction: the
    // solve uses the velocity's in-plane part only), else nullptr (three components).
    const d3* split_basis() const { return solve.velocity_correction == 0 ? dm.solve_basis : nullptr; }

    void step_matrix() {
        if (dynamic) {
            // FP32 records unless the sweeps run in FP64
            ck(launch_unit_matrix(row0_64.p, precision == 2 ? nullptr : rec32.p, ctrl.p, N, dm.symmetry, dm.neglect_self,
                                  wing_of_line.p, factors.p,
                                  factors_split.p, split_basis(), stream),
               "unit matrix");
            launches += 1;
        } else {
            const auto& q = setup.quasi_steady_wake;
            double wl = q.wake_length_factor * dm.rep_chord;
            ck(launch_horseshoe_matrix(dm, static_cast<int>(q.viscous_core_length.kind), q.viscous_core_length.value, wl,
                                       qs_wake_vec.p, qs_rc.p, static_cast<int>(q.symmetry_condition), factors.p,
                                       factors_split.p, split_basis(), stream),
               "horseshoe matrix");
            launches += 2;
            record(3);
        }
        record(4);
    }

    SolveBuffers solve_buffers() const {
        SolveBuffers sb;
        sb.fixed = fixed.p;
        sb.factors = factors.p;
        sb.factors_split = factors_split.p;
        // off-diagonal lo parts are zero when the unit matrix came from the FP32 records
        sb.split_full = (dynamic && precision != 2) ? 0 : 1;
        sb.basis = split_basis();
        sb.split_comps = sb.basis ? 2 : 3;
        sb.gamma_prev = gamma_p;
        sb.vel_out = vel_out.p;
        sb.scalars = scalars.p;
        sb.lin_work = lin_work.p;
        sb.err = err.p;
        sb.candidate[0] = candidate_p[0];
        sb.candidate[1] = candidate_p[1];
        if (dynamic) {
            sb.wake_str_row0 = str[cur].p;
            sb.rec32_row0 = rec32.p;
            sb.rec64_row0 = precision == 2 ? rec64.p : nullptr;
        }
        return sb;
    }

    // A quasi-steady case with the Linearized solver: its solve depends on nothing that
    // changes between steps (device pointers and settings), so a batch solves all such
    // cases in one launch of k_solve_lin_jobs.
    bool linearized_quasi_steady() const { return !dynamic && solver_kind == 1; }
    SolveJob linearized_job() const {
        SolveJob j;
        j.m = dm;
        j.st = solve;
        j.b = solve_buffers();
        return j;
    }

    void step_solve() {
        const SolveBuffers sb = solve_buffers();
        if (solver_kind == 0) {
            SolveSettings st = solve;
            if (solve.start_with_linearized) {
                SolveBuffers lb = sb;
                lb.gamma_prev = gamma_tmp.p;
                lb.wake_str_row0 = nullptr;
                lb.rec32_row0 = nullptr;
                lb.rec64_row0 = nullptr;
                SolveSettings ls;  // Linearized::default()
                ck(launch_solve_linearized(dm, ls, lb, stream), "linearized start");
                launches += 1;
                ck(cudaMemcpyAsync(gamma_p, gamma_tmp.p, N * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
                st.correction_factor_initial = 1.0;
            }
            ck(launch_solve_simple_iterative(dm, st, sb, stream), "simple iterative solve");
        } else {
            ck(launch_solve_linearized(dm, solve, sb, stream), "linearized solve");
        }
        launches += 1;
    }

    void step_after_solve() {
        // chain records of the wake with this step's solution in row 0, for the roll-up
        if (dynamic && use_chains() && rollup_active()) build_chains();
        record(5);
        if (!dynamic) record(6);
    }

    void step_matrix_and_solve() {
        step_matrix();
        step_solve();
        step_after_solve();
    }

    // Forces and the output block (force_calculations.rs:669-698).
    ForceJob force_job() const {
        ForceJob j;
        j.m = dm;
        j.p = params;
        j.f.gamma = gamma_p;
        j.f.vel = vel_out.p;
        j.f.hist0 = hist0.p;
        j.f.hist1 = hist1.p;
        j.f.fd_count = fd_count;
        j.f.out = out.p;
        j.f.scalars = scalars.p;
        return j;
    }

    void step_end() {
        const ForceJob j = force_job();
        ck(launch_forces(j.m, j.p, j.f, stream), "forces");
        after_forces();
    }

    // what follows the forces launch, also when a batch launches them for all its cases
    void after_forces() {
        launches += 1;
        last_counters[5] = static_cast<double>(launches);
        fd_count += 1;
        record(7);
    }

    void finish_step() {
        ck(cudaMemcpyAsync(h_out.p, out.p, L.total * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H output");
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H status");
        ck(cudaStreamSynchronize(stream), "step");
        collect_timing();
        check_device_status();
        if (writer) writer->push(result_record());
        if (dynamic && setup.dynamic_wake.write_wake_data_to_file) push_wake_file();
    }

    // Phase and kernel times of the step just synchronised (sb_sim_enable_timing).
    void collect_timing() {
        if (timing) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[0], ev[7]); last_ms[0] = ms;
            cudaEventElapsedTime(&ms, ev[1], ev[2]); last_ms[1] = ms;
            cudaEventElapsedTime(&ms, ev[2], ev[3]); last_ms[2] = ms;
            cudaEventElapsedTime(&ms, ev[3], ev[4]); last_ms[3] = ms;
            cudaEventElapsedTime(&ms, ev[4], ev[5]); last_ms[4] = ms;
            cudaEventElapsedTime(&ms, ev[5], ev[6]); last_ms[5] = ms;
            cudaEventElapsedTime(&ms, ev[6], ev[7]); last_ms[6] = ms;
            last_ms[7] = last_ms[8] = last_ms[9] = last_ms[10] = last_ms[11] = 0.0;
            if (swept[1]) { cudaEventElapsedTime(&ms, ev[10], ev[11]); last_ms[7] = ms; }
            if (swept[0]) { cudaEventElapsedTime(&ms, ev[8], ev[9]); last_ms[8] = ms; }
            if (dynamic) {
                cudaEventElapsedTime(&ms, ev[1], ev[12]); last_ms[9] = ms;
                cudaEventElapsedTime(&ms, ev[12], ev[2]); last_ms[10] = ms;
            }
            if (chains_built) { cudaEventElapsedTime(&ms, ev[13], ev[14]); last_ms[11] = ms; }
        }
    }

    // The wake after the step as a VTK file `{wake_files_folder_path}/wake_{time / dt}.vtp`
    // (Simulation::do_step, simulation.rs:183-185; export.rs:11-23, 75-163), written on a
    // background thread.
    std::unique_ptr<sbhost::WakeFileWriter> wake_writer;
    std::vector<int> wing_of_line_h;
    std::vector<int> wing_start_h;  // first line of each wing
    std::vector<double> panel_core_h;

    void push_wake_file() {
        if (!wake_writer) wake_writer.reset(new sbhost::WakeFileWriter());
        sbhost::WakeRecord w;
        const double q = params.dt != 0.0 ? params.time / params.dt : 0.0;
        const unsigned long long index = q > 0.0 ? static_cast<unsigned long long>(q) : 0ull;  // `as usize`
        w.path = setup.dynamic_wake.wake_files_folder_path + "/wake_" + std::to_string(index) + ".vtp";
        w.N = N;
        w.Np = Np;
        w.W = W;
        w.wing_of_line = wing_of_line_h;
        w.pts.resize(static_cast<size_t>(P_pts) * 3);
        w.str.resize(static_cast<size_t>(P_pan));
        ck(cudaMemcpyAsync(w.pts.data(), pts[cur].p, P_pts * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H wake points");
        ck(cudaMemcpyAsync(w.str.data(), str[cur].p, P_pan * sizeof(double), cudaMemcpyDeviceToHost, stream),
           "D2H wake strengths");
        ck(cudaStreamSynchronize(stream), "wake file");
        w.core = panel_core_h;
        wake_writer->push(std::move(w));
    }

    // ---------------------------------------------------------------- result output
    std::unique_ptr<sbhost::ResultWriter> writer;
    mutable std::vector<std::pair<int, int>> wing_ranges_h;  // line range of each wing (filled once)

    // The last step's SimulationResult from the host copy of the output block.
    sbhost::ResultRecord result_record() const {
        if (wing_ranges_h.empty()) {
            std::vector<int> ws(S), we(S);
            ck(cudaMemcpy(ws.data(), wing_start.p, S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
            ck(cudaMemcpy(we.data(), wing_end.p, S * sizeof(int), cudaMemcpyDeviceToHost), "D2H");
            for (int w = 0; w < S; ++w) wing_ranges_h.emplace_back(ws[w], we[w]);
        }
        sbhost::ResultRecord r;
        r.time = params.time;
        r.N = N;
        r.S = S;
        r.body = dm.output_body != 0;
        r.motion = params;
        r.wings = wing_ranges_h;
        r.out.assign(h_out.p, h_out.p + L.total);
        return r;
    }

    void set_result_file(const char* path, int format) {
        writer.reset();
        if (!path || format == sbhost::kResultsOff) return;
        try {
            writer.reset(new sbhost::ResultWriter(path, format));
        } catch (const std::exception& e) {
            raise(SB_ERR_STATE, e.what());
        }
    }

    void check_device_status() {
        int e = h_err.p[0];
        if (e != kDevOk) {
            ck(cudaMemsetAsync(err.p, 0, sizeof(int), stream), "memset");
            if (e == kDevTimeout) raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out");
            if (e == kDevSingular) raise(SB_ERR_STATE, "Matrix is singular or nearly singular");
            raise(SB_ERR_CUDA, "device error word " + std::to_string(e));
        }
    }

    void write_output(sb_step_output* o) const {
        const double* h = h_out.p;
        auto cp = [](double* dst, const double* src, size_t n) { if (dst) std::memcpy(dst, src, n * sizeof(double)); };
        cp(o->circulation_strength, h + L.gamma, N);
        cp(o->ctrl_points_velocity, h + L.vel, 3 * N);
        cp(o->solver_input_velocity, h + L.felt, 3 * N);
        cp(o->angles_of_attack, h + L.aoa, N);
        cp(o->force_input_velocity, h + L.fvel, 3 * N);
        cp(o->acceleration, h + L.acc, 3 * N);
        cp(o->ctrl_points, h + L.ctrl, 3 * N);
        cp(o->sectional_forces, h + L.sect, 18 * N);
        cp(o->integrated_forces, h + L.intf, 18 * S);
        cp(o->integrated_moments, h + L.intm, 18 * S);
        for (int k = 0; k < 3; ++k) {
            o->force_sum[k] = h[L.fsum + k];
            o->moment_sum[k] = h[L.msum + k];
        }
        o->residual = h[L.residual];
        o->iterations = static_cast<int64_t>(h[L.iterations]);
        o->converged = h[L.converged] != 0.0 ? 1 : 0;
        o->reserved = 0;
    }

    void do_step(double time, double dt, const double* fs_host, size_t n, sb_step_output* o) {
        if (static_cast<long long>(n) != nfs) raise(SB_ERR_SIZE, "freestream has " + std::to_string(n) + " points, expected " + std::to_string(nfs));
        const size_t cnt = n * 3;
        const size_t bad = copy_finite(fs_host, h_fs.p, cnt);
        if (bad < cnt) raise(SB_ERR_NONFINITE, "non-finite freestream value at index " + std::to_string(bad / 3));
        ck(cudaMemcpyAsync(fs_p, h_fs.p, cnt * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D freestream");
        enqueue_step(time, dt);
        finish_step();
        if (o) write_output(o);
    }

    void do_step_device(double time, double dt, const double* fs_dev, size_t n) {
        if (static_cast<long long>(n) != nfs) raise(SB_ERR_SIZE, "freestream length mismatch");
        order_after_caller(stream);
        ck(cudaMemcpyAsync(fs_p, fs_dev, n * sizeof(d3), cudaMemcpyDeviceToDevice, stream), "D2D freestream");
        enqueue_step(time, dt);
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H status");
        ck(cudaStreamSynchronize(stream), "step");
        collect_timing();
        check_device_status();
    }

    void read_output(sb_step_output* o) {
        ck(cudaMemcpyAsync(h_out.p, out.p, L.total * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H output");
        ck(cudaStreamSynchronize(stream), "read output");
        write_output(o);
    }

    // ---------------------------------------------------------------- state between steps
    // What a step reads from the steps before it, as the public fields of the reference's
    // Simulation (simulation.rs:20-28) and DynamicWake (wake/dynamic_wake/mod.rs:41-64) hold
    // it: [0] wake steps completed, [1] first step completed (0/1), [2] flow-derivative
    // updates, then (dynamic) wake points [P_pts][3], velocity at the points [P_pts][3],
    // panel strengths [P_pan], then the previous circulation [N] and the flow-derivative
    // history (two earlier control-point velocities) [2][N][3]. Rigid-body motion and wing
    // angles are not part of it (their setters set them).
    static constexpr size_t kStateHead = 3;
    size_t state_size() const {
        const size_t wake = dynamic ? static_cast<size_t>(P_pts) * 6 + static_cast<size_t>(P_pan) : 0;
        return kStateHead + wake + static_cast<size_t>(N) * 7;
    }

    void get_state(double* o, size_t n) {
        if (n != state_size()) raise(SB_ERR_SIZE, "state buffer has " + std::to_string(n) + " values, expected " +
                                                      std::to_string(state_size()));
        o[0] = dynamic ? static_cast<double>(steps_completed) : 0.0;
        o[1] = first_step_completed ? 1.0 : 0.0;
        o[2] = static_cast<double>(fd_count);
        double* p = o + kStateHead;
        auto d2h = [&](const void* src, size_t count) {
            ck(cudaMemcpyAsync(p, src, count * sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H state");
            p += count;
        };
        if (dynamic) {
            d2h(pts[cur].p, static_cast<size_t>(P_pts) * 3);
            d2h(vel.p, static_cast<size_t>(P_pts) * 3);
            d2h(str[cur].p, static_cast<size_t>(P_pan));
        }
        d2h(gamma_p, static_cast<size_t>(N));
        d2h(hist0.p, static_cast<size_t>(N) * 3);
        d2h(hist1.p, static_cast<size_t>(N) * 3);
        ck(cudaStreamSynchronize(stream), "get state");
    }

    void set_state(const double* s, size_t n) {
        if (n != state_size()) raise(SB_ERR_SIZE, "state buffer has " + std::to_string(n) + " values, expected " +
                                                      std::to_string(state_size()));
        for (size_t i = 0; i < n; ++i)
            if (!std::isfinite(s[i])) raise(SB_ERR_NONFINITE, "non-finite state value at index " + std::to_string(i));
        if (s[0] < 0.0 || s[0] > 2e9 || s[2] < 0.0 || s[2] > 2e9) raise(SB_ERR_SIZE, "step counters out of range");
        const double* p = s + kStateHead;
        auto h2d = [&](void* dst, size_t count) {
            ck(cudaMemcpyAsync(dst, p, count * sizeof(double), cudaMemcpyHostToDevice, stream), "H2D state");
            p += count;
        };
        row_extra = 0;
        if (dynamic) {
            h2d(pts[cur].p, static_cast<size_t>(P_pts) * 3);
            h2d(vel.p, static_cast<size_t>(P_pts) * 3);
            const double* g = p;
            h2d(str[cur].p, static_cast<size_t>(P_pan));
            // sweeps stop after the rows a wake of this age can have filled (active_rows);
            // a loaded wake may hold strengths further downstream
            long long last = -1;
            for (long long i = P_pan - 1; i >= 0; --i)
                if (g[i] != 0.0) { last = i / N; break; }
            steps_completed = static_cast<int>(s[0]);
            row_extra = static_cast<int>(std::max<long long>(0, last - steps_completed - 1));
        }
        h2d(gamma_p, static_cast<size_t>(N));
        h2d(hist0.p, static_cast<size_t>(N) * 3);
        h2d(hist1.p, static_cast<size_t>(N) * 3);
        first_step_completed = s[1] != 0.0;
        fd_count = static_cast<int>(s[2]);
        // panel records of the loaded wake (sb_sim_induced_velocities may come before a step)
        if (dynamic) ck(launch_wake_panels(dm, wake(false), 0, stream), "wake panels");
        ck(cudaStreamSynchronize(stream), "set state");
    }

    // ---------------------------------------------------------------- wind model
    void set_wind(const char* env_json, const char* cond_json) {
        sbsetup::WindEnvironment env;
        sbsetup::WindCondition cond;
        try {
            env = sbsetup::parse_wind_environment(env_json);
            cond = sbsetup::parse_wind_condition(cond_json);
        } catch (const sbsetup::SetupError& e) {
            raise(SB_ERR_BAD_JSON, e.what());
        }
        WindDevice w;
        auto d3of = [](const sbsetup::Vec3& v) { return mk(v.x, v.y, v.z); };
        w.up = d3of(env.up_direction);
        w.axis = d3of(env.wind_rotation_axis);
        w.zero = d3of(env.zero_direction_vector);
        w.water_plane_height = env.water_plane_height;
        w.direction_coming_from = cond.direction_coming_from;
        const auto& v = cond.velocity_variation;
        w.vv_kind = static_cast<int>(v.kind);
        w.vv_constant = v.constant;
        w.reference_velocity = v.reference_velocity;
        w.reference_height = v.reference_height;
        w.power_factor = v.power_factor;
        w.friction_velocity = v.friction_velocity;
        w.surface_roughness = v.surface_roughness;
        w.has_obukhov = v.has_obukhov_length ? 1 : 0;
        w.obukhov_length = v.obukhov_length;
        w.von_karman = v.von_karman_constant;
        w.stable_coefficient = v.stable_coefficient;
        w.unstable_coefficient = v.unstable_coefficient;
        std::vector<double> data;
        const sbsetup::Spectrum* gusts[3] = {&cond.parallel_gust, &cond.perpendicular_gust, &cond.vertical_gust};
        for (int k = 0; k < 3; ++k) {
            if (!gusts[k]->present) continue;
            w.spec_off[k] = static_cast<int>(data.size());
            w.spec_n[k] = static_cast<int>(gusts[k]->frequencies.size());
            data.insert(data.end(), gusts[k]->frequencies.begin(), gusts[k]->frequencies.end());
            data.insert(data.end(), gusts[k]->amplitudes.begin(), gusts[k]->amplitudes.end());
            data.insert(data.end(), gusts[k]->phases.begin(), gusts[k]->phases.end());
        }
        std::vector<int> ints;
        std::vector<long long> ranges;
        const auto& ic = env.inflow_corrections;
        size_t dirs_off = data.size(), corr_base = 0;
        if (ic.present) {
            // the reference indexes each direction's wing ranges by wing (inflow_corrections.rs:28)
            for (const auto& c : ic.corrections)
                if (c.wing_indices.size() < static_cast<size_t>(S))
                    raise(SB_ERR_SIZE, "inflow corrections need one height range per wing");
            w.n_dirs = static_cast<int>(ic.apparent_wind_directions.size());
            w.S = S;
            data.insert(data.end(), ic.apparent_wind_directions.begin(), ic.apparent_wind_directions.end());
            corr_base = data.size();
            std::vector<int> offs, lens;
            for (const auto& c : ic.corrections) {
                offs.push_back(static_cast<int>(data.size() - corr_base));
                lens.push_back(static_cast<int>(c.height_values.size()));
                data.insert(data.end(), c.height_values.begin(), c.height_values.end());
                data.insert(data.end(), c.magnitude_corrections.begin(), c.magnitude_corrections.end());
                data.insert(data.end(), c.angle_corrections.begin(), c.angle_corrections.end());
                for (int wg = 0; wg < S; ++wg) {
                    ranges.push_back(c.wing_indices[wg].first);
                    ranges.push_back(c.wing_indices[wg].second);
                }
            }
            ints = offs;
            ints.insert(ints.end(), lens.begin(), lens.end());
        }
        wind_data.upload(data.empty() ? std::vector<double>{0.0} : data);
        wind_ints.upload(ints.empty() ? std::vector<int>{0} : ints);
        wind_ranges.upload(ranges.empty() ? std::vector<long long>{0} : ranges);
        w.spectra = wind_data.p;
        if (ic.present) {
            w.dirs = wind_data.p + dirs_off;
            w.corr = wind_data.p + corr_base;
            w.corr_off = wind_ints.p;
            w.corr_len = wind_ints.p + w.n_dirs;
            w.ranges = wind_ranges.p;
        }
        if (wind_step_own.n == 0) {
            wind_step_own.alloc(2);
            h_wind_step.alloc(2);
        }
        w.step = has_wind && wind.step ? wind.step : wind_step_own.p;
        wind = w;
        has_wind = true;
    }

    void set_wind_step(double time, double ship_velocity) {
        h_wind_step.p[0] = time;
        h_wind_step.p[1] = ship_velocity;
        ck(cudaMemcpyAsync(wind_step_own.p, h_wind_step.p, 2 * sizeof(double), cudaMemcpyHostToDevice, stream),
           "H2D wind step");
    }

    // CompleteSailModel::freestream_velocity (complete_sail_model/mod.rs:213-257) into fs_p at
    // the current freestream points (control points of the current geometry, wake points).
    void enqueue_wind_freestream() {
        ck(launch_prep_geometry(dm, params, nullptr, nullptr, stream), "prep geometry");
        ck(launch_wind_freestream(wind, ctrl.p, wing_of_line.p, N, dynamic ? pts[cur].p : nullptr, dynamic ? P_pts : 0,
                                  fs_p, stream),
           "wind freestream");
        launches += 2;
    }

    void do_step_wind(double time, double dt, double ship_velocity, sb_step_output* o) {
        if (!has_wind) raise(SB_ERR_STATE, "no wind model: call sb_sim_set_wind first");
        set_wind_step(time, ship_velocity);
        enqueue_wind_freestream();
        enqueue_step(time, dt);
        finish_step();
        if (o) write_output(o);
    }

    void wind_freestream(double time, double ship_velocity, double* outp, size_t n) {
        if (!has_wind) raise(SB_ERR_STATE, "no wind model: call sb_sim_set_wind first");
        if (static_cast<long long>(n) != nfs) raise(SB_ERR_SIZE, "freestream buffer length mismatch");
        set_wind_step(time, ship_velocity);
        enqueue_wind_freestream();
        ck(cudaMemcpyAsync(outp, fs_p, n * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H freestream");
        ck(cudaStreamSynchronize(stream), "wind freestream");
    }

    void freestream_points(double* outp, size_t n) {
        if (static_cast<long long>(n) != nfs) raise(SB_ERR_SIZE, "points buffer length mismatch");
        ck(launch_prep_geometry(dm, params, nullptr, nullptr, stream), "prep geometry");
        ck(cudaMemcpyAsync(outp, ctrl.p, N * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H");
        if (dynamic) ck(cudaMemcpyAsync(outp + 3 * N, pts[cur].p, P_pts * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "freestream points");
    }

    void induced_velocities(const double* p, size_t n, double* o) {
        if (!dynamic) raise(SB_ERR_STATE, "Induced velocities not implemented for pure quasi-steady simulations yet");
        if (n == 0) return;
        ensure_rec64();
        if (aux_targets.n < n) { aux_targets.alloc(n); aux_out.alloc(n); }
        ck(cudaMemcpyAsync(aux_targets.p, p, n * sizeof(d3), cudaMemcpyHostToDevice, stream), "H2D points");
        sweep({aux_targets.p, static_cast<long long>(n), 0, P_pan, nullptr, nullptr, static_cast<long long>(n), aux_out.p},
              2);
        ck(cudaMemcpyAsync(o, aux_out.p, n * sizeof(d3), cudaMemcpyDeviceToHost, stream), "D2H velocities");
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H status");
        ck(cudaStreamSynchronize(stream), "induced velocities");
        check_device_status();
    }
};
