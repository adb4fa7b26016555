// Circulation solvers and force output (sm_103a), f64.
//
// k_solve_si: the damped fixed-point solve SimpleIterative::solve
// (stormbird/src/lifting_line/solvers/simple_iterative.rs:86-212) for one case on one
// thread-block cluster. Every CTA of the cluster keeps the full circulation vector in
// shared memory; CTA r owns a contiguous block of control points. Per iteration:
//   1. induced velocity of its rows: fixed + M * Gamma (frozen_wake.rs:268-301), one warp
//      per row, matrix rows read from L2 as (hi, lo) float pairs and the products summed
//      in double-float arithmetic on the FP32 pipes (~2^-44 relative per product; this
//      part's FP64 rate is 1/64 of its FP32 rate);
//   2. per row, in f64: total velocity (velocity_corrections.rs:28-100), span component
//      removed (line_force_model/mod.rs:235-254), angle of attack
//      (force_calculations.rs:79-107), Foil lift, circulation estimate
//      (force_calculations.rs:271-292), residual term (force_calculations.rs:552-627) and
//      the damped update; the thread's own f64 circulation stays in registers;
//   3. new Gamma (as a float pair) and residual terms are stored into every CTA's shared
//      memory through distributed shared memory, the per-CTA max |dGamma| likewise, one
//      cluster barrier;
//   4. every CTA sums the residual terms with one warp in a fixed order (the same value,
//      hence the same stopping decision, in every CTA) and takes the max.
// All waits are hardware cluster barriers; no spin loops.
//
// k_solve_lin / k_solve_lin_jobs: Linearized::solve (solvers/linearized.rs:54-222) with
// the Gaussian elimination with partial pivoting of stormath/src/matrix/linalg.rs:41-103,
// one CTA per case: one case, or all linearized quasi-steady cases of a batch in one
// launch.
//
// k_forces: SimulationResult of one step (force_calculations.rs:322-452, 669-698;
// common_utils/forces_and_moments.rs:163-245; flow_derivatives.rs:31-63).
#include <cooperative_groups.h>

#include <map>
#include <mutex>
#include <tuple>

#include "sb_device.cuh"
#include "sb_kernels.h"
#include "sb_ptx.cuh"

namespace cg = cooperative_groups;

namespace sbgpu {

constexpr int kSolveThreads = 256;
constexpr int kSolveRowsPerThread = 4;  // most rows per thread (1024 per CTA)
constexpr int kMaxCluster = 8;

__host__ __device__ inline int si_cluster_size(int N) {
    if (N <= 64) return 1;
    if (N <= 256) return 4;
    return 8;
}
int solve_cluster_size(int N) { return si_cluster_size(N); }

// Matrix slab of a CTA (its rows of the split matrix) in shared memory. Bytes of one row:
// 2 or 3 components (SolveBuffers::split_comps) x stride floats, twice with the lo plane. When all of the CTA's rows fit
// kSlabBudget they are copied once per solve and stay; else chunks of 4 to 8 rows (a row per
// warp) stream through two buffers of half the budget each, every iteration. 0: not even 4
// rows fit a buffer (N above about 900): the warps read their rows from global memory.
constexpr long long kSlabBudget = 88 * 1024;
__host__ __device__ inline long long si_row_bytes(int N, int full, int comps) {
    return 4LL * comps * si_matrix_stride(N) * (full ? 2 : 1);
}
// Shared memory before the slab, in doubles: circulation pairs 2 x stride, residual terms
// 2 x N, maxima 2 x kMaxCluster, the CTA's M * Gamma pairs (3 doubles per row), the own
// panels' lo parts (2 doubles per row), the own rows' in-plane bases (6 doubles per row),
// rounded to 16 bytes.
__host__ __device__ inline long long si_slab_offset(int N) {
    const int CS = si_cluster_size(N);
    const long long rp = (N + CS - 1) / CS;
    const long long d = 2LL * si_matrix_stride(N) + 2LL * N + 2 * kMaxCluster + 3 * rp + 2 * rp + 6 * rp;
    return (d + 1) & ~1LL;
}
__host__ __device__ inline int si_slab_rows(int N, int full, int comps) {
    const int CS = si_cluster_size(N);
    const int rp = (N + CS - 1) / CS;
    const long long rowb = si_row_bytes(N, full, comps);
    // two CTAs of a cluster per SM: at most ~110 KB of shared memory each
    const long long rest = 110 * 1024 - si_slab_offset(N) * 8;
    const long long budget = rest < kSlabBudget ? rest : kSlabBudget;
    if (rp * rowb <= budget) return rp;
    const long long r = budget / (2 * rowb);
    return r < 4 ? 0 : (r > 8 ? 8 : static_cast<int>(r));
}

struct RowGeom {
    d3 felt, span_dir, chord, span_rel_out;  // span_dir = normalize(span end - span start)
    double chord_len, area;
    double chord_norm;  // |chord vector|
    double cl_gamma;    // 2 |span_rel| / area (0 if the area or density is 0): see residual_of_row
    int wing;
};

__device__ inline RowGeom row_geom(const DevModel& m, int i) {
    RowGeom g;
    g.felt = m.felt_ctrl[i];
    const d3 span_rel = m.span_e[i] - m.span_s[i];
    g.span_dir = normalize(span_rel);
    g.chord = m.chord_global[i];
    g.span_rel_out = m.output_body ? (m.span_e_local[i] - m.span_s_local[i]) : span_rel;
    g.chord_len = m.chord_len[i];
    g.area = m.chord_len[i] * m.span_len_local[i];
    g.chord_norm = len(g.chord);
    g.cl_gamma = (g.area == 0.0 || m.density == 0.0) ? 0.0 : 2.0 * len(span_rel) / g.area;
    g.wing = m.wing_of_line[i];
    return g;
}

// signed_angle_between(chord, u, span_dir) (vector_math.rs:65-95) with |chord| and |u| known:
// cos = chord.u / (|chord| |u|) instead of / sqrt(|chord|^2 |u|^2) (the same to an ulp)
__device__ inline double row_angle(const RowGeom& g, d3 u, double ul) {
    const double triple = dot(g.chord, cross(u, g.span_dir));
    double ang = 0.0;
    if (!(g.chord_norm == 0.0 || ul == 0.0)) {
        double c = dot(g.chord, u) / (g.chord_norm * ul);
        c = fmin(fmax(c, -1.0), 1.0);
        ang = acos(c);
    }
    return triple > 0.0 ? ang : -ang;
}

// velocity_corrections.rs:28-100 (returns freestream + induced, corrected)
__device__ inline d3 total_velocity(const SolveSettings& st, d3 fs, d3 ind) {
    if (st.velocity_correction == 1) {
        double im = len(ind), fm = len(fs);
        double mx = st.velocity_correction_ratio * fm;
        d3 c = im > mx ? normalize(ind) * mx : ind;
        return fs + c;
    }
    if (st.velocity_correction == 2) return normalize(fs + ind) * len(fs);
    return fs + ind;
}

__device__ inline double circulation_cl(const DevModel& m, const FoilP& f, double aoa) {
    double cl = foil_cl_pre_stall(f, aoa);
    if (m.include_viscous_lift) cl += foil_cl_post_stall(f, aoa);
    return cl;
}

// |cl_gamma - cl_direct| of force_calculations.rs:552-607, given cl_direct = the foil's
// pre-stall lift coefficient at the line's angle of attack
__device__ inline double residual_from_cl(const DevModel& m, const RowGeom& g, double gam, d3 u, double cl_pre) {
    double ul = len(u);
    d3 force = ul == 0.0 ? mk(0, 0, 0) : (gam * cross(u, g.span_rel_out)) * m.density;
    double sign = -1.0 * signum(gam);
    double ff = 0.5 * g.area * m.density * len2(u);
    double clg = ff == 0.0 ? 0.0 : len(force) * sign / ff;
    return fabs(clg - cl_pre);
}
__device__ inline double residual_term(const DevModel& m, const RowGeom& g, const FoilP& f, double gam, d3 u, double aoa) {
    return residual_from_cl(m, g, gam, u, foil_cl_pre_stall(f, aoa));
}
// The same in the iterations, with |u| known. In the global output frame the line's span
// vector is span_rel, to which u was made perpendicular (the projection before the angle),
// so |u x span_rel| = |u| |span_rel| and the lift coefficient of the force is
// -gam |u| |span_rel| rho / (area rho |u|^2 / 2) = -gam cl_gamma / |u|: one division for
// the cross product, two square roots and the quotient of residual_from_cl. (Body-frame
// output keeps that function: there the span vector is the body frame's.)
__device__ inline double residual_of_row(const DevModel& m, const RowGeom& g, double gam, d3 u, double ul, double cl_pre) {
    if (m.output_body) return residual_from_cl(m, g, gam, u, cl_pre);
    const double clg = ul == 0.0 ? 0.0 : -gam * g.cl_gamma / ul;
    return fabs(clg - cl_pre);
}

// Double-float accumulation for the matrix-vector product: (S, C) += (xh + xl) * (gh + gl).
// The product's head xh*gh is added to S by an error-free two-sum (Knuth); its rounding error
// (an exact FMA) and the cross terms xh*gl + xl*gh go into C; xl*gl (~2^-48 of the product)
// is dropped. The _rn intrinsics keep the compiler from fusing the steps.
__device__ __forceinline__ void ff_mac(float& S, float& C, float2 x, float2 g) {
    const float p = __fmul_rn(x.x, g.x);
    float t = fmaf(x.x, g.x, -p);
    t = fmaf(x.x, g.y, t);
    t = fmaf(x.y, g.x, t);
    const float s = __fadd_rn(S, p);
    const float bv = __fsub_rn(s, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bv)), __fsub_rn(p, bv));
    S = s;
    C = __fadd_rn(C, __fadd_rn(err, t));
}
// Four consecutive columns into one component's double-float sum (S, C): matrix entries
// (a + al) (al = 0 without lo parts) against the circulation pairs (g01.x + g01.y),
// (g01.z + g01.w), (g23.x + g23.y), (g23.z + g23.w), each by ff_mac (two-sum: exact for any
// magnitudes; a Kahan-compensated sum, two operations cheaper, is exact only while the
// running sum outweighs the new term and left the solve a residual floor near 1e-11).
__device__ __forceinline__ void ff_mac4(float& S, float& C, float4 a, float4 al, float4 g01, float4 g23) {
    ff_mac(S, C, make_float2(a.x, al.x), make_float2(g01.x, g01.y));
    ff_mac(S, C, make_float2(a.y, al.y), make_float2(g01.z, g01.w));
    ff_mac(S, C, make_float2(a.z, al.z), make_float2(g23.x, g23.y));
    ff_mac(S, C, make_float2(a.w, al.w), make_float2(g23.z, g23.w));
}

// One lane's share of a row of the split matrix times the circulation: columns 4*lane + 128*t,
// NC components (planes of S floats), hi plane fh and (full) lo plane fl.
template <int NC>
__device__ __forceinline__ void row_dot_lane(const float* fh, const float* fl, const float2* Gc, float (&acc)[6], int S,
                                             int lane, int full) {
#pragma unroll 2
    for (int k = 4 * lane; k < S; k += 128) {
        const float4 g01 = *reinterpret_cast<const float4*>(Gc + k);  // (hi, lo) of columns k, k + 1
        const float4 g23 = *reinterpret_cast<const float4*>(Gc + k + 2);
#pragma unroll
        for (int q = 0; q < NC; ++q) {
            const float4 a = *reinterpret_cast<const float4*>(fh + q * S + k);
            const float4 al = full ? *reinterpret_cast<const float4*>(fl + q * S + k) : make_float4(0.f, 0.f, 0.f, 0.f);
            ff_mac4(acc[2 * q], acc[2 * q + 1], a, al, g01, g23);
        }
    }
}
// (S, C) += (h, l), another double-float partial sum
__device__ __forceinline__ void ff_add(float& S, float& C, float h, float l) {
    const float s = __fadd_rn(S, h);
    const float bv = __fsub_rn(s, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bv)), __fsub_rn(h, bv));
    S = s;
    C = __fadd_rn(C, __fadd_rn(err, l));
}

// Sum / max over a warp in a fixed order (lane 0 gets the result): every CTA of a cluster
// reduces the same residual terms the same way and takes the same stopping decision.
__device__ __forceinline__ double warp_sum_to_lane0(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
// Maxima of magnitudes on the integer pipe (this part's FP64 pipe costs a full warp
// instruction per compare): |v| as its IEEE bit pattern, which orders like an unsigned
// integer for non-negative values; a NaN maps to 0, as fmax(x, NaN) = x leaves it out.
__device__ __forceinline__ unsigned long long mag_bits(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7FFFFFFFFFFFFFFFull;
    return b > 0x7FF0000000000000ull ? 0ull : b;
}
__device__ __forceinline__ double bits_value(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }
__device__ __forceinline__ unsigned long long warp_umax_to_lane0(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// SimpleIterative::solve for one case on the calling thread-block cluster (see the top of
// the file). Run by k_solve_si (one case) and k_solve_si_jobs (a cluster per case of a batch).
// RPT = rows per thread: 1 while a CTA owns at most kSolveThreads rows (registers for two
// CTAs per SM), else kSolveRowsPerThread.
template <int RPT>
__device__ void si_solve(const DevModel& m, const SolveSettings& st, const SolveBuffers& b) {
    cg::cluster_group cl = cg::this_cluster();
    const int CS = static_cast<int>(cl.num_blocks());
    const int rank = static_cast<int>(cl.block_rank());
    const int N = m.N;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = kSolveThreads / 32;
    extern __shared__ __align__(16) double smem[];
    // circulation of every line as (hi, lo) float pairs for the matrix-vector products, padded
    // with zeros to the matrix's row stride; the f64 circulation of the thread's own rows
    // stays in registers (gown)
    const int S = si_matrix_stride(N);
    float2* G[2] = {reinterpret_cast<float2*>(smem), reinterpret_cast<float2*>(smem + S)};
    double* RR[2] = {smem + 2 * S, smem + 2 * S + N};
    double* MX[2] = {smem + 2 * S + 2 * N, smem + 2 * S + 2 * N + kMaxCluster};
    const int rp = (N + CS - 1) / CS;
    const int r0 = min(N, rank * rp), r1 = min(N, r0 + rp);
    // The thread's k-th own row (offset from r0): consecutive rows on consecutive threads, so
    // that a CTA owning fewer than 256 rows fills as few warps as possible (this part's FP64
    // pipe costs the same per warp instruction however few lanes are active).
    auto own_row = [&](int k) { return tid + k * kSolveThreads; };
    // M * Gamma of the CTA's rows as double-float pairs (x hi, x lo, y hi, y lo, z hi, z lo);
    // the row's owner adds them to the fixed part in f64
    float* uff = reinterpret_cast<float*>(smem + 2 * S + 2 * N + 2 * kMaxCluster);
    const int rp_max = (N + CS - 1) / CS;
    // lo parts of the own panels' entries (x, y, z), when the matrix has none elsewhere
    float* diag_lo = reinterpret_cast<float*>(smem + 2 * S + 2 * N + 2 * kMaxCluster + 3 * rp_max);
    d3* basis_sm = reinterpret_cast<d3*>(smem + 2 * S + 2 * N + 2 * kMaxCluster + 5 * rp_max);  // e1, e2 per own row
    float* slab = reinterpret_cast<float*>(smem + si_slab_offset(N));
    __shared__ double s_res;
    __shared__ unsigned long long s_umax[kSolveThreads / 32];
    __shared__ int s_conv;
    __shared__ __align__(8) uint64_t s_mbar[2];

    const bool scale0 = fabs(st.correction_factor_initial - 1.0) > kMinPositive;
    for (int i = tid; i < N; i += kSolveThreads) {
        double g = b.gamma_prev[i];
        if (scale0) g *= st.correction_factor_initial;
        G[0][i] = split_f64(g);
    }
    for (int i = N + tid; i < S; i += kSolveThreads) G[0][i] = G[1][i] = make_float2(0.f, 0.f);
    // per-thread rows
    RowGeom rg[RPT];
    d3 u_last[RPT];
    double aoa_last[RPT], gown[RPT];
    int nrows = 0;
    for (int k = 0; k < RPT; ++k) {
        int i = r0 + own_row(k);
        if (i < r1) {
            double g = b.gamma_prev[i];
            if (scale0) g *= st.correction_factor_initial;
            gown[k] = g;
            rg[k] = row_geom(m, i);
            u_last[k] = mk(0, 0, 0);
            aoa_last[k] = 0.0;
            nrows = k + 1;
        }
    }
    __syncthreads();

    const int full = b.split_full;
    const int C = b.split_comps;  // 2: in-plane components in the rows' bases, 3: x, y, z
    const int slab_rows = si_slab_rows(N, full, C);
    const int nrows_cta = r1 - r0;
    const int nch = slab_rows > 0 ? (nrows_cta + slab_rows - 1) / slab_rows : 0;
    const bool resident = slab_rows > 0 && slab_rows >= rp_max;  // copied once, kept
    const long long rowf = static_cast<long long>(C) * S;         // floats of a row, one plane
    const long long buf_floats = static_cast<long long>(slab_rows) * rowf * (full ? 2 : 1);
    const long long lo_plane = static_cast<long long>(C) * N * S;
    if (tid == 0) {
        mbar_init(&s_mbar[0], 1);
        mbar_init(&s_mbar[1], 1);
        fence_mbar_init();
    }
    for (int k = tid; k < nrows_cta; k += kSolveThreads) {
        const long long row = r0 + k;
        if (!full) {
            const float* fl = b.factors_split + lo_plane + row * rowf;
            for (int q = 0; q < C; ++q) diag_lo[3 * k + q] = fl[q * S + row];
        }
        if (C == 2) {
            basis_sm[2 * k] = b.basis[2 * row];
            basis_sm[2 * k + 1] = b.basis[2 * row + 1];
        }
    }

    // residual of the initial solution with zero velocity (simple_iterative.rs:180-184)
    double residual = 0.0;
    if (st.max_iterations == 0) {
        if (tid == 0) {
            double s = 0.0;
            for (int i = 0; i < N; ++i) s += fabs(0.0 - foil_cl_pre_stall(m.foils[m.wing_of_line[i]], 0.0));
            s_res = s / static_cast<double>(N);
        }
        __syncthreads();
        residual = s_res;
    }
    cl.sync();

    // induced velocity of own rows for the circulation Gc: fixed + M * Gc. One warp per row;
    // double-float arithmetic on the FP32 pipes (this part's FP64 rate is 1/64 of its FP32
    // rate), a lane taking four consecutive columns per 16-byte shared-memory load. The
    // CTA's matrix rows come from its slab in shared memory: thread 0 copies them by bulk
    // asynchronous copies (cp.async.bulk, completion on an mbarrier; bounded waits), kept for
    // the whole solve when they fit, else streamed in chunks through two buffers (the copy
    // of chunk c + 1 runs while the warps work on chunk c).
    // A slab wait that runs out records kDevTimeout (the host raises SB_ERR_TIMEOUT after the
    // launch); that thread then waits no more and thread 0 issues no more copies, and the
    // solve runs its remaining (bounded) iterations on whatever the buffers hold, through the
    // same barriers as the other CTAs of the cluster, so that none waits for it forever.
    uint32_t mph[2] = {0u, 0u};
    bool pending[2] = {false, false};  // thread 0: a copy into the buffer not yet waited for
    bool slab_loaded = false, dead = false;
    auto issue = [&](int c, int bufi) {  // thread 0
        const long long row0 = r0 + static_cast<long long>(c) * slab_rows;
        const int nr = min(slab_rows, r1 - static_cast<int>(row0));
        const uint32_t bytes = static_cast<uint32_t>(nr * rowf * 4);
        float* dst = slab + bufi * buf_floats;
        mbar_expect_tx(&s_mbar[bufi], full ? 2 * bytes : bytes);
        bulk_g2s(dst, b.factors_split + row0 * rowf, bytes, &s_mbar[bufi]);
        if (full) bulk_g2s(dst + slab_rows * rowf, b.factors_split + lo_plane + row0 * rowf, bytes, &s_mbar[bufi]);
        pending[bufi] = true;
    };
    // (S, C) += row . Gc over the lane's columns, from fh (hi) and fl (lo, full only)
    auto row_dot = [&](const float* fh, const float* fl, const float2* Gc, float (&acc)[6]) {
        if (C == 2) row_dot_lane<2>(fh, fl, Gc, acc, S, lane, full);
        else row_dot_lane<3>(fh, fl, Gc, acc, S, lane, full);
    };
    auto finish_row = [&](int row, float (&acc)[6], const float2* Gc) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 3; ++q)
                if (q < C)
                    ff_add(acc[2 * q], acc[2 * q + 1], __shfl_down_sync(0xffffffffu, acc[2 * q], o),
                           __shfl_down_sync(0xffffffffu, acc[2 * q + 1], o));
        if (lane == 0) {
            if (!full) {  // the own panel's entry is f64: its lo parts times Gamma hi
                const float2 g = Gc[row];
                const float* dl = diag_lo + 3 * (row - r0);
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    if (q < C) ff_mac(acc[2 * q], acc[2 * q + 1], make_float2(0.f, dl[q]), g);
            }
            float* o = uff + 6 * (row - r0);
#pragma unroll
            for (int q = 0; q < 6; ++q) o[q] = acc[q];
        }
    };
    auto induced_rows = [&](const float2* Gc) {
        if (slab_rows == 0) {  // rows from global memory
            for (int row = r0 + warp; row < r1; row += nwarps) {
                const float* fh = b.factors_split + static_cast<long long>(row) * rowf;
                float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                row_dot(fh, fh + lo_plane, Gc, acc);
                finish_row(row, acc, Gc);
            }
            __syncthreads();
            return;
        }
        const bool copy = !(resident && slab_loaded);
        if (copy && tid == 0 && !dead) {
            issue(0, 0);
            if (nch > 1) issue(1, 1);
        }
        for (int c = 0; c < nch; ++c) {
            const int bufi = c & 1;
            if (copy) {
                if (!dead) {
                    if (mbar_wait_bounded(&s_mbar[bufi], mph[bufi], b.err)) pending[bufi] = false;
                    else dead = true;
                }
                mph[bufi] ^= 1u;
            }
            const int row0 = r0 + c * slab_rows;
            const int nr = min(slab_rows, r1 - row0);
            const float* base = slab + bufi * buf_floats;
            for (int w = warp; w < nr; w += nwarps) {
                float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                row_dot(base + w * rowf, base + (slab_rows + w) * rowf, Gc, acc);
                finish_row(row0 + w, acc, Gc);
            }
            __syncthreads();  // every warp is done with this buffer
            if (copy && !resident && tid == 0 && !dead && c + 2 < nch) issue(c + 2, bufi);
        }
        slab_loaded = true;
    };
    // Velocity of own row i with its span component taken out (project(u, span_rel) before
    // the angle): freestream + fixed + M * Gamma. With two components the products are already
    // the in-plane coordinates along the row's basis (e1, e2), and the velocity correction is
    // off (the only mode the two-component matrix is built for).
    auto row_velocity = [&](int i, const RowGeom& g) {
        const float* o = uff + 6 * (i - r0);
        const d3 fx = b.fixed[i];
        if (C == 2) {
            const d3 e1 = basis_sm[2 * (i - r0)], e2 = basis_sm[2 * (i - r0) + 1];
            const d3 base = g.felt + fx;
            const double a = dot(base, e1) + (static_cast<double>(o[0]) + static_cast<double>(o[1]));
            const double c = dot(base, e2) + (static_cast<double>(o[2]) + static_cast<double>(o[3]));
            return e1 * a + e2 * c;
        }
        const d3 ind = mk(fx.x + (static_cast<double>(o[0]) + static_cast<double>(o[1])),
                          fx.y + (static_cast<double>(o[2]) + static_cast<double>(o[3])),
                          fx.z + (static_cast<double>(o[4]) + static_cast<double>(o[5])));
        const d3 u = total_velocity(st, g.felt, ind);
        return u - g.span_dir * dot(u, g.span_dir);
    };

    // Guarded warm start: residual (simple_iterative.rs:160-176) of the plain start G[0]
    // and of each candidate (staged in G[1]). A candidate replaces the current start only
    // when both its mean residual (the solver's own measure) and its largest per-line term
    // are lower: the solver stops on the mean, which a start with its error on a few lines
    // could pass while those lines are still off. The plain start wins ties. The second
    // candidate (the network's) must beat the best start so far by b.second_margin (0.5 by
    // default) on both measures: its per-line error is noise-like, and a start that is only slightly
    // better by the initial residual took more iterations than the extrapolation (566 of
    // 2,560 solves of the uneven-case batch: 108 iterations against 107 from the plain start).
    if (b.candidate[0] || b.candidate[1]) {
        double best = 0.0, best_max = 0.0;
        int taken = 0;
        for (int v = 0; v < 3; ++v) {
            const double* src = v == 0 ? nullptr : b.candidate[v - 1];
            if (v > 0 && !src) continue;
            float2* Gv = v == 0 ? G[0] : G[1];
            if (v > 0) {
                for (int i = tid; i < N; i += kSolveThreads) G[1][i] = split_f64(src[i]);
                __syncthreads();
            }
            induced_rows(Gv);
            for (int k = 0; k < nrows; ++k) {
                int i = r0 + own_row(k);
                const RowGeom& g = rg[k];
                const FoilP f = m.foils[g.wing];
                const d3 u = row_velocity(i, g);
                double aoa = len(u) > kMinPositive ? signed_angle_between(g.chord, u, g.span_dir) : 0.0;
                double r = residual_term(m, g, f, v == 0 ? gown[k] : src[i], u, aoa);
                for (int q = 0; q < CS; ++q) cl.map_shared_rank(RR[0], q)[i] = r;
            }
            cl.sync();
            if (warp == 0) {
                double s = 0.0;
                unsigned long long mx = 0;
                for (int i = lane; i < N; i += 32) {
                    s += RR[0][i];
                    const unsigned long long bi = mag_bits(RR[0][i]);
                    mx = bi > mx ? bi : mx;
                }
                s = warp_sum_to_lane0(s);
                mx = warp_umax_to_lane0(mx);
                if (lane == 0) {
                    s_res = s;
                    s_umax[0] = mx;
                }
            }
            __syncthreads();
            const double rv = s_res, rmax = bits_value(s_umax[0]);
            if (v == 0) {
                best = rv;
                best_max = rmax;
            } else if (isfinite(rv) && rv < (v == 2 ? b.second_margin : 1.0) * best &&
                       rmax < (v == 2 ? b.second_margin : 1.0) * best_max) {  // same decision in every CTA
                best = rv;
                best_max = rmax;
                taken = v;
                for (int i = tid; i < N; i += kSolveThreads) G[0][i] = G[1][i];
                for (int k = 0; k < nrows; ++k) gown[k] = src[r0 + own_row(k)];
            }
            cl.sync();  // RR[0] and G[1] are written again by the next pass or the first iteration
        }
        if (rank == 0 && tid == 0) b.scalars[4] = static_cast<double>(taken);
    } else if (rank == 0 && tid == 0) {
        b.scalars[4] = -1.0;
    }

    int it = 0, cur = 0;
    bool conv = false;
    const bool want_max = st.strength_tolerance > 0.0;
    while (it < st.max_iterations && !conv) {
        it += 1;
        const float2* Gc = G[cur];
        // 1. induced velocity of own rows
        induced_rows(Gc);
        // 2. row updates
        unsigned long long lmax = 0;  // max |dGamma| of the thread's rows (mag_bits)
        for (int k = 0; k < nrows; ++k) {
            int i = r0 + own_row(k);
            const RowGeom& g = rg[k];
            const FoilP f = m.foils[g.wing];
            const d3 u = row_velocity(i, g);
            const double ul = len(u);
            double aoa = ul > kMinPositive ? row_angle(g, u, ul) : 0.0;
            // the pre-stall lift coefficient serves the estimate and the residual alike
            const double clp = foil_cl_pre_stall(f, aoa);
            const double clc = m.include_viscous_lift ? clp + foil_cl_post_stall(f, aoa) : clp;  // circulation_cl
            double est = -0.5 * g.chord_len * ul * clc;
            double gold = gown[k];
            double r = residual_of_row(m, g, gold, u, ul, clp);
            double d = est - gold;
            if (want_max) {
                const unsigned long long db = mag_bits(d);
                lmax = db > lmax ? db : lmax;
            }
            double gnew = gold + st.damping * d;
            gown[k] = gnew;
            u_last[k] = u;
            aoa_last[k] = aoa;
            const float2 gs = split_f64(gnew);
            for (int q = 0; q < CS; ++q) {
                float2* Gr = cl.map_shared_rank(G[cur ^ 1], q);
                double* Rr = cl.map_shared_rank(RR[cur], q);
                Gr[i] = gs;
                Rr[i] = r;
            }
        }
        // block max of |dGamma|, only where a strength tolerance can stop the solve (with a
        // tolerance <= 0 the test `max < tolerance` never holds)
        if (want_max) {
            lmax = warp_umax_to_lane0(lmax);
            if (lane == 0) s_umax[warp] = lmax;
            __syncthreads();
            if (tid == 0) {
                unsigned long long v = 0;
                for (int w = 0; w < nwarps; ++w) v = s_umax[w] > v ? s_umax[w] : v;
                for (int q = 0; q < CS; ++q) cl.map_shared_rank(MX[cur], q)[rank] = bits_value(v);
            }
        }
        cl.sync();
        if (warp == 0) {
            double s = 0.0;
            for (int i = lane; i < N; i += 32) s += RR[cur][i];
            s = warp_sum_to_lane0(s);
            if (lane == 0) {
                double res = s / static_cast<double>(N);
                unsigned long long mb = 0;
                if (want_max)
                    for (int q = 0; q < CS; ++q) {
                        const unsigned long long bq = static_cast<unsigned long long>(__double_as_longlong(MX[cur][q]));
                        mb = bq > mb ? bq : mb;
                    }
                const double mx = bits_value(mb);
                s_res = res;
                s_conv = (res < st.residual_tolerance) || (want_max && mx < st.strength_tolerance);
            }
        }
        __syncthreads();
        residual = s_res;
        conv = s_conv != 0;
        cur ^= 1;
    }

    // final circulation from the last velocities (simple_iterative.rs:200-203)
    for (int k = 0; k < nrows; ++k) {
        int i = r0 + own_row(k);
        const RowGeom& g = rg[k];
        double gam = -0.5 * g.chord_len * len(u_last[k]) * circulation_cl(m, m.foils[g.wing], aoa_last[k]);
        b.gamma_prev[i] = gam;
        b.vel_out[i] = u_last[k];
        if (b.wake_str_row0) b.wake_str_row0[i] = gam;
        if (b.rec32_row0) b.rec32_row0[i].v[kRec32Gamma] = static_cast<float>(gam);
        if (b.rec64_row0) b.rec64_row0[i].v[kRec64Gamma] = gam;
    }
    if (rank == 0 && tid == 0) {
        b.scalars[0] = residual;
        b.scalars[1] = static_cast<double>(it);
        b.scalars[2] = conv ? 1.0 : 0.0;
    }
    // a copy whose wait ran out may still be in flight: wait for it (bounded) before leaving
    if (tid == 0)
        for (int q = 0; q < 2; ++q)
            if (pending[q]) mbar_wait_bounded(&s_mbar[q], mph[q] ^ 1u, b.err);
    cl.sync();  // no CTA leaves while others may still write into its shared memory
}

template <int RPT>
__global__ void __launch_bounds__(kSolveThreads, RPT == 1 ? 2 : 1) k_solve_si(DevModel m, SolveSettings st, SolveBuffers b) {
    si_solve<RPT>(m, st, b);
}

// Every case of a batch whose cluster size (and rows per thread) is this launch's: cluster i
// solves jobs[i].
template <int RPT>
__global__ void __launch_bounds__(kSolveThreads, RPT == 1 ? 2 : 1) k_solve_si_jobs(const SolveJob* jobs) {
    cg::cluster_group cl = cg::this_cluster();
    const SolveJob& j = jobs[blockIdx.x / cl.num_blocks()];
    si_solve<RPT>(j.m, j.st, j.b);
}

// rows per thread of a solve of N span lines
int si_rows_per_thread(int N) {
    const int CS = solve_cluster_size(N);
    const int rp = (N + CS - 1) / CS;
    return rp <= kSolveThreads ? 1 : kSolveRowsPerThread;
}

size_t si_smem_bytes(int N, int full, int comps) {
    const int CS = si_cluster_size(N);
    const int rp = (N + CS - 1) / CS;
    const int sr = si_slab_rows(N, full, comps);
    const long long bufs = sr == 0 ? 0 : (sr >= rp ? 1 : 2);
    return static_cast<size_t>(si_slab_offset(N) * 8 + bufs * sr * si_row_bytes(N, full, comps));
}

cudaError_t launch_solve_simple_iterative_jobs(const SolveJob* jobs, int n, int cluster, int rows_per_thread,
                                               size_t smem, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (cluster != 1 && cluster != 4 && cluster != 8) return cudaErrorInvalidValue;
    if (rows_per_thread != 1 && rows_per_thread != kSolveRowsPerThread) return cudaErrorInvalidValue;
    auto kernel = rows_per_thread == 1 ? k_solve_si_jobs<1> : k_solve_si_jobs<kSolveRowsPerThread>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(n * cluster), 1, 1);
    cfg.blockDim = dim3(kSolveThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, jobs);
}

cudaError_t launch_solve_simple_iterative(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, cudaStream_t s) {
    const int CS = solve_cluster_size(m.N);
    const int rp = (m.N + CS - 1) / CS;
    if (rp > kSolveThreads * kSolveRowsPerThread) return cudaErrorInvalidValue;
    size_t smem = si_smem_bytes(m.N, b.split_full, b.split_comps);
    auto kernel = si_rows_per_thread(m.N) == 1 ? k_solve_si<1> : k_solve_si<kSolveRowsPerThread>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CS, 1, 1);
    cfg.blockDim = dim3(kSolveThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, m, st, b);
}

// ---------------------------------------------------------------------------------------
// Linearized solver: one CTA per case (one case, or every case of a batch in one launch)
// ---------------------------------------------------------------------------------------
constexpr int kLinThreads = 512;
constexpr int kLinMaxCluster = 16;  // non-portable cluster size (16 SMs of one GPC)

// Per case in shared memory: control-point velocities, induced velocities and the
// circulation, then the augmented matrix [N][N+1] when it fits in what the launch gave.
__host__ __device__ inline size_t lin_vec_bytes(int N) {
    return static_cast<size_t>(N) * (2 * sizeof(d3) + sizeof(double));
}
__host__ __device__ inline size_t lin_mat_bytes(int N) { return static_cast<size_t>(N) * (N + 1) * sizeof(double); }

// Cluster of C CTAs: the vectors, the pivot row, the row permutation and its inverse, and
// the CTA's share of rows ((N + C - 1) / C rows of N + 1 values).
__host__ __device__ inline size_t lin_cluster_bytes(int N, int C) {
    const size_t W1 = static_cast<size_t>(N) + 1;
    return lin_vec_bytes(N) + W1 * sizeof(double) + 2 * static_cast<size_t>(N) * sizeof(int) +
           static_cast<size_t>((N + C - 1) / C) * W1 * sizeof(double);
}

// One row of the linearized system (linearized.rs:61-136): the velocity with the fixed part
// and the span component removed, the coefficients row[0..N-1] and the right-hand side row[N].
__device__ inline void lin_build_row(const DevModel& m, const SolveBuffers& b, int i, double* row) {
    const int N = m.N;
    RowGeom g = row_geom(m, i);
    d3 v = g.felt + b.fixed[i];
    v = v - g.span_dir * dot(v, g.span_dir);  // project(v, span_rel)
    d3 un = normalize(v);
    const d3 sd = g.span_dir;
    d3 nd = cross(un, sd);
    double aoa = len(v) > kMinPositive ? signed_angle_between(g.chord, v, g.span_dir) : 0.0;
    const FoilP f = m.foils[g.wing];
    double cll = foil_cl_linear(f, aoa);
    double ut = dot(v, un);
    double dcl = f.cl_initial_slope;
    for (int c = 0; c < N; ++c) {
        double uin = dot(b.factors[static_cast<long long>(i) * N + c], nd);
        double a = -dcl * uin / ut;
        if (i == c) a += 2.0 / (g.chord_len * ut);
        row[c] = a;
    }
    row[N] = -cll;
}

// After the solve, on one CTA: induced and total velocities, the viscous correction, the
// residual and the outputs (linearized.rs:141-213).
__device__ void lin_finish(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, d3* vel, d3* ind,
                           double* gam) {
    const int N = m.N, tid = threadIdx.x, nt = blockDim.x;
    // induced velocity and the total velocity (linearized.rs:141-156)
    auto update_induced = [&]() {
        for (int i = tid; i < N; i += nt) {
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int c = 0; c < N; ++c) {
                d3 f = b.factors[static_cast<long long>(i) * N + c];
                sx += f.x * gam[c];
                sy += f.y * gam[c];
                sz += f.z * gam[c];
            }
            d3 fx = b.fixed[i];
            ind[i] = mk(fx.x + sx, fx.y + sy, fx.z + sz);
        }
        __syncthreads();
    };
    update_induced();
    for (int i = tid; i < N; i += nt) vel[i] = total_velocity(st, m.felt_ctrl[i], ind[i]);
    __syncthreads();
    // viscous correction (linearized.rs:158-202)
    if (!st.disable_viscous_corrections) {
        for (int i = tid; i < N; i += nt) {
            RowGeom g = row_geom(m, i);
            const FoilP f = m.foils[g.wing];
            double aoa = len(vel[i]) > kMinPositive ? signed_angle_between(g.chord, vel[i], g.span_dir) : 0.0;
            double cll = foil_cl_linear(f, aoa);
            double clf = foil_cl_pre_stall(f, aoa);
            if (fabs(cll) > kMinPositive) gam[i] *= clf / cll;
        }
        __syncthreads();
        if (st.full_induced_correction) update_induced();
        for (int i = tid; i < N; i += nt) vel[i] = total_velocity(st, m.felt_ctrl[i], ind[i]);
        __syncthreads();
    }
    // residual (linearized.rs:204-213): the terms in parallel (into the induced-velocity
    // storage, no longer needed), summed in control-point order by one thread
    double* terms = reinterpret_cast<double*>(ind);
    for (int i = tid; i < N; i += nt) {
        RowGeom g = row_geom(m, i);
        const FoilP f = m.foils[g.wing];
        double aoa = len(vel[i]) > kMinPositive ? signed_angle_between(g.chord, vel[i], g.span_dir) : 0.0;
        terms[i] = residual_term(m, g, f, gam[i], vel[i], aoa);
    }
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += terms[i];
        b.scalars[0] = s / static_cast<double>(N);
        b.scalars[1] = 1.0;
        b.scalars[2] = 1.0;
    }
    for (int i = tid; i < N; i += nt) {
        b.gamma_prev[i] = gam[i];
        b.vel_out[i] = vel[i];
        if (b.wake_str_row0) b.wake_str_row0[i] = gam[i];
        if (b.rec32_row0) b.rec32_row0[i].v[kRec32Gamma] = static_cast<float>(gam[i]);
        if (b.rec64_row0) b.rec64_row0[i].v[kRec64Gamma] = gam[i];
    }
}

// Linearized::solve (linearized.rs:54-222) for one case on the calling CTA. The Gaussian
// elimination (linalg.rs:41-103) keeps the reference's arithmetic per element: the pivot is
// the first row of largest |A[i][k]| (warp 0: per-lane scan, then a butterfly on (value,
// lowest index)); row i -= (A[i][k] / pivot) * row k over columns k..N (a warp per row);
// back substitution by warp 0, one row at a time. Where the matrix lives (shared memory or
// the case's global scratch) does not change any result.
__device__ void lin_solve_case(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, unsigned char* dyn,
                               size_t dyn_bytes) {
    const int N = m.N, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    const int W1 = N + 1;
    d3* vel = reinterpret_cast<d3*>(dyn);                 // [N]
    d3* ind = vel + N;                                    // [N]
    double* gam = reinterpret_cast<double*>(ind + N);     // [N]
    double* A = lin_vec_bytes(N) + lin_mat_bytes(N) <= dyn_bytes ? gam + N : b.lin_work;  // [N][N+1]
    __shared__ int s_piv;

    for (int i = tid; i < N; i += nt) lin_build_row(m, b, i, A + static_cast<long long>(i) * W1);
    __syncthreads();
    // forward elimination with partial pivoting
    for (int k = 0; k < N; ++k) {
        double* Ak = A + static_cast<long long>(k) * W1;
        if (warp == 0) {
            double bv = -1.0;
            int bi = N;
            for (int i = k + lane; i < N; i += 32) {
                const double v = fabs(A[static_cast<long long>(i) * W1 + k]);
                if (v > bv) {
                    bv = v;
                    bi = i;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) s_piv = bi < N ? bi : k;
        }
        __syncthreads();
        const int mr = s_piv;
        if (mr != k) {
            double* Am = A + static_cast<long long>(mr) * W1;
            for (int j = tid; j <= N; j += nt) {
                const double t = Ak[j];
                Ak[j] = Am[j];
                Am[j] = t;
            }
        }
        __syncthreads();
        const double piv = Ak[k];
        if (fabs(piv) < 1e-12) {  // the same value in every thread: the whole CTA leaves
            if (tid == 0) {
                atomicExch(b.err, kDevSingular);
                b.scalars[3] = 1.0;
            }
            return;
        }
        for (int i = k + 1 + warp; i < N; i += nw) {
            double* Ai = A + static_cast<long long>(i) * W1;
            const double f = Ai[k] / piv;
            __syncwarp();  // every lane has read A[i][k] before lane 0 overwrites it
            for (int j = k + lane; j <= N; j += 32) Ai[j] -= f * Ak[j];
        }
        __syncthreads();
    }
    // back substitution
    if (warp == 0) {
        for (int i = N - 1; i >= 0; --i) {
            const double* Ai = A + static_cast<long long>(i) * W1;
            double part = 0.0;
            for (int j = i + 1 + lane; j < N; j += 32) part += Ai[j] * gam[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
            if (lane == 0) gam[i] = (Ai[N] - part) / Ai[i];
            __syncwarp();
        }
    }
    __syncthreads();
    lin_finish(m, st, b, vel, ind, gam);
}

__global__ void __launch_bounds__(kLinThreads) k_solve_lin(DevModel m, SolveSettings st, SolveBuffers b, unsigned smem) {
    extern __shared__ __align__(16) unsigned char lin_dyn[];
    lin_solve_case(m, st, b, lin_dyn, smem);
}

// Every case of a batch in one launch: CTA i solves jobs[i].
__global__ void __launch_bounds__(kLinThreads) k_solve_lin_jobs(const SolveJob* jobs, unsigned smem) {
    extern __shared__ __align__(16) unsigned char lin_dyn[];
    const SolveJob& j = jobs[blockIdx.x];
    lin_solve_case(j.m, j.st, j.b, lin_dyn, smem);
}

// Linearized::solve for a system whose matrix does not fit one CTA's shared memory, on a
// thread-block cluster of C CTAs: physical row r lives in the shared memory of CTA r mod C
// (row r / C there). Row exchanges are kept as a permutation held by every CTA (at[k] =
// physical row at position k, pos[r] its inverse), so rows never move. Per column k, one
// cluster barrier: each CTA's warp 0 has put its candidate for column k (the rows at
// positions >= k: largest |A[r][k]|, then lowest position, i.e. the reference's first
// largest row after its swaps) into a double-buffered slot; after the barrier every CTA
// reduces the C candidates (one per lane, the same butterfly), applies the same exchange
// to its permutation,
// copies the pivot row (columns k..N; a pivot row never changes again) through distributed
// shared memory, eliminates its own rows at positions > k with lin_solve_case's per-element
// arithmetic, and posts its candidate for column k + 1. Back substitution runs on CTA 0,
// reading each pivot row from its owner as lin_solve_case reads it (warp 0, lane-strided
// sum, butterfly), while the other CTAs wait at the final barrier. CTA 0 then finishes the
// solve. The result is bit-identical to lin_solve_case; all waits are cluster barriers.
__device__ void lin_solve_cluster(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, unsigned char* dyn) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = static_cast<int>(cl.num_blocks()), rank = static_cast<int>(cl.block_rank());
    const int N = m.N, W1 = N + 1, R = (N + C - 1) / C;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    d3* vel = reinterpret_cast<d3*>(dyn);              // [N] (CTA 0)
    d3* ind = vel + N;                                 // [N] (CTA 0)
    double* gam = reinterpret_cast<double*>(ind + N);  // [N] (CTA 0)
    double* prow = gam + N;                            // [N + 1] pivot row of the current column
    int* at = reinterpret_cast<int*>(prow + W1);       // [N] physical row at each position
    int* pos = at + N;                                 // [N] position of each physical row
    double* A = reinterpret_cast<double*>(pos + N);    // [R][N + 1] rows rank, rank + C, ...
    __shared__ double s_cand_v[2];
    __shared__ int s_cand_p[2], s_piv;

    // the candidate of this CTA for column k: first largest |A[r][k]| over its rows at
    // positions >= k (lowest position among equal values), into slot k & 1
    auto post_candidate = [&](int k) {
        double bv = -1.0;
        int bp = N;
        for (int l = lane; l < R; l += 32) {
            const int r = rank + l * C;
            if (r >= N) break;
            const int p = pos[r];
            if (p < k) continue;
            const double v = fabs(A[static_cast<long long>(l) * W1 + k]);
            if (v > bv || (v == bv && p < bp)) {
                bv = v;
                bp = p;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int op = __shfl_xor_sync(0xffffffffu, bp, o);
            if (ov > bv || (ov == bv && op < bp)) {
                bv = ov;
                bp = op;
            }
        }
        if (lane == 0) {
            s_cand_v[k & 1] = bv;
            s_cand_p[k & 1] = bp;
        }
    };

    for (int i = tid; i < N; i += nt) {
        at[i] = i;
        pos[i] = i;
    }
    for (int l = tid; l < R; l += nt) {
        const int r = rank + l * C;
        if (r < N) lin_build_row(m, b, r, A + static_cast<long long>(l) * W1);
    }
    __syncthreads();
    if (warp == 0) post_candidate(0);
    for (int k = 0; k < N; ++k) {
        cl.sync();  // every CTA's candidate for column k is posted; column k of every row is final
        if (warp == 0) {  // lane q reads CTA q's candidate; the same butterfly as post_candidate
            double bv = -1.0;
            int bp = N;
            if (lane < C) {
                bv = *cl.map_shared_rank(&s_cand_v[k & 1], lane);
                bp = *cl.map_shared_rank(&s_cand_p[k & 1], lane);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int op = __shfl_xor_sync(0xffffffffu, bp, o);
                if (ov > bv || (ov == bv && op < bp)) {
                    bv = ov;
                    bp = op;
                }
            }
            if (lane == 0) {  // the cluster's first largest row: apply the exchange
                const int mr = bp < N ? bp : k;  // position of the pivot row
                const int rk = at[k], rm = at[mr];
                at[k] = rm;
                at[mr] = rk;
                pos[rm] = k;
                pos[rk] = mr;
                s_piv = rm;
            }
        }
        __syncthreads();
        const int pr = s_piv;  // physical pivot row
        {
            const double* src = cl.map_shared_rank(A, pr % C) + static_cast<long long>(pr / C) * W1;
            for (int j = k + tid; j <= N; j += nt) prow[j] = src[j];
        }
        __syncthreads();
        const double piv = prow[k];
        if (fabs(piv) < 1e-12) {  // the same value in every CTA: the whole cluster leaves
            if (rank == 0 && tid == 0) {
                atomicExch(b.err, kDevSingular);
                b.scalars[3] = 1.0;
            }
            cl.sync();  // no CTA leaves while another may still read its rows
            return;
        }
        for (int l = warp; l < R; l += nw) {
            const int r = rank + l * C;
            if (r >= N) break;
            if (pos[r] <= k) continue;
            double* Ai = A + static_cast<long long>(l) * W1;
            const double f = Ai[k] / piv;
            __syncwarp();  // every lane has read A[i][k] before lane 0 overwrites it
            for (int j = k + lane; j <= N; j += 32) Ai[j] -= f * prow[j];
        }
        __syncthreads();
        if (warp == 0 && k + 1 < N) post_candidate(k + 1);
    }
    cl.sync();  // every row is final
    if (rank == 0) {
        if (warp == 0) {
            for (int i = N - 1; i >= 0; --i) {
                const int r = at[i];
                const double* Ai = cl.map_shared_rank(A, r % C) + static_cast<long long>(r / C) * W1;
                double part = 0.0;
                for (int j = i + 1 + lane; j < N; j += 32) part += Ai[j] * gam[j];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if (lane == 0) gam[i] = (Ai[N] - part) / Ai[i];
                __syncwarp();
            }
        }
        __syncthreads();
    }
    cl.sync();  // CTA 0 has read every row it needs
    if (rank == 0) lin_finish(m, st, b, vel, ind, gam);
}

__global__ void __launch_bounds__(kLinThreads) k_solve_lin_cluster(DevModel m, SolveSettings st, SolveBuffers b) {
    extern __shared__ __align__(16) unsigned char lin_dyn[];
    lin_solve_cluster(m, st, b, lin_dyn);
}

// Every case of a batch that needs a cluster of this launch's size: cluster i solves jobs[i].
__global__ void __launch_bounds__(kLinThreads) k_solve_lin_cluster_jobs(const SolveJob* jobs) {
    extern __shared__ __align__(16) unsigned char lin_dyn[];
    cg::cluster_group cl = cg::this_cluster();
    const SolveJob& j = jobs[blockIdx.x / cl.num_blocks()];
    lin_solve_cluster(j.m, j.st, j.b, lin_dyn);
}

namespace {

void cluster_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute& attr, int clusters, int C, size_t smem, cudaStream_t s) {
    cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(clusters * C), 1, 1);
    cfg.blockDim = dim3(kLinThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = static_cast<unsigned>(C);
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
}

template <class K>
cudaError_t prepare_cluster_kernel(K kernel, int C, size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e == cudaSuccess && C > 8) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

// Whether clusters of C CTAs with `smem` bytes of shared memory each can be resident on the
// current device (cached per device and shape).
bool cluster_fits(int C, size_t smem) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, size_t>, bool> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, C, smem);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    bool ok = prepare_cluster_kernel(k_solve_lin_cluster, C, smem) == cudaSuccess &&
              prepare_cluster_kernel(k_solve_lin_cluster_jobs, C, smem) == cudaSuccess;
    if (ok) {
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr;
        cluster_config(cfg, attr, 1, C, smem, nullptr);
        int n = 0;
        ok = cudaOccupancyMaxActiveClusters(&n, k_solve_lin_cluster, &cfg) == cudaSuccess && n > 0;
    }
    if (!ok) (void)cudaGetLastError();  // a refused shape is not an error of the caller
    cache[key] = ok;
    return ok;
}

}  // namespace

LinPlan linearized_plan(int N) {
    const size_t v = lin_vec_bytes(N), a = lin_mat_bytes(N);
    if (v + a <= kLinSmemLimit) return {1, v + a};
    for (int C = 2; C <= kLinMaxCluster; C *= 2) {
        const size_t bytes = lin_cluster_bytes(N, C);
        if (bytes <= kLinSmemLimit && cluster_fits(C, bytes)) return {C, bytes};
    }
    return {1, v};  // matrix in the case's global scratch
}

cudaError_t launch_solve_linearized(const DevModel& m, const SolveSettings& st, const SolveBuffers& b, cudaStream_t s) {
    const LinPlan p = linearized_plan(m.N);
    if (p.cluster == 1) {
        if (p.smem > 48 * 1024) {
            cudaError_t e =
                cudaFuncSetAttribute(k_solve_lin, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(p.smem));
            if (e != cudaSuccess) return e;
        }
        k_solve_lin<<<1, kLinThreads, p.smem, s>>>(m, st, b, static_cast<unsigned>(p.smem));
        return cudaGetLastError();
    }
    cudaError_t e = prepare_cluster_kernel(k_solve_lin_cluster, p.cluster, p.smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_config(cfg, attr, 1, p.cluster, p.smem, s);
    return cudaLaunchKernelEx(&cfg, k_solve_lin_cluster, m, st, b);
}

cudaError_t launch_solve_linearized_jobs(const SolveJob* jobs, int n, const LinPlan& plan, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (plan.smem > kLinSmemLimit) return cudaErrorInvalidValue;
    if (plan.cluster == 1) {
        if (plan.smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(k_solve_lin_jobs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(plan.smem));
            if (e != cudaSuccess) return e;
        }
        k_solve_lin_jobs<<<n, kLinThreads, plan.smem, s>>>(jobs, static_cast<unsigned>(plan.smem));
        return cudaGetLastError();
    }
    cudaError_t e = prepare_cluster_kernel(k_solve_lin_cluster_jobs, plan.cluster, plan.smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr;
    cluster_config(cfg, attr, n, plan.cluster, plan.smem, s);
    return cudaLaunchKernelEx(&cfg, k_solve_lin_cluster_jobs, jobs);
}

// ---------------------------------------------------------------------------------------
// Forces, one CTA
// ---------------------------------------------------------------------------------------
constexpr int kForceThreads = 256;

// One case's forces on the calling CTA (k_forces: one case; k_forces_jobs: a CTA per case
// of a batch, all cases side by side instead of one SM per case on a few streams).
__device__ void forces_case(const DevModel& m, const StepParams& p, const ForceArgs& f) {
    const int N = m.N, S = m.S, tid = threadIdx.x, nt = blockDim.x;
    const OutLayout L = OutLayout::make(N, S);
    double* o = f.out;
    const bool body = m.output_body != 0;
    for (int i = tid; i < N; i += nt) {
        double g = f.gamma[i];
        d3 v = f.vel[i];
        d3 sr = m.span_e[i] - m.span_s[i];
        double aoa = len(v) > kMinPositive ? signed_angle_between(m.chord_global[i], v, normalize(sr)) : 0.0;
        d3 acc = mk(0, 0, 0);
        if (f.fd_count >= 2) acc = (v * 3.0 - f.hist1[i] * 4.0 + f.hist0[i]) / (2.0 * p.dt);
        f.hist0[i] = f.hist1[i];
        f.hist1[i] = v;
        d3 fv = body ? to_body(v, p.rotation) : v;
        d3 fa = body ? to_body(acc, p.rotation) : acc;
        d3 sl_local = m.span_e_local[i] - m.span_s_local[i];
        d3 sl_out = body ? sl_local : sr;
        d3 cv_out = body ? m.chord_local[i] : m.chord_global[i];
        const FoilP fo = m.foils[m.wing_of_line[i]];
        double area = m.chord_len[i] * m.span_len_local[i];
        double ff = 0.5 * area * m.density * len2(fv);
        d3 circ = len(fv) == 0.0 ? mk(0, 0, 0) : (g * cross(fv, sl_out)) * m.density;
        d3 visc = mk(0, 0, 0);
        if (!m.include_viscous_lift) visc = normalize(cross(sl_local, fv)) * foil_cl_post_stall(fo, aoa) * ff;
        d3 drag = normalize(fv) * foil_cd(fo, aoa) * ff;
        double strip = m.chord_len[i] * len(sl_out);
        d3 ra = fa - project(fa, normalize(sl_out));
        ra = ra - project(ra, cv_out);
        d3 am = mk(0, 0, 0);
        if (len(ra) != 0.0) am = (fo.added_mass_factor * len(ra)) * m.density * strip * normalize(ra);
        d3 gy = mk(0, 0, 0);
        d3 tot = circ;
        tot = tot + visc;
        tot = tot + drag;
        tot = tot + am;
        tot = tot + gy;
        d3 comps[6] = {circ, visc, drag, am, gy, tot};
        o[L.gamma + i] = g;
        d3 ctrl = m.ctrl[i];
        d3 felt = m.felt_ctrl[i];
        const d3* src[6] = {&v, &felt, &fv, &fa, &ctrl, nullptr};
        long long offs[5] = {L.vel, L.felt, L.fvel, L.acc, L.ctrl};
        for (int q = 0; q < 5; ++q) {
            o[offs[q] + 3 * i] = src[q]->x;
            o[offs[q] + 3 * i + 1] = src[q]->y;
            o[offs[q] + 3 * i + 2] = src[q]->z;
        }
        o[L.aoa + i] = aoa;
        for (int c = 0; c < 6; ++c) {
            long long base = L.sect + (static_cast<long long>(c) * N + i) * 3;
            o[base] = comps[c].x;
            o[base + 1] = comps[c].y;
            o[base + 2] = comps[c].z;
        }
    }
    __syncthreads();
    // integrated force and moment of each (wing, component), summed in line order
    for (int t = tid; t < S * 6; t += nt) {
        const int w = t / 6, c = t % 6;
        d3 fs = mk(0, 0, 0), ms = mk(0, 0, 0);
        for (int i = m.wing_start[w]; i < m.wing_end[w]; ++i) {
            if (m.is_virtual[i]) continue;
            d3 cp = body ? 0.5 * (m.span_s_local[i] + m.span_e_local[i]) : 0.5 * (m.span_s[i] + m.span_e[i]);
            long long base = L.sect + (static_cast<long long>(c) * N + i) * 3;
            d3 sf = mk(o[base], o[base + 1], o[base + 2]);
            fs = fs + sf;
            ms = ms + cross(cp, sf);
        }
        long long bf = L.intf + (static_cast<long long>(w) * 6 + c) * 3, bm = L.intm + (static_cast<long long>(w) * 6 + c) * 3;
        o[bf] = fs.x;
        o[bf + 1] = fs.y;
        o[bf + 2] = fs.z;
        o[bm] = ms.x;
        o[bm + 1] = ms.y;
        o[bm + 2] = ms.z;
    }
    __syncthreads();
    if (tid == 0) {
        d3 fsum = mk(0, 0, 0), msum = mk(0, 0, 0);
        for (int w = 0; w < S; ++w) {
            long long bf = L.intf + (static_cast<long long>(w) * 6 + 5) * 3, bm = L.intm + (static_cast<long long>(w) * 6 + 5) * 3;
            fsum = fsum + mk(o[bf], o[bf + 1], o[bf + 2]);
            msum = msum + mk(o[bm], o[bm + 1], o[bm + 2]);
        }
        o[L.fsum] = fsum.x;
        o[L.fsum + 1] = fsum.y;
        o[L.fsum + 2] = fsum.z;
        o[L.msum] = msum.x;
        o[L.msum + 1] = msum.y;
        o[L.msum + 2] = msum.z;
        o[L.residual] = f.scalars[0];
        o[L.iterations] = f.scalars[1];
        o[L.converged] = f.scalars[2];
    }
}

__global__ void __launch_bounds__(kForceThreads) k_forces(DevModel m, StepParams p, ForceArgs f) { forces_case(m, p, f); }

__global__ void __launch_bounds__(kForceThreads) k_forces_jobs(const ForceJob* jobs) {
    const ForceJob& j = jobs[blockIdx.x];
    forces_case(j.m, j.p, j.f);
}

cudaError_t launch_forces(const DevModel& m, const StepParams& p, const ForceArgs& f, cudaStream_t s) {
    k_forces<<<1, kForceThreads, 0, s>>>(m, p, f);
    return cudaGetLastError();
}

cudaError_t launch_forces_jobs(const ForceJob* jobs, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_forces_jobs<<<static_cast<unsigned>(n), kForceThreads, 0, s>>>(jobs);
    return cudaGetLastError();
}

}  // namespace sbgpu
