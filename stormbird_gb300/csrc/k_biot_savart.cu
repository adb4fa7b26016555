// Biot-Savart sweeps of vortex-ring panels (sm_103a).
//
// Reference: DynamicWake::induced_velocities_local_include_self_induced
// (stormbird/src/lifting_line/wake/dynamic_wake/induced_velocity_calc.rs:111-126) with
// Panel::induced_velocity_with_unit_strength (singularity_elements/panel.rs:61-118),
// the vortex line of vortex_line.rs:18-106 and the symmetry correction of
// symmetry_condition.rs:27-43.
//
// k_bs_sweep: an N-body sweep over (target tile x source chunk) work items, taken from an
// atomic work counter by a persistent grid. Panel records of a chunk are streamed into
// shared memory in tiles by one thread with bulk asynchronous copies (cp.async.bulk,
// completion on an mbarrier), double-buffered. Each thread holds T targets in registers.
// Near/far classification follows panel.rs:53-57 per pair; a warp evaluates the vortex
// ring only if one of its lanes needs it and the point doublet only if one needs that.
// Sums: FP32 within a tile, then an error-free TwoSum fold across tiles (compensated
// accumulation); plain FP32 and FP64 variants exist for the precision study.
// Zero-strength panels are skipped (induced_velocity_calc.rs:203).
//
// k_unit_matrix: the unit-strength influence of the first-row panels at the control
// points (frozen_wake.rs:198-249), in FP64: the control point lies on its own bound
// vortex, where the reference's 1e-10 closeness cut-off must fire exactly as in f64.
#include <atomic>
#include <cfloat>
#include <cstdio>
#include <math_constants.h>

#include "sb_device.cuh"
#include "sb_kernels.h"
#include "sb_ptx.cuh"

namespace sbgpu {

// ---------------------------------------------------------------------------------------
// FP64 element functions (literal restatement, used by k_unit_matrix and the FP64 sweep)
// ---------------------------------------------------------------------------------------
// vortex_line.rs:18-106
__device__ inline d3 line_unit_f64(d3 a, d3 b, d3 x, double rc) {
    d3 r1 = x - a, r2 = x - b;
    double r1sq = len2(r1), r2sq = len2(r2);
    double l1 = sqrt(r1sq), l2 = sqrt(r2sq);
    double r1r2 = l1 * l2;
    double den = r1r2 * (r1r2 + dot(r1, r2));
    if (fabs(den) > 1.0e-10) {
        double core = 1.0;
        if (rc != 0.0) {
            d3 rl = b - a;
            double ll = sqrt(len2(rl));
            d3 dir = rl / ll;
            double t = dot(r1, dir);
            double d2 = t < 0.0 ? r1sq : (t > ll ? r2sq : len2(r1) - t * t);
            double rc2 = rc * rc;
            double cden = sqrt(rc2 * rc2 + d2 * d2);
            core = cden > 0.0 ? d2 / cden : 0.0;
        }
        double k = (l1 + l2) / den;
        return (core * cross(r1, r2)) * (k * kFourPiInv);
    }
    return mk(0, 0, 0);
}

// panel.rs:61-118 (record layout of PanelRec<double>: [25] holds the core length itself)
__device__ inline d3 panel_unit_f64(const double* v, d3 x) {
    d3 c = mk(v[16], v[17], v[18]);
    d3 t = x - c;
    double d2 = len2(t);
    if (d2 <= v[19]) {
        d3 p[4] = {mk(v[0], v[1], v[2]), mk(v[3], v[4], v[5]), mk(v[6], v[7], v[8]), mk(v[9], v[10], v[11])};
        d3 u = mk(0, 0, 0);
        for (int i = 0; i < 4; ++i) u = u + line_unit_f64(p[i], p[(i + 1) & 3], x, v[25]);
        return u;
    }
    d3 n = mk(v[20], v[21], v[22]);
    double d5 = d2 * d2 * sqrt(d2);
    double h = dot(t, n);
    return (v[23] * ((3.0 * h) * t - d2 * n)) / d5;
}

__device__ inline d3 mirror(int sym, d3 p) {
    if (sym == 1) return mk(-p.x, p.y, p.z);
    if (sym == 2) return mk(p.x, -p.y, p.z);
    return mk(p.x, p.y, -p.z);
}
__device__ inline d3 sym_correct(int sym, d3 u, d3 m) {
    if (sym == 1) return mk(u.x - m.x, u.y + m.y, u.z + m.z);
    if (sym == 2) return mk(u.x + m.x, u.y - m.y, u.z + m.z);
    return mk(u.x + m.x, u.y + m.y, u.z - m.z);
}

// ---------------------------------------------------------------------------------------
// Sweep kernel
// ---------------------------------------------------------------------------------------
template <class R>
struct TileSize;
template <>
struct TileSize<float> { static constexpr int value = 64; };
template <>
struct TileSize<double> { static constexpr int value = 32; };

template <class R>
__device__ __forceinline__ void two_sum_acc(R& s, R& c, R t) {
    R sum = s + t;
    R bp = sum - s;
    R err = (s - (sum - bp)) + (t - bp);
    s = sum;
    c += err;
}

// ---------------------------------------------------------------------------------------
// Packed FP32 helpers (Blackwell f32x2: two FP32 operations per instruction)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as one packed FMA (b * -1 is exact, so the result is the rounded difference)
__device__ __forceinline__ float2 sub2s(float2 a, float b) { return __ffma2_rn(make_float2(b, b), make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sel2(bool cx, float2 a, bool cy, float2 b) {
    return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}
// The hardware reciprocal square root (PTX rsqrt.approx.ftz.f32). Every argument below is
// first clamped to a normal float, where this is the same approximation rsqrtf returns,
// without the handling of subnormal arguments around it.
__device__ __forceinline__ float rsqrt_n(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Point doublet (panel.rs:82-96) at two targets, e = target - centre, |e|^2 = e2, added to
// (TX, TY, TZ): Gamma area/(4 pi) (3 (n.e) e / |e|^5 - n / |e|^3). The record's slot 35 holds
// area/(4 pi) / (3 sqrt 3) and f = Gamma x slot 35 per lane (0 for a lane that takes no
// doublet). With q = 1/sqrt(|e|^2 / 3): q^2 = 3/|e|^2, f q^3 = Gamma area/(4 pi) / |e|^3, so
// the doublet is B (g e - n) with B = f q^3 and g = q^2 (n.e): 20 packed operations. The
// floor keeps q finite where a degenerate panel meets a target at its centre (its doublet
// then overflows, as the f64 formula would).
__device__ __forceinline__ void doublet2(float2 f, const float* v, float2 ex, float2 ey, float2 ez, float2 e2,
                                         float2& TX, float2& TY, float2& TZ) {
    const float2 e3 = fma2(e2, bc(1.f / 3.f), bc(FLT_MIN));
    const float2 q = make_float2(rsqrt_n(e3.x), rsqrt_n(e3.y));
    const float2 q2 = mul2(q, q);
    const float2 B = mul2(mul2(f, q), q2);
    const float nx = v[36], ny = v[37], nz = v[38];
    const float2 g = mul2(q2, fma2(ex, bc(nx), fma2(ey, bc(ny), mul2(ez, bc(nz)))));
    TX = fma2(B, fma2(g, ex, bc(-nx)), TX);
    TY = fma2(B, fma2(g, ey, bc(-ny)), TY);
    TZ = fma2(B, fma2(g, ez, bc(-nz)), TZ);
}

// Vortex ring of one FP32 panel record at two targets (the two lanes of the float2s), given
// e = x - centre (float-float difference). r_k = e - o_k. Per segment, with c = d x r1 = r1 x r2:
//   r1.r2 = |r1|^2 - r1.d,
//   den = l1 l2 (l1 l2 + r1.r2) = B / A without cancellation
//        (A, B) = (l1 l2 - r1.r2, l1 l2 |c|^2) if r1.r2 < 0, else (1, l1 l2 (l1 l2 + r1.r2)),
//   distance^2 to the segment = |c|^2 / |d|^2 inside it, the end-point distance outside,
//   core * k = d2 (l1 + l2) A / (B sqrt(d2^2 + rc^4)) with a single rsqrt,
// which is the reference's (vortex_line.rs:18-106) value, evaluated without the FP32
// cancellations of its literal form. Returns sum_k core_k k_k c_k (times Gamma/4pi = velocity).
// Corner vector r = e - o (o: FP32 offset of the corner from the record's anchor), |r|^2, |r|.
__device__ __forceinline__ void corner2(float2 ex, float2 ey, float2 ez, const float* o, float2& rx, float2& ry,
                                        float2& rz, float2& rs, float2& rl) {
    rx = sub2s(ex, o[0]);
    ry = sub2s(ey, o[1]);
    rz = sub2s(ez, o[2]);
    rs = fma2(rx, rx, fma2(ry, ry, mul2(rz, rz)));
    // r = 0 (target on a corner) gives l = 0: the floor is one packed add on the FMA pipe
    // (the same value as a maximum wherever |r|^2 > 4e-23, where 1e-30 is below its rounding)
    const float2 rsf = add2(rs, bc(1e-30f));
    rl = mul2(rs, make_float2(rsqrt_n(rsf.x), rsqrt_n(rsf.y)));
}

// One segment from corner 1 (r1) to corner 2 (r2 = r1 - d): s * c with c = d x r1, i.e.
// core * k * (r1 x r2) of vortex_line.rs:18-106 (see above), added to (ax, ay, az), times the
// weight g when WEIGHTED.
template <bool WEIGHTED>
__device__ __forceinline__ void segment2(float2 rx, float2 ry, float2 rz, float2 rs1, float2 rl1, float2 rs2,
                                         float2 rl2, float dx, float dy, float dz, float il, float dd, float rc4, float g,
                                         float2& ax, float2& ay, float2& az) {
    const float2 p = mul2(rl1, rl2);
    // projection on the segment, and r1.r2 = |r1|^2 - r1.d (r2 = r1 - d)
    const float2 tp = fma2(rx, bc(dx), fma2(ry, bc(dy), mul2(rz, bc(dz))));
    const float2 q = fma2(tp, bc(-1.f), rs1);
    const float2 cx = fma2(bc(dy), rz, mul2(bc(-dz), ry));
    const float2 cy = fma2(bc(dz), rx, mul2(bc(-dx), rz));
    const float2 cz = fma2(bc(dx), ry, mul2(bc(-dy), rx));
    const float2 c2 = fma2(cx, cx, fma2(cy, cy, mul2(cz, cz)));
    const bool n0 = q.x < 0.f, n1 = q.y < 0.f;
    // both branches use l1 l2 + |r1.r2|: p - q for q < 0 (A), p + q otherwise (B)
    const float2 pa = add2(p, make_float2(fabsf(q.x), fabsf(q.y)));
    const float2 Ax = make_float2(n0 ? pa.x : 1.f, n1 ? pa.y : 1.f);
    const float2 Bx = mul2(p, make_float2(n0 ? c2.x : pa.x, n1 ? c2.y : pa.y));
    // past the segment's end (projection r1.d > |d|^2): the end-point distance
    float2 d2 = mul2(c2, bc(il));
    d2.x = tp.x > dd ? rs2.x : d2.x;
    d2.y = tp.y > dd ? rs2.y : d2.y;
    d2.x = tp.x < 0.f ? rs1.x : d2.x;
    d2.y = tp.y < 0.f ? rs1.y : d2.y;
    // X = 0 only where B = 0 too (target on the segment or a corner); the select below
    // then discards the lane, so the floor (a packed add) only keeps rsqrt finite
    const float2 X = add2(mul2(mul2(Bx, Bx), fma2(d2, d2, bc(rc4))), bc(1e-37f));
    const float2 Aw = WEIGHTED ? mul2(Ax, bc(g)) : Ax;
    const float2 s0 = mul2(mul2(mul2(d2, add2(rl1, rl2)), Aw),
                           make_float2(rsqrt_n(X.x), rsqrt_n(X.y)));
    const float2 lim = mul2(Ax, bc(1.0e-10f));
    const float2 sg = make_float2(Bx.x > lim.x ? s0.x : 0.f, Bx.y > lim.y ? s0.y : 0.f);
    ax = fma2(sg, cx, ax);
    ay = fma2(sg, cy, ay);
    az = fma2(sg, cz, az);
}

__device__ __forceinline__ void ring2(const float* v, float2 ex, float2 ey, float2 ez, float2& ax, float2& ay,
                                      float2& az) {
    float2 rx[4], ry[4], rz[4], rs[4], rl[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) corner2(ex, ey, ez, v + 3 * k, rx[k], ry[k], rz[k], rs[k], rl[k]);
    const float rc4 = v[40];
    ax = ay = az = bc(0.f);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int k1 = (k + 1) & 3;
        segment2<false>(rx[k], ry[k], rz[k], rs[k], rl[k], rs[k1], rl[k1], v[12 + 3 * k], v[12 + 3 * k + 1],
                        v[12 + 3 * k + 2], v[24 + k], v[kRec32DD + k], rc4, 1.f, ax, ay, az);
    }
}

// Open chain of a chain record (kChain* layout) at two targets: five corners shared by four
// segments, each weighted by its strength difference / 4 pi. Corners are computed as the
// chain advances (two live at a time).
__device__ __forceinline__ void chain2(const float* v, float2 ex, float2 ey, float2 ez, float2& ax, float2& ay,
                                       float2& az) {
    float2 rxa, rya, rza, rsa, rla;
    corner2(ex, ey, ez, v + kChainOff, rxa, rya, rza, rsa, rla);
    const float rc4 = v[kChainRc4];
    ax = ay = az = bc(0.f);
#pragma unroll
    for (int k = 0; k < kChainSegs; ++k) {
        float2 rxb, ryb, rzb, rsb, rlb;
        corner2(ex, ey, ez, v + kChainOff + 3 * (k + 1), rxb, ryb, rzb, rsb, rlb);
        segment2<true>(rxa, rya, rza, rsa, rla, rsb, rlb, v[kChainD + 3 * k], v[kChainD + 3 * k + 1],
                       v[kChainD + 3 * k + 2], v[kChainIl + k], v[kChainDD + k], rc4, v[kChainG + k], ax, ay, az);
        rxa = rxb;
        rya = ryb;
        rza = rzb;
        rsa = rsb;
        rla = rlb;
    }
}

// panel.rs:53-57 in f64 for one target given as float-float coordinates: the squared
// distance of the float-float target from the float-float centre against the far-field
// length squared (hi + lo). The points are the f64 points to within 2^-48 relative.
__device__ inline bool near_f64(const float* v, float xh, float xl, float yh, float yl, float zh, float zl) {
    const double dx = (static_cast<double>(xh) - v[28]) + (static_cast<double>(xl) - v[32]);
    const double dy = (static_cast<double>(yh) - v[29]) + (static_cast<double>(yl) - v[33]);
    const double dz = (static_cast<double>(zh) - v[30]) + (static_cast<double>(zl) - v[34]);
    return dx * dx + dy * dy + dz * dz <= static_cast<double>(v[31]) + static_cast<double>(v[kRec32FF2Lo]);
}

// The near/far decision of the targets in `which` (bit 0: the first lane of the pair, bit 1:
// the second) from the float-float difference, and where that lies within kNearFarBand of
// ff2, by near_f64; bit k of the result: target k is near. Out of line: the rare branch's
// registers stay out of the sweep's loop.
__device__ __noinline__ int near_recheck(const float* v, float2 X2h, float2 Y2h, float2 Z2h, float2 X2l, float2 Y2l,
                                         float2 Z2l, int which) {
    const float ff2 = v[31];
    const float2 ex = add2(sub2s(X2h, v[28]), sub2s(X2l, v[32]));
    const float2 ey = add2(sub2s(Y2h, v[29]), sub2s(Y2l, v[33]));
    const float2 ez = add2(sub2s(Z2h, v[30]), sub2s(Z2l, v[34]));
    const float2 f2 = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
    const float2 g = sub2s(f2, ff2);
    const float nb = kNearFarBand * ff2;
    int n = 0;
    if (which & 1)
        n |= (fabsf(g.x) <= nb ? near_f64(v, X2h.x, X2l.x, Y2h.x, Y2l.x, Z2h.x, Z2l.x) : f2.x <= ff2) ? 1 : 0;
    if (which & 2)
        n |= (fabsf(g.y) <= nb ? near_f64(v, X2h.y, X2l.y, Y2h.y, Y2l.y, Z2h.y, Z2l.y) : f2.y <= ff2) ? 2 : 0;
    return n;
}

// Near/far test (panel.rs:53-57) of one FP32 panel record at two targets, from e2 = the
// FP32 |x_hi - c_hi|^2 (the far-field doublet's own distance): outside the record's band
// around ff2 (kRec32FF2Band bounds the error of e2 there) that is the f64 decision. A target
// inside it (rare) is decided from the float-float difference, and where that one lies within
// kNearFarBand of ff2, by near_f64. VOTE: every lane of the warp calls it together, and the
// rare branch is taken as one warp-uniform branch.
template <bool VOTE>
__device__ __forceinline__ void near_far2(const float* v, float2 e2, float2 X2h, float2 Y2h, float2 Z2h, float2 X2l,
                                          float2 Y2l, float2 Z2l, bool& n0, bool& n1) {
    const float ff2 = v[31], w = v[kRec32FF2Band];
    n0 = e2.x <= ff2;
    n1 = e2.y <= ff2;
    const float2 d = sub2s(e2, ff2);
    const bool u0 = fabsf(d.x) <= w, u1 = fabsf(d.y) <= w;
    if (VOTE ? __any_sync(0xffffffffu, u0 || u1) : (u0 || u1)) {
        const int n = near_recheck(v, X2h, Y2h, Z2h, X2l, Y2l, Z2l, (u0 ? 1 : 0) | (u1 ? 2 : 0));
        if (u0) n0 = (n & 1) != 0;
        if (u1) n1 = (n & 2) != 0;
    }
}

// Job holding global item `item` of a batched launch: the last job whose first item is
// at or before it (item_begin ascending, jobs[0].item_begin == 0).
__device__ __forceinline__ int find_job(const BsJob* jobs, int n, long long item) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// FP32 panel sweeps: at most 96 registers, five CTAs (20 warps) per SM; this issue-bound
// kernel lost a fifth of its speed at four (98 registers round up to 104 per thread)
template <class R, int T, bool KAHAN, int SYM, bool NEGLECT, bool CHAIN, int TILE_PANELS = 0>
__global__ void __launch_bounds__(kBsThreads, (sizeof(R) == 4 && !CHAIN) ? 5 : 1) k_bs_sweep(const BsArgs a) {
    // panels per shared-memory stage: the precision's default, or a tuned shape (batched sweeps)
    constexpr int TILE = TILE_PANELS ? TILE_PANELS : TileSize<R>::value;
    constexpr int TT = SYM ? 2 * T : T;  // mirrored targets ride along as extra targets
    constexpr bool F32 = sizeof(R) == 4;
    static_assert(!F32 || TT == 2, "the packed FP32 path holds exactly two targets per thread");
    static_assert(!CHAIN || (F32 && !NEGLECT), "chain records: FP32 sweeps without neglect-self only");
    // Stages of panel tiles: three where five CTAs per SM still fit (the 64-panel FP32 tile),
    // else two. A warp runs ahead of the CTA's slowest by up to the stages less one: a stage
    // is refilled by the warp that releases it last, with no CTA barrier per tile (the far-field
    // fast path takes warps through a tile at different speeds).
    constexpr int NS = (TILE * sizeof(PanelRec<R>) <= 12288) ? 3 : 2;
    constexpr int kWarps = kBsThreads / 32;
    __shared__ __align__(128) PanelRec<R> tile[NS][TILE];
    __shared__ __align__(8) uint64_t bar[NS];
    __shared__ unsigned s_done[NS];    // releases of the stage in this launch (kWarps per tile)
    __shared__ unsigned s_issued[NS];  // copies issued into the stage in this launch
    // FP32 panel sweeps (capped at 96 registers): a thread's running sums and compensations (x,
    // y, z sums of its two targets, then their compensations) between tiles. Touched once a
    // tile, they leave the registers to the tile loop. (The chain sweeps keep them in registers.)
    constexpr bool SMEM_ACC = F32 && !CHAIN;
    __shared__ float s_acc[SMEM_ACC ? 12 : 1][kBsThreads];
    __shared__ long long s_item;
    // the item's target tile, source chunk and panel range (read from shared memory where used,
    // so that no register holds them through the tile loop)
    __shared__ long long s_ttile, s_pb, s_pe;
    __shared__ int s_chunk;
    __shared__ int s_timed_out;  // a tile wait of this CTA ran out
    // far-field fast path (FP32 panel sweeps): bounding box of each warp's targets (hi parts)
    __shared__ float s_wbox[kBsThreads / 32][6];
    constexpr bool FAST_FAR = F32 && !CHAIN && !NEGLECT;
    __shared__ BsJob s_job;  // the current item's sweep (one copy per item, by thread 0)

    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0) {
        for (int q = 0; q < NS; ++q) {
            mbar_init(&bar[q], 1);
            s_done[q] = 0;
            s_issued[q] = 0;
        }
        fence_mbar_init();
        s_timed_out = 0;
    }
    __syncthreads();
    uint32_t phases = 0;  // bit q: parity of stage q's phase that the next wait on it waits for
    const long long n_items = a.jobs ? a.jobs[a.n_jobs].item_begin : a.job0.n_ttiles * static_cast<long long>(a.job0.n_chunks);
    constexpr int TM = kBsThreads * T;

    while (true) {
        __syncthreads();  // every thread is done with the previous item's s_item, s_job and tiles
        if (s_timed_out) {
            // A tile wait ran out (every warp has left its tile loop): the launch's results are
            // void. Thread 0 waits, bounded again, for the last copy issued into each stage, so
            // that no copy is in flight into the CTA's shared memory when it exits; the n-th copy
            // into a stage completes its phase n - 1.
            if (tid == 0)
                for (int q = 0; q < NS; ++q)
                    if (s_issued[q] > 0) mbar_wait_bounded(&bar[q], (s_issued[q] - 1u) & 1u, a.err);
            return;
        }
        if (tid == 0) {
            // once a wait of any CTA has run out the launch's results are void: take no more items
            const bool stop = *reinterpret_cast<volatile const int*>(a.err) == kDevTimeout;
            const long long it = stop ? n_items : static_cast<long long>(atomicAdd(a.work_counter, 1ULL));
            s_item = it;
            if (it < n_items) {
                const BsJob& Jt = a.jobs ? a.jobs[find_job(a.jobs, a.n_jobs, it)] : a.job0;
                s_job = Jt;
                const long long local = it - Jt.item_begin;
                // chunk-major order: CTAs running together share a source chunk in L2
                const int chunk = static_cast<int>(local / Jt.n_ttiles);
                s_chunk = chunk;
                s_ttile = local % Jt.n_ttiles;
                const long long pb = Jt.p_begin + static_cast<long long>(chunk) * Jt.chunk_panels;
                s_pb = pb;
                s_pe = min(pb + static_cast<long long>(Jt.chunk_panels), Jt.p_end);
            }
        }
        __syncthreads();
        if (s_item >= n_items) break;
        const BsJob& J = s_job;
        const long long ttile = s_ttile;

        // targets: float-float pairs (FP32) or doubles (FP64 path, lo parts 0)
        R xh[TT], yh[TT], zh[TT], xl[TT], yl[TT], zl[TT];
        bool valid[TT];
        int tw[TT];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            // with the far-field fast path a thread's targets are adjacent (a warp's 64 targets
            // are consecutive points, a compact box); else T rows of the tile apart
            const long long slot = ttile * TM + (FAST_FAR ? static_cast<long long>(tid) * T + t
                                                          : static_cast<long long>(t) * kBsThreads + tid);
            const long long idx = FAST_FAR ? bs_slot_target(J, slot) : slot;
            valid[t] = slot < bs_slots(J) && idx < J.M;
            d3 p = valid[t] ? J.targets[idx] : mk(0, 0, 0);
            tw[t] = (NEGLECT && valid[t]) ? J.target_wing[idx] : -1;
            d3 q[2] = {p, SYM ? mirror(SYM, p) : p};
#pragma unroll
            for (int m = 0; m < (SYM ? 2 : 1); ++m) {
                const int u = t + m * T;
                xh[u] = static_cast<R>(q[m].x);
                yh[u] = static_cast<R>(q[m].y);
                zh[u] = static_cast<R>(q[m].z);
                xl[u] = static_cast<R>(q[m].x - static_cast<double>(xh[u]));
                yl[u] = static_cast<R>(q[m].y - static_cast<double>(yh[u]));
                zl[u] = static_cast<R>(q[m].z - static_cast<double>(zh[u]));
                valid[u] = valid[t];
                tw[u] = tw[t];
            }
        }
        // running sums and compensations; for FP32 lane j of a float2 is target j (s_acc)
        R sx[TT], sy[TT], sz[TT], cx[TT], cy[TT], cz[TT];
        if constexpr (SMEM_ACC) {
#pragma unroll
            for (int q = 0; q < 12; ++q) s_acc[q][tid] = 0.f;
        } else {
#pragma unroll
            for (int t = 0; t < TT; ++t) sx[t] = sy[t] = sz[t] = cx[t] = cy[t] = cz[t] = R(0);
        }
        float2 X2h, Y2h, Z2h, X2l, Y2l, Z2l;
        if constexpr (F32) {
            X2h = make_float2(xh[0], xh[1]); Y2h = make_float2(yh[0], yh[1]); Z2h = make_float2(zh[0], zh[1]);
            X2l = make_float2(xl[0], xl[1]); Y2l = make_float2(yl[0], yl[1]); Z2l = make_float2(zl[0], zl[1]);
        }
        if constexpr (FAST_FAR) {
            // box of the warp's valid targets (both lanes: 64 consecutive target points, compact
            // along a wake row), reduced over the warp by butterflies
            float b6[6] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F};
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (valid[u]) {
                    b6[0] = fminf(b6[0], xh[u]);
                    b6[1] = fminf(b6[1], yh[u]);
                    b6[2] = fminf(b6[2], zh[u]);
                    b6[3] = fmaxf(b6[3], xh[u]);
                    b6[4] = fmaxf(b6[4], yh[u]);
                    b6[5] = fmaxf(b6[5], zh[u]);
                }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const float w = __shfl_xor_sync(0xffffffffu, b6[q], o);
                    b6[q] = q < 3 ? fminf(b6[q], w) : fmaxf(b6[q], w);
                }
            if ((tid & 31) == 0)
#pragma unroll
                for (int q = 0; q < 6; ++q) s_wbox[tid >> 5][q] = b6[q];
            __syncwarp();
        }

        const int ntiles = static_cast<int>((s_pe - s_pb + TILE - 1) / TILE);
        // panels of tile k
        auto tile_panels = [&](int k) {
            return static_cast<int>(min(static_cast<long long>(TILE), s_pe - s_pb - static_cast<long long>(k) * TILE));
        };
        // tile k goes into stage k % NS
        auto issue = [&](int k, int q) {
            const long long p0 = s_pb + static_cast<long long>(k) * TILE;
            const uint32_t bytes = static_cast<uint32_t>(tile_panels(k)) * static_cast<uint32_t>(sizeof(PanelRec<R>));
            uint64_t* b = &bar[q];
            atomicAdd(&s_issued[q], 1u);
            mbar_expect_tx(b, bytes);
            bulk_g2s(&tile[q][0], reinterpret_cast<const PanelRec<R>*>(s_job.panels) + p0, bytes, b);
        };
        if (tid == 0)
            for (int q = 0; q < NS && q < ntiles; ++q) issue(q, q);

        int buf = 0;  // stage of tile k
        for (int k = 0; k < ntiles; ++k, buf = buf + 1 == NS ? 0 : buf + 1) {
            // a wait of another warp ran out: the item's sums are void, and the stages that
            // warp did not release are never refilled
            if (__any_sync(0xffffffffu, *reinterpret_cast<volatile int*>(&s_timed_out) != 0)) break;
            const bool ok = mbar_wait_bounded(&bar[buf], (phases >> buf) & 1u, a.err, a.wait_polls);
            phases ^= 1u << buf;
            // A warp with a lane whose wait ran out leaves the tile alone: its copy may still be
            // landing, and lanes reading a word while it lands can see different values, which
            // would split the warp at the uniform branches, votes and shuffles below.
            if (__any_sync(0xffffffffu, !ok)) {
                if (lane == 0) s_timed_out = 1;
                break;
            }
            const int np = tile_panels(k);
            {
                if constexpr (F32) {
                    float2 TX = bc(0.f), TY = bc(0.f), TZ = bc(0.f);
                    // Far-field fast path, per quarter of the tile (a sub-tile of TILE / 4 panels):
                    // when the box of the sub-tile's panel centres lies farther from the box of the
                    // warp's targets than the sub-tile's largest far-field radius (with a margin well
                    // beyond the FP32 rounding of the per-pair distance), every pair of it is a point
                    // doublet (panel.rs:53-57, 82-96) and the per-pair test below would decide so for
                    // every lane: the warp evaluates the doublets alone, without the test and the
                    // votes. Quarters keep the boxes compact where a tile holds the end of one wing's
                    // row of panels and the start of the next.
                    unsigned far_mask = 0;   // bit q: sub-tile q is all far
                    unsigned zero_mask = 0;  // bit q: sub-tile q holds a zero-strength panel
                    if constexpr (FAST_FAR) {
                        static_assert(TILE % 32 == 0, "the fast path's sub-tiles are 8 lanes x TILE / 32 panels");
                        constexpr int PPL = TILE / 32;  // panels per lane; sub-tile q = lanes 8q .. 8q + 7
                        float c7[7] = {CUDART_INF_F, CUDART_INF_F, CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F, -CUDART_INF_F,
                                       0.f};
                        bool zero = false;  // a zero-strength panel: skipped, so not in the box
#pragma unroll
                        for (int j = 0; j < PPL; ++j) {
                            const int q = PPL * lane + j;
                            if (q < np && tile[buf][q].v[kRec32Gamma] == 0.f) zero = true;
                            else if (q < np) {
                                const float4 c = *reinterpret_cast<const float4*>(&tile[buf][q].v[28]);  // centre hi, ff2
                                c7[0] = fminf(c7[0], c.x);
                                c7[1] = fminf(c7[1], c.y);
                                c7[2] = fminf(c7[2], c.z);
                                c7[3] = fmaxf(c7[3], c.x);
                                c7[4] = fmaxf(c7[4], c.y);
                                c7[5] = fmaxf(c7[5], c.z);
                                c7[6] = fmaxf(c7[6], c.w);
                            }
                        }
#pragma unroll
                        for (int o = 4; o > 0; o >>= 1)
#pragma unroll
                            for (int q = 0; q < 7; ++q) {
                                const float w = __shfl_xor_sync(0xffffffffu, c7[q], o);
                                c7[q] = q < 3 ? fminf(c7[q], w) : fmaxf(c7[q], w);
                            }
                        const float* wb = s_wbox[tid >> 5];
                        // the boxes are of hi parts, each within 2^-24 |x| of its point: the gaps
                        // shrink by both sides' bound before the test (an empty sub-tile's box
                        // gives a gap of 0: not far, and no panels to take)
                        auto gap = [&](int q) {
                            const float m = fmaxf(fmaxf(fabsf(c7[q]), fabsf(c7[q + 3])), fmaxf(fabsf(wb[q]), fabsf(wb[q + 3])));
                            return fmaxf(0.f, fmaxf(c7[q] - wb[q + 3], wb[q] - c7[q + 3]) - 0x1p-23f * m);
                        };
                        const float gx = gap(0), gy = gap(1), gz = gap(2);
                        const unsigned b =
                            __ballot_sync(0xffffffffu, c7[6] < CUDART_INF_F && gx * gx + gy * gy + gz * gz > 1.001f * c7[6]);
                        far_mask = (b & 1u) | ((b >> 7) & 2u) | ((b >> 14) & 4u) | ((b >> 21) & 8u);
                        const unsigned z = __ballot_sync(0xffffffffu, zero);
                        zero_mask = ((z & 0xffu) ? 1u : 0u) | ((z & 0xff00u) ? 2u : 0u) | ((z & 0xff0000u) ? 4u : 0u) |
                                    ((z & 0xff000000u) ? 8u : 0u);
                    }
                    constexpr int NSUB = FAST_FAR ? 4 : 1;
                    constexpr int SUB = TILE / NSUB;
#pragma unroll 1
                    for (int sq = 0; sq < NSUB; ++sq) {
                    const int pa = sq * SUB, pz = min(np, pa + SUB);
                    if ((far_mask >> sq) & 1u) {
                        // lanes of targets past the end compute values that are never stored; four
                        // panels per trip give the scheduler independent chains to interleave, which
                        // it can only do without a branch per panel: a sub-tile with no
                        // zero-strength panel takes every panel
                        if (!((zero_mask >> sq) & 1u)) {
#pragma unroll 4
                            for (int p = pa; p < pz; ++p) {
                                const float* v = reinterpret_cast<const float*>(tile[buf][p].v);
                                const float2 ex = sub2s(X2h, v[28]);
                                const float2 ey = sub2s(Y2h, v[29]);
                                const float2 ez = sub2s(Z2h, v[30]);
                                const float2 e2s = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
                                doublet2(bc(v[35] * v[kRec32Gamma]), v, ex, ey, ez, e2s, TX, TY, TZ);
                            }
                            continue;
                        }
                        // a zero-strength panel must be skipped: only its strength slot is written
                        // (its other fields may hold anything, and 0 times NaN is NaN)
#pragma unroll 4
                        for (int p = pa; p < pz; ++p) {
                            const float* v = reinterpret_cast<const float*>(tile[buf][p].v);
                            const float gam = v[kRec32Gamma];
                            if (gam == 0.f) continue;  // uniform across the CTA
                            const float2 ex = sub2s(X2h, v[28]);
                            const float2 ey = sub2s(Y2h, v[29]);
                            const float2 ez = sub2s(Z2h, v[30]);
                            const float2 e2s = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
                            doublet2(bc(v[35] * gam), v, ex, ey, ez, e2s, TX, TY, TZ);
                        }
                        continue;
                    }
                    for (int p = pa; p < pz; ++p) {
                        const float* v = reinterpret_cast<const float*>(tile[buf][p].v);
                        if constexpr (CHAIN) {  // every pair near-field: the chain's segments
                            if (v[kChainAny] == 0.f) continue;  // uniform across the CTA
                            const float2 ex = add2(sub2s(X2h, v[0]), sub2s(X2l, v[3]));
                            const float2 ey = add2(sub2s(Y2h, v[1]), sub2s(Y2l, v[4]));
                            const float2 ez = add2(sub2s(Z2h, v[2]), sub2s(Z2l, v[5]));
                            float2 ax, ay, az;
                            chain2(v, ex, ey, ez, ax, ay, az);
                            TX = add2(TX, ax);
                            TY = add2(TY, ay);
                            TZ = add2(TZ, az);
                            continue;
                        }
                        const float gam = v[kRec32Gamma];
                        if (gam == 0.f) continue;  // uniform across the CTA
                        // target - centre from the hi parts: the near/far test's first look and the
                        // far-field doublet's (at least ff_ratio panel sizes away), as in the fast
                        // path above; the ring below adds the lo parts
                        float2 ex = sub2s(X2h, v[28]);
                        float2 ey = sub2s(Y2h, v[29]);
                        float2 ez = sub2s(Z2h, v[30]);
                        float2 e2 = bc(0.f);
                        bool n0 = true, n1 = true;
                        if (v[31] != CUDART_INF_F) {  // panel.rs:53-57; uniform per panel
                            e2 = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
                            near_far2<true>(v, e2, X2h, Y2h, Z2h, X2l, Y2l, Z2l, n0, n1);
                        }
                        bool a0 = valid[0], a1 = valid[1];
                        if (NEGLECT) {
                            const int pw = static_cast<int>(v[41]);
                            a0 = a0 && tw[0] != pw;
                            a1 = a1 && tw[1] != pw;
                        }
                        const bool any_near = __any_sync(0xffffffffu, (a0 && n0) || (a1 && n1));
                        const bool any_far = __any_sync(0xffffffffu, (a0 && !n0) || (a1 && !n1));
                        if (any_far) {  // point doublet (panel.rs:82-96), the fast path's arithmetic
                            const float2 e2s = make_float2(n0 ? 1.f : e2.x, n1 ? 1.f : e2.y);
                            const float at = v[35] * gam;
                            const float2 sm = make_float2((a0 && !n0) ? at : 0.f, (a1 && !n1) ? at : 0.f);
                            doublet2(sm, v, ex, ey, ez, e2s, TX, TY, TZ);
                        }
                        if (any_near) {  // vortex ring (panel.rs:99-118)
                            // float-float difference: (x_hi - c_hi) + (x_lo - c_lo)
                            ex = add2(ex, sub2s(X2l, v[32]));
                            ey = add2(ey, sub2s(Y2l, v[33]));
                            ez = add2(ez, sub2s(Z2l, v[34]));
                            float2 ax, ay, az;
                            ring2(v, ex, ey, ez, ax, ay, az);
                            const float g4 = gam * static_cast<float>(kFourPiInv);
                            const float2 gm = make_float2((a0 && n0) ? g4 : 0.f, (a1 && n1) ? g4 : 0.f);
                            TX = fma2(gm, ax, TX);
                            TY = fma2(gm, ay, TY);
                            TZ = fma2(gm, az, TZ);
                        }
                    }
                    }
                    const float txa[2] = {TX.x, TX.y}, tya[2] = {TY.x, TY.y}, tza[2] = {TZ.x, TZ.y};
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        if constexpr (!SMEM_ACC) {
                            if (KAHAN) {
                                two_sum_acc(sx[t], cx[t], txa[t]);
                                two_sum_acc(sy[t], cy[t], tya[t]);
                                two_sum_acc(sz[t], cz[t], tza[t]);
                            } else {
                                sx[t] += txa[t];
                                sy[t] += tya[t];
                                sz[t] += tza[t];
                            }
                        } else {
                            float ax = s_acc[t][tid], ay = s_acc[2 + t][tid], az = s_acc[4 + t][tid];
                            if (KAHAN) {
                                float bx = s_acc[6 + t][tid], by = s_acc[8 + t][tid], bz = s_acc[10 + t][tid];
                                two_sum_acc(ax, bx, txa[t]);
                                two_sum_acc(ay, by, tya[t]);
                                two_sum_acc(az, bz, tza[t]);
                                s_acc[6 + t][tid] = bx;
                                s_acc[8 + t][tid] = by;
                                s_acc[10 + t][tid] = bz;
                            } else {
                                ax += txa[t];
                                ay += tya[t];
                                az += tza[t];
                            }
                            s_acc[t][tid] = ax;
                            s_acc[2 + t][tid] = ay;
                            s_acc[4 + t][tid] = az;
                        }
                    }
                } else {
                    R tx[TT], ty[TT], tz[TT];
#pragma unroll
                    for (int t = 0; t < TT; ++t) tx[t] = ty[t] = tz[t] = R(0);
                    for (int p = 0; p < np; ++p) {
                        const double* v = reinterpret_cast<const double*>(tile[buf][p].v);
                        const double gam = v[kRec64Gamma];
                        if (gam == 0.0) continue;
                        const int pw = NEGLECT ? static_cast<int>(v[26]) : 0;
#pragma unroll
                        for (int t = 0; t < TT; ++t) {
                            if (!valid[t] || (NEGLECT && tw[t] == pw)) continue;
                            d3 u = panel_unit_f64(v, mk(xh[t], yh[t], zh[t]));
                            tx[t] += gam * u.x;
                            ty[t] += gam * u.y;
                            tz[t] += gam * u.z;
                        }
                    }
#pragma unroll
                    for (int t = 0; t < TT; ++t) {
                        sx[t] += tx[t];
                        sy[t] += ty[t];
                        sz[t] += tz[t];
                    }
                }
            }
            // Release the stage: every lane of the warp is done reading it. The warp that
            // releases it last (the kWarps-th release of this tile) refills it with tile k + NS.
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                if (atomicAdd(&s_done[buf], 1u) % kWarps == kWarps - 1 && k + NS < ntiles) {
                    __threadfence_block();
                    issue(k + NS, buf);
                }
            }
        }

        const long long ttile_out = s_ttile;
        const int chunk = s_chunk;
        if constexpr (SMEM_ACC) {
#pragma unroll
            for (int t = 0; t < TT; ++t) {
                sx[t] = s_acc[t][tid];
                sy[t] = s_acc[2 + t][tid];
                sz[t] = s_acc[4 + t][tid];
                cx[t] = s_acc[6 + t][tid];
                cy[t] = s_acc[8 + t][tid];
                cz[t] = s_acc[10 + t][tid];
            }
        }
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const long long slot = ttile_out * TM + (FAST_FAR ? static_cast<long long>(tid) * T + t
                                                              : static_cast<long long>(t) * kBsThreads + tid);
            const long long idx = FAST_FAR ? bs_slot_target(J, slot) : slot;
            if (slot < bs_slots(J) && idx < J.M) {
                d3 u = mk(static_cast<double>(sx[t]) + static_cast<double>(cx[t]),
                          static_cast<double>(sy[t]) + static_cast<double>(cy[t]),
                          static_cast<double>(sz[t]) + static_cast<double>(cz[t]));
                if (SYM) {
                    d3 m = mk(static_cast<double>(sx[T + t]) + static_cast<double>(cx[T + t]),
                              static_cast<double>(sy[T + t]) + static_cast<double>(cy[T + t]),
                              static_cast<double>(sz[T + t]) + static_cast<double>(cz[T + t]));
                    u = sym_correct(SYM, u, m);
                }
                double* o = J.partial + (static_cast<long long>(chunk) * J.M + idx) * 3;
                o[0] = u.x;
                o[1] = u.y;
                o[2] = u.z;
            }
        }
    }
}

// Sums the per-chunk partials in chunk order and adds an optional base velocity.
// Points in [M, M_total) get the base only (update_data.rs:125-141).
__global__ void k_bs_reduce(const double* partial, int n_chunks, long long M, long long M_total, const d3* base, d3* out) {
    long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= M_total) return;
    d3 b = base ? base[i] : mk(0, 0, 0);
    if (i < M) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < n_chunks; ++k) {
            const double* p = partial + (static_cast<long long>(k) * M + i) * 3;
            s0 += p[0];
            s1 += p[1];
            s2 += p[2];
        }
        b.x += s0;
        b.y += s1;
        b.z += s2;
    }
    out[i] = b;
}

// The same reduction when there are many chunks (a few targets against many panels, as the
// control points against the whole wake: 1,200 chunks): one warp per target, the lanes
// over chunks lane, lane + 32, ... in f64, then a fixed-order shuffle tree (deterministic).
// A thread per target would walk the chunks one dependent L2 load after another.
constexpr int kBsReduceWideChunks = 64;  // from this many chunks on
__global__ void k_bs_reduce_wide(const double* partial, int n_chunks, long long M, long long M_total, const d3* base,
                                 d3* out) {
    const long long i = (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= M_total) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    if (i < M) {
#pragma unroll 4
        for (int k = lane; k < n_chunks; k += 32) {
            const double* p = partial + (static_cast<long long>(k) * M + i) * 3;
            s0 += p[0];
            s1 += p[1];
            s2 += p[2];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, o);
            s1 += __shfl_down_sync(0xffffffffu, s1, o);
            s2 += __shfl_down_sync(0xffffffffu, s2, o);
        }
    }
    if (lane == 0) {
        d3 b = base ? base[i] : mk(0, 0, 0);
        b.x += s0;
        b.y += s1;
        b.z += s2;
        out[i] = b;
    }
}

// The same reduction for every job of a batched sweep: block b belongs to the last job whose
// block_begin is at or before it.
__global__ void __launch_bounds__(kBsReduceThreads) k_bs_reduce_jobs(const BsJob* jobs, int n_jobs) {
    const long long b = blockIdx.x;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].block_begin <= b) lo = mid;
        else hi = mid - 1;
    }
    const BsJob& J = jobs[lo];
    const long long i = (b - J.block_begin) * kBsReduceThreads + threadIdx.x;
    if (i >= J.M_total) return;
    d3 v = J.base ? J.base[i] : mk(0, 0, 0);
    if (i < J.M) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < J.n_chunks; ++k) {
            const double* p = J.partial + (static_cast<long long>(k) * J.M + i) * 3;
            s0 += p[0];
            s1 += p[1];
            s2 += p[2];
        }
        v.x += s0;
        v.y += s1;
        v.z += s2;
    }
    J.out[i] = v;
}

// one matrix entry into the f64 and/or split matrix (row c, column j). With a basis (two
// components per entry, the influence matrix of the SimpleIterative solve) the entry is
// projected on the in-plane basis of row c: in FP32 for an FP32-evaluated entry (fp32: its
// components stay single floats, lo parts 0), else in f64.
__device__ inline void store_factor(d3* factors, float* split, int N, const d3* basis, long long id, int c, int j, d3 u,
                                    bool fp32 = false) {
    if (factors) factors[id] = u;
    if (split) {  // hi plane [N][C][stride], then the lo plane
        const int S = si_matrix_stride(N);
        const int C = basis ? 2 : 3;
        double comp[3] = {u.x, u.y, u.z};
        if (basis) {
            const d3 e1 = basis[2 * c], e2 = basis[2 * c + 1];
            if (fp32) {
                const float ux = static_cast<float>(u.x), uy = static_cast<float>(u.y), uz = static_cast<float>(u.z);
                comp[0] = fmaf(ux, static_cast<float>(e1.x), fmaf(uy, static_cast<float>(e1.y), uz * static_cast<float>(e1.z)));
                comp[1] = fmaf(ux, static_cast<float>(e2.x), fmaf(uy, static_cast<float>(e2.y), uz * static_cast<float>(e2.z)));
            } else {
                comp[0] = dot(u, e1);
                comp[1] = dot(u, e2);
            }
        }
        float* r = split + static_cast<long long>(c) * C * S + j;
        const long long lo = static_cast<long long>(C) * N * S;
        for (int q = 0; q < C; ++q) {
            const float2 h = split_f64(comp[q]);
            r[q * S] = h.x;
            r[lo + q * S] = h.y;
        }
    }
}

// frozen_wake.rs:198-249: factors[c][p] = unit velocity of first-row panel p at control point c
__device__ inline void unit_matrix_elem(const PanelRec<double>* row0, const d3* ctrl, int N, int sym, int neglect,
                                        const int* wing_of_line, d3* factors, float* split, const d3* basis,
                                        long long id) {
    if (id >= static_cast<long long>(N) * N) return;
    int c = static_cast<int>(id / N), p = static_cast<int>(id % N);
    d3 u = mk(0, 0, 0);
    if (!(neglect && wing_of_line[c] == wing_of_line[p])) {
        d3 x = ctrl[c];
        u = panel_unit_f64(row0[p].v, x);
        if (sym) u = sym_correct(sym, u, panel_unit_f64(row0[p].v, mirror(sym, x)));
    }
    store_factor(factors, split, N, basis, id, c, p, u);
}

__global__ void k_unit_matrix(const PanelRec<double>* row0, const d3* ctrl, int N, int sym, int neglect,
                              const int* wing_of_line, d3* factors, float* split, const d3* basis) {
    unit_matrix_elem(row0, ctrl, N, sym, neglect, wing_of_line, factors, split, basis,
                     blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

// The same matrix from the FP32 panel records of row 0, two control points per thread as the
// lanes of the sweep's f32x2 arithmetic (the per-pair rule of panel.rs:53-57, vortex ring or
// point doublet, exactly as k_bs_sweep evaluates it). A control point lies on the bound
// vortex of its own panel, where the reference's 1e-10 cut-off decides a segment: that entry
// (c == p) is evaluated in FP64 as in k_unit_matrix. The other entries carry FP32 rounding,
// like the frozen-wake sweep over the rows behind.
__device__ __forceinline__ void split2(double a, double b, float2& h, float2& l) {
    const float ha = static_cast<float>(a), hb = static_cast<float>(b);
    h = make_float2(ha, hb);
    l = make_float2(static_cast<float>(a - static_cast<double>(ha)), static_cast<float>(b - static_cast<double>(hb)));
}
__device__ __forceinline__ void panel_unit2(const float* v, float2 X2h, float2 Y2h, float2 Z2h, float2 X2l, float2 Y2l,
                                            float2 Z2l, float2& ux, float2& uy, float2& uz) {
    float2 ex = sub2s(X2h, v[28]), ey = sub2s(Y2h, v[29]), ez = sub2s(Z2h, v[30]);
    float2 e2 = bc(0.f);
    bool n0 = true, n1 = true;
    if (v[31] != CUDART_INF_F) {
        e2 = fma2(ex, ex, fma2(ey, ey, mul2(ez, ez)));
        near_far2<false>(v, e2, X2h, Y2h, Z2h, X2l, Y2l, Z2l, n0, n1);
    }
    ux = uy = uz = bc(0.f);
    if (!n0 || !n1) {  // point doublet (panel.rs:82-96), unit strength
        const float2 e2s = make_float2(n0 ? 1.f : e2.x, n1 ? 1.f : e2.y);
        doublet2(make_float2(n0 ? 0.f : v[35], n1 ? 0.f : v[35]), v, ex, ey, ez, e2s, ux, uy, uz);
    }
    if (n0 || n1) {  // vortex ring (panel.rs:99-118), unit strength
        ex = add2(ex, sub2s(X2l, v[32]));
        ey = add2(ey, sub2s(Y2l, v[33]));
        ez = add2(ez, sub2s(Z2l, v[34]));
        float2 ax, ay, az;
        ring2(v, ex, ey, ez, ax, ay, az);
        const float g4 = static_cast<float>(kFourPiInv);
        const float2 gm = make_float2(n0 ? g4 : 0.f, n1 ? g4 : 0.f);
        ux = fma2(gm, ax, ux);
        uy = fma2(gm, ay, uy);
        uz = fma2(gm, az, uz);
    }
}

__device__ inline void unit_matrix_f32_elem(const PanelRec<float>* row0_32, const PanelRec<double>* row0, const d3* ctrl,
                                            int N, int sym, int neglect, const int* wing_of_line, d3* factors,
                                            float* split, const d3* basis, long long id) {
    const int pairs = (N + 1) / 2;
    if (id >= static_cast<long long>(pairs) * N) return;
    const int cp = static_cast<int>(id / N), p = static_cast<int>(id % N);
    const int c0 = 2 * cp, c1 = min(c0 + 1, N - 1);  // an odd N repeats the last control point
    const d3 x0 = ctrl[c0], x1 = ctrl[c1];
    float2 Xh, Yh, Zh, Xl, Yl, Zl;
    split2(x0.x, x1.x, Xh, Xl);
    split2(x0.y, x1.y, Yh, Yl);
    split2(x0.z, x1.z, Zh, Zl);
    const float* v = row0_32[p].v;
    float2 ux, uy, uz;
    panel_unit2(v, Xh, Yh, Zh, Xl, Yl, Zl, ux, uy, uz);
    if (sym) {  // symmetry_condition.rs:27-43: the mirrored control points
        float2 mx, my, mz;
        const float2 nXh = mul2(Xh, bc(-1.f)), nXl = mul2(Xl, bc(-1.f)), nYh = mul2(Yh, bc(-1.f)),
                     nYl = mul2(Yl, bc(-1.f)), nZh = mul2(Zh, bc(-1.f)), nZl = mul2(Zl, bc(-1.f));
        if (sym == 1) panel_unit2(v, nXh, Yh, Zh, nXl, Yl, Zl, mx, my, mz);
        else if (sym == 2) panel_unit2(v, Xh, nYh, Zh, Xl, nYl, Zl, mx, my, mz);
        else panel_unit2(v, Xh, Yh, nZh, Xl, Yl, nZl, mx, my, mz);
        if (sym == 1) {
            ux = add2(ux, mul2(mx, bc(-1.f)));
            uy = add2(uy, my);
            uz = add2(uz, mz);
        } else if (sym == 2) {
            ux = add2(ux, mx);
            uy = add2(uy, mul2(my, bc(-1.f)));
            uz = add2(uz, mz);
        } else {
            ux = add2(ux, mx);
            uy = add2(uy, my);
            uz = add2(uz, mul2(mz, bc(-1.f)));
        }
    }
    const float uxa[2] = {ux.x, ux.y}, uya[2] = {uy.x, uy.y}, uza[2] = {uz.x, uz.y};
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const int c = l == 0 ? c0 : c1;
        if (l == 1 && c1 == c0) break;
        d3 u = mk(uxa[l], uya[l], uza[l]);
        bool fp32 = true;
        if (neglect && wing_of_line[c] == wing_of_line[p]) {
            u = mk(0, 0, 0);
        } else if (c == p) {
            const d3 x = ctrl[c];
            u = panel_unit_f64(row0[p].v, x);
            if (sym) u = sym_correct(sym, u, panel_unit_f64(row0[p].v, mirror(sym, x)));
            fp32 = false;
        }
        store_factor(factors, split, N, basis, static_cast<long long>(c) * N + p, c, p, u, fp32);
    }
}

__global__ void k_unit_matrix_f32(const PanelRec<float>* row0_32, const PanelRec<double>* row0, const d3* ctrl, int N,
                                  int sym, int neglect, const int* wing_of_line, d3* factors, float* split,
                                  const d3* basis) {
    unit_matrix_f32_elem(row0_32, row0, ctrl, N, sym, neglect, wing_of_line, factors, split, basis,
                         blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x);
}

constexpr int kUnitMatrixThreads = 128;

// The unit-strength matrices of every case of a batch in one launch (block -> case by a
// binary search over the cases' first blocks, as the other job-list kernels).
__global__ void k_unit_matrix_jobs(const CaseStepJob* jobs, int n) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk_matrix <= static_cast<long long>(blockIdx.x)) lo = mid;
        else hi = mid - 1;
    }
    const CaseStepJob& J = jobs[lo];
    const long long id = (blockIdx.x - J.blk_matrix) * static_cast<long long>(kUnitMatrixThreads) + threadIdx.x;
    const DevModel& m = J.m;
    if (J.row0_32)
        unit_matrix_f32_elem(J.row0_32, J.w.row0_64, m.ctrl, m.N, m.symmetry, m.neglect_self, m.wing_of_line, J.factors,
                             J.split, J.basis, id);
    else
        unit_matrix_elem(J.w.row0_64, m.ctrl, m.N, m.symmetry, m.neglect_self, m.wing_of_line, J.factors, J.split,
                         J.basis, id);
}

long long unit_matrix_blocks(int N, bool fp32) {
    const long long tot = fp32 ? static_cast<long long>((N + 1) / 2) * N : static_cast<long long>(N) * N;
    return (tot + kUnitMatrixThreads - 1) / kUnitMatrixThreads;
}

cudaError_t launch_unit_matrix_jobs(const CaseStepJob* jobs, int n, long long blocks, cudaStream_t s) {
    if (n <= 0 || blocks <= 0) return cudaSuccess;
    k_unit_matrix_jobs<<<static_cast<unsigned>(blocks), kUnitMatrixThreads, 0, s>>>(jobs, n);
    return cudaGetLastError();
}

// Quasi-steady wake: core length and wake vectors (frozen_wake.rs:74-100). One CTA: the
// span line lengths and the wake vectors in parallel (FP64 square roots and divisions are
// slow on this part, so a serial loop over them costs microseconds per line), the mean
// length summed in line order by one thread.
constexpr int kQsPrepThreads = 256;
__global__ void __launch_bounds__(kQsPrepThreads) k_qs_prep(DevModel m, int core_kind, double core_value,
                                                            double wake_length, d3* wake_vec, double* rc_out) {
    const int tid = threadIdx.x;
    for (int k = tid; k < m.Np; k += kQsPrepThreads) wake_vec[k] = normalize(m.felt_span[k]) * wake_length;
    if (core_kind != 0) {
        if (tid == 0) *rc_out = core_kind == 1 ? core_value : 0.0;
        return;
    }
    extern __shared__ double lens[];  // [N]
    for (int i = tid; i < m.N; i += kQsPrepThreads) lens[i] = len(m.span_e[i] - m.span_s[i]);
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int i = 0; i < m.N; ++i) s += lens[i];
        *rc_out = core_value * (s / static_cast<double>(m.N));
    }
}

// Horseshoe influence matrix (frozen_wake.rs:102-128, horseshoe_vortex.rs:23-103):
// factors[c][j] = unit velocity of horseshoe j (bound + start trailing + end trailing) at
// control point c. Horseshoe j of wing w uses wake vectors j + w and j + w + 1.
__global__ void k_horseshoe_matrix(DevModel m, const d3* wake_vec, const double* rc_dev, int sym, d3* factors,
                                   float* split, const d3* basis) {
    long long id = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    const int N = m.N;
    if (id >= static_cast<long long>(N) * N) return;
    int c = static_cast<int>(id / N), j = static_cast<int>(id % N);
    const double rc = *rc_dev;
    const int k = j + m.wing_of_line[j];
    d3 s = m.span_s[j], e = m.span_e[j];
    d3 st0 = s + wake_vec[k], en1 = e + wake_vec[k + 1];
    auto hs = [&](d3 x) {
        d3 u = mk(0, 0, 0);
        u = u + line_unit_f64(s, e, x, rc);
        u = u + line_unit_f64(st0, s, x, rc);
        u = u + line_unit_f64(e, en1, x, rc);
        return u;
    };
    d3 x = m.ctrl[c];
    d3 u = hs(x);
    if (sym) u = sym_correct(sym, u, hs(mirror(sym, x)));
    store_factor(factors, split, N, basis, id, c, j, u);
}

cudaError_t launch_horseshoe_matrix(const DevModel& m, int core_kind, double core_value, double wake_length, d3* wake_vec,
                                    double* rc_dev, int sym, d3* factors, float* split, const d3* basis,
                                    cudaStream_t s) {
    const size_t smem = static_cast<size_t>(m.N) * sizeof(double);
    if (smem > 48 * 1024) {
        cudaError_t a = cudaFuncSetAttribute(k_qs_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (a != cudaSuccess) return a;
    }
    k_qs_prep<<<1, kQsPrepThreads, smem, s>>>(m, core_kind, core_value, wake_length, wake_vec, rc_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    long long tot = static_cast<long long>(m.N) * m.N;
    k_horseshoe_matrix<<<static_cast<unsigned>((tot + 127) / 128), 128, 0, s>>>(m, wake_vec, rc_dev, sym, factors, split,
                                                                               basis);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------
template <class R, int T, bool KAHAN, int SYM, bool NEGLECT, bool CHAIN = false, int TILE_PANELS = 0>
static cudaError_t launch_t(const BsArgs& a, int grid, cudaStream_t s) {
    k_bs_sweep<R, T, KAHAN, SYM, NEGLECT, CHAIN, TILE_PANELS><<<grid, kBsThreads, 0, s>>>(a);
    return cudaGetLastError();
}

// Tile shapes the autotuner may pick for the compensated FP32 panel sweeps without symmetry
// (the batch's sweeps): panels per shared-memory stage. 64 is the default.
constexpr int kTunedTiles[3] = {64, 32, 96};
static bool tuned_tile_variant(int precision, int symmetry, int chain, int tile) {
    return precision == 0 && symmetry == 0 && !chain && (tile == 32 || tile == 96);
}

template <bool KAHAN>
static cudaError_t launch_chain(const BsArgs& a, int grid, cudaStream_t s) {
    switch (a.symmetry) {
        case 0: return launch_t<float, 2, KAHAN, 0, false, true>(a, grid, s);
        case 1: return launch_t<float, 1, KAHAN, 1, false, true>(a, grid, s);
        case 2: return launch_t<float, 1, KAHAN, 2, false, true>(a, grid, s);
        default: return launch_t<float, 1, KAHAN, 3, false, true>(a, grid, s);
    }
}

template <class R, bool KAHAN>
static cudaError_t launch_sym(const BsArgs& a, int grid, cudaStream_t s) {
    if constexpr (KAHAN) {
        if (a.symmetry == 0 && a.tile == 32)
            return a.neglect ? launch_t<R, 2, KAHAN, 0, true, false, 32>(a, grid, s)
                             : launch_t<R, 2, KAHAN, 0, false, false, 32>(a, grid, s);
        if (a.symmetry == 0 && a.tile == 96)
            return a.neglect ? launch_t<R, 2, KAHAN, 0, true, false, 96>(a, grid, s)
                             : launch_t<R, 2, KAHAN, 0, false, false, 96>(a, grid, s);
    }
    if (a.neglect) {
        switch (a.symmetry) {
            case 0: return launch_t<R, 2, KAHAN, 0, true>(a, grid, s);
            case 1: return launch_t<R, 1, KAHAN, 1, true>(a, grid, s);
            case 2: return launch_t<R, 1, KAHAN, 2, true>(a, grid, s);
            default: return launch_t<R, 1, KAHAN, 3, true>(a, grid, s);
        }
    }
    switch (a.symmetry) {
        case 0: return launch_t<R, 2, KAHAN, 0, false>(a, grid, s);
        case 1: return launch_t<R, 1, KAHAN, 1, false>(a, grid, s);
        case 2: return launch_t<R, 1, KAHAN, 2, false>(a, grid, s);
        default: return launch_t<R, 1, KAHAN, 3, false>(a, grid, s);
    }
}

int bs_targets_per_thread(int symmetry) { return symmetry == 0 ? 2 : 1; }
int bs_tile_panels(int precision) { return precision == 2 ? TileSize<double>::value : TileSize<float>::value; }
int bs_tile_panels(int precision, int symmetry, int chain, int tile) {
    return tuned_tile_variant(precision, symmetry, chain, tile) ? tile : bs_tile_panels(precision);
}
int bs_tile_choices(int* tiles, int n) {
    int k = 0;
    for (int t : kTunedTiles)
        if (k < n) tiles[k++] = t;
    return k;
}

static std::atomic<int> g_sweep_wait_polls{-1};

void set_sweep_wait_polls(int polls) { g_sweep_wait_polls.store(polls < 0 ? -1 : polls); }

cudaError_t launch_bs_sweep(const BsArgs& args, int precision, int grid, cudaStream_t s) {
    BsArgs a = args;
    const int polls = g_sweep_wait_polls.load();
    if (polls >= 0) a.wait_polls = polls;
    if (a.chain) {
        if (precision == 2 || a.neglect) return cudaErrorInvalidValue;
        return precision == 1 ? launch_chain<false>(a, grid, s) : launch_chain<true>(a, grid, s);
    }
    if (precision == 2) return launch_sym<double, false>(a, grid, s);
    if (precision == 1) return launch_sym<float, false>(a, grid, s);
    if (!tuned_tile_variant(precision, a.symmetry, a.chain, a.tile)) a.tile = 0;
    return launch_sym<float, true>(a, grid, s);
}

int bs_occupancy_blocks_per_sm(int precision, int symmetry, int neglect, int tile) {
    int nb = 0;
    cudaError_t e;
    if (tuned_tile_variant(precision, symmetry, 0, tile)) {
        if (tile == 32) e = neglect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<float, 2, true, 0, true, false, 32>, kBsThreads, 0)
                                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<float, 2, true, 0, false, false, 32>, kBsThreads, 0);
        else e = neglect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<float, 2, true, 0, true, false, 96>, kBsThreads, 0)
                         : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<float, 2, true, 0, false, false, 96>, kBsThreads, 0);
        return (e != cudaSuccess || nb < 1) ? 1 : nb;
    }
#define SB_OCC(R, T, K, S, NG) \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<R, T, K, S, NG, false>, kBsThreads, 0)
    if (precision == 2) {
        if (symmetry == 0) { if (neglect) SB_OCC(double, 2, false, 0, true); else SB_OCC(double, 2, false, 0, false); }
        else { if (neglect) SB_OCC(double, 1, false, 1, true); else SB_OCC(double, 1, false, 1, false); }
    } else if (precision == 1) {
        if (symmetry == 0) { if (neglect) SB_OCC(float, 2, false, 0, true); else SB_OCC(float, 2, false, 0, false); }
        else { if (neglect) SB_OCC(float, 1, false, 1, true); else SB_OCC(float, 1, false, 1, false); }
    } else {
        if (symmetry == 0) { if (neglect) SB_OCC(float, 2, true, 0, true); else SB_OCC(float, 2, true, 0, false); }
        else { if (neglect) SB_OCC(float, 1, true, 1, true); else SB_OCC(float, 1, true, 1, false); }
    }
#undef SB_OCC
    if (e != cudaSuccess || nb < 1) nb = 1;
    return nb;
}

cudaError_t launch_bs_reduce(const double* partial, int n_chunks, long long M, long long M_total, const d3* base, d3* out,
                             cudaStream_t s) {
    if (M_total <= 0) return cudaSuccess;
    int threads = 256;
    if (n_chunks >= kBsReduceWideChunks) {
        const long long blocks = (M_total * 32 + threads - 1) / threads;
        k_bs_reduce_wide<<<static_cast<unsigned>(blocks), threads, 0, s>>>(partial, n_chunks, M, M_total, base, out);
        return cudaGetLastError();
    }
    long long blocks = (M_total + threads - 1) / threads;
    k_bs_reduce<<<static_cast<unsigned>(blocks), threads, 0, s>>>(partial, n_chunks, M, M_total, base, out);
    return cudaGetLastError();
}

cudaError_t launch_bs_reduce_jobs(const BsJob* jobs, int n_jobs, long long blocks, cudaStream_t s) {
    if (n_jobs <= 0 || blocks <= 0) return cudaSuccess;
    k_bs_reduce_jobs<<<static_cast<unsigned>(blocks), kBsReduceThreads, 0, s>>>(jobs, n_jobs);
    return cudaGetLastError();
}

cudaError_t launch_unit_matrix(const PanelRec<double>* row0, const PanelRec<float>* row0_32, const d3* ctrl, int N,
                               int sym, int neglect, const int* wing_of_line, d3* factors, float* split, const d3* basis,
                               cudaStream_t s) {
    const long long blocks = unit_matrix_blocks(N, row0_32 != nullptr);
    if (row0_32) {
        k_unit_matrix_f32<<<static_cast<unsigned>(blocks), kUnitMatrixThreads, 0, s>>>(row0_32, row0, ctrl, N, sym, neglect,
                                                                                        wing_of_line, factors, split, basis);
        return cudaGetLastError();
    }
    k_unit_matrix<<<static_cast<unsigned>(blocks), kUnitMatrixThreads, 0, s>>>(row0, ctrl, N, sym, neglect, wing_of_line,
                                                                                factors, split, basis);
    return cudaGetLastError();
}

}  // namespace sbgpu
