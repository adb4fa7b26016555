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
#include <cstdio>

#include "sb_device.cuh"
#include "sb_kernels.h"

namespace sbgpu {

// ---------------------------------------------------------------------------------------
// PTX helpers: mbarrier and bulk async copy
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after a fixed number of polls and records kDevTimeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(err, kDevTimeout);
    return false;
}

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

// One FP32 vortex ring (4 segments) at one target, from float-float corners; returns the
// unscaled sum sum_k core_k * kk_k * (r_k x r_{k+1}) (times Gamma / 4 pi gives the velocity).
// r_k = (x_hi - p_hi_k) + (x_lo - p_lo_k); d_k = p_{k+1} - p_k (precomputed per panel).
__device__ __forceinline__ void ring_f32(const float (&ph)[12], const float (&pl)[12], const float (&dx)[4],
                                         const float (&dy)[4], const float (&dz)[4], const float (&il)[4], float rc4,
                                         bool nocore, float xh, float yh, float zh, float xl, float yl, float zl,
                                         float& ax, float& ay, float& az) {
    float rx[4], ry[4], rz[4], rs[4], rl[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        rx[k] = (xh - ph[3 * k]) + (xl - pl[3 * k]);
        ry[k] = (yh - ph[3 * k + 1]) + (yl - pl[3 * k + 1]);
        rz[k] = (zh - ph[3 * k + 2]) + (zl - pl[3 * k + 2]);
        rs[k] = fmaf(rx[k], rx[k], fmaf(ry[k], ry[k], rz[k] * rz[k]));
        rl[k] = rs[k] * rsqrtf(fmaxf(rs[k], 1e-30f));
    }
    ax = 0.f;
    ay = 0.f;
    az = 0.f;
    // The reference's den = l1 l2 (l1 l2 + r1.r2) and its segment distance |r1|^2 - t^2 both
    // cancel catastrophically in FP32 when the target is close to the segment's interior
    // (r1.r2 -> -l1 l2). They are evaluated through exact identities instead:
    //   c = r1 x r2 = d x r1,  l1 l2 + r1.r2 = |c|^2 / (l1 l2 - r1.r2)  (for r1.r2 < 0),
    //   distance^2 to the segment's line = |c|^2 / |d|^2.
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int k1 = (k + 1) & 3;
        const float p = rl[k] * rl[k1];
        const float q = fmaf(rx[k], rx[k1], fmaf(ry[k], ry[k1], rz[k] * rz[k1]));
        const float cx = dy[k] * rz[k] - dz[k] * ry[k];
        const float cy = dz[k] * rx[k] - dx[k] * rz[k];
        const float cz = dx[k] * ry[k] - dy[k] * rx[k];
        const float c2 = fmaf(cx, cx, fmaf(cy, cy, cz * cz));
        // den = B / A without cancellation
        const bool neg = q < 0.f;
        const float A = neg ? p - q : 1.f;
        const float B = neg ? p * c2 : p * (p + q);
        // distance^2 to the segment, clamped to the end points (vortex_line.rs:59-84)
        const float tp = fmaf(rx[k], dx[k], fmaf(ry[k], dy[k], rz[k] * dz[k]));
        float d2 = c2 * il[k];
        d2 = (tp * il[k] > 1.f) ? rs[k1] : d2;
        d2 = (tp < 0.f) ? rs[k] : d2;
        const float core = nocore ? 1.f : d2 * rsqrtf(fmaxf(fmaf(d2, d2, rc4), 1e-37f));
        // closeness cut-off |den| > 1e-10 (vortex_line.rs:35); den >= 0 here
        const bool ok = (B > 1.0e-10f * A) && il[k] > 0.f;
        const float s = ok ? core * __fdividef((rl[k] + rl[k1]) * A, B) : 0.f;
        ax = fmaf(s, cx, ax);
        ay = fmaf(s, cy, ay);
        az = fmaf(s, cz, az);
    }
}

template <class R, int T, bool KAHAN, int SYM, bool NEGLECT>
__global__ void __launch_bounds__(kBsThreads) k_bs_sweep(BsArgs a) {
    constexpr int TILE = TileSize<R>::value;
    constexpr int TT = SYM ? 2 * T : T;  // mirrored targets ride along as extra targets
    constexpr bool F32 = sizeof(R) == 4;
    __shared__ __align__(128) PanelRec<R> tile[2][TILE];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ long long s_item;

    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase0 = 0, phase1 = 0;
    const PanelRec<R>* P = reinterpret_cast<const PanelRec<R>*>(a.panels);
    const long long n_items = a.n_ttiles * static_cast<long long>(a.n_chunks);
    constexpr int TM = kBsThreads * T;

    while (true) {
        if (tid == 0) s_item = atomicAdd(a.work_counter, 1ULL);
        __syncthreads();
        const long long item = s_item;
        __syncthreads();
        if (item >= n_items) break;
        // chunk-major order: CTAs running together share a source chunk in L2
        const int chunk = static_cast<int>(item / a.n_ttiles);
        const long long ttile = item % a.n_ttiles;
        const long long pb = a.p_begin + static_cast<long long>(chunk) * a.chunk_panels;
        const long long pe = min(pb + static_cast<long long>(a.chunk_panels), a.p_end);

        // targets: FP32 as float-float pairs, FP64 as is (the lo parts stay 0)
        R xh[TT], yh[TT], zh[TT], xl[TT], yl[TT], zl[TT];
        bool valid[TT];
        int tw[TT];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            long long idx = ttile * TM + static_cast<long long>(t) * kBsThreads + tid;
            valid[t] = idx < a.M;
            d3 p = valid[t] ? a.targets[idx] : mk(0, 0, 0);
            tw[t] = (NEGLECT && valid[t]) ? a.target_wing[idx] : -1;
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
        R sx[TT], sy[TT], sz[TT], cx[TT], cy[TT], cz[TT];
#pragma unroll
        for (int t = 0; t < TT; ++t) sx[t] = sy[t] = sz[t] = cx[t] = cy[t] = cz[t] = R(0);

        const int ntiles = static_cast<int>((pe - pb + TILE - 1) / TILE);
        auto issue = [&](int k) {
            long long p0 = pb + static_cast<long long>(k) * TILE;
            int np = static_cast<int>(min(static_cast<long long>(TILE), pe - p0));
            uint32_t bytes = static_cast<uint32_t>(np) * static_cast<uint32_t>(sizeof(PanelRec<R>));
            uint64_t* b = &bar[k & 1];
            mbar_expect_tx(b, bytes);
            bulk_g2s(&tile[k & 1][0], P + p0, bytes, b);
        };
        if (tid == 0 && ntiles > 0) issue(0);

        for (int k = 0; k < ntiles; ++k) {
            const int buf = k & 1;
            if (tid == 0 && k + 1 < ntiles) issue(k + 1);
            if (buf == 0) {
                mbar_wait_bounded(&bar[0], phase0, a.err);
                phase0 ^= 1;
            } else {
                mbar_wait_bounded(&bar[1], phase1, a.err);
                phase1 ^= 1;
            }
            const int np = static_cast<int>(min(static_cast<long long>(TILE), pe - (pb + static_cast<long long>(k) * TILE)));

            R tx[TT], ty[TT], tz[TT];
#pragma unroll
            for (int t = 0; t < TT; ++t) tx[t] = ty[t] = tz[t] = R(0);

            for (int p = 0; p < np; ++p) {
                const R* v = tile[buf][p].v;
                const R gam = F32 ? v[kRec32Gamma] : v[kRec64Gamma];
                if (gam == R(0)) continue;  // uniform across the CTA
                R ccx, ccy, ccz, ff2, clx = 0, cly = 0, clz = 0;
                int pw = 0;
                if constexpr (F32) {
                    ccx = v[24]; ccy = v[25]; ccz = v[26]; ff2 = v[27];
                    clx = v[28]; cly = v[29]; clz = v[30];
                    if (NEGLECT) pw = static_cast<int>(v[41]);
                } else {
                    ccx = v[16]; ccy = v[17]; ccz = v[18]; ff2 = v[19];
                    if (NEGLECT) pw = static_cast<int>(v[26]);
                }
                R ex[TT], ey[TT], ez[TT], e2[TT];
                bool nr[TT], act[TT];
                bool my_near = false, my_far = false;
#pragma unroll
                for (int t = 0; t < TT; ++t) {
                    ex[t] = (xh[t] - ccx) + (xl[t] - clx);
                    ey[t] = (yh[t] - ccy) + (yl[t] - cly);
                    ez[t] = (zh[t] - ccz) + (zl[t] - clz);
                    e2[t] = ex[t] * ex[t] + ey[t] * ey[t] + ez[t] * ez[t];
                    nr[t] = e2[t] <= ff2;
                    act[t] = valid[t] && (!NEGLECT || tw[t] != pw);
                    my_near |= act[t] && nr[t];
                    my_far |= act[t] && !nr[t];
                }
                const bool any_near = __any_sync(0xffffffffu, my_near);
                const bool any_far = __any_sync(0xffffffffu, my_far);
                if (any_far) {
                    R nx, ny, nz, at;
                    if constexpr (F32) {
                        nx = v[32]; ny = v[33]; nz = v[34]; at = v[31] * gam;
                    } else {
                        nx = v[20]; ny = v[21]; nz = v[22]; at = v[23] * gam;
                    }
#pragma unroll
                    for (int t = 0; t < TT; ++t) {
                        if (act[t] && !nr[t]) {
                            R h = ex[t] * nx + ey[t] * ny + ez[t] * nz;
                            R h3 = R(3) * h;
                            R s;
                            if constexpr (F32) {
                                float ir = rsqrtf(e2[t]);
                                float ir2 = ir * ir;
                                s = at * (ir2 * ir2 * ir);
                            } else {
                                s = at / (e2[t] * e2[t] * sqrt(e2[t]));
                            }
                            tx[t] += s * (h3 * ex[t] - e2[t] * nx);
                            ty[t] += s * (h3 * ey[t] - e2[t] * ny);
                            tz[t] += s * (h3 * ez[t] - e2[t] * nz);
                        }
                    }
                }
                if (any_near) {
                    if constexpr (F32) {
                        float ph[12], pl[12], il[4], dx[4], dy[4], dz[4];
#pragma unroll
                        for (int i = 0; i < 12; ++i) {
                            ph[i] = v[i];
                            pl[i] = v[12 + i];
                        }
#pragma unroll
                        for (int k2 = 0; k2 < 4; ++k2) {
                            const int n2 = (k2 + 1) & 3;
                            il[k2] = v[36 + k2];
                            dx[k2] = (ph[3 * n2] - ph[3 * k2]) + (pl[3 * n2] - pl[3 * k2]);
                            dy[k2] = (ph[3 * n2 + 1] - ph[3 * k2 + 1]) + (pl[3 * n2 + 1] - pl[3 * k2 + 1]);
                            dz[k2] = (ph[3 * n2 + 2] - ph[3 * k2 + 2]) + (pl[3 * n2 + 2] - pl[3 * k2 + 2]);
                        }
                        const float rc4 = v[40];
                        const bool nocore = v[42] != 0.f;
                        const float g4 = gam * static_cast<float>(kFourPiInv);
#pragma unroll
                        for (int t = 0; t < TT; ++t) {
                            if (act[t] && nr[t]) {
                                float ax, ay, az;
                                ring_f32(ph, pl, dx, dy, dz, il, rc4, nocore, xh[t], yh[t], zh[t], xl[t], yl[t], zl[t],
                                         ax, ay, az);
                                tx[t] = fmaf(g4, ax, tx[t]);
                                ty[t] = fmaf(g4, ay, ty[t]);
                                tz[t] = fmaf(g4, az, tz[t]);
                            }
                        }
                    } else {
#pragma unroll
                        for (int t = 0; t < TT; ++t) {
                            if (act[t] && nr[t]) {
                                d3 u = mk(0, 0, 0);
                                d3 pp[4] = {mk(v[0], v[1], v[2]), mk(v[3], v[4], v[5]), mk(v[6], v[7], v[8]),
                                            mk(v[9], v[10], v[11])};
                                d3 X = mk(xh[t], yh[t], zh[t]);
                                for (int i = 0; i < 4; ++i) u = u + line_unit_f64(pp[i], pp[(i + 1) & 3], X, v[25]);
                                tx[t] += gam * u.x;
                                ty[t] += gam * u.y;
                                tz[t] += gam * u.z;
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < TT; ++t) {
                if (KAHAN) {
                    two_sum_acc(sx[t], cx[t], tx[t]);
                    two_sum_acc(sy[t], cy[t], ty[t]);
                    two_sum_acc(sz[t], cz[t], tz[t]);
                } else {
                    sx[t] += tx[t];
                    sy[t] += ty[t];
                    sz[t] += tz[t];
                }
            }
            __syncthreads();  // the buffer is refilled in the next-but-one tile
        }

#pragma unroll
        for (int t = 0; t < T; ++t) {
            long long idx = ttile * TM + static_cast<long long>(t) * kBsThreads + tid;
            if (idx < a.M) {
                d3 u = mk(static_cast<double>(sx[t]) + static_cast<double>(cx[t]),
                          static_cast<double>(sy[t]) + static_cast<double>(cy[t]),
                          static_cast<double>(sz[t]) + static_cast<double>(cz[t]));
                if (SYM) {
                    d3 m = mk(static_cast<double>(sx[T + t]) + static_cast<double>(cx[T + t]),
                              static_cast<double>(sy[T + t]) + static_cast<double>(cy[T + t]),
                              static_cast<double>(sz[T + t]) + static_cast<double>(cz[T + t]));
                    u = sym_correct(SYM, u, m);
                }
                double* o = a.partial + (static_cast<long long>(chunk) * a.M + idx) * 3;
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

// frozen_wake.rs:198-249: factors[c][p] = unit velocity of first-row panel p at control point c
__global__ void k_unit_matrix(const PanelRec<double>* row0, const d3* ctrl, int N, int sym, int neglect,
                              const int* wing_of_line, d3* factors) {
    long long id = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (id >= static_cast<long long>(N) * N) return;
    int c = static_cast<int>(id / N), p = static_cast<int>(id % N);
    d3 u = mk(0, 0, 0);
    if (!(neglect && wing_of_line[c] == wing_of_line[p])) {
        d3 x = ctrl[c];
        u = panel_unit_f64(row0[p].v, x);
        if (sym) u = sym_correct(sym, u, panel_unit_f64(row0[p].v, mirror(sym, x)));
    }
    factors[id] = u;
}

// Quasi-steady wake: core length and wake vectors (frozen_wake.rs:74-100). One thread.
__global__ void k_qs_prep(DevModel m, int core_kind, double core_value, double wake_length, d3* wake_vec, double* rc_out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double rc = 0.0;
    if (core_kind == 0) {
        double s = 0.0;
        for (int i = 0; i < m.N; ++i) s += len(m.span_e[i] - m.span_s[i]);
        rc = core_value * (s / static_cast<double>(m.N));
    } else if (core_kind == 1) {
        rc = core_value;
    }
    *rc_out = rc;
    for (int k = 0; k < m.Np; ++k) wake_vec[k] = normalize(m.felt_span[k]) * wake_length;
}

// Horseshoe influence matrix (frozen_wake.rs:102-128, horseshoe_vortex.rs:23-103):
// factors[c][j] = unit velocity of horseshoe j (bound + start trailing + end trailing) at
// control point c. Horseshoe j of wing w uses wake vectors j + w and j + w + 1.
__global__ void k_horseshoe_matrix(DevModel m, const d3* wake_vec, const double* rc_dev, int sym, d3* factors) {
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
    factors[id] = u;
}

cudaError_t launch_horseshoe_matrix(const DevModel& m, int core_kind, double core_value, double wake_length, d3* wake_vec,
                                    double* rc_dev, int sym, d3* factors, cudaStream_t s) {
    k_qs_prep<<<1, 32, 0, s>>>(m, core_kind, core_value, wake_length, wake_vec, rc_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    long long tot = static_cast<long long>(m.N) * m.N;
    k_horseshoe_matrix<<<static_cast<unsigned>((tot + 127) / 128), 128, 0, s>>>(m, wake_vec, rc_dev, sym, factors);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------
template <class R, int T, bool KAHAN, int SYM, bool NEGLECT>
static cudaError_t launch_t(const BsArgs& a, int grid, cudaStream_t s) {
    k_bs_sweep<R, T, KAHAN, SYM, NEGLECT><<<grid, kBsThreads, 0, s>>>(a);
    return cudaGetLastError();
}

template <class R, bool KAHAN>
static cudaError_t launch_sym(const BsArgs& a, int grid, cudaStream_t s) {
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

cudaError_t launch_bs_sweep(const BsArgs& a, int precision, int grid, cudaStream_t s) {
    if (precision == 2) return launch_sym<double, false>(a, grid, s);
    if (precision == 1) return launch_sym<float, false>(a, grid, s);
    return launch_sym<float, true>(a, grid, s);
}

int bs_occupancy_blocks_per_sm(int precision, int symmetry, int neglect) {
    int nb = 0;
    cudaError_t e;
#define SB_OCC(R, T, K, S, NG) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bs_sweep<R, T, K, S, NG>, kBsThreads, 0)
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
    long long blocks = (M_total + threads - 1) / threads;
    k_bs_reduce<<<static_cast<unsigned>(blocks), threads, 0, s>>>(partial, n_chunks, M, M_total, base, out);
    return cudaGetLastError();
}

cudaError_t launch_unit_matrix(const PanelRec<double>* row0, const d3* ctrl, int N, int sym, int neglect,
                               const int* wing_of_line, d3* factors, cudaStream_t s) {
    long long tot = static_cast<long long>(N) * N;
    int threads = 128;
    long long blocks = (tot + threads - 1) / threads;
    k_unit_matrix<<<static_cast<unsigned>(blocks), threads, 0, s>>>(row0, ctrl, N, sym, neglect, wing_of_line, factors);
    return cudaGetLastError();
}

}  // namespace sbgpu
