// Warm-start network kernels (sm_103a).
//
// k_mlp_gemm: C[M][N] = A[M][K] B[N][K]^T on the 5th-generation tensor cores. One CTA of
// eight warps owns a 128 x N output tile whose FP32 accumulator lives in tensor memory
// (256 columns allocated with tcgen05.alloc). The operands arrive by TMA: per 64-wide K
// step one thread issues two cp.async.bulk.tensor.2d copies (A: 64 x 128, B: 64 x N BF16)
// into a stage of shared memory in the 128-byte-swizzled K-major layout (one 128-byte row
// per matrix row, 16-byte chunks XOR-ed with the row index mod 8, 8-row atoms 1024 B
// apart), completing on the stage's `full` mbarrier. Two stages run ahead of the tensor
// cores; the same thread waits for a stage, issues four tcgen05.mma.cta_group::1.kind::f16
// (K = 16 each: the descriptor start advances 32 B inside the swizzle atom) and commits to
// the stage's `empty` mbarrier, and refills the stage of the previous step once its MMAs
// have completed, so one step of MMAs is always queued behind the running one. Two CTAs
// fit on an SM (shared memory), so one CTA's epilogue overlaps the other's MMAs. The
// epilogue reads the accumulator with tcgen05.ld (32 lanes x 32 columns per warp and
// instruction; warps w and w + 4 own tensor-memory lanes 32 (w mod 4) .. + 31 = rows and
// half of the columns each) and applies the layer's bias and GELU (forward), the GELU
// derivative (backward), or stores split-K partial sums (weight gradients). Waits are
// bounded: a wait that runs out records kDevTimeout, skips the epilogue, waits (bounded)
// for the copies and MMAs in flight and frees the tensor memory.
//
// The rest are CUDA-core kernels: the width->1 output layer with the MSE loss, input
// packing, deterministic fixed-order reductions, Adam, weight casts, and the batch-side
// feature / candidate / target kernels of the warm start.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "sb_mlp.h"
#include "sb_ptx.cuh"

namespace sbgpu {

namespace {

constexpr int kGemmThreads = 256;  // 8 warps: warps w and w + 4 drain one lane quadrant
constexpr int kKStep = 64;       // one 128-byte swizzle row of BF16
constexpr int kStages = 2;
constexpr uint32_t kSBO = 1024;  // bytes between 8-row atoms
constexpr uint32_t kStageA = kMlpRowTile * kKStep * 2;
constexpr uint32_t kStageB = kMlpWidth * kKStep * 2;
constexpr uint32_t kStage = kStageA + kStageB;
constexpr uint32_t kTmemCols = 256;
static_assert(kStageA % 1024 == 0 && kStage % 1024 == 0, "stages keep the 1024-byte swizzle alignment");

// tcgen05 shared-memory matrix descriptor of a K-major 128-byte-swizzled tile: start
// address (>> 4), leading offset 16 B (unused by this layout), SBO 1024 B (>> 4), version
// 1, layout type 2 (128-byte swizzle), base offset 0 (atoms are 1024-byte aligned).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (1ull << 16) |
           (static_cast<uint64_t>((kSBO >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}

// 2-D tiled TMA copy of the box at (x, y) (x in elements along the contiguous dimension)
// into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 32 consecutive FP32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// GELU with the error function, and its derivative
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ void store_bf16x32(bf16* dst, const float (&v)[32]) {
    uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        __nv_bfloat162 p[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) p[j] = __floats2bfloat162_rn(v[q * 8 + 2 * j], v[q * 8 + 2 * j + 1]);
        d[q] = *reinterpret_cast<uint4*>(p);
    }
}

__global__ void __launch_bounds__(kGemmThreads) k_mlp_gemm(const __grid_constant__ CUtensorMap map_a,
                                                           const __grid_constant__ CUtensorMap map_b, GemmArgs g) {
    extern __shared__ unsigned char dyn[];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ __align__(8) uint64_t empty[kStages];
    __shared__ uint32_t s_tmem;
    __shared__ int s_issued, s_ok;
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(dyn) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kMlpRowTile;
    const int split = blockIdx.y;
    const int k_begin = split * g.k_split;
    const int k_end = min(g.K, k_begin + g.k_split);
    const int nk = (k_end - k_begin) / kKStep;

    if (warp == 0) tmem_alloc(&s_tmem, kTmemCols);
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (tid == 0) {
        const uint32_t idesc = idesc_bf16(kMlpRowTile, g.N);
        const uint32_t tx = kStageA + static_cast<uint32_t>(g.N) * kKStep * 2;
        auto load = [&](int kt) {
            const int s = kt % kStages;
            unsigned char* sa = base + s * kStage;
            mbar_expect_tx(&full[s], tx);
            tma_load_2d(sa, &map_a, k_begin + kt * kKStep, m0, &full[s]);
            tma_load_2d(sa + kStageA, &map_b, k_begin + kt * kKStep, 0, &full[s]);
        };
        int loaded = 0;  // K steps whose copies were issued
        for (; loaded < min(nk, kStages); ++loaded) load(loaded);
        bool ok = true;
        int issued = 0;  // K steps whose MMAs were issued
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % kStages;
            if (!mbar_wait_bounded(&full[s], (kt / kStages) & 1, g.err)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t a_addr = smem_u32(base + s * kStage), b_addr = a_addr + kStageA;
#pragma unroll
            for (int j = 0; j < kKStep / 16; ++j)
                mma_bf16(tmem, smem_desc_sw128(a_addr + j * 32), smem_desc_sw128(b_addr + j * 32), idesc,
                         (kt > 0 || j > 0) ? 1u : 0u);
            mma_commit(&empty[s]);
            issued = kt + 1;
            // refill the stage of step kt - 1 once its MMAs are done (those of step kt stay queued)
            if (kt >= 1 && loaded < nk) {
                const int p = kt - 1;
                if (!mbar_wait_bounded(&empty[p % kStages], (p / kStages) & 1, g.err)) {
                    ok = false;
                    break;
                }
                load(loaded);
                ++loaded;
            }
        }
        // copies issued but never consumed still write shared memory: wait for them
        if (!ok)
            for (int kt = issued; kt < loaded; ++kt) mbar_wait_bounded(&full[kt % kStages], (kt / kStages) & 1, g.err);
        s_issued = issued;
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    const int issued = s_issued;
    // the last commit arrives when every MMA issued before it has completed
    bool done = s_ok && issued == nk && nk > 0;
    if (issued > 0) {
        const int p = issued - 1;
        const bool w = mbar_wait_bounded(&empty[p % kStages], (p / kStages) & 1, g.err);
        done = done && w;
    }
    done = __syncthreads_and(done);
    tc_fence_after();

    if (done) {
        // a warp reads the tensor-memory lanes of its quadrant (warp mod 4); the two warps of
        // a quadrant take half of the columns each
        const int quad = warp & 3, half = warp >> 2;
        const int row = m0 + quad * 32 + lane;
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(quad * 32) << 16);
        const int c_end = (half + 1) * (g.N / 2);
        for (int c0 = half * (g.N / 2); c0 < c_end; c0 += 32) {
            float v[32];
            tmem_ld32(lane_addr + static_cast<uint32_t>(c0), v);
            if (g.mode == kGemmPartial) {
                float4* o = reinterpret_cast<float4*>(g.part_out + (static_cast<long long>(split) * g.M + row) * g.N + c0);
#pragma unroll
                for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                continue;
            }
            if (g.mode == kGemmForward) {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] += g.bias[c0 + j];
                if (g.z_out) {
                    float4* o = reinterpret_cast<float4*>(g.z_out + static_cast<long long>(row) * g.N + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = gelu(v[j]);
            } else {  // backward through the GELU of the layer below
                const float4* zi = reinterpret_cast<const float4*>(g.z_in + static_cast<long long>(row) * g.N + c0);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 z = zi[q];
                    v[4 * q] *= gelu_grad(z.x);
                    v[4 * q + 1] *= gelu_grad(z.y);
                    v[4 * q + 2] *= gelu_grad(z.z);
                    v[4 * q + 3] *= gelu_grad(z.w);
                }
            }
            if (g.h_out) store_bf16x32(g.h_out + static_cast<long long>(row) * g.N + c0, v);
            if (g.hT_out) {
#pragma unroll
                for (int j = 0; j < 32; ++j) g.hT_out[static_cast<long long>(c0 + j) * g.ldt + row] = __float2bfloat16_rn(v[j]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

__global__ void __launch_bounds__(32 * kHeadRowsPerCta) k_mlp_head(HeadArgs a) {
    __shared__ float wacc[kHeadRowsPerCta][kMlpWidth + 2];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r = blockIdx.x * kHeadRowsPerCta + warp;  // < rows_pad
    const int f0 = lane * 8;
    float hv[8];
    {
        const uint4 raw = *reinterpret_cast<const uint4*>(a.h + static_cast<long long>(r) * kMlpWidth + f0);
        const __nv_bfloat162* p = reinterpret_cast<const __nv_bfloat162*>(&raw);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 f = __bfloat1622float2(p[j]);
            hv[2 * j] = f.x;
            hv[2 * j + 1] = f.y;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s = fmaf(hv[j], a.w[f0 + j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float y = s + a.w[kMlpWidth];
    if (!a.target) {
        if (lane == 0 && r < a.rows) a.y[r] = y;
        return;
    }
    const float res = r < a.rows ? y - a.target[r] : 0.f;
    const float dy = 2.f * res * a.inv_n;
    const float4* zp = reinterpret_cast<const float4*>(a.z + static_cast<long long>(r) * kMlpWidth + f0);
    const float4 z0 = zp[0], z1 = zp[1];
    const float zz[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
    float dz[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) dz[j] = dy * a.w[f0 + j] * gelu_grad(zz[j]);
    __nv_bfloat162 pk[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) pk[j] = __floats2bfloat162_rn(dz[2 * j], dz[2 * j + 1]);
    *reinterpret_cast<uint4*>(a.dz + static_cast<long long>(r) * kMlpWidth + f0) = *reinterpret_cast<uint4*>(pk);
#pragma unroll
    for (int j = 0; j < 8; ++j) a.dzT[static_cast<long long>(f0 + j) * a.rows_pad + r] = __float2bfloat16_rn(dz[j]);
#pragma unroll
    for (int j = 0; j < 8; ++j) wacc[warp][f0 + j] = dy * hv[j];
    if (lane == 0) {
        wacc[warp][kMlpWidth] = dy;
        wacc[warp][kMlpWidth + 1] = res * res;
    }
    __syncthreads();
    for (int i = tid; i < kMlpWidth + 2; i += blockDim.x) {
        float t = 0.f;
        for (int w = 0; w < kHeadRowsPerCta; ++w) t += wacc[w][i];
        a.part[static_cast<long long>(blockIdx.x) * (kMlpWidth + 2) + i] = t;
    }
}

__global__ void k_mlp_pack(const float* x, int rows, int n_in, int rows_pad, bf16* X, bf16* XT) {
    const long long id = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (id >= static_cast<long long>(rows_pad) * kMlpInPad) return;
    const int r = static_cast<int>(id / kMlpInPad), c = static_cast<int>(id % kMlpInPad);
    const float v = (r < rows && c < n_in) ? x[static_cast<long long>(r) * n_in + c] : 0.f;
    const bf16 b = __float2bfloat16_rn(v);
    X[id] = b;
    if (XT) XT[static_cast<long long>(c) * rows_pad + r] = b;
}

__global__ void k_mlp_sum_partials(const float* part, int splits, long long n, long long stride, float* out) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    float t = 0.f;
    for (int s = 0; s < splits; ++s) t += part[static_cast<long long>(s) * stride + i];
    out[i] = t;
}

__global__ void __launch_bounds__(256) k_mlp_colsum(const bf16* XT, int rows_pad, float* out) {
    __shared__ float red[256];
    const bf16* row = XT + static_cast<long long>(blockIdx.x) * rows_pad;
    float t = 0.f;
    for (int r = threadIdx.x; r < rows_pad; r += 256) t += __bfloat162float(row[r]);
    red[threadIdx.x] = t;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void k_mlp_adam(float* p, const float* g, float* m, float* v, long long n, float lr_t, float b1, float b2,
                           float eps) {
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

__global__ void k_mlp_cast(const float* W, int out, int in, bf16* Wb, bf16* WbT) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= out * in) return;
    const int o = id / in, i = id % in;
    const bf16 b = __float2bfloat16_rn(W[id]);
    Wb[id] = b;
    if (WbT) WbT[static_cast<long long>(i) * out + o] = b;
}

// ---- batch side ------------------------------------------------------------------------
__device__ inline double geometric_aoa(d3 chord, d3 span_rel, d3 u) {
    const d3 v = u - project(u, span_rel);
    return len(v) > kMinPositive ? signed_angle_between(chord, v, normalize(span_rel)) : 0.0;
}

__global__ void k_batch_features(const FeatJob* jobs, int n_jobs, long long rows, float* feat, double* q_out,
                                 double* g0_out, double* tr_out) {
    const long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (r >= rows) return;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].row0 <= r) lo = mid;
        else hi = mid - 1;
    }
    const FeatJob& J = jobs[lo];
    const int i = static_cast<int>(r - J.row0);
    const int w = J.wing_of_line[i];
    const int ws = J.wing_start[w], we = J.wing_end[w];
    const d3 fs = J.fs[i];
    const double U = len(fs);
    auto qf = [&](int k) { return 0.5 * J.chord_len[k] * len(J.fs[k]); };
    auto gn = [&](int k) {
        const double qk = qf(k);
        return qk > 0.0 ? -J.gamma[k] / qk : 0.0;
    };
    const double q = 0.5 * J.chord_len[i] * U;
    const double g0 = gn(i);
    const double gl = gn(i > ws ? i - 1 : i), gr = gn(i + 1 < we ? i + 1 : i);
    double gm = 0.0;
    for (int k = ws; k < we; ++k) gm += gn(k);
    gm /= static_cast<double>(we - ws);
    const d3 fs_prev = J.hist > 0 ? J.fs_old[i] : fs;
    const double Up = len(fs_prev);
    const double gold = J.hist > 1 ? J.gamma_old[i] : J.gamma[i];
    const double trend = q > 0.0 ? -(J.gamma[i] - gold) / q : 0.0;
    const d3 span_rel = J.span_e[i] - J.span_s[i];
    const double a_t = geometric_aoa(J.chord[i], span_rel, fs);
    const double a_p = geometric_aoa(J.chord[i], span_rel, fs_prev);
    const int P = we - ws;
    const double sp = P > 1 ? static_cast<double>(i - ws) / static_cast<double>(P - 1) : 0.5;
    const double k = static_cast<double>(J.steps);
    const double Wd = static_cast<double>(J.W > 0 ? J.W : 1);
    float* f = feat + r * kMlpFeatures;
    f[0] = static_cast<float>(g0);
    f[1] = static_cast<float>(gl);
    f[2] = static_cast<float>(gr);
    f[3] = static_cast<float>(gm);
    f[4] = static_cast<float>(10.0 * trend);
    f[5] = static_cast<float>(Up > 0.0 ? 10.0 * (U / Up - 1.0) : 0.0);
    f[6] = static_cast<float>(a_t);
    f[7] = static_cast<float>(10.0 * (a_t - a_p));
    f[8] = static_cast<float>(2.0 * sp - 1.0);
    f[9] = static_cast<float>(J.chord_len[i] / 10.0);
    f[10] = static_cast<float>(J.S > 1 ? static_cast<double>(w) / (J.S - 1) : 0.0);
    f[11] = static_cast<float>(J.S / 6.0);
    f[12] = static_cast<float>(P / 96.0);
    f[13] = static_cast<float>(J.W / 400.0);
    f[14] = static_cast<float>(fmin(k, Wd) / Wd);
    f[15] = static_cast<float>(1.0 / (1.0 + k));
    q_out[r] = q;
    g0_out[r] = g0;
    tr_out[r] = trend;
    // history for the next step (only this thread touches row i of these two arrays)
    J.gamma_old[i] = J.gamma[i];
    J.fs_old[i] = fs;
}

__global__ void k_batch_candidate(const float* y, const double* q, const double* g0, const double* tr, long long rows,
                                  double* cand_ex, double* cand_net) {
    const long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (r >= rows) return;
    const double e = g0[r] + tr[r];
    cand_ex[r] = -e * q[r];
    cand_net[r] = -(e + static_cast<double>(y[r])) * q[r];
}

__global__ void k_batch_targets(const double* gamma_new, const double* q, const double* g0, const double* tr,
                                long long rows, float* t) {
    const long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (r >= rows) return;
    t[r] = q[r] > 0.0 ? static_cast<float>(-gamma_new[r] / q[r] - g0[r] - tr[r]) : 0.f;
}

unsigned blocks_for(long long n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace

size_t mlp_gemm_smem_bytes() { return kStages * static_cast<size_t>(kStage) + 1024; }

cudaError_t configure_mlp_gemm() {
    return cudaFuncSetAttribute(k_mlp_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(mlp_gemm_smem_bytes()));
}

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver
// library); null when the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// Row-major BF16 matrix [rows][cols] with leading dimension ld, copied in boxes of 64
// columns x box_rows rows into 128-byte-swizzled shared memory.
bool encode_bf16_map(CUtensorMap* map, const bf16* ptr, long long rows, long long cols, long long ld, int box_rows) {
    const auto encode = tensor_map_encoder();
    if (!encode) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * sizeof(bf16)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(kKStep), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t elem[2] = {1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(ptr), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launch_mlp_gemm(const GemmArgs& g, cudaStream_t s) {
    // TMA: 16-byte aligned bases and row strides; every box lies inside its matrix
    if (g.M <= 0 || g.M % kMlpRowTile || g.K <= 0 || g.K % kKStep || g.k_split <= 0 || g.k_split % kKStep ||
        (g.N != 64 && g.N != 128 && g.N != 256) || g.lda % 8 || g.ldb % 8 || g.lda < g.K || g.ldb < g.K ||
        reinterpret_cast<uintptr_t>(g.A) % 16 || reinterpret_cast<uintptr_t>(g.B) % 16)
        return cudaErrorInvalidValue;
    CUtensorMap ma, mb;
    if (!encode_bf16_map(&ma, g.A, g.M, g.K, g.lda, kMlpRowTile) || !encode_bf16_map(&mb, g.B, g.N, g.K, g.ldb, g.N))
        return cudaErrorInvalidValue;
    const int splits = (g.K + g.k_split - 1) / g.k_split;
    k_mlp_gemm<<<dim3(g.M / kMlpRowTile, splits), kGemmThreads, mlp_gemm_smem_bytes(), s>>>(ma, mb, g);
    return cudaGetLastError();
}

cudaError_t launch_mlp_head(const HeadArgs& a, cudaStream_t s) {
    if (a.rows_pad % kHeadRowsPerCta) return cudaErrorInvalidValue;
    k_mlp_head<<<a.rows_pad / kHeadRowsPerCta, 32 * kHeadRowsPerCta, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mlp_pack(const float* x, int rows, int n_in, int rows_pad, bf16* X, bf16* XT, cudaStream_t s) {
    const long long n = static_cast<long long>(rows_pad) * kMlpInPad;
    k_mlp_pack<<<blocks_for(n, 256), 256, 0, s>>>(x, rows, n_in, rows_pad, X, XT);
    return cudaGetLastError();
}

cudaError_t launch_mlp_sum_partials(const float* part, int splits, long long n, long long stride, float* out,
                                    cudaStream_t s) {
    k_mlp_sum_partials<<<blocks_for(n, 256), 256, 0, s>>>(part, splits, n, stride, out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_colsum(const bf16* XT, int n_out, int rows_pad, float* out, cudaStream_t s) {
    k_mlp_colsum<<<n_out, 256, 0, s>>>(XT, rows_pad, out);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* p, const float* g, float* m, float* v, long long n, float lr_t, float b1, float b2,
                            float eps, cudaStream_t s) {
    k_mlp_adam<<<blocks_for(n, 256), 256, 0, s>>>(p, g, m, v, n, lr_t, b1, b2, eps);
    return cudaGetLastError();
}

cudaError_t launch_mlp_cast(const float* W, int out, int in, bf16* Wb, bf16* WbT, cudaStream_t s) {
    k_mlp_cast<<<blocks_for(static_cast<long long>(out) * in, 256), 256, 0, s>>>(W, out, in, Wb, WbT);
    return cudaGetLastError();
}

cudaError_t launch_batch_features(const FeatJob* jobs, int n_jobs, long long rows, float* feat, double* q, double* g0,
                                  double* tr, cudaStream_t s) {
    if (rows <= 0 || n_jobs <= 0) return cudaSuccess;
    k_batch_features<<<blocks_for(rows, 128), 128, 0, s>>>(jobs, n_jobs, rows, feat, q, g0, tr);
    return cudaGetLastError();
}

cudaError_t launch_batch_candidate(const float* y, const double* q, const double* g0, const double* tr, long long rows,
                                   double* cand_ex, double* cand_net, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    k_batch_candidate<<<blocks_for(rows, 256), 256, 0, s>>>(y, q, g0, tr, rows, cand_ex, cand_net);
    return cudaGetLastError();
}

cudaError_t launch_batch_targets(const double* gamma_new, const double* q, const double* g0, const double* tr,
                                 long long rows, float* target, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    k_batch_targets<<<blocks_for(rows, 256), 256, 0, s>>>(gamma_new, q, g0, tr, rows, target);
    return cudaGetLastError();
}

}  // namespace sbgpu
