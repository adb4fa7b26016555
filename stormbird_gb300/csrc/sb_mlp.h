// Kernels of the warm-start network (k_mlp.cu): a multilayer perceptron with BF16
// weights and activations on the tensor cores (tcgen05, FP32 accumulation in tensor
// memory), its training kernels, and the batch-side feature and candidate kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sb_device.cuh"

namespace sbgpu {

constexpr int kMlpWidth = 256;     // hidden width
constexpr int kMlpHidden = 4;      // hidden layers
constexpr int kMlpInPad = 64;      // input features padded to one K tile
constexpr int kMlpRowTile = 128;   // rows per GEMM tile (tcgen05 M)
constexpr int kMlpFeatures = 16;   // features per panel built by the batch

using bf16 = __nv_bfloat16;

// C[M][N] = A[M][K] * B[N][K]^T with A and B row-major BF16 (K contiguous), FP32 accumulate.
// M a multiple of 128, N in {64, 128, 256}, K a multiple of 64 (split over gridDim.y in
// chunks of k_split).
enum GemmMode : int {
    kGemmForward = 0,   // z = acc + bias; h = gelu(z) -> h_out (row-major), hT_out (transposed)
    kGemmBackward = 1,  // dz = acc * gelu'(z_in) -> h_out (row-major), hT_out (transposed)
    kGemmPartial = 2,   // part_out[split][M][N] = acc
};
struct GemmArgs {
    const bf16* A = nullptr;
    long long lda = 0;
    const bf16* B = nullptr;
    long long ldb = 0;
    int M = 0, N = 0, K = 0, k_split = 0;
    int mode = 0;
    const float* bias = nullptr;
    float* z_out = nullptr;   // [M][N] or nullptr
    bf16* h_out = nullptr;    // [M][N] or nullptr
    bf16* hT_out = nullptr;   // [N][ldt] or nullptr
    long long ldt = 0;
    const float* z_in = nullptr;
    float* part_out = nullptr;
    int* err = nullptr;
};
size_t mlp_gemm_smem_bytes();
// Raises the GEMM kernel's dynamic shared-memory limit (once, before any stream capture).
cudaError_t configure_mlp_gemm();
cudaError_t launch_mlp_gemm(const GemmArgs& g, cudaStream_t s);

// Output layer (width -> 1) on the CUDA cores. Inference: y[r] = h[r] . w + w[width].
// Training (target != nullptr): MSE residuals, dz of the last hidden layer (row-major and
// transposed) and per-CTA partials [grid][width + 2] of (dw, db, sum of squared residuals).
struct HeadArgs {
    const bf16* h = nullptr;
    const float* z = nullptr;
    const float* w = nullptr;   // [width + 1]
    const float* target = nullptr;
    int rows = 0, rows_pad = 0;
    float* y = nullptr;
    bf16* dz = nullptr;
    bf16* dzT = nullptr;
    float* part = nullptr;
    float inv_n = 0.f;
};
constexpr int kHeadRowsPerCta = 8;
cudaError_t launch_mlp_head(const HeadArgs& a, cudaStream_t s);

// Input packing: x [rows][n_in] f32 -> X [rows_pad][64] BF16 (zero padded) and, when XT is
// not null, its transpose [64][rows_pad].
cudaError_t launch_mlp_pack(const float* x, int rows, int n_in, int rows_pad, bf16* X, bf16* XT, cudaStream_t s);
// out[i] = sum over s < splits of part[s * stride + i], i < n, in split order.
cudaError_t launch_mlp_sum_partials(const float* part, int splits, long long n, long long stride, float* out,
                                    cudaStream_t s);
// out[o] = sum over r < rows_pad of XT[o][r] (bias gradients from a transposed dz), o < n_out.
cudaError_t launch_mlp_colsum(const bf16* XT, int n_out, int rows_pad, float* out, cudaStream_t s);
// Adam update of n parameters (bias-corrected step sizes precomputed on the host).
cudaError_t launch_mlp_adam(float* p, const float* g, float* m, float* v, long long n, float lr_t, float b1, float b2,
                            float eps, cudaStream_t s);
// W [out][in] f32 -> Wb [out][in] BF16 and, when WbT is not null, WbT [in][out].
cudaError_t launch_mlp_cast(const float* W, int out, int in, bf16* Wb, bf16* WbT, cudaStream_t s);

// ---- batch side ----------------------------------------------------------------------
// One case of a batch, for the per-panel features of the warm start.
struct FeatJob {
    const d3* fs = nullptr;          // [N] freestream at the control points, this step
    const double* gamma = nullptr;   // [N] previous solution
    double* gamma_old = nullptr;     // [N] solution of the step before (updated in place)
    d3* fs_old = nullptr;            // [N] freestream of the previous step (updated in place)
    const d3* chord = nullptr;       // [N] global chord vectors
    const d3* span_s = nullptr;
    const d3* span_e = nullptr;
    const double* chord_len = nullptr;
    const int* wing_of_line = nullptr;
    const int* wing_start = nullptr;
    const int* wing_end = nullptr;
    int N = 0, S = 0, W = 0, steps = 0;
    int hist = 0;                    // steps whose history this job's arrays hold (0, 1 or 2):
                                     // fs_old is read from 1, gamma_old from 2
    long long row0 = 0;              // first row of the case in the batch arrays
};
// Per panel, with q = chord |U| / 2 and the lift-coefficient-like variable g = -Gamma / q:
// feat [rows][kMlpFeatures], q, g0 = g of the previous solution and tr = its change over
// the previous step (zero before two solutions exist), the linear-extrapolation baseline.
cudaError_t launch_batch_features(const FeatJob* jobs, int n_jobs, long long rows, float* feat, double* q, double* g0,
                                  double* tr, cudaStream_t s);
// cand_ex = -(g0 + tr) q: extrapolation in time; cand_net = -(g0 + tr + y) q: plus the
// network's correction y
cudaError_t launch_batch_candidate(const float* y, const double* q, const double* g0, const double* tr, long long rows,
                                   double* cand_ex, double* cand_net, cudaStream_t s);
// target = -gamma_new / q - g0 - tr: the correction the network is trained to predict
cudaError_t launch_batch_targets(const double* gamma_new, const double* q, const double* g0, const double* tr,
                                 long long rows, float* target, cudaStream_t s);

}  // namespace sbgpu

// The network as the batch uses it (mlp_host.cu).
struct sb_mlp;
namespace sbhost {
int mlp_inputs(const sb_mlp* m);
// Buffers for `rows` inference rows (allocates: call outside any stream capture).
void mlp_reserve(sb_mlp* m, long long rows);
// y [rows] = network(x [rows][inputs]) enqueued on s (no synchronisation).
void mlp_forward_async(sb_mlp* m, const float* x, long long rows, float* y, cudaStream_t s);
// Throws when a bounded wait in the network's kernels ran out (synchronises the device).
void mlp_check(sb_mlp* m);
}  // namespace sbhost
