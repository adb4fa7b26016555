// Warm-start network: host side and the sb_mlp_* C ABI.
//
// A multilayer perceptron with kMlpHidden hidden layers of width kMlpWidth (GELU) and one
// output, trained by mean-squared error with Adam. Parameters are kept in FP32 (the master
// copy the optimizer updates) and cast to BF16 for the tensor-core GEMMs after every update
// (row-major W for the forward pass, W^T for the input gradients). Activations are BF16;
// every GEMM accumulates in FP32. The flat parameter order is
//   W1 [256][64] (input columns >= n_in stay zero), b1 [256],
//   W2 [256][256], b2, W3, b3, W4, b4, w_out [256], b_out [1].
// Every reduction (split-K weight gradients, bias sums, output-layer partials) runs in a
// fixed order, so a training step is deterministic.
#include <cmath>
#include <cstring>
#include <vector>

#include "sb_mlp.h"
#include "sim_core.hpp"

using namespace sbgpu;

struct sb_mlp {
    int device = 0;
    int n_in = 0;
    cudaStream_t stream = nullptr;
    long long off_W[kMlpHidden] = {0}, off_b[kMlpHidden] = {0}, off_out = 0, n_params = 0;
    int in_dim[kMlpHidden] = {0};
    DevBuf<float> params, grads, adam_m, adam_v;
    DevBuf<bf16> Wb[kMlpHidden], WbT[kMlpHidden];
    int cap = 0;   // rows the activation buffers hold (multiple of 128)
    bool cap_train = false;
    DevBuf<bf16> X0, X0T, H[kMlpHidden], HT[kMlpHidden], DZ[kMlpHidden], DZT[kMlpHidden];
    DevBuf<float> Z[kMlpHidden], part, head_part, loss;
    DevBuf<float> y_tmp, t_tmp;
    DevBuf<int> err;
    PinnedBuf<float> h_loss;
    PinnedBuf<int> h_err;
    int adam_step = 0;
    int splits = 1;

    ~sb_mlp() {
        if (stream) cudaStreamDestroy(stream);
    }

    void build(int dev, int n_inputs, unsigned long long seed) {
        if (n_inputs < 1 || n_inputs > kMlpInPad) raise(SB_ERR_SIZE, "the network takes 1 to 64 inputs");
        device = dev;
        n_in = n_inputs;
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        long long at = 0;
        for (int l = 0; l < kMlpHidden; ++l) {
            in_dim[l] = l == 0 ? kMlpInPad : kMlpWidth;
            off_W[l] = at;
            at += static_cast<long long>(kMlpWidth) * in_dim[l];
            off_b[l] = at;
            at += kMlpWidth;
        }
        off_out = at;
        at += kMlpWidth + 1;
        n_params = at;
        // He-uniform initialisation from a seeded splitmix64 stream, biases zero
        std::vector<float> p(static_cast<size_t>(n_params), 0.f);
        unsigned long long s = seed;
        auto next = [&]() {
            s += 0x9E3779B97F4A7C15ull;
            unsigned long long z = s;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
        };
        for (int l = 0; l < kMlpHidden; ++l) {
            const int fan_in = l == 0 ? n_in : kMlpWidth;
            const double a = std::sqrt(6.0 / fan_in);
            for (int o = 0; o < kMlpWidth; ++o)
                for (int i = 0; i < in_dim[l]; ++i) {
                    const double u = next();
                    if (l == 0 && i >= n_in) continue;
                    p[static_cast<size_t>(off_W[l] + static_cast<long long>(o) * in_dim[l] + i)] =
                        static_cast<float>((2.0 * u - 1.0) * a);
                }
        }
        const double ao = std::sqrt(3.0 / kMlpWidth);
        for (int i = 0; i < kMlpWidth; ++i) p[static_cast<size_t>(off_out + i)] = static_cast<float>((2.0 * next() - 1.0) * ao);
        params.upload(p);
        grads.alloc(n_params);
        adam_m.alloc(n_params);
        adam_v.alloc(n_params);
        ck(cudaMemset(grads.p, 0, n_params * sizeof(float)), "memset");
        ck(cudaMemset(adam_m.p, 0, n_params * sizeof(float)), "memset");
        ck(cudaMemset(adam_v.p, 0, n_params * sizeof(float)), "memset");
        for (int l = 0; l < kMlpHidden; ++l) {
            Wb[l].alloc(static_cast<size_t>(kMlpWidth) * in_dim[l]);
            if (l > 0) WbT[l].alloc(static_cast<size_t>(kMlpWidth) * in_dim[l]);
        }
        loss.alloc(1);
        err.alloc(1);
        ck(cudaMemset(err.p, 0, sizeof(int)), "memset");
        h_loss.alloc(1);
        h_err.alloc(1);
        ck(configure_mlp_gemm(), "GEMM shared-memory limit");
        cast_weights(stream);
        ck(cudaStreamSynchronize(stream), "mlp build");
    }

    void cast_weights(cudaStream_t s) {
        for (int l = 0; l < kMlpHidden; ++l)
            ck(launch_mlp_cast(params.p + off_W[l], kMlpWidth, in_dim[l], Wb[l].p, l > 0 ? WbT[l].p : nullptr, s),
               "weight cast");
    }

    static int pad_rows(long long rows) {
        return static_cast<int>(((rows + kMlpRowTile - 1) / kMlpRowTile) * kMlpRowTile);
    }

    // Activation buffers for `rows` rows (allocation: call outside any stream capture).
    void ensure(long long rows, bool train) {
        const int need = pad_rows(std::max<long long>(rows, 1));
        if (need <= cap && (!train || cap_train)) return;
        const int c = std::max(need, cap);
        const size_t w = static_cast<size_t>(c) * kMlpWidth;
        X0.alloc(static_cast<size_t>(c) * kMlpInPad);
        for (int l = 0; l < kMlpHidden; ++l) {
            H[l].alloc(w);
            Z[l].alloc(train ? w : 0);
            HT[l].alloc(train ? w : 0);
            DZ[l].alloc(train ? w : 0);
            DZT[l].alloc(train ? w : 0);
        }
        X0T.alloc(train ? static_cast<size_t>(c) * kMlpInPad : 0);
        head_part.alloc(train ? static_cast<size_t>(c / kHeadRowsPerCta) * (kMlpWidth + 2) : 0);
        // split-K over the batch rows for the weight gradients: about one wave of CTAs
        splits = std::max(1, std::min(c / 64, 76));
        part.alloc(train ? static_cast<size_t>(splits) * kMlpWidth * kMlpWidth : 0);
        y_tmp.alloc(static_cast<size_t>(c));
        cap = c;
        cap_train = train;
    }

    GemmArgs gemm(const bf16* A, long long lda, const bf16* B, long long ldb, int M, int N, int K, int mode) const {
        GemmArgs g;
        g.A = A;
        g.lda = lda;
        g.B = B;
        g.ldb = ldb;
        g.M = M;
        g.N = N;
        g.K = K;
        g.k_split = K;
        g.mode = mode;
        g.err = err.p;
        return g;
    }

    // Forward pass over rows of x [rows][n_in] (device). Inference writes y [rows]; training
    // (target != nullptr) keeps what the backward pass needs.
    void forward(const float* x, long long rows, float* y, const float* target, cudaStream_t s) {
        const bool train = target != nullptr;
        const int R = pad_rows(rows);
        ck(launch_mlp_pack(x, static_cast<int>(rows), n_in, R, X0.p, train ? X0T.p : nullptr, s), "pack inputs");
        const bf16* in = X0.p;
        long long ld = kMlpInPad;
        for (int l = 0; l < kMlpHidden; ++l) {
            GemmArgs g = gemm(in, ld, Wb[l].p, in_dim[l], R, kMlpWidth, in_dim[l], kGemmForward);
            g.bias = params.p + off_b[l];
            g.z_out = train ? Z[l].p : nullptr;
            g.h_out = H[l].p;
            g.hT_out = train ? HT[l].p : nullptr;
            g.ldt = R;
            ck(launch_mlp_gemm(g, s), "forward GEMM");
            in = H[l].p;
            ld = kMlpWidth;
        }
        HeadArgs h;
        h.h = H[kMlpHidden - 1].p;
        h.z = train ? Z[kMlpHidden - 1].p : nullptr;
        h.w = params.p + off_out;
        h.target = target;
        h.rows = static_cast<int>(rows);
        h.rows_pad = R;
        h.y = y;
        h.dz = train ? DZ[kMlpHidden - 1].p : nullptr;
        h.dzT = train ? DZT[kMlpHidden - 1].p : nullptr;
        h.part = train ? head_part.p : nullptr;
        h.inv_n = 1.f / static_cast<float>(std::max<long long>(rows, 1));
        ck(launch_mlp_head(h, s), "output layer");
    }

    // Gradients of the mean squared error into `grads` (after a training forward pass).
    void backward(long long rows, cudaStream_t s) {
        const int R = pad_rows(rows);
        const int nh = R / kHeadRowsPerCta;
        // output layer: dw_out, db_out and the loss from the per-CTA partials
        ck(launch_mlp_sum_partials(head_part.p, nh, kMlpWidth + 1, kMlpWidth + 2, grads.p + off_out, s),
           "head gradient");
        ck(launch_mlp_sum_partials(head_part.p + kMlpWidth + 1, nh, 1, kMlpWidth + 2, loss.p, s), "loss");
        for (int l = kMlpHidden - 1; l >= 0; --l) {
            // dW_l = dZ_l^T X_{l-1}: M = 256 outputs, N = inputs, K = rows (split)
            const bf16* XT = l == 0 ? X0T.p : HT[l - 1].p;
            GemmArgs g = gemm(DZT[l].p, R, XT, R, kMlpWidth, in_dim[l], R, kGemmPartial);
            int ks = ((R / splits + 63) / 64) * 64;
            if (ks < 64) ks = 64;
            g.k_split = ks;
            g.part_out = part.p;
            ck(launch_mlp_gemm(g, s), "weight-gradient GEMM");
            const int ns = (R + ks - 1) / ks;
            const long long nw = static_cast<long long>(kMlpWidth) * in_dim[l];
            ck(launch_mlp_sum_partials(part.p, ns, nw, nw, grads.p + off_W[l], s), "weight-gradient reduce");
            ck(launch_mlp_colsum(DZT[l].p, kMlpWidth, R, grads.p + off_b[l], s), "bias gradient");
            if (l > 0) {
                // dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1})
                GemmArgs b = gemm(DZ[l].p, kMlpWidth, WbT[l].p, kMlpWidth, R, kMlpWidth, kMlpWidth, kGemmBackward);
                b.z_in = Z[l - 1].p;
                b.h_out = DZ[l - 1].p;
                b.hT_out = DZT[l - 1].p;
                b.ldt = R;
                ck(launch_mlp_gemm(b, s), "input-gradient GEMM");
            }
        }
    }

    void check_err(cudaStream_t s) {
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, s), "D2H status");
        ck(cudaStreamSynchronize(s), "mlp");
        if (h_err.p[0] != kDevOk) {
            ck(cudaMemset(err.p, 0, sizeof(int)), "memset");
            raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out in the network kernels");
        }
    }

    double read_loss(cudaStream_t s) {
        ck(cudaMemcpyAsync(h_loss.p, loss.p, sizeof(float), cudaMemcpyDeviceToHost, s), "D2H loss");
        check_err(s);
        return static_cast<double>(h_loss.p[0]);
    }

    void adam(float lr, cudaStream_t s) {
        adam_step += 1;
        const double b1 = 0.9, b2 = 0.999;
        const double lr_t = lr * std::sqrt(1.0 - std::pow(b2, adam_step)) / (1.0 - std::pow(b1, adam_step));
        ck(launch_mlp_adam(params.p, grads.p, adam_m.p, adam_v.p, n_params, static_cast<float>(lr_t),
                           static_cast<float>(b1), static_cast<float>(b2), 1e-8f, s),
           "adam");
        cast_weights(s);
    }
};

namespace sbhost {
int mlp_inputs(const sb_mlp* m) { return m->n_in; }
void mlp_reserve(sb_mlp* m, long long rows) { m->ensure(rows, m->cap_train); }
void mlp_forward_async(sb_mlp* m, const float* x, long long rows, float* y, cudaStream_t s) {
    m->forward(x, rows, y, nullptr, s);
}
void mlp_check(sb_mlp* m) {
    ck(cudaDeviceSynchronize(), "network");
    m->check_err(m->stream);
}
}  // namespace sbhost

namespace {
int null_arg() {
    report_error(SB_ERR_NULL_ARG, "null argument");
    return SB_ERR_NULL_ARG;
}
}  // namespace

extern "C" {

sb_mlp* sb_mlp_new(int device, int n_inputs, unsigned long long seed) {
    std::unique_ptr<sb_mlp> m(new sb_mlp());
    if (guard([&] { m->build(device, n_inputs, seed); }) != SB_OK) return nullptr;
    return m.release();
}

void sb_mlp_free(sb_mlp* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    delete m;
}

int sb_mlp_num_params(const sb_mlp* m, size_t* n) {
    if (!m || !n) return null_arg();
    *n = static_cast<size_t>(m->n_params);
    return SB_OK;
}

int sb_mlp_get_params(sb_mlp* m, float* p, size_t n) {
    if (!m || !p) return null_arg();
    return guard([&] {
        if (static_cast<long long>(n) != m->n_params) raise(SB_ERR_SIZE, "parameter count mismatch");
        ck(cudaMemcpyAsync(p, m->params.p, n * sizeof(float), cudaMemcpyDeviceToHost, m->stream), "D2H");
        ck(cudaStreamSynchronize(m->stream), "sync");
    });
}

int sb_mlp_set_params(sb_mlp* m, const float* p, size_t n) {
    if (!m || !p) return null_arg();
    return guard([&] {
        if (static_cast<long long>(n) != m->n_params) raise(SB_ERR_SIZE, "parameter count mismatch");
        ck(cudaMemcpyAsync(m->params.p, p, n * sizeof(float), cudaMemcpyHostToDevice, m->stream), "H2D");
        m->cast_weights(m->stream);
        ck(cudaStreamSynchronize(m->stream), "sync");
    });
}

int sb_mlp_forward(sb_mlp* m, const float* x_dev, size_t rows, float* y_dev) {
    if (!m || (rows && (!x_dev || !y_dev))) return null_arg();
    if (rows == 0) return SB_OK;
    return guard([&] {
        m->ensure(static_cast<long long>(rows), m->cap_train);
        order_after_caller(m->stream);
        m->forward(x_dev, static_cast<long long>(rows), y_dev, nullptr, m->stream);
        m->check_err(m->stream);
    });
}

int sb_mlp_gradients(sb_mlp* m, const float* x_dev, const float* target_dev, size_t rows, float* grads_host,
                     double* loss) {
    if (!m || !x_dev || !target_dev || !grads_host) return null_arg();
    if (rows == 0) {
        report_error(SB_ERR_SIZE, "no rows");
        return SB_ERR_SIZE;
    }
    return guard([&] {
        m->ensure(static_cast<long long>(rows), true);
        order_after_caller(m->stream);
        m->forward(x_dev, static_cast<long long>(rows), m->y_tmp.p, target_dev, m->stream);
        m->backward(static_cast<long long>(rows), m->stream);
        ck(cudaMemcpyAsync(grads_host, m->grads.p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost, m->stream),
           "D2H gradients");
        const double l = m->read_loss(m->stream);
        if (loss) *loss = l / static_cast<double>(rows);
    });
}

int sb_mlp_train_step(sb_mlp* m, const float* x_dev, const float* target_dev, size_t rows, float learning_rate,
                      double* loss) {
    if (!m || !x_dev || !target_dev) return null_arg();
    if (rows == 0) {
        report_error(SB_ERR_SIZE, "no rows");
        return SB_ERR_SIZE;
    }
    return guard([&] {
        m->ensure(static_cast<long long>(rows), true);
        order_after_caller(m->stream);
        m->forward(x_dev, static_cast<long long>(rows), m->y_tmp.p, target_dev, m->stream);
        m->backward(static_cast<long long>(rows), m->stream);
        m->adam(learning_rate, m->stream);
        // the inputs are read by the time the call returns (the caller may reuse them)
        if (loss) *loss = m->read_loss(m->stream) / static_cast<double>(rows);
        else m->check_err(m->stream);
    });
}

}  // extern "C"
