// Allocation-free variant of the standalone Biot-Savart sweep (sb_panel_sweep).
//
// Who needs it: callers that may not allocate device memory while they run — for example a
// co-simulation master stepping the lifting line in real time (the FMU's do_step), where
// allocation after initialisation is forbidden, or a host framework whose pool manager owns
// all of the GPU's memory. They pass inputs and outputs in device memory they already own;
// the sweep's scratch (panel records, per-chunk partial sums, the work counter and the error
// word) lives in one file-scope device array of fixed size that every GPU which loads this
// library holds until the process exits.
//
// The array is shared by every call on a device and keeps the last call's contents: the work
// counter and the error word are cleared on every call, the records and partial sums are
// fully rewritten. Calls that overlap on the GPU (two streams, or two host threads) race on
// it and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address, so the entry point resolves the
// address once per device, with that device current, by cudaGetSymbolAddress (set-up on the
// first call). A context reset (cudaDeviceReset) reloads the module and can move the array,
// so the resolved address is kept together with the identity of the context it belongs to
// and resolved again when the device's current context has changed.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/stormbird_gb300.h"
#include "sb_device.cuh"
#include "sb_kernels.h"

namespace {

using namespace sbgpu;

constexpr long long kMaxPanels = SB_NO_ALLOC_MAX_PANELS;
constexpr long long kMaxTargets = SB_NO_ALLOC_MAX_TARGETS;
constexpr size_t kRecordBytes = static_cast<size_t>(kMaxPanels) * sizeof(PanelRec<float>);  // 3 MiB
constexpr size_t kPartialBytes = static_cast<size_t>(4) << 20;                            // 4 MiB
constexpr size_t kControlBytes = 256;  // work counter + error word
constexpr size_t kScratchBytes = kRecordBytes + kPartialBytes + kControlBytes;

static __device__ __align__(256) unsigned char g_sweep_scratch[kScratchBytes];

// Resolved address of g_sweep_scratch per device, and the id of the context it was resolved in.
struct Resolved {
    unsigned long long ctx_id = 0;
    unsigned char* addr = nullptr;
};
std::mutex g_mu;
Resolved g_resolved[256];

int fail(int code, const std::string& m) {
    report_error(code, m);  // sb_last_error / sb_last_status
    return code;
}

int ok() {
    report_error(SB_OK, "");
    return SB_OK;
}

// Id of the calling thread's current context (cuCtxGetId, unique for the life of the
// process), through the runtime's driver entry points; 0 when it cannot be read.
unsigned long long current_context_id() {
    static const auto fns = [] {
        std::pair<PFN_cuCtxGetCurrent_v4000, PFN_cuCtxGetId_v12000> f{nullptr, nullptr};
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.first = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.second = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
        return f;
    }();
    if (!fns.first || !fns.second) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (fns.first(&ctx) != CUDA_SUCCESS || !ctx || fns.second(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// The caller's current device, restored when the call returns.
struct RestoreDevice {
    int dev = -1;
    RestoreDevice() {
        if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    }
    ~RestoreDevice() {
        if (dev >= 0) cudaSetDevice(dev);
    }
};

}  // namespace

extern "C" int sb_panel_sweep_no_alloc(int device, const double* corners, const double* strengths,
                                       const double* core_lengths, size_t n_panels, double far_field_ratio,
                                       int symmetry, const double* targets, size_t n_targets, double* velocities,
                                       void* stream) {
    if ((n_panels && (!corners || !strengths || !core_lengths)) || (n_targets && (!targets || !velocities)))
        return fail(SB_ERR_NULL_ARG, "null argument");
    if (symmetry < 0 || symmetry > 3) return fail(SB_ERR_SIZE, "symmetry must be 0..3");
    if (static_cast<long long>(n_panels) > kMaxPanels || static_cast<long long>(n_targets) > kMaxTargets)
        return fail(SB_ERR_SIZE, "sb_panel_sweep_no_alloc handles at most " + std::to_string(kMaxPanels) +
                                     " panels and " + std::to_string(kMaxTargets) + " targets per call (got " +
                                     std::to_string(n_panels) + " panels, " + std::to_string(n_targets) + " targets)");
    if (device < 0 || device >= 256) return fail(SB_ERR_SIZE, "device ordinal out of range");
    if (n_targets == 0) return ok();
    RestoreDevice restore;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(SB_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    unsigned char* base = nullptr;
    {
        // set-up, once per device (again after a context reset), with that device current
        std::lock_guard<std::mutex> lk(g_mu);
        Resolved& r = g_resolved[device];
        const unsigned long long id = current_context_id();
        if (!r.addr || id == 0 || id != r.ctx_id) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_sweep_scratch);
            if (e != cudaSuccess || !p)
                return fail(SB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            r.addr = static_cast<unsigned char*>(p);
            r.ctx_id = id;
        }
        base = r.addr;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PanelRec<float>* rec = reinterpret_cast<PanelRec<float>*>(base);
    double* partial = reinterpret_cast<double*>(base + kRecordBytes);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(base + kRecordBytes + kPartialBytes);
    int* err = reinterpret_cast<int*>(base + kRecordBytes + kPartialBytes + 16);
    const long long P = static_cast<long long>(n_panels), M = static_cast<long long>(n_targets);

    auto check = [&](cudaError_t x, const char* what) {
        if (x != cudaSuccess) {
            fail(SB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(x));
            return false;
        }
        return true;
    };
    if (!check(cudaMemsetAsync(err, 0, sizeof(int), st), "clear error word")) return SB_ERR_CUDA;
    if (P == 0) {
        if (!check(launch_bs_reduce(nullptr, 0, 0, M, nullptr, reinterpret_cast<d3*>(velocities), st), "reduce"))
            return SB_ERR_CUDA;
        return check(cudaStreamSynchronize(st), "sweep") ? ok() : SB_ERR_CUDA;
    }
    if (!check(launch_panels_from_corners(corners, strengths, core_lengths, P, far_field_ratio, rec, nullptr, st),
               "panel records"))
        return SB_ERR_CUDA;

    // work decomposition: target tiles x source chunks, the chunks limited by the partial-sum space
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (sms < 1) sms = 1;
    const int T = bs_targets_per_thread(symmetry);
    const long long TM = static_cast<long long>(kBsThreads) * T;
    const long long n_ttiles = (M + TM - 1) / TM;
    const int tile = bs_tile_panels(0);
    const long long slots = static_cast<long long>(sms) * bs_occupancy_blocks_per_sm(0, symmetry, 0);
    const long long cap_chunks = std::max<long long>(1, static_cast<long long>(kPartialBytes / sizeof(double)) / (M * 3));
    long long nc = (4 * slots + n_ttiles - 1) / n_ttiles;
    nc = std::min(std::max<long long>(nc, 1), std::min(cap_chunks, (P + tile - 1) / tile));
    long long chunk = (P + nc - 1) / nc;
    chunk = std::max<long long>(tile, ((chunk + tile - 1) / tile) * tile);
    const int n_chunks = static_cast<int>((P + chunk - 1) / chunk);

    BsArgs a;
    a.job0.panels = rec;
    a.job0.p_begin = 0;
    a.job0.p_end = P;
    a.job0.targets = reinterpret_cast<const d3*>(targets);
    a.job0.M = M;
    a.job0.chunk_panels = static_cast<int>(chunk);
    a.job0.n_chunks = n_chunks;
    a.job0.n_ttiles = n_ttiles;
    a.job0.partial = partial;
    a.work_counter = counter;
    a.err = err;
    a.symmetry = symmetry;
    const int grid = static_cast<int>(std::max<long long>(1, std::min(slots, n_ttiles * n_chunks)));
    if (!check(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st), "clear work counter")) return SB_ERR_CUDA;
    if (!check(launch_bs_sweep(a, 0, grid, st), "Biot-Savart sweep")) return SB_ERR_CUDA;
    if (!check(launch_bs_reduce(partial, n_chunks, M, M, nullptr, reinterpret_cast<d3*>(velocities), st), "reduce"))
        return SB_ERR_CUDA;
    int herr = 0;
    if (!check(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st), "read error word")) return SB_ERR_CUDA;
    if (!check(cudaStreamSynchronize(st), "sweep")) return SB_ERR_CUDA;
    if (herr == kDevTimeout) return fail(SB_ERR_TIMEOUT, "a bounded device-side wait ran out");
    return ok();
}
