// Batched execution of independent lifting-line cases: the sb_batch_* functions of the C ABI.
//
// A batch owns one simulation handle per case (each built from its own setup JSON, with any
// sail count, panel count and wake length) and steps them all together. Per step:
//   1. one host->device copy of every case's freestream (one contiguous buffer) and of the
//      step's sweep work lists;
//   2. the per-case kernels before solving (geometry, wake advection, panels), spread over a
//      pool of forked streams so that small cases run side by side;
//   3. ONE persistent sweep launch for the frozen-wake sweeps of all cases and ONE for all
//      roll-up sweeps: every (case, source chunk, target tile) item sits in one work list,
//      costliest items first, taken from one atomic counter (k_bs_sweep with a job list);
//   4. the per-case solves and force kernels on the pool streams, then one gather kernel
//      that packs every case's circulation and force summary for one device->host copy.
// With a warm-start network attached, the per-panel features of every case, the network's
// forward pass and the candidate initial solutions (linear extrapolation of the solution in
// time plus the network's correction) run on the main stream between 2 and 4;
// each case's solve starts from the plain start, the extrapolation or the network's
// candidate, whichever has the lowest residual (k_solve_si), and the change of the
// solution beyond the extrapolation is kept as a training target.
// After three steps (when the step's kernel arguments stop changing except for the wake
// buffer parity) the whole step is captured into a CUDA graph per parity and replayed; the
// work lists are refreshed through the graph's copy node from pinned host memory.
//
// Work decomposition: each sweep's source chunk size is fixed per case by a target item
// size (total steady-state pairs / (persistent grid x waves)), so items are of similar
// cost across cases; `waves` and the CTAs per SM of the persistent grid come from the
// autotuner (sb_batch_autotune), which times the batch's own roll-up sweep for each
// candidate and keeps the best per workload bucket for the life of the process.
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>

#include "batch_access.hpp"
#include "sb_mlp.h"
#include "sim_core.hpp"

namespace {

constexpr int kPoolStreams = 16;
constexpr int kMaxChunksPerJob = 64;

// summary record of one case after a step
struct GatherJob {
    const double* out = nullptr;  // the case's output block
    long long fsum = 0, msum = 0, residual = 0, iterations = 0, converged = 0;
    int N = 0;
    const int* err = nullptr;
    const double* scalars = nullptr;  // solver scalars ([4]: start taken)
    double* gamma_dst = nullptr;
    double* summary_dst = nullptr;
};

// One CTA per case: circulation and SB_BATCH_SUMMARY summary values into the compact buffer.
__global__ void k_gather(const GatherJob* jobs) {
    const GatherJob& g = jobs[blockIdx.x];
    for (int i = threadIdx.x; i < g.N; i += blockDim.x) g.gamma_dst[i] = g.out[i];
    if (threadIdx.x == 0) {
        double* s = g.summary_dst;
        for (int k = 0; k < 3; ++k) {
            s[k] = g.out[g.fsum + k];
            s[3 + k] = g.out[g.msum + k];
        }
        s[6] = g.out[g.residual];
        s[7] = g.out[g.iterations];
        s[8] = g.out[g.converged];
        s[9] = static_cast<double>(*g.err);
        s[10] = g.scalars[4];
    }
}

// Tuned parameters of the batched sweeps.
struct Tuning {
    int waves = 8;          // items per persistent CTA the item size aims at
    int blocks_per_sm = 0;  // persistent CTAs per SM (0: the occupancy limit)
    int tile = 0;           // panels per shared-memory stage of the compensated FP32 sweeps (0: default)
    int order = 0;          // item schedule: 0 the costliest case's items first, 1 case order
};

// Process-wide tuning results per workload bucket.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, Tuning> g_tune_cache;

}  // namespace

struct sb_batch {
    int device = 0;
    int sms = 1;
    int precision = 0;
    std::vector<std::unique_ptr<sb_sim>> cases;
    std::vector<long long> line_off, fs_off;
    long long N_total = 0, nfs_total = 0;
    bool any_dynamic = false;

    cudaStream_t main = nullptr;
    cudaStream_t pool[kPoolStreams] = {nullptr};
    cudaEvent_t ev_fork[3] = {nullptr}, ev_join[3][kPoolStreams] = {{nullptr}};
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;

    DevBuf<d3> fs_all;
    PinnedBuf<double> h_fs_all;
    DevBuf<double> gamma_all;
    DevBuf<double> compact;  // [N_total] circulation, then [cases][SB_BATCH_SUMMARY]
    PinnedBuf<double> h_compact;
    DevBuf<GatherJob> gather_jobs;
    // quasi-steady cases with the Linearized solver: one launch per plan shape and step
    // (group g: clusters of 2^g CTAs; g = 0 one CTA per case)
    struct LinGroup {
        LinPlan plan;
        int n = 0;
        DevBuf<SolveJob> jobs;
    };
    static constexpr int kLinGroups = 5;
    LinGroup lin_groups[kLinGroups];
    // SimpleIterative solves: one launch per cluster size (1, 4, 8 CTAs, solve_cluster_size),
    // a cluster per case; the job list is refilled every step from pinned memory, since it
    // names the wake buffer of the step's parity
    struct SiGroup {
        int cluster = 0, rows_per_thread = 1;
        std::vector<int> cases;
        long long off = 0;
    };
    static constexpr int kSiGroups = 6;  // cluster size 1, 4, 8 x rows per thread 1, 4
    SiGroup si_groups[kSiGroups];
    long long si_entries = 0;
    std::vector<char> si_batched;  // per case: its solve runs in a k_solve_si_jobs launch
    PinnedBuf<SolveJob> h_si_jobs;
    DevBuf<SolveJob> d_si_jobs;
    // forces of every case, one launch (refilled each step: step parameters can change)
    PinnedBuf<ForceJob> h_force_jobs;
    DevBuf<ForceJob> d_force_jobs;
    // geometry, wake update, unit-strength matrix and chain records of the dynamic cases past
    // their first step: one launch per kind for all of them (refilled each step: the jobs
    // name the step's wake buffers and time step)
    std::vector<char> case_batched;  // per case, in the current step
    PinnedBuf<CaseStepJob> h_case_jobs;
    DevBuf<CaseStepJob> d_case_jobs;
    int n_case_jobs = 0;
    long long blk_advect = 0, blk_panels = 0, blk_matrix = 0, blk_chain = 0;

    // Sweep work lists: group = (sweep kind, symmetry, neglect); one launch each.
    struct Group {
        int kind = 0;  // 0 frozen-wake sweep, 1 roll-up sweep
        int sym = 0, neglect = 0;
        int chain = 0;  // sources are chain records (shared-segment roll-up)
        std::vector<int> cases;           // case of each job, costliest items first
        int tile = 64;                    // panels per shared-memory stage of this group's launch
        std::vector<int> chunk;           // panels per source chunk of each job
        std::vector<long long> part_off;  // offset of each job's partial sums
        std::vector<long long> block_off; // first reduce block of each job
        long long reduce_blocks = 0;
        long long job_off = 0;            // first entry in the job staging buffer
        int grid = 1;
        long long items = 0;              // items in the current step
    };
    std::vector<Group> groups;
    Tuning tuning;
    bool tuned = false;
    double tune_best_ms = 0.0;
    int tune_candidates = 0;
    long long job_entries = 0;
    PinnedBuf<BsJob> h_jobs;
    DevBuf<BsJob> d_jobs;
    DevBuf<double> partial;
    DevBuf<unsigned long long> counters;
    DevBuf<int> err;
    PinnedBuf<int> h_err;

    // warm start: 0 off, 1 network candidates, 2 features and targets only (training data)
    sb_mlp* mlp = nullptr;
    int warm_mode = 0;
    double warm_margin = 0.5;  // SolveBuffers::second_margin of every case
    DevBuf<float> w_feat, w_y, w_target;
    DevBuf<double> w_q, w_g0, w_tr, w_cand_ex, w_cand, w_gamma_old;
    DevBuf<d3> w_fs_old;
    PinnedBuf<FeatJob> h_feat;
    DevBuf<FeatJob> d_feat;
    // per case, the steps whose freestream and solution w_fs_old / w_gamma_old hold (capped at
    // 2): a case's own step count says nothing about them after a loaded state or a mode change
    std::vector<int> warm_hist;

    // freestream from per-case wind models: [cases][time, ship velocity] staged per step
    bool has_wind = false;
    DevBuf<double> wind_steps;
    PinnedBuf<double> h_wind_steps;
    // controller measurements [3 * N_total] and per-wing force/moment totals (CompleteSailModel sweeps)
    DevBuf<double> ctrl_in;
    PinnedBuf<double> h_ctrl_in;
    PinnedBuf<double> h_wing_totals;

    bool use_graph = true;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    double graph_dt = 0.0;
    int graph_precision = -1;
    int graph_wind = -1;
    int steps = 0;
    double last_ms = 0.0;
    long long last_pairs = 0;  // panel-target pairs of the last step's sweeps

    ~sb_batch() {
        cudaSetDevice(device);
        if (main) cudaStreamSynchronize(main);
        drop_graphs();
        cases.clear();
        for (auto& e : ev_fork) if (e) cudaEventDestroy(e);
        for (auto& r : ev_join) for (auto& e : r) if (e) cudaEventDestroy(e);
        if (ev_t0) cudaEventDestroy(ev_t0);
        if (ev_t1) cudaEventDestroy(ev_t1);
        for (auto& s : pool) if (s) cudaStreamDestroy(s);
        if (main) cudaStreamDestroy(main);
    }

    void drop_graphs() {
        for (auto& g : graph) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
    }

    // ------------------------------------------------------------------ construction
    void build(const char* const* jsons, size_t n, int dev) {
        device = dev;
        if (n == 0) raise(SB_ERR_SIZE, "a batch needs at least one case");
        for (size_t i = 0; i < n; ++i) {
            if (!jsons[i]) raise(SB_ERR_NULL_ARG, "setup JSON of case " + std::to_string(i) + " is NULL");
            std::unique_ptr<sb_sim> s(new sb_sim());
            try {
                s->build(jsons[i], dev);
            } catch (const SbFail& e) {
                raise(e.code, "case " + std::to_string(i) + ": " + e.msg);
            }
            cases.push_back(std::move(s));
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        sms = num_sms(device);
        ck(cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto& s : pool) ck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto& e : ev_fork) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        for (auto& r : ev_join) for (auto& e : r) ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreate(&ev_t0), "cudaEventCreate");
        ck(cudaEventCreate(&ev_t1), "cudaEventCreate");

        // contiguous freestream and circulation; every case works on its slice
        for (auto& c : cases) {
            line_off.push_back(N_total);
            fs_off.push_back(nfs_total);
            N_total += c->N;
            nfs_total += c->nfs;
            any_dynamic = any_dynamic || c->dynamic;
        }
        fs_all.alloc(nfs_total);
        h_fs_all.alloc(static_cast<size_t>(nfs_total) * 3);
        gamma_all.alloc(N_total);
        ck(cudaMemset(gamma_all.p, 0, N_total * sizeof(double)), "memset");
        const size_t ncomp = static_cast<size_t>(N_total) + cases.size() * SB_BATCH_SUMMARY;
        compact.alloc(ncomp);
        ck(cudaMemset(compact.p, 0, ncomp * sizeof(double)), "memset");
        h_compact.alloc(ncomp);
        std::memset(h_compact.p, 0, ncomp * sizeof(double));
        std::vector<GatherJob> gj;
        for (size_t i = 0; i < cases.size(); ++i) {
            sb_sim& c = *cases[i];
            c.fs_p = fs_all.p + fs_off[i];
            c.gamma_p = gamma_all.p + line_off[i];
            c.stream = pool[i % kPoolStreams];
            GatherJob g;
            g.out = c.out.p;
            g.fsum = c.L.fsum;
            g.msum = c.L.msum;
            g.residual = c.L.residual;
            g.iterations = c.L.iterations;
            g.converged = c.L.converged;
            g.N = c.N;
            g.err = c.err.p;
            g.scalars = c.scalars.p;
            g.gamma_dst = compact.p + line_off[i];
            g.summary_dst = compact.p + N_total + static_cast<long long>(i) * SB_BATCH_SUMMARY;
            gj.push_back(g);
        }
        gather_jobs.upload(gj);
        std::vector<SolveJob> lj[kLinGroups];
        for (size_t i = 0; i < cases.size(); ++i)
            if (cases[i]->linearized_quasi_steady()) {
                const LinPlan p = linearized_plan(cases[i]->N);
                int g = 0;
                while ((1 << g) < p.cluster) ++g;
                lin_groups[g].plan.cluster = p.cluster;
                lin_groups[g].plan.smem = std::max(lin_groups[g].plan.smem, p.smem);
                lj[g].push_back(cases[i]->linearized_job());
            }
        for (int g = 0; g < kLinGroups; ++g) {
            lin_groups[g].n = static_cast<int>(lj[g].size());
            if (!lj[g].empty()) lin_groups[g].jobs.upload(lj[g]);
        }
        si_batched.assign(cases.size(), 0);
        for (size_t i = 0; i < cases.size(); ++i) {
            const sb_sim& c = *cases[i];
            if (c.solver_kind != 0 || c.solve.start_with_linearized) continue;
            const int CS = solve_cluster_size(c.N);
            if ((c.N + CS - 1) / CS > 1024) continue;  // too many rows per CTA: the single path reports it
            const int rpt = si_rows_per_thread(c.N);
            const int g = (CS == 1 ? 0 : (CS == 4 ? 1 : 2)) + (rpt == 1 ? 0 : 3);
            si_groups[g].cluster = CS;
            si_groups[g].rows_per_thread = rpt;
            si_groups[g].cases.push_back(static_cast<int>(i));
            si_batched[i] = 1;
        }
        for (auto& g : si_groups) {
            g.off = si_entries;
            si_entries += static_cast<long long>(g.cases.size());
        }
        if (si_entries > 0) {
            h_si_jobs.alloc(si_entries);
            d_si_jobs.alloc(si_entries);
        }
        h_force_jobs.alloc(cases.size());
        d_force_jobs.alloc(cases.size());
        case_batched.assign(cases.size(), 0);
        h_case_jobs.alloc(cases.size());
        d_case_jobs.alloc(cases.size());
        counters.alloc(16);
        err.alloc(1);
        ck(cudaMemset(err.p, 0, sizeof(int)), "memset");
        h_err.alloc(1);
        make_groups();
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(bucket());
            if (it != g_tune_cache.end()) {
                tuning = it->second;
                tuned = true;
            }
        }
        plan(tuning);
        ck(cudaDeviceSynchronize(), "batch build");
    }

    // Groups of sweeps that share a kernel variant.
    void make_groups() {
        groups.clear();
        std::map<std::tuple<int, int, int, int>, int> index;
        for (size_t i = 0; i < cases.size(); ++i) {
            sb_sim& c = *cases[i];
            if (!c.dynamic) continue;
            c.precision = precision;
            for (int kind = 0; kind < 2; ++kind) {
                const int neglect = kind == 0 ? c.dm.neglect_self : 0;
                const int chain = kind == 1 && c.use_chains() ? 1 : 0;
                auto key = std::make_tuple(kind, c.dm.symmetry, neglect, chain);
                auto it = index.find(key);
                if (it == index.end()) {
                    Group g;
                    g.kind = kind;
                    g.sym = c.dm.symmetry;
                    g.neglect = neglect;
                    g.chain = chain;
                    it = index.emplace(key, static_cast<int>(groups.size())).first;
                    groups.push_back(g);
                }
                groups[it->second].cases.push_back(static_cast<int>(i));
            }
        }
        if (groups.size() > 16) raise(SB_ERR_UNSUPPORTED, "too many sweep variants in one batch");
    }

    // Workload bucket of the tuning cache: precision, log2 of the steady-state roll-up pairs,
    // log2 of the number of cases, and the number of sweep variants.
    std::tuple<int, int, int, int> bucket() const {
        double pairs = 0.0;
        for (const auto& c : cases)
            if (c->dynamic) pairs += static_cast<double>(std::min<long long>(c->dm.end_index, c->P_pts)) * c->P_pan;
        return std::make_tuple(precision, static_cast<int>(std::lround(std::log2(std::max(pairs, 1.0)))),
                               static_cast<int>(std::lround(std::log2(static_cast<double>(cases.size())))),
                               static_cast<int>(groups.size()));
    }

    // Steady-state sweep sizes (all wake rows active) of case c.
    static void full_sizes(const sb_sim& c, int kind, long long& M, long long& P, long long& M_total) {
        if (kind == 0) {
            M = c.N;
            P = c.P_pan - c.N;
            M_total = c.N;
        } else {
            M = c.dm.end_index > 0 ? std::min<long long>(c.dm.end_index, c.P_pts) : 0;
            P = c.use_chains() ? c.chain_Q * c.chain_Bq : c.P_pan;  // chain and panel records cost alike
            M_total = c.P_pts;
        }
    }

    // Chunk sizes, item order, partial-sum offsets and grids for the tuning t.
    void plan(const Tuning& t) {
        drop_graphs();
        long long part_total = 0;
        job_entries = 0;
        for (auto& g : groups) {
            const int tile = bs_tile_panels(precision, g.sym, g.chain, t.tile);
            g.tile = tile;
            const int T = bs_targets_per_thread(g.sym);
            const long long TM = static_cast<long long>(kBsThreads) * T;
            const int occ = bs_occupancy_blocks_per_sm(precision, g.sym, g.neglect, g.chain ? 0 : t.tile);
            const int bps = t.blocks_per_sm > 0 ? std::min(t.blocks_per_sm, occ) : occ;
            g.grid = sms * bps;
            double total = 0.0;
            for (int c : g.cases) {
                long long M, P, Mt;
                full_sizes(*cases[c], g.kind, M, P, Mt);
                total += static_cast<double>(M) * static_cast<double>(P);
            }
            const double item_pairs = std::max(total / (static_cast<double>(g.grid) * t.waves),
                                               static_cast<double>(TM) * tile);
            const size_t n = g.cases.size();
            g.chunk.assign(n, tile);
            for (size_t k = 0; k < n; ++k) {
                long long M, P, Mt;
                full_sizes(*cases[g.cases[k]], g.kind, M, P, Mt);
                long long ch = static_cast<long long>(std::ceil(item_pairs / static_cast<double>(TM)));
                ch = ((ch + tile - 1) / tile) * tile;
                const long long whole = std::max<long long>(tile, ((P + tile - 1) / tile) * tile);
                const long long min_for_cap = (((P + kMaxChunksPerJob - 1) / kMaxChunksPerJob + tile - 1) / tile) * tile;
                ch = std::min(std::max<long long>({ch, static_cast<long long>(tile), min_for_cap}), whole);
                g.chunk[k] = static_cast<int>(ch);
            }
            // schedule 0: costliest items first (LPT order); 1: case order. Fixed until re-planned
            std::vector<size_t> order(n);
            std::iota(order.begin(), order.end(), 0);
            if (t.order == 0)
                std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return g.chunk[a] > g.chunk[b]; });
            std::vector<int> cs(n), ch(n);
            for (size_t k = 0; k < n; ++k) {
                cs[k] = g.cases[order[k]];
                ch[k] = g.chunk[order[k]];
            }
            g.cases = cs;
            g.chunk = ch;
            g.part_off.assign(n, 0);
            g.block_off.assign(n, 0);
            long long blocks = 0;
            for (size_t k = 0; k < n; ++k) {
                long long M, P, Mt;
                full_sizes(*cases[g.cases[k]], g.kind, M, P, Mt);
                const long long nch = P > 0 ? (P + g.chunk[k] - 1) / g.chunk[k] : 0;
                g.part_off[k] = part_total;
                part_total += nch * M * 3;
                g.block_off[k] = blocks;
                blocks += (Mt + kBsReduceThreads - 1) / kBsReduceThreads;
            }
            g.reduce_blocks = blocks;
            g.job_off = job_entries;
            job_entries += static_cast<long long>(n) + 1;  // + sentinel
        }
        if (partial.n < static_cast<size_t>(std::max<long long>(part_total, 1))) partial.alloc(std::max<long long>(part_total, 1));
        if (h_jobs.n < static_cast<size_t>(std::max<long long>(job_entries, 1))) {
            h_jobs.alloc(std::max<long long>(job_entries, 1));
            d_jobs.alloc(std::max<long long>(job_entries, 1));
        }
        tuning = t;
    }

    // Work lists of the current step (host), for every group.
    void fill_jobs() {
        last_pairs = 0;
        for (auto& g : groups) {
            const int T = bs_targets_per_thread(g.sym);
            const long long TM = static_cast<long long>(kBsThreads) * T;
            long long item = 0;
            for (size_t k = 0; k < g.cases.size(); ++k) {
                sb_sim& c = *cases[g.cases[k]];
                sb_sim::SweepDesc d = g.kind == 0 ? c.fixed_desc() : c.rollup_desc();
                BsJob J;
                J.panels = d.src ? d.src
                                 : precision == 2 ? static_cast<const void*>(c.rec64.p) : static_cast<const void*>(c.rec32.p);
                J.p_begin = d.p0;
                J.p_end = d.p1;
                J.targets = d.targets;
                J.target_wing = d.twing;
                J.M = d.M;
                J.chunk_panels = g.chunk[k];
                const long long P = d.p1 - d.p0;
                J.n_chunks = (P > 0 && d.M > 0) ? static_cast<int>((P + g.chunk[k] - 1) / g.chunk[k]) : 0;
                c.target_layout(d, J);
                J.n_ttiles = (bs_slots(J) + TM - 1) / TM;
                J.partial = partial.p + g.part_off[k];
                J.item_begin = item;
                J.M_total = d.M_total;
                J.base = d.base;
                J.out = d.dst;
                J.block_begin = g.block_off[k];
                item += J.n_ttiles * static_cast<long long>(J.n_chunks);
                if (J.n_chunks > 0) last_pairs += d.M * P;
                h_jobs.p[g.job_off + static_cast<long long>(k)] = J;
            }
            BsJob sentinel;
            sentinel.item_begin = item;
            sentinel.block_begin = g.reduce_blocks;
            h_jobs.p[g.job_off + static_cast<long long>(g.cases.size())] = sentinel;
            g.items = item;
        }
    }

    // ------------------------------------------------------------------ one step
    void fork(int slot) {
        ck(cudaEventRecord(ev_fork[slot], main), "fork");
        for (auto& s : pool) ck(cudaStreamWaitEvent(s, ev_fork[slot], 0), "fork");
    }
    void join(int slot) {
        for (int k = 0; k < kPoolStreams; ++k) {
            ck(cudaEventRecord(ev_join[slot][k], pool[k]), "join");
            ck(cudaStreamWaitEvent(main, ev_join[slot][k], 0), "join");
        }
    }

    void launch_group(Group& g) {
        BsArgs a;
        a.jobs = d_jobs.p + g.job_off;
        a.n_jobs = static_cast<int>(g.cases.size());
        a.work_counter = counters.p + (&g - groups.data());
        a.err = err.p;
        a.symmetry = g.sym;
        a.neglect = g.neglect;
        a.chain = g.chain;
        a.tile = g.tile;
        ck(cudaMemsetAsync(a.work_counter, 0, sizeof(unsigned long long), main), "memset counter");
        ck(launch_bs_sweep(a, precision, g.grid, main), "batched Biot-Savart sweep");
        ck(launch_bs_reduce_jobs(a.jobs, a.n_jobs, g.reduce_blocks, main), "batched sweep reduce");
    }

    void sweeps(int kind) {
        for (auto& g : groups)
            if (g.kind == kind) launch_group(g);
    }

    // Enqueues one step of every case on main + pool (the freestream is in fs_all and the
    // work lists in h_jobs).
    void enqueue(double time, double dt, bool wind) {
        if (job_entries > 0)
            ck(cudaMemcpyAsync(d_jobs.p, h_jobs.p, job_entries * sizeof(BsJob), cudaMemcpyHostToDevice, main), "H2D jobs");
        if (si_entries > 0)
            ck(cudaMemcpyAsync(d_si_jobs.p, h_si_jobs.p, si_entries * sizeof(SolveJob), cudaMemcpyHostToDevice, main),
               "H2D solve jobs");
        if (wind)
            ck(cudaMemcpyAsync(wind_steps.p, h_wind_steps.p, cases.size() * 2 * sizeof(double), cudaMemcpyHostToDevice, main),
               "H2D wind steps");
        if (n_case_jobs > 0)
            ck(cudaMemcpyAsync(d_case_jobs.p, h_case_jobs.p, n_case_jobs * sizeof(CaseStepJob), cudaMemcpyHostToDevice,
                               main),
               "H2D case jobs");
        fork(0);
        for (size_t i = 0; i < cases.size(); ++i) {
            sb_sim& c = *cases[i];
            if (wind) c.enqueue_wind_freestream();  // complete_sail_model/mod.rs:213-257
            if (case_batched[i]) c.step_begin_host(time, dt);
            else c.step_begin(time, dt);
        }
        join(0);
        if (n_case_jobs > 0) {  // geometry, then wake advection and panels, of the batched cases
            ck(launch_prep_geometry_jobs(d_case_jobs.p, n_case_jobs, main), "batched geometry");
            ck(launch_wake_jobs(d_case_jobs.p, n_case_jobs, blk_advect, blk_panels, main), "batched wake update");
        }
        if (warm_mode != 0) warm_start_before_solve();
        sweeps(0);
        for (auto& c : cases) if (c->dynamic) c->after_fixed_sweep();
        if (n_case_jobs > 0) ck(launch_unit_matrix_jobs(d_case_jobs.p, n_case_jobs, blk_matrix, main), "batched unit matrix");
        fork(1);
        for (size_t i = 0; i < cases.size(); ++i) {
            sb_sim& c = *cases[i];
            if (case_batched[i]) {
                if (!si_batched[i]) c.step_solve();  // matrix and chain records come from the batch
            } else if (c.linearized_quasi_steady() || si_batched[i]) {
                c.step_matrix();
            } else {
                c.step_matrix_and_solve();
            }
        }
        join(1);
        // the batched solves: a launch per Linearized plan shape and per SimpleIterative
        // cluster size, side by side on the pool streams
        int n_launch = 0;
        for (const auto& g : lin_groups) n_launch += g.n > 0 ? 1 : 0;
        for (const auto& g : si_groups) n_launch += g.cases.empty() ? 0 : 1;
        if (n_launch > 0) {
            if (n_launch > 1) fork(1);
            int k = 0;
            for (const auto& g : lin_groups)
                if (g.n > 0)
                    ck(launch_solve_linearized_jobs(g.jobs.p, g.n, g.plan, n_launch > 1 ? pool[k++] : main),
                       "batched linearized solve");
            for (const auto& g : si_groups)
                if (!g.cases.empty()) {
                    // shared memory of the group's largest case (its matrix slab depends on
                    // whether the matrix has lo parts off the diagonal, i.e. on the precision)
                    size_t smem = 0;
                    for (int ci : g.cases)
                        smem = std::max(smem, si_smem_bytes(cases[ci]->N, cases[ci]->solve_buffers().split_full,
                                                              cases[ci]->solve_buffers().split_comps));
                    ck(launch_solve_simple_iterative_jobs(d_si_jobs.p + g.off, static_cast<int>(g.cases.size()), g.cluster,
                                                          g.rows_per_thread, smem, n_launch > 1 ? pool[k++] : main),
                       "batched simple iterative solve");
                }
            if (n_launch > 1) join(1);
        }
        // what follows a solve in its case (chain records of the wake), after the batched solves
        bool after = false;
        for (size_t i = 0; i < cases.size(); ++i) after = after || (si_batched[i] && !case_batched[i]);
        if (after) {
            fork(1);
            for (size_t i = 0; i < cases.size(); ++i)
                if (si_batched[i] && !case_batched[i]) cases[i]->step_after_solve();
            join(1);
        }
        if (n_case_jobs > 0 && blk_chain > 0)
            ck(launch_chain_records_jobs(d_case_jobs.p, n_case_jobs, blk_chain, main), "batched chain records");
        if (warm_mode != 0)
            ck(launch_batch_targets(gamma_all.p, w_q.p, w_g0.p, w_tr.p, N_total, w_target.p, main), "warm-start targets");
        sweeps(1);
        for (auto& c : cases) if (c->dynamic) c->after_rollup_sweep();
        fill_force_jobs();
        ck(cudaMemcpyAsync(d_force_jobs.p, h_force_jobs.p, cases.size() * sizeof(ForceJob), cudaMemcpyHostToDevice, main),
           "H2D force jobs");
        ck(launch_forces_jobs(d_force_jobs.p, static_cast<int>(cases.size()), main), "batched forces");
        for (auto& c : cases) c->after_forces();
        k_gather<<<static_cast<unsigned>(cases.size()), 128, 0, main>>>(gather_jobs.p);
        ck(cudaGetLastError(), "gather");
        const size_t ncomp = static_cast<size_t>(N_total) + cases.size() * SB_BATCH_SUMMARY;
        ck(cudaMemcpyAsync(h_compact.p, compact.p, ncomp * sizeof(double), cudaMemcpyDeviceToHost, main), "D2H summary");
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, main), "D2H status");
    }

    // ------------------------------------------------------------------ warm start
    void set_warm_start(sb_mlp* m, int mode) {
        if (mode < 0 || mode > 2) raise(SB_ERR_SIZE, "warm-start mode must be 0, 1 or 2");
        if (mode == 1 && !m) raise(SB_ERR_NULL_ARG, "warm-start mode 1 needs a network");
        if (mode == 1 && mlp_inputs(m) != kMlpFeatures)
            raise(SB_ERR_SIZE, "the warm-start network must take " + std::to_string(kMlpFeatures) + " inputs");
        for (const auto& c : cases)
            if (mode != 0 && c->solver_kind != 0) raise(SB_ERR_UNSUPPORTED, "the warm start needs SimpleIterative solvers");
        ck(cudaStreamSynchronize(main), "sync");
        drop_graphs();
        if (mode != 0 && w_feat.n == 0) {
            w_feat.alloc(static_cast<size_t>(N_total) * kMlpFeatures);
            w_y.alloc(N_total);
            w_target.alloc(N_total);
            w_q.alloc(N_total);
            w_g0.alloc(N_total);
            w_tr.alloc(N_total);
            w_cand.alloc(N_total);
            w_cand_ex.alloc(N_total);
            w_gamma_old.alloc(N_total);
            w_fs_old.alloc(N_total);
            ck(cudaMemset(w_target.p, 0, N_total * sizeof(float)), "memset");
            h_feat.alloc(cases.size());
            d_feat.alloc(cases.size());
        }
        if (mode == 1) mlp_reserve(m, N_total);
        mlp = mode == 1 ? m : nullptr;
        warm_mode = mode;
        warm_hist.assign(cases.size(), 0);
        for (size_t i = 0; i < cases.size(); ++i) {
            cases[i]->candidate_p[0] = mode == 1 ? w_cand_ex.p + line_off[i] : nullptr;
            cases[i]->candidate_p[1] = mode == 1 ? w_cand.p + line_off[i] : nullptr;
        }
    }

    // Feature jobs of this step (host; steps completed before the step).
    void fill_feature_jobs() {
        for (size_t i = 0; i < cases.size(); ++i) {
            const sb_sim& c = *cases[i];
            FeatJob f;
            f.fs = c.fs_p;
            f.gamma = c.gamma_p;
            f.gamma_old = w_gamma_old.p + line_off[i];
            f.fs_old = w_fs_old.p + line_off[i];
            f.chord = c.chord_global.p;
            f.span_s = c.span_s.p;
            f.span_e = c.span_e.p;
            f.chord_len = c.chord_len.p;
            f.wing_of_line = c.wing_of_line.p;
            f.wing_start = c.wing_start.p;
            f.wing_end = c.wing_end.p;
            f.N = c.N;
            f.S = c.S;
            f.W = c.W;
            f.steps = c.dynamic ? c.steps_completed : c.fd_count;
            f.hist = warm_hist[i];
            f.row0 = line_off[i];
            h_feat.p[i] = f;
        }
    }

    void warm_start_before_solve() {
        ck(cudaMemcpyAsync(d_feat.p, h_feat.p, cases.size() * sizeof(FeatJob), cudaMemcpyHostToDevice, main),
           "H2D feature jobs");
        ck(launch_batch_features(d_feat.p, static_cast<int>(cases.size()), N_total, w_feat.p, w_q.p, w_g0.p, w_tr.p,
                                 main),
           "warm-start features");
        if (warm_mode == 1) {
            mlp_forward_async(mlp, w_feat.p, N_total, w_y.p, main);
            ck(launch_batch_candidate(w_y.p, w_q.p, w_g0.p, w_tr.p, N_total, w_cand_ex.p, w_cand.p, main),
               "warm-start candidates");
        }
    }

    void copy_warm_start_data(float* feat, float* target, size_t rows) {
        if (warm_mode == 0) raise(SB_ERR_STATE, "the batch records no warm-start data (mode 0)");
        if (static_cast<long long>(rows) != N_total) raise(SB_ERR_SIZE, "rows must equal the batch's span lines");
        order_after_caller(main);  // the caller's buffers may still be in use on its stream
        if (feat)
            ck(cudaMemcpyAsync(feat, w_feat.p, rows * kMlpFeatures * sizeof(float), cudaMemcpyDefault, main), "copy");
        if (target) ck(cudaMemcpyAsync(target, w_target.p, rows * sizeof(float), cudaMemcpyDefault, main), "copy");
        ck(cudaStreamSynchronize(main), "copy");
    }

    // Host state a replayed graph step leaves behind (the same as enqueue's bookkeeping).
    void replay_bookkeeping(double time, double dt) {
        for (auto& c : cases) {
            c->params.time = time;
            c->params.dt = dt;
            if (c->dynamic) {
                c->cur ^= 1;
                c->after_fixed_sweep();
                c->after_rollup_sweep();
            }
            c->fd_count += 1;
        }
    }

    bool steady() const {
        for (const auto& c : cases) {
            if (!c->first_step_completed || c->fd_count < 2) return false;
            if (c->dynamic && c->steps_completed < 3) return false;
        }
        return true;
    }

    void step(double time, double dt, bool wind = false) {
        for (auto& c : cases) {
            if (c->timing) c->timing = false;
            c->precision = precision;
            c->ensure_rec64();  // FP64 records (allocation) before any capture
        }
        if (graph_dt != dt || graph_precision != precision || graph_wind != (wind ? 1 : 0)) drop_graphs();
        if (warm_mode != 0) fill_feature_jobs();
        // the parity of the wake buffers at the start of the step selects the graph
        const int parity = any_dynamic ? first_dynamic().cur : (steps & 1);
        ck(cudaEventRecord(ev_t0, main), "event");
        fill_case_jobs(time, dt);
        if (use_graph && steady()) {
            // job lists of this step, read by the graph's copy node at launch
            fill_jobs_after_begin();
            if (!graph[parity]) {
                // capture: the host-side state advances as in an eager step
                cudaGraph_t g = nullptr;
                ck(cudaStreamBeginCapture(main, cudaStreamCaptureModeRelaxed), "begin capture");
                try {
                    enqueue(time, dt, wind);
                } catch (...) {
                    cudaStreamEndCapture(main, &g);
                    if (g) cudaGraphDestroy(g);
                    throw;
                }
                ck(cudaStreamEndCapture(main, &g), "end capture");
                cudaError_t e = cudaGraphInstantiate(&graph[parity], g, 0);
                cudaGraphDestroy(g);
                ck(e, "graph instantiate");
                graph_dt = dt;
                graph_precision = precision;
                graph_wind = wind ? 1 : 0;
            } else {
                // host state of the step as an eager step leaves it before its forces
                replay_bookkeeping(time, dt);
                for (auto& c : cases) c->fd_count -= 1;
                fill_force_jobs();
                for (auto& c : cases) c->fd_count += 1;
            }
            ck(cudaGraphLaunch(graph[parity], main), "graph launch");
        } else {
            fill_jobs_after_begin();
            enqueue(time, dt, wind);
        }
        ck(cudaEventRecord(ev_t1, main), "event");
        ck(cudaStreamSynchronize(main), "batch step");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev_t0, ev_t1);
        last_ms = ms;
        steps += 1;
        if (warm_mode != 0)
            for (auto& h : warm_hist) h = std::min(h + 1, 2);
        if (mlp) mlp_check(mlp);
        if (h_err.p[0] != kDevOk) {
            ck(cudaMemset(err.p, 0, sizeof(int)), "memset");
            raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out in a batched sweep");
        }
        for (size_t i = 0; i < cases.size(); ++i) {
            const double st = h_compact.p[N_total + static_cast<long long>(i) * SB_BATCH_SUMMARY + 9];
            if (st != 0.0) {
                sb_sim& c = *cases[i];
                ck(cudaMemset(c.err.p, 0, sizeof(int)), "memset");
                if (st == kDevTimeout) raise(SB_ERR_TIMEOUT, "case " + std::to_string(i) + ": a bounded device-side wait ran out");
                if (st == kDevSingular) raise(SB_ERR_STATE, "case " + std::to_string(i) + ": Matrix is singular or nearly singular");
                raise(SB_ERR_CUDA, "case " + std::to_string(i) + ": device error word " + std::to_string(st));
            }
        }
    }

    // Loads case i's state (sb_sim_set_state layout). Every dynamic case of a batch must be
    // at the same wake-buffer parity and step count for the batched step; a state taken from
    // another batch's case i at the same step keeps that. The case's warm-start history starts
    // again: its extrapolation candidate waits for two solutions of this batch's own.
    void set_case_state(size_t i, const double* state, size_t n) {
        ck(cudaStreamSynchronize(main), "sync");
        sb_sim& c = *cases[i];
        c.set_state(state, n);
        if (i < warm_hist.size()) warm_hist[i] = 0;
        drop_graphs();
    }

    const sb_sim& first_dynamic() const {
        for (const auto& c : cases) if (c->dynamic) return *c;
        return *cases[0];
    }

    // The work lists describe the sweeps as they will be after step_begin (which swaps the
    // wake buffers): compute them with the parity flipped for the duration.
    // The job of every dynamic case past its first step (state before the step).
    void fill_case_jobs(double time, double dt) {
        n_case_jobs = 0;
        blk_advect = blk_panels = blk_matrix = blk_chain = 0;
        for (size_t i = 0; i < cases.size(); ++i) {
            const sb_sim& c = *cases[i];
            case_batched[i] = c.batch_kernels_ok() ? 1 : 0;
            if (!case_batched[i]) continue;
            CaseStepJob j = c.step_job(time, dt);
            j.blk_advect = blk_advect;
            j.blk_panels = blk_panels;
            j.blk_matrix = blk_matrix;
            j.blk_chain = blk_chain;
            blk_advect += wake_advect_blocks(c.dm);
            blk_panels += wake_panels_blocks(c.dm);
            blk_matrix += unit_matrix_blocks(c.N, j.row0_32 != nullptr);
            blk_chain += chain_records_blocks(j.chain_n);
            h_case_jobs.p[n_case_jobs++] = j;
        }
    }

    void fill_jobs_after_begin() {
        for (auto& c : cases) if (c->dynamic) c->cur ^= 1;
        fill_jobs();
        fill_si_jobs();
        for (auto& c : cases) if (c->dynamic) c->cur ^= 1;
    }

    // The forces job of every case (read by the graph's copy node at launch when replayed).
    void fill_force_jobs() {
        for (size_t i = 0; i < cases.size(); ++i) h_force_jobs.p[i] = cases[i]->force_job();
    }

    // The SimpleIterative jobs of the step (each case's model, settings and buffers, with the
    // wake buffer its solve writes row 0 into).
    void fill_si_jobs() {
        for (const auto& g : si_groups)
            for (size_t k = 0; k < g.cases.size(); ++k) {
                const sb_sim& c = *cases[g.cases[k]];
                SolveJob& j = h_si_jobs.p[g.off + static_cast<long long>(k)];
                j.m = c.dm;
                j.st = c.solve;
                j.b = c.solve_buffers();
                j.b.second_margin = warm_margin;
            }
    }

    void do_step(double time, double dt, const double* fs_host, size_t n) {
        if (static_cast<long long>(n) != nfs_total)
            raise(SB_ERR_SIZE, "freestream has " + std::to_string(n) + " points, expected " + std::to_string(nfs_total));
        const size_t cnt = n * 3;
        const size_t bad = copy_finite(fs_host, h_fs_all.p, cnt);
        if (bad < cnt) raise(SB_ERR_NONFINITE, "non-finite freestream value at index " + std::to_string(bad / 3));
        ck(cudaMemcpyAsync(fs_all.p, h_fs_all.p, cnt * sizeof(double), cudaMemcpyHostToDevice, main), "H2D freestream");
        step(time, dt);
    }

    // ------------------------------------------------------------------ wind models
    void set_wind(const char* env_json, const char* const* cond_jsons) {
        ck(cudaStreamSynchronize(main), "sync");
        drop_graphs();
        if (wind_steps.n == 0) {
            wind_steps.alloc(cases.size() * 2);
            h_wind_steps.alloc(cases.size() * 2);
        }
        for (size_t i = 0; i < cases.size(); ++i) {
            if (!cond_jsons[i]) raise(SB_ERR_NULL_ARG, "wind condition of case " + std::to_string(i) + " is NULL");
            try {
                cases[i]->set_wind(env_json, cond_jsons[i]);
            } catch (const SbFail& e) {
                raise(e.code, "case " + std::to_string(i) + ": " + e.msg);
            }
            cases[i]->wind.step = wind_steps.p + 2 * i;
        }
        has_wind = true;
    }

    void do_step_wind(double time, double dt, const double* ship_velocities) {
        if (!has_wind) raise(SB_ERR_STATE, "no wind models: call sb_batch_set_wind first");
        for (size_t i = 0; i < cases.size(); ++i) {
            if (!std::isfinite(ship_velocities[i])) raise(SB_ERR_NONFINITE, "non-finite ship velocity of case " + std::to_string(i));
            h_wind_steps.p[2 * i] = time;
            h_wind_steps.p[2 * i + 1] = ship_velocities[i];
        }
        step(time, dt, true);
    }

    // The flow measurements every case's controller reads before a steady-state step
    // (CompleteSailModel::apply_controller_based_on_freestream, complete_sail_model/mod.rs:
    // 259-288): each case's wind freestream at its control points for (time, ship velocity),
    // then |u|, the angle of attack and the apparent wind direction per line. Returns the
    // host copy: case i's lines at 3 * line_off[i] (|u| [N], angle [N], direction [N]).
    const double* controller_inputs(double time, const double* ship_velocities) {
        if (!has_wind) raise(SB_ERR_STATE, "no wind models: call sb_batch_set_wind first");
        for (size_t i = 0; i < cases.size(); ++i) {
            if (!std::isfinite(ship_velocities[i])) raise(SB_ERR_NONFINITE, "non-finite ship velocity of case " + std::to_string(i));
            h_wind_steps.p[2 * i] = time;
            h_wind_steps.p[2 * i + 1] = ship_velocities[i];
        }
        if (ctrl_in.n == 0) {
            ctrl_in.alloc(static_cast<size_t>(N_total) * 3);
            h_ctrl_in.alloc(static_cast<size_t>(N_total) * 3);
        }
        ck(cudaMemcpyAsync(wind_steps.p, h_wind_steps.p, cases.size() * 2 * sizeof(double), cudaMemcpyHostToDevice, main),
           "H2D wind steps");
        fork(0);
        for (size_t i = 0; i < cases.size(); ++i) {
            sb_sim& c = *cases[i];
            c.enqueue_wind_freestream();
            double* d = ctrl_in.p + 3 * line_off[i];
            ck(launch_controller_input(c.dm, c.params, c.fs_p, d, c.stream), "controller input");
            ck(cudaMemcpyAsync(h_ctrl_in.p + 3 * line_off[i], d, 3 * c.N * sizeof(double), cudaMemcpyDeviceToHost,
                               c.stream),
               "D2H controller input");
        }
        join(0);
        ck(cudaStreamSynchronize(main), "controller input");
        return h_ctrl_in.p;
    }

    // Integrated forces [S][6][3] then moments [S][6][3] of every case after the last step,
    // case after case (what SimulationResult::as_simplified reads, results/simulation.rs:150-166).
    const double* wing_totals() {
        size_t total = 0;
        for (const auto& c : cases) total += static_cast<size_t>(c->S) * 36;
        if (h_wing_totals.n < total) h_wing_totals.alloc(total);
        size_t off = 0;
        for (const auto& c : cases) {
            const size_t n = static_cast<size_t>(c->S) * 18;
            ck(cudaMemcpyAsync(h_wing_totals.p + off, c->out.p + c->L.intf, n * sizeof(double), cudaMemcpyDeviceToHost,
                               main),
               "D2H wing forces");
            ck(cudaMemcpyAsync(h_wing_totals.p + off + n, c->out.p + c->L.intm, n * sizeof(double),
                               cudaMemcpyDeviceToHost, main),
               "D2H wing moments");
            off += 2 * n;
        }
        ck(cudaStreamSynchronize(main), "wing totals");
        return h_wing_totals.p;
    }

    void do_step_device(double time, double dt, const double* fs_dev, size_t n) {
        if (static_cast<long long>(n) != nfs_total) raise(SB_ERR_SIZE, "freestream length mismatch");
        order_after_caller(main);
        ck(cudaMemcpyAsync(fs_all.p, fs_dev, n * sizeof(d3), cudaMemcpyDeviceToDevice, main), "D2D freestream");
        step(time, dt);
    }

    // ------------------------------------------------------------------ autotuner
    // Times the roll-up sweeps of the current wake state for each candidate (waves x CTAs per
    // SM) and keeps the fastest. The sweeps only rewrite the wake-point velocities, which the
    // last run (with the chosen plan) leaves as an eager sweep of this state would.
    void autotune(double budget_s) {
        bool active = false;
        for (const auto& c : cases) active = active || (c->dynamic && c->rollup_active());
        if (!active) raise(SB_ERR_STATE, "autotuning needs a batch whose wake roll-up has started (4 steps)");
        ck(cudaStreamSynchronize(main), "sync");
        // times the roll-up sweeps of the current state under tuning t (best of two)
        double spent = 0.0;
        tune_candidates = 0;
        auto time_candidate = [&](const Tuning& t) {
            plan(t);
            fill_jobs();
            ck(cudaMemcpyAsync(d_jobs.p, h_jobs.p, job_entries * sizeof(BsJob), cudaMemcpyHostToDevice, main), "H2D jobs");
            auto t0 = std::chrono::steady_clock::now();
            double ms = 1e300;
            for (int rep = 0; rep < 2; ++rep) {
                ck(cudaEventRecord(ev_t0, main), "event");
                sweeps(1);
                ck(cudaEventRecord(ev_t1, main), "event");
                ck(cudaStreamSynchronize(main), "tuning sweep");
                float f = 0.f;
                cudaEventElapsedTime(&f, ev_t0, ev_t1);
                ms = std::min(ms, static_cast<double>(f));
            }
            spent += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            tune_candidates += 1;
            return ms;
        };
        Tuning best = tuning;
        double best_ms = 1e300;
        auto consider = [&](const Tuning& t) {
            if (spent > budget_s) return;
            const double ms = time_candidate(t);
            if (ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        };
        // 1. tile shape (panels per shared-memory stage) at the default decomposition
        int tiles[4] = {0, 0, 0, 0};
        const int n_tiles = bs_tile_choices(tiles, 4);
        for (int k = 0; k < n_tiles; ++k) consider(Tuning{8, 0, tiles[k] == 64 ? 0 : tiles[k], 0});
        // 2. items per persistent CTA x CTAs per SM for that tile
        int occ = 1;
        for (const auto& g : groups)
            occ = std::max(occ, bs_occupancy_blocks_per_sm(precision, g.sym, g.neglect, g.chain ? 0 : best.tile));
        const Tuning after_tile = best;
        std::vector<int> blocks = {0};  // 0: the occupancy limit
        if (occ >= 2) blocks.push_back(occ - 1);
        for (int w : {1, 2, 4, 8, 16, 32})
            for (int b : blocks)
                if (!(w == after_tile.waves && b == after_tile.blocks_per_sm)) consider(Tuning{w, b, after_tile.tile, 0});
        // 3. item schedule
        Tuning alt = best;
        alt.order = 1;
        consider(alt);
        plan(best);
        fill_jobs();
        ck(cudaMemcpyAsync(d_jobs.p, h_jobs.p, job_entries * sizeof(BsJob), cudaMemcpyHostToDevice, main), "H2D jobs");
        sweeps(1);
        ck(cudaMemcpyAsync(h_err.p, err.p, sizeof(int), cudaMemcpyDeviceToHost, main), "D2H status");
        ck(cudaStreamSynchronize(main), "tuning");
        if (h_err.p[0] != kDevOk) {
            ck(cudaMemset(err.p, 0, sizeof(int)), "memset");
            raise(SB_ERR_TIMEOUT, "a bounded device-side wait ran out in a batched sweep");
        }
        tuned = true;
        tune_best_ms = best_ms;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[bucket()] = best;
    }
};

// =======================================================================================
// C ABI
// =======================================================================================
namespace sbhost {

size_t batch_case_count(const sb_batch* b) { return b->cases.size(); }
sb_sim* batch_case(sb_batch* b, size_t i) { return b->cases.at(i).get(); }
long long batch_line_offset(const sb_batch* b, size_t i) { return b->line_off.at(i); }
const double* batch_controller_inputs(sb_batch* b, double time, const double* ship_velocities) {
    return b->controller_inputs(time, ship_velocities);
}
const double* batch_wing_totals(sb_batch* b) { return b->wing_totals(); }

}  // namespace sbhost

namespace {
int null_arg() {
    report_error(SB_ERR_NULL_ARG, "null argument");
    return SB_ERR_NULL_ARG;
}
}  // namespace

extern "C" {

sb_batch* sb_batch_new(const char* const* setup_jsons, size_t n_cases, int device) {
    if (!setup_jsons) {
        null_arg();
        return nullptr;
    }
    std::unique_ptr<sb_batch> b(new sb_batch());
    int rc = guard([&] { b->build(setup_jsons, n_cases, device); });
    if (rc != SB_OK) return nullptr;
    return b.release();
}

void sb_batch_free(sb_batch* b) { delete b; }

int sb_batch_sizes(const sb_batch* b, size_t* n_cases, size_t* total_lines, size_t* total_freestream) {
    if (!b) return null_arg();
    if (n_cases) *n_cases = b->cases.size();
    if (total_lines) *total_lines = static_cast<size_t>(b->N_total);
    if (total_freestream) *total_freestream = static_cast<size_t>(b->nfs_total);
    return SB_OK;
}

int sb_batch_case_sizes(const sb_batch* b, size_t i, size_t* n, size_t* s, size_t* nfs, size_t* line_offset,
                        size_t* freestream_offset) {
    if (!b) return null_arg();
    if (i >= b->cases.size()) {
        report_error(SB_ERR_SIZE, "case index out of range");
        return SB_ERR_SIZE;
    }
    const sb_sim& c = *b->cases[i];
    if (n) *n = static_cast<size_t>(c.N);
    if (s) *s = static_cast<size_t>(c.S);
    if (nfs) *nfs = static_cast<size_t>(c.nfs);
    if (line_offset) *line_offset = static_cast<size_t>(b->line_off[i]);
    if (freestream_offset) *freestream_offset = static_cast<size_t>(b->fs_off[i]);
    return SB_OK;
}

int sb_batch_get_freestream_points(sb_batch* b, double* points, size_t n) {
    if (!b || !points) return null_arg();
    return guard([&] {
        if (static_cast<long long>(n) != b->nfs_total) raise(SB_ERR_SIZE, "points buffer length mismatch");
        for (size_t i = 0; i < b->cases.size(); ++i) {
            sb_sim& c = *b->cases[i];
            c.freestream_points(points + 3 * b->fs_off[i], static_cast<size_t>(c.nfs));
        }
    });
}

int sb_batch_do_step(sb_batch* b, double time, double dt, const double* freestream, size_t n) {
    if (!b || !freestream) return null_arg();
    return guard([&] { b->do_step(time, dt, freestream, n); });
}

int sb_batch_do_step_device(sb_batch* b, double time, double dt, const double* freestream_dev, size_t n) {
    if (!b || !freestream_dev) return null_arg();
    return guard([&] { b->do_step_device(time, dt, freestream_dev, n); });
}

int sb_batch_set_wind(sb_batch* b, const char* environment_json, const char* const* condition_jsons) {
    if (!b || !environment_json || !condition_jsons) return null_arg();
    return guard([&] { b->set_wind(environment_json, condition_jsons); });
}

int sb_batch_do_step_wind(sb_batch* b, double time, double dt, const double* ship_velocities) {
    if (!b || !ship_velocities) return null_arg();
    return guard([&] { b->do_step_wind(time, dt, ship_velocities); });
}

int sb_batch_get_circulation(const sb_batch* b, double* gamma, size_t n) {
    if (!b || !gamma) return null_arg();
    if (static_cast<long long>(n) != b->N_total) {
        report_error(SB_ERR_SIZE, "circulation buffer length mismatch");
        return SB_ERR_SIZE;
    }
    std::memcpy(gamma, b->h_compact.p, n * sizeof(double));
    return SB_OK;
}

int sb_batch_get_summary(const sb_batch* b, double* summary, size_t n) {
    if (!b || !summary) return null_arg();
    if (n != b->cases.size() * SB_BATCH_SUMMARY) {
        report_error(SB_ERR_SIZE, "summary buffer length mismatch");
        return SB_ERR_SIZE;
    }
    std::memcpy(summary, b->h_compact.p + b->N_total, n * sizeof(double));
    return SB_OK;
}

int sb_batch_read_case_output(sb_batch* b, size_t i, sb_step_output* out) {
    if (!b || !out) return null_arg();
    if (i >= b->cases.size()) {
        report_error(SB_ERR_SIZE, "case index out of range");
        return SB_ERR_SIZE;
    }
    return guard([&] { b->cases[i]->read_output(out); });
}

int sb_batch_case_state_size(const sb_batch* b, size_t i, size_t* n) {
    if (!b || !n) return null_arg();
    if (i >= b->cases.size()) {
        report_error(SB_ERR_SIZE, "case index out of range");
        return SB_ERR_SIZE;
    }
    *n = b->cases[i]->state_size();
    return SB_OK;
}

int sb_batch_get_case_state(sb_batch* b, size_t i, double* state, size_t n) {
    if (!b || !state) return null_arg();
    if (i >= b->cases.size()) {
        report_error(SB_ERR_SIZE, "case index out of range");
        return SB_ERR_SIZE;
    }
    return guard([&] { b->cases[i]->get_state(state, n); });
}

int sb_batch_set_case_state(sb_batch* b, size_t i, const double* state, size_t n) {
    if (!b || !state) return null_arg();
    if (i >= b->cases.size()) {
        report_error(SB_ERR_SIZE, "case index out of range");
        return SB_ERR_SIZE;
    }
    return guard([&] { b->set_case_state(i, state, n); });
}

int sb_batch_set_initial_circulation(sb_batch* b, const double* gamma, size_t n) {
    if (!b || !gamma) return null_arg();
    return guard([&] {
        if (static_cast<long long>(n) != b->N_total) raise(SB_ERR_SIZE, "circulation length mismatch");
        ck(cudaMemcpyAsync(b->gamma_all.p, gamma, n * sizeof(double), cudaMemcpyHostToDevice, b->main), "H2D");
        ck(cudaStreamSynchronize(b->main), "sync");
    });
}

int sb_batch_set_initial_circulation_device(sb_batch* b, const double* gamma_dev, size_t n) {
    if (!b || !gamma_dev) return null_arg();
    return guard([&] {
        if (static_cast<long long>(n) != b->N_total) raise(SB_ERR_SIZE, "circulation length mismatch");
        order_after_caller(b->main);
        ck(cudaMemcpyAsync(b->gamma_all.p, gamma_dev, n * sizeof(double), cudaMemcpyDeviceToDevice, b->main), "D2D");
        ck(cudaStreamSynchronize(b->main), "sync");
    });
}

int sb_batch_previous_circulation_device(sb_batch* b, double** gamma_dev) {
    if (!b || !gamma_dev) return null_arg();
    *gamma_dev = b->gamma_all.p;
    return SB_OK;
}

int sb_batch_set_precision(sb_batch* b, int mode) {
    if (!b) return null_arg();
    if (mode < 0 || mode > 2) {
        report_error(SB_ERR_SIZE, "precision mode must be 0, 1 or 2");
        return SB_ERR_SIZE;
    }
    return guard([&] {
        if (mode != b->precision) {
            b->precision = mode;
            b->make_groups();  // chain records are FP32 only
            b->plan(b->tuning);
        }
    });
}

int sb_batch_use_graph(sb_batch* b, int enable) {
    if (!b) return null_arg();
    b->use_graph = enable != 0;
    if (!b->use_graph) b->drop_graphs();
    return SB_OK;
}

int sb_batch_autotune(sb_batch* b, double budget_seconds) {
    if (!b) return null_arg();
    return guard([&] { b->autotune(budget_seconds > 0.0 ? budget_seconds : 5.0); });
}

int sb_batch_set_warm_start(sb_batch* b, sb_mlp* network, int mode) {
    if (!b) return null_arg();
    return guard([&] { b->set_warm_start(network, mode); });
}

int sb_batch_set_warm_start_guard(sb_batch* b, double margin) {
    if (!b) return null_arg();
    return guard([&] {
        if (!(margin > 0.0 && margin <= 1.0)) raise(SB_ERR_SIZE, "the warm-start guard must lie in (0, 1]");
        b->warm_margin = margin;
    });
}

int sb_batch_copy_warm_start_data(sb_batch* b, float* features, float* targets, size_t rows) {
    if (!b) return null_arg();
    return guard([&] { b->copy_warm_start_data(features, targets, rows); });
}

int sb_batch_info(const sb_batch* b, double* info, size_t n) {
    if (!b || !info) return null_arg();
    long long items = 0;
    int grid = 0;
    for (const auto& g : b->groups) {
        if (g.kind == 1) {
            items += g.items;
            grid = std::max(grid, g.grid);
        }
    }
    const double v[SB_BATCH_INFO] = {b->last_ms,
                                     static_cast<double>(b->last_pairs),
                                     static_cast<double>(b->tuning.waves),
                                     static_cast<double>(b->tuning.blocks_per_sm),
                                     static_cast<double>(grid),
                                     static_cast<double>(items),
                                     b->tuned ? 1.0 : 0.0,
                                     static_cast<double>(b->tune_candidates),
                                     b->tune_best_ms,
                                     (b->graph[0] || b->graph[1]) ? 1.0 : 0.0,
                                     static_cast<double>(b->steps),
                                     static_cast<double>(bs_tile_panels(b->precision, 0, 0, b->tuning.tile)),
                                     static_cast<double>(b->tuning.order)};
    for (size_t i = 0; i < n && i < SB_BATCH_INFO; ++i) info[i] = v[i];
    return SB_OK;
}

}  // extern "C"
