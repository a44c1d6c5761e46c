// C-ABI of the device numeric phase (include/uchol_gpu.h): symbolic upload,
// plan cache, arena allocation, launch sequencing of the factorisation, the
// solves and the FP64-residual refinement.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/uchol_gpu.h"
#include "factor_kernels.cuh"
#include "panel_kernels.cuh"
#include "plan.hpp"
#include "solve_kernels.cuh"
#include "tc_gemm.cuh"
#include "inv_solve.cuh"

using namespace uchol_dev;

namespace {

thread_local std::string g_error;
std::atomic<long long> g_launches{0};          // kernel launches issued by this library
std::atomic<int> g_phase_timing{-1};           // -1: not yet read from UCHOL_PHASE_TIMES
inline void counted(int k = 1) { g_launches += k; }
inline bool phase_timing() {
    int v = g_phase_timing.load();
    if (v < 0) {
        const char* e = getenv("UCHOL_PHASE_TIMES");
        v = (e && *e && strcmp(e, "0") != 0) ? 1 : 0;
        g_phase_timing.store(v);
    }
    return v != 0;
}

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw Error(UCHOL_OOM, std::string(what) + ": device memory exhausted");
    }
    throw Error(UCHOL_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call) check((call), #call)

template <class F>
int guarded(F&& f) {
    try {
        f();
        g_error.clear();
        return UCHOL_OK;
    } catch (const Error& e) {
        g_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_error = "host allocation failed";
        return UCHOL_OOM;
    } catch (const std::exception& e) {
        g_error = e.what();
        return UCHOL_INTERNAL;
    }
}

// Owning device allocation.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t b, const char* what) {
        release();
        if (b == 0) b = 16;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            throw Error(UCHOL_OOM, std::string("cudaMalloc of ") + std::to_string(b) + " bytes for " + what +
                                       " failed: " + cudaGetErrorString(e));
        }
        bytes = b;
    }
    template <class V>
    void upload(const std::vector<V>& v, cudaStream_t s, const char* what) {
        alloc(v.size() * sizeof(V), what);
        if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, s));
    }
    template <class V>
    V* as() const { return static_cast<V*>(p); }
};

struct DevPlan {
    Plan plan;
    DBuf sn, rel, asm_pos, ea_items, ea_entries, small, pivot_tasks, panel_tasks, simt_jobs, tc_jobs,
        stage;
    DBuf fvec_off, solve_fronts, solve_tasks, inv_blocks, inv_tasks;
    DBuf rows, child_ptr, children;   // structure of the device fronts
};

// Device memory a factor of this plan reserves when it is created (the solve workspace,
// which depends on the number of right-hand sides, comes on top).
int64_t planned_bytes(const Plan& P, int precision, long long nnz, long long full_nnz, int n) {
    const int64_t elem = precision == UCHOL_PRECISION_FP64 ? 8 : 4;
    const int64_t op = precision == UCHOL_PRECISION_BF16 ? 2 : 4;
    const int64_t sb = P.cfg.solve_block;
    int64_t b = (P.factor_elems + P.contrib_elems) * elem;
    if (P.cfg.tensor_core)
        b += 2 * P.stage_elems * op + (int64_t)std::max(1, P.diag_slots) * kMinvStride * 4 +
             (int64_t)tc_ws_floats(152) * 4 + (int64_t)tc_counter_count(152) * 4;
    b += ((int64_t)P.inv_blocks.size() + P.inv_off_blocks) * sb * sb * elem;
    b += (nnz + full_nnz) * 8 + (int64_t)n * 8;
    return b;
}

void check_budget(int64_t budget, int64_t need) {
    if (budget > 0 && need > budget)
        throw Error(UCHOL_OOM, "the factorisation needs " + std::to_string(need) + " bytes of device memory, more than "
                                   "the budget of " + std::to_string(budget) + " bytes");
}

inline int grid_for(long long work, int block, int cap = 152 * 16) {
    long long g = (work + block - 1) / block;
    return (int)std::max<long long>(1, std::min<long long>(g, cap));
}

}  // namespace

struct uchol_symbolic_s {
    // held by its handle and by every factor made from it: the caller may destroy the handle
    // before its factors (a garbage collector picks any order), the object outlives them
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int n = 0, nnz = 0, count = 0;
    // host copies of the symbolic arrays (plans are built lazily per configuration)
    std::vector<int> row_ptr, col, perm, diag_idx, pat_ptr, pat_rows, lower_start, lower_ptr, lower_idx;
    std::vector<int> first_col, parent, child_ptr, children, front_ptr, front_rows;
    DBuf d_perm, d_diag_idx, d_full_ptr, d_full_col, d_full_src;
    long long full_nnz = 0;
    std::map<std::string, std::unique_ptr<DevPlan>> plans;
    std::mutex mu;

    // The plan of a configuration, built once and uploaded; `budget` > 0 rejects a plan whose
    // factor would need more device memory (UCHOL_OOM) before anything is uploaded.
    DevPlan* get_plan(const PlanConfig& c, int precision = UCHOL_PRECISION_FP64, int64_t budget = 0) {
        std::string key = std::to_string(c.pivot_block) + "/" + std::to_string(c.outer_block) + "/" +
                          std::to_string(c.small_mask) + "/" + std::to_string(c.tensor_core) + "/" +
                          std::to_string(c.solve_block) + "/" + std::to_string(c.merge_cols) + "/" +
                          std::to_string(c.merge_fill) + "/" + std::to_string(c.inv_cols) + "/" +
                          std::to_string(c.side_extend_add) + "/" + std::to_string(c.sms);
        auto it = plans.find(key);
        if (it != plans.end()) {
            check_budget(budget, planned_bytes(it->second->plan, precision, nnz, full_nnz, n));
            return it->second.get();
        }
        auto dp = std::make_unique<DevPlan>();
        try {
            dp->plan = build_plan(n, count, first_col.data(), parent.data(), child_ptr.data(), children.data(),
                                  front_ptr.data(), front_rows.data(), diag_idx.data(), pat_ptr.data(), pat_rows.data(),
                                  lower_start.data(), lower_ptr.data(), lower_idx.data(), nnz, c);
        } catch (const std::runtime_error& e) {
            throw Error(UCHOL_BAD_ARG, std::string("inconsistent symbolic factorization: ") + e.what());
        }
        const Plan& P = dp->plan;
        check_budget(budget, planned_bytes(P, precision, nnz, full_nnz, n));
        dp->sn.upload(P.sn, stream, "supernode table");
        dp->rel.upload(P.rel, stream, "relative indices");
        dp->asm_pos.upload(P.assemble_pos, stream, "assembly map");
        dp->ea_items.upload(P.ea_items, stream, "plan");
        dp->ea_entries.upload(P.ea_entries, stream, "plan");
        dp->small.upload(P.small_fronts, stream, "plan");
        dp->pivot_tasks.upload(P.pivot_tasks, stream, "plan");
        dp->panel_tasks.upload(P.panel_tasks, stream, "plan");
        dp->simt_jobs.upload(P.simt_jobs, stream, "plan");
        dp->tc_jobs.upload(P.tc_jobs, stream, "plan");
        dp->stage.upload(P.stage, stream, "plan");
        dp->fvec_off.upload(P.fvec_off, stream, "plan");
        dp->solve_fronts.upload(P.solve_fronts, stream, "plan");
        dp->solve_tasks.upload(P.solve_tasks, stream, "plan");
        dp->inv_blocks.upload(P.inv_blocks, stream, "plan");
        dp->inv_tasks.upload(P.inv_tasks, stream, "plan");
        dp->rows.upload(P.front_rows, stream, "front rows");
        dp->child_ptr.upload(P.child_ptr, stream, "children");
        dp->children.upload(P.children, stream, "children");
        CK(cudaStreamSynchronize(stream));
        DevPlan* raw = dp.get();
        plans[key] = std::move(dp);
        return raw;
    }
};

struct uchol_factor_s {
    uchol_symbolic sym = nullptr;
    DevPlan* dp = nullptr;
    uchol_options opts{};
    int precision = UCHOL_PRECISION_FP64;
    size_t elem = 8;              // bytes per front element
    DBuf panel, contrib, stage_a, stage_b, diag, values, full_val, stats, ctl;
    DBuf work, fv, fv2, vec[6], scal;   // solve workspace
    DBuf bwd_partial;                   // backward column dots split in row chunks: partial sums
    DBuf linv;                          // inverses of the diagonal blocks (solves)
    DBuf linv_off;                      // inverse fronts: off-diagonal blocks of the diagonal block's inverse
    DBuf inv_partial;                   // inverse fronts: backward partial sums (solve workspace)
    DBuf inv_diag_partial, inv_diag_cnt;   // inverse fronts: chunk partial sums of the diagonal products, counters
    DBuf minv;                          // mixed path: per outer block X^T, D, D^{-1} of each diagonal block
    DBuf solve_flags;                   // per diagonal block: forward and backward "solution published" flags
    DBuf solve_maps;                    // per front: tensor maps of its panel, boxes SB x SB, SB x SB/2, SB/2 x SB
    DBuf solve_status;                  // nonzero once a bounded wait of a solve expired
    int coop_fwd = 0, coop_bwd = 0;     // resident CTAs of the level solve kernels (whole device)
    int ws_nrhs = 0;
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t solve_graph = nullptr;
    int solve_graph_nrhs = 0, solve_graph_nodes = 0;
    cudaGraphExec_t factor_graph = nullptr;
    int factor_graph_nodes = 0;
    cudaStream_t side_stream = nullptr;   // captured factorisation: the side-stream extend-add launches
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    ~uchol_factor_s();
    DBuf maps;                    // tensor-map pairs of the staging regions
    DBuf tc_ws, tc_counters;      // K-split tiles of the tensor-core updates: partial tiles, arrival counts
    int sms = 148;
    uchol_factor_stats last{};
    uchol_phase_times phases{};
    std::mutex mu;
};

// Drops one reference; the last one frees the symbolic object and its own stream.
void symbolic_release(uchol_symbolic_s* s) {
    if (s->refs.fetch_sub(1) != 1) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaStream_t st = s->stream;
    const bool own = s->own_stream;
    delete s;
    if (own && st) cudaStreamDestroy(st);
}

uchol_factor_s::~uchol_factor_s() {
    if (solve_graph) cudaGraphExecDestroy(solve_graph);
    if (factor_graph) cudaGraphExecDestroy(factor_graph);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    if (side_stream) cudaStreamDestroy(side_stream);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (sym) symbolic_release(sym);
}

namespace {

struct StreamTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s;
    explicit StreamTimer(cudaStream_t st) : s(st) {
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        CK(cudaEventRecord(a, s));
    }
    double stop() {
        CK(cudaEventRecord(b, s));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        return ms;
    }
    ~StreamTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// K blocks of a tensor-core tile below which a launch is never split in K.
int split_min_kb(const uchol_options& o) { return o.split_min_kblocks == 0 ? kTcMinSplitKb : o.split_min_kblocks; }

PlanConfig config_for(const uchol_options& o) {
    PlanConfig c;
    c.small_mask = o.small_front_buckets ? o.small_front_buckets : 0x7;
    c.pivot_block = std::min(kMaxPivotBlock, std::max(4, std::min(128, o.panel_width)));
    c.merge_cols = o.chain_merge_width == 0 ? kDefaultMergeCols : std::max(0, o.chain_merge_width);
    c.inv_cols = o.inverse_block_width == 0 ? kDefaultInvCols : std::max(0, o.inverse_block_width);
    c.side_extend_add = o.extend_add_overlap >= 0;
    if (o.chain_merge_fill > 0.0) c.merge_fill = o.chain_merge_fill;
    if (o.precision == UCHOL_PRECISION_FP64) {
        c.tensor_core = false;
        c.outer_block = c.pivot_block;
        c.solve_block = 64;
    } else {
        c.solve_block = 128;
        c.tensor_core = true;
        c.pivot_block = std::min(c.pivot_block, 32);
        // outer block: 64 or 128 columns (the diagonal-block kernel holds at most kDiagMax)
        int nb = o.block_width > 0 ? o.block_width : kDiagMax;
        c.outer_block = std::max(64, std::min(kDiagMax, nb / 64 * 64));
    }
    return c;
}

template <class T>
void run_factor_launches(uchol_factor_s* F, cudaStream_t st) {
    DevPlan& D = *F->dp;
    const Plan& P = D.plan;
    T* panel = F->panel.as<T>();
    T* contrib = F->contrib.as<T>();
    double* diag = F->diag.as<double>();
    PivotStats* stats = F->stats.as<PivotStats>();
    FactorCtl* ctl = F->ctl.as<FactorCtl>();
    const SnDev* sn = D.sn.as<SnDev>();
    int launches = 0;
    // Optional per-kind device timing (UCHOL_PHASE_TIMES=1): one event pair per launch.
    const bool timing = phase_timing();
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    std::vector<int> ev_kind;
    const size_t small_smem = (size_t)P.max_small_m * P.max_small_m * sizeof(double);
    // side-stream launches fork from the main stream and are joined before the launch that
    // needs them (plan.hpp, Launch::stream); under per-launch timing everything runs in order
    const bool overlap = !timing && F->side_stream;
    bool side_busy = false;
    auto join_side = [&]() {
        CK(cudaEventRecord(F->join_ev, F->side_stream));
        CK(cudaStreamWaitEvent(st, F->join_ev, 0));
        side_busy = false;
    };
    for (const Launch& L : P.launches) {
        cudaStream_t ls = st;
        if (overlap && L.stream == 2 && side_busy) join_side();
        if (overlap && L.stream == 1) {
            if (side_busy) join_side();
            CK(cudaEventRecord(F->fork_ev, st));
            CK(cudaStreamWaitEvent(F->side_stream, F->fork_ev, 0));
            ls = F->side_stream;
            side_busy = true;
        }
        if (timing) {
            cudaEvent_t a, b;
            CK(cudaEventCreate(&a));
            CK(cudaEventCreate(&b));
            CK(cudaEventRecord(a, st));
            ev.push_back({a, b});
            ev_kind.push_back((int)L.kind);
        }
        switch (L.kind) {
            case Launch::ExtendAdd: {
                const int grid = (L.count + 7) / 8;
                if (ls == st)
                    k_extend_add<T><<<grid, 256, 0, ls>>>(D.ea_items.as<EaItem>() + L.begin, L.count,
                                                          D.ea_entries.as<EaEntry>(), sn, D.rel.as<int>(), panel,
                                                          contrib);
                else
                    k_extend_add<T, true><<<grid, 256, 0, ls>>>(D.ea_items.as<EaItem>() + L.begin, L.count,
                                                                D.ea_entries.as<EaEntry>(), sn, D.rel.as<int>(), panel,
                                                                contrib);
                break;
            }
            case Launch::SmallFronts:
                k_small_fronts<T><<<L.count, 256, small_smem, st>>>(D.small.as<int>() + L.begin, sn, panel, contrib,
                                                                    diag, ctl, stats);
                break;
            case Launch::PivotBlock:
            case Launch::Trsm:
            case Launch::SimtUpdate:
                // FP64 path: 32- or 64-column pivot blocks, TRSM and right-looking updates in FP64
                if constexpr (sizeof(T) == 8) {
                    const PanelTask* pt = D.pivot_tasks.as<PanelTask>() + L.begin;
                    const PanelTask* tk = D.panel_tasks.as<PanelTask>() + L.begin;
                    if (L.kind == Launch::PivotBlock)
                        k_pivot_block<T><<<L.count, 128, 0, st>>>(pt, sn, panel, diag, ctl, stats);
                    else if (L.kind == Launch::SimtUpdate)
                        k_simt_update<T, double><<<(unsigned)L.tiles, 256, 0, st>>>(
                            D.simt_jobs.as<UpdJob>() + L.begin, L.count, sn, panel, contrib, diag);
                    else if (P.cfg.pivot_block <= 32)
                        k_trsm<T, double, 32><<<L.count, 128, 0, st>>>(tk, sn, panel, diag);
                    else
                        k_trsm<T, double, 64><<<L.count, 128, 0, st>>>(tk, sn, panel, diag);
                } else {
                    throw Error(UCHOL_INTERNAL, "FP64 panel launch in a mixed-precision plan");
                }
                break;
            case Launch::DiagBlock:
            case Launch::PanelSolve:
                // mixed path: diagonal block, then its rows below as a GEMM with the block's inverse
                if constexpr (sizeof(T) == 4) {
                    if (L.kind == Launch::DiagBlock)
                        k_diag_block<<<L.count, 256, kDiagSmemBytes, st>>>(D.pivot_tasks.as<PanelTask>() + L.begin, sn,
                                                                           panel, diag, F->minv.as<float>(), ctl, stats);
                    else if (F->precision == UCHOL_PRECISION_BF16)
                        k_panel_solve<__nv_bfloat16><<<L.count, 256, kPanelSmemBytes, st>>>(
                            D.panel_tasks.as<PanelTask>() + L.begin, sn, panel, F->minv.as<float>(),
                            F->stage_a.as<__nv_bfloat16>(), F->stage_b.as<__nv_bfloat16>(), D.stage.as<StageInfo>());
                    else
                        k_panel_solve<float><<<L.count, 256, kPanelSmemBytes, st>>>(
                            D.panel_tasks.as<PanelTask>() + L.begin, sn, panel, F->minv.as<float>(),
                            F->stage_a.as<float>(), F->stage_b.as<float>(), D.stage.as<StageInfo>());
                } else {
                    throw Error(UCHOL_INTERNAL, "mixed-precision panel launch in an FP64 plan");
                }
                break;
            case Launch::KindCount:
                throw Error(UCHOL_INTERNAL, "invalid launch kind");
            case Launch::TcUpdate: {
                // K blocks of every job when all share one K (the launch may then be split in K)
                const bool bf16 = F->precision == UCHOL_PRECISION_BF16;
                const int kbe = bf16 ? 64 : 32;
                int nkb = (P.tc_jobs[L.begin].kn + kbe - 1) / kbe;
                for (int j = L.begin + 1; j < L.begin + L.count; ++j)
                    if (P.tc_jobs[j].kn != P.tc_jobs[L.begin].kn) nkb = 0;
                const TcPlanned tp = tc_schedule(L.tiles, nkb, F->sms, split_min_kb(F->opts));
                const TcSched S{L.tiles, tp.dp_tiles, tp.sk_nkb, F->tc_ws.as<float>(), F->tc_counters.as<int>()};
                launch_tc_gemm(bf16, D.tc_jobs.as<TcJob>() + L.begin, L.count, S, tp.grid, sn, (float*)panel,
                               (float*)contrib, F->maps.as<CUtensorMap>(), &stats->status, st);
                break;
            }
        }
        if (timing) CK(cudaEventRecord(ev.back().second, st));
        ++launches;
        counted();
    }
    if (side_busy) join_side();
    CK(cudaGetLastError());
    F->phases.launches = launches;
    F->phases.schur_tensor_flops = P.tc_flops;
    F->phases.schur_tensor_launches = 0;
    for (const Launch& L : P.launches) F->phases.schur_tensor_launches += L.kind == Launch::TcUpdate;
    if (timing) {
        CK(cudaStreamSynchronize(st));
        double sum[Launch::KindCount] = {0};
        // optional per-launch record (diagnostics): kind, tasks, tiles, algorithmic tensor flops, largest K, ms
        const char* log_path = getenv("UCHOL_LAUNCH_LOG");
        FILE* log = log_path && *log_path ? fopen(log_path, "w") : nullptr;
        if (log) fprintf(log, "kind,count,tiles,flops,max_k,ms\n");
        for (size_t q = 0; q < ev.size(); ++q) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[q].first, ev[q].second));
            sum[ev_kind[q]] += ms;
            cudaEventDestroy(ev[q].first);
            cudaEventDestroy(ev[q].second);
            if (log) {
                const Launch& L = P.launches[q];
                double flops = 0.0;
                int max_k = 0;
                if (L.kind == Launch::TcUpdate)
                    for (int j = L.begin; j < L.begin + L.count; ++j) {
                        const TcJobHost& J = P.tc_jobs[j];
                        flops += job_flops(UpdJob{0, J.s, J.c0, J.cend, J.kbeg, J.kn, -1}, P.sn[J.s]);
                        max_k = std::max(max_k, J.kn);
                    }
                fprintf(log, "%d,%d,%lld,%.6e,%d,%.6f\n", (int)L.kind, L.count, L.tiles, flops, max_k, ms);
            }
        }
        if (log) fclose(log);
        F->phases.extend_add_ms = sum[Launch::ExtendAdd];
        F->phases.small_fronts_ms = sum[Launch::SmallFronts];
        F->phases.panel_ms = sum[Launch::PivotBlock] + sum[Launch::Trsm] + sum[Launch::DiagBlock] + sum[Launch::PanelSolve];
        F->phases.schur_ms = sum[Launch::SimtUpdate] + sum[Launch::TcUpdate];
        F->phases.pivot_block_ms = sum[Launch::PivotBlock] + sum[Launch::DiagBlock];
        F->phases.schur_tensor_ms = sum[Launch::TcUpdate];
    }
}

// Raises the dynamic shared-memory limits of every kernel a factorisation of
// this configuration launches (done once, before any stream capture).  The
// small-front kernel gets the limit of its largest bucket: the attribute is a
// per-function maximum shared by every factor, so it never goes down.
void prepare_factor_kernels(uchol_factor_s* F) {
    const int small = (int)((size_t)kSmallFrontLimit * kSmallFrontLimit * sizeof(double));
    if (F->elem == 8) {
        CK(cudaFuncSetAttribute(k_small_fronts<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, std::max(small, 1)));
        CK(cudaFuncSetAttribute(k_invert_blocks<double, double, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(2 * 64 * 64 * sizeof(double))));
        CK(cudaFuncSetAttribute(k_inv_offdiag<double, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_offdiag_smem<double, 64>()));
    } else {
        CK(cudaFuncSetAttribute(k_small_fronts<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, std::max(small, 1)));
        CK(cudaFuncSetAttribute(k_invert_blocks<float, float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(2 * 128 * 128 * sizeof(float))));
        CK(cudaFuncSetAttribute(k_inv_offdiag<float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_offdiag_smem<float, 128>()));
        CK(cudaFuncSetAttribute(k_diag_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDiagSmemBytes));
        CK(cudaFuncSetAttribute(k_panel_solve<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kPanelSmemBytes));
        CK(cudaFuncSetAttribute(k_panel_solve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemBytes));
        CK(cudaFuncSetAttribute(k_tc_gemm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
        CK(cudaFuncSetAttribute(k_tc_gemm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
    }
}

// Inverses of the diagonal blocks used by the solves (FP64 factor: FP64,
// 64-wide blocks; FP32 factor: FP32, 128-wide blocks).
void invert_diagonal_blocks(uchol_factor_s* F, cudaStream_t st) {
    DevPlan& D = *F->dp;
    const Plan& P = D.plan;
    const int nb = (int)P.inv_blocks.size();
    if (nb == 0) return;
    if (F->elem == 8) {
        constexpr int SB = 64;
        const size_t smem = 2 * SB * SB * sizeof(double);
        k_invert_blocks<double, double, SB><<<nb, SB, smem, st>>>(D.inv_blocks.as<SolveBlockTask>(), D.sn.as<SnDev>(),
                                                                  F->panel.as<double>(), F->linv.as<double>());
        // inverse fronts: off-diagonal blocks of the inverse, one launch per block diagonal
        for (const InvLaunch& L : P.inv_launches) {
            k_inv_offdiag<double, SB><<<L.count, 256, inv_offdiag_smem<double, SB>(), st>>>(
                D.inv_tasks.as<SolveBlockTask>() + L.begin, D.sn.as<SnDev>(), F->panel.as<double>(),
                F->linv.as<double>(), F->linv_off.as<double>());
            counted();
        }
    } else {
        constexpr int SB = 128;
        const size_t smem = 2 * SB * SB * sizeof(float);
        k_invert_blocks<float, float, SB><<<nb, SB, smem, st>>>(D.inv_blocks.as<SolveBlockTask>(), D.sn.as<SnDev>(),
                                                                F->panel.as<float>(), F->linv.as<float>());
        for (const InvLaunch& L : P.inv_launches) {
            k_inv_offdiag<float, SB><<<L.count, 256, inv_offdiag_smem<float, SB>(), st>>>(
                D.inv_tasks.as<SolveBlockTask>() + L.begin, D.sn.as<SnDev>(), F->panel.as<float>(),
                F->linv.as<float>(), F->linv_off.as<float>());
            counted();
        }
    }
    counted();
    CK(cudaGetLastError());
}

// Full-matrix product structure (both triangles) for the FP64 residual.
void build_full_csr(uchol_symbolic_s* S) {
    const int n = S->n;
    std::vector<int> cnt(n + 1, 0);
    for (int r = 0; r < n; ++r)
        for (int k = S->row_ptr[r]; k < S->row_ptr[r + 1]; ++k) {
            int c = S->col[k];
            cnt[r + 1]++;
            if (c != r) cnt[c + 1]++;
        }
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> fcol(cnt[n]), fsrc(cnt[n]);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int r = 0; r < n; ++r)
        for (int k = S->row_ptr[r]; k < S->row_ptr[r + 1]; ++k) {
            int c = S->col[k];
            fcol[fill[r]] = c;
            fsrc[fill[r]++] = k;
            if (c != r) {
                fcol[fill[c]] = r;
                fsrc[fill[c]++] = k;
            }
        }
    S->full_nnz = cnt[n];
    S->d_full_ptr.upload(cnt, S->stream, "product structure");
    S->d_full_col.upload(fcol, S->stream, "product structure");
    S->d_full_src.upload(fsrc, S->stream, "product structure");
}

// Every device operation of one numeric factorisation after the values are
// in place: statistics reset, diagonal scale, product values, assembly,
// the planned launches and the inverses of the diagonal blocks.
void enqueue_factorization(uchol_factor_s* F, cudaStream_t st) {
    uchol_symbolic_s* S = F->sym;
    PivotStats* stats = F->stats.as<PivotStats>();
    CK(cudaMemsetAsync(stats, 0, sizeof(PivotStats), st));
    if (S->n > 0) {
        k_diag_scale<<<grid_for(S->n, 256), 256, 0, st>>>(F->values.as<double>(), S->d_diag_idx.as<int>(), S->n, stats);
        counted();
    }
    k_finish_scale<<<1, 1, 0, st>>>(stats, F->ctl.as<FactorCtl>(), F->opts.pivot_tolerance,
                                    F->opts.diagonal_regularization, F->opts.allow_diagonal_regularization);
    counted();
    if (S->full_nnz > 0)
        k_gather_values<<<grid_for(S->full_nnz, 256), 256, 0, st>>>(F->values.as<double>(), S->d_full_src.as<int>(),
                                                                     S->full_nnz, F->full_val.as<double>());
    if (S->full_nnz > 0) counted();
    if (S->count > 0) {
        CK(cudaMemsetAsync(F->panel.p, 0, F->panel.bytes, st));
        // arrival counts of K-split tiles start at zero (also after a factorisation that timed out)
        if (F->tc_counters.p) CK(cudaMemsetAsync(F->tc_counters.p, 0, F->tc_counters.bytes, st));
        if (F->elem == 8)
            k_assemble<double><<<grid_for(S->nnz, 256), 256, 0, st>>>(F->values.as<double>(), F->dp->asm_pos.as<long long>(),
                                                                      S->nnz, F->panel.as<double>());
        else
            k_assemble<float><<<grid_for(S->nnz, 256), 256, 0, st>>>(F->values.as<double>(), F->dp->asm_pos.as<long long>(),
                                                                     S->nnz, F->panel.as<float>());
        counted();
        if (F->elem == 8) run_factor_launches<double>(F, st);
        else run_factor_launches<float>(F, st);
        invert_diagonal_blocks(F, st);
    }
}

// Kernel nodes of a captured factorisation: the side-stream extend-add at the lowest
// priority, every other kernel at the highest, so that CTAs of the latency-bound chain
// (diagonal blocks, panel solves, own-column updates) are scheduled before pending
// extend-add CTAs.
cudaError_t prioritise_main_stream(cudaGraph_t g) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    size_t count = 0;
    if ((e = cudaGraphGetNodes(g, nullptr, &count)) != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> nodes(count);
    if ((e = cudaGraphGetNodes(g, nodes.data(), &count)) != cudaSuccess) return e;
    const void* side_f = reinterpret_cast<const void*>(&k_extend_add<float, true>);
    const void* side_d = reinterpret_cast<const void*>(&k_extend_add<double, true>);
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType type;
        if ((e = cudaGraphNodeGetType(nd, &type)) != cudaSuccess) return e;
        if (type != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        if ((e = cudaGraphKernelNodeGetParams(nd, &kp)) != cudaSuccess) return e;
        cudaLaunchAttributeValue v;
        memset(&v, 0, sizeof(v));
        v.priority = (kp.func == side_f || kp.func == side_d) ? least : greatest;
        if ((e = cudaGraphKernelNodeSetAttribute(nd, cudaLaunchAttributePriority, &v)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void factorize_impl(uchol_factor_s* F, const double* values, bool on_device) {
    uchol_symbolic_s* S = F->sym;
    cudaStream_t st = S->stream;
    const Plan& P = F->dp->plan;
    // the whole launch sequence is captured once per factor and replayed:
    // refactorisations with the same pattern cost one graph launch.  The capture
    // (host work) and the graph's upload come before the timed region, so that
    // factor_ms of a first factorisation equals that of a refactorisation.
    if (!phase_timing() && !F->factor_graph) {
        if (!F->capture_stream) CK(cudaStreamCreateWithFlags(&F->capture_stream, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        const long long before = g_launches.load();
        CK(cudaStreamBeginCapture(F->capture_stream, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_factorization(F, F->capture_stream);
        } catch (...) {
            cudaStreamEndCapture(F->capture_stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        CK(cudaStreamEndCapture(F->capture_stream, &g));
        F->factor_graph_nodes = (int)(g_launches.load() - before);
        g_launches -= F->factor_graph_nodes;   // counted when the graph runs
        unsigned long long flags = 0;
        if (F->side_stream) {
            cudaError_t pe = prioritise_main_stream(g);
            if (pe != cudaSuccess) {
                cudaGraphDestroy(g);
                CK(pe);
            }
            flags = cudaGraphInstantiateFlagUseNodePriority;
        }
        cudaError_t e = cudaGraphInstantiateWithFlags(&F->factor_graph, g, flags);
        cudaGraphDestroy(g);
        CK(e);
        CK(cudaGraphUpload(F->factor_graph, st));
    }
    StreamTimer total(st);
    if (on_device)
        CK(cudaMemcpyAsync(F->values.p, values, (size_t)S->nnz * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else
        CK(cudaMemcpyAsync(F->values.p, values, (size_t)S->nnz * sizeof(double), cudaMemcpyHostToDevice, st));
    PivotStats* stats = F->stats.as<PivotStats>();
    if (phase_timing()) {
        enqueue_factorization(F, st);   // direct launches, one event pair each
    } else {
        CK(cudaGraphLaunch(F->factor_graph, st));
        counted(F->factor_graph_nodes);
    }
    PivotStats hs;
    CK(cudaMemcpyAsync(&hs, stats, sizeof(PivotStats), cudaMemcpyDeviceToHost, st));
    double ms = total.stop();
    (void)P;
    uchol_factor_stats& o = F->last;
    o.regularized_pivot_count = hs.regularized;
    o.negative_pivot_count = hs.negative;
    o.smallest_pivot_magnitude = S->count ? __builtin_bit_cast(double, hs.min_bits) : 0.0;
    o.largest_pivot_magnitude = S->count ? __builtin_bit_cast(double, hs.max_bits) : 0.0;
    if (S->count == 0) o.smallest_pivot_magnitude = o.largest_pivot_magnitude = 0.0;
    o.failed_pivot = hs.failed == INT_MAX ? -1 : hs.failed;
    o.factor_ms = ms;
    o.device_bytes = (int64_t)(F->panel.bytes + F->contrib.bytes + F->stage_a.bytes + F->stage_b.bytes + F->diag.bytes +
                               F->values.bytes + F->full_val.bytes);
    F->phases.total_ms = ms;
    if (hs.status != 0)
        throw Error(UCHOL_TIMEOUT, "a bounded device wait expired during the factorization (status " +
                                       std::to_string(hs.status) + ")");
    if (o.failed_pivot >= 0)
        throw Error(UCHOL_NOT_SPD, "Pivot in equation " + std::to_string(o.failed_pivot) +
                                       " (in elimination order) is not positive: the matrix is not positive definite. "
                                       "Enable diagonal regularization if factorization must be completed.");
}

void check_options(const uchol_options* o) {
    if (!o) return;
    if (o->precision < UCHOL_PRECISION_FP64 || o->precision > UCHOL_PRECISION_BF16)
        throw Error(UCHOL_BAD_ARG, "unknown precision mode");
    if (!(o->pivot_tolerance >= 0.0) || !(o->diagonal_regularization > 0.0))
        throw Error(UCHOL_BAD_ARG, "pivot tolerance must be >= 0 and regularization > 0");
    if (o->device_memory_budget < 0) throw Error(UCHOL_BAD_ARG, "the device memory budget must be >= 0");
    if (!(o->chain_merge_fill >= 0.0) || o->chain_merge_fill > 10.0)
        throw Error(UCHOL_BAD_ARG, "chain_merge_fill must be in [0, 10]");
    if (o->small_front_buckets < 0 || o->small_front_buckets >= (1 << kSmallBuckets))
        throw Error(UCHOL_BAD_ARG, "small_front_buckets has bits beyond the " + std::to_string(kSmallBuckets) +
                                       " front-size buckets");
}

uchol_factor_s* create_factor(uchol_symbolic_s* S, int n, int nnz, const uchol_options* opts) {
    if (!S) throw Error(UCHOL_BAD_ARG, "symbolic handle is null");
    if (n != S->n)
        throw Error(UCHOL_PATTERN_MISMATCH, "Matrix size " + std::to_string(n) +
                                                " does not match the symbolic factorization built for " +
                                                std::to_string(S->n) + " equations.");
    if (nnz != S->nnz)
        throw Error(UCHOL_PATTERN_MISMATCH,
                    "The matrix sparse structure has changed since symbolic analysis (previously " +
                        std::to_string(S->nnz) + " nonzero elements, now " + std::to_string(nnz) +
                        "). Symbolic factorization can be reused only when the structure is unchanged. Run Analyze again.");
    check_options(opts);
    auto F = std::make_unique<uchol_factor_s>();
    F->sym = S;
    S->refs.fetch_add(1);
    if (opts) F->opts = *opts; else uchol_default_options(&F->opts);
    F->precision = F->opts.precision;
    F->elem = F->precision == UCHOL_PRECISION_FP64 ? 8 : 4;
    PlanConfig cfg = config_for(F->opts);
    CK(cudaDeviceGetAttribute(&F->sms, cudaDevAttrMultiProcessorCount, S->device));
    cfg.sms = F->sms;
    F->dp = S->get_plan(cfg, F->precision, F->opts.device_memory_budget);
    const Plan& P = F->dp->plan;
    cudaStream_t st = S->stream;
    F->panel.alloc((size_t)P.factor_elems * F->elem, "factor panels");
    F->contrib.alloc((size_t)P.contrib_elems * F->elem, "contribution blocks");
    bool side = false;
    for (const Launch& L : P.launches) side |= L.stream == 1;
    if (side) {
        CK(cudaStreamCreateWithFlags(&F->side_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&F->fork_ev, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&F->join_ev, cudaEventDisableTiming));
    }
    if (cfg.tensor_core && P.stage_elems > 0) {
        const bool bf16 = F->precision == UCHOL_PRECISION_BF16;
        const size_t op = bf16 ? 2 : 4;
        F->stage_a.alloc((size_t)P.stage_elems * op, "operand staging");
        F->stage_b.alloc((size_t)P.stage_elems * op, "operand staging");
        CK(cudaMemsetAsync(F->stage_a.p, 0, F->stage_a.bytes, st));
        CK(cudaMemsetAsync(F->stage_b.p, 0, F->stage_b.bytes, st));
        std::vector<CUtensorMap> maps(2 * P.map_front.size());
        for (size_t k = 0; k < P.map_front.size(); ++k) {
            const int s = P.map_front[k];
            const StageInfo& g = P.stage[s];
            try {
                make_stage_maps(bf16, (char*)F->stage_a.p + g.off * op, (char*)F->stage_b.p + g.off * op, P.sn[s].m,
                                g.ld, &maps[2 * k]);
            } catch (const std::runtime_error& e) {
                throw Error(UCHOL_CUDA_ERROR, e.what());
            }
        }
        F->maps.upload(maps, st, "tensor maps");
        F->tc_ws.alloc(tc_ws_floats(F->sms) * sizeof(float), "K-split workspace");
        F->tc_counters.alloc(tc_counter_count(F->sms) * sizeof(int), "K-split workspace");
        CK(cudaMemsetAsync(F->tc_counters.p, 0, F->tc_counters.bytes, st));
        CK(cudaStreamSynchronize(st));
    }
    if (cfg.tensor_core)
        F->minv.alloc((size_t)std::max(1, P.diag_slots) * kMinvStride * sizeof(float), "diagonal-block inverses");
    F->diag.alloc((size_t)std::max(1, S->n) * sizeof(double), "pivots");
    F->linv.alloc((size_t)std::max<size_t>(1, P.inv_blocks.size()) * cfg.solve_block * cfg.solve_block * F->elem,
                  "inverse diagonal blocks");
    F->linv_off.alloc((size_t)std::max<long long>(1, P.inv_off_blocks) * cfg.solve_block * cfg.solve_block * F->elem,
                      "inverse blocks of the inverse fronts");
    F->values.alloc((size_t)std::max(1, S->nnz) * sizeof(double), "matrix values");
    F->full_val.alloc((size_t)std::max<long long>(1, S->full_nnz) * sizeof(double), "matrix values");
    F->stats.alloc(sizeof(PivotStats), "statistics");
    F->ctl.alloc(sizeof(FactorCtl), "statistics");
    prepare_factor_kernels(F.get());
    return F.release();
}

// ---- solves ----

// Cooperative launch: every CTA of the grid is resident at once (the level
// solve kernels wait on one another), or the launch fails.
template <class... KArgs, class... Args>
void launch_cooperative(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelEx(&cfg, kernel, args...));
}

// Reports an expired bounded wait of the level solve kernels (after a synchronisation).
void check_solve_status(uchol_factor_s* F) {
    if (!F->solve_status.p) return;
    int h = 0;
    CK(cudaMemcpy(&h, F->solve_status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h != 0) {
        CK(cudaMemset(F->solve_status.p, 0, sizeof(int)));
        throw Error(UCHOL_TIMEOUT, "a bounded device wait expired during a triangular solve (status " +
                                       std::to_string(h) + ")");
    }
}

// RG: right-hand sides the level kernels and the backward column dots carry together.
// Optional per-launch device timing of a solve (direct launches, one event pair each).
struct SolveTimer {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    std::vector<int> kind;
    void begin(int k, cudaStream_t st) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        CK(cudaEventRecord(a, st));
        ev.push_back({a, b});
        kind.push_back(k);
    }
    void end(cudaStream_t st) { CK(cudaEventRecord(ev.back().second, st)); }
    // sums per launch kind into t (after the stream has completed)
    void collect(uchol_phase_times& t) {
        for (double& v : t.solve_kind_ms) v = 0.0;
        t.solve_total_ms = 0.0;
        t.solve_launches = (int)ev.size();
        for (size_t q = 0; q < ev.size(); ++q) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[q].first, ev[q].second));
            if (kind[q] >= 0 && kind[q] < UCHOL_SOLVE_KINDS) t.solve_kind_ms[kind[q]] += ms;
            t.solve_total_ms += ms;
        }
    }
    ~SolveTimer() {
        for (auto& e : ev) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
    }
};

SolveArgs solve_args(uchol_factor_s* F, int nrhs) {
    DevPlan& D = *F->dp;
    SolveArgs A;
    A.sn = D.sn.as<SnDev>();
    A.rel = D.rel.as<int>();
    A.rows = D.rows.as<int>();
    A.child_ptr = D.child_ptr.as<int>();
    A.children = D.children.as<int>();
    A.fvec_off = D.fvec_off.as<long long>();
    A.fv_stride = D.plan.fvec_elems;
    A.n = F->sym->n;
    A.nrhs = nrhs;
    A.ldw = F->sym->n;
    return A;
}

// RG: right-hand sides the level kernels and the backward column dots carry together.
template <class T, class Cv, int SB, int RG>
void run_solve(uchol_factor_s* F, int nrhs, Cv* work, Cv* fv, Cv* fv2, cudaStream_t st, SolveTimer* timer = nullptr) {
    DevPlan& D = *F->dp;
    const Plan& P = D.plan;
    const SolveArgs A = solve_args(F, nrhs);
    const T* panel = F->panel.as<T>();
    const Cv* linv = F->linv.as<Cv>();
    const SolveBlockTask* tasks = D.solve_tasks.as<SolveBlockTask>();
    const double* diag = F->diag.as<double>();
    const int nblocks = (int)P.inv_blocks.size();
    int* fwd_flags = F->solve_flags.as<int>();
    int* bwd_flags = fwd_flags + nblocks;
    int* progress = bwd_flags + nblocks;
    int* status = F->solve_status.as<int>();
    CK(cudaMemsetAsync(fwd_flags, 0, sizeof(int) * ((size_t)2 * nblocks + P.progress_count), st));
    const size_t smem = level_smem_bytes<T, Cv, SB, RG>();
    constexpr int RGD = RG == 1 ? 1 : 8;   // right-hand sides per CTA of the inverse-front diagonal kernels
    auto level_args = [&](const SolveLaunch& L, int* flags, int grid) {
        LevelArgs la;
        la.chains = tasks + L.begin;
        la.nchains = L.count;
        la.bulk = tasks + L.bulk_begin;
        la.nbulk = L.bulk_count;
        // CTAs split between chains and bulk in proportion to their work (a block solve counted as
        // two chunk updates), each side at least one
        const double share = 2.0 * L.chain_work / std::max(1.0, 2.0 * L.chain_work + (double)L.bulk_work);
        const int want = std::max(L.long_chains, (int)std::lround(grid * share));
        la.nchain_cta = std::max(1, std::min({L.count, grid - 1, want}));
        // bulk CTAs split between the diagonal-block chunks (which the chains wait for: weighted
        // up) and the trailing-row chunks
        const int nbulk_cta = grid - la.nchain_cta;
        const long long trail_work = L.bulk_work - L.diag_work;
        la.ndiag = L.ndiag;
        if (L.ndiag == 0) {
            la.ndiag_cta = 0;
        } else if (L.ndiag == L.bulk_count) {
            la.ndiag_cta = nbulk_cta;
        } else {
            const double dshare = 2.0 * L.diag_work / std::max(1.0, 2.0 * L.diag_work + (double)trail_work);
            la.ndiag_cta = std::max(1, std::min(nbulk_cta - 1, (int)std::lround(nbulk_cta * dshare)));
        }
        la.steps = L.steps;
        la.flags = flags;
        la.progress = progress + L.progress_off;
        la.status = status;
        la.maps = F->solve_maps.as<CUtensorMap>();
        return la;
    };
    for (const SolveLaunch& L : P.fwd_launches) {
        if (L.count == 0) continue;
        if (timer) timer->begin((int)L.kind, st);
        if (L.kind == SolveLaunch::FwdGather) {
            k_fwd_gather<Cv><<<dim3(L.count, std::min(nrhs, 65535)), 256, 0, st>>>(tasks + L.begin, A, work, fv);
        } else if (L.kind == SolveLaunch::FwdSolo) {
            k_fwd_solo<T, Cv, SB><<<L.count, 256, 0, st>>>(tasks + L.begin, A, panel, linv, fv, fv2, diag, work);
        } else if (L.kind == SolveLaunch::FwdInvDiag) {
            k_fwd_inv_diag<T, Cv, SB, RGD><<<dim3(L.count, (nrhs + RGD - 1) / RGD), 256, inv_solve_smem<T, Cv, SB, RGD>(), st>>>(
                tasks + L.begin, A, linv, F->linv_off.as<Cv>(), fv, fv2, diag, work, F->inv_diag_partial.as<Cv>(),
                F->inv_diag_cnt.as<unsigned>(), status);
        } else if (L.kind == SolveLaunch::FwdInvTail) {
            k_fwd_inv_tail<T, Cv, SB, RG><<<L.count, 256, inv_tail_smem<T, Cv, SB, RG, false>(), st>>>(
                tasks + L.begin, A, F->solve_maps.as<CUtensorMap>() + P.count, fv2, fv, status);
        } else if (L.kind == SolveLaunch::FwdTail) {
            if (nrhs == 1)
                k_fwd_tail<T, Cv, SB, 1><<<L.count, kTailRows / 4, 0, st>>>(tasks + L.begin, A, panel, fv2, fv);
            else
                k_fwd_tail<T, Cv, SB, 4><<<L.count, kTailRows / 4, 0, st>>>(tasks + L.begin, A, panel, fv2, fv);
        } else {
            const int grid = F->coop_fwd;
            launch_cooperative(k_fwd_level<T, Cv, SB, RG>, grid, 256, smem, st, level_args(L, fwd_flags, grid), A, panel,
                               linv, fv, fv2, diag, work);
        }
        if (timer) timer->end(st);
    }
    for (const SolveLaunch& L : P.bwd_launches) {
        if (L.count == 0) continue;
        if (timer) timer->begin((int)L.kind, st);
        if (L.kind == SolveLaunch::BwdGather) {
            k_bwd_gather<Cv><<<dim3(L.count, std::min(nrhs, 65535)), 256, 0, st>>>(tasks + L.begin, A, work, fv);
        } else if (L.kind == SolveLaunch::BwdTail) {
            k_bwd_cols<T, Cv, RG><<<L.count, 256, 0, st>>>(tasks + L.begin, A, panel, fv, F->bwd_partial.as<Cv>());
        } else if (L.kind == SolveLaunch::BwdTailReduce) {
            k_bwd_cols_reduce<Cv><<<L.count, 128, 0, st>>>(tasks + L.begin, A, F->bwd_partial.as<Cv>(), fv);
        } else if (L.kind == SolveLaunch::BwdInvCols) {
            k_bwd_inv_cols<T, Cv, SB, RG><<<L.count, 256, inv_tail_smem<T, Cv, SB, RG, true>(), st>>>(
                tasks + L.begin, A, F->solve_maps.as<CUtensorMap>() + 2 * P.count, fv, F->inv_partial.as<Cv>(), status);
        } else if (L.kind == SolveLaunch::BwdInvReduce) {
            k_bwd_inv_reduce<Cv, SB><<<dim3(L.count, std::min(nrhs, 65535)), SB, 0, st>>>(tasks + L.begin, A, fv,
                                                                                        F->inv_partial.as<Cv>());
        } else if (L.kind == SolveLaunch::BwdInvDiag) {
            k_bwd_inv_diag<T, Cv, SB, RGD><<<dim3(L.count, (nrhs + RGD - 1) / RGD), 256, inv_solve_smem<T, Cv, SB, RGD>(), st>>>(
                tasks + L.begin, A, linv, F->linv_off.as<Cv>(), fv, work, F->inv_diag_partial.as<Cv>(),
                F->inv_diag_cnt.as<unsigned>(), status);
        } else if (L.kind == SolveLaunch::BwdSolo) {
            k_bwd_solo<Cv, SB><<<L.count, 256, 0, st>>>(tasks + L.begin, A, linv, fv, fv2, work);
        } else {
            const int grid = F->coop_bwd;
            launch_cooperative(k_bwd_level<T, Cv, SB, RG>, grid, 256, smem, st, level_args(L, bwd_flags, grid), A, panel,
                               linv, fv, fv2, work);
        }
        if (timer) timer->end(st);
    }
    CK(cudaGetLastError());
}

static_assert(kTailRows == kTailRowsPlan, "forward tail chunk of the plan and the kernel");

int solve_launch_count(const Plan& P) {
    int c = 0;
    for (const SolveLaunch& L : P.fwd_launches) c += L.count > 0;
    for (const SolveLaunch& L : P.bwd_launches) c += L.count > 0;
    return c + 1;   // + the flag reset
}

// The triangular solves of a factor for nrhs columns, captured once into a
// CUDA graph over the factor's fixed work buffers and replayed on each call.
template <class T, class Cv, int SB>
void launch_solve_graph(uchol_factor_s* F, int nrhs, Cv* work, cudaStream_t st) {
    if (!F->solve_graph || F->solve_graph_nrhs != nrhs) {
        if (F->solve_graph) {
            CK(cudaGraphExecDestroy(F->solve_graph));
            F->solve_graph = nullptr;
        }
        if (!F->capture_stream) CK(cudaStreamCreateWithFlags(&F->capture_stream, cudaStreamNonBlocking));
        // the level kernels run as cooperative launches: at most as many CTAs as the device holds at once
        auto level_kernels = [&](auto* fwd, auto* bwd, int smem) {
            CK(cudaFuncSetAttribute(fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            CK(cudaFuncSetAttribute(bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            int per_sm = 0;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd, 256, smem));
            F->coop_fwd = per_sm * F->sms;
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bwd, 256, smem));
            F->coop_bwd = per_sm * F->sms;
        };
        if (nrhs == 1)
            level_kernels(k_fwd_level<T, Cv, SB, 1>, k_bwd_level<T, Cv, SB, 1>, (int)level_smem_bytes<T, Cv, SB, 1>());
        else
            level_kernels(k_fwd_level<T, Cv, SB, kSolveRhsGroup>, k_bwd_level<T, Cv, SB, kSolveRhsGroup>,
                          (int)level_smem_bytes<T, Cv, SB, kSolveRhsGroup>());
        // inverse-front kernels of both groupings
        CK(cudaFuncSetAttribute(k_fwd_inv_diag<T, Cv, SB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_solve_smem<T, Cv, SB, 1>()));
        CK(cudaFuncSetAttribute(k_fwd_inv_diag<T, Cv, SB, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_solve_smem<T, Cv, SB, 8>()));
        CK(cudaFuncSetAttribute(k_bwd_inv_diag<T, Cv, SB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_solve_smem<T, Cv, SB, 1>()));
        CK(cudaFuncSetAttribute(k_bwd_inv_diag<T, Cv, SB, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_solve_smem<T, Cv, SB, 8>()));
        CK(cudaFuncSetAttribute(k_fwd_inv_tail<T, Cv, SB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_tail_smem<T, Cv, SB, 1, false>()));
        CK(cudaFuncSetAttribute(k_fwd_inv_tail<T, Cv, SB, kSolveRhsGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_tail_smem<T, Cv, SB, kSolveRhsGroup, false>()));
        CK(cudaFuncSetAttribute(k_bwd_inv_cols<T, Cv, SB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_tail_smem<T, Cv, SB, 1, true>()));
        CK(cudaFuncSetAttribute(k_bwd_inv_cols<T, Cv, SB, kSolveRhsGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)inv_tail_smem<T, Cv, SB, kSolveRhsGroup, true>()));
        if (F->coop_fwd < 2 || F->coop_bwd < 2) throw Error(UCHOL_CUDA_ERROR, "the level solve kernels do not fit");
        if (!F->solve_maps.p) {
            // tile copies of the solves: each front's panel (m x w), in boxes of SB x SB (level
            // kernels), SB x SB/2 and SB/2 x SB (half tiles of the inverse-front kernels)
            const Plan& P = F->dp->plan;
            const size_t nf = P.sn.size();
            std::vector<CUtensorMap> maps(std::max<size_t>(1, 3 * nf));
            std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
            const size_t es = sizeof(T);
            const cuuint32_t boxes[3][2] = {{(cuuint32_t)SB, (cuuint32_t)SB}, {(cuuint32_t)SB, (cuuint32_t)(SB / 2)},
                                            {(cuuint32_t)(SB / 2), (cuuint32_t)SB}};
            for (int kind = 0; kind < 3; ++kind)
                for (size_t s2 = 0; s2 < nf; ++s2) {
                    const SnDev& d = P.sn[s2];   // every front: its trailing rows are bulk tiles too
                    cuuint64_t dims[2] = {(cuuint64_t)d.m, (cuuint64_t)d.w};
                    cuuint64_t strides[1] = {(cuuint64_t)d.ldp * es};
                    cuuint32_t box[2] = {boxes[kind][0], boxes[kind][1]};
                    cuuint32_t estr[2] = {1, 1};
                    CUresult r = tensor_map_encoder()(&maps[kind * nf + s2],
                                                      es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                                                      2, (char*)F->panel.p + (size_t)d.panel_off * es, dims, strides, box,
                                                      estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
                    if (r != CUDA_SUCCESS)
                        throw Error(UCHOL_CUDA_ERROR,
                                    "cuTensorMapEncodeTiled failed for a solve tile map: " + std::to_string((int)r));
                }
            F->solve_maps.upload(maps, st, "solve tile maps");
            CK(cudaStreamSynchronize(st));
        }
        if (!F->solve_flags.p) {
            const Plan& P = F->dp->plan;
            F->solve_flags.alloc(sizeof(int) * (2 * std::max<size_t>(1, P.inv_blocks.size()) + P.progress_count),
                                 "solve flags");
            F->solve_status.alloc(sizeof(int), "solve flags");
            CK(cudaMemsetAsync(F->solve_status.p, 0, sizeof(int), st));
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(F->capture_stream, cudaStreamCaptureModeThreadLocal));
        try {
            if (nrhs == 1)
                run_solve<T, Cv, SB, 1>(F, nrhs, work, F->fv.as<Cv>(), F->fv2.as<Cv>(), F->capture_stream);
            else
                run_solve<T, Cv, SB, kSolveRhsGroup>(F, nrhs, work, F->fv.as<Cv>(), F->fv2.as<Cv>(), F->capture_stream);
        } catch (...) {
            cudaStreamEndCapture(F->capture_stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        CK(cudaStreamEndCapture(F->capture_stream, &g));
        cudaError_t e = cudaGraphInstantiate(&F->solve_graph, g, 0);
        cudaGraphDestroy(g);
        CK(e);
        F->solve_graph_nrhs = nrhs;
        F->solve_graph_nodes = solve_launch_count(F->dp->plan);
    }
    if (phase_timing()) {
        // direct launches with one event pair each (the graph above stays for untimed calls)
        SolveTimer timer;
        if (nrhs == 1)
            run_solve<T, Cv, SB, 1>(F, nrhs, work, F->fv.as<Cv>(), F->fv2.as<Cv>(), st, &timer);
        else
            run_solve<T, Cv, SB, kSolveRhsGroup>(F, nrhs, work, F->fv.as<Cv>(), F->fv2.as<Cv>(), st, &timer);
        CK(cudaStreamSynchronize(st));
        timer.collect(F->phases);
        counted(F->solve_graph_nodes);
        return;
    }
    CK(cudaGraphLaunch(F->solve_graph, st));
    counted(F->solve_graph_nodes);
}

void ensure_workspace(uchol_factor_s* F, int nrhs);

// Failure check of the bounded waits: the plan's first forward level launch whose front has
// three or more diagonal blocks, with every CTA a chain CTA, so that the chains' waits for the
// bulk CTAs' progress counters can only expire.  The solve set-up (workspace, tile maps, flags,
// kernel attributes) is that of a one-column solve, made first.
template <class T, class Cv, int SB>
void starved_level_launch(uchol_factor_s* F, cudaStream_t st) {
    DevPlan& D = *F->dp;
    const Plan& P = D.plan;
    const SolveLaunch* Lp = nullptr;
    for (const SolveLaunch& L : P.fwd_launches)
        if (L.kind == SolveLaunch::FwdLevel && L.steps >= 3 && L.count > 0) {
            Lp = &L;
            break;
        }
    if (!Lp)
        throw Error(UCHOL_BAD_ARG, "the factor has no level-solve launch with a chain of three diagonal blocks "
                                   "(use inverse_block_width < 0 and a front wider than three solve blocks)");
    ensure_workspace(F, 1);
    CK(cudaMemsetAsync(F->work.p, 0, F->work.bytes, st));
    launch_solve_graph<T, Cv, SB>(F, 1, F->work.as<Cv>(), st);   // set-up, and a normal solve of zeros
    CK(cudaStreamSynchronize(st));
    const SolveBlockTask* tasks = D.solve_tasks.as<SolveBlockTask>();
    const int nblocks = (int)P.inv_blocks.size();
    int* fwd_flags = F->solve_flags.as<int>();
    int* progress = fwd_flags + 2 * nblocks;
    CK(cudaMemsetAsync(fwd_flags, 0, sizeof(int) * ((size_t)2 * nblocks + P.progress_count), st));
    const int grid = std::max(1, std::min(Lp->count, F->coop_fwd));
    LevelArgs la;
    la.chains = tasks + Lp->begin;
    la.nchains = Lp->count;
    la.bulk = tasks + Lp->bulk_begin;
    la.nbulk = Lp->bulk_count;
    la.nchain_cta = grid;   // no bulk CTA: the progress counters never move
    la.ndiag = Lp->ndiag;
    la.ndiag_cta = 0;
    la.steps = Lp->steps;
    la.flags = fwd_flags;
    la.progress = progress + Lp->progress_off;
    la.status = F->solve_status.as<int>();
    la.maps = F->solve_maps.as<CUtensorMap>();
    launch_cooperative(k_fwd_level<T, Cv, SB, 1>, grid, 256, level_smem_bytes<T, Cv, SB, 1>(), st, la,
                       solve_args(F, 1), F->panel.as<T>(), F->linv.as<Cv>(), F->fv.as<Cv>(), F->fv2.as<Cv>(),
                       F->diag.as<double>(), F->work.as<Cv>());
    counted();
    CK(cudaStreamSynchronize(st));
}

void ensure_workspace(uchol_factor_s* F, int nrhs) {
    if (F->ws_nrhs >= nrhs) return;
    uchol_symbolic_s* S = F->sym;
    const Plan& P = F->dp->plan;
    size_t cv = F->precision == UCHOL_PRECISION_FP64 ? 8 : 4;
    F->work.alloc((size_t)std::max(1, S->n) * nrhs * cv, "solve workspace");
    F->fv.alloc((size_t)P.fvec_elems * nrhs * cv, "solve workspace");
    F->fv2.alloc((size_t)P.fvec_elems * nrhs * cv, "solve workspace");
    F->bwd_partial.alloc((size_t)std::max(1, P.bwd_partial_slots) * 8 * nrhs * cv, "solve workspace");
    F->inv_partial.alloc((size_t)std::max(1, P.inv_partial_slots) * P.cfg.solve_block * nrhs * cv, "solve workspace");
    F->inv_diag_partial.alloc((size_t)std::max(1, P.inv_diag_slots) * P.cfg.solve_block * nrhs * cv, "solve workspace");
    F->inv_diag_cnt.alloc((size_t)std::max(1, P.inv_diag_slots) * nrhs * sizeof(unsigned), "solve workspace");
    CK(cudaMemsetAsync(F->inv_diag_cnt.p, 0, F->inv_diag_cnt.bytes, S->stream));   // the last chunk resets each
    if (F->solve_graph) {
        CK(cudaGraphExecDestroy(F->solve_graph));
        F->solve_graph = nullptr;
    }
    for (auto& v : F->vec) v.alloc((size_t)std::max(1, S->n) * nrhs * sizeof(double), "refinement vectors");
    F->scal.alloc((size_t)(kDotBlocks * nrhs + 16 * nrhs) * sizeof(double), "refinement scalars");
    F->ws_nrhs = nrhs;
}

// x = A^-1 b through the factor only (device buffers, original order).
void apply_factor(uchol_factor_s* F, int nrhs, const double* b, int ldb, double* x, int ldx) {
    uchol_symbolic_s* S = F->sym;
    cudaStream_t st = S->stream;
    const int n = S->n;
    if (n == 0) return;
    dim3 g(grid_for(n, 256, 1024), std::min(nrhs, 65535));
    if (F->precision == UCHOL_PRECISION_FP64) {
        double* work = F->work.as<double>();
        k_permute_in<double><<<g, 256, 0, st>>>(b, ldb, S->d_perm.as<int>(), n, nrhs, work, n);
        if (S->count) launch_solve_graph<double, double, 64>(F, nrhs, work, st);
        k_permute_out<double><<<g, 256, 0, st>>>(work, n, S->d_perm.as<int>(), n, nrhs, x, ldx);
        counted(2);
    } else {
        float* work = F->work.as<float>();
        k_permute_in<float><<<g, 256, 0, st>>>(b, ldb, S->d_perm.as<int>(), n, nrhs, work, n);
        if (S->count) launch_solve_graph<float, float, 128>(F, nrhs, work, st);
        k_permute_out<float><<<g, 256, 0, st>>>(work, n, S->d_perm.as<int>(), n, nrhs, x, ldx);
        counted(2);
    }
    CK(cudaGetLastError());
}

void residual(uchol_factor_s* F, int nrhs, const double* x, int ldx, const double* b, int ldb, double* r, int ldr) {
    uchol_symbolic_s* S = F->sym;
    if (S->n == 0) return;
    k_spmv_residual<<<(S->n + 7) / 8, 256, 0, S->stream>>>(S->d_full_ptr.as<int>(), S->d_full_col.as<int>(),
                                                          F->full_val.as<double>(), S->n, nrhs, x, ldx, b, ldb, r, ldr);
    counted();
}

// out[r] = u_r . v_r (deterministic two-stage reduction) on the device.
void dots(uchol_factor_s* F, int nrhs, const double* u, int ldu, const double* v, int ldv, double* out) {
    uchol_symbolic_s* S = F->sym;
    double* partial = F->scal.as<double>();
    dim3 g(kDotBlocks, nrhs);
    k_dot_partial<<<g, 256, 0, S->stream>>>(u, ldu, v, ldv, S->n, partial);
    k_dot_finish<<<1, 32 * ((nrhs + 31) / 32), 0, S->stream>>>(partial, kDotBlocks, nrhs, out);
    counted(2);
}

__global__ void k_fill(double* p, double v, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_cg_scalars(const double* num, const double* den, double* out, int nrhs) {
    int r = threadIdx.x;
    if (r < nrhs) out[r] = den[r] != 0.0 ? num[r] / den[r] : 0.0;
}

void solve_refined(uchol_factor_s* F, int nrhs, const double* b, int ldb, double* x, int ldx,
                   const uchol_refine_options* ro, uchol_refine_stats* rs) {
    uchol_symbolic_s* S = F->sym;
    cudaStream_t st = S->stream;
    const int n = S->n;
    ensure_workspace(F, nrhs);
    StreamTimer timer(st);
    uchol_refine_options opt{1e-10, 50, 0};
    if (ro) opt = *ro;
    int method = opt.method;
    if (method == 0)
        method = (F->precision == UCHOL_PRECISION_FP64 || F->last.regularized_pivot_count > 0) ? 1 : 2;
    if (n == 0) {
        if (rs) *rs = {0, 0.0, 0.0, timer.stop()};
        return;
    }
    double* r = F->vec[0].as<double>();
    double* z = F->vec[1].as<double>();
    double* p = F->vec[2].as<double>();
    double* q = F->vec[3].as<double>();
    double* sc = F->scal.as<double>() + kDotBlocks * nrhs;   // scalar area: 16 * nrhs doubles
    double* bnorm2 = sc, *rnorm2 = sc + nrhs, *rz = sc + 2 * nrhs, *rz_new = sc + 3 * nrhs, *pq = sc + 4 * nrhs;
    double* alpha = sc + 5 * nrhs, *beta = sc + 6 * nrhs;
    std::vector<double> hb(nrhs), hr(nrhs);
    dots(F, nrhs, b, ldb, b, ldb, bnorm2);
    CK(cudaMemcpyAsync(hb.data(), bnorm2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
    auto rel_max = [&]() {
        CK(cudaMemcpyAsync(hr.data(), rnorm2, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        double worst = 0.0;
        for (int j = 0; j < nrhs; ++j) {
            double nb = std::sqrt(hb[j]), nr = std::sqrt(hr[j]);
            const double rel = nb > 0.0 ? nr / nb : nr;
            if (!std::isfinite(rel)) return std::numeric_limits<double>::quiet_NaN();   // any column
            worst = std::max(worst, rel);
        }
        return worst;
    };
    dim3 g(grid_for(n, 256, 1024), nrhs);
    int it = 0;
    double initial = 0.0, current = 0.0;
    // x0 = M^-1 b
    apply_factor(F, nrhs, b, ldb, x, ldx);
    residual(F, nrhs, x, ldx, b, ldb, r, n);
    dots(F, nrhs, r, n, r, n, rnorm2);
    initial = current = rel_max();
    if (method == 1) {
        double* ones = sc + 15 * nrhs;
        k_fill<<<(nrhs + 31) / 32, 32, 0, st>>>(ones, 1.0, nrhs); counted();
        while (current > opt.tolerance && std::isfinite(current) && it < opt.max_iterations) {
            apply_factor(F, nrhs, r, n, z, n);
            k_axpy_cols<<<g, 256, 0, st>>>(x, ldx, z, n, ones, 1.0, n, nrhs); counted();
            residual(F, nrhs, x, ldx, b, ldb, r, n);
            dots(F, nrhs, r, n, r, n, rnorm2);
            current = rel_max();
            ++it;
        }
    } else {
        // Conjugate gradients on A preconditioned by the factor, started from x0.
        apply_factor(F, nrhs, r, n, z, n);
        CK(cudaMemcpyAsync(p, z, (size_t)n * nrhs * sizeof(double), cudaMemcpyDeviceToDevice, st));
        dots(F, nrhs, r, n, z, n, rz);
        while (current > opt.tolerance && std::isfinite(current) && it < opt.max_iterations) {
            residual(F, nrhs, p, n, nullptr, 0, q, n);   // q = A p
            dots(F, nrhs, p, n, q, n, pq);
            k_cg_scalars<<<1, 32 * ((nrhs + 31) / 32), 0, st>>>(rz, pq, alpha, nrhs); counted();
            k_axpy_cols<<<g, 256, 0, st>>>(x, ldx, p, n, alpha, 1.0, n, nrhs); counted();
            k_axpy_cols<<<g, 256, 0, st>>>(r, n, q, n, alpha, -1.0, n, nrhs); counted();
            ++it;
            // true residual for the stopping test (FP64 product, no drift)
            residual(F, nrhs, x, ldx, b, ldb, z, n);
            dots(F, nrhs, z, n, z, n, rnorm2);
            current = rel_max();
            if (current <= opt.tolerance) break;
            apply_factor(F, nrhs, r, n, z, n);
            dots(F, nrhs, r, n, z, n, rz_new);
            k_cg_scalars<<<1, 32 * ((nrhs + 31) / 32), 0, st>>>(rz_new, rz, beta, nrhs); counted();
            k_xpby_cols<<<g, 256, 0, st>>>(z, n, p, n, beta, n, nrhs); counted();
            CK(cudaMemcpyAsync(rz, rz_new, nrhs * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
    }
    CK(cudaGetLastError());
    double ms = timer.stop();
    check_solve_status(F);
    if (rs) *rs = {it, current, initial, ms};
    if (!std::isfinite(current))
        throw Error(UCHOL_NO_CONVERGENCE,
                    "refinement stopped after " + std::to_string(it) +
                        " steps: the residual is not finite (a non-finite right-hand side, or a reduced-precision "
                        "factor whose pivots broke down; refactorise with a higher precision)");
    if (current > opt.tolerance)
        throw Error(UCHOL_NO_CONVERGENCE, "refinement stopped at relative residual " + std::to_string(current) +
                                              " after " + std::to_string(it) + " steps (target " +
                                              std::to_string(opt.tolerance) + ")");
}

}  // namespace

extern "C" {

const char* uchol_last_error(void) { return g_error.c_str(); }

int64_t uchol_kernel_launches(void) { return g_launches.load(); }

void uchol_set_phase_timing(int on) { g_phase_timing.store(on ? 1 : 0); }

int uchol_set_wait_limits(double solve_ms, double factor_ms) {
    return guarded([&] {
        const unsigned long long s = solve_ms > 0.0 ? (unsigned long long)(solve_ms * 1e6) : kDefaultSolveWaitNs;
        const unsigned long long f = factor_ms > 0.0 ? (unsigned long long)(factor_ms * 1e6) : kDefaultFactorWaitNs;
        CK(cudaMemcpyToSymbol(g_solve_wait_ns, &s, sizeof(s)));
        CK(cudaMemcpyToSymbol(g_factor_wait_ns, &f, sizeof(f)));
    });
}

int uchol_check_solve_wait(uchol_factor f, double wait_ms) {
    return guarded([&] {
        if (!f) throw Error(UCHOL_BAD_ARG, "factor handle is null");
        if (!(wait_ms > 0.0)) throw Error(UCHOL_BAD_ARG, "the wait limit must be positive");
        std::lock_guard<std::mutex> lk(f->mu);
        cudaStream_t st = f->sym->stream;
        unsigned long long old = kDefaultSolveWaitNs;
        CK(cudaMemcpyFromSymbol(&old, g_solve_wait_ns, sizeof(old)));
        const unsigned long long lim = (unsigned long long)(wait_ms * 1e6);
        CK(cudaMemcpyToSymbol(g_solve_wait_ns, &lim, sizeof(lim)));
        try {
            if (f->precision == UCHOL_PRECISION_FP64) starved_level_launch<double, double, 64>(f, st);
            else starved_level_launch<float, float, 128>(f, st);
        } catch (...) {
            cudaMemcpyToSymbol(g_solve_wait_ns, &old, sizeof(old));
            throw;
        }
        CK(cudaMemcpyToSymbol(g_solve_wait_ns, &old, sizeof(old)));
        check_solve_status(f);   // UCHOL_TIMEOUT when the wait expired, status cleared
        throw Error(UCHOL_INTERNAL, "the starved level solve completed: its wait did not expire");
    });
}

void uchol_default_options(uchol_options* o) {
    if (!o) return;
    o->allow_diagonal_regularization = 1;
    o->pivot_tolerance = 1e-13;
    o->diagonal_regularization = 1e-10;
    o->panel_width = 32;
    o->precision = UCHOL_PRECISION_FP64;
    o->block_width = 0;
    o->small_front_buckets = 0;
    o->chain_merge_width = 0;
    o->inverse_block_width = 0;
    o->device_memory_budget = 0;
    o->split_min_kblocks = 0;
    o->extend_add_overlap = 0;
    o->chain_merge_fill = 0.0;
}

int uchol_symbolic_create(const uchol_symbolic_desc* d, uchol_symbolic* out) {
    return guarded([&] {
        if (!d || !out) throw Error(UCHOL_BAD_ARG, "null argument");
        *out = nullptr;
        const int n = d->n, nnz = d->nnz, count = d->supernode_count;
        if (n < 0 || nnz < 0 || count < 0) throw Error(UCHOL_BAD_ARG, "negative size");
        if (n > 0 && (!d->row_ptr || !d->col || !d->permutation || !d->diag_value_index || !d->pattern_ptr ||
                      !d->lower_start || !d->lower_value_ptr || !d->first_column || !d->parent || !d->child_ptr ||
                      !d->front_ptr))
            throw Error(UCHOL_BAD_ARG, "null symbolic array");
        if ((n == 0) != (count == 0)) throw Error(UCHOL_BAD_ARG, "supernode count inconsistent with the size");
        auto S = std::make_unique<uchol_symbolic_s>();
        CK(cudaGetDevice(&S->device));
        CK(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
        S->own_stream = true;
        S->n = n;
        S->nnz = nnz;
        S->count = count;
        auto cp = [](const int* p, long long len) { return p ? std::vector<int>(p, p + len) : std::vector<int>(); };
        if (n > 0) {
            S->row_ptr = cp(d->row_ptr, n + 1);
            if (S->row_ptr[0] != 0 || S->row_ptr[n] != nnz) throw Error(UCHOL_BAD_ARG, "row pointers do not match nnz");
            S->col = cp(d->col, nnz);
            for (int r = 0; r < n; ++r) {
                if (S->row_ptr[r + 1] < S->row_ptr[r]) throw Error(UCHOL_BAD_ARG, "row pointers are not monotone");
                for (int k = S->row_ptr[r]; k < S->row_ptr[r + 1]; ++k)
                    if (S->col[k] < r || S->col[k] >= n) throw Error(UCHOL_BAD_ARG, "column index outside the upper triangle");
            }
            S->perm = cp(d->permutation, n);
            {
                std::vector<char> seen(n, 0);
                for (int v : S->perm) {
                    if (v < 0 || v >= n || seen[v]) throw Error(UCHOL_BAD_ARG, "permutation is not a permutation");
                    seen[v] = 1;
                }
            }
            S->diag_idx = cp(d->diag_value_index, n);
            for (int v : S->diag_idx)
                if (v < -1 || v >= nnz) throw Error(UCHOL_BAD_ARG, "diagonal value index out of range");
            S->pat_ptr = cp(d->pattern_ptr, n + 1);
            if (S->pat_ptr[0] != 0) throw Error(UCHOL_BAD_ARG, "pattern pointers must start at 0");
            for (int j = 0; j < n; ++j)
                if (S->pat_ptr[j + 1] < S->pat_ptr[j]) throw Error(UCHOL_BAD_ARG, "pattern pointers are not monotone");
            S->pat_rows = cp(d->pattern_rows, S->pat_ptr[n]);
            S->lower_start = cp(d->lower_start, n);
            S->lower_ptr = cp(d->lower_value_ptr, n + 1);
            if (S->lower_ptr[0] != 0) throw Error(UCHOL_BAD_ARG, "lower pointers must start at 0");
            for (int j = 0; j < n; ++j) {
                if (S->lower_ptr[j + 1] < S->lower_ptr[j]) throw Error(UCHOL_BAD_ARG, "lower pointers are not monotone");
                int len = S->lower_ptr[j + 1] - S->lower_ptr[j];
                if (S->lower_start[j] != S->pat_ptr[j + 1] - len || S->lower_start[j] < S->pat_ptr[j])
                    throw Error(UCHOL_BAD_ARG, "lower start inconsistent with the pattern");
            }
            S->lower_idx = cp(d->lower_value_index, S->lower_ptr[n]);
            S->first_col = cp(d->first_column, count + 1);
            S->parent = cp(d->parent, count);
            S->child_ptr = cp(d->child_ptr, count + 1);
            if (S->child_ptr[0] != 0 || S->child_ptr[count] < 0) throw Error(UCHOL_BAD_ARG, "child pointers invalid");
            S->children = cp(d->children, S->child_ptr[count]);
            S->front_ptr = cp(d->front_ptr, count + 1);
            if (S->front_ptr[count] < 0) throw Error(UCHOL_BAD_ARG, "front pointers invalid");
            for (int s = 0; s < count; ++s)
                if (S->front_ptr[s + 1] < S->front_ptr[s]) throw Error(UCHOL_BAD_ARG, "front pointers are not monotone");
            S->front_rows = cp(d->front_rows, S->front_ptr[count]);
            // validates the whole structure (throws on any inconsistency)
            PlanConfig probe;
            try {
                (void)build_plan(n, count, S->first_col.data(), S->parent.data(), S->child_ptr.data(),
                                 S->children.data(), S->front_ptr.data(), S->front_rows.data(), S->diag_idx.data(),
                                 S->pat_ptr.data(), S->pat_rows.data(), S->lower_start.data(), S->lower_ptr.data(),
                                 S->lower_idx.data(), nnz, probe);
            } catch (const std::runtime_error& e) {
                throw Error(UCHOL_BAD_ARG, std::string("inconsistent symbolic factorization: ") + e.what());
            }
            S->d_perm.upload(S->perm, S->stream, "permutation");
            S->d_diag_idx.upload(S->diag_idx, S->stream, "diagonal indices");
            build_full_csr(S.get());
            CK(cudaStreamSynchronize(S->stream));
        }
        *out = S.release();
    });
}

int uchol_estimate_device_bytes(const uchol_symbolic_desc* d, const uchol_options* opts, int64_t* factor_bytes,
                                int64_t* contribution_bytes, int64_t* staging_bytes, int* levels, int* launches) {
    return guarded([&] {
        if (!d) throw Error(UCHOL_BAD_ARG, "null argument");
        check_options(opts);
        uchol_options o;
        if (opts) o = *opts; else uchol_default_options(&o);
        PlanConfig cfg = config_for(o);
        const int n = d->n, count = d->supernode_count;
        if (n < 0 || count < 0) throw Error(UCHOL_BAD_ARG, "negative size");
        Plan P;
        try {
            P = build_plan(n, count, d->first_column, d->parent, d->child_ptr, d->children, d->front_ptr, d->front_rows,
                           d->diag_value_index, d->pattern_ptr, d->pattern_rows, d->lower_start, d->lower_value_ptr,
                           d->lower_value_index, d->nnz, cfg);
        } catch (const std::runtime_error& e) {
            throw Error(UCHOL_BAD_ARG, std::string("inconsistent symbolic factorization: ") + e.what());
        }
        const int64_t elem = o.precision == UCHOL_PRECISION_FP64 ? 8 : 4;
        const int64_t op = o.precision == UCHOL_PRECISION_BF16 ? 2 : 4;
        if (factor_bytes) *factor_bytes = P.factor_elems * elem;
        if (contribution_bytes) *contribution_bytes = P.contrib_elems * elem;
        if (staging_bytes)
            *staging_bytes = cfg.tensor_core ? 2 * P.stage_elems * op + (int64_t)P.diag_slots * kMinvStride * 4 +
                                                   (int64_t)tc_ws_floats(152) * 4 + (int64_t)tc_counter_count(152) * 4
                                             : 0;
        if (levels) *levels = P.levels;
        if (launches) *launches = (int)P.launches.size();
        const long long nnz = d->nnz;
        check_budget(o.device_memory_budget, planned_bytes(P, o.precision, nnz, 2 * nnz - n, n));
    });
}

int uchol_symbolic_destroy(uchol_symbolic s) {
    return guarded([&] {
        if (s) symbolic_release(s);
    });
}

int uchol_symbolic_set_stream(uchol_symbolic s, void* stream) {
    return guarded([&] {
        if (!s) throw Error(UCHOL_BAD_ARG, "null handle");
        CK(cudaStreamSynchronize(s->stream));
        if (s->own_stream) CK(cudaStreamDestroy(s->stream));
        if (stream) {
            s->stream = (cudaStream_t)stream;
            s->own_stream = false;
        } else {
            CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
            s->own_stream = true;
        }
    });
}

static int factorize_common(uchol_symbolic s, int n, int nnz, const double* values, bool on_device,
                            const uchol_options* opts, uchol_factor* out, uchol_factor_stats* stats) {
    return guarded([&] {
        if (!out) throw Error(UCHOL_BAD_ARG, "null output handle");
        *out = nullptr;
        if (!s) throw Error(UCHOL_BAD_ARG, "symbolic handle is null");
        if (!values && nnz > 0) throw Error(UCHOL_BAD_ARG, "values is null");
        std::lock_guard<std::mutex> lk(s->mu);
        std::unique_ptr<uchol_factor_s> F(create_factor(s, n, nnz, opts));
        factorize_impl(F.get(), values, on_device);
        if (stats) *stats = F->last;
        *out = F.release();
    });
}

int uchol_factorize(uchol_symbolic s, int n, int nnz, const double* values, const uchol_options* opts,
                    uchol_factor* out, uchol_factor_stats* stats) {
    return factorize_common(s, n, nnz, values, false, opts, out, stats);
}

int uchol_factorize_device(uchol_symbolic s, int n, int nnz, const double* d_values, const uchol_options* opts,
                           uchol_factor* out, uchol_factor_stats* stats) {
    return factorize_common(s, n, nnz, d_values, true, opts, out, stats);
}

int uchol_refactorize(uchol_factor f, const double* values, int on_device, uchol_factor_stats* stats) {
    return guarded([&] {
        if (!f || (!values && f->sym->nnz > 0)) throw Error(UCHOL_BAD_ARG, "null argument");
        std::lock_guard<std::mutex> lk(f->mu);
        factorize_impl(f, values, on_device != 0);
        if (stats) *stats = f->last;
    });
}

int uchol_autotune(uchol_symbolic s, int n, int nnz, const double* values, const uchol_options* base,
                   uchol_options* best, uchol_autotune_report* report) {
    return guarded([&] {
        if (!s || !best || (!values && nnz > 0)) throw Error(UCHOL_BAD_ARG, "null argument");
        check_options(base);
        uchol_options o0;
        if (base) o0 = *base; else uchol_default_options(&o0);
        std::lock_guard<std::mutex> lk(s->mu);
        if (n != s->n || nnz != s->nnz)
            throw Error(UCHOL_PATTERN_MISMATCH, "the values do not match the symbolic factorization");
        DBuf dv;
        dv.alloc((size_t)std::max(1, nnz) * sizeof(double), "autotune values");
        if (nnz > 0) CK(cudaMemcpy(dv.p, values, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice));
        const bool mixed = o0.precision != UCHOL_PRECISION_FP64;
        int candidates = 0;
        // refactorisation time of one configuration: a factor of its own, a first factorisation
        // (graph capture), then the best of two replays; +inf when the configuration fails
        auto timed = [&](int mask, int bw, int merge, int split) -> double {
            ++candidates;
            uchol_options o = o0;
            o.small_front_buckets = mask;
            o.block_width = bw;
            o.chain_merge_width = merge;
            o.split_min_kblocks = split;
            try {
                std::unique_ptr<uchol_factor_s> F(create_factor(s, n, nnz, &o));
                factorize_impl(F.get(), dv.as<double>(), true);
                double t = std::numeric_limits<double>::infinity();
                for (int r = 0; r < 2; ++r) {
                    factorize_impl(F.get(), dv.as<double>(), true);
                    t = std::min(t, F->last.factor_ms);
                }
                CK(cudaStreamSynchronize(s->stream));
                return t;
            } catch (const Error& e) {
                if (e.code == UCHOL_CUDA_ERROR || e.code == UCHOL_TIMEOUT) throw;   // not a property of the candidate
                return std::numeric_limits<double>::infinity();
            }
        };
        int mask = o0.small_front_buckets ? o0.small_front_buckets : 0x7;
        int bw = mixed ? (o0.block_width > 0 ? o0.block_width : kDiagMax) : 0;
        int merge = o0.chain_merge_width, split = o0.split_min_kblocks;
        const double t_default = timed(mask, bw, merge, split);
        double t_best = t_default;
        auto keep = [&](double t) {
            if (t < t_best) {
                t_best = t;
                return true;
            }
            return false;
        };
        for (int b = kSmallBuckets - 1; b >= 0; --b) {
            const int m2 = mask ^ (1 << b);
            if (keep(timed(m2, bw, merge, split))) mask = m2;
        }
        if (mixed) {
            const int bw2 = bw == kDiagMax ? 64 : kDiagMax;
            if (keep(timed(mask, bw2, merge, split))) bw = bw2;
        }
        // device fronts from supernode chains: narrower, wider, or one front per supernode
        for (int m2 : {512, 1024, -1}) {
            if (m2 == merge) continue;
            if (keep(timed(mask, bw, m2, split))) merge = m2;
        }
        // stream-K threshold of the tensor-core updates
        if (mixed)
            for (int s2 : {4, 16, -1}) {
                if (s2 == split) continue;
                if (keep(timed(mask, bw, merge, s2))) split = s2;
            }
        *best = o0;
        best->small_front_buckets = mask;
        best->block_width = bw;
        best->chain_merge_width = merge;
        best->split_min_kblocks = split;
        if (report) *report = {candidates, t_default, t_best, mask, bw, merge, split};
    });
}

int uchol_factor_destroy(uchol_factor f) {
    return guarded([&] {
        if (!f) return;
        cudaStreamSynchronize(f->sym->stream);
        delete f;
    });
}

int uchol_factor_diagonal(uchol_factor f, double* out) {
    return guarded([&] {
        if (!f || (!out && f->sym->n > 0)) throw Error(UCHOL_BAD_ARG, "null argument");
        if (f->sym->n == 0) return;
        CK(cudaMemcpyAsync(out, f->diag.p, (size_t)f->sym->n * sizeof(double), cudaMemcpyDeviceToHost, f->sym->stream));
        CK(cudaStreamSynchronize(f->sym->stream));
    });
}

int uchol_factor_get_stats(uchol_factor f, uchol_factor_stats* stats) {
    return guarded([&] {
        if (!f || !stats) throw Error(UCHOL_BAD_ARG, "null argument");
        *stats = f->last;
    });
}

int uchol_factor_phase_times(uchol_factor f, uchol_phase_times* t) {
    return guarded([&] {
        if (!f || !t) throw Error(UCHOL_BAD_ARG, "null argument");
        *t = f->phases;
    });
}

static void check_solve_args(uchol_factor f, int n, int nrhs, const void* b, int ldb, const void* x, int ldx) {
    if (!f) throw Error(UCHOL_BAD_ARG, "factor handle is null");
    if (n != f->sym->n)
        throw Error(UCHOL_BAD_ARG, "The right-hand side length " + std::to_string(n) +
                                       " does not match the matrix size " + std::to_string(f->sym->n) + ".");
    if (nrhs < 0 || nrhs > 65535) throw Error(UCHOL_BAD_ARG, "invalid number of right-hand sides");
    if (n > 0 && nrhs > 0 && (!b || !x)) throw Error(UCHOL_BAD_ARG, "null vector");
    if (ldb < std::max(1, n) || ldx < std::max(1, n)) throw Error(UCHOL_BAD_ARG, "leading dimension smaller than n");
}

int uchol_solve_device(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx) {
    return guarded([&] {
        check_solve_args(f, n, nrhs, b, ldb, x, ldx);
        if (n == 0 || nrhs == 0) return;
        std::lock_guard<std::mutex> lk(f->mu);
        ensure_workspace(f, nrhs);
        apply_factor(f, nrhs, b, ldb, x, ldx);
        CK(cudaStreamSynchronize(f->sym->stream));
        check_solve_status(f);
    });
}

int uchol_solve(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx) {
    return guarded([&] {
        check_solve_args(f, n, nrhs, b, ldb, x, ldx);
        if (n == 0 || nrhs == 0) return;
        std::lock_guard<std::mutex> lk(f->mu);
        cudaStream_t st = f->sym->stream;
        ensure_workspace(f, nrhs);
        double* db = f->vec[4].as<double>();
        double* dx = f->vec[5].as<double>();
        CK(cudaMemcpy2DAsync(db, (size_t)n * 8, b, (size_t)ldb * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice, st));
        apply_factor(f, nrhs, db, n, dx, n);
        CK(cudaMemcpy2DAsync(x, (size_t)ldx * 8, dx, (size_t)n * 8, (size_t)n * 8, nrhs, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        check_solve_status(f);
    });
}

int uchol_solve_refined_device(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx,
                               const uchol_refine_options* ro, uchol_refine_stats* rs) {
    return guarded([&] {
        check_solve_args(f, n, nrhs, b, ldb, x, ldx);
        if (rs) *rs = {0, 0.0, 0.0, 0.0};
        if (n == 0 || nrhs == 0) return;
        std::lock_guard<std::mutex> lk(f->mu);
        solve_refined(f, nrhs, b, ldb, x, ldx, ro, rs);
    });
}

int uchol_solve_refined(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx,
                        const uchol_refine_options* ro, uchol_refine_stats* rs) {
    return guarded([&] {
        check_solve_args(f, n, nrhs, b, ldb, x, ldx);
        if (rs) *rs = {0, 0.0, 0.0, 0.0};
        if (n == 0 || nrhs == 0) return;
        std::lock_guard<std::mutex> lk(f->mu);
        cudaStream_t st = f->sym->stream;
        ensure_workspace(f, nrhs);
        DBuf db, dx;
        db.alloc((size_t)n * nrhs * 8, "right-hand sides");
        dx.alloc((size_t)n * nrhs * 8, "solutions");
        CK(cudaMemcpy2DAsync(db.p, (size_t)n * 8, b, (size_t)ldb * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice, st));
        int code = UCHOL_OK;
        std::string msg;
        try {
            solve_refined(f, nrhs, db.as<double>(), n, dx.as<double>(), n, ro, rs);
        } catch (const Error& e) {
            if (e.code != UCHOL_NO_CONVERGENCE) throw;
            code = e.code;
            msg = e.what();
        }
        CK(cudaMemcpy2DAsync(x, (size_t)ldx * 8, dx.p, (size_t)n * 8, (size_t)n * 8, nrhs, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (code != UCHOL_OK) throw Error(code, msg);
    });
}

int uchol_residual_norms(uchol_factor f, int n, int nrhs, const double* b, int ldb, const double* x, int ldx,
                         double* out) {
    return guarded([&] {
        check_solve_args(f, n, nrhs, b, ldb, x, ldx);
        if (!out && nrhs > 0) throw Error(UCHOL_BAD_ARG, "null output");
        if (nrhs == 0) return;
        if (n == 0) {
            for (int j = 0; j < nrhs; ++j) out[j] = 0.0;
            return;
        }
        std::lock_guard<std::mutex> lk(f->mu);
        cudaStream_t st = f->sym->stream;
        ensure_workspace(f, nrhs);
        double* db = f->vec[4].as<double>();
        double* dx = f->vec[5].as<double>();
        double* r = f->vec[0].as<double>();
        CK(cudaMemcpy2DAsync(db, (size_t)n * 8, b, (size_t)ldb * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpy2DAsync(dx, (size_t)n * 8, x, (size_t)ldx * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice, st));
        residual(f, nrhs, dx, n, db, n, r, n);
        double* nr = f->scal.as<double>() + kDotBlocks * nrhs;
        dots(f, nrhs, r, n, r, n, nr);
        std::vector<double> h(nrhs);
        CK(cudaMemcpyAsync(h.data(), nr, nrhs * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int j = 0; j < nrhs; ++j) out[j] = std::sqrt(h[j]);
    });
}

}  // extern "C"

#include "kernel_checks.cuh"
#include "device_matrix.cuh"
