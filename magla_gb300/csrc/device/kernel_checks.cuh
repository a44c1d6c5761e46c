// Kernel checks: single launches of the mixed path's factorisation kernels on
// caller data (host buffers), so that tests can compare each kernel with an
// FP64 product or LDL^T of the same operands, tile class by tile class.  They
// have no counterpart in the reference, whose numeric phase is one CPU routine.
// Included by capi.cu (the kernels are defined once, in that translation unit).
#pragma once

namespace {

inline int round_up_int(int x, int a) { return (x + a - 1) / a * a; }

// Front of m rows and w columns in the device layout (panel m x w with ldp, contribution
// t x t with ldc), from / to a column-major m x m host array (lower triangle used).
struct CheckFront {
    SnDev d{};
    DBuf panel, contrib, sn;
    void setup(int m, int w, cudaStream_t st) {
        d.m = m;
        d.w = w;
        d.ldp = round_up_int(m, 8);
        const int t = m - w;
        d.ldc = t > 0 ? round_up_int(t, 8) : 0;
        d.panel_off = 0;
        d.contrib_off = 0;
        d.first_col = 0;
        d.rows_off = 0;
        d.rel_off = 0;
        d.parent = -1;
        panel.alloc((size_t)d.ldp * w * sizeof(float), "check front");
        contrib.alloc((size_t)std::max(1, d.ldc * t) * sizeof(float), "check front");
        std::vector<SnDev> v{d};
        sn.upload(v, st, "check front");
    }
    void upload(const float* full, cudaStream_t st) {
        const int m = d.m, w = d.w, t = m - w;
        std::vector<float> p((size_t)d.ldp * w, 0.f), c((size_t)std::max(1, d.ldc * t), 0.f);
        for (int j = 0; j < w; ++j)
            for (int i = 0; i < m; ++i) p[i + (size_t)j * d.ldp] = full[i + (size_t)j * m];
        for (int j = 0; j < t; ++j)
            for (int i = 0; i < t; ++i) c[i + (size_t)j * d.ldc] = full[(w + i) + (size_t)(w + j) * m];
        CK(cudaMemcpyAsync(panel.p, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(contrib.p, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    }
    void download(float* full, cudaStream_t st) {
        const int m = d.m, w = d.w, t = m - w;
        std::vector<float> p((size_t)d.ldp * w), c((size_t)std::max(1, d.ldc * t));
        CK(cudaMemcpyAsync(p.data(), panel.p, p.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(c.data(), contrib.p, c.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int j = 0; j < w; ++j)
            for (int i = 0; i < m; ++i) full[i + (size_t)j * m] = p[i + (size_t)j * d.ldp];
        for (int j = 0; j < t; ++j)
            for (int i = 0; i < t; ++i) full[(w + i) + (size_t)(w + j) * m] = c[i + (size_t)j * d.ldc];
    }
};

// Round to nearest even BF16 (the staging copies' rounding, __floats2bfloat162_rn).
inline uint16_t to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);   // inf / nan kept
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

}  // namespace

extern "C" {

int uchol_check_schur_update(int bf16, int m, int w, int c0, int cend, int kbeg, int kn, const float* front,
                             const float* w_op, const float* l_op, int ld, int max_ctas, float* front_out,
                             int64_t* tiles_out, int* split_out) {
    return guarded([&] {
        if (!front || !w_op || !l_op || !front_out) throw Error(UCHOL_BAD_ARG, "null argument");
        if (m <= 0 || w <= 0 || w > m || c0 < 0 || cend <= c0 || cend > m || (c0 < w && cend > w))
            throw Error(UCHOL_BAD_ARG, "the columns must lie in [0, m), all in the panel or all in the contribution");
        if (ld <= 0 || ld % 64 != 0 || kbeg < 0 || kn <= 0 || kbeg + kn > ld)
            throw Error(UCHOL_BAD_ARG, "ld must be a positive multiple of 64 holding [kbeg, kbeg + kn)");
        const int kbe = bf16 ? 64 : 32;
        if (kbeg % kbe != 0) throw Error(UCHOL_BAD_ARG, "kbeg must start a 128-byte K block");
        int dev = 0, sms = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (max_ctas > 0) sms = std::min(sms, max_ctas);
        cudaStream_t st = nullptr;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } guard{st};
        CheckFront F;
        F.setup(m, w, st);
        F.upload(front, st);
        // staging operands, K-major rows x ld (BF16: rounded to nearest even on the host)
        const size_t es = bf16 ? 2 : 4;
        DBuf sa, sb, maps, jobs, ws, counters, status;
        sa.alloc((size_t)m * ld * es, "check operands");
        sb.alloc((size_t)m * ld * es, "check operands");
        if (bf16) {
            std::vector<uint16_t> a((size_t)m * ld), b((size_t)m * ld);
            for (size_t i = 0; i < a.size(); ++i) {
                a[i] = to_bf16(w_op[i]);
                b[i] = to_bf16(l_op[i]);
            }
            CK(cudaMemcpyAsync(sa.p, a.data(), a.size() * 2, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(sb.p, b.data(), b.size() * 2, cudaMemcpyHostToDevice, st));
        } else {
            CK(cudaMemcpyAsync(sa.p, w_op, (size_t)m * ld * 4, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(sb.p, l_op, (size_t)m * ld * 4, cudaMemcpyHostToDevice, st));
        }
        std::vector<CUtensorMap> mp(2);
        try {
            make_stage_maps(bf16 != 0, sa.p, sb.p, m, ld, mp.data());
        } catch (const std::runtime_error& e) {
            throw Error(UCHOL_CUDA_ERROR, e.what());
        }
        maps.upload(mp, st, "check maps");
        const long long tiles = tc_job_tiles(c0, cend, m);
        std::vector<TcJob> jv{TcJob{0, 0, c0, cend, kbeg, kn, 0}};
        jobs.upload(jv, st, "check job");
        ws.alloc(tc_ws_floats(sms) * sizeof(float), "check workspace");
        counters.alloc(tc_counter_count(sms) * sizeof(int), "check workspace");
        status.alloc(sizeof(int), "check workspace");
        CK(cudaMemsetAsync(counters.p, 0, counters.bytes, st));
        CK(cudaMemsetAsync(status.p, 0, sizeof(int), st));
        CK(cudaFuncSetAttribute(k_tc_gemm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
        CK(cudaFuncSetAttribute(k_tc_gemm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
        const TcPlanned tp = tc_schedule(tiles, (kn + kbe - 1) / kbe, sms);
        const TcSched S{tiles, tp.dp_tiles, tp.sk_nkb, ws.as<float>(), counters.as<int>()};
        launch_tc_gemm(bf16 != 0, jobs.as<TcJob>(), 1, S, tp.grid, F.sn.as<SnDev>(), F.panel.as<float>(),
                       F.contrib.as<float>(), maps.as<CUtensorMap>(), status.as<int>(), st);
        counted();
        CK(cudaGetLastError());
        int hs = 0;
        CK(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        F.download(front_out, st);
        if (hs != 0) throw Error(UCHOL_TIMEOUT, "a bounded device wait expired in the tensor-core update");
        if (tiles_out) *tiles_out = tiles;
        if (split_out) *split_out = tp.sk_nkb > 0 ? 1 : 0;
    });
}

int uchol_check_diag_panel(int m, int nb, const float* front, double threshold, double regularization,
                           int allow_regularization, float* l_out, double* d_out, float* w_stage_out,
                           int* counts_out) {
    return guarded([&] {
        if (!front || !l_out || !d_out) throw Error(UCHOL_BAD_ARG, "null argument");
        if (nb <= 0 || nb > kDiagMax || m < nb) throw Error(UCHOL_BAD_ARG, "need 0 < nb <= 128 and m >= nb");
        cudaStream_t st = nullptr;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } guard{st};
        // a front of m rows whose first nb columns are the block (w = nb); only the panel is used
        CheckFront F;
        F.setup(m, nb, st);
        std::vector<float> full((size_t)m * m, 0.f);
        for (int j = 0; j < nb; ++j)
            for (int i = 0; i < m; ++i) full[i + (size_t)j * m] = front[i + (size_t)j * m];
        F.upload(full.data(), st);
        const int ld = round_up_int(nb, 64);
        DBuf diag, minv, sa, sb, info, ptask, ttask, ctl, stats;
        diag.alloc(sizeof(double) * nb, "check");
        minv.alloc(sizeof(float) * kMinvStride, "check");
        sa.alloc((size_t)m * ld * sizeof(float), "check");
        sb.alloc((size_t)m * ld * sizeof(float), "check");
        CK(cudaMemsetAsync(sa.p, 0, sa.bytes, st));
        CK(cudaMemsetAsync(sb.p, 0, sb.bytes, st));
        std::vector<StageInfo> si{StageInfo{0, ld, 0}};
        info.upload(si, st, "check");
        std::vector<PanelTask> pt{PanelTask{0, 0, nb, nb, 0, -1, 0, 0}};
        ptask.upload(pt, st, "check");
        std::vector<PanelTask> tt;
        for (int r = nb; r < m; r += kSolveRows)
            tt.push_back(PanelTask{0, 0, nb, r, std::min(kSolveRows, m - r), 1, 0, 0});
        if (!tt.empty()) ttask.upload(tt, st, "check");
        std::vector<FactorCtl> cv{FactorCtl{threshold, regularization, allow_regularization}};
        ctl.upload(cv, st, "check");
        PivotStats ps0{};
        ps0.failed = INT_MAX;
        ps0.min_bits = 0x7fefffffffffffffull;   // DBL_MAX, as k_finish_scale leaves it
        std::vector<PivotStats> pv{ps0};
        stats.upload(pv, st, "check");
        CK(cudaFuncSetAttribute(k_diag_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDiagSmemBytes));
        CK(cudaFuncSetAttribute(k_panel_solve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPanelSmemBytes));
        k_diag_block<<<1, 256, kDiagSmemBytes, st>>>(ptask.as<PanelTask>(), F.sn.as<SnDev>(), F.panel.as<float>(),
                                                      diag.as<double>(), minv.as<float>(), ctl.as<FactorCtl>(),
                                                      stats.as<PivotStats>());
        counted();
        if (!tt.empty()) {
            k_panel_solve<float><<<(unsigned)tt.size(), 256, kPanelSmemBytes, st>>>(
                ttask.as<PanelTask>(), F.sn.as<SnDev>(), F.panel.as<float>(), minv.as<float>(), sa.as<float>(),
                sb.as<float>(), info.as<StageInfo>());
            counted();
        }
        CK(cudaGetLastError());
        F.download(full.data(), st);
        for (int j = 0; j < nb; ++j)
            for (int i = 0; i < m; ++i) l_out[i + (size_t)j * m] = full[i + (size_t)j * m];
        CK(cudaMemcpyAsync(d_out, diag.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
        PivotStats hs{};
        CK(cudaMemcpyAsync(&hs, stats.p, sizeof(PivotStats), cudaMemcpyDeviceToHost, st));
        if (w_stage_out) {
            // the W = L D staging rows of the panel solve, K-major m x ld -> column-major m x nb (rows >= nb)
            std::vector<float> h((size_t)m * ld);
            CK(cudaMemcpyAsync(h.data(), sa.p, h.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            for (int j = 0; j < nb; ++j)
                for (int i = 0; i < m; ++i) w_stage_out[i + (size_t)j * m] = h[(size_t)i * ld + j];
        }
        CK(cudaStreamSynchronize(st));
        if (counts_out) {
            counts_out[0] = hs.regularized;
            counts_out[1] = hs.negative;
            counts_out[2] = hs.failed == INT_MAX ? -1 : hs.failed;
        }
    });
}


// Plan check (host only): builds the execution plan of a symbolic factorisation for the
// given options and SM count and verifies the invariants its launches rely on; no GPU needed.
int uchol_check_plan(const uchol_symbolic_desc* d, const uchol_options* opts, int sms, int* counts) {
    return guarded([&] {
        // counts (optional, 5 ints): extend-add items, side-stream launches, inverse-diagonal rows
        // split in more than one chunk, backward row chunks, forward trailing-row chunks
        int n_items = 0, n_side = 0, n_split = 0, n_bchunks = 0, n_fchunks = 0;
        if (!d) throw Error(UCHOL_BAD_ARG, "null argument");
        check_options(opts);
        uchol_options o;
        if (opts) o = *opts; else uchol_default_options(&o);
        PlanConfig cfg = config_for(o);
        cfg.sms = sms;
        Plan P;
        try {
            P = build_plan(d->n, d->supernode_count, d->first_column, d->parent, d->child_ptr, d->children,
                           d->front_ptr, d->front_rows, d->diag_value_index, d->pattern_ptr, d->pattern_rows,
                           d->lower_start, d->lower_value_ptr, d->lower_value_index, d->nnz, cfg);
        } catch (const std::runtime_error& e) {
            throw Error(UCHOL_BAD_ARG, std::string("inconsistent symbolic factorization: ") + e.what());
        }
        auto fail = [](const std::string& m) { throw Error(UCHOL_INTERNAL, "plan check: " + m); };
        // (1) extend-add: every receiving column of a front with children exactly once; side-stream
        //     items only for the contribution columns of fronts not factorised whole; a side launch
        //     is joined by the next contribution update before another one forks
        std::map<std::pair<int, int>, int> seen;
        bool pending = false;
        for (const Launch& L : P.launches) {
            if (L.kind == Launch::ExtendAdd) n_items += L.count;
            if (L.stream == 1) ++n_side;
            if (L.kind == Launch::ExtendAdd)
                for (int q = L.begin; q < L.begin + L.count; ++q) {
                    const EaItem& it = P.ea_items[q];
                    const SnDev& pd = P.sn[it.parent];
                    if (++seen[{it.parent, it.pcol}] != 1) fail("a receiving column appears twice");
                    if (L.stream == 1 && (it.pcol < pd.w || small_front(P.cfg, pd.m)))
                        fail("a side-stream extend-add item outside the contribution columns of a large front");
                    for (int e = it.begin; e < it.end; ++e)
                        if (e < 0 || e >= (int)P.ea_entries.size()) fail("extend-add entry out of range");
                }
            if (L.stream == 1) {
                if (pending) fail("a side launch forks before the previous one is joined");
                pending = true;
            } else if (L.stream == 2) {
                if (!pending) fail("a join without a side launch");
                if (L.kind != Launch::TcUpdate) fail("a join on a launch other than a contribution update");
                for (int j = L.begin; j < L.begin + L.count; ++j) {
                    const TcJobHost& J = P.tc_jobs[j];
                    if (J.c0 != P.sn[J.s].w || J.kbeg != 0 || J.kn != P.sn[J.s].w) fail("the join is not a contribution update");
                }
                pending = false;
            }
        }
        if (pending) fail("a side launch is never joined");
        for (int s = 0; s < P.count; ++s) {
            const SnDev& sd = P.sn[s];
            if (sd.parent < 0) continue;
            for (int a = 0; a < sd.m - sd.w; ++a)
                if (!seen.count({sd.parent, P.rel[sd.rel_off + a]})) fail("a child's trailing row is not received");
        }
        // (2) solve tasks
        const int SB = P.cfg.solve_block;
        auto check_chunks = [&](const SolveLaunch& L, bool fwd) {
            std::map<std::pair<int, int>, std::vector<const SolveBlockTask*>> rows;
            std::map<int, int> slots;
            for (int q = L.begin; q < L.begin + L.count; ++q) {
                const SolveBlockTask& t = P.solve_tasks[q];
                rows[{t.s, t.k0}].push_back(&t);
            }
            for (auto& kv : rows) {
                const int lo = fwd ? 0 : kv.first.second;
                const int hi = fwd ? kv.first.second : kv.second[0]->kn - 1;
                int next = lo;
                const int nc = (int)kv.second.size();
                n_split += nc > 1;
                for (const SolveBlockTask* t : kv.second) {
                    if (t->c0 != next || t->c1 < t->c0 || t->c1 - t->c0 + 1 > kInvDiagChunk) fail("diagonal chunks do not tile the row");
                    if (t->flags != nc || t->r1 != kv.second[0]->r1) fail("diagonal chunk count or slot base differs");
                    const int slot = t->r1 + (t->c0 - lo) / kInvDiagChunk;
                    if (slot >= std::max(1, P.inv_diag_slots) || ++slots[slot] != 1) fail("diagonal chunk slot reused or out of range");
                    next = t->c1 + 1;
                }
                if (next != hi + 1) fail("diagonal chunks do not reach the row's end");
            }
        };
        for (const SolveLaunch& L : P.fwd_launches) {
            if (L.kind == SolveLaunch::FwdInvDiag) check_chunks(L, true);
            if (L.kind == SolveLaunch::FwdInvTail) {
                std::map<int, std::vector<std::pair<int, int>>> rr;
                for (int q = L.begin; q < L.begin + L.count; ++q)
                    rr[P.solve_tasks[q].s].push_back({P.solve_tasks[q].r0, P.solve_tasks[q].r1});
                for (auto& kv : rr) {
                    std::sort(kv.second.begin(), kv.second.end());
                    int next = P.sn[kv.first].w;
                    for (auto& r : kv.second) {
                        ++n_fchunks;
                        if (r.first != next || r.second <= r.first || r.second - r.first > SB) fail("forward tail chunks do not tile the rows");
                        next = r.second;
                    }
                    if (next != P.sn[kv.first].m) fail("forward tail chunks do not reach the front's end");
                }
            }
        }
        for (size_t li = 0; li < P.bwd_launches.size(); ++li) {
            const SolveLaunch& L = P.bwd_launches[li];
            if (L.kind == SolveLaunch::BwdInvDiag) check_chunks(L, false);
            if (L.kind == SolveLaunch::BwdInvCols) {
                std::map<std::pair<int, int>, std::vector<const SolveBlockTask*>> cols;
                std::map<int, int> slots;
                for (int q = L.begin; q < L.begin + L.count; ++q) cols[{P.solve_tasks[q].s, P.solve_tasks[q].k0}].push_back(&P.solve_tasks[q]);
                for (auto& kv : cols) {
                    int next = P.sn[kv.first.first].w;
                    for (const SolveBlockTask* t : kv.second) {
                        ++n_bchunks;
                        if (t->r0 != next || t->r1 <= t->r0) fail("backward chunks do not tile the rows");
                        if (t->blk >= std::max(1, P.inv_partial_slots) || ++slots[t->blk] != 1) fail("backward chunk slot reused or out of range");
                        next = t->r1;
                    }
                    if (next != P.sn[kv.first.first].m) fail("backward chunks do not reach the front's end");
                }
                if (li + 1 >= P.bwd_launches.size() || P.bwd_launches[li + 1].kind != SolveLaunch::BwdInvReduce)
                    fail("backward chunks without their reduction");
                const SolveLaunch& R = P.bwd_launches[li + 1];
                for (int q = R.begin; q < R.begin + R.count; ++q) {
                    const SolveBlockTask& t = P.solve_tasks[q];
                    auto it = cols.find({t.s, t.k0});
                    if (it == cols.end() || t.r1 != (int)it->second.size() || t.r0 != it->second[0]->blk)
                        fail("a reduction does not match its chunks");
                }
            }
        }
        if (counts) {
            counts[0] = n_items;
            counts[1] = n_side;
            counts[2] = n_split;
            counts[3] = n_bchunks;
            counts[4] = n_fchunks;
        }
    });
}

}  // extern "C"
