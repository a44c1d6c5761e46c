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

}  // extern "C"
