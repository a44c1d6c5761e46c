// Tensor-core Schur update on sm_103a: C -= W L^T over a front's trailing
// lower triangle, with W = L21 D and L21 staged K-major in low precision (FP32
// read as TF32, or BF16).  A tile is 128 columns x 256 rows of C computed
// transposed, D = L_cols W_rows^T, by one M=128, N=256 tcgen05.mma per K step:
// 48 KB of operands per 128-byte K block for 4.2 MFLOP (a 128 x 128 tile
// moves 32 KB for half the flops), which is what bounds the kernel, since the
// SM's operand bandwidth from L2 and HBM, not the tensor pipe, is the limit.
// Operands arrive through TMA (128-byte swizzle) into a four-stage ring, the
// accumulator lives in TMEM (two 256-column buffers), and eight epilogue warps
// subtract it from the FP32 front in place: each warp's 32 columns x 32 rows go
// through a shared-memory transpose, so that every global access of the warp
// covers 32 consecutive rows of one column, and C takes the update as an L2
// reduction (each entry exactly once per launch: the same sum as a
// read-modify-write, without waiting for a load).
//
// Launches with fewer tiles than SMs can be split in K (stream-K): their K
// blocks are divided evenly over the grid.  A CTA that ends with a partial tile
// writes it to a workspace slot; the last of the tile's CTAs to arrive adds the
// partial tiles in CTA order (deterministic) and updates C.  The kernel also
// takes a whole-tile prefix (TcSched::dp_tiles) before the split tiles; the
// host schedule leaves it empty.
//
// Every wait on an mbarrier is bounded in time; on expiry the kernel records
// a status word, waits once more (bounded) for its own operations, frees
// its TMEM and returns.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace uchol_dev {

constexpr int kTcStatusTimeout = 1;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns(), limit = g_factor_wait_ns;
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row atoms 1024 bytes apart (SBO); LBO unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor: D = FP32, A/B format fmt (TF32 = 2 for kind::tf32,
// BF16 = 1 for kind::f16), both K-major, M x N.
__host__ __device__ constexpr uint32_t mma_idesc(uint32_t fmt, uint32_t M, uint32_t N) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

template <bool BF16>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accumulate) {
    if constexpr (BF16) {
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "setp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
            "}\n" ::"r"(tmem_d),
            "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "setp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
            "}\n" ::"r"(tmem_d),
            "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
            : "memory");
    }
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- kernel
constexpr int kTcABytes = kTcCols * 128;   // one 128-byte K block of the L operand (columns of C)
constexpr int kTcBBytes = kTcRows * 128;   // one 128-byte K block of the W operand (rows of C)
constexpr int kTcStages = 4;               // shared-memory ring of (A, B) K blocks: 192 KB
constexpr int kTcEpiWarps = 8;             // two warps per TMEM lane quadrant, four 32-row chunks each
constexpr int kTcThreads = 64 + 32 * kTcEpiWarps;   // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int kTcPartial = kTcCols * kTcRows;       // floats of one partial tile
constexpr int kTcEpiLd = 33;                        // epilogue transpose buffer: 32 x 33 floats per warp
constexpr int kTcMinSplitKb = 8;           // K blocks of a tile below which it is never split
constexpr int kTcMaxParts = 4;             // most CTAs sharing one split tile (bounds the fixup's reads)

// One rank-kn update C[rows, cols] -= W[rows, kbeg:kbeg+kn] L[cols, kbeg:kbeg+kn]^T of front s,
// operands in the front's staging region (tensor maps 2*map (W, 256-row box), 2*map+1 (L,
// 128-row box); staging row = front row).  Columns [c0, cend) lie all in the panel or all in
// the contribution block.
struct TcJob {
    long long tile_begin;
    int s, c0, cend, kbeg, kn, map;
};

// Work split of one launch (see the file comment).
struct TcSched {
    long long tiles;      // tiles of the launch
    long long dp_tiles;   // tiles [0, dp_tiles): whole tiles, round robin over the grid
    int sk_nkb;           // > 0: tiles [dp_tiles, tiles) are split in K over the grid, sk_nkb K blocks each
    float* ws;            // partial tiles: slots 2b and 2b + 1 of CTA b
    int* counters;        // per split tile: partial tiles arrived (zero between launches)
};

// One unit of a CTA's work: K blocks [kb0, kb1) of tile t (kb1 < 0: all of the job's).
struct TcSeg {
    long long t;
    int kb0, kb1;
    int parts;   // 1: the whole tile; > 1: CTAs sharing the tile
    int slot;    // workspace slot of a partial tile
};

// The segments of CTA b, in order; every role of the CTA walks the same sequence.
struct TcSegIter {
    long long t, dp, W, G, u, u0, u1;
    int nkb, b;
    __device__ TcSegIter(const TcSched& S, int b_, int G_) : t(b_), dp(S.dp_tiles), G(G_), nkb(S.sk_nkb), b(b_) {
        W = nkb > 0 ? (S.tiles - dp) * nkb : 0;
        u0 = u = W > 0 ? (long long)b * W / G : 0;
        u1 = W > 0 ? (long long)(b + 1) * W / G : 0;
    }
    // CTA holding split unit v (units [b W / G, (b + 1) W / G) belong to CTA b)
    __device__ long long owner(long long v) const { return ((v + 1) * G + W - 1) / W - 1; }
    __device__ long long first_cta(long long tt) const { return owner(tt * nkb); }
    __device__ long long last_cta(long long tt) const { return owner(tt * nkb + nkb - 1); }
    // slot of CTA c's partial of split tile tt: its first segment uses 2c, its last 2c + 1
    __device__ long long slot_of(long long c, long long tt) const { return c * W / G >= tt * nkb ? 2 * c : 2 * c + 1; }
    __device__ bool next(TcSeg& g) {
        if (t < dp) {
            g.t = t;
            g.kb0 = 0;
            g.kb1 = -1;
            g.parts = 1;
            g.slot = 0;
            t += G;
            return true;
        }
        if (u < u1) {
            const long long tt = u / nkb;
            const int kb0 = (int)(u - tt * nkb);
            const int kb1 = (int)min((long long)nkb, (long long)kb0 + (u1 - u));
            g.t = dp + tt;
            g.kb0 = kb0;
            g.kb1 = kb1;
            g.parts = (int)(last_cta(tt) - first_cta(tt) + 1);
            g.slot = (int)(2 * b + (u == u0 ? 0 : 1));
            u += kb1 - kb0;
            return true;
        }
        return false;
    }
};

__device__ __forceinline__ int tc_find_job(const TcJob* __restrict__ jobs, int njobs, long long t) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Tile t of job J (front of m rows): first row i0, first column j0, column limit jend.
__device__ __forceinline__ void tc_tile(const TcJob& J, int m, long long t, int& i0, int& j0, int& jend) {
    tc_decode_tile(J.c0, J.cend, m, t, i0, j0, jend);
}

// Barriers of the epilogue warps only (named barrier 1).  Every epilogue warp walks the
// same segments and meets the same barriers; tc_epi_any also returns the OR of a
// predicate over them, so that a decision to stop is the same in every warp.
// Column j of C (indexed by front row) for the tile whose first column is j0.
__device__ __forceinline__ float* tc_column(float* panel, float* contrib, const SnDev& d, int j0, int j) {
    return j0 < d.w ? panel + d.panel_off + (long long)j * d.ldp
                    : contrib + d.contrib_off + (long long)(j - d.w) * d.ldc - d.w;
}

__device__ __forceinline__ void tc_epi_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * kTcEpiWarps) : "memory"); }
__device__ __forceinline__ bool tc_epi_any(bool pred) {
    uint32_t r;
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 p, %1, 0;\n"
        "bar.red.or.pred q, 1, %2, p;\n"
        "selp.u32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)pred), "n"(32 * kTcEpiWarps)
        : "memory");
    return r != 0;
}

// C[i0 + cc*32 + r, j] -= v[r] for the lower-triangle entries of rows below m; whole
// float4 groups are read and written back (entries outside the triangle unchanged).
__device__ __forceinline__ void tc_update_chunk(float* __restrict__ col, int ib, int j, int m, const float* v) {
    float4 o[8];
#pragma unroll
    for (int r4 = 0; r4 < 8; ++r4) {
        const int i = ib + 4 * r4;
        if (i < m && i + 3 >= j) o[r4] = *reinterpret_cast<const float4*>(col + i);
    }
#pragma unroll
    for (int r4 = 0; r4 < 8; ++r4) {
        const int i = ib + 4 * r4;
        if (i < m && i + 3 >= j) {
            float4 x = o[r4];
            if (i >= j && i + 3 < m) {
                x.x -= v[4 * r4];
                x.y -= v[4 * r4 + 1];
                x.z -= v[4 * r4 + 2];
                x.w -= v[4 * r4 + 3];
            } else {
                if (i >= j && i < m) x.x -= v[4 * r4];
                if (i + 1 >= j && i + 1 < m) x.y -= v[4 * r4 + 1];
                if (i + 2 >= j && i + 2 < m) x.z -= v[4 * r4 + 2];
                if (i + 3 >= j && i + 3 < m) x.w -= v[4 * r4 + 3];
            }
            *reinterpret_cast<float4*>(col + i) = x;
        }
    }
}

template <bool BF16>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_gemm(const TcJob* __restrict__ jobs, int njobs, TcSched S, const SnDev* __restrict__ sn,
              float* __restrict__ panel, float* __restrict__ contrib, const CUtensorMap* __restrict__ maps,
              int* status) {
    constexpr int KBE = BF16 ? 64 : 32;  // K elements per 128-byte block
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;                              // L rows (C columns)
    uint8_t* sB = smem + kTcStages * kTcABytes;      // W rows (C rows)
    uint64_t* full = reinterpret_cast<uint64_t*>(sB + kTcStages * kTcBBytes);
    uint64_t* empty = full + kTcStages;
    uint64_t* acc_full = empty + kTcStages;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* last_flag = reinterpret_cast<volatile int*>(tmem_slot + 2);
    float* epi_buf = reinterpret_cast<float*>(full + 16);   // after the barriers and flags (128 bytes)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int q = 0; q < kTcStages; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], 32 * kTcEpiWarps);
        }
        *abort_flag = 0;
        *last_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 2 * kTcRows);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    auto fail = [&]() {
        atomicExch(status, kTcStatusTimeout);
        *abort_flag = 1;
    };

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            TcSegIter it(S, blockIdx.x, gridDim.x);
            TcSeg g;
            while (!*abort_flag && it.next(g)) {
                const TcJob J = jobs[tc_find_job(jobs, njobs, g.t)];
                int i0, j0, jend;
                tc_tile(J, sn[J.s].m, g.t - J.tile_begin, i0, j0, jend);
                const CUtensorMap* mw = maps + 2 * J.map;
                const CUtensorMap* ml = mw + 1;
                const int kb1 = g.kb1 < 0 ? (J.kn + KBE - 1) / KBE : g.kb1;
                bool ok = true;
                for (int kb = g.kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1)) { fail(); ok = false; break; }
                    mbar_arrive_expect_tx(&full[stage], kTcABytes + kTcBBytes);
                    const int kx = J.kbeg + kb * KBE;
                    tma_load_2d(sA + stage * kTcABytes, ml, &full[stage], kx, j0);
                    tma_load_2d(sB + stage * kTcBBytes, mw, &full[stage], kx, i0);
                    if (++stage == kTcStages) { stage = 0; phase ^= 1; }
                }
                if (!ok) break;
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int acc = 0;
            uint32_t acc_phase = 0;
            constexpr uint32_t idesc = mma_idesc(BF16 ? 1u : 2u, kTcCols, kTcRows);
            TcSegIter it(S, blockIdx.x, gridDim.x);
            TcSeg g;
            while (!*abort_flag && it.next(g)) {
                const int kb1 = g.kb1 < 0 ? (jobs[tc_find_job(jobs, njobs, g.t)].kn + KBE - 1) / KBE : g.kb1;
                if (!mbar_wait(&acc_empty[acc], acc_phase ^ 1)) { fail(); break; }
                tc_fence_after();
                const uint32_t dt = tmem + (uint32_t)(acc * kTcRows);
                bool ok = true;
                for (int kb = g.kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&full[stage], phase)) { fail(); ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA + stage * kTcABytes);
                    const uint32_t b0 = smem_u32(sB + stage * kTcBBytes);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma<BF16>(dt, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc,
                                   (kb != g.kb0 || kk != 0) ? 1u : 0u);
                    umma_commit(&empty[stage]);
                    if (++stage == kTcStages) { stage = 0; phase ^= 1; }
                }
                if (!ok) break;
                umma_commit(&acc_full[acc]);
                if (++acc == 2) { acc = 0; acc_phase ^= 1; }
            }
        }
    } else {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 (columns of C)
        // and 32-row chunks [4h, 4h + 4), h = (w - 2) / 4
        const int q = warp & 3;
        const int c_first = ((warp - 2) >> 2) * 4;
        const int jl = q * 32 + lane;
        int acc = 0;
        uint32_t acc_phase = 0;
        TcSegIter it(S, blockIdx.x, gridDim.x);
        TcSeg g;
        for (;;) {
            const bool have = it.next(g);
            if (tc_epi_any(!have || *abort_flag)) break;
            const TcJob J = jobs[tc_find_job(jobs, njobs, g.t)];
            const SnDev d = sn[J.s];
            int i0, j0, jend;
            tc_tile(J, d.m, g.t - J.tile_begin, i0, j0, jend);
            // on an expired wait this thread skips its work but still meets the barriers below
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[acc], acc_phase));   // warp-uniform
            if (!ok) fail();
            tc_fence_after();
            const int j = j0 + jl;
            float* col = tc_column(panel, contrib, d, j0, j);   // column j of C, indexed by front row
            const uint32_t ta = tmem + (uint32_t)(acc * kTcRows) + ((uint32_t)(q * 32) << 16);
            if (g.parts == 1) {
                if (ok) {
                    // the warp's 32 columns x 32 rows go through a shared-memory transpose, so that
                    // every global access of the warp is 32 consecutive rows of one column
                    float* tb = epi_buf + (warp - 2) * 32 * kTcEpiLd;
                    const int jw = j0 + q * 32;   // the warp's first column
                    const long long ld = jw < d.w ? d.ldp : d.ldc;
                    float* colw = tc_column(panel, contrib, d, j0, jw);
#pragma unroll 1
                    for (int cc = c_first; cc < c_first + 4; ++cc) {
                        float v[32];
                        tmem_ld32(ta + (uint32_t)(cc * 32), v);
#pragma unroll
                        for (int r = 0; r < 32; ++r) tb[r * kTcEpiLd + lane] = v[r];
                        __syncwarp();
                        const int i = i0 + cc * 32 + lane;   // this thread's row from here on
                        // each entry of C takes exactly one update per launch, so a reduction in L2
                        // (no load, nothing to wait for) gives the same sum as a read-modify-write
                        if (i < d.m && i0 + cc * 32 + 31 >= jw) {
#pragma unroll
                            for (int c = 0; c < 32; ++c)
                                if (jw + c < jend && i >= jw + c) atomicAdd(colw + (long long)c * ld + i, -tb[lane * kTcEpiLd + c]);
                        }
                        __syncwarp();
                    }
                }
            } else {
                // partial tile: to the workspace; the last CTA of the tile adds all of them
                if (ok) {
                    float* mine = S.ws + (long long)g.slot * kTcPartial + (long long)jl * kTcRows;
#pragma unroll 1
                    for (int cc = c_first; cc < c_first + 4; ++cc) {
                        float v[32];
                        tmem_ld32(ta + (uint32_t)(cc * 32), v);
#pragma unroll
                        for (int r4 = 0; r4 < 8; ++r4)
                            __stcg(reinterpret_cast<float4*>(mine + cc * 32) + r4,
                                   make_float4(v[4 * r4], v[4 * r4 + 1], v[4 * r4 + 2], v[4 * r4 + 3]));
                    }
                }
                __threadfence();
                const bool bad = tc_epi_any(!ok);
                const long long tt = g.t - it.dp;
                if (threadIdx.x == 64) {
                    int last = 0;
                    if (!bad) {
                        const int before = atomicAdd(&S.counters[tt], 1);
                        last = before == g.parts - 1;
                        if (last) S.counters[tt] = 0;
                    }
                    *last_flag = last;
                    __threadfence();
                }
                tc_epi_sync();
                if (*last_flag) {
                    __threadfence();
                    const long long c_lo = it.first_cta(tt), c_hi = it.last_cta(tt);
#pragma unroll 1
                    for (int cc = c_first; cc < c_first + 4; ++cc) {
                        float v[32];
#pragma unroll
                        for (int r = 0; r < 32; ++r) v[r] = 0.f;
                        // two partial tiles in flight per step, added in CTA order
#pragma unroll 1
                        for (long long c = c_lo; c <= c_hi; c += 2) {
                            const float4* p0 = reinterpret_cast<const float4*>(
                                S.ws + it.slot_of(c, tt) * kTcPartial + (long long)jl * kTcRows + cc * 32);
                            const bool two = c + 1 <= c_hi;
                            const float4* p1 = reinterpret_cast<const float4*>(
                                S.ws + it.slot_of(two ? c + 1 : c, tt) * kTcPartial + (long long)jl * kTcRows + cc * 32);
                            float4 x0[8], x1[8];
#pragma unroll
                            for (int r4 = 0; r4 < 8; ++r4) {
                                x0[r4] = __ldcg(p0 + r4);
                                if (two) x1[r4] = __ldcg(p1 + r4);
                            }
#pragma unroll
                            for (int r4 = 0; r4 < 8; ++r4) {
                                v[4 * r4] += x0[r4].x;
                                v[4 * r4 + 1] += x0[r4].y;
                                v[4 * r4 + 2] += x0[r4].z;
                                v[4 * r4 + 3] += x0[r4].w;
                            }
                            if (two) {
#pragma unroll
                                for (int r4 = 0; r4 < 8; ++r4) {
                                    v[4 * r4] += x1[r4].x;
                                    v[4 * r4 + 1] += x1[r4].y;
                                    v[4 * r4 + 2] += x1[r4].z;
                                    v[4 * r4 + 3] += x1[r4].w;
                                }
                            }
                        }
                        if (j < jend) tc_update_chunk(col, i0 + cc * 32, j, d.m, v);
                    }
                }
            }
            // the accumulator is free once every thread has read it (for a partial tile: written it out)
            tc_fence_before();
            mbar_arrive(&acc_empty[acc]);
            if (++acc == 2) { acc = 0; acc_phase ^= 1; }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*abort_flag && threadIdx.x == 0) {
        // a wait expired: give copies and MMAs still in flight a bounded time to land before the CTA exits
        const unsigned long long t0 = global_ns();
        while (global_ns() - t0 < 10000000ull) {
        }
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 2 * kTcRows);
}

// ---------------------------------------------------------------- host side
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            throw std::runtime_error("cuTensorMapEncodeTiled is not available from the driver");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// A K-major [rows x ld] operand region: box = 128 bytes of K x box_rows rows,
// 128-byte swizzle, zero fill outside (rows beyond the front, K beyond ld).
inline CUtensorMap make_region_map(bool bf16, void* base, long long rows, int ld, int box_rows) {
    CUtensorMap m;
    const size_t es = bf16 ? 2 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * es};
    cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(&m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                      base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return m;
}

// The tensor-map pair of one front's staging regions: W rows (256-row box), L rows (128-row box).
inline void make_stage_maps(bool bf16, void* w_base, void* l_base, long long rows, int ld, CUtensorMap* out) {
    out[0] = make_region_map(bf16, w_base, rows, ld, kTcRows);
    out[1] = make_region_map(bf16, l_base, rows, ld, kTcCols);
}

inline size_t tc_smem_bytes() {
    static_assert((2 * kTcStages + 4) * 8 + 12 <= 128, "barriers and flags fit before the epilogue buffers");
    return 1024 + (size_t)kTcStages * (kTcABytes + kTcBBytes) + 128 +
           (size_t)kTcEpiWarps * 32 * kTcEpiLd * sizeof(float);
}

// Workspace of the K-split tiles: two partial tiles per CTA, one counter per split tile.
inline size_t tc_ws_floats(int sms) { return (size_t)2 * sms * kTcPartial; }
inline size_t tc_counter_count(int sms) { return (size_t)2 * sms; }

// Grid and split of one launch of `tiles` tiles.  nkb: K blocks of every tile when all
// tiles have the same K (0 otherwise: never split).  A launch with fewer tiles than SMs is
// split in K when that is estimated faster: time in K blocks per CTA, a split tile costing
// about kTcMinSplitKb more (its partial tiles through L2).  Larger launches take whole
// tiles round robin: the CTAs working on the column tiles that share W rows then stay at
// the same K offsets, which a split tail breaks (operands read from HBM several times).
struct TcPlanned {
    unsigned grid;
    long long dp_tiles;
    int sk_nkb;
};
// min_kb: K blocks of a tile below which it is never split (kTcMinSplitKb by default, < 0: never).
inline TcPlanned tc_schedule(long long tiles, int nkb, int sms, int min_kb = kTcMinSplitKb) {
    TcPlanned p{(unsigned)std::max<long long>(1, std::min<long long>(tiles, sms)), tiles, 0};
    if (min_kb < 0 || nkb < std::max(1, min_kb) || tiles <= 0 || tiles >= sms) return p;
    const long long W = tiles * nkb;
    const long long G = std::max<long long>(1, std::min<long long>({(long long)sms, W / std::max(1, min_kb),
                                                                     tiles * kTcMaxParts}));
    const double t_whole = nkb;   // one wave of whole tiles
    const double t_split = (double)((W + G - 1) / G) + std::max(1, min_kb);
    if (t_split < 0.9 * t_whole) {
        p.grid = (unsigned)G;
        p.dp_tiles = 0;
        p.sk_nkb = nkb;
    }
    return p;
}

inline void launch_tc_gemm(bool bf16, const TcJob* jobs, int njobs, const TcSched& S, unsigned grid, const SnDev* sn,
                           float* panel, float* contrib, const CUtensorMap* maps, int* status, cudaStream_t st) {
    const size_t smem = tc_smem_bytes();
    if (bf16) {
        k_tc_gemm<true><<<grid, kTcThreads, smem, st>>>(jobs, njobs, S, sn, panel, contrib, maps, status);
    } else {
        k_tc_gemm<false><<<grid, kTcThreads, smem, st>>>(jobs, njobs, S, sn, panel, contrib, maps, status);
    }
}

}  // namespace uchol_dev
