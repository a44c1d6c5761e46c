// Tensor-core Schur update on sm_103a: C -= W L^T for 128 x 128 tiles of a
// front's trailing lower triangle, with W = L21 D and L21 staged K-major in
// low precision (FP32 read as TF32, or BF16).  Operands arrive through TMA
// (128-byte swizzle) into shared memory, tcgen05.mma accumulates in TMEM
// (FP32), and the epilogue subtracts the accumulator from the FP32 front in
// place (column-major, one warp per 32 rows -> coalesced 128-byte columns).
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

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per bounded wait
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
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > kWaitLimitNs) return false;
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
constexpr int kTcTile = 128;                  // M = N = 128
constexpr int kTcBlockBytes = kTcTile * 128;  // one 128-row x 128-byte K block of one operand
constexpr int kTcStages = 6;                  // shared-memory ring of (A, B) K blocks (192 KB: enough bytes in flight to cover load latency)
constexpr int kTcGroup = 8;                   // column tiles per group of the tile order (L2 reuse)
constexpr int kTcThreads = 192;               // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue

// One rank-kn update C[rows, cols] -= W[rows, kbeg:kbeg+kn] L[cols, kbeg:kbeg+kn]^T of front s,
// operands in the front's staging region (tensor maps 2*map, 2*map+1; staging row = front row).
struct TcJob {
    long long tile_begin;
    int s, c0, cend, kbeg, kn, map;
};

// Tile t of a trapezoid of nc column tiles (first row tile count R), in
// groups of G column tiles: inside a group, rows first, then the group's
// columns, so the CTAs working at the same time share operand panels.
__device__ __forceinline__ void decode_grouped(long long t, long long nc, long long R, int G, long long& jt,
                                               long long& rt) {
    for (long long jg = 0; jg < nc; jg += G) {
        const long long g = min((long long)G, nc - jg);
        const long long tri = g * (g + 1) / 2;
        const long long count = tri + (R - jg - g) * g;
        if (t < count) {
            if (t < tri) {
                long long dr = (long long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
                while (dr * (dr + 1) / 2 > t) --dr;
                while ((dr + 1) * (dr + 2) / 2 <= t) ++dr;
                rt = jg + dr;
                jt = jg + (t - dr * (dr + 1) / 2);
            } else {
                const long long u = t - tri;
                rt = jg + g + u / g;
                jt = jg + u % g;
            }
            return;
        }
        t -= count;
    }
    jt = rt = 0;
}

__device__ __forceinline__ int tc_find_job(const TcJob* __restrict__ jobs, int njobs, long long t) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void tc_tile(const TcJob& J, const SnDev& d, long long t, int& i0, int& j0, int& jend) {
    int base = J.c0, lim = J.cend;
    if (J.c0 < d.w && d.w < J.cend) {
        const long long nc1 = (d.w - J.c0 + kTcTile - 1) / kTcTile;
        const long long R1 = (d.m - J.c0 + kTcTile - 1) / kTcTile;
        const long long n1 = region_tiles(nc1, R1);
        if (t < n1) lim = d.w; else { t -= n1; base = d.w; }
    }
    const long long nc = (lim - base + kTcTile - 1) / kTcTile;
    const long long R = (d.m - base + kTcTile - 1) / kTcTile;
    long long jt, rt;
    decode_grouped(t, nc, R, kTcGroup, jt, rt);
    j0 = base + (int)jt * kTcTile;
    i0 = base + (int)rt * kTcTile;
    jend = min(j0 + kTcTile, lim);
}

template <bool BF16>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_gemm(const TcJob* __restrict__ jobs, int njobs, long long total_tiles, const SnDev* __restrict__ sn,
              float* __restrict__ panel, float* __restrict__ contrib, const CUtensorMap* __restrict__ maps,
              int* status) {
    constexpr int KBE = BF16 ? 64 : 32;  // K elements per 128-byte block
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;
    uint8_t* sB = smem + kTcStages * kTcBlockBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(sB + kTcStages * kTcBlockBytes);
    uint64_t* empty = full + kTcStages;
    uint64_t* acc_full = empty + kTcStages;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int q = 0; q < kTcStages; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], 128);
        }
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 256);
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
            for (long long t = blockIdx.x; t < total_tiles && !*abort_flag; t += gridDim.x) {
                const TcJob J = jobs[tc_find_job(jobs, njobs, t)];
                const SnDev d = sn[J.s];
                int i0, j0, jend;
                tc_tile(J, d, t - J.tile_begin, i0, j0, jend);
                const CUtensorMap* ma = maps + 2 * J.map;
                const CUtensorMap* mb = ma + 1;
                const int nkb = (J.kn + KBE - 1) / KBE;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1)) { fail(); break; }
                    mbar_arrive_expect_tx(&full[stage], 2 * kTcBlockBytes);
                    const int kx = J.kbeg + kb * KBE;
                    tma_load_2d(sA + stage * kTcBlockBytes, ma, &full[stage], kx, i0);
                    tma_load_2d(sB + stage * kTcBlockBytes, mb, &full[stage], kx, j0);
                    if (++stage == kTcStages) { stage = 0; phase ^= 1; }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int acc = 0;
            uint32_t acc_phase = 0;
            constexpr uint32_t idesc = mma_idesc(BF16 ? 1u : 2u, kTcTile, kTcTile);
            for (long long t = blockIdx.x; t < total_tiles && !*abort_flag; t += gridDim.x) {
                const int nkb = (jobs[tc_find_job(jobs, njobs, t)].kn + KBE - 1) / KBE;
                if (!mbar_wait(&acc_empty[acc], acc_phase ^ 1)) { fail(); break; }
                tc_fence_after();
                const uint32_t dt = tmem + (uint32_t)(acc * kTcTile);
                bool ok = true;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&full[stage], phase)) { fail(); ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA + stage * kTcBlockBytes);
                    const uint32_t b0 = smem_u32(sB + stage * kTcBlockBytes);
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma<BF16>(dt, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc,
                                   (kb | kk) != 0 ? 1u : 0u);
                    umma_commit(&empty[stage]);
                    if (++stage == kTcStages) { stage = 0; phase ^= 1; }
                }
                if (!ok) break;
                umma_commit(&acc_full[acc]);
                if (++acc == 2) { acc = 0; acc_phase ^= 1; }
            }
        }
    } else {
        // ---------------- epilogue: warps 2..5 own TMEM lanes 32*(warp%4) .. +31
        const int q = warp & 3;
        int acc = 0;
        uint32_t acc_phase = 0;
        for (long long t = blockIdx.x; t < total_tiles; t += gridDim.x) {
            const TcJob J = jobs[tc_find_job(jobs, njobs, t)];
            const SnDev d = sn[J.s];
            int i0, j0, jend;
            tc_tile(J, d, t - J.tile_begin, i0, j0, jend);
            if (!mbar_wait(&acc_full[acc], acc_phase)) { fail(); break; }
            tc_fence_after();
            const int i = i0 + q * 32 + lane;
            const bool in_panel = j0 < d.w;
            float* base = in_panel ? panel + d.panel_off + i : contrib + d.contrib_off + (i - d.w);
            const long long ldc = in_panel ? d.ldp : d.ldc;
            const int jshift = in_panel ? 0 : d.w;
            const bool row_ok = i < d.m;
            const uint32_t ta = tmem + (uint32_t)(acc * kTcTile) + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
            for (int cc = 0; cc < kTcTile / 32; ++cc) {
                float v[32], old[32];
                tmem_ld32(ta + (uint32_t)(cc * 32), v);
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const int j = j0 + cc * 32 + c;
                    old[c] = (row_ok && j < jend && i >= j) ? base[(long long)(j - jshift) * ldc] : 0.f;
                }
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const int j = j0 + cc * 32 + c;
                    if (row_ok && j < jend && i >= j) base[(long long)(j - jshift) * ldc] = old[c] - v[c];
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[acc]);
            if (++acc == 2) { acc = 0; acc_phase ^= 1; }
            if (*abort_flag) break;
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
    if (warp == 0) tmem_dealloc(tmem, 256);
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

// A K-major [rows x ld] operand region: box = 128 bytes of K x 128 rows,
// 128-byte swizzle, zero fill outside (rows beyond the front, K beyond ld).
inline CUtensorMap make_region_map(bool bf16, void* base, long long rows, int ld) {
    CUtensorMap m;
    const size_t es = bf16 ? 2 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * es};
    cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)kTcTile};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = tensor_map_encoder()(&m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                      base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return m;
}

inline size_t tc_smem_bytes() {
    return (size_t)kTcStages * 2 * kTcBlockBytes + 1024 + (2 * kTcStages + 4) * 8 + 16;
}

inline void launch_tc_gemm(bool bf16, const TcJob* jobs, int njobs, long long tiles, const SnDev* sn, float* panel,
                           float* contrib, const CUtensorMap* maps, int* status, int sms, cudaStream_t st) {
    const size_t smem = tc_smem_bytes();
    const unsigned grid = (unsigned)std::min<long long>(tiles, (long long)sms);
    if (bf16) {
        k_tc_gemm<true><<<grid, kTcThreads, smem, st>>>(jobs, njobs, tiles, sn, panel, contrib, maps, status);
    } else {
        k_tc_gemm<false><<<grid, kTcThreads, smem, st>>>(jobs, njobs, tiles, sn, panel, contrib, maps, status);
    }
}

}  // namespace uchol_dev
