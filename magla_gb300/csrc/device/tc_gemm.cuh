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

struct TcMaps {
    CUtensorMap a;
    CUtensorMap b;
    bool valid = false;
};

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
constexpr int kTcBlockBytes = kTcTile * 128;  // one 128-row x 128-byte K block

template <bool BF16>
__global__ void __launch_bounds__(128, 1)
    k_tc_update(const UpdJob* __restrict__ jobs, int njobs, const SnDev* __restrict__ sn, float* __restrict__ panel,
                float* __restrict__ contrib, const __grid_constant__ CUtensorMap map_a,
                const __grid_constant__ CUtensorMap map_b, int max_kblocks, int* status) {
    constexpr int KBE = BF16 ? 64 : 32;  // K elements per 128-byte block
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* sA = smem;
    uint8_t* sB = smem + max_kblocks * kTcBlockBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + max_kblocks * kTcBlockBytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
    int* flag = reinterpret_cast<int*>(tmem_slot + 1);

    const UpdJob J = jobs[find_job(jobs, njobs, blockIdx.x)];
    const SnDev d = sn[J.s];
    TileTask tk;
    tk.s = J.s;
    tk.k0 = J.k0;
    tk.kn = J.kn;
    decode_tile(J, d, kTcTile, (long long)blockIdx.x - J.tile_begin, tk.i0, tk.j0, tk.jend);
    tk.a_row = J.stage_row0 + (tk.i0 - J.c0);
    tk.b_row = J.stage_row0 + (tk.j0 - J.c0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nkb = min(max_kblocks, (tk.kn + KBE - 1) / KBE);

    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
        *flag = 1;
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 128);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bars[0], (uint32_t)(nkb * 2 * kTcBlockBytes));
        for (int kb = 0; kb < nkb; ++kb) {
            tma_load_2d(sA + kb * kTcBlockBytes, &map_a, &bars[0], kb * KBE, tk.a_row);
            tma_load_2d(sB + kb * kTcBlockBytes, &map_b, &bars[0], kb * KBE, tk.b_row);
        }
        if (mbar_wait(&bars[0], 0)) {
            tc_fence_after();
            constexpr uint32_t idesc = mma_idesc(BF16 ? 1u : 2u, kTcTile, kTcTile);
            for (int kb = 0; kb < nkb; ++kb) {
                const uint32_t a0 = smem_u32(sA + kb * kTcBlockBytes);
                const uint32_t b0 = smem_u32(sB + kb * kTcBlockBytes);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)  // 4 MMAs of 32 bytes of K per 128-byte block
                    umma<BF16>(tmem, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc,
                               (kb | kk) != 0 ? 1u : 0u);
            }
            umma_commit(&bars[1]);
        } else {
            atomicExch(status, kTcStatusTimeout);
            *flag = 0;
            mbar_wait(&bars[0], 0);  // one more bounded wait for the copies in flight
        }
    }
    __syncthreads();
    const bool ok = *flag != 0;
    bool done = ok && mbar_wait(&bars[1], 0);
    if (ok && !done) {
        atomicExch(status, kTcStatusTimeout);
        mbar_wait(&bars[1], 0);
    }
    tc_fence_after();
    if (done) {
        const bool in_panel = tk.j0 < d.w;
        const int i = tk.i0 + warp * 32 + lane;
        float* base = in_panel ? panel + d.panel_off + i : contrib + d.contrib_off + (i - d.w);
        const long long ldc = in_panel ? d.ldp : d.ldc;
        const int jshift = in_panel ? 0 : d.w;
        const bool row_ok = i < d.m;
#pragma unroll 1
        for (int cc = 0; cc < kTcTile / 32; ++cc) {
            float v[32], old[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
            // all 32 loads are issued before any store so they overlap
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const int j = tk.j0 + cc * 32 + c;
                old[c] = (row_ok && j < tk.jend && i >= j) ? base[(long long)(j - jshift) * ldc] : 0.f;
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                const int j = tk.j0 + cc * 32 + c;
                if (row_ok && j < tk.jend && i >= j) base[(long long)(j - jshift) * ldc] = old[c] - v[c];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 128);
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

// One map per operand over the whole staging arena [rows x nb], K-major:
// box = 128 bytes of K x 128 rows, 128-byte swizzle, zero fill outside.
inline TcMaps make_tc_maps(bool bf16, void* a, void* b, long long rows, int nb) {
    TcMaps m;
    auto enc = tensor_map_encoder();
    const size_t es = bf16 ? 2 : 4;
    CUtensorMapDataType dt = bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    cuuint64_t dims[2] = {(cuuint64_t)nb, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)nb * es};
    cuuint32_t box[2] = {(cuuint32_t)(128 / es), (cuuint32_t)kTcTile};
    cuuint32_t estr[2] = {1, 1};
    for (int w = 0; w < 2; ++w) {
        CUresult r = enc(w == 0 ? &m.a : &m.b, dt, 2, w == 0 ? a : b, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    }
    m.valid = true;
    return m;
}
inline void destroy_tc_maps(TcMaps& m) { m.valid = false; }

inline size_t tc_smem_bytes(int kblocks) { return (size_t)kblocks * 2 * kTcBlockBytes + 1024 + 64; }

inline void launch_tc_update(bool bf16, const UpdJob* jobs, int njobs, long long tiles, const SnDev* sn, float* panel,
                             float* contrib, const TcMaps& maps, int nb, int* status, cudaStream_t st) {
    const int kblocks = nb / (bf16 ? 64 : 32);
    const size_t smem = tc_smem_bytes(kblocks);
    if (bf16) {
        cudaFuncSetAttribute(k_tc_update<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_tc_update<true><<<(unsigned)tiles, 128, smem, st>>>(jobs, njobs, sn, panel, contrib, maps.a, maps.b, kblocks,
                                                             status);
    } else {
        cudaFuncSetAttribute(k_tc_update<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_tc_update<false><<<(unsigned)tiles, 128, smem, st>>>(jobs, njobs, sn, panel, contrib, maps.a, maps.b, kblocks,
                                                              status);
    }
}

}  // namespace uchol_dev
