// Solves of inverse fronts: fronts of solve_block < w <= inv_cols columns keep
// the whole inverse of the unit-lower triangle of their diagonal block, so that
// a level's solve needs no chain of block solves.  Forward, per front:
//   y_1 = Linv_11 f_1                  (k_fwd_inv_diag: one CTA per block row),
//   f_2 -= L_21 y_1                    (k_fwd_inv_tail: one CTA per chunk of trailing rows);
// backward:
//   g_1 -= L_21^T g_2                  (k_bwd_inv_cols: partial sums per chunk of rows;
//                                       k_bwd_inv_reduce adds them in chunk order),
//   x_1 = Linv_11^T g_1                (k_bwd_inv_diag: one CTA per block column).
// The algebra is the reference's supernodal substitution
// (CAESolvers/UCHOL/UtduNumericFactorization.cs:139-207) with the triangular solve of
// the diagonal block written as a product with its inverse; the result differs only
// in rounding.  The inverse is built once per factorisation from the inverses of the
// SB x SB diagonal blocks (k_invert_blocks): block (i, j), i > j, is
// -Linv(i, i) sum_{j <= k < i} L(i, k) Linv(k, j), by increasing i - j (k_inv_offdiag).
#pragma once

#include "solve_kernels.cuh"

namespace uchol_dev {

// SB x SB block of the inverse, column-major: (i, i) in the diagonal-block arena, (i, j), i > j,
// in the off-diagonal arena.
template <class Cv, int SB>
__device__ __forceinline__ const Cv* inv_block(const Cv* linv, const Cv* linv_off, int blk, int ob, int i, int j) {
    return i == j ? linv + (long long)(blk + i) * SB * SB
                  : linv_off + ((long long)ob + (long long)i * (i - 1) / 2 + j) * SB * SB;
}

// C (SB x SB, in registers: thread (tx, ty) holds rows tx TM .. +TM, columns ty TN .. +TN)
// += A B for column-major SB x SB A and B in shared memory.
template <class T, int SB>
struct BlockGemm {
    static constexpr int TM = SB / 16, TN = SB / 16;
    T c[TM][TN];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) c[a][b] = T(0);
    }
    __device__ __forceinline__ void mma(const T* A, const T* B, int tx, int ty) {
#pragma unroll 4
        for (int kk = 0; kk < SB; ++kk) {
            T a[TM], b[TN];
#pragma unroll
            for (int u = 0; u < TM; ++u) a[u] = A[tx * TM + u + kk * SB];
#pragma unroll
            for (int v = 0; v < TN; ++v) b[v] = B[kk + (ty * TN + v) * SB];
#pragma unroll
            for (int u = 0; u < TM; ++u)
#pragma unroll
                for (int v = 0; v < TN; ++v) c[u][v] += a[u] * b[v];
        }
    }
};

// Off-diagonal inverse block (i, j) of an inverse front (task {s, i, j, ob, -, -, blk}).
template <class T, int SB>
__global__ void __launch_bounds__(256) k_inv_offdiag(const SolveBlockTask* __restrict__ tasks, const SnDev* __restrict__ sn,
                                                     const T* __restrict__ panel, const T* __restrict__ linv,
                                                     T* __restrict__ linv_off) {
    extern __shared__ __align__(16) unsigned char inv_smem[];
    T* A = reinterpret_cast<T*>(inv_smem);
    T* B = A + SB * SB;
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const int i = tk.k0, j = tk.kn, ob = tk.r0, blk = tk.blk;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const T* P = panel + d.panel_off;
    BlockGemm<T, SB> g;
    g.zero();
    for (int k = j; k < i; ++k) {
        __syncthreads();
        // A = L(i, k), rows past the front's columns (its trailing rows) read as zero
        for (int e = tid; e < SB * SB; e += blockDim.x) {
            const int r = e % SB, c = e / SB, gr = i * SB + r;
            A[e] = gr < d.w ? P[gr + (long long)(k * SB + c) * d.ldp] : T(0);
        }
        const T* Bk = inv_block<T, SB>(linv, linv_off, blk, ob, k, j);
        for (int e = tid; e < SB * SB; e += blockDim.x) B[e] = Bk[e];
        __syncthreads();
        g.mma(A, B, tx, ty);
    }
    // X = the sum, into B; then -Linv(i, i) X
    __syncthreads();
#pragma unroll
    for (int u = 0; u < BlockGemm<T, SB>::TM; ++u)
#pragma unroll
        for (int v = 0; v < BlockGemm<T, SB>::TN; ++v)
            B[tx * BlockGemm<T, SB>::TM + u + (ty * BlockGemm<T, SB>::TN + v) * SB] = g.c[u][v];
    const T* Di = linv + (long long)(blk + i) * SB * SB;
    for (int e = tid; e < SB * SB; e += blockDim.x) A[e] = Di[e];
    __syncthreads();
    g.zero();
    g.mma(A, B, tx, ty);
    T* out = linv_off + ((long long)ob + (long long)i * (i - 1) / 2 + j) * SB * SB;
#pragma unroll
    for (int u = 0; u < BlockGemm<T, SB>::TM; ++u)
#pragma unroll
        for (int v = 0; v < BlockGemm<T, SB>::TN; ++v)
            out[tx * BlockGemm<T, SB>::TM + u + (ty * BlockGemm<T, SB>::TN + v) * SB] = -g.c[u][v];
}

template <class T, int SB>
constexpr size_t inv_offdiag_smem() { return (size_t)2 * SB * SB * sizeof(T); }

// Shared memory of the inverse-front solve kernels: two SB x SB tile stages, two
// right-hand blocks (SB rows x RG, stride RS) and the partial sums.
template <class T, class Cv, int SB, int RG>
constexpr size_t inv_solve_smem() {
    return (size_t)2 * SB * SB * sizeof(T) + LevelRhs<Cv, SB, RG>::bytes + kLevelSmemSlack;
}

// Register prefetch of an SB x RG right-hand block: thread t holds elements t + 256 q;
// fetch() issues the global loads of the next block before the current tile's products,
// commit() stores them into shared memory (row c at c RS, right-hand side g at + g) after.
template <class Cv, int SB, int RG>
struct RhsPrefetch {
    static constexpr int PQ = (SB * RG + 255) / 256;
    static constexpr int RS = LevelRhs<Cv, SB, RG>::RS;
    Cv v[PQ];
    // f(c, g) -> the value of row c, right-hand side g (zero where absent)
    template <class F>
    __device__ __forceinline__ void fetch(F&& f) {
#pragma unroll
        for (int q = 0; q < PQ; ++q) {
            const int e = (int)threadIdx.x + 256 * q, g = e / SB, c = e - g * SB;
            v[q] = e < SB * RG ? f(c, g) : Cv(0);
        }
    }
    __device__ __forceinline__ void commit(Cv* buf) const {
#pragma unroll
        for (int q = 0; q < PQ; ++q) {
            const int e = (int)threadIdx.x + 256 * q, g = e / SB, c = e - g * SB;
            if (e < SB * RG) buf[c * RS + g] = v[q];
        }
    }
};

// Inverse-diagonal products split in chunks of blocks (plan.hpp, FwdInvDiag): a CTA stores
// the partial sums v of its chunk (row `row`, right-hand sides g0 .. g0+FG-1 of the group) in
// slot slot0 + chunk and counts itself in; the CTA that completes the row's nc chunks adds
// the nc partial sums in chunk order into v and returns true, the others return false.  No
// CTA waits for another.  nc = 1: v is already complete.
template <class Cv, int SB, int FG>
__device__ __forceinline__ bool inv_chunk_combine(Cv (&v)[FG], bool fin, int row, int g0, int ng, int rg, int nrhs,
                                                  int slot0, int chunk, int nc, Cv* __restrict__ pbuf,
                                                  unsigned* __restrict__ cnt) {
    if (nc == 1) return true;
    __shared__ int last;
    if (fin) {
#pragma unroll
        for (int q = 0; q < FG; ++q)
            if (g0 + q < ng) pbuf[((long long)(slot0 + chunk) * nrhs + rg + g0 + q) * SB + row] = v[q];
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned* c = cnt + (long long)slot0 * gridDim.y + blockIdx.y;
        last = atomicAdd(c, 1u) == (unsigned)(nc - 1);
        if (last) *c = 0u;   // every chunk has counted in: ready for the next launch
    }
    __syncthreads();
    if (!last) return false;
    if (fin) {
#pragma unroll
        for (int q = 0; q < FG; ++q) {
            Cv s = Cv(0);
            if (g0 + q < ng)
                for (int k = 0; k < nc; ++k) s += __ldcg(&pbuf[((long long)(slot0 + k) * nrhs + rg + g0 + q) * SB + row]);
            v[q] = s;
        }
    }
    return true;
}

// Forward y_i = sum_{j <= i} Linv(i, j) f_j for right-hand sides [RG blockIdx.y, +RG);
// writes y_i (front vector yv) and y_i / D (work).  Thread (row, pid) sums columns
// [pid CPT, pid CPT + CPT) of each block.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 1) k_fwd_inv_diag(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                         const Cv* __restrict__ linv, const Cv* __restrict__ linv_off,
                                                         const Cv* __restrict__ fv, Cv* __restrict__ yv,
                                                         const double* __restrict__ diag, Cv* __restrict__ work,
                                                         Cv* __restrict__ pbuf, unsigned* __restrict__ cnt,
                                                         int* status) {
    using R = LevelRhs<Cv, SB, RG>;
    constexpr int TPR = R::TP, CPT = SB / TPR, RS = R::RS, FG = R::FG;
    extern __shared__ __align__(128) unsigned char blk_smem[];
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    Cv* const stage0 = reinterpret_cast<Cv*>(sm);        // two Linv tile stages
    auto stage = [&](int k) { return stage0 + k * SB * SB; };
    Cv* const fb0 = stage0 + 2 * SB * SB;                // two blocks f_j: SB rows x RG
    auto fbuf = [&](int k) { return fb0 + k * SB * RS; };
    Cv* part = fb0 + 2 * SB * RS;
    __shared__ unsigned long long bar[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int i = tk.k0, ob = tk.r0, blk = tk.blk, j0 = tk.c0, j1 = tk.c1;
    const int rg = blockIdx.y * RG, ng = min(RG, A.nrhs - rg);
    const int tid = threadIdx.x, row = tid % SB, pid = tid / SB;
    const bool fin = RG >= TPR || pid == 0;
    const int g0 = RG >= TPR ? pid * FG : 0;
    const long long fo = A.fvec_off[tk.s];
    if (tid == 0) {
        bar_init(&bar[0]);
        bar_init(&bar[1]);
    }
    constexpr unsigned kTileBytes = SB * SB * sizeof(Cv);
    auto issue = [&](int jj) {
        if (tid == 0) {
            const int st = (jj - j0) & 1;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bar_expect(&bar[st], kTileBytes);
            bulk_g2s(stage(st), inv_block<Cv, SB>(linv, linv_off, blk, ob, i, jj), kTileBytes, &bar[st]);
        }
    };
    // f_j, zero past the front's columns and the group's right-hand sides
    RhsPrefetch<Cv, SB, RG> pf;
    auto fetch = [&](int j) {
        pf.fetch([&](int c, int g) {
            const int col = j * SB + c;
            return (g < ng && col < d.w) ? fv[fo + (long long)(rg + g) * A.fv_stride + col] : Cv(0);
        });
    };
    fetch(j0);
    __syncthreads();   // barriers initialised
    issue(j0);
    if (j0 + 1 <= j1) issue(j0 + 1);
    pf.commit(fbuf(0));
    if (j0 + 1 <= j1) fetch(j0 + 1);
    RhsAcc<Cv, RG> acc;
    acc.zero();
    unsigned phase = 0;
    for (int j = j0; j <= j1; ++j) {
        const int st = (j - j0) & 1;
        if (!__syncthreads_and(bar_wait(&bar[st], (phase >> st) & 1u, status))) return;
        phase ^= 1u << st;
        const Cv* tile = stage(st);
        const Cv* fb = fbuf(st);
#pragma unroll 2
        for (int u0 = 0; u0 < CPT; u0 += 4)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = pid * CPT + u0 + q;
                acc.add(q, tile[row + c * SB], fb + c * RS);
            }
        if (j + 1 <= j1) pf.commit(fbuf(st ^ 1));
        if (j + 2 <= j1) fetch(j + 2);
        __syncthreads();   // the stage is free again
        if (j + 2 <= j1) issue(j + 2);
    }
    acc.store(part + (pid * SB + row) * RG);
    __syncthreads();
    Cv y[FG];
#pragma unroll
    for (int q = 0; q < FG; ++q) {
        const int g = g0 + q;
        y[q] = Cv(0);
        if (fin && g < ng) {
            y[q] = part[row * RG + g];
#pragma unroll
            for (int p = 1; p < TPR; ++p) y[q] += part[(p * SB + row) * RG + g];
        }
    }
    if (!inv_chunk_combine<Cv, SB, FG>(y, fin, row, g0, ng, rg, A.nrhs, tk.r1, j0 / kInvDiagChunk, tk.flags, pbuf,
                                       cnt))
        return;
    if (fin) {
        const int kn = min(SB, d.w - i * SB);
#pragma unroll
        for (int q = 0; q < FG; ++q) {
            const int g = g0 + q;
            if (g >= ng || row >= kn) break;
            const int col = i * SB + row;
            yv[fo + (long long)(rg + g) * A.fv_stride + col] = y[q];
            work[d.first_col + col + (long long)(rg + g) * A.ldw] = (Cv)((double)y[q] / diag[d.first_col + col]);
        }
    }
}

// Register tiles of the trailing-row kernels.  A thread accumulates RT rows (forward) or
// RT columns (backward) by GT right-hand sides; RT elements are 16 bytes, so the forward
// kernel reads them as one vector.  NG groups of RT rows (columns) cover SB, NH groups of
// GT cover the RG right-hand sides, and the NS remaining thread groups split the half
// tile's columns (forward) or rows (backward); their partial sums are added at the end.
template <class Cv, int SB, int RG>
struct TailTiles {
    static constexpr int RT = 16 / (int)sizeof(Cv);
    static constexpr int GT = RG < 8 ? RG : 8;
    static constexpr int NH = RG / GT;
    static constexpr int NG = SB / RT;
    static constexpr int NS = 256 / (NG * NH);
    static constexpr int RS = LevelRhs<Cv, SB, RG>::RS;   // row stride of the right-hand blocks
    static_assert(NG * NH * NS == 256 && RG % GT == 0, "thread tiles must cover the CTA");
};

// Shared memory of the trailing-row kernels: two half-tile stages, the transposed half tile
// (backward only; rows of SB + 1 so that the transpose and the column reads are free of
// bank conflicts), two right-hand blocks of SB/2 rows; the partial sums (NS x SB x RG) reuse
// the stages after the last tile.  Two CTAs fit on an SM.
template <class T, class Cv, int SB, int RG, bool kTransposed>
constexpr size_t inv_tail_smem() {
    return (size_t)SB * SB * sizeof(T) + (kTransposed ? (size_t)(SB / 2) * (SB + 1) * sizeof(T) : 0) +
           (size_t)2 * (SB / 2) * TailTiles<Cv, SB, RG>::RS * sizeof(Cv) + kLevelSmemSlack;
}
static_assert((size_t)TailTiles<float, 128, 16>::NS * 128 * 16 * sizeof(float) <= (size_t)128 * 128 * sizeof(float),
              "the partial sums fit in the tile stages");
static_assert((size_t)TailTiles<double, 64, 16>::NS * 64 * 16 * sizeof(double) <= (size_t)64 * 64 * sizeof(double),
              "the partial sums fit in the tile stages");

// Starts a tensor-map tile copy of `bytes` bytes at (x, y) into dst, completing on bar (one thread).
__device__ __forceinline__ void start_box_tile(void* dst, const CUtensorMap* map, int x, int y, unsigned bytes,
                                               unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bar_expect(bar, bytes);
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// RT consecutive elements of shared memory (16-byte aligned), widened.
__device__ __forceinline__ void lds_vec(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
__device__ __forceinline__ void lds_vec(const double* p, double (&v)[2]) {
    const double2 q = *reinterpret_cast<const double2*>(p);
    v[0] = q.x;
    v[1] = q.y;
}
// GT values of a right-hand row (16-byte aligned when GT is a multiple of 16 bytes)
template <class Cv, int GT>
__device__ __forceinline__ void lds_rhs(const Cv* p, Cv (&v)[GT]) {
    if constexpr (GT * sizeof(Cv) % 16 == 0) {
#pragma unroll
        for (int g = 0; g < GT; g += 16 / (int)sizeof(Cv)) {
            Cv w[16 / sizeof(Cv)];
            lds_vec(p + g, w);
#pragma unroll
            for (int k = 0; k < 16 / (int)sizeof(Cv); ++k) v[g + k] = w[k];
        }
    } else {
#pragma unroll
        for (int g = 0; g < GT; ++g) v[g] = p[g];
    }
}

// Forward trailing rows [r0, r1) of an inverse front: f -= L[r0:r1, 0:w] y, by half tiles
// of SB rows x SB/2 columns (tensor map `maps`: box {SB, SB/2}); the tiles start at r0
// rounded down to 16 bytes.  Thread (row group, right-hand group, column split) keeps an
// RT x GT tile of sums.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 2) k_fwd_inv_tail(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                         const CUtensorMap* __restrict__ maps,
                                                         const Cv* __restrict__ yv, Cv* __restrict__ fv, int* status) {
    static_assert(sizeof(T) == sizeof(Cv), "factor and vector elements of one size");
    using W = TailTiles<Cv, SB, RG>;
    constexpr int HC = SB / 2, RT = W::RT, GT = W::GT, NG = W::NG, NH = W::NH, NS = W::NS, RS = W::RS;
    constexpr int CPS = HC / NS;                          // columns of a half tile per split
    constexpr int kAlign = 16 / (int)sizeof(T);
    constexpr unsigned kBytes = SB * HC * sizeof(T);
    extern __shared__ __align__(128) unsigned char blk_smem[];
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    T* const stage0 = reinterpret_cast<T*>(sm);          // two half-tile stages (SB x HC, column-major)
    auto stage = [&](int k) { return stage0 + k * SB * HC; };
    Cv* const yb0 = reinterpret_cast<Cv*>(stage0 + 2 * SB * HC);   // two blocks of y: HC rows x RG
    auto ybuf = [&](int k) { return yb0 + k * HC * RS; };
    Cv* const part = reinterpret_cast<Cv*>(stage0);      // after the last tile: NS x SB x RG
    __shared__ unsigned long long bar[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int nh = (d.w + HC - 1) / HC, r0 = tk.r0, r1 = tk.r1, ra = r0 & ~(kAlign - 1);
    const int tid = threadIdx.x, rgp = tid % NG, rh = (tid / NG) % NH, cs = tid / (NG * NH);
    const long long fo = A.fvec_off[tk.s];
    if (tid == 0) {
        bar_init(&bar[0]);
        bar_init(&bar[1]);
    }
    __syncthreads();
    unsigned phase = 0;
    RhsPrefetch<Cv, HC, RG> pf;
    for (int rg = 0; rg < A.nrhs; rg += RG) {
        const int ng = min(RG, A.nrhs - rg);
        auto fetch = [&](int h) {
            const int kn = min(HC, d.w - h * HC);
            pf.fetch([&](int c, int g) {
                return (g < ng && c < kn) ? yv[fo + (long long)(rg + g) * A.fv_stride + h * HC + c] : Cv(0);
            });
        };
        fetch(0);
        if (tid == 0) {
            start_box_tile(stage(0), maps + tk.s, ra, 0, kBytes, &bar[0]);
            if (nh > 1) start_box_tile(stage(1), maps + tk.s, ra, HC, kBytes, &bar[1]);
        }
        pf.commit(ybuf(0));
        if (nh > 1) fetch(1);
        Cv acc[RT][GT];
#pragma unroll
        for (int a = 0; a < RT; ++a)
#pragma unroll
            for (int g = 0; g < GT; ++g) acc[a][g] = Cv(0);
        for (int h = 0; h < nh; ++h) {
            if (!__syncthreads_and(bar_wait(&bar[h & 1], (phase >> (h & 1)) & 1u, status))) return;
            phase ^= 1u << (h & 1);
            const T* tile = stage(h & 1) + rgp * RT;
            const Cv* yb = ybuf(h & 1) + rh * GT;
#pragma unroll 4
            for (int u = 0; u < CPS; ++u) {
                const int c = cs * CPS + u;
                Cv l[RT], y[GT];
                lds_vec(tile + c * SB, l);
                lds_rhs<Cv, GT>(yb + c * RS, y);
#pragma unroll
                for (int a = 0; a < RT; ++a)
#pragma unroll
                    for (int g = 0; g < GT; ++g) acc[a][g] += l[a] * y[g];
            }
            if (h + 1 < nh) pf.commit(ybuf((h + 1) & 1));
            if (h + 2 < nh) fetch(h + 2);
            __syncthreads();   // the stage is free again
            if (tid == 0 && h + 2 < nh) start_box_tile(stage(h & 1), maps + tk.s, ra, (h + 2) * HC, kBytes, &bar[h & 1]);
        }
        // partial sums of the column splits, then f -= their sum for the chunk's rows
#pragma unroll
        for (int a = 0; a < RT; ++a)
#pragma unroll
            for (int g = 0; g < GT; ++g) part[(cs * SB + rgp * RT + a) * RG + rh * GT + g] = acc[a][g];
        __syncthreads();
        for (int e = tid; e < SB * RG; e += blockDim.x) {
            const int g = e / SB, lr = e - g * SB, i = ra + lr;
            if (g >= ng || i < r0 || i >= r1) continue;
            Cv sum = part[lr * RG + g];
#pragma unroll
            for (int p = 1; p < NS; ++p) sum += part[(p * SB + lr) * RG + g];
            fv[fo + (long long)(rg + g) * A.fv_stride + i] -= sum;
        }
        __syncthreads();
    }
}

// Backward: column block kb of an inverse front against its trailing rows [r0, r1) (task
// {s, kb, nb, r0, r1, nq, slot}), by half tiles of SB/2 rows x SB columns (tensor map `maps`:
// box {SB/2, SB}), each transposed in shared memory so that a thread's RT columns are read
// without bank conflicts and g is a broadcast.  Thread (column group, right-hand group, row
// split) keeps an RT x GT tile of sums; column group q holds columns q + NG a.  The sums go
// to partial slot `slot` ((slot nrhs + r) SB + c for right-hand side r, column c), which
// k_bwd_inv_reduce adds to g of the block's columns.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 2) k_bwd_inv_cols(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                         const CUtensorMap* __restrict__ maps, const Cv* __restrict__ fv,
                                                         Cv* __restrict__ partial, int* status) {
    static_assert(sizeof(T) == sizeof(Cv), "factor and vector elements of one size");
    using W = TailTiles<Cv, SB, RG>;
    constexpr int HR = SB / 2, RT = W::RT, GT = W::GT, NG = W::NG, NH = W::NH, NS = W::NS, RS = W::RS;
    constexpr int RPS = HR / NS;                          // rows of a half tile per split
    constexpr int TS = SB + 1;                            // row stride of the transposed half tile
    constexpr int kAlign = 16 / (int)sizeof(T);
    constexpr unsigned kBytes = HR * SB * sizeof(T);
    extern __shared__ __align__(128) unsigned char blk_smem[];
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    T* const stage0 = reinterpret_cast<T*>(sm);          // two half-tile stages (HR x SB, column-major)
    auto stage = [&](int k) { return stage0 + k * HR * SB; };
    T* const tt = stage0 + 2 * HR * SB;                   // transposed half tile: row r at r TS
    Cv* const xb0 = reinterpret_cast<Cv*>(tt + HR * TS);  // two blocks of g: HR rows x RG
    auto xbuf = [&](int k) { return xb0 + k * HR * RS; };
    Cv* const part = reinterpret_cast<Cv*>(stage0);      // after the last tile: NS x SB x RG
    __shared__ unsigned long long bar[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int kb = tk.k0, r0 = tk.r0, r1 = tk.r1, ra = r0 & ~(kAlign - 1);
    const int ntile = (r1 - ra + HR - 1) / HR;
    const int tid = threadIdx.x, cgp = tid % NG, rh = (tid / NG) % NH, rsp = tid / (NG * NH);
    const long long fo = A.fvec_off[tk.s];
    if (tid == 0) {
        bar_init(&bar[0]);
        bar_init(&bar[1]);
    }
    __syncthreads();
    unsigned phase = 0;
    RhsPrefetch<Cv, HR, RG> pf;
    for (int rg = 0; rg < A.nrhs; rg += RG) {
        const int ng = min(RG, A.nrhs - rg);
        auto fetch = [&](int t) {
            const int tr = ra + t * HR;
            pf.fetch([&](int r, int g) {
                const int gr = tr + r;
                return (g < ng && gr >= r0 && gr < r1) ? fv[fo + (long long)(rg + g) * A.fv_stride + gr] : Cv(0);
            });
        };
        fetch(0);
        if (tid == 0) {
            start_box_tile(stage(0), maps + tk.s, ra, kb * SB, kBytes, &bar[0]);
            if (ntile > 1) start_box_tile(stage(1), maps + tk.s, ra + HR, kb * SB, kBytes, &bar[1]);
        }
        pf.commit(xbuf(0));
        if (ntile > 1) fetch(1);
        Cv acc[RT][GT];
#pragma unroll
        for (int a = 0; a < RT; ++a)
#pragma unroll
            for (int g = 0; g < GT; ++g) acc[a][g] = Cv(0);
        for (int t = 0; t < ntile; ++t) {
            if (!__syncthreads_and(bar_wait(&bar[t & 1], (phase >> (t & 1)) & 1u, status))) return;
            phase ^= 1u << (t & 1);
            {
                // 16 bytes (RT consecutive rows of one column) per read
                const T* src = stage(t & 1);
                constexpr int QR = HR / RT;   // 16-byte groups per column
                for (int e = tid; e < QR * SB; e += blockDim.x) {
                    const int r = (e % QR) * RT, c = e / QR;
                    T v[RT];
                    lds_vec(src + c * HR + r, v);
#pragma unroll
                    for (int k = 0; k < RT; ++k) tt[(r + k) * TS + c] = v[k];
                }
            }
            __syncthreads();   // tt is ready, the stage is free again
            if (tid == 0 && t + 2 < ntile) start_box_tile(stage(t & 1), maps + tk.s, ra + (t + 2) * HR, kb * SB, kBytes, &bar[t & 1]);
            const Cv* xb = xbuf(t & 1) + rh * GT;
#pragma unroll 4
            for (int u = 0; u < RPS; ++u) {
                const int r = rsp * RPS + u;
                Cv l[RT], x[GT];
#pragma unroll
                for (int a = 0; a < RT; ++a) l[a] = (Cv)tt[r * TS + cgp + NG * a];
                lds_rhs<Cv, GT>(xb + r * RS, x);
#pragma unroll
                for (int a = 0; a < RT; ++a)
#pragma unroll
                    for (int g = 0; g < GT; ++g) acc[a][g] += l[a] * x[g];
            }
            if (t + 1 < ntile) pf.commit(xbuf((t + 1) & 1));
            if (t + 2 < ntile) fetch(t + 2);
            __syncthreads();   // tt and the right-hand block are free again
        }
#pragma unroll
        for (int a = 0; a < RT; ++a)
#pragma unroll
            for (int g = 0; g < GT; ++g) part[(rsp * SB + cgp + NG * a) * RG + rh * GT + g] = acc[a][g];
        __syncthreads();
        for (int e = tid; e < SB * RG; e += blockDim.x) {
            const int g = e / SB, c = e - g * SB;
            if (g >= ng) continue;
            Cv sum = part[c * RG + g];
#pragma unroll
            for (int p = 1; p < NS; ++p) sum += part[(p * SB + c) * RG + g];
            partial[((long long)tk.blk * A.nrhs + rg + g) * SB + c] = sum;
        }
        __syncthreads();
    }
}

// Backward: g of column block kb of an inverse front -= its nq partial sums, added in chunk
// order (task {s, kb, nb, slot0, nq, -, -}: the block's chunks have slots slot0 .. slot0+nq-1),
// one CTA per block and right-hand side (blockIdx.y), one thread per column.
template <class Cv, int SB>
__global__ void __launch_bounds__(SB) k_bwd_inv_reduce(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                       Cv* __restrict__ fv, const Cv* __restrict__ partial) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int kb = tk.k0, slot0 = tk.r0, nq = tk.r1, c = threadIdx.x;
    if (kb * SB + c >= d.w) return;
    for (int r = blockIdx.y; r < A.nrhs; r += gridDim.y) {
        Cv* gp = fv + A.fvec_off[tk.s] + (long long)r * A.fv_stride + kb * SB + c;
        Cv v = *gp;
        const Cv* pp = partial + ((long long)slot0 * A.nrhs + r) * SB + c;
        for (int q0 = 0; q0 < nq; q0 += 8) {   // eight loads in flight, subtracted in chunk order
            Cv p8[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) p8[k] = q0 + k < nq ? pp[(long long)(q0 + k) * A.nrhs * SB] : Cv(0);
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (q0 + k < nq) v -= p8[k];
        }
        *gp = v;
    }
}

// Backward x_j = sum_{i >= j} Linv(i, j)^T g_i (g_i already reduced by k_bwd_inv_cols),
// right-hand sides [RG blockIdx.y, +RG); writes x_j to the work vector.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 1) k_bwd_inv_diag(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                         const Cv* __restrict__ linv, const Cv* __restrict__ linv_off,
                                                         const Cv* __restrict__ fv, Cv* __restrict__ work,
                                                         Cv* __restrict__ pbuf, unsigned* __restrict__ cnt,
                                                         int* status) {
    using R = LevelRhs<Cv, SB, RG>;
    constexpr int TPC = R::TP, RPT = SB / TPC, RS = R::RS, FG = R::FG;
    extern __shared__ __align__(128) unsigned char blk_smem[];
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    Cv* const stage0 = reinterpret_cast<Cv*>(sm);        // two Linv tile stages
    auto stage = [&](int k) { return stage0 + k * SB * SB; };
    Cv* const gb0 = stage0 + 2 * SB * SB;                // two blocks g_i: SB rows x RG
    auto gbuf = [&](int k) { return gb0 + k * SB * RS; };
    Cv* part = gb0 + 2 * SB * RS;
    __shared__ unsigned long long bar[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int j = tk.k0, ob = tk.r0, blk = tk.blk, i0 = tk.c0, i1 = tk.c1;
    const int rg = blockIdx.y * RG, ng = min(RG, A.nrhs - rg);
    const int tid = threadIdx.x, ccol = tid % SB, cpart = tid / SB;
    const bool fin = RG >= TPC || cpart == 0;
    const int g0 = RG >= TPC ? cpart * FG : 0;
    const long long fo = A.fvec_off[tk.s];
    if (tid == 0) {
        bar_init(&bar[0]);
        bar_init(&bar[1]);
    }
    constexpr unsigned kTileBytes = SB * SB * sizeof(Cv);
    auto issue = [&](int ii) {
        if (tid == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const int st = (ii - i0) & 1;
            bar_expect(&bar[st], kTileBytes);
            bulk_g2s(stage(st), inv_block<Cv, SB>(linv, linv_off, blk, ob, ii, j), kTileBytes, &bar[st]);
        }
    };
    RhsPrefetch<Cv, SB, RG> pf;
    auto fetch = [&](int i) {
        pf.fetch([&](int c, int g) {
            const int col = i * SB + c;
            return (g < ng && col < d.w) ? fv[fo + (long long)(rg + g) * A.fv_stride + col] : Cv(0);
        });
    };
    fetch(i0);
    __syncthreads();   // barriers initialised
    issue(i0);
    if (i0 + 1 <= i1) issue(i0 + 1);
    pf.commit(gbuf(0));
    if (i0 + 1 <= i1) fetch(i0 + 1);
    RhsAcc<Cv, RG> acc;
    acc.zero();
    unsigned phase = 0;
    for (int i = i0; i <= i1; ++i) {
        const int st = (i - i0) & 1;
        if (!__syncthreads_and(bar_wait(&bar[st], (phase >> st) & 1u, status))) return;
        phase ^= 1u << st;
        const Cv* tile = stage(st);
        const Cv* gb = gbuf(st);
#pragma unroll 2
        for (int u0 = 0; u0 < RPT; u0 += 4)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = cpart * RPT + ((u0 + q + ccol) & (RPT - 1));
                acc.add(q, tile[c + ccol * SB], gb + c * RS);
            }
        if (i + 1 <= i1) pf.commit(gbuf(st ^ 1));
        if (i + 2 <= i1) fetch(i + 2);
        __syncthreads();
        if (i + 2 <= i1) issue(i + 2);
    }
    acc.store(part + (cpart * SB + ccol) * RG);
    __syncthreads();
    Cv x[FG];
#pragma unroll
    for (int q = 0; q < FG; ++q) {
        const int g = g0 + q;
        x[q] = Cv(0);
        if (fin && g < ng) {
            x[q] = part[ccol * RG + g];
#pragma unroll
            for (int p = 1; p < TPC; ++p) x[q] += part[(p * SB + ccol) * RG + g];
        }
    }
    if (!inv_chunk_combine<Cv, SB, FG>(x, fin, ccol, g0, ng, rg, A.nrhs, tk.r1, (i0 - j) / kInvDiagChunk, tk.flags,
                                       pbuf, cnt))
        return;
    if (fin) {
        const int kn = min(SB, d.w - j * SB);
#pragma unroll
        for (int q = 0; q < FG; ++q) {
            const int g = g0 + q;
            if (g >= ng || ccol >= kn) break;
            work[d.first_col + j * SB + ccol + (long long)(rg + g) * A.ldw] = x[q];
        }
    }
}

}  // namespace uchol_dev
