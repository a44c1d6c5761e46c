// Supernodal triangular solves (multifrontal form), FP64 symmetric product
// and vector kernels for refinement.
//
// Forward U^T y = b follows the multifrontal schedule: each supernode
// gathers its right-hand side plus the update vectors of its children
// (extend-add of vectors, child order, no atomics), solves with its
// diagonal block and leaves the update vector of its trailing rows for the
// parent.  Backward U x = z reads the final values of the trailing rows
// (ancestors) directly.  The result equals the reference's supernodal
// substitutions (CAESolvers/UCHOL/UtduNumericFactorization.cs:139-207);
// only the order of the floating-point sums differs.
#pragma once

#include <cuda.h>

#include <type_traits>

#include "common.cuh"
#include "plan.hpp"

namespace uchol_dev {

__device__ __forceinline__ SolveBlockTask blocks_or_tasks(const SolveBlockTask* __restrict__ t) { return t[blockIdx.x]; }

struct SolveArgs {
    const SnDev* sn;
    const int* rel;
    const int* rows;        // front_rows
    const int* child_ptr;
    const int* children;
    const long long* fvec_off;
    long long fv_stride;    // elements between RHS columns in the front-vector workspace
    int n, nrhs, ldw;       // ldw: leading dimension of the work vector
};

template <class Cv>
__global__ void k_permute_in(const double* __restrict__ b, int ldb, const int* __restrict__ perm, int n, int nrhs,
                             Cv* __restrict__ work, int ldw) {
    for (int r = blockIdx.y; r < nrhs; r += gridDim.y)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            work[i + (long long)r * ldw] = (Cv)b[perm[i] + (long long)r * ldb];
}

template <class Cv>
__global__ void k_permute_out(const Cv* __restrict__ work, int ldw, const int* __restrict__ perm, int n, int nrhs,
                              double* __restrict__ x, int ldx) {
    for (int r = blockIdx.y; r < nrhs; r += gridDim.y)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[perm[i] + (long long)r * ldx] = (double)work[i + (long long)r * ldw];
}

// Rows [r0, r1) of a front vector: the supernode's right-hand side (own
// columns) plus, child by child, the child's update vector entries that map
// into these rows (relative indices are sorted, so each child contributes a
// contiguous range, found once per child for every right-hand side).
//
// First index in the sorted array a[0, n) whose value is >= key, by one warp: each round
// probes 32 evenly spaced entries and keeps the gap between the last one below the key and
// the first one not below it (a 32-way search: three rounds for 30,000 entries).
__device__ __forceinline__ int warp_lower_bound(const int* __restrict__ a, int n, int key, int lane) {
    int lo = 0, hi = n;   // the answer lies in [lo, hi]
    while (hi - lo > 32) {
        const long long span = hi - lo;
        const int pos = lo + (int)(span * lane / 32);
        const int below = __popc(__ballot_sync(0xffffffffu, a[pos] < key));   // a prefix of the probes
        const int nlo = below == 0 ? lo : lo + (int)(span * (below - 1) / 32) + 1;
        const int nhi = below == 32 ? hi : lo + (int)(span * below / 32);
        lo = nlo;
        hi = nhi;
    }
    const int pos = lo + lane;
    return lo + __popc(__ballot_sync(0xffffffffu, pos < hi && a[pos] < key));
}

template <class Cv>
__global__ void k_fwd_gather(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const Cv* __restrict__ work,
                             Cv* __restrict__ fv) {
    __shared__ int range[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // right-hand sides blockIdx.y, blockIdx.y + gridDim.y, ...
    for (int r = blockIdx.y; r < A.nrhs; r += gridDim.y) {
        Cv* f = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x)
            f[a] = a < d.w ? work[d.first_col + a + (long long)r * A.ldw] : Cv(0);
    }
    __syncthreads();
    const bool whole = tk.r0 == 0 && tk.r1 == d.m;   // the chunk is the whole front
    for (int c = A.child_ptr[s]; c < A.child_ptr[s + 1]; ++c) {
        const int ch = A.children[c];
        const SnDev cd = A.sn[ch];
        const int t = cd.m - cd.w;
        const int* rl = A.rel + cd.rel_off;
        if (whole) {
            if (threadIdx.x == 0) {
                range[0] = 0;
                range[1] = t;
            }
        } else if (warp < 2) {   // warp 0: the chunk's first row, warp 1: its end
            const int v = warp_lower_bound(rl, t, warp == 0 ? tk.r0 : tk.r1, lane);
            if (lane == 0) range[warp] = v;
        }
        __syncthreads();
        for (int r = blockIdx.y; r < A.nrhs; r += gridDim.y) {
            Cv* f = fv + A.fvec_off[s] + r * A.fv_stride;
            const Cv* u = fv + A.fvec_off[ch] + r * A.fv_stride + cd.w;
            for (int b = range[0] + threadIdx.x; b < range[1]; b += blockDim.x) f[rl[b]] += u[b];
        }
        __syncthreads();
    }
}

// Inverse of every unit-lower diagonal block (SB x SB, column-major), one
// CTA per block, thread c computing column c by forward substitution.
template <class T, class Cv, int SB>
__global__ void __launch_bounds__(SB) k_invert_blocks(const SolveBlockTask* __restrict__ blocks, const SnDev* __restrict__ sn,
                                                      const T* __restrict__ panel, Cv* __restrict__ linv) {
    extern __shared__ unsigned char inv_smem[];
    Cv* Lb = reinterpret_cast<Cv*>(inv_smem);
    Cv* X = Lb + SB * SB;
    const SolveBlockTask tk = blocks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const T* P = panel + d.panel_off;
    const int kn = tk.kn;
    for (int idx = threadIdx.x; idx < kn * kn; idx += blockDim.x) {
        int r = idx % kn, c = idx / kn;
        Lb[r + c * SB] = r > c ? (Cv)P[(tk.k0 + r) + (long long)(tk.k0 + c) * d.ldp] : Cv(0);
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c < kn) {
        for (int r = 0; r < kn; ++r) {
            Cv v = r == c ? Cv(1) : Cv(0);
            if (r > c)
                for (int k = c; k < r; ++k) v -= Lb[r + k * SB] * X[k + c * SB];
            X[r + c * SB] = v;
        }
    }
    __syncthreads();
    Cv* out = linv + (long long)tk.blk * SB * SB;
    for (int idx = threadIdx.x; idx < SB * SB; idx += blockDim.x) {
        int r = idx % SB, cc = idx / SB;
        out[idx] = (r < kn && cc < kn) ? X[r + cc * SB] : Cv(0);
    }
}

// ---- persistent block solves: one cooperative launch per tree level ----
//
// The diagonal blocks of a front must be solved in order, and each block
// solution updates every row (forward) or column (backward) after it.  One
// kernel per level runs the whole chain with two kinds of CTA, all resident
// at once (cooperative launch):
//   chain CTAs (one or more fronts each) solve the blocks in order.  For
//     block b+1 a chain needs the rows (columns) of that block updated with
//     every earlier solution: all but the latest come from the bulk CTAs (it
//     waits for the chunk's progress counter), the latest it applies itself
//     from an SB x SB tile of L that it prefetched into shared memory, with
//     the block's inverse, while it waited.  It then publishes the block's
//     solution with a release flag.
//   bulk CTAs own chunks of SB rows (columns) and apply each published
//     solution to them, then advance the chunk's progress counter.
// Everything proceeds step-major: a wait at step b is only ever for a flag
// or counter of step b-1, so no CTA can block its own producer.

constexpr size_t kLevelSmemSlack = 1024;                      // alignment slack of the level kernels' dynamic smem
constexpr int kSolveRhsGroup = 16;                            // right-hand sides per group of the multi-column solves
constexpr int kSolveStatusTimeout = 2;

__device__ __forceinline__ unsigned long long solve_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bulk copies global -> shared on an mbarrier (the copy engine moves the
// bytes; the issuing threads do not wait for them).
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bar_expect(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Waits (bounded) for phase `parity` of the mbarrier; false if the wait expired.
// The clock is read only once the first try has failed (copies issued a tile ahead have
// usually landed by then).
__device__ __forceinline__ bool bar_try(unsigned long long* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, unsigned parity, int* status) {
    if (bar_try(bar, parity)) return true;
    const unsigned long long t0 = solve_ns();
    for (;;) {
        if (bar_try(bar, parity)) return true;
        if (solve_ns() - t0 > g_solve_wait_ns) {
            atomicExch(status, kSolveStatusTimeout);
            return false;
        }
    }
}

// Thread 0 starts the copy of the SB x SB tile of L at rows [r0, r0+SB),
// columns [c0, c0+SB) of a front's diagonal region (one tensor-map copy: a
// column-major box, rows past the region read as zero) and of the first
// inv_cols columns of an inverse block (SB x SB, contiguous) into shared
// memory, completing on `bar`.
template <class T, class Cv, int SB>
__device__ __forceinline__ void start_tile_copy(T* Tl, Cv* Li, const CUtensorMap* map, int r0, int c0,
                                                bool with_tile, const Cv* inv, int inv_cols, unsigned long long* bar) {
    if (threadIdx.x != 0) return;
    const unsigned inv_bytes = (unsigned)(inv_cols * SB * sizeof(Cv));
    const unsigned total = (with_tile ? (unsigned)(SB * SB * sizeof(T)) : 0u) + inv_bytes;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bar_expect(bar, total);
    if (with_tile)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                smem_addr(Tl)),
            "l"(reinterpret_cast<unsigned long long>(map)), "r"(r0), "r"(c0), "r"(smem_addr(bar))
            : "memory");
    bulk_g2s(Li, inv, inv_bytes, bar);
}

// Thread 0 waits for *flag >= target, giving up after g_solve_wait_ns (status :=
// timeout) or as soon as another CTA has given up; the CTA learns the outcome.
__device__ __forceinline__ bool wait_at_least(const int* flag, int target, int* status, int* ok) {
    if (threadIdx.x == 0) {
        int good = 1;
        if (ld_acquire_gpu(flag) < target) {
            const unsigned long long t0 = solve_ns();
            unsigned ns = 32;
            for (;;) {
                __nanosleep(ns);
                if (ld_acquire_gpu(flag) >= target) break;
                if (ns < 256) ns <<= 1;
                if (ld_acquire_gpu(status) != 0) {
                    good = 0;
                    break;
                }
                if (solve_ns() - t0 > g_solve_wait_ns) {
                    atomicExch(status, kSolveStatusTimeout);
                    good = 0;
                    break;
                }
            }
        }
        *ok = good;
    }
    __syncthreads();
    const bool r = *ok != 0;
    __syncthreads();
    return r;
}

// Every thread's writes, then the flag: the CTA barrier orders the other threads' writes
// before thread 0's release store, and release is cumulative, so a reader that acquires the
// flag (ld.acquire.gpu, then a CTA barrier) sees all of them.
__device__ __forceinline__ void publish(int* flag, int value) {
    __syncthreads();
    if (threadIdx.x == 0) st_release_gpu(flag, value);
}

// A level launch.  chains: the level's fronts (task: s; blk = first diagonal
// block; k0 = bulk index of the chunk of its block 0, its other diagonal
// blocks following in order), taken round-robin by CTAs [0, nchain_cta).
// bulk: the chunks, taken round-robin by the other CTAs.
struct LevelArgs {
    const SolveBlockTask* chains;
    int nchains;
    const SolveBlockTask* bulk;
    int nbulk;
    int nchain_cta;
    int steps;       // most diagonal blocks of one front
    int* flags;      // per diagonal block: solution published
    int* progress;   // per bulk chunk: solutions applied
    int* status;
    const CUtensorMap* maps;   // per supernode: its panel (m x w)
    int ndiag;                 // bulk chunks [0, ndiag): diagonal blocks, taken by bulk CTAs [0, ndiag_cta)
    int ndiag_cta;             // the other bulk CTAs take the trailing-row chunks
};

// Tile copy of a bulk item into a stage buffer: rows [x, x+SB), columns
// [y, y+SB) of a front's panel (zero past its m rows and w columns).
template <class T, int SB>
__device__ __forceinline__ void start_bulk_tile(T* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bar_expect(bar, (unsigned)(SB * SB * sizeof(T)));
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// The bulk CTA's share of the chunks: diagonal-block chunks or trailing-row chunks.
struct BulkRange {
    int begin, end, step;
};
__device__ __forceinline__ BulkRange bulk_range(const LevelArgs& L) {
    const int k = blockIdx.x - L.nchain_cta, nbulk_cta = gridDim.x - L.nchain_cta;
    if (k < L.ndiag_cta) return {k, L.ndiag, L.ndiag_cta};
    return {L.ndiag + (k - L.ndiag_cta), L.nbulk, nbulk_cta - L.ndiag_cta};
}

// Next duty (front index q, step b) of a chain CTA after (q, b), in step-major
// order; false when there is none.  Front q (chain task kn = its number of
// diagonal blocks) has duties at steps -1 .. nblk - 2 (step b solves block
// b + 1).
__device__ __forceinline__ bool next_chain_duty(const LevelArgs& L, int& q, int& b, int nblk_q) {
    if (q >= 0 && (int)blockIdx.x + L.nchain_cta >= L.nchains) {
        // the CTA's only front (nblk_q: its number of diagonal blocks)
        if (b + 1 < nblk_q - 1) {
            ++b;
            return true;
        }
        return false;
    }
    int nq = q < 0 ? (int)blockIdx.x : q + L.nchain_cta, nb = q < 0 ? -1 : b;
    for (;;) {
        if (nq >= L.nchains) {
            nq = blockIdx.x;
            if (++nb >= L.steps - 1) return false;
        }
        if (nb < L.chains[nq].kn - 1) {
            q = nq;
            b = nb;
            return true;
        }
        nq += L.nchain_cta;
    }
}

// Right-hand sides of the level kernels.  RG columns of the solve go through
// each chain duty and each bulk item together: the current solution block
// (y or x) and the solved block's right-hand side (f or g) sit in shared memory
// as SB rows of RG values (row stride RS, padded so that the backward kernel's
// skewed rows are read without bank conflicts), next to the partial sums of the
// TP thread groups that split each product.
template <class Cv, int SB, int RG>
struct LevelRhs {
    static constexpr int TP = 256 / SB;                  // thread groups splitting one product
    static constexpr int RS = RG >= 4 ? RG + 4 : RG;     // row stride of the solution and right-hand blocks
    static constexpr int FG = RG >= TP ? RG / TP : RG;   // right-hand sides one thread finishes
    static constexpr size_t bytes = (size_t)(2 * SB * RS + TP * SB * RG) * sizeof(Cv);
};

// Dynamic shared memory of a level kernel: two tile buffers, then the right-hand-side area.
template <class T, class Cv, int SB, int RG>
constexpr size_t level_smem_bytes() {
    return (size_t)SB * SB * (sizeof(T) + sizeof(Cv)) + LevelRhs<Cv, SB, RG>::bytes + kLevelSmemSlack;
}

// Sums of RG right-hand sides.  With one right-hand side four independent sums
// hide the latency of the multiply-adds; with several, the right-hand sides do.
template <class Cv, int RG>
struct RhsAcc {
    static constexpr int NA = RG >= 4 ? 1 : 4;
    Cv v[NA][RG];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int g = 0; g < RG; ++g) v[a][g] = Cv(0);
    }
    // v[j] += t * y[0, RG) (y: 16-byte aligned when RG is a multiple of 4); j is a compile-time index
    __device__ __forceinline__ void add(int j, Cv t, const Cv* y) {
        Cv* a = v[j & (NA - 1)];
        if constexpr (RG % 4 == 0 && sizeof(Cv) == 4) {
#pragma unroll
            for (int g = 0; g < RG; g += 4) {
                const float4 q = *reinterpret_cast<const float4*>(y + g);
                a[g] += t * q.x;
                a[g + 1] += t * q.y;
                a[g + 2] += t * q.z;
                a[g + 3] += t * q.w;
            }
        } else if constexpr (RG % 2 == 0 && sizeof(Cv) == 8) {
#pragma unroll
            for (int g = 0; g < RG; g += 2) {
                const double2 q = *reinterpret_cast<const double2*>(y + g);
                a[g] += t * q.x;
                a[g + 1] += t * q.y;
            }
        } else {
#pragma unroll
            for (int g = 0; g < RG; ++g) a[g] += t * y[g];
        }
    }
    __device__ __forceinline__ Cv sum(int g) const {
        if constexpr (NA == 4) return (v[0][g] + v[1][g]) + (v[2][g] + v[3][g]);
        else return v[0][g];
    }
    // p[0, RG) = the sums (16-byte aligned when RG is a multiple of 4)
    __device__ __forceinline__ void store(Cv* p) const {
        if constexpr (RG % 4 == 0 && sizeof(Cv) == 4) {
#pragma unroll
            for (int g = 0; g < RG; g += 4)
                *reinterpret_cast<float4*>(p + g) = make_float4(sum(g), sum(g + 1), sum(g + 2), sum(g + 3));
        } else {
#pragma unroll
            for (int g = 0; g < RG; ++g) p[g] = sum(g);
        }
    }
};

// Forward.  Chain duty (front, b): y_{b+1} = L_{b+1}^-1 (f_{b+1} - L[b+1, b] y_b),
// where the bulk has already applied y_0 .. y_{b-1} to f_{b+1}; writes y and
// y / D (the work vector).  Bulk chunk of diagonal block `own` applies
// y_0 .. y_{own-2}; a chunk of trailing rows applies every y_b and ends as
// the front's update vector.  Both sides: SB rows, 256 / SB threads per row
// splitting the columns, RG right-hand sides at a time.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 1) k_fwd_level(LevelArgs L, SolveArgs A, const T* __restrict__ panel,
                                                      const Cv* __restrict__ linv, Cv* fv, Cv* yv,
                                                      const double* __restrict__ diag, Cv* work) {
    using R = LevelRhs<Cv, SB, RG>;
    constexpr int TPR = R::TP;       // threads per row
    constexpr int CPT = SB / TPR;    // columns per thread
    constexpr int RS = R::RS, FG = R::FG;
    extern __shared__ __align__(128) unsigned char blk_smem[];
    // copy destinations aligned to 1024 bytes (the launch adds kLevelSmemSlack)
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    T* Tl = reinterpret_cast<T*>(sm);                          // tile L[b+1, b], column-major
    Cv* Li = reinterpret_cast<Cv*>(sm + SB * SB * sizeof(T));  // inverse of block b+1, column-major
    Cv* yb = Li + SB * SB;                                     // y_b: SB rows x RG
    Cv* fb = yb + SB * RS;                                     // f_{b+1} - L[b+1, b] y_b
    Cv* part = fb + SB * RS;                                   // [TPR][SB][RG] partial sums
    __shared__ int ok;
    __shared__ unsigned long long tbar;
    __shared__ unsigned long long sbar[2];
    const int tid = threadIdx.x, row = tid % SB, pid = tid / SB;
    // the thread finishing right-hand sides [g0, g0 + FG) of its row
    const bool fin = RG >= TPR || pid == 0;
    const int g0 = RG >= TPR ? pid * FG : 0;
    const int nr = A.nrhs;
    const bool one_group = nr <= RG;
    // y_b of right-hand sides [rg, rg + ng) into yb (zero past kb rows and ng columns)
    auto load_y = [&](long long fo, int rg, int ng, int b, int kb) {
        for (int t = tid; t < SB * RG; t += blockDim.x) {
            const int g = t / SB, k = t - g * SB;
            yb[k * RS + g] = (g < ng && k < kb) ? __ldcg(yv + fo + (long long)(rg + g) * A.fv_stride + b * SB + k) : Cv(0);
        }
    };
    if ((int)blockIdx.x < L.nchain_cta) {
        // tile rows past a partial block are multiplied by zero: start from zeros, not stale bits
        for (int i = tid; i < SB * SB; i += blockDim.x) {
            Tl[i] = T(0);
            Li[i] = Cv(0);
        }
        if (tid == 0) bar_init(&tbar);
        __syncthreads();
        unsigned phase = 0;
        int q = -1, b = -1;
        if (!next_chain_duty(L, q, b, 0)) return;
        // descriptors of the current front, reloaded only when the front changes
        int cq = -1;
        SolveBlockTask c;
        SnDev d;
        auto front = [&](int qq) {
            if (qq != cq) {
                c = L.chains[qq];
                d = A.sn[c.s];
                cq = qq;
            }
        };
        auto prefetch = [&](int qq, int bb) {
            front(qq);
            const int r0 = (bb + 1) * SB, kn = min(SB, d.w - r0);
            start_tile_copy<T, Cv, SB>(Tl, Li, L.maps + c.s, r0, bb * SB, bb >= 0,
                                       linv + (long long)(c.blk + bb + 1) * SB * SB, kn, &tbar);
        };
        prefetch(q, b);
        int held = -1;   // front whose y_b is in yb (all right-hand sides in one group)
        for (;;) {
            front(q);
            const int r0 = (b + 1) * SB, kn = min(SB, d.w - r0);
            const int kb = b >= 0 ? min(SB, d.w - b * SB) : 0;
            const long long fo = A.fvec_off[c.s];
            for (int rg = 0; rg < nr; rg += RG) {
                const int ng = min(RG, nr - rg);
                if (b >= 0 && !(one_group && held == q)) {
                    __syncthreads();
                    load_y(fo, rg, ng, b, kb);
                }
                if (rg == 0) {
                    if (!__syncthreads_and(bar_wait(&tbar, phase, L.status))) return;
                    phase ^= 1;
                }
                __syncthreads();
                // f_{b+1} - L[b+1, b] y_b: thread (row, pid) sums columns [pid CPT, pid CPT + CPT)
                RhsAcc<Cv, RG> acc;
                acc.zero();
                if (b >= 0) {
#pragma unroll 2
                    for (int u0 = 0; u0 < CPT; u0 += 4)
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int k = pid * CPT + u0 + j;
                            acc.add(j, (Cv)Tl[row + k * SB], yb + k * RS);
                        }
                }
                acc.store(part + (pid * SB + row) * RG);
                // only now the bulk's part: chunk b+1 has applied y_0 .. y_{b-1} (the product above
                // needs neither it nor f, so it overlaps the bulk's last update)
                if (rg == 0 && b >= 1 && !wait_at_least(L.progress + c.k0 + b + 1, b, L.status, &ok)) return;
                Cv f0[FG];
#pragma unroll
                for (int j = 0; j < FG; ++j) {
                    const int g = g0 + j;
                    f0[j] = (fin && row < kn && g < ng) ? __ldcg(fv + fo + (long long)(rg + g) * A.fv_stride + r0 + row)
                                                        : Cv(0);
                }
                __syncthreads();
                if (fin) {
#pragma unroll
                    for (int j = 0; j < FG; ++j) {
                        const int g = g0 + j;
                        Cv v = f0[j];
#pragma unroll
                        for (int p = 0; p < TPR; ++p) v -= part[(p * SB + row) * RG + g];
                        fb[row * RS + g] = row < kn ? v : Cv(0);
                    }
                }
                __syncthreads();
                // y = L_{b+1}^-1 f: thread (row, pid) sums k in [pid CPT, pid CPT + CPT), k <= row
                acc.zero();
                {
                    const int kend = min(pid * CPT + CPT, row + 1);
                    int k = pid * CPT;
                    for (; k + 4 <= kend; k += 4)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc.add(j, Li[row + (k + j) * SB], fb + (k + j) * RS);
                    for (; k < kend; ++k) acc.add(0, Li[row + k * SB], fb + k * RS);
                }
                acc.store(part + (pid * SB + row) * RG);
                __syncthreads();
                if (fin) {
#pragma unroll
                    for (int j = 0; j < FG; ++j) {
                        const int g = g0 + j;
                        Cv y = part[row * RG + g];
#pragma unroll
                        for (int p = 1; p < TPR; ++p) y += part[(p * SB + row) * RG + g];
                        const bool live = row < kn && g < ng;
                        if (live) {
                            const int col = r0 + row;
                            yv[fo + (long long)(rg + g) * A.fv_stride + col] = y;
                            work[d.first_col + col + (long long)(rg + g) * A.ldw] =
                                (Cv)((double)y / diag[d.first_col + col]);
                        }
                        yb[row * RS + g] = live ? y : Cv(0);   // y_{b+1}, kept for this front's next duty
                    }
                }
            }
            held = q;
            publish(L.flags + c.blk + b + 1, 1);
            if (!next_chain_duty(L, q, b, c.kn)) return;
            prefetch(q, b);
        }
    }
    // ---- bulk CTA: work items (step b, chunk q) in step-major order over its share of the chunks.
    // Tiles come by tensor-map copies into two stage buffers (the chain's tile and inverse space),
    // the next item's copy in flight while the current one is applied; the flag and y_b of
    // consecutive items of one front are shared.
    const BulkRange Rg = bulk_range(L);
    if (Rg.begin >= Rg.end || Rg.step <= 0) return;
    auto stage = [&](int k) { return k ? reinterpret_cast<T*>(Li) : Tl; };
    if (tid == 0) {
        bar_init(&sbar[0]);
        bar_init(&sbar[1]);
    }
    __syncthreads();
    unsigned phbits = 0;   // expected parity of each stage barrier
    auto next_item = [&](int& b, int& q) {
        for (;;) {
            q = q < 0 ? Rg.begin : q + Rg.step;
            if (q >= Rg.end) {
                q = -1;
                if (++b >= L.steps) return false;
                continue;
            }
            if (b < L.bulk[q].kn) return true;   // kn = the chunk's number of solutions to apply
        }
    };
    // tile rows start at the chunk's first row rounded down to 16 bytes (trailing-row chunks are
    // SB - 16 / sizeof(T) rows high, so the box still covers them)
    constexpr int kAlign = 16 / (int)sizeof(T);
    auto issue = [&](int st_, int b, int q) {
        if (tid == 0)
            start_bulk_tile<T, SB>(stage(st_), L.maps + L.bulk[q].s, L.bulk[q].r0 & ~(kAlign - 1), b * SB, &sbar[st_]);
    };
    int seen_blk = -1, seen_b = -1, prev_q = -1;
    Cv fcur[FG];   // f of this thread's row after the previous item (all right-hand sides in one group)
#pragma unroll
    for (int j = 0; j < FG; ++j) fcur[j] = Cv(0);
    int b0 = 0, q0 = -1;
    if (!next_item(b0, q0)) return;
    int b1 = b0, q1 = q0;
    bool has1 = next_item(b1, q1);
    issue(0, b0, q0);
    if (has1) issue(1, b1, q1);
    int cur = 0;
    for (;;) {
        const SolveBlockTask c = L.bulk[q0];
        const SnDev d = A.sn[c.s];
        const int kb = min(SB, d.w - b0 * SB), i = c.r0 + row;
        const bool same = c.blk == seen_blk && b0 == seen_b;
        const long long fo = A.fvec_off[c.s];
        // f of the row, issued before the waits (this thread wrote it last, if anyone did)
        Cv fold[FG];
#pragma unroll
        for (int j = 0; j < FG; ++j) {
            const int g = g0 + j;
            fold[j] = (one_group && fin && i < c.r1 && g < nr)
                          ? (q0 == prev_q ? fcur[j] : fv[fo + (long long)g * A.fv_stride + i])
                          : Cv(0);
        }
        if (!same && !wait_at_least(L.flags + c.blk + b0, 1, L.status, &ok)) return;
        for (int rg = 0; rg < nr; rg += RG) {
            const int ng = min(RG, nr - rg);
            if (!(same && one_group)) {
                __syncthreads();
                load_y(fo, rg, ng, b0, kb);
            }
            if (rg == 0) {
                if (!__syncthreads_and(bar_wait(&sbar[cur], (phbits >> cur) & 1u, L.status))) return;
                phbits ^= 1u << cur;
            }
            __syncthreads();
            const T* tile = stage(cur);
            const int trow = min(row + (c.r0 & (kAlign - 1)), SB - 1);   // idle rows past the chunk: clamped
            RhsAcc<Cv, RG> acc;
            acc.zero();
#pragma unroll 2
            for (int u0 = 0; u0 < CPT; u0 += 4)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int k = pid * CPT + u0 + j;
                    acc.add(j, (Cv)tile[trow + k * SB], yb + k * RS);
                }
            acc.store(part + (pid * SB + row) * RG);
            __syncthreads();
            if (fin && i < c.r1) {
#pragma unroll
                for (int j = 0; j < FG; ++j) {
                    const int g = g0 + j;
                    if (g >= ng) break;
                    Cv sum = part[row * RG + g];
#pragma unroll
                    for (int p = 1; p < TPR; ++p) sum += part[(p * SB + row) * RG + g];
                    Cv* fp = fv + fo + (long long)(rg + g) * A.fv_stride + i;
                    const Cv f = (one_group ? fold[j] : *fp) - sum;
                    *fp = f;
                    fcur[j] = f;
                }
            }
        }
        seen_blk = c.blk;
        seen_b = b0;
        prev_q = q0;
        if (c.r0 < d.w) publish(L.progress + q0, b0 + 1);
        __syncthreads();   // the stage buffer is free again
        if (!has1) return;
        int b2 = b1, q2 = q1;
        const bool has2 = next_item(b2, q2);
        if (has2) issue(cur, b2, q2);
        b0 = b1;
        q0 = q1;
        b1 = b2;
        q1 = q2;
        has1 = has2;
        cur ^= 1;
    }
}

// Backward.  Chain duty (front, t) for block b = nblk-1-t: x_{b-1} =
// L_{b-1}^-T (g_{b-1} - L[b, b-1]^T x_b), where the bulk has already applied
// x_{nblk-1} .. x_{b+1} to g_{b-1} (t = -1 solves the last block from g after
// the trailing rows' contribution); writes x to the work vector.  Bulk chunk
// of own columns of block `own` applies x_{nblk-1} .. x_{own+2}.  Both sides:
// thread (column, part) sums its part of the rows in skewed order (row
// part*RPT + (u + column) mod RPT), so that the threads of a warp read
// different banks of the column-major tile; RG right-hand sides at a time.
template <class T, class Cv, int SB, int RG>
__global__ void __launch_bounds__(256, 1) k_bwd_level(LevelArgs L, SolveArgs A, const T* __restrict__ panel,
                                                      const Cv* __restrict__ linv, Cv* fv, Cv* xv, Cv* work) {
    using R = LevelRhs<Cv, SB, RG>;
    constexpr int TPC = R::TP;      // threads per column
    constexpr int RPT = SB / TPC;   // rows per thread (a power of two)
    constexpr int RS = R::RS, FG = R::FG;
    extern __shared__ __align__(128) unsigned char blk_smem[];
    unsigned char* sm = blk_smem + ((1024u - (smem_addr(blk_smem) & 1023u)) & 1023u);
    T* Tl = reinterpret_cast<T*>(sm);                          // tile L[b, b-1], column-major
    Cv* Li = reinterpret_cast<Cv*>(sm + SB * SB * sizeof(T));  // inverse of block b-1, column-major
    Cv* xb = Li + SB * SB;                                     // x_b: SB rows x RG
    Cv* gb = xb + SB * RS;                                     // g_{b-1} - L[b, b-1]^T x_b
    Cv* part = gb + SB * RS;                                   // [TPC][SB][RG] partial sums
    __shared__ int ok;
    __shared__ unsigned long long tbar;
    __shared__ unsigned long long sbar[2];
    const int tid = threadIdx.x, ccol = tid % SB, cpart = tid / SB;
    const bool fin = RG >= TPC || cpart == 0;
    const int g0 = RG >= TPC ? cpart * FG : 0;
    const int nr = A.nrhs;
    const bool one_group = nr <= RG;
    auto load_x = [&](long long fo, int rg, int ng, int b, int kb) {
        for (int e = tid; e < SB * RG; e += blockDim.x) {
            const int g = e / SB, i = e - g * SB;
            xb[i * RS + g] = (g < ng && i < kb) ? __ldcg(xv + fo + (long long)(rg + g) * A.fv_stride + b * SB + i) : Cv(0);
        }
    };
    // acc += tile^T x over this thread's rows of column ccol (skewed order)
    auto tile_t_x = [&](RhsAcc<Cv, RG>& acc, const T* tile) {
#pragma unroll 2
        for (int u0 = 0; u0 < RPT; u0 += 4)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = cpart * RPT + ((u0 + j + ccol) & (RPT - 1));
                acc.add(j, (Cv)tile[i + ccol * SB], xb + i * RS);
            }
    };
    if ((int)blockIdx.x < L.nchain_cta) {
        // tile rows past a partial block are multiplied by zero: start from zeros, not stale bits
        for (int i = tid; i < SB * SB; i += blockDim.x) {
            Tl[i] = T(0);
            Li[i] = Cv(0);
        }
        if (tid == 0) bar_init(&tbar);
        __syncthreads();
        unsigned phase = 0;
        int q = -1, t = -1;
        if (!next_chain_duty(L, q, t, 0)) return;
        int cq = -1;
        SolveBlockTask c;
        SnDev d;
        auto front = [&](int qq) {
            if (qq != cq) {
                c = L.chains[qq];
                d = A.sn[c.s];
                cq = qq;
            }
        };
        auto prefetch = [&](int qq, int tt) {
            front(qq);
            const int bb = c.kn - 1 - tt;   // duty tt solves block bb - 1
            start_tile_copy<T, Cv, SB>(Tl, Li, L.maps + c.s, bb * SB, (bb - 1) * SB, tt >= 0,
                                       linv + (long long)(c.blk + bb - 1) * SB * SB, min(SB, d.w - (bb - 1) * SB), &tbar);
        };
        prefetch(q, t);
        int held = -1;   // front whose x_b is in xb (all right-hand sides in one group)
        for (;;) {
            front(q);
            const int b = c.kn - 1 - t;                        // x_b is applied (t >= 0)
            const int tgt = b - 1;                             // block solved by this duty
            const int c0 = tgt * SB, kn = min(SB, d.w - c0);
            const int kb = t >= 0 ? min(SB, d.w - b * SB) : 0;  // rows of block b
            const long long fo = A.fvec_off[c.s];
            for (int rg = 0; rg < nr; rg += RG) {
                const int ng = min(RG, nr - rg);
                if (t >= 0 && !(one_group && held == q)) {
                    __syncthreads();
                    load_x(fo, rg, ng, b, kb);
                }
                if (rg == 0) {
                    if (!__syncthreads_and(bar_wait(&tbar, phase, L.status))) return;
                    phase ^= 1;
                }
                __syncthreads();
                // g_{b-1} -= L[b, b-1]^T x_b
                RhsAcc<Cv, RG> acc;
                acc.zero();
                if (t >= 0) tile_t_x(acc, Tl);
                acc.store(part + (cpart * SB + ccol) * RG);
                // only now the bulk's part: chunk b-1 has applied x_{nblk-1} .. x_{b+1}; then g of
                // the block's columns
                if (rg == 0 && t >= 1 && !wait_at_least(L.progress + c.k0 + tgt, t, L.status, &ok)) return;
                for (int e = tid; e < SB * RG; e += blockDim.x) {
                    const int g = e / SB, k = e - g * SB;
                    gb[k * RS + g] = (g < ng && k < kn) ? __ldcg(fv + fo + (long long)(rg + g) * A.fv_stride + c0 + k) : Cv(0);
                }
                __syncthreads();
                if (t >= 0 && fin && ccol < kn) {
#pragma unroll
                    for (int j = 0; j < FG; ++j) {
                        const int g = g0 + j;
                        Cv sum = part[ccol * RG + g];
#pragma unroll
                        for (int p = 1; p < TPC; ++p) sum += part[(p * SB + ccol) * RG + g];
                        gb[ccol * RS + g] -= sum;
                    }
                }
                __syncthreads();
                // x = Li^T g: column ccol of the inverse against g, the same skewed split (k >= ccol)
                acc.zero();
#pragma unroll 2
                for (int u0 = 0; u0 < RPT; u0 += 4)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int k = cpart * RPT + ((u0 + j + ccol) & (RPT - 1));
                        if (k >= ccol && k < kn) acc.add(j, Li[k + ccol * SB], gb + k * RS);
                    }
                acc.store(part + (cpart * SB + ccol) * RG);
                __syncthreads();
                if (fin) {
#pragma unroll
                    for (int j = 0; j < FG; ++j) {
                        const int g = g0 + j;
                        Cv x = part[ccol * RG + g];
#pragma unroll
                        for (int p = 1; p < TPC; ++p) x += part[(p * SB + ccol) * RG + g];
                        const bool live = ccol < kn && g < ng;
                        if (live) {
                            xv[fo + (long long)(rg + g) * A.fv_stride + c0 + ccol] = x;
                            work[d.first_col + c0 + ccol + (long long)(rg + g) * A.ldw] = x;
                        }
                        xb[ccol * RS + g] = live ? x : Cv(0);   // x_{b-1}, kept for this front's next duty
                    }
                }
            }
            held = q;
            publish(L.flags + c.blk + tgt, 1);
            if (!next_chain_duty(L, q, t, c.kn)) return;
            prefetch(q, t);
        }
    }
    // ---- bulk CTA: work items (step t, chunk q) over its share of the chunks; tiles by tensor-map
    // copies into two stage buffers, as in the forward kernel
    const BulkRange Rg = bulk_range(L);
    if (Rg.begin >= Rg.end || Rg.step <= 0) return;
    auto stage = [&](int k) { return k ? reinterpret_cast<T*>(Li) : Tl; };
    if (tid == 0) {
        bar_init(&sbar[0]);
        bar_init(&sbar[1]);
    }
    __syncthreads();
    unsigned phbits = 0;   // expected parity of each stage barrier
    auto next_item = [&](int& t, int& q) {
        for (;;) {
            q = q < 0 ? Rg.begin : q + Rg.step;
            if (q >= Rg.end) {
                q = -1;
                if (++t >= L.steps) return false;
                continue;
            }
            if (t < L.bulk[q].kn) return true;   // kn = the chunk's number of solutions to apply
        }
    };
    // rows of block b (x), the chunk's columns (y)
    auto issue = [&](int st_, int t, int q) {
        if (tid == 0)
            start_bulk_tile<T, SB>(stage(st_), L.maps + L.bulk[q].s, (L.bulk[q].k0 - t) * SB, L.bulk[q].r0, &sbar[st_]);
    };
    int seen_blk = -1, seen_b = -1, prev_q = -1;
    Cv gcur[FG];   // g of this thread's column after the previous item (all right-hand sides in one group)
#pragma unroll
    for (int j = 0; j < FG; ++j) gcur[j] = Cv(0);
    int t0 = 0, q0 = -1;
    if (!next_item(t0, q0)) return;
    int t1 = t0, q1 = q0;
    bool has1 = next_item(t1, q1);
    issue(0, t0, q0);
    if (has1) issue(1, t1, q1);
    int cur = 0;
    for (;;) {
        const SolveBlockTask c = L.bulk[q0];
        const SnDev d = A.sn[c.s];
        const int b = c.k0 - t0, kb = min(SB, d.w - b * SB);
        const bool same = c.blk == seen_blk && b == seen_b;
        const int col = c.r0 + ccol;
        const long long fo = A.fvec_off[c.s];
        // g of this thread's column, issued before the waits (this thread wrote it last, if anyone did)
        Cv gold[FG];
#pragma unroll
        for (int j = 0; j < FG; ++j) {
            const int g = g0 + j;
            gold[j] = (one_group && fin && col < c.r1 && g < nr)
                          ? (q0 == prev_q ? gcur[j] : fv[fo + (long long)g * A.fv_stride + col])
                          : Cv(0);
        }
        if (!same && !wait_at_least(L.flags + c.blk + b, 1, L.status, &ok)) return;
        for (int rg = 0; rg < nr; rg += RG) {
            const int ng = min(RG, nr - rg);
            if (!(same && one_group)) {
                __syncthreads();
                load_x(fo, rg, ng, b, kb);
            }
            if (rg == 0) {
                if (!__syncthreads_and(bar_wait(&sbar[cur], (phbits >> cur) & 1u, L.status))) return;
                phbits ^= 1u << cur;
            }
            __syncthreads();
            RhsAcc<Cv, RG> acc;
            acc.zero();
            tile_t_x(acc, stage(cur));
            acc.store(part + (cpart * SB + ccol) * RG);
            __syncthreads();
            if (fin && col < c.r1) {
#pragma unroll
                for (int j = 0; j < FG; ++j) {
                    const int g = g0 + j;
                    if (g >= ng) break;
                    Cv sum = part[ccol * RG + g];
#pragma unroll
                    for (int p = 1; p < TPC; ++p) sum += part[(p * SB + ccol) * RG + g];
                    Cv* gp = fv + fo + (long long)(rg + g) * A.fv_stride + col;
                    const Cv gv = (one_group ? gold[j] : *gp) - sum;
                    *gp = gv;
                    gcur[j] = gv;
                }
            }
        }
        seen_blk = c.blk;
        seen_b = b;
        prev_q = q0;
        publish(L.progress + q0, t0 + 1);
        __syncthreads();
        if (!has1) return;
        int t2 = t1, q2 = q1;
        const bool has2 = next_item(t2, q2);
        if (has2) issue(cur, t2, q2);
        t0 = t1;
        q0 = q1;
        t1 = t2;
        q1 = q2;
        has1 = has2;
        cur ^= 1;
    }
}

// Fronts of one diagonal block (most fronts low in the tree) need no chain:
// one CTA per front solves its block and, forward, updates its trailing rows.

// Forward: y = L_0^-1 f_0 (thread per row), y / D to the work vector, then
// f[i] -= L[i, 0:w] y for the trailing rows (thread per row, coalesced columns).
template <class T, class Cv, int SB>
__global__ void __launch_bounds__(256) k_fwd_solo(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                  const T* __restrict__ panel, const Cv* __restrict__ linv,
                                                  Cv* __restrict__ fv, Cv* __restrict__ yv,
                                                  const double* __restrict__ diag, Cv* __restrict__ work) {
    __shared__ Cv f0[SB];
    __shared__ Cv y[SB];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int w = d.w, tid = threadIdx.x;
    const Cv* Li = linv + (long long)tk.blk * SB * SB;
    const T* P = panel + d.panel_off;
    for (int r = 0; r < A.nrhs; ++r) {
        const long long base = A.fvec_off[tk.s] + r * A.fv_stride;
        Cv* f = fv + base;
        __syncthreads();
        for (int t = tid; t < w; t += blockDim.x) f0[t] = f[t];
        __syncthreads();
        for (int t = tid; t < w; t += blockDim.x) {
            Cv a0 = Cv(0), a1 = Cv(0);
            int k = 0;
            for (; k + 1 <= t; k += 2) {
                a0 += Li[t + k * SB] * f0[k];
                a1 += Li[t + (k + 1) * SB] * f0[k + 1];
            }
            for (; k <= t; ++k) a0 += Li[t + k * SB] * f0[k];
            const Cv v = a0 + a1;
            y[t] = v;
            yv[base + t] = v;
            work[d.first_col + t + (long long)r * A.ldw] = (Cv)((double)v / diag[d.first_col + t]);
        }
    }
}

// Four consecutive entries of a factor column (16- or 32-byte aligned), widened.
__device__ __forceinline__ void load4(const float* p, float* v) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x;
    v[1] = x.y;
    v[2] = x.z;
    v[3] = x.w;
}
__device__ __forceinline__ void load4(const double* p, double* v) {
    const double2 x = reinterpret_cast<const double2*>(p)[0], z = reinterpret_cast<const double2*>(p)[1];
    v[0] = x.x;
    v[1] = x.y;
    v[2] = z.x;
    v[3] = z.y;
}

// Forward, trailing rows of single-block fronts (after k_fwd_solo): f[i] -= sum_k L[i, k] y[k]
// for rows [r0, r1) of the task's front (r0 a multiple of 4; rows below w are skipped).
// Four consecutive rows per thread, one aligned group per column, eight columns in flight,
// so a front's trailing block streams at HBM speed over many CTAs instead of one.  The
// right-hand sides go in groups of G: each factor entry is read once per group.
constexpr int kTailRows = 1024;
template <class T, class Cv, int SB, int G>
__global__ void __launch_bounds__(kTailRows / 4) k_fwd_tail(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                            const T* __restrict__ panel, const Cv* __restrict__ yv,
                                                            Cv* __restrict__ fv) {
    __shared__ Cv y[G][SB];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int w = d.w;
    const int i = tk.r0 + 4 * (int)threadIdx.x;
    const T* p = panel + d.panel_off + i;
    for (int r0 = 0; r0 < A.nrhs; r0 += G) {
        const int ng = min(G, A.nrhs - r0);
        __syncthreads();
        for (int t = threadIdx.x; t < G * SB; t += blockDim.x) {
            const int g = t / SB, kk = t - g * SB;
            y[g][kk] = (g < ng && kk < w) ? __ldcg(yv + A.fvec_off[tk.s] + (r0 + g) * A.fv_stride + kk) : Cv(0);
        }
        __syncthreads();
        if (i >= tk.r1) continue;
        Cv a[G][4];
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
            for (int e = 0; e < 4; ++e) a[g][e] = Cv(0);
        int k = 0;
        for (; k + 8 <= w; k += 8) {
            T v[8][4];
#pragma unroll
            for (int u = 0; u < 8; ++u) load4(p + (long long)(k + u) * d.ldp, v[u]);
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const Cv yk = y[g][k + u];
#pragma unroll
                    for (int e = 0; e < 4; ++e) a[g][e] += (Cv)v[u][e] * yk;
                }
        }
        for (; k < w; ++k) {
            T v[4];
            load4(p + (long long)k * d.ldp, v);
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const Cv yk = y[g][k];
#pragma unroll
                for (int e = 0; e < 4; ++e) a[g][e] += (Cv)v[e] * yk;
            }
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            if (g >= ng) break;
            Cv* f = fv + A.fvec_off[tk.s] + (r0 + g) * A.fv_stride;
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (i + e >= w && i + e < tk.r1) f[i + e] -= a[g][e];
        }
    }
}

// Backward: x = L_0^-T g (warp per output, lanes over the inverse's column),
// after the trailing rows' contribution; x to the work vector.
template <class Cv, int SB>
__global__ void __launch_bounds__(256) k_bwd_solo(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                  const Cv* __restrict__ linv, Cv* __restrict__ fv,
                                                  Cv* __restrict__ xv, Cv* __restrict__ work) {
    __shared__ Cv g0[SB];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const SnDev d = A.sn[tk.s];
    const int w = d.w, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
    const Cv* Li = linv + (long long)tk.blk * SB * SB;
    for (int r = 0; r < A.nrhs; ++r) {
        const long long base = A.fvec_off[tk.s] + r * A.fv_stride;
        __syncthreads();
        for (int t = tid; t < w; t += blockDim.x) g0[t] = fv[base + t];
        __syncthreads();
        for (int t = warp; t < w; t += nwarps) {
            Cv acc = Cv(0);
            for (int k = t + lane; k < w; k += 32) acc += Li[k + t * SB] * g0[k];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) {
                xv[base + t] = acc;
                work[d.first_col + t + (long long)r * A.ldw] = acc;
            }
        }
    }
}

template <class Cv>
__global__ void k_bwd_gather(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const Cv* __restrict__ work,
                             Cv* __restrict__ fv) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    const int* rows = A.rows + d.rows_off;
    for (int r = blockIdx.y; r < A.nrhs; r += gridDim.y) {
        Cv* g = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x) g[a] = work[rows[a] + (long long)r * A.ldw];
    }
}

// g[k] -= sum_{i in [r0, r1)} L[i,k] g[i] for columns k in [k0, k0+kn), one warp per column,
// RG right-hand sides at a time (each column entry is loaded once per group).
// Rows are read 16 bytes at a time between a scalar head and tail: a panel
// column and the front vector start on 16-byte boundaries (panel offsets are
// multiples of 64 elements, ldp, front-vector offsets and their stride of 8),
// so row i of both is aligned exactly when i is a multiple of 16 / sizeof(element).
template <class T, class Cv, int RG>
__global__ void k_bwd_cols(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const T* __restrict__ panel,
                           Cv* __restrict__ fv, Cv* __restrict__ partial) {
    static_assert(sizeof(T) == sizeof(Cv), "factor and vector elements of one size");
    constexpr int V = 16 / (int)sizeof(T);
    using Vec = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp >= tk.kn) return;
    const SnDev d = A.sn[tk.s];
    const int k = tk.k0 + warp;
    const T* col = panel + d.panel_off + (long long)k * d.ldp;
    const Vec* cv = reinterpret_cast<const Vec*>(col);
    const int head = min(tk.r1, (tk.r0 + V - 1) / V * V), body = max(head, tk.r1 / V * V);
    auto dot = [](const Vec& a, const Vec& b) -> Cv {
        if constexpr (V == 4) return (Cv)a.x * b.x + (Cv)a.y * b.y + (Cv)a.z * b.z + (Cv)a.w * b.w;
        else return (Cv)a.x * b.x + (Cv)a.y * b.y;
    };
    for (int rg = 0; rg < A.nrhs; rg += RG) {
        const int ng = min(RG, A.nrhs - rg);
        Cv* g = fv + A.fvec_off[tk.s] + (long long)rg * A.fv_stride;
        Cv acc[RG];
#pragma unroll
        for (int r = 0; r < RG; ++r) acc[r] = Cv(0);
        for (int i = tk.r0 + lane; i < head; i += 32) {
            const Cv a = (Cv)col[i];
#pragma unroll
            for (int r = 0; r < RG; ++r)
                if (r < ng) acc[r] += a * g[r * A.fv_stride + i];
        }
        int v = head / V + lane;
        if constexpr (RG == 1) {
            for (; v + 32 < body / V; v += 64) {   // two 16-byte loads of each in flight per lane
                const Vec* gv = reinterpret_cast<const Vec*>(g);
                const Vec a0 = cv[v], a1 = cv[v + 32], b0 = gv[v], b1 = gv[v + 32];
                acc[0] += dot(a0, b0);
                acc[0] += dot(a1, b1);
            }
        }
        for (; v < body / V; v += 32) {
            const Vec a = cv[v];
#pragma unroll
            for (int r = 0; r < RG; ++r)
                if (r < ng) acc[r] += dot(a, reinterpret_cast<const Vec*>(g + r * A.fv_stride)[v]);
        }
        for (int i = body + lane; i < tk.r1; i += 32) {
            const Cv a = (Cv)col[i];
#pragma unroll
            for (int r = 0; r < RG; ++r)
                if (r < ng) acc[r] += a * g[r * A.fv_stride + i];
        }
#pragma unroll
        for (int r = 0; r < RG; ++r)
            for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < RG; ++r) {
                if (r >= ng) break;
                if (tk.flags) partial[((long long)tk.blk * 8 + warp) * A.nrhs + rg + r] = acc[r];   // one row chunk
                else g[r * A.fv_stride + k] -= acc[r];
            }
        }
    }
}

// Columns split into row chunks: g[k] -= the chunks' partial sums, added in chunk order.
// Task: columns [k0, k0 + kn) of front s, partial slots [r0, r0 + r1).
template <class Cv>
__global__ void k_bwd_cols_reduce(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                  const Cv* __restrict__ partial, Cv* __restrict__ fv) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    for (int t = threadIdx.x; t < tk.kn * A.nrhs; t += blockDim.x) {
        const int kk = t % tk.kn, r = t / tk.kn;
        Cv sum = Cv(0);
        for (int q = 0; q < tk.r1; ++q) sum += partial[((long long)(tk.r0 + q) * 8 + kk) * A.nrhs + r];
        fv[A.fvec_off[tk.s] + r * A.fv_stride + tk.k0 + kk] -= sum;
    }
}

// ---- FP64 symmetric product through a full (both triangles) CSR ----

// full_val[k] = values[full_src[k]] — refreshed once per factorisation.
__global__ void k_gather_values(const double* __restrict__ values, const int* __restrict__ src, long long count,
                                double* __restrict__ out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count; k += (long long)gridDim.x * blockDim.x)
        out[k] = values[src[k]];
}

// r = b - A x (or y = A x when b is null), one warp per row.
__global__ void k_spmv_residual(const int* __restrict__ ptr, const int* __restrict__ col, const double* __restrict__ val,
                                int n, int nrhs, const double* __restrict__ x, int ldx, const double* __restrict__ b,
                                int ldb, double* __restrict__ out, int ldo) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int row = warp;
    if (row >= n) return;
    const int p0 = ptr[row], p1 = ptr[row + 1];
    for (int r = 0; r < nrhs; ++r) {
        const double* xr = x + (long long)r * ldx;
        double acc = 0.0;
        for (int p = p0 + lane; p < p1; p += 32) acc += val[p] * xr[col[p]];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[row + (long long)r * ldo] = b ? b[row + (long long)r * ldb] - acc : acc;
    }
}

// Deterministic column dot products: stage 1 per-block partial sums.
constexpr int kDotBlocks = 256;
__global__ void k_dot_partial(const double* __restrict__ u, int ldu, const double* __restrict__ v, int ldv, int n,
                              double* __restrict__ partial) {
    __shared__ double red[256];
    const int r = blockIdx.y;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc += u[i + (long long)r * ldu] * v[i + (long long)r * ldv];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x + r * gridDim.x] = red[0];
}
__global__ void k_dot_finish(const double* __restrict__ partial, int blocks, int nrhs, double* __restrict__ out) {
    const int r = threadIdx.x;
    if (r >= nrhs) return;
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += partial[b + r * blocks];
    out[r] = s;
}

// x += alpha_r * p (per column), with alpha read from device memory.
__global__ void k_axpy_cols(double* __restrict__ x, int ldx, const double* __restrict__ p, int ldp,
                            const double* __restrict__ alpha, double sign, int n, int nrhs) {
    for (int r = blockIdx.y; r < nrhs; r += gridDim.y) {
        const double a = sign * alpha[r];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i + (long long)r * ldx] += a * p[i + (long long)r * ldp];
    }
}

// p = z + beta_r * p
__global__ void k_xpby_cols(const double* __restrict__ z, int ldz, double* __restrict__ p, int ldp,
                            const double* __restrict__ beta, int n, int nrhs) {
    for (int r = blockIdx.y; r < nrhs; r += gridDim.y) {
        const double bt = beta[r];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            p[i + (long long)r * ldp] = z[i + (long long)r * ldz] + bt * p[i + (long long)r * ldp];
    }
}

}  // namespace uchol_dev
