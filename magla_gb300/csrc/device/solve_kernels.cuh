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
// contiguous range found by binary search).
__device__ __forceinline__ int lower_bound_int(const int* a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <class Cv>
__global__ void k_fwd_gather(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const Cv* __restrict__ work,
                             Cv* __restrict__ fv) {
    __shared__ int range[2];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    for (int r = 0; r < A.nrhs; ++r) {
        Cv* f = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x)
            f[a] = a < d.w ? work[d.first_col + a + (long long)r * A.ldw] : Cv(0);
        __syncthreads();
        for (int c = A.child_ptr[s]; c < A.child_ptr[s + 1]; ++c) {
            const int ch = A.children[c];
            const SnDev cd = A.sn[ch];
            const int t = cd.m - cd.w;
            const int* rl = A.rel + cd.rel_off;
            if (tk.r0 == 0 && tk.r1 == d.m) {   // the chunk is the whole front
                if (threadIdx.x == 0) {
                    range[0] = 0;
                    range[1] = t;
                }
            } else if (threadIdx.x == 0) {
                range[0] = lower_bound_int(rl, t, tk.r0);
                range[1] = lower_bound_int(rl, t, tk.r1);
            }
            __syncthreads();
            const Cv* u = fv + A.fvec_off[ch] + r * A.fv_stride + cd.w;
            for (int b = range[0] + threadIdx.x; b < range[1]; b += blockDim.x) f[rl[b]] += u[b];
            __syncthreads();
        }
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

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// Starts copying inverse block `src` (SB x SB) into shared memory.
template <class Cv, int SB>
__device__ __forceinline__ void prefetch_inverse(Cv* dst, const Cv* src) {
    constexpr int chunks = SB * SB * (int)sizeof(Cv) / 16;
    for (int q = threadIdx.x; q < chunks; q += blockDim.x) cp_async16(reinterpret_cast<char*>(dst) + 16 * q,
                                                                       reinterpret_cast<const char*>(src) + 16 * q);
}

// First block solution of each front: forward y_0 = L_00^-1 f_0 (after the
// gather), backward x_last = L_ll^-T g_last (after the trailing-row dots).
template <class Cv, int SB, bool FORWARD>
__global__ void __launch_bounds__(256) k_block_start(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                     const Cv* __restrict__ linv, const Cv* __restrict__ fv,
                                                     Cv* __restrict__ sol) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    Cv* Ls = reinterpret_cast<Cv*>(blk_smem);
    __shared__ Cv v[SB];
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int kn = tk.kn;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    prefetch_inverse<Cv, SB>(Ls, linv + (long long)tk.blk * SB * SB);
    cp_async_wait_all();
    for (int r = 0; r < A.nrhs; ++r) {
        const long long base = A.fvec_off[tk.s] + r * A.fv_stride;
        __syncthreads();
        for (int t = threadIdx.x; t < kn; t += blockDim.x) v[t] = fv[base + tk.k0 + t];
        __syncthreads();
        if (FORWARD) {
            // thread per output row: consecutive threads read consecutive words of each inverse column
            for (int t = threadIdx.x; t < kn; t += blockDim.x) {
                Cv acc = Cv(0);
                for (int k = 0; k <= t; ++k) acc += Ls[t + k * SB] * v[k];
                sol[base + tk.k0 + t] = acc;
            }
        } else {
            // warp per output: lanes read consecutive words of one inverse column
            for (int t = warp; t < kn; t += nwarps) {
                Cv acc = Cv(0);
                for (int k = t + lane; k < kn; k += 32) acc += Ls[k + t * SB] * v[k];
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) sol[base + tk.k0 + t] = acc;
            }
        }
    }
}

// Forward step of diagonal block b of a front: y_b (in the solution buffer)
// updates the task's rows, f[i] -= L[i, b] y_b.  The task whose rows are
// block b+1 then computes y_{b+1} from their final values with the inverse
// it prefetched at the start.
template <class T, class Cv, int SB>
__global__ void __launch_bounds__(128) k_fwd_block(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                   const T* __restrict__ panel, const Cv* __restrict__ linv,
                                                   Cv* __restrict__ fv, Cv* __restrict__ yv) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    Cv* Ls = reinterpret_cast<Cv*>(blk_smem);
    __shared__ Cv y[SB];
    __shared__ Cv fn[SB];
    const SolveBlockTask tk = blocks_or_tasks(tasks);
    const SnDev d = A.sn[tk.s];
    const T* P = panel + d.panel_off;
    const int kn = tk.kn;
    const bool next = tk.flags & kSolveNext;
    const int kn_next = next ? min(SB, d.w - (tk.k0 + kn)) : 0;
    if (next) prefetch_inverse<Cv, SB>(Ls, linv + (long long)(tk.blk + 1) * SB * SB);
    for (int r = 0; r < A.nrhs; ++r) {
        const long long base = A.fvec_off[tk.s] + r * A.fv_stride;
        Cv* f = fv + base;
        __syncthreads();
        for (int t = threadIdx.x; t < kn; t += blockDim.x) y[t] = yv[base + tk.k0 + t];
        __syncthreads();
        const int i = tk.r0 + threadIdx.x;
        if (i < tk.r1) {
            const T* row = P + i + (long long)tk.k0 * d.ldp;
            Cv acc[4] = {Cv(0), Cv(0), Cv(0), Cv(0)};
            int k = 0;
            for (; k + 32 <= kn; k += 32) {
                T vv[32];
#pragma unroll
                for (int u = 0; u < 32; ++u) vv[u] = row[(long long)(k + u) * d.ldp];
#pragma unroll
                for (int u = 0; u < 32; ++u) acc[u & 3] += (Cv)vv[u] * y[k + u];
            }
            for (; k < kn; ++k) acc[0] += (Cv)row[(long long)k * d.ldp] * y[k];
            const Cv nv = f[i] - ((acc[0] + acc[1]) + (acc[2] + acc[3]));
            f[i] = nv;
            if (next && threadIdx.x < kn_next) fn[threadIdx.x] = nv;
        }
        if (next) {
            if (r == 0) cp_async_wait_all();
            __syncthreads();
            for (int t = threadIdx.x; t < kn_next; t += blockDim.x) {
                Cv acc = Cv(0);
                for (int k = 0; k <= t; ++k) acc += Ls[t + k * SB] * fn[k];
                yv[base + tk.k0 + kn + t] = acc;
            }
        }
    }
}

// Backward step of diagonal block b of a front: x_b (in the solution buffer)
// updates the task's columns c < k0, g[c] -= L[b, c]^T x_b (warp-cooperative
// dots, four columns per warp pass).  The task whose columns are block b-1
// then computes x_{b-1}.
template <class T, class Cv, int SB>
__global__ void __launch_bounds__(256) k_bwd_block(const SolveBlockTask* __restrict__ tasks, SolveArgs A,
                                                   const T* __restrict__ panel, const Cv* __restrict__ linv,
                                                   Cv* __restrict__ fv, Cv* __restrict__ xv) {
    extern __shared__ __align__(16) unsigned char blk_smem[];
    Cv* Ls = reinterpret_cast<Cv*>(blk_smem);
    __shared__ Cv x[SB];
    __shared__ Cv gn[SB];
    const SolveBlockTask tk = blocks_or_tasks(tasks);
    const SnDev d = A.sn[tk.s];
    const T* P = panel + d.panel_off;
    const int kn = tk.kn;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const bool next = tk.flags & kSolveNext;
    if (next) prefetch_inverse<Cv, SB>(Ls, linv + (long long)(tk.blk - 1) * SB * SB);
    for (int r = 0; r < A.nrhs; ++r) {
        const long long base = A.fvec_off[tk.s] + r * A.fv_stride;
        Cv* g = fv + base;
        __syncthreads();
        for (int t = threadIdx.x; t < kn; t += blockDim.x) x[t] = xv[base + tk.k0 + t];
        __syncthreads();
        for (int c0 = tk.r0 + 4 * warp; c0 < tk.r1; c0 += 4 * nwarps) {
            Cv acc[4] = {Cv(0), Cv(0), Cv(0), Cv(0)};
            T vv[4][SB / 32];
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int u = 0; u < SB / 32; ++u) {
                    const int i = lane + 32 * u;
                    vv[q][u] = (c0 + q < tk.r1 && i < kn) ? P[(long long)(c0 + q) * d.ldp + tk.k0 + i] : T(0);
                }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int u = 0; u < SB / 32; ++u) {
                    const int i = lane + 32 * u;
                    if (i < kn) acc[q] += (Cv)vv[q][u] * x[i];
                }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                Cv a = acc[q];
                for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                if (lane == 0 && c0 + q < tk.r1) {
                    const Cv nv = g[c0 + q] - a;
                    g[c0 + q] = nv;
                    if (next) gn[c0 + q - tk.r0] = nv;
                }
            }
        }
        if (next) {
            if (r == 0) cp_async_wait_all();
            __syncthreads();
            for (int t = warp; t < SB; t += nwarps) {   // the previous block is always full width
                Cv acc = Cv(0);
                for (int k = t + lane; k < SB; k += 32) acc += Ls[k + t * SB] * gn[k];
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) xv[base + tk.r0 + t] = acc;
            }
        }
    }
}

// y = f / D for the supernode's own columns (the diagonal step of the solve).
template <class Cv>
__global__ void k_fwd_finish(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const double* __restrict__ diag,
                             const Cv* __restrict__ fv, Cv* __restrict__ work) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    for (int r = 0; r < A.nrhs; ++r) {
        const Cv* f = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x)
            work[d.first_col + a + (long long)r * A.ldw] = (Cv)((double)f[a] / diag[d.first_col + a]);
    }
}

template <class Cv>
__global__ void k_bwd_gather(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const Cv* __restrict__ work,
                             Cv* __restrict__ fv) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    const int* rows = A.rows + d.rows_off;
    for (int r = 0; r < A.nrhs; ++r) {
        Cv* g = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x) g[a] = work[rows[a] + (long long)r * A.ldw];
    }
}

// g[k] -= sum_{i in [r0, r1)} L[i,k] g[i] for columns k in [k0, k0+kn), one warp per column.
template <class T, class Cv>
__global__ void k_bwd_cols(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const T* __restrict__ panel,
                           Cv* __restrict__ fv) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp >= tk.kn) return;
    const SnDev d = A.sn[tk.s];
    const int k = tk.k0 + warp;
    const T* col = panel + d.panel_off + (long long)k * d.ldp;
    for (int r = 0; r < A.nrhs; ++r) {
        Cv* g = fv + A.fvec_off[tk.s] + r * A.fv_stride;
        Cv acc = Cv(0);
        for (int i = tk.r0 + lane; i < tk.r1; i += 32) acc += (Cv)col[i] * g[i];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) g[k] -= acc;
    }
}

template <class Cv>
__global__ void k_bwd_finish(const SolveBlockTask* __restrict__ tasks, SolveArgs A, const Cv* __restrict__ fv,
                             Cv* __restrict__ work) {
    const SolveBlockTask tk = tasks[blockIdx.x];
    const int s = tk.s;
    const SnDev d = A.sn[s];
    for (int r = 0; r < A.nrhs; ++r) {
        const Cv* g = fv + A.fvec_off[s] + r * A.fv_stride;
        for (int a = tk.r0 + threadIdx.x; a < tk.r1; a += blockDim.x) work[d.first_col + a + (long long)r * A.ldw] = g[a];
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
