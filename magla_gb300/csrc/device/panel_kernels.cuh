// Mixed-precision factorisation of one outer block [k0, k0+nb) (nb <= 128) of
// every large front of a level, once the block has received the updates of
// all earlier columns of its supernode:
//
//   k_diag_block   one CTA per front: A11 = L11 D L11^T in FP32 shared memory
//                  (32-column sub-blocks: a register-resident warp LDL^T
//                  that also yields the sub-block's inverse, the rows below
//                  by a small product with that inverse, a rank-32 trailing
//                  update), then X = L11^{-1}.  Writes L11
//                  and D to the factor, X^T, D and D^{-1} to a workspace slot.
//   k_panel_solve  128 rows per CTA: W21 = A21 X^T as an FP32 register-tiled
//                  GEMM, L21 = W21 D^{-1}; L21 goes to the factor and, K-major,
//                  W21 and L21 go to the staging operands of the tensor-core
//                  updates.
//
// Together they replace the reference's per-column panel loop for these
// blocks (CAESolvers/UCHOL/UtduNumericFactorization.cs:520-610): the same
// L, D and pivot rule, computed in two launches per 128 columns instead of a
// chain of small steps.  The fronts of the mixed path are stored in FP32 and L,
// X and the products are FP32; the pivots are FP64: each diagonal entry of the
// block is carried in FP64 through every elimination step inside the block
// (d_r -= d_k L_rk^2 with the FP32 L), and the pivot test !(d > tol * scale),
// the regularisation and D itself are FP64 (the FP32 elimination divides by D
// rounded to FP32).  That is O(nb^2) FP64 work per block.  The FP64 residual
// refinement recovers full accuracy of the solution.
#pragma once

#include <cfloat>
#include <climits>
#include <cuda_bf16.h>

#include "common.cuh"

namespace uchol_dev {

constexpr int kDiagMax = 128;
constexpr int kDiagLd = kDiagMax + 1;
// workspace slot: X^T as kDiagMax x kDiagMax (row k, column j: X[j][k], zero for k > j
// and beyond nb), then D and D^{-1} (kDiagMax floats each)
constexpr int kMinvStride = kDiagMax * kDiagMax + 2 * kDiagMax;
constexpr int kSolveRows = 128;
// float part: S and X (kDiagMax x kDiagLd each), Wt (kDiagMax x 33), D and D^{-1} in FP32;
// then the FP64 part: the running diagonal and D (kDiagMax doubles each)
constexpr size_t kDiagSmemFloats = 2 * kDiagMax * kDiagLd + kDiagMax * 33 + 2 * kDiagMax;
constexpr size_t kDiagSmemBytes = sizeof(float) * kDiagSmemFloats + sizeof(double) * 2 * kDiagMax;
static_assert(sizeof(float) * kDiagSmemFloats % sizeof(double) == 0, "the FP64 part is aligned");

// Pivot acceptance of the reference, !(d > tol*scale) -> regularise or reject,
// on FP64 pivots (UtduNumericFactorization.cs:553-592).  Only the decision is
// taken per pivot; the smallest and largest |d| of the block are taken from D
// once it is complete (FP64 instructions are scarce on this GPU).
struct PivotAccD {
    int regularized = 0, negative = 0, failed = INT_MAX;
    __device__ __forceinline__ double accept(double piv, int column, double thr, double reg, int allow) {
        if (!(piv > thr)) {
            if (!allow) failed = min(failed, column);
            if (piv < 0.0) ++negative;
            ++regularized;
            piv = reg;
        }
        return piv;
    }
    __device__ __forceinline__ void flush(PivotStats* st) const {
        if (regularized) atomicAdd(&st->regularized, regularized);
        if (negative) atomicAdd(&st->negative, negative);
        if (failed != INT_MAX) atomicMin(&st->failed, failed);
    }
};

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// LDL^T of the bn x bn (bn <= 32) diagonal sub-block at S[b0][b0] by one
// warp, with the same eliminations applied to the identity so that
// X_bb = L_bb^{-1} comes out with it.  Lane r holds row b0 + r in registers
// as a shift register: at pivot k, a[j] is F[r][k + j] and x[c] is X[r][c];
// its diagonal entry is carried separately in FP64 (dd, from dg), and the pivot
// d_k is lane k's dd.
// Every lane below the pivot applies F[r][k+j] -= L[r][k] (d_k L[k+j][k])
// (the reference's association) and shifts its row by one, so the loop over
// pivots stays rolled (short code) while every register index is a constant.
// The pivot column (times d_k) and row k of X reach every lane through the
// 64-float shared scratch `scr` (16-byte aligned) as eight 16-byte broadcast
// loads each: lane r stores d_k L[r][k] at slot (r - k) mod 32, so slot j is
// row k + j (rows above the pivot store zero).  Entries right of the
// diagonal take meaningless updates and are never read.
__device__ __forceinline__ void warp_ldlt32(float* S, float* X, int b0, int bn, int lane, int col0, double thr,
                                            double reg, int allow, float* sd, float* sdi, double* dg, double* sd64,
                                            PivotAccD& acc, float* scr) {
    float a[32], x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        a[j] = (lane < bn && j <= lane) ? S[(b0 + lane) * kDiagLd + b0 + j] : 0.f;
        x[j] = j == lane ? 1.f : 0.f;
    }
    double dd = lane < bn ? dg[b0 + lane] : 0.0;   // this row's diagonal entry, FP64
    for (int k = 0; k < bn; ++k) {
        const double raw = __shfl_sync(0xffffffffu, dd, k);   // F[k][k]
        const double piv64 = acc.accept(raw, col0 + k, thr, reg, allow);   // the same in every lane
        const float piv = (float)piv64;
        const float inv = rcp_approx(piv);
        const bool below = lane > k && lane < bn;
        const float l = below ? a[0] * inv : 0.f;
        if (below) {
            S[(b0 + lane) * kDiagLd + b0 + k] = l;
            const double ld = (double)l;
            dd = fma(-piv64, ld * ld, dd);   // l^2 is exact in FP64
        }
        if (lane == k) {
            S[(b0 + k) * kDiagLd + b0 + k] = 1.f;
            sd[b0 + k] = piv;
            sdi[b0 + k] = inv;
            sd64[b0 + k] = piv64;
        }
        scr[(lane - k) & 31] = piv * l;
        if (lane == k) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                reinterpret_cast<float4*>(scr + 32)[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
        }
        __syncwarp();
        float pl[32], xk[32];   // d_k L[k+j][k] (zero past the block), X[k][c]
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 u = reinterpret_cast<const float4*>(scr)[q];
            const float4 v = reinterpret_cast<const float4*>(scr + 32)[q];
            pl[4 * q] = u.x;
            pl[4 * q + 1] = u.y;
            pl[4 * q + 2] = u.z;
            pl[4 * q + 3] = u.w;
            xk[4 * q] = v.x;
            xk[4 * q + 1] = v.y;
            xk[4 * q + 2] = v.z;
            xk[4 * q + 3] = v.w;
        }
        __syncwarp();   // the scratch is rewritten at the next pivot
#pragma unroll
        for (int j = 1; j < 32; ++j) a[j - 1] = fmaf(-l, pl[j], a[j]);
        a[31] = 0.f;
#pragma unroll
        for (int c = 0; c < 32; ++c) x[c] = fmaf(-l, xk[c], x[c]);
    }
    if (lane < bn) {
#pragma unroll
        for (int c = 0; c < 32; ++c)
            if (c <= lane) X[(b0 + lane) * kDiagLd + b0 + c] = x[c];
    }
}

__global__ void __launch_bounds__(256, 1) k_diag_block(const PanelTask* __restrict__ tasks, const SnDev* __restrict__ sn,
                                                    float* __restrict__ panel, double* __restrict__ diag,
                                                    float* __restrict__ minv, const FactorCtl* __restrict__ ctlp,
                                                    PivotStats* st) {
    extern __shared__ float smem[];
    float* S = smem;                         // block, row-major (S[r * kDiagLd + c]); L11 after the factorisation
    float* X = S + kDiagMax * kDiagLd;       // L11^{-1}, row-major
    float* Wt = X + kDiagMax * kDiagLd;      // W = L D of the current sub-block's rows below it
    float* sd = Wt + kDiagMax * 33;          // D
    float* sdi = sd + kDiagMax;              // D^{-1}
    double* dg = reinterpret_cast<double*>(smem + kDiagSmemFloats);   // running diagonal, FP64
    double* sd64 = dg + kDiagMax;            // D, FP64
    const PanelTask tk = tasks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const FactorCtl ctl = *ctlp;
    const double thr = ctl.threshold, reg = ctl.regularization;
    const int nb = tk.nb, k0 = tk.j0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* P = panel + d.panel_off + k0 + (long long)k0 * d.ldp;   // A11 origin, column-major, ld = ldp

    for (int i = tid; i < kDiagMax * kDiagLd; i += 256) X[i] = 0.f;
    // lower triangle of A11: 16 independent loads in flight per thread
    for (int q0 = 0; q0 < kDiagMax * kDiagMax / 256; q0 += 16) {
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int idx = tid + 256 * (q0 + q), r = idx & (kDiagMax - 1), c = idx >> 7;
            v[q] = (r < nb && c <= r) ? P[r + (long long)c * d.ldp] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int idx = tid + 256 * (q0 + q), r = idx & (kDiagMax - 1), c = idx >> 7;
            S[r * kDiagLd + c] = v[q];
        }
    }
    if (tid < kDiagMax) dg[tid] = tid < nb ? (double)P[tid + (long long)tid * d.ldp] : 0.0;
    __syncthreads();

    PivotAccD acc;
    for (int b0 = 0; b0 < nb; b0 += 32) {
        const int bn = min(32, nb - b0);
        // (1) LDL^T of the sub-block and X_bb = L_bb^{-1}, by one warp
        if (warp == 0)   // Wt is free until step (3): its first 64 floats are the warp's scratch
            warp_ldlt32(S, X, b0, bn, lane, d.first_col + k0 + b0, thr, reg, ctl.allow_regularization, sd, sdi, dg,
                        sd64, acc, Wt);
        __syncthreads();
        // (3) rows below the sub-block: w[r][j] = sum_{k<=j} A[r][b0+k] X_bb[j][k], l = w / d_j;
        //     lane j, rows r0 + 8 q (four independent sums per lane)
        const int rb0 = b0 + bn;
        for (int r0 = rb0 + warp; r0 < nb; r0 += 32) {
            float w[4] = {0.f, 0.f, 0.f, 0.f};
            if (lane < bn) {
#pragma unroll 4
                for (int k = 0; k < bn; ++k) {
                    const float x = X[(b0 + lane) * kDiagLd + b0 + k];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int r = min(r0 + 8 * q, nb - 1);
                        w[q] = fmaf(S[r * kDiagLd + b0 + k], x, w[q]);
                    }
                }
            }
            __syncwarp();
            if (lane < bn) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int r = r0 + 8 * q;
                    if (r < nb) {
                        Wt[r * 33 + lane] = w[q];
                        S[r * kDiagLd + b0 + lane] = w[q] * sdi[b0 + lane];
                    }
                }
            }
        }
        __syncthreads();
        // (3b) the diagonal entries of the rows below, in FP64: d_r -= sum_k d_k L_rk^2, two threads per
        //      row (16 of the sub-block's columns each, four independent sums); reads only the
        //      sub-block's columns of S, which step (4) does not write
        {
            const int r = rb0 + (tid >> 1), kh = (tid & 1) * 16;
            double v[4] = {0.0, 0.0, 0.0, 0.0};
            if (r < nb) {
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    if (kh + k < bn) {
                        const double l = (double)S[r * kDiagLd + b0 + kh + k];
                        v[k & 3] = fma(sd64[b0 + kh + k], l * l, v[k & 3]);
                    }
                }
            }
            double sum = (v[0] + v[1]) + (v[2] + v[3]);
            sum += __shfl_xor_sync(0xffffffffu, sum, 1);
            if (r < nb && kh == 0) dg[r] -= sum;
        }
        // (4) trailing update of the block: S[r][c] -= sum_k W[r][k] L[c][k], rb0 <= c <= r < nb
        if (rb0 < nb) {
            const int tx = tid & 15, ty = tid >> 4;
            float accu[6][6];
#pragma unroll
            for (int p = 0; p < 6; ++p)
#pragma unroll
                for (int q = 0; q < 6; ++q) accu[p][q] = 0.f;
#pragma unroll 2
            for (int k = 0; k < bn; ++k) {
                float wv[6], lv[6];
#pragma unroll
                for (int p = 0; p < 6; ++p) {
                    const int r = rb0 + ty + 16 * p;
                    wv[p] = r < nb ? Wt[r * 33 + k] : 0.f;
                }
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const int c = rb0 + tx + 16 * q;
                    lv[q] = c < nb ? S[c * kDiagLd + b0 + k] : 0.f;
                }
#pragma unroll
                for (int p = 0; p < 6; ++p)
#pragma unroll
                    for (int q = 0; q < 6; ++q) accu[p][q] = fmaf(wv[p], lv[q], accu[p][q]);
            }
#pragma unroll
            for (int p = 0; p < 6; ++p)
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const int r = rb0 + ty + 16 * p, c = rb0 + tx + 16 * q;
                    if (r < nb && c <= r) S[r * kDiagLd + c] -= accu[p][q];
                }
        }
        __syncthreads();
    }

    // (5) off-diagonal blocks of X = L11^{-1}: X_ij = -X_ii sum_{j<=k<i} L_ik X_kj, by block diagonals;
    //     64 threads per block pair, each a 4 x 4 tile (rows rr + 8q, columns cc + 8p)
    const int nblk = (nb + 31) >> 5;
    float* T = Wt;   // (nblk - dd) blocks of 32 x 33
    for (int dd = 1; dd < nblk; ++dd) {
        const int pairs = nblk - dd;
        const int pr = tid >> 6, cc = tid & 7, rr = (tid >> 3) & 7, i = pr + dd;
        const bool active = pr < pairs;
        float t[4][4];
        if (active) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int p = 0; p < 4; ++p) t[q][p] = 0.f;
#pragma unroll 2
            for (int k = pr * 32; k < i * 32; ++k) {
                float xv[4], sv[4];
#pragma unroll
                for (int p = 0; p < 4; ++p) xv[p] = X[k * kDiagLd + pr * 32 + cc + 8 * p];
#pragma unroll
                for (int q = 0; q < 4; ++q) sv[q] = S[(i * 32 + rr + 8 * q) * kDiagLd + k];
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) t[q][p] = fmaf(sv[q], xv[p], t[q][p]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int p = 0; p < 4; ++p) T[pr * 32 * 33 + (rr + 8 * q) * 33 + cc + 8 * p] = t[q][p];
        }
        __syncthreads();
        if (active) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int p = 0; p < 4; ++p) t[q][p] = 0.f;
            // X_ii is lower triangular (zero above its diagonal), so the sums run over all 32 columns
#pragma unroll 2
            for (int tt = 0; tt < 32; ++tt) {
                float yv[4], xv[4];
#pragma unroll
                for (int p = 0; p < 4; ++p) yv[p] = T[pr * 32 * 33 + tt * 33 + cc + 8 * p];
#pragma unroll
                for (int q = 0; q < 4; ++q) xv[q] = X[(i * 32 + rr + 8 * q) * kDiagLd + i * 32 + tt];
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int p = 0; p < 4; ++p) t[q][p] = fmaf(xv[q], yv[p], t[q][p]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int row = i * 32 + rr + 8 * q;
                if (row < nb) {
#pragma unroll
                    for (int p = 0; p < 4; ++p) X[row * kDiagLd + pr * 32 + cc + 8 * p] = -t[q][p];
                }
            }
        }
        __syncthreads();
    }

    // (6) write L11 (unit diagonal), D, and the workspace slot
    for (int c = warp; c < nb; c += 8)
        for (int r = c + lane; r < nb; r += 32) P[r + (long long)c * d.ldp] = r == c ? 1.f : S[r * kDiagLd + c];
    if (tid < nb) diag[d.first_col + k0 + tid] = sd64[tid];
    float* M = minv + (size_t)tk.slot * kMinvStride;
    for (int idx = tid; idx < kDiagMax * kDiagMax; idx += 256) {
        const int k = idx >> 7, j = idx & (kDiagMax - 1);
        M[idx] = (j < nb && k <= j) ? X[j * kDiagLd + k] : 0.f;
    }
    if (tid < kDiagMax) {
        M[kDiagMax * kDiagMax + tid] = tid < nb ? sd[tid] : 0.f;
        M[kDiagMax * kDiagMax + kDiagMax + tid] = tid < nb ? sdi[tid] : 0.f;
    }
    if (tid == 0) acc.flush(st);
    // smallest and largest |d| of the block, by the first warp
    if (warp == 0) {
        double lo = DBL_MAX, hi = 0.0;
        for (int k = lane; k < nb; k += 32) {
            const double a = fabs(sd64[k]);
            lo = fmin(lo, a);
            hi = fmax(hi, a);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0 && nb > 0) {
            atomicMin(&st->min_bits, (unsigned long long)__double_as_longlong(lo));
            atomicMax(&st->max_bits, (unsigned long long)__double_as_longlong(hi));
        }
    }
}

// 4-byte asynchronous copy global -> shared (zero fill when !valid: nothing is read then).
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Shared memory of k_panel_solve: two stages of (A21 chunk, X^T chunk), 32 K columns each.
constexpr int kPanelKc = 32, kPanelLds = kSolveRows + 4;
constexpr size_t kPanelSmemBytes = sizeof(float) * 2 * 2 * kPanelKc * kPanelLds;

__device__ __forceinline__ void store_op4(__nv_bfloat16* p, float a, float b, float c, float e) {
    __nv_bfloat162 lo = __floats2bfloat162_rn(a, b), hi = __floats2bfloat162_rn(c, e);
    uint2 v;
    v.x = *reinterpret_cast<unsigned*>(&lo);
    v.y = *reinterpret_cast<unsigned*>(&hi);
    *reinterpret_cast<uint2*>(p) = v;
}
// TF32 operands: rounded to TF32 precision (nearest, ties away) as they are staged, so that
// the tensor core, which reads only the top 19 bits of each FP32 operand, multiplies rounded
// rather than truncated values (truncation biases every product the same way, and over the
// many updates of a deep tree that bias accumulates in the factor).
__device__ __forceinline__ float round_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ void store_op4(float* p, float a, float b, float c, float e) {
    *reinterpret_cast<float4*>(p) = make_float4(round_tf32(a), round_tf32(b), round_tf32(c), round_tf32(e));
}
__device__ __forceinline__ void store_op1(__nv_bfloat16* p, float a) { *p = __float2bfloat16_rn(a); }
__device__ __forceinline__ void store_op1(float* p, float a) { *p = a; }

// W21 = A21 X^T and L21 = W21 D^{-1} for rows [row0, row0 + rows) of the
// front, 256 threads: thread (ty, tx) owns rows {4ty..4ty+3, 64+4ty..} and
// columns {4tx..4tx+3, 64+4tx..} of the 128 x 128 tile (conflict-free 128-bit
// shared loads).  X^T is upper triangular, so columns below 64 take no
// updates from K >= 64.
template <class Op>
__global__ void __launch_bounds__(256, 2) k_panel_solve(const PanelTask* __restrict__ tasks,
                                                     const SnDev* __restrict__ sn, float* __restrict__ panel,
                                                     const float* __restrict__ minv, Op* __restrict__ stage_a,
                                                     Op* __restrict__ stage_b,
                                                     const StageInfo* __restrict__ stage_info) {
    constexpr int KC = kPanelKc, LDS = kPanelLds;
    extern __shared__ __align__(16) float psm[];   // stage s: As = psm + 2 s KC LDS, Ms = As + KC LDS
    const PanelTask tk = tasks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const int nb = tk.nb, k0 = tk.j0, row0 = tk.row0, rows = tk.rows;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const float* M = minv + (size_t)tk.slot * kMinvStride;
    float* A = panel + d.panel_off + row0 + (long long)k0 * d.ldp;   // A21 rows of this task, column-major
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    // K chunks of KC columns copied asynchronously into two stages: every copy of a chunk in
    // flight at once, and the next chunk's copies under the current chunk's products
    auto issue_chunk = [&](int kc, int st) {
        float* As = psm + 2 * st * KC * LDS;
        float* Ms = As + KC * LDS;
#pragma unroll
        for (int q = 0; q < (KC * kSolveRows) / 256; ++q) {
            const int idx = tid + 256 * q, r = idx & (kSolveRows - 1), k = idx >> 7;
            const bool ok = r < rows && kc + k < nb;
            cp_async4(&As[k * LDS + r], ok ? A + r + (long long)(kc + k) * d.ldp : A, ok);
            cp_async4(&Ms[k * LDS + r], M + (kc + k) * kDiagMax + r, true);
        }
        cp_async_commit();
    };
    issue_chunk(0, 0);
    for (int kc = 0, st = 0; kc < nb; kc += KC, st ^= 1) {
        if (kc + KC < nb) {
            issue_chunk(kc + KC, st ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float* As = psm + 2 * st * KC * LDS;
        const float* Ms = As + KC * LDS;
        const bool low_cols = kc < 64;   // X^T[k][j] = 0 for j < k: columns 0..63 see K < 64 only
#pragma unroll 4
        for (int k = 0; k < KC; ++k) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[k * LDS + 4 * ty]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[k * LDS + 64 + 4 * ty]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Ms[k * LDS + 64 + 4 * tx]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bh[4] = {b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][4 + j] = fmaf(av[i], bh[j], acc[i][4 + j]);
            if (low_cols) {
                const float4 b0 = *reinterpret_cast<const float4*>(&Ms[k * LDS + 4 * tx]);
                const float bl[4] = {b0.x, b0.y, b0.z, b0.w};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bl[j], acc[i][j]);
            }
        }
        __syncthreads();   // this stage is refilled two chunks later
    }
    // epilogue: L21 = W21 D^{-1} to the factor (column-major), W21 and L21 to the staging rows (K-major)
    const float* dinv = M + kDiagMax * kDiagMax + kDiagMax;
    const bool vec_rows = ((d.panel_off + row0) & 3) == 0;
#pragma unroll
    for (int jg = 0; jg < 2; ++jg) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int col = 64 * jg + 4 * tx + j;
            if (col >= nb) continue;
            const float di = dinv[col];
#pragma unroll
            for (int ig = 0; ig < 2; ++ig) {
                const int r = 64 * ig + 4 * ty;
                float* dst = A + r + (long long)col * d.ldp;
                const float l0 = acc[4 * ig + 0][4 * jg + j] * di, l1 = acc[4 * ig + 1][4 * jg + j] * di;
                const float l2 = acc[4 * ig + 2][4 * jg + j] * di, l3 = acc[4 * ig + 3][4 * jg + j] * di;
                if (vec_rows && r + 4 <= rows) {
                    *reinterpret_cast<float4*>(dst) = make_float4(l0, l1, l2, l3);
                } else {
                    if (r + 0 < rows) dst[0] = l0;
                    if (r + 1 < rows) dst[1] = l1;
                    if (r + 2 < rows) dst[2] = l2;
                    if (r + 3 < rows) dst[3] = l3;
                }
            }
        }
    }
    if (!tk.stage) return;
    const StageInfo g = stage_info[tk.s];
#pragma unroll
    for (int ig = 0; ig < 2; ++ig) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = 64 * ig + 4 * ty + i;
            if (r >= rows) continue;
            const long long so = g.off + (long long)(row0 + r) * g.ld + k0;
#pragma unroll
            for (int jg = 0; jg < 2; ++jg) {
                const int col = 64 * jg + 4 * tx;
                const float* w = &acc[4 * ig + i][4 * jg];
                if (col + 4 <= nb) {
                    store_op4(stage_a + so + col, w[0], w[1], w[2], w[3]);
                    store_op4(stage_b + so + col, w[0] * dinv[col], w[1] * dinv[col + 1], w[2] * dinv[col + 2],
                              w[3] * dinv[col + 3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (col + j < nb) {
                            store_op1(stage_a + so + col + j, w[j]);
                            store_op1(stage_b + so + col + j, w[j] * dinv[col + j]);
                        }
                }
            }
        }
    }
    if (tk.stage_zero_to > k0 + nb) {
        const int zc = tk.stage_zero_to - (k0 + nb);
        for (int idx = tid; idx < rows * zc; idx += 256) {
            const int r = idx / zc, c = idx - r * zc;
            const long long o = g.off + (long long)(row0 + r) * g.ld + k0 + nb + c;
            store_op1(stage_a + o, 0.f);
            store_op1(stage_b + o, 0.f);
        }
    }
}

}  // namespace uchol_dev
