// Factorisation kernels: assembly, extend-add and small fronts for both
// paths (front storage type T is double on the FP64 path, float on the mixed
// path; their pivots are FP64), and the FP64 path's pivot block, TRSM and
// right-looking updates.  The mixed path's panel kernels are in
// panel_kernels.cuh.
#pragma once

#include <cfloat>
#include <climits>
#include <cuda_bf16.h>

#include "common.cuh"

namespace uchol_dev {

__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(fabs(x));
}

// max |A_ii| over the stored diagonal (ComputeDiagonalScale,
// CAESolvers/UCHOL/UtduNumericFactorization.cs:411-418).
__global__ void k_diag_scale(const double* __restrict__ values, const int* __restrict__ diag_index, int n,
                             PivotStats* st) {
    unsigned long long best = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        int di = diag_index[j];
        if (di >= 0) {
            unsigned long long b = abs_bits(values[di]);
            if (b > best) best = b;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, best, o);
        if (v > best) best = v;
    }
    if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(&st->min_bits, best);  // temporarily holds the scale bits
}

// Resets the statistics and turns the scale bits into the pivot controls.
__global__ void k_finish_scale(PivotStats* st, FactorCtl* ctl, double pivot_tolerance, double diagonal_regularization,
                               int allow) {
    double scale = __longlong_as_double((long long)st->min_bits);
    if (!(scale > 0.0)) scale = 1.0;
    st->scale = scale;
    st->regularized = 0;
    st->negative = 0;
    st->failed = INT_MAX;
    st->min_bits = 0x7fefffffffffffffull;  // DBL_MAX
    st->max_bits = 0;
    ctl->threshold = pivot_tolerance * scale;
    ctl->regularization = diagonal_regularization * scale;
    ctl->allow_regularization = allow;
}

// Pivot acceptance exactly as the reference: !(d > tol*scale) (which also
// catches NaN) is regularised or rejected (UtduNumericFactorization.cs:557-575).
struct PivotAcc {
    int regularized = 0, negative = 0, failed = INT_MAX;
    unsigned long long min_bits = 0x7fefffffffffffffull, max_bits = 0;
    __device__ __forceinline__ double accept(double piv, int column, const FactorCtl& ctl) {
        if (!(piv > ctl.threshold)) {
            if (!ctl.allow_regularization) failed = min(failed, column);
            if (piv < 0.0) ++negative;
            ++regularized;
            piv = ctl.regularization;
        }
        unsigned long long b = abs_bits(piv);
        if (b < min_bits) min_bits = b;
        if (b > max_bits) max_bits = b;
        return piv;
    }
    __device__ __forceinline__ void flush(PivotStats* st) const {
        if (regularized) atomicAdd(&st->regularized, regularized);
        if (negative) atomicAdd(&st->negative, negative);
        if (failed != INT_MAX) atomicMin(&st->failed, failed);
        atomicMin(&st->min_bits, min_bits);
        atomicMax(&st->max_bits, max_bits);
    }
};

template <class T>
__global__ void k_assemble(const double* __restrict__ values, const long long* __restrict__ pos, int nnz,
                           T* __restrict__ panel) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x)
        panel[pos[k]] = (T)values[k];
}

// Extend-add: one warp per receiving parent column; the children's columns
// that land in it are added in child order (deterministic, no atomics).
// UtduNumericFactorization.cs:471-509.  A column of the parent's contribution
// block is first cleared from its diagonal down (the reference zeroes the
// whole front, :441-447; only the lower triangle is ever read), so the
// clearing costs no pass of its own and the adds find the lines in L2.
// Side = true: the instance launched on the side stream (its graph nodes run at
// the lowest priority, so that the main stream's CTAs are scheduled first).
template <class T, bool Side = false>
__global__ void k_extend_add(const EaItem* __restrict__ items, int count, const EaEntry* __restrict__ entries,
                             const SnDev* __restrict__ sn, const int* __restrict__ rel, T* __restrict__ panel,
                             T* __restrict__ contrib) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp < count; warp += warps) {
        const EaItem it = items[warp];
        const SnDev P = sn[it.parent];
        T* dst;
        int shift;
        if (it.pcol < P.w) {
            dst = panel + P.panel_off + (long long)it.pcol * P.ldp;
            shift = 0;
        } else {
            const int c = it.pcol - P.w, t = P.m - P.w;
            dst = contrib + P.contrib_off + (long long)c * P.ldc;
            shift = P.w;
            // rows [c, t): 16-byte stores between a scalar head and tail (the column starts on a
            // 16-byte boundary: contribution offsets are multiples of 64 elements, ldc of 8)
            constexpr int V = 16 / (int)sizeof(T);
            const int head = min(t, (c + V - 1) / V * V), body = max(head, t / V * V);
            for (int r = c + lane; r < head; r += 32) dst[r] = T(0);
            for (int v = head / V + lane; v < body / V; v += 32) reinterpret_cast<uint4*>(dst)[v] = make_uint4(0u, 0u, 0u, 0u);
            for (int r = body + lane; r < t; r += 32) dst[r] = T(0);
            __syncwarp();
        }
        for (int e = it.begin; e < it.end; ++e) {
            const EaEntry en = entries[e];
            const SnDev C = sn[en.child];
            const int t = C.m - C.w;
            const int* r = rel + C.rel_off;
            const T* src = contrib + C.contrib_off + (long long)en.a * C.ldc;
            // rows of one child column are distinct, so loads of a batch are issued before its stores
            constexpr int D = 8;   // loads of a batch in flight per lane
            for (int b0 = en.a + lane; b0 < t; b0 += 32 * D) {
                int idx[D];
                T sv[D], dv[D];
#pragma unroll
                for (int u = 0; u < D; ++u) {
                    const int b = b0 + 32 * u;
                    idx[u] = b < t ? r[b] - shift : -1;
                    sv[u] = b < t ? src[b] : T(0);
                }
#pragma unroll
                for (int u = 0; u < D; ++u) dv[u] = idx[u] >= 0 ? dst[idx[u]] : T(0);
#pragma unroll
                for (int u = 0; u < D; ++u)
                    if (idx[u] >= 0) dst[idx[u]] = dv[u] + sv[u];
            }
            __syncwarp();
        }
    }
}

// Whole small front in shared memory (FP64), unblocked right-looking LDL^T
// of its w pivots; writes the unit factor block and the contribution.
template <class T>
__global__ void __launch_bounds__(256) k_small_fronts(const int* __restrict__ fronts, const SnDev* __restrict__ sn,
                                                      T* __restrict__ panel, T* __restrict__ contrib,
                                                      double* __restrict__ diag, const FactorCtl* __restrict__ ctlp,
                                                      PivotStats* st) {
    extern __shared__ double S[];
    const SnDev d = sn[fronts[blockIdx.x]];
    const FactorCtl ctl = *ctlp;
    const int m = d.m, w = d.w, ld = m;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int idx = tid; idx < m * m; idx += nt) {
        int i = idx % m, j = idx / m;
        if (i < j) continue;
        S[i + j * ld] = j < w ? (double)panel[d.panel_off + i + (long long)j * d.ldp]
                              : (double)contrib[d.contrib_off + (i - w) + (long long)(j - w) * d.ldc];
    }
    PivotAcc acc;
    __syncthreads();
    for (int k = 0; k < w; ++k) {
        double piv = acc.accept(S[k + k * ld], d.first_col + k, ctl);  // identical in every thread
        const double inv = 1.0 / piv;
        __syncthreads();
        for (int i = k + 1 + tid; i < m; i += nt) S[i + k * ld] *= inv;
        if (tid == 0) {
            diag[d.first_col + k] = piv;
            S[k + k * ld] = 1.0;
        }
        __syncthreads();
        const int r = m - k - 1;
        for (int idx = tid; idx < r * r; idx += nt) {
            int ii = idx % r, jj = idx / r;
            if (ii < jj) continue;
            int i = k + 1 + ii, j = k + 1 + jj;
            S[i + j * ld] -= S[i + k * ld] * (piv * S[j + k * ld]);
        }
        __syncthreads();
    }
    for (int idx = tid; idx < m * m; idx += nt) {
        int i = idx % m, j = idx / m;
        if (i < j) continue;
        if (j < w) panel[d.panel_off + i + (long long)j * d.ldp] = (T)S[i + j * ld];
        else contrib[d.contrib_off + (i - w) + (long long)(j - w) * d.ldc] = (T)S[i + j * ld];
    }
    if (tid == 0) acc.flush(st);
}

// Pivot block [j0, j0+nb) of a large front: FP64 LDL^T of the nb x nb
// diagonal block in shared memory, one CTA per block; writes the unit L11,
// the pivots D and the statistics (UtduNumericFactorization.cs:553-592
// restricted to the diagonal block).
constexpr int kMaxPivotBlock = 64;

template <class T>
__global__ void __launch_bounds__(128) k_pivot_block(const PanelTask* __restrict__ tasks, const SnDev* __restrict__ sn,
                                                     T* __restrict__ panel, double* __restrict__ diag,
                                                     const FactorCtl* __restrict__ ctlp, PivotStats* st) {
    __shared__ double Dg[kMaxPivotBlock * (kMaxPivotBlock + 1)];
    const PanelTask tk = tasks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const FactorCtl ctl = *ctlp;
    const int nb = tk.nb, j0 = tk.j0, ld = kMaxPivotBlock + 1;
    const int tid = threadIdx.x, nt = blockDim.x;
    T* P = panel + d.panel_off;
    for (int idx = tid; idx < nb * nb; idx += nt) {
        int r = idx % nb, c = idx / nb;
        if (r >= c) Dg[r + c * ld] = (double)P[(j0 + r) + (long long)(j0 + c) * d.ldp];
    }
    PivotAcc acc;
    __syncthreads();
    for (int k = 0; k < nb; ++k) {
        const double piv = acc.accept(Dg[k + k * ld], d.first_col + j0 + k, ctl);
        const double inv = 1.0 / piv;
        __syncthreads();
        for (int r = k + 1 + tid; r < nb; r += nt) Dg[r + k * ld] *= inv;
        if (tid == 0) {
            diag[d.first_col + j0 + k] = piv;
            Dg[k + k * ld] = 1.0;
        }
        __syncthreads();
        const int q = nb - k - 1;
        for (int idx = tid; idx < q * q; idx += nt) {
            int rr = idx % q, cc = idx / q;
            if (rr < cc) continue;
            int r = k + 1 + rr, c = k + 1 + cc;
            Dg[r + c * ld] -= Dg[r + k * ld] * (piv * Dg[c + k * ld]);
        }
        __syncthreads();
    }
    for (int idx = tid; idx < nb * nb; idx += nt) {
        int r = idx % nb, c = idx / nb;
        if (r >= c) P[(j0 + r) + (long long)(j0 + c) * d.ldp] = (T)Dg[r + c * ld];
    }
    if (tid == 0) acc.flush(st);
}

// Rows [row0, row0+rows) under the pivot block (FP64 path): Y = F21 L11^-T
// (forward substitution per row), L21 = Y / D.
template <class T, class Cc, int NBMAX>
__global__ void __launch_bounds__(128) k_trsm(const PanelTask* __restrict__ tasks, const SnDev* __restrict__ sn,
                                              T* __restrict__ panel, const double* __restrict__ diag) {
    __shared__ Cc L11[NBMAX * (NBMAX + 1)];
    __shared__ double dinv[NBMAX];
    const PanelTask tk = tasks[blockIdx.x];
    const SnDev d = sn[tk.s];
    const int nb = tk.nb, j0 = tk.j0, ld = NBMAX + 1;
    const int tid = threadIdx.x, nt = blockDim.x;
    T* P = panel + d.panel_off;
    for (int idx = tid; idx < nb * nb; idx += nt) {
        int r = idx % nb, c = idx / nb;
        L11[r + c * ld] = r > c ? (Cc)P[(j0 + r) + (long long)(j0 + c) * d.ldp] : Cc(0);
    }
    if (tid < nb) dinv[tid] = 1.0 / diag[d.first_col + j0 + tid];
    __syncthreads();
    if (tid < tk.rows) {
        const int i = tk.row0 + tid;
        Cc y[NBMAX];
#pragma unroll
        for (int k = 0; k < NBMAX; ++k) {
            if (k < nb) {
                Cc v = (Cc)P[i + (long long)(j0 + k) * d.ldp];
#pragma unroll
                for (int j = 0; j < k; ++j) v -= y[j] * L11[k + j * ld];
                y[k] = v;
            }
        }
#pragma unroll
        for (int k = 0; k < NBMAX; ++k)
            if (k < nb) P[i + (long long)(j0 + k) * d.ldp] = (T)((double)y[k] * dinv[k]);
    }
}

// SIMT tile update C[i, j] -= sum_k L[i,k] d_k L[j,k] over a 64 x 64 tile,
// lower triangle only (i >= j).  Compute type C: double on the FP64 path,
// float for the inner updates of the mixed path.
template <class T, class C>
__global__ void __launch_bounds__(256) k_simt_update(const UpdJob* __restrict__ jobs, int njobs,
                                                     const SnDev* __restrict__ sn, T* __restrict__ panel,
                                                     T* __restrict__ contrib, const double* __restrict__ diag) {
    constexpr int TS = 64, KC = 32;
    __shared__ C As[KC][TS + 1];
    __shared__ C Bs[KC][TS + 1];
    const UpdJob J = jobs[find_job(jobs, njobs, blockIdx.x)];
    const SnDev d = sn[J.s];
    TileTask tk;
    tk.s = J.s;
    tk.k0 = J.k0;
    tk.kn = J.kn;
    decode_tile(J, d, TS, (long long)blockIdx.x - J.tile_begin, tk.i0, tk.j0, tk.jend);
    const T* Pn = panel + d.panel_off;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    C acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = C(0);
    for (int kc = 0; kc < tk.kn; kc += KC) {
        const int kl = min(KC, tk.kn - kc);
        __syncthreads();
        for (int idx = threadIdx.x; idx < KC * TS; idx += 256) {
            int r = idx % TS, k = idx / TS;
            int kk = tk.k0 + kc + k;
            C av = C(0), bv = C(0);
            if (k < kl) {
                int i = tk.i0 + r, j = tk.j0 + r;
                if (i < d.m) av = (C)Pn[i + (long long)kk * d.ldp];
                if (j < d.m) bv = (C)((double)Pn[j + (long long)kk * d.ldp] * diag[d.first_col + kk]);
            }
            As[k][r] = av;
            Bs[k][r] = bv;
        }
        __syncthreads();
        for (int k = 0; k < kl; ++k) {
            C a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = As[k][ty + 16 * q];
                b[q] = Bs[k][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] += a[p] * b[q];
        }
    }
    const bool in_panel = tk.j0 < d.w;
    T* base = in_panel ? panel : contrib;
    long long off[4][4];
    T old[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int j = tk.j0 + tx + 16 * q;
            const int i = tk.i0 + ty + 16 * p;
            const bool ok = j < tk.jend && i < d.m && i >= j;
            off[p][q] = !ok ? -1
                            : in_panel ? d.panel_off + i + (long long)j * d.ldp
                                       : d.contrib_off + (i - d.w) + (long long)(j - d.w) * d.ldc;
            old[p][q] = ok ? base[off[p][q]] : T(0);   // loads first, then stores: no serialised round trips
        }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p)
            if (off[p][q] >= 0) base[off[p][q]] = (T)((C)old[p][q] - acc[p][q]);
}

}  // namespace uchol_dev
