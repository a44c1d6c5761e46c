// Device-resident values of a SymmetricCSRMatrix (uchol_dmatrix): the
// values-refresh operations of the reference's container run as kernels on
// the handle's stream, the factorisation reads the refreshed values without a
// host round trip, and a Jacobi-preconditioned CG runs on the FP64 product.
//
//   ClearValues        CAESolvers/SymmetricCSRMatrix.cs:113-116   cudaMemsetAsync of the values
//   AccumulateAt       CAESolvers/SymmetricCSRMatrix.cs:98-110    k_accumulate over a planned item list
//   LineCross          CAESolvers/SymmetricCSRMatrix.cs:125-167   k_line_cross_rhs + k_line_cross_values
//   Multiply           CAESolvers/SymmetricCSRMatrix.cs:293-324   k_spmv_residual on the both-triangle structure
//   Jacobi-PCG         CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs:78-165,
//                      CAESolvers/CGGP/JacobiPreconditioner.cs:12-57
//
// Positions are resolved on the host once per item list (a plan): the device
// work is then a fixed set of launches with no search and no atomics, and every
// entry receives its additions in the list's order, so the refreshed values are
// bit-identical to the reference's sequential calls.
//
// Included by capi.cu (one translation unit with the helpers it uses).
#pragma once

struct uchol_dmatrix_s {
    int n = 0, nnz = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<int> row_ptr, col, diag;          // host pattern (plans, validation)
    std::vector<int> col_ptr, col_row, col_pos;   // column view of the upper half (LineCross plans)
    DBuf values, d_diag, full_ptr, full_col, full_src, full_val;
    long long full_nnz = 0;
    DBuf ws;                                      // PCG / host-variant workspace
    int ws_nrhs = 0;
    const void* checked_symbolic = nullptr;       // last symbolic whose pattern matched
    std::mutex mu;
};

struct uchol_values_plan_s {
    uchol_dmatrix_s* m = nullptr;   // compared, never dereferenced after creation
    int kind = 0;   // 0: AccumulateAt list, 1: LineCross list
    int count = 0;
    // AccumulateAt: targets (distinct positions, ascending) and their items in list order
    int targets = 0;
    DBuf tgt_pos, tgt_ptr, item_perm, items;
    // LineCross: per affected right-hand-side row its events in list order; value positions to
    // zero and diagonal positions to set to one
    int rows = 0, nzero = 0, nones = 0;
    DBuf ev_ptr, ev_row, ev_pos, ev_t, zero_pos, one_pos, rhs_ws, pres_ws;
};

namespace {

constexpr int kEvSet = -2;      // LineCross event: rhs[row] = prescribed
constexpr int kEvZeroed = -1;   // LineCross event: the entry was already zeroed by an earlier call
constexpr int kCgBlocks = 296;  // CTAs of the PCG reductions (two per SM)
constexpr int kCgPoll = 16;     // PCG steps between host checks of the active columns

// values[tgt_pos[t]] += items of target t, one after the other in list order.
__global__ void k_accumulate(const int* __restrict__ tgt_pos, const int* __restrict__ tgt_ptr,
                             const int* __restrict__ perm, int targets, const double* __restrict__ items,
                             double* __restrict__ values) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < targets; t += gridDim.x * blockDim.x) {
        const int pos = tgt_pos[t];
        double v = values[pos];
        for (int k = tgt_ptr[t]; k < tgt_ptr[t + 1]; ++k) v = __dadd_rn(v, items[perm[k]]);
        values[pos] = v;
    }
}

// Right-hand-side rows touched by a LineCross list, one thread per (row, column): the
// row's events in list order, with the multiplicands read before k_line_cross_values
// zeroes them (an entry zeroed by an earlier call of the list multiplies as +0.0).
__global__ void k_line_cross_rhs(const int* __restrict__ ev_ptr, const int* __restrict__ ev_row,
                                 const int* __restrict__ ev_pos, const int* __restrict__ ev_t, int rows,
                                 const double* __restrict__ values, double* __restrict__ rhs, int ldr,
                                 const double* __restrict__ pres, int ldp, int nrhs) {
    for (int r = blockIdx.y; r < nrhs; r += gridDim.y)
        for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < rows; a += gridDim.x * blockDim.x) {
            double* y = rhs + (long long)r * ldr + ev_row[a];
            const double* p = pres + (long long)r * ldp;
            double x = *y;
            for (int e = ev_ptr[a]; e < ev_ptr[a + 1]; ++e) {
                const int pos = ev_pos[e];
                const double pv = p[ev_t[e]];
                if (pos == kEvSet) {
                    x = pv;
                } else {
                    const double v = pos >= 0 ? values[pos] : 0.0;
                    x = __dsub_rn(x, __dmul_rn(v, pv));
                }
            }
            *y = x;
        }
}

__global__ void k_line_cross_values(const int* __restrict__ zero_pos, int nzero, const int* __restrict__ one_pos,
                                    int nones, double* __restrict__ values) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nzero + nones; i += gridDim.x * blockDim.x) {
        if (i < nzero) values[zero_pos[i]] = 0.0;
        else values[one_pos[i - nzero]] = 1.0;
    }
}

// ---- Jacobi-preconditioned CG, several right-hand sides (columns) at once -----
// Each column follows the reference's iteration on its own and stops when its
// residual norm reaches its threshold (or after max_it steps): later steps leave it
// untouched.  Reductions are two-stage and deterministic (per-CTA partial sums, then
// the last CTA to finish adds them in CTA order).

struct CgCol {
    double thr, scale, rz, rnorm2, alpha, beta;
    int active, iters, failed, pad;
};

__device__ __forceinline__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s;   // valid in thread 0
}

// Thread 0 of every CTA stores its partial sums; returns true in the CTA that finished last
// (its thread 0 then reads every partial), after which the column's counter is reset.
__device__ __forceinline__ bool last_cta(unsigned* counter) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

// z = M^-1 r, p = z, rz = r . z (the step before the first iteration).
__global__ void __launch_bounds__(256) k_cg_start(const double* __restrict__ inv, const double* __restrict__ r,
                                                  double* __restrict__ z, double* __restrict__ p, int n, int ld,
                                                  CgCol* cols, double* partial, unsigned* counters) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    if (!cols[c].active) return;
    const double* rc = r + (long long)c * ld;
    double* zc = z + (long long)c * ld;
    double* pc = p + (long long)c * ld;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double zi = __dmul_rn(inv[i], rc[i]);
        zc[i] = zi;
        pc[i] = zi;
        acc = __dadd_rn(acc, __dmul_rn(rc[i], zi));
    }
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) partial[(long long)c * gridDim.x + blockIdx.x] = s;
    if (last_cta(&counters[c]) && threadIdx.x == 0) {
        double t = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(&partial[(long long)c * gridDim.x + b]);
        cols[c].rz = t;
        counters[c] = 0;
    }
}

// q = A p for the active columns (one warp per row of the both-triangle structure).
__global__ void k_cg_spmv(const int* __restrict__ ptr, const int* __restrict__ col, const double* __restrict__ val,
                          int n, int nrhs, const double* __restrict__ p, int ld, double* __restrict__ q,
                          const CgCol* __restrict__ cols) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= n) return;
    const int p0 = ptr[row], p1 = ptr[row + 1];
    for (int c = 0; c < nrhs; ++c) {
        if (!cols[c].active) continue;
        const double* pc = p + (long long)c * ld;
        double acc = 0.0;
        for (int k = p0 + lane; k < p1; k += 32) acc += val[k] * pc[col[k]];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) q[row + (long long)c * ld] = acc;
    }
}

// pAp = p . q; alpha = rz / pAp (a column whose pAp <= 0 fails and stops).
__global__ void __launch_bounds__(256) k_cg_alpha(const double* __restrict__ p, const double* __restrict__ q, int n,
                                                  int ld, CgCol* cols, double* partial, unsigned* counters) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    if (!cols[c].active) return;
    const double* pc = p + (long long)c * ld;
    const double* qc = q + (long long)c * ld;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc = __dadd_rn(acc, __dmul_rn(pc[i], qc[i]));
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) partial[(long long)c * gridDim.x + blockIdx.x] = s;
    if (last_cta(&counters[c]) && threadIdx.x == 0) {
        double pap = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) pap += __ldcg(&partial[(long long)c * gridDim.x + b]);
        counters[c] = 0;
        if (pap <= 0.0) {
            cols[c].failed = 1;
            cols[c].active = 0;
        } else {
            cols[c].alpha = cols[c].rz / pap;
        }
    }
}

// x += alpha p, r -= alpha q, z = M^-1 r; |r|^2 and r . z; then the stopping test and beta.
__global__ void __launch_bounds__(256) k_cg_update(double* __restrict__ x, int ldx, double* __restrict__ r,
                                                   double* __restrict__ z, const double* __restrict__ p,
                                                   const double* __restrict__ q, const double* __restrict__ inv,
                                                   int n, int ld, int max_it, CgCol* cols, double* partial,
                                                   unsigned* counters) {
    __shared__ double red[8];
    const int c = blockIdx.y;
    if (!cols[c].active) return;
    const double alpha = cols[c].alpha;
    double* xc = x + (long long)c * ldx;
    double* rc = r + (long long)c * ld;
    double* zc = z + (long long)c * ld;
    const double* pc = p + (long long)c * ld;
    const double* qc = q + (long long)c * ld;
    double rr = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        xc[i] = __dadd_rn(xc[i], __dmul_rn(alpha, pc[i]));
        const double ri = __dsub_rn(rc[i], __dmul_rn(alpha, qc[i]));
        rc[i] = ri;
        const double zi = __dmul_rn(inv[i], ri);
        zc[i] = zi;
        rr = __dadd_rn(rr, __dmul_rn(ri, ri));
        rz = __dadd_rn(rz, __dmul_rn(ri, zi));
    }
    const double s1 = block_sum(rr, red);
    const double s2 = block_sum(rz, red);
    const long long base = (long long)c * gridDim.x * 2;
    if (threadIdx.x == 0) {
        partial[base + 2 * blockIdx.x] = s1;
        partial[base + 2 * blockIdx.x + 1] = s2;
    }
    if (last_cta(&counters[c]) && threadIdx.x == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
            t1 += __ldcg(&partial[base + 2 * b]);
            t2 += __ldcg(&partial[base + 2 * b + 1]);
        }
        counters[c] = 0;
        CgCol& C = cols[c];
        C.rnorm2 = t1;
        C.iters += 1;
        if (sqrt(t1) <= C.thr || C.iters >= max_it) {
            C.active = 0;
        } else {
            C.beta = t2 / C.rz;
            C.rz = t2;
        }
    }
}

// p = z + beta p
__global__ void k_cg_direction(const double* __restrict__ z, double* __restrict__ p, int n, int ld,
                               const CgCol* __restrict__ cols) {
    const int c = blockIdx.y;
    if (!cols[c].active) return;
    const double beta = cols[c].beta;
    const double* zc = z + (long long)c * ld;
    double* pc = p + (long long)c * ld;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        pc[i] = __dadd_rn(zc[i], __dmul_rn(beta, pc[i]));
}

// Column setup: threshold from |b| and the first residual; a column already within it
// makes no step.
__global__ void k_cg_init(const double* bnorm2, const double* rnorm2, double tol, int nrhs, CgCol* cols) {
    const int c = threadIdx.x;
    if (c >= nrhs) return;
    const double bn = sqrt(bnorm2[c]);
    CgCol C{};
    C.scale = bn > 0.0 ? bn : 1.0;
    C.thr = tol * C.scale;
    C.rnorm2 = rnorm2[c];
    C.active = sqrt(rnorm2[c]) <= C.thr ? 0 : 1;
    cols[c] = C;
}

// inv[i] = 1 / A(i, i) (JacobiPreconditioner); *bad = the first row whose diagonal is
// zero, absent or not finite.  Without the preconditioner inv = 1 (z = r exactly).
__global__ void k_jacobi_inverse(const double* __restrict__ values, const int* __restrict__ diag, int n,
                                 double pivot_tol, int use, double* __restrict__ inv, int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!use) {
            inv[i] = 1.0;
            continue;
        }
        const double d = diag[i] >= 0 ? values[diag[i]] : 0.0;
        if (!isfinite(d) || fabs(d) <= pivot_tol) {
            atomicMin(bad, i);
            inv[i] = 0.0;
        } else {
            inv[i] = 1.0 / d;
        }
    }
}

uchol_dmatrix_s* check_dmatrix(uchol_dmatrix m) {
    if (!m) throw Error(UCHOL_BAD_ARG, "matrix handle is null");
    return m;
}

void check_plan(uchol_dmatrix_s* m, uchol_values_plan p, int kind) {
    if (!p) throw Error(UCHOL_BAD_ARG, "plan handle is null");
    if (p->m != m) throw Error(UCHOL_BAD_ARG, "the plan was built for another matrix");
    if (p->kind != kind)
        throw Error(UCHOL_BAD_ARG, kind == 0 ? "the plan is a LineCross list, not an AccumulateAt list"
                                             : "the plan is an AccumulateAt list, not a LineCross list");
}

int find_position(const uchol_dmatrix_s* m, int row, int c) {
    if (row == c) return m->diag[row];
    const int* b = m->col.data() + m->row_ptr[row];
    const int* e = m->col.data() + m->row_ptr[row + 1];
    const int* it = std::lower_bound(b, e, c);
    return (it != e && *it == c) ? (int)(it - m->col.data()) : -1;
}

// Product structure of both triangles and the values gathered into it.
void dmatrix_full_values(uchol_dmatrix_s* m) {
    if (m->full_nnz > 0) {
        k_gather_values<<<grid_for(m->full_nnz, 256), 256, 0, m->stream>>>(m->values.as<double>(), m->full_src.as<int>(),
                                                                           m->full_nnz, m->full_val.as<double>());
        counted();
    }
}

// Workspace layout for nrhs columns: r z p q xd bd (n * nrhs each), inv (n), partial
// (2 * kCgBlocks * nrhs), norms (2 * nrhs), cols (nrhs), counters (nrhs), bad (1).
struct CgWs {
    double *r, *z, *p, *q, *xd, *bd, *inv, *partial, *bn2, *rn2;
    CgCol* cols;
    unsigned* counters;
    int* bad;
};

CgWs dmatrix_ws(uchol_dmatrix_s* m, int nrhs) {
    const size_t n = (size_t)std::max(1, m->n);
    const size_t nv = n * nrhs;
    auto bytes = [&](int k) {
        return (6 * nv + n + 2 * (size_t)kCgBlocks * k + 2 * (size_t)k) * 8 + (size_t)k * sizeof(CgCol) +
               (size_t)k * 4 + 16;
    };
    if (m->ws_nrhs < nrhs) {
        CK(cudaStreamSynchronize(m->stream));
        m->ws.alloc(bytes(nrhs), "matrix workspace");
        CK(cudaMemsetAsync(m->ws.p, 0, m->ws.bytes, m->stream));   // reduction counters start at zero
        m->ws_nrhs = nrhs;
    }
    const size_t cap = (size_t)m->ws_nrhs;
    const size_t nvc = n * cap;
    char* b = (char*)m->ws.p;
    CgWs w;
    double* d = (double*)b;
    w.r = d; w.z = d + nvc; w.p = d + 2 * nvc; w.q = d + 3 * nvc; w.xd = d + 4 * nvc; w.bd = d + 5 * nvc;
    w.inv = d + 6 * nvc;
    w.partial = w.inv + n;
    w.bn2 = w.partial + 2 * (size_t)kCgBlocks * cap;
    w.rn2 = w.bn2 + cap;
    w.cols = (CgCol*)(w.rn2 + cap);
    w.counters = (unsigned*)(w.cols + cap);
    w.bad = (int*)(w.counters + cap);
    return w;
}

// out[c] = u_c . v_c, deterministic (the kernels of the factor's refinement).
void dm_dots(uchol_dmatrix_s* m, int nrhs, const double* u, int ldu, const double* v, int ldv, double* partial,
             double* out) {
    dim3 g(kDotBlocks, nrhs);
    k_dot_partial<<<g, 256, 0, m->stream>>>(u, ldu, v, ldv, m->n, partial);
    k_dot_finish<<<1, 32 * ((nrhs + 31) / 32), 0, m->stream>>>(partial, kDotBlocks, nrhs, out);
    counted(2);
}

void jacobi_pcg(uchol_dmatrix_s* m, int nrhs, const double* b, int ldb, double* x, int ldx, bool on_device,
                const uchol_cg_options& o, uchol_cg_result* res) {
    const int n = m->n;
    cudaStream_t st = m->stream;
    StreamTimer timer(st);
    if (n == 0) {
        const double ms = timer.stop();
        for (int c = 0; c < nrhs; ++c) res[c] = {0, 1, 0.0, 0.0, ms};
        return;
    }
    CgWs w = dmatrix_ws(m, nrhs);
    const double* db = b;
    double* dx = x;
    int ldbd = ldb, ldxd = ldx;
    if (!on_device) {
        CK(cudaMemcpy2DAsync(w.bd, (size_t)n * 8, b, (size_t)ldb * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice, st));
        if (o.use_initial_guess)
            CK(cudaMemcpy2DAsync(w.xd, (size_t)n * 8, x, (size_t)ldx * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice,
                                 st));
        db = w.bd;
        dx = w.xd;
        ldbd = ldxd = n;
    }
    if (!o.use_initial_guess) CK(cudaMemset2DAsync(dx, (size_t)ldxd * 8, 0, (size_t)n * 8, nrhs, st));
    dmatrix_full_values(m);
    // b norms, first residual r = b - A x0 and its norm
    dm_dots(m, nrhs, db, ldbd, db, ldbd, w.partial, w.bn2);
    k_spmv_residual<<<(n + 7) / 8, 256, 0, st>>>(m->full_ptr.as<int>(), m->full_col.as<int>(), m->full_val.as<double>(),
                                                 n, nrhs, dx, ldxd, db, ldbd, w.r, n);
    counted();
    dm_dots(m, nrhs, w.r, n, w.r, n, w.partial, w.rn2);
    k_cg_init<<<1, 32 * ((nrhs + 31) / 32), 0, st>>>(w.bn2, w.rn2, o.relative_tolerance, nrhs, w.cols);
    const int bad_init = INT_MAX;
    CK(cudaMemcpyAsync(w.bad, &bad_init, sizeof(int), cudaMemcpyHostToDevice, st));
    k_jacobi_inverse<<<grid_for(n, 256), 256, 0, st>>>(m->values.as<double>(), m->d_diag.as<int>(), n,
                                                       o.pivot_tolerance, o.use_preconditioner ? 1 : 0, w.inv, w.bad);
    counted(2);
    std::vector<CgCol> hc(nrhs);
    int hbad = INT_MAX;
    CK(cudaMemcpyAsync(hc.data(), w.cols, nrhs * sizeof(CgCol), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hbad, w.bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    bool any = false;
    for (int c = 0; c < nrhs; ++c) any |= hc[c].active != 0;
    if (any && hbad != INT_MAX)
        throw Error(UCHOL_NOT_SPD, "The diagonal element in row " + std::to_string(hbad) +
                                       " is zero or invalid while building the Jacobi preconditioner.");
    const int max_it = o.max_iterations > 0 ? o.max_iterations : n;
    const int gx = std::min(kCgBlocks, grid_for(n, 256));
    const dim3 gv(gx, nrhs);
    if (any) {
        k_cg_start<<<gv, 256, 0, st>>>(w.inv, w.r, w.z, w.p, n, n, w.cols, w.partial, w.counters);
        counted();
    }
    int steps = 0;
    while (any) {
        const int chunk = std::min(kCgPoll, max_it - steps);
        for (int k = 0; k < chunk; ++k) {
            k_cg_spmv<<<(n + 7) / 8, 256, 0, st>>>(m->full_ptr.as<int>(), m->full_col.as<int>(), m->full_val.as<double>(),
                                                   n, nrhs, w.p, n, w.q, w.cols);
            k_cg_alpha<<<gv, 256, 0, st>>>(w.p, w.q, n, n, w.cols, w.partial, w.counters);
            k_cg_update<<<gv, 256, 0, st>>>(dx, ldxd, w.r, w.z, w.p, w.q, w.inv, n, n, max_it, w.cols, w.partial,
                                            w.counters);
            k_cg_direction<<<gv, 256, 0, st>>>(w.z, w.p, n, n, w.cols);
            counted(4);
        }
        steps += chunk;
        CK(cudaMemcpyAsync(hc.data(), w.cols, nrhs * sizeof(CgCol), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        any = false;
        for (int c = 0; c < nrhs; ++c) {
            if (hc[c].failed)
                throw Error(UCHOL_NOT_SPD,
                            "p^T A p <= 0. The matrix is not positive definite, so the CG method cannot be applied.");
            any |= hc[c].active != 0;
        }
        if (steps >= max_it) any = false;   // every column has stopped by its own count
    }
    CK(cudaGetLastError());
    if (!on_device)
        CK(cudaMemcpy2DAsync(x, (size_t)ldx * 8, w.xd, (size_t)n * 8, (size_t)n * 8, nrhs, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hc.data(), w.cols, nrhs * sizeof(CgCol), cudaMemcpyDeviceToHost, st));
    const double ms = timer.stop();
    for (int c = 0; c < nrhs; ++c) {
        const double rn = std::sqrt(hc[c].rnorm2);
        const double rel = rn / hc[c].scale;
        res[c] = {hc[c].iters, rel <= o.relative_tolerance ? 1 : 0, rn, rel, ms};
    }
}

}  // namespace

extern "C" {

int uchol_dmatrix_create(int n, int nnz, const int* row_ptr, const int* col, const double* values, void* stream,
                         uchol_dmatrix* out) {
    return guarded([&] {
        if (!out) throw Error(UCHOL_BAD_ARG, "null output handle");
        *out = nullptr;
        if (n < 0 || nnz < 0) throw Error(UCHOL_BAD_ARG, "negative size");
        if (!row_ptr || (nnz > 0 && !col)) throw Error(UCHOL_BAD_ARG, "null structure");
        if (row_ptr[0] != 0 || row_ptr[n] != nnz) throw Error(UCHOL_BAD_ARG, "row pointers do not span nnz entries");
        auto M = std::make_unique<uchol_dmatrix_s>();
        M->n = n;
        M->nnz = nnz;
        M->row_ptr.assign(row_ptr, row_ptr + n + 1);
        M->col.assign(col, col + nnz);
        M->diag.assign(n, -1);
        for (int r = 0; r < n; ++r) {
            if (row_ptr[r + 1] < row_ptr[r]) throw Error(UCHOL_BAD_ARG, "row pointers decrease");
            for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                if (col[k] < r || col[k] >= n || (k > row_ptr[r] && col[k] <= col[k - 1]))
                    throw Error(UCHOL_BAD_ARG, "the structure is not an upper-triangle CSR with ascending columns");
            }
            if (row_ptr[r + 1] > row_ptr[r] && col[row_ptr[r]] == r) M->diag[r] = row_ptr[r];
        }
        // column view of the upper half: for column c the rows r < c holding (r, c), ascending
        M->col_ptr.assign(n + 1, 0);
        for (int k = 0; k < nnz; ++k) M->col_ptr[col[k] + 1]++;
        for (int c = 0; c < n; ++c) M->col_ptr[c + 1] += M->col_ptr[c];
        M->col_row.resize(nnz);
        M->col_pos.resize(nnz);
        {
            std::vector<int> fill(M->col_ptr.begin(), M->col_ptr.end() - 1);
            for (int r = 0; r < n; ++r)
                for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                    const int c = col[k];
                    M->col_row[fill[c]] = r;
                    M->col_pos[fill[c]++] = k;
                }
        }
        if (stream) {
            M->stream = (cudaStream_t)stream;
        } else {
            CK(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking));
            M->own_stream = true;
        }
        cudaStream_t st = M->stream;
        M->values.alloc((size_t)std::max(1, nnz) * 8, "matrix values");
        if (values && nnz > 0)
            CK(cudaMemcpyAsync(M->values.p, values, (size_t)nnz * 8, cudaMemcpyHostToDevice, st));
        else
            CK(cudaMemsetAsync(M->values.p, 0, M->values.bytes, st));
        M->d_diag.upload(M->diag, st, "matrix structure");
        // product structure of both triangles (transposed entries first, then the row's own)
        std::vector<int> cnt(n + 1, 0);
        for (int r = 0; r < n; ++r)
            for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                cnt[r + 1]++;
                if (col[k] != r) cnt[col[k] + 1]++;
            }
        for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
        std::vector<int> fcol(cnt[n]), fsrc(cnt[n]);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int r = 0; r < n; ++r)
            for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                const int c = col[k];
                fcol[fill[r]] = c;
                fsrc[fill[r]++] = k;
                if (c != r) {
                    fcol[fill[c]] = r;
                    fsrc[fill[c]++] = k;
                }
            }
        M->full_nnz = cnt[n];
        M->full_ptr.upload(cnt, st, "product structure");
        M->full_col.upload(fcol, st, "product structure");
        M->full_src.upload(fsrc, st, "product structure");
        M->full_val.alloc((size_t)std::max<long long>(1, M->full_nnz) * 8, "product values");
        CK(cudaStreamSynchronize(st));
        *out = M.release();
    });
}

int uchol_dmatrix_destroy(uchol_dmatrix m) {
    return guarded([&] {
        if (!m) return;
        cudaStream_t st = m->stream;
        const bool own = m->own_stream;
        if (st) cudaStreamSynchronize(st);
        delete m;
        if (own && st) cudaStreamDestroy(st);
    });
}

int uchol_dmatrix_set_stream(uchol_dmatrix m, void* stream) {
    return guarded([&] {
        check_dmatrix(m);
        std::lock_guard<std::mutex> lk(m->mu);
        CK(cudaStreamSynchronize(m->stream));
        if (m->own_stream) CK(cudaStreamDestroy(m->stream));
        if (stream) {
            m->stream = (cudaStream_t)stream;
            m->own_stream = false;
        } else {
            CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
            m->own_stream = true;
        }
    });
}

int uchol_dmatrix_values(uchol_dmatrix m, double** d_values) {
    return guarded([&] {
        check_dmatrix(m);
        if (!d_values) throw Error(UCHOL_BAD_ARG, "null output");
        *d_values = m->values.as<double>();
    });
}

int uchol_dmatrix_set_values(uchol_dmatrix m, const double* values, int on_device) {
    return guarded([&] {
        check_dmatrix(m);
        if (!values && m->nnz > 0) throw Error(UCHOL_BAD_ARG, "values is null");
        std::lock_guard<std::mutex> lk(m->mu);
        if (m->nnz == 0) return;
        CK(cudaMemcpyAsync(m->values.p, values, (size_t)m->nnz * 8,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, m->stream));
        if (!on_device) CK(cudaStreamSynchronize(m->stream));
    });
}

int uchol_dmatrix_get_values(uchol_dmatrix m, double* out, int on_device) {
    return guarded([&] {
        check_dmatrix(m);
        if (!out && m->nnz > 0) throw Error(UCHOL_BAD_ARG, "null output");
        std::lock_guard<std::mutex> lk(m->mu);
        if (m->nnz == 0) return;
        CK(cudaMemcpyAsync(out, m->values.p, (size_t)m->nnz * 8,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, m->stream));
        if (!on_device) CK(cudaStreamSynchronize(m->stream));
    });
}

int uchol_dmatrix_clear_values(uchol_dmatrix m) {
    return guarded([&] {
        check_dmatrix(m);
        std::lock_guard<std::mutex> lk(m->mu);
        CK(cudaMemsetAsync(m->values.p, 0, m->values.bytes, m->stream));
    });
}

int uchol_accumulate_plan_create(uchol_dmatrix m, int count, const int* rows, const int* cols,
                                 uchol_values_plan* out) {
    return guarded([&] {
        check_dmatrix(m);
        if (!out) throw Error(UCHOL_BAD_ARG, "null output handle");
        *out = nullptr;
        if (count < 0) throw Error(UCHOL_BAD_ARG, "negative item count");
        if (count > 0 && (!rows || !cols)) throw Error(UCHOL_BAD_ARG, "null item positions");
        std::vector<int> pos(count);
        for (int i = 0; i < count; ++i) {
            int r = rows[i], c = cols[i];
            if (r < 0 || r >= m->n || c < 0 || c >= m->n)
                throw Error(UCHOL_OUT_OF_RANGE, "Indices are out of range: (" + std::to_string(r) + ", " +
                                                    std::to_string(c) + ") (item " + std::to_string(i) + ").");
            if (r > c) std::swap(r, c);
            pos[i] = find_position(m, r, c);
            if (pos[i] < 0)
                throw Error(UCHOL_NOT_IN_PATTERN,
                            "Position (" + std::to_string(r) + ", " + std::to_string(c) +
                                ") is absent from the sparse structure. Add this position to "
                                "SymmetricSparseMatrixCSRBuilder before assembly.");
        }
        // stable counting sort of the items by position
        std::vector<int> cnt(m->nnz + 1, 0);
        for (int i = 0; i < count; ++i) cnt[pos[i] + 1]++;
        std::vector<int> tpos, tptr{0}, perm(count);
        std::vector<int> start(m->nnz + 1, 0);
        for (int k = 0; k < m->nnz; ++k) start[k + 1] = start[k] + cnt[k + 1];
        {
            std::vector<int> fill(start.begin(), start.end() - 1);
            for (int i = 0; i < count; ++i) perm[fill[pos[i]]++] = i;
        }
        for (int k = 0; k < m->nnz; ++k)
            if (cnt[k + 1] > 0) {
                tpos.push_back(k);
                tptr.push_back(start[k + 1]);
            }
        auto P = std::make_unique<uchol_values_plan_s>();
        P->m = m;
        P->kind = 0;
        P->count = count;
        P->targets = (int)tpos.size();
        P->tgt_pos.upload(tpos, m->stream, "accumulate plan");
        P->tgt_ptr.upload(tptr, m->stream, "accumulate plan");
        P->item_perm.upload(perm, m->stream, "accumulate plan");
        CK(cudaStreamSynchronize(m->stream));
        *out = P.release();
    });
}

int uchol_accumulate(uchol_dmatrix m, uchol_values_plan p, const double* items, int on_device) {
    return guarded([&] {
        check_dmatrix(m);
        check_plan(m, p, 0);
        if (!items && p->count > 0) throw Error(UCHOL_BAD_ARG, "item values are null");
        std::lock_guard<std::mutex> lk(m->mu);
        if (p->targets == 0) return;
        const double* d = items;
        if (!on_device) {
            if (!p->items.p) p->items.alloc((size_t)p->count * 8, "accumulate items");
            CK(cudaMemcpyAsync(p->items.p, items, (size_t)p->count * 8, cudaMemcpyHostToDevice, m->stream));
            d = p->items.as<double>();
        }
        k_accumulate<<<grid_for(p->targets, 256), 256, 0, m->stream>>>(p->tgt_pos.as<int>(), p->tgt_ptr.as<int>(),
                                                                       p->item_perm.as<int>(), p->targets, d,
                                                                       m->values.as<double>());
        counted();
        CK(cudaGetLastError());
        if (!on_device) CK(cudaStreamSynchronize(m->stream));
    });
}

int uchol_line_cross_plan_create(uchol_dmatrix m, int count, const int* indices, uchol_values_plan* out) {
    return guarded([&] {
        check_dmatrix(m);
        if (!out) throw Error(UCHOL_BAD_ARG, "null output handle");
        *out = nullptr;
        if (count < 0) throw Error(UCHOL_BAD_ARG, "negative index count");
        if (count > 0 && !indices) throw Error(UCHOL_BAD_ARG, "null index list");
        const int n = m->n;
        std::vector<std::vector<std::pair<int, int>>> ev(n);   // per rhs row: (position or code, list item)
        std::vector<char> zeroed(m->nnz, 0), one(n, 0);
        std::vector<int> zero_pos, one_pos;
        for (int t = 0; t < count; ++t) {
            const int k = indices[t];
            if (k < 0 || k >= n)
                throw Error(UCHOL_OUT_OF_RANGE, "index " + std::to_string(k) + " (item " + std::to_string(t) +
                                                    ") is out of range");
            if (m->diag[k] < 0)
                throw Error(UCHOL_NOT_IN_PATTERN, "Diagonal position (" + std::to_string(k) + ", " + std::to_string(k) +
                                                      ") is absent from the sparse structure.");
            auto hit = [&](int pos, int other) {
                ev[other].push_back({zeroed[pos] ? kEvZeroed : pos, t});
                if (!zeroed[pos]) {
                    zeroed[pos] = 1;
                    zero_pos.push_back(pos);
                }
            };
            for (int a = m->col_ptr[k]; a < m->col_ptr[k + 1]; ++a)   // (r, k), r < k
                if (m->col_row[a] != k) hit(m->col_pos[a], m->col_row[a]);
            for (int pos = m->row_ptr[k]; pos < m->row_ptr[k + 1]; ++pos)   // (k, c), c > k
                if (m->col[pos] != k) hit(pos, m->col[pos]);
            ev[k].push_back({kEvSet, t});
            if (!one[k]) {
                one[k] = 1;
                one_pos.push_back(m->diag[k]);
            }
        }
        std::vector<int> eptr{0}, erow, epos, et;
        for (int r = 0; r < n; ++r) {
            if (ev[r].empty()) continue;
            erow.push_back(r);
            for (auto& e : ev[r]) {
                epos.push_back(e.first);
                et.push_back(e.second);
            }
            eptr.push_back((int)epos.size());
        }
        auto P = std::make_unique<uchol_values_plan_s>();
        P->m = m;
        P->kind = 1;
        P->count = count;
        P->rows = (int)erow.size();
        P->nzero = (int)zero_pos.size();
        P->nones = (int)one_pos.size();
        cudaStream_t st = m->stream;
        P->ev_ptr.upload(eptr, st, "LineCross plan");
        P->ev_row.upload(erow, st, "LineCross plan");
        P->ev_pos.upload(epos, st, "LineCross plan");
        P->ev_t.upload(et, st, "LineCross plan");
        P->zero_pos.upload(zero_pos, st, "LineCross plan");
        P->one_pos.upload(one_pos, st, "LineCross plan");
        CK(cudaStreamSynchronize(st));
        *out = P.release();
    });
}

int uchol_line_cross(uchol_dmatrix m, uchol_values_plan p, double* rhs, int ldr, int nrhs, const double* prescribed,
                     int ldp, int on_device) {
    return guarded([&] {
        check_dmatrix(m);
        check_plan(m, p, 1);
        if (nrhs < 0) throw Error(UCHOL_BAD_ARG, "negative right-hand-side count");
        if (nrhs > 0 && (!rhs || (!prescribed && p->count > 0)))
            throw Error(UCHOL_BAD_ARG, "null right-hand side or prescribed values");
        if (nrhs > 0 && (ldr < m->n || ldp < p->count)) throw Error(UCHOL_BAD_ARG, "leading dimension too small");
        std::lock_guard<std::mutex> lk(m->mu);
        cudaStream_t st = m->stream;
        const int n = m->n;
        double* drhs = rhs;
        const double* dpres = prescribed;
        int ldr_d = ldr, ldp_d = ldp;
        if (!on_device && nrhs > 0) {
            if (p->rhs_ws.bytes < (size_t)n * nrhs * 8) p->rhs_ws.alloc((size_t)n * nrhs * 8, "LineCross right-hand side");
            if (p->pres_ws.bytes < (size_t)std::max(1, p->count) * nrhs * 8)
                p->pres_ws.alloc((size_t)std::max(1, p->count) * nrhs * 8, "LineCross prescribed values");
            CK(cudaMemcpy2DAsync(p->rhs_ws.p, (size_t)n * 8, rhs, (size_t)ldr * 8, (size_t)n * 8, nrhs,
                                 cudaMemcpyHostToDevice, st));
            if (p->count > 0)
                CK(cudaMemcpy2DAsync(p->pres_ws.p, (size_t)p->count * 8, prescribed, (size_t)ldp * 8,
                                     (size_t)p->count * 8, nrhs, cudaMemcpyHostToDevice, st));
            drhs = p->rhs_ws.as<double>();
            dpres = p->pres_ws.as<double>();
            ldr_d = n;
            ldp_d = std::max(1, p->count);
        }
        if (nrhs > 0 && p->rows > 0) {
            dim3 g(grid_for(p->rows, 256), std::min(nrhs, 65535));
            k_line_cross_rhs<<<g, 256, 0, st>>>(p->ev_ptr.as<int>(), p->ev_row.as<int>(), p->ev_pos.as<int>(),
                                                p->ev_t.as<int>(), p->rows, m->values.as<double>(), drhs, ldr_d, dpres,
                                                ldp_d, nrhs);
            counted();
        }
        if (p->nzero + p->nones > 0) {
            k_line_cross_values<<<grid_for(p->nzero + p->nones, 256), 256, 0, st>>>(
                p->zero_pos.as<int>(), p->nzero, p->one_pos.as<int>(), p->nones, m->values.as<double>());
            counted();
        }
        CK(cudaGetLastError());
        if (!on_device) {
            if (nrhs > 0)
                CK(cudaMemcpy2DAsync(rhs, (size_t)ldr * 8, drhs, (size_t)n * 8, (size_t)n * 8, nrhs,
                                     cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    });
}

int uchol_values_plan_destroy(uchol_values_plan p) {
    // The plan's matrix may already be destroyed (the two are released in any order): the
    // plan only keeps its address for the check that it is applied to that matrix, and is
    // freed without touching it (cudaFree waits for the device work that reads the buffers).
    return guarded([&] {
        if (!p) return;
        delete p;
    });
}

int uchol_dmatrix_multiply(uchol_dmatrix m, int nrhs, const double* x, int ldx, double* y, int ldy, int on_device) {
    return guarded([&] {
        check_dmatrix(m);
        if (nrhs < 0) throw Error(UCHOL_BAD_ARG, "negative right-hand-side count");
        if (nrhs > 0 && (!x || !y)) throw Error(UCHOL_BAD_ARG, "null vector");
        if (nrhs > 0 && (ldx < m->n || ldy < m->n)) throw Error(UCHOL_BAD_ARG, "leading dimension too small");
        std::lock_guard<std::mutex> lk(m->mu);
        const int n = m->n;
        if (n == 0 || nrhs == 0) return;
        cudaStream_t st = m->stream;
        dmatrix_full_values(m);
        if (on_device) {
            k_spmv_residual<<<(n + 7) / 8, 256, 0, st>>>(m->full_ptr.as<int>(), m->full_col.as<int>(),
                                                         m->full_val.as<double>(), n, nrhs, x, ldx, nullptr, 0, y, ldy);
            counted();
        } else {
            CgWs w = dmatrix_ws(m, nrhs);
            CK(cudaMemcpy2DAsync(w.xd, (size_t)n * 8, x, (size_t)ldx * 8, (size_t)n * 8, nrhs, cudaMemcpyHostToDevice,
                                 st));
            k_spmv_residual<<<(n + 7) / 8, 256, 0, st>>>(m->full_ptr.as<int>(), m->full_col.as<int>(),
                                                         m->full_val.as<double>(), n, nrhs, w.xd, n, nullptr, 0, w.bd, n);
            counted();
            CK(cudaMemcpy2DAsync(y, (size_t)ldy * 8, w.bd, (size_t)n * 8, (size_t)n * 8, nrhs, cudaMemcpyDeviceToHost,
                                 st));
            CK(cudaStreamSynchronize(st));
        }
        CK(cudaGetLastError());
    });
}

void uchol_default_cg_options(uchol_cg_options* o) {
    if (!o) return;
    o->relative_tolerance = 1e-8;
    o->max_iterations = 0;
    o->use_preconditioner = 1;
    o->use_initial_guess = 0;
    o->pivot_tolerance = 1e-300;
}

int uchol_jacobi_pcg(uchol_dmatrix m, int nrhs, const double* b, int ldb, double* x, int ldx, int on_device,
                     const uchol_cg_options* opts, uchol_cg_result* results) {
    return guarded([&] {
        check_dmatrix(m);
        uchol_cg_options o;
        uchol_default_cg_options(&o);
        if (opts) o = *opts;
        if (!std::isfinite(o.relative_tolerance) || o.relative_tolerance < 0.0)
            throw Error(UCHOL_OUT_OF_RANGE, "RelativeTolerance must be finite and >= 0");
        if (o.max_iterations < 0)
            throw Error(UCHOL_OUT_OF_RANGE, "MaxIterations: the maximum iteration count cannot be negative.");
        if (!std::isfinite(o.pivot_tolerance) || o.pivot_tolerance <= 0.0)
            throw Error(UCHOL_OUT_OF_RANGE, "pivotTolerance must be finite and > 0");
        if (nrhs < 0 || nrhs > 1024) throw Error(UCHOL_BAD_ARG, "nrhs must be in [0, 1024]");
        if (nrhs > 0 && (!b || !x || !results)) throw Error(UCHOL_BAD_ARG, "null argument");
        if (nrhs > 0 && (ldb < m->n || ldx < m->n)) throw Error(UCHOL_BAD_ARG, "leading dimension too small");
        if (nrhs == 0) return;
        std::lock_guard<std::mutex> lk(m->mu);
        jacobi_pcg(m, nrhs, b, ldb, x, ldx, on_device != 0, o, results);
    });
}

int uchol_refactorize_dmatrix(uchol_factor f, uchol_dmatrix m, uchol_factor_stats* stats) {
    return guarded([&] {
        if (!f) throw Error(UCHOL_BAD_ARG, "factor handle is null");
        check_dmatrix(m);
        uchol_symbolic_s* S = f->sym;
        if (m->n != S->n || m->nnz != S->nnz)
            throw Error(UCHOL_PATTERN_MISMATCH, "the matrix does not have the structure of the symbolic factorization");
        std::lock_guard<std::mutex> lk(f->mu);
        std::lock_guard<std::mutex> lm(m->mu);
        if (m->checked_symbolic != (const void*)S) {
            if (m->row_ptr != S->row_ptr || m->col != S->col)
                throw Error(UCHOL_PATTERN_MISMATCH,
                            "the matrix does not have the structure of the symbolic factorization");
            m->checked_symbolic = S;
        }
        // the factorisation's stream waits for the refresh work queued on the matrix's stream
        if (m->stream != S->stream) {
            cudaEvent_t ev;
            CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            cudaError_t e1 = cudaEventRecord(ev, m->stream);
            cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(S->stream, ev, 0) : e1;
            cudaEventDestroy(ev);
            CK(e2);
        }
        factorize_impl(f, m->values.as<double>(), true);
        if (stats) *stats = f->last;
    });
}

}  // extern "C"
