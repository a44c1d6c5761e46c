// ORACLE — test infrastructure only.  CPU restatement of the reference's
// values-refresh operations on a SymmetricCSRMatrix and of its
// Jacobi-preconditioned conjugate gradients, the checker of the device
// refresh kernels and the device PCG.  Scalar, sequential, in the reference's
// own loop order; compiled without floating-point contraction.
//
//   oracle_accumulate  SymmetricCSRMatrix.AccumulateAt   CAESolvers/SymmetricCSRMatrix.cs:98-110
//                      (bounds check :208-212, normalisation :198-206, search :219-240)
//   oracle_line_cross  SymmetricCSRMatrix.LineCross      CAESolvers/SymmetricCSRMatrix.cs:125-167
//   oracle_jacobi_pcg  ConjugateGradientGaussPreSolver   CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs:78-165
//                      JacobiPreconditioner              CAESolvers/CGGP/JacobiPreconditioner.cs:12-57
//                      allocation-free Multiply          CAESolvers/SymmetricCSRMatrix.cs:293-324
//                      CalculateNorm                     CAESolvers/ResidualCalculator.cs:23-31
#include <cmath>
#include <cstring>
#include <vector>

namespace {

// Position of (row, col), row <= col, in the upper CSR; -1 when structurally absent.
int find_index(const int* row_ptr, const int* col, const int* diag, int row, int c) {
    if (row == c) return diag[row];
    int lo = row_ptr[row], hi = row_ptr[row + 1] - 1;
    while (lo <= hi) {
        const int mid = lo + (hi - lo) / 2;
        if (col[mid] == c) return mid;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// result = A x through the stored upper half, in the reference's order: the
// row's own entries accumulate separately and are added after the transposed
// contributions of the earlier rows.
void multiply(int n, const int* row_ptr, const int* col, const double* val, const double* x, double* result) {
    for (int i = 0; i < n; ++i) result[i] = 0.0;
    for (int row = 0; row < n; ++row) {
        const double xrow = x[row];
        double accumulated = 0.0;
        for (int k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
            const int c = col[k];
            const double v = val[k];
            accumulated = accumulated + v * x[c];
            if (c != row) result[c] = result[c] + v * xrow;
        }
        result[row] = result[row] + accumulated;
    }
}

double norm(const double* v, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + v[i] * v[i];
    return std::sqrt(s);
}

double dot(const double* a, const double* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
    return s;
}

}  // namespace

extern "C" {

// values[pos(rows[i], cols[i])] += items[i] for i = 0..count-1 in order.
// Returns 0, 1 (index out of range: IndexOutOfRangeException) or
// 2 (position absent: InvalidOperationException); *bad = the failing item.
int oracle_accumulate(int n, const int* row_ptr, const int* col, const int* diag, double* val, int count,
                      const int* rows, const int* cols, const double* items, int* bad) {
    *bad = -1;
    for (int i = 0; i < count; ++i) {
        int r = rows[i], c = cols[i];
        if (r < 0 || r >= n || c < 0 || c >= n) {
            *bad = i;
            return 1;
        }
        if (r > c) {
            const int t = r;
            r = c;
            c = t;
        }
        const int k = find_index(row_ptr, col, diag, r, c);
        if (k < 0) {
            *bad = i;
            return 2;
        }
        val[k] += items[i];
    }
    return 0;
}

// One LineCross(rhs, prescribed, index).  Returns 0, 1 (index out of range) or
// 2 (diagonal absent from the structure).
int oracle_line_cross(int n, const int* row_ptr, const int* col, const int* diag, double* val, double* rhs,
                      double prescribed, int index) {
    if (index < 0 || index >= n) return 1;
    const int di = diag[index];
    if (di < 0) return 2;
    for (int row = 0; row < n; ++row)
        for (int pos = row_ptr[row]; pos < row_ptr[row + 1]; ++pos) {
            const int c = col[pos];
            if (row == c) continue;
            int other;
            if (row == index) other = c;
            else if (c == index) other = row;
            else continue;
            rhs[other] -= val[pos] * prescribed;
            val[pos] = 0.0;
        }
    val[di] = 1.0;
    rhs[index] = prescribed;
    return 0;
}

// Jacobi-preconditioned CG from x (in: the initial guess, or zeros; out: the
// solution).  Returns 0, 3 (a diagonal entry zero or not finite, *bad = its
// row) or 4 (p^T A p <= 0: InvalidOperationException).  out = {iterations,
// converged, residual norm, relative residual}.
int oracle_jacobi_pcg(int n, const int* row_ptr, const int* col, const int* diag, const double* val,
                      const double* b, double* x, double tolerance, int max_iterations, int use_preconditioner,
                      double pivot_tolerance, double* out, int* bad) {
    *bad = -1;
    const double bnorm = norm(b, n);
    const double scale = bnorm > 0.0 ? bnorm : 1.0;
    auto complete = [&](int it, double rnorm) {
        out[0] = it;
        out[2] = rnorm;
        out[3] = rnorm / scale;
        out[1] = out[3] <= tolerance ? 1.0 : 0.0;
        return 0;
    };
    if (n == 0) return complete(0, 0.0);
    const double threshold = tolerance * scale;
    std::vector<double> r(n), z(n), p(n), ap(n), inv;
    multiply(n, row_ptr, col, val, x, ap.data());
    for (int i = 0; i < n; ++i) r[i] = b[i] - ap[i];
    double rnorm = norm(r.data(), n);
    if (rnorm <= threshold) return complete(0, rnorm);
    if (use_preconditioner) {
        inv.resize(n);
        for (int i = 0; i < n; ++i) {
            const double d = diag[i] >= 0 ? val[diag[i]] : 0.0;
            if (!std::isfinite(d) || std::fabs(d) <= pivot_tolerance) {
                *bad = i;
                return 3;
            }
            inv[i] = 1.0 / d;
        }
    }
    auto precondition = [&]() {
        if (use_preconditioner)
            for (int i = 0; i < n; ++i) z[i] = inv[i] * r[i];
        else
            std::memcpy(z.data(), r.data(), sizeof(double) * n);
    };
    precondition();
    p = z;
    double rz_old = dot(r.data(), z.data(), n);
    const int max_it = max_iterations > 0 ? max_iterations : n;
    for (int it = 1; it <= max_it; ++it) {
        multiply(n, row_ptr, col, val, p.data(), ap.data());
        const double pap = dot(p.data(), ap.data(), n);
        if (pap <= 0.0) return 4;
        const double alpha = rz_old / pap;
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * ap[i];
        }
        rnorm = norm(r.data(), n);
        if (rnorm <= threshold) return complete(it, rnorm);
        precondition();
        const double rz_new = dot(r.data(), z.data(), n);
        const double beta = rz_new / rz_old;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz_old = rz_new;
    }
    return complete(max_it, rnorm);
}

}  // extern "C"
