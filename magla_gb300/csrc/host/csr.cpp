// Matrix construction for the upper-triangle symmetric CSR format and the
// adjacency graph used by the ordering.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "symbolic.hpp"

namespace uchol {

// Entries whose summed value has magnitude <= this are dropped from the
// structure (CAESolvers/SymmetricCSRMatrix.cs:29,57).
static constexpr double kDropTolerance = 1e-15;

UpperCsr csr_from_triplets(int n, int64_t count, const int* rows, const int* cols, const double* vals) {
    if (n < 0) throw std::invalid_argument("matrix size must be non-negative");
    // Bucket the normalised entries by row, keeping input order (stable), then
    // order each row's bucket by column (stable) so duplicates are summed in
    // the order they were supplied.
    std::vector<int64_t> row_count(static_cast<size_t>(n) + 1, 0);
    for (int64_t t = 0; t < count; ++t) {
        int r = rows[t], c = cols[t];
        if (r < 0 || r >= n || c < 0 || c >= n)
            throw std::out_of_range("triplet index out of range");
        row_count[std::min(r, c) + 1]++;
    }
    for (int i = 0; i < n; ++i) row_count[i + 1] += row_count[i];
    std::vector<int64_t> cursor(row_count.begin(), row_count.end() - 1);
    std::vector<int> bucket_col(static_cast<size_t>(count));
    std::vector<double> bucket_val(static_cast<size_t>(count));
    for (int64_t t = 0; t < count; ++t) {
        int r = rows[t], c = cols[t];
        int lo = std::min(r, c), hi = std::max(r, c);
        int64_t pos = cursor[lo]++;
        bucket_col[pos] = hi;
        bucket_val[pos] = vals[t];
    }

    UpperCsr m;
    m.n = n;
    m.row_ptr.assign(static_cast<size_t>(n) + 1, 0);
    m.diag_index.assign(static_cast<size_t>(n), -1);
    m.col.reserve(static_cast<size_t>(count));
    m.val.reserve(static_cast<size_t>(count));

    std::vector<int64_t> order;
    for (int r = 0; r < n; ++r) {
        m.row_ptr[r] = static_cast<int>(m.col.size());
        int64_t b = row_count[r], e = row_count[r + 1];
        order.resize(static_cast<size_t>(e - b));
        std::iota(order.begin(), order.end(), b);
        std::stable_sort(order.begin(), order.end(),
                         [&](int64_t x, int64_t y) { return bucket_col[x] < bucket_col[y]; });
        size_t q = 0;
        while (q < order.size()) {
            int c = bucket_col[order[q]];
            double sum = 0.0;
            for (; q < order.size() && bucket_col[order[q]] == c; ++q) sum += bucket_val[order[q]];
            if (std::fabs(sum) > kDropTolerance) {
                if (c == r) m.diag_index[r] = static_cast<int>(m.col.size());
                m.col.push_back(c);
                m.val.push_back(sum);
            }
        }
    }
    m.row_ptr[n] = static_cast<int>(m.col.size());
    if (m.col.size() > static_cast<size_t>(INT32_MAX))
        throw std::length_error("nonzero count exceeds the 32-bit index range");
    return m;
}

AdjacencyGraph adjacency_from_upper(int n, const int* row_ptr, const int* col) {
    AdjacencyGraph g;
    g.n = n;
    g.ptr.assign(static_cast<size_t>(n) + 1, 0);
    for (int r = 0; r < n; ++r)
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            if (c == r) continue;
            g.ptr[r + 1]++;
            g.ptr[c + 1]++;
        }
    for (int i = 0; i < n; ++i) g.ptr[i + 1] += g.ptr[i];
    g.adj.assign(static_cast<size_t>(g.ptr[n]), 0);
    std::vector<int> fill(g.ptr.begin(), g.ptr.end() - 1);
    for (int r = 0; r < n; ++r)
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            if (c == r) continue;
            g.adj[fill[r]++] = c;
            g.adj[fill[c]++] = r;
        }
    return g;
}

}  // namespace uchol
