// C-ABI of the host half (include/uchol_host.h).
#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

#include "../../../include/uchol_host.h"
#include "generators.hpp"
#include "symbolic.hpp"

struct uchol_csr_s {
    uchol::UpperCsr m;
};
struct uchol_analysis_s {
    uchol::Symbolic s;
};

namespace {
thread_local std::string g_error;

template <class F>
int guarded(F&& f) {
    try {
        f();
        g_error.clear();
        return UCHOL_OK;
    } catch (const std::out_of_range& e) {
        g_error = e.what();
        return UCHOL_BAD_ARG;
    } catch (const std::invalid_argument& e) {
        g_error = e.what();
        return UCHOL_BAD_ARG;
    } catch (const std::length_error& e) {
        g_error = e.what();
        return UCHOL_TOO_DENSE;
    } catch (const std::bad_alloc&) {
        g_error = "host allocation failed";
        return UCHOL_OOM;
    } catch (const std::exception& e) {
        g_error = e.what();
        return UCHOL_INTERNAL;
    }
}

template <class V>
void copy_vec(const V& v, int* out) {
    if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(int));
}
}  // namespace

extern "C" {

const char* uchol_host_last_error(void) { return g_error.c_str(); }

int uchol_csr_from_triplets(int n, int64_t count, const int* rows, const int* cols, const double* values,
                            uchol_csr* out) {
    return guarded([&] {
        if (!out || (count > 0 && (!rows || !cols || !values))) throw std::invalid_argument("null argument");
        if (count < 0) throw std::invalid_argument("negative triplet count");
        *out = new uchol_csr_s{uchol::csr_from_triplets(n, count, rows, cols, values)};
    });
}

int uchol_csr_grid(int nx, int ny, int nz, int dof, uchol_csr* out) {
    return guarded([&] {
        if (!out || nx < 1 || ny < 1 || nz < 1 || dof < 1) throw std::invalid_argument("bad grid arguments");
        *out = new uchol_csr_s{uchol::grid_matrix(nx, ny, nz, dof)};
    });
}

int uchol_csr_laplacian3d(int nx, int ny, int nz, uchol_csr* out) {
    return guarded([&] {
        if (!out || nx < 1 || ny < 1 || nz < 1) throw std::invalid_argument("bad grid arguments");
        *out = new uchol_csr_s{uchol::laplacian3d(nx, ny, nz)};
    });
}

int uchol_csr_laplacian2d(int n, int stencil, const double* shift, uchol_csr* out) {
    return guarded([&] {
        if (!out || n < 1 || (stencil != 5 && stencil != 9)) throw std::invalid_argument("bad 2D Laplacian arguments");
        *out = new uchol_csr_s{uchol::laplacian2d(n, stencil, shift)};
    });
}

int uchol_csr_elasticity(int ex, int ey, int ez, const double* youngs, double nu, int clamp_bottom,
                         double* body_load, uchol_csr* out) {
    return guarded([&] {
        if (!out || ex < 1 || ey < 1 || ez < 1 || !(nu > -1.0 && nu < 0.5))
            throw std::invalid_argument("bad elasticity arguments");
        auto p = uchol::elasticity_q1(ex, ey, ez, youngs, nu, clamp_bottom != 0);
        if (body_load) {
            for (int idx : p.clamped) p.body_load[idx] = 0.0;
            std::memcpy(body_load, p.body_load.data(), p.body_load.size() * sizeof(double));
        }
        *out = new uchol_csr_s{std::move(p.matrix)};
    });
}

int uchol_csr_shape(uchol_csr m, int* n, int* nnz) {
    return guarded([&] {
        if (!m) throw std::invalid_argument("null matrix");
        if (n) *n = m->m.n;
        if (nnz) *nnz = m->m.nnz();
    });
}

int uchol_csr_copy(uchol_csr m, int* row_ptr, int* col, double* values, int* diag_index) {
    return guarded([&] {
        if (!m) throw std::invalid_argument("null matrix");
        if (row_ptr) copy_vec(m->m.row_ptr, row_ptr);
        if (col) copy_vec(m->m.col, col);
        if (values && !m->m.val.empty()) std::memcpy(values, m->m.val.data(), m->m.val.size() * sizeof(double));
        if (diag_index) copy_vec(m->m.diag_index, diag_index);
    });
}

void uchol_csr_destroy(uchol_csr m) { delete m; }

int uchol_analyze(int n, int nnz, const int* row_ptr, const int* col, int ordering, int amalgamation_limit,
                  uchol_analysis* out) {
    return guarded([&] {
        if (!out || n < 0 || nnz < 0 || (n > 0 && !row_ptr) || (nnz > 0 && !col))
            throw std::invalid_argument("null or negative argument");
        if (ordering != UCHOL_ORDERING_NATURAL && ordering != UCHOL_ORDERING_AMD)
            throw std::invalid_argument("unknown ordering");
        if (n > 0 && (row_ptr[0] != 0 || row_ptr[n] != nnz)) throw std::invalid_argument("row pointers do not match nnz");
        for (int r = 0; r < n; ++r) {
            if (row_ptr[r + 1] < row_ptr[r]) throw std::invalid_argument("row pointers are not monotone");
            for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
                if (col[k] < r || col[k] >= n) throw std::out_of_range("column index outside the upper triangle");
                if (k > row_ptr[r] && col[k] <= col[k - 1]) throw std::invalid_argument("columns not strictly ascending");
            }
        }
        auto a = new uchol_analysis_s;
        try {
            a->s = uchol::analyze(n, row_ptr, col, nnz,
                                  ordering == UCHOL_ORDERING_AMD ? uchol::Ordering::ApproximateMinimumDegree
                                                                 : uchol::Ordering::Natural,
                                  amalgamation_limit);
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

int uchol_analysis_get_info(uchol_analysis a, uchol_analysis_info* info) {
    return guarded([&] {
        if (!a || !info) throw std::invalid_argument("null argument");
        const auto& s = a->s;
        info->n = s.n;
        info->nnz = s.matrix_nonzero_count;
        info->supernode_count = s.supernodes.count();
        info->max_front_size = s.supernodes.max_front_size;
        info->max_supernode_width = s.supernodes.max_supernode_width;
        info->pattern_entries = static_cast<int>(s.pattern.rows.size());
        info->lower_entries = static_cast<int>(s.pattern.lower_value_index.size());
        info->front_row_entries = static_cast<int>(s.supernodes.pattern_rows.size());
        info->child_entries = static_cast<int>(s.supernodes.children.size());
        info->slab_count = static_cast<int>(s.layout.slab_lengths.size());
        info->factor_entry_count = s.supernodes.factor_entry_count;
        info->strict_factor_nonzero_count = s.strict_factor_nonzero_count;
        info->factor_operation_count = s.supernodes.factor_operation_count;
        info->peak_contribution_entries = s.supernodes.peak_contribution_entries;
    });
}

int uchol_analysis_copy(uchol_analysis a, int which, int* out) {
    return guarded([&] {
        if (!a || !out) throw std::invalid_argument("null argument");
        const auto& s = a->s;
        switch (which) {
            case UCHOL_A_PERMUTATION: copy_vec(s.permutation, out); break;
            case UCHOL_A_INVERSE_PERMUTATION: copy_vec(s.inverse_permutation, out); break;
            case UCHOL_A_PATTERN_PTR: copy_vec(s.pattern.ptr, out); break;
            case UCHOL_A_PATTERN_ROWS: copy_vec(s.pattern.rows, out); break;
            case UCHOL_A_LOWER_START: copy_vec(s.pattern.lower_start, out); break;
            case UCHOL_A_LOWER_VALUE_PTR: copy_vec(s.pattern.lower_value_ptr, out); break;
            case UCHOL_A_LOWER_VALUE_INDEX: copy_vec(s.pattern.lower_value_index, out); break;
            case UCHOL_A_DIAG_VALUE_INDEX: copy_vec(s.pattern.diag_value_index, out); break;
            case UCHOL_A_ETREE_PARENT: copy_vec(s.etree_parent, out); break;
            case UCHOL_A_COLUMN_COUNTS: copy_vec(s.column_counts, out); break;
            case UCHOL_A_FIRST_COLUMN: copy_vec(s.supernodes.first_column, out); break;
            case UCHOL_A_SUPERNODE_OF: copy_vec(s.supernodes.supernode_of, out); break;
            case UCHOL_A_SN_PARENT: copy_vec(s.supernodes.parent, out); break;
            case UCHOL_A_CHILD_PTR: copy_vec(s.supernodes.child_ptr, out); break;
            case UCHOL_A_CHILDREN: copy_vec(s.supernodes.children, out); break;
            case UCHOL_A_FRONT_PTR: copy_vec(s.supernodes.pattern_ptr, out); break;
            case UCHOL_A_FRONT_ROWS: copy_vec(s.supernodes.pattern_rows, out); break;
            case UCHOL_A_SLAB_INDEX: copy_vec(s.layout.slab_index, out); break;
            case UCHOL_A_SLAB_OFFSET: copy_vec(s.layout.slab_offset, out); break;
            case UCHOL_A_SLAB_LENGTHS: copy_vec(s.layout.slab_lengths, out); break;
            default: throw std::invalid_argument("unknown array selector");
        }
    });
}

void uchol_analysis_destroy(uchol_analysis a) { delete a; }

// Validates one upper-CSR system of a batch.
static void check_upper(int n, const int* row_ptr, const int* col) {
    if (n < 0 || (n > 0 && (!row_ptr || !col))) throw std::invalid_argument("null or negative argument in a batch system");
    if (n > 0 && row_ptr[0] != 0) throw std::invalid_argument("row pointers of a batch system do not start at 0");
    for (int r = 0; r < n; ++r) {
        if (row_ptr[r + 1] < row_ptr[r]) throw std::invalid_argument("row pointers are not monotone");
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            if (col[k] < r || col[k] >= n) throw std::out_of_range("column index outside the upper triangle");
            if (k > row_ptr[r] && col[k] <= col[k - 1]) throw std::invalid_argument("columns not strictly ascending");
        }
    }
}

int uchol_batch_csr(int count, const int* sizes, const int* const* row_ptrs, const int* const* cols,
                    const double* const* values, uchol_csr* out) {
    return guarded([&] {
        if (!out || count < 0 || (count > 0 && (!sizes || !row_ptrs || !cols || !values)))
            throw std::invalid_argument("null or negative argument");
        uchol::UpperCsr m;
        int64_t n = 0, nnz = 0;
        for (int q = 0; q < count; ++q) {
            check_upper(sizes[q], row_ptrs[q], cols[q]);
            if (sizes[q] > 0 && !values[q]) throw std::invalid_argument("null values of a batch system");
            n += sizes[q];
            nnz += sizes[q] > 0 ? row_ptrs[q][sizes[q]] : 0;
        }
        if (n > INT32_MAX || nnz > INT32_MAX) throw std::length_error("the batch exceeds the 32-bit index range");
        m.n = (int)n;
        m.row_ptr.reserve(n + 1);
        m.row_ptr.push_back(0);
        m.col.reserve(nnz);
        m.val.reserve(nnz);
        m.diag_index.assign(n, -1);
        int off = 0;
        for (int q = 0; q < count; ++q) {
            const int nq = sizes[q];
            for (int r = 0; r < nq; ++r) {
                for (int k = row_ptrs[q][r]; k < row_ptrs[q][r + 1]; ++k) {
                    if (cols[q][k] == r) m.diag_index[off + r] = (int)m.col.size();
                    m.col.push_back(off + cols[q][k]);
                    m.val.push_back(values[q][k]);
                }
                m.row_ptr.push_back((int)m.col.size());
            }
            off += nq;
        }
        *out = new uchol_csr_s{std::move(m)};
    });
}

int uchol_batch_analyze(int count, const int* sizes, const int* const* row_ptrs, const int* const* cols, int ordering,
                        int amalgamation_limit, uchol_analysis* out) {
    return guarded([&] {
        if (!out || count < 0 || (count > 0 && (!sizes || !row_ptrs || !cols)))
            throw std::invalid_argument("null or negative argument");
        if (ordering != UCHOL_ORDERING_NATURAL && ordering != UCHOL_ORDERING_AMD)
            throw std::invalid_argument("unknown ordering");
        int64_t n = 0, nnz = 0;
        for (int q = 0; q < count; ++q) {
            check_upper(sizes[q], row_ptrs[q], cols[q]);
            n += sizes[q];
            nnz += sizes[q] > 0 ? row_ptrs[q][sizes[q]] : 0;
        }
        if (n > INT32_MAX || nnz > INT32_MAX) throw std::length_error("the batch exceeds the 32-bit index range");
        // the union's pattern, and each system's own fill-reducing order shifted to its rows
        std::vector<int> rp, cl, order;
        rp.reserve(n + 1);
        rp.push_back(0);
        cl.reserve(nnz);
        order.reserve(n);
        int off = 0;
        for (int q = 0; q < count; ++q) {
            const int nq = sizes[q];
            for (int r = 0; r < nq; ++r) {
                for (int k = row_ptrs[q][r]; k < row_ptrs[q][r + 1]; ++k) cl.push_back(off + cols[q][k]);
                rp.push_back((int)cl.size());
            }
            if (ordering == UCHOL_ORDERING_AMD) {
                auto p = uchol::amd_order(uchol::adjacency_from_upper(nq, row_ptrs[q], cols[q]));
                for (int v : p) order.push_back(off + v);
            } else {
                for (int v = 0; v < nq; ++v) order.push_back(off + v);
            }
            off += nq;
        }
        auto a = new uchol_analysis_s;
        try {
            a->s = uchol::analyze_ordered((int)n, rp.data(), cl.data(), (int)nnz, order, amalgamation_limit);
        } catch (...) {
            delete a;
            throw;
        }
        *out = a;
    });
}

int uchol_amd_order(int n, const int* row_ptr, const int* col, int* perm_out) {
    return guarded([&] {
        if (n < 0 || (n > 0 && (!row_ptr || !col || !perm_out))) throw std::invalid_argument("null argument");
        auto g = uchol::adjacency_from_upper(n, row_ptr, col);
        auto p = uchol::amd_order(g);
        copy_vec(p, perm_out);
    });
}

}  // extern "C"
