// Host half of the UCHOL solver: matrix construction semantics and the
// symbolic phase (fill-reducing ordering, elimination tree, column counts,
// supernode partition).  Every structure produced here is integer-only and
// must agree bit for bit with the reference implementation, so each routine
// keeps the reference's tie-breaking rules; the code itself is organised for
// this library (flat std::vector arrays that are handed to the device
// library unchanged).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace uchol {

// Upper-triangle CSR (row <= col), columns strictly ascending inside a row,
// so the diagonal, when present, is the first entry of its row.
// Mirrors CAESolvers/SymmetricCSRMatrix.cs:19-90.
struct UpperCsr {
    int n = 0;
    std::vector<int> row_ptr;     // n + 1
    std::vector<int> col;         // nnz
    std::vector<double> val;      // nnz
    std::vector<int> diag_index;  // n, -1 when the diagonal is structurally absent
    int nnz() const { return static_cast<int>(col.size()); }
};

// Builds the matrix from coordinate triplets: (row, col) is normalised to
// (min, max), duplicates are summed in input order, sums with
// |v| <= 1e-15 are dropped (SymmetricCSRMatrix.cs:29,36-90).
UpperCsr csr_from_triplets(int n, int64_t count, const int* rows, const int* cols, const double* vals);

// Undirected adjacency of the pattern without the diagonal
// (CAESolvers/AMD/SymmetricPatternGraph.cs:71-121).  Neighbour lists keep
// the reference's fill order (row-major sweep of the stored upper half).
struct AdjacencyGraph {
    int n = 0;
    std::vector<int> ptr;   // n + 1
    std::vector<int> adj;   // 2 * off-diagonal count
};
AdjacencyGraph adjacency_from_upper(int n, const int* row_ptr, const int* col);

// Approximate minimum degree ordering (CAESolvers/AMD/ApproximateMinimumDegreeOrdering.cs).
// Returns perm with perm[k] = original index eliminated k-th.
std::vector<int> amd_order(const AdjacencyGraph& g);

// Pattern of P^T A P (CAESolvers/UCHOL/PermutedSymmetricPattern.cs:81-184).
struct PermutedPattern {
    int n = 0;
    std::vector<int> ptr;                 // n + 1, full structure (both triangles, no diagonal)
    std::vector<int> rows;                // sorted ascending inside each column
    std::vector<int> lower_start;         // n, start of rows > j inside column j
    std::vector<int> lower_value_ptr;     // n + 1
    std::vector<int> lower_value_index;   // index into the CSR values for each lower entry
    std::vector<int> diag_value_index;    // n, -1 if absent
};
PermutedPattern permute_pattern(int n, const int* row_ptr, const int* col, const std::vector<int>& inverse_perm);

// Elimination tree and friends (CAESolvers/UCHOL/EliminationTree.cs).
std::vector<int> etree_build(int n, const std::vector<int>& ptr, const std::vector<int>& rows);
std::vector<int> etree_postorder(int n, const std::vector<int>& parent);
std::vector<int> etree_column_counts(int n, const std::vector<int>& ptr, const std::vector<int>& rows,
                                     const std::vector<int>& parent, const std::vector<int>& post);

// Supernode partition and assembly tree (CAESolvers/UCHOL/SupernodalStructure.cs).
struct Supernodes {
    int n = 0;
    std::vector<int> first_column;     // count + 1
    std::vector<int> supernode_of;     // n
    std::vector<int> parent;           // count, -1 for roots
    std::vector<int> child_ptr;        // count + 1
    std::vector<int> children;         // grouped by parent, ascending
    std::vector<int> pattern_ptr;      // count + 1
    std::vector<int> pattern_rows;     // sorted row lists; first width entries are the columns
    int64_t factor_entry_count = 0;
    int64_t factor_operation_count = 0;
    int max_front_size = 0;
    int max_supernode_width = 0;
    int64_t peak_contribution_entries = 0;

    int count() const { return static_cast<int>(first_column.size()) - 1; }
    int width(int s) const { return first_column[s + 1] - first_column[s]; }
    int front_size(int s) const { return pattern_ptr[s + 1] - pattern_ptr[s]; }
};
Supernodes build_supernodes(const PermutedPattern& pattern, const std::vector<int>& parent,
                            const std::vector<int>& column_counts, int amalgamation_limit);

// Slab packing of the factor blocks (CAESolvers/UCHOL/FactorStorageLayout.cs:55-103).
struct FactorLayout {
    std::vector<int> slab_index, slab_offset, block_length, slab_lengths;
};
FactorLayout build_layout(const Supernodes& sn);

enum class Ordering : int { Natural = 0, ApproximateMinimumDegree = 1 };

// Result of the symbolic phase (CAESolvers/UCHOL/UtduSymbolicFactorization.cs:109-295).
struct Symbolic {
    int n = 0;
    int matrix_nonzero_count = 0;
    std::vector<int> permutation;          // perm[k] = original index of the k-th eliminated equation
    std::vector<int> inverse_permutation;
    PermutedPattern pattern;
    Supernodes supernodes;
    std::vector<int> etree_parent;
    std::vector<int> column_counts;
    FactorLayout layout;
    int64_t strict_factor_nonzero_count = 0;
};

Symbolic analyze(int n, const int* row_ptr, const int* col, int nnz, Ordering ordering, int amalgamation_limit);
// The analysis from a given fill-reducing order (position -> original index), e.g. one AMD
// ordering per diagonal block of a block-diagonal system.
Symbolic analyze_ordered(int n, const int* row_ptr, const int* col, int nnz, const std::vector<int>& fill_reducing,
                         int amalgamation_limit);

}  // namespace uchol
