/*
 * uchol_host.h — host half of the UCHOL direct solver: matrix construction
 * and the symbolic phase (ordering, elimination tree, column counts,
 * supernodes).  In a MAGLA deployment this half stays the reference's own
 * C# code; this C++ restatement exists for hosts without a .NET runtime and
 * produces the same integer arrays, which are then handed unchanged to the
 * device library (uchol_gpu.h, uchol_symbolic_create).
 *
 * Reference interfaces replaced (paths within the MAGLA project):
 *   uchol_csr_from_triplets   CAESolvers/SymmetricCSRMatrix.cs:36-90 (COO constructor)
 *                             CAESolvers/SymmetricCSRMatrixBuilder.cs:22-51 (Build)
 *   uchol_analyze             CAESolvers/UCHOL/UtduSymbolicFactorization.cs:240-295 (Analyze)
 *   uchol_analysis_info       CAESolvers/UCHOL/UtduSymbolicFactorization.cs:127-234 (statistics)
 *   uchol_csr_grid            CAESolvers/UCHOL/UtduSolverBenchmark.cs:220-261 (BuildGridMatrix)
 *
 * Every function returns UCHOL_OK (0) or a non-zero status; the message of
 * the last failure on the calling thread is available from
 * uchol_host_last_error().
 */
#ifndef UCHOL_HOST_H
#define UCHOL_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct uchol_csr_s* uchol_csr;
typedef struct uchol_analysis_s* uchol_analysis;

/* Status codes shared with uchol_gpu.h. */
#define UCHOL_OK 0
#define UCHOL_BAD_ARG 1           /* ArgumentException / ArgumentNullException / out of range */
#define UCHOL_PATTERN_MISMATCH 2  /* ArgumentException from EnsureCompatible */
#define UCHOL_NOT_SPD 3           /* InvalidOperationException: pivot rejected, regularization off */
#define UCHOL_OOM 4
#define UCHOL_TIMEOUT 5           /* a bounded device wait ran out */
#define UCHOL_CUDA_ERROR 6
#define UCHOL_TOO_DENSE 7         /* InvalidOperationException: front/block too large */
#define UCHOL_NO_CONVERGENCE 8    /* refinement did not reach its tolerance */
#define UCHOL_INTERNAL 9          /* InvalidOperationException from an internal consistency check */

/* Orderings (CAESolvers/UCHOL/UtduSymbolicFactorization.cs:8-24). */
#define UCHOL_ORDERING_NATURAL 0
#define UCHOL_ORDERING_AMD 1

/* ---- matrices -------------------------------------------------------- */
int uchol_csr_from_triplets(int n, int64_t count, const int* rows, const int* cols, const double* values,
                            uchol_csr* out);
int uchol_csr_grid(int nx, int ny, int nz, int dof, uchol_csr* out);
int uchol_csr_laplacian3d(int nx, int ny, int nz, uchol_csr* out);
int uchol_csr_laplacian2d(int n, int stencil, const double* shift, uchol_csr* out);
/* Q1 hexahedral elasticity; youngs: ex*ey*ez moduli or NULL; body_load: out, 3*(ex+1)(ey+1)(ez+1) */
int uchol_csr_elasticity(int ex, int ey, int ez, const double* youngs, double nu, int clamp_bottom,
                         double* body_load, uchol_csr* out);
int uchol_csr_shape(uchol_csr m, int* n, int* nnz);
/* row_ptr: n+1, col: nnz, values: nnz, diag_index: n (any may be NULL) */
int uchol_csr_copy(uchol_csr m, int* row_ptr, int* col, double* values, int* diag_index);
void uchol_csr_destroy(uchol_csr m);

/* ---- symbolic phase --------------------------------------------------- */
int uchol_analyze(int n, int nnz, const int* row_ptr, const int* col, int ordering, int amalgamation_limit,
                  uchol_analysis* out);

typedef struct {
    int n;
    int nnz;                              /* MatrixNonZeroCount */
    int supernode_count;
    int max_front_size;
    int max_supernode_width;
    int pattern_entries;                  /* PermutedSymmetricPattern.Rows length */
    int lower_entries;                    /* LowerValueIndices length */
    int front_row_entries;                /* SupernodalStructure.PatternRows length */
    int child_entries;                    /* Children length */
    int slab_count;
    int64_t factor_entry_count;           /* FactorEntryCount */
    int64_t strict_factor_nonzero_count;  /* StrictFactorNonZeroCount */
    int64_t factor_operation_count;       /* FactorOperationCount */
    int64_t peak_contribution_entries;    /* PeakContributionEntries */
} uchol_analysis_info;

int uchol_analysis_get_info(uchol_analysis a, uchol_analysis_info* info);

/* Array selectors for uchol_analysis_copy (lengths in brackets). */
#define UCHOL_A_PERMUTATION 0          /* [n] */
#define UCHOL_A_INVERSE_PERMUTATION 1  /* [n] */
#define UCHOL_A_PATTERN_PTR 2          /* [n+1] */
#define UCHOL_A_PATTERN_ROWS 3         /* [pattern_entries] */
#define UCHOL_A_LOWER_START 4          /* [n] */
#define UCHOL_A_LOWER_VALUE_PTR 5      /* [n+1] */
#define UCHOL_A_LOWER_VALUE_INDEX 6    /* [lower_entries] */
#define UCHOL_A_DIAG_VALUE_INDEX 7     /* [n] */
#define UCHOL_A_ETREE_PARENT 8         /* [n] */
#define UCHOL_A_COLUMN_COUNTS 9        /* [n] */
#define UCHOL_A_FIRST_COLUMN 10        /* [supernode_count+1] */
#define UCHOL_A_SUPERNODE_OF 11        /* [n] */
#define UCHOL_A_SN_PARENT 12           /* [supernode_count] */
#define UCHOL_A_CHILD_PTR 13           /* [supernode_count+1] */
#define UCHOL_A_CHILDREN 14            /* [child_entries] */
#define UCHOL_A_FRONT_PTR 15           /* [supernode_count+1] */
#define UCHOL_A_FRONT_ROWS 16          /* [front_row_entries] */
#define UCHOL_A_SLAB_INDEX 17          /* [supernode_count] */
#define UCHOL_A_SLAB_OFFSET 18         /* [supernode_count] */
#define UCHOL_A_SLAB_LENGTHS 19        /* [slab_count] */

int uchol_analysis_copy(uchol_analysis a, int which, int* out);
void uchol_analysis_destroy(uchol_analysis a);

/* Individual symbolic steps, exposed for parity tests against the
 * reference's own unit tests (AMD permutation validity, etc.). */
/* Batches of independent systems (many small problems at once; no counterpart in the
 * reference, whose solvers take one SymmetricCSRMatrix per call): the block-diagonal
 * union of `count` upper-CSR systems, system q occupying rows and columns
 * [sum_{p<q} sizes[p], ...).  uchol_batch_csr builds the union matrix (values in the
 * systems' CSR order, concatenated).  uchol_batch_analyze orders every system on its
 * own (the reference's AMD or natural order, as UtduSymbolicFactorization.Analyze does
 * for one matrix) and analyses the union with that order: the elimination forest has
 * one tree per system, each with the supernodes of that system's own analysis, so one
 * numeric factorisation and one solve of the union treat every system in each launch. */
int uchol_batch_csr(int count, const int* sizes, const int* const* row_ptrs, const int* const* cols,
                    const double* const* values, uchol_csr* out);
int uchol_batch_analyze(int count, const int* sizes, const int* const* row_ptrs, const int* const* cols, int ordering,
                        int amalgamation_limit, uchol_analysis* out);

int uchol_amd_order(int n, const int* row_ptr, const int* col, int* perm_out);

const char* uchol_host_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* UCHOL_HOST_H */
