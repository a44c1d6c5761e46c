/*
 * uchol_gpu.h — device numeric phase of the MAGLA UCHOL direct solver on one
 * GB300 (sm_103a): supernodal multifrontal U^T D U (= L D L^T) factorisation
 * of a symmetric upper-CSR matrix, forward / diagonal / backward solves, the
 * FP64 residual product and iterative refinement.
 *
 * This is the drop-in boundary: the managed MAGLA code keeps its public
 * classes and replaces two internal calls with these entry points.
 *
 *   uchol_symbolic_create   uploads the integer output of
 *       UtduSymbolicFactorization.Analyze (CAESolvers/UCHOL/UtduSymbolicFactorization.cs:240-295):
 *       the permutation, PermutedSymmetricPattern arrays
 *       (CAESolvers/UCHOL/PermutedSymmetricPattern.cs:41-72) and SupernodalStructure arrays
 *       (CAESolvers/UCHOL/SupernodalStructure.cs:44-96).  Done once per sparsity pattern.
 *   uchol_factorize         replaces SupernodalMultifrontalFactorizer.Factorize
 *       (CAESolvers/UCHOL/UtduNumericFactorization.cs:281-403), called from
 *       SymmetricUtduSolver.Factorize (CAESolvers/UCHOL/SymmetricUtduSolver.cs:95),
 *       including EnsureCompatible (UtduSymbolicFactorization.cs:306-319).
 *   uchol_factor_diagonal   UtduNumericFactorization.Diagonal (UtduNumericFactorization.cs:84).
 *   uchol_solve             replaces the body of UtduNumericFactorization.Solve
 *       (UtduNumericFactorization.cs:90-112), for nrhs columns at once.
 *   uchol_residual_norms    UtduNumericFactorization.ResidualNorm (UtduNumericFactorization.cs:222-234)
 *       and ResidualCalculator.CalculateResidualNorm (CAESolvers/ResidualCalculator.cs:5-20).
 *   uchol_solve_refined     a low-precision factor plus FP64-residual refinement;
 *       has no single counterpart in the reference (its solves are FP64 only).
 *
 * Conventions: every function returns a status (UCHOL_OK = 0, codes below);
 * uchol_last_error() gives the message of the calling thread's last failure.
 * Host pointers are only read during the call (the library copies them).
 * Handles are not thread-safe for concurrent factorisations of the same
 * symbolic handle; solves on one factor are serialised internally.
 */
#ifndef UCHOL_GPU_H
#define UCHOL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef UCHOL_OK
#define UCHOL_OK 0
#define UCHOL_BAD_ARG 1           /* ArgumentException / ArgumentNullException */
#define UCHOL_PATTERN_MISMATCH 2  /* ArgumentException from EnsureCompatible */
#define UCHOL_NOT_SPD 3           /* InvalidOperationException (pivot rejected, regularization off) */
#define UCHOL_OOM 4               /* device memory exhausted (checked before any arithmetic) */
#define UCHOL_TIMEOUT 5           /* a bounded device wait ran out */
#define UCHOL_CUDA_ERROR 6
#define UCHOL_TOO_DENSE 7         /* InvalidOperationException: front too large */
#define UCHOL_NO_CONVERGENCE 8    /* refinement did not reach its tolerance */
#define UCHOL_INTERNAL 9
#endif
#define UCHOL_OUT_OF_RANGE 10     /* IndexOutOfRangeException / ArgumentOutOfRangeException */
#define UCHOL_NOT_IN_PATTERN 11   /* InvalidOperationException: position absent from the sparse structure */

typedef struct uchol_symbolic_s* uchol_symbolic;
typedef struct uchol_factor_s* uchol_factor;

/* Arithmetic of the factorisation. */
#define UCHOL_PRECISION_FP64 0   /* FP64 fronts, FP64 Schur updates (plain form) */
#define UCHOL_PRECISION_TF32 1   /* FP32 fronts, Schur GEMMs on tcgen05 kind::tf32, FP32 accumulation */
#define UCHOL_PRECISION_BF16 2   /* FP32 fronts, Schur GEMMs on tcgen05 kind::f16 (BF16), FP32 accumulation */

/* Integer output of the symbolic phase; array lengths in brackets. */
typedef struct {
    int n;                        /* Size */
    int nnz;                      /* matrix NonZeroCount (upper half incl. diagonal) */
    const int* row_ptr;           /* [n+1]  upper-CSR pattern of A (SymmetricCSRMatrix.RowPointers) */
    const int* col;               /* [nnz]  SymmetricCSRMatrix.ColumnIndices */
    const int* permutation;       /* [n]    UtduSymbolicFactorization.Permutation */
    const int* diag_value_index;  /* [n]    PermutedSymmetricPattern.DiagonalValueIndices */
    const int* pattern_ptr;       /* [n+1]  PermutedSymmetricPattern.Pointers */
    const int* pattern_rows;      /* [pattern_ptr[n]] PermutedSymmetricPattern.Rows */
    const int* lower_start;       /* [n]    PermutedSymmetricPattern.LowerStart */
    const int* lower_value_ptr;   /* [n+1]  PermutedSymmetricPattern.LowerValuePointers */
    const int* lower_value_index; /* [lower_value_ptr[n]] PermutedSymmetricPattern.LowerValueIndices */
    int supernode_count;          /* SupernodalStructure.Count */
    const int* first_column;      /* [count+1] SupernodalStructure.FirstColumn */
    const int* parent;            /* [count]   SupernodalStructure.Parent */
    const int* child_ptr;         /* [count+1] SupernodalStructure.ChildPointers */
    const int* children;          /* [child_ptr[count]] SupernodalStructure.Children */
    const int* front_ptr;         /* [count+1] SupernodalStructure.PatternPointers */
    const int* front_rows;        /* [front_ptr[count]] SupernodalStructure.PatternRows */
} uchol_symbolic_desc;

/* UtduSolverOptions (CAESolvers/UCHOL/UtduSymbolicFactorization.cs:31-98), numeric part. */
typedef struct {
    int allow_diagonal_regularization;  /* AllowDiagonalRegularization (default 1) */
    double pivot_tolerance;             /* PivotTolerance (default 1e-13) */
    double diagonal_regularization;     /* DiagonalRegularization (default 1e-10) */
    int panel_width;                    /* PanelWidth, clamped to 4..64: pivot-block width of the FP64 path */
    int precision;                      /* UCHOL_PRECISION_* */
    int block_width;                    /* mixed paths: outer block, 64 or 128 columns (0 = 128) */
    int small_front_buckets;            /* bit b (b < 5): fronts with 32b < m <= 32(b+1) rows are factorised
                                           whole by one CTA in shared memory, the others by the blocked
                                           path; 0 = the default 0x7 (m <= 96).  uchol_autotune picks it. */
    int chain_merge_width;              /* device fronts: runs of supernodes in which each is the only child of
                                           the next are factorised as one front of at most this many columns
                                           when that adds at most 5% stored entries (exact zeros); the symbolic
                                           partition itself is unchanged.  0 = 2048, < 0 = one front per
                                           supernode. */
    int inverse_block_width;            /* solves: fronts of more than one solve block (128 columns mixed, 64
                                           FP64) and at most this many columns keep the inverse of their
                                           diagonal block's unit-lower triangle (built after each
                                           factorisation), so that their triangular solves are products
                                           instead of a chain of block solves.  0 = 2048, < 0 = off. */
    int64_t device_memory_budget;       /* > 0: a factorisation whose factor, contribution arena, staging,
                                           inverses and value copies (uchol_estimate_device_bytes) exceed
                                           this many bytes fails with UCHOL_OOM before any of it is
                                           allocated; 0 = no budget.  The reference's counterpart is its
                                           EstimatePeakBytes (UtduSymbolicFactorization.cs:203-219). */
    int split_min_kblocks;              /* mixed paths: a tensor-core update launch with fewer tiles than SMs is
                                           split in K (stream-K) only when its tiles have at least this many
                                           128-byte K blocks; 0 = 8, < 0 = never split.  uchol_autotune picks
                                           it. */
    int extend_add_overlap;             /* mixed paths: the extend-add into the contribution columns of the
                                           large fronts of a level runs on a second stream, beside the level's
                                           outer blocks, and is joined before the level's contribution update;
                                           0 = on, < 0 = off (one stream). */
    double chain_merge_fill;            /* device fronts from supernode chains: the largest relative growth
                                           of the stored entries a grouping may cost; 0 = 0.05. */
} uchol_options;

/* Pivot statistics (UtduNumericFactorization.cs:57-84) and timings. */
typedef struct {
    int regularized_pivot_count;
    int negative_pivot_count;
    double smallest_pivot_magnitude;
    double largest_pivot_magnitude;
    int failed_pivot;       /* elimination-order index of a rejected pivot (strict mode), else -1 */
    double factor_ms;       /* device time of the numeric factorisation (CUDA events) */
    int64_t device_bytes;   /* device memory held by the factor */
} uchol_factor_stats;

typedef struct {
    double tolerance;       /* target ||b - A x||_2 / ||b||_2 per column (e.g. 1e-10) */
    int max_iterations;     /* refinement steps after the first solve */
    int method;             /* 0 = automatic, 1 = classical refinement, 2 = factor-preconditioned CG */
} uchol_refine_options;

typedef struct {
    int iterations;             /* refinement steps taken (max over columns) */
    double relative_residual;   /* final max over columns of ||b - A x|| / ||b|| (FP64) */
    double initial_relative_residual;
    double solve_ms;            /* device time of the whole solve / refinement */
} uchol_refine_stats;

void uchol_default_options(uchol_options* o);

int uchol_symbolic_create(const uchol_symbolic_desc* desc, uchol_symbolic* out);
int uchol_symbolic_destroy(uchol_symbolic s);
/* Streams: all work of a symbolic handle and its factors runs on this CUDA stream
 * (cudaStream_t passed as void*; NULL = a private stream created by the library). */
int uchol_symbolic_set_stream(uchol_symbolic s, void* stream);

/* Numeric factorisation from host values [nnz] (SymmetricCSRMatrix.Values order). */
int uchol_factorize(uchol_symbolic s, int n, int nnz, const double* values, const uchol_options* opts,
                    uchol_factor* out, uchol_factor_stats* stats);
/* Same with the values already resident in device memory. */
int uchol_factorize_device(uchol_symbolic s, int n, int nnz, const double* d_values, const uchol_options* opts,
                           uchol_factor* out, uchol_factor_stats* stats);
/* Refactorise an existing factor in place with new values (same pattern, same options). */
int uchol_refactorize(uchol_factor f, const double* values, int on_device, uchol_factor_stats* stats);
int uchol_factor_destroy(uchol_factor f);

int uchol_factor_diagonal(uchol_factor f, double* out_n);
int uchol_factor_get_stats(uchol_factor f, uchol_factor_stats* stats);

/* X = A^-1 B for nrhs columns (column-major, leading dimension ld >= n), host
 * buffers, original equation order; one pass of the factor (no refinement). */
int uchol_solve(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx);
/* Device-buffer variant. */
int uchol_solve_device(uchol_factor f, int n, int nrhs, const double* d_b, int ldb, double* d_x, int ldx);
/* Solve with FP64-residual refinement against the factorised matrix. */
int uchol_solve_refined(uchol_factor f, int n, int nrhs, const double* b, int ldb, double* x, int ldx,
                        const uchol_refine_options* ro, uchol_refine_stats* rs);
int uchol_solve_refined_device(uchol_factor f, int n, int nrhs, const double* d_b, int ldb, double* d_x, int ldx,
                               const uchol_refine_options* ro, uchol_refine_stats* rs);

/* ||b_j - A x_j||_2 for each column j with the FP64 symmetric product of the
 * factorised values (host buffers); out_norms[nrhs]. */
int uchol_residual_norms(uchol_factor f, int n, int nrhs, const double* b, int ldb, const double* x, int ldx,
                         double* out_norms);

#define UCHOL_SOLVE_KINDS 14

/* Device-time of the last call on the handle's stream, per phase. */
typedef struct {
    double pivot_block_ms, extend_add_ms, small_fronts_ms, panel_ms, schur_ms, total_ms;  /* filled when UCHOL_PHASE_TIMES is set */
    int launches;            /* kernel launches of the last factorisation */
    double schur_tensor_flops;   /* algorithmic flops of the tensor-core Schur updates (lower triangle) */
    double schur_tensor_ms;      /* their device time (UCHOL_PHASE_TIMES) */
    int schur_tensor_launches;
    /* Triangular solves (filled by a solve made while phase timing is on; that solve
     * launches its kernels directly instead of replaying its graph).  Index: 0 forward
     * gather, 1 forward single-block fronts, 2 forward level kernels, 3 backward gather,
     * 4 backward column dots, 5 backward single-block fronts, 6 backward level kernels,
     * 7 forward trailing rows of single-block fronts, 8 backward partial-sum reductions,
     * 9-13 inverse fronts: forward diagonal, forward trailing rows, backward partial sums,
     * backward diagonal, backward partial-sum reductions. */
    double solve_kind_ms[UCHOL_SOLVE_KINDS];
    double solve_total_ms;       /* sum over the solve's launches */
    int solve_launches;
} uchol_phase_times;
int uchol_factor_phase_times(uchol_factor f, uchol_phase_times* t);

/* Autotuner: per front-size bucket, the kernel that factorises the fronts (one CTA with
 * the whole front in shared memory, or the blocked path); on the mixed paths the
 * outer-block width (64 or 128 columns); the widest device front grouped from a supernode
 * chain (512, 1024, 2048 columns or none); and on the mixed paths the stream-K threshold of
 * the tensor-core updates (4, 8, 16 K blocks or never).  uchol_autotune times graph-replayed
 * refactorisations of these values for each candidate: the default first, then one
 * bucket toggled at a time from the largest down, each change kept when it is faster,
 * then the other block width, the merge widths and the thresholds in the same way.  It writes the fastest options to *best (the base options
 * with small_front_buckets and block_width set) and a report.  Every candidate builds its
 * own factor (device memory of one factorisation at a time).  No counterpart in the
 * reference, which has one CPU kernel per operation; the device has several shapes and
 * the right one depends on the pattern's front sizes. */
typedef struct {
    int candidates;              /* configurations timed (failed ones count, with no time) */
    double default_ms;           /* refactorisation time of the default configuration */
    double best_ms;              /* of the chosen configuration */
    int small_front_buckets;     /* chosen bucket mask */
    int block_width;             /* chosen outer-block width (mixed paths; 0 on the FP64 path) */
    int chain_merge_width;       /* chosen chain_merge_width (0 = the default, 2048) */
    int split_min_kblocks;       /* chosen split_min_kblocks (0 = the default, 8) */
} uchol_autotune_report;
int uchol_autotune(uchol_symbolic s, int n, int nnz, const double* values, const uchol_options* base,
                   uchol_options* best, uchol_autotune_report* report);

/* Device memory a factorisation with these options will reserve, computed on
 * the host from the symbolic arrays alone (no GPU needed): factor panels,
 * the planned contribution arena and the tensor-core operand staging (with
 * the K-split workspace of the tensor-core updates, 40 MB for a 152-SM GPU).
 * With opts->device_memory_budget > 0 it returns UCHOL_OOM when the whole
 * reservation (also the inverses and the value copies) exceeds the budget.
 * Counterpart of UtduSymbolicFactorization.EstimatePeakBytes
 * (CAESolvers/UCHOL/UtduSymbolicFactorization.cs:203-219). */
int uchol_estimate_device_bytes(const uchol_symbolic_desc* desc, const uchol_options* opts, int64_t* factor_bytes,
                                int64_t* contribution_bytes, int64_t* staging_bytes, int* levels, int* launches);

/* Residual norms without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory while
 * they solve — an application that has reserved all device memory for its
 * own pool, a caller recording into a CUDA stream capture, or a loop that
 * must not take the synchronisation of cudaMalloc.  It computes
 * out[j] = ||b_j - A x_j||_2 for the symmetric matrix given by its upper
 * triangle (SymmetricCSRMatrix layout: d_row_ptr [n+1], d_col and d_values
 * [nnz]), with every buffer in device memory and supplied by the caller
 * (d_norms: nrhs doubles).  Its only scratch is a static device array of
 * 2^20 doubles (8 MiB, held on every device that loads the library until
 * exit): n * nrhs + 128 * nrhs must not exceed 2^20 and nrhs must not exceed
 * 64, otherwise UCHOL_BAD_ARG.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture; so is the first call after a device reset or
 * under another context, which looks the address up again.  All calls share the array: calls that overlap
 * on the GPU (other streams, other threads) race and must be serialised by
 * the caller.  Work is queued on `stream` (cudaStream_t, NULL = default);
 * results are valid once that stream has completed.  The mirrored half of
 * the product is accumulated with atomics, so results can differ from call
 * to call in the last bits. */
int uchol_residual_norms_static(int n, int nnz, int nrhs, const int* d_row_ptr, const int* d_col,
                                const double* d_values, const double* d_b, int ldb, const double* d_x, int ldx,
                                double* d_norms, void* stream);
const char* uchol_residual_norms_static_error(void);

/* Bounded waits of the kernels, in milliseconds, on the current device: waits of the
 * triangular solves (default 1000) and of the tensor-core Schur update (default 2000);
 * a value <= 0 restores the default.  An expired wait makes the call report UCHOL_TIMEOUT
 * with the device context still usable.  No counterpart in the reference (CPU threads). */
int uchol_set_wait_limits(double solve_ms, double factor_ms);

/* Failure check of the bounded waits: runs the factor's first level-solve launch (forward)
 * whose front has at least three diagonal blocks with its bulk CTAs withheld, so that a
 * chain waits on a progress counter that is never published, under a solve wait limit of
 * wait_ms.  Returns UCHOL_TIMEOUT when the wait expired, as designed, and leaves the factor
 * usable; UCHOL_BAD_ARG when the factor has no such launch (use inverse_block_width < 0 and
 * a front wider than three solve blocks).  No counterpart in the reference. */
int uchol_check_solve_wait(uchol_factor f, double wait_ms);

/* Kernel checks: one launch of a factorisation kernel of the mixed path on caller data
 * (host buffers), so that tests can compare each kernel with an FP64 computation on the
 * same operands.  No counterpart in the reference, whose numeric phase is one CPU routine.
 *
 * uchol_check_schur_update: the tensor-core Schur update (k_tc_gemm) of one job,
 * C[rows, cols] -= W[rows, kbeg:kbeg+kn] L[cols, kbeg:kbeg+kn]^T over the lower triangle of
 * result columns [c0, cend) (all in the panel, c < w, or all in the contribution block) of
 * a front of m rows and w columns.  front / front_out: column-major m x m (lower triangle);
 * w_op, l_op: row-major m x ld FP32 operands (ld a multiple of 64; BF16 rounds them to
 * nearest even first); K runs in whole 128-byte blocks, so the operand columns from kbeg + kn
 * to the end of its block must be zero (as the factorisation's staging copies are).  max_ctas > 0 caps the grid, which decides whether the launch is split
 * in K (stream-K).  Outputs the tile count and whether the launch was split. */
int uchol_check_schur_update(int bf16, int m, int w, int c0, int cend, int kbeg, int kn, const float* front,
                             const float* w_op, const float* l_op, int ld, int max_ctas, float* front_out,
                             int64_t* tiles_out, int* split_out);
/* uchol_check_diag_panel: the outer block of the mixed path (k_diag_block + k_panel_solve) on
 * the first nb <= 128 columns of an m-row front: front, l_out column-major m x nb (l_out: unit
 * L11 and L21), d_out the nb FP64 pivots, w_stage_out (optional) the staged W = L D rows,
 * column-major m x nb (rows >= nb); counts_out = {regularized, negative, failed column or -1}
 * under the pivot rule !(d > threshold) with the given regularization value. */
int uchol_check_diag_panel(int m, int nb, const float* front, double threshold, double regularization,
                           int allow_regularization, float* l_out, double* d_out, float* w_stage_out,
                           int* counts_out);

/* ---- Device-resident matrix values ------------------------------------
 * A uchol_dmatrix holds a SymmetricCSRMatrix on the device: its upper-triangle
 * structure (row_ptr [n+1], col [nnz], ascending columns, row <= col, as
 * CAESolvers/SymmetricCSRMatrix.cs:373-390 exposes it) and its values [nnz].
 * The values are refreshed on the device by the reference's container
 * operations and fed to a refactorisation without a host round trip:
 *   ClearValues   (SymmetricCSRMatrix.cs:113-116)  uchol_dmatrix_clear_values
 *   AccumulateAt  (SymmetricCSRMatrix.cs:98-110)   uchol_accumulate over a planned item list
 *   LineCross     (SymmetricCSRMatrix.cs:125-167)  uchol_line_cross over a planned index list
 *   Multiply      (SymmetricCSRMatrix.cs:293-324)  uchol_dmatrix_multiply
 * Work is queued on the handle's stream (`stream`, NULL = a stream of its own);
 * entry points with on_device = 0 take host buffers and return after the stream
 * has completed, those with on_device = 1 take device buffers and return at once.
 * A plan resolves each listed position on the host once (the errors of the
 * reference's calls are reported when it is built); applying it is a fixed set
 * of launches whose results equal the reference's sequential calls bit for bit. */
typedef struct uchol_dmatrix_s* uchol_dmatrix;
typedef struct uchol_values_plan_s* uchol_values_plan;

/* values: host array [nnz] or NULL (zeros).  UCHOL_BAD_ARG for a structure that is not
 * an upper-triangle CSR with strictly ascending columns. */
int uchol_dmatrix_create(int n, int nnz, const int* row_ptr, const int* col, const double* values, void* stream,
                         uchol_dmatrix* out);
int uchol_dmatrix_destroy(uchol_dmatrix m);
int uchol_dmatrix_set_stream(uchol_dmatrix m, void* stream);
/* The device array of the values (owned by the handle; valid until it is destroyed). */
int uchol_dmatrix_values(uchol_dmatrix m, double** d_values);
int uchol_dmatrix_set_values(uchol_dmatrix m, const double* values, int on_device);
int uchol_dmatrix_get_values(uchol_dmatrix m, double* out, int on_device);
int uchol_dmatrix_clear_values(uchol_dmatrix m);
/* AccumulateAt(rows[i], cols[i], item_i) for i = 0..count-1, in order: positions are
 * normalised to (min, max); UCHOL_OUT_OF_RANGE for an index outside [0, n)
 * (IndexOutOfRangeException), UCHOL_NOT_IN_PATTERN for a position absent from the
 * structure (InvalidOperationException).  Several items may name one position: it
 * receives their values in list order. */
int uchol_accumulate_plan_create(uchol_dmatrix m, int count, const int* rows, const int* cols,
                                 uchol_values_plan* out);
/* values[pos_i] += items[i] (items: count values, host or device). */
int uchol_accumulate(uchol_dmatrix m, uchol_values_plan p, const double* items, int on_device);
/* LineCross(rhs, prescribed[t], indices[t]) for t = 0..count-1, in order:
 * UCHOL_OUT_OF_RANGE for an index outside [0, n) (ArgumentOutOfRangeException),
 * UCHOL_NOT_IN_PATTERN for an index whose diagonal is absent. */
int uchol_line_cross_plan_create(uchol_dmatrix m, int count, const int* indices, uchol_values_plan* out);
/* rhs: nrhs columns of n (leading dimension ldr); prescribed: nrhs columns of count
 * (leading dimension ldp), column j holding the values of rhs column j.  Every column
 * receives what the list of calls does to one right-hand side of the matrix as it was
 * before this call; the values are then those after the list.  nrhs = 0 changes the
 * values only. */
int uchol_line_cross(uchol_dmatrix m, uchol_values_plan p, double* rhs, int ldr, int nrhs, const double* prescribed,
                     int ldp, int on_device);
/* Plans and their matrix may be destroyed in either order. */
int uchol_values_plan_destroy(uchol_values_plan p);
/* y = A x in FP64 (nrhs columns). */
int uchol_dmatrix_multiply(uchol_dmatrix m, int nrhs, const double* x, int ldx, double* y, int ldy, int on_device);

/* Jacobi-preconditioned conjugate gradients on the device
 * (CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs:78-165, JacobiPreconditioner.cs:12-57):
 * x0 = the initial guess or 0; stop when ||b - A x_k|| <= tolerance * ||b|| (||b|| = 0: 1);
 * at most max_iterations steps (0: n).  Each column iterates on its own.  UCHOL_NOT_SPD for
 * a diagonal entry that is zero, absent, not finite or within pivot_tolerance of zero (only
 * when a step is needed) and for p^T A p <= 0; UCHOL_OUT_OF_RANGE for a negative tolerance
 * or iteration limit.  Not converging is not an error: results[j].converged = 0. */
typedef struct {
    double relative_tolerance;   /* RelativeTolerance, default 1e-8 */
    int max_iterations;          /* MaxIterations, default 0 (= n) */
    int use_preconditioner;      /* UsePreconditioner, default 1 */
    int use_initial_guess;       /* 1: x holds the initial guess on entry */
    double pivot_tolerance;      /* JacobiPreconditioner pivotTolerance, default 1e-300 */
} uchol_cg_options;
typedef struct {
    int iterations;
    int converged;
    double residual_norm;        /* ||b - A x|| of the iteration's recurrence */
    double relative_residual;
    double ms;                   /* whole call, device time */
} uchol_cg_result;
void uchol_default_cg_options(uchol_cg_options* o);
int uchol_jacobi_pcg(uchol_dmatrix m, int nrhs, const double* b, int ldb, double* x, int ldx, int on_device,
                     const uchol_cg_options* opts, uchol_cg_result* results);

/* Refactorise f with the values of m (same structure as f's symbolic factorisation,
 * else UCHOL_PATTERN_MISMATCH).  The factorisation's stream waits for the work queued on
 * m's stream; the values do not leave the device. */
int uchol_refactorize_dmatrix(uchol_factor f, uchol_dmatrix m, uchol_factor_stats* stats);

/* Plan check (host only, no GPU needed): builds the execution plan of `desc` for the options
 * and an SM count (0 = unknown) and verifies the invariants its launches rely on (every
 * received column assembled once, side-stream launches joined, solve chunks tiling their
 * rows and blocks with distinct partial slots).  UCHOL_INTERNAL with the violated invariant
 * in uchol_last_error.  counts (optional, 5 ints): extend-add items, side-stream launches,
 * inverse-diagonal rows split in chunks, backward row chunks, forward trailing-row chunks.
 * No counterpart in the reference. */
int uchol_check_plan(const uchol_symbolic_desc* desc, const uchol_options* opts, int sms, int* counts);

/* Number of kernel launches this library has issued since it was loaded. */
int64_t uchol_kernel_launches(void);
/* Per-phase device timing of factorisations (one CUDA event pair per launch);
 * also enabled by the environment variable UCHOL_PHASE_TIMES. */
void uchol_set_phase_timing(int on);

const char* uchol_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* UCHOL_GPU_H */
