// Shared device-side types for the UCHOL numeric phase on sm_103a.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace uchol_dev {

// Front of one supernode.  Rows are local indices 0..m-1 (the supernode's
// sorted row pattern); columns 0..w-1 are the pivots.  Storage is split in
// two column-major pieces:
//   panel   (m x w, leading dimension ldp)  — becomes the factor block,
//   contrib (t x t, leading dimension ldc)  — the Schur complement passed
//                                              to the parent, t = m - w.
// Element (i, j), i >= j, lives in panel[i + j*ldp] when j < w, otherwise in
// contrib[(i-w) + (j-w)*ldc].
struct SnDev {
    long long panel_off;    // element offset of the panel in the factor arena
    long long contrib_off;  // element offset of the block in the contribution arena (t > 0)
    int m, w, ldp, ldc;
    int first_col;          // first pivot column in elimination order
    int rows_off;           // offset of the row pattern in front_rows
    int rel_off;            // offset of the parent-local indices of the t trailing rows
    int parent;
};

// Scalars shared by every factorisation kernel of one call.
struct FactorCtl {
    double threshold;         // PivotTolerance * max|A_ii|
    double regularization;    // DiagonalRegularization * max|A_ii|
    int allow_regularization;
};

// Pivot statistics, updated with atomics (one update per front / task).
struct PivotStats {
    int regularized;
    int negative;
    int failed;                        // smallest rejected pivot index, INT_MAX if none
    int status;                        // non-zero: a bounded device wait expired
    unsigned long long min_bits;       // |d| as ordered bit pattern (non-negative doubles)
    unsigned long long max_bits;
    double scale;                      // max|A_ii| (1 when zero)
};

struct EaItem {        // one parent column gathered by one warp
    int parent;
    int pcol;
    int begin, end;    // range in the entry list
};
struct EaEntry {
    int child;
    int a;             // child trailing column
};

struct PanelTask {     // FP64 pivot block [j0, j0+nb) of front s plus TRSM of rows [row0, row0+rows)
    int s, j0, nb, row0, rows;
    int stage_row;     // first staging row of this task's rows (-1: no staging)
    int stage_k;       // K offset of column j0 inside the staging block
    int stage_zero_to; // > 0: also clear staging columns [stage_k + nb, stage_zero_to)
};

struct TileTask {      // C[i0:i0+TM, j0:j0+TN] -= sum_k A[i,k] B[j,k], k in [k0, k0+kn)
    int s, i0, j0, k0, kn;
    int a_row, b_row;  // staging rows of i0 and j0 (tensor-core path)
    int jend;          // column limit of this tile (does not cross the panel/contrib split)
};

__device__ __forceinline__ long long elem_offset(const SnDev& d, int i, int j, bool& in_panel) {
    in_panel = j < d.w;
    return in_panel ? d.panel_off + i + (long long)j * d.ldp
                    : d.contrib_off + (i - d.w) + (long long)(j - d.w) * d.ldc;
}

}  // namespace uchol_dev
