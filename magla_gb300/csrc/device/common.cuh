// Shared device-side types for the UCHOL numeric phase on sm_103a.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace uchol_dev {

#ifdef __CUDACC__
// Limits of the kernels' bounded waits, in ns (uchol_set_wait_limits changes them on the
// current device): the solves' waits on flags, counters and copies, and the tensor-core
// update's waits on its mbarriers.  On expiry a kernel records a status word and returns,
// and the host call reports UCHOL_TIMEOUT.
constexpr unsigned long long kDefaultSolveWaitNs = 1000000000ull;    // 1 s
constexpr unsigned long long kDefaultFactorWaitNs = 2000000000ull;   // 2 s
static __device__ unsigned long long g_solve_wait_ns = kDefaultSolveWaitNs;
static __device__ unsigned long long g_factor_wait_ns = kDefaultFactorWaitNs;
#endif

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

struct PanelTask {     // pivot block [j0, j0+nb) of front s, or its solve for rows [row0, row0+rows)
    int s, j0, nb, row0, rows;
    int stage;         // 1: also write the K-major staging copies W = L D and L (tensor-core path)
    int slot;          // mixed path: workspace slot of the block's inverse (index within its launch)
    int stage_zero_to; // > 0: also clear staging columns [j0 + nb, stage_zero_to) of these rows
};

// Staging region of a large front on the tensor-core path: m rows (front
// rows) x ld K columns (the supernode's columns, ld = w rounded up to 64),
// one region for W = L D (A operand) and one for L (B operand).
struct StageInfo {
    long long off;     // element offset of the front's region in each staging arena
    int ld;
    int map;           // index of the front's tensor-map pair
};

struct TileTask {      // C[i0:i0+TM, j0:j0+TN] -= sum_k A[i,k] B[j,k], k in [k0, k0+kn)
    int s, i0, j0, k0, kn;
    int a_row, b_row;  // staging rows of i0 and j0 (tensor-core path)
    int jend;          // column limit of this tile (does not cross the panel/contrib split)
};

// All tiles of one rank-kn update of front s: result columns [c0, cend),
// rows from each tile's first column down to m, lower triangle only.
// Column tiles are T wide and restart at the panel/contribution split w, so
// a tile never spans both storage pieces.  tile_begin is the prefix of tile
// counts inside one launch; a CTA decodes its tile from blockIdx.x.
struct UpdJob {
    long long tile_begin;
    int s, c0, cend, k0, kn;
    int stage_row0;    // staging row of front row c0 (tensor-core path), -1 otherwise
};

// Tiles of a region of nc column tiles whose first row tile count is R:
// column tile j holds R - j row tiles.
__host__ __device__ __forceinline__ long long region_tiles(long long nc, long long R) {
    return nc * R - nc * (nc - 1) / 2;
}

// Tensor-core update tiles: 128 columns of C (the MMA's M side, TMEM lanes) by
// 256 rows (its N side).  Column tile q of a job whose columns start h rows
// above the front's end holds R_q = ceil((h - 128 q) / 256) row tiles, which
// is R_0 - floor((q + delta) / 2) with delta = R_0 - R_1, so tile counts and
// their prefixes have closed forms.
constexpr int kTcCols = 128;
constexpr int kTcRows = 256;

// sum_{q < X} floor(q / 2)
__host__ __device__ __forceinline__ long long tc_half_sum(long long X) {
    const long long P = X >> 1;
    return P * (P - 1) + ((X & 1) ? P : 0);
}
// R_0 and delta of a job with columns from c0 in a front of m rows.
__host__ __device__ __forceinline__ void tc_col_shape(int c0, int m, int& R0, int& delta) {
    const int h = m - c0;
    R0 = (h + kTcRows - 1) / kTcRows;
    delta = (h > kTcCols && (h - kTcCols + kTcRows - 1) / kTcRows < R0) ? 1 : 0;
}
// Tiles of the first Q column tiles.
__host__ __device__ __forceinline__ long long tc_col_prefix(long long Q, int R0, int delta) {
    return Q * R0 - tc_half_sum(Q + delta);
}
// Tiles of a whole update job: result columns [c0, cend) of a front with m rows.
__host__ __device__ __forceinline__ long long tc_job_tiles(int c0, int cend, int m) {
    if (cend <= c0) return 0;
    int R0, delta;
    tc_col_shape(c0, m, R0, delta);
    return tc_col_prefix((cend - c0 + kTcCols - 1) / kTcCols, R0, delta);
}

// Tile t (0 <= t < tc_job_tiles) of the job with columns [c0, cend) of a front of m rows:
// first row i0, first column j0, column limit jend.  Column tiles go in groups of
// kTcGroup; inside a group, row tile r of every column that has one, then r + 1, so the
// CTAs working at the same time share operand rows.  Row tile r of a column group whose
// R_g is the first column's row-tile count is held by 2 (R_g - r) - delta of its columns
// (all g of them for the first F rows), a prefix since R_q does not grow with q.
constexpr int kTcGroup = 8;
__host__ __device__ __forceinline__ void tc_decode_tile(int c0, int cend, int m, long long t, int& i0, int& j0,
                                                        int& jend) {
    const int nc = (cend - c0 + kTcCols - 1) / kTcCols;
    int R0, delta;
    tc_col_shape(c0, m, R0, delta);
    int lo = 0, hi = (nc - 1) / kTcGroup;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tc_col_prefix((long long)mid * kTcGroup, R0, delta) <= t) lo = mid; else hi = mid - 1;
    }
    t -= tc_col_prefix((long long)lo * kTcGroup, R0, delta);
    const int g = kTcGroup < nc - lo * kTcGroup ? kTcGroup : nc - lo * kTcGroup;
    const int Rg = R0 - lo * (kTcGroup / 2);
    const int Fr = Rg - (g + delta + 1) / 2 + 1;
    const int F = Fr > 0 ? Fr : 0;   // rows every column of the group has
    int r, q;
    if (t < (long long)F * g) {
        r = (int)(t / g);
        q = (int)(t % g);
    } else {
        t -= (long long)F * g;
        r = F;
        q = 0;
        for (int guard = 0; guard < kTcGroup; ++guard, ++r) {
            const int cr = 2 * (Rg - r) - delta;
            const int c = cr < 0 ? 0 : (cr < g ? cr : g);
            if (t < c) {
                q = (int)t;
                break;
            }
            t -= c;
        }
    }
    j0 = c0 + (lo * kTcGroup + q) * kTcCols;
    i0 = j0 + r * kTcRows;
    jend = j0 + kTcCols < cend ? j0 + kTcCols : cend;
}

#ifdef __CUDACC__
// Decodes tile t of job J (front d) for tile edge T into (i0, j0, jend).
__device__ __forceinline__ void decode_tile(const UpdJob& J, const SnDev& d, int T, long long t, int& i0, int& j0,
                                            int& jend) {
    const int split = d.w;
    int base = J.c0, lim = J.cend;
    if (J.c0 < split && split < J.cend) {
        const int l1 = split - J.c0;
        const long long nc1 = (l1 + T - 1) / T;
        const long long R1 = (d.m - J.c0 + T - 1) / T;
        const long long n1 = region_tiles(nc1, R1);
        if (t < n1) {
            lim = split;
        } else {
            t -= n1;
            base = split;
        }
    }
    const long long R = (d.m - base + T - 1) / T;
    // largest j with j*R - j(j-1)/2 <= t
    const double b2 = 2.0 * (double)R + 1.0;
    long long j = (long long)floor((b2 - sqrt(b2 * b2 - 8.0 * (double)t)) * 0.5);
    if (j < 0) j = 0;
    while (j > 0 && region_tiles(j, R) > t) --j;
    while (region_tiles(j + 1, R) <= t) ++j;
    const long long it = t - region_tiles(j, R);
    j0 = base + (int)j * T;
    i0 = j0 + (int)it * T;
    jend = min(j0 + T, lim);
}

__device__ __forceinline__ int find_job(const UpdJob* __restrict__ jobs, int njobs, long long bid) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_begin <= bid) lo = mid; else hi = mid - 1;
    }
    return lo;
}
#endif  // __CUDACC__

#ifdef __CUDACC__
__device__ __forceinline__ long long elem_offset(const SnDev& d, int i, int j, bool& in_panel) {
    in_panel = j < d.w;
    return in_panel ? d.panel_off + i + (long long)j * d.ldp
                    : d.contrib_off + (i - d.w) + (long long)(j - d.w) * d.ldc;
}
#endif

}  // namespace uchol_dev
