// Host-side execution plan of the device numeric phase: tree levels, memory
// layout of fronts, and the task lists every kernel launch consumes.  Built
// once per (symbolic pattern, block configuration) and reused by every
// factorisation and solve.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "common.cuh"

namespace uchol_dev {

constexpr int kSolveRowsPlan = 128;   // rows per panel-solve task (kSolveRows of the kernel)
constexpr int kTailRowsPlan = 1024;  // trailing rows per forward tail task (kTailRows of the kernel)
constexpr int kColRowsPlan = 2048;   // trailing rows per backward column-dot task (longer columns: partial sums)
constexpr int kInvColRowsPlan = 1024;   // trailing rows per backward partial-sum task of an inverse front
constexpr int kDefaultInvCols = 2048;   // widest front whose diagonal block is kept inverted for the solves
constexpr int kSuperBlocks = 4;       // tensor-core path: outer blocks per super-block of the own-column updates
constexpr int kDefaultMergeCols = 2048;   // widest device front made of a chain of supernodes (merge_chains)
constexpr int kInvDiagChunk = 2;         // inverse blocks per task of the inverse-front diagonal products

struct PlanConfig {
    int pivot_block = 32;     // FP64 pivot block (the reference's PanelWidth)
    int outer_block = 32;     // Schur-update block (== pivot_block on the FP64 path)
    int small_mask = 0x7;     // bit b: fronts with 32b < m <= 32(b+1) are factorised by one CTA in shared memory
    int tile = 64;            // SIMT tile edge (update kernels)
    bool tensor_core = false; // outer updates on tcgen05 from staged operands
    int solve_block = 64;     // column block of the triangular solves
    int inv_cols = 0;         // > 0: fronts of solve_block < w <= inv_cols columns keep the whole inverse of their
                              // unit-lower diagonal block, and their solves run without a block chain
    int merge_cols = 0;       // > 0: single-child chains of supernodes grouped into device fronts of at most
                              // this many columns (see merge_chains); 0: one device front per supernode
    double merge_fill = 0.05; // largest growth of the stored entries a grouping may cost
    bool side_extend_add = false;   // tensor-core path: the extend-add into the contribution columns of
                                    // large fronts runs on a second stream, beside the level's outer blocks
    int sms = 0;                    // > 0: the device's SM count (sizes the backward inverse-front chunks)
};

// Device fronts from the supernode partition: runs of supernodes in which each
// one is the only child of the next are grouped into one front, as long as the
// group stays within cfg.merge_cols columns and its lower-trapezoid entries
// exceed the members' own by at most cfg.merge_fill.  A group's rows are its
// columns followed by the last member's trailing rows (every earlier member's
// trailing rows outside the group are among them), so the group is a valid
// front of the same elimination order: the entries it adds are structural zeros
// that stay exactly zero, and its parent's front contains its trailing rows.
struct FrontStructure {
    int count = 0;
    std::vector<int> first_column, parent, child_ptr, children, front_ptr, front_rows;
    std::vector<int> group_of;   // per supernode: its device front
};
FrontStructure merge_chains(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                            const int* children, const int* front_ptr, const int* front_rows, int max_cols,
                            double max_fill);

// One kernel launch: a contiguous range of tasks in one of the task arrays.
struct Launch {
    enum Kind : int {
        ExtendAdd, SmallFronts, PivotBlock, Trsm, SimtUpdate, TcUpdate, DiagBlock, PanelSolve,
        KindCount
    } kind;
    int begin, count;   // task range
    long long tiles;    // update launches: total tiles (= grid size)
    int stream = 0;     // 0: main stream; 1: side stream, forked from the main stream at this point;
                        // 2: main stream after joining the side stream
};

struct SolveLaunch {
    enum Kind : int {
        FwdGather, FwdSolo, FwdLevel, BwdGather, BwdTail, BwdSolo, BwdLevel, FwdTail, BwdTailReduce,
        FwdInvDiag, FwdInvTail, BwdInvCols, BwdInvDiag, BwdInvReduce, KindCount
    } kind;
    int begin, count;   // tasks; level launches: the chains (one per front)
    int steps;          // level launches: most diagonal blocks of one front of the level
    int bulk_begin, bulk_count;   // level launches: the bulk chunks
    int progress_off;             // level launches: first progress counter of the bulk chunks
    long long chain_work, bulk_work;   // level launches: block solves and chunk updates (CTA split)
    int long_chains;                   // level launches: fronts of three or more diagonal blocks
    int ndiag;                         // level launches: bulk chunks [0, ndiag) are diagonal blocks
    long long diag_work;               // level launches: chunk updates of those
};

// Inverse fronts (cfg.inv_cols): the off-diagonal blocks (i, j), i > j, of the
// inverse of the unit-lower diagonal block, SB x SB column-major each, front s's
// at block index ob_s + i (i - 1) / 2 + j of the off-diagonal arena.  Tasks:
//   inversion            {s, i, j, ob_s, -, -, blk}: block (i, j) from the blocks
//                        (k, j), j <= k < i (launched by diagonal i - j);
//   FwdInvDiag           {s, i, nb, ob_s, slot0, nc, blk, j0, j1}: the part j0 <= j <= j1 of
//                        y_i = sum_{j <= i} Linv(i, j) f_j; block row i is split in nc chunks of
//                        kInvDiagChunk blocks (partial slots slot0 .. slot0+nc-1; nc = 1: no split);
//   FwdInvTail           {s, -, nb, r0, r1, -, -}: f[r0, r1) -= L[r0:r1, 0:w] y;
//   BwdInvCols           {s, kb, nb, r0, r1, -, slot}: partial sums of L[r0:r1, block kb]^T g
//                        into partial slot `slot` (a block's nq chunks have consecutive slots);
//   BwdInvReduce         {s, kb, nb, slot0, nq, -, -}: g of block kb -= its nq partial sums;
//   BwdInvDiag           {s, j, nb, ob_s, slot0, nc, blk, i0, i1}: the part i0 <= i <= i1 of
//                        x_j = sum_{i >= j} Linv(i, j)^T g_i, in chunks as FwdInvDiag.
// blk is the diagonal-inverse index of the front's block 0.
struct InvLaunch {
    int begin, count;   // inversion tasks of one diagonal i - j
};

// Solve task of supernode s.  Gathers: rows [r0, r1) of the front vector.
// Level launches: a chain (k0 = bulk index of the chunk of the front's
// diagonal block 0, blk = its first diagonal block) or a bulk chunk of rows
// (forward) or own columns (backward) [r0, r1) (blk as for chains).
// Trailing-row dots: columns [k0, k0+kn) against rows [r0, r1).  Inversion:
// diagonal block [k0, k0+kn), blk = its index in the inverse arena.
struct SolveBlockTask {
    int s, k0, kn, r0, r1;
    int flags, blk;
    int c0 = 0, c1 = 0;   // inverse-front diagonal tasks: the range of inverse blocks summed
};

// Host mirror of the device TcJob (tc_gemm.cuh): one rank-kn update of a front.
struct TcJobHost {
    long long tile_begin;
    int s, c0, cend, kbeg, kn, map;
};

// Front-size buckets of the one-CTA small-front kernel: 32 rows each, up to kSmallFrontLimit
// rows (the whole front in FP64 shared memory: 160^2 * 8 bytes = 200 KB).
constexpr int kSmallBucketRows = 32;
constexpr int kSmallFrontLimit = 160;
constexpr int kSmallBuckets = kSmallFrontLimit / kSmallBucketRows;
inline bool small_front(const PlanConfig& cfg, int m) {
    return m <= kSmallFrontLimit && ((cfg.small_mask >> ((m - 1) / kSmallBucketRows)) & 1);
}

// Rows in 16 bytes of the factor storage type (float on the tensor-core path, else double):
// tile copies by tensor map must start on a multiple of it.
inline int kTileAlignRows(const PlanConfig& cfg) { return cfg.tensor_core ? 4 : 2; }

struct Plan {
    PlanConfig cfg;
    int n = 0, count = 0, levels = 0;          // count: device fronts
    int supernodes = 0;                        // supernodes of the symbolic partition
    std::vector<int> front_rows, child_ptr, children;   // structure of the device fronts (solves)
    std::vector<int> level_of;                 // per supernode
    std::vector<SnDev> sn;                     // per supernode
    std::vector<int> rel;                      // parent-local index of each trailing row
    std::vector<long long> assemble_pos;       // per matrix value: offset in the factor arena
    long long factor_elems = 0;                // panels
    long long contrib_elems = 0;               // contribution arena (planned peak)
    long long fvec_elems = 0;                  // front-vector workspace of the solves (per RHS)
    std::vector<long long> fvec_off;           // per supernode offset into the front-vector workspace

    // factorisation tasks
    std::vector<EaItem> ea_items;
    std::vector<EaEntry> ea_entries;
    std::vector<int> small_fronts;
    std::vector<PanelTask> pivot_tasks;   // one per (front, pivot block); mixed path: per (front, outer block)
    std::vector<PanelTask> panel_tasks;   // TRSM / panel-solve row chunks
    int diag_slots = 0;                   // mixed path: most diagonal blocks of one launch (inverse workspace slots)
    double panel_flops = 0.0;             // mixed path: flops of the panel-solve products
    std::vector<UpdJob> simt_jobs;
    std::vector<TcJobHost> tc_jobs;
    std::vector<StageInfo> stage;              // per supernode (tensor-core path)
    std::vector<int> map_front;                // front of each tensor-map pair
    std::vector<Launch> launches;
    int max_small_m = 0;
    long long stage_elems = 0;                 // elements of each operand staging arena (tensor-core path)
    double tc_flops = 0.0;                     // algorithmic flops of the tensor-core updates (lower triangle)
    double simt_flops = 0.0;                   // algorithmic flops of the SIMT updates

    // solve tasks
    std::vector<int> solve_fronts;             // supernode lists for gather/finish launches
    std::vector<SolveBlockTask> solve_tasks;
    std::vector<SolveBlockTask> inv_blocks;    // every diagonal block, for the inversion after a factorisation
    std::vector<SolveLaunch> fwd_launches, bwd_launches;
    std::vector<SolveBlockTask> inv_tasks;     // inverse fronts: off-diagonal inverse blocks, by diagonal
    std::vector<InvLaunch> inv_launches;
    long long inv_off_blocks = 0;              // blocks of the off-diagonal inverse arena
    int inv_partial_slots = 0;                 // most BwdInvCols partial slots of one launch (SB x nrhs each)
    int inv_diag_slots = 0;                    // most inverse-diagonal partial slots of one launch (SB x nrhs each)
    int progress_count = 0;                    // progress counters of all level launches
    int bwd_partial_slots = 0;                 // most backward column-dot partial slots of one launch (8 x nrhs each)
};

// Algorithmic flops (2 per multiply-add, lower triangle) and tiles of an update job.
double job_flops(const UpdJob& J, const SnDev& d);
long long job_tiles(const UpdJob& J, const SnDev& d, int T);

// Throws std::runtime_error on inconsistent symbolic input.
Plan build_plan(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                const int* children, const int* front_ptr, const int* front_rows, const int* diag_value_index,
                const int* pattern_ptr, const int* pattern_rows, const int* lower_start, const int* lower_value_ptr,
                const int* lower_value_index, int nnz, const PlanConfig& cfg);

}  // namespace uchol_dev
