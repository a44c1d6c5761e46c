// Execution plan of the device numeric phase (see plan.hpp).
#include "plan.hpp"

#include <algorithm>
#include <map>
#include <stdexcept>

namespace uchol_dev {

namespace {

inline long long round_up(long long x, long long a) { return (x + a - 1) / a * a; }

void fail(const std::string& m) { throw std::runtime_error(m); }

// First-fit allocator over one arena, used to plan the lifetimes of the
// contribution blocks ahead of time (no device allocation at run time).
class ArenaPlanner {
public:
    long long alloc(long long size) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= size) {
                long long off = it->first;
                long long rest = it->second - size;
                free_.erase(it);
                if (rest > 0) free_[off + size] = rest;
                return off;
            }
        }
        long long off = top_;
        // extend the last free block if it touches the top
        if (!free_.empty()) {
            auto last = std::prev(free_.end());
            if (last->first + last->second == top_) {
                off = last->first;
                free_.erase(last);
            }
        }
        top_ = off + size;
        peak_ = std::max(peak_, top_);
        return off;
    }
    void release(long long off, long long size) {
        auto it = free_.emplace(off, size).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
                it = prev;
            }
        }
        if (it->first + it->second == top_) {
            top_ = it->first;
            free_.erase(it);
        }
    }
    long long peak() const { return peak_; }

private:
    std::map<long long, long long> free_;
    long long top_ = 0, peak_ = 0;
};

}  // namespace

// Useful flops of an update job: 2 * kn per lower-triangle entry of columns [c0, cend), rows j..m-1.
double job_flops(const UpdJob& J, const SnDev& d) {
    const double cols = J.cend - J.c0;
    const double entries = cols * d.m - (double)(J.c0 + J.cend - 1) * cols / 2.0;
    return 2.0 * J.kn * entries;
}

// Tile count of an update job (must match decode_tile).
long long job_tiles(const UpdJob& J, const SnDev& d, int T) {
    auto region = [&](int base, int lim) -> long long {
        if (lim <= base) return 0;
        long long nc = (lim - base + T - 1) / T;
        long long R = (d.m - base + T - 1) / T;
        return region_tiles(nc, R);
    };
    if (J.c0 < d.w && d.w < J.cend) return region(J.c0, d.w) + region(d.w, J.cend);
    return region(J.c0, J.cend);
}


namespace {

// Checks the front structure (every device index the plan derives from it).
void validate_fronts(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                     const int* children, const int* front_ptr, const int* front_rows) {
    if (first_column[0] != 0 || first_column[count] != n) fail("first_column does not span 0..n");
    if (front_ptr[0] != 0) fail("front_ptr must start at 0");
    for (int s = 0; s < count; ++s) {
        int w = first_column[s + 1] - first_column[s];
        int m = front_ptr[s + 1] - front_ptr[s];
        if (w < 1 || m < w) fail("supernode " + std::to_string(s) + " has an invalid width or front size");
        if (parent[s] != -1 && (parent[s] <= s || parent[s] >= count)) fail("supernode parents must follow their children");
        const int* rows = front_rows + front_ptr[s];
        for (int a = 0; a < m; ++a) {
            if (rows[a] < 0 || rows[a] >= n) fail("front row index out of range");
            if (a > 0 && rows[a] <= rows[a - 1]) fail("front rows are not strictly ascending");
            if (a < w && rows[a] != first_column[s] + a) fail("front rows must start with the supernode's columns");
        }
        if (m > w && parent[s] < 0) fail("a root supernode cannot have trailing rows");
        if (child_ptr[s + 1] < child_ptr[s]) fail("child pointers are not monotone");
        for (int c = child_ptr[s]; c < child_ptr[s + 1]; ++c)
            if (children[c] < 0 || children[c] >= s || parent[children[c]] != s) fail("children list inconsistent with parents");
    }
}

Plan build_from_fronts(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                       const int* children, const int* front_ptr, const int* front_rows, const int* diag_value_index,
                       const int* pattern_ptr, const int* pattern_rows, const int* lower_start,
                       const int* lower_value_ptr, const int* lower_value_index, int nnz, const PlanConfig& cfg) {
    Plan P;
    P.cfg = cfg;
    P.n = n;
    P.count = count;
    if (count == 0) return P;
    validate_fronts(n, count, first_column, parent, child_ptr, children, front_ptr, front_rows);
    if ((long long)pattern_ptr[n] < 0 || lower_value_ptr[n] < 0) fail("negative pattern length");

    // ---- levels (height in the assembly tree) ----
    P.level_of.assign(count, 0);
    for (int s = 0; s < count; ++s)
        if (parent[s] >= 0) P.level_of[parent[s]] = std::max(P.level_of[parent[s]], P.level_of[s] + 1);
    P.levels = 0;
    for (int s = 0; s < count; ++s) P.levels = std::max(P.levels, P.level_of[s] + 1);
    std::vector<std::vector<int>> at_level(P.levels);
    for (int s = 0; s < count; ++s) at_level[P.level_of[s]].push_back(s);

    // ---- per-supernode geometry, relative indices ----
    P.sn.resize(count);
    long long rel_total = 0;
    for (int s = 0; s < count; ++s) {
        SnDev& d = P.sn[s];
        d.w = first_column[s + 1] - first_column[s];
        d.m = front_ptr[s + 1] - front_ptr[s];
        d.first_col = first_column[s];
        d.rows_off = front_ptr[s];
        d.parent = parent[s];
        d.ldp = (int)round_up(d.m, 8);
        int t = d.m - d.w;
        d.ldc = t > 0 ? (int)round_up(t, 8) : 0;
        d.rel_off = (int)rel_total;
        rel_total += t;
    }
    if (rel_total > INT32_MAX) fail("too many trailing rows for 32-bit offsets");
    P.rel.assign(rel_total, 0);
    for (int s = 0; s < count; ++s) {
        const SnDev& d = P.sn[s];
        int t = d.m - d.w;
        if (t == 0) continue;
        const SnDev& pd = P.sn[parent[s]];
        const int* prow = front_rows + front_ptr[parent[s]];
        const int* crow = front_rows + front_ptr[s] + d.w;
        int q = 0;
        for (int a = 0; a < t; ++a) {
            while (q < pd.m && prow[q] < crow[a]) ++q;
            if (q == pd.m || prow[q] != crow[a])
                fail("trailing row of supernode " + std::to_string(s) + " is missing from its parent's pattern");
            P.rel[d.rel_off + a] = q;
        }
    }

    // ---- factor panels (persistent) ----
    long long off = 0;
    for (int s = 0; s < count; ++s) {
        SnDev& d = P.sn[s];
        d.panel_off = off;
        off += round_up((long long)d.ldp * d.w, 64);
    }
    P.factor_elems = off;

    // ---- contribution blocks: lifetime [level(s), level(parent)] ----
    {
        ArenaPlanner arena;
        std::vector<long long> size(count, 0);
        for (int L = 0; L < P.levels; ++L) {
            for (int s : at_level[L]) {
                SnDev& d = P.sn[s];
                int t = d.m - d.w;
                if (t == 0) {
                    d.contrib_off = -1;
                    continue;
                }
                size[s] = round_up((long long)d.ldc * t, 64);
                d.contrib_off = arena.alloc(size[s]);
            }
            for (int s : at_level[L])
                for (int c = child_ptr[s]; c < child_ptr[s + 1]; ++c) {
                    int ch = children[c];
                    if (size[ch] > 0) arena.release(P.sn[ch].contrib_off, size[ch]);
                }
        }
        P.contrib_elems = std::max<long long>(arena.peak(), 64);
    }

    // ---- assembly map ----
    P.assemble_pos.assign(nnz, -1);
    {
        std::vector<int> row_map(n, -1);
        for (int s = 0; s < count; ++s) {
            const SnDev& d = P.sn[s];
            const int* rows = front_rows + front_ptr[s];
            for (int a = 0; a < d.m; ++a) row_map[rows[a]] = a;
            for (int lc = 0; lc < d.w; ++lc) {
                int j = d.first_col + lc;
                int di = diag_value_index[j];
                if (di >= 0) {
                    if (di >= nnz || P.assemble_pos[di] != -1) fail("diagonal value index invalid or repeated");
                    P.assemble_pos[di] = d.panel_off + lc + (long long)lc * d.ldp;
                }
                int lb = lower_value_ptr[j];
                for (int p = lower_start[j]; p < pattern_ptr[j + 1]; ++p) {
                    int r = pattern_rows[p];
                    if (r <= j || r >= n) fail("lower pattern row out of range");
                    int lr = row_map[r];
                    if (lr < 0 || rows[lr] != r) fail("matrix entry outside the supernode's row pattern");
                    int vi = lower_value_index[lb + (p - lower_start[j])];
                    if (vi < 0 || vi >= nnz || P.assemble_pos[vi] != -1) fail("lower value index invalid or repeated");
                    P.assemble_pos[vi] = d.panel_off + lr + (long long)lc * d.ldp;
                }
            }
            for (int a = 0; a < d.m; ++a) row_map[rows[a]] = -1;
        }
        for (int k = 0; k < nnz; ++k)
            if (P.assemble_pos[k] < 0) fail("a matrix value is not referenced by the symbolic pattern");
    }

    // ---- factorisation launches, level by level ----
    P.stage.assign(count, StageInfo{0, 0, -1});
    const int PB = cfg.pivot_block;
    const int NB = cfg.tensor_core ? cfg.outer_block : cfg.pivot_block;
    const int TS = cfg.tile;
    for (int L = 0; L < P.levels; ++L) {
        const auto& fronts = at_level[L];
        // extend-add: one item per receiving parent column.  With side_extend_add the items of
        // the contribution columns of large fronts form a launch of their own, run on the side
        // stream: nothing before the level's contribution update reads or writes those columns
        // (the own-column updates, diagonal blocks and panel solves stay within the panel).
        const bool side = cfg.tensor_core && cfg.side_extend_add;
        std::vector<EaItem> side_items;
        std::vector<EaEntry> side_entries;
        int ib = (int)P.ea_items.size();
        for (int s : fronts) {
            struct Rec { int pcol, order, child, a; };
            std::vector<Rec> recs;
            for (int c = child_ptr[s]; c < child_ptr[s + 1]; ++c) {
                int ch = children[c];
                const SnDev& cd = P.sn[ch];
                int t = cd.m - cd.w;
                for (int a = 0; a < t; ++a) recs.push_back({P.rel[cd.rel_off + a], c, ch, a});
            }
            std::stable_sort(recs.begin(), recs.end(), [](const Rec& x, const Rec& y) {
                return x.pcol != y.pcol ? x.pcol < y.pcol : x.order < y.order;
            });
            // panel columns that receive entries, then every contribution column (its item also
            // clears the column's lower part before adding, so no separate clearing pass exists)
            const SnDev& pd = P.sn[s];
            size_t q = 0;
            while (q < recs.size() && recs[q].pcol < pd.w) {
                EaItem it{s, recs[q].pcol, (int)P.ea_entries.size(), 0};
                for (const int pc = it.pcol; q < recs.size() && recs[q].pcol == pc; ++q)
                    P.ea_entries.push_back({recs[q].child, recs[q].a});
                it.end = (int)P.ea_entries.size();
                P.ea_items.push_back(it);
            }
            const bool to_side = side && !small_front(cfg, pd.m);
            std::vector<EaItem>& items = to_side ? side_items : P.ea_items;
            std::vector<EaEntry>& ents = to_side ? side_entries : P.ea_entries;
            for (int pc = pd.w; pc < pd.m; ++pc) {
                EaItem it{s, pc, (int)ents.size(), 0};
                for (; q < recs.size() && recs[q].pcol == pc; ++q) ents.push_back({recs[q].child, recs[q].a});
                it.end = (int)ents.size();
                items.push_back(it);
            }
        }
        const int main_items = (int)P.ea_items.size() - ib;
        bool side_pending = false;
        if (!side_items.empty()) {
            const int base = (int)P.ea_entries.size(), sb0 = (int)P.ea_items.size();
            P.ea_entries.insert(P.ea_entries.end(), side_entries.begin(), side_entries.end());
            for (EaItem it : side_items) {
                it.begin += base;
                it.end += base;
                P.ea_items.push_back(it);
            }
            Launch Ls{Launch::ExtendAdd, sb0, (int)side_items.size(), 0};
            Ls.stream = 1;
            P.launches.push_back(Ls);
            side_pending = true;
        }
        if (main_items > 0) P.launches.push_back({Launch::ExtendAdd, ib, main_items, 0});

        // small fronts: one CTA each
        int sb = (int)P.small_fronts.size();
        std::vector<int> large;
        for (int s : fronts) {
            if (small_front(cfg, P.sn[s].m)) {
                P.small_fronts.push_back(s);
                P.max_small_m = std::max(P.max_small_m, P.sn[s].m);
            } else {
                large.push_back(s);
            }
        }
        if ((int)P.small_fronts.size() > sb) P.launches.push_back({Launch::SmallFronts, sb, (int)P.small_fronts.size() - sb, 0});

        // large fronts: blocked right-looking factorisation in lockstep
        int max_w = 0;
        for (int s : large) max_w = std::max(max_w, P.sn[s].w);
        if (cfg.tensor_core) {
            // one staging region per large front of the level (the arena is reused by every level)
            long long top = 0;
            for (int s : large) {
                const SnDev& d = P.sn[s];
                StageInfo& g = P.stage[s];
                g.ld = (int)round_up(d.w, 64);
                g.off = top;
                g.map = (int)P.map_front.size();
                P.map_front.push_back(s);
                top += round_up((long long)d.m * g.ld, 256);
            }
            P.stage_elems = std::max(P.stage_elems, top);
        }
        // tensor-core path, left-looking in two levels.  At the start of each super-block of
        // kSuperBlocks outer blocks, one update brings all of its columns up to date with every
        // earlier column of the supernode (K = sb0); each later outer block of the super-block
        // then takes only the super-block's own earlier columns (K = k0 - sb0).  The operands
        // W and L of K columns are read once per super-block instead of once per outer block:
        // at 128-column blocks that update moves 2 bytes of W per 128 flops and is HBM-bound.
        const int SBW = kSuperBlocks * NB;
        for (int k0 = 0; k0 < max_w; k0 += NB) {
            const int sb0 = k0 / SBW * SBW;
            if (cfg.tensor_core && k0 > 0) {
                int jb = (int)P.tc_jobs.size();
                long long tiles = 0;
                for (int s : large) {
                    const SnDev& d = P.sn[s];
                    if (d.w <= k0) continue;
                    const bool super = k0 == sb0;
                    const int cend = std::min(d.w, k0 + (super ? SBW : NB));
                    const int kbeg = super ? 0 : sb0;
                    const int kn = super ? k0 : k0 - sb0;
                    UpdJob U{tiles, s, k0, cend, kbeg, kn, -1};
                    P.tc_jobs.push_back({tiles, s, k0, cend, kbeg, kn, P.stage[s].map});
                    tiles += tc_job_tiles(k0, cend, d.m);
                    P.tc_flops += job_flops(U, d);
                }
                if ((int)P.tc_jobs.size() > jb) P.launches.push_back({Launch::TcUpdate, jb, (int)P.tc_jobs.size() - jb, tiles});
            }
            // mixed path: the whole outer block in two launches (diagonal block, then its rows below)
            if (cfg.tensor_core) {
                int qb = (int)P.pivot_tasks.size();
                int pb = (int)P.panel_tasks.size();
                int slot = 0;
                for (int s : large) {
                    const SnDev& d = P.sn[s];
                    if (d.w <= k0) continue;
                    int nbo = std::min(NB, d.w - k0);
                    P.pivot_tasks.push_back({s, k0, nbo, k0 + nbo, 0, -1, slot, 0});
                    int zero_to = (k0 + nbo == d.w && P.stage[s].ld > d.w) ? P.stage[s].ld : 0;
                    for (int r = k0 + nbo; r < d.m; r += kSolveRowsPlan) {
                        int rows = std::min(kSolveRowsPlan, d.m - r);
                        P.panel_tasks.push_back({s, k0, nbo, r, rows, 1, slot, zero_to});
                        P.panel_flops += 2.0 * rows * nbo * nbo;
                    }
                    ++slot;
                }
                P.diag_slots = std::max(P.diag_slots, slot);
                if ((int)P.pivot_tasks.size() > qb) P.launches.push_back({Launch::DiagBlock, qb, (int)P.pivot_tasks.size() - qb, 0});
                if ((int)P.panel_tasks.size() > pb) P.launches.push_back({Launch::PanelSolve, pb, (int)P.panel_tasks.size() - pb, 0});
                continue;
            }
            for (int j0r = 0; j0r < NB; j0r += PB) {
                int qb = (int)P.pivot_tasks.size();
                int pb = (int)P.panel_tasks.size();
                int ub = (int)P.simt_jobs.size();
                long long utiles = 0;
                for (int s : large) {
                    const SnDev& d = P.sn[s];
                    if (d.w <= k0) continue;
                    int nbo = std::min(NB, d.w - k0);
                    int j0 = k0 + j0r;
                    if (j0r >= nbo) continue;
                    int nbi = std::min(PB, k0 + nbo - j0);
                    int outer_end = k0 + nbo;
                    P.pivot_tasks.push_back({s, j0, nbi, j0 + nbi, 0, -1, 0, 0});
                    // TRSM tasks over rows [j0+nbi, m)
                    int r = j0 + nbi;
                    while (r < d.m) {
                        int rows = std::min(128, d.m - r);
                        int stage = cfg.tensor_core ? 1 : 0, zero_to = 0;
                        if (cfg.tensor_core && j0 + nbi == d.w && P.stage[s].ld > d.w) zero_to = P.stage[s].ld;
                        P.panel_tasks.push_back({s, j0, nbi, r, rows, stage, 0, zero_to});
                        r += rows;
                    }
                    // inner update of the rest of the outer block (tensor-core configuration only)
                    if (NB != PB && j0 + nbi < outer_end) {
                        UpdJob J{utiles, s, j0 + nbi, outer_end, j0, nbi, -1};
                        utiles += job_tiles(J, d, TS);
                        P.simt_flops += job_flops(J, d);
                        P.simt_jobs.push_back(J);
                    }
                }
                if ((int)P.pivot_tasks.size() > qb) P.launches.push_back({Launch::PivotBlock, qb, (int)P.pivot_tasks.size() - qb, 0});
                if ((int)P.panel_tasks.size() > pb) P.launches.push_back({Launch::Trsm, pb, (int)P.panel_tasks.size() - pb, 0});
                if ((int)P.simt_jobs.size() > ub)
                    P.launches.push_back({Launch::SimtUpdate, ub, (int)P.simt_jobs.size() - ub, utiles});
                if (!cfg.tensor_core) break;  // FP64 path: one pivot block per outer step
            }
            // FP64 path: right-looking update of the whole trailing triangle per step
            if (!cfg.tensor_core) {
                int jb = (int)P.simt_jobs.size();
                long long tiles = 0;
                for (int s : large) {
                    const SnDev& d = P.sn[s];
                    if (d.w <= k0) continue;
                    int nbo = std::min(NB, d.w - k0);
                    int c0 = k0 + nbo;
                    if (c0 >= d.m) continue;
                    UpdJob J{tiles, s, c0, d.m, k0, nbo, -1};
                    tiles += job_tiles(J, d, TS);
                    P.simt_flops += job_flops(J, d);
                    P.simt_jobs.push_back(J);
                }
                if ((int)P.simt_jobs.size() > jb)
                    P.launches.push_back({Launch::SimtUpdate, jb, (int)P.simt_jobs.size() - jb, tiles});
            }
        }
        // tensor-core path: contribution block of every large front, K = its whole width
        if (cfg.tensor_core) {
            int jb = (int)P.tc_jobs.size();
            long long tiles = 0;
            for (int s : large) {
                const SnDev& d = P.sn[s];
                if (d.m == d.w) continue;
                UpdJob U{tiles, s, d.w, d.m, 0, d.w, -1};
                P.tc_jobs.push_back({tiles, s, d.w, d.m, 0, d.w, P.stage[s].map});
                tiles += tc_job_tiles(d.w, d.m, d.m);
                P.tc_flops += job_flops(U, d);
            }
            if ((int)P.tc_jobs.size() > jb) {
                Launch Lc{Launch::TcUpdate, jb, (int)P.tc_jobs.size() - jb, tiles};
                Lc.stream = side_pending ? 2 : 0;   // the contribution columns are complete first
                P.launches.push_back(Lc);
                side_pending = false;
            }
        }
        if (side_pending) fail("side-stream extend-add without a contribution update to join it");
    }

    // ---- solves ----
    P.fvec_off.assign(count, 0);
    long long fo = 0;
    for (int s = 0; s < count; ++s) {
        P.fvec_off[s] = fo;
        fo += round_up(P.sn[s].m, 8);
    }
    P.fvec_elems = std::max<long long>(fo, 8);
    const int SB = cfg.solve_block;
    // diagonal blocks of every supernode (inverted once per factorisation)
    std::vector<int> first_blk(count, 0);
    for (int s = 0; s < count; ++s) {
        first_blk[s] = (int)P.inv_blocks.size();
        for (int k0 = 0; k0 < P.sn[s].w; k0 += SB)
            P.inv_blocks.push_back({s, k0, std::min(SB, P.sn[s].w - k0), 0, 0, 1, (int)P.inv_blocks.size()});
    }
    // inverse fronts: SB < w <= inv_cols; their off-diagonal inverse blocks, by diagonal i - j
    std::vector<int> inv_ob(count, -1);
    {
        int max_nb = 0;
        for (int s = 0; s < count; ++s) {
            const int w = P.sn[s].w;
            if (cfg.inv_cols <= 0 || w <= SB || w > cfg.inv_cols) continue;
            const int nb = (w + SB - 1) / SB;
            if (P.inv_off_blocks + (long long)nb * (nb - 1) / 2 > INT32_MAX) fail("too many inverse blocks");
            inv_ob[s] = (int)P.inv_off_blocks;
            P.inv_off_blocks += (long long)nb * (nb - 1) / 2;
            max_nb = std::max(max_nb, nb);
        }
        for (int dg = 1; dg < max_nb; ++dg) {
            const int b0 = (int)P.inv_tasks.size();
            for (int s = 0; s < count; ++s) {
                if (inv_ob[s] < 0) continue;
                const int nb = (P.sn[s].w + SB - 1) / SB;
                for (int i = dg; i < nb; ++i) P.inv_tasks.push_back({s, i, i - dg, inv_ob[s], 0, 0, first_blk[s]});
            }
            if ((int)P.inv_tasks.size() > b0) P.inv_launches.push_back({b0, (int)P.inv_tasks.size() - b0});
        }
    }
    constexpr int kGatherChunk = 512;   // rows per gather CTA (one CTA per chunk and right-hand side)
    // chunked per-front tasks: rows [r0, r1) of the front vector
    auto gather_tasks = [&](const std::vector<int>& fronts) {
        int b = (int)P.solve_tasks.size();
        for (int s : fronts)
            for (int r = 0; r < P.sn[s].m; r += kGatherChunk)
                P.solve_tasks.push_back({s, 0, 0, r, std::min(P.sn[s].m, r + kGatherChunk), 0, 0});
        return std::make_pair(b, (int)P.solve_tasks.size() - b);
    };
    // level launch: chains (one per front), then the bulk chunks that take updates.  The
    // diagonal-block chunks of a front that the bulk updates are contiguous and in block order,
    // from block 2 (forward; blocks 0 and 1 take theirs from the chain) or block 0 up to
    // nblk - 3 (backward); the chain finds them by index (task k0 = the index its block-0
    // chunk would have).  Trailing-row chunks (forward only) come after all of them.
    auto level_launch = [&](SolveLaunch::Kind kind, const std::vector<int>& fronts, bool forward) {
        SolveLaunch Lh{kind, (int)P.solve_tasks.size(), (int)fronts.size(), 0, 0, 0, P.progress_count, 0, 0, 0, 0, 0};
        std::vector<SolveBlockTask> bulk;
        // chains longest first: CTA k takes chains k, k + nchain_cta, ..., so every long chain
        // gets a CTA of its own when there are enough
        std::vector<int> order(fronts.begin(), fronts.end());
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return P.sn[a].w > P.sn[b].w; });
        for (int s : order) Lh.long_chains += (P.sn[s].w + SB - 1) / SB >= 3;
        const size_t chain_base = P.solve_tasks.size();
        P.solve_tasks.resize(chain_base + order.size());
        std::map<int, int> pos;
        for (size_t k = 0; k < order.size(); ++k) pos[order[k]] = (int)k;
        for (int s : fronts) {
            const SnDev& d = P.sn[s];
            const int nblk = (d.w + SB - 1) / SB;
            Lh.steps = std::max(Lh.steps, nblk);
            Lh.chain_work += nblk;
            Lh.bulk_work += (long long)std::max(0, nblk - 1) * (nblk - 2 > 0 ? nblk - 2 : 0) / 2;
            const int lo = forward ? 2 : 0, hi = forward ? nblk - 1 : nblk - 3;   // bulk diagonal blocks [lo, hi]
            P.solve_tasks[chain_base + pos[s]] = {s, (int)bulk.size() - lo, nblk, 0, 0, 0, first_blk[s]};
            // kn: the number of solutions the chunk applies (forward y_0 .. y_{k-2}; backward
            // x_{nblk-1} .. x_{k+2}); backward k0 = nblk - 1 (step t applies block k0 - t)
            for (int k = lo; k <= hi; ++k)
                bulk.push_back({s, forward ? 0 : nblk - 1, forward ? k - 1 : nblk - 2 - k, k * SB,
                                std::min(d.w, (k + 1) * SB), 0, first_blk[s]});
        }
        Lh.ndiag = (int)bulk.size();
        Lh.diag_work = Lh.bulk_work;
        const bool trailing = forward;
        if (trailing)
            for (int s : fronts) {
                const SnDev& d = P.sn[s];
                const int nblk = (d.w + SB - 1) / SB;
                // SB - A rows each: the tile copy starts at the row rounded down to 16 bytes
                // (A rows), so that the chunk still fits in one SB-row box
                const int height = SB - kTileAlignRows(cfg);
                for (int r = d.w; r < d.m; r += height) {
                    bulk.push_back({s, 0, nblk, r, std::min(d.m, r + height), 0, first_blk[s]});
                    Lh.bulk_work += nblk;
                }
            }
        Lh.bulk_begin = (int)P.solve_tasks.size();
        Lh.bulk_count = (int)bulk.size();
        P.solve_tasks.insert(P.solve_tasks.end(), bulk.begin(), bulk.end());
        P.progress_count += (int)bulk.size();
        return Lh;
    };
    // fronts of one diagonal block go to the solo kernels, inverse fronts to their own kernels,
    // the others to the level kernels
    auto split = [&](const std::vector<int>& fronts, std::vector<int>& multi, std::vector<int>& inv) {
        SolveLaunch S{SolveLaunch::FwdSolo, (int)P.solve_tasks.size(), 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        multi.clear();
        inv.clear();
        for (int s : fronts) {
            if (P.sn[s].w <= SB) P.solve_tasks.push_back({s, 0, P.sn[s].w, 0, 0, 0, first_blk[s]});
            else if (inv_ob[s] >= 0) inv.push_back(s);
            else multi.push_back(s);
        }
        S.count = (int)P.solve_tasks.size() - S.begin;
        return S;
    };
    auto simple = [&](SolveLaunch::Kind kind, int begin) {
        return SolveLaunch{kind, begin, (int)P.solve_tasks.size() - begin, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    };
    std::vector<int> multi, inv;
    for (int L = 0; L < P.levels; ++L) {
        const auto& fronts = at_level[L];
        auto g = gather_tasks(fronts);
        P.fwd_launches.push_back({SolveLaunch::FwdGather, g.first, g.second, 0, 0, 0, 0, 0, 0, 0, 0, 0});
        SolveLaunch solo = split(fronts, multi, inv);
        if (solo.count > 0) P.fwd_launches.push_back(solo);
        // trailing rows of the single-block fronts, in chunks from w rounded down to 4
        int tb = (int)P.solve_tasks.size();
        for (int s : fronts) {
            const SnDev& d = P.sn[s];
            if (d.w > SB || d.m == d.w) continue;
            for (int r = d.w & ~3; r < d.m; r += kTailRowsPlan)
                P.solve_tasks.push_back({s, 0, d.w, r, std::min(d.m, r + kTailRowsPlan), 0, 0});
        }
        if ((int)P.solve_tasks.size() > tb)
            P.fwd_launches.push_back({SolveLaunch::FwdTail, tb, (int)P.solve_tasks.size() - tb, 0, 0, 0, 0, 0, 0, 0, 0, 0});
        if (!multi.empty()) P.fwd_launches.push_back(level_launch(SolveLaunch::FwdLevel, multi, true));
        if (!inv.empty()) {
            // y_1 per block row, then the trailing rows in chunks of SB - A rows (the tile copy starts
            // at the chunk's first row rounded down to 16 bytes)
            int b = (int)P.solve_tasks.size(), dslots = 0;
            for (int s : inv) {
                const int nb = (P.sn[s].w + SB - 1) / SB;
                for (int i = 0; i < nb; ++i) {
                    const int nc = (i + kInvDiagChunk) / kInvDiagChunk;   // blocks 0 .. i
                    for (int c = 0; c < nc; ++c) {
                        SolveBlockTask t{s, i, nb, inv_ob[s], dslots, nc, first_blk[s]};
                        t.c0 = c * kInvDiagChunk;
                        t.c1 = std::min(i, t.c0 + kInvDiagChunk - 1);
                        P.solve_tasks.push_back(t);
                    }
                    dslots += nc;
                }
            }
            P.inv_diag_slots = std::max(P.inv_diag_slots, dslots);
            P.fwd_launches.push_back(simple(SolveLaunch::FwdInvDiag, b));
            b = (int)P.solve_tasks.size();
            const int height = SB - kTileAlignRows(cfg);
            for (int s : inv) {
                const SnDev& d = P.sn[s];
                const int nb = (d.w + SB - 1) / SB;
                for (int r = d.w; r < d.m; r += height) P.solve_tasks.push_back({s, 0, nb, r, std::min(d.m, r + height), 0, 0});
            }
            if ((int)P.solve_tasks.size() > b) P.fwd_launches.push_back(simple(SolveLaunch::FwdInvTail, b));
        }
    }
    for (int L = P.levels - 1; L >= 0; --L) {
        const auto& fronts = at_level[L];
        auto g = gather_tasks(fronts);
        P.bwd_launches.push_back({SolveLaunch::BwdGather, g.first, g.second, 0, 0, 0, 0, 0, 0, 0, 0, 0});
        // column dots against the trailing rows, 8 columns per task; columns longer than
        // kColRowsPlan rows are split into row chunks (flags = 1, blk = partial slot) whose
        // partial sums a reduction task (k0, kn; r0 = first slot, r1 = slots) adds in order
        int tb = (int)P.solve_tasks.size();
        std::vector<SolveBlockTask> reduce;
        int slot = 0;
        for (int s : fronts) {
            const SnDev& d = P.sn[s];
            if (d.m == d.w || inv_ob[s] >= 0) continue;
            const int nch = (d.m - d.w + kColRowsPlan - 1) / kColRowsPlan;
            for (int c = 0; c < d.w; c += 8) {
                const int kn = std::min(8, d.w - c);
                if (nch == 1) {
                    P.solve_tasks.push_back({s, c, kn, d.w, d.m, 0, 0});
                    continue;
                }
                reduce.push_back({s, c, kn, slot, nch, 0, 0});
                for (int q = 0; q < nch; ++q) {
                    const int r0 = d.w + q * kColRowsPlan;
                    P.solve_tasks.push_back({s, c, kn, r0, std::min(d.m, r0 + kColRowsPlan), 1, slot++});
                }
            }
        }
        if ((int)P.solve_tasks.size() > tb)
            P.bwd_launches.push_back({SolveLaunch::BwdTail, tb, (int)P.solve_tasks.size() - tb, 0, 0, 0, 0, 0, 0, 0, 0, 0});
        if (!reduce.empty()) {
            const int rb = (int)P.solve_tasks.size();
            P.solve_tasks.insert(P.solve_tasks.end(), reduce.begin(), reduce.end());
            P.bwd_launches.push_back({SolveLaunch::BwdTailReduce, rb, (int)reduce.size(), 0, 0, 0, 0, 0, 0, 0, 0, 0});
        }
        P.bwd_partial_slots = std::max(P.bwd_partial_slots, slot);
        SolveLaunch solo = split(fronts, multi, inv);
        solo.kind = SolveLaunch::BwdSolo;
        if (solo.count > 0) P.bwd_launches.push_back(solo);
        if (!multi.empty()) P.bwd_launches.push_back(level_launch(SolveLaunch::BwdLevel, multi, false));
        if (!inv.empty()) {
            // partial sums per (column block, chunk of trailing rows), their sums per column block
            // in chunk order, then x_1 per block column.  With the SM count known, the level's
            // trailing rows are cut into as many chunks as make at most two tasks per SM (one
            // round of the two CTAs an SM holds); otherwise chunks of kInvColRowsPlan rows.
            int b = (int)P.solve_tasks.size(), slots = 0, dslots = 0;
            std::vector<SolveBlockTask> diag_tasks, reduce_tasks;
            int level_blocks = 0;
            for (int s : inv) level_blocks += (P.sn[s].w + SB - 1) / SB;
            for (int s : inv) {
                const SnDev& d = P.sn[s];
                const int nb = (d.w + SB - 1) / SB;
                const int t = d.m - d.w;
                int nq = (t + kInvColRowsPlan - 1) / kInvColRowsPlan, height = kInvColRowsPlan;
                if (cfg.sms > 0 && t > 0) {
                    nq = std::max(1, std::min((t + SB / 2 - 1) / (SB / 2), 2 * cfg.sms / std::max(1, level_blocks)));
                    height = (t + nq - 1) / nq;
                    nq = (t + height - 1) / height;
                }
                for (int kb = 0; kb < nb; ++kb)
                    for (int q = 0; q < nq; ++q) {
                        const int r0 = d.w + q * height;
                        P.solve_tasks.push_back({s, kb, nb, r0, std::min(d.m, r0 + height), 0, slots + kb * nq + q});
                    }
                if (nq > 0)
                    for (int kb = 0; kb < nb; ++kb) reduce_tasks.push_back({s, kb, nb, slots + kb * nq, nq, 0, 0});
                for (int j = 0; j < nb; ++j) {
                    const int nc = (nb - j + kInvDiagChunk - 1) / kInvDiagChunk;   // blocks j .. nb-1
                    for (int c = 0; c < nc; ++c) {
                        SolveBlockTask t{s, j, nb, inv_ob[s], dslots, nc, first_blk[s]};
                        t.c0 = j + c * kInvDiagChunk;
                        t.c1 = std::min(nb - 1, t.c0 + kInvDiagChunk - 1);
                        diag_tasks.push_back(t);
                    }
                    dslots += nc;
                }
                slots += nb * nq;
            }
            if ((int)P.solve_tasks.size() > b) P.bwd_launches.push_back(simple(SolveLaunch::BwdInvCols, b));
            if (!reduce_tasks.empty()) {
                b = (int)P.solve_tasks.size();
                P.solve_tasks.insert(P.solve_tasks.end(), reduce_tasks.begin(), reduce_tasks.end());
                P.bwd_launches.push_back(simple(SolveLaunch::BwdInvReduce, b));
            }
            P.inv_partial_slots = std::max(P.inv_partial_slots, slots);
            P.inv_diag_slots = std::max(P.inv_diag_slots, dslots);
            b = (int)P.solve_tasks.size();
            P.solve_tasks.insert(P.solve_tasks.end(), diag_tasks.begin(), diag_tasks.end());
            P.bwd_launches.push_back(simple(SolveLaunch::BwdInvDiag, b));
        }
    }
    return P;
}

}  // namespace

FrontStructure merge_chains(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                            const int* children, const int* front_ptr, const int* front_rows, int max_cols,
                            double max_fill) {
    FrontStructure F;
    F.group_of.assign(count, 0);
    // lower-trapezoid entries of a front of m rows and w columns
    auto entries = [](long long m, long long w) { return (double)(w * m - w * (w - 1) / 2); };
    std::vector<std::pair<int, int>> groups;   // first and last member
    for (int a = 0; a < count;) {
        int e = a;
        double own = entries(front_ptr[a + 1] - front_ptr[a], first_column[a + 1] - first_column[a]);
        while (max_cols > 0) {
            const int p = parent[e];
            if (p != e + 1 || child_ptr[p + 1] - child_ptr[p] != 1) break;   // not the next supernode's only child
            const int wg = first_column[p + 1] - first_column[a];
            if (wg > max_cols) break;
            const int wp = first_column[p + 1] - first_column[p], mp = front_ptr[p + 1] - front_ptr[p];
            const double with_p = own + entries(mp, wp);
            if (entries(wg + (mp - wp), wg) > (1.0 + max_fill) * with_p) break;
            own = with_p;
            e = p;
        }
        for (int q = a; q <= e; ++q) F.group_of[q] = (int)groups.size();
        groups.push_back({a, e});
        a = e + 1;
    }
    F.count = (int)groups.size();
    F.first_column.resize(F.count + 1);
    F.parent.resize(F.count);
    F.child_ptr.assign(F.count + 1, 0);
    F.front_ptr.assign(F.count + 1, 0);
    for (int g = 0; g < F.count; ++g) {
        const int a = groups[g].first, e = groups[g].second;
        F.first_column[g] = first_column[a];
        F.parent[g] = parent[e] < 0 ? -1 : F.group_of[parent[e]];
        // the group's columns, then the last member's trailing rows
        for (int c = first_column[a]; c < first_column[e + 1]; ++c) F.front_rows.push_back(c);
        const int we = first_column[e + 1] - first_column[e];
        F.front_rows.insert(F.front_rows.end(), front_rows + front_ptr[e] + we, front_rows + front_ptr[e + 1]);
        F.front_ptr[g + 1] = (int)F.front_rows.size();
        // children from outside the group: those of its first member (each later member's only
        // child is the member before it); ascending, as group numbers follow supernode numbers
        for (int c = child_ptr[a]; c < child_ptr[a + 1]; ++c) F.children.push_back(F.group_of[children[c]]);
        F.child_ptr[g + 1] = (int)F.children.size();
    }
    F.first_column[F.count] = count > 0 ? first_column[count] : 0;
    (void)n;
    return F;
}

Plan build_plan(int n, int count, const int* first_column, const int* parent, const int* child_ptr,
                const int* children, const int* front_ptr, const int* front_rows, const int* diag_value_index,
                const int* pattern_ptr, const int* pattern_rows, const int* lower_start, const int* lower_value_ptr,
                const int* lower_value_index, int nnz, const PlanConfig& cfg) {
    if (count == 0) {
        Plan P;
        P.cfg = cfg;
        P.n = n;
        P.child_ptr.assign(1, 0);
        return P;
    }
    validate_fronts(n, count, first_column, parent, child_ptr, children, front_ptr, front_rows);
    FrontStructure F = merge_chains(n, count, first_column, parent, child_ptr, children, front_ptr, front_rows,
                                    cfg.merge_cols, cfg.merge_fill);
    Plan P = build_from_fronts(n, F.count, F.first_column.data(), F.parent.data(), F.child_ptr.data(),
                               F.children.data(), F.front_ptr.data(), F.front_rows.data(), diag_value_index,
                               pattern_ptr, pattern_rows, lower_start, lower_value_ptr, lower_value_index, nnz, cfg);
    P.supernodes = count;
    P.front_rows = std::move(F.front_rows);
    P.child_ptr = std::move(F.child_ptr);
    P.children = std::move(F.children);
    return P;
}

}  // namespace uchol_dev
