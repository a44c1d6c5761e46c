// Permuted pattern, elimination tree, column counts, supernodes, slab layout
// and the Analyze driver.  Integer-only; every array must match the reference
// symbolic phase exactly, so the traversal orders below follow it.
#include "symbolic.hpp"

#include <algorithm>
#include <numeric>

namespace uchol {

namespace {
constexpr int kNone = -1;

std::vector<int> invert(const std::vector<int>& perm) {
    std::vector<int> inv(perm.size());
    for (size_t k = 0; k < perm.size(); ++k) inv[perm[k]] = static_cast<int>(k);
    return inv;
}
}  // namespace

// PermutedSymmetricPattern.cs:81-184: two passes over the stored upper half,
// then every column is sorted (keys are unique row numbers).
PermutedPattern permute_pattern(int n, const int* row_ptr, const int* col, const std::vector<int>& inv) {
    if (static_cast<int>(inv.size()) != n) throw std::invalid_argument("permutation length does not match the matrix size");
    PermutedPattern pp;
    pp.n = n;
    pp.ptr.assign(n + 1, 0);
    pp.lower_value_ptr.assign(n + 1, 0);
    pp.diag_value_index.assign(n, kNone);
    for (int r = 0; r < n; ++r) {
        int pr = inv[r];
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            if (c == r) { pp.diag_value_index[pr] = k; continue; }
            int pc = inv[c];
            pp.ptr[pr + 1]++;
            pp.ptr[pc + 1]++;
            pp.lower_value_ptr[std::min(pr, pc) + 1]++;
        }
    }
    for (int j = 0; j < n; ++j) {
        pp.ptr[j + 1] += pp.ptr[j];
        pp.lower_value_ptr[j + 1] += pp.lower_value_ptr[j];
    }
    pp.rows.assign(pp.ptr[n], 0);
    pp.lower_value_index.assign(pp.lower_value_ptr[n], 0);
    std::vector<int> lower_rows(pp.lower_value_ptr[n]);
    std::vector<int> fill(pp.ptr.begin(), pp.ptr.end() - 1);
    std::vector<int> lower_fill(pp.lower_value_ptr.begin(), pp.lower_value_ptr.end() - 1);
    for (int r = 0; r < n; ++r) {
        int pr = inv[r];
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            if (c == r) continue;
            int pc = inv[c];
            pp.rows[fill[pr]++] = pc;
            pp.rows[fill[pc]++] = pr;
            int lo = std::min(pr, pc), hi = pr + pc - lo;
            int pos = lower_fill[lo]++;
            lower_rows[pos] = hi;
            pp.lower_value_index[pos] = k;
        }
    }
    std::vector<std::pair<int, int>> tmp;
    for (int j = 0; j < n; ++j) {
        std::sort(pp.rows.begin() + pp.ptr[j], pp.rows.begin() + pp.ptr[j + 1]);
        int b = pp.lower_value_ptr[j], e = pp.lower_value_ptr[j + 1];
        if (e - b > 1) {
            tmp.resize(e - b);
            for (int t = b; t < e; ++t) tmp[t - b] = {lower_rows[t], pp.lower_value_index[t]};
            std::sort(tmp.begin(), tmp.end());
            for (int t = b; t < e; ++t) pp.lower_value_index[t] = tmp[t - b].second;
        }
    }
    pp.lower_start.resize(n);
    for (int j = 0; j < n; ++j)
        pp.lower_start[j] = pp.ptr[j + 1] - (pp.lower_value_ptr[j + 1] - pp.lower_value_ptr[j]);
    return pp;
}

// EliminationTree.cs:39-71 (Liu's algorithm with path compression through ancestor[]).
std::vector<int> etree_build(int n, const std::vector<int>& ptr, const std::vector<int>& rows) {
    std::vector<int> parent(n, kNone), ancestor(n, kNone);
    for (int k = 0; k < n; ++k) {
        for (int p = ptr[k]; p < ptr[k + 1]; ++p) {
            int i = rows[p];
            if (i >= k) break;
            while (i != kNone && i < k) {
                int up = ancestor[i];
                ancestor[i] = k;
                if (up == kNone) parent[i] = k;
                i = up;
            }
        }
    }
    return parent;
}

// EliminationTree.cs:80-130: children visited in ascending order, explicit stack.
std::vector<int> etree_postorder(int n, const std::vector<int>& parent) {
    std::vector<int> head(n, kNone), next(n, kNone), stack(n), post(n);
    for (int j = n - 1; j >= 0; --j) {
        if (parent[j] == kNone) continue;
        next[j] = head[parent[j]];
        head[parent[j]] = j;
    }
    int written = 0;
    for (int root = 0; root < n; ++root) {
        if (parent[root] != kNone) continue;
        int top = 0;
        stack[0] = root;
        while (top >= 0) {
            int v = stack[top];
            int c = head[v];
            if (c == kNone) {
                --top;
                post[written++] = v;
            } else {
                head[v] = next[c];
                stack[++top] = c;
            }
        }
    }
    return post;
}

// EliminationTree.cs:152-249 (Gilbert-Ng-Peyton column counts, symmetric case).
std::vector<int> etree_column_counts(int n, const std::vector<int>& ptr, const std::vector<int>& rows,
                                     const std::vector<int>& parent, const std::vector<int>& post) {
    std::vector<int> delta(n, 0), ancestor(n), max_first(n, kNone), prev_leaf(n, kNone), first(n, kNone);
    for (int k = 0; k < n; ++k) {
        int j = post[k];
        delta[j] = first[j] == kNone ? 1 : 0;
        for (; j != kNone && first[j] == kNone; j = parent[j]) first[j] = k;
    }
    std::iota(ancestor.begin(), ancestor.end(), 0);
    for (int k = 0; k < n; ++k) {
        int j = post[k];
        if (parent[j] != kNone) delta[parent[j]]--;
        for (int p = ptr[j]; p < ptr[j + 1]; ++p) {
            int i = rows[p];
            if (i <= j || first[j] <= max_first[i]) continue;
            max_first[i] = first[j];
            int jprev = prev_leaf[i];
            prev_leaf[i] = j;
            delta[j]++;
            if (jprev == kNone) continue;
            int root = jprev;
            while (root != ancestor[root]) root = ancestor[root];
            for (int s = jprev; s != root;) {
                int up = ancestor[s];
                ancestor[s] = root;
                s = up;
            }
            delta[root]--;
        }
        if (parent[j] != kNone) ancestor[j] = parent[j];
    }
    for (int j = 0; j < n; ++j)
        if (parent[j] != kNone) delta[parent[j]] += delta[j];
    return delta;
}

namespace {

// SupernodalStructure.cs:175-193.
std::vector<int> fundamental_starts(int n, const std::vector<int>& parent, const std::vector<int>& cc,
                                    const std::vector<int>& child_count) {
    std::vector<int> starts;
    for (int j = 0; j < n; ++j) {
        bool fresh = j == 0 || parent[j - 1] != j || child_count[j] > 1 || cc[j - 1] != cc[j] + 1;
        if (fresh) starts.push_back(j);
    }
    starts.push_back(n);
    return starts;
}

// SupernodalStructure.cs:271-286: graded explicit-zero tolerance.
bool merge_worthwhile(int columns, int64_t added_zeros, int64_t stored) {
    if (added_zeros <= 0) return true;
    double fraction = static_cast<double>(added_zeros) / static_cast<double>(stored);
    if (columns <= 4) return fraction <= 0.8;
    if (columns <= 16) return fraction <= 0.1;
    if (columns <= 48) return fraction <= 0.05;
    return false;
}

// SupernodalStructure.cs:203-262: relaxed amalgamation up the chain.
std::vector<int> amalgamate(int n, const std::vector<int>& fs, const std::vector<int>& parent,
                            const std::vector<int>& cc, int limit, std::vector<int>& front_sizes) {
    int fcount = static_cast<int>(fs.size()) - 1;
    std::vector<int64_t> prefix(n + 1, 0);
    for (int j = 0; j < n; ++j) prefix[j + 1] = prefix[j] + cc[j];
    std::vector<int> bounds;
    front_sizes.clear();
    int index = 0;
    while (index < fcount) {
        int first = fs[index];
        int last = fs[index + 1] - 1;
        int columns = last - first + 1;
        int front = cc[first];
        int64_t nonzeros = prefix[last + 1] - prefix[first];
        while (index + 1 < fcount) {
            if (parent[last] != last + 1) break;
            int next_last = fs[index + 2] - 1;
            int next_first = fs[index + 1];
            int merged_columns = columns + (next_last - next_first + 1);
            if (merged_columns > limit) break;
            int64_t merged_front = static_cast<int64_t>(columns) + cc[next_first];
            int64_t stored = merged_front * merged_columns - static_cast<int64_t>(merged_columns) * (merged_columns - 1) / 2;
            int64_t merged_nonzeros = nonzeros + (prefix[next_last + 1] - prefix[next_first]);
            if (!merge_worthwhile(merged_columns, stored - merged_nonzeros, stored)) break;
            last = next_last;
            columns = merged_columns;
            front = static_cast<int>(merged_front);
            nonzeros = merged_nonzeros;
            ++index;
        }
        bounds.push_back(first);
        front_sizes.push_back(front);
        ++index;
    }
    bounds.push_back(n);
    return bounds;
}

}  // namespace

Supernodes build_supernodes(const PermutedPattern& pattern, const std::vector<int>& parent,
                            const std::vector<int>& cc, int limit) {
    const int n = pattern.n;
    std::vector<int> child_count(n, 0);
    for (int j = 0; j < n; ++j)
        if (parent[j] >= 0) child_count[parent[j]]++;
    std::vector<int> front_sizes;
    auto fs = fundamental_starts(n, parent, cc, child_count);
    Supernodes sn;
    sn.n = n;
    sn.first_column = amalgamate(n, fs, parent, cc, limit, front_sizes);
    const int count = sn.count();

    sn.supernode_of.assign(n, 0);
    for (int s = 0; s < count; ++s)
        for (int j = sn.first_column[s]; j < sn.first_column[s + 1]; ++j) sn.supernode_of[j] = s;

    sn.parent.assign(count, kNone);
    std::vector<int> kids(count, 0);
    for (int s = 0; s < count; ++s) {
        int pc = parent[sn.first_column[s + 1] - 1];
        sn.parent[s] = pc < 0 ? kNone : sn.supernode_of[pc];
        if (sn.parent[s] >= 0) kids[sn.parent[s]]++;
    }
    sn.child_ptr.assign(count + 1, 0);
    for (int s = 0; s < count; ++s) sn.child_ptr[s + 1] = sn.child_ptr[s] + kids[s];
    sn.children.assign(count == 0 ? 0 : sn.child_ptr[count], 0);
    std::vector<int> cursor(sn.child_ptr.begin(), sn.child_ptr.end() - 1);
    for (int s = 0; s < count; ++s)
        if (sn.parent[s] >= 0) sn.children[cursor[sn.parent[s]]++] = s;

    sn.pattern_ptr.assign(count + 1, 0);
    for (int s = 0; s < count; ++s) sn.pattern_ptr[s + 1] = sn.pattern_ptr[s] + front_sizes[s];
    sn.pattern_rows.assign(count == 0 ? 0 : sn.pattern_ptr[count], 0);

    // Row structure of each supernode: own columns, lower parts of its
    // columns, then the trailing rows of every child (SupernodalStructure.cs:296-355).
    std::vector<int> flag(n, kNone);
    for (int s = 0; s < count; ++s) {
        int first = sn.first_column[s], last = sn.first_column[s + 1] - 1;
        int write = sn.pattern_ptr[s];
        for (int j = first; j <= last; ++j) {
            flag[j] = s;
            sn.pattern_rows[write++] = j;
        }
        for (int j = first; j <= last; ++j)
            for (int p = pattern.lower_start[j]; p < pattern.ptr[j + 1]; ++p) {
                int r = pattern.rows[p];
                if (flag[r] == s) continue;
                flag[r] = s;
                if (write >= sn.pattern_ptr[s + 1])
                    throw std::runtime_error("symbolic phase: front size prediction exceeded (internal error)");
                sn.pattern_rows[write++] = r;
            }
        // the rows so far in any order; each child's trailing rows follow as a segment in its
        // own (ascending) order, so the distinct rows are sorted by one small sort and a merge
        // per child instead of a sort of the whole front
        auto base = sn.pattern_rows.begin() + sn.pattern_ptr[s];
        std::sort(base, sn.pattern_rows.begin() + write);
        for (int c = sn.child_ptr[s]; c < sn.child_ptr[s + 1]; ++c) {
            int child = sn.children[c];
            const int seg = write;
            for (int q = sn.pattern_ptr[child] + sn.width(child); q < sn.pattern_ptr[child + 1]; ++q) {
                int r = sn.pattern_rows[q];
                if (flag[r] == s) continue;
                flag[r] = s;
                if (write >= sn.pattern_ptr[s + 1])
                    throw std::runtime_error("symbolic phase: front size prediction exceeded (internal error)");
                sn.pattern_rows[write++] = r;
            }
            std::inplace_merge(base, sn.pattern_rows.begin() + seg, sn.pattern_rows.begin() + write);
        }
        if (write != sn.pattern_ptr[s + 1])
            throw std::runtime_error("symbolic phase: predicted front size of supernode " + std::to_string(s) +
                                     " does not match the actual one (internal error)");
    }

    // Costs and the exact peak of live contribution blocks (SupernodalStructure.cs:370-418).
    std::vector<int64_t> contribution(count, 0);
    int64_t live = 0, peak = 0;
    for (int s = 0; s < count; ++s) {
        int64_t m = sn.front_size(s), w = sn.width(s);
        sn.factor_entry_count += m * w - w * (w - 1) / 2;
        for (int64_t k = 0; k < w; ++k) sn.factor_operation_count += (m - k) * (m - k);
        sn.max_front_size = std::max<int>(sn.max_front_size, static_cast<int>(m));
        sn.max_supernode_width = std::max<int>(sn.max_supernode_width, static_cast<int>(w));
        peak = std::max(peak, live + m * (m + 1) / 2);
        for (int c = sn.child_ptr[s]; c < sn.child_ptr[s + 1]; ++c) live -= contribution[sn.children[c]];
        int64_t t = m - w;
        contribution[s] = t * (t + 1) / 2;
        live += contribution[s];
        peak = std::max(peak, live);
    }
    sn.peak_contribution_entries = peak;
    return sn;
}

FactorLayout build_layout(const Supernodes& sn) {
    constexpr int64_t kSlab = int64_t(1) << 23;  // FactorStorageLayout.cs:33
    FactorLayout L;
    const int count = sn.count();
    L.slab_index.resize(count);
    L.slab_offset.resize(count);
    L.block_length.resize(count);
    int slab = 0;
    int64_t used = 0, capacity = 0;
    for (int s = 0; s < count; ++s) {
        int64_t m = sn.front_size(s), w = sn.width(s);
        int64_t length = m * w - w * (w - 1) / 2;
        if (length > INT32_MAX) throw std::length_error("factor block of a supernode exceeds the 32-bit range");
        L.block_length[s] = static_cast<int>(length);
        if (used + length > capacity) {
            if (capacity > 0) {
                L.slab_lengths.push_back(static_cast<int>(used));
                ++slab;
            }
            capacity = std::max(kSlab, length);
            used = 0;
        }
        L.slab_index[s] = slab;
        L.slab_offset[s] = static_cast<int>(used);
        used += length;
    }
    if (capacity > 0) L.slab_lengths.push_back(static_cast<int>(used));
    return L;
}

// UtduSymbolicFactorization.cs:240-295.
Symbolic analyze(int n, const int* row_ptr, const int* col, int nnz, Ordering ordering, int amalgamation_limit) {
    std::vector<int> fill_reducing(n);
    if (ordering == Ordering::ApproximateMinimumDegree) {
        AdjacencyGraph g = adjacency_from_upper(n, row_ptr, col);
        fill_reducing = amd_order(g);
    } else {
        std::iota(fill_reducing.begin(), fill_reducing.end(), 0);
    }
    return analyze_ordered(n, row_ptr, col, nnz, fill_reducing, amalgamation_limit);
}

// The same analysis from a given fill-reducing order (position -> original index).
Symbolic analyze_ordered(int n, const int* row_ptr, const int* col, int nnz, const std::vector<int>& fill_reducing,
                         int amalgamation_limit) {
    Symbolic S;
    S.n = n;
    S.matrix_nonzero_count = nnz;
    if ((int)fill_reducing.size() != n) throw std::invalid_argument("ordering length does not match the matrix size");
    // Postorder the elimination tree of the ordered matrix so that every
    // supernode and every subtree occupies a contiguous column range.
    std::vector<int> first_inv = invert(fill_reducing);
    PermutedPattern first_pattern = permute_pattern(n, row_ptr, col, first_inv);
    std::vector<int> first_parent = etree_build(n, first_pattern.ptr, first_pattern.rows);
    std::vector<int> post = etree_postorder(n, first_parent);
    S.permutation.resize(n);
    for (int k = 0; k < n; ++k) S.permutation[k] = fill_reducing[post[k]];
    S.inverse_permutation = invert(S.permutation);
    std::vector<int> final_post;
    bool post_is_identity = true;
    for (int k = 0; k < n && post_is_identity; ++k) post_is_identity = post[k] == k;
    if (post_is_identity) {
        // the order is already a postorder (a chain, for instance): the second pass would
        // rebuild the same pattern, tree and postorder
        S.pattern = std::move(first_pattern);
        S.etree_parent = std::move(first_parent);
        final_post = std::move(post);
    } else {
        S.pattern = permute_pattern(n, row_ptr, col, S.inverse_permutation);
        S.etree_parent = etree_build(n, S.pattern.ptr, S.pattern.rows);
        final_post = etree_postorder(n, S.etree_parent);
    }
    S.column_counts = etree_column_counts(n, S.pattern.ptr, S.pattern.rows, S.etree_parent, final_post);
    S.supernodes = build_supernodes(S.pattern, S.etree_parent, S.column_counts, std::max(1, amalgamation_limit));
    for (int j = 0; j < n; ++j) S.strict_factor_nonzero_count += S.column_counts[j];
    S.layout = build_layout(S.supernodes);
    return S;
}

}  // namespace uchol
