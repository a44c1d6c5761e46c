// Approximate minimum degree ordering on a quotient graph.
//
// The ordering decides the whole factor structure, so it has to reproduce
// the reference ordering exactly (CAESolvers/AMD/ApproximateMinimumDegreeOrdering.cs
// and its helpers FactorGraph.cs, DegreeBuckets.cs, HashBuckets.cs,
// MemberLists.cs).  The tie-breaking rules that matter are kept:
//   * degree lists are LIFO with a moving lower bound (DegreeBuckets.cs:57-114);
//   * supervariable detection hashes with `hash % n` and scans buckets in
//     first-use order (HashBuckets.cs:54-67, ApproximateMinimumDegreeOrdering.cs:531-592);
//   * compaction moves live lists in ascending start order (FactorGraph.cs:95-143);
//   * dense rows (degree > max(16, 10 sqrt n), capped at n) are ordered last
//     and isolated vertices first (ApproximateMinimumDegreeOrdering.cs:231-269).
#include <algorithm>
#include <climits>
#include <cmath>

#include "symbolic.hpp"

namespace uchol {
namespace {

constexpr int kNone = -1;
inline int flip(int i) { return -i - 2; }

// Doubly linked degree lists with a lower bound on the smallest non-empty list.
struct DegreeLists {
    std::vector<int> head, next, prev;
    int lowest = 0;
    explicit DegreeLists(int n) : head(n + 1, kNone), next(n, kNone), prev(n, kNone) {}
    void insert(int v, int d) {
        int h = head[d];
        if (h != kNone) prev[h] = v;
        next[v] = h;
        prev[v] = kNone;
        head[d] = v;
        if (d < lowest) lowest = d;
    }
    void remove(int v, int d) {
        int p = prev[v], q = next[v];
        if (q != kNone) prev[q] = p;
        if (p != kNone) next[p] = q; else head[d] = q;
    }
    int pop_min(int max_degree) {
        for (int d = lowest; d <= max_degree; ++d) {
            int v = head[d];
            if (v == kNone) continue;
            lowest = d;
            int q = next[v];
            if (q != kNone) prev[q] = kNone;
            head[d] = q;
            return v;
        }
        throw std::runtime_error("AMD: no vertex left to eliminate in a non-empty graph (internal error)");
    }
};

// Chained hash table over the variables of the newest element.
struct HashChains {
    std::vector<int> head, next, prev, used;
    int used_count = 0;
    int n;
    explicit HashChains(int n_) : head(n_, kNone), next(n_, kNone), prev(n_, kNone), used(n_, 0), n(n_) {}
    void add(long long hash, int v) {
        int b = static_cast<int>(hash % n);
        int h = head[b];
        if (h == kNone) used[used_count++] = b; else prev[h] = v;
        next[v] = h;
        prev[v] = kNone;
        head[b] = v;
    }
    void unlink(int v) {  // v is never a chain head here
        int p = prev[v], q = next[v];
        next[p] = q;
        if (q != kNone) prev[q] = p;
    }
};

class AmdState {
public:
    explicit AmdState(const AdjacencyGraph& g)
        : n_(g.n), nv_(n_, 1), degree_(n_), w_(n_, 1), lists_(n_), chains_(n_),
          member_head_(n_), member_tail_(n_), member_next_(n_, kNone), dense_(n_), perm_(n_) {
        const int edges = static_cast<int>(g.adj.size());
        iw_len_ = edges + edges / 5 + n_ + 16;
        iw_.assign(static_cast<size_t>(iw_len_), 0);
        std::copy(g.adj.begin(), g.adj.end(), iw_.begin());
        pfree_ = edges;
        pe_.resize(n_);
        len_.resize(n_);
        elen_.assign(n_, 0);
        for (int i = 0; i < n_; ++i) {
            pe_[i] = g.ptr[i];
            len_[i] = g.ptr[i + 1] - g.ptr[i];
            degree_[i] = len_[i];
            member_head_[i] = member_tail_[i] = i;
        }
        wbig_ = INT_MAX - n_ - 1;
    }

    std::vector<int> run() {
        int eliminated = initial_lists();
        wflg_ = 2;
        lists_.lowest = 0;
        int max_element = 0;
        while (eliminated < n_) {
            reserve_marks(2 * n_ + 2);
            const int pivot = lists_.pop_min(n_);
            const int pivot_elen = elen_[pivot];
            int pivot_nv = nv_[pivot];
            eliminated += pivot_nv;
            nv_[pivot] = -pivot_nv;

            int elem_degree, first, last;
            if (pivot_elen == 0) element_from_variables(pivot, elem_degree, first, last);
            else element_from_elements(pivot, pivot_elen, elem_degree, first, last);

            pe_[pivot] = first;
            len_[pivot] = last - first + 1;

            outside_counts(first, last);
            approximate_degrees(pivot, first, last, elem_degree, pivot_nv, eliminated);

            degree_[pivot] = elem_degree;
            elen_[pivot] = flip(pivot_nv + elem_degree);
            max_element = std::max(max_element, elem_degree);

            merge_indistinguishable();
            relink_degrees(pivot, pivot_elen, elem_degree, pivot_nv, eliminated, first, last);
            emit(pivot);
            wflg_ += max_element + 1;
        }
        for (int t = 0; t < dense_count_; ++t) emit(dense_[t]);
        if (written_ != n_)
            throw std::runtime_error("AMD: incomplete permutation (internal error)");
        return perm_;
    }

private:
    int n_;
    std::vector<int> iw_;
    int iw_len_ = 0, pfree_ = 0;
    std::vector<int> pe_, len_, elen_;
    std::vector<int> nv_, degree_, w_;
    int wflg_ = 0, wbig_ = 0;
    DegreeLists lists_;
    HashChains chains_;
    std::vector<int> member_head_, member_tail_, member_next_;
    std::vector<int> dense_;
    int dense_count_ = 0;
    std::vector<int> perm_;
    int written_ = 0;
    std::vector<int> compact_keys_, compact_order_;

    void append_members(int target, int source) {
        member_next_[member_tail_[target]] = member_head_[source];
        member_tail_[target] = member_tail_[source];
    }
    void emit(int rep) {
        for (int v = member_head_[rep]; v != kNone; v = member_next_[v]) perm_[written_++] = v;
    }

    int initial_lists() {
        int dense = static_cast<int>(10.0 * std::sqrt(static_cast<double>(n_)));
        dense = std::max(16, dense);
        dense = std::min(n_, dense);
        int eliminated = 0;
        for (int i = 0; i < n_; ++i) {
            int d = degree_[i];
            if (d == 0) {
                pe_[i] = kNone;
                w_[i] = 0;
                nv_[i] = 0;
                elen_[i] = kNone;
                ++eliminated;
                emit(i);
            } else if (d > dense) {
                pe_[i] = kNone;
                nv_[i] = 0;
                elen_[i] = kNone;
                ++eliminated;
                dense_[dense_count_++] = i;
            } else {
                lists_.insert(i, d);
            }
        }
        return eliminated;
    }

    void reserve_marks(int required) {
        if (static_cast<long long>(wflg_) + required < wbig_) return;
        for (int x = 0; x < n_; ++x)
            if (w_[x] != 0) w_[x] = 1;
        wflg_ = 2;
    }

    // Pivot without adjacent elements: the new element is written over the
    // pivot's own variable list.
    void element_from_variables(int pivot, int& elem_degree, int& first, int& last) {
        elem_degree = 0;
        first = pe_[pivot];
        last = first - 1;
        const int end = first + len_[pivot];
        for (int p = first; p < end; ++p) {
            int i = iw_[p];
            int nvi = nv_[i];
            if (nvi <= 0) continue;
            elem_degree += nvi;
            nv_[i] = -nvi;
            iw_[++last] = i;
            lists_.remove(i, degree_[i]);
        }
    }

    // Compacts the workspace, moving every live list to the front in order of
    // its start; the element under construction (first .. pfree) follows them.
    void compact(int& first) {
        if (compact_keys_.empty()) {
            compact_keys_.resize(n_);
            compact_order_.resize(n_);
        }
        int count = 0;
        for (int j = 0; j < n_; ++j)
            if (pe_[j] >= 0 && len_[j] > 0) {
                compact_keys_[count] = pe_[j];
                compact_order_[count] = j;
                ++count;
            }
        // Start positions of live lists are distinct, so any sort agrees.
        std::vector<std::pair<int, int>> order(count);
        for (int t = 0; t < count; ++t) order[t] = {compact_keys_[t], compact_order_[t]};
        std::sort(order.begin(), order.end());
        int dst = 0;
        for (int t = 0; t < count; ++t) {
            int j = order[t].second;
            int src = pe_[j], length = len_[j];
            if (dst != src) std::copy(iw_.begin() + src, iw_.begin() + src + length, iw_.begin() + dst);
            pe_[j] = dst;
            dst += length;
        }
        int partial = pfree_ - first;
        if (partial > 0 && dst != first)
            std::copy(iw_.begin() + first, iw_.begin() + first + partial, iw_.begin() + dst);
        first = dst;
        pfree_ = dst + partial;
        int required = pfree_ + n_ + 16;
        if (required > iw_len_) {
            iw_len_ = std::max(required, iw_len_ + iw_len_ / 2);
            iw_.resize(static_cast<size_t>(iw_len_), 0);
        }
    }

    // General case: the new element is the union of all adjacent elements and
    // the pivot's live variables, built in the free tail of the workspace;
    // every adjacent element is absorbed.
    void element_from_elements(int pivot, int pivot_elen, int& elem_degree, int& first, int& last) {
        elem_degree = 0;
        int p = pe_[pivot];
        first = pfree_;
        const int own_variables = len_[pivot] - pivot_elen;
        for (int outer = 1; outer <= pivot_elen + 1; ++outer) {
            const bool own = outer > pivot_elen;
            int e, cursor, count;
            if (own) {
                e = pivot;
                cursor = p;
                count = own_variables;
            } else {
                e = iw_[p++];
                cursor = pe_[e];
                count = len_[e];
            }
            for (int inner = 1; inner <= count; ++inner) {
                int i = iw_[cursor++];
                int nvi = nv_[i];
                if (nvi <= 0) continue;
                if (pfree_ >= iw_len_) {
                    if (!own) {
                        pe_[pivot] = p;
                        len_[pivot] = (pivot_elen - outer) + own_variables;
                        if (len_[pivot] == 0) pe_[pivot] = kNone;
                    }
                    pe_[e] = cursor;
                    len_[e] = count - inner;
                    if (len_[e] == 0) pe_[e] = kNone;
                    compact(first);
                    cursor = pe_[e];
                    p = own ? cursor : pe_[pivot];
                }
                elem_degree += nvi;
                nv_[i] = -nvi;
                iw_[pfree_++] = i;
                lists_.remove(i, degree_[i]);
            }
            if (e != pivot) {
                pe_[e] = flip(pivot);
                w_[e] = 0;
            }
        }
        last = pfree_ - 1;
    }

    // Pass 1: w[e] - wflg becomes |Le \ Lme| for every element e adjacent to
    // a variable of the new element.
    void outside_counts(int first, int last) {
        for (int pos = first; pos <= last; ++pos) {
            int i = iw_[pos];
            int ecount = elen_[i];
            if (ecount <= 0) continue;
            int nvi = -nv_[i];
            int wnvi = wflg_ - nvi;
            int end = pe_[i] + ecount;
            for (int p = pe_[i]; p < end; ++p) {
                int e = iw_[p];
                int we = w_[e];
                if (we >= wflg_) we -= nvi;
                else if (we != 0) we = degree_[e] + wnvi;
                w_[e] = we;
            }
        }
    }

    // Pass 2: approximate external degrees, aggressive absorption, mass
    // elimination and hashing of the survivors.
    void approximate_degrees(int pivot, int first, int last, int& elem_degree, int& pivot_nv, int& eliminated) {
        chains_.used_count = 0;
        for (int pos = first; pos <= last; ++pos) {
            int i = iw_[pos];
            int start = pe_[i];
            int elem_end = start + elen_[i];
            int write = start;
            long long hash = 0;
            int deg = 0;
            for (int p = start; p < elem_end; ++p) {
                int e = iw_[p];
                if (w_[e] == 0) continue;
                int external = w_[e] - wflg_;
                if (external > 0) {
                    deg += external;
                    iw_[write++] = e;
                    hash += e;
                } else if (external == 0) {
                    pe_[e] = flip(pivot);
                    w_[e] = 0;
                }
            }
            elen_[i] = write - start + 1;
            int var_start = write;
            int list_end = start + len_[i];
            for (int p = elem_end; p < list_end; ++p) {
                int j = iw_[p];
                int nvj = nv_[j];
                if (nvj <= 0) continue;
                deg += nvj;
                iw_[write++] = j;
                hash += j;
            }
            if (elen_[i] == 1 && var_start == write) {
                pe_[i] = flip(pivot);
                int nvi = -nv_[i];
                elem_degree -= nvi;
                pivot_nv += nvi;
                eliminated += nvi;
                nv_[i] = 0;
                elen_[i] = kNone;
                append_members(pivot, i);
            } else {
                degree_[i] = std::min(degree_[i], deg);
                iw_[write] = iw_[var_start];
                iw_[var_start] = iw_[start];
                iw_[start] = pivot;
                len_[i] = write - start + 1;
                chains_.add(hash, i);
            }
        }
    }

    // Merges variables of the new element whose adjacency lists coincide.
    void merge_indistinguishable() {
        for (int b = 0; b < chains_.used_count; ++b) {
            int bucket = chains_.used[b];
            for (int i = chains_.head[bucket]; i != kNone; i = chains_.next[i]) {
                if (nv_[i] >= 0) continue;
                int length = len_[i];
                int ecount = elen_[i];
                for (int p = pe_[i] + 1; p < pe_[i] + length; ++p) w_[iw_[p]] = wflg_;
                int j = chains_.next[i];
                while (j != kNone) {
                    bool same = nv_[j] < 0 && len_[j] == length && elen_[j] == ecount;
                    if (same) {
                        for (int p = pe_[j] + 1; p < pe_[j] + length; ++p)
                            if (w_[iw_[p]] != wflg_) { same = false; break; }
                    }
                    int following = chains_.next[j];
                    if (same) {
                        pe_[j] = flip(i);
                        nv_[i] += nv_[j];
                        nv_[j] = 0;
                        elen_[j] = kNone;
                        append_members(i, j);
                        chains_.unlink(j);
                    }
                    j = following;
                }
                ++wflg_;
            }
            chains_.head[bucket] = kNone;
        }
    }

    void relink_degrees(int pivot, int pivot_elen, int elem_degree, int pivot_nv, int eliminated,
                        int first, int last) {
        int write = first;
        int remaining = n_ - eliminated;
        for (int pos = first; pos <= last; ++pos) {
            int i = iw_[pos];
            int nvi = -nv_[i];
            if (nvi <= 0) continue;
            nv_[i] = nvi;
            int deg = degree_[i] + elem_degree - nvi;
            deg = std::min(deg, remaining - nvi);
            if (deg < 0) deg = 0;
            degree_[i] = deg;
            lists_.insert(i, deg);
            iw_[write++] = i;
        }
        nv_[pivot] = pivot_nv;
        len_[pivot] = write - first;
        if (len_[pivot] == 0) {
            pe_[pivot] = kNone;
            w_[pivot] = 0;
        }
        if (pivot_elen != 0) pfree_ = write;
    }
};

}  // namespace

std::vector<int> amd_order(const AdjacencyGraph& g) {
    if (g.n == 0) return {};
    AmdState state(g);
    return state.run();
}

}  // namespace uchol
