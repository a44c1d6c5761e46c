// ORACLE — test infrastructure only.  CPU restatement of the MAGLA UCHOL
// numeric phase (supernodal multifrontal U^T D U factorisation and the
// forward / diagonal / backward solves).  Only the test-suite, the smoke
// check and the CPU-baseline leg of the benchmark load this library; the
// product never does.
//
// It follows CAESolvers/UCHOL/UtduNumericFactorization.cs step for step:
//   * packed lower-triangular column-major fronts, column k of a front of
//     size m holding m - k entries (ColumnOffset, :213-214, :437-440);
//   * assembly of A through DiagonalValueIndices / LowerValueIndices and the
//     extend-add of each child's packed contribution (:449-509);
//   * panels of PanelWidth pivots with the pivot test !(d > tol * scale),
//     regularisation or failure, scaling by 1/d and the intra-panel
//     right-looking updates (:541-601);
//   * the rank-P trailing update with the panel x D packed in blocks of
//     RowBlock = 128 rows, four result columns per register tile, the
//     triangular corner and single-column remainders (:624-852);
//   * a ready stack of leaf supernodes, child counters and worker threads
//     (:313-379, :943-1023), with the second level of parallelism inside
//     large trailing updates (:660-672);
//   * the supernodal forward / backward substitutions (:139-207).
// The element arithmetic keeps the reference's mul-then-add (no fused
// multiply-add: compiled with -ffp-contract=off) and its summation orders;
// the vectorised dot product uses four lanes (Vector<double>.Count on AVX2
// x64) folded lane 0..3, DenseKernels.cs:91-113.
//
// Symbolic arrays are inputs (they come from the host symbolic phase, as
// the reference's numeric phase receives a UtduSymbolicFactorization).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kRowBlock = 128;   // UtduNumericFactorization.cs:619
constexpr int kColumnTile = 4;   // UtduNumericFactorization.cs:622
constexpr int kLanes = 4;        // Vector<double>.Count assumed for the dot product

struct Sym {
    int n, count;
    const int* diag_value_index;
    const int* pattern_ptr;
    const int* pattern_rows;
    const int* lower_start;
    const int* lower_value_ptr;
    const int* lower_value_index;
    const int* first_column;
    const int* parent;
    const int* child_ptr;
    const int* children;
    const int* front_ptr;
    const int* front_rows;
    int width(int s) const { return first_column[s + 1] - first_column[s]; }
    int front(int s) const { return front_ptr[s + 1] - front_ptr[s]; }
};

struct Options {
    int allow_regularization;
    double pivot_tolerance;
    double diagonal_regularization;
    int panel_width;
    long long parallel_threshold;
    int workers;
};

struct Stats {
    int regularized = 0, negative = 0;
    double smallest = 1.7976931348623157e308, largest = 0.0;
    void observe(double p) {
        double a = std::fabs(p);
        if (a < smallest) smallest = a;
        if (a > largest) largest = a;
    }
};

struct Failure : std::exception {
    std::string msg;
    int column;
    explicit Failure(std::string m, int c) : msg(std::move(m)), column(c) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

// target[t] -= source[t] * f, DenseKernels.SubtractScaled
inline void subtract_scaled(double* target, const double* source, int length, double f) {
    for (int t = 0; t < length; ++t) target[t] = target[t] - source[t] * f;
}
inline void scale(double* x, int length, double f) {
    for (int t = 0; t < length; ++t) x[t] = x[t] * f;
}
// DenseKernels.Dot with kLanes accumulators folded in lane order.
inline double dot(const double* a, const double* b, int length) {
    int t = 0;
    double sum = 0.0;
    if (length >= kLanes) {
        double acc[kLanes] = {0.0, 0.0, 0.0, 0.0};
        for (; t <= length - kLanes; t += kLanes)
            for (int l = 0; l < kLanes; ++l) acc[l] = acc[l] + a[t + l] * b[t + l];
        double s = 0.0;
        for (int l = 0; l < kLanes; ++l) s = s + acc[l] * 1.0;
        sum = s;
    }
    for (; t < length; ++t) sum = sum + a[t] * b[t];
    return sum;
}

// --- trailing update (UpdateTrailingColumns / GatherPanelTile / PanelDot / UpdateColumnTile) ---
void gather_tile(const double* front, const int* off, int ps, int pw, int first, int columns, double* tile) {
    for (int k = 0; k < pw; ++k) {
        int column = ps + k;
        int row_base = off[column] - column;
        for (int t = 0; t < columns; ++t) tile[k * kColumnTile + t] = front[row_base + first + t];
    }
}
inline double panel_dot(const double* buf, int row_index, int pw, const double* tile, int t) {
    double sum = 0.0;
    for (int k = 0; k < pw; ++k) sum = sum + buf[row_index + k * kRowBlock] * tile[k * kColumnTile + t];
    return sum;
}
void update_column_tile(double* front, const int* off, const double* buf, int block_base, int block_first,
                        int from, int to, int pw, int first, const double* tile) {
    const int o0 = off[first] - first, o1 = off[first + 1] - first - 1;
    const int o2 = off[first + 2] - first - 2, o3 = off[first + 3] - first - 3;
    for (int i = from; i < to; ++i) {
        const double* row = buf + block_base + (i - block_first);
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int k = 0; k < pw; ++k) {
            double p = row[k * kRowBlock];
            const double* sc = tile + k * kColumnTile;
            s0 = s0 + p * sc[0];
            s1 = s1 + p * sc[1];
            s2 = s2 + p * sc[2];
            s3 = s3 + p * sc[3];
        }
        front[o0 + i] = front[o0 + i] - s0;
        front[o1 + i] = front[o1 + i] - s1;
        front[o2 + i] = front[o2 + i] - s2;
        front[o3 + i] = front[o3 + i] - s3;
    }
}
void update_trailing(double* front, const int* off, int m, int ps, int pe, const double* buf, int cfrom, int cto) {
    const int pw = pe - ps;
    const int blocks = (m - pe + kRowBlock - 1) / kRowBlock;
    std::vector<double> tile(static_cast<size_t>(pw) * kColumnTile);
    for (int block = 0; block < blocks; ++block) {
        int block_base = block * (kRowBlock * pw);
        int block_first = pe + block * kRowBlock;
        int block_last = std::min(block_first + kRowBlock, m);
        int limit = std::min(cto, block_last);
        int j = cfrom;
        for (; j + kColumnTile - 1 < limit; j += kColumnTile) {
            gather_tile(front, off, ps, pw, j, kColumnTile, tile.data());
            int full_from = std::max(j + kColumnTile - 1, block_first);
            update_column_tile(front, off, buf, block_base, block_first, full_from, block_last, pw, j, tile.data());
            for (int i = std::max(j, block_first); i < full_from; ++i)
                for (int t = 0; t <= i - j; ++t)
                    front[off[j + t] + (i - j - t)] -= panel_dot(buf, block_base + (i - block_first), pw, tile.data(), t);
        }
        for (; j < limit; ++j) {
            gather_tile(front, off, ps, pw, j, 1, tile.data());
            int oj = off[j];
            for (int i = std::max(j, block_first); i < block_last; ++i)
                front[oj + (i - j)] -= panel_dot(buf, block_base + (i - block_first), pw, tile.data(), 0);
        }
    }
}

void apply_panel_update(double* front, const int* off, int m, int ps, int pe, int first_column, const double* diag,
                        double* buf, int inner_degree, long long threshold) {
    const int pw = pe - ps;
    const int trailing = m - pe;
    const int blocks = (trailing + kRowBlock - 1) / kRowBlock;
    for (int block = 0; block < blocks; ++block) {
        int block_base = block * (kRowBlock * pw);
        int block_first = pe + block * kRowBlock;
        int rows = std::min(kRowBlock, m - block_first);
        for (int kk = 0; kk < pw; ++kk) {
            int column = ps + kk;
            int src = off[column] + (block_first - column);
            double piv = diag[first_column + column];
            int dst = block_base + kk * kRowBlock;
            for (int r = 0; r < rows; ++r) buf[dst + r] = front[src + r] * piv;
            for (int r = rows; r < kRowBlock; ++r) buf[dst + r] = 0.0;
        }
    }
    long long work = static_cast<long long>(trailing) * trailing * pw;
    if (inner_degree > 1 && work > threshold) {
        int chunks = std::min(trailing, inner_degree * 8);
        std::atomic<int> next{0};
        auto run = [&] {
            for (int c = next++; c < chunks; c = next++) {
                int from = pe + static_cast<int>(static_cast<long long>(trailing) * c / chunks);
                int to = pe + static_cast<int>(static_cast<long long>(trailing) * (c + 1) / chunks);
                update_trailing(front, off, m, ps, pe, buf, from, to);
            }
        };
        std::vector<std::thread> helpers;
        for (int h = 1; h < inner_degree; ++h) helpers.emplace_back(run);
        run();
        for (auto& t : helpers) t.join();
    } else {
        update_trailing(front, off, m, ps, pe, buf, pe, m);
    }
}

struct Worker {
    std::vector<int> row_map, offsets, relative;
    std::vector<double> panel, front;
    Stats stats;
};

void factorize_front(double* front, const int* off, int m, int w, int first_column, double* diag, Worker& ctx,
                     const Options& o, double scale_value, int pw_opt, int inner_degree) {
    const double threshold = o.pivot_tolerance * scale_value;
    const double reg = o.diagonal_regularization * scale_value;
    for (int ps = 0; ps < w; ps += pw_opt) {
        int pe = std::min(ps + pw_opt, w);
        for (int k = ps; k < pe; ++k) {
            int co = off[k];
            int len = m - k;
            double piv = front[co];
            if (!(piv > threshold)) {
                if (!o.allow_regularization)
                    throw Failure("Pivot in equation " + std::to_string(first_column + k) +
                                  " (in elimination order) is not positive: the matrix is not positive definite.",
                                  first_column + k);
                if (piv < 0.0) ctx.stats.negative++;
                ctx.stats.regularized++;
                piv = reg;
            }
            diag[first_column + k] = piv;
            ctx.stats.observe(piv);
            scale(front + co + 1, len - 1, 1.0 / piv);
            for (int j = k + 1; j < pe; ++j) {
                double f = piv * front[co + (j - k)];
                if (f == 0.0) continue;
                subtract_scaled(front + off[j], front + co + (j - k), m - j, f);
            }
            front[co] = 1.0;
        }
        if (pe < m)
            apply_panel_update(front, off, m, ps, pe, first_column, diag, ctx.panel.data(), inner_degree,
                               o.parallel_threshold);
    }
}

struct Result {
    std::vector<std::vector<double>> blocks;   // packed factor block per supernode
    std::vector<double> diag;
    Stats stats;
};

void factorize_supernode(int s, const Sym& S, const double* values, Result& R,
                         std::vector<std::vector<double>>& updates, Worker& ctx, const Options& o,
                         double scale_value, int pw, int inner_degree) {
    const int first = S.first_column[s];
    const int w = S.width(s);
    const int m = S.front(s);
    const int pstart = S.front_ptr[s];
    const size_t length = static_cast<size_t>(m) * (m + 1) / 2;
    auto& off = ctx.offsets;
    off[0] = 0;
    for (int j = 0; j < m; ++j) off[j + 1] = off[j] + (m - j);
    if (ctx.front.size() < length) ctx.front.resize(length);
    double* front = ctx.front.data();
    std::fill(front, front + length, 0.0);
    for (int t = 0; t < m; ++t) ctx.row_map[S.front_rows[pstart + t]] = t;

    for (int local = 0; local < w; ++local) {
        int column = first + local;
        int di = S.diag_value_index[column];
        if (di >= 0) front[off[local]] += values[di];
        int lb = S.lower_value_ptr[column];
        int start = S.lower_start[column];
        int end = S.pattern_ptr[column + 1];
        int cb = off[local] - local;
        for (int p = start; p < end; ++p) {
            int row = ctx.row_map[S.pattern_rows[p]];
            front[cb + row] += values[S.lower_value_index[lb + (p - start)]];
        }
    }
    for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; ++c) {
        int child = S.children[c];
        auto& upd = updates[child];
        if (upd.empty()) continue;
        int cw = S.width(child);
        int cps = S.front_ptr[child];
        int trailing = S.front(child) - cw;
        for (int a = 0; a < trailing; ++a) ctx.relative[a] = ctx.row_map[S.front_rows[cps + cw + a]];
        size_t src = 0;
        for (int a = 0; a < trailing; ++a) {
            int tc = ctx.relative[a];
            int tb = off[tc] - tc;
            for (int b = a; b < trailing; ++b) front[tb + ctx.relative[b]] += upd[src + (b - a)];
            src += trailing - a;
        }
        std::vector<double>().swap(upd);
    }
    factorize_front(front, off.data(), m, w, first, R.diag.data(), ctx, o, scale_value, pw, inner_degree);
    size_t block_length = static_cast<size_t>(off[w]);
    R.blocks[s].assign(front, front + block_length);
    if (m - w > 0) updates[s].assign(front + block_length, front + length);
}

}  // namespace

struct oracle_factor_s {
    Sym sym;
    std::vector<int> owned;   // copies of the symbolic arrays (keeps the factor self-contained)
    Result result;
    int n;
};

namespace {
thread_local std::string g_error;

std::vector<int> copy_ints(const int* p, size_t n) { return std::vector<int>(p, p + n); }
}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_error.c_str(); }

typedef struct oracle_factor_s* oracle_factor;

// Status: 0 ok, 1 bad argument, 3 pivot rejected (regularisation off), 9 other failure.
int oracle_factorize(int n, int count, const int* diag_value_index, const int* pattern_ptr, const int* pattern_rows,
                     const int* lower_start, const int* lower_value_ptr, const int* lower_value_index,
                     const int* first_column, const int* parent, const int* child_ptr, const int* children,
                     const int* front_ptr, const int* front_rows, int max_front, const double* values,
                     int allow_regularization, double pivot_tolerance, double diagonal_regularization,
                     int panel_width, long long parallel_threshold, int workers, oracle_factor* out,
                     int* regularized, int* negative, double* smallest, double* largest, int* failed_column) {
    if (!out) return 1;
    *failed_column = -1;
    auto* F = new oracle_factor_s;
    F->n = n;
    auto& S = F->sym;
    S.n = n;
    S.count = count;
    // Keep private copies of every symbolic array.
    std::vector<std::vector<int>> keep;
    keep.push_back(copy_ints(diag_value_index, n));
    keep.push_back(copy_ints(pattern_ptr, n + 1));
    keep.push_back(copy_ints(pattern_rows, n ? pattern_ptr[n] : 0));
    keep.push_back(copy_ints(lower_start, n));
    keep.push_back(copy_ints(lower_value_ptr, n + 1));
    keep.push_back(copy_ints(lower_value_index, n ? lower_value_ptr[n] : 0));
    keep.push_back(copy_ints(first_column, count + 1));
    keep.push_back(copy_ints(parent, count));
    keep.push_back(copy_ints(child_ptr, count + 1));
    keep.push_back(copy_ints(children, count ? child_ptr[count] : 0));
    keep.push_back(copy_ints(front_ptr, count + 1));
    keep.push_back(copy_ints(front_rows, count ? front_ptr[count] : 0));
    size_t owned_len = 0;
    for (auto& v : keep) owned_len += v.size();
    F->owned.reserve(owned_len);
    std::vector<size_t> at;
    for (auto& v : keep) {
        at.push_back(F->owned.size());
        F->owned.insert(F->owned.end(), v.begin(), v.end());
    }
    const int* base = F->owned.data();
    S.diag_value_index = base + at[0];
    S.pattern_ptr = base + at[1];
    S.pattern_rows = base + at[2];
    S.lower_start = base + at[3];
    S.lower_value_ptr = base + at[4];
    S.lower_value_index = base + at[5];
    S.first_column = base + at[6];
    S.parent = base + at[7];
    S.child_ptr = base + at[8];
    S.children = base + at[9];
    S.front_ptr = base + at[10];
    S.front_rows = base + at[11];

    Options o{allow_regularization, pivot_tolerance, diagonal_regularization,
              std::min(128, std::max(4, panel_width)), parallel_threshold, std::max(1, workers)};
    auto& R = F->result;
    R.diag.assign(n, 0.0);
    R.blocks.assign(count, {});
    if (count == 0) {
        *out = F;
        *regularized = *negative = 0;
        *smallest = *largest = 0.0;
        return 0;
    }
    // ComputeDiagonalScale: max |A_ii| over the stored diagonal, 1 if zero.
    double scale_value = 0.0;
    for (int j = 0; j < n; ++j)
        if (diag_value_index[j] >= 0) scale_value = std::max(scale_value, std::fabs(values[diag_value_index[j]]));
    if (!(scale_value > 0.0)) scale_value = 1.0;

    const int worker_count = std::min(o.workers, count);
    std::vector<std::vector<double>> updates(count);
    std::vector<int> remaining(count);
    std::vector<int> ready;
    for (int s = 0; s < count; ++s) {
        remaining[s] = S.child_ptr[s + 1] - S.child_ptr[s];
        if (remaining[s] == 0) ready.push_back(s);
    }
    std::mutex mu;
    std::condition_variable cv;
    int completed = 0, active = 0;
    bool stop = false;
    std::exception_ptr failure;
    std::vector<Worker> ctxs(worker_count);

    auto worker = [&](int wi) {
        Worker& ctx = ctxs[wi];
        ctx.row_map.assign(n, 0);
        ctx.offsets.assign(max_front + 1, 0);
        ctx.relative.assign(std::max(1, max_front), 0);
        int blocks = (max_front + kRowBlock - 1) / kRowBlock + 1;
        ctx.panel.assign(std::max(1, blocks * kRowBlock * o.panel_width), 0.0);
        try {
            for (;;) {
                int s;
                int inner;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&] { return stop || !ready.empty(); });
                    if (stop) return;
                    s = ready.back();   // LIFO, as the reference's ConcurrentStack
                    ready.pop_back();
                    ++active;
                    inner = std::max(1, worker_count - active + 1);
                }
                factorize_supernode(s, S, values, R, updates, ctx, o, scale_value, o.panel_width, inner);
                {
                    std::lock_guard<std::mutex> lk(mu);
                    --active;
                    int p = S.parent[s];
                    if (p >= 0 && --remaining[p] == 0) ready.push_back(p);
                    if (++completed == count) stop = true;
                }
                cv.notify_all();
            }
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            if (!failure) failure = std::current_exception();
            stop = true;
            cv.notify_all();
        }
    };
    if (worker_count == 1) {
        worker(0);
    } else {
        std::vector<std::thread> threads;
        for (int wi = 0; wi < worker_count; ++wi) threads.emplace_back(worker, wi);
        for (auto& t : threads) t.join();
    }
    if (failure) {
        try {
            std::rethrow_exception(failure);
        } catch (const Failure& f) {
            g_error = f.msg;
            *failed_column = f.column;
            delete F;
            return 3;
        } catch (const std::exception& e) {
            g_error = e.what();
            delete F;
            return 9;
        }
    }
    Stats total;
    for (auto& c : ctxs) {
        total.regularized += c.stats.regularized;
        total.negative += c.stats.negative;
        total.smallest = std::min(total.smallest, c.stats.smallest);
        total.largest = std::max(total.largest, c.stats.largest);
    }
    if (total.smallest == 1.7976931348623157e308) total.smallest = 0.0;
    R.stats = total;
    *regularized = total.regularized;
    *negative = total.negative;
    *smallest = total.smallest;
    *largest = total.largest;
    *out = F;
    return 0;
}

int oracle_diagonal(oracle_factor f, double* out) {
    if (!f || !out) return 1;
    std::copy(f->result.diag.begin(), f->result.diag.end(), out);
    return 0;
}

// Packed factor block of supernode s (length m*w - w(w-1)/2).
int oracle_block(oracle_factor f, int s, double* out) {
    if (!f || s < 0 || s >= f->sym.count) return 1;
    const auto& b = f->result.blocks[s];
    std::copy(b.begin(), b.end(), out);
    return 0;
}

// x = P U^-1 D^-1 U^-T P^T b (UtduNumericFactorization.Solve, :90-207).
int oracle_solve(oracle_factor f, const int* permutation, const double* b, double* x) {
    if (!f) return 1;
    const Sym& S = f->sym;
    const int n = f->n;
    std::vector<double> work(n);
    for (int i = 0; i < n; ++i) work[i] = b[permutation[i]];
    int max_front = 1;
    for (int s = 0; s < S.count; ++s) max_front = std::max(max_front, S.front(s));
    std::vector<double> scratch(max_front);
    for (int s = 0; s < S.count; ++s) {
        int m = S.front(s), w = S.width(s), ps = S.front_ptr[s];
        const double* block = f->result.blocks[s].data();
        for (int t = 0; t < m; ++t) scratch[t] = work[S.front_rows[ps + t]];
        int offset = 0;
        for (int k = 0; k < w; ++k) {
            int len = m - k;
            double v = scratch[k];
            if (v != 0.0) subtract_scaled(scratch.data() + k + 1, block + offset + 1, len - 1, v);
            offset += len;
        }
        for (int t = 0; t < m; ++t) work[S.front_rows[ps + t]] = scratch[t];
    }
    for (int i = 0; i < n; ++i) work[i] /= f->result.diag[i];
    for (int s = S.count - 1; s >= 0; --s) {
        int m = S.front(s), w = S.width(s), ps = S.front_ptr[s];
        const double* block = f->result.blocks[s].data();
        for (int t = 0; t < m; ++t) scratch[t] = work[S.front_rows[ps + t]];
        for (int k = w - 1; k >= 0; --k) {
            int offset = k * m - k * (k - 1) / 2;
            int len = m - k;
            scratch[k] -= dot(block + offset + 1, scratch.data() + k + 1, len - 1);
        }
        for (int t = 0; t < w; ++t) work[S.front_rows[ps + t]] = scratch[t];
    }
    for (int i = 0; i < n; ++i) x[permutation[i]] = work[i];
    return 0;
}

void oracle_destroy(oracle_factor f) { delete f; }

// Symmetric upper-CSR product y = A x (SymmetricCSRMatrix.Multiply, :259-283)
// and ||b - A x||_2 (UtduNumericFactorization.ResidualNorm, :222-234).
double oracle_residual_norm(int n, const int* row_ptr, const int* col, const double* val, const double* b,
                            const double* x) {
    std::vector<double> y(n, 0.0);
    for (int r = 0; r < n; ++r)
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            double v = val[k];
            y[r] = y[r] + v * x[c];
            if (c != r) y[c] = y[c] + v * x[r];
        }
    double sum = 0.0;
    for (int i = 0; i < n; ++i) {
        double d = b[i] - y[i];
        sum = sum + d * d;
    }
    return std::sqrt(sum);
}

void oracle_multiply(int n, const int* row_ptr, const int* col, const double* val, const double* x, double* y) {
    std::fill(y, y + n, 0.0);
    for (int r = 0; r < n; ++r)
        for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k) {
            int c = col[k];
            double v = val[k];
            y[r] = y[r] + v * x[c];
            if (c != r) y[c] = y[c] + v * x[r];
        }
}

}  // extern "C"
