// Linear-dependency presolve: remove the rows of A that are linear
// combinations of other rows, after checking that b agrees (else the LP is
// infeasible).  Same purpose, tolerances and first stage as the reference's
// Presolve_Lindep.cpp (empty rows, a triangular crash, then a numerical test
// of the rows the crash leaves; TOLAPIV and TOLPRIMAL = 1e-8, LP.h:95-96),
// which tests those rows against a basis factorised with LUSOL; here they are
// reduced against the crash's triangular block and eliminated directly, with
// no third-party factorisation:
//
// 1. Crash (crash()): rows peeled through columns no other remaining row
//    holds, the densest remaining row deferred when none is left.  Peeled
//    rows are independent; every dependency runs through deferred rows.
// 2. Reduction (residuals()): each deferred row's entries in the peeled
//    rows' pivot columns eliminated in peel order, leaving a row over the
//    free columns.  Multicommodity flow peels all but one node row per
//    commodity with multipliers of +-1 (0.15 s for 234,640 rows, against
//    0.21 s for the reference's own presolve).  Where a multiplier passes
//    kCrashGrowth or the work passes its limit, the crash is dropped and
//    stage 3 takes the whole matrix (random matrices); where it is dropped
//    with more than 4 x kDenseMaxRows deferred rows, the call returns -4.
// 3. Elimination (eliminate()): the remaining rows held as sparse rows with
//    row lists per column; each step picks a pivot (i, j) among the columns
//    of fewest active entries, the row of fewest entries whose |a_ij| is at
//    least 0.1 of its column's largest (Markowitz cost (r_i - 1)(c_j - 1),
//    threshold partial pivoting), eliminates column j from the other rows
//    (and the same from b), and retires row i and column j.  Once the active
//    entries pass 4 x nnz + 16 m or the entry updates 64 x nnz + 2^28, the
//    remaining rows (at most kDenseMaxRows) finish densely (dense_finish),
//    else the call returns -4: the presolve does not apply to that matrix.
//
// Entries that cancel below tol x their row's largest original entry are
// dropped; rows left with no entry are dependent: such a row is y^T A = 0 for
// the y its reductions built (y_i = 1), and y^T b must be within
// 1e-8 sqrt(1 + |b|_2^2) of zero, else the LP is infeasible.  A removed row
// has no column of its own (it is a combination of kept rows, so each of its
// nonzeros sits in a kept row too): no column of the reduced LP is empty.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <utility>
#include <vector>

#include "../../include/help_lp.h"
#include "guard.h"

namespace {

struct Entry {
    int32_t col;
    double val;
};

constexpr double kThreshold = 0.1;  // pivot at least this fraction of its column's largest entry
constexpr int kSearchColumns = 4;   // columns examined per pivot search
constexpr int64_t kDenseMaxRows = 4096;        // largest remainder the dense finish takes
constexpr int64_t kDenseMaxEntries = 1 << 24;  // per dense array (128 MB of doubles)
constexpr int kOversample = 8;                 // sketch columns beyond the remaining rows
constexpr double kTolPrimal = 1e-8;            // agreement of b along a dependency, relative to |b|_2

// One row of the active submatrix: entries [0, sorted) ordered by column,
// then an unsorted tail of fill; an entry whose value is exactly 0 is dead
// (live entries exceed tol x the row's scale > 0).  Updating a long row
// costs the pivot row's length (times the tail's), not its own: the tail is
// merged back once it passes 2 sqrt(sorted part), which balances the tail
// scans against the merges.
struct Row {
    std::vector<Entry> e;
    int32_t sorted = 0;
    int32_t live = 0;
};

struct Lindep {
    int32_t m, n;
    std::vector<Row> rows;
    std::vector<std::vector<int32_t>> col_rows;  // rows that hold (or once held) the column
    std::vector<int32_t> colcount;               // live entries per column in active rows
    std::vector<char> row_active, col_active;
    std::vector<double> row_scale, b;
    // active columns bucketed by their count: doubly linked lists
    std::vector<int32_t> bhead, bnext, bprev;
    int32_t cmin = 1;  // no nonempty bucket below this
    std::vector<uint32_t> stamp;  // per row: the last column scan that met it
    uint32_t scan_id = 0;
    std::vector<Entry> cand;
    int64_t entries = 0;
    int64_t work = 0;  // row entries scanned or updated so far

    bool in_bucket(int32_t j) const { return col_active[j] && colcount[j] > 0; }
    void unlink(int32_t j) {
        if (!in_bucket(j)) return;
        const int32_t p = bprev[j], q = bnext[j];
        if (p >= 0) bnext[p] = q;
        else bhead[colcount[j]] = q;
        if (q >= 0) bprev[q] = p;
    }
    void link(int32_t j) {
        if (!in_bucket(j)) return;
        const int32_t c = colcount[j];
        bprev[j] = -1;
        bnext[j] = bhead[c];
        if (bhead[c] >= 0) bprev[bhead[c]] = j;
        bhead[c] = j;
        cmin = std::min(cmin, c);
    }
    void set_count(int32_t j, int32_t c) {
        unlink(j);
        colcount[j] = c;
        link(j);
    }
    // slot of column j in row i (live or dead), or -1
    int64_t slot(int32_t i, int32_t j) {
        const Row& r = rows[i];
        const size_t tail = r.e.size() - (size_t)r.sorted;
        work += 1 + (int64_t)std::log2((double)r.sorted + 1.0) + (int64_t)tail;
        auto end = r.e.begin() + r.sorted;
        auto it = std::lower_bound(r.e.begin(), end, j, [](const Entry& x, int32_t c) { return x.col < c; });
        if (it != end && it->col == j) return (int64_t)(it - r.e.begin());
        for (size_t k = (size_t)r.sorted; k < r.e.size(); ++k)
            if (r.e[k].col == j) return (int64_t)k;
        return -1;
    }
    // slot of a live entry of column j in row i, or -1
    int64_t find(int32_t i, int32_t j) {
        const int64_t k = slot(i, j);
        return (k >= 0 && rows[i].e[(size_t)k].val != 0.0) ? k : -1;
    }
    // sort the tail into the row and drop its dead entries
    void compact(int32_t i) {
        Row& r = rows[i];
        work += (int64_t)r.e.size();
        std::sort(r.e.begin() + r.sorted, r.e.end(), [](const Entry& x, const Entry& y) { return x.col < y.col; });
        std::inplace_merge(r.e.begin(), r.e.begin() + r.sorted, r.e.end(),
                           [](const Entry& x, const Entry& y) { return x.col < y.col; });
        r.e.erase(std::remove_if(r.e.begin(), r.e.end(), [](const Entry& x) { return x.val == 0.0; }), r.e.end());
        r.sorted = (int32_t)r.e.size();
    }
    // cand = (row, |a_ij|) for the active rows holding column j, each once;
    // col_rows[j] is compacted to those rows on the way
    void column(int32_t j) {
        if (++scan_id == 0) {  // stamps wrapped: start over
            std::fill(stamp.begin(), stamp.end(), 0u);
            scan_id = 1;
        }
        std::vector<int32_t>& cr = col_rows[j];
        cand.clear();
        size_t k = 0;
        for (int32_t i : cr) {
            if (!row_active[i] || stamp[i] == scan_id) continue;
            stamp[i] = scan_id;
            const int64_t e = find(i, j);
            if (e < 0) continue;
            cr[k++] = i;
            cand.push_back({i, std::fabs(rows[i].e[(size_t)e].val)});
        }
        cr.resize(k);
    }
    // row i -= l * row r, the pivot column pc set to exactly zero and entries
    // of i at most tol x its scale dropped
    void axpy_row(int32_t i, int32_t r, int32_t pc, double l, double tol) {
        const double drop = tol * row_scale[i];
        for (const Entry& pe : rows[r].e) {
            if (pe.val == 0.0) continue;
            const int64_t k = slot(i, pe.col);
            if (k >= 0) {
                Entry& x = rows[i].e[(size_t)k];
                const bool was_live = x.val != 0.0;
                const double v = (pe.col == pc) ? 0.0 : x.val - l * pe.val;
                const bool keep = std::fabs(v) > drop;
                x.val = keep ? v : 0.0;
                if (was_live && !keep) {
                    set_count(pe.col, colcount[pe.col] - 1);
                    --rows[i].live;
                    --entries;
                } else if (!was_live && keep) {
                    col_rows[pe.col].push_back(i);
                    set_count(pe.col, colcount[pe.col] + 1);
                    ++rows[i].live;
                    ++entries;
                }
            } else {
                const double v = -l * pe.val;
                if (!(std::fabs(v) > drop)) continue;
                rows[i].e.push_back({pe.col, v});
                col_rows[pe.col].push_back(i);
                set_count(pe.col, colcount[pe.col] + 1);
                ++rows[i].live;
                ++entries;
            }
        }
        Row& ri = rows[i];
        const size_t tail = ri.e.size() - (size_t)ri.sorted;
        const size_t tail_max = std::max<size_t>(16, (size_t)(2.0 * std::sqrt((double)ri.sorted)));
        if (tail > tail_max || (int64_t)ri.e.size() > 2 * (int64_t)ri.live + 16)
            compact(i);
    }
};

// Standard normal deviates from a fixed-seed splitmix64 stream (Box-Muller).
struct Normal {
    uint64_t s;
    bool have = false;
    double spare = 0.0;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double operator()() {
        if (have) {
            have = false;
            return spare;
        }
        const double u1 = ((double)(next() >> 11) + 1.0) * 0x1.0p-53;  // (0, 1]
        const double u2 = (double)(next() >> 11) * 0x1.0p-53;
        const double rad = std::sqrt(-2.0 * std::log(u1)), th = 6.283185307179586 * u2;
        spare = rad * std::sin(th);
        have = true;
        return rad * std::cos(th);
    }
};

// Dense finish once sparse elimination fills in: the remaining active rows
// (r of them) are copied into a dense r x w array -- their active columns
// as they are when there are few, else a Gaussian sketch Y = A_act G with
// w = r + kOversample columns, which has the same row dependencies as A_act
// with probability one -- and reduced to row echelon form in row order: each
// row's largest entry left is its pivot, or the row is dependent when that
// entry is at most tol x the row's scale.  Independent rows are retired;
// dependent ones are left active and empty with their eliminated b.
// Returns 0, or -4 when the remainder is beyond the dense limits.
int dense_finish(Lindep& S, double tol) {
    std::vector<int32_t> R;
    for (int32_t i = 0; i < S.m; ++i)
        if (S.row_active[i] && S.rows[i].live > 0) R.push_back(i);
    const int64_t r = (int64_t)R.size();
    if (r == 0) return 0;
    if (r > kDenseMaxRows) return -4;
    std::vector<int32_t> cidx((size_t)S.n, -1);
    int64_t c = 0;
    for (int32_t i : R)
        for (const Entry& e : S.rows[i].e)
            if (e.val != 0.0 && cidx[e.col] < 0) cidx[e.col] = (int32_t)c++;
    const bool sketch = c > 2 * (r + kOversample);
    const int64_t w = sketch ? r + kOversample : c;
    if (r * w > kDenseMaxEntries || (sketch && c * w > kDenseMaxEntries)) return -4;
    std::vector<double> Y((size_t)(r * w), 0.0), scale((size_t)r);
    if (sketch) {
        std::vector<double> G((size_t)(c * w));
        Normal nrm{0x5DEECE66DULL};
        for (double& g : G) g = nrm();
        for (int64_t k = 0; k < r; ++k) {
            double* yk = &Y[(size_t)(k * w)];
            for (const Entry& e : S.rows[R[k]].e) {
                if (e.val == 0.0) continue;
                const double* gr = &G[(size_t)cidx[e.col] * (size_t)w];
                for (int64_t t = 0; t < w; ++t) yk[t] += e.val * gr[t];
            }
            double mx = 0.0;
            for (int64_t t = 0; t < w; ++t) mx = std::max(mx, std::fabs(yk[t]));
            scale[k] = std::max(mx, S.row_scale[R[k]]);
        }
    } else {
        for (int64_t k = 0; k < r; ++k) {
            for (const Entry& e : S.rows[R[k]].e)
                if (e.val != 0.0) Y[(size_t)(k * w + cidx[e.col])] = e.val;
            scale[k] = S.row_scale[R[k]];
        }
    }
    for (int64_t k = 0; k < r; ++k) {
        double* yk = &Y[(size_t)(k * w)];
        int64_t jm = -1;
        double vm = 0.0;
        for (int64_t t = 0; t < w; ++t)
            if (std::fabs(yk[t]) > vm) {
                vm = std::fabs(yk[t]);
                jm = t;
            }
        const int32_t ik = R[k];
        if (vm <= tol * scale[k]) {  // dependent: left active and empty
            S.rows[ik] = Row();
            continue;
        }
        S.row_active[ik] = 0;
        const double piv = yk[jm];
        for (int64_t kk = k + 1; kk < r; ++kk) {
            double* y = &Y[(size_t)(kk * w)];
            if (y[jm] == 0.0) continue;
            const double l = y[jm] / piv;
            for (int64_t t = 0; t < w; ++t) y[t] -= l * yk[t];
            y[jm] = 0.0;
            S.b[R[kk]] -= l * S.b[ik];
        }
    }
    return 0;
}

// A by rows, entries of each row in column order (zeros skipped).
struct RowMajor {
    std::vector<int64_t> ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
};

RowMajor by_rows(const help_lp* in) {
    RowMajor R;
    R.ptr.assign((size_t)in->m + 1, 0);
    for (int64_t q = 0; q < in->nnz; ++q)
        if (in->val[q] != 0.0) R.ptr[(size_t)in->row_ind[q] + 1]++;
    for (int32_t i = 0; i < in->m; ++i) R.ptr[(size_t)i + 1] += R.ptr[(size_t)i];
    R.col.resize((size_t)R.ptr[(size_t)in->m]);
    R.val.resize((size_t)R.ptr[(size_t)in->m]);
    std::vector<int64_t> fill(R.ptr.begin(), R.ptr.end() - 1);
    for (int32_t j = 0; j < in->n; ++j)
        for (int32_t q = in->col_ptr[j]; q < in->col_ptr[j + 1]; ++q) {
            if (in->val[q] == 0.0) continue;
            const int64_t p = fill[(size_t)in->row_ind[q]]++;
            R.col[(size_t)p] = j;
            R.val[(size_t)p] = in->val[q];
        }
    return R;
}

// Triangular crash (the structure of Andersen's method, which the reference
// follows: Presolve_Lindep.cpp:34-167): a row with a column no other
// remaining row holds is independent of the remaining rows -- it is peeled
// with that column as its pivot; when no such column is left, the remaining
// row with the most entries is deferred, which may free new columns.  The
// peeled rows against their pivot columns form a triangular block with a
// nonzero diagonal (row k holds no pivot column of a row peeled before it),
// so they are independent; every dependency runs through deferred rows.
enum RowState : char { kRemaining = 0, kPeeled = 1, kDeferred = 2, kEmpty = 3 };
constexpr double kCrashPivot = 1e-2;   // a peel's pivot is at least this x its row's largest entry
constexpr double kCrashGrowth = 1e2;   // largest multiplier the reduction against the crash takes

struct Crash {
    std::vector<char> state;           // per row
    std::vector<int32_t> order;        // peeled rows, in peel order
    std::vector<int32_t> pcol;         // pivot column of each peeled row
    std::vector<double> pval;          // its entry there
    std::vector<int32_t> peel_of_col;  // column -> index in order, or -1
    std::vector<int32_t> deferred;
};

void crash(const help_lp* in, const RowMajor& R, const std::vector<double>& row_scale, Crash& C) {
    const int32_t m = in->m, n = in->n;
    C.state.assign((size_t)m, kRemaining);
    C.peel_of_col.assign((size_t)n, -1);
    std::vector<int32_t> cnt((size_t)n, 0), queue, by_len;
    for (int32_t i = 0; i < m; ++i) {
        if (R.ptr[(size_t)i + 1] == R.ptr[(size_t)i]) {
            C.state[(size_t)i] = kEmpty;
            continue;
        }
        by_len.push_back(i);
        for (int64_t p = R.ptr[(size_t)i]; p < R.ptr[(size_t)i + 1]; ++p) cnt[(size_t)R.col[(size_t)p]]++;
    }
    for (int32_t j = 0; j < n; ++j)
        if (cnt[(size_t)j] == 1) queue.push_back(j);
    std::stable_sort(by_len.begin(), by_len.end(), [&](int32_t x, int32_t y) {
        return R.ptr[(size_t)x + 1] - R.ptr[(size_t)x] > R.ptr[(size_t)y + 1] - R.ptr[(size_t)y];
    });
    auto leave = [&](int32_t i) {  // row i no longer remaining
        for (int64_t p = R.ptr[(size_t)i]; p < R.ptr[(size_t)i + 1]; ++p)
            if (--cnt[(size_t)R.col[(size_t)p]] == 1) queue.push_back(R.col[(size_t)p]);
    };
    size_t head = 0, next = 0;
    for (;;) {
        while (head < queue.size()) {
            const int32_t j = queue[head++];
            if (cnt[(size_t)j] != 1) continue;
            int32_t i = -1;
            double v = 0.0;
            for (int32_t q = in->col_ptr[j]; q < in->col_ptr[j + 1]; ++q)
                if (in->val[q] != 0.0 && C.state[(size_t)in->row_ind[q]] == kRemaining) {
                    i = in->row_ind[q];
                    v = in->val[q];
                    break;
                }
            if (i < 0 || std::fabs(v) < kCrashPivot * row_scale[(size_t)i]) continue;
            C.state[(size_t)i] = kPeeled;
            C.peel_of_col[(size_t)j] = (int32_t)C.order.size();
            C.order.push_back(i);
            C.pcol.push_back(j);
            C.pval.push_back(v);
            leave(i);
        }
        while (next < by_len.size() && C.state[(size_t)by_len[next]] != kRemaining) ++next;
        if (next == by_len.size()) break;
        const int32_t d = by_len[next++];
        C.state[(size_t)d] = kDeferred;
        C.deferred.push_back(d);
        leave(d);
    }
}

// Each deferred row reduced against the peeled rows: its entries in pivot
// columns are eliminated in peel order (a row peeled k-th holds pivot
// columns of rows peeled after it only, so the order never reintroduces an
// eliminated column), leaving a row over the free columns; b follows.  The
// rows go into S (peeled rows inactive).  The triangular block has no
// pivoting of its own, so a multiplier above kCrashGrowth (random matrices:
// chains of ratios reach 1e5) means the crash is ill-conditioned for this
// matrix.  Returns false then, or when the entry updates pass work_limit.
bool residuals(const help_lp* in, const RowMajor& R, const Crash& C, double tol, int64_t work_limit, Lindep& S) {
    const int32_t n = in->n;
    std::vector<double> r((size_t)n, 0.0);
    std::vector<char> mark((size_t)n, 0), queued(C.order.size(), 0);
    std::vector<int32_t> touched, heap;
    const std::greater<int32_t> later;
    int64_t work = 0;
    auto touch = [&](int32_t c) {
        if (!mark[(size_t)c]) {
            mark[(size_t)c] = 1;
            touched.push_back(c);
        }
        const int32_t k = C.peel_of_col[(size_t)c];
        if (k >= 0 && !queued[(size_t)k]) {
            queued[(size_t)k] = 1;
            heap.push_back(k);
            std::push_heap(heap.begin(), heap.end(), later);
        }
    };
    for (int32_t d : C.deferred) {
        touched.clear();
        for (int64_t p = R.ptr[(size_t)d]; p < R.ptr[(size_t)d + 1]; ++p) {
            r[(size_t)R.col[(size_t)p]] = R.val[(size_t)p];
            touch(R.col[(size_t)p]);
        }
        double bd = in->b[d];
        while (!heap.empty()) {
            std::pop_heap(heap.begin(), heap.end(), later);
            const int32_t k = heap.back();
            heap.pop_back();
            queued[(size_t)k] = 0;
            const int32_t j = C.pcol[(size_t)k];
            if (r[(size_t)j] == 0.0) continue;
            const double l = r[(size_t)j] / C.pval[(size_t)k];
            if (!(std::fabs(l) <= kCrashGrowth)) return false;
            const int32_t i = C.order[(size_t)k];
            for (int64_t p = R.ptr[(size_t)i]; p < R.ptr[(size_t)i + 1]; ++p) {
                const int32_t c = R.col[(size_t)p];
                touch(c);
                r[(size_t)c] -= l * R.val[(size_t)p];
            }
            r[(size_t)j] = 0.0;
            bd -= l * in->b[i];
            work += R.ptr[(size_t)i + 1] - R.ptr[(size_t)i];
            if (work > work_limit) return false;
        }
        const double drop = tol * S.row_scale[(size_t)d];
        Row& row = S.rows[(size_t)d];
        for (int32_t c : touched) {
            if (C.peel_of_col[(size_t)c] < 0 && std::fabs(r[(size_t)c]) > drop) row.e.push_back({c, r[(size_t)c]});
            r[(size_t)c] = 0.0;
            mark[(size_t)c] = 0;
        }
        std::sort(row.e.begin(), row.e.end(), [](const Entry& x, const Entry& y) { return x.col < y.col; });
        S.b[(size_t)d] = bd;
    }
    return true;
}

// S sized for m rows and n columns, every row active and empty.
void setup(Lindep& S, const help_lp* in, const std::vector<double>& row_scale) {
    const int32_t m = in->m, n = in->n;
    S.m = m;
    S.n = n;
    S.rows.assign((size_t)m, Row());
    S.col_rows.assign((size_t)n, {});
    S.colcount.assign((size_t)n, 0);
    S.row_active.assign((size_t)m, 1);
    S.col_active.assign((size_t)n, 1);
    S.row_scale = row_scale;
    S.b.assign(in->b, in->b + m);
    S.bhead.assign((size_t)m + 1, -1);
    S.bnext.assign((size_t)n, -1);
    S.bprev.assign((size_t)n, -1);
    S.stamp.assign((size_t)m, 0u);
}

// After the rows are filled (each sorted by column): counts and buckets.
void finish_setup(Lindep& S) {
    for (int32_t i = 0; i < S.m; ++i) {
        Row& r = S.rows[(size_t)i];
        r.sorted = r.live = (int32_t)r.e.size();
        S.entries += r.live;
        for (const Entry& e : r.e) {
            S.col_rows[(size_t)e.col].push_back(i);
            S.colcount[(size_t)e.col]++;
        }
    }
    for (int32_t j = S.n - 1; j >= 0; --j) S.link(j);  // bucket lists in column order
}

// Markowitz elimination of S's active rows until no active column is left,
// or the dense finish once the active entries or the work pass their limits.
// Returns 0 or -4.
int eliminate(Lindep& S, double tol, int64_t fill_limit, int64_t work_limit) {
    const int32_t m = S.m;
    int32_t pivots = 0;
    std::vector<int32_t> targets;
    while (pivots < m) {
        if (S.entries > fill_limit || S.work > work_limit) return dense_finish(S, tol);
        // Markowitz search over the columns of fewest active entries; a
        // candidate is at least kThreshold of its column's largest entry, so
        // every multiplier is at most 1 / kThreshold
        while (S.cmin <= m && S.bhead[(size_t)S.cmin] < 0) ++S.cmin;
        if (S.cmin > m) break;  // no active column left
        int32_t bi = -1, bj = -1;
        int64_t best = -1;
        int examined = 0;
        for (int32_t c = S.cmin; c <= m && examined < kSearchColumns && best != 0; ++c) {
            if (best >= 0 && c > S.cmin + 2 * kSearchColumns) break;
            for (int32_t j = S.bhead[(size_t)c]; j >= 0 && examined < kSearchColumns; j = S.bnext[j]) {
                ++examined;
                S.column(j);
                double cmax = 0.0;
                for (const Entry& ce : S.cand) cmax = std::max(cmax, ce.val);
                for (const Entry& ce : S.cand) {
                    const int32_t i = ce.col;
                    if (ce.val < kThreshold * cmax) continue;
                    const int64_t cost = (int64_t)(S.rows[i].live - 1) * (c - 1);
                    if (best < 0 || cost < best || (cost == best && i < bi)) {
                        best = cost;
                        bi = i;
                        bj = j;
                    }
                }
                if (best == 0) break;
            }
        }
        if (bi < 0) break;  // cannot happen: an active column has an active row
        // eliminate column bj from the other active rows
        S.column(bj);
        targets.clear();
        for (const Entry& ce : S.cand)
            if (ce.col != bi) targets.push_back(ce.col);
        const double piv = S.rows[bi].e[(size_t)S.find(bi, bj)].val;
        for (int32_t i : targets) {
            const double l = S.rows[i].e[(size_t)S.find(i, bj)].val / piv;
            S.axpy_row(i, bi, bj, l, tol);
            S.b[i] -= l * S.b[bi];
            if (S.work > 2 * work_limit) return -4;  // one pivot alone ran far past the limit
        }
        // retire the pivot row and column
        for (const Entry& e : S.rows[bi].e)
            if (e.val != 0.0) S.set_count(e.col, S.colcount[e.col] - 1);
        S.entries -= S.rows[bi].live;
        S.rows[bi] = Row();
        S.row_active[bi] = 0;
        S.unlink(bj);
        S.col_active[bj] = 0;
        ++pivots;
    }
    return 0;
}

int remove_dependent_rows(const help_lp* in, double tol, help_lp* out, int32_t* removed) {
    const int32_t m = in->m, n = in->n;
    const int64_t nnz = in->nnz;
    std::vector<double> row_scale((size_t)m, 0.0);  // largest |entry| of each row
    for (int64_t q = 0; q < nnz; ++q)
        row_scale[(size_t)in->row_ind[q]] = std::max(row_scale[(size_t)in->row_ind[q]], std::fabs(in->val[q]));
    double bnorm2 = 1.0;  // 1 + |b|_2^2
    for (int32_t i = 0; i < m; ++i) bnorm2 += in->b[i] * in->b[i];
    const double b_tol = kTolPrimal * std::sqrt(bnorm2);
    // sparse elimination until the active entries or the work pass these,
    // then the dense finish
    const int64_t fill_limit = 4 * std::max<int64_t>(nnz, 1) + 16 * (int64_t)m;
    const int64_t work_limit = 64 * std::max<int64_t>(nnz, 1) + (int64_t(1) << 28);

    // the crash, then the deferred rows' remainders eliminated; where
    // reducing the deferred rows grows or passes the work limit, the whole
    // matrix is eliminated instead
    Lindep S;
    bool reduced;
    {
        const RowMajor R = by_rows(in);
        Crash C;
        crash(in, R, row_scale, C);
        setup(S, in, row_scale);
        for (int32_t i = 0; i < m; ++i)
            if (C.state[(size_t)i] == kPeeled) S.row_active[(size_t)i] = 0;
        reduced = residuals(in, R, C, tol, work_limit, S);
        // an ill-conditioned crash that left more rows without a column of
        // their own than four dense finishes take marks a random-like core:
        // its elimination fills in past the limits (random 100,000-row and
        // block-angular 1.9M-row instances), so stop here
        if (!reduced && (int64_t)C.deferred.size() > 4 * kDenseMaxRows) return -4;
    }
    if (!reduced) {
        S = Lindep();
        setup(S, in, row_scale);
        for (int32_t j = 0; j < n; ++j)  // rows come out sorted by column
            for (int32_t q = in->col_ptr[j]; q < in->col_ptr[j + 1]; ++q)
                if (in->val[q] != 0.0) S.rows[(size_t)in->row_ind[q]].e.push_back({j, in->val[q]});
    }
    finish_setup(S);
    const int rc = eliminate(S, tol, fill_limit, work_limit);
    if (rc) return rc;
    // rows never pivoted are dependent (all their entries cancelled)
    std::vector<char> dep((size_t)m, 0);
    int32_t n_dep = 0;
    for (int32_t i = 0; i < m; ++i) {
        if (!S.row_active[i]) continue;
        if (S.rows[i].live > 0) continue;  // cannot happen: an entry left is a pivot candidate
        // b agrees when y^T b (y_i = 1) is within 1e-8 sqrt(1 + |b|_2^2): the
        // reference's test of the dependent row's basic value against
        // TOLPRIMAL sqrt(1 + |x_B|_2^2) (Presolve_Lindep.cpp:263-284, LP.h:96)
        // with b standing in for the basic solution x_B
        if (std::fabs(S.b[i]) > b_tol) return -3;  // primal infeasible
        dep[i] = 1;
        ++n_dep;
    }
    // the reduced LP: the kept rows, renumbered in order
    std::vector<int32_t> new_row((size_t)m, -1);
    int32_t mr = 0;
    for (int32_t i = 0; i < m; ++i)
        if (!dep[i]) new_row[i] = mr++;
    int64_t nnz_r = 0;
    for (int64_t q = 0; q < nnz; ++q)
        if (!dep[in->row_ind[q]]) ++nnz_r;
    out->m = mr;
    out->n = n;
    out->n_struct = in->n_struct;
    out->nnz = nnz_r;
    out->col_ptr = (int32_t*)std::malloc(sizeof(int32_t) * ((size_t)n + 1));
    out->row_ind = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz_r, 1));
    out->val = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(nnz_r, 1));
    out->b = (double*)std::malloc(sizeof(double) * (size_t)std::max(mr, 1));
    out->c = (double*)std::malloc(sizeof(double) * (size_t)n);
    out->row_type = (char*)std::malloc((size_t)std::max(mr, 1));
    if (!out->col_ptr || !out->row_ind || !out->val || !out->b || !out->c || !out->row_type) {
        help_lp_free(out);
        return -2;
    }
    int64_t p = 0;
    for (int32_t j = 0; j < n; ++j) {
        out->col_ptr[j] = (int32_t)p;
        for (int32_t q = in->col_ptr[j]; q < in->col_ptr[j + 1]; ++q)
            if (!dep[in->row_ind[q]]) {
                out->row_ind[p] = new_row[in->row_ind[q]];
                out->val[p] = in->val[q];
                ++p;
            }
    }
    out->col_ptr[n] = (int32_t)p;
    std::memcpy(out->c, in->c, sizeof(double) * (size_t)n);
    for (int32_t i = 0; i < m; ++i)
        if (!dep[i]) {
            out->b[new_row[i]] = in->b[i];
            out->row_type[new_row[i]] = in->row_type ? in->row_type[i] : 'E';
        }
    if (removed)
        for (int32_t i = 0; i < m; ++i) removed[i] = dep[i];
    return n_dep;
}

}  // namespace

extern "C" {

int help_lp_remove_dependent_rows(const help_lp* in, double tol, help_lp* out, int32_t* removed) {
    if (!in || !out || in->m <= 0 || in->n <= 0 || !(tol > 0.0)) return -1;
    std::memset(out, 0, sizeof(*out));
    const int rc = c_guard(-2, [&] { return remove_dependent_rows(in, tol, out, removed); });
    if (rc == -2) help_lp_free(out);
    return rc;
}

}  // extern "C"
