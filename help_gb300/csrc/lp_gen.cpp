// Seeded generators for the benchmark LP families and the MPS writer.
//
// Reproducibility across hosts (x86-64 here, aarch64 on the GPU hosts) is a
// requirement: the same seed must give bit-identical instances everywhere, so
// this file uses only IEEE-754 basic operations (+ - * / sqrt, rounding to
// integers) and is compiled with -ffp-contract=off.  The logarithm and the
// exponential needed by the normal and Zipf samplers are computed here from
// their series rather than taken from the platform libm, whose last-bit
// behaviour differs between architectures.
//
// Every value is rounded to a 1e-6 decimal grid.  The reference reads MPS
// values with atof() at fixed card position 24 and also scans a second
// name/value pair at position 39 (MPSRead.cpp:144-169), so each value must be
// short (<= 15 characters) yet round-trip exactly; k / 1e6 printed as %.6f
// parses back to the same double because both sides are the correctly
// rounded value of the same decimal.

#include "../../include/help_lp.h"
#include "guard.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// xoshiro256** (Blackman & Vigna), seeded through splitmix64.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            s[i] = z ^ (z >> 31);
        }
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    // Uniform in [0, 1) with 53 random bits.
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    // Uniform in (0, 1].
    double uniform_pos() { return ((double)(next() >> 11) + 1.0) * (1.0 / 9007199254740992.0); }
    // Uniform integer in [0, n) by 128-bit multiply-shift (Lemire), no modulo bias worth noting.
    int32_t below(int32_t n) {
        unsigned __int128 p = (unsigned __int128)next() * (unsigned __int128)(uint64_t)n;
        return (int32_t)(p >> 64);
    }
    double uniform_range(double lo, double hi) { return lo + (hi - lo) * uniform(); }
};

const double kLn2 = 0.6931471805599453094;

// Natural log for x > 0: x = f * 2^e with f in [sqrt(1/2), sqrt(2)),
// log f = 2 atanh(u), u = (f - 1) / (f + 1), |u| < 0.1716, series to u^41.
double det_log(double x) {
    int e = 0;
    double f = std::frexp(x, &e);  // exact: f in [0.5, 1)
    if (f < 0.70710678118654752440) {
        f *= 2.0;
        e -= 1;
    }
    const double u = (f - 1.0) / (f + 1.0);
    const double u2 = u * u;
    double term = u, sum = 0.0;
    for (int k = 1; k <= 41; k += 2) {
        sum += term / (double)k;
        term *= u2;
    }
    return 2.0 * sum + (double)e * kLn2;
}

// exp(x) for moderate |x|: x = k ln2 + r, |r| <= ln2/2, Taylor series to r^24.
double det_exp(double x) {
    const double kd = std::nearbyint(x / kLn2);
    const double r = x - kd * kLn2;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 24; ++k) {
        term *= r / (double)k;
        sum += term;
    }
    return std::ldexp(sum, (int)kd);
}

// Standard normal by Marsaglia's polar method.
struct Normal {
    bool has_spare = false;
    double spare = 0.0;
    double operator()(Rng& g) {
        if (has_spare) {
            has_spare = false;
            return spare;
        }
        double u, v, s;
        do {
            u = 2.0 * g.uniform() - 1.0;
            v = 2.0 * g.uniform() - 1.0;
            s = u * u + v * v;
        } while (s >= 1.0 || s == 0.0);
        const double f = std::sqrt(-2.0 * det_log(s) / s);
        spare = v * f;
        has_spare = true;
        return u * f;
    }
};

inline double q6(double v) { return std::nearbyint(v * 1e6) / 1e6; }

// A nonzero N(0,1) value on the 1e-6 grid.
double nonzero_normal(Rng& g, Normal& nd) {
    for (;;) {
        const double v = q6(nd(g));
        if (v != 0.0) return v;
    }
}

struct Triplets {
    std::vector<int32_t> col_ptr;
    std::vector<int32_t> rows;
    std::vector<double> vals;
};

int alloc_out(help_lp* out, int32_t m, int32_t n, int64_t nnz) {
    std::memset(out, 0, sizeof(*out));
    out->m = m;
    out->n = n;
    out->n_struct = n;
    out->nnz = nnz;
    out->col_ptr = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)(n + 1));
    out->row_ind = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
    out->val = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
    out->b = (double*)std::calloc((size_t)std::max(m, 1), sizeof(double));
    out->c = (double*)std::calloc((size_t)std::max(n, 1), sizeof(double));
    out->row_type = (char*)std::malloc((size_t)std::max(m, 1));
    if (!out->col_ptr || !out->row_ind || !out->val || !out->b || !out->c || !out->row_type) {
        help_lp_free(out);
        return -2;
    }
    std::memset(out->row_type, 'E', (size_t)std::max(m, 1));
    return 0;
}

// Sort rows inside every column (values follow), as the reference's presolve
// leaves its column lists (Presolve.cpp:60-75).
void sort_columns(Triplets& t, int32_t n) {
    std::vector<std::pair<int32_t, double>> tmp;
    for (int32_t j = 0; j < n; ++j) {
        const int32_t a = t.col_ptr[j], e = t.col_ptr[j + 1];
        tmp.clear();
        for (int32_t p = a; p < e; ++p) tmp.emplace_back(t.rows[p], t.vals[p]);
        std::sort(tmp.begin(), tmp.end(),
                  [](const std::pair<int32_t, double>& x, const std::pair<int32_t, double>& y) {
                      return x.first < y.first;
                  });
        for (int32_t p = a; p < e; ++p) {
            t.rows[p] = tmp[p - a].first;
            t.vals[p] = tmp[p - a].second;
        }
    }
}

// Every row must hold at least one nonzero, otherwise A D^-1 A^T is singular.
// An empty row i receives one entry in column (i * 7919) mod n.
void cover_empty_rows(Triplets& t, int32_t m, int32_t n, Rng& g, Normal& nd) {
    std::vector<int32_t> cnt(m, 0);
    for (int32_t r : t.rows) cnt[r]++;
    std::vector<std::vector<std::pair<int32_t, double>>> extra(n);
    bool any = false;
    for (int32_t i = 0; i < m; ++i) {
        if (cnt[i] == 0) {
            const int32_t j = (int32_t)(((int64_t)i * 7919) % n);
            extra[j].emplace_back(i, nonzero_normal(g, nd));
            any = true;
        }
    }
    if (!any) return;
    Triplets u;
    u.col_ptr.assign(n + 1, 0);
    u.rows.reserve(t.rows.size() + m);
    u.vals.reserve(t.rows.size() + m);
    for (int32_t j = 0; j < n; ++j) {
        u.col_ptr[j] = (int32_t)u.rows.size();
        for (int32_t p = t.col_ptr[j]; p < t.col_ptr[j + 1]; ++p) {
            u.rows.push_back(t.rows[p]);
            u.vals.push_back(t.vals[p]);
        }
        for (auto& e : extra[j]) {
            u.rows.push_back(e.first);
            u.vals.push_back(e.second);
        }
    }
    u.col_ptr[n] = (int32_t)u.rows.size();
    t = std::move(u);
    sort_columns(t, n);
}

// Feasible-by-construction right-hand sides (the configuration recipe):
// x0 ~ U(0.5, 2), b = A x0, y0 ~ N(0, 1), s0 ~ U(0.5, 2), c = A^T y0 + s0,
// all rounded to the 1e-6 grid.
void finish_random_lp(const Triplets& t, int32_t m, int32_t n, Rng& g, Normal& nd, help_lp* out) {
    std::vector<double> x0(n), y0(m), s0(n);
    for (int32_t j = 0; j < n; ++j) x0[j] = q6(g.uniform_range(0.5, 2.0));
    for (int32_t i = 0; i < m; ++i) y0[i] = q6(nd(g));
    for (int32_t j = 0; j < n; ++j) s0[j] = q6(g.uniform_range(0.5, 2.0));
    std::vector<double> bb(m, 0.0);
    for (int32_t j = 0; j < n; ++j)
        for (int32_t p = t.col_ptr[j]; p < t.col_ptr[j + 1]; ++p) bb[t.rows[p]] += t.vals[p] * x0[j];
    for (int32_t i = 0; i < m; ++i) out->b[i] = q6(bb[i]);
    for (int32_t j = 0; j < n; ++j) {
        double s = 0.0;
        for (int32_t p = t.col_ptr[j]; p < t.col_ptr[j + 1]; ++p) s += t.vals[p] * y0[t.rows[p]];
        out->c[j] = q6(s + s0[j]);
    }
}

int emit(const Triplets& t, int32_t m, int32_t n, help_lp* out) {
    const int64_t nnz = (int64_t)t.rows.size();
    if (nnz > 2147483647LL) return -3;
    int rc = alloc_out(out, m, n, nnz);
    if (rc) return rc;
    std::memcpy(out->col_ptr, t.col_ptr.data(), sizeof(int32_t) * (size_t)(n + 1));
    std::memcpy(out->row_ind, t.rows.data(), sizeof(int32_t) * (size_t)nnz);
    std::memcpy(out->val, t.vals.data(), sizeof(double) * (size_t)nnz);
    return 0;
}

// k distinct rows per column drawn by `draw`, values N(0,1).
template <class Draw>
void fill_columns(Triplets& t, int32_t n, int32_t k, Rng& g, Normal& nd, Draw draw,
                  int32_t forced_rows_below) {
    t.col_ptr.assign(n + 1, 0);
    t.rows.reserve((size_t)n * k);
    t.vals.reserve((size_t)n * k);
    int32_t picked[64];
    for (int32_t j = 0; j < n; ++j) {
        t.col_ptr[j] = (int32_t)t.rows.size();
        int32_t cnt = 0;
        if (j < forced_rows_below) picked[cnt++] = j;
        while (cnt < k) {
            const int32_t r = draw(g);
            bool dup = false;
            for (int32_t q = 0; q < cnt; ++q) dup |= (picked[q] == r);
            if (!dup) picked[cnt++] = r;
        }
        std::sort(picked, picked + cnt);
        for (int32_t q = 0; q < cnt; ++q) {
            t.rows.push_back(picked[q]);
            t.vals.push_back(nonzero_normal(g, nd));
        }
    }
    t.col_ptr[n] = (int32_t)t.rows.size();
}

int gen_random(const help_lp_spec* s, uint64_t seed, help_lp* out) {
    const int32_t m = s->m, n = s->n, k = s->nnz_per_col;
    if (m <= 0 || n <= 0 || k <= 0 || k > m || k > 64) return -1;
    Rng g(seed);
    Normal nd;
    Triplets t;
    fill_columns(t, n, k, g, nd, [m](Rng& r) { return r.below(m); }, 0);
    cover_empty_rows(t, m, n, g, nd);
    int rc = emit(t, m, n, out);
    if (rc) return rc;
    finish_random_lp(t, m, n, g, nd, out);
    return 0;
}

// Zipf rank law: row of rank r is drawn with weight (r + offset)^-s; ranks are
// mapped to rows by a seeded permutation so heavy rows are scattered; column
// j < m always contains row j so no row is empty.
int gen_zipf(const help_lp_spec* s, uint64_t seed, help_lp* out) {
    const int32_t m = s->m, n = s->n, k = s->nnz_per_col;
    if (m <= 0 || n <= 0 || k <= 1 || k > m || k > 64 || !(s->zipf_s > 0.0)) return -1;
    Rng g(seed);
    Normal nd;
    std::vector<double> cdf(m);
    double acc = 0.0;
    for (int32_t r = 0; r < m; ++r) {
        acc += det_exp(-s->zipf_s * det_log((double)r + (double)std::max(1, s->zipf_offset)));
        cdf[r] = acc;
    }
    std::vector<int32_t> perm(m);
    for (int32_t i = 0; i < m; ++i) perm[i] = i;
    for (int32_t i = m - 1; i > 0; --i) std::swap(perm[i], perm[g.below(i + 1)]);
    const double total = acc;
    Triplets t;
    fill_columns(
        t, n, k, g, nd,
        [&](Rng& r) {
            const double u = r.uniform() * total;
            int32_t idx = (int32_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
            if (idx >= m) idx = m - 1;
            return perm[idx];
        },
        m);
    cover_empty_rows(t, m, n, g, nd);
    int rc = emit(t, m, n, out);
    if (rc) return rc;
    finish_random_lp(t, m, n, g, nd, out);
    return 0;
}

// Block-angular: `blocks` diagonal blocks of block_rows x block_cols with k
// uniform nonzeros per column inside the block's rows, plus link_rows dense-ish
// coupling rows at the bottom in which each column appears with probability
// link_prob (geometric skips over the linking rows).
int gen_block(const help_lp_spec* s, uint64_t seed, help_lp* out) {
    const int32_t B = s->blocks, R = s->block_rows, C = s->block_cols, L = s->link_rows;
    const int32_t k = s->nnz_per_col;
    const double q = s->link_prob;
    if (B <= 0 || R <= 0 || C <= 0 || L < 0 || k <= 0 || k > R || k > 64 || q < 0.0 || q >= 1.0)
        return -1;
    const int64_t m64 = (int64_t)B * R + L, n64 = (int64_t)B * C;
    if (m64 > 2000000000LL || n64 > 2000000000LL) return -1;
    const int32_t m = (int32_t)m64, n = (int32_t)n64;
    Rng g(seed);
    Normal nd;
    Triplets t;
    t.col_ptr.assign(n + 1, 0);
    const double expect = (double)n * (k + q * L);
    t.rows.reserve((size_t)(expect * 1.02) + 16);
    t.vals.reserve((size_t)(expect * 1.02) + 16);
    const double log1mq = (q > 0.0) ? det_log(1.0 - q) : 0.0;
    int32_t picked[64];
    for (int32_t j = 0; j < n; ++j) {
        t.col_ptr[j] = (int32_t)t.rows.size();
        const int32_t base = (j / C) * R;
        int32_t cnt = 0;
        while (cnt < k) {
            const int32_t r = base + g.below(R);
            bool dup = false;
            for (int32_t z = 0; z < cnt; ++z) dup |= (picked[z] == r);
            if (!dup) picked[cnt++] = r;
        }
        std::sort(picked, picked + cnt);
        for (int32_t z = 0; z < cnt; ++z) {
            t.rows.push_back(picked[z]);
            t.vals.push_back(nonzero_normal(g, nd));
        }
        if (q > 0.0 && L > 0) {
            int64_t l = -1;
            for (;;) {
                const double skip = std::floor(det_log(g.uniform_pos()) / log1mq);
                l += 1 + (int64_t)skip;
                if (l >= L) break;
                t.rows.push_back((int32_t)((int64_t)B * R + l));
                t.vals.push_back(nonzero_normal(g, nd));
            }
        }
    }
    t.col_ptr[n] = (int32_t)t.rows.size();
    if ((int64_t)t.rows.size() > 2147483647LL) return -3;
    cover_empty_rows(t, m, n, g, nd);
    int rc = emit(t, m, n, out);
    if (rc) return rc;
    finish_random_lp(t, m, n, g, nd, out);
    return 0;
}

// Multicommodity flow on a G x G grid with 4-neighbour bidirectional arcs.
// Rows: per commodity the node-balance rows of nodes 1..N-1 (node 0 is
// grounded: each commodity's incidence matrix has rank N-1), or of all N
// nodes with mcf_ungrounded (then each commodity's rows sum to zero and A is
// K rows short of full rank, as the reference's inputs are when its
// dependent-row presolve is needed), then one 'L' capacity row per arc.  Columns: flow (commodity, arc) with +1 at the tail
// row, -1 at the head row and +1 at the arc's capacity row; then one slack
// column per capacity row (Crushing.cpp:71-99 adds these for 'L' rows).
// Demands come from routing, per commodity, `pairs` random source/sink pairs
// along random monotone lattice paths with amounts U(1, 10); capacities are
// the summed flow + U(1, 10); costs are U(1, 10).
int gen_mcf(const help_lp_spec* s, uint64_t seed, help_lp* out) {
    const int32_t G = s->grid, K = s->commodities, P = std::max(1, s->pairs_per_commodity);
    if (G < 2 || K <= 0) return -1;
    const int32_t N = G * G;
    // Arc list: for every node, neighbours in the order right, down, left, up.
    std::vector<int32_t> tail, head;
    std::vector<int32_t> arc_of(4 * (size_t)N, -1);  // node*4 + dir -> arc id
    for (int32_t r = 0; r < G; ++r)
        for (int32_t c = 0; c < G; ++c) {
            const int32_t u = r * G + c;
            const int32_t dr[4] = {0, 1, 0, -1}, dc[4] = {1, 0, -1, 0};
            for (int d = 0; d < 4; ++d) {
                const int32_t rr = r + dr[d], cc = c + dc[d];
                if (rr < 0 || rr >= G || cc < 0 || cc >= G) continue;
                arc_of[(size_t)u * 4 + d] = (int32_t)tail.size();
                tail.push_back(u);
                head.push_back(rr * G + cc);
            }
        }
    const int32_t A = (int32_t)tail.size();
    const int32_t NR = s->mcf_ungrounded ? N : N - 1;  // node rows per commodity
    const int64_t m64 = (int64_t)K * NR + A;
    const int64_t n64 = (int64_t)K * A + A;
    if (m64 > 2000000000LL || n64 > 2000000000LL) return -1;
    const int32_t m = (int32_t)m64, n = (int32_t)n64;
    Rng g(seed);
    std::vector<double> flow((size_t)K * A, 0.0);
    std::vector<double> supply((size_t)K * N, 0.0);
    for (int32_t k = 0; k < K; ++k) {
        for (int32_t pidx = 0; pidx < P; ++pidx) {
            int32_t src = g.below(N), dst = g.below(N);
            while (dst == src) dst = g.below(N);
            const double amt = q6(g.uniform_range(1.0, 10.0));
            int32_t r = src / G, c = src % G;
            const int32_t tr = dst / G, tc = dst % G;
            while (r != tr || c != tc) {
                int d;
                const bool can_r = (c != tc), can_d = (r != tr);
                if (can_r && can_d) d = (g.below(2) == 0) ? 0 : 1;
                else d = can_r ? 0 : 1;
                int dir;
                if (d == 0) dir = (tc > c) ? 0 : 2;
                else dir = (tr > r) ? 1 : 3;
                const int32_t u = r * G + c;
                const int32_t a = arc_of[(size_t)u * 4 + dir];
                flow[(size_t)k * A + a] += amt;
                if (dir == 0) ++c;
                else if (dir == 2) --c;
                else if (dir == 1) ++r;
                else --r;
            }
            supply[(size_t)k * N + src] += amt;
            supply[(size_t)k * N + dst] -= amt;
        }
    }
    int rc = alloc_out(out, m, n, (int64_t)K * A * 3 + A);
    if (rc) return rc;
    out->n_struct = K * A;
    auto node_row = [&](int32_t k, int32_t node) -> int32_t {
        if (s->mcf_ungrounded) return k * N + node;
        return node == 0 ? -1 : k * (N - 1) + (node - 1);
    };
    int64_t p = 0;
    for (int32_t k = 0; k < K; ++k) {
        for (int32_t a = 0; a < A; ++a) {
            const int32_t j = k * A + a;
            out->col_ptr[j] = (int32_t)p;
            int32_t rr[3];
            double vv[3];
            int cnt = 0;
            const int32_t rt = node_row(k, tail[a]), rh = node_row(k, head[a]);
            if (rt >= 0) { rr[cnt] = rt; vv[cnt++] = 1.0; }
            if (rh >= 0) { rr[cnt] = rh; vv[cnt++] = -1.0; }
            rr[cnt] = K * NR + a;
            vv[cnt++] = 1.0;
            // sort the (at most 3) rows
            for (int x = 0; x < cnt; ++x)
                for (int y = x + 1; y < cnt; ++y)
                    if (rr[y] < rr[x]) { std::swap(rr[x], rr[y]); std::swap(vv[x], vv[y]); }
            for (int x = 0; x < cnt; ++x) {
                out->row_ind[p] = rr[x];
                out->val[p] = vv[x];
                ++p;
            }
            out->c[j] = q6(g.uniform_range(1.0, 10.0));
        }
    }
    for (int32_t a = 0; a < A; ++a) {
        const int32_t j = K * A + a;
        out->col_ptr[j] = (int32_t)p;
        out->row_ind[p] = K * NR + a;
        out->val[p] = 1.0;
        ++p;
        out->c[j] = 0.0;
    }
    out->col_ptr[n] = (int32_t)p;
    out->nnz = p;
    for (int32_t k = 0; k < K; ++k)
        for (int32_t node = s->mcf_ungrounded ? 0 : 1; node < N; ++node)
            out->b[node_row(k, node)] = q6(supply[(size_t)k * N + node]);
    for (int32_t a = 0; a < A; ++a) {
        double tot = 0.0;
        for (int32_t k = 0; k < K; ++k) tot += flow[(size_t)k * A + a];
        out->b[K * NR + a] = q6(tot + g.uniform_range(1.0, 10.0));
        out->row_type[K * NR + a] = 'L';
    }
    return 0;
}

}  // namespace

extern "C" {

int help_lp_generate(const help_lp_spec* spec, uint64_t seed, help_lp* out) {
    if (!spec || !out) return -1;
    std::memset(out, 0, sizeof(*out));
    const int rc = c_guard(-2, [&] {
        switch (spec->kind) {
            case HELP_LP_RANDOM: return gen_random(spec, seed, out);
            case HELP_LP_ZIPF: return gen_zipf(spec, seed, out);
            case HELP_LP_MCF: return gen_mcf(spec, seed, out);
            case HELP_LP_BLOCK: return gen_block(spec, seed, out);
            default: return -1;
        }
    });
    if (rc < -1) help_lp_free(out);  // allocation failed part way
    return rc;
}

void help_lp_free(help_lp* lp) {
    if (!lp) return;
    std::free(lp->col_ptr);
    std::free(lp->row_ind);
    std::free(lp->val);
    std::free(lp->b);
    std::free(lp->c);
    std::free(lp->row_type);
    std::memset(lp, 0, sizeof(*lp));
}

int help_lp_write_mps(const help_lp* lp, const char* path) {
    if (!lp || !path) return -1;
    if (lp->m > 10000000 || lp->n_struct > 10000000) return -1;  // 8-character names
    FILE* f = std::fopen(path, "w");
    if (!f) return -2;
    std::fprintf(f, "NAME          HELPLP\nROWS\n N  COST\n");
    for (int32_t i = 0; i < lp->m; ++i)
        std::fprintf(f, " %c  R%07d\n", lp->row_type[i] == 'L' ? 'L' : 'E', i);
    std::fprintf(f, "COLUMNS\n");
    for (int32_t j = 0; j < lp->n_struct; ++j) {
        std::fprintf(f, "    C%07d  COST      %.6f\n", j, lp->c[j]);
        for (int32_t p = lp->col_ptr[j]; p < lp->col_ptr[j + 1]; ++p)
            std::fprintf(f, "    C%07d  R%07d  %.6f\n", j, lp->row_ind[p], lp->val[p]);
    }
    std::fprintf(f, "RHS\n");
    for (int32_t i = 0; i < lp->m; ++i)
        if (lp->b[i] != 0.0) std::fprintf(f, "    RHS       R%07d  %.6f\n", i, lp->b[i]);
    std::fprintf(f, "ENDATA\n");
    return std::fclose(f) == 0 ? 0 : -2;
}

int help_csc_to_csr(int32_t m, int32_t n, const int32_t* col_ptr, const int32_t* row_ind,
                    const double* val, int32_t* row_ptr, int32_t* col_ind, double* val_out) {
    if (m < 0 || n < 0) return -1;
    return c_guard(-2, [&] {
        for (int32_t i = 0; i <= m; ++i) row_ptr[i] = 0;
        const int32_t nnz = col_ptr[n];
        for (int32_t p = 0; p < nnz; ++p) row_ptr[row_ind[p] + 1]++;
        for (int32_t i = 0; i < m; ++i) row_ptr[i + 1] += row_ptr[i];
        std::vector<int32_t> fill(row_ptr, row_ptr + m);
        for (int32_t j = 0; j < n; ++j)
            for (int32_t p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
                const int32_t q = fill[row_ind[p]]++;
                col_ind[q] = j;
                if (val_out) val_out[q] = val[p];
            }
        return 0;
    });
}

}  // extern "C"
