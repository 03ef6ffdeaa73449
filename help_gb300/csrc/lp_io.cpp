// LP input: an MPS reader for the standard-form problems the HSD driver
// solves, and a binary format for large instances.
//
// The MPS reader follows the reference's MPSRead.cpp (sections ROWS,
// COLUMNS, RHS; MPSRead.cpp:76-219) and its row standardisation
// (Crushing.cpp:71-99: an L row gets slack +1, a G row slack -1, slacks
// appended after the structural columns in row order).  Unlike the reference
// it tokenises on blanks rather than card positions, so it reads both the
// fixed layout (names without blanks) and free MPS; it keeps the reference's
// tolerance for dropped entries (1e-8, LP.h:66) and its handling of unknown
// row names (entry dropped).  Bounds other than x >= 0 and RANGES are
// rejected: the HSD driver takes all-lower-bounded columns only.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#include <algorithm>

#include "../../include/help_lp.h"
#include "guard.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

const double kInputTolerance = 1e-8;  // LP.h:66

// Splits a line into blank-separated fields.
void fields(const char* line, std::vector<std::string>& out) {
    out.clear();
    const char* p = line;
    while (*p) {
        while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') ++p;
        if (!*p) break;
        const char* q = p;
        while (*q && *q != ' ' && *q != '\t' && *q != '\r' && *q != '\n') ++q;
        out.emplace_back(p, q - p);
        p = q;
    }
}

bool parse_double(const std::string& s, double* v) {
    char* end = nullptr;
    errno = 0;
    *v = std::strtod(s.c_str(), &end);
    return end && *end == '\0' && errno == 0 && std::isfinite(*v);
}

// Reads one whole line (any length) into buf; false at end of file.
bool read_line(FILE* f, std::string& buf) {
    buf.clear();
    char chunk[4096];
    while (std::fgets(chunk, sizeof(chunk), f)) {
        buf += chunk;
        if (!buf.empty() && buf.back() == '\n') return true;
    }
    return !buf.empty();
}

int alloc_lp(help_lp* out, int32_t m, int32_t n, int64_t nnz) {
    std::memset(out, 0, sizeof(*out));
    out->m = m;
    out->n = n;
    out->nnz = nnz;
    out->col_ptr = (int32_t*)std::malloc(sizeof(int32_t) * ((size_t)n + 1));
    out->row_ind = (int32_t*)std::malloc(sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
    out->val = (double*)std::malloc(sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
    out->b = (double*)std::calloc((size_t)std::max(m, 1), sizeof(double));
    out->c = (double*)std::calloc((size_t)std::max(n, 1), sizeof(double));
    out->row_type = (char*)std::malloc((size_t)std::max(m, 1));
    if (!out->col_ptr || !out->row_ind || !out->val || !out->b || !out->c || !out->row_type) {
        help_lp_free(out);
        return -2;
    }
    return 0;
}

struct Column {
    double cost = 0.0;
    std::vector<std::pair<int32_t, double>> entries;
};

int read_mps_impl(const char* path, help_lp* out) {
    ScopedFile file(std::fopen(path, "r"));
    if (!file.f) return fail(-2, std::string("cannot open ") + path);
    FILE* f = file.f;
    std::unordered_map<std::string, int32_t> row_id, col_id;
    std::vector<char> row_type;
    std::vector<double> rhs;
    std::vector<Column> cols;
    std::string obj_name, line;
    std::vector<std::string> tok;
    enum { kNone, kRows, kColumns, kRhs, kBounds, kDone } sec = kNone;
    long long lineno = 0;
    auto err = [&](const std::string& why) { return fail(-3, "line " + std::to_string(lineno) + ": " + why); };
    while (read_line(f, line)) {
        ++lineno;
        if (line.empty() || line[0] == '*') continue;
        fields(line.c_str(), tok);
        if (tok.empty()) continue;
        if (line[0] != ' ' && line[0] != '\t') {  // section header
            const std::string& h = tok[0];
            if (h == "NAME") continue;
            if (h == "ROWS") sec = kRows;
            else if (h == "COLUMNS") sec = kColumns;
            else if (h == "RHS") sec = kRhs;
            else if (h == "BOUNDS") sec = kBounds;
            else if (h == "RANGES") return err("RANGES are not supported (the HSD driver takes E, L, G rows only)");
            else if (h == "ENDATA") { sec = kDone; break; }
            else if (h == "OBJSENSE" || h == "OBJSENSE MAX") return err("OBJSENSE is not supported (minimisation only)");
            else return err("unknown section " + h);
            continue;
        }
        switch (sec) {
            case kRows: {
                if (tok.size() != 2 || tok[0].size() != 1) return err("ROWS: expected <type> <name>");
                const char t = tok[0][0];
                if (t == 'N') {
                    if (obj_name.empty()) obj_name = tok[1];  // later N rows are free rows, ignored
                    continue;
                }
                if (t != 'E' && t != 'L' && t != 'G') return err("ROWS: unknown row type " + tok[0]);
                if (row_id.count(tok[1])) return err("ROWS: duplicate row " + tok[1]);
                row_id.emplace(tok[1], (int32_t)row_type.size());
                row_type.push_back(t);
                rhs.push_back(0.0);
                break;
            }
            case kColumns: {
                if (tok.size() >= 3 && tok[1] == "'MARKER'") return err("integer markers are not supported");
                if (tok.size() != 3 && tok.size() != 5) return err("COLUMNS: expected <col> <row> <value> [<row> <value>]");
                auto it = col_id.find(tok[0]);
                int32_t j;
                if (it == col_id.end()) {
                    j = (int32_t)cols.size();
                    col_id.emplace(tok[0], j);
                    cols.emplace_back();
                } else {
                    j = it->second;
                }
                for (size_t q = 1; q + 1 < tok.size(); q += 2) {
                    double v;
                    if (!parse_double(tok[q + 1], &v)) return err("COLUMNS: bad value " + tok[q + 1]);
                    if (tok[q] == obj_name) {
                        cols[j].cost = v;
                        continue;
                    }
                    auto r = row_id.find(tok[q]);
                    if (r == row_id.end()) continue;  // unknown row: dropped (MPSRead.cpp:148-152)
                    if (std::fabs(v) < kInputTolerance) continue;  // MPSRead.cpp:158-162
                    cols[j].entries.emplace_back(r->second, v);
                }
                break;
            }
            case kRhs: {
                if (tok.size() != 3 && tok.size() != 5 && tok.size() != 2 && tok.size() != 4)
                    return err("RHS: expected [<set>] <row> <value> [<row> <value>]");
                // the set name is optional in free MPS: an even count means it is absent
                const size_t first = (tok.size() % 2 == 1) ? 1 : 0;
                for (size_t q = first; q + 1 < tok.size(); q += 2) {
                    double v;
                    if (!parse_double(tok[q + 1], &v)) return err("RHS: bad value " + tok[q + 1]);
                    auto r = row_id.find(tok[q]);
                    if (r == row_id.end()) continue;  // objective constant or unknown row
                    rhs[r->second] = v;
                }
                break;
            }
            case kBounds: {
                // <type> <set> <col> [<value>]: only x >= 0 (LO 0, PL) is accepted
                if (tok.size() < 3) return err("BOUNDS: expected <type> <set> <column> [<value>]");
                const std::string& t = tok[0];
                double v = 0.0;
                if (tok.size() >= 4 && !parse_double(tok[3], &v)) return err("BOUNDS: bad value " + tok[3]);
                if (t == "PL" || (t == "LO" && v == 0.0)) continue;
                return err("BOUNDS: only x >= 0 is supported (got " + t + ")");
            }
            default:
                return err("data line outside a section");
        }
    }
    file.close();
    if (sec != kDone) return fail(-3, "missing ENDATA");
    if (obj_name.empty()) return fail(-3, "no objective (N) row");
    const int32_t m = (int32_t)row_type.size();
    int32_t n_slack = 0;
    for (char t : row_type) n_slack += (t != 'E');
    const int64_t n_struct = (int64_t)cols.size();
    const int64_t n = n_struct + n_slack;
    if (m <= 0 || n_struct <= 0) return fail(-3, "empty problem");
    if (n > 2000000000LL) return fail(-3, "too many columns");
    int64_t nnz = n_slack;
    for (auto& c : cols) {
        std::sort(c.entries.begin(), c.entries.end(),
                  [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) { return a.first < b.first; });
        for (size_t q = 1; q < c.entries.size(); ++q)
            if (c.entries[q].first == c.entries[q - 1].first) return fail(-3, "repeated (row, column) entry");
        nnz += (int64_t)c.entries.size();
    }
    if (nnz > 2000000000LL) return fail(-3, "too many nonzeros");
    if (alloc_lp(out, m, (int32_t)n, nnz) != 0) return fail(-2, "out of memory");
    out->n_struct = (int32_t)n_struct;
    int64_t p = 0;
    for (int64_t j = 0; j < n_struct; ++j) {
        out->col_ptr[j] = (int32_t)p;
        out->c[j] = cols[j].cost;
        for (auto& e : cols[j].entries) {
            out->row_ind[p] = e.first;
            out->val[p] = e.second;
            ++p;
        }
    }
    int64_t j = n_struct;
    for (int32_t i = 0; i < m; ++i) {
        out->b[i] = rhs[i];
        out->row_type[i] = row_type[i];
        if (row_type[i] == 'E') continue;
        out->col_ptr[j] = (int32_t)p;
        out->c[j] = 0.0;
        out->row_ind[p] = i;
        out->val[p] = row_type[i] == 'L' ? 1.0 : -1.0;
        ++p;
        ++j;
    }
    out->col_ptr[n] = (int32_t)p;
    return 0;
}

}  // namespace

extern "C" {

const char* help_lp_last_error(void) { return g_err.c_str(); }

int help_lp_read_mps(const char* path, help_lp* out) {
    g_err.clear();
    if (!path || !out) return fail(-1, "bad arguments");
    std::memset(out, 0, sizeof(*out));
    const int rc = c_guard(-4, [&] { return read_mps_impl(path, out); });
    if (rc != -4) return rc;
    help_lp_free(out);
    return fail(-2, "out of memory");
}

int help_lp_write_bin(const help_lp* lp, const char* path) {
    g_err.clear();
    if (!lp || !path || lp->m <= 0 || lp->n <= 0) return fail(-1, "bad arguments");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(-2, std::string("cannot open ") + path);
    int64_t hdr[8] = {0};
    std::memcpy(hdr, "HELPLP01", 8);
    hdr[1] = lp->m;
    hdr[2] = lp->n;
    hdr[3] = lp->n_struct;
    hdr[4] = lp->nnz;
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1;
    auto put = [&](const void* p, size_t bytes) {
        if (ok && bytes) ok = std::fwrite(p, 1, bytes, f) == bytes;
    };
    put(lp->col_ptr, sizeof(int32_t) * ((size_t)lp->n + 1));
    put(lp->row_ind, sizeof(int32_t) * (size_t)lp->nnz);
    put(lp->val, sizeof(double) * (size_t)lp->nnz);
    put(lp->b, sizeof(double) * (size_t)lp->m);
    put(lp->c, sizeof(double) * (size_t)lp->n);
    put(lp->row_type, (size_t)lp->m);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? 0 : fail(-2, "write failed");
}

int help_lp_read_bin(const char* path, help_lp* out) {
    g_err.clear();
    if (!path || !out) return fail(-1, "bad arguments");
    std::memset(out, 0, sizeof(*out));
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(-2, std::string("cannot open ") + path);
    int64_t hdr[8];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || std::memcmp(hdr, "HELPLP01", 8) != 0) {
        std::fclose(f);
        return fail(-3, "not a HELPLP01 file");
    }
    const int64_t m = hdr[1], n = hdr[2], ns = hdr[3], nnz = hdr[4];
    if (m <= 0 || n <= 0 || ns < 0 || ns > n || nnz < 0 || m > 2000000000LL || n > 2000000000LL ||
        nnz > 2000000000LL) {
        std::fclose(f);
        return fail(-3, "bad header");
    }
    if (alloc_lp(out, (int32_t)m, (int32_t)n, nnz) != 0) {
        std::fclose(f);
        return fail(-2, "out of memory");
    }
    out->n_struct = (int32_t)ns;
    bool ok = true;
    auto get = [&](void* p, size_t bytes) {
        if (ok && bytes) ok = std::fread(p, 1, bytes, f) == bytes;
    };
    get(out->col_ptr, sizeof(int32_t) * ((size_t)n + 1));
    get(out->row_ind, sizeof(int32_t) * (size_t)nnz);
    get(out->val, sizeof(double) * (size_t)nnz);
    get(out->b, sizeof(double) * (size_t)m);
    get(out->c, sizeof(double) * (size_t)n);
    get(out->row_type, (size_t)m);
    std::fclose(f);
    if (!ok) {
        help_lp_free(out);
        return fail(-3, "truncated file");
    }
    // the arrays must describe a valid CSC matrix before anyone indexes with them
    bool valid = out->col_ptr[0] == 0 && out->col_ptr[n] == nnz;
    for (int64_t j = 0; valid && j < n; ++j) {
        if (out->col_ptr[j + 1] < out->col_ptr[j]) valid = false;
        for (int64_t q = out->col_ptr[j]; valid && q < out->col_ptr[j + 1]; ++q)
            if (out->row_ind[q] < 0 || out->row_ind[q] >= m || (q > out->col_ptr[j] && out->row_ind[q] <= out->row_ind[q - 1]))
                valid = false;
    }
    if (!valid) {
        help_lp_free(out);
        return fail(-3, "inconsistent column pointers or row indices");
    }
    return 0;
}

}  // extern "C"
