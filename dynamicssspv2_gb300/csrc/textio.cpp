// textio.cpp -- readers and writer for the reference's three text formats
// (graph "u v w", changes "u v w op", SSSP "node parent dist"; README.md:25-37).
//
// The reference reads them with fgets + sscanf (all_structure_undir.cuh:89-198).  These
// readers keep its field semantics and parse the file in parallel chunks split at line
// boundaries.  Deliberate differences: a line with too few fields is skipped (sscanf would
// leave stale values), and an out-of-range vertex id is an error code instead of an
// uncaught std::out_of_range.
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <omp.h>

#include "../../include/dsssp.h"
#include "host_common.h"

namespace dsssp {
namespace {

// "no out-of-range vertex id in this chunk" (any id a file can name, -1 included, is reported)
constexpr long long kNoBadId = LLONG_MIN;

struct FileBuf {
    std::vector<char> data;
};

int slurp(const char* path, FileBuf& fb) {
    FILE* f = fopen(path, "rb");
    if (!f) return fail(DSSSP_E_IO, "cannot open %s: %s", path, strerror(errno));
    if (fseek(f, 0, SEEK_END) != 0) { fclose(f); return fail(DSSSP_E_IO, "cannot seek %s", path); }
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    fb.data.resize((size_t)(sz > 0 ? sz : 0) + 1);
    size_t got = sz > 0 ? fread(fb.data.data(), 1, (size_t)sz, f) : 0;
    fclose(f);
    fb.data.resize(got + 1);
    fb.data[got] = '\n';
    return DSSSP_OK;
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Parses one integer field; returns false at end of line or when the next token is not a
// number.  Without flt it reads like the reference's sscanf("%d"): the integer prefix of the
// token ("2.5" gives 2, and ".5" then counts as a field that is not a number).  With flt (the
// distance column of an SSSP file, which the reference's Dijkstra writes through cout, e.g.
// "1.2e+06") a token in floating-point form is read whole and rounded, and *flt is set.
inline bool next_int(const char*& p, const char* end, long long& out, bool* flt) {
    while (p < end && is_space(*p)) p++;
    if (p >= end || *p == '\n') return false;
    const char* s = p;
    bool neg = false;
    if (*p == '-' || *p == '+') { neg = *p == '-'; p++; }
    long long v = 0;
    bool any = false;
    while (p < end && *p >= '0' && *p <= '9') {  // saturates: such a value is out of range anyway
        const int d = *p - '0';
        v = v > (LLONG_MAX - d) / 10 ? LLONG_MAX : v * 10 + d;
        p++;
        any = true;
    }
    if (flt && p < end && (*p == '.' || *p == 'e' || *p == 'E')) {
        char* q = nullptr;
        double d = strtod(s, &q);
        p = q;
        if (flt) *flt = true;
        out = (long long)llround(d);
        return true;
    }
    if (!any) {  // not a number: skip the token, report no value
        while (p < end && !is_space(*p) && *p != '\n') p++;
        return false;
    }
    out = neg ? -v : v;
    return true;
}

// Splits the buffer into T chunks at newlines; calls parse(t, lo, hi) per chunk in parallel.
template <class F>
void parallel_lines(const FileBuf& fb, F parse, int T) {
    const char* base = fb.data.data();
    const size_t n = fb.data.size();
    std::vector<size_t> cut((size_t)T + 1, n);
    cut[0] = 0;
    for (int t = 1; t < T; t++) {
        size_t c = n * (size_t)t / (size_t)T;
        if (c < cut[(size_t)t - 1]) c = cut[(size_t)t - 1];
        while (c < n && base[c - 1] != '\n') c++;
        cut[(size_t)t] = c;
    }
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; t++) parse(t, base + cut[(size_t)t], base + cut[(size_t)t + 1]);
}

int chunks_for(size_t bytes) {
    int T = omp_get_max_threads();
    int byb = (int)(bytes / (1 << 20)) + 1;
    return T < byb ? T : byb;
}

}  // namespace
}  // namespace dsssp

using namespace dsssp;

extern "C" {

int dsssp_read_graph_file(const char* path, int32_t n, int32_t** u, int32_t** v, int32_t** w,
                          int64_t* m) {
    if (!path || n <= 0 || !u || !v || !w || !m) return fail(DSSSP_E_INVAL, "read_graph: bad arguments");
    FileBuf fb;
    int rc = slurp(path, fb);
    if (rc) return rc;
    const int T = chunks_for(fb.data.size());
    std::vector<std::vector<int32_t>> A((size_t)T), B((size_t)T), W((size_t)T);
    std::vector<long long> bad((size_t)T, kNoBadId);
    parallel_lines(fb, [&](int t, const char* p, const char* end) {
        while (p < end) {
            long long x[3];
            int k = 0;
            while (k < 3 && next_int(p, end, x[k], nullptr)) k++;
            while (p < end && *p != '\n') p++;
            p++;
            if (k < 3) continue;
            if (x[0] < 0 || x[0] >= n || x[1] < 0 || x[1] >= n) { bad[(size_t)t] = x[0] < 0 || x[0] >= n ? x[0] : x[1]; continue; }
            A[(size_t)t].push_back((int32_t)x[0]);
            B[(size_t)t].push_back((int32_t)x[1]);
            W[(size_t)t].push_back((int32_t)x[2]);
        }
    }, T);
    for (int t = 0; t < T; t++)
        if (bad[(size_t)t] != kNoBadId)
            return fail(DSSSP_E_BAD_VERTEX, "%s: vertex id %lld outside 0..%d", path, bad[(size_t)t], n - 1);
    size_t tot = 0;
    for (int t = 0; t < T; t++) tot += A[(size_t)t].size();
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (tot ? tot : 1));
    int32_t* b = (int32_t*)malloc(sizeof(int32_t) * (tot ? tot : 1));
    int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (tot ? tot : 1));
    if (!a || !b || !c) { free(a); free(b); free(c); return fail(DSSSP_E_OOM, "read_graph: out of host memory"); }
    size_t o = 0;
    for (int t = 0; t < T; t++) {
        size_t s = A[(size_t)t].size();
        if (s == 0) continue;
        memcpy(a + o, A[(size_t)t].data(), s * 4);
        memcpy(b + o, B[(size_t)t].data(), s * 4);
        memcpy(c + o, W[(size_t)t].data(), s * 4);
        o += s;
    }
    *u = a; *v = b; *w = c; *m = (int64_t)tot;
    return DSSSP_OK;
}

int dsssp_read_changes_file(const char* path, int32_t n, dsssp_change** changes, int64_t* k) {
    if (!path || n <= 0 || !changes || !k) return fail(DSSSP_E_INVAL, "read_changes: bad arguments");
    FileBuf fb;
    int rc = slurp(path, fb);
    if (rc) return rc;
    const int T = chunks_for(fb.data.size());
    std::vector<std::vector<dsssp_change>> C((size_t)T);
    std::vector<long long> bad((size_t)T, kNoBadId);
    parallel_lines(fb, [&](int t, const char* p, const char* end) {
        while (p < end) {
            long long x[4];
            int q = 0;
            while (q < 4 && next_int(p, end, x[q], nullptr)) q++;
            while (p < end && *p != '\n') p++;
            p++;
            if (q < 4) continue;
            if ((x[3] == 0 || x[3] == 1) && (x[0] < 0 || x[0] >= n || x[1] < 0 || x[1] >= n)) {
                bad[(size_t)t] = x[0] < 0 || x[0] >= n ? x[0] : x[1];
                continue;
            }
            C[(size_t)t].push_back(dsssp_change{(int32_t)x[0], (int32_t)x[1], (int32_t)x[2], (int32_t)x[3]});
        }
    }, T);
    for (int t = 0; t < T; t++)
        if (bad[(size_t)t] != kNoBadId)
            return fail(DSSSP_E_BAD_VERTEX, "%s: vertex id %lld outside 0..%d", path, bad[(size_t)t], n - 1);
    size_t tot = 0;
    for (auto& c : C) tot += c.size();
    dsssp_change* out = (dsssp_change*)malloc(sizeof(dsssp_change) * (tot ? tot : 1));
    if (!out) return fail(DSSSP_E_OOM, "read_changes: out of host memory");
    size_t o = 0;
    for (auto& c : C) {
        if (c.empty()) continue;
        memcpy(out + o, c.data(), c.size() * sizeof(dsssp_change));
        o += c.size();
    }
    *changes = out;
    *k = (int64_t)tot;
    return DSSSP_OK;
}

int dsssp_read_sssp_file(const char* path, int32_t n, int32_t* parent, int64_t* dist,
                         int64_t* lossy) {
    if (!path || n <= 0 || !parent || !dist) return fail(DSSSP_E_INVAL, "read_sssp: bad arguments");
    FileBuf fb;
    int rc = slurp(path, fb);
    if (rc) return rc;
    for (int32_t i = 0; i < n; i++) { parent[i] = -1; dist[i] = DSSSP_UNREACHABLE; }
    const int T = chunks_for(fb.data.size());
    std::vector<long long> bad((size_t)T, kNoBadId), nflt((size_t)T, 0);
    // every vertex appears on at most one line in a well-formed file; with duplicates the
    // last line in file order wins (as in the reference), so chunks are applied in order
    std::vector<std::vector<long long>> rows((size_t)T);
    parallel_lines(fb, [&](int t, const char* p, const char* end) {
        while (p < end) {
            long long x[3];
            bool flt = false;
            int q = 0;
            while (q < 3 && next_int(p, end, x[q], q == 2 ? &flt : nullptr)) q++;
            while (p < end && *p != '\n') p++;
            p++;
            if (q < 3) continue;
            if (x[0] < 0 || x[0] >= n) { bad[(size_t)t] = x[0]; continue; }
            if (flt) nflt[(size_t)t]++;
            rows[(size_t)t].push_back(x[0]);
            rows[(size_t)t].push_back(x[1]);
            rows[(size_t)t].push_back(x[2]);
        }
    }, T);
    for (int t = 0; t < T; t++)
        if (bad[(size_t)t] != kNoBadId)
            return fail(DSSSP_E_BAD_VERTEX, "%s: vertex id %lld outside 0..%d", path, bad[(size_t)t], n - 1);
    long long nl = 0;
    for (int t = 0; t < T; t++) {
        nl += nflt[(size_t)t];
        const auto& r = rows[(size_t)t];
        for (size_t i = 0; i + 2 < r.size(); i += 3) {
            int32_t node = (int32_t)r[i];
            long long par = r[i + 1];
            if (par == -1) { parent[node] = -1; dist[node] = DSSSP_UNREACHABLE; }  // read_SSSP:153-156
            else { parent[node] = (int32_t)par; dist[node] = r[i + 2]; }
        }
    }
    if (lossy) *lossy = nl;
    return DSSSP_OK;
}

int dsssp_write_sssp_file(const char* path, int32_t n, const int32_t* parent, const int64_t* dist) {
    if (!path || n < 0 || !parent || !dist) return fail(DSSSP_E_INVAL, "write_sssp: bad arguments");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DSSSP_E_IO, "cannot create %s: %s", path, strerror(errno));
    std::vector<char> buf;
    buf.reserve(1 << 22);
    char tmp[80];
    for (int32_t i = 0; i < n; i++) {
        int len;
        if (parent[i] == -1) len = snprintf(tmp, sizeof(tmp), "%d -1 -1\n", i);
        else len = snprintf(tmp, sizeof(tmp), "%d %d %lld\n", i, parent[i], (long long)dist[i]);
        buf.insert(buf.end(), tmp, tmp + len);
        if (buf.size() > (1 << 22) - 100) {
            if (fwrite(buf.data(), 1, buf.size(), f) != buf.size()) { fclose(f); return fail(DSSSP_E_IO, "write to %s failed", path); }
            buf.clear();
        }
    }
    if (!buf.empty() && fwrite(buf.data(), 1, buf.size(), f) != buf.size()) { fclose(f); return fail(DSSSP_E_IO, "write to %s failed", path); }
    if (fclose(f) != 0) return fail(DSSSP_E_IO, "closing %s failed", path);
    return DSSSP_OK;
}

// Change records in the line format the reference's generator prints (createChangedEdges.cpp:
// 104 for insertions, 116 for deletions): "u  v w 1 " and "u v w 0 ", each with a trailing
// space.  Records with another op keep the deletion layout with their op.
int dsssp_write_changes_file(const char* path, const dsssp_change* changes, int64_t k) {
    if (!path || k < 0 || (k > 0 && !changes)) return fail(DSSSP_E_INVAL, "write_changes: bad arguments");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DSSSP_E_IO, "cannot create %s: %s", path, strerror(errno));
    std::vector<char> buf;
    buf.reserve(1 << 22);
    char tmp[96];
    for (int64_t i = 0; i < k; i++) {
        const dsssp_change& c = changes[i];
        const int len = c.op == 1 ? snprintf(tmp, sizeof(tmp), "%d  %d %d 1 \n", c.u, c.v, c.w)
                                  : snprintf(tmp, sizeof(tmp), "%d %d %d %d \n", c.u, c.v, c.w, c.op);
        buf.insert(buf.end(), tmp, tmp + len);
        if (buf.size() > (1 << 22) - 128) {
            if (fwrite(buf.data(), 1, buf.size(), f) != buf.size()) { fclose(f); return fail(DSSSP_E_IO, "write to %s failed", path); }
            buf.clear();
        }
    }
    if (!buf.empty() && fwrite(buf.data(), 1, buf.size(), f) != buf.size()) { fclose(f); return fail(DSSSP_E_IO, "write to %s failed", path); }
    if (fclose(f) != 0) return fail(DSSSP_E_IO, "closing %s failed", path);
    return DSSSP_OK;
}

}  // extern "C"
