// gen.cpp -- seeded synthetic graphs and change batches (ER, RMAT, grid), plus the host
// helpers they share (error message, parallel radix sort).
//
// Every random value is a pure function of (seed, stream, index), so a generator gives the
// same output on any host and with any thread count.  "Exactly m distinct pairs" is defined
// as: draw candidates 0..D-1, deduplicate, and keep the m distinct pairs with the smallest
// hash; D grows until at least m distinct pairs exist.
#include <cmath>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <unordered_set>

#include <omp.h>

#include "../../include/dsssp.h"
#include "host_common.h"

namespace dsssp {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

const char* last_error() { return g_err; }

int num_host_threads() { return omp_get_max_threads(); }

void radix_sort_u64(std::vector<uint64_t>& keys) {
    const size_t n = keys.size();
    if (n < 2) return;
    uint64_t orv = 0, andv = ~0ull;
#pragma omp parallel for reduction(| : orv) reduction(& : andv)
    for (size_t i = 0; i < n; i++) {
        orv |= keys[i];
        andv &= keys[i];
    }
    const uint64_t varying = orv ^ andv;
    if (n < (1u << 16)) {
        std::sort(keys.begin(), keys.end());
        return;
    }
    std::vector<uint64_t> tmp(n);
    uint64_t* src = keys.data();
    uint64_t* dst = tmp.data();
    const int T = omp_get_max_threads();
    std::vector<size_t> hist((size_t)T * 256);
    for (int shift = 0; shift < 64; shift += 8) {
        if (((varying >> shift) & 0xFF) == 0) continue;
        std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(T)
        {
            const int t = omp_get_thread_num();
            const size_t lo = n * t / T, hi = n * (t + 1) / T;
            size_t* h = &hist[(size_t)t * 256];
            for (size_t i = lo; i < hi; i++) h[(src[i] >> shift) & 0xFF]++;
#pragma omp barrier
#pragma omp single
            {
                size_t sum = 0;
                for (int d = 0; d < 256; d++)
                    for (int q = 0; q < T; q++) {
                        size_t c = hist[(size_t)q * 256 + d];
                        hist[(size_t)q * 256 + d] = sum;
                        sum += c;
                    }
            }
            for (size_t i = lo; i < hi; i++) dst[h[(src[i] >> shift) & 0xFF]++] = src[i];
        }
        std::swap(src, dst);
    }
    if (src != keys.data()) memcpy(keys.data(), src, n * sizeof(uint64_t));
}

// Draws candidates with draw(i) -> key (~0ull = rejected), keeps the m distinct keys with the
// smallest hash, returns them sorted by that hash (a random order).  Gives up (false) once the
// draws pass 64 m + 2^20 without m distinct keys: the parameters cannot give that many (too
// few possible pairs, or a distribution that keeps drawing the same ones).
template <class Draw>
static bool distinct_keys(int64_t m, const Stream& hs, Draw draw, std::vector<uint64_t>& out) {
    int64_t D = m + m / 8 + 64;
    for (int attempt = 0; attempt < 40; attempt++) {
        std::vector<uint64_t> keys((size_t)D);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < D; i++) keys[(size_t)i] = draw((uint64_t)i);
        radix_sort_u64(keys);
        size_t u = 0;
        for (size_t i = 0; i < keys.size(); i++) {
            if (keys[i] == ~0ull) break;
            if (u == 0 || keys[u - 1] != keys[i]) keys[u++] = keys[i];
        }
        if ((int64_t)u >= m) {
            keys.resize(u);
            // rank by hash of the key: (hash, key) pairs sorted by hash; keep the first m
            std::vector<std::pair<uint64_t, uint64_t>> hk(u);
#pragma omp parallel for schedule(static)
            for (size_t i = 0; i < u; i++) hk[i] = {hs.at(keys[i]), keys[i]};
            std::nth_element(hk.begin(), hk.begin() + (m - 1 < 0 ? 0 : m - 1), hk.end());
            hk.resize((size_t)m);
            std::sort(hk.begin(), hk.end());
            out.resize((size_t)m);
            for (int64_t i = 0; i < m; i++) out[(size_t)i] = hk[(size_t)i].second;
            return true;
        }
        D = D + D / 2 + (m - (int64_t)u) * 2;
        if (D > 64 * m + (1 << 20)) break;
    }
    return false;
}

static int emit_edges(const std::vector<uint64_t>& keys, const Stream& ws, int32_t wlo,
                      int32_t whi, int32_t** u, int32_t** v, int32_t** w) {
    const size_t m = keys.size();
    int32_t* a = (int32_t*)malloc(sizeof(int32_t) * (m ? m : 1));
    int32_t* b = (int32_t*)malloc(sizeof(int32_t) * (m ? m : 1));
    int32_t* c = (int32_t*)malloc(sizeof(int32_t) * (m ? m : 1));
    if (!a || !b || !c) {
        free(a); free(b); free(c);
        return fail(DSSSP_E_OOM, "host allocation of %zu edges failed", m);
    }
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < m; i++) {
        a[i] = (int32_t)(keys[i] >> 32);
        b[i] = (int32_t)(keys[i] & 0xFFFFFFFFu);
        c[i] = (int32_t)ws.range(i, wlo, whi);
    }
    *u = a; *v = b; *w = c;
    return DSSSP_OK;
}

// RMAT quadrant walk: one uniform draw per level.
static inline uint64_t rmat_pair(const Stream& s, uint64_t i, int scale, double a, double ab,
                                 double abc) {
    uint32_t x = 0, y = 0;
    for (int l = 0; l < scale; l++) {
        double r = s.unit(i * (uint64_t)scale + (uint64_t)l);
        uint32_t bx = 0, by = 0;
        if (r < a) {
        } else if (r < ab) {
            by = 1;
        } else if (r < abc) {
            bx = 1;
        } else {
            bx = 1;
            by = 1;
        }
        x = (x << 1) | bx;
        y = (y << 1) | by;
    }
    return ((uint64_t)x << 32) | y;
}

}  // namespace dsssp

using namespace dsssp;

extern "C" {

const char* dsssp_last_error(void) { return dsssp::last_error(); }

void dsssp_free(void* p) { free(p); }

int dsssp_gen_er(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed, int32_t** u,
                 int32_t** v, int32_t** w) {
    if (n < 2 || m < 0 || wlo < 0 || whi < wlo || !u || !v || !w)
        return fail(DSSSP_E_INVAL, "gen_er: bad arguments");
    if ((double)m > (double)n * (n - 1) / 2.0)
        return fail(DSSSP_E_INVAL, "gen_er: %lld pairs do not exist on %d vertices", (long long)m, n);
    Stream ps(seed, 1), hs(seed, 2), ws(seed, 3);
    std::vector<uint64_t> keys;
    bool ok = distinct_keys(m, hs, [&](uint64_t i) {
        uint32_t a = (uint32_t)ps.range(2 * i, 0, n - 1), b = (uint32_t)ps.range(2 * i + 1, 0, n - 1);
        return a == b ? (uint64_t)~0ull : pair_key(a, b);
    }, keys);
    if (!ok) return fail(DSSSP_E_INVAL, "gen_er: could not draw %lld distinct pairs", (long long)m);
    return emit_edges(keys, ws, wlo, whi, u, v, w);
}

int dsssp_gen_rmat(int32_t scale, int64_t m, double a, double b, double c, int32_t wlo,
                   int32_t whi, uint64_t seed, int32_t** u, int32_t** v, int32_t** w) {
    if (scale < 1 || scale > 30 || m < 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 ||
        wlo < 0 || whi < wlo || !u || !v || !w)
        return fail(DSSSP_E_INVAL, "gen_rmat: bad arguments");
    if ((double)m > std::ldexp(1.0, scale) * (std::ldexp(1.0, scale) - 1) / 2.0)
        return fail(DSSSP_E_INVAL, "gen_rmat: %lld pairs do not exist on 2^%d vertices", (long long)m, scale);
    Stream ps(seed, 11), hs(seed, 12), ws(seed, 13);
    const double ab = a + b, abc = a + b + c;
    std::vector<uint64_t> keys;
    bool ok = distinct_keys(m, hs, [&](uint64_t i) {
        uint64_t p = rmat_pair(ps, i, scale, a, ab, abc);
        uint32_t x = (uint32_t)(p >> 32), y = (uint32_t)p;
        return x == y ? (uint64_t)~0ull : pair_key(x, y);
    }, keys);
    if (!ok) return fail(DSSSP_E_INVAL, "gen_rmat: could not draw %lld distinct pairs", (long long)m);
    return emit_edges(keys, ws, wlo, whi, u, v, w);
}

int dsssp_gen_grid(int32_t rows, int32_t cols, double remove_frac, int64_t n_diag, int32_t wlo,
                   int32_t whi, uint64_t seed, int32_t** u, int32_t** v, int32_t** w,
                   int64_t* m_out) {
    if (rows < 1 || cols < 1 || (int64_t)rows * cols > INT32_MAX || remove_frac < 0 ||
        remove_frac >= 1 || n_diag < 0 || wlo < 0 || whi < wlo || !u || !v || !w || !m_out)
        return fail(DSSSP_E_INVAL, "gen_grid: bad arguments");
    const int64_t nh = (int64_t)rows * (cols - 1), nv = (int64_t)(rows - 1) * cols;
    const int64_t E = nh + nv;
    const int64_t n_remove = (int64_t)(remove_frac * (double)E);
    Stream rs(seed, 21), ds(seed, 22), hs(seed, 23), ws(seed, 24);
    // keep the E - n_remove grid edges with the largest hash rank: rank by (hash, index)
    std::vector<uint64_t> keep_keys;
    {
        std::vector<std::pair<uint64_t, int64_t>> hk((size_t)E);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < E; i++) hk[(size_t)i] = {rs.at((uint64_t)i), i};
        if (n_remove > 0) std::nth_element(hk.begin(), hk.begin() + (n_remove - 1), hk.end());
        std::vector<int64_t> idx;
        idx.reserve((size_t)(E - n_remove));
        for (int64_t i = n_remove; i < E; i++) idx.push_back(hk[(size_t)i].second);
        std::sort(idx.begin(), idx.end());
        keep_keys.resize(idx.size());
#pragma omp parallel for schedule(static)
        for (size_t j = 0; j < idx.size(); j++) {
            int64_t i = idx[j];
            uint32_t a, b;
            if (i < nh) {
                int64_t r = i / (cols - 1), c = i % (cols - 1);
                a = (uint32_t)(r * cols + c);
                b = a + 1;
            } else {
                int64_t k = i - nh, r = k / cols, c = k % cols;
                a = (uint32_t)(r * cols + c);
                b = a + (uint32_t)cols;
            }
            keep_keys[j] = pair_key(a, b);
        }
    }
    std::vector<uint64_t> diag;
    if (n_diag > 0) {
        if (rows < 2 || cols < 2) return fail(DSSSP_E_INVAL, "gen_grid: no diagonals on a line");
        if (n_diag > 2 * (int64_t)(rows - 1) * (cols - 1))
            return fail(DSSSP_E_INVAL, "gen_grid: a %d x %d grid has only %lld diagonals", rows, cols,
                        2 * (long long)(rows - 1) * (cols - 1));
        bool ok = distinct_keys(n_diag, hs, [&](uint64_t i) {
            int64_t r = ds.range(3 * i, 0, rows - 1), c = ds.range(3 * i + 1, 0, cols - 1);
            int64_t d = ds.range(3 * i + 2, 0, 3);
            int64_t r2 = r + ((d & 1) ? 1 : -1), c2 = c + ((d & 2) ? 1 : -1);
            if (r2 < 0 || r2 >= rows || c2 < 0 || c2 >= cols) return (uint64_t)~0ull;
            return pair_key((uint32_t)(r * cols + c), (uint32_t)(r2 * cols + c2));
        }, diag);
        if (!ok) return fail(DSSSP_E_INVAL, "gen_grid: could not draw %lld diagonals", (long long)n_diag);
    }
    keep_keys.insert(keep_keys.end(), diag.begin(), diag.end());
    *m_out = (int64_t)keep_keys.size();
    return emit_edges(keep_keys, ws, wlo, whi, u, v, w);
}

int32_t dsssp_max_degree_vertex(int32_t n, int64_t m, const int32_t* u, const int32_t* v) {
    if (n <= 0) return -1;
    std::vector<int64_t> deg((size_t)n, 0);
    for (int64_t i = 0; i < m; i++) {
        if (u[i] >= 0 && u[i] < n) deg[(size_t)u[i]]++;
        if (v[i] >= 0 && v[i] < n) deg[(size_t)v[i]]++;
    }
    int32_t best = 0;
    for (int32_t x = 1; x < n; x++)
        if (deg[(size_t)x] > deg[(size_t)best]) best = x;
    return best;
}

int dsssp_gen_changes(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                      const int32_t* ew, int64_t n_ins, int64_t n_del, int32_t ins_kind,
                      int32_t scale, double p0, double p1, double p2, int32_t wlo, int32_t whi,
                      uint64_t seed, dsssp_change** changes) {
    if (n < 2 || m < 0 || n_ins < 0 || n_del < 0 || n_del > m || wlo < 0 || whi < wlo || !changes)
        return fail(DSSSP_E_INVAL, "gen_changes: bad arguments");
    if (ins_kind == DSSSP_INS_RMAT && (scale < 1 || (1ll << scale) > n))
        return fail(DSSSP_E_INVAL, "gen_changes: rmat scale %d does not fit %d vertices", scale, n);
    if (ins_kind == DSSSP_INS_LOCAL && (scale < 1 || n % scale != 0 || p0 < 1))
        return fail(DSSSP_E_INVAL, "gen_changes: local insertions need cols | n and radius >= 1");
    Stream is(seed, 31), ws(seed, 32), dsel(seed, 33), sh(seed, 34);
    std::vector<uint64_t> existing((size_t)m);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; i++) existing[(size_t)i] = pair_key((uint32_t)eu[i], (uint32_t)ev[i]);
    radix_sort_u64(existing);

    std::vector<dsssp_change> out;
    out.reserve((size_t)(n_ins + n_del));
    // insertions: sequential draws, new pairs only, distinct within the batch
    std::unordered_set<uint64_t> seen;
    seen.reserve((size_t)n_ins * 2 + 16);
    const double ab = p0 + p1, abc = p0 + p1 + p2;
    const int64_t radius = (int64_t)p0, cols = scale, rows = scale > 0 ? n / scale : 0;
    uint64_t i = 0;
    const uint64_t draw_cap = (uint64_t)(n_ins + 16) * 1000;
    while ((int64_t)seen.size() < n_ins) {
        if (i > draw_cap) return fail(DSSSP_E_INVAL, "gen_changes: cannot find %lld new pairs", (long long)n_ins);
        const uint64_t draw = i++;
        uint32_t a, b;
        if (ins_kind == DSSSP_INS_RMAT) {
            uint64_t p = rmat_pair(is, draw, scale, p0, ab, abc);
            a = (uint32_t)(p >> 32);
            b = (uint32_t)p;
        } else if (ins_kind == DSSSP_INS_LOCAL) {
            int64_t r = is.range(4 * draw, 0, rows - 1), c = is.range(4 * draw + 1, 0, cols - 1);
            int64_t r2 = r + is.range(4 * draw + 2, -radius, radius);
            int64_t c2 = c + is.range(4 * draw + 3, -radius, radius);
            if (r2 < 0 || r2 >= rows || c2 < 0 || c2 >= cols) continue;
            a = (uint32_t)(r * cols + c);
            b = (uint32_t)(r2 * cols + c2);
        } else {
            a = (uint32_t)is.range(2 * draw, 0, n - 1);
            b = (uint32_t)is.range(2 * draw + 1, 0, n - 1);
        }
        if (a == b) continue;
        uint64_t key = pair_key(a, b);
        if (std::binary_search(existing.begin(), existing.end(), key)) continue;
        if (!seen.insert(key).second) continue;
        out.push_back(dsssp_change{(int32_t)a, (int32_t)b, (int32_t)ws.range(draw, wlo, whi), 1});
    }
    // deletions: Floyd's sampling of n_del distinct line indices
    {
        std::unordered_set<int64_t> pick;
        pick.reserve((size_t)n_del * 2 + 16);
        std::vector<int64_t> order;
        order.reserve((size_t)n_del);
        for (int64_t j = m - n_del; j < m; j++) {
            int64_t t = dsel.range((uint64_t)j, 0, j);
            int64_t chosen = pick.count(t) ? j : t;
            pick.insert(chosen);
            order.push_back(chosen);
        }
        for (int64_t li : order) out.push_back(dsssp_change{eu[li], ev[li], ew[li], 0});
    }
    // shuffle (Fisher-Yates)
    for (int64_t j = (int64_t)out.size() - 1; j > 0; j--) {
        int64_t t = sh.range((uint64_t)j, 0, j);
        std::swap(out[(size_t)j], out[(size_t)t]);
    }
    dsssp_change* res = (dsssp_change*)malloc(sizeof(dsssp_change) * (out.size() ? out.size() : 1));
    if (!res) return fail(DSSSP_E_OOM, "gen_changes: host allocation failed");
    if (!out.empty()) memcpy(res, out.data(), sizeof(dsssp_change) * out.size());
    *changes = res;
    return DSSSP_OK;
}

// The reference generator's sampling (createChangedEdges.cpp:75-122) with a seeded stream in
// place of rand(): num_changes records, (int)(num_changes * ins_pct / 100) of them insertions.
// Each step flips a coin; heads draws an insertion -- a uniform pair, redrawn when both ends
// are equal, ordered u < v, weight uniform in [wlo, whi] (the reference: rand() % 100, i.e.
// [0, 99]), possibly an existing edge or a repeat -- and tails a deletion of a uniform line of
// the edge list, with replacement.  Records come out in draw order.  Allocates *changes.
int dsssp_gen_changes_ref(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev, const int32_t* ew,
                          int64_t num_changes, int32_t ins_pct, int32_t wlo, int32_t whi, uint64_t seed,
                          dsssp_change** changes) {
    if (n < 2 || m < 0 || num_changes < 0 || ins_pct < 0 || ins_pct > 100 || wlo < 0 || whi < wlo || !changes)
        return fail(DSSSP_E_INVAL, "gen_changes_ref: bad arguments");
    const int64_t n_ins = (int64_t)((double)num_changes * ((double)ins_pct / 100.0));
    const int64_t n_del = num_changes - n_ins;
    if (n_del > 0 && (m == 0 || !eu || !ev || !ew)) return fail(DSSSP_E_INVAL, "gen_changes_ref: no lines to delete");
    Stream coin(seed, 41), pick(seed, 42), wt(seed, 43), del(seed, 44);
    std::vector<dsssp_change> out;
    out.reserve((size_t)num_changes);
    int64_t ii = 0, id = 0;
    uint64_t step = 0;
    const uint64_t cap = (uint64_t)(num_changes + 16) * 64;
    while (ii < n_ins || id < n_del) {
        if (step > cap) return fail(DSSSP_E_INVAL, "gen_changes_ref: too many redraws");
        const uint64_t s = step++;
        if (coin.at(s) & 1) {
            if (ii >= n_ins) continue;
            const int32_t x = (int32_t)pick.range(2 * s, 0, n - 1), y = (int32_t)pick.range(2 * s + 1, 0, n - 1);
            if (x == y) continue;
            out.push_back(dsssp_change{x < y ? x : y, x < y ? y : x, (int32_t)wt.range(s, wlo, whi), 1});
            ii++;
        } else {
            if (id >= n_del) continue;
            const int64_t li = del.range(s, 0, m - 1);
            out.push_back(dsssp_change{eu[li], ev[li], ew[li], 0});
            id++;
        }
    }
    dsssp_change* res = (dsssp_change*)malloc(sizeof(dsssp_change) * (out.size() ? out.size() : 1));
    if (!res) return fail(DSSSP_E_OOM, "gen_changes_ref: host allocation failed");
    if (!out.empty()) memcpy(res, out.data(), sizeof(dsssp_change) * out.size());
    *changes = res;
    return DSSSP_OK;
}

}  // extern "C"
