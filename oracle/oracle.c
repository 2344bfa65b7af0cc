/*
 * oracle.c -- CPU oracle for the dynamic SSSP batch update (test infrastructure only;
 * see oracle.h for what it restates and how it is pinned).
 */
#include "oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------ */
/* Updated graph (all_structure_undir.cuh:89-126 + gpuFunctions_undir.cuh:179-215)       */
/* ------------------------------------------------------------------------------------ */

static uint64_t pair_key(int32_t a, int32_t b) {
    uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
    return ((uint64_t)lo << 32) | hi;
}

/* open-addressing set of (endpoint pair, weight) deletion keys */
typedef struct {
    uint64_t* pair;
    int32_t* w;
    uint8_t* used;
    uint64_t mask;
} del_set;

static uint64_t mix_key(uint64_t p, int32_t w) {
    uint64_t z = p ^ ((uint64_t)(uint32_t)w * 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void del_set_init(del_set* s, int64_t n) {
    uint64_t cap = 16;
    while (cap < (uint64_t)n * 2 + 16) cap <<= 1;
    s->pair = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    s->w = (int32_t*)malloc(sizeof(int32_t) * cap);
    s->used = (uint8_t*)calloc(cap, 1);
    s->mask = cap - 1;
}

static void del_set_free(del_set* s) { free(s->pair); free(s->w); free(s->used); }

static void del_set_add(del_set* s, uint64_t p, int32_t w) {
    uint64_t h = mix_key(p, w) & s->mask;
    while (s->used[h]) {
        if (s->pair[h] == p && s->w[h] == w) return;
        h = (h + 1) & s->mask;
    }
    s->used[h] = 1; s->pair[h] = p; s->w[h] = w;
}

static int del_set_has(const del_set* s, uint64_t p, int32_t w) {
    uint64_t h = mix_key(p, w) & s->mask;
    while (s->used[h]) {
        if (s->pair[h] == p && s->w[h] == w) return 1;
        h = (h + 1) & s->mask;
    }
    return 0;
}

/* Marks which lines (m base lines followed by the insertions, in batch order) survive. */
static int64_t mark_lines(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                          const int32_t* ew, int64_t k, const int32_t* cu, const int32_t* cv,
                          const int32_t* cw, const int32_t* cop, uint8_t* keep,
                          int64_t* n_lines_out) {
    int64_t n_ins = 0, n_del = 0;
    for (int64_t i = 0; i < k; i++) {
        if (cop[i] == 1) n_ins++;
        else if (cop[i] == 0) n_del++;
    }
    del_set ds;
    del_set_init(&ds, n_del);
    for (int64_t i = 0; i < k; i++) {
        if (cop[i] != 0 && cop[i] != 1) continue;
        if (cu[i] < 0 || cu[i] >= n || cv[i] < 0 || cv[i] >= n) {
            del_set_free(&ds);
            return -1;
        }
        if (cop[i] == 0) del_set_add(&ds, pair_key(cu[i], cv[i]), cw[i]);
    }
    int64_t L = m + n_ins, line = 0, nnz = 0;
    for (int64_t i = 0; i < m + k; i++) {
        int32_t a, b, w;
        if (i < m) {
            a = eu[i]; b = ev[i]; w = ew[i];
            if (a < 0 || a >= n || b < 0 || b >= n) { del_set_free(&ds); return -1; }
        } else {
            int64_t c = i - m;
            if (cop[c] != 1) continue;
            a = cu[c]; b = cv[c]; w = cw[c];
        }
        int alive = n_del == 0 || !del_set_has(&ds, pair_key(a, b), w);
        keep[line++] = (uint8_t)alive;
        if (alive) nnz += 2;
    }
    del_set_free(&ds);
    *n_lines_out = L;
    return nnz;
}

int64_t orc_updated_graph_nnz(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                              const int32_t* ew, int64_t k, const int32_t* cu, const int32_t* cv,
                              const int32_t* cw, const int32_t* cop) {
    uint8_t* keep = (uint8_t*)malloc((size_t)(m + k + 1));
    int64_t L = 0;
    int64_t nnz = mark_lines(n, m, eu, ev, ew, k, cu, cv, cw, cop, keep, &L);
    free(keep);
    return nnz;
}

int64_t orc_updated_graph(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                          const int32_t* ew, int64_t k, const int32_t* cu, const int32_t* cv,
                          const int32_t* cw, const int32_t* cop, int64_t* off, int32_t* col,
                          int32_t* wt, uint8_t* kept_lines) {
    uint8_t* keep = (uint8_t*)malloc((size_t)(m + k + 1));
    int64_t L = 0;
    int64_t nnz = mark_lines(n, m, eu, ev, ew, k, cu, cv, cw, cop, keep, &L);
    if (nnz < 0) { free(keep); return -1; }
    if (kept_lines) memcpy(kept_lines, keep, (size_t)L);
    /* counting sort by row, keeping line order inside each row */
    memset(off, 0, sizeof(int64_t) * (size_t)(n + 1));
    int64_t line = 0;
    for (int64_t i = 0; i < m + k; i++) {
        int32_t a, b;
        if (i < m) { a = eu[i]; b = ev[i]; }
        else { int64_t c = i - m; if (cop[c] != 1) continue; a = cu[c]; b = cv[c]; }
        if (keep[line++]) { off[a + 1]++; off[b + 1]++; }
    }
    for (int32_t v = 0; v < n; v++) off[v + 1] += off[v];
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)n);
    line = 0;
    for (int64_t i = 0; i < m + k; i++) {
        int32_t a, b, w;
        if (i < m) { a = eu[i]; b = ev[i]; w = ew[i]; }
        else {
            int64_t c = i - m;
            if (cop[c] != 1) continue;
            a = cu[c]; b = cv[c]; w = cw[c];
        }
        if (!keep[line++]) continue;
        /* seqSSSPwithDist_undir.cpp:50-58: row n1 gets n2, then row n2 gets n1 */
        col[cur[a]] = b; wt[cur[a]] = w; cur[a]++;
        col[cur[b]] = a; wt[cur[b]] = w; cur[b]++;
    }
    free(cur);
    free(keep);
    return nnz;
}

int64_t orc_csr_from_edges(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                           const int32_t* ew, int64_t* off, int32_t* col, int32_t* wt) {
    return orc_updated_graph(n, m, eu, ev, ew, 0, NULL, NULL, NULL, NULL, off, col, wt, NULL);
}

/* ------------------------------------------------------------------------------------ */
/* Sequential Dijkstra (seqSSSPwithDist_undir.cpp:66-128)                                */
/* ------------------------------------------------------------------------------------ */

/* The reference keys its min-heap by pair<int,double>(dist at push time, vertex); a vertex
 * is in the heap at most once (the inQ flag), so all keys are distinct and any correct
 * priority queue pops them in the same order. */
typedef struct {
    int64_t key;
    int32_t v;
} heap_item;

static int item_less(heap_item a, heap_item b) {
    return a.key < b.key || (a.key == b.key && a.v < b.v);
}

static void heap_push(heap_item* h, int64_t* sz, heap_item it) {
    int64_t i = (*sz)++;
    while (i > 0) {
        int64_t p = (i - 1) >> 1;
        if (!item_less(it, h[p])) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = it;
}

static heap_item heap_pop(heap_item* h, int64_t* sz) {
    heap_item top = h[0];
    heap_item last = h[--(*sz)];
    int64_t i = 0, s = *sz;
    for (;;) {
        int64_t c = 2 * i + 1;
        if (c >= s) break;
        if (c + 1 < s && item_less(h[c + 1], h[c])) c++;
        if (!item_less(h[c], last)) break;
        h[i] = h[c];
        i = c;
    }
    if (s > 0) h[i] = last;
    return top;
}

int64_t orc_dijkstra(int32_t n, const int64_t* off, const int32_t* col, const int32_t* wt,
                     int32_t src, int64_t inf_cap, int64_t* dist, int32_t* parent) {
    for (int32_t v = 0; v < n; v++) { dist[v] = inf_cap; parent[v] = -1; }
    if (src < 0 || src >= n) return 0;
    dist[src] = 0;
    parent[src] = src;
    uint8_t* inq = (uint8_t*)calloc((size_t)n, 1);
    heap_item* h = (heap_item*)malloc(sizeof(heap_item) * (size_t)n);
    int64_t sz = 0, pops = 0;
    heap_item s0 = {0, src};
    heap_push(h, &sz, s0);
    inq[src] = 1;
    while (sz > 0) {
        heap_item it = heap_pop(h, &sz);
        int32_t u = it.v;
        inq[u] = 0;
        pops++;
        int64_t du = dist[u];
        for (int64_t j = off[u]; j < off[u + 1]; j++) {
            int32_t v = col[j];
            int64_t nd = du + (int64_t)wt[j];
            if (dist[v] > nd) {
                dist[v] = nd;
                parent[v] = u;
                if (!inq[v]) {
                    heap_item x = {nd, v};
                    heap_push(h, &sz, x);
                    inq[v] = 1;
                }
            }
            du = dist[u]; /* the reference re-reads dist[u] every iteration */
        }
    }
    free(h);
    free(inq);
    return pops;
}

/* ------------------------------------------------------------------------------------ */
/* Shortest-path-tree validator                                                         */
/* ------------------------------------------------------------------------------------ */

static int fail(char* msg, int32_t len, int code, const char* fmt, long long a, long long b,
                long long c) {
    if (msg && len > 0) snprintf(msg, (size_t)len, fmt, a, b, c);
    return code;
}

int orc_validate_tree(int32_t n, const int64_t* off, const int32_t* col, const int32_t* wt,
                      int32_t src, const int64_t* dist, const int32_t* parent, int64_t unreach,
                      char* msg, int32_t msglen) {
    if (n <= 0 || src < 0 || src >= n) return fail(msg, msglen, 1, "bad source %lld%lld%lld", src, 0, 0);
    if (dist[src] != 0 || parent[src] != src)
        return fail(msg, msglen, 2, "source %lld has dist %lld parent %lld", src, dist[src],
                    parent[src]);
    for (int32_t v = 0; v < n; v++) {
        if (v == src) continue;
        int32_t p = parent[v];
        if (p == -1) {
            if (dist[v] != unreach)
                return fail(msg, msglen, 3, "vertex %lld unreachable but dist %lld%lld", v,
                            dist[v], 0);
            continue;
        }
        if (p < 0 || p >= n || parent[p] == -1)
            return fail(msg, msglen, 4, "vertex %lld has bad parent %lld%lld", v, p, 0);
        int64_t need = dist[v] - dist[p];
        int ok = 0;
        for (int64_t j = off[v]; j < off[v + 1] && !ok; j++)
            if (col[j] == p && wt[j] >= 0 && (int64_t)wt[j] == need) ok = 1;
        if (!ok)
            return fail(msg, msglen, 5, "vertex %lld: no live edge from parent %lld of weight %lld",
                        v, p, need);
    }
    for (int32_t u = 0; u < n; u++) {
        if (parent[u] == -1) continue;
        for (int64_t j = off[u]; j < off[u + 1]; j++) {
            if (wt[j] < 0) continue;
            int32_t c = col[j];
            if (parent[c] == -1)
                return fail(msg, msglen, 6, "vertex %lld unreachable but neighbour %lld is reachable%lld",
                            c, u, 0);
            if (dist[u] + (int64_t)wt[j] < dist[c])
                return fail(msg, msglen, 7, "edge %lld->%lld relaxes (dist %lld)", u, c, dist[c]);
        }
    }
    /* acyclicity: 0 = unknown, 1 = on the current walk, 2 = reaches the source */
    uint8_t* st = (uint8_t*)calloc((size_t)n, 1);
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    st[src] = 2;
    int rc = 0;
    for (int32_t v = 0; v < n && !rc; v++) {
        if (parent[v] == -1 || st[v] == 2) continue;
        int64_t top = 0;
        int32_t x = v;
        while (st[x] == 0) {
            st[x] = 1;
            stack[top++] = x;
            x = parent[x];
        }
        if (st[x] == 1) rc = fail(msg, msglen, 8, "parent cycle through vertex %lld%lld%lld", x, 0, 0);
        while (top > 0) st[stack[--top]] = 2;
    }
    free(stack);
    free(st);
    return rc;
}

/* ------------------------------------------------------------------------------------ */
/* Reference GPU update, run one thread at a time (SSSPmainForUndirected.cu:42-281)        */
/* ------------------------------------------------------------------------------------ */

void orc_read_sssp_semantics(int32_t n, int64_t rows, const int32_t* node, const int32_t* par,
                             const int32_t* dist, int32_t* out_parent, int32_t* out_dist) {
    /* fresh managed memory reads as zero */
    memset(out_parent, 0, sizeof(int32_t) * (size_t)n);
    memset(out_dist, 0, sizeof(int32_t) * (size_t)n);
    int32_t prev = 0;
    for (int64_t r = 0; r < rows; r++) {
        int32_t v = node[r], p = par[r], d = dist[r];
        if (v > prev + 1)
            for (int32_t i = prev + 1; i < v && i < n; i++) { out_dist[i] = 9999999; out_parent[i] = -1; }
        if (p == -1) d = 9999999;
        if (v >= 0 && v < n) { out_parent[v] = p; out_dist[v] = d; }
        prev = v;
    }
    for (int32_t j = prev + 1; j < n; j++) { out_dist[j] = 9999999; out_parent[j] = -1; }
}

#define REF_INVALID 999999 /* gpuFunctions_undir.cuh:190 */

int orc_ref_update(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev, const int32_t* ew,
                   int64_t k, const int32_t* cu, const int32_t* cv, const int32_t* cw,
                   const int32_t* cop, const int32_t* in_parent, const int32_t* in_dist,
                   int32_t* out_dist, int32_t* out_parent, int64_t* rounds_del,
                   int64_t* rounds_relax) {
    /* adjacency: base lines, then insertions appended (all_structure_undir.cuh:106-117);
     * row order is line order (MAIN:68-72 flattens the vector-of-vectors) */
    int64_t* off = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int64_t n_ins = 0, n_del = 0;
    for (int64_t i = 0; i < m; i++) {
        if (eu[i] < 0 || eu[i] >= n || ev[i] < 0 || ev[i] >= n) { free(off); return -1; }
        off[eu[i] + 1]++; off[ev[i] + 1]++;
    }
    for (int64_t i = 0; i < k; i++) {
        if (cop[i] != 0 && cop[i] != 1) continue;
        if (cu[i] < 0 || cu[i] >= n || cv[i] < 0 || cv[i] >= n) { free(off); return -1; }
        if (cop[i] == 1) { off[cu[i] + 1]++; off[cv[i] + 1]++; n_ins++; }
        else n_del++;
    }
    for (int32_t v = 0; v < n; v++) off[v + 1] += off[v];
    int64_t nnz = off[n];
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
    int32_t* wt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    memcpy(cur, off, sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < m; i++) {
        /* read_graphEdges: row n2 gets n1 first, then row n1 gets n2 */
        int32_t a = eu[i], b = ev[i];
        col[cur[b]] = a; wt[cur[b]] = ew[i]; cur[b]++;
        col[cur[a]] = b; wt[cur[a]] = ew[i]; cur[a]++;
    }
    int64_t* ins = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_ins ? n_ins : 1));
    int64_t* del = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n_del ? n_del : 1));
    int64_t ni = 0, nd = 0;
    for (int64_t i = 0; i < k; i++) {
        if (cop[i] == 1) {
            int32_t a = cu[i], b = cv[i];
            col[cur[b]] = a; wt[cur[b]] = cw[i]; cur[b]++;
            col[cur[a]] = b; wt[cur[a]] = cw[i]; cur[a]++;
            ins[ni++] = i;
        } else if (cop[i] == 0) {
            del[nd++] = i;
        }
    }
    free(cur);

    int32_t* P = out_parent;
    int32_t* D = out_dist;
    int32_t* U = (int32_t*)calloc((size_t)(n ? n : 1), sizeof(int32_t));
    memcpy(P, in_parent, sizeof(int32_t) * (size_t)n);
    memcpy(D, in_dist, sizeof(int32_t) * (size_t)n);
    /* +1024 slack: updateNeighbors_del reads the list before its bounds check (GPU:314) */
    int32_t* list = (int32_t*)calloc((size_t)n + 1024, sizeof(int32_t));
    int64_t cnt = 0, r_del = 0, r_rel = 0;
    int rc = 0;

    /* STEP1: deleteEdge (gpuFunctions_undir.cuh:179-215), one thread per deletion */
    for (int64_t t = 0; t < nd; t++) {
        int64_t i = del[t];
        int32_t n1 = cu[i], n2 = cv[i], w = cw[i];
        if (P[n2] == n1) { D[n2] = REF_INVALID; U[n2] = 1; }
        else if (P[n1] == n2) { D[n1] = REF_INVALID; U[n1] = 1; }
        for (int64_t j = off[n2]; j < off[n2 + 1]; j++)
            if (col[j] == n1 && wt[j] == w) wt[j] = -1;
        for (int64_t j = off[n1]; j < off[n1 + 1]; j++)
            if (col[j] == n2 && wt[j] == w) wt[j] = -1;
    }
    /* insertEdge (gpuFunctions_undir.cuh:217-251), one thread per insertion */
    for (int64_t t = 0; t < ni; t++) {
        int64_t i = ins[t];
        int32_t x1 = cu[i], x2 = cv[i], w = cw[i], a, b;
        if (D[x2] > D[x1]) { a = x1; b = x2; } else { a = x2; b = x1; }
        int flag = 1;
        if (P[a] == b) flag = 0;
        if (D[b] == REF_INVALID && U[b] == 1) flag = 0;
        if (D[b] > D[a] + w && flag == 1) { P[b] = a; D[b] = D[a] + w; U[b] = 2; }
    }
    int64_t cap_rounds = 4 * (int64_t)n + 16;
    /* STEP2A: filterAffectedNodes + updateNeighbors_del (MAIN:219-239) */
    if (nd > 0) {
        cnt = 0;
        for (int32_t v = 0; v < n; v++) if (U[v] == 1) list[cnt++] = v;
        int change = 1;
        while (change > 0) {
            change = 0;
            r_del++;
            if (r_del > cap_rounds) { rc = -2; break; }
            for (int64_t t = 0; t < cnt; t++) {
                int32_t x = list[t];
                U[x] = 2;
                for (int64_t j = off[x]; j < off[x + 1]; j++) {
                    int32_t c = col[j], w = wt[j];
                    if (w < 0) continue;
                    if (P[c] == list[t] && D[c] != REF_INVALID) { D[c] = REF_INVALID; U[c] = 1; change = 1; }
                }
            }
            cnt = 0;
            for (int32_t v = 0; v < n; v++) if (U[v] == 1) list[cnt++] = v;
        }
    }
    /* STEP2B: filterAllAffected + updateNeighbors (MAIN:263-281) */
    cnt = 0;
    for (int32_t v = 0; v < n; v++) if (U[v] == 2 || U[v] == 1) list[cnt++] = v;
    int change = 1;
    while (rc == 0 && change == 1) {
        change = 0;
        r_rel++;
        if (r_rel > cap_rounds) { rc = -2; break; }
        for (int64_t t = 0; t < cnt; t++) {
            int32_t x = list[t];
            U[x] = 0;
            for (int64_t j = off[x]; j < off[x + 1]; j++) {
                int32_t c = col[j], w = wt[j];
                if (w < 0) continue;
                if (D[x] > D[c] + w) {
                    if (P[c] != x) { D[x] = D[c] + w; U[x] = 2; P[x] = c; change = 1; continue; }
                }
                if (D[c] > D[x] + w) {
                    if (P[x] != c) { D[c] = D[x] + w; U[c] = 2; P[c] = x; change = 1; }
                }
            }
        }
        cnt = 0;
        for (int32_t v = 0; v < n; v++) if (U[v] == 2 || U[v] == 1) list[cnt++] = v;
    }
    if (rounds_del) *rounds_del = r_del;
    if (rounds_relax) *rounds_relax = r_rel;
    free(list); free(U); free(ins); free(del); free(col); free(wt); free(off);
    return rc;
}
