/*
 * oracle_gen.c -- the seeded synthetic inputs, restated in C for the CPU side.
 *
 * TEST INFRASTRUCTURE ONLY (part of oracle/liboracle.so).  bench.py's CPU reference arm builds
 * its workload with these functions so that it loads no product library; tests check that
 * they give exactly what the dsssp library's generators give (Erdos-Renyi and RMAT edge lists,
 * change batches with uniform or RMAT insertions, the highest-degree vertex).
 *
 * The generators are defined by their random streams, not by an implementation: value i of
 * stream s of a seed is mix(key(seed, s) + i * golden) with SplitMix64's finaliser as mix; a
 * uniform integer in [lo, hi] is lo + ((value * (hi - lo + 1)) >> 64); a unit double is
 * (value >> 11) * 2^-53.  "Exactly m distinct pairs": draw candidates 0..D-1 (a rejected draw
 * gives ~0), sort, deduplicate, and keep the m distinct keys with the smallest (hash, key),
 * hash = stream 2 (ER) or 12 (RMAT) at the key; D starts at m + m/8 + 64 and grows by half plus
 * twice the shortfall.  Edge weights are stream 3 / 13 at the edge's rank.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

static const uint64_t kGolden = 0x9E3779B97F4A7C15ull;

static uint64_t mix64(uint64_t z) {
    z += kGolden;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t stream_key(uint64_t seed, uint64_t s) { return mix64(mix64(seed) ^ mix64(s * 0xD1B54A32D192ED03ull)); }
static uint64_t at(uint64_t key, uint64_t i) { return mix64(key + i * kGolden); }
static int64_t range(uint64_t key, uint64_t i, int64_t lo, int64_t hi) {
    unsigned __int128 p = (unsigned __int128)at(key, i) * (uint64_t)(hi - lo + 1);
    return lo + (int64_t)(uint64_t)(p >> 64);
}
static double unit(uint64_t key, uint64_t i) { return (double)(at(key, i) >> 11) * (1.0 / 9007199254740992.0); }
static uint64_t pair_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
}

/* LSD radix sort of n 64-bit keys (stable; payload moves along when pay != NULL). */
static int radix_sort(uint64_t* key, uint64_t* pay, size_t n) {
    if (n < 2) return 0;
    uint64_t* k2 = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    uint64_t* p2 = pay ? (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1)) : NULL;
    if (!k2 || (pay && !p2)) {
        free(k2);
        free(p2);
        return -1;
    }
    uint64_t* ks = key; uint64_t* kd = k2;
    uint64_t* ps = pay; uint64_t* pd = p2;
    for (int shift = 0; shift < 64; shift += 8) {
        size_t cnt[257];
        memset(cnt, 0, sizeof cnt);
        for (size_t i = 0; i < n; i++) cnt[((ks[i] >> shift) & 0xFF) + 1]++;
        if (cnt[((ks[0] >> shift) & 0xFF) + 1] == n) continue;  /* this digit is the same everywhere */
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (size_t i = 0; i < n; i++) {
            const size_t at_ = cnt[(ks[i] >> shift) & 0xFF]++;
            kd[at_] = ks[i];
            if (pay) pd[at_] = ps[i];
        }
        uint64_t* t = ks; ks = kd; kd = t;
        if (pay) { t = ps; ps = pd; pd = t; }
    }
    if (ks != key) {
        memcpy(key, ks, sizeof(uint64_t) * n);
        if (pay) memcpy(pay, ps, sizeof(uint64_t) * n);
    }
    free(k2);
    free(p2);
    return 0;
}

typedef struct {
    int kind; /* 0 = ER (uniform pairs), 1 = RMAT */
    int32_t n;
    int scale;
    double a, ab, abc;
    uint64_t ps; /* pair stream */
} drawer;

static uint64_t rmat_pair(uint64_t key, uint64_t i, int scale, double a, double ab, double abc) {
    uint32_t x = 0, y = 0;
    for (int l = 0; l < scale; l++) {
        const double r = unit(key, i * (uint64_t)scale + (uint64_t)l);
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

static uint64_t draw(const drawer* d, uint64_t i) {
    uint32_t a, b;
    if (d->kind == 0) {
        a = (uint32_t)range(d->ps, 2 * i, 0, d->n - 1);
        b = (uint32_t)range(d->ps, 2 * i + 1, 0, d->n - 1);
    } else {
        const uint64_t p = rmat_pair(d->ps, i, d->scale, d->a, d->ab, d->abc);
        a = (uint32_t)(p >> 32);
        b = (uint32_t)p;
    }
    return a == b ? ~0ull : pair_key(a, b);
}

/* The m distinct keys with the smallest (hash, key), in that order; 0 or -1. */
static int distinct_keys(int64_t m, uint64_t hs, const drawer* d, uint64_t* out) {
    int64_t D = m + m / 8 + 64;
    for (int attempt = 0; attempt < 40; attempt++) {
        uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)D);
        if (!keys) return -1;
        for (int64_t i = 0; i < D; i++) keys[i] = draw(d, (uint64_t)i);
        if (radix_sort(keys, NULL, (size_t)D)) {
            free(keys);
            return -1;
        }
        int64_t u = 0;
        for (int64_t i = 0; i < D; i++) {
            if (keys[i] == ~0ull) break;
            if (u == 0 || keys[u - 1] != keys[i]) keys[u++] = keys[i];
        }
        if (u >= m) {
            /* stable sort of the key-sorted distinct keys by hash: order (hash, key) */
            uint64_t* h = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(u ? u : 1));
            if (!h) {
                free(keys);
                return -1;
            }
            for (int64_t i = 0; i < u; i++) h[i] = at(hs, keys[i]);
            const int rc = radix_sort(h, keys, (size_t)u);
            if (!rc) memcpy(out, keys, sizeof(uint64_t) * (size_t)m);
            free(h);
            free(keys);
            return rc;
        }
        free(keys);
        D = D + D / 2 + (m - u) * 2;
        if (D > 64 * m + (1 << 20)) break;
    }
    return -1;
}

static int emit(const uint64_t* keys, int64_t m, uint64_t ws, int32_t wlo, int32_t whi, int32_t* u, int32_t* v,
                int32_t* w) {
    for (int64_t i = 0; i < m; i++) {
        u[i] = (int32_t)(keys[i] >> 32);
        v[i] = (int32_t)(keys[i] & 0xFFFFFFFFu);
        w[i] = (int32_t)range(ws, (uint64_t)i, wlo, whi);
    }
    return 0;
}

int orc_gen_er(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed, int32_t* u, int32_t* v, int32_t* w) {
    if (n < 2 || m < 0 || (double)m > (double)n * (n - 1) / 2.0) return -1;
    drawer d = {0, n, 0, 0, 0, 0, stream_key(seed, 1)};
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(m ? m : 1));
    if (!keys) return -1;
    int rc = distinct_keys(m, stream_key(seed, 2), &d, keys);
    if (!rc) rc = emit(keys, m, stream_key(seed, 3), wlo, whi, u, v, w);
    free(keys);
    return rc;
}

int orc_gen_rmat(int32_t scale, int64_t m, double a, double b, double c, int32_t wlo, int32_t whi, uint64_t seed,
                 int32_t* u, int32_t* v, int32_t* w) {
    if (scale < 1 || scale > 30 || m < 0) return -1;
    drawer d = {1, 1 << scale, scale, a, a + b, a + b + c, stream_key(seed, 11)};
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(m ? m : 1));
    if (!keys) return -1;
    int rc = distinct_keys(m, stream_key(seed, 12), &d, keys);
    if (!rc) rc = emit(keys, m, stream_key(seed, 13), wlo, whi, u, v, w);
    free(keys);
    return rc;
}

int32_t orc_max_degree_vertex(int32_t n, int64_t m, const int32_t* u, const int32_t* v) {
    if (n <= 0) return -1;
    int64_t* deg = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    if (!deg) return -1;
    for (int64_t i = 0; i < m; i++) {
        if (u[i] >= 0 && u[i] < n) deg[u[i]]++;
        if (v[i] >= 0 && v[i] < n) deg[v[i]]++;
    }
    int32_t best = 0;
    for (int32_t x = 1; x < n; x++)
        if (deg[x] > deg[best]) best = x;
    free(deg);
    return best;
}

/* open-addressing set of 64-bit keys (~0 never inserted) */
typedef struct {
    uint64_t* slot;
    uint64_t mask;
} kset;

static int kset_init(kset* s, int64_t n) {
    uint64_t cap = 64;
    while (cap < (uint64_t)(2 * n + 16)) cap <<= 1;
    s->slot = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    if (!s->slot) return -1;
    memset(s->slot, 0xFF, sizeof(uint64_t) * cap);
    s->mask = cap - 1;
    return 0;
}

/* 1 if newly inserted, 0 if present */
static int kset_insert(kset* s, uint64_t k) {
    uint64_t h = mix64(k) & s->mask;
    while (s->slot[h] != ~0ull) {
        if (s->slot[h] == k) return 0;
        h = (h + 1) & s->mask;
    }
    s->slot[h] = k;
    return 1;
}

static int kset_has(const kset* s, uint64_t k) {
    uint64_t h = mix64(k) & s->mask;
    while (s->slot[h] != ~0ull) {
        if (s->slot[h] == k) return 1;
        h = (h + 1) & s->mask;
    }
    return 0;
}

static int has_sorted(const uint64_t* a, int64_t n, uint64_t k) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && a[lo] == k;
}

int orc_gen_changes(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev, const int32_t* ew, int64_t n_ins,
                    int64_t n_del, int32_t ins_kind, int32_t scale, double p0, double p1, double p2, int32_t wlo,
                    int32_t whi, uint64_t seed, int32_t* cu, int32_t* cv, int32_t* cw, int32_t* cop) {
    if (n < 2 || m < 0 || n_ins < 0 || n_del < 0 || n_del > m || (ins_kind != 0 && ins_kind != 1)) return -1;
    if (ins_kind == 1 && (scale < 1 || (1ll << scale) > n)) return -1;
    const uint64_t is = stream_key(seed, 31), ws = stream_key(seed, 32), dsel = stream_key(seed, 33),
                   sh = stream_key(seed, 34);
    uint64_t* existing = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(m ? m : 1));
    if (!existing) return -1;
    for (int64_t i = 0; i < m; i++) existing[i] = pair_key((uint32_t)eu[i], (uint32_t)ev[i]);
    if (radix_sort(existing, NULL, (size_t)m)) {
        free(existing);
        return -1;
    }
    const int64_t k = n_ins + n_del;
    int64_t at_ = 0;
    kset seen;
    if (kset_init(&seen, n_ins)) {
        free(existing);
        return -1;
    }
    const double ab = p0 + p1, abc = p0 + p1 + p2;
    const uint64_t cap = (uint64_t)(n_ins + 16) * 1000;
    int64_t got = 0;
    for (uint64_t i = 0; got < n_ins; i++) {
        if (i > cap) {
            free(existing);
            free(seen.slot);
            return -1;
        }
        uint32_t a, b;
        if (ins_kind == 1) {
            const uint64_t p = rmat_pair(is, i, scale, p0, ab, abc);
            a = (uint32_t)(p >> 32);
            b = (uint32_t)p;
        } else {
            a = (uint32_t)range(is, 2 * i, 0, n - 1);
            b = (uint32_t)range(is, 2 * i + 1, 0, n - 1);
        }
        if (a == b) continue;
        const uint64_t key = pair_key(a, b);
        if (has_sorted(existing, m, key)) continue;
        if (!kset_insert(&seen, key)) continue;
        cu[at_] = (int32_t)a;
        cv[at_] = (int32_t)b;
        cw[at_] = (int32_t)range(ws, i, wlo, whi);
        cop[at_] = 1;
        at_++;
        got++;
    }
    free(seen.slot);
    free(existing);
    /* deletions: Floyd's sampling of n_del distinct line indices */
    kset pick;
    if (kset_init(&pick, n_del)) return -1;
    for (int64_t j = m - n_del; j < m; j++) {
        const int64_t t = range(dsel, (uint64_t)j, 0, j);
        const int64_t chosen = kset_has(&pick, (uint64_t)t) ? j : t;
        kset_insert(&pick, (uint64_t)chosen);
        cu[at_] = eu[chosen];
        cv[at_] = ev[chosen];
        cw[at_] = ew[chosen];
        cop[at_] = 0;
        at_++;
    }
    free(pick.slot);
    /* shuffle (Fisher-Yates) */
    for (int64_t j = k - 1; j > 0; j--) {
        const int64_t t = range(sh, (uint64_t)j, 0, j);
        int32_t x;
        x = cu[j]; cu[j] = cu[t]; cu[t] = x;
        x = cv[j]; cv[j] = cv[t]; cv[t] = x;
        x = cw[j]; cw[j] = cw[t]; cw[t] = x;
        x = cop[j]; cop[j] = cop[t]; cop[t] = x;
    }
    return 0;
}
