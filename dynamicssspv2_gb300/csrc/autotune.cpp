// autotune.cpp -- the autotuner of the update's launch and frontier-switch settings, as host
// C++ over the engine's C ABI.
//
// For a graph and a representative change batch it times a list of candidate settings --
// edges per thread item and the CTA-chunk thresholds (the degree buckets), the subtree-walk
// depth before pointer jumping, CTA size and residency, the width of solo steps on one CTA,
// and near-far bucket widths scaled by the batch's mean weight -- each on the same batch from
// the same starting state (device snapshot and restore), in rounds that time every candidate
// once (so drift of the device's speed touches all alike), compares their median times, keeps
// the first setting (the graph's own) unless another is at least 3 % faster, sets the winner
// on the graph and caches it per size class (log2 vertices, log2 adjacency entries, log2 batch size)
// in a text file, so that later graphs of the same class (the command line's --autotune, the
// server's tune_cache, the Python binding) take it without timing.  The reference has no
// tunables: its block size is a compile-time macro (SSSPmainForUndirected.cu:11).
//
// Cache file: one line per size class, "<key> <ms> <field>=<value> ...", written whole to a
// temporary file and renamed over the old one.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/dsssp.h"
#include "host_common.h"

using namespace dsssp;

namespace {

// The settings the tuner varies, by name (the cache stores these fields).
struct Field {
    const char* name;
    int32_t dsssp_opts::*i32;
};
const Field kFields[] = {
    {"small_deg", &dsssp_opts::small_deg},   {"large_deg", &dsssp_opts::large_deg},
    {"chunk", &dsssp_opts::chunk},           {"bfs_levels", &dsssp_opts::bfs_levels},
    {"block", &dsssp_opts::block},           {"ctas_per_sm", &dsssp_opts::ctas_per_sm},
    {"delta", &dsssp_opts::delta},           {"solo_waves", &dsssp_opts::solo_waves},
    {"group_ctas", &dsssp_opts::group_ctas}, {"group_waves", &dsssp_opts::group_waves},
    {"warp_agg", &dsssp_opts::warp_agg},     {"auto_rounds", &dsssp_opts::auto_rounds},
};

struct Override {
    const char* name;
    int32_t value;
};

// Candidate i: the base options with a few fields changed.
const std::vector<std::vector<Override>> kCandidates = {
    {},
    {{"small_deg", 8}},
    {{"small_deg", 4}, {"large_deg", 1024}, {"chunk", 1024}},
    {{"small_deg", 4}, {"large_deg", 4096}, {"chunk", 2048}},
    {{"bfs_levels", 0}},
    {{"bfs_levels", 8}},
    {{"block", 128}},
    {{"ctas_per_sm", 2}},
    {{"solo_waves", 0}},
    {{"solo_waves", 4}},
};

bool set_field(dsssp_opts& o, const char* name, int32_t v) {
    for (const Field& f : kFields)
        if (!strcmp(f.name, name)) {
            o.*(f.i32) = v;
            return true;
        }
    return false;
}

int lg(long long x) { return (int)std::lround(std::log2((double)(x > 1 ? x : 1))); }

struct Entry {
    double ms = 0;
    std::vector<std::pair<std::string, int32_t>> fields;
};

// Parses a cache file (missing or unreadable: empty).
std::map<std::string, Entry> read_cache(const char* path) {
    std::map<std::string, Entry> out;
    FILE* f = path ? fopen(path, "r") : nullptr;
    if (!f) return out;
    char line[1024];
    while (fgets(line, sizeof line, f)) {
        char* save = nullptr;
        char* tok = strtok_r(line, " \t\r\n", &save);
        if (!tok || tok[0] == '#') continue;
        std::string key = tok;
        tok = strtok_r(nullptr, " \t\r\n", &save);
        if (!tok) continue;
        Entry e;
        e.ms = atof(tok);
        while ((tok = strtok_r(nullptr, " \t\r\n", &save))) {
            char* eq = strchr(tok, '=');
            if (!eq) continue;
            *eq = 0;
            char* end = nullptr;
            const long v = strtol(eq + 1, &end, 10);
            if (end == eq + 1 || *end) continue;
            e.fields.emplace_back(tok, (int32_t)v);
        }
        out[key] = e;
    }
    fclose(f);
    return out;
}

int write_cache(const char* path, const std::map<std::string, Entry>& c) {
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) return fail(DSSSP_E_IO, "autotune: cannot write %s", tmp.c_str());
    fprintf(f, "# dsssp autotune cache: <size class> <ms> <option>=<value> ...\n");
    for (const auto& kv : c) {
        fprintf(f, "%s %.6f", kv.first.c_str(), kv.second.ms);
        for (const auto& fv : kv.second.fields) fprintf(f, " %s=%d", fv.first.c_str(), fv.second);
        fprintf(f, "\n");
    }
    const bool ok = fclose(f) == 0;
    if (!ok || rename(tmp.c_str(), path) != 0) return fail(DSSSP_E_IO, "autotune: cannot replace %s", path);
    return DSSSP_OK;
}

std::mutex g_cache_mu;  // tuners of one process share a cache file

void fill(dsssp_tune_result* out, const std::string& key, const dsssp_opts& o, double ms, int trials, int cached) {
    if (!out) return;
    memset(out, 0, sizeof(*out));
    snprintf(out->key, sizeof out->key, "%s", key.c_str());
    out->opts = o;
    out->ms = ms;
    out->trials = trials;
    out->cached = cached;
}

}  // namespace

extern "C" {

int dsssp_tune_size_class(int64_t n, int64_t entries, int64_t k, char* key, size_t cap) {
    if (!key || cap < 8 || n < 0 || entries < 0 || k < 0) return fail(DSSSP_E_INVAL, "tune_size_class: bad arguments");
    snprintf(key, cap, "v%d_e%d_b%d", lg(n), lg(entries), lg(k));
    return DSSSP_OK;
}

int dsssp_tune_candidates(const dsssp_opts* base, const dsssp_change* changes, int64_t k, dsssp_opts* out, int32_t cap,
                          int32_t* count) {
    if (!base || (k > 0 && !changes) || k < 0 || cap < 0 || (cap > 0 && !out) || !count)
        return fail(DSSSP_E_INVAL, "tune_candidates: bad arguments");
    std::vector<dsssp_opts> c;
    for (const auto& ov : kCandidates) {
        dsssp_opts o = *base;
        for (const Override& x : ov) set_field(o, x.name, x.value);
        c.push_back(o);
    }
    // near-far bucket widths scaled by the batch's mean weight: a multiple of the typical edge
    // keeps a few hops per bucket (narrow: fewer relaxations; wide: fewer rounds)
    double sw = 0;
    long long live = 0;
    for (int64_t i = 0; i < k; i++)
        if (changes[i].op == 0 || changes[i].op == 1) {
            sw += changes[i].w;
            live++;
        }
    const double wbar = live ? sw / (double)live : 0.0;
    if (wbar > 0)
        for (double f : {8.0, 96.0}) {
            dsssp_opts o = *base;
            const double d = std::floor(f * wbar + 0.5);
            o.delta = d < 1 ? 1 : (d > 2147483647.0 ? 2147483647 : (int32_t)d);
            c.push_back(o);
        }
    *count = (int32_t)c.size();
    for (int32_t i = 0; i < cap && i < (int32_t)c.size(); i++) out[i] = c[(size_t)i];
    return DSSSP_OK;
}

int dsssp_autotune_lookup(dsssp_graph* g, int64_t k, const char* cache_path, dsssp_tune_result* out) {
    if (!g || k < 0 || !cache_path) return fail(DSSSP_E_INVAL, "autotune_lookup: bad arguments");
    int64_t n = 0, entries = 0;
    int rc = dsssp_graph_info(g, &n, &entries, nullptr, nullptr, nullptr);
    if (rc) return rc;
    char key[32];
    dsssp_tune_size_class(n, entries, k, key, sizeof key);
    std::map<std::string, Entry> cache;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        cache = read_cache(cache_path);
    }
    auto it = cache.find(key);
    if (it == cache.end()) return fail(DSSSP_E_INVAL, "autotune_lookup: no entry for size class %s in %s", key, cache_path);
    dsssp_opts o;
    rc = dsssp_graph_get_opts(g, &o);
    if (rc) return rc;
    for (const auto& fv : it->second.fields) set_field(o, fv.first.c_str(), fv.second);
    rc = dsssp_graph_set_opts(g, &o);
    if (rc) return rc;
    fill(out, key, o, it->second.ms, 0, 1);
    return DSSSP_OK;
}

int dsssp_autotune(dsssp_graph* g, const dsssp_change* changes, int64_t k, const char* cache_path, int32_t reps,
                   int32_t force, dsssp_tune_result* out) {
    if (!g || k < 1 || !changes || reps < 0) return fail(DSSSP_E_INVAL, "autotune: bad arguments");
    if (cache_path && !force && dsssp_autotune_lookup(g, k, cache_path, out) == DSSSP_OK) return DSSSP_OK;
    int64_t n = 0, entries = 0;
    int rc = dsssp_graph_info(g, &n, &entries, nullptr, nullptr, nullptr);
    if (rc) return rc;
    char key[32];
    dsssp_tune_size_class(n, entries, k, key, sizeof key);
    dsssp_opts base;
    rc = dsssp_graph_get_opts(g, &base);
    if (rc) return rc;
    std::vector<dsssp_opts> cands(32);
    int32_t nc = 0;
    rc = dsssp_tune_candidates(&base, changes, k, cands.data(), (int32_t)cands.size(), &nc);
    if (rc) return rc;
    cands.resize((size_t)(nc < 32 ? nc : 32));
    rc = dsssp_graph_snapshot(g);  // every candidate starts from this state
    if (rc) return rc;
    const int r = reps > 0 ? reps : 3;
    std::vector<std::vector<double>> times(cands.size());
    std::vector<bool> ok(cands.size(), true);
    for (int round = 0; round < r; round++)
        for (size_t c = 0; c < cands.size(); c++) {
            if (!ok[c]) continue;
            dsssp_stats st;
            // a setting the device cannot run, or a batch that failed or was recovered: not a candidate
            if (dsssp_graph_set_opts(g, &cands[c]) != DSSSP_OK || dsssp_graph_restore(g, nullptr) != DSSSP_OK ||
                dsssp_apply_batch(g, changes, k, nullptr, &st) != DSSSP_OK) {
                ok[c] = false;
                continue;
            }
            times[c].push_back(st.t_total_ms);
        }
    double best_ms = -1;
    dsssp_opts best = base;
    int trials = 0;
    for (size_t c = 0; c < cands.size(); c++) {
        if (!ok[c] || times[c].empty()) continue;
        std::vector<double> t = times[c];
        std::sort(t.begin(), t.end());
        const double med = t[t.size() / 2];
        trials++;
        // the first candidate is the graph's own setting: another must beat it by 3 %
        if (best_ms < 0 || med < best_ms * (c == 0 || trials == 1 ? 1.0 : 0.97)) {
            best_ms = med;
            best = cands[c];
        }
    }
    rc = dsssp_graph_restore(g, nullptr);
    if (!rc) rc = dsssp_graph_set_opts(g, &best);
    if (rc) return rc;
    if (trials == 0) return fail(DSSSP_E_CUDA, "autotune: no candidate could be timed");
    if (cache_path) {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        std::map<std::string, Entry> cache = read_cache(cache_path);
        Entry e;
        e.ms = best_ms;
        for (const Field& f : kFields) e.fields.emplace_back(f.name, best.*(f.i32));
        cache[key] = e;
        rc = write_cache(cache_path, cache);
        if (rc) return rc;
    }
    fill(out, key, best, best_ms, trials, 0);
    return DSSSP_OK;
}

}  // extern "C"
