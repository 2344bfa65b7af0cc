// serve.cpp -- the batching and serving layers: a pooled graph store of many graphs and a
// request loop with continuous batching, as C++ host code over the engine's C ABI.
//
// Pool: the graphs lie side by side in one vertex id space (graph i owns ids [first[i],
// first[i] + n_i)), so one engine graph holds their disjoint union and every graph is a
// separate part with its own root.  A set of change batches -- at most one per graph --
// becomes one change batch of the union (ids shifted), applied by one launch sequence; the
// update of one graph never reads another graph's data, so each graph's result equals
// applying its batch alone (distances bit-exact, parents a valid tree).  A pool may hold
// spare vertex ids (a reserve): a graph added later takes a free id range, gets its source
// as a new root and its edges as one insertion batch (whose relaxation builds its tree); a
// removed graph's edges become tombstones (reclaimed by compaction) and its ids a free range.
//
// Server: tenants are admitted in order while their estimated device footprint fits the
// memory budget and live in one pool; the others wait and are admitted when a removal frees
// memory and ids (tenants can also be added and removed while serving).  dsssp_submit
// validates a request, queues a copy of its batch and returns at once; a worker thread serves
// epochs back to back: every admitted tenant with a waiting request contributes its oldest
// one, the epoch's records are copied once into a pinned staging buffer with ids shifted into
// the pool's id space, and the epoch runs as one union batch; its requests complete together.
// A tenant never has two requests in one epoch, so its batches apply in arrival order and each
// result equals applying that batch alone.  Requests for tenants that are waiting or removed
// are refused and malformed ones fail at submission, without touching any epoch.  While no
// request waits, the worker compacts the store when its tombstones or its spare-region use pass
// the configured fractions.
//
// No counterpart in the reference, which applies one batch per process run.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/dsssp.h"
#include "host_common.h"

using namespace dsssp;

struct dsssp_pool {
    dsssp_graph* g = nullptr;
    std::vector<int64_t> first;  // per graph: its first id in the store
    std::vector<int32_t> nv;     // per graph: its vertex count (0 once removed)
    int64_t capacity = 0;        // vertex ids of the store
    std::map<int64_t, int64_t> free_ids;  // unused id ranges: first -> count
    dsssp_change* stage = nullptr;  // pinned staging buffer of union batches
    int64_t stage_cap = 0;

    int32_t count() const { return (int32_t)first.size(); }
    int32_t size(int32_t i) const { return nv[(size_t)i]; }
    ~dsssp_pool() {
        if (stage) dsssp_host_free(stage);
        if (g) dsssp_graph_destroy(g);
    }
    int ensure_stage(int64_t k) {
        if (k <= stage_cap) return DSSSP_OK;
        if (stage) dsssp_host_free(stage);
        stage_cap = 0;
        const int64_t cap = k + k / 2 + 1024;
        stage = (dsssp_change*)dsssp_host_alloc(sizeof(dsssp_change) * (size_t)cap);
        if (!stage) return fail(DSSSP_E_OOM, "pool: pinned staging buffer of %lld records", (long long)cap);
        stage_cap = cap;
        return DSSSP_OK;
    }
    // first fit: the lowest free range of at least n ids, -1 if none
    int64_t find_ids(int64_t n) const {
        for (const auto& r : free_ids)
            if (r.second >= n) return r.first;
        return -1;
    }
    void take_ids(int64_t at, int64_t n) {
        auto it = free_ids.find(at);
        const int64_t len = it->second;
        free_ids.erase(it);
        if (len > n) free_ids[at + n] = len - n;
    }
    void give_ids(int64_t at, int64_t n) {
        auto it = free_ids.emplace(at, n).first;
        auto next = std::next(it);
        if (next != free_ids.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_ids.erase(next);
        }
        if (it != free_ids.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_ids.erase(it);
            }
        }
    }
};

namespace {

// Why a batch cannot be applied to a graph of n vertices, or empty.
std::string check_batch(const dsssp_change* ch, int64_t k, int32_t n) {
    for (int64_t i = 0; i < k; i++) {
        const dsssp_change& c = ch[i];
        if (c.op != 0 && c.op != 1) continue;  // ignored records, as in the engine
        if (c.u < 0 || c.u >= n || c.v < 0 || c.v >= n) {
            char buf[96];
            snprintf(buf, sizeof buf, "change %lld names a vertex outside 0..%d", (long long)i, n - 1);
            return buf;
        }
        if (c.op == 1 && c.w < 0) {
            char buf[96];
            snprintf(buf, sizeof buf, "insertion %lld has a negative weight", (long long)i);
            return buf;
        }
    }
    return std::string();
}

// Copies batch records into out with ids shifted by `shift` (one pass).
void copy_shifted(const dsssp_change* src, int64_t k, int32_t shift, dsssp_change* out) {
    for (int64_t i = 0; i < k; i++) {
        dsssp_change c = src[i];
        c.u += shift;
        c.v += shift;
        out[i] = c;
    }
}

int union_batch(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                const int64_t* sizes, dsssp_change* out, int64_t cap, int64_t* k) {
    std::vector<char> seen((size_t)p->count(), 0);
    int64_t total = 0;
    for (int32_t b = 0; b < nb; b++) {
        const int32_t gi = graphs[b];
        if (gi < 0 || gi >= p->count()) return fail(DSSSP_E_INVAL, "pool: no graph %d", gi);
        if (p->size(gi) == 0) return fail(DSSSP_E_INVAL, "pool: graph %d was removed", gi);
        if (seen[(size_t)gi]) return fail(DSSSP_E_INVAL, "pool: graph %d has two batches in one union", gi);
        seen[(size_t)gi] = 1;
        if (sizes[b] < 0 || (sizes[b] > 0 && !batches[b])) return fail(DSSSP_E_INVAL, "pool: bad batch for graph %d", gi);
        if (!out) {
            const std::string why = check_batch(batches[b], sizes[b], p->size(gi));
            if (!why.empty())
                return fail(why.find("weight") != std::string::npos ? DSSSP_E_BAD_WEIGHT : DSSSP_E_BAD_VERTEX,
                            "pool graph %d: %s", gi, why.c_str());
        }
        total += sizes[b];
    }
    *k = total;
    if (!out) return DSSSP_OK;
    if (total > cap) return fail(DSSSP_E_INVAL, "pool: union batch of %lld records exceeds %lld", (long long)total, (long long)cap);
    int64_t at = 0;
    for (int32_t b = 0; b < nb; b++) {
        copy_shifted(batches[b], sizes[b], (int32_t)p->first[(size_t)graphs[b]], out + at);
        at += sizes[b];
    }
    return DSSSP_OK;
}

int check_edges(int32_t n, int64_t m, const int32_t* u, const int32_t* v, const int32_t* w, const char* what) {
    for (int64_t j = 0; j < m; j++) {
        if (u[j] < 0 || u[j] >= n || v[j] < 0 || v[j] >= n)
            return fail(DSSSP_E_BAD_VERTEX, "%s: edge %lld names a vertex outside 0..%d", what, (long long)j, n - 1);
        if (w[j] < 0) return fail(DSSSP_E_BAD_WEIGHT, "%s: edge %lld has a negative weight", what, (long long)j);
    }
    return DSSSP_OK;
}

int pool_create_impl(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                     const int32_t* const* v, const int32_t* const* w, int64_t reserve, const dsssp_opts* o,
                     dsssp_pool** out) {
    if (count < 0 || (count > 0 && (!n || !m || !u || !v || !w)) || !out || reserve < 0 || (count == 0 && reserve == 0))
        return fail(DSSSP_E_INVAL, "pool_create: bad arguments");
    dsssp_pool* p = new dsssp_pool();
    int64_t edges = 0, at = 0;
    for (int32_t i = 0; i < count; i++) {
        if (n[i] <= 0 || m[i] < 0 || (m[i] > 0 && (!u[i] || !v[i] || !w[i]))) {
            delete p;
            return fail(DSSSP_E_INVAL, "pool_create: graph %d needs at least one vertex and its edge arrays", i);
        }
        p->first.push_back(at);
        p->nv.push_back(n[i]);
        at += n[i];
        edges += m[i];
    }
    p->capacity = at + reserve;
    if (p->capacity >= (1ll << 31) - 16) {
        delete p;
        return fail(DSSSP_E_INVAL, "pool_create: the pool's vertex count must stay below 2^31");
    }
    if (reserve > 0) p->free_ids[at] = reserve;
    std::vector<int32_t> U((size_t)edges), V((size_t)edges), W((size_t)edges);
    int64_t e = 0;
    for (int32_t i = 0; i < count; i++) {
        const int32_t shift = (int32_t)p->first[(size_t)i];
        for (int64_t j = 0; j < m[i]; j++, e++) {
            if (u[i][j] < 0 || u[i][j] >= n[i] || v[i][j] < 0 || v[i][j] >= n[i]) {
                delete p;
                return fail(DSSSP_E_BAD_VERTEX, "pool_create: graph %d edge %lld names a vertex outside 0..%d", i,
                            (long long)j, n[i] - 1);
            }
            U[(size_t)e] = u[i][j] + shift;
            V[(size_t)e] = v[i][j] + shift;
            W[(size_t)e] = w[i][j];
        }
    }
    const int rc = dsssp_graph_create((int32_t)p->capacity, edges, U.data(), V.data(), W.data(), o, &p->g);
    if (rc) {
        delete p;
        return rc;
    }
    *out = p;
    return DSSSP_OK;
}

}  // namespace

extern "C" {

int64_t dsssp_estimate_footprint(int32_t n, int64_t m, int32_t slack_pct, int32_t slack_min) {
    // per vertex: state 8, row descriptor 16, sorted-prefix length 4, four tags 16, cut-off
    // root list 4, three thread-item lists 48; per slot: entry 8, twin 4, three thread-item
    // lists (16 bytes per small_deg slots); plus a margin for the batch buffers
    const double slots = 2.0 * (double)m * (1.0 + slack_pct / 100.0) + (double)n * slack_min;
    return (int64_t)((double)n * (8 + 16 + 4 + 16 + 4 + 48) + slots * (8 + 4 + 3 * 16 / 4.0) + (1 << 20));
}

int dsssp_pool_create(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                      const int32_t* const* v, const int32_t* const* w, const dsssp_opts* o, dsssp_pool** out) {
    if (count < 1) return fail(DSSSP_E_INVAL, "pool_create: no graph");
    return pool_create_impl(count, n, m, u, v, w, 0, o, out);
}

int dsssp_pool_create_reserved(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                               const int32_t* const* v, const int32_t* const* w, int64_t reserve_vertices,
                               const dsssp_opts* o, dsssp_pool** out) {
    return pool_create_impl(count, n, m, u, v, w, reserve_vertices, o, out);
}

void dsssp_pool_destroy(dsssp_pool* p) { delete p; }

dsssp_graph* dsssp_pool_graph(dsssp_pool* p) { return p ? p->g : nullptr; }

int dsssp_pool_offsets(const dsssp_pool* p, int64_t* offsets) {
    if (!p || !offsets) return fail(DSSSP_E_INVAL, "pool_offsets: bad arguments");
    for (int32_t i = 0; i < p->count(); i++) offsets[i] = p->first[(size_t)i];
    offsets[p->count()] = p->count() ? p->first.back() + p->nv.back() : 0;
    return DSSSP_OK;
}

int dsssp_pool_graph_range(const dsssp_pool* p, int32_t graph, int64_t* first, int32_t* n) {
    if (!p || graph < 0 || graph >= p->count() || !first || !n) return fail(DSSSP_E_INVAL, "pool_graph_range: bad arguments");
    *first = p->first[(size_t)graph];
    *n = p->nv[(size_t)graph];
    return DSSSP_OK;
}

int dsssp_pool_capacity(const dsssp_pool* p, int64_t* vertices, int64_t* free_vertices, int64_t* largest_free) {
    if (!p) return fail(DSSSP_E_INVAL, "pool_capacity: NULL pool");
    int64_t fr = 0, big = 0;
    for (const auto& r : p->free_ids) {
        fr += r.second;
        big = std::max(big, r.second);
    }
    if (vertices) *vertices = p->capacity;
    if (free_vertices) *free_vertices = fr;
    if (largest_free) *largest_free = big;
    return DSSSP_OK;
}

int dsssp_pool_tree_compute(dsssp_pool* p, const int32_t* sources, dsssp_stats* st) {
    if (!p || !sources) return fail(DSSSP_E_INVAL, "pool_tree_compute: bad arguments");
    std::vector<int32_t> s;
    for (int32_t i = 0; i < p->count(); i++) {
        if (p->size(i) == 0) continue;  // removed
        if (sources[i] < 0 || sources[i] >= p->size(i))
            return fail(DSSSP_E_BAD_VERTEX, "pool_tree_compute: source %d of graph %d out of range", sources[i], i);
        s.push_back(sources[i] + (int32_t)p->first[(size_t)i]);
    }
    if (s.empty()) return fail(DSSSP_E_INVAL, "pool_tree_compute: the pool holds no graph");
    return dsssp_tree_compute_multi(p->g, s.data(), (int32_t)s.size(), st);
}

int dsssp_pool_forest_load(dsssp_pool* p, const int32_t* const* parent, const int64_t* const* dist) {
    if (!p || !parent || !dist) return fail(DSSSP_E_INVAL, "pool_forest_load: bad arguments");
    const size_t N = (size_t)p->capacity;
    std::vector<int32_t> par(N, -1);
    std::vector<int64_t> d(N, DSSSP_UNREACHABLE);
    for (int32_t i = 0; i < p->count(); i++) {
        if (p->size(i) == 0) continue;
        if (!parent[i] || !dist[i]) return fail(DSSSP_E_INVAL, "pool_forest_load: no tree for graph %d", i);
        const int64_t a = p->first[(size_t)i];
        for (int32_t x = 0; x < p->size(i); x++) {
            const int32_t q = parent[i][x];
            par[(size_t)(a + x)] = q < 0 ? -1 : q + (int32_t)a;
            d[(size_t)(a + x)] = dist[i][x];
        }
    }
    return dsssp_forest_load(p->g, par.data(), d.data());
}

int dsssp_pool_union(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                     const int64_t* sizes, dsssp_change* out, int64_t cap, int64_t* k) {
    if (!p || nb < 0 || (nb > 0 && (!graphs || !batches || !sizes)) || !k)
        return fail(DSSSP_E_INVAL, "pool_union: bad arguments");
    int rc = union_batch(p, nb, graphs, batches, sizes, nullptr, 0, k);  // validates
    if (rc || !out) return rc;
    return union_batch(p, nb, graphs, batches, sizes, out, cap, k);
}

int dsssp_pool_apply(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                     const int64_t* sizes, dsssp_stats* st) {
    if (!p || nb < 0 || (nb > 0 && (!graphs || !batches || !sizes)))
        return fail(DSSSP_E_INVAL, "pool_apply: bad arguments");
    int64_t total = 0;
    int rc = union_batch(p, nb, graphs, batches, sizes, nullptr, 0, &total);  // validates
    if (rc) return rc;
    rc = p->ensure_stage(total);
    if (rc) return rc;
    rc = union_batch(p, nb, graphs, batches, sizes, p->stage, p->stage_cap, &total);
    if (rc) return rc;
    return dsssp_apply_batch(p->g, p->stage, total, nullptr, st);
}

int dsssp_pool_tree_read(dsssp_pool* p, int32_t graph, int32_t* parent, int64_t* dist) {
    if (!p || graph < 0 || graph >= p->count() || !parent || !dist) return fail(DSSSP_E_INVAL, "pool_tree_read: bad arguments");
    if (p->size(graph) == 0) return fail(DSSSP_E_INVAL, "pool_tree_read: graph %d was removed", graph);
    const int32_t a = (int32_t)p->first[(size_t)graph], nn = p->size(graph);
    const int rc = dsssp_tree_read_range(p->g, a, nn, parent, dist);
    if (rc) return rc;
    for (int32_t x = 0; x < nn; x++)
        if (parent[x] >= 0) parent[x] -= a;
    return DSSSP_OK;
}

int dsssp_pool_add_graph(dsssp_pool* p, int32_t n, int64_t m, const int32_t* u, const int32_t* v, const int32_t* w,
                         int32_t src, int32_t* graph) {
    if (!p || n < 1 || m < 0 || (m > 0 && (!u || !v || !w)) || !graph) return fail(DSSSP_E_INVAL, "pool_add_graph: bad arguments");
    if (src < 0 || src >= n) return fail(DSSSP_E_BAD_VERTEX, "pool_add_graph: source %d outside 0..%d", src, n - 1);
    int rc = check_edges(n, m, u, v, w, "pool_add_graph");
    if (rc) return rc;
    const int64_t at = p->find_ids(n);
    if (at < 0) return fail(DSSSP_E_OOM, "pool_add_graph: no free range of %d vertex ids in the pool", n);
    // the source becomes a root of its own (isolated) part first; the insertion batch then
    // relaxes outward from it, which builds the graph's tree
    const int32_t root = (int32_t)at + src;
    rc = dsssp_tree_add_sources(p->g, &root, 1, nullptr);
    if (rc < 0) {
        dsssp_graph_clear_range(p->g, (int32_t)at, n);
        return rc;
    }
    if (m > 0) {
        rc = p->ensure_stage(m);
        if (!rc) {
            for (int64_t j = 0; j < m; j++) p->stage[j] = dsssp_change{u[j] + (int32_t)at, v[j] + (int32_t)at, w[j], 1};
            rc = dsssp_apply_batch(p->g, p->stage, m, nullptr, nullptr);
        }
        if (rc < 0) {
            char why[200];
            snprintf(why, sizeof why, "%s", dsssp_last_error());
            dsssp_graph_clear_range(p->g, (int32_t)at, n);
            return fail(rc, "pool_add_graph: %s", why);
        }
    }
    p->take_ids(at, n);
    p->first.push_back(at);
    p->nv.push_back(n);
    *graph = p->count() - 1;
    return DSSSP_OK;
}

int dsssp_pool_remove_graph(dsssp_pool* p, int32_t graph) {
    if (!p || graph < 0 || graph >= p->count()) return fail(DSSSP_E_INVAL, "pool_remove_graph: bad arguments");
    if (p->size(graph) == 0) return fail(DSSSP_E_INVAL, "pool_remove_graph: graph %d was removed already", graph);
    const int rc = dsssp_graph_clear_range(p->g, (int32_t)p->first[(size_t)graph], p->size(graph));
    if (rc) return rc;
    p->give_ids(p->first[(size_t)graph], p->size(graph));
    p->nv[(size_t)graph] = 0;
    return DSSSP_OK;
}

}  // extern "C"

// ---- serving ------------------------------------------------------------------------------

namespace {

using clk = std::chrono::steady_clock;

struct Req {
    dsssp_request_info info;
    std::vector<dsssp_change> ch;  // validated at submission; tenant-local ids
};

enum TenantState { kWaiting = DSSSP_TENANT_WAITING, kAdmitted = DSSSP_TENANT_ADMITTED, kRemoved = DSSSP_TENANT_REMOVED };

struct TenantRec {
    int32_t n = 0;
    int64_t m = 0;
    int32_t src = 0;
    int64_t footprint = 0;
    int state = kWaiting;
    int32_t graph = -1;  // pool graph while admitted
    std::vector<int32_t> u, v, w;  // the edges, kept while the tenant waits for admission
    std::deque<Req*> queue;        // waiting requests, arrival order
};

}  // namespace

struct dsssp_server {
    dsssp_pool* pool = nullptr;
    std::vector<TenantRec> tenants;  // guarded by mu (graph, state, queue)
    int64_t used = 0;                // footprint of the admitted tenants (guarded by dev)
    int32_t slack_pct = 25, slack_min = 4;
    dsssp_server_opts so{};
    clk::time_point t0;
    std::mutex dev;  // device work: epochs, reads, upkeep, admission; taken before mu
    std::mutex mu;   // tenants, queues, completed list, counters
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> done;
    std::unordered_map<int64_t, std::pair<std::vector<int32_t>, std::vector<int64_t>>> results;
    int64_t pending = 0, inflight = 0, next_id = 0, epochs = 0, compactions = 0, recovered = 0;
    bool upkeep = false;  // the idle upkeep after the last epoch has not finished yet
    std::atomic<int> record{0};
    double compact_ms = 0;
    bool stop = false;
    std::thread worker;

    double now_us() const { return std::chrono::duration<double, std::micro>(clk::now() - t0).count(); }

    void complete(Req* r) {  // with mu held
        done.push_back(r);
        cv_done.notify_all();
    }

    bool fits(const TenantRec& t) const {  // with dev held
        if (so.memory_budget > 0 && used + t.footprint > so.memory_budget) return false;
        return pool->find_ids(t.n) >= 0;
    }

    // Brings tenant t into the pool (with dev held; t is waiting and fits).
    int admit(int32_t t, const int32_t* u, const int32_t* v, const int32_t* w) {
        TenantRec& r = tenants[(size_t)t];
        int32_t gi = -1;
        const int rc = dsssp_pool_add_graph(pool, r.n, r.m, u, v, w, r.src, &gi);
        if (rc < 0) return rc;
        used += r.footprint;
        std::lock_guard<std::mutex> lk(mu);
        r.graph = gi;
        r.state = kAdmitted;
        std::vector<int32_t>().swap(r.u);
        std::vector<int32_t>().swap(r.v);
        std::vector<int32_t>().swap(r.w);
        return DSSSP_OK;
    }

    // Admits waiting tenants in the order they came while they fit (with dev held).
    void admit_waiting() {
        for (int32_t t = 0; t < (int32_t)tenants.size(); t++) {
            TenantRec& r = tenants[(size_t)t];
            if (r.state != kWaiting || !fits(r)) continue;
            admit(t, r.u.data(), r.v.data(), r.w.data());
        }
    }

    bool needs_compaction() {
        if (so.compact_dead_frac < 0) return false;
        int64_t live = 0, dead = 0, sp_used = 0, total = 0;
        if (dsssp_graph_health(pool->g, &live, &dead, &sp_used, &total) != DSSSP_OK) return false;
        if ((double)dead > so.compact_dead_frac * (double)(live > 0 ? live : 1)) return true;
        return total > 0 && (double)sp_used > so.compact_spare_frac * (double)total;
    }

    void idle_upkeep(std::unique_lock<std::mutex>& lk) {  // lk holds mu; released meanwhile
        upkeep = true;
        lk.unlock();
        double took = -1;
        {
            std::lock_guard<std::mutex> d(dev);
            if (needs_compaction()) {
                const auto c0 = clk::now();
                if (dsssp_graph_compact(pool->g) == DSSSP_OK)
                    took = std::chrono::duration<double, std::milli>(clk::now() - c0).count();
            }
        }
        lk.lock();
        if (took >= 0) {
            compactions++;
            compact_ms += took;
        }
        upkeep = false;
        cv_done.notify_all();
    }

    // An epoch: its requests and the id shift of each (its tenant's first id in the pool).
    struct Epoch {
        std::vector<Req*> reqs;
        std::vector<int32_t> shift;
        int64_t total = 0;
        double start = 0;
    };
    std::string tune_cache;  // autotuner cache (empty: none)
    std::string tune_key;    // size class whose cached options are set now
    dsssp_opts base_opts{};  // the options given at creation (classes the cache does not know)

    // Sets the cached options of the epoch's size class when it differs from the last epoch's
    // (with dev held, no batch pending).
    void tune_for(int64_t k) {
        if (tune_cache.empty()) return;
        int64_t n = 0, entries = 0;
        if (dsssp_graph_info(pool->g, &n, &entries, nullptr, nullptr, nullptr) != DSSSP_OK) return;
        char key[32];
        dsssp_tune_size_class(n, entries, k, key, sizeof key);
        if (tune_key == key) return;
        tune_key = key;
        dsssp_tune_result r;
        if (dsssp_autotune_lookup(pool->g, k, tune_cache.c_str(), &r) != DSSSP_OK)
            dsssp_graph_set_opts(pool->g, &base_opts);
    }

    dsssp_change* stage[2] = {nullptr, nullptr};  // pinned staging of two epochs' records
    int64_t stage_cap[2] = {0, 0};
    std::atomic<int> dev_waiters{0};  // threads waiting for the device between epochs

    // The oldest waiting request of every admitted tenant, oldest first (with dev held).
    void form(Epoch& e) {
        e.reqs.clear();
        e.shift.clear();
        e.total = 0;
        std::lock_guard<std::mutex> lk(mu);
        std::vector<std::pair<double, int32_t>> order;
        for (int32_t t = 0; t < (int32_t)tenants.size(); t++)
            if (!tenants[(size_t)t].queue.empty()) order.emplace_back(tenants[(size_t)t].queue.front()->info.arrival_us, t);
        std::sort(order.begin(), order.end());
        if (so.max_epoch_requests > 0 && (int32_t)order.size() > so.max_epoch_requests)
            order.resize((size_t)so.max_epoch_requests);
        for (auto& o : order) {
            TenantRec& tr = tenants[(size_t)o.second];
            e.reqs.push_back(tr.queue.front());
            tr.queue.pop_front();
            e.shift.push_back((int32_t)pool->first[(size_t)tr.graph]);
            e.total += (int64_t)e.reqs.back()->ch.size();
        }
        pending -= (int64_t)e.reqs.size();
        inflight += (int64_t)e.reqs.size();
    }

    // One pass over the records: copied into pinned stage b with ids shifted into the pool's
    // id space (they were validated at submission).
    int assemble(const Epoch& e, int b) {
        if (e.total > stage_cap[b]) {
            if (stage[b]) dsssp_host_free(stage[b]);
            stage_cap[b] = 0;
            const int64_t cap = e.total + e.total / 2 + 4096;
            stage[b] = (dsssp_change*)dsssp_host_alloc(sizeof(dsssp_change) * (size_t)cap);
            if (!stage[b]) return fail(DSSSP_E_OOM, "server: pinned staging buffer of %lld records", (long long)cap);
            stage_cap[b] = cap;
        }
        int64_t at = 0;
        for (size_t i = 0; i < e.reqs.size(); i++) {
            copy_shifted(e.reqs[i]->ch.data(), (int64_t)e.reqs[i]->ch.size(), e.shift[i], stage[b] + at);
            at += (int64_t)e.reqs[i]->ch.size();
        }
        return DSSSP_OK;
    }

    // Completes an epoch's requests with status rc (with dev held).
    void complete_epoch(Epoch& e, int rc, double end) {
        char why[96] = {0};
        if (rc) snprintf(why, sizeof why, "%s", dsssp_last_error());
        if (rc >= 0 && record.load()) {
            for (Req* r : e.reqs) {
                const int32_t gi = tenants[(size_t)r->info.tenant].graph, nn = pool->size(gi);
                std::vector<int32_t> par((size_t)nn);
                std::vector<int64_t> dist((size_t)nn);
                if (dsssp_pool_tree_read(pool, gi, par.data(), dist.data()) == DSSSP_OK) {
                    std::lock_guard<std::mutex> lk(mu);
                    results[r->info.id] = {std::move(par), std::move(dist)};
                }
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        for (Req* r : e.reqs) {
            r->info.epoch = epochs;
            r->info.start_us = e.start;
            r->info.done_us = end;
            r->info.status = rc;
            if (rc) snprintf(r->info.error, sizeof r->info.error, "%s", why);
            std::vector<dsssp_change>().swap(r->ch);
            complete(r);
        }
        if (rc == DSSSP_W_RECOMPUTED) recovered++;
        epochs++;
        inflight -= (int64_t)e.reqs.size();
        e.reqs.clear();
    }

    // Epochs are pipelined: while epoch i runs on the device, the host forms epoch i + 1 and
    // copies its records into the other pinned buffer; then it waits for epoch i, completes its
    // requests (reading recorded trees) and enqueues epoch i + 1.  The device mutex is held
    // while epochs are in flight and released between them as soon as another thread waits
    // for it (reads, admission, removal) or no request is left.
    void run() {
        Epoch ep[2];
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                if (pending == 0 && !stop) {  // idle: storage upkeep is off the latency path
                    idle_upkeep(lk);
                    cv_work.wait(lk, [&] { return stop || pending > 0; });
                }
                if (pending == 0 && stop) return;
            }
            while (dev_waiters.load() > 0) std::this_thread::sleep_for(std::chrono::microseconds(20));
            std::lock_guard<std::mutex> d(dev);  // before mu: no admission or removal mid-epoch
            int cur = 0;
            bool flying = false;  // ep[cur ^ 1] is on the device
            for (;;) {
                const bool more = dev_waiters.load() == 0;
                if (more) form(ep[cur]);
                const int arc = ep[cur].reqs.empty() ? DSSSP_OK : assemble(ep[cur], cur);
                if (flying) {
                    dsssp_stats st;
                    const int rc = dsssp_batch_finish(pool->g, &st);
                    complete_epoch(ep[cur ^ 1], rc, now_us());
                    flying = false;
                }
                if (ep[cur].reqs.empty()) break;
                tune_for(ep[cur].total);
                ep[cur].start = now_us();
                int rc = arc;
                if (!rc) rc = dsssp_apply_batch_host_async(pool->g, stage[cur], ep[cur].total, nullptr);
                if (rc) {  // nothing was enqueued
                    complete_epoch(ep[cur], rc, now_us());
                    break;
                }
                flying = true;
                cur ^= 1;
            }
            std::lock_guard<std::mutex> lk(mu);
            upkeep = pending == 0;  // the idle upkeep comes next; drain waits for it
        }
    }

    ~dsssp_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        if (worker.joinable()) worker.join();
        for (auto& t : tenants)
            for (Req* r : t.queue) delete r;
        for (Req* r : done) delete r;
        for (auto* b : stage)
            if (b) dsssp_host_free(b);
        dsssp_pool_destroy(pool);
    }
};

namespace {

// Takes the server's device mutex from a thread other than the worker: announced first, so
// that the worker leaves its epoch pipeline after the epoch in flight.
struct DevLock {
    dsssp_server* s;
    explicit DevLock(dsssp_server* sv) : s(sv) {
        s->dev_waiters.fetch_add(1);
        s->dev.lock();
        s->dev_waiters.fetch_sub(1);
    }
    ~DevLock() { s->dev.unlock(); }
};

}  // namespace

extern "C" {

void dsssp_default_server_opts(dsssp_server_opts* so) {
    if (!so) return;
    memset(so, 0, sizeof(*so));
    so->memory_budget = 0;
    so->max_epoch_requests = 0;
    so->record = 0;
    so->compact_dead_frac = 0.25;
    so->compact_spare_frac = 0.75;
    so->reserve_vertices = 0;
    so->tune_cache = nullptr;
}

int dsssp_server_create(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                        const int32_t* const* v, const int32_t* const* w, const int32_t* sources,
                        const dsssp_server_opts* so, const dsssp_opts* o, dsssp_server** out) {
    if (count < 0 || (count > 0 && (!n || !m || !u || !v || !w || !sources)) || !out)
        return fail(DSSSP_E_INVAL, "server_create: bad arguments");
    dsssp_server* s = new dsssp_server();
    if (so) s->so = *so;
    else dsssp_default_server_opts(&s->so);
    if (s->so.reserve_vertices < 0) {
        delete s;
        return fail(DSSSP_E_INVAL, "server_create: negative vertex reserve");
    }
    dsssp_opts opts;
    if (o) opts = *o;
    else dsssp_default_opts(&opts);
    s->slack_pct = opts.slack_pct;
    s->slack_min = opts.slack_min;
    s->base_opts = opts;
    if (s->so.tune_cache) s->tune_cache = s->so.tune_cache;
    s->so.tune_cache = nullptr;  // the caller's string is not kept
    // admission: tenants in order while their estimated footprint fits the budget; the others
    // wait (their ids are reserved in the pool, so that they can come in when memory frees)
    std::vector<int32_t> an, asrc;
    std::vector<int64_t> am;
    std::vector<const int32_t*> au, av, aw;
    int64_t waiting_ids = 0;
    s->tenants.resize((size_t)count);
    for (int32_t t = 0; t < count; t++) {
        TenantRec& r = s->tenants[(size_t)t];
        if (n[t] < 1 || m[t] < 0 || (m[t] > 0 && (!u[t] || !v[t] || !w[t])) || sources[t] < 0 || sources[t] >= n[t]) {
            delete s;
            return fail(DSSSP_E_INVAL, "server_create: tenant %d needs at least one vertex, its edges and a source in range", t);
        }
        r.n = n[t];
        r.m = m[t];
        r.src = sources[t];
        r.footprint = dsssp_estimate_footprint(n[t], m[t], opts.slack_pct, opts.slack_min);
        if (s->so.memory_budget > 0 && s->used + r.footprint > s->so.memory_budget) {
            int rc = check_edges(n[t], m[t], u[t], v[t], w[t], "server_create");
            if (rc) {
                delete s;
                return rc;
            }
            r.u.assign(u[t], u[t] + m[t]);
            r.v.assign(v[t], v[t] + m[t]);
            r.w.assign(w[t], w[t] + m[t]);
            waiting_ids += n[t];
            continue;
        }
        s->used += r.footprint;
        r.state = kAdmitted;
        r.graph = (int32_t)an.size();
        an.push_back(n[t]);
        am.push_back(m[t]);
        au.push_back(u[t]);
        av.push_back(v[t]);
        aw.push_back(w[t]);
        asrc.push_back(sources[t]);
    }
    const int64_t reserve = s->so.reserve_vertices + waiting_ids;
    if (an.empty() && reserve == 0) {
        delete s;
        return fail(DSSSP_E_INVAL, "server_create: no tenant and no vertex reserve");
    }
    int rc = pool_create_impl((int32_t)an.size(), an.data(), am.data(), au.data(), av.data(), aw.data(), reserve,
                              &opts, &s->pool);
    if (!rc && !an.empty()) rc = dsssp_pool_tree_compute(s->pool, asrc.data(), nullptr);
    if (rc) {
        delete s;
        return rc;
    }
    s->record = s->so.record;
    s->t0 = clk::now();
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return DSSSP_OK;
}

void dsssp_server_destroy(dsssp_server* s) { delete s; }

int dsssp_server_slot(const dsssp_server* s, int32_t tenant) {
    if (!s) return -1;
    dsssp_server* ms = const_cast<dsssp_server*>(s);
    std::lock_guard<std::mutex> lk(ms->mu);
    if (tenant < 0 || tenant >= (int32_t)s->tenants.size()) return -1;
    const TenantRec& r = s->tenants[(size_t)tenant];
    return r.state == kAdmitted ? r.graph : -1;
}

int dsssp_server_tenant_state(const dsssp_server* s, int32_t tenant) {
    if (!s) return fail(DSSSP_E_INVAL, "server_tenant_state: NULL server");
    dsssp_server* ms = const_cast<dsssp_server*>(s);
    std::lock_guard<std::mutex> lk(ms->mu);
    if (tenant < 0 || tenant >= (int32_t)s->tenants.size()) return fail(DSSSP_E_INVAL, "no tenant %d", tenant);
    return s->tenants[(size_t)tenant].state;
}

int dsssp_server_add_tenant(dsssp_server* s, int32_t n, int64_t m, const int32_t* u, const int32_t* v,
                            const int32_t* w, int32_t src, int32_t* tenant) {
    if (!s || n < 1 || m < 0 || (m > 0 && (!u || !v || !w)) || !tenant)
        return fail(DSSSP_E_INVAL, "server_add_tenant: bad arguments");
    if (src < 0 || src >= n) return fail(DSSSP_E_BAD_VERTEX, "server_add_tenant: source %d outside 0..%d", src, n - 1);
    int rc = check_edges(n, m, u, v, w, "server_add_tenant");
    if (rc) return rc;
    TenantRec r;
    r.n = n;
    r.m = m;
    r.src = src;
    r.footprint = dsssp_estimate_footprint(n, m, s->slack_pct, s->slack_min);
    DevLock d(s);  // after any running epoch
    int32_t t;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        t = (int32_t)s->tenants.size();
        s->tenants.push_back(std::move(r));
    }
    *tenant = t;
    if (s->fits(s->tenants[(size_t)t]) && s->admit(t, u, v, w) == DSSSP_OK) return DSSSP_OK;
    std::lock_guard<std::mutex> lk(s->mu);  // waits: keep its edges for a later admission
    TenantRec& tr = s->tenants[(size_t)t];
    tr.u.assign(u, u + m);
    tr.v.assign(v, v + m);
    tr.w.assign(w, w + m);
    return DSSSP_OK;
}

int dsssp_server_remove_tenant(dsssp_server* s, int32_t tenant) {
    if (!s) return fail(DSSSP_E_INVAL, "server_remove_tenant: NULL server");
    DevLock d(s);  // after any running epoch
    int32_t gi = -1;
    int64_t fp = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (tenant < 0 || tenant >= (int32_t)s->tenants.size()) return fail(DSSSP_E_INVAL, "no tenant %d", tenant);
        TenantRec& r = s->tenants[(size_t)tenant];
        if (r.state == kRemoved) return fail(DSSSP_E_INVAL, "tenant %d was removed already", tenant);
        const double t = s->now_us();
        for (Req* q : r.queue) {  // its waiting requests are refused
            q->info.status = DSSSP_REFUSED;
            snprintf(q->info.error, sizeof q->info.error, "tenant removed");
            q->info.start_us = q->info.done_us = t;
            std::vector<dsssp_change>().swap(q->ch);
            s->complete(q);
        }
        s->pending -= (int64_t)r.queue.size();
        r.queue.clear();
        if (r.state == kAdmitted) {
            gi = r.graph;
            fp = r.footprint;
        }
        r.state = kRemoved;
        r.graph = -1;
        std::vector<int32_t>().swap(r.u);
        std::vector<int32_t>().swap(r.v);
        std::vector<int32_t>().swap(r.w);
    }
    if (gi >= 0) {
        const int rc = dsssp_pool_remove_graph(s->pool, gi);
        if (rc) return rc;
        s->used -= fp;
    }
    s->admit_waiting();  // memory and ids freed: waiting tenants may come in now
    s->cv_done.notify_all();
    return DSSSP_OK;
}

int dsssp_submit_many(dsssp_server* s, int32_t count, const int32_t* tenants, const dsssp_change* const* batches,
                      const int64_t* sizes, int64_t* ids) {
    if (!s || count < 0 || (count > 0 && (!tenants || !batches || !sizes || !ids)))
        return fail(DSSSP_E_INVAL, "submit: bad arguments");
    // Requests are taken in chunks (up to 64 requests or about 2^20 records): a chunk is
    // validated and copied outside the queue lock and then queued, so the worker starts on the
    // first chunk while the later ones are still being copied, and a large submission stays
    // off the other requests' latency.  Every request carries the call's arrival time.
    const double t = s->now_us();
    std::vector<int32_t> tn((size_t)count, -1);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (int32_t i = 0; i < count; i++)
            if (tenants[i] >= 0 && tenants[i] < (int32_t)s->tenants.size()) tn[(size_t)i] = s->tenants[(size_t)tenants[i]].n;
    }
    int32_t a = 0;
    while (a < count) {
        int32_t b = a;
        int64_t recs = 0;
        while (b < count && b - a < 64 && (b == a || recs + (sizes[b] > 0 ? sizes[b] : 0) <= (1 << 20))) {
            recs += sizes[b] > 0 ? sizes[b] : 0;
            b++;
        }
        std::vector<Req*> reqs;
        reqs.reserve((size_t)(b - a));
        for (int32_t i = a; i < b; i++) {
            Req* r = new Req();
            reqs.push_back(r);
            memset(&r->info, 0, sizeof(r->info));
            r->info.tenant = tenants[i];
            r->info.changes = sizes[i];
            r->info.arrival_us = t;
            r->info.epoch = -1;
            if (tn[(size_t)i] < 0) {
                r->info.status = DSSSP_REFUSED;
                snprintf(r->info.error, sizeof r->info.error, "no such tenant");
            } else if (sizes[i] < 0 || (sizes[i] > 0 && !batches[i])) {
                r->info.status = DSSSP_E_INVAL;
                snprintf(r->info.error, sizeof r->info.error, "bad batch");
            } else {
                const std::string why = check_batch(batches[i], sizes[i], tn[(size_t)i]);
                if (!why.empty()) {
                    r->info.status = why.find("weight") != std::string::npos ? DSSSP_E_BAD_WEIGHT : DSSSP_E_BAD_VERTEX;
                    snprintf(r->info.error, sizeof r->info.error, "%s", why.c_str());
                } else {
                    r->ch.assign(batches[i], batches[i] + sizes[i]);
                }
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (int32_t i = a; i < b; i++) {
                Req* r = reqs[(size_t)(i - a)];
                r->info.id = s->next_id++;
                ids[i] = r->info.id;
                if (r->info.status == 0) {
                    TenantRec& tr = s->tenants[(size_t)r->info.tenant];
                    if (tr.state != kAdmitted) {
                        r->info.status = DSSSP_REFUSED;
                        snprintf(r->info.error, sizeof r->info.error, "%s",
                                 tr.state == kWaiting ? "tenant not admitted (waiting for memory)" : "tenant removed");
                        std::vector<dsssp_change>().swap(r->ch);
                    }
                }
                if (r->info.status == 0) {
                    s->tenants[(size_t)r->info.tenant].queue.push_back(r);
                    s->pending++;
                } else {
                    r->info.start_us = r->info.done_us = t;
                    s->complete(r);
                }
            }
        }
        s->cv_work.notify_one();
        a = b;
    }
    return DSSSP_OK;
}

int dsssp_submit(dsssp_server* s, int32_t tenant, const dsssp_change* changes, int64_t k, int64_t* id) {
    return dsssp_submit_many(s, 1, &tenant, &changes, &k, id);
}

int dsssp_poll(dsssp_server* s, dsssp_request_info* out, int32_t cap, int32_t wait_ms, int32_t* count) {
    if (!s || cap < 0 || (cap > 0 && !out) || !count) return fail(DSSSP_E_INVAL, "poll: bad arguments");
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
    int32_t k = 0;
    while (k < cap && !s->done.empty()) {
        Req* r = s->done.front();
        s->done.pop_front();
        out[k++] = r->info;
        delete r;
    }
    *count = k;
    return DSSSP_OK;
}

int dsssp_server_drain(dsssp_server* s, int32_t timeout_ms) {
    if (!s) return fail(DSSSP_E_INVAL, "drain: NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms > 0 ? timeout_ms : 1),
                                        [&] { return s->pending == 0 && s->inflight == 0 && !s->upkeep; });
    return ok ? DSSSP_OK : fail(DSSSP_E_TIMEOUT, "drain: requests still waiting after %d ms", timeout_ms);
}

int dsssp_server_result(dsssp_server* s, int64_t id, int32_t* parent, int64_t* dist) {
    if (!s || !parent || !dist) return fail(DSSSP_E_INVAL, "server_result: bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->results.find(id);
    if (it == s->results.end()) return fail(DSSSP_E_INVAL, "server_result: no recorded tree for request %lld", (long long)id);
    memcpy(parent, it->second.first.data(), sizeof(int32_t) * it->second.first.size());
    memcpy(dist, it->second.second.data(), sizeof(int64_t) * it->second.second.size());
    s->results.erase(it);
    return DSSSP_OK;
}

int dsssp_server_tree_read(dsssp_server* s, int32_t tenant, int32_t* parent, int64_t* dist) {
    if (!s) return fail(DSSSP_E_INVAL, "server_tree_read: NULL server");
    DevLock d(s);
    const int32_t gi = dsssp_server_slot(s, tenant);
    if (gi < 0) return fail(DSSSP_E_INVAL, "server_tree_read: tenant %d is not served", tenant);
    return dsssp_pool_tree_read(s->pool, gi, parent, dist);
}

int dsssp_server_info(dsssp_server* s, int64_t* epochs, int64_t* compactions, double* compact_ms,
                      int64_t* pending) {
    if (!s) return fail(DSSSP_E_INVAL, "server_info: NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (epochs) *epochs = s->epochs;
    if (compactions) *compactions = s->compactions;
    if (compact_ms) *compact_ms = s->compact_ms;
    if (pending) *pending = s->pending + s->inflight;
    return DSSSP_OK;
}

int dsssp_server_recovered_epochs(dsssp_server* s, int64_t* epochs) {
    if (!s || !epochs) return fail(DSSSP_E_INVAL, "server_recovered_epochs: bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    *epochs = s->recovered;
    return DSSSP_OK;
}

dsssp_pool* dsssp_server_pool(dsssp_server* s) { return s ? s->pool : nullptr; }

int dsssp_server_validate(dsssp_server* s, int64_t* violations, int64_t* roots) {
    if (!s || !violations) return fail(DSSSP_E_INVAL, "server_validate: bad arguments");
    DevLock d(s);
    return dsssp_tree_validate(s->pool->g, violations, roots, nullptr);
}

int dsssp_server_set_record(dsssp_server* s, int32_t on) {
    if (!s) return fail(DSSSP_E_INVAL, "server_set_record: NULL server");
    s->record = on ? 1 : 0;
    if (!on) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->results.clear();
    }
    return DSSSP_OK;
}

int dsssp_server_debug_set(dsssp_server* s, int32_t what, int64_t value) {
    if (!s) return fail(DSSSP_E_INVAL, "server_debug_set: NULL server");
    DevLock d(s);  // between epochs
    return dsssp_debug_set(s->pool->g, what, value);
}

}  // extern "C"
