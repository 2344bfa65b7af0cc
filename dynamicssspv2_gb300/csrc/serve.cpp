// serve.cpp -- the batching and serving layers: a pooled graph store of many graphs and a
// request loop with continuous batching, as C++ host code over the engine's C ABI.
//
// Pool: the graphs are laid out side by side in one vertex id space (graph i owns ids
// [off[i], off[i] + n_i)), so one engine graph holds their disjoint union and every graph is
// a separate part with its own root.  A set of change batches -- at most one per graph --
// becomes one change batch of the union (ids shifted), applied by one launch sequence; the
// update of one graph never reads another graph's data, so each graph's result equals
// applying its batch alone (distances bit-exact, parents a valid tree).
//
// Server: tenants are admitted in order while their estimated device footprint fits the
// memory budget and live in one pool.  dsssp_submit queues a request (a copy of its batch)
// and returns at once; a worker thread serves epochs back to back: every tenant with a
// waiting request contributes its oldest one, the epoch's batches run as one union batch,
// and the requests complete together.  A tenant never has two requests in one epoch, so its
// batches apply in arrival order and each result equals applying that batch alone.
// Requests for tenants that were not admitted are refused and malformed ones fail at
// submission, without touching any epoch.  While no request waits, the worker compacts the
// store when its tombstones or its spare-region use pass the configured fractions.
//
// No counterpart in the reference, which applies one batch per process run.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
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
    std::vector<int64_t> off;  // count + 1 offsets into the union's id space
    dsssp_change* stage = nullptr;  // pinned staging buffer of the union batch
    int64_t stage_cap = 0;
    std::vector<int32_t> par;  // tree-read staging
    std::vector<int64_t> dst;

    int32_t count() const { return (int32_t)off.size() - 1; }
    int32_t size(int32_t i) const { return (int32_t)(off[(size_t)i + 1] - off[(size_t)i]); }
    ~dsssp_pool() {
        if (stage) dsssp_host_free(stage);
        if (g) dsssp_graph_destroy(g);
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

int union_batch(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                const int64_t* sizes, dsssp_change* out, int64_t cap, int64_t* k) {
    std::vector<char> seen((size_t)p->count(), 0);
    int64_t total = 0;
    for (int32_t b = 0; b < nb; b++) {
        const int32_t gi = graphs[b];
        if (gi < 0 || gi >= p->count()) return fail(DSSSP_E_INVAL, "pool: no graph %d", gi);
        if (seen[(size_t)gi]) return fail(DSSSP_E_INVAL, "pool: graph %d has two batches in one union", gi);
        seen[(size_t)gi] = 1;
        if (sizes[b] < 0 || (sizes[b] > 0 && !batches[b])) return fail(DSSSP_E_INVAL, "pool: bad batch for graph %d", gi);
        const std::string why = check_batch(batches[b], sizes[b], p->size(gi));
        if (!why.empty())
            return fail(why.find("weight") != std::string::npos ? DSSSP_E_BAD_WEIGHT : DSSSP_E_BAD_VERTEX, "pool graph %d: %s",
                        gi, why.c_str());
        total += sizes[b];
    }
    *k = total;
    if (!out) return DSSSP_OK;
    if (total > cap) return fail(DSSSP_E_INVAL, "pool: union batch of %lld records exceeds %lld", (long long)total, (long long)cap);
    int64_t at = 0;
    for (int32_t b = 0; b < nb; b++) {
        const int32_t shift = (int32_t)p->off[(size_t)graphs[b]];
        const dsssp_change* src = batches[b];
        for (int64_t i = 0; i < sizes[b]; i++) {
            dsssp_change c = src[i];
            c.u += shift;
            c.v += shift;
            out[at++] = c;
        }
    }
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
    if (count < 1 || !n || !m || !u || !v || !w || !out) return fail(DSSSP_E_INVAL, "pool_create: bad arguments");
    dsssp_pool* p = new dsssp_pool();
    p->off.assign((size_t)count + 1, 0);
    int64_t edges = 0;
    for (int32_t i = 0; i < count; i++) {
        if (n[i] <= 0 || m[i] < 0 || (m[i] > 0 && (!u[i] || !v[i] || !w[i]))) {
            delete p;
            return fail(DSSSP_E_INVAL, "pool_create: graph %d needs at least one vertex and its edge arrays", i);
        }
        p->off[(size_t)i + 1] = p->off[(size_t)i] + n[i];
        edges += m[i];
    }
    if (p->off.back() >= (1ll << 31) - 16) {
        delete p;
        return fail(DSSSP_E_INVAL, "pool_create: the pool's vertex count must stay below 2^31");
    }
    std::vector<int32_t> U((size_t)edges), V((size_t)edges), W((size_t)edges);
    int64_t at = 0;
    for (int32_t i = 0; i < count; i++) {
        const int32_t shift = (int32_t)p->off[(size_t)i];
        for (int64_t j = 0; j < m[i]; j++, at++) {
            if (u[i][j] < 0 || u[i][j] >= n[i] || v[i][j] < 0 || v[i][j] >= n[i]) {
                delete p;
                return fail(DSSSP_E_BAD_VERTEX, "pool_create: graph %d edge %lld names a vertex outside 0..%d", i,
                            (long long)j, n[i] - 1);
            }
            U[(size_t)at] = u[i][j] + shift;
            V[(size_t)at] = v[i][j] + shift;
            W[(size_t)at] = w[i][j];
        }
    }
    const int rc = dsssp_graph_create((int32_t)p->off.back(), edges, U.data(), V.data(), W.data(), o, &p->g);
    if (rc) {
        delete p;
        return rc;
    }
    *out = p;
    return DSSSP_OK;
}

void dsssp_pool_destroy(dsssp_pool* p) { delete p; }

dsssp_graph* dsssp_pool_graph(dsssp_pool* p) { return p ? p->g : nullptr; }

int dsssp_pool_offsets(const dsssp_pool* p, int64_t* offsets) {
    if (!p || !offsets) return fail(DSSSP_E_INVAL, "pool_offsets: bad arguments");
    memcpy(offsets, p->off.data(), sizeof(int64_t) * p->off.size());
    return DSSSP_OK;
}

int dsssp_pool_tree_compute(dsssp_pool* p, const int32_t* sources, dsssp_stats* st) {
    if (!p || !sources) return fail(DSSSP_E_INVAL, "pool_tree_compute: bad arguments");
    std::vector<int32_t> s((size_t)p->count());
    for (int32_t i = 0; i < p->count(); i++) {
        if (sources[i] < 0 || sources[i] >= p->size(i))
            return fail(DSSSP_E_BAD_VERTEX, "pool_tree_compute: source %d of graph %d out of range", sources[i], i);
        s[(size_t)i] = sources[i] + (int32_t)p->off[(size_t)i];
    }
    return dsssp_tree_compute_multi(p->g, s.data(), p->count(), st);
}

int dsssp_pool_forest_load(dsssp_pool* p, const int32_t* const* parent, const int64_t* const* dist) {
    if (!p || !parent || !dist) return fail(DSSSP_E_INVAL, "pool_forest_load: bad arguments");
    const size_t N = (size_t)p->off.back();
    std::vector<int32_t> par(N);
    std::vector<int64_t> d(N);
    for (int32_t i = 0; i < p->count(); i++) {
        const int64_t a = p->off[(size_t)i];
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
    return union_batch(p, nb, graphs, batches, sizes, out, cap, k);
}

int dsssp_pool_apply(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                     const int64_t* sizes, dsssp_stats* st) {
    if (!p || nb < 0 || (nb > 0 && (!graphs || !batches || !sizes)))
        return fail(DSSSP_E_INVAL, "pool_apply: bad arguments");
    int64_t total = 0;
    int rc = union_batch(p, nb, graphs, batches, sizes, nullptr, 0, &total);
    if (rc) return rc;
    if (total > p->stage_cap) {
        if (p->stage) dsssp_host_free(p->stage);
        p->stage_cap = 0;
        const int64_t cap = total + total / 2 + 1024;
        p->stage = (dsssp_change*)dsssp_host_alloc(sizeof(dsssp_change) * (size_t)cap);
        if (!p->stage) return fail(DSSSP_E_OOM, "pool_apply: pinned staging buffer");
        p->stage_cap = cap;
    }
    rc = union_batch(p, nb, graphs, batches, sizes, p->stage, p->stage_cap, &total);
    if (rc) return rc;
    return dsssp_apply_batch(p->g, p->stage, total, nullptr, st);
}

int dsssp_pool_tree_read(dsssp_pool* p, int32_t graph, int32_t* parent, int64_t* dist) {
    if (!p || graph < 0 || graph >= p->count() || !parent || !dist) return fail(DSSSP_E_INVAL, "pool_tree_read: bad arguments");
    const int32_t a = (int32_t)p->off[(size_t)graph], nn = p->size(graph);
    const int rc = dsssp_tree_read_range(p->g, a, nn, parent, dist);
    if (rc) return rc;
    for (int32_t x = 0; x < nn; x++)
        if (parent[x] >= 0) parent[x] -= a;
    return DSSSP_OK;
}

}  // extern "C"

// ---- serving ------------------------------------------------------------------------------

namespace {

using clk = std::chrono::steady_clock;

struct Req {
    dsssp_request_info info;
    std::vector<dsssp_change> ch;
};

}  // namespace

struct dsssp_server {
    dsssp_pool* pool = nullptr;
    std::vector<int32_t> slot;  // tenant -> pool graph, -1 = not admitted
    std::vector<int32_t> tenant_of;  // pool graph -> tenant
    dsssp_server_opts so{};
    clk::time_point t0;
    std::mutex mu;  // queues, completed list, counters
    std::condition_variable cv_work, cv_done;
    std::mutex dev;  // device work: epochs, reads, upkeep
    std::vector<std::deque<Req*>> queues;  // per pool graph, arrival order
    std::deque<Req*> done;
    std::unordered_map<int64_t, std::pair<std::vector<int32_t>, std::vector<int64_t>>> results;
    int64_t pending = 0, inflight = 0, next_id = 0, epochs = 0, compactions = 0;
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

    bool needs_compaction() {
        if (so.compact_dead_frac < 0) return false;
        int64_t live = 0, dead = 0, used = 0, total = 0;
        if (dsssp_graph_health(pool->g, &live, &dead, &used, &total) != DSSSP_OK) return false;
        if ((double)dead > so.compact_dead_frac * (double)(live > 0 ? live : 1)) return true;
        return total > 0 && (double)used > so.compact_spare_frac * (double)total;
    }

    void run() {
        std::vector<Req*> ep;
        std::vector<int32_t> graphs;
        std::vector<const dsssp_change*> batches;
        std::vector<int64_t> sizes;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                if (pending == 0 && !stop) {  // idle: storage upkeep is off the latency path
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
                    cv_work.wait(lk, [&] { return stop || pending > 0; });
                }
                if (pending == 0 && stop) return;
                // the epoch: the oldest waiting request of every tenant, oldest first
                std::vector<std::pair<double, int32_t>> order;
                for (int32_t gi = 0; gi < (int32_t)queues.size(); gi++)
                    if (!queues[(size_t)gi].empty()) order.emplace_back(queues[(size_t)gi].front()->info.arrival_us, gi);
                std::sort(order.begin(), order.end());
                if (so.max_epoch_requests > 0 && (int32_t)order.size() > so.max_epoch_requests)
                    order.resize((size_t)so.max_epoch_requests);
                ep.clear();
                for (auto& o : order) {
                    ep.push_back(queues[(size_t)o.second].front());
                    queues[(size_t)o.second].pop_front();
                }
                pending -= (int64_t)ep.size();
                inflight = (int64_t)ep.size();
            }
            graphs.clear();
            batches.clear();
            sizes.clear();
            for (Req* r : ep) {
                graphs.push_back(slot[(size_t)r->info.tenant]);
                batches.push_back(r->ch.data());
                sizes.push_back((int64_t)r->ch.size());
            }
            int rc;
            double start, end;
            {
                std::lock_guard<std::mutex> d(dev);
                start = now_us();
                dsssp_stats st;
                rc = dsssp_pool_apply(pool, (int32_t)ep.size(), graphs.data(), batches.data(), sizes.data(), &st);
                end = now_us();
                if (rc == DSSSP_OK && record.load()) {
                    for (Req* r : ep) {
                        const int32_t gi = slot[(size_t)r->info.tenant], nn = pool->size(gi);
                        std::vector<int32_t> par((size_t)nn);
                        std::vector<int64_t> dist((size_t)nn);
                        if (dsssp_pool_tree_read(pool, gi, par.data(), dist.data()) == DSSSP_OK) {
                            std::lock_guard<std::mutex> lk(mu);
                            results[r->info.id] = {std::move(par), std::move(dist)};
                        }
                    }
                }
            }
            std::lock_guard<std::mutex> lk(mu);
            for (Req* r : ep) {
                r->info.epoch = epochs;
                r->info.start_us = start;
                r->info.done_us = end;
                r->info.status = rc;
                if (rc) snprintf(r->info.error, sizeof r->info.error, "%s", dsssp_last_error());
                r->ch.clear();
                r->ch.shrink_to_fit();
                complete(r);
            }
            epochs++;
            inflight = 0;
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
        for (auto& q : queues)
            for (Req* r : q) delete r;
        for (Req* r : done) delete r;
        dsssp_pool_destroy(pool);
    }
};

extern "C" {

void dsssp_default_server_opts(dsssp_server_opts* so) {
    if (!so) return;
    memset(so, 0, sizeof(*so));
    so->memory_budget = 0;
    so->max_epoch_requests = 0;
    so->record = 0;
    so->compact_dead_frac = 0.25;
    so->compact_spare_frac = 0.75;
}

int dsssp_server_create(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                        const int32_t* const* v, const int32_t* const* w, const int32_t* sources,
                        const dsssp_server_opts* so, const dsssp_opts* o, dsssp_server** out) {
    if (count < 1 || !n || !m || !u || !v || !w || !sources || !out) return fail(DSSSP_E_INVAL, "server_create: bad arguments");
    dsssp_server* s = new dsssp_server();
    if (so) s->so = *so;
    else dsssp_default_server_opts(&s->so);
    dsssp_opts opts;
    if (o) opts = *o;
    else dsssp_default_opts(&opts);
    // admission: tenants in order while their estimated footprint fits the budget
    s->slot.assign((size_t)count, -1);
    std::vector<int32_t> an, asrc;
    std::vector<int64_t> am;
    std::vector<const int32_t*> au, av, aw;
    int64_t used = 0;
    for (int32_t t = 0; t < count; t++) {
        const int64_t fp = dsssp_estimate_footprint(n[t], m[t], opts.slack_pct, opts.slack_min);
        if (s->so.memory_budget > 0 && used + fp > s->so.memory_budget) continue;
        used += fp;
        s->slot[(size_t)t] = (int32_t)an.size();
        s->tenant_of.push_back(t);
        an.push_back(n[t]);
        am.push_back(m[t]);
        au.push_back(u[t]);
        av.push_back(v[t]);
        aw.push_back(w[t]);
        asrc.push_back(sources[t]);
    }
    if (an.empty()) {
        delete s;
        return fail(DSSSP_E_OOM, "server_create: no tenant fits the memory budget");
    }
    int rc = dsssp_pool_create((int32_t)an.size(), an.data(), am.data(), au.data(), av.data(), aw.data(), &opts, &s->pool);
    if (!rc) rc = dsssp_pool_tree_compute(s->pool, asrc.data(), nullptr);
    if (rc) {
        delete s;
        return rc;
    }
    s->queues.resize(an.size());
    s->record = s->so.record;
    s->t0 = clk::now();
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return DSSSP_OK;
}

void dsssp_server_destroy(dsssp_server* s) { delete s; }

int dsssp_server_slot(const dsssp_server* s, int32_t tenant) {
    if (!s || tenant < 0 || tenant >= (int32_t)s->slot.size()) return -1;
    return s->slot[(size_t)tenant];
}

int dsssp_submit_many(dsssp_server* s, int32_t count, const int32_t* tenants, const dsssp_change* const* batches,
                      const int64_t* sizes, int64_t* ids) {
    if (!s || count < 0 || (count > 0 && (!tenants || !batches || !sizes || !ids)))
        return fail(DSSSP_E_INVAL, "submit: bad arguments");
    // Validation and the copy of each batch happen before the lock: the worker takes the same
    // lock between epochs, so holding it only to number and queue the requests keeps a large
    // submission off the other requests' latency.  (Admission and tenant sizes are fixed.)
    const double t = s->now_us();
    std::vector<Req*> reqs((size_t)count);
    for (int32_t i = 0; i < count; i++) {
        Req* r = new Req();
        reqs[(size_t)i] = r;
        memset(&r->info, 0, sizeof(r->info));
        r->info.tenant = tenants[i];
        r->info.changes = sizes[i];
        r->info.arrival_us = t;
        r->info.epoch = -1;
        const bool known = tenants[i] >= 0 && tenants[i] < (int32_t)s->slot.size();
        if (!known || s->slot[(size_t)tenants[i]] < 0) {
            r->info.status = DSSSP_REFUSED;
            snprintf(r->info.error, sizeof r->info.error, "%s", known ? "tenant not admitted" : "no such tenant");
        } else if (sizes[i] < 0 || (sizes[i] > 0 && !batches[i])) {
            r->info.status = DSSSP_E_INVAL;
            snprintf(r->info.error, sizeof r->info.error, "bad batch");
        } else {
            const std::string why = check_batch(batches[i], sizes[i], s->pool->size(s->slot[(size_t)tenants[i]]));
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
        for (int32_t i = 0; i < count; i++) {
            Req* r = reqs[(size_t)i];
            r->info.id = s->next_id++;
            ids[i] = r->info.id;
            if (r->info.status == 0) {
                s->queues[(size_t)s->slot[(size_t)r->info.tenant]].push_back(r);
                s->pending++;
            } else {
                r->info.start_us = r->info.done_us = t;
                s->complete(r);
            }
        }
    }
    s->cv_work.notify_one();
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
    const int32_t gi = dsssp_server_slot(s, tenant);
    if (gi < 0) return fail(DSSSP_E_INVAL, "server_tree_read: tenant %d is not served", tenant);
    std::lock_guard<std::mutex> d(s->dev);
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

dsssp_pool* dsssp_server_pool(dsssp_server* s) { return s ? s->pool : nullptr; }

int dsssp_server_validate(dsssp_server* s, int64_t* violations, int64_t* roots) {
    if (!s || !violations) return fail(DSSSP_E_INVAL, "server_validate: bad arguments");
    std::lock_guard<std::mutex> d(s->dev);
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

}  // extern "C"
