// graph.cu -- device graph store (CSR with per-row slack), tree load/read, batch
// orchestration and the C ABI of include/dsssp.h.
//
// The graph store replaces the reference's host vector-of-vectors adjacency that is rebuilt
// and re-copied for every batch (all_structure_undir.cuh:178-198, SSSPmainForUndirected.cu:
// 42-91): rows live on the device, sorted by neighbour, each with free slots so insertions
// append in place.  A row that runs out of slots triggers a repack (rows re-sorted, tombstones
// dropped, slack restored) and the batch resumes after it.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include "../../include/dsssp.h"
#include "engine.cuh"
#include "host_common.h"

namespace dsssp {

cudaError_t launch_front(const UpdParams& p, int grid, cudaStream_t s, cudaEvent_t after_prepare,
                         cudaEvent_t after_delete);
cudaError_t update_occupancy(int block, int* blocks_per_sm);
cudaError_t launch_update(const UpdParams& p, int grid, int block, cudaStream_t s);
void batch_kernels(const void* fns[4]);
const void* update_kernel(bool warp_agg);
const void* delete_kernel(bool tails);

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---- build / repack kernels ------------------------------------------------------------

__global__ void k_check_edges(const int* u, const int* v, const int* w, long long m, int n, Ctl* ctl) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    if (u[i] < 0 || u[i] >= n || v[i] < 0 || v[i] >= n) set_status(ctl, DSSSP_E_BAD_VERTEX);
    else if (w[i] < 0) set_status(ctl, DSSSP_E_BAD_WEIGHT);
}

__global__ void k_degree(const int* u, const int* v, long long m, int* deg) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    atomicAdd(&deg[u[i]], 1);
    atomicAdd(&deg[v[i]], 1);
}

// cap = deg + max(slack_min, deg * slack_pct / 100)
__global__ void k_caps(const long long* deg, int n, int slack_pct, int slack_min, long long* cap) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const long long d = deg[v];
    long long s = d * slack_pct / 100;
    if (s < slack_min) s = slack_min;
    cap[v] = d + s;
}

__device__ __forceinline__ unsigned long long make_key(int col, int wt) {
    return ((unsigned long long)(unsigned)col << 32) | (unsigned)wt;
}

__global__ void k_scatter_packed(const int* u, const int* v, const int* w, long long m, const long long* poff,
                                 int* cursor, unsigned long long* keys) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int a = u[i], b = v[i];
    keys[poff[a] + atomicAdd(&cursor[a], 1)] = make_key(b, w[i]);
    keys[poff[b] + atomicAdd(&cursor[b], 1)] = make_key(a, w[i]);
}

// First index in keys[lo, hi) that is >= key.
__device__ __forceinline__ long long lower_key(const unsigned long long* keys, long long lo, long long hi,
                                               unsigned long long key) {
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (keys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Packed (contiguous) sorted rows -> slack layout.  Thread per entry.
// With twin != nullptr also the slot of the reverse entry: the i-th copy of (c, w) in row r
// pairs with the i-th copy of (r, w) in row c.
// row[e] = the row of entry e (sorted alongside the keys).
__global__ void k_spread(const unsigned long long* keys, const unsigned* row, const long long* poff,
                         const long long* start, long long total, int2* adj, unsigned* twin) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int lo = (int)row[e];
    const unsigned long long k = keys[e];
    const long long slot = start[lo] + (e - poff[lo]);
    const int c = (int)(k >> 32), w = (int)(unsigned)k;
    adj[slot] = make_int2(c, w);
    if (twin) {
        const long long rank = e - lower_key(keys, poff[lo], poff[lo + 1], k);
        const unsigned long long rk = ((unsigned long long)(unsigned)lo << 32) | (unsigned)w;
        const long long pos = lower_key(keys, poff[c], poff[c + 1], rk);
        twin[slot] = (unsigned)(start[c] + (pos - poff[c]) + rank);
    }
}

// Row id of every packed entry: warp per row r fills its segment [poff[r], poff[r+1]).
__global__ void k_row_ids(const long long* poff, int n, unsigned* ids) {
    const unsigned lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps)
        for (long long e = poff[r] + lane; e < poff[r + 1]; e += 32) ids[e] = (unsigned)r;
}

__global__ void k_rows_init(const long long* start, const long long* deg, const long long* cap, int n,
                            RowDesc* rows, int* sorted_len) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    RowDesc r;
    r.start = start[v];
    r.deg = (int)deg[v];
    r.cap = (int)cap[v];
    rows[v] = r;
    sorted_len[v] = (int)deg[v];
}

// live entries of each row (warp per row); an overflowed row holds cap entries
__global__ void k_count_live(const RowDesc* rows, const int2* adj, int n, int* live) {
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (gw >= n) return;
    const RowDesc r = rows[gw];
    const int len = r.deg < r.cap ? r.deg : r.cap;
    int c = 0;
    for (int j = (int)lane; j < len; j += 32) c += adj[r.start + j].y >= 0;
    c = __reduce_add_sync(0xFFFFFFFFu, (unsigned)c);
    if (lane == 0) live[gw] = c;
}

__global__ void k_ovf_count(const int4* ovf, int novf, int* live) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < novf) atomicAdd(&live[ovf[i].x], 1);
}

__global__ void k_pack_live(const RowDesc* rows, const int2* adj, int n, const long long* poff, int* cursor,
                            unsigned long long* keys) {
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (gw >= n) return;
    const RowDesc r = rows[gw];
    const int len = r.deg < r.cap ? r.deg : r.cap;
    int out = 0;
    for (int b = 0; b < len; b += 32) {
        const int j = b + (int)lane;
        int2 e = make_int2(0, -1);
        if (j < len) e = adj[r.start + j];
        const bool keep = e.y >= 0;
        const unsigned mask = __ballot_sync(0xFFFFFFFFu, keep);
        if (keep) keys[poff[gw] + out + __popc(mask & ((1u << lane) - 1u))] = make_key(e.x, e.y);
        out += __popc(mask);
    }
    if (lane == 0) cursor[gw] = out;
}

__global__ void k_pack_ovf(const int4* ovf, int novf, const long long* poff, int* cursor, unsigned long long* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= novf) return;
    const int4 o = ovf[i];
    keys[poff[o.x] + atomicAdd(&cursor[o.x], 1)] = make_key(o.y, o.z);
}

// ---- row growth: rows that ran out of slack are compacted in place or move to the spare region ----

struct GrowParams {
    RowDesc* rows;
    int2* adj;
    unsigned* twin;
    const int4* ovf;
    int novf;
    const int4* chg;
    long long k;
    const int* ins_state;
    long long* slot;
    int* need;                 // per vertex: overflowed entries of its row (0 = row not growing)
    int* gidx;                 // per vertex: 1 + index in the grow list (0 = not growing)
    unsigned* grow_list;       // rows that grow
    unsigned* grow_count;
    long long* old_start;      // per grow-list entry
    int* old_cap;
    unsigned long long* spare; // {top, end} of the spare region (bump allocator)
    int* fail;
    int slack_min;
    long long cap_total;
    // compacting growth (with the twin index)
    int* sorted_len;
    long long* new_start;             // per grow-list entry: the row's first slot after growth
    long long* scratch;               // per grow-list entry: scratch of a row compacted in place, -1: moves
    int* live;                        // per grow-list entry: live entries (tombstones are dropped)
    int* live_sorted;                 // ... of them in the neighbour-sorted prefix
    int* ncap;                        // per grow-list entry: capacity after growth
    unsigned long long* scr_used;     // scratch slots taken from the free end of the spare region
    unsigned long long* dropped;      // tombstones dropped
};

__global__ void k_grow_count(GrowParams q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.novf) return;
    const int r = q.ovf[i].x;
    if (atomicAdd(&q.need[r], 1) == 0) {
        const unsigned j = atomicAdd(q.grow_count, 1u);
        q.grow_list[j] = (unsigned)r;
        q.gidx[r] = (int)j + 1;
    }
}

// Without the twin index (slot counts above 32 bits): warp per growing row, a region of
// 2 * (cap + need) + slack_min slots from the spare region, the row's cap stored entries
// (tombstones included) copied there.
__global__ void k_grow_move(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count) return;
    const unsigned r = q.grow_list[j];
    const RowDesc rd = q.rows[r];
    const long long ncap = 2LL * (rd.cap + q.need[r]) + q.slack_min;
    unsigned long long pos = 0;
    if (lane == 0) pos = atomicAdd(&q.spare[0], (unsigned long long)ncap);
    pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
    if (pos + (unsigned long long)ncap > q.spare[1] || ncap > 0x7FFFFFFFLL) {
        if (lane == 0) atomicExch(q.fail, 1);
        return;
    }
    for (int e = (int)lane; e < rd.cap; e += 32) {
        q.adj[pos + e] = q.adj[rd.start + e];
        if (q.twin) q.twin[pos + e] = q.twin[rd.start + e];
    }
    if (lane == 0) {
        q.old_start[j] = rd.start;
        q.old_cap[j] = rd.cap;
        RowDesc nr;
        nr.start = (long long)pos;
        nr.deg = rd.cap;  // the entries actually stored; overflowed ones are placed next
        nr.cap = (int)ncap;
        q.rows[r] = nr;
    }
}

// Warp per grown row: every live entry re-links with its reverse entry, wherever either moved.
// Each moved entry reads only its own twin word, which no other thread writes.
__global__ void k_grow_fix(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count || !q.twin) return;
    const unsigned r = q.grow_list[j];
    const long long ns = q.rows[r].start;
    for (int e = (int)lane; e < q.old_cap[j]; e += 32) {
        const long long at = ns + e;
        const int2 x = q.adj[at];
        const unsigned t = q.twin[at];
        if (x.y < 0 || t == kNoTwin) continue;
        const int c = x.x;  // the reverse entry lives in row c
        const int gc = q.gidx[c];
        // A moved partner re-links itself from its own (old) twin word, so only our own word
        // is written for it; a partner that stayed gets our new slot.
        const long long t2 = gc ? q.rows[c].start + ((long long)t - q.old_start[gc - 1]) : (long long)t;
        if (t2 < 0 || t2 >= q.cap_total) {  // internal error: report, skip the access
            atomicExch(q.fail, 2);
            continue;
        }
        q.twin[at] = (unsigned)t2;
        if (!gc) q.twin[t2] = (unsigned)at;
    }
}

// Places the overflowed ends of every surviving insertion into its grown row and pairs twins.
__global__ void k_grow_place(GrowParams q) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.k) return;
    const int4 c = q.chg[i];
    if (c.w != 1 || q.ins_state[i] != 1) return;
    long long at[2] = {q.slot[2 * i], q.slot[2 * i + 1]};
    if (at[0] >= 0 && at[1] >= 0) return;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        if (at[side] >= 0) {
            // the end that fitted may sit in a row that moved in this growth step
            const int r = side ? c.y : c.x;
            const int gr = q.gidx[r];
            if (gr) at[side] = q.rows[r].start + (at[side] - q.old_start[gr - 1]);
            continue;
        }
        const int r = side ? c.y : c.x, col = side ? c.x : c.y;
        const int pos = atomicAdd(&q.rows[r].deg, 1);
        at[side] = q.rows[r].start + pos;
        q.adj[at[side]] = make_int2(col, c.z);
        q.slot[2 * i + side] = at[side];
    }
    if (q.twin) {
        q.twin[at[0]] = (unsigned)at[1];
        q.twin[at[1]] = (unsigned)at[0];
    }
}

__global__ void k_grow_reset(GrowParams q) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= *q.grow_count) return;
    const unsigned r = q.grow_list[j];
    q.need[r] = 0;
    q.gidx[r] = 0;
}

// ---- compacting growth (twin index): a growing row keeps only its live entries, in their
// order (the sorted prefix stays sorted).  A row whose live entries and overflow fit its own
// region with room to spare is compacted in place (through scratch slots at the free end of the
// spare region, so it uses none of that region); the others move to a region of
// 2 * (live + need) + slack_min slots.  Every moved live entry leaves its final slot in its old
// twin word (a forwarding pointer), through which the twins and the batch's recorded slots are
// re-linked.  Warp per growing row unless noted.

__global__ void k_grow_plan(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count) return;
    const unsigned r = q.grow_list[j];
    const RowDesc rd = q.rows[r];
    const int sl = q.sorted_len[r];
    int live = 0, ls = 0;
    for (int e = (int)lane; e < rd.cap; e += 32) {
        const bool l = q.adj[rd.start + e].y >= 0;
        live += l ? 1 : 0;
        ls += l && e < sl ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        live += __shfl_xor_sync(0xFFFFFFFFu, live, o);
        ls += __shfl_xor_sync(0xFFFFFFFFu, ls, o);
    }
    if (lane != 0) return;
    const long long need = q.need[r];
    const long long room = live / 8 > 1 ? live / 8 : 1;  // free slots left after an in-place compaction
    q.live[j] = live;
    q.live_sorted[j] = ls;
    atomicAdd(q.dropped, (unsigned long long)(rd.cap - live));
    if (live + need + room <= rd.cap) {
        const unsigned long long at = atomicAdd(q.scr_used, (unsigned long long)live);
        q.new_start[j] = rd.start;
        q.scratch[j] = (long long)(q.spare[1] - at - (unsigned long long)live);  // checked on the host
        q.ncap[j] = rd.cap;
    } else {
        const long long nc = 2 * (live + need) + q.slack_min;
        const unsigned long long pos = atomicAdd(&q.spare[0], (unsigned long long)nc);
        if (pos + (unsigned long long)nc > q.spare[1] || nc > 0x7FFFFFFFLL) atomicExch(q.fail, 1);
        q.new_start[j] = (long long)pos;
        q.scratch[j] = -1;
        q.ncap[j] = (int)(nc > 0x7FFFFFFFLL ? 0x7FFFFFFFLL : nc);
    }
    q.old_start[j] = rd.start;
    q.old_cap[j] = rd.cap;
}

__global__ void k_grow_out(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count) return;
    const long long os = q.old_start[j], fin = q.new_start[j];
    const long long dst = q.scratch[j] >= 0 ? q.scratch[j] : fin;
    const int cap = q.old_cap[j];
    int idx = 0;
    for (int b = 0; b < cap; b += 32) {
        const int e = b + (int)lane;
        const int2 x = e < cap ? q.adj[os + e] : make_int2(0, -1);
        const bool l = x.y >= 0;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, l);
        const int at = idx + __popc(m & ((1u << lane) - 1u));
        if (l) {
            q.adj[dst + at] = x;
            q.twin[dst + at] = q.twin[os + e];  // the partner's old slot, re-linked below
            q.twin[os + e] = (unsigned)(fin + at);
        }
        idx += __popc(m);
    }
}

// Each compacted entry takes its partner's final slot: from the partner's forwarding pointer
// when the partner's row grows too, else the partner stays and gets this entry's final slot.
__global__ void k_grow_relink(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count) return;
    const long long fin = q.new_start[j];
    const long long at0 = q.scratch[j] >= 0 ? q.scratch[j] : fin;
    const int live = q.live[j];
    for (int e = (int)lane; e < live; e += 32) {
        const unsigned t = q.twin[at0 + e];
        if (t == kNoTwin) continue;
        const int c = q.adj[at0 + e].x;  // the partner lives in row c
        if ((long long)t >= q.cap_total) {  // internal error: report, skip the access
            atomicExch(q.fail, 2);
            continue;
        }
        unsigned t2 = t;
        if (q.gidx[c]) t2 = q.twin[t];
        else q.twin[t] = (unsigned)(fin + e);
        if ((long long)t2 >= q.cap_total) {
            atomicExch(q.fail, 2);
            continue;
        }
        q.twin[at0 + e] = t2;
    }
}

// Thread per record: the recorded slot of an inserted end that fitted into a growing row.
__global__ void k_grow_translate(GrowParams q) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.k) return;
    const int4 c = q.chg[i];
    if (c.w != 1 || q.ins_state[i] != 1) return;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const long long at = q.slot[2 * i + side];
        const int r = side ? c.y : c.x;
        if (at >= 0 && q.gidx[r]) q.slot[2 * i + side] = (long long)q.twin[at];
    }
}

__global__ void k_grow_back(GrowParams q) {
    const unsigned j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (j >= *q.grow_count) return;
    const long long fin = q.new_start[j], scr = q.scratch[j];
    const int live = q.live[j];
    if (scr >= 0)
        for (int e = (int)lane; e < live; e += 32) {
            q.adj[fin + e] = q.adj[scr + e];
            q.twin[fin + e] = q.twin[scr + e];
        }
    if (lane == 0) {
        const unsigned r = q.grow_list[j];
        RowDesc nr;
        nr.start = fin;
        nr.deg = live;
        nr.cap = q.ncap[j];
        q.rows[r] = nr;
        q.sorted_len[r] = q.live_sorted[j];
    }
}

// Thread per record: the overflowed ends go after the live entries of their grown rows, and
// every surviving insertion's two ends are paired.
__global__ void k_grow_place2(GrowParams q) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.k) return;
    const int4 c = q.chg[i];
    if (c.w != 1 || q.ins_state[i] != 1) return;
    long long at[2] = {q.slot[2 * i], q.slot[2 * i + 1]};
    if (at[0] >= 0 && at[1] >= 0) return;  // paired by the batch (and re-linked if moved)
#pragma unroll
    for (int side = 0; side < 2; side++) {
        if (at[side] >= 0) continue;
        const int r = side ? c.y : c.x, col = side ? c.x : c.y;
        const int pos = atomicAdd(&q.rows[r].deg, 1);
        if (pos >= q.rows[r].cap) {  // cannot happen: growth sized the row for its overflow
            atomicExch(q.fail, 3);
            return;
        }
        at[side] = q.rows[r].start + pos;
        q.adj[at[side]] = make_int2(col, c.z);
        q.slot[2 * i + side] = at[side];
    }
    q.twin[at[0]] = (unsigned)at[1];
    q.twin[at[1]] = (unsigned)at[0];
}

__global__ void k_int_to_ll(const int* a, int n, long long* b) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) b[v] = a[v];
}

// ---- tree kernels --------------------------------------------------------------------------

// parent -1 -> unreachable; otherwise parent in range and 0 <= dist < 2^32-1; the root is the
// single vertex with parent[v] == v and it must have dist 0.
__global__ void k_tree_pack(const int* parent, const long long* dist, int n, unsigned long long* state, Ctl* ctl) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int p = parent[v];
    if (p == -1) {
        state[v] = kInfState;
        return;
    }
    if (p < 0 || p >= n) {
        set_status(ctl, DSSSP_E_BAD_TREE);
        state[v] = kInfState;
        return;
    }
    const long long d = dist[v];
    if (d < 0 || d >= (long long)kDistInf) {
        set_status(ctl, d < 0 ? DSSSP_E_BAD_TREE : DSSSP_E_OVERFLOW);
        state[v] = kInfState;
        return;
    }
    if (p == v) {
        atomicAdd(&ctl->stat[0], 1ull);             // number of roots
        atomicMin(&ctl->stat[1], (unsigned long long)v);  // root id
        if (d != 0) set_status(ctl, DSSSP_E_BAD_TREE);
    }
    state[v] = ((unsigned long long)d << 32) | (unsigned)p;
}

__global__ void k_tree_unpack(const unsigned long long* state, int n, int* parent, long long* dist) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const unsigned long long s = state[v];
    if (s == kInfState) {
        if (parent) parent[v] = -1;
        if (dist) dist[v] = DSSSP_UNREACHABLE;
    } else {
        if (parent) parent[v] = (int)(unsigned)s;
        if (dist) dist[v] = (long long)(s >> 32);
    }
}

// The same with 32-bit distances (0xFFFFFFFF = unreachable, which is the state's own top half).
__global__ void k_tree_unpack32(const unsigned long long* state, int n, int* parent, unsigned* dist) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const unsigned long long s = state[v];
    if (parent) parent[v] = s == kInfState ? -1 : (int)(unsigned)s;
    if (dist) dist[v] = (unsigned)(s >> 32);
}

// Vertices the last batch may have changed: cut off in this epoch, or holding a push tag or
// far-list generation of the batch's tag range [lo, hi).  CTA-aggregated append.
__global__ void k_tree_changed(const unsigned long long* state, const unsigned* inv_tag, const unsigned* chg_tag,
                               const unsigned* push_tag, const unsigned* far_tag, int n, unsigned epoch, unsigned lo,
                               unsigned hi, int* vertex, int* parent, long long* dist, unsigned* count) {
    __shared__ unsigned s_n, s_base;
    __shared__ int s_v[kThreads];
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    bool ch = false;
    if (v < n) {
        const unsigned pt = push_tag[v];
        ch = inv_tag[v] == epoch || chg_tag[v] == epoch || (pt >= lo && pt < hi);
        if (!ch && far_tag) {
            const unsigned ft = far_tag[v];
            ch = ft >= lo && ft < hi;
        }
    }
    if (ch) s_v[atomicAdd(&s_n, 1u)] = v;
    __syncthreads();
    if (threadIdx.x == 0 && s_n) s_base = atomicAdd(count, s_n);
    __syncthreads();
    if (threadIdx.x < s_n) {
        const int x = s_v[threadIdx.x];
        const unsigned long long s = state[x];
        const unsigned i = s_base + threadIdx.x;
        vertex[i] = x;
        parent[i] = s == kInfState ? -1 : (int)(unsigned)s;
        dist[i] = s == kInfState ? (long long)DSSSP_UNREACHABLE : (long long)(s >> 32);
    }
}

// ---- certificate of the resident tree (dsssp_tree_validate) -------------------------------
// A warp per vertex v checks v's live adjacency entries: no entry (u, w) offers a shorter
// distance (dist[u] + w < dist[v], an unreachable v included), a reachable non-root v has a
// live entry to its parent p with dist[p] + w == dist[v], and a root (its own parent) has
// distance 0.  out[0] counts violations, out[1] roots, out[2] the least violating vertex.
// Checks of one row's entries (a range of them): a shorter distance on offer (bad), the tight
// live parent edge (tight).
__device__ __forceinline__ void validate_entries(const unsigned long long* state, const int2* adj, long long lo,
                                                 long long hi, long long step, bool reach, unsigned long long dv,
                                                 unsigned pv, bool& bad, bool& tight) {
    for (long long i = lo; i < hi; i += step) {
        const int2 e = adj[i];
        if (e.y < 0) continue;
        const unsigned long long su = state[e.x];
        if (su == kInfState) continue;
        const unsigned long long du = su >> 32;
        if (du + (unsigned)e.y < dv) bad = true;  // a shorter distance is on offer
        if (reach && (unsigned)e.x == pv && du + (unsigned)e.y == dv) tight = true;
    }
}

// The verdict on vertex v once its row is checked (one thread).
__device__ __forceinline__ void validate_vertex(long long v, int n, bool reach, unsigned long long dv, unsigned pv,
                                                bool bad, bool tight, unsigned* jm, unsigned long long* out) {
    const bool root = reach && pv == (unsigned)v;
    if (reach && !root && (pv >= (unsigned)n || !tight)) bad = true;  // no tight live parent edge
    if (root && dv != 0) bad = true;
    if (root) atomicAdd(&out[1], 1ull);
    if (bad) {
        atomicAdd(&out[0], 1ull);
        atomicMin(&out[2], (unsigned long long)v);
    }
    // pointer-jumping word: terminal (kTagOk) at roots and unreachable vertices
    jm[v] = (!reach || root || pv >= (unsigned)n) ? kTagOk : pv;
}

constexpr int kValidateLongRow = 2048;  // rows above this are checked by a whole CTA

// Warp per row; rows above kValidateLongRow entries are listed (long, *nlong) for k_validate_long.
__global__ void k_validate_rows(const unsigned long long* state, const RowDesc* rows, const int2* adj, int n,
                                unsigned* jm, unsigned long long* out, unsigned* lng, unsigned* nlong) {
    const unsigned lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long v = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const RowDesc rd = rows[v];
        if (rd.deg > kValidateLongRow) {
            if (lane == 0) lng[atomicAdd(nlong, 1u)] = (unsigned)v;
            continue;
        }
        const unsigned long long sv = state[v];
        const bool reach = sv != kInfState;
        const unsigned long long dv = reach ? (sv >> 32) : (unsigned long long)kDistInf;
        const unsigned pv = (unsigned)sv;
        bool bad = false, tight = false;
        validate_entries(state, adj, rd.start + lane, rd.start + rd.deg, 32, reach, dv, pv, bad, tight);
        bad = __any_sync(0xFFFFFFFFu, bad);
        tight = __any_sync(0xFFFFFFFFu, tight);
        if (lane == 0) validate_vertex(v, n, reach, dv, pv, bad, tight, jm, out);
    }
}

// CTA per long row (hubs of up to millions of entries would keep one warp busy for ms).
__global__ void k_validate_long(const unsigned long long* state, const RowDesc* rows, const int2* adj, int n,
                                unsigned* jm, unsigned long long* out, const unsigned* lng, const unsigned* nlong) {
    const unsigned count = *nlong;
    for (unsigned i = blockIdx.x; i < count; i += gridDim.x) {
        const long long v = lng[i];
        const RowDesc rd = rows[v];
        const unsigned long long sv = state[v];
        const bool reach = sv != kInfState;
        const unsigned long long dv = reach ? (sv >> 32) : (unsigned long long)kDistInf;
        const unsigned pv = (unsigned)sv;
        bool bad = false, tight = false;
        validate_entries(state, adj, rd.start + threadIdx.x, rd.start + rd.deg, blockDim.x, reach, dv, pv, bad, tight);
        bad = __syncthreads_or(bad);
        tight = __syncthreads_or(tight);
        if (threadIdx.x == 0) validate_vertex(v, n, reach, dv, pv, bad, tight, jm, out);
    }
}

// One pointer-jumping pass: jm[v] <- jm[jm[v]] until it is terminal.
__global__ void k_validate_jump(unsigned* jm, int n) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const unsigned j = jm[v];
        if (j < kTagInv) jm[v] = jm[j];
    }
}

// Vertices whose parent chain is still not terminal after 32 doublings lie on a cycle.
__global__ void k_validate_cycles(const unsigned* jm, int n, unsigned long long* out) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        if (jm[v] < kTagInv) {
            atomicAdd(&out[0], 1ull);
            atomicMin(&out[2], (unsigned long long)v);
        }
    }
}

// Rows [first, first + count): live entries whose column lies outside the range (out[0]).
__global__ void k_range_crossing(const RowDesc* rows, const int2* adj, int first, int count,
                                 unsigned long long* out) {
    const unsigned lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    unsigned long long cross = 0;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < count; i += warps) {
        const RowDesc rd = rows[first + i];
        for (int j = (int)lane; j < rd.deg; j += 32) {
            const int2 e = adj[rd.start + j];
            if (e.y >= 0 && (e.x < first || (long long)e.x >= (long long)first + count)) cross++;
        }
    }
    if (cross) atomicAdd(&out[0], cross);
}

// Tombstones every live entry of rows [first, first + count) -- both directions of each edge
// lie in the range -- and makes the range's vertices unreachable.  out[1] counts the entries.
__global__ void k_range_clear(unsigned long long* state, const RowDesc* rows, int2* adj, int first, int count,
                              unsigned long long* out) {
    const unsigned lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    unsigned long long dead = 0;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < count; i += warps) {
        const RowDesc rd = rows[first + i];
        for (int j = (int)lane; j < rd.deg; j += 32) {
            int2* e = &adj[rd.start + j];
            if (e->y >= 0) {
                e->y = -1;
                dead++;
            }
        }
        if (lane == 0) state[first + i] = kInfState;
    }
    if (dead) atomicAdd(&out[1], dead);
}

__global__ void k_state_reset(unsigned long long* state, int n) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) state[v] = kInfState;
}

// Sources: distance 0, own parent.  Ids are checked; a bad one sets DSSSP_E_BAD_VERTEX.
__global__ void k_set_sources(unsigned long long* state, int n, const int* srcs, int k, Ctl* ctl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k) return;
    const int s = srcs[i];
    if (s < 0 || s >= n) set_status(ctl, DSSSP_E_BAD_VERTEX);
    else state[s] = (unsigned long long)(unsigned)s;
}

// ---- host helpers --------------------------------------------------------------------------

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(DSSSP_E_OOM, "%s: out of device memory", what);
    }
    return fail(DSSSP_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

template <class T>
int dalloc(T** p, size_t count, const char* what) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, what);
    }
    return DSSSP_OK;
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

}  // namespace
}  // namespace dsssp

using namespace dsssp;

struct dsssp_graph {
    int dev = 0;
    int n = 0;
    int src = -1;
    int num_sms = 0;
    dsssp_opts o{};
    cudaStream_t stream = nullptr;
    long long cap_total = 0;
    double mean_w = 1.0;       // mean edge weight (automatic near-far width)
    long long last_rounds = 0; // relaxation rounds of the last batch or tree computation
    long long entries = 0;     // live adjacency entries
    long long dead = 0;        // tombstoned entries since the last layout
    long long spare_lo = 0;    // first slot of the spare region
    long long spare_top = 0;   // its bump pointer as of the last row growth
    DevGraph dg{};
    // batch buffers
    int4* d_chg = nullptr;
    long long chg_cap = 0;
    int* d_ins_state = nullptr;
    int4* d_ovf = nullptr;
    long long* d_slot = nullptr;        // per record: slots of both appended ends
    unsigned* d_seedq = nullptr;        // vertices seeded by the insertions of a batch
    // in-place row growth
    unsigned long long* d_spare = nullptr;  // {top, end} of the spare region
    int* d_need = nullptr;
    int* d_gidx = nullptr;
    unsigned* d_grow_list = nullptr;
    unsigned* d_grow_count = nullptr;
    long long* d_old_start = nullptr;
    int* d_old_cap = nullptr;
    long long* d_gnew = nullptr;            // per grow-list entry: first slot after growth
    long long* d_gscr = nullptr;            // per grow-list entry: scratch of an in-place compaction
    int* d_glive = nullptr;                 // per grow-list entry: live entries, of them sorted, capacity
    int* d_gsorted = nullptr;
    int* d_gncap = nullptr;
    unsigned long long* d_gwords = nullptr; // scratch slots used, tombstones dropped
    long long grow_dropped = 0;             // tombstones the last row growth dropped
    int* d_fail = nullptr;
    long long grow_cap = 0;
    unsigned long long s_spare[2] = {0, 0};  // spare words saved with the snapshot
    long long s_spare_lo = 0;                // and the first slot of its spare region
    DelSlot* d_hset = nullptr;  // deletion set of the batch
    unsigned long long hcap = 0;
    Ctl* h_ctl = nullptr;  // pinned mirror of the control block
    // batch timing: 0 start, 1 before k_update, 2 end, 3 spare, 4 after k_prepare, 5 after k_delete
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    unsigned epoch = 0;
    int coop_grid = 0;
    // the batch launch sequence as an instantiated CUDA graph (opts.launch_graph)
    cudaGraph_t bgraph = nullptr;
    cudaGraphExec_t bexec = nullptr;
    cudaGraphNode_t bn_hash = nullptr, bn_kern[4] = {nullptr, nullptr, nullptr, nullptr};
    int bgraph_timing = 0;  // the timing level the instantiated graph records
    int bgraph_agg = 0;     // the update kernel it launches (opts.warp_agg)
    int bgraph_tails = 0;   // the deletion kernel it launches (tails)
    // rows may hold unsorted tails: set by a batch that appends, cleared by a fresh layout
    bool tails = false;
    bool s_tails = false;   // ... as of the snapshot
    bool bgraph_failed = false;
    // pending batch
    bool pending = false;
    long long pend_k = 0;
    const int4* pend_chg = nullptr;
    cudaStream_t pend_stream = nullptr;
    bool pend_events = false;
    bool pend_graph = false;
    // tag range of the last successful batch (tree_read_changed); delta_ok false after a
    // tree load or computation, a failed batch or a tag reset
    unsigned delta_lo = 0, delta_hi = 0, delta_epoch = 0;
    bool delta_ok = false;
    bool delta_empty = false;  // the last batch had no records: nothing changed
    unsigned pend_rb0 = 0;
    int* d_vtx = nullptr;
    unsigned* d_count = nullptr;
    // tree staging
    int* d_par = nullptr;
    long long* d_dist = nullptr;
    // asynchronous tree reads: their own staging, copied to the host on a copy stream
    int* a_par = nullptr;
    unsigned* a_dist = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_unpacked = nullptr;  // the staging holds the tree (later batches may start)
    cudaEvent_t ev_copied = nullptr;    // the host arrays hold it (the staging is free again)
    bool copy_pending = false;
    // snapshot
    unsigned long long* s_state = nullptr;
    RowDesc* s_rows = nullptr;
    int* s_sorted = nullptr;
    int2* s_adj = nullptr;
    unsigned* s_twin = nullptr;
    long long s_cap = 0;
    long long s_entries = 0;
    long long s_dead = 0;
    int s_src = -1;
    bool has_snap = false;
    bool has_tree = false;
    bool s_has_tree = false;
    int* d_srcs = nullptr;  // sources of the last from-scratch computation
    int srcs_cap = 0;
    // the roots of the resident forest (vertices that are their own parent), kept on the host
    // so that a failed batch can be recovered by recomputing the trees from them
    std::vector<int> roots;
    std::vector<int> s_roots;  // with the snapshot
};

namespace dsssp {
namespace {

int set_device(const dsssp_graph* g) {
    cudaError_t e = cudaSetDevice(g->dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return DSSSP_OK;
}

// Work-list capacities.  A vertex enters a given list at most once per step (push tags,
// cut-off tags), so a list holds at most sum_v ceil(deg_v / te) thread items and
// sum over rows above large_deg of ceil(deg_v / chunk) CTA items.
long long thread_item_capacity(long long cap_total, long long n, const dsssp_opts& o) {
    return cap_total / o.small_deg + n + 64;
}

long long cta_item_capacity(long long cap_total, const dsssp_opts& o) {
    return cap_total / o.chunk + cap_total / (o.large_deg > 0 ? o.large_deg : 1) + 64;
}

// Near-far lists: one entry per vertex at most; allocated when near-far rounds first run.
int ensure_far(dsssp_graph* g) {
    DevGraph& d = g->dg;
    if (d.far_tag) return DSSSP_OK;
    int rc = dalloc(&d.far0, (size_t)g->n, "far list");
    if (!rc) rc = dalloc(&d.far1, (size_t)g->n, "far list");
    if (!rc) rc = dalloc(&d.far_tag, (size_t)g->n, "far tags");
    if (rc) {
        dfree(d.far0); dfree(d.far1); dfree(d.far_tag);
        return rc;
    }
    CK(cudaMemsetAsync(d.far_tag, 0, sizeof(unsigned) * (size_t)g->n, g->stream), "far tags");
    return DSSSP_OK;
}

// Near-far bucket width of the next batch or tree computation.  delta > 0 is used as given;
// delta < 0 (automatic) turns near-far rounds on with 32 times the mean edge weight once the
// last batch or tree computation needed more than opts.auto_rounds rounds (a high-diameter graph);
// 0 keeps plain rounds.
unsigned long long effective_delta(const dsssp_graph* g) {
    if (g->o.delta > 0) return (unsigned long long)g->o.delta;
    if (g->o.delta < 0 && g->last_rounds > (long long)g->o.auto_rounds) {
        // wide buckets: a round costs a dependent chain and a grid barrier whatever its size,
        // so fewer rounds beat fewer relaxations (the 4096^2 grid: 103 ms at 8x, 87 ms at 32x,
        // 83 ms at 64-96x with 4-6x the relaxations)
        const double d = 32.0 * g->mean_w;
        return d < 1.0 ? 1ull : (unsigned long long)(d + 0.5);
    }
    return 0;
}

int ensure_work(dsssp_graph* g) {
    const long long nt = thread_item_capacity(g->cap_total, g->n, g->o);
    const long long nc = cta_item_capacity(g->cap_total, g->o);
    DevGraph& d = g->dg;
    if (g->o.delta > 0) {
        const int rc = ensure_far(g);
        if (rc) return rc;
    }
    if (d.tcap >= nt && d.ccap >= nc && d.rt0) return DSSSP_OK;
    dfree(d.rt0); dfree(d.rt1); dfree(d.rc0); dfree(d.rc1); dfree(d.it); dfree(d.ic);
    d.tcap = d.ccap = 0;
    int rc = dalloc(&d.rt0, (size_t)nt, "work list");
    if (!rc) rc = dalloc(&d.rt1, (size_t)nt, "work list");
    if (!rc) rc = dalloc(&d.it, (size_t)nt, "work list");
    if (!rc) rc = dalloc(&d.rc0, (size_t)nc, "work list");
    if (!rc) rc = dalloc(&d.rc1, (size_t)nc, "work list");
    if (!rc) rc = dalloc(&d.ic, (size_t)nc, "work list");
    if (!rc) {
        d.tcap = nt;
        d.ccap = nc;
    }
    return rc;
}

int ensure_batch(dsssp_graph* g, long long k) {
    if (k <= g->chg_cap) return DSSSP_OK;
    long long cap = k + k / 4 + 1024;
    unsigned long long h = 64;
    while (h < 2ull * (unsigned long long)cap) h <<= 1;
    dfree(g->d_chg);
    dfree(g->d_ins_state);
    dfree(g->d_ovf);
    dfree(g->d_hset);
    dfree(g->d_slot);
    dfree(g->d_seedq);
    dfree(g->d_grow_list);
    dfree(g->d_old_start);
    dfree(g->d_old_cap);
    dfree(g->d_gnew); dfree(g->d_gscr); dfree(g->d_glive); dfree(g->d_gsorted); dfree(g->d_gncap);
    g->grow_cap = 0;
    g->chg_cap = 0;
    g->hcap = 0;
    int rc = dalloc(&g->d_chg, (size_t)cap, "change buffer");
    if (!rc) rc = dalloc(&g->d_ins_state, (size_t)cap, "insertion state");
    if (!rc) rc = dalloc(&g->d_ovf, (size_t)cap * 2, "overflow buffer");
    if (!rc) rc = dalloc(&g->d_hset, (size_t)h, "deletion set");
    if (!rc) rc = dalloc(&g->d_slot, (size_t)cap * 2, "slot buffer");
    const long long gl = 2 * cap < g->n ? 2 * cap : g->n;
    if (!rc) rc = dalloc(&g->d_grow_list, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_seedq, (size_t)gl, "seed list");
    if (!rc) rc = dalloc(&g->d_old_start, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_old_cap, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_gnew, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_gscr, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_glive, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_gsorted, (size_t)gl, "grow list");
    if (!rc) rc = dalloc(&g->d_gncap, (size_t)gl, "grow list");
    if (!rc && !g->d_gwords) rc = dalloc(&g->d_gwords, 2, "grow list");
    if (!rc) g->grow_cap = gl;
    if (!rc) {
        g->chg_cap = cap;
        g->hcap = h;
    }
    return rc;
}

// deg (int, n) -> deg64 (n+1, last 0) and poff = exclusive scan (n+1, last = total)
int row_offsets(dsssp_graph* g, const int* d_deg, long long** deg64, long long** poff, cudaStream_t s) {
    const int n = g->n;
    *deg64 = nullptr;
    *poff = nullptr;
    int rc = dalloc(deg64, (size_t)n + 1, "row degrees");
    if (!rc) rc = dalloc(poff, (size_t)n + 1, "row offsets");
    if (rc) return rc;
    CK(cudaMemsetAsync(*deg64 + n, 0, sizeof(long long), s), "memset");
    if (n > 0) {
        k_int_to_ll<<<blocks_for(n), kThreads, 0, s>>>(d_deg, n, *deg64);
        count_launch(1);
    }
    size_t tb = 0;
    CK(cub::DeviceScan::ExclusiveSum(nullptr, tb, *deg64, *poff, n + 1, s), "scan");
    void* tmp = nullptr;
    CK(cudaMalloc(&tmp, tb ? tb : 1), "scan scratch");
    cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, tb, *deg64, *poff, n + 1, s);
    cudaFree(tmp);
    CK(e, "scan");
    return DSSSP_OK;
}

// Packed rows (keys at poff, row v holding deg64[v] keys) -> sorted rows in a fresh
// slack-layout adjacency; replaces g's adjacency, rows and sorted prefix lengths.
int layout_rows(dsssp_graph* g, unsigned long long* keys_in, long long total, const long long* deg64,
                const long long* poff, cudaStream_t s) {
    g->tails = false;  // every row is sorted: no tails until a batch appends
    const int n = g->n;
    long long *cap = nullptr, *start = nullptr;
    unsigned long long* keys_out = nullptr;
    unsigned *ids_a = nullptr, *ids_b = nullptr;
    const unsigned long long* keys_sorted = keys_in;
    const unsigned* rows_sorted = ids_a;
    void* tmp = nullptr;
    int2* adj = nullptr;
    long long cap_total = 0;
    int rc = dalloc(&cap, (size_t)n + 1, "row caps");
    if (!rc) rc = dalloc(&start, (size_t)n + 1, "row starts");
    if (!rc) rc = dalloc(&keys_out, (size_t)total, "sort buffer");
    if (!rc) rc = dalloc(&ids_a, (size_t)total, "sort buffer");
    if (!rc) rc = dalloc(&ids_b, (size_t)total, "sort buffer");
    if (!rc) {
        cudaError_t e = cudaMemsetAsync(cap + n, 0, sizeof(long long), s);
        if (n > 0 && e == cudaSuccess) {
            k_caps<<<blocks_for(n), kThreads, 0, s>>>(deg64, n, g->o.slack_pct, g->o.slack_min, cap);
            count_launch(1);
        }
        // Rows sorted by (neighbour, weight) with two stable radix sorts over all entries: by the
        // (col << 32 | wt) key carrying the row id, then by row id carrying the key, so no row is
        // sorted by one CTA alone (a segmented sort leaves hub rows of 10^5 entries to one block).
        int row_bits = 1;
        while (row_bits < 32 && (1ll << row_bits) < (long long)n) row_bits++;
        int key_bits = 32 + row_bits;  // column < n, weight < 2^31
        cub::DoubleBuffer<unsigned long long> dk(keys_in, keys_out);
        cub::DoubleBuffer<unsigned> dv(ids_a, ids_b);
        size_t tb1 = 0, tb2 = 0, tb3 = 0;
        if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, tb1, cap, start, n + 1, s);
        if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(nullptr, tb2, dk, dv, total, 0, key_bits, s);
        if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(nullptr, tb3, dv, dk, total, 0, row_bits, s);
        size_t tb = tb1 > tb2 ? tb1 : tb2;
        tb = tb > tb3 ? tb : tb3;
        if (e == cudaSuccess) e = cudaMalloc(&tmp, tb ? tb : 1);
        if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(tmp, tb1, cap, start, n + 1, s);
        if (e == cudaSuccess && total > 0) {
            k_row_ids<<<(unsigned)(((long long)n * 32 + kThreads - 1) / kThreads), kThreads, 0, s>>>(poff, n, ids_a);
            count_launch(1);
            e = cub::DeviceRadixSort::SortPairs(tmp, tb2, dk, dv, total, 0, key_bits, s);
            if (e == cudaSuccess) e = cub::DeviceRadixSort::SortPairs(tmp, tb3, dv, dk, total, 0, row_bits, s);
            keys_sorted = dk.Current();
            rows_sorted = dv.Current();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&cap_total, start + n, sizeof(long long), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "row layout");
    }
    // rows take [0, main); [main, cap_total) is the spare region that rows running out of
    // slack move into (bump allocator, reset by the next layout)
    const long long main_slots = cap_total;
    cap_total = main_slots + main_slots * g->o.spare_pct / 100 + 1024;
    const long long spare_lo = main_slots;
    if (!rc) {
        const unsigned long long sp[2] = {(unsigned long long)main_slots, (unsigned long long)cap_total};
        cudaError_t e = cudaMemcpyAsync(g->d_spare, sp, sizeof(sp), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "spare region");
    }
    unsigned* twin = nullptr;
    if (!rc) rc = dalloc(&adj, (size_t)cap_total, "adjacency");
    if (!rc && cap_total < 0xFFFFFFFFll) rc = dalloc(&twin, (size_t)cap_total, "twin index");
    if (!rc) {
        if (total > 0) {
            k_spread<<<blocks_for(total), kThreads, 0, s>>>(keys_sorted, rows_sorted, poff, start, total, adj, twin);
            count_launch(1);
        }
        if (n > 0) {
            k_rows_init<<<blocks_for(n), kThreads, 0, s>>>(start, deg64, cap, n, g->dg.rows, g->dg.sorted_len);
            count_launch(1);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "row layout");
    }
    if (!rc) {
        dfree(g->dg.adj);
        dfree(g->dg.twin);
        g->dg.adj = adj;
        g->dg.twin = twin;
        adj = nullptr;
        twin = nullptr;
        g->cap_total = cap_total;
        g->entries = total;
        g->dead = 0;
        g->spare_lo = spare_lo;
        g->spare_top = spare_lo;
        rc = ensure_work(g);
    }
    dfree(cap);
    dfree(start);
    dfree(keys_out);
    dfree(ids_a);
    dfree(ids_b);
    if (tmp) cudaFree(tmp);
    dfree(adj);
    dfree(twin);
    return rc;
}

// Drops tombstones, folds n_ovf overflow entries (row, col, wt) in, re-sorts every row and
// restores slack.
int repack(dsssp_graph* g, const int4* d_ovf, int n_ovf, cudaStream_t s) {
    const int n = g->n;
    int *live = nullptr, *cursor = nullptr;
    long long *deg64 = nullptr, *poff = nullptr;
    unsigned long long* keys = nullptr;
    long long total = 0;
    int rc = dalloc(&live, (size_t)n, "live counts");
    if (!rc) rc = dalloc(&cursor, (size_t)n, "row cursors");
    if (!rc && n > 0) {
        const unsigned wb = (unsigned)(((long long)n * 32 + kThreads - 1) / kThreads);
        k_count_live<<<wb, kThreads, 0, s>>>(g->dg.rows, g->dg.adj, n, live);
        count_launch(1);
        if (n_ovf > 0) {
            k_ovf_count<<<blocks_for(n_ovf), kThreads, 0, s>>>(d_ovf, n_ovf, live);
            count_launch(1);
        }
    }
    if (!rc) rc = row_offsets(g, live, &deg64, &poff, s);
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(&total, poff + n, sizeof(long long), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "repack");
    }
    if (!rc) rc = dalloc(&keys, (size_t)total, "repack keys");
    if (!rc && n > 0) {
        const unsigned wb = (unsigned)(((long long)n * 32 + kThreads - 1) / kThreads);
        k_pack_live<<<wb, kThreads, 0, s>>>(g->dg.rows, g->dg.adj, n, poff, cursor, keys);
        count_launch(1);
        if (n_ovf > 0) {
            k_pack_ovf<<<blocks_for(n_ovf), kThreads, 0, s>>>(d_ovf, n_ovf, poff, cursor, keys);
            count_launch(1);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "repack");
    }
    if (!rc) rc = layout_rows(g, keys, total, deg64, poff, s);
    dfree(live);
    dfree(cursor);
    dfree(deg64);
    dfree(poff);
    dfree(keys);
    return rc;
}

UpdParams make_params(const dsssp_graph* g, const int4* chg, long long k, int mode) {
    UpdParams p;
    p.g = g->dg;
    p.g.n = g->n;
    p.g.src = g->src;
    p.g.cap_total = g->cap_total;
    p.chg = chg;
    p.k = k;
    p.ins_state = g->d_ins_state;
    p.hset = g->d_hset;
    p.hmask = g->hcap ? g->hcap - 1 : 0;
    p.ovf = g->d_ovf;
    p.slot = g->d_slot;
    p.epoch = g->epoch;
    p.te = g->o.small_deg;
    p.large_deg = g->o.large_deg;
    p.chunk = g->o.chunk;
    p.bfs_levels = g->o.bfs_levels;
    p.mode = mode;
    p.delta = g->dg.far_tag ? effective_delta(g) : 0ull;  // the caller ensured the lists
    p.seedq = g->d_seedq;
    p.srcs = g->d_srcs;
    p.nsrc = 0;
    p.max_rounds = g->o.max_rounds > 0 ? g->o.max_rounds : 2LL * g->n + 16;
    p.solo_waves = (unsigned)g->o.solo_waves;
    p.group_ctas = (unsigned)g->o.group_ctas;
    p.group_waves = (unsigned)g->o.group_waves;
    p.warp_agg = g->o.warp_agg;
    p.tails = g->tails ? 1 : 0;
    return p;
}

int clear_ctl(dsssp_graph* g, cudaStream_t s) {
    const size_t off = offsetof(Ctl, status);  // line 1 onwards
    CK(cudaMemsetAsync((char*)g->dg.ctl + off, 0, sizeof(Ctl) - off, s), "control block reset");
    return DSSSP_OK;
}

int next_epoch(dsssp_graph* g, cudaStream_t s) {
    if (g->epoch >= 0xFFFFFFF0u) {
        CK(cudaMemsetAsync(g->dg.inv_tag, 0, sizeof(unsigned) * (size_t)g->n, s), "tag reset");
        CK(cudaMemsetAsync(g->dg.chg_tag, 0, sizeof(unsigned) * (size_t)g->n, s), "tag reset");
        g->epoch = 0;
    }
    g->epoch++;
    return DSSSP_OK;
}

// After a failed batch the device may not have advanced its round base: clear the frontier
// tags and restart the tag sequence so no stale tag can suppress a later push.
void reset_tags(dsssp_graph* g, cudaStream_t s) {
    cudaMemsetAsync(g->dg.push_tag, 0, sizeof(unsigned) * (size_t)g->n, s);
    if (g->dg.far_tag) cudaMemsetAsync(g->dg.far_tag, 0, sizeof(unsigned) * (size_t)g->n, s);
    const unsigned one = 1;
    cudaMemcpyAsync(&g->dg.ctl->round_base, &one, sizeof(one), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    g->h_ctl->round_base = 1;
}

int status_code(int st) {
    switch (st) {
        case 0: return DSSSP_OK;
        case DSSSP_E_BAD_VERTEX: return fail(st, "change batch names a vertex outside 0..n-1");
        case DSSSP_E_BAD_WEIGHT: return fail(st, "change batch inserts an edge with a negative weight");
        case DSSSP_E_NO_CONVERGENCE: return fail(st, "relaxation did not converge within the round cap");
        case DSSSP_E_TIMEOUT: return fail(st, "a device-side grid barrier timed out");  // detail set by caller
        case DSSSP_E_BAD_TREE: return fail(st, "the shortest-path tree has a parent cycle");
        case DSSSP_E_OVERFLOW: return fail(st, "a distance does not fit below 2^32-1");
        default: return fail(DSSSP_E_CUDA, "device status %d", st);
    }
}

void fill_stats(const dsssp_graph* g, const Ctl& c, dsssp_stats* st, bool events, long long k, int repacks) {
    if (!st) return;
    memset(st, 0, sizeof(*st));
    st->n_ins = (int64_t)c.stat[ST_INS];
    st->n_del = (int64_t)c.stat[ST_DEL];
    st->n_ignored = (int64_t)c.stat[ST_IGN];
    st->n_roots = (int64_t)c.stat[ST_ROOTS];
    st->n_invalidated = (int64_t)c.stat[ST_INV];
    st->inv_levels = (int64_t)c.stat[ST_LEVELS];
    st->pj_passes = (int64_t)c.stat[ST_PJ];
    st->rounds = (int64_t)c.stat[ST_ROUNDS];
    // totals of the batch; the seeds' share (k_append) is kept apart for the byte model
    const double live_ins = (double)c.stat[ST_LIVE_INS], seed_upd = (double)c.stat[ST_SEED_UPD],
                 seed_front = (double)c.stat[ST_SEED_FRONT];
    st->frontier_total = (int64_t)(c.stat[ST_FRONTIER] + c.stat[ST_SEED_FRONT]);
    st->edges_relaxed = (int64_t)(c.stat[ST_EDGES_RELAX] + 2 * c.stat[ST_LIVE_INS]);
    st->edges_inval = (int64_t)(c.stat[ST_EDGES_INV] + c.stat[ST_EDGES_PULL]);
    st->del_probed = (int64_t)c.stat[ST_DEL_PROBED];
    st->updates = (int64_t)(c.stat[ST_UPDATES] + c.stat[ST_SEED_UPD]);
    st->overflow_entries = (int64_t)c.stat[ST_OVF];
    st->repacks = repacks;
    if (c.ts[1] > c.ts[0]) st->t_inval_ms = (double)(c.ts[1] - c.ts[0]) * 1e-6;
    if (c.ts[3] > c.ts[2]) st->t_relax_ms = (double)(c.ts[3] - c.ts[2]) * 1e-6;
    if (c.ts[2] > c.ts[1] && c.ts[1] > 0) {
        st->t_seed_ms = (double)(c.ts[2] - c.ts[1]) * 1e-6;
        st->t_relax_ms += st->t_seed_ms;
    }
    if (events) {
        float a = 0, b = 0, t = 0;
        if (cudaEventElapsedTime(&a, g->ev[0], g->ev[1]) == cudaSuccess) st->t_step1_ms = a;
        if (cudaEventElapsedTime(&b, g->ev[1], g->ev[2]) == cudaSuccess) st->t_update_ms = b;
        if (cudaEventElapsedTime(&t, g->ev[0], g->ev[2]) == cudaSuccess) st->t_total_ms = t;
        if (k > 0 && g->o.timing >= 2) {  // a batch: the front kernels one by one
            float d = 0, ap = 0;
            if (cudaEventElapsedTime(&d, g->ev[4], g->ev[5]) == cudaSuccess) st->t_delete_ms = d;
            if (cudaEventElapsedTime(&ap, g->ev[5], g->ev[1]) == cudaSuccess) st->t_append_ms = ap;
        }
    }
    st->n_killed = (int64_t)c.killed;
    st->work_items = (int64_t)c.stat[ST_ITEMS];
    st->advances = (int64_t)c.stat[ST_ADVANCES];
    st->tombstoned = (int64_t)c.stat[ST_TOMBS];
    st->graph_launch = g->pend_graph ? 1 : 0;
    // algorithmic bytes.  The update kernel's figure uses the per-unit bytes of the task's
    // byte model: per cut-off vertex 16 (state write, child-range offsets) + 4 per child, per
    // frontier vertex 20 (queue id, row offset and length, own state) + 16 per scanned edge
    // ((col, wt) + neighbour state), per distance-lowering atomic 12 (word, next-frontier
    // push).  A cut-off vertex's pull counts as a frontier vertex with its scanned edges; the
    // walk's scans of whole rows to find children are work beyond the model (no credit).
    const double inv = (double)st->n_invalidated, roots = (double)st->n_roots;
    const double upd = 16.0 * inv + 4.0 * (inv > roots ? inv - roots : 0.0) +
                       20.0 * ((double)c.stat[ST_FRONTIER] + inv) +
                       16.0 * ((double)c.stat[ST_EDGES_RELAX] + (double)c.stat[ST_EDGES_PULL]) +
                       12.0 * (double)c.stat[ST_UPDATES];
    //   the engine's own count of what the update kernel touches (reported beside it): per
    //   adjacency entry scanned 16, per work item 40, per pushed vertex 20, per lowering
    //   atomic 8, per cut-off vertex 12, per seed expanded 8, per pointer-jumping pass 12 n
    const double n = (double)g->n;
    double eng = 16.0 * (double)(c.stat[ST_EDGES_RELAX] + c.stat[ST_EDGES_INV] + c.stat[ST_EDGES_PULL]) +
                 40.0 * (double)st->work_items + 20.0 * (double)c.stat[ST_FRONTIER] + 8.0 * (double)c.stat[ST_UPDATES] +
                 12.0 * inv + 8.0 * (double)c.seed_count;
    if (st->pj_passes > 0) eng += n * (12.0 + 12.0 * (double)st->pj_passes);
    st->bytes_engine_update = eng;
    //   front kernels: 16 per record (read by each of the three), 48 per insertion (two
    //   descriptor atomics + two entries + hash probe), 56 per deletion (two descriptors, two
    //   prefix lengths, two states, hash slot) + 8 per probed entry + 16 per root; per
    //   surviving insertion 16 (both end states), per seed relaxation 8, per claimed end 8
    const double front = 48.0 * (double)k + 48.0 * (double)st->n_ins + 56.0 * (double)st->n_del +
                         8.0 * (double)st->del_probed + 16.0 * (double)st->n_roots + 16.0 * live_ins +
                         8.0 * seed_upd + 8.0 * seed_front;
    st->bytes_alg_update = upd;
    st->bytes_alg = upd + front;
}

constexpr int kSpareExhausted = 1;

// Moves every row that overflowed in this batch into the spare region and places its
// overflowed entries; kSpareExhausted if the region is too small (nothing lost: the caller
// repacks, which folds the overflow list in).
// Row growth with the twin index: rows compacted in place or moved, tombstones dropped (the
// kernels above).  kSpareExhausted when the moves and the scratch do not both fit the spare
// region (nothing has been written then: the caller repacks).
int grow_rows_compacting(dsssp_graph* g, const GrowParams& q, int novf, long long rows_max, unsigned wb,
                         cudaStream_t s) {
    CK(cudaMemsetAsync(g->d_gwords, 0, 2 * sizeof(unsigned long long), s), "row growth");
    k_grow_count<<<blocks_for(novf), kThreads, 0, s>>>(q);
    k_grow_plan<<<wb, kThreads, 0, s>>>(q);
    count_launch(2);
    int fail = 0;
    unsigned long long sp[2] = {0, 0}, words[2] = {0, 0};
    CK(cudaMemcpyAsync(&fail, g->d_fail, sizeof(int), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaMemcpyAsync(sp, g->d_spare, sizeof(sp), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaMemcpyAsync(words, g->d_gwords, sizeof(words), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaStreamSynchronize(s), "row growth");
    if (fail || sp[0] + words[0] > sp[1]) {
        k_grow_reset<<<blocks_for(rows_max), kThreads, 0, s>>>(q);
        count_launch(1);
        CK(cudaStreamSynchronize(s), "row growth");
        return kSpareExhausted;
    }
    k_grow_out<<<wb, kThreads, 0, s>>>(q);
    k_grow_relink<<<wb, kThreads, 0, s>>>(q);
    k_grow_translate<<<blocks_for(g->pend_k), kThreads, 0, s>>>(q);
    k_grow_back<<<wb, kThreads, 0, s>>>(q);
    k_grow_place2<<<blocks_for(g->pend_k), kThreads, 0, s>>>(q);
    k_grow_reset<<<blocks_for(rows_max), kThreads, 0, s>>>(q);
    count_launch(6);
    CK(cudaMemcpyAsync(&fail, g->d_fail, sizeof(int), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaStreamSynchronize(s), "row growth");
    if (fail) return dsssp::fail(DSSSP_E_CUDA, "row growth: internal error %d", fail);
    g->spare_top = (long long)sp[0];
    g->grow_dropped = (long long)words[1];
    return DSSSP_OK;
}

int grow_rows(dsssp_graph* g, int novf, cudaStream_t s) {
    if (novf <= 0) return DSSSP_OK;
    if (!g->d_need) {
        int rc = dalloc(&g->d_need, (size_t)g->n, "row growth");
        if (!rc) rc = dalloc(&g->d_gidx, (size_t)g->n, "row growth");
        if (rc) return rc;
        CK(cudaMemsetAsync(g->d_need, 0, sizeof(int) * (size_t)g->n, s), "row growth");
        CK(cudaMemsetAsync(g->d_gidx, 0, sizeof(int) * (size_t)g->n, s), "row growth");
    }
    GrowParams q;
    q.rows = g->dg.rows;
    q.adj = g->dg.adj;
    q.twin = g->dg.twin;
    q.ovf = g->d_ovf;
    q.novf = novf;
    q.chg = g->pend_chg;
    q.k = g->pend_k;
    q.ins_state = g->d_ins_state;
    q.slot = g->d_slot;
    q.need = g->d_need;
    q.gidx = g->d_gidx;
    q.grow_list = g->d_grow_list;
    q.grow_count = g->d_grow_count;
    q.old_start = g->d_old_start;
    q.old_cap = g->d_old_cap;
    q.spare = g->d_spare;
    q.fail = g->d_fail;
    q.slack_min = g->o.slack_min > 4 ? g->o.slack_min : 4;
    q.cap_total = g->cap_total;
    q.sorted_len = g->dg.sorted_len;
    q.new_start = g->d_gnew;
    q.scratch = g->d_gscr;
    q.live = g->d_glive;
    q.live_sorted = g->d_gsorted;
    q.ncap = g->d_gncap;
    q.scr_used = g->d_gwords;
    q.dropped = g->d_gwords + 1;
    g->grow_dropped = 0;
    CK(cudaMemsetAsync(g->d_grow_count, 0, sizeof(unsigned), s), "row growth");
    CK(cudaMemsetAsync(g->d_fail, 0, sizeof(int), s), "row growth");
    const long long rows_max = novf < g->grow_cap ? novf : g->grow_cap;
    const unsigned wb = (unsigned)((rows_max * 32 + kThreads - 1) / kThreads);
    if (g->dg.twin) return grow_rows_compacting(g, q, novf, rows_max, wb, s);
    k_grow_count<<<blocks_for(novf), kThreads, 0, s>>>(q);
    k_grow_move<<<wb, kThreads, 0, s>>>(q);
    count_launch(2);
    int fail = 0;
    CK(cudaMemcpyAsync(&fail, g->d_fail, sizeof(int), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaStreamSynchronize(s), "row growth");
    if (fail) {
        k_grow_reset<<<blocks_for(rows_max), kThreads, 0, s>>>(q);
        count_launch(1);
        CK(cudaStreamSynchronize(s), "row growth");
        return kSpareExhausted;
    }
    k_grow_fix<<<wb, kThreads, 0, s>>>(q);
    k_grow_place<<<blocks_for(g->pend_k), kThreads, 0, s>>>(q);
    k_grow_reset<<<blocks_for(rows_max), kThreads, 0, s>>>(q);
    count_launch(3);
    CK(cudaMemcpyAsync(&fail, g->d_fail, sizeof(int), cudaMemcpyDeviceToHost, s), "row growth");
    unsigned long long top = 0;
    CK(cudaMemcpyAsync(&top, g->d_spare, sizeof(top), cudaMemcpyDeviceToHost, s), "row growth");
    CK(cudaStreamSynchronize(s), "row growth");
    if (fail) return dsssp::fail(DSSSP_E_CUDA, "row growth: twin index out of range (internal error)");
    g->spare_top = (long long)top;
    return DSSSP_OK;
}

// Kernel-node parameters of the batch kernels for the parameter block p.
struct BatchNodes {
    UpdParams p;
    void* args[1];
    cudaKernelNodeParams kp[4];
    cudaMemsetParams hash;
};

void batch_nodes(const dsssp_graph* g, const UpdParams& p, unsigned long long h, BatchNodes& b) {
    const void* fns[4];
    batch_kernels(fns);
    fns[1] = delete_kernel(p.tails != 0);
    fns[3] = update_kernel(p.warp_agg != 0);
    b.p = p;
    b.args[0] = &b.p;
    const long long need = (p.k + 255) / 256;
    const unsigned front = (unsigned)(need < g->num_sms * 8 ? need : g->num_sms * 8);  // as launch_front
    for (int i = 0; i < 4; i++) {
        cudaKernelNodeParams& k = b.kp[i];
        k = cudaKernelNodeParams{};
        k.func = const_cast<void*>(fns[i]);
        k.gridDim = dim3(i < 3 ? front : (unsigned)g->coop_grid);
        k.blockDim = dim3(i < 3 ? 256u : (unsigned)g->o.block);
        k.sharedMemBytes = 0;
        k.kernelParams = b.args;
        k.extra = nullptr;
    }
    memset(&b.hash, 0, sizeof(b.hash));
    b.hash.dst = g->d_hset;
    b.hash.value = 0xFF;
    b.hash.elementSize = 1;
    b.hash.width = sizeof(DelSlot) * (size_t)h;
    b.hash.height = 1;
    b.hash.pitch = 0;
}

void drop_batch_graph(dsssp_graph* g) {
    if (g->bexec) cudaGraphExecDestroy(g->bexec);
    if (g->bgraph) cudaGraphDestroy(g->bgraph);
    g->bexec = nullptr;
    g->bgraph = nullptr;
}

// Builds and instantiates the batch graph: [event 0] control-block reset, deletion-set reset,
// k_prepare, [event 4], k_delete, [event 5], k_append, [event 1] k_update (cooperative),
// [event 2] status read.  Events 0-2 are recorded at timing level 1, events 4-5 at level 2.
cudaError_t build_batch_graph(dsssp_graph* g, const BatchNodes& b, int timing) {
    drop_batch_graph(g);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaGraphCreate(&gr, 0);
    if (e != cudaSuccess) return e;
    g->bgraph = gr;
    cudaGraphNode_t prev = nullptr, n = nullptr;
    auto dep = [&]() { return prev ? 1 : 0; };
    if (timing && (e = cudaGraphAddEventRecordNode(&n, gr, &prev, dep(), g->ev[0])) == cudaSuccess) prev = n;
    if (e == cudaSuccess) {
        cudaMemsetParams c;
        memset(&c, 0, sizeof(c));
        const size_t off = offsetof(Ctl, status);  // line 1 onwards, as clear_ctl
        c.dst = (char*)g->dg.ctl + off;
        c.value = 0;
        c.elementSize = 1;
        c.width = sizeof(Ctl) - off;
        c.height = 1;
        if ((e = cudaGraphAddMemsetNode(&n, gr, &prev, dep(), &c)) == cudaSuccess) prev = n;
    }
    if (e == cudaSuccess && (e = cudaGraphAddMemsetNode(&n, gr, &prev, dep(), &b.hash)) == cudaSuccess) {
        prev = n;
        g->bn_hash = n;
    }
    for (int i = 0; i < 4 && e == cudaSuccess; i++) {
        if (i == 3 && timing && (e = cudaGraphAddEventRecordNode(&n, gr, &prev, dep(), g->ev[1])) == cudaSuccess)
            prev = n;
        if (e != cudaSuccess) break;
        if ((e = cudaGraphAddKernelNode(&n, gr, &prev, dep(), &b.kp[i])) != cudaSuccess) break;
        g->bn_kern[i] = n;
        if (i < 2 && timing >= 2) {  // after k_prepare and after k_delete
            prev = n;
            if ((e = cudaGraphAddEventRecordNode(&n, gr, &prev, dep(), g->ev[4 + i])) != cudaSuccess) break;
        }
        if (i == 3) {  // the update kernel's grid barrier needs all CTAs resident
            cudaLaunchAttributeValue v;
            memset(&v, 0, sizeof(v));
            v.cooperative = 1;
            if ((e = cudaGraphKernelNodeSetAttribute(n, cudaLaunchAttributeCooperative, &v)) != cudaSuccess) break;
        }
        prev = n;
    }
    if (e == cudaSuccess && timing && (e = cudaGraphAddEventRecordNode(&n, gr, &prev, dep(), g->ev[2])) == cudaSuccess)
        prev = n;
    if (e == cudaSuccess &&
        (e = cudaGraphAddMemcpyNode1D(&n, gr, &prev, dep(), g->h_ctl, g->dg.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost)) ==
            cudaSuccess)
        prev = n;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->bexec, gr, 0);
    if (e != cudaSuccess) {
        drop_batch_graph(g);
        cudaGetLastError();
    }
    g->bgraph_timing = timing;
    g->bgraph_agg = b.p.warp_agg;
    g->bgraph_tails = b.p.tails;
    return e;
}

// Replays the batch graph with this batch's parameters; false = use plain launches.
bool launch_batch_graph(dsssp_graph* g, const UpdParams& p, unsigned long long h, cudaStream_t s) {
    if (!g->o.launch_graph || g->bgraph_failed || p.k <= 0) return false;
    BatchNodes b;
    batch_nodes(g, p, h, b);
    const int timing = g->o.timing;
    cudaError_t e = cudaSuccess;
    if (!g->bexec || g->bgraph_timing != timing || g->bgraph_agg != p.warp_agg || g->bgraph_tails != p.tails) {
        e = build_batch_graph(g, b, timing);
    } else {
        e = cudaGraphExecMemsetNodeSetParams(g->bexec, g->bn_hash, &b.hash);
        for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaGraphExecKernelNodeSetParams(g->bexec, g->bn_kern[i], &b.kp[i]);
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(g->bexec, s);
    if (e != cudaSuccess) {  // never again for this graph: plain launches
        cudaGetLastError();
        drop_batch_graph(g);
        g->bgraph_failed = true;
        return false;
    }
    count_launch(4);
    return true;
}

// Enqueues one batch (records already on the device).
int enqueue_batch(dsssp_graph* g, const int4* d_chg, long long k, cudaStream_t s) {
    // k_append already claims frontier tags: restart the tag sequence before it could wrap
    // (the mirror holds the round base the last kernel left)
    if (g->h_ctl->round_base > 0xF0000000u) reset_tags(g, g->stream);
    if (effective_delta(g) > 0) {
        const int rc = ensure_far(g);
        if (rc) return rc;
    }
    const size_t hb = (size_t)(2ull * (unsigned long long)k);
    unsigned long long h = 64;
    while (h < hb) h <<= 1;  // this batch uses the first h slots of the deletion set
    UpdParams p = make_params(g, d_chg, k, 0);
    p.hmask = h - 1;
    g->pend_rb0 = g->h_ctl->round_base;  // the device reads the same value (mirror)
    g->pend_graph = launch_batch_graph(g, p, h, s);
    if (g->pend_graph) return DSSSP_OK;
    const bool ev = g->o.timing != 0;
    if (ev) CK(cudaEventRecord(g->ev[0], s), "event");
    int rc = clear_ctl(g, s);
    if (rc) return rc;
    CK(cudaMemsetAsync(g->d_hset, 0xFF, sizeof(DelSlot) * h, s), "deletion set reset");
    const bool fev = g->o.timing >= 2;
    CK(launch_front(p, g->num_sms * 8, s, fev ? g->ev[4] : nullptr, fev ? g->ev[5] : nullptr), "insert/delete kernels");
    if (ev) CK(cudaEventRecord(g->ev[1], s), "event");
    CK(launch_update(p, g->coop_grid, g->o.block, s), "update kernel");
    if (ev) CK(cudaEventRecord(g->ev[2], s), "event");
    CK(cudaMemcpyAsync(g->h_ctl, g->dg.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s), "status read");
    return DSSSP_OK;
}

// Statuses of the update kernel that leave the batch's adjacency edits in place and the tree
// unfinished: a timed-out grid barrier, the round cap, an internal list capacity, a parent
// cycle found by pointer jumping.  (Refused records, found before anything is modified, and a
// distance overflow, which a recomputation would meet again, are not among them.)
bool recoverable(int dev_status) {
    return dev_status == DSSSP_E_TIMEOUT || dev_status == DSSSP_E_NO_CONVERGENCE || dev_status == -4 ||
           dev_status == DSSSP_E_BAD_TREE;
}

// After a recoverable failure the graph holds the whole batch (every deletion and insertion
// is in the adjacency) but the tree is unfinished.  With opts.recover the trees are computed
// again from the roots on the updated graph, which gives exactly the result of a successful
// batch: DSSSP_W_RECOMPUTED, and st->recovered_from names the failure.  If that computation
// fails too, the tree is marked unusable (later batches are refused until a tree is loaded or
// computed) and the original error is returned.  Without opts.recover the error is returned
// and the tree is left as the kernel left it.
int recover_after_failure(dsssp_graph* g, int rc, dsssp_stats* st) {
    if (!g->o.recover || g->roots.empty()) {
        if (g->o.recover) g->has_tree = false;
        return rc;
    }
    char why[200];
    snprintf(why, sizeof why, "%s", dsssp_last_error());
    const std::vector<int> roots = g->roots;
    dsssp_stats rs;
    // the recomputation runs with the default round cap (2n + 16): after round r of a
    // computation from the sources every vertex with a shortest path of at most r edges is
    // final, so it needs fewer than n rounds
    const long long cap = g->o.max_rounds;
    g->o.max_rounds = 0;
    const int rr = dsssp_tree_compute_multi(g, roots.data(), (int32_t)roots.size(), &rs);
    g->o.max_rounds = cap;
    if (rr != DSSSP_OK) {
        g->has_tree = false;
        return fail(rc, "%s; recomputing the trees from %zu roots failed too (%d): the tree must be loaded or "
                        "computed again", why, roots.size(), rr);
    }
    if (st) {
        st->recovered_from = rc;
        st->t_recompute_ms = rs.t_total_ms;
    }
    return fail(DSSSP_W_RECOMPUTED, "%s; the batch is applied and the trees were recomputed from %zu roots", why,
                roots.size());
}

int finish_batch(dsssp_graph* g, dsssp_stats* st) {
    if (!g->pending) {
        if (st) memset(st, 0, sizeof(*st));
        return DSSSP_OK;
    }
    g->pending = false;
    cudaStream_t s = g->pend_stream;
    CK(cudaStreamSynchronize(s), "batch");
    int repacks = 0;
    if (g->h_ctl->status == kStatusOverflowPending) {
        // deletions are applied and the insertions that fit are placed.  The rows that ran
        // out of slack drop their tombstones and are compacted in place or move to the spare
        // region with room to grow; only when that region is used up is the whole adjacency
        // repacked.  Then the update kernel runs.
        int rc = grow_rows(g, g->h_ctl->ovf_count, s);
        if (rc == kSpareExhausted) {
            rc = repack(g, g->d_ovf, g->h_ctl->ovf_count, s);
            repacks = 1;
        }
        if (rc) return rc;
        CK(cudaMemsetAsync(&g->dg.ctl->status, 0, sizeof(int), s), "status reset");
        UpdParams p = make_params(g, g->pend_chg, g->pend_k, 0);
        // the front interval now spans the repack; the update interval is the resumed launch
        if (g->pend_events) CK(cudaEventRecord(g->ev[1], s), "event");
        CK(launch_update(p, g->coop_grid, g->o.block, s), "update kernel");
        if (g->pend_events) CK(cudaEventRecord(g->ev[2], s), "event");
        CK(cudaMemcpyAsync(g->h_ctl, g->dg.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s), "status read");
        CK(cudaStreamSynchronize(s), "batch");
    }
    fill_stats(g, *g->h_ctl, st, g->pend_events, g->pend_k, repacks);
    if (!repacks) {  // a repack counts the live entries itself
        const long long tombs = (long long)g->h_ctl->stat[ST_TOMBS];
        g->entries += 2 * (long long)g->h_ctl->stat[ST_LIVE_INS] - tombs;
        g->dead += tombs - g->grow_dropped;  // row growth drops the tombstones of the rows it compacts
        if (g->h_ctl->stat[ST_LIVE_INS] > 0) g->tails = true;  // insertions appended to row tails
    }
    g->grow_dropped = 0;
    g->delta_ok = g->h_ctl->status == 0 && g->h_ctl->stat[ST_DIST_OVF] == 0;
    g->delta_empty = false;
    if (g->h_ctl->status == 0) g->last_rounds = (long long)g->h_ctl->stat[ST_ROUNDS];
    g->delta_lo = g->pend_rb0;
    g->delta_hi = g->h_ctl->round_base;
    g->delta_epoch = g->epoch;
    const int dev_status = g->h_ctl->status;
    if (dev_status != 0) reset_tags(g, s);
    if (g->h_ctl->stat[ST_DIST_OVF] > 0 && dev_status == 0) return status_code(DSSSP_E_OVERFLOW);
    int rc;
    if (dev_status == DSSSP_E_TIMEOUT) {
        const unsigned* d = g->h_ctl->diag;
        rc = fail(DSSSP_E_TIMEOUT,
                  "grid barrier #%u timed out with %u of %d CTAs arrived; %u CTAs timed out; "
                  "CTA barrier counts at exit: min %u max %u",
                  d[0], d[1], g->coop_grid, d[2], 0xFFFFFFFFu - d[4], d[3]);
    } else {
        rc = status_code(dev_status);
    }
    if (rc == DSSSP_OK || !recoverable(dev_status)) return rc;
    return recover_after_failure(g, rc, st);
}

}  // namespace
}  // namespace dsssp

// =========================================================================================
// C ABI
// =========================================================================================

extern "C" {

int dsssp_abi_sizes(size_t* out, int32_t cap) {
    const size_t sz[] = {sizeof(dsssp_opts), sizeof(dsssp_stats), sizeof(dsssp_server_opts), sizeof(dsssp_request_info),
                         sizeof(dsssp_tune_result)};
    int32_t k = 0;
    for (; out && k < cap && k < (int32_t)(sizeof sz / sizeof sz[0]); k++) out[k] = sz[k];
    return k;
}

void dsssp_default_opts(dsssp_opts* o) {
    if (!o) return;
    o->device = 0;
    o->slack_pct = 25;
    o->slack_min = 4;
    o->small_deg = 4;
    o->large_deg = 256;
    o->chunk = 1024;
    o->bfs_levels = 48;
    o->block = 256;
    o->ctas_per_sm = 0;
    o->timing = 1;
    o->max_rounds = 0;
    o->spare_pct = 12;
    o->delta = -1;
    o->launch_graph = 1;
    o->recover = 1;
    o->warp_agg = 0;
    o->solo_waves = 2;
    o->auto_rounds = 256;
    o->group_ctas = 0;
    o->group_waves = 2;
}

const char* dsssp_strerror(int code) {
    switch (code) {
        case DSSSP_OK: return "ok";
        case DSSSP_E_INVAL: return "invalid argument";
        case DSSSP_E_OOM: return "out of memory";
        case DSSSP_E_BAD_VERTEX: return "vertex id out of range";
        case DSSSP_E_CUDA: return "CUDA error";
        case DSSSP_E_NO_CONVERGENCE: return "no convergence within the round cap";
        case DSSSP_E_TIMEOUT: return "device-side wait timed out";
        case DSSSP_E_BAD_TREE: return "invalid shortest-path tree";
        case DSSSP_E_OVERFLOW: return "distance overflow";
        case DSSSP_E_IO: return "file I/O error";
        case DSSSP_E_BAD_WEIGHT: return "negative edge weight";
        case DSSSP_E_NO_DEVICE: return "no CUDA device";
        case DSSSP_E_COOP: return "persistent kernel cannot be co-resident";
        case DSSSP_W_RECOMPUTED: return "batch applied; tree recomputed after a failed update";
        default: return "unknown error";
    }
}

int64_t dsssp_launch_count(void) { return (int64_t)g_launches.load(); }

void* dsssp_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void dsssp_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

void dsssp_graph_destroy(dsssp_graph* g) {
    if (!g) return;
    cudaSetDevice(g->dev);
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->copy_stream) cudaStreamSynchronize(g->copy_stream);
    DevGraph& d = g->dg;
    dfree(g->a_par); dfree(g->a_dist);
    if (g->ev_unpacked) cudaEventDestroy(g->ev_unpacked);
    if (g->ev_copied) cudaEventDestroy(g->ev_copied);
    if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
    dfree(d.state); dfree(d.rows); dfree(d.sorted_len); dfree(d.adj); dfree(d.inv_tag);
    dfree(d.push_tag); dfree(d.jm); dfree(d.invq); dfree(d.rt0); dfree(d.rt1); dfree(d.rc0); dfree(d.rc1);
    dfree(d.it); dfree(d.ic); dfree(d.ctl); dfree(d.far0); dfree(d.far1); dfree(d.far_tag); dfree(d.chg_tag);
    dfree(g->d_chg); dfree(g->d_ins_state); dfree(g->d_ovf); dfree(g->d_hset); dfree(d.twin); dfree(g->s_twin);
    dfree(g->d_par); dfree(g->d_dist); dfree(g->d_vtx); dfree(g->d_count); dfree(g->d_srcs); dfree(g->d_slot); dfree(g->d_seedq); dfree(g->d_spare);
    dfree(g->d_need); dfree(g->d_gidx); dfree(g->d_grow_list); dfree(g->d_grow_count); dfree(g->d_old_start);
    dfree(g->d_old_cap); dfree(g->d_fail);
    dfree(g->d_gnew); dfree(g->d_gscr); dfree(g->d_glive); dfree(g->d_gsorted); dfree(g->d_gncap); dfree(g->d_gwords);
    dfree(g->s_state); dfree(g->s_rows); dfree(g->s_sorted); dfree(g->s_adj);
    if (g->bexec) cudaGraphExecDestroy(g->bexec);
    if (g->bgraph) cudaGraphDestroy(g->bgraph);
    if (g->h_ctl) cudaFreeHost(g->h_ctl);
    for (auto& e : g->ev)
        if (e) cudaEventDestroy(e);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

static int check_opts(const dsssp_opts& o) {
    if (o.slack_pct < 0 || o.slack_min < 0 || o.small_deg < 4 || o.small_deg > 64 || o.small_deg % 4 ||
        o.large_deg < o.small_deg || o.chunk < 32 ||
        o.bfs_levels < 0 || o.block < 32 || o.block > 256 || o.block % 32 || o.ctas_per_sm < 0 || o.max_rounds < 0 ||
        o.spare_pct < 0 || o.spare_pct > 400 || o.delta < -1 || o.timing < 0 || o.timing > 2 || o.recover < 0 ||
        o.recover > 1 || o.warp_agg < 0 || o.warp_agg > 1 || o.solo_waves < 0 || o.solo_waves > 64 ||
        o.auto_rounds < 0 || o.group_ctas < 0 || o.group_ctas > 1024 || o.group_waves < 1 || o.group_waves > 64)
        return fail(DSSSP_E_INVAL, "invalid dsssp_opts");
    return DSSSP_OK;
}

int dsssp_graph_create(int32_t n, int64_t m, const int32_t* u, const int32_t* v, const int32_t* w,
                       const dsssp_opts* opts, dsssp_graph** out) {
    if (!out) return fail(DSSSP_E_INVAL, "graph_create: out is NULL");
    *out = nullptr;
    if (n <= 0 || n >= 0x7FFFFFF0 || m < 0 || (m > 0 && (!u || !v || !w)))
        return fail(DSSSP_E_INVAL, "graph_create: bad sizes or NULL edge arrays");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(DSSSP_E_NO_DEVICE, "no CUDA device is available");
    }
    dsssp_graph* g = new dsssp_graph();
    if (opts) g->o = *opts;
    else dsssp_default_opts(&g->o);
    if (m > 0) {  // mean weight for the automatic near-far width
        double sw = 0;
#pragma omp parallel for reduction(+ : sw)
        for (int64_t i = 0; i < m; i++) sw += (double)(w[i] > 0 ? w[i] : 0);
        g->mean_w = sw / (double)m;
    }
    int rc = check_opts(g->o);
    if (rc) { delete g; return rc; }
    if (g->o.device < 0 || g->o.device >= ndev) {
        const int dev = g->o.device;
        delete g;
        return fail(DSSSP_E_INVAL, "device %d does not exist", dev);
    }
    g->dev = g->o.device;
    g->n = n;
    rc = set_device(g);
    if (rc) { delete g; return rc; }
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->dev);
    cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->dev);
    if (!coop) { delete g; return fail(DSSSP_E_COOP, "device does not support cooperative launch"); }
    int per_sm = 0;
    if (update_occupancy(g->o.block, &per_sm) != cudaSuccess || per_sm < 1) {
        const int block = g->o.block;
        delete g;
        return fail(DSSSP_E_COOP, "update kernel has no occupancy at block %d", block);
    }
    if (g->o.ctas_per_sm > 0 && g->o.ctas_per_sm < per_sm) per_sm = g->o.ctas_per_sm;
    g->coop_grid = per_sm * g->num_sms;
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { dsssp_graph_destroy(g); return cuda_fail(e, "stream"); }
    for (auto& ev : g->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) { dsssp_graph_destroy(g); return cuda_fail(e, "event"); }
    if (cudaMallocHost((void**)&g->h_ctl, sizeof(Ctl)) != cudaSuccess) {
        dsssp_graph_destroy(g);
        return fail(DSSSP_E_OOM, "pinned control block");
    }
    memset(g->h_ctl, 0, sizeof(Ctl));
    DevGraph& d = g->dg;
    const size_t N = (size_t)n;
    rc = dalloc(&d.state, N, "state");
    if (!rc) rc = dalloc(&d.rows, N, "rows");
    if (!rc) rc = dalloc(&d.sorted_len, N, "sorted_len");
    if (!rc) rc = dalloc(&d.inv_tag, N, "inv_tag");
    if (!rc) rc = dalloc(&d.push_tag, N, "push_tag");
    if (!rc) rc = dalloc(&d.jm, N, "jm");
    if (!rc) rc = dalloc(&d.invq, N, "invq");
    if (!rc) rc = dalloc(&d.chg_tag, N, "change tags");
    if (!rc) rc = dalloc(&d.ctl, 1, "control block");
    if (!rc) rc = dalloc(&g->d_spare, 2, "spare region words");
    if (!rc) rc = dalloc(&g->d_grow_count, 1, "row growth");
    if (!rc) rc = dalloc(&g->d_fail, 1, "row growth");
    if (rc) { dsssp_graph_destroy(g); return rc; }
    cudaStream_t s = g->stream;
    cudaMemsetAsync(d.state, 0xFF, sizeof(unsigned long long) * N, s);
    cudaMemsetAsync(d.inv_tag, 0, sizeof(unsigned) * N, s);
    cudaMemsetAsync(d.chg_tag, 0, sizeof(unsigned) * N, s);
    cudaMemsetAsync(d.push_tag, 0, sizeof(unsigned) * N, s);
    cudaMemsetAsync(d.ctl, 0, sizeof(Ctl), s);
    Ctl init{};
    init.round_base = 1;
    cudaMemcpyAsync(d.ctl, &init, sizeof(Ctl), cudaMemcpyHostToDevice, s);

    // edges -> packed rows -> sorted slack layout
    int *du = nullptr, *dv = nullptr, *dw = nullptr, *deg = nullptr, *cursor = nullptr;
    long long *deg64 = nullptr, *poff = nullptr;
    unsigned long long* keys = nullptr;
    rc = dalloc(&du, (size_t)m, "edge upload");
    if (!rc) rc = dalloc(&dv, (size_t)m, "edge upload");
    if (!rc) rc = dalloc(&dw, (size_t)m, "edge upload");
    if (!rc) rc = dalloc(&deg, N, "degrees");
    if (!rc) rc = dalloc(&cursor, N, "cursors");
    if (!rc && m > 0) {
        e = cudaMemcpyAsync(du, u, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dw, w, sizeof(int) * (size_t)m, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "edge upload");
    }
    if (!rc) {
        cudaMemsetAsync(deg, 0, sizeof(int) * N, s);
        cudaMemsetAsync(cursor, 0, sizeof(int) * N, s);
        if (m > 0) {
            k_check_edges<<<blocks_for(m), kThreads, 0, s>>>(du, dv, dw, m, n, d.ctl);
            count_launch(1);
        }
        e = cudaMemcpyAsync(g->h_ctl, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = cuda_fail(e, "edge check");
        else if (g->h_ctl->status != 0)
            rc = fail(g->h_ctl->status, g->h_ctl->status == DSSSP_E_BAD_WEIGHT ? "graph has a negative edge weight"
                                                                               : "graph names a vertex outside 0..n-1");
    }
    if (!rc && m > 0) {
        k_degree<<<blocks_for(m), kThreads, 0, s>>>(du, dv, m, deg);
        count_launch(1);
    }
    if (!rc) rc = row_offsets(g, deg, &deg64, &poff, s);
    if (!rc) rc = dalloc(&keys, (size_t)(2 * m), "build keys");
    if (!rc && m > 0) {
        k_scatter_packed<<<blocks_for(m), kThreads, 0, s>>>(du, dv, dw, m, poff, cursor, keys);
        count_launch(1);
    }
    dfree(du); dfree(dv); dfree(dw);
    if (!rc) rc = layout_rows(g, keys, 2 * m, deg64, poff, s);
    dfree(deg); dfree(cursor); dfree(deg64); dfree(poff); dfree(keys);
    if (rc) { dsssp_graph_destroy(g); return rc; }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { dsssp_graph_destroy(g); return cuda_fail(e, "graph build"); }
    *out = g;
    return DSSSP_OK;
}

int dsssp_graph_info(const dsssp_graph* g, int64_t* n, int64_t* entries, int64_t* capacity,
                     int64_t* device_bytes, int32_t* source) {
    if (!g) return fail(DSSSP_E_INVAL, "graph_info: NULL graph");
    if (n) *n = g->n;
    if (entries) *entries = g->entries;
    if (capacity) *capacity = g->cap_total;
    if (source) *source = g->src;
    if (device_bytes) {
        const long long N = g->n;
        long long b = N * (8 + 16 + 4 + 4 + 4 + 4 + 4) + g->cap_total * 8 + 3 * g->dg.tcap * 8 +
                      3 * g->dg.ccap * 8 + g->chg_cap * (16 + 4 + 32) + (long long)g->hcap * 16 +
                      (g->dg.twin ? g->cap_total * 4 : 0) +
                      (long long)sizeof(Ctl);
        if (g->d_par) b += N * 12;
        if (g->has_snap) b += N * (8 + 16 + 4) + g->s_cap * 8;
        *device_bytes = b;
    }
    return DSSSP_OK;
}

static int tree_load_impl(dsssp_graph* g, const int32_t* parent, const int64_t* dist, bool forest) {
    if (!g || !parent || !dist) return fail(DSSSP_E_INVAL, "tree_load: NULL argument");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_load: a batch is still pending");
    cudaStream_t s = g->stream;
    if (!g->d_par) {
        rc = dalloc(&g->d_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    rc = clear_ctl(g, s);
    if (rc) return rc;
    const unsigned long long big = ~0ull;
    CK(cudaMemcpyAsync(&g->dg.ctl->stat[1], &big, sizeof(big), cudaMemcpyHostToDevice, s), "tree load");
    CK(cudaMemcpyAsync(g->d_par, parent, sizeof(int) * (size_t)g->n, cudaMemcpyHostToDevice, s), "tree upload");
    CK(cudaMemcpyAsync(g->d_dist, dist, sizeof(long long) * (size_t)g->n, cudaMemcpyHostToDevice, s), "tree upload");
    k_tree_pack<<<blocks_for(g->n), kThreads, 0, s>>>(g->d_par, g->d_dist, g->n, g->dg.state, g->dg.ctl);
    count_launch(1);
    CK(cudaMemcpyAsync(g->h_ctl, g->dg.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s), "tree load");
    CK(cudaStreamSynchronize(s), "tree load");
    const unsigned long long roots = g->h_ctl->stat[0];
    int bad = 0;
    if (g->h_ctl->status != 0) {
        bad = fail(g->h_ctl->status, "tree_load: %s", g->h_ctl->status == DSSSP_E_OVERFLOW
                                                          ? "a distance does not fit below 2^32-1"
                                                          : "bad parent id, negative distance or root distance != 0");
    } else if (forest ? roots == 0 : roots != 1) {
        bad = fail(DSSSP_E_BAD_TREE, "tree_load: %llu vertices are their own parent (need %s)", roots,
                   forest ? "at least one root" : "exactly one root");
    }
    if (bad) {
        cudaMemsetAsync(g->dg.state, 0xFF, sizeof(unsigned long long) * (size_t)g->n, s);
        cudaStreamSynchronize(s);
        g->src = -1;
        g->has_tree = false;
        return bad;
    }
    g->src = (int)g->h_ctl->stat[1];
    g->has_tree = true;
    g->delta_ok = false;
    g->roots.clear();
    for (int v = 0; v < g->n; v++)
        if (parent[v] == v) g->roots.push_back(v);
    return DSSSP_OK;
}

int dsssp_tree_load(dsssp_graph* g, const int32_t* parent, const int64_t* dist) {
    return tree_load_impl(g, parent, dist, false);
}

int dsssp_forest_load(dsssp_graph* g, const int32_t* parent, const int64_t* dist) {
    return tree_load_impl(g, parent, dist, true);
}

static int compute_from_sources(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st, bool reset);

int dsssp_tree_compute_multi(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st) {
    return compute_from_sources(g, srcs, k, st, true);
}

int dsssp_tree_add_sources(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st) {
    return compute_from_sources(g, srcs, k, st, false);
}

// reset: every vertex starts unreachable (a computation from scratch); otherwise the current
// distances stay as upper bounds (each is the length of a real path from a root) and the new
// sources join the roots: relaxation from them lowers what they improve, which converges to the
// exact distances from the enlarged set of roots.
static int compute_from_sources(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st, bool reset) {
    if (!g || k < 1 || !srcs) return fail(DSSSP_E_INVAL, "tree_compute: NULL graph or no source");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_compute: a batch is still pending");
    for (int32_t i = 0; i < k; i++)
        if (srcs[i] < 0 || srcs[i] >= g->n)
            return fail(DSSSP_E_BAD_VERTEX, "tree_compute: source %d outside 0..%d", srcs[i], g->n - 1);
    cudaStream_t s = g->stream;
    if (k > g->srcs_cap) {
        dfree(g->d_srcs);
        g->srcs_cap = 0;
        rc = dalloc(&g->d_srcs, (size_t)k, "source list");
        if (rc) return rc;
        g->srcs_cap = k;
    }
    // the sources are de-duplicated so each is pushed once
    std::vector<int32_t> uniq(srcs, srcs + k);
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    const int nsrc = (int)uniq.size();
    rc = clear_ctl(g, s);
    if (rc) return rc;
    CK(cudaMemcpyAsync(g->d_srcs, uniq.data(), sizeof(int) * (size_t)nsrc, cudaMemcpyHostToDevice, s), "sources");
    const bool ev = g->o.timing != 0;
    if (ev) CK(cudaEventRecord(g->ev[0], s), "event");
    if (reset) {
        k_state_reset<<<blocks_for(g->n), kThreads, 0, s>>>(g->dg.state, g->n);
        count_launch(1);
    }
    k_set_sources<<<blocks_for(nsrc), kThreads, 0, s>>>(g->dg.state, g->n, g->d_srcs, nsrc, g->dg.ctl);
    count_launch(1);
    if (ev) CK(cudaEventRecord(g->ev[1], s), "event");
    if (effective_delta(g) > 0) {
        rc = ensure_far(g);
        if (rc) return rc;
    }
    UpdParams p = make_params(g, nullptr, 0, 1);
    p.nsrc = nsrc;
    CK(launch_update(p, g->coop_grid, g->o.block, s), "update kernel");
    if (ev) CK(cudaEventRecord(g->ev[2], s), "event");
    CK(cudaMemcpyAsync(g->h_ctl, g->dg.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s), "status read");
    CK(cudaStreamSynchronize(s), "tree compute");
    if (reset || !g->has_tree) {
        g->src = uniq[0];
        g->roots = uniq;
    } else {
        std::vector<int> all(g->roots);
        all.insert(all.end(), uniq.begin(), uniq.end());
        std::sort(all.begin(), all.end());
        all.erase(std::unique(all.begin(), all.end()), all.end());
        g->roots.swap(all);
        g->src = g->roots[0];
    }
    g->has_tree = g->h_ctl->status == 0;
    g->last_rounds = (long long)g->h_ctl->stat[ST_ROUNDS];
    g->delta_ok = false;
    g->pend_graph = false;
    fill_stats(g, *g->h_ctl, st, ev, 0, 0);
    if (g->h_ctl->status != 0) reset_tags(g, s);
    if (g->h_ctl->stat[ST_DIST_OVF] > 0 && g->h_ctl->status == 0) return status_code(DSSSP_E_OVERFLOW);
    return status_code(g->h_ctl->status);
}

int dsssp_tree_compute(dsssp_graph* g, int32_t src, dsssp_stats* st) {
    if (g && (src < 0 || src >= g->n))
        return fail(DSSSP_E_BAD_VERTEX, "tree_compute: source %d outside 0..%d", src, g->n - 1);
    return dsssp_tree_compute_multi(g, &src, 1, st);
}

int dsssp_tree_read(dsssp_graph* g, int32_t* parent, int64_t* dist) {
    if (!g) return fail(DSSSP_E_INVAL, "tree_read: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_read: a batch is still pending");
    cudaStream_t s = g->stream;
    if (!g->d_par) {
        rc = dalloc(&g->d_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    k_tree_unpack<<<blocks_for(g->n), kThreads, 0, s>>>(g->dg.state, g->n, parent ? g->d_par : nullptr,
                                                        dist ? g->d_dist : nullptr);
    count_launch(1);
    if (parent) CK(cudaMemcpyAsync(parent, g->d_par, sizeof(int) * (size_t)g->n, cudaMemcpyDeviceToHost, s), "tree read");
    if (dist) CK(cudaMemcpyAsync(dist, g->d_dist, sizeof(long long) * (size_t)g->n, cudaMemcpyDeviceToHost, s), "tree read");
    CK(cudaStreamSynchronize(s), "tree read");
    return DSSSP_OK;
}

int dsssp_tree_read32(dsssp_graph* g, int32_t* parent, uint32_t* dist) {
    if (!g) return fail(DSSSP_E_INVAL, "tree_read32: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_read32: a batch is still pending");
    cudaStream_t s = g->stream;
    if (!g->d_par) {
        rc = dalloc(&g->d_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    unsigned* d_dist32 = reinterpret_cast<unsigned*>(g->d_dist);  // n int64 slots hold n uint32
    k_tree_unpack32<<<blocks_for(g->n), kThreads, 0, s>>>(g->dg.state, g->n, parent ? g->d_par : nullptr,
                                                          dist ? d_dist32 : nullptr);
    count_launch(1);
    if (parent) CK(cudaMemcpyAsync(parent, g->d_par, sizeof(int) * (size_t)g->n, cudaMemcpyDeviceToHost, s), "tree read");
    if (dist) CK(cudaMemcpyAsync(dist, d_dist32, sizeof(unsigned) * (size_t)g->n, cudaMemcpyDeviceToHost, s), "tree read");
    CK(cudaStreamSynchronize(s), "tree read");
    return DSSSP_OK;
}

int dsssp_tree_read32_async(dsssp_graph* g, int32_t* parent, uint32_t* dist) {
    if (!g) return fail(DSSSP_E_INVAL, "tree_read32_async: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_read32_async: a batch is still pending");
    if (!g->copy_stream) {
        CK(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking), "copy stream");
        CK(cudaEventCreateWithFlags(&g->ev_unpacked, cudaEventDisableTiming), "copy events");
        CK(cudaEventCreateWithFlags(&g->ev_copied, cudaEventDisableTiming), "copy events");
    }
    if (!g->a_par) {
        rc = dalloc(&g->a_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->a_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    cudaStream_t s = g->stream;
    if (g->copy_pending) CK(cudaStreamWaitEvent(s, g->ev_copied, 0), "tree read");  // staging in use
    k_tree_unpack32<<<blocks_for(g->n), kThreads, 0, s>>>(g->dg.state, g->n, parent ? g->a_par : nullptr,
                                                          dist ? g->a_dist : nullptr);
    count_launch(1);
    CK(cudaEventRecord(g->ev_unpacked, s), "tree read");
    CK(cudaStreamWaitEvent(g->copy_stream, g->ev_unpacked, 0), "tree read");
    if (parent)
        CK(cudaMemcpyAsync(parent, g->a_par, sizeof(int) * (size_t)g->n, cudaMemcpyDeviceToHost, g->copy_stream),
           "tree read");
    if (dist)
        CK(cudaMemcpyAsync(dist, g->a_dist, sizeof(unsigned) * (size_t)g->n, cudaMemcpyDeviceToHost, g->copy_stream),
           "tree read");
    CK(cudaEventRecord(g->ev_copied, g->copy_stream), "tree read");
    g->copy_pending = true;
    return DSSSP_OK;
}

int dsssp_tree_read_wait(dsssp_graph* g) {
    if (!g) return fail(DSSSP_E_INVAL, "tree_read_wait: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (!g->copy_pending) return DSSSP_OK;
    CK(cudaEventSynchronize(g->ev_copied), "tree read");
    g->copy_pending = false;
    return DSSSP_OK;
}

int dsssp_tree_read_range(dsssp_graph* g, int32_t first, int32_t count, int32_t* parent, int64_t* dist) {
    if (!g || first < 0 || count < 0 || (long long)first + count > g->n || (count > 0 && (!parent || !dist)))
        return fail(DSSSP_E_INVAL, "tree_read_range: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_read_range: a batch is still pending");
    if (count == 0) return DSSSP_OK;
    cudaStream_t s = g->stream;
    if (!g->d_par) {
        rc = dalloc(&g->d_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    k_tree_unpack<<<blocks_for(count), kThreads, 0, s>>>(g->dg.state + first, count, g->d_par, g->d_dist);
    count_launch(1);
    CK(cudaMemcpyAsync(parent, g->d_par, sizeof(int) * (size_t)count, cudaMemcpyDeviceToHost, s), "tree read");
    CK(cudaMemcpyAsync(dist, g->d_dist, sizeof(long long) * (size_t)count, cudaMemcpyDeviceToHost, s), "tree read");
    CK(cudaStreamSynchronize(s), "tree read");
    return DSSSP_OK;
}

int dsssp_tree_read_changed(dsssp_graph* g, int32_t* vertex, int32_t* parent, int64_t* dist, int64_t cap,
                            int64_t* count) {
    if (!g || !vertex || !parent || !dist || cap < 0 || !count) return fail(DSSSP_E_INVAL, "tree_read_changed: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_read_changed: a batch is still pending");
    if (!g->delta_ok) return fail(DSSSP_E_INVAL, "tree_read_changed: no successful batch since the tree was set");
    if (g->delta_empty) {
        *count = 0;
        return DSSSP_OK;
    }
    cudaStream_t s = g->stream;
    if (!g->d_par) {
        rc = dalloc(&g->d_par, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_dist, (size_t)g->n, "tree staging");
        if (rc) return rc;
    }
    if (!g->d_vtx) {
        rc = dalloc(&g->d_vtx, (size_t)g->n, "tree staging");
        if (!rc) rc = dalloc(&g->d_count, 1, "tree staging");
        if (rc) return rc;
    }
    unsigned cnt = 0;
    CK(cudaMemsetAsync(g->d_count, 0, sizeof(unsigned), s), "tree read");
    k_tree_changed<<<blocks_for(g->n), kThreads, 0, s>>>(g->dg.state, g->dg.inv_tag, g->dg.chg_tag, g->dg.push_tag,
                                                         g->dg.far_tag,
                                                         g->n, g->delta_epoch, g->delta_lo, g->delta_hi, g->d_vtx,
                                                         g->d_par, g->d_dist, g->d_count);
    count_launch(1);
    CK(cudaMemcpyAsync(&cnt, g->d_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "tree read");
    CK(cudaStreamSynchronize(s), "tree read");
    *count = cnt;
    if ((int64_t)cnt > cap) return fail(DSSSP_E_INVAL, "tree_read_changed: %u changed vertices exceed cap %lld", cnt, (long long)cap);
    if (cnt) {
        CK(cudaMemcpyAsync(vertex, g->d_vtx, sizeof(int) * cnt, cudaMemcpyDeviceToHost, s), "tree read");
        CK(cudaMemcpyAsync(parent, g->d_par, sizeof(int) * cnt, cudaMemcpyDeviceToHost, s), "tree read");
        CK(cudaMemcpyAsync(dist, g->d_dist, sizeof(long long) * cnt, cudaMemcpyDeviceToHost, s), "tree read");
        CK(cudaStreamSynchronize(s), "tree read");
    }
    return DSSSP_OK;
}

int dsssp_debug_set(dsssp_graph* g, int32_t what, int64_t value) {
    if (!g) return fail(DSSSP_E_INVAL, "debug_set: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "debug_set: a batch is still pending");
    unsigned* field = nullptr;
    if (what == DSSSP_DEBUG_SPIN_LIMIT && value >= 0 && value <= (1ll << 24)) field = &g->dg.ctl->spin_limit;
    else if (what == DSSSP_DEBUG_STALL_US && value >= 0 && value <= 1000000) field = &g->dg.ctl->stall_us;
    if (!field) return fail(DSSSP_E_INVAL, "debug_set: unknown hook %d or value %lld out of range", what, (long long)value);
    const unsigned v = (unsigned)value;
    CK(cudaMemcpyAsync(field, &v, sizeof(v), cudaMemcpyHostToDevice, g->stream), "debug_set");
    CK(cudaStreamSynchronize(g->stream), "debug_set");
    return DSSSP_OK;
}

int dsssp_tree_validate(dsssp_graph* g, int64_t* violations, int64_t* roots, int32_t* first_bad) {
    if (!g || !violations) return fail(DSSSP_E_INVAL, "tree_validate: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "tree_validate: a batch is still pending");
    cudaStream_t s = g->stream;
    unsigned long long* d_out = nullptr;
    unsigned* d_long = nullptr;  // [0] count, then the long rows
    rc = dalloc(&d_out, 3, "validation counters");
    const long long long_cap = g->cap_total / kValidateLongRow + 2;
    if (!rc) rc = dalloc(&d_long, (size_t)long_cap, "validation rows");
    if (rc) {
        dfree(d_out);
        return rc;
    }
    const unsigned long long init[3] = {0, 0, ~0ull};
    unsigned long long out[3] = {0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(d_out, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_long, 0, sizeof(unsigned), s);
    const unsigned grid = (unsigned)(g->num_sms * 8);
    if (e == cudaSuccess) {
        k_validate_rows<<<grid, kThreads, 0, s>>>(g->dg.state, g->dg.rows, g->dg.adj, g->n, g->dg.jm, d_out,
                                                  d_long + 1, d_long);
        k_validate_long<<<grid, kThreads, 0, s>>>(g->dg.state, g->dg.rows, g->dg.adj, g->n, g->dg.jm, d_out,
                                                  d_long + 1, d_long);
        for (int pass = 0; pass < 32; pass++) k_validate_jump<<<grid, kThreads, 0, s>>>(g->dg.jm, g->n);
        k_validate_cycles<<<grid, kThreads, 0, s>>>(g->dg.jm, g->n, d_out);
        count_launch(35);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(d_out);
    dfree(d_long);
    if (e != cudaSuccess) return cuda_fail(e, "tree_validate");
    *violations = (int64_t)out[0];
    if (roots) *roots = (int64_t)out[1];
    if (first_bad) *first_bad = out[0] ? (int32_t)out[2] : -1;
    return DSSSP_OK;
}

int dsssp_apply_batch_async(dsssp_graph* g, const dsssp_change* d_changes, int64_t k, void* stream) {
    if (!g || k < 0 || (k > 0 && !d_changes)) return fail(DSSSP_E_INVAL, "apply_batch: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "apply_batch: previous batch not finished");
    if (!g->has_tree) return fail(DSSSP_E_BAD_TREE, "apply_batch: no tree loaded");
    cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
    if (k == 0) {  // nothing to do; the changed-entries read of this batch is empty
        g->delta_ok = true;
        g->delta_empty = true;
        return DSSSP_OK;
    }
    rc = ensure_batch(g, k);
    if (!rc && g->copy_pending) CK(cudaStreamWaitEvent(s, g->ev_unpacked, 0), "apply_batch");  // a read's unpack
    if (!rc) rc = next_epoch(g, s);
    if (!rc) rc = enqueue_batch(g, (const int4*)d_changes, k, s);
    if (rc) return rc;
    g->pending = true;
    g->pend_k = k;
    g->pend_chg = (const int4*)d_changes;
    g->pend_stream = s;
    g->pend_events = g->o.timing != 0;
    return DSSSP_OK;
}

int dsssp_batch_finish(dsssp_graph* g, dsssp_stats* st) {
    if (!g) return fail(DSSSP_E_INVAL, "batch_finish: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    return finish_batch(g, st);
}

int dsssp_apply_batch_host_async(dsssp_graph* g, const dsssp_change* changes, int64_t k, void* stream) {
    if (!g || k < 0 || (k > 0 && !changes)) return fail(DSSSP_E_INVAL, "apply_batch: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "apply_batch: previous batch not finished");
    if (k == 0) return dsssp_apply_batch_async(g, nullptr, 0, stream);
    rc = ensure_batch(g, k);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
    CK(cudaMemcpyAsync(g->d_chg, changes, sizeof(int4) * (size_t)k, cudaMemcpyHostToDevice, s), "batch upload");
    return dsssp_apply_batch_async(g, (const dsssp_change*)g->d_chg, k, s);
}

int dsssp_apply_batch(dsssp_graph* g, const dsssp_change* changes, int64_t k, void* stream, dsssp_stats* st) {
    if (st) memset(st, 0, sizeof(*st));
    const int rc = dsssp_apply_batch_host_async(g, changes, k, stream);
    if (rc || k == 0) return rc;
    return finish_batch(g, st);
}

int dsssp_graph_set_opts(dsssp_graph* g, const dsssp_opts* o) {
    if (!g || !o) return fail(DSSSP_E_INVAL, "set_opts: NULL argument");
    int rc = check_opts(*o);
    if (rc) return rc;
    if (o->device != g->dev) return fail(DSSSP_E_INVAL, "set_opts: the device of a graph cannot change");
    rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "set_opts: a batch is still pending");
    int per_sm = 0;
    if (update_occupancy(o->block, &per_sm) != cudaSuccess || per_sm < 1)
        return fail(DSSSP_E_COOP, "set_opts: update kernel has no occupancy at block %d", o->block);
    if (o->ctas_per_sm > 0 && o->ctas_per_sm < per_sm) per_sm = o->ctas_per_sm;
    const dsssp_opts old = g->o;
    g->o = *o;
    g->o.slack_pct = old.slack_pct;  // slack is fixed when rows are laid out
    g->o.slack_min = old.slack_min;
    rc = ensure_work(g);
    if (rc) {
        g->o = old;
        return rc;
    }
    g->coop_grid = per_sm * g->num_sms;
    return DSSSP_OK;
}

int dsssp_graph_get_opts(const dsssp_graph* g, dsssp_opts* o) {
    if (!g || !o) return fail(DSSSP_E_INVAL, "get_opts: NULL argument");
    *o = g->o;
    return DSSSP_OK;
}

int dsssp_graph_snapshot(dsssp_graph* g) {
    if (!g) return fail(DSSSP_E_INVAL, "snapshot: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "snapshot: a batch is still pending");
    if (!g->s_state) {
        rc = dalloc(&g->s_state, (size_t)g->n, "snapshot");
        if (!rc) rc = dalloc(&g->s_rows, (size_t)g->n, "snapshot");
        if (!rc) rc = dalloc(&g->s_sorted, (size_t)g->n, "snapshot");
        if (rc) return rc;
    }
    if (g->s_cap != g->cap_total || (g->dg.twin && !g->s_twin)) {
        dfree(g->s_adj);
        dfree(g->s_twin);
        g->s_cap = 0;
        rc = dalloc(&g->s_adj, (size_t)g->cap_total, "snapshot");
        if (!rc && g->dg.twin) rc = dalloc(&g->s_twin, (size_t)g->cap_total, "snapshot");
        if (rc) return rc;
        g->s_cap = g->cap_total;
    }
    cudaStream_t s = g->stream;
    const size_t N = (size_t)g->n;
    CK(cudaMemcpyAsync(g->s_state, g->dg.state, N * 8, cudaMemcpyDeviceToDevice, s), "snapshot");
    CK(cudaMemcpyAsync(g->s_rows, g->dg.rows, N * sizeof(RowDesc), cudaMemcpyDeviceToDevice, s), "snapshot");
    CK(cudaMemcpyAsync(g->s_sorted, g->dg.sorted_len, N * 4, cudaMemcpyDeviceToDevice, s), "snapshot");
    CK(cudaMemcpyAsync(g->s_adj, g->dg.adj, (size_t)g->cap_total * 8, cudaMemcpyDeviceToDevice, s), "snapshot");
    if (g->dg.twin)
        CK(cudaMemcpyAsync(g->s_twin, g->dg.twin, (size_t)g->cap_total * 4, cudaMemcpyDeviceToDevice, s), "snapshot");
    CK(cudaMemcpyAsync(g->s_spare, g->d_spare, sizeof(g->s_spare), cudaMemcpyDeviceToHost, s), "snapshot");
    CK(cudaStreamSynchronize(s), "snapshot");
    g->s_entries = g->entries;
    g->s_dead = g->dead;
    g->s_tails = g->tails;
    g->s_spare_lo = g->spare_lo;
    g->s_src = g->src;
    g->s_has_tree = g->has_tree;
    g->s_roots = g->roots;
    g->has_snap = true;
    return DSSSP_OK;
}

int dsssp_graph_restore(dsssp_graph* g, void* stream) {
    if (!g || !g->has_snap) return fail(DSSSP_E_INVAL, "restore: no snapshot");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "restore: a batch is still pending");
    cudaStream_t s = stream ? (cudaStream_t)stream : g->stream;
    if (g->copy_pending) CK(cudaStreamWaitEvent(s, g->ev_unpacked, 0), "restore");  // a read's unpack
    if (g->cap_total != g->s_cap || (g->s_twin && !g->dg.twin)) {
        CK(cudaStreamSynchronize(s), "restore");
        dfree(g->dg.adj);
        dfree(g->dg.twin);
        rc = dalloc(&g->dg.adj, (size_t)g->s_cap, "adjacency");
        if (!rc && g->s_twin) rc = dalloc(&g->dg.twin, (size_t)g->s_cap, "twin index");
        if (rc) return rc;
        g->cap_total = g->s_cap;
        rc = ensure_work(g);
        if (rc) return rc;
    }
    const size_t N = (size_t)g->n;
    CK(cudaMemcpyAsync(g->dg.state, g->s_state, N * 8, cudaMemcpyDeviceToDevice, s), "restore");
    CK(cudaMemcpyAsync(g->dg.rows, g->s_rows, N * sizeof(RowDesc), cudaMemcpyDeviceToDevice, s), "restore");
    CK(cudaMemcpyAsync(g->dg.sorted_len, g->s_sorted, N * 4, cudaMemcpyDeviceToDevice, s), "restore");
    CK(cudaMemcpyAsync(g->dg.adj, g->s_adj, (size_t)g->s_cap * 8, cudaMemcpyDeviceToDevice, s), "restore");
    if (g->s_twin)
        CK(cudaMemcpyAsync(g->dg.twin, g->s_twin, (size_t)g->s_cap * 4, cudaMemcpyDeviceToDevice, s), "restore");
    CK(cudaMemcpyAsync(g->d_spare, g->s_spare, sizeof(g->s_spare), cudaMemcpyHostToDevice, s), "restore");
    g->entries = g->s_entries;
    g->dead = g->s_dead;
    g->spare_top = (long long)g->s_spare[0];
    g->spare_lo = g->s_spare_lo;
    g->tails = g->s_tails;
    g->src = g->s_src;
    g->has_tree = g->s_has_tree;
    g->roots = g->s_roots;
    g->delta_ok = false;  // the tags name batches after the snapshot
    return DSSSP_OK;
}

int dsssp_graph_health(const dsssp_graph* g, int64_t* live_entries, int64_t* dead_entries, int64_t* spare_used,
                       int64_t* spare_total) {
    if (!g) return fail(DSSSP_E_INVAL, "graph_health: NULL graph");
    if (live_entries) *live_entries = g->entries;
    if (dead_entries) *dead_entries = g->dead;
    if (spare_used) *spare_used = g->spare_top - g->spare_lo;
    if (spare_total) *spare_total = g->cap_total - g->spare_lo;
    return DSSSP_OK;
}

int dsssp_graph_clear_range(dsssp_graph* g, int32_t first, int32_t count) {
    if (!g || first < 0 || count < 0 || (long long)first + count > g->n)
        return fail(DSSSP_E_INVAL, "clear_range: bad arguments");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "clear_range: a batch is still pending");
    if (count == 0) return DSSSP_OK;
    cudaStream_t s = g->stream;
    unsigned long long* d_out = nullptr;
    rc = dalloc(&d_out, 2, "range counters");
    if (rc) return rc;
    unsigned long long out[2] = {0, 0};
    const unsigned grid = (unsigned)(g->num_sms * 8);
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(out), s);
    if (e == cudaSuccess) {
        k_range_crossing<<<grid, kThreads, 0, s>>>(g->dg.rows, g->dg.adj, first, count, d_out);
        count_launch(1);
        e = cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && out[0] == 0) {
        k_range_clear<<<grid, kThreads, 0, s>>>(g->dg.state, g->dg.rows, g->dg.adj, first, count, d_out);
        count_launch(1);
        e = cudaMemcpyAsync(out, d_out, sizeof(out), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    dfree(d_out);
    if (e != cudaSuccess) return cuda_fail(e, "clear_range");
    if (out[0] != 0)
        return fail(DSSSP_E_INVAL, "clear_range: %llu live entries join [%d, %lld) to the rest of the graph", out[0],
                    first, (long long)first + count);
    g->entries -= (long long)out[1];
    g->dead += (long long)out[1];
    std::vector<int> keep;
    for (int r : g->roots)
        if (r < first || (long long)r >= (long long)first + count) keep.push_back(r);
    g->roots.swap(keep);
    if (g->src >= first && (long long)g->src < (long long)first + count) g->src = g->roots.empty() ? -1 : g->roots[0];
    g->delta_ok = false;
    return DSSSP_OK;
}

int dsssp_graph_compact(dsssp_graph* g) {
    if (!g) return fail(DSSSP_E_INVAL, "compact: NULL graph");
    int rc = set_device(g);
    if (rc) return rc;
    if (g->pending) return fail(DSSSP_E_INVAL, "compact: a batch is still pending");
    return repack(g, nullptr, 0, g->stream);
}

}  // extern "C"
