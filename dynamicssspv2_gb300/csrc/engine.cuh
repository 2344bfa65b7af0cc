// engine.cuh -- device data layout and primitives of the dynamic SSSP engine (sm_103a).
//
// Layout in HBM (one graph of n vertices):
//   state[n]      u64  (dist << 32) | parent      dist 0xFFFFFFFF = unreachable, parent
//                                                 0xFFFFFFFF = none; one atomicMin keeps
//                                                 distance and parent consistent
//   rows[n]       16 B {start, deg, cap}          row v = adj[start, start+deg), capacity cap
//   sorted_len[n] i32  length of the neighbour-sorted prefix of each row
//   adj[]         8 B  (col, wt) per directed entry; wt < 0 marks a deleted entry
//   twin[]        u32  per adjacency slot: slot of the reverse entry (v -> u for u -> v), so a
//                      deletion searches only the shorter of its two rows
//   inv_tag[n]    u32  batch epoch in which the vertex was cut off
//   push_tag[n]   u32  round tag of the last frontier push (de-duplication)
//   jm[n]         u32  pointer-jumping word (ancestor or terminal tag)
//   invq[n]       u32  vertices cut off directly by a deleted tree edge
//   work items    16 B (first slot, vertex, count): a pushed vertex of degree d becomes
//                      ceil(d/te) thread items of te edges, or, above large_deg, ceil(d/chunk)
//                      CTA items; an item names its adjacency slots itself, so processing it
//                      needs no row-descriptor load.  rt/rc = relaxation frontier (double
//                      buffer), it/ic = cut-off vertices
//   ctl           control block: grid barrier, status word, list counters, statistics, one
//                 128-byte line per group of fields that different CTAs hit at the same time
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace dsssp {

constexpr unsigned long long kInfState = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned kNone = 0xFFFFFFFFu;
constexpr unsigned long long kDistInf = 0xFFFFFFFFull;
constexpr unsigned kTagOk = 0xFFFFFFFFu;   // pointer jumping: reaches the root untouched
constexpr unsigned kTagInv = 0xFFFFFFFEu;  // pointer jumping: below a cut-off vertex
constexpr int kStatusOverflowPending = 1;  // internal: an insertion did not fit its row
constexpr unsigned kNoTwin = 0xFFFFFFFFu;   // twin not known yet (the other end overflowed)
constexpr unsigned long long kHashEmpty = 0xFFFFFFFFFFFFFFFFull;
constexpr int kHashNoWeight = -1;  // 0xFF byte fill; deletions with w < 0 are not hashed

// One slot of the batch's deletion set (endpoint pair, weight): one 16-byte sector.
struct __align__(16) DelSlot {
    unsigned long long pair;
    int w;
    int pad;
};

struct __align__(16) RowDesc {
    long long start;
    int deg;
    int cap;
};

enum StatIdx {
    ST_INS = 0,
    ST_DEL,
    ST_IGN,
    ST_ROOTS,
    ST_INV,
    ST_LEVELS,
    ST_PJ,
    ST_ROUNDS,
    ST_FRONTIER,
    ST_EDGES_RELAX,
    ST_EDGES_INV,
    ST_DEL_PROBED,
    ST_UPDATES,
    ST_OVF,
    ST_ITEMS,
    ST_DIST_OVF,
    ST_ADVANCES,
    ST_TOMBS,
    ST_LIVE_INS,
    ST_SEED_UPD,    // k_append: distance-lowering seed relaxations
    ST_SEED_FRONT,  // k_append: ends claimed for the first frontier (or the far list)
    ST_EDGES_PULL,  // adjacency entries scanned by the pulls of cut-off vertices
    ST_COUNT
};

// Device control block.  Everything from line 1 on is cleared before every batch.
struct __align__(128) Ctl {
    // line 0 (persistent)
    unsigned bar_gen;
    unsigned round_base;
    unsigned spin_limit;  // grid-barrier poll limit (0 = default); persistent, set by the host
    unsigned stall_us;    // test hook: the last CTA of k_update waits this long before its first barrier
    unsigned grp_gen;     // generation of the group barrier (the first group_ctas CTAs)
    unsigned pad0[27];
    // line 1
    int status;
    int ovf_count;
    unsigned inv_count;  // roots appended by k_delete
    unsigned killed;     // insertions removed by a deletion of the same batch
    unsigned seed_count;  // vertices k_append seeded into the first frontier
    unsigned pad1[27];
    // line 2
    unsigned bar_count;
    unsigned pad2[31];
    // line 2b: arrivals at the group barrier (its own line: the grid's CTAs poll bar_gen meanwhile)
    unsigned grp_count;
    unsigned pad2b[31];
    // line 3: relaxation lists, round r reads slot r%3
    unsigned rcT[3];
    unsigned rcC[3];
    unsigned pad3[26];
    // line 4: cut-off lists (level L appends to slot (L+1)%3), pointer jumping
    unsigned ltT[3];
    unsigned ltC[3];
    unsigned pjT;
    unsigned pjC;
    unsigned pjf[3];
    unsigned fc[2];  // near-far: far-list counts (double buffer)
    unsigned pad4[19];
    // line 4b: near-far threshold reduction (double buffer)
    unsigned long long fmin[2];
    // small steps run by CTA 0 alone hand their end state to the grid here
    unsigned long long solo[4];
    unsigned solo_n[2];  // list sizes of the first round after solo relaxation rounds
    unsigned pad4b[18];
    // line 5: barrier diagnostics (first timed-out barrier, arrivals then, CTAs that timed
    // out, max barrier count at exit, 0xFFFFFFFF - min barrier count at exit)
    unsigned diag[8];
    unsigned pad5[24];
    // lines 6-7
    unsigned long long stat[ST_COUNT];
    // line 8: %globaltimer stamps: 0 start, 1 after invalidation, 2 after seeding, 3 end
    unsigned long long ts[8];
    unsigned long long pad6[8];
};

// A work item: adjacency slots [lo, lo + cnt) of vertex v's row, as {lo low word, lo high
// word, v, cnt} (one 16-byte load).
using Item = uint4;

__device__ __forceinline__ Item make_item(unsigned v, long long lo, unsigned cnt) {
    return make_uint4((unsigned)lo, (unsigned)((unsigned long long)lo >> 32), v, cnt);
}
__device__ __forceinline__ long long item_lo(const Item& it) {
    return (long long)(((unsigned long long)it.y << 32) | it.x);
}

struct DevGraph {
    unsigned long long* state;
    RowDesc* rows;
    int* sorted_len;
    int2* adj;
    unsigned* twin;  // nullptr when the slot count does not fit 32 bits
    unsigned* inv_tag;
    unsigned* push_tag;
    unsigned* jm;
    unsigned* invq;
    Item* rt0;  // relaxation thread items, double buffer
    Item* rt1;
    Item* rc0;  // relaxation CTA items, double buffer
    Item* rc1;
    Item* it;   // cut-off vertices' thread items
    Item* ic;   // cut-off vertices' CTA items
    unsigned* far0;     // near-far: vertices whose distance is at or above the threshold
    unsigned* far1;
    unsigned* far_tag;  // far-list membership tag (de-duplication)
    unsigned* chg_tag;  // batch epoch of an equal-distance parent swap (changed-vertex set)
    long long tcap;
    long long ccap;
    long long cap_total;  // adjacency slots (bounds of twin-derived indices)
    Ctl* ctl;
    int n;
    int src;  // lowest root (informational; kernels treat any vertex that is its own parent as a root)
};

struct UpdParams {
    DevGraph g;
    const int4* chg;  // (u, v, w, op) records
    long long k;
    int* ins_state;   // per record: 1 = insertion that survives the batch
    DelSlot* hset;    // deletion set: endpoint pair -> weight (open addressing)
    unsigned long long hmask;
    int4* ovf;        // insertions that did not fit their row: (row, col, wt, record)
    long long* slot;  // per record, both directions: slot of the appended entry, -1 = overflowed
    unsigned epoch;
    int te;           // edges per thread item
    int large_deg;    // rows above this become CTA items
    int chunk;        // edges per CTA item
    int bfs_levels;
    int mode;         // 0 = batch update, 1 = from scratch (state already reset)
    unsigned long long delta;  // near-far bucket width; 0 = plain frontier relaxation
    unsigned* seedq;  // vertices seeded by k_append (claimed, expanded by k_update)
    const int* srcs;  // mode 1: the sources (every root is its own parent)
    int nsrc;
    long long max_rounds;
    unsigned solo_waves;  // steps of at most this many CTA-waves of items run on CTA 0 alone
    unsigned group_ctas;  // mid-size steps run on CTAs [0, group_ctas) with a group barrier (0 = off)
    unsigned group_waves; // ... a step is mid-size up to group_ctas * group_waves CTA-waves of items
    int warp_agg;         // 1 = warp-aggregated distance offers (one atomicMin per target and warp)
    int tails;            // 1 = rows may hold unsorted tails (k_delete scans long ones warp-wide)
};

// ---- memory-order helpers -------------------------------------------------------------

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void set_status(Ctl* ctl, int code) { atomicCAS(&ctl->status, 0, code); }

__device__ __forceinline__ unsigned long long dmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long dpair_key(unsigned a, unsigned b) {
    return a < b ? ((unsigned long long)a << 32) | b : ((unsigned long long)b << 32) | a;
}

// ---- warp helpers (must be called by all 32 lanes) -------------------------------------

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Appends val for every lane with pred set, one atomic per warp.
__device__ __forceinline__ void warp_append(bool pred, unsigned val, unsigned* list, unsigned* counter) {
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, pred);
    if (mask == 0) return;
    const unsigned lane = lane_id();
    const unsigned leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (pred) list[base + __popc(mask & ((1u << lane) - 1u))] = val;
}

// Adjacency entries are read once per push: streaming loads (evict-first in L1 and L2) keep
// the randomly accessed per-vertex arrays (state, row descriptors, tags) resident in L2.
__device__ __forceinline__ int2 ld_stream(const int2* a) { return __ldcs(a); }

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

}  // namespace dsssp
