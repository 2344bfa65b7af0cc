// engine.cuh -- device data layout and primitives of the dynamic SSSP engine (sm_103a).
//
// Layout in HBM (one graph):
//   state[n]      u64  (dist << 32) | parent      dist 0xFFFFFFFF = unreachable, parent
//                                                 0xFFFFFFFF = none; one atomicMin keeps
//                                                 distance and parent consistent
//   rows[n]       16 B {start, deg, cap}          row v = adj[start, start+deg), capacity cap
//   sorted_len[n] i32  length of the neighbour-sorted prefix of each row
//   adj[]         8 B  (col, wt) per directed entry; wt < 0 marks a deleted entry
//   inv_tag[n]    u32  batch epoch in which the vertex was cut off
//   push_tag[n]   u32  round tag of the last frontier push (de-duplication)
//   jm[n]         u32  pointer-jumping word (ancestor or terminal tag)
//   invq[n]       u32  every vertex cut off in this batch, in discovery order
//   q[2][n]       u32  frontier double buffer, h[2][n] heavy-vertex lists
//   ctl           control block: grid barrier, status word, queue counters, statistics
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
    ST_PUSHES,
    ST_DIST_OVF,
    ST_COUNT
};

// Device control block.  Fields from `status` on are cleared before every batch.
struct Ctl {
    unsigned bar_gen;
    unsigned round_base;
    unsigned pad0[2];
    // ---- cleared per batch ----
    int status;
    int ovf_count;
    unsigned bar_count;
    unsigned inv_count;
    unsigned cq[3];   // frontier counts (round r reads cq[r%3])
    unsigned ch[3];   // heavy-list counts of the relaxation rounds
    unsigned bh[3];   // heavy-list counts of the subtree walk
    unsigned ph;      // heavy-list count of the pull pass
    unsigned pjf[3];  // pointer-jumping "still moving" flags
    unsigned lc[3];   // subtree walk: vertices cut off during level L counted in lc[(L+1)%3]
    unsigned pj_cnt;  // vertices cut off by pointer jumping
    unsigned pad1[2];
    // barrier diagnostics: first timed-out barrier index, arrivals seen then, CTAs that timed
    // out, and per-CTA barrier counts at exit (max, 0xFFFFFFFF - min)
    unsigned diag[6];
    unsigned pad2[2];
    unsigned long long stat[ST_COUNT];
    unsigned long long ts[8];  // %globaltimer stamps: 0 start, 1 after invalidation,
                               // 2 after seeding, 3 end
};

struct DevGraph {
    unsigned long long* state;
    RowDesc* rows;
    int* sorted_len;
    int2* adj;
    unsigned* inv_tag;
    unsigned* push_tag;
    unsigned* jm;
    unsigned* invq;
    unsigned* q0;
    unsigned* q1;
    uint2* h0;  // heavy lists: (vertex, chunk index) work items
    uint2* h1;
    long long hcap;
    Ctl* ctl;
    int n;
    int src;
};

struct UpdParams {
    DevGraph g;
    const int4* chg;        // (u, v, w, op) records
    long long k;
    const long long* slot;  // per change: 2 adjacency indices of an inserted entry
    unsigned epoch;
    int small_deg;
    int large_deg;
    int chunk;
    int bfs_levels;
    int mode;  // 0 = batch update, 1 = from scratch (state already reset, src seeded)
    long long max_rounds;
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

// Appends cnt items (val, 0..cnt-1) for every lane with pred set, one atomic per warp.
// Returns false (and appends nothing) if the list would exceed cap.
__device__ __forceinline__ bool warp_append_chunks(bool pred, unsigned val, unsigned cnt, uint2* list,
                                                   unsigned* counter, long long cap) {
    unsigned c = pred ? cnt : 0u;
    const unsigned lane = lane_id();
    unsigned incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += t;
    }
    const unsigned total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (total == 0) return true;
    unsigned base = 0;
    if (lane == 31) base = atomicAdd(counter, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    if ((long long)base + total > cap) return false;
    const unsigned first = base + incl - c;
    for (unsigned k = 0; k < c; k++) list[first + k] = make_uint2(val, k);
    return true;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w < v ? w : v;
    }
    return v;
}

}  // namespace dsssp
