// update.cu -- the batch-update kernels of the dynamic SSSP engine (sm_103a).
//
// One batch (replaces SSSPmainForUndirected.cu:196-281) is four launches on one stream:
//   k_prepare   validate and count the change records
//   k_delete    the child end of a deleted tree edge is cut off and every adjacency entry
//               matching a deletion is tombstoned (binary search in the sorted row prefix +
//               scan of older appended entries); deletions also go into a device hash set
//               (replaces deleteEdge, gpuFunctions_undir.cuh:179-215)
//   k_append    insertions that no deletion of the batch removes go into row slack (atomic
//               degree bump, both directions).  The reference appends every insertion and
//               then tombstones matches (all_structure_undir.cuh:106-117 before
//               gpuFunctions_undir.cuh:201-213); skipping the removed ones gives the same graph.
//               Each surviving insertion then relaxes both ends and seeds the first frontier
//               (replaces insertEdge, gpuFunctions_undir.cuh:217-251)
//   k_update    one persistent cooperative kernel with a bounded grid barrier:
//               A. cut-off subtrees are walked level by level from the roots (replaces
//                  filterAffectedNodes + updateNeighbors_del and its host loop,
//                  gpuFunctions_undir.cuh:125-144, 312-349, MAIN:219-239); after bfs_levels
//                  levels it switches to pointer jumping over the parent array.  The walk
//                  follows the parent words as k_append left them, so an end relaxed from a
//                  vertex that turns out to be cut off is cut off with it.
//               B. every cut-off vertex pulls its best live neighbour
//               C. frontier relaxation rounds with 64-bit atomicMin on the packed
//                  (dist, parent) word until the frontier is empty (replaces
//                  filterAllAffected + updateNeighbors and its host loop,
//                  gpuFunctions_undir.cuh:162-174, 370-433, MAIN:263-281).  With a bucket
//                  width delta > 0 the rounds are near-far ordered: a vertex whose new
//                  distance is at or above the threshold T waits in a de-duplicated far list;
//                  when the near frontier runs dry, T moves to (least far distance) + delta
//                  and the far list is split again.  High-diameter graphs then settle most
//                  vertices once instead of once per improving wave.  The result is the same
//                  fixpoint: exact distances, the same parents.
// Load balance: a vertex entering a frontier is split by degree into work items -- rows of
// at most te edges are one thread's item, longer rows up to large_deg become ceil(deg/te)
// thread items (a warp's worth for a few hundred edges), longer ones become CTA items of
// `chunk` edges -- so every round is one even wave over all threads.
#include <cuda_runtime.h>

#include "engine.cuh"

namespace dsssp {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned kSpinLimit = 1u << 20;  // polls of ~1 us: a barrier gives up after ~1 s
constexpr int kMaxWarps = 8;               // update kernel blocks have at most 256 threads
constexpr int kBuf = 176;                  // per-warp push buffer entries (16 bytes each: four
                                           // CTAs of the update kernel stay within 100 KB of
                                           // shared memory, which leaves the L1 its 156 KB)
constexpr int kListRegion = 512;           // per-warp u32 staging of the batch front kernels
constexpr int kAddsPerCheck = 32;          // entries a warp may add between two flush checks
                                           // (one add of up to 32 lanes; visit4 reserves room
                                           // for its four adds instead)
static_assert(kBuf > kAddsPerCheck, "a push buffer must take one visit's adds after a check");
constexpr int kSoloSteps = 256;            // consecutive solo steps before the grid re-syncs

__shared__ unsigned s_nbar;        // grid barriers this CTA has passed
__shared__ unsigned s_gen;         // barrier generation this CTA waits on next (ctl->bar_gen)
__shared__ unsigned s_ggen;        // group-barrier generation this CTA waits on next (ctl->grp_gen)
// List counters of solo steps (CTA 0 alone): (thread items, CTA items) per slot, slots used
// like the control block's three rotating counters.  Shared-memory atomics and reads save a
// global round trip each per step.
__shared__ unsigned s_solo_cnt[3][2];
__shared__ unsigned s_spin_limit;  // polls before a grid barrier gives up
__shared__ uint4 s_pbuf[kMaxWarps][kBuf];  // (vertex, degree, row start) pushed, not yet expanded
__shared__ unsigned s_wlist[kMaxWarps][kListRegion];  // k_delete / k_append list staging

// Per-thread counters (32 bits: a thread's share stays far below 2^32 in any run; the block
// sums in flush_stats are 64-bit), few registers in the register-bound update kernel.
struct LocalStats {
    unsigned edges_relax = 0, edges_inv = 0, updates = 0, dist_ovf = 0, frontier = 0, items = 0, marked = 0,
             edges_pull = 0;
};

// Grid-wide barrier for a cooperative launch.  The wait is bounded: on timeout the status
// word gets DSSSP_E_TIMEOUT (with where it happened in ctl->diag) and every CTA leaves at
// its next barrier.  Returns false when the kernel must stop (timeout or any error).  Each
// CTA tracks the generation it waits on (s_gen, read once at kernel start: no barrier can
// complete before every CTA has arrived), so arriving costs no load.  With a and b given,
// the two counters the caller needs next are read once per CTA together with the status
// word and returned in va and vb.
__device__ bool grid_sync(Ctl* ctl, const unsigned* a, const unsigned* b, unsigned& va, unsigned& vb) {
    __shared__ int s_go;
    __shared__ unsigned s_va, s_vb;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = s_gen;
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->bar_count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            st_release(&ctl->bar_gen, gen + 1);
        } else {
            unsigned spins = 0;
            while (ld_acquire(&ctl->bar_gen) == gen) {
                if (++spins > s_spin_limit) {
                    if (atomicCAS(&ctl->status, 0, -6 /* DSSSP_E_TIMEOUT */) == 0) {
                        ctl->diag[0] = s_nbar;
                        ctl->diag[1] = atomicAdd(&ctl->bar_count, 0u);
                    }
                    atomicAdd(&ctl->diag[2], 1u);
                    break;
                }
                __nanosleep(spins < 32 ? 32 : (spins < 2048 ? 200 : 1000));  // long waits: solo steps
            }
        }
        __threadfence();
        s_gen = gen + 1;
        s_nbar++;
        const int st = __ldcg(&ctl->status);
        s_va = a ? __ldcg(a) : 0u;
        s_vb = b ? __ldcg(b) : 0u;
        s_go = st == 0;
    }
    __syncthreads();
    va = s_va;
    vb = s_vb;
    return s_go != 0;
}

// Barrier of the first G CTAs (a group running mid-size steps while the others wait at the
// next grid barrier): like grid_sync, bounded, with the counters the caller needs next read
// once per CTA after the release.  Every CTA of the group calls it the same number of times.
__device__ bool group_sync(Ctl* ctl, unsigned G, const unsigned* a, const unsigned* b, unsigned& va, unsigned& vb) {
    __shared__ int s_go;
    __shared__ unsigned s_va, s_vb;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = s_ggen;
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->grp_count, 1u);
        if (arrived == G - 1) {
            atomicExch(&ctl->grp_count, 0u);
            __threadfence();
            st_release(&ctl->grp_gen, gen + 1);
        } else {
            unsigned spins = 0;
            while (ld_acquire(&ctl->grp_gen) == gen) {
                if (++spins > s_spin_limit) {
                    if (atomicCAS(&ctl->status, 0, -6 /* DSSSP_E_TIMEOUT */) == 0) {
                        ctl->diag[0] = 0x80000000u | s_nbar;  // high bit: a group barrier
                        ctl->diag[1] = atomicAdd(&ctl->grp_count, 0u);
                    }
                    atomicAdd(&ctl->diag[2], 1u);
                    break;
                }
                if (spins > 32) __nanosleep(spins < 4096 ? 64 : 1000);
            }
        }
        __threadfence();
        s_ggen = gen + 1;
        const int st = __ldcg(&ctl->status);
        s_va = __ldcg(a);
        s_vb = __ldcg(b);
        s_go = st == 0;
    }
    __syncthreads();
    va = s_va;
    vb = s_vb;
    return s_go != 0;
}

__device__ __forceinline__ bool grid_sync(Ctl* ctl) {
    unsigned x, y;
    return grid_sync(ctl, nullptr, nullptr, x, y);
}

// Offers distance nd through parent u to vertex c whose current word is cur.  Returns true
// when c's distance went down (c must then be pushed).  Zero-weight edges only replace a
// strictly larger distance, so equal-distance parent swaps can never close a cycle.  A swap
// to a smaller parent id at the same distance (the packed minimum's tie rule) is recorded in
// chg_tag, so the batch's set of changed vertices stays complete.
__device__ __forceinline__ bool relax_to(const DevGraph& g, unsigned epoch, unsigned c, unsigned long long nd,
                                         unsigned u, int w, unsigned long long cur, LocalStats& ls) {
    unsigned long long* state = g.state;
    if (nd >= kDistInf) {
        if (cur == kInfState) ls.dist_ovf++;
        return false;
    }
    const unsigned long long cand = (nd << 32) | u;
    if (cand >= cur) return false;
    if (w > 0) {
        const unsigned long long old = atomicMin(&state[c], cand);
        if ((old >> 32) > nd) {
            ls.updates++;
            return true;
        }
        if (old > cand && g.chg_tag) g.chg_tag[c] = epoch;
        return false;
    }
    while ((cur >> 32) > nd) {
        const unsigned long long prev = atomicCAS(&state[c], cur, cand);
        if (prev == cur) {
            ls.updates++;
            return true;
        }
        cur = prev;
    }
    return false;
}

// The two seed relaxations of an insertion (u, v, w) with w > 0: v is offered ndv = d(u) + w
// through u and u is offered ndu = d(v) + w through v, from the states su, sv read before.
// Both atomicMin go out before either result is used; the outcome is that of two relax_to
// calls.  pu / pv: u / v went down and must be pushed.
__device__ __forceinline__ void relax_both(const DevGraph& g, unsigned epoch, unsigned u, unsigned v,
                                           unsigned long long ndv, unsigned long long ndu, unsigned long long su,
                                           unsigned long long sv, bool& pu, bool& pv, LocalStats& ls) {
    const bool from_u = (su >> 32) != kDistInf, from_v = (sv >> 32) != kDistInf;
    if (from_u && ndv >= kDistInf && sv == kInfState) ls.dist_ovf++;
    if (from_v && ndu >= kDistInf && su == kInfState) ls.dist_ovf++;
    const unsigned long long cv = (ndv << 32) | u, cu = (ndu << 32) | v;
    const bool tv = from_u && ndv < kDistInf && cv < sv;
    const bool tu = from_v && ndu < kDistInf && cu < su;
    const unsigned long long ov = tv ? atomicMin(&g.state[v], cv) : kInfState;
    const unsigned long long ou = tu ? atomicMin(&g.state[u], cu) : kInfState;
    pv = tv && (ov >> 32) > ndv;
    pu = tu && (ou >> 32) > ndu;
    ls.updates += (pv ? 1 : 0) + (pu ? 1 : 0);
    if (g.chg_tag) {
        if (tv && !pv && ov > cv) g.chg_tag[v] = epoch;
        if (tu && !pu && ou > cu) g.chg_tag[u] = epoch;
    }
}

// Destination of pushed vertices: a thread-item list and a CTA-item list with counters.
struct Out {
    Item* tl;
    unsigned* tcnt;
    long long tcap;
    Item* cl;
    unsigned* ccnt;
    long long ccap;
};

// Work items of the entries a lane holds in a push buffer (entries lane, lane + 32, ...).
__device__ __forceinline__ void buf_counts(const uint4* buf, int count, const UpdParams& p, unsigned& nt,
                                           unsigned& nc) {
    nt = nc = 0;
    for (int e = (int)lane_id(); e < count; e += 32) {
        const int deg = (int)buf[e].y;
        if (deg > p.large_deg) nc += (unsigned)((deg + p.chunk - 1) / p.chunk);
        else if (deg > 0) nt += (unsigned)((deg + p.te - 1) / p.te);
    }
}

// Writes those items from list positions ft (thread items) and fc (CTA items) on.
__device__ __forceinline__ void buf_write(const uint4* buf, int count, const UpdParams& p, const Out& o, unsigned ft,
                                          unsigned fc) {
    for (int e = (int)lane_id(); e < count; e += 32) {
        const uint4 x = buf[e];
        const int deg = (int)x.y;
        const long long start = (long long)(((unsigned long long)x.w << 32) | x.z);
        if (deg > p.large_deg) {
            for (int k = 0; k < deg; k += p.chunk) o.cl[fc++] = make_item(x.x, start + k, (unsigned)min(p.chunk, deg - k));
        } else if (deg > 0) {
            for (int k = 0; k < deg; k += p.te) o.tl[ft++] = make_item(x.x, start + k, (unsigned)min(p.te, deg - k));
        }
    }
}

__device__ __forceinline__ unsigned warp_incl_scan(unsigned x) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(kFull, x, o);
        if (lane_id() >= (unsigned)o) x += t;
    }
    return x;
}

// Per-warp shared-memory buffer of pushed (vertex, degree, row start).  Entries are split into work
// items when the buffer is nearly full (one list-counter atomic per warp for up to kBuf
// vertices) and at the end of a phase (one atomic per CTA): the list counters are single
// words that every CTA appends to, so their atomics are kept few.
struct PushBuf {
    uint4* buf;
    int count;  // warp-uniform

    // pushes v with its row (start, deg) for every lane with pred
    __device__ __forceinline__ void add(bool pred, unsigned v, const RowDesc& rd) {
        const unsigned mask = __ballot_sync(kFull, pred);
        if (pred)
            buf[count + __popc(mask & ((1u << lane_id()) - 1u))] =
                make_uint4(v, (unsigned)rd.deg, (unsigned)rd.start, (unsigned)((unsigned long long)rd.start >> 32));
        count += __popc(mask);
        __syncwarp();
    }

    // warp-collective: expands the buffer once it could not take another kAddsPerCheck
    __device__ __forceinline__ void flush(const UpdParams& p, const Out& o, LocalStats& ls) {
        if (count <= kBuf - kAddsPerCheck) return;
        expand_all(p, o, ls);
    }

    // warp-collective: makes room for n more entries (n warp-uniform, at most kBuf)
    __device__ __forceinline__ void reserve(unsigned n, const UpdParams& p, const Out& o, LocalStats& ls) {
        if ((unsigned)count + n <= (unsigned)kBuf) return;
        expand_all(p, o, ls);
    }

    // warp-collective: splits every buffered entry into work items (one atomic per list)
    __device__ __forceinline__ void expand_all(const UpdParams& p, const Out& o, LocalStats& ls) {
        unsigned nt, nc;
        buf_counts(buf, count, p, nt, nc);
        const unsigned it = warp_incl_scan(nt), ic = warp_incl_scan(nc);
        const unsigned tt = __shfl_sync(kFull, it, 31), tc = __shfl_sync(kFull, ic, 31);
        unsigned bt = 0, bc = 0;
        if (lane_id() == 0) {
            if (tt) bt = atomicAdd(o.tcnt, tt);
            if (tc) bc = atomicAdd(o.ccnt, tc);
        }
        bt = __shfl_sync(kFull, bt, 0);
        bc = __shfl_sync(kFull, bc, 0);
        if ((long long)bt + tt > o.tcap || (long long)bc + tc > o.ccap) {
            if (lane_id() == 0) set_status(p.g.ctl, -4 /* work list capacity: internal error */);
        } else {
            buf_write(buf, count, p, o, bt + it - nt, bc + ic - nc);
        }
        ls.items += nt + nc;
        count = 0;
        __syncwarp();
    }

    // CTA-collective (every thread of the CTA): expands what every warp still holds
    __device__ void flush_cta(const UpdParams& p, const Out& o, LocalStats& ls) {
        __shared__ unsigned s_t[kMaxWarps], s_c[kMaxWarps], s_bt, s_bc, s_ok;
        const unsigned w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        unsigned nt, nc;
        buf_counts(buf, count, p, nt, nc);
        const unsigned it = warp_incl_scan(nt), ic = warp_incl_scan(nc);
        if (lane_id() == 31) {
            s_t[w] = it;
            s_c[w] = ic;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tt = 0, tc = 0;
            for (unsigned k = 0; k < nw; k++) {
                const unsigned a = s_t[k], b = s_c[k];
                s_t[k] = tt;
                s_c[k] = tc;
                tt += a;
                tc += b;
            }
            s_bt = tt ? atomicAdd(o.tcnt, tt) : 0u;
            s_bc = tc ? atomicAdd(o.ccnt, tc) : 0u;
            s_ok = (long long)s_bt + tt <= o.tcap && (long long)s_bc + tc <= o.ccap;
            if (!s_ok) set_status(p.g.ctl, -4 /* work list capacity: internal error */);
        }
        __syncthreads();
        if (s_ok) buf_write(buf, count, p, o, s_bt + s_t[w] + it - nt, s_bc + s_c[w] + ic - nc);
        ls.items += nt + nc;
        count = 0;
        __syncthreads();
    }
};

// Claims c for the next frontier; its row descriptor (for the work items) is loaded alongside
// the claim.
__device__ __forceinline__ bool claim_with_row(const UpdParams& p, bool want, unsigned c, unsigned tag, RowDesc& rd) {
    rd = RowDesc{0, 0, 0};
    if (!want) return false;
    const RowDesc r = p.g.rows[c];
    const bool won = atomicExch(&p.g.push_tag[c], tag) != tag;
    rd = r;
    return won;
}

// The row descriptor of v when pred holds (an empty row otherwise).
__device__ __forceinline__ RowDesc row_if(const UpdParams& p, bool pred, unsigned v) {
    return pred ? p.g.rows[v] : RowDesc{0, 0, 0};
}

// Near-far ordering: pushes whose new distance is at or above the threshold T go to a far
// list, each vertex at most once per list generation (far_tag).  T = ~0 turns it off.
struct Far {
    unsigned* list;
    unsigned* cnt;
    unsigned* tag;
    unsigned gen;
    unsigned cap;
    unsigned long long T;
};

// Appends c to the far list for every lane with pred (warp-collective).
__device__ __forceinline__ void far_push(const UpdParams& p, const Far& f, bool pred, unsigned c) {
    if (pred) pred = atomicExch(&f.tag[c], f.gen) != f.gen;
    const unsigned mask = __ballot_sync(kFull, pred);
    if (mask == 0) return;
    const unsigned lane = lane_id();
    const unsigned leader = __ffs(mask) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(f.cnt, (unsigned)__popc(mask));
    base = __shfl_sync(kFull, base, leader);
    if ((unsigned long long)base + __popc(mask) > f.cap) {  // cannot happen: one entry per vertex
        if (lane == leader) set_status(p.g.ctl, -4);
        return;
    }
    if (pred) f.list[base + __popc(mask & ((1u << lane) - 1u))] = c;
}

// Appends c[q] for every pred[q] of every lane to the far list with one atomic per warp
// (warp-collective; the far tags are already claimed).
__device__ __forceinline__ void far_append4(const UpdParams& p, const Far& f, const bool (&pred)[4],
                                            const unsigned (&c)[4]) {
    unsigned cnt = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) cnt += pred[q] ? 1u : 0u;
    if (!__any_sync(kFull, cnt != 0)) return;
    const unsigned incl = warp_incl_scan(cnt);
    const unsigned total = __shfl_sync(kFull, incl, 31);
    unsigned base = 0;
    if (lane_id() == 31) base = atomicAdd(f.cnt, total);
    base = __shfl_sync(kFull, base, 31);
    if ((unsigned long long)base + total > f.cap) {  // cannot happen: one entry per vertex
        if (lane_id() == 31) set_status(p.g.ctl, -4);
        return;
    }
    unsigned at = base + incl - cnt;
#pragma unroll
    for (int q = 0; q < 4; q++)
        if (pred[q]) f.list[at++] = c[q];
}

// Warp-aggregated offers: lanes offering to the same vertex c (offer set) are grouped with
// __match_any_sync; the group's least candidate word goes to its lowest lane (lead), the only
// one that issues the atomicMin, so a vertex offered by several lanes of a warp takes one
// atomic instead of one per lane.  Warp-collective; the loop runs (largest group - 1) times.
__device__ __forceinline__ void warp_agg_min(bool offer, unsigned c, unsigned long long& best, bool& lead) {
    const unsigned lane = lane_id();
    if (!__any_sync(kFull, offer)) return;
    // lanes without an offer get keys no vertex id takes (ids are below 2^31)
    const unsigned grp = __match_any_sync(kFull, offer ? c : 0x80000000u | lane);
    unsigned rem = grp & ~(1u << lane);
    while (__any_sync(kFull, rem != 0)) {
        const int src = rem ? __ffs(rem) - 1 : (int)lane;
        const unsigned long long o = __shfl_sync(kFull, best, src);
        best = o < best ? o : best;
        rem &= rem - 1;
    }
    lead = offer && (__ffs(grp) - 1) == (int)lane;
}

// ---- per-edge operations ---------------------------------------------------------------
// visit4 handles up to four adjacency entries per lane and is called by all 32 lanes.

template <bool kAgg>
struct RelaxOp {
    const UpdParams* p;
    unsigned tag;
    Out out;
    PushBuf pb;
    LocalStats* ls;
    Far far;
    // Offer by atomicMin alone, without first loading the neighbour's state to skip offers
    // that cannot win: one memory latency less per item, one atomic per edge instead of per
    // winning edge.  Used for steps of at most one wave of items, which wait on latency.
    bool direct;

    __device__ __forceinline__ unsigned long long prep(unsigned v) const { return __ldcg(&p->g.state[v]) >> 32; }
    __device__ __forceinline__ bool skip(unsigned long long du) const { return du >= kDistInf; }
    __device__ __forceinline__ void begin_lane(unsigned) {}
    __device__ __forceinline__ void end_lane(unsigned, bool) {}
    __device__ __forceinline__ void begin_group(unsigned) {}
    __device__ __forceinline__ void end_group(unsigned) {}
    __device__ __forceinline__ void finish() { pb.flush_cta(*p, out, *ls); }

    __device__ __forceinline__ void visit4(unsigned u, unsigned long long du, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        unsigned long long* state = p->g.state;
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? ld_stream(&p->g.adj[j[q]]) : make_int2(0, -1);
        unsigned long long cur[4];
#pragma unroll
        for (int q = 0; q < 4; q++) cur[q] = e[q].y >= 0 && !direct ? __ldcg(&state[e[q].x]) : kInfState;
        // The lane's four offers go out before any result is used, then its claims: two
        // memory latencies for the four edges instead of two per improving edge.  The
        // adjacency loads above were issued alongside the load of du (an unreachable u offers
        // nothing).
        const bool live = du < kDistInf;
        bool push[4], later[4];
        if constexpr (!kAgg) {
            unsigned long long old[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned long long nd = du + (unsigned)e[q].y;
                const bool offer = live && e[q].y > 0 && nd < kDistInf && ((nd << 32) | u) < cur[q];
                if (live && e[q].y > 0 && nd >= kDistInf &&
                    (direct ? __ldcg(&state[e[q].x]) : cur[q]) == kInfState)
                    ls->dist_ovf++;
                old[q] = offer ? atomicMin(&state[e[q].x], (nd << 32) | u) : 0ull;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned long long nd = du + (unsigned)e[q].y;
                const unsigned long long cand = (nd << 32) | u;
                push[q] = false;
                if (live && e[q].y > 0 && nd < kDistInf && cand < cur[q]) {
                    push[q] = (old[q] >> 32) > nd;
                    if (push[q]) ls->updates++;
                    else if (old[q] > cand && p->g.chg_tag) p->g.chg_tag[e[q].x] = p->epoch;
                } else if (live && e[q].y == 0) {  // zero weight: strict improvements only (compare-and-swap)
                    push[q] = relax_to(p->g, p->epoch, (unsigned)e[q].x, nd, u, 0,
                                       direct ? __ldcg(&state[e[q].x]) : cur[q], *ls);
                }
                later[q] = push[q] && nd >= far.T;
            }
        } else {
            // the lanes' offers to one vertex are reduced in the warp first: only the group's
            // least candidate word is issued, by the group's lowest lane
            unsigned long long old[4], best[4];
            bool lead[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned long long nd = du + (unsigned)e[q].y;
                const bool offer = live && e[q].y > 0 && nd < kDistInf && ((nd << 32) | u) < cur[q];
                if (live && e[q].y > 0 && nd >= kDistInf &&
                    (direct ? __ldcg(&state[e[q].x]) : cur[q]) == kInfState)
                    ls->dist_ovf++;
                best[q] = offer ? (nd << 32) | u : kInfState;
                lead[q] = offer;
                warp_agg_min(offer, (unsigned)e[q].x, best[q], lead[q]);
                old[q] = lead[q] ? atomicMin(&state[e[q].x], best[q]) : 0ull;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned long long nd = best[q] >> 32;  // the group's least distance
                push[q] = false;
                if (lead[q]) {
                    push[q] = (old[q] >> 32) > nd;
                    if (push[q]) ls->updates++;
                    else if (old[q] > best[q] && p->g.chg_tag) p->g.chg_tag[e[q].x] = p->epoch;
                } else if (live && e[q].y == 0) {  // zero weight: strict improvements only (compare-and-swap)
                    push[q] = relax_to(p->g, p->epoch, (unsigned)e[q].x, du, u, 0,
                                       direct ? __ldcg(&state[e[q].x]) : cur[q], *ls);
                }
                later[q] = push[q] && (e[q].y == 0 ? du : nd) >= far.T;
            }
        }
        unsigned ftag[4], ctag[4];
        RowDesc rd[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const unsigned c = (unsigned)e[q].x;
            const bool want = push[q] && !later[q];
            ftag[q] = later[q] ? atomicExch(&far.tag[c], far.gen) : far.gen;
            rd[q] = row_if(*p, want, c);
            ctag[q] = want ? atomicExch(&p->g.push_tag[c], tag) : tag;
        }
        bool fl[4], doit[4];
        unsigned fc[4], nadd = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            fl[q] = later[q] && ftag[q] != far.gen;
            fc[q] = (unsigned)e[q].x;
            doit[q] = push[q] && !later[q] && ctag[q] != tag;
            nadd += __popc(__ballot_sync(kFull, doit[q]));
        }
        pb.reserve(nadd, *p, out, *ls);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            ls->frontier += doit[q] ? 1 : 0;
            pb.add(doit[q], (unsigned)e[q].x, rd[q]);
            ls->edges_relax += ok[q] && live ? 1 : 0;
        }
        far_append4(*p, far, fl, fc);
    }
};

struct MarkOp {
    const UpdParams* p;
    Out out;
    PushBuf pb;
    LocalStats* ls;

    __device__ __forceinline__ unsigned long long prep(unsigned) const { return 0; }
    __device__ __forceinline__ bool skip(unsigned long long) const { return false; }
    __device__ __forceinline__ void begin_lane(unsigned) {}
    __device__ __forceinline__ void end_lane(unsigned, bool) {}
    __device__ __forceinline__ void begin_group(unsigned) {}
    __device__ __forceinline__ void end_group(unsigned) {}
    __device__ __forceinline__ void finish() { pb.flush_cta(*p, out, *ls); }

    __device__ __forceinline__ void visit4(unsigned x, unsigned long long, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        unsigned long long* state = p->g.state;
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? ld_stream(&p->g.adj[j[q]]) : make_int2(0, -1);
        unsigned long long s[4];
#pragma unroll
        for (int q = 0; q < 4; q++) s[q] = e[q].y >= 0 ? __ldcg(&state[e[q].x]) : kInfState;
        // a child is cut off even when already tagged: a root that an insertion of this batch
        // re-parented onto a vertex of a cut-off subtree must lose that distance.  The four
        // tag exchanges and degree loads go out before any result is used.
        unsigned old[4];
        RowDesc rd[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const unsigned c = (unsigned)e[q].x;
            const bool child = e[q].y >= 0 && (unsigned)s[q] == x;
            if (child) state[c] = kInfState;
            old[q] = child ? atomicExch(&p->g.inv_tag[c], p->epoch) : p->epoch;
            rd[q] = row_if(*p, child, c);
        }
        unsigned nadd = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) nadd += __popc(__ballot_sync(kFull, old[q] != p->epoch));
        pb.reserve(nadd, *p, out, *ls);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const bool mark = old[q] != p->epoch;
            ls->marked += mark ? 1 : 0;
            pb.add(mark, (unsigned)e[q].x, rd[q]);
            ls->edges_inv += ok[q] ? 1 : 0;
        }
    }
};

struct PullOp {
    const UpdParams* p;
    unsigned tag;
    Out out;
    PushBuf pb;
    LocalStats* ls;
    Far far;
    unsigned long long best;
    bool need;

    // pushes x (pred) to the next round or, at or above the threshold, to the far list; d is
    // x's distance when the caller knows it (its own lowering atomicMin), else kDistInf
    __device__ __forceinline__ void route(bool pred, unsigned x, unsigned long long d) {
        const bool later = pred && far.T != ~0ull && (d < kDistInf ? d : __ldcg(&p->g.state[x]) >> 32) >= far.T;
        far_push(*p, far, later, x);
        RowDesc rd;
        const bool doit = claim_with_row(*p, pred && !later, x, tag, rd);
        ls->frontier += doit ? 1 : 0;
        pb.add(doit, x, rd);
        pb.flush(*p, out, *ls);
    }

    __device__ __forceinline__ unsigned long long prep(unsigned) const { return 0; }
    __device__ __forceinline__ bool skip(unsigned long long) const { return false; }
    __device__ __forceinline__ void begin_lane(unsigned) { best = kInfState; need = false; }
    __device__ __forceinline__ void begin_group(unsigned) { best = kInfState; need = false; }
    __device__ __forceinline__ void finish() { pb.flush_cta(*p, out, *ls); }

    __device__ __forceinline__ void visit4(unsigned x, unsigned long long, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        unsigned long long* state = p->g.state;
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? ld_stream(&p->g.adj[j[q]]) : make_int2(0, -1);
        unsigned long long s[4];
#pragma unroll
        for (int q = 0; q < 4; q++) s[q] = e[q].y >= 0 ? __ldcg(&state[e[q].x]) : kInfState;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            ls->edges_pull += ok[q] ? 1 : 0;
            if (e[q].y < 0 || s[q] == kInfState) continue;
            const unsigned long long nd = (s[q] >> 32) + (unsigned)e[q].y;
            if (nd >= kDistInf) {
                ls->dist_ovf++;
                continue;
            }
            if (e[q].y > 0) {
                const unsigned long long cand = (nd << 32) | (unsigned)e[q].x;
                best = cand < best ? cand : best;
            } else if (relax_to(p->g, p->epoch, x, nd, (unsigned)e[q].x, 0, __ldcg(&state[x]), *ls)) {
                need = true;
            }
        }
    }
    // a lane's own item
    __device__ __forceinline__ void end_lane(unsigned x, bool valid) {
        bool improved = false;
        if (valid && best != kInfState) {
            const unsigned long long old = atomicMin(&p->g.state[x], best);
            if ((old >> 32) > (best >> 32)) {
                improved = true;
                ls->updates++;
            }
        }
        route(valid && (need || improved), x, improved ? best >> 32 : kDistInf);
    }
    // an item shared by the warp (part of a CTA item)
    __device__ __forceinline__ void end_group(unsigned x) {
        const unsigned long long b = warp_min_u64(best);
        const bool nd = __any_sync(kFull, need);
        bool improved = false;
        if (lane_id() == 0 && b != kInfState) {
            const unsigned long long old = atomicMin(&p->g.state[x], b);
            if ((old >> 32) > (b >> 32)) {
                improved = true;
                ls->updates++;
            }
        }
        route(lane_id() == 0 && (nd || improved), x, improved ? b >> 32 : kDistInf);
    }
};

// A step of nt thread items and nc CTA items is small when CTA 0 alone finishes it in at most
// `solo` waves (opts.solo_waves, default 2): then it skips the grid barrier, whose cost (~2.5 us
// plus the wait for the slowest CTA) exceeds the work.  solo 0: every step runs on the grid.
__device__ __forceinline__ bool small_step(unsigned nt, unsigned nc, unsigned solo) {
    return solo > 0 && (nt + blockDim.x - 1) / blockDim.x + nc <= solo;
}

// A step is mid-size when the group (the first G CTAs) finishes it in at most p.group_waves
// waves: it runs there with the group barrier, shorter than the grid's and waiting for the
// slowest of G chains instead of all CTAs'.
__device__ __forceinline__ bool group_step(const UpdParams& p, unsigned nt, unsigned nc) {
    const unsigned G = p.group_ctas;
    if (G < 2 || G >= gridDim.x || small_step(nt, nc, p.solo_waves)) return false;
    return (unsigned long long)(nt + blockDim.x - 1) / blockDim.x + nc <= (unsigned long long)G * p.group_waves;
}

// Processes one step's work on ncta CTAs (the whole grid, or CTA 0 alone for a small step;
// this CTA is number cta of them): CTA items first (one CTA per chunk of a long row; CTA
// items cta, cta + ncta, ...), then thread items (te edges each) in one grid-stride wave over
// the ncta CTAs' threads.
template <class Op>
__device__ void run_items(Op& op, const UpdParams& p, const Item* tl, unsigned nt, const Item* cl, unsigned nc,
                          unsigned cta, unsigned ncta) {
    const unsigned lane = lane_id();
    const unsigned gtid = cta * blockDim.x + threadIdx.x;
    const unsigned nthreads = ncta * blockDim.x;
    for (unsigned t = cta; t < nc; t += ncta) {
        const Item it = __ldcg(&cl[t]);
        const unsigned long long du = __shfl_sync(kFull, op.prep(it.z), 0);
        if (op.skip(du)) continue;
        const long long lo = item_lo(it), hi = lo + (long long)it.w;
        op.begin_group(it.z);
        for (long long b = lo; b < hi; b += 4LL * blockDim.x) {
            long long j[4];
            bool ok[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                j[q] = b + (long long)q * blockDim.x + threadIdx.x;
                ok[q] = j[q] < hi;
            }
            op.visit4(it.z, du, j, ok);
        }
        op.end_group(it.z);
    }
    // thread items: the item names its slots, so the adjacency loads go out alongside the
    // load of the vertex's own state (prep)
    for (unsigned base = gtid - lane; base < nt; base += nthreads) {
        const unsigned i = base + lane;
        const bool has = i < nt;
        const Item it = has ? __ldcg(&tl[i]) : make_uint4(0u, 0u, 0u, 0u);
        const unsigned long long du = has ? op.prep(it.z) : kDistInf;
        const long long lo = item_lo(it);
        const int cnt = (int)it.w;
        op.begin_lane(it.z);
        for (int b = 0; b < p.te; b += 4) {  // warp-uniform trip count (visit4 is warp-collective)
            long long j[4];
            bool ok[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                ok[q] = b + q < cnt;
                j[q] = lo + b + q;
            }
            op.visit4(it.z, du, j, ok);
        }
        op.end_lane(it.z, has && !op.skip(du));
    }
    op.finish();
}

// Block-reduced statistics: one atomic per block and counter.
__device__ void flush_stats(Ctl* ctl, const LocalStats& ls) {
    __shared__ unsigned long long s_acc[8];
    if (threadIdx.x < 8) s_acc[threadIdx.x] = 0;
    __syncthreads();
    const unsigned long long v[8] = {ls.edges_relax, ls.edges_inv, ls.updates, ls.dist_ovf,
                                     ls.frontier, ls.items, ls.marked, ls.edges_pull};
#pragma unroll
    for (int s = 0; s < 8; s++) {
        const unsigned long long x = warp_sum_u64(v[s]);
        if (lane_id() == 0 && x) atomicAdd(&s_acc[s], x);
    }
    __syncthreads();
    const int idx[8] = {ST_EDGES_RELAX, ST_EDGES_INV, ST_UPDATES, ST_DIST_OVF, ST_FRONTIER, ST_ITEMS, ST_INV,
                        ST_EDGES_PULL};
    if (threadIdx.x < 8 && s_acc[threadIdx.x]) atomicAdd(&ctl->stat[idx[threadIdx.x]], s_acc[threadIdx.x]);
}

__device__ void block_max(unsigned long long* dst, unsigned long long x) {
    __shared__ unsigned long long s_max;
    __syncthreads();
    if (threadIdx.x == 0) s_max = 0;
    __syncthreads();
    x = warp_max_u64(x);
    if (lane_id() == 0 && x) atomicMax(&s_max, x);
    __syncthreads();
    if (threadIdx.x == 0 && s_max) atomicMax(dst, s_max);
}

__device__ void block_add(unsigned long long* dst, unsigned long long x) {
    __shared__ unsigned long long s_sum;
    __syncthreads();
    if (threadIdx.x == 0) s_sum = 0;
    __syncthreads();
    x = warp_sum_u64(x);
    if (lane_id() == 0 && x) atomicAdd(&s_sum, x);
    __syncthreads();
    if (threadIdx.x == 0 && s_sum) atomicAdd(dst, s_sum);
}

// Per-warp staging of appends to a plain u32 list.  A warp writes its region of shared memory
// and appends it to the list with one atomic when the region is nearly full; at the end the
// CTA appends what its warps still hold with one atomic (flush_cta).  The list counters are
// single words that every CTA hits, so their atomics are kept few, and no CTA-wide barrier
// is needed while the warps work.
struct WarpList {
    unsigned* buf;  // this warp's region of shared memory
    int cap;        // entries in the region
    int count;      // warp-uniform

    __device__ __forceinline__ void add(bool pred, unsigned v) {
        const unsigned mask = __ballot_sync(kFull, pred);
        if (pred) buf[count + __popc(mask & ((1u << lane_id()) - 1u))] = v;
        count += __popc(mask);
        __syncwarp();
    }

    // warp-collective: appends the region once fewer than `room` entries are free
    __device__ __forceinline__ void flush(unsigned* list, unsigned* counter, unsigned list_cap, int room, Ctl* ctl) {
        if (count + room <= cap) return;
        unsigned b = 0;
        if (lane_id() == 0) b = atomicAdd(counter, (unsigned)count);
        b = __shfl_sync(kFull, b, 0);
        if ((unsigned long long)b + (unsigned)count > list_cap) {
            if (lane_id() == 0) set_status(ctl, -4 /* list capacity: internal error */);
        } else {
            for (int j = (int)lane_id(); j < count; j += 32) list[b + j] = buf[j];
        }
        count = 0;
        __syncwarp();
    }

    // CTA-collective (every thread of the CTA)
    __device__ void flush_cta(unsigned* list, unsigned* counter, unsigned list_cap, Ctl* ctl) {
        __shared__ unsigned s_off[kMaxWarps], s_base, s_ok;
        const unsigned w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane_id() == 0) s_off[w] = (unsigned)count;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (unsigned k = 0; k < nw; k++) {
                const unsigned c = s_off[k];
                s_off[k] = t;
                t += c;
            }
            s_base = t ? atomicAdd(counter, t) : 0u;
            s_ok = (unsigned long long)s_base + t <= list_cap;
            if (!s_ok) set_status(ctl, -4 /* list capacity: internal error */);
        }
        __syncthreads();
        if (s_ok)
            for (int j = (int)lane_id(); j < count; j += 32) list[s_base + s_off[w] + j] = buf[j];
        count = 0;
        __syncthreads();
    }
};

// ---- row search and the deletion set -------------------------------------------------------

// First index in adj[lo, hi) whose column is >= c (the prefix is sorted by column).
__device__ __forceinline__ long long lower_col(const int2* adj, long long lo, long long hi, int c) {
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (adj[mid].x < c) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Inserts (pair, w) into the open-addressing deletion set.  Probing depends only on the pair;
// a slot whose pair matches but whose weight is taken by another weight is skipped.
__device__ bool hash_insert(const UpdParams& p, unsigned long long pair, int w) {
    unsigned long long h = dmix64(pair) & p.hmask;
    for (unsigned long long probe = 0; probe <= p.hmask; probe++) {
        DelSlot* slot = &p.hset[h];
        const unsigned long long old = atomicCAS(&slot->pair, kHashEmpty, pair);
        if (old == kHashEmpty || old == pair) {
            const int ow = atomicCAS(&slot->w, kHashNoWeight, w);
            if (ow == kHashNoWeight || ow == w) return true;
        }
        h = (h + 1) & p.hmask;
    }
    return false;
}

__device__ bool hash_contains(const UpdParams& p, unsigned long long pair, int w) {
    unsigned long long h = dmix64(pair) & p.hmask;
    for (unsigned long long probe = 0; probe <= p.hmask; probe++) {
        const DelSlot slot = p.hset[h];
        if (slot.pair == kHashEmpty) return false;
        if (slot.pair == pair && slot.w == w) return true;
        h = (h + 1) & p.hmask;
    }
    return false;
}

// Writes the entry (col, w) at position pos of row r, described by rd (read before the degree
// bump).  Returns its slot, or -1 after listing it for the host-side row growth when the row
// is full (record i).
__device__ __forceinline__ long long place_entry(const UpdParams& p, const RowDesc& rd, int pos, int r, int col,
                                                 int w, long long i, unsigned long long& ovf) {
    if (pos < rd.cap) {
        const long long at = rd.start + pos;
        p.g.adj[at] = make_int2(col, w);
        return at;
    }
    const int o = atomicAdd(&p.g.ctl->ovf_count, 1);
    p.ovf[o] = make_int4(r, col, w, (int)i);
    ovf++;
    atomicCAS(&p.g.ctl->status, 0, kStatusOverflowPending);
    return -1;
}

// Tombstones the reverse entry of slot j.  A twin word outside the adjacency is an internal
// error: it is reported in the status word and the access is skipped.
__device__ __forceinline__ void tombstone_twin(const UpdParams& p, long long j) {
    const unsigned t = p.g.twin[j];
    if ((long long)t < p.g.cap_total) p.g.adj[t].y = -1;
    else set_status(p.g.ctl, -4 /* twin index out of range: internal error */);
}

// Tombstones one matching entry; the compare-and-swap makes the count exact when a batch
// deletes one line twice.  Returns the entries tombstoned (2 with the twin).
__device__ __forceinline__ unsigned tombstone_at(const UpdParams& p, long long j, int w, bool with_twin) {
    // a negative weight matches no live entry (tombstones hold -1)
    if (w < 0 || atomicCAS(&p.g.adj[j].y, w, -1) != w) return 0;
    if (with_twin) tombstone_twin(p, j);
    return with_twin ? 2u : 1u;
}

// Tombstones every live entry (col, w) in the neighbour-sorted prefix of a row (binary search)
// and returns the row's unsorted tail [tlo, thi): the entries appended since the row was laid
// out, which the caller scans.  With the twin index the reverse entries are tombstoned too.
// Returns the number of entries examined; `dead` counts the entries tombstoned.
__device__ unsigned long long tombstone_prefix(const UpdParams& p, const RowDesc& rd, int sorted_len, int col, int w,
                                               bool with_twin, unsigned long long& dead, long long& tlo,
                                               long long& thi) {
    const int2* adj = p.g.adj;
    const long long sl = rd.start + sorted_len;
    long long j = lower_col(adj, rd.start, sl, col);
    unsigned long long probed = 1;
    for (; j < sl && adj[j].x == col; j++, probed++)
        if (adj[j].y == w) dead += tombstone_at(p, j, w, with_twin);
    tlo = sl;
    thi = rd.start + rd.deg;
    return probed;
}

__device__ unsigned long long tombstone_tail(const UpdParams& p, long long lo, long long hi, int col, int w,
                                             bool with_twin, unsigned long long& dead) {
    for (long long j = lo; j < hi; j++)
        if (p.g.adj[j].x == col && p.g.adj[j].y == w) dead += tombstone_at(p, j, w, with_twin);
    return (unsigned long long)(hi > lo ? hi - lo : 0);
}

// The whole row: the sorted prefix by binary search, the tail by this thread.
__device__ unsigned long long tombstone_row(const UpdParams& p, const RowDesc& rd, int sorted_len, int col, int w,
                                            bool with_twin, unsigned long long& dead) {
    const int2* adj = p.g.adj;
    const long long sl = rd.start + sorted_len, end = rd.start + rd.deg;
    long long j = lower_col(adj, rd.start, sl, col);
    unsigned long long probed = 1;
    for (; j < sl && adj[j].x == col; j++, probed++)
        if (adj[j].y == w) dead += tombstone_at(p, j, w, with_twin);
    for (j = sl; j < end; j++, probed++)
        if (adj[j].x == col && adj[j].y == w) dead += tombstone_at(p, j, w, with_twin);
    return probed;
}

// Unsorted tails longer than this are scanned by the whole warp, 32 consecutive entries per
// step, instead of by the deletion's own lane: under sustained insertion and deletion the tails
// of hub rows grow to thousands of entries until the row is compacted or the adjacency is
// repacked.  The deletion's lane lists such a tail in its warp's staging; the warp scans the
// listed tails after its records (a lane whose warp's list is full scans its tail itself).
constexpr long long kCoopTail = 64;
constexpr int kTailList = 32;
struct LongTail {
    long long lo, hi;
    int col, w;
};
__shared__ LongTail s_tails[kMaxWarps][kTailList];
__shared__ unsigned s_ntails[kMaxWarps];

}  // namespace

// ---- kernels -----------------------------------------------------------------------------

__global__ void k_prepare(UpdParams p) {
    Ctl* ctl = p.g.ctl;
    unsigned long long ins = 0, del = 0, ign = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.k;
         i += (long long)gridDim.x * blockDim.x) {
        const int4 c = p.chg[i];
        if (c.w == 1 || c.w == 0) {
            if (c.x < 0 || c.x >= p.g.n || c.y < 0 || c.y >= p.g.n) set_status(ctl, -3 /* BAD_VERTEX */);
            else if (c.w == 1 && c.z < 0) set_status(ctl, -10 /* BAD_WEIGHT */);
            if (c.w == 1) ins++;
            else del++;
        } else {
            ign++;
        }
    }
    block_add(&ctl->stat[ST_INS], ins);
    block_add(&ctl->stat[ST_DEL], del);
    block_add(&ctl->stat[ST_IGN], ign);
}

// Deletions: cut off the child end of a deleted tree edge, tombstone every matching entry,
// record the deletion in the batch's deletion set.
// kTails: rows may hold unsorted tails (entries appended since the last layout), and long ones
// are scanned warp-wide; without, every tail is scanned by its deletion's lane (the host picks
// this form after a layout, a repack or a compaction, until a batch appends again: the long-tail
// path alone costs the kernel a few percent).
template <bool kTails>
__global__ void k_delete(UpdParams p) {
    Ctl* ctl = p.g.ctl;
    if (__ldcg(&ctl->status) != 0) return;  // set by k_prepare: same for every thread
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    unsigned long long probed = 0, roots = 0, dead = 0;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    if constexpr (kTails) {
        if (lane == 0) s_ntails[warp] = 0;
        __syncwarp();
    }
    WarpList roots_list{s_wlist[warp], kListRegion, 0};
    for (long long base = (long long)blockIdx.x * blockDim.x + threadIdx.x - lane; base < p.k; base += nthreads) {
        const long long i = base + lane;
        const int4 c = i < p.k ? p.chg[i] : make_int4(0, 0, 0, -1);
        bool cut = false;
        unsigned cutv = 0;
        if (c.w == 0) {
            const unsigned a = (unsigned)c.x, b = (unsigned)c.y;
            // gpuFunctions_undir.cuh:189-198: the child end is checked as b first, then as a.
            // A self-loop never cuts: its only parent relation is a root's (parent == itself),
            // and roots are never cut off.
            if (a != b) {
                const unsigned pb = (unsigned)__ldcg(&p.g.state[b]), pa = (unsigned)__ldcg(&p.g.state[a]);
                if (pb == a) cutv = b, cut = true;
                else if (pa == b) cutv = a, cut = true;
            }
            if (cut) {
                cut = atomicExch(&p.g.inv_tag[cutv], p.epoch) != p.epoch;
                if (cut) p.g.state[cutv] = kInfState;
            }
            const RowDesc ra = p.g.rows[a], rb = p.g.rows[b];
            if (p.g.twin) {
                // search the shorter row; each match's reverse entry is found through twin[]
                const bool use_a = ra.deg <= rb.deg;
                const RowDesc& rs = use_a ? ra : rb;
                const int sl = p.g.sorted_len[use_a ? a : b];
                const int col = (int)(use_a ? b : a);
                if (!kTails || rs.deg - sl <= kCoopTail) {  // a short unsorted tail: this lane scans it too
                    probed += tombstone_row(p, rs, sl, col, c.z, true, dead);
                } else {  // a long one goes to the warp's list (or, when that is full, to this lane)
                    long long tlo, thi;
                    probed += tombstone_prefix(p, rs, sl, col, c.z, true, dead, tlo, thi);
                    const unsigned at = atomicAdd(&s_ntails[warp], 1u);
                    if (at < (unsigned)kTailList) s_tails[warp][at] = LongTail{tlo, thi, col, c.z};
                    else probed += tombstone_tail(p, tlo, thi, col, c.z, true, dead);
                }
            } else {
                probed += tombstone_row(p, ra, p.g.sorted_len[a], (int)b, c.z, false, dead);
                probed += tombstone_row(p, rb, p.g.sorted_len[b], (int)a, c.z, false, dead);
            }
            if (c.z >= 0 && !hash_insert(p, dpair_key(a, b), c.z)) set_status(ctl, -4 /* deletion set full */);
        }
        roots_list.add(cut, cutv);
        roots += cut ? 1 : 0;
        roots_list.flush(p.g.invq, &ctl->inv_count, (unsigned)p.g.n, 32, ctl);
    }
    if constexpr (kTails) {  // the listed long tails, each by the whole warp (32 entries per step)
        __syncwarp();
        const unsigned nt = min(s_ntails[warp], (unsigned)kTailList);
        for (unsigned t = 0; t < nt; t++) {
            const LongTail lt = s_tails[warp][t];
            for (long long j = lt.lo + lane; j < lt.hi; j += 32) {
                const int2 e = p.g.adj[j];
                if (e.x == lt.col && e.y == lt.w) dead += tombstone_at(p, j, lt.w, true);
            }
            if (lane == 0) probed += (unsigned long long)(lt.hi - lt.lo);
        }
    }
    roots_list.flush_cta(p.g.invq, &ctl->inv_count, (unsigned)p.g.n, ctl);
    block_add(&ctl->stat[ST_ROOTS], roots);
    block_add(&ctl->stat[ST_DEL_PROBED], probed);
    block_add(&ctl->stat[ST_TOMBS], dead);
}

// Insertions that no deletion of the batch removes go into row slack, both directions.  An
// entry that does not fit is written to the overflow list and the batch is deferred to a
// host-side row growth (status 1).  Every surviving insertion then relaxes both of its ends
// (replaces insertEdge, gpuFunctions_undir.cuh:217-251); an improved end is claimed for the
// first frontier and listed in seedq (k_update splits it into work items once every row has
// its final degree) or, in near-far mode, put in the far list.  Doing this before the
// subtree walk is exact: k_delete has already cut off the roots (their distance is
// infinite, so nothing relaxes from them), an end relaxed from a vertex that the walk later
// cuts off takes that vertex as its parent and is cut off with it, and every other relaxed
// distance is the length of a live path.
__global__ void k_append(UpdParams p) {
    Ctl* ctl = p.g.ctl;
    if (__ldcg(&ctl->status) < 0) return;  // same for every thread
    DevGraph& g = p.g;
    const unsigned lane = lane_id();
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const unsigned rbase = __ldcg(&ctl->round_base);
    const unsigned tag0 = rbase + 1;
    // near-far: a batch starts with threshold 0, so every seed waits in the far list
    const bool nf = p.delta != 0 && g.far0 != nullptr && g.far1 != nullptr && g.far_tag != nullptr;
    const unsigned long long T = nf ? 0ull : ~0ull;
    // seeds are staged per warp (half of the warp's staging region each for near and far)
    unsigned* region = s_wlist[threadIdx.x >> 5];
    WarpList near_list{region, kListRegion / 2, 0}, far_list{region + kListRegion / 2, kListRegion / 2, 0};
    const unsigned seed_cap = (unsigned)min(2 * p.k, (long long)g.n);  // distinct claimed ends
    LocalStats ls;
    unsigned long long killed = 0, ovf = 0, live_ins = 0;
    for (long long base = (long long)blockIdx.x * blockDim.x + threadIdx.x - lane; base < p.k; base += nthreads) {
        const long long i = base + lane;
        const int4 c = i < p.k ? p.chg[i] : make_int4(0, 0, 0, -1);
        // Independent accesses of one record go out together (states, rows and the deletion-set
        // probe; both degree bumps; both seed relaxations; both claims).
        int alive = 0;
        unsigned long long sa = kInfState, sb = kInfState;
        if (c.w == 1) {
            sa = __ldcg(&g.state[c.x]);
            sb = __ldcg(&g.state[c.y]);
            const RowDesc rx = g.rows[c.x], ry = g.rows[c.y];  // start and cap are fixed in this kernel
            if (hash_contains(p, dpair_key((unsigned)c.x, (unsigned)c.y), c.z)) {
                killed++;
            } else {
                alive = 1;
                live_ins++;
                const int pos0 = atomicAdd(&g.rows[c.x].deg, 1);
                const int pos1 = atomicAdd(&g.rows[c.y].deg, 1);
                const long long at0 = place_entry(p, rx, pos0, c.x, c.y, c.z, i, ovf);
                const long long at1 = place_entry(p, ry, pos1, c.y, c.x, c.z, i, ovf);
                p.slot[2 * i] = at0;
                p.slot[2 * i + 1] = at1;
                if (g.twin) {  // an overflowed end is placed (and paired) by the row growth
                    if (at0 >= 0) g.twin[at0] = at1 >= 0 ? (unsigned)at1 : kNoTwin;
                    if (at1 >= 0) g.twin[at1] = at0 >= 0 ? (unsigned)at0 : kNoTwin;
                }
            }
        }
        if (i < p.k) p.ins_state[i] = alive;
        // seed: relax both ends through the new edge
        bool pa = false, pbv = false;
        const unsigned long long ndb = (sa >> 32) + (unsigned)c.z, nda = (sb >> 32) + (unsigned)c.z;
        if (alive) {
            if (c.z > 0) {
                relax_both(g, p.epoch, (unsigned)c.x, (unsigned)c.y, ndb, nda, sa, sb, pa, pbv, ls);
            } else {  // zero weight: strict improvements only (compare-and-swap)
                if ((sa >> 32) != kDistInf) pbv = relax_to(g, p.epoch, (unsigned)c.y, ndb, (unsigned)c.x, c.z, sb, ls);
                if ((sb >> 32) != kDistInf)
                    pa = relax_to(g, p.epoch, (unsigned)c.x, nda, (unsigned)c.y, c.z, __ldcg(&g.state[c.x]), ls);
            }
            ls.edges_relax += 2;
        }
        // claim: far-list tag for an end at or above the threshold, frontier tag otherwise
        const bool lb = pbv && ndb >= T, la = pa && nda >= T;
        unsigned* tb = lb ? g.far_tag + c.y : g.push_tag + c.y;
        unsigned* ta = la ? g.far_tag + c.x : g.push_tag + c.x;
        const unsigned vb = lb ? rbase : tag0, va = la ? rbase : tag0;
        const unsigned ob = pbv ? atomicExch(tb, vb) : vb;
        const unsigned oa = pa ? atomicExch(ta, va) : va;
        const bool fb = lb && ob != vb, db = pbv && !lb && ob != vb;
        const bool fa = la && oa != va, da = pa && !la && oa != va;
        ls.frontier += (db ? 1 : 0) + (da ? 1 : 0) + (fb ? 1 : 0) + (fa ? 1 : 0);
        near_list.add(db, (unsigned)c.y);  // claimed: one entry per vertex
        near_list.add(da, (unsigned)c.x);
        far_list.add(fb, (unsigned)c.y);  // far-tagged: one entry per vertex
        far_list.add(fa, (unsigned)c.x);
        near_list.flush(p.seedq, &ctl->seed_count, seed_cap, 64, ctl);
        far_list.flush(g.far0, &ctl->fc[0], (unsigned)g.n, 64, ctl);
    }
    near_list.flush_cta(p.seedq, &ctl->seed_count, seed_cap, ctl);
    far_list.flush_cta(g.far0, &ctl->fc[0], (unsigned)g.n, ctl);
    block_add(&ctl->stat[ST_SEED_UPD], ls.updates);  // kept apart from k_update's counters
    block_add(&ctl->stat[ST_SEED_FRONT], ls.frontier);
    block_add(&ctl->stat[ST_DIST_OVF], ls.dist_ovf);
    block_add(&ctl->stat[ST_OVF], ovf);
    block_add(&ctl->stat[ST_LIVE_INS], live_ins);
    unsigned long long kk = warp_sum_u64(killed);
    if (lane_id() == 0 && kk) atomicAdd(&ctl->killed, (unsigned)kk);
}

template <bool kAgg>
__device__ void update_body(UpdParams& p);

// 3 CTAs of 256 threads per SM: 80 registers a thread without spills.  Every walk level and
// relaxation round waits on its slowest CTA's chain of dependent accesses, so shorter chains
// and fewer CTAs at each barrier beat more resident warps here (4 CTAs per SM with 64
// registers and spills was slower on every workload but the throughput-bound 256-graph batch).
// kAgg: warp-aggregated distance offers (opts.warp_agg), compiled as its own kernel so that
// the default kernel keeps its register allocation.
template <bool kAgg>
__global__ void __launch_bounds__(256, 3) k_update(UpdParams p) {
    if (threadIdx.x == 0) {
        s_nbar = 0;
        s_gen = ld_acquire(&p.g.ctl->bar_gen);
        s_ggen = ld_acquire(&p.g.ctl->grp_gen);
        const unsigned lim = __ldcg(&p.g.ctl->spin_limit);
        s_spin_limit = lim ? lim : kSpinLimit;
    }
    __syncthreads();
    update_body<kAgg>(p);
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMax(&p.g.ctl->diag[3], s_nbar);
        atomicMax(&p.g.ctl->diag[4], 0xFFFFFFFFu - s_nbar);
    }
}

template <bool kAgg>
__device__ void update_body(UpdParams& p) {
    Ctl* ctl = p.g.ctl;
    DevGraph& g = p.g;
    __shared__ int s_skip;
    if (threadIdx.x == 0) s_skip = __ldcg(&ctl->status) != 0;  // set before launch: same for every CTA
    __syncthreads();
    if (s_skip) return;
    const unsigned stall_us = __ldcg(&ctl->stall_us);
    if (stall_us && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        // test hook (failure detection): arrive late at the first barrier so that the others
        // run out of polls; a bounded wait (at most 2^21 sleeps of 1 us).  One launch only: the
        // hook clears itself, so a recomputation after the failed batch runs normally.
        const unsigned long long t0 = globaltimer();
        for (unsigned i = 0; i < (1u << 21) && globaltimer() - t0 < 1000ull * stall_us; i++) __nanosleep(1000);
        ctl->stall_us = 0;
    }
    const unsigned lane = lane_id();
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const bool leader = gtid == 0;
    uint4* pbuf = s_pbuf[threadIdx.x >> 5];
    LocalStats ls;
    if (leader) ctl->ts[0] = globaltimer();

    unsigned rbase = __ldcg(&ctl->round_base);
    if (rbase > 0xF0000000u) {  // push and far tags would wrap: clear them
        for (unsigned v = gtid; v < (unsigned)g.n; v += nthreads) {
            g.push_tag[v] = 0;
            if (g.far_tag) g.far_tag[v] = 0;
        }
        if (!grid_sync(ctl)) return;
        rbase = 1;
    }
    const unsigned tag0 = rbase + 1;
    const Out relax0{g.rt0, &ctl->rcT[0], g.tcap, g.rc0, &ctl->rcC[0], g.ccap};
    // Near-far state (identical in every thread).  A batch update starts with T = 0, so every
    // seed waits in the far list and the first advance picks the threshold; a computation
    // from scratch starts with the sources (distance 0) near and T = delta.  Far generations
    // of this call are rbase, rbase + 1, ... (at most one per round, so below the next
    // call's round base).
    const bool nf = p.delta != 0 && g.far0 != nullptr && g.far1 != nullptr && g.far_tag != nullptr;
    unsigned long long T = nf ? (p.mode == 1 ? p.delta : 0ull) : ~0ull;
    unsigned fgen = rbase;
    int cf = 0;
    unsigned adv = 0;
    auto far_of = [&](int which, unsigned gen, unsigned long long thr) {
        return Far{which ? g.far1 : g.far0, &ctl->fc[which], g.far_tag, gen, (unsigned)g.n, thr};
    };

    unsigned nT = 0, nC = 0;  // the sizes of the next relaxation round's lists
    if (p.mode == 1) {
        PushBuf pb{pbuf, 0};
        for (unsigned base = gtid - lane; base < (unsigned)p.nsrc; base += nthreads) {
            const unsigned i = base + lane;
            const unsigned v = i < (unsigned)p.nsrc ? (unsigned)p.srcs[i] : 0u;
            if (i < (unsigned)p.nsrc) g.push_tag[v] = tag0;
            pb.add(i < (unsigned)p.nsrc, v, row_if(p, i < (unsigned)p.nsrc, v));
            pb.flush(p, relax0, ls);
            ls.frontier += i < (unsigned)p.nsrc ? 1 : 0;
        }
        pb.flush_cta(p, relax0, ls);
        if (!grid_sync(ctl, &ctl->rcT[0], &ctl->rcC[0], nT, nC)) return;
    } else {
        // ---- A. cut-off subtrees ------------------------------------------------------------
        // Level L processes items [lo, hi) of the lists it/ic and appends the items of the
        // vertices it cuts off after hi through the level's own counters lt*[(L+1)%3], so
        // every CTA derives the same level bounds while faster CTAs already append.
        const unsigned nroots = __ldcg(&ctl->inv_count);  // written by k_delete
        {
            const Out lvl0{g.it, &ctl->ltT[0], g.tcap, g.ic, &ctl->ltC[0], g.ccap};
            PushBuf pb{pbuf, 0};
            for (unsigned base = gtid - lane; base < nroots; base += nthreads) {
                const unsigned i = base + lane;
                const unsigned v = i < nroots ? __ldcg(&g.invq[i]) : 0u;
                pb.add(i < nroots, v, row_if(p, i < nroots, v));
                pb.flush(p, lvl0, ls);
            }
            pb.flush_cta(p, lvl0, ls);
        }
        if (leader) ls.marked += nroots;
        unsigned loT = 0, loC = 0, hiT, hiC;
        if (!grid_sync(ctl, &ctl->ltT[0], &ctl->ltC[0], hiT, hiC)) return;
        int level = 0;
        bool need_pj = false;
        for (;;) {
            if (loT >= hiT && loC >= hiC) break;
            if (level >= p.bfs_levels) {
                need_pj = true;
                break;
            }
            if (small_step(hiT - loT, hiC - loC, p.solo_waves)) {
                // small levels: CTA 0 walks on alone while they stay small; the others wait
                if (blockIdx.x == 0) {
                    if (threadIdx.x < 6) s_solo_cnt[threadIdx.x / 2][threadIdx.x % 2] = 0;
                    __syncthreads();
                    for (int steps = 0; steps < kSoloSteps; steps++) {
                        if ((loT >= hiT && loC >= hiC) || level >= p.bfs_levels || !small_step(hiT - loT, hiC - loC, p.solo_waves))
                            break;
                        unsigned* cnt = s_solo_cnt[(level + 1) % 3];
                        if (threadIdx.x == 0) {
                            s_solo_cnt[(level + 2) % 3][0] = 0;
                            s_solo_cnt[(level + 2) % 3][1] = 0;
                        }
                        MarkOp op{&p, Out{g.it + hiT, &cnt[0], g.tcap - hiT, g.ic + hiC, &cnt[1], g.ccap - hiC},
                                  PushBuf{pbuf, 0}, &ls};
                        run_items(op, p, g.it + loT, hiT - loT, g.ic + loC, hiC - loC, 0, 1);
                        __syncthreads();
                        loT = hiT;
                        loC = hiC;
                        hiT += cnt[0];
                        hiC += cnt[1];
                        level++;
                        __syncthreads();  // every thread has read the counters before the next reset
                    }
                    if (threadIdx.x == 0) {
                        ctl->solo[0] = ((unsigned long long)hiT << 32) | loT;
                        ctl->solo[1] = ((unsigned long long)hiC << 32) | loC;
                        ctl->solo[2] = (unsigned long long)level;
                        ctl->ltT[(level + 1) % 3] = 0;  // the grid's next level appends here
                        ctl->ltC[(level + 1) % 3] = 0;
                    }
                }
                if (!grid_sync(ctl)) return;
                const unsigned long long a = __ldcg(&ctl->solo[0]), b = __ldcg(&ctl->solo[1]);
                loT = (unsigned)a;
                hiT = (unsigned)(a >> 32);
                loC = (unsigned)b;
                hiC = (unsigned)(b >> 32);
                level = (int)__ldcg(&ctl->solo[2]);
                continue;
            }
            if (leader) {
                ctl->ltT[(level + 2) % 3] = 0;
                ctl->ltC[(level + 2) % 3] = 0;
            }
            MarkOp op{&p,
                      Out{g.it + hiT, &ctl->ltT[(level + 1) % 3], g.tcap - hiT, g.ic + hiC, &ctl->ltC[(level + 1) % 3],
                          g.ccap - hiC},
                      PushBuf{pbuf, 0}, &ls};
            run_items(op, p, g.it + loT, hiT - loT, g.ic + loC, hiC - loC, blockIdx.x, gridDim.x);
            unsigned addT, addC;
            if (!grid_sync(ctl, &ctl->ltT[(level + 1) % 3], &ctl->ltC[(level + 1) % 3], addT, addC)) return;
            loT = hiT;
            loC = hiC;
            hiT += addT;
            hiC += addC;
            level++;
        }
        if (leader) ctl->stat[ST_LEVELS] = (unsigned long long)level;
        if (need_pj) {
            // pointer jumping: jm[v] climbs towards the root until it meets a cut-off vertex
            // (kTagInv) or the root / an unreachable vertex (kTagOk); O(log depth) passes
            for (unsigned v = gtid; v < (unsigned)g.n; v += nthreads) {
                unsigned t;
                if (__ldcg(&g.inv_tag[v]) == p.epoch) {
                    t = kTagInv;
                } else {
                    const unsigned par = (unsigned)__ldcg(&g.state[v]);
                    t = (par == v || par == kNone) ? kTagOk : par;  // a root, or unreachable
                }
                g.jm[v] = t;
            }
            if (!grid_sync(ctl)) return;
            int pass = 0;
            for (;; pass++) {
                if (pass >= 64) {
                    if (leader) set_status(ctl, -7 /* BAD_TREE: parent cycle */);
                    grid_sync(ctl);
                    return;
                }
                if (leader) ctl->pjf[(pass + 1) % 3] = 0;
                int moving = 0;
                for (unsigned v = gtid; v < (unsigned)g.n; v += nthreads) {
                    const unsigned j = __ldcg(&g.jm[v]);
                    if (j < kTagInv) {
                        const unsigned jj = __ldcg(&g.jm[j]);
                        g.jm[v] = jj;
                        moving |= jj < kTagInv;
                    }
                }
                moving = __syncthreads_or(moving);
                if (moving && threadIdx.x == 0) atomicOr(&ctl->pjf[pass % 3], 1u);
                if (!grid_sync(ctl)) return;
                if (__ldcg(&ctl->pjf[pass % 3]) == 0) break;
            }
            if (leader) ctl->stat[ST_PJ] = (unsigned long long)(pass + 1);
            const Out pjo{g.it + hiT, &ctl->pjT, g.tcap - hiT, g.ic + hiC, &ctl->pjC, g.ccap - hiC};
            PushBuf pb{pbuf, 0};
            for (unsigned base = gtid - lane; base < (unsigned)g.n; base += nthreads) {
                const unsigned v = base + lane;
                bool newinv = false;
                const bool inv = v < (unsigned)g.n && __ldcg(&g.jm[v]) == kTagInv;
                if (inv && __ldcg(&g.inv_tag[v]) != p.epoch) {
                    g.inv_tag[v] = p.epoch;
                    newinv = true;
                }
                // also the roots: one that an insertion re-parented may hold a distance
                // through a cut-off vertex (the pull gives it its best live value again)
                if (inv) g.state[v] = kInfState;
                ls.marked += newinv ? 1 : 0;
                pb.add(newinv, v, row_if(p, newinv, v));
                pb.flush(p, pjo, ls);
            }
            pb.flush_cta(p, pjo, ls);
            if (!grid_sync(ctl)) return;
            hiT += __ldcg(&ctl->pjT);
            hiC += __ldcg(&ctl->pjC);
        }
        if (leader) ctl->ts[1] = globaltimer();

        // ---- B. the seeds of k_append become work items; cut-off vertices pull their best
        // live neighbour --------------------------------------------------------------------
        {
            const unsigned ns = __ldcg(&ctl->seed_count);
            PushBuf pb{pbuf, 0};
            for (unsigned base = gtid - lane; base < ns; base += nthreads) {
                const unsigned i = base + lane;
                const unsigned v = i < ns ? __ldcg(&p.seedq[i]) : 0u;
                pb.add(i < ns, v, row_if(p, i < ns, v));
                pb.flush(p, relax0, ls);
            }
            pb.flush_cta(p, relax0, ls);
        }
        {
            PullOp op{&p, tag0, relax0, PushBuf{pbuf, 0}, &ls, far_of(cf, fgen, T), kInfState, false};
            run_items(op, p, g.it, hiT, g.ic, hiC, blockIdx.x, gridDim.x);
        }
        if (!grid_sync(ctl, &ctl->rcT[0], &ctl->rcC[0], nT, nC)) return;
    }
    if (leader) ctl->ts[2] = globaltimer();

    // ---- C. relaxation rounds ---------------------------------------------------------------
    long long r = 0;
    for (;; r++) {
        // nT, nC: the sizes of round r's lists (read at the barrier before)
        if (nT == 0 && nC == 0) {
            if (!nf) break;
            // near frontier empty: advance the threshold past the least waiting distance
            const unsigned nfar = __ldcg(&ctl->fc[cf]);
            if (nfar == 0) break;
            const unsigned* fl = cf ? g.far1 : g.far0;
            unsigned long long mn = ~0ull;
            for (unsigned i = gtid; i < nfar; i += nthreads) {
                const unsigned long long d = __ldcg(&g.state[__ldcg(&fl[i])]) >> 32;
                if (d >= T && d < mn) mn = d;  // below T: settled by an earlier near phase
            }
            block_max(&ctl->fmin[adv & 1], ~mn);  // max of ~d = min of d; 0 = nothing waits
            if (leader) {
                ctl->fmin[(adv + 1) & 1] = 0;  // read by every CTA before the last barrier
                ctl->fc[cf ^ 1] = 0;           // the previous advance's source list
            }
            if (!grid_sync(ctl)) break;
            const unsigned long long fm = __ldcg(&ctl->fmin[adv & 1]);
            if (fm == 0) break;
            const unsigned long long tn = ~fm + p.delta;
            const Far nxt = far_of(cf ^ 1, fgen + 1, tn);
            const Out near{(r & 1) ? g.rt1 : g.rt0, &ctl->rcT[r % 3], g.tcap, (r & 1) ? g.rc1 : g.rc0,
                           &ctl->rcC[r % 3], g.ccap};
            const unsigned tagr = rbase + (unsigned)r + 1u;  // the tag of round r's list
            PushBuf pb{pbuf, 0};
            for (unsigned base = gtid - lane; base < nfar; base += nthreads) {
                const unsigned i = base + lane;
                const unsigned v = i < nfar ? __ldcg(&fl[i]) : 0u;
                const unsigned long long d = i < nfar ? __ldcg(&g.state[v]) >> 32 : 0ull;
                const bool live = i < nfar && d >= T;
                far_push(p, nxt, live && d >= tn, v);
                RowDesc rd;
                const bool doit = claim_with_row(p, live && d < tn, v, tagr, rd);
                ls.frontier += doit ? 1 : 0;
                pb.add(doit, v, rd);
                pb.flush(p, near, ls);
            }
            pb.flush_cta(p, near, ls);
            T = tn;
            fgen++;
            cf ^= 1;
            adv++;
            if (!grid_sync(ctl, &ctl->rcT[r % 3], &ctl->rcC[r % 3], nT, nC)) break;
        }
        if (r >= p.max_rounds) {
            if (leader) set_status(ctl, -5 /* NO_CONVERGENCE */);
            break;
        }
        if (small_step(nT, nC, p.solo_waves)) {
            // small rounds: CTA 0 relaxes on alone while they stay small; the others wait.  An
            // empty frontier goes back to the grid (near-far advance or the end).
            if (blockIdx.x == 0) {
                long long rr = r;
                unsigned t = nT, c = nC;
                if (threadIdx.x < 6) s_solo_cnt[threadIdx.x / 2][threadIdx.x % 2] = 0;
                __syncthreads();
                for (int steps = 0; steps < kSoloSteps; steps++) {
                    if ((t == 0 && c == 0) || !small_step(t, c, p.solo_waves) || rr >= p.max_rounds) break;
                    unsigned* cnt = s_solo_cnt[(rr + 1) % 3];
                    if (threadIdx.x == 0) {
                        s_solo_cnt[(rr + 2) % 3][0] = 0;
                        s_solo_cnt[(rr + 2) % 3][1] = 0;
                    }
                    const bool odd = (rr & 1) != 0;
                    RelaxOp<kAgg> op{&p, rbase + (unsigned)rr + 2u,
                               Out{odd ? g.rt0 : g.rt1, &cnt[0], g.tcap, odd ? g.rc0 : g.rc1, &cnt[1], g.ccap},
                               PushBuf{pbuf, 0}, &ls, far_of(cf, fgen, T), true};
                    run_items(op, p, odd ? g.rt1 : g.rt0, t, odd ? g.rc1 : g.rc0, c, 0, 1);
                    __syncthreads();
                    rr++;
                    t = cnt[0];
                    c = cnt[1];
                    __syncthreads();  // every thread has read the counters before the next reset
                }
                if (threadIdx.x == 0) {
                    ctl->solo[3] = (unsigned long long)rr;
                    ctl->solo_n[0] = t;
                    ctl->solo_n[1] = c;
                    ctl->rcT[rr % 3] = t;  // round rr's lists (the near-far advance appends here when empty)
                    ctl->rcC[rr % 3] = c;
                    ctl->rcT[(rr + 1) % 3] = 0;  // the grid's round rr appends here
                    ctl->rcC[(rr + 1) % 3] = 0;
                }
            }
            if (!grid_sync(ctl, &ctl->solo_n[0], &ctl->solo_n[1], nT, nC)) break;
            r = (long long)__ldcg(&ctl->solo[3]) - 1;  // the loop steps to the first round left
            continue;
        }
        if (group_step(p, nT, nC)) {
            // mid-size rounds: the group relaxes on with its own barrier while they stay
            // mid-size (at most kSoloSteps); the others wait at the next grid barrier.  Lists and
            // counters are the grid's, so the hand-over is the same as after solo rounds.
            const unsigned G = p.group_ctas;
            if (blockIdx.x < G) {
                long long rr = r;
                unsigned t = nT, c = nC;
                for (int steps = 0; steps < kSoloSteps; steps++) {
                    if ((t == 0 && c == 0) || !group_step(p, t, c) || rr >= p.max_rounds) break;
                    if (blockIdx.x == 0 && threadIdx.x == 0) {
                        ctl->rcT[(rr + 2) % 3] = 0;
                        ctl->rcC[(rr + 2) % 3] = 0;
                    }
                    const bool odd = (rr & 1) != 0;
                    RelaxOp<kAgg> op{&p, rbase + (unsigned)rr + 2u,
                                     Out{odd ? g.rt0 : g.rt1, &ctl->rcT[(rr + 1) % 3], g.tcap, odd ? g.rc0 : g.rc1,
                                         &ctl->rcC[(rr + 1) % 3], g.ccap},
                                     PushBuf{pbuf, 0}, &ls, far_of(cf, fgen, T),
                                     (unsigned long long)t + (unsigned long long)c * blockDim.x <=
                                         (unsigned long long)G * blockDim.x};
                    run_items(op, p, odd ? g.rt1 : g.rt0, t, odd ? g.rc1 : g.rc0, c, blockIdx.x, G);
                    unsigned t2, c2;
                    const bool go = group_sync(ctl, G, &ctl->rcT[(rr + 1) % 3], &ctl->rcC[(rr + 1) % 3], t2, c2);
                    rr++;
                    t = t2;
                    c = c2;
                    if (!go) break;
                }
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    ctl->solo[3] = (unsigned long long)rr;
                    ctl->solo_n[0] = t;
                    ctl->solo_n[1] = c;
                    ctl->rcT[rr % 3] = t;  // round rr's lists (the near-far advance appends here when empty)
                    ctl->rcC[rr % 3] = c;
                    ctl->rcT[(rr + 1) % 3] = 0;  // the grid's round rr appends here
                    ctl->rcC[(rr + 1) % 3] = 0;
                }
            }
            if (!grid_sync(ctl, &ctl->solo_n[0], &ctl->solo_n[1], nT, nC)) break;
            r = (long long)__ldcg(&ctl->solo[3]) - 1;  // the loop steps to the first round left
            continue;
        }
        if (leader) {
            ctl->rcT[(r + 2) % 3] = 0;
            ctl->rcC[(r + 2) % 3] = 0;
        }
        const bool odd = (r & 1) != 0;
        RelaxOp<kAgg> op{&p, rbase + (unsigned)r + 2u,
                   Out{odd ? g.rt0 : g.rt1, &ctl->rcT[(r + 1) % 3], g.tcap, odd ? g.rc0 : g.rc1,
                       &ctl->rcC[(r + 1) % 3], g.ccap},
                   PushBuf{pbuf, 0}, &ls, far_of(cf, fgen, T),
                   (unsigned long long)nT + (unsigned long long)nC * blockDim.x <= (unsigned long long)nthreads};
        run_items(op, p, odd ? g.rt1 : g.rt0, nT, odd ? g.rc1 : g.rc0, nC, blockIdx.x, gridDim.x);
        if (!grid_sync(ctl, &ctl->rcT[(r + 1) % 3], &ctl->rcC[(r + 1) % 3], nT, nC)) break;
    }
    flush_stats(ctl, ls);
    if (leader) {
        ctl->stat[ST_ROUNDS] = (unsigned long long)r;
        ctl->stat[ST_ADVANCES] = (unsigned long long)adv;
        ctl->round_base = rbase + (unsigned)r + 4u;
        ctl->ts[3] = globaltimer();
    }
}

}  // namespace dsssp

// ---- host launch wrappers (the kernels above are launched only through these) -----------
namespace dsssp {

void count_launch(int n);

// after_prepare / after_delete: events recorded between the kernels (nullptr = none)
cudaError_t launch_front(const UpdParams& p, int grid, cudaStream_t s, cudaEvent_t after_prepare,
                         cudaEvent_t after_delete) {
    if (p.k <= 0) return cudaSuccess;
    const long long need = (p.k + 255) / 256;
    const unsigned g = (unsigned)(need < grid ? need : grid);
    k_prepare<<<g, 256, 0, s>>>(p);
    if (after_prepare) cudaEventRecord(after_prepare, s);
    if (p.tails) k_delete<true><<<g, 256, 0, s>>>(p);
    else k_delete<false><<<g, 256, 0, s>>>(p);
    if (after_delete) cudaEventRecord(after_delete, s);
    k_append<<<g, 256, 0, s>>>(p);
    count_launch(3);
    return cudaGetLastError();
}

// The batch kernels as graph-node functions: k_prepare, k_delete, k_append, k_update.
void batch_kernels(const void* fns[4]) {
    fns[0] = (const void*)k_prepare;
    fns[1] = (const void*)k_delete<true>;
    fns[2] = (const void*)k_append;
    fns[3] = (const void*)k_update<false>;
}

const void* delete_kernel(bool tails) {
    return tails ? (const void*)k_delete<true> : (const void*)k_delete<false>;
}

const void* update_kernel(bool warp_agg) {
    return warp_agg ? (const void*)k_update<true> : (const void*)k_update<false>;
}

cudaError_t update_occupancy(int block, int* blocks_per_sm) {
    int a = 0, b = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_update<false>, block, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_update<true>, block, 0);
    *blocks_per_sm = a < b ? a : b;
    return e;
}

cudaError_t launch_update(const UpdParams& p, int grid, int block, cudaStream_t s) {
    UpdParams copy = p;
    void* args[] = {&copy};
    cudaError_t e = cudaLaunchCooperativeKernel(update_kernel(p.warp_agg != 0), dim3((unsigned)grid),
                                                dim3((unsigned)block), args, 0, s);
    count_launch(1);
    return e;
}

}  // namespace dsssp
