// update.cu -- the batch-update kernels of the dynamic SSSP engine (sm_103a).
//
// One batch (replaces SSSPmainForUndirected.cu:196-281) is four launches on one stream:
//   k_prepare   validate and count the change records
//   k_append    insertions go into row slack (atomic degree bump), both directions
//               (replaces the host-side append of all_structure_undir.cuh:106-117)
//   k_delete    every adjacency entry matching a deletion is tombstoned (binary search in
//               the sorted row prefix + scan of the appended tail) and the child end of a
//               deleted tree edge is cut off (replaces deleteEdge, gpuFunctions_undir.cuh:179-215)
//   k_update    one persistent cooperative kernel with a bounded grid barrier:
//               A. cut-off subtrees are walked level by level from the cut-off roots
//                  (replaces filterAffectedNodes + updateNeighbors_del and its host loop,
//                  gpuFunctions_undir.cuh:125-144, 312-349, MAIN:219-239); after
//                  bfs_levels levels it switches to pointer jumping over the parent array
//               B. surviving insertions relax their endpoints (replaces insertEdge,
//                  gpuFunctions_undir.cuh:217-251) and every cut-off vertex pulls its best
//                  live neighbour
//               C. frontier relaxation rounds with degree buckets (thread / warp per vertex,
//                  CTA per chunk for heavy rows) and 64-bit atomicMin on the packed
//                  (dist, parent) word until the frontier is empty (replaces
//                  filterAllAffected + updateNeighbors and its host loop,
//                  gpuFunctions_undir.cuh:162-174, 370-433, MAIN:263-281)
#include <cuda_runtime.h>

#include "engine.cuh"

namespace dsssp {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned kSpinLimit = 1u << 24;  // x ~200 ns sleeps: a barrier gives up after ~3 s

__shared__ unsigned s_nbar;  // grid barriers this CTA has passed

struct LocalStats {
    unsigned long long edges_relax = 0, edges_inv = 0, updates = 0, dist_ovf = 0;
};

// Grid-wide barrier for a cooperative launch.  The wait is bounded: on timeout the status
// word gets DSSSP_E_TIMEOUT and every CTA leaves at its next barrier.  Returns false when
// the kernel must stop (timeout or any error status).
__device__ bool grid_sync(Ctl* ctl) {
    __shared__ int s_go;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire(&ctl->bar_gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->bar_count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            st_release(&ctl->bar_gen, gen + 1);
        } else {
            unsigned spins = 0;
            while (ld_acquire(&ctl->bar_gen) == gen) {
                if (++spins > kSpinLimit) {
                    if (atomicCAS(&ctl->status, 0, -6 /* DSSSP_E_TIMEOUT */) == 0) {
                        ctl->diag[0] = s_nbar;
                        ctl->diag[1] = atomicAdd(&ctl->bar_count, 0u);
                    }
                    atomicAdd(&ctl->diag[2], 1u);
                    break;
                }
                __nanosleep(spins < 32 ? 32 : 200);
            }
        }
        s_nbar++;
        __threadfence();
        s_go = __ldcg(&ctl->status) == 0;
    }
    __syncthreads();
    return s_go != 0;
}

__device__ __forceinline__ bool claim_push(unsigned* push_tag, unsigned c, unsigned tag) {
    if (__ldcg(&push_tag[c]) == tag) return false;
    return atomicExch(&push_tag[c], tag) != tag;
}

// Offers distance nd through parent u to vertex c whose current word is cur.  Returns true
// when c's distance went down (c must then be pushed).  Zero-weight edges only replace a
// strictly larger distance, so equal-distance parent swaps can never close a cycle.
__device__ __forceinline__ bool relax_to(unsigned long long* state, unsigned c, unsigned long long nd,
                                         unsigned u, int w, unsigned long long cur, LocalStats& ls) {
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

// ---- per-edge operations ---------------------------------------------------------------
// visit4 handles up to four adjacency entries per lane and is called by all 32 lanes.

struct RelaxOp {
    unsigned long long* state;
    const int2* adj;
    unsigned* push_tag;
    unsigned tag;
    unsigned* qout;
    unsigned* qcnt;
    LocalStats* ls;

    __device__ __forceinline__ unsigned long long prep(unsigned v) const { return __ldcg(&state[v]) >> 32; }
    __device__ __forceinline__ bool skip(unsigned long long du) const { return du >= kDistInf; }
    __device__ __forceinline__ void begin_lane(unsigned) {}
    __device__ __forceinline__ void end_lane(unsigned, bool) {}
    __device__ __forceinline__ void begin_warp(unsigned) {}
    __device__ __forceinline__ void end_warp(unsigned) {}

    __device__ __forceinline__ void visit4(unsigned u, unsigned long long du, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? __ldg(&adj[j[q]]) : make_int2(0, -1);
        unsigned long long cur[4];
#pragma unroll
        for (int q = 0; q < 4; q++) cur[q] = e[q].y >= 0 ? __ldcg(&state[e[q].x]) : 0ull;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            bool push = false;
            if (e[q].y >= 0) push = relax_to(state, (unsigned)e[q].x, du + (unsigned)e[q].y, u, e[q].y, cur[q], *ls);
            const bool doit = push && claim_push(push_tag, (unsigned)e[q].x, tag);
            warp_append(doit, (unsigned)e[q].x, qout, qcnt);
            ls->edges_relax += ok[q] ? 1 : 0;
        }
    }
};

struct MarkOp {
    unsigned long long* state;
    const int2* adj;
    unsigned* inv_tag;
    unsigned epoch;
    unsigned* invq;
    unsigned* inv_count;
    LocalStats* ls;

    __device__ __forceinline__ unsigned long long prep(unsigned) const { return 0; }
    __device__ __forceinline__ bool skip(unsigned long long) const { return false; }
    __device__ __forceinline__ void begin_lane(unsigned) {}
    __device__ __forceinline__ void end_lane(unsigned, bool) {}
    __device__ __forceinline__ void begin_warp(unsigned) {}
    __device__ __forceinline__ void end_warp(unsigned) {}

    __device__ __forceinline__ void visit4(unsigned x, unsigned long long, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? __ldg(&adj[j[q]]) : make_int2(0, -1);
        unsigned long long s[4];
#pragma unroll
        for (int q = 0; q < 4; q++) s[q] = e[q].y >= 0 ? __ldcg(&state[e[q].x]) : kInfState;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const unsigned c = (unsigned)e[q].x;
            bool mark = e[q].y >= 0 && (unsigned)s[q] == x;
            if (mark) mark = atomicExch(&inv_tag[c], epoch) != epoch;
            if (mark) state[c] = kInfState;
            warp_append(mark, c, invq, inv_count);
            ls->edges_inv += ok[q] ? 1 : 0;
        }
    }
};

struct PullOp {
    unsigned long long* state;
    const int2* adj;
    unsigned* push_tag;
    unsigned tag;
    unsigned* qout;
    unsigned* qcnt;
    LocalStats* ls;
    unsigned long long best;
    bool need;

    __device__ __forceinline__ unsigned long long prep(unsigned) const { return 0; }
    __device__ __forceinline__ bool skip(unsigned long long) const { return false; }
    __device__ __forceinline__ void begin_lane(unsigned) { best = kInfState; need = false; }
    __device__ __forceinline__ void begin_warp(unsigned) { best = kInfState; need = false; }

    __device__ __forceinline__ void visit4(unsigned x, unsigned long long, const long long (&j)[4],
                                           const bool (&ok)[4]) {
        int2 e[4];
#pragma unroll
        for (int q = 0; q < 4; q++) e[q] = ok[q] ? __ldg(&adj[j[q]]) : make_int2(0, -1);
        unsigned long long s[4];
#pragma unroll
        for (int q = 0; q < 4; q++) s[q] = e[q].y >= 0 ? __ldcg(&state[e[q].x]) : kInfState;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            ls->edges_inv += ok[q] ? 1 : 0;
            if (e[q].y < 0 || s[q] == kInfState) continue;
            const unsigned long long nd = (s[q] >> 32) + (unsigned)e[q].y;
            if (nd >= kDistInf) {
                ls->dist_ovf++;
                continue;
            }
            if (e[q].y > 0) {
                const unsigned long long cand = (nd << 32) | (unsigned)e[q].x;
                best = cand < best ? cand : best;
            } else if (relax_to(state, x, nd, (unsigned)e[q].x, 0, __ldcg(&state[x]), *ls)) {
                need = true;
            }
        }
    }
    // flush of one lane's own vertex
    __device__ __forceinline__ void end_lane(unsigned x, bool valid) {
        bool improved = false;
        if (valid && best != kInfState) {
            const unsigned long long old = atomicMin(&state[x], best);
            if ((old >> 32) > (best >> 32)) {
                improved = true;
                ls->updates++;
            }
        }
        const bool doit = valid && (need || improved) && claim_push(push_tag, x, tag);
        warp_append(doit, x, qout, qcnt);
    }
    // flush of a vertex shared by the warp
    __device__ __forceinline__ void end_warp(unsigned x) {
        const unsigned long long b = warp_min_u64(best);
        const bool nd = __any_sync(kFull, need);
        bool improved = false;
        if (lane_id() == 0 && b != kInfState) {
            const unsigned long long old = atomicMin(&state[x], b);
            if ((old >> 32) > (b >> 32)) {
                improved = true;
                ls->updates++;
            }
        }
        const bool doit = lane_id() == 0 && (nd || improved) && claim_push(push_tag, x, tag);
        warp_append(doit, x, qout, qcnt);
    }
};

// ---- granularities ---------------------------------------------------------------------

template <class Op>
__device__ __forceinline__ void lane_row(Op& op, unsigned v, unsigned long long du, long long start, int deg,
                                         int maxd, bool valid) {
    op.begin_lane(v);
    for (int b = 0; b < maxd; b += 4) {
        long long j[4];
        bool ok[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            ok[q] = b + q < deg;
            j[q] = start + b + q;
        }
        op.visit4(v, du, j, ok);
    }
    op.end_lane(v, valid);
}

template <class Op>
__device__ __forceinline__ void warp_row(Op& op, unsigned v, unsigned long long du, long long start, int deg) {
    const int lane = (int)lane_id();
    op.begin_warp(v);
    for (int b = 0; b < deg; b += 128) {
        long long j[4];
        bool ok[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int idx = b + q * 32 + lane;
            ok[q] = idx < deg;
            j[q] = start + idx;
        }
        op.visit4(v, du, j, ok);
    }
    op.end_warp(v);
}

template <class Op>
__device__ __forceinline__ void cta_chunk(Op& op, unsigned v, unsigned long long du, long long start, int deg,
                                          unsigned chunk_id, int chunk) {
    const long long lo = (long long)chunk_id * chunk;
    const long long hi = min((long long)deg, lo + chunk);
    op.begin_warp(v);
    for (long long b = lo; b < hi; b += 4LL * blockDim.x) {
        long long j[4];
        bool ok[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const long long idx = b + (long long)q * blockDim.x + threadIdx.x;
            ok[q] = idx < hi;
            j[q] = start + idx;
        }
        op.visit4(v, du, j, ok);
    }
    op.end_warp(v);
}

// Processes a work list with degree buckets: heavy vertices handed over by the previous
// step (CTA per chunk), then the light items 32 per warp -- degree <= small_deg one thread
// each, up to large_deg one warp each; heavier ones go to heavy_out for the next step.
template <class Op>
__device__ void run_items(Op& op, const UpdParams& p, const unsigned* items, unsigned count,
                          const uint2* heavy, unsigned hcount, uint2* heavy_out,
                          unsigned* heavy_out_cnt) {
    const RowDesc* rows = p.g.rows;
    const unsigned lane = lane_id();
    const unsigned gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    // heavy rows handed over by the previous step: one CTA per (vertex, chunk) item
    for (unsigned t = blockIdx.x; t < hcount; t += gridDim.x) {
        const uint2 it = __ldcg(&heavy[t]);
        const RowDesc rd = rows[it.x];
        const unsigned long long du = __shfl_sync(kFull, op.prep(it.x), 0);
        if (!op.skip(du)) cta_chunk(op, it.x, du, rd.start, rd.deg, it.y, p.chunk);
    }
    for (unsigned base = gwarp * 32; base < count; base += nwarps * 32) {
        const unsigned i = base + lane;
        const bool has = i < count;
        const unsigned v = has ? __ldcg(&items[i]) : 0u;
        RowDesc rd;
        rd.start = 0;
        rd.deg = 0;
        rd.cap = 0;
        if (has) rd = rows[v];
        const unsigned long long du = has ? op.prep(v) : kDistInf;
        const bool live = has && !op.skip(du) && rd.deg > 0;
        const int deg = live ? rd.deg : 0;
        const bool is_small = live && deg <= p.small_deg;
        const bool is_heavy = live && deg > p.large_deg;
        const unsigned nch = is_heavy ? (unsigned)((deg + p.chunk - 1) / p.chunk) : 0u;
        if (!warp_append_chunks(is_heavy, v, nch, heavy_out, heavy_out_cnt, p.g.hcap) && lane == 0)
            set_status(p.g.ctl, -4 /* heavy list capacity: internal error */);
        const int sdeg = is_small ? deg : 0;
        const int maxd = (int)__reduce_max_sync(kFull, (unsigned)sdeg);
        if (maxd > 0) lane_row(op, v, du, rd.start, sdeg, maxd, is_small);
        unsigned mm = __ballot_sync(kFull, live && !is_small && !is_heavy);
        while (mm) {
            const int l = __ffs(mm) - 1;
            mm &= mm - 1;
            const unsigned vv = __shfl_sync(kFull, v, l);
            const long long st = __shfl_sync(kFull, rd.start, l);
            const int dg = __shfl_sync(kFull, deg, l);
            const unsigned long long dd = __shfl_sync(kFull, du, l);
            warp_row(op, vv, dd, st, dg);
        }
    }
}

__device__ void flush_stats(Ctl* ctl, const LocalStats& ls) {
    unsigned long long v[4] = {ls.edges_relax, ls.edges_inv, ls.updates, ls.dist_ovf};
    const int idx[4] = {ST_EDGES_RELAX, ST_EDGES_INV, ST_UPDATES, ST_DIST_OVF};
#pragma unroll
    for (int s = 0; s < 4; s++) {
        unsigned long long x = v[s];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
        if (lane_id() == 0 && x) atomicAdd(&ctl->stat[idx[s]], x);
    }
}

// ---- row search -------------------------------------------------------------------------

// First index in adj[lo, hi) whose column is >= c (the prefix is sorted by column).
__device__ __forceinline__ long long lower_col(const int2* adj, long long lo, long long hi, int c) {
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (adj[mid].x < c) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace

// ---- kernels -----------------------------------------------------------------------------

__global__ void k_prepare(UpdParams p) {
    Ctl* ctl = p.g.ctl;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned ins = 0, del = 0, ign = 0;
    if (i < p.k) {
        const int4 c = p.chg[i];
        if (c.w == 1 || c.w == 0) {
            if (c.x < 0 || c.x >= p.g.n || c.y < 0 || c.y >= p.g.n) set_status(ctl, -3 /* BAD_VERTEX */);
            else if (c.w == 1 && c.z < 0) set_status(ctl, -10 /* BAD_WEIGHT */);
            if (c.w == 1) ins = 1;
            else del = 1;
        } else {
            ign = 1;
        }
    }
    ins = __reduce_add_sync(kFull, ins);
    del = __reduce_add_sync(kFull, del);
    ign = __reduce_add_sync(kFull, ign);
    if (lane_id() == 0) {
        if (ins) atomicAdd(&ctl->stat[ST_INS], ins);
        if (del) atomicAdd(&ctl->stat[ST_DEL], del);
        if (ign) atomicAdd(&ctl->stat[ST_IGN], ign);
    }
}

// Insertions: both directions go into row slack.  An entry that does not fit is written to
// the overflow list and the batch is deferred to a host-side repack (status 1).
__global__ void k_append(UpdParams p, int4* ovf) {
    Ctl* ctl = p.g.ctl;
    if (__ldcg(&ctl->status) < 0) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.k) return;
    const int4 c = p.chg[i];
    if (c.w != 1) return;
    long long* slot = const_cast<long long*>(p.slot);
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int r = side ? c.y : c.x, col = side ? c.x : c.y;
        RowDesc* rd = &p.g.rows[r];
        const int pos = atomicAdd(&rd->deg, 1);
        if (pos < rd->cap) {
            const long long at = rd->start + pos;
            p.g.adj[at] = make_int2(col, c.z);
            slot[2 * i + side] = at;
        } else {
            const int o = atomicAdd(&ctl->ovf_count, 1);
            ovf[o] = make_int4(r, col, c.z, (int)i);
            slot[2 * i + side] = -1;
            atomicAdd(&ctl->stat[ST_OVF], 1ull);
            atomicCAS(&ctl->status, 0, kStatusOverflowPending);
        }
    }
}

// Deletions: cut off the child end of a deleted tree edge, tombstone every matching entry.
__global__ void k_delete(UpdParams p) {
    Ctl* ctl = p.g.ctl;
    if (__ldcg(&ctl->status) != 0) return;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool cut = false;
    unsigned cutv = 0;
    unsigned long long probed = 0;
    if (i < p.k) {
        const int4 c = p.chg[i];
        if (c.w == 0) {
            const unsigned a = (unsigned)c.x, b = (unsigned)c.y;
            // gpuFunctions_undir.cuh:189-198: child end first checked as b, then as a
            if (b != (unsigned)p.g.src && (unsigned)__ldcg(&p.g.state[b]) == a) cutv = b, cut = true;
            else if (a != (unsigned)p.g.src && (unsigned)__ldcg(&p.g.state[a]) == b) cutv = a, cut = true;
            if (cut) {
                cut = atomicExch(&p.g.inv_tag[cutv], p.epoch) != p.epoch;
                if (cut) p.g.state[cutv] = kInfState;
            }
#pragma unroll
            for (int side = 0; side < 2; side++) {
                const int r = side ? c.y : c.x, col = side ? c.x : c.y;
                const RowDesc rd = p.g.rows[r];
                const long long sl = rd.start + p.g.sorted_len[r], end = rd.start + rd.deg;
                long long j = lower_col(p.g.adj, rd.start, sl, col);
                probed += 1;
                for (; j < sl && p.g.adj[j].x == col; j++, probed++)
                    if (p.g.adj[j].y == c.z) p.g.adj[j].y = -1;
                for (j = sl; j < end; j++, probed++)
                    if (p.g.adj[j].x == col && p.g.adj[j].y == c.z) p.g.adj[j].y = -1;
            }
        }
    }
    warp_append(cut, cutv, p.g.invq, &ctl->inv_count);
    const unsigned nc = __popc(__ballot_sync(kFull, cut));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) probed += __shfl_xor_sync(kFull, probed, o);
    if (lane_id() == 0) {
        if (nc) atomicAdd(&ctl->stat[ST_ROOTS], (unsigned long long)nc);
        if (probed) atomicAdd(&ctl->stat[ST_DEL_PROBED], probed);
    }
}

// After a repack: point each insertion's slots at an entry (col, w) of its two rows.
__global__ void k_relocate(UpdParams p) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.k) return;
    const int4 c = p.chg[i];
    if (c.w != 1) return;
    long long* slot = const_cast<long long*>(p.slot);
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int r = side ? c.y : c.x, col = side ? c.x : c.y;
        const RowDesc rd = p.g.rows[r];
        const long long sl = rd.start + p.g.sorted_len[r], end = rd.start + rd.deg;
        long long j = lower_col(p.g.adj, rd.start, sl, col), at = -1;
        for (; j < sl && p.g.adj[j].x == col && at < 0; j++)
            if (p.g.adj[j].y == c.z) at = j;
        for (j = sl; j < end && at < 0; j++)
            if (p.g.adj[j].x == col && p.g.adj[j].y == c.z) at = j;
        slot[2 * i + side] = at;
    }
}

__device__ void update_body(UpdParams& p);

__global__ void __launch_bounds__(256) k_update(UpdParams p) {
    if (threadIdx.x == 0) s_nbar = 0;
    __syncthreads();
    update_body(p);
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMax(&p.g.ctl->diag[3], s_nbar);
        atomicMax(&p.g.ctl->diag[4], 0xFFFFFFFFu - s_nbar);
    }
}

__device__ void update_body(UpdParams& p) {
    Ctl* ctl = p.g.ctl;
    DevGraph& g = p.g;
    __shared__ int s_skip;
    if (threadIdx.x == 0) s_skip = __ldcg(&ctl->status) != 0;  // set before launch: same for every CTA
    __syncthreads();
    if (s_skip) return;
    const unsigned lane = lane_id();
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const bool leader = gtid == 0;
    LocalStats ls;
    if (leader) ctl->ts[0] = globaltimer();

    unsigned rbase = __ldcg(&ctl->round_base);
    if (rbase > 0xF0000000u) {  // push tags would wrap: clear them
        for (unsigned v = gtid; v < (unsigned)g.n; v += nthreads) g.push_tag[v] = 0;
        if (!grid_sync(ctl)) return;
        rbase = 1;
    }

    if (p.mode == 1) {
        if (leader) {
            g.q0[0] = (unsigned)g.src;
            g.push_tag[g.src] = rbase + 1;
            ctl->cq[0] = 1;
        }
        if (!grid_sync(ctl)) return;
    } else {
        // ---- A. cut-off subtrees: level-synchronous walk over children -------------------
        // Level L reads invq[lo, hi) and appends the children it cuts off at invq[hi...]
        // through its own counter lc[(L+1)%3], so every CTA derives the same level bounds
        // even while faster CTAs already append the next level.  inv_count (the roots,
        // written by k_delete) is not written by this kernel.
        unsigned lo = 0, hi = __ldcg(&ctl->inv_count);
        int level = 0;
        bool need_pj = false;
        for (;;) {
            const unsigned nh = __ldcg(&ctl->bh[level % 3]);
            if (lo >= hi && nh == 0) break;
            if (level >= p.bfs_levels) {
                need_pj = true;
                break;
            }
            if (leader) {
                ctl->bh[(level + 2) % 3] = 0;
                ctl->lc[(level + 2) % 3] = 0;
            }
            MarkOp op{g.state, g.adj, g.inv_tag, p.epoch, g.invq + hi, &ctl->lc[(level + 1) % 3], &ls};
            run_items(op, p, g.invq + lo, hi - lo, (level & 1) ? g.h1 : g.h0, nh, (level & 1) ? g.h0 : g.h1,
                      &ctl->bh[(level + 1) % 3]);
            if (!grid_sync(ctl)) return;
            lo = hi;
            hi += __ldcg(&ctl->lc[(level + 1) % 3]);
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
                    t = (v == (unsigned)g.src || par == kNone) ? kTagOk : par;
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
            for (unsigned base = gtid - lane; base < (unsigned)g.n; base += nthreads) {
                const unsigned v = base + lane;
                bool newinv = false;
                if (v < (unsigned)g.n && __ldcg(&g.jm[v]) == kTagInv && __ldcg(&g.inv_tag[v]) != p.epoch) {
                    g.inv_tag[v] = p.epoch;
                    g.state[v] = kInfState;
                    newinv = true;
                }
                warp_append(newinv, v, g.invq + hi, &ctl->pj_cnt);
            }
            if (!grid_sync(ctl)) return;
            hi += __ldcg(&ctl->pj_cnt);
        }
        if (leader) {
            ctl->ts[1] = globaltimer();
            ctl->stat[ST_INV] = hi;
        }

        // ---- B. seeds: surviving insertions relax both ends; cut-off vertices pull -------
        const unsigned tag0 = rbase + 1;
        for (long long base = (long long)(gtid - lane); base < p.k; base += nthreads) {
            const long long i = base + lane;
            const bool has = i < p.k;
            const int4 c = has ? p.chg[i] : make_int4(0, 0, 0, -1);
            bool alive = false;
            if (has && c.w == 1) {
                const long long s0 = p.slot[2 * i], s1 = p.slot[2 * i + 1];
                const long long s = s0 >= 0 ? s0 : s1;
                alive = s >= 0 && __ldg(&g.adj[s]).y >= 0;
            }
            bool pa = false, pb = false;
            if (alive) {
                const unsigned a = (unsigned)c.x, b = (unsigned)c.y;
                const unsigned long long sa = __ldcg(&g.state[a]), sb = __ldcg(&g.state[b]);
                if ((sa >> 32) != kDistInf) pb = relax_to(g.state, b, (sa >> 32) + (unsigned)c.z, a, c.z, sb, ls);
                if ((sb >> 32) != kDistInf)
                    pa = relax_to(g.state, a, (sb >> 32) + (unsigned)c.z, b, c.z, __ldcg(&g.state[a]), ls);
                ls.edges_relax += 2;
            }
            const bool db = pb && claim_push(g.push_tag, (unsigned)c.y, tag0);
            warp_append(db, (unsigned)c.y, g.q0, &ctl->cq[0]);
            const bool da = pa && claim_push(g.push_tag, (unsigned)c.x, tag0);
            warp_append(da, (unsigned)c.x, g.q0, &ctl->cq[0]);
        }
        const unsigned ninv = hi;
        {
            PullOp op{g.state, g.adj, g.push_tag, tag0, g.q0, &ctl->cq[0], &ls, kInfState, false};
            run_items(op, p, g.invq, ninv, nullptr, 0, g.h0, &ctl->ph);
        }
        if (!grid_sync(ctl)) return;
        const unsigned nph = __ldcg(&ctl->ph);
        if (nph > 0) {
            PullOp op{g.state, g.adj, g.push_tag, tag0, g.q0, &ctl->cq[0], &ls, kInfState, false};
            run_items(op, p, nullptr, 0, g.h0, nph, g.h1, &ctl->ph);
            if (!grid_sync(ctl)) return;
        }
    }
    if (leader) ctl->ts[2] = globaltimer();

    // ---- C. relaxation rounds ---------------------------------------------------------
    long long r = 0;
    unsigned long long frontier = 0;
    for (;; r++) {
        const unsigned nq = __ldcg(&ctl->cq[r % 3]), nh = __ldcg(&ctl->ch[r % 3]);
        if (nq == 0 && nh == 0) break;
        if (r >= p.max_rounds) {
            if (leader) set_status(ctl, -5 /* NO_CONVERGENCE */);
            break;
        }
        frontier += (unsigned long long)nq + nh;
        if (leader) {
            ctl->cq[(r + 2) % 3] = 0;
            ctl->ch[(r + 2) % 3] = 0;
        }
        const bool odd = (r & 1) != 0;
        RelaxOp op{g.state, g.adj, g.push_tag, rbase + (unsigned)r + 2u, odd ? g.q0 : g.q1,
                   &ctl->cq[(r + 1) % 3], &ls};
        run_items(op, p, odd ? g.q1 : g.q0, nq, odd ? g.h1 : g.h0, nh, odd ? g.h0 : g.h1, &ctl->ch[(r + 1) % 3]);
        if (!grid_sync(ctl)) break;
    }
    flush_stats(ctl, ls);
    if (leader) {
        ctl->stat[ST_ROUNDS] = (unsigned long long)r;
        ctl->stat[ST_FRONTIER] = frontier;
        ctl->round_base = rbase + (unsigned)r + 4u;
        ctl->ts[3] = globaltimer();
    }
}

}  // namespace dsssp

// ---- host launch wrappers (the kernels above are launched only through these) -----------
namespace dsssp {

void count_launch(int n);

cudaError_t launch_front(const UpdParams& p, int4* ovf, bool with_append, cudaStream_t s) {
    const unsigned grid = (unsigned)((p.k + 255) / 256);
    if (grid == 0) return cudaSuccess;
    if (with_append) {
        k_prepare<<<grid, 256, 0, s>>>(p);
        k_append<<<grid, 256, 0, s>>>(p, ovf);
        count_launch(2);
    }
    k_delete<<<grid, 256, 0, s>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_relocate(const UpdParams& p, cudaStream_t s) {
    const unsigned grid = (unsigned)((p.k + 255) / 256);
    if (grid == 0) return cudaSuccess;
    k_relocate<<<grid, 256, 0, s>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t update_occupancy(int block, int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_update, block, 0);
}

cudaError_t launch_update(const UpdParams& p, int grid, int block, cudaStream_t s) {
    UpdParams copy = p;
    void* args[] = {&copy};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_update, dim3((unsigned)grid), dim3((unsigned)block),
                                                args, 0, s);
    count_launch(1);
    return e;
}

}  // namespace dsssp
