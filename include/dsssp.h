/*
 * dsssp.h -- C ABI of the GB300-native dynamic single-source-shortest-path engine.
 *
 * The engine keeps an undirected, integer-weighted graph and a shortest-path tree resident
 * on one GPU and applies batches of edge insertions and deletions to them.  It is a drop-in
 * for the update path of ArindamK92/DynamicSSSPv2 (SSSPmainForUndirected.cu, whose only
 * interface is its command line and three text formats); each entry point below names the
 * part of the reference it replaces.
 *
 * Conventions
 *   - Every function that can fail returns 0 (DSSSP_OK) or a negative DSSSP_E* code;
 *     dsssp_last_error() gives a message for the calling thread's last failure.  A batch
 *     may also return the positive DSSSP_W_RECOMPUTED: it succeeded by a slower route.
 *   - Host buffers are owned by the caller; device memory is owned by the library.
 *   - Vertex ids are 0..n-1.  Weights are int32 >= 0.  A distance is an integer below
 *     2^32-1; an unreachable vertex has parent -1 and distance DSSSP_UNREACHABLE.
 *   - A dsssp_graph is not thread-safe; separate graphs may be used from separate threads.
 *   - Memory returned by the text readers and generators is released with dsssp_free().
 */
#ifndef DSSSP_H
#define DSSSP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSSSP_OK 0
#define DSSSP_E_INVAL (-1)          /* bad argument */
#define DSSSP_E_OOM (-2)            /* device or host allocation failed */
#define DSSSP_E_BAD_VERTEX (-3)     /* vertex id outside 0..n-1 */
#define DSSSP_E_CUDA (-4)           /* CUDA runtime error */
#define DSSSP_E_NO_CONVERGENCE (-5) /* relaxation round cap reached */
#define DSSSP_E_TIMEOUT (-6)        /* a bounded device-side wait gave up */
#define DSSSP_E_BAD_TREE (-7)       /* tree has no unique root, a parent cycle or bad ids */
#define DSSSP_E_OVERFLOW (-8)       /* a distance does not fit below 2^32-1 */
#define DSSSP_E_IO (-9)             /* file could not be opened or written */
#define DSSSP_E_BAD_WEIGHT (-10)    /* negative weight on an edge that is added */
#define DSSSP_E_NO_DEVICE (-11)     /* no usable CUDA device */
#define DSSSP_E_COOP (-12)          /* the persistent update kernel could not be co-resident */

/* A batch whose update kernel failed (a timed-out device wait, the round cap, an internal list
 * capacity or a parent cycle) after its edits reached the adjacency, recovered by computing
 * the trees again from the roots on the updated graph (opts.recover): the graph and tree are
 * exactly what a successful batch gives; stats.recovered_from holds the failure's code and
 * dsssp_last_error() describes it.  A success code, not an error. */
#define DSSSP_W_RECOMPUTED 2

#define DSSSP_UNREACHABLE (-1)

typedef struct dsssp_graph dsssp_graph;

/* One change record: op 1 = insert, op 0 = delete, any other op is ignored
 * (the reference's changeEdge, all_structure_undir.cuh:52-57, read by readin_changes,
 * all_structure_undir.cuh:89-126).  16 bytes. */
typedef struct {
    int32_t u, v, w, op;
} dsssp_change;

/* Tunables.  dsssp_default_opts() fills defaults; the autotuner writes the same fields. */
typedef struct {
    int32_t device;       /* CUDA device ordinal */
    int32_t slack_pct;    /* per-row insertion slack, percent of the row's degree */
    int32_t slack_min;    /* minimum free slots per row */
    int32_t small_deg;    /* edges per thread work item (multiple of 4, 4..64): a frontier
                             vertex of degree d <= small_deg is one thread's item, a longer row
                             up to large_deg is split into ceil(d/small_deg) thread items */
    int32_t large_deg;    /* rows above this degree are split into CTA items of `chunk` edges */
    int32_t chunk;        /* edges per CTA work item */
    int32_t bfs_levels;   /* subtree walk levels before switching to pointer jumping */
    int32_t block;        /* threads per CTA of the update kernel (multiple of 32) */
    int32_t ctas_per_sm;  /* resident CTAs per SM of the update kernel; 0 = occupancy max */
    int32_t timing;       /* 1 = record CUDA events and phase timestamps into the stats; 2 = also
                             events between the batch front kernels (t_delete_ms, t_append_ms),
                             which costs a batch a few microseconds */
    int64_t max_rounds;   /* relaxation round cap; 0 = 2n + 16 */
    int32_t spare_pct;    /* extra adjacency slots, percent of the laid-out rows, into which a
                             row that runs out of slack moves (no full repack) unless dropping
                             its tombstones leaves it room in place; 0..400 */
    int32_t delta;        /* near-far bucket width of the relaxation rounds: 0 = plain frontier
                             rounds; > 0 = a round relaxes only vertices whose distance is below
                             a threshold T, the others wait until the near frontier is empty and
                             T moves to (least waiting distance) + delta.  Same results; far
                             fewer rounds and relaxations on high-diameter graphs.  -1 (the
                             default) = automatic: near-far with 32 x the mean edge weight once
                             the last batch or tree computation needed more than auto_rounds
                             rounds, plain rounds otherwise.  Costs 12 bytes per vertex, allocated when
                             first used. */
    int32_t launch_graph; /* 1 = a batch's launch sequence (control-block reset, deletion-set
                             reset, the four kernels, the status read) is replayed from an
                             instantiated CUDA graph whose node parameters are updated per
                             batch; 0 = plain stream launches.  Falls back to plain launches
                             if the graph cannot be built. */
    int32_t recover;      /* 1 (the default) = a batch whose update kernel fails after its edits
                             reached the adjacency recomputes the trees from the roots and returns
                             DSSSP_W_RECOMPUTED (or, if that fails too, the error, and the tree
                             must be loaded or computed before the next batch); 0 = return the
                             error and leave the tree as the kernel left it (unfinished) */
    int32_t warp_agg;     /* 1 = warp-aggregated distance offers: lanes of a warp offering to the
                             same vertex are grouped (__match_any_sync) and only the least offer
                             is issued as a 64-bit atomicMin; 0 (the default) = one atomicMin per
                             improving offer.  Same results either way. */
    int32_t solo_waves;   /* a walk level or relaxation round with at most this many CTA-waves of
                             work items runs on one CTA with block barriers instead of the whole
                             grid (0..64; 0 = never; default 2) */
    int32_t auto_rounds;  /* delta = -1: near-far rounds start once the last batch or tree
                             computation needed more than this many rounds (default 256) */
    int32_t group_ctas;   /* a relaxation round too large for one CTA (solo_waves) but at most
                             group_waves CTA-waves on group_ctas CTAs runs on the first group_ctas
                             CTAs with a barrier of their own while the other CTAs wait: a shorter
                             barrier and the slowest of group_ctas dependent chains instead of all
                             CTAs' (high-diameter graphs run thousands of such rounds); 0 (the
                             default) = off: measured slower, the rounds wait on their items'
                             dependent chains more than on the barrier */
    int32_t group_waves;  /* see group_ctas (1..64, default 2) */
} dsssp_opts;

/* Counters of one batch (or one tree computation), read back from the device. */
typedef struct {
    int64_t n_ins;             /* insertion records (op 1) */
    int64_t n_del;             /* deletion records (op 0) */
    int64_t n_ignored;         /* records with another op */
    int64_t n_roots;           /* vertices cut off directly by a deleted tree edge */
    int64_t n_invalidated;     /* all vertices of the cut-off subtrees (roots included) */
    int64_t inv_levels;        /* subtree-walk levels */
    int64_t pj_passes;         /* pointer-jumping passes (0 if the walk finished) */
    int64_t rounds;            /* relaxation rounds */
    int64_t frontier_total;    /* sum of frontier sizes over the rounds */
    int64_t edges_relaxed;     /* adjacency entries scanned by relaxation rounds and seeds */
    int64_t edges_inval;       /* adjacency entries scanned by the subtree walk and pulls */
    int64_t del_probed;        /* adjacency entries examined to find deleted edges */
    int64_t updates;           /* atomic updates that lowered a distance */
    int64_t overflow_entries;  /* inserted entries that did not fit a row's slack */
    int64_t repacks;           /* adjacency repacks this call triggered */
    int64_t n_killed;          /* insertions removed again by a deletion of the same batch */
    int64_t work_items;        /* work items (te-edge thread items + CTA chunks) created */
    double t_step1_ms;         /* insert + delete kernels (CUDA events) */
    double t_inval_ms;         /* subtree invalidation (device timestamps) */
    double t_relax_ms;         /* seeding + relaxation rounds (device timestamps) */
    double t_update_ms;        /* the persistent update kernel (CUDA events) */
    double t_total_ms;         /* the whole batch on the device (CUDA events) */
    double bytes_alg;          /* algorithmic bytes of the batch (byte model of the engine) */
    double bytes_alg_update;   /* the update kernel's algorithmic bytes (per-unit byte model:
                                  cut-off vertices and children, frontier vertices and their
                                  scanned edges, lowering atomics) */
    int64_t advances;          /* near-far threshold advances (0 when delta = 0) */
    int64_t tombstoned;        /* adjacency entries the batch's deletions tombstoned */
    int64_t graph_launch;      /* 1 = the batch was replayed from the instantiated CUDA graph */
    double bytes_engine_update; /* the update kernel's bytes by the engine's own count (all row
                                   scans of the subtree walk included; bytes_alg_update credits
                                   only the task byte model's units) */
    double t_delete_ms;        /* k_delete alone (CUDA events; batches at timing level 2) */
    double t_append_ms;        /* k_append alone, seeds included (CUDA events; batches at timing
                                  level 2; with row growth it spans the growth too) */
    int64_t recovered_from;    /* DSSSP_W_RECOMPUTED: the code of the failure recovered from */
    double t_recompute_ms;     /* DSSSP_W_RECOMPUTED: the recomputation of the trees (CUDA events) */
    double t_seed_ms;          /* the seeding and pull phase alone (part of t_relax_ms) */
} dsssp_stats;

/* ---- engine ------------------------------------------------------------------------ */

void dsssp_default_opts(dsssp_opts* o);

/* sizeof of the ABI's structs as this library was built: dsssp_opts, dsssp_stats,
 * dsssp_server_opts, dsssp_request_info, dsssp_tune_result (out[0..4]), so that a binding
 * (ctypes, cgo, JNI) can refuse to run against a header it was not written for.  Returns
 * the number of sizes written, at most cap. */
int dsssp_abi_sizes(size_t* out, int32_t cap);

/* Builds the device-resident graph (CSR rows sorted by neighbour, with per-row slack) from
 * an undirected edge list; each line (u[i], v[i], w[i]) adds both directions.
 * Replaces read_graphEdges + the CSR flatten and copy (all_structure_undir.cuh:178-198,
 * SSSPmainForUndirected.cu:42-91).  o may be NULL for defaults. */
int dsssp_graph_create(int32_t n, int64_t m, const int32_t* u, const int32_t* v,
                       const int32_t* w, const dsssp_opts* o, dsssp_graph** out);

void dsssp_graph_destroy(dsssp_graph* g);

/* n, live adjacency entries, slot capacity, device bytes held, source (-1 if no tree). */
int dsssp_graph_info(const dsssp_graph* g, int64_t* n, int64_t* entries, int64_t* capacity,
                     int64_t* device_bytes, int32_t* source);

/* Loads a shortest-path tree: parent[v] (-1 = unreachable, the root has parent[root]==root
 * and dist 0) and dist[v].  Replaces read_SSSP's copy into managed memory
 * (all_structure_undir.cuh:133-171, SSSPmainForUndirected.cu:147-165). */
int dsssp_tree_load(dsssp_graph* g, const int32_t* parent, const int64_t* dist);

/* Computes the tree from scratch on the GPU from source src (replaces running
 * seqSSSPwithDist_undir.cpp to make the initial SSSP file). */
int dsssp_tree_compute(dsssp_graph* g, int32_t src, dsssp_stats* st);

/* Several sources at once: each vertex gets its distance to the nearest source.  With one
 * source per connected component this is one tree per component, as used by the batching
 * and serving layers (one graph store holding many tenant graphs).  No counterpart in the
 * reference (its Dijkstra has one hard-coded source, seqSSSPwithDist_undir.cpp:196). */
int dsssp_tree_compute_multi(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st);

/* Adds k sources to the resident forest without recomputing it: each becomes a root
 * (distance 0, its own parent) and relaxation from them lowers every distance they improve,
 * so the result is the exact forest from the old roots and the new ones together (the current
 * distances stay valid upper bounds).  On a graph with no tree yet it is dsssp_tree_compute_multi.
 * Used to bring a new tenant's part of a pooled store to life.  No counterpart in the reference. */
int dsssp_tree_add_sources(dsssp_graph* g, const int32_t* srcs, int32_t k, dsssp_stats* st);

/* Removes every edge of the vertex range [first, first + count) and makes its vertices
 * unreachable (roots in it stop being roots); the range must be closed under adjacency (no
 * live edge between it and the rest: DSSSP_E_INVAL otherwise, nothing changed).  The entries
 * become tombstones that dsssp_graph_compact reclaims.  Used to retire a tenant's part of a
 * pooled store.  No counterpart in the reference. */
int dsssp_graph_clear_range(dsssp_graph* g, int32_t first, int32_t count);

/* Like dsssp_tree_load, but any number (>= 1) of roots: a forest of shortest-path trees,
 * e.g. one per tenant graph of a pooled graph store. */
int dsssp_forest_load(dsssp_graph* g, const int32_t* parent, const int64_t* dist);

/* Reads the current tree back into host arrays of n entries (either may be NULL).
 * Replaces printSSSP and the host print of SSSPmainForUndirected.cu:298-312. */
int dsssp_tree_read(dsssp_graph* g, int32_t* parent, int64_t* dist);

/* Like dsssp_tree_read with 32-bit distances, the width of RT_Vertex.Dist in the reference
 * (all_structure_undir.cuh:66-75): dist[v] is the exact distance as an unsigned 32-bit integer
 * (every distance the engine holds fits), DSSSP_UNREACHABLE32 for an unreachable vertex,
 * whose parent is -1.  8 bytes per vertex cross the host link instead of 12. */
#define DSSSP_UNREACHABLE32 0xFFFFFFFFu
int dsssp_tree_read32(dsssp_graph* g, int32_t* parent, uint32_t* dist);

/* dsssp_tree_read32 without waiting: the tree as it is now is unpacked on the device at once
 * (into staging of its own) and copied to the host arrays on a copy stream of the graph, and
 * the call returns.  The next batch may be applied meanwhile (it waits only for the unpack),
 * so the copy overlaps its upload and kernels; the host arrays hold the tree once
 * dsssp_tree_read_wait returns (pinned host memory makes the copy asynchronous; with pageable
 * memory it completes inside the call).  A read unpacks only after the previous read's copy has
 * finished, so once a batch applied after read i + 1 has completed, read i's arrays are
 * filled.  Either array may be NULL.  No counterpart in the reference, which prints
 * the first distances after the update (SSSPmainForUndirected.cu:298-312). */
int dsssp_tree_read32_async(dsssp_graph* g, int32_t* parent, uint32_t* dist);
/* Waits for the copies of dsssp_tree_read32_async (returns at once if none is outstanding). */
int dsssp_tree_read_wait(dsssp_graph* g);

/* Test hooks for failure detection (not for production use).
 * DSSSP_DEBUG_SPIN_LIMIT: polls of about 1 us before a grid barrier of the update kernel
 *   gives up with DSSSP_E_TIMEOUT (0 = the default 2^20, about 1 s).
 * DSSSP_DEBUG_STALL_US: the last CTA of the next launch of the update kernel waits this many
 *   microseconds (0..1,000,000; 0 = off) before its first grid barrier, so that a small spin
 *   limit runs out: the batch fails with DSSSP_E_TIMEOUT and the device stays usable.  The
 *   hook applies to one launch and then clears itself. */
#define DSSSP_DEBUG_SPIN_LIMIT 1
#define DSSSP_DEBUG_STALL_US 2
int dsssp_debug_set(dsssp_graph* g, int32_t what, int64_t value);

/* Certificate of the resident tree on the device: counts violations of (a) no live edge
 * (u, v, w) with dist[u] + w < dist[v] (an unreachable v included), (b) every reachable
 * vertex other than a root has a live edge to its parent p with dist[p] + w == dist[v],
 * (c) a root (its own parent) has distance 0, (d) parent chains end at a root (no cycle).
 * Zero violations means the distances are the exact shortest distances from the set of
 * roots and the parents form a shortest-path forest.  *roots gets the number of roots and
 * *first_bad the least violating vertex (-1 if none); either may be NULL. */
int dsssp_tree_validate(dsssp_graph* g, int64_t* violations, int64_t* roots, int32_t* first_bad);

/* Reads parent and dist of vertices [first, first + count) into caller arrays of count
 * entries (the part of a pooled store that belongs to one graph). */
int dsssp_tree_read_range(dsssp_graph* g, int32_t first, int32_t count, int32_t* parent, int64_t* dist);

/* Reads back only the part of the tree the last batch may have changed: every vertex that
 * the batch cut off or whose distance it lowered (a superset of the vertices whose parent or
 * distance differs from before the batch), in no particular order.  vertex/parent/dist get
 * *count entries (at most cap; cap = n always suffices).  A caller that keeps the previous
 * tree on the host applies these entries to have the updated tree, at a fraction of the
 * copy volume of dsssp_tree_read.  After a batch with no records *count is 0.  DSSSP_E_INVAL
 * when there is no successful batch since the tree was loaded or computed (a batch that
 * returned DSSSP_W_RECOMPUTED computed the whole tree again: read it with dsssp_tree_read), or
 * when the set exceeds cap (then *count is its size). */
int dsssp_tree_read_changed(dsssp_graph* g, int32_t* vertex, int32_t* parent, int64_t* dist,
                            int64_t cap, int64_t* count);

/* Applies one change batch from host memory and waits for it: copies the records to the
 * device, appends insertions into row slack, deletes every entry matching a deletion,
 * invalidates cut-off subtrees and relaxes to the new shortest-path tree.
 * Replaces STEP1 + STEP2 of SSSPmainForUndirected.cu:196-292 (deleteEdge, insertEdge,
 * filterAffectedNodes, updateNeighbors_del, filterAllAffected, updateNeighbors).
 * stream is a cudaStream_t (NULL = the library's own stream).  st may be NULL. */
int dsssp_apply_batch(dsssp_graph* g, const dsssp_change* changes, int64_t k, void* stream,
                      dsssp_stats* st);

/* Asynchronous form of dsssp_apply_batch: enqueues the copy of the k host records and the
 * update on stream and returns without waiting; dsssp_batch_finish() waits and reports.  The
 * records must stay unchanged until then (the copy runs on the stream; pinned memory makes it
 * truly asynchronous), so the caller can prepare its next batch meanwhile. */
int dsssp_apply_batch_host_async(dsssp_graph* g, const dsssp_change* changes, int64_t k, void* stream);

/* Asynchronous form for callers that keep the batch on the device: enqueues the update
 * of k records at device address d_changes on stream and returns without waiting.
 * dsssp_batch_finish() waits, handles a slack overflow and reports the status. */
int dsssp_apply_batch_async(dsssp_graph* g, const dsssp_change* d_changes, int64_t k,
                            void* stream);
int dsssp_batch_finish(dsssp_graph* g, dsssp_stats* st);

/* Changes the launch tunables of a graph (all fields but device and the slack, which are
 * fixed when the rows are laid out); used by the autotuner.  No counterpart in the reference
 * (its block size is a compile-time macro, SSSPmainForUndirected.cu:11). */
int dsssp_graph_set_opts(dsssp_graph* g, const dsssp_opts* o);
int dsssp_graph_get_opts(const dsssp_graph* g, dsssp_opts* o);

/* Device-side copy of the graph and tree, and its restore (benchmark repetition). */
int dsssp_graph_snapshot(dsssp_graph* g);
int dsssp_graph_restore(dsssp_graph* g, void* stream);

/* Removes tombstones and re-sorts every row, restoring full slack (off the update path). */
int dsssp_graph_compact(dsssp_graph* g);

/* Storage health, to decide when to compact: live adjacency entries, tombstoned entries
 * since the last layout, and used / total slots of the spare region that rows move into
 * when they run out of slack.  Any pointer may be NULL. */
int dsssp_graph_health(const dsssp_graph* g, int64_t* live_entries, int64_t* dead_entries,
                       int64_t* spare_used, int64_t* spare_total);

/* Pinned host memory for fast copies (cudaMallocHost) and its release. */
void* dsssp_host_alloc(size_t bytes);
void dsssp_host_free(void* p);

/* Number of kernels this library has launched in this process. */
int64_t dsssp_launch_count(void);

const char* dsssp_last_error(void);
const char* dsssp_strerror(int code);
void dsssp_free(void* p);

/* ---- autotuner ----------------------------------------------------------------------
 * Times candidate settings of the update -- edges per thread item and the CTA-chunk
 * thresholds (degree buckets), walk depth before pointer jumping, CTA size and residency,
 * solo-step width, near-far bucket widths scaled by the batch's mean weight -- on a
 * representative batch from one starting state (device snapshot and restore), sets the
 * fastest on the graph and caches it per size class (log2 vertices, log2 adjacency entries,
 * log2 batch size) in a text file.  No counterpart in the reference (its block size is a
 * compile-time macro, SSSPmainForUndirected.cu:11). */
typedef struct {
    char key[32];      /* size class "v<log2 n>_e<log2 entries>_b<log2 k>" */
    dsssp_opts opts;   /* the chosen options (also set on the graph) */
    double ms;         /* their device time on the batch (median of reps) */
    int32_t trials;    /* candidates timed; 0 when taken from the cache */
    int32_t cached;    /* 1 = taken from the cache without timing */
} dsssp_tune_result;

/* Tunes g for batches like changes[0..k): a cached size class is applied without timing
 * (unless force); otherwise every candidate runs the batch once per round for reps rounds
 * (0 = 3), and the candidate with the least median time is set and written to cache_path
 * (NULL: not cached) -- the graph's own setting (the first candidate) unless another is at
 * least 3 % faster.  Replaces the graph's snapshot and leaves
 * the graph and tree as they were before the call. */
int dsssp_autotune(dsssp_graph* g, const dsssp_change* changes, int64_t k, const char* cache_path,
                   int32_t reps, int32_t force, dsssp_tune_result* out);
/* Sets the cached options of g's size class for batches of k records; DSSSP_E_INVAL if the
 * cache has none (nothing changed). */
int dsssp_autotune_lookup(dsssp_graph* g, int64_t k, const char* cache_path, dsssp_tune_result* out);
/* The size-class key of a graph of n vertices and `entries` adjacency entries with k-record
 * batches (no device needed). */
int dsssp_tune_size_class(int64_t n, int64_t entries, int64_t k, char* key, size_t cap);
/* The candidate options the tuner times for batch changes[0..k) starting from base: *count of
 * them, the first cap written to out (no device needed). */
int dsssp_tune_candidates(const dsssp_opts* base, const dsssp_change* changes, int64_t k,
                          dsssp_opts* out, int32_t cap, int32_t* count);

/* ---- shortest-path tree without device allocation ---------------------------------- */

/* Largest graph dsssp_sssp_noalloc() accepts: its work space is a fixed static device array
 * of about 8.2 MB that every GPU that loads this library keeps until the process exits. */
#define DSSSP_NOALLOC_MAX_VERTICES 65536
#define DSSSP_NOALLOC_MAX_ENTRIES 1048576

/* Shortest-path tree from src of a graph held in the caller's device memory, for callers
 * that must not allocate device memory where they call it (for example a plugin's enqueue
 * callback inside an inference or streaming runtime that owns the memory budget, or a
 * pipeline that reserved all device memory up front; cudaMalloc may also synchronize the
 * device).  No counterpart in the reference: it has no library interface, and its CLI
 * allocates per run.
 *   d_row_off  n+1 int64 row offsets (d_row_off[0] == 0, d_row_off[n] == nnz)
 *   d_adj      nnz (column, weight) int32 pairs, 8-byte aligned, weights >= 0; an
 *              undirected edge appears in both rows
 *   d_parent   n int32 outputs (-1 = unreachable, src is its own parent)
 *   d_dist     n int64 outputs (DSSSP_UNREACHABLE = -1 for unreachable vertices)
 * All pointers are device addresses on the current device, each aligned to its element size
 * (d_row_off, d_adj and d_dist to 8 bytes, d_parent to 4); stream is a cudaStream_t (NULL =
 * legacy default stream).  n <= DSSSP_NOALLOC_MAX_VERTICES and nnz <=
 * DSSSP_NOALLOC_MAX_ENTRIES, else DSSSP_E_INVAL; so is a NULL or misaligned pointer (refused
 * before anything is launched) and a malformed CSR (offsets not monotone from 0 to nnz, a
 * column outside 0..n-1 or a negative weight; found on the device, outputs then undefined).
 * The call is blocking: it synchronizes stream and copies the status word to the host before
 * it returns, so the calling thread waits for the whole computation, and no call (the first
 * or any later one) may be made while stream is being captured into a CUDA graph: the
 * synchronization would invalidate the capture.
 * It calls no cudaMalloc, cudaFree or other allocating routine.  The first call on a device
 * also looks up the work space's device address (cudaGetSymbolAddress) and the update
 * kernel's occupancy.  All calls on a device share
 * the one work space (each call re-initialises what it needs), so calls that overlap on the
 * GPU, from any thread or stream, race and must be serialised by the caller. */
int dsssp_sssp_noalloc(int32_t n, int64_t nnz, const int64_t* d_row_off, const int32_t* d_adj,
                       int32_t src, int32_t* d_parent, int64_t* d_dist, void* stream);

/* ---- reference text formats (all_structure_undir.cuh:89-198, README.md:25-37) ---- */

/* graph file: "u v w" per line, each undirected edge once.  Vertex ids must be < n
 * (the reference's AdjList.at throws otherwise).  Allocates *u, *v, *w. */
int dsssp_read_graph_file(const char* path, int32_t n, int32_t** u, int32_t** v, int32_t** w,
                          int64_t* m);

/* change file: "u v w op" per line.  Allocates *changes (all lines with 4 fields; the
 * engine ignores ops other than 0/1 as the reference does). */
int dsssp_read_changes_file(const char* path, int32_t n, dsssp_change** changes, int64_t* k);

/* SSSP file: "node parent dist" per line, read with the semantics of read_SSSP: missing
 * vertices and parent -1 mean unreachable.  dist may be written as an integer or in the
 * %g form the reference's Dijkstra prints; *lossy counts values that were not integers.
 * Fills caller arrays parent[n], dist[n]. */
int dsssp_read_sssp_file(const char* path, int32_t n, int32_t* parent, int64_t* dist,
                         int64_t* lossy);

/* Writes "node parent dist" lines (integers; unreachable: parent -1 dist -1). */
int dsssp_write_sssp_file(const char* path, int32_t n, const int32_t* parent,
                          const int64_t* dist);

/* Writes change records in the reference generator's line format (createChangedEdges.cpp:104,
 * 116): "u  v w 1 " for an insertion, "u v w 0 " for a deletion; readable by
 * dsssp_read_changes_file and by the reference's readin_changes. */
int dsssp_write_changes_file(const char* path, const dsssp_change* changes, int64_t k);

/* ---- binary cache ------------------------------------------------------------------
 * Binary images of an edge list and of a tree (32-byte header with magic, sizes and a
 * checksum, then the arrays) that load at file-system speed instead of being parsed.  A
 * reader fails with DSSSP_E_IO on another magic, other sizes than expected, a short file or a
 * checksum mismatch.  Replaces nothing in the reference (it parses text on every run,
 * all_structure_undir.cuh:133-198). */
int dsssp_write_graph_binary(const char* path, int32_t n, int64_t m, const int32_t* u,
                             const int32_t* v, const int32_t* w);
/* Allocates *u, *v, *w (free with dsssp_free); vertex ids are range-checked like the text
 * reader's (DSSSP_E_BAD_VERTEX). */
int dsssp_read_graph_binary(const char* path, int32_t n, int32_t** u, int32_t** v, int32_t** w,
                            int64_t* m);
int dsssp_write_sssp_binary(const char* path, int32_t n, const int32_t* parent,
                            const int64_t* dist);
/* parent[n] and dist[n] are caller-owned. */
int dsssp_read_sssp_binary(const char* path, int32_t n, int32_t* parent, int64_t* dist);

/* ---- seeded synthetic inputs (SplitMix64-based counter PRNG, same result on any host) --- */

/* Erdos-Renyi: exactly m distinct undirected pairs u<v, w uniform in [wlo, whi]. */
int dsssp_gen_er(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed, int32_t** u,
                 int32_t** v, int32_t** w);

/* RMAT(a, b, c, 1-a-b-c) on 2^scale vertices: exactly m distinct non-self-loop pairs
 * (u<v after normalisation, ids not permuted), w uniform in [wlo, whi]. */
int dsssp_gen_rmat(int32_t scale, int64_t m, double a, double b, double c, int32_t wlo,
                   int32_t whi, uint64_t seed, int32_t** u, int32_t** v, int32_t** w);

/* rows x cols grid, id = r*cols + c: 4-neighbour edges with a fraction remove_frac removed
 * uniformly, plus n_diag distinct random diagonals (r+-1, c+-1); w uniform in [wlo, whi]. */
int dsssp_gen_grid(int32_t rows, int32_t cols, double remove_frac, int64_t n_diag,
                   int32_t wlo, int32_t whi, uint64_t seed, int32_t** u, int32_t** v,
                   int32_t** w, int64_t* m);

/* Insertion endpoint models for dsssp_gen_changes. */
#define DSSSP_INS_UNIFORM 0 /* uniform random pairs */
#define DSSSP_INS_RMAT 1    /* pairs drawn from RMAT(p0, p1, p2) on 2^scale vertices */
#define DSSSP_INS_LOCAL 2   /* pairs within Chebyshev distance p0 on a grid of `scale` columns */

/* A change batch over the graph (eu, ev, ew): n_ins insertions of pairs that are not edges
 * of the graph (and distinct), w uniform in [wlo, whi]; n_del deletions sampled without
 * replacement from the graph's lines.  Records are shuffled.  Allocates *changes. */
int dsssp_gen_changes(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                      const int32_t* ew, int64_t n_ins, int64_t n_del, int32_t ins_kind,
                      int32_t scale, double p0, double p1, double p2, int32_t wlo, int32_t whi,
                      uint64_t seed, dsssp_change** changes);

/* The reference generator's sampling (createChangedEdges.cpp:49-125: `op_cE graph N k pct`)
 * with a seeded stream instead of rand(): num_changes records of which
 * (int)(num_changes*ins_pct/100) are insertions, interleaved by coin flips; insertions are
 * uniform pairs u<v (u != v) with w uniform in [wlo, whi] (the reference uses [0, 99]) and
 * may repeat or duplicate existing edges; deletions are lines of the edge list drawn with
 * replacement.  Allocates *changes (num_changes records). */
int dsssp_gen_changes_ref(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                          const int32_t* ew, int64_t num_changes, int32_t ins_pct, int32_t wlo,
                          int32_t whi, uint64_t seed, dsssp_change** changes);

/* ---- batching: a pooled graph store ------------------------------------------------
 * Many graphs side by side in one engine graph (graph i owns ids [off[i], off[i] + n[i])):
 * one launch sequence applies a set of batches, at most one per graph, and each graph's
 * result equals applying its batch alone.  Graph-local vertex ids throughout; the pool
 * validates every batch against its graph (DSSSP_E_BAD_VERTEX / DSSSP_E_BAD_WEIGHT, nothing
 * applied).  No counterpart in the reference, which updates one graph per process run. */
typedef struct dsssp_pool dsssp_pool;
int dsssp_pool_create(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                      const int32_t* const* v, const int32_t* const* w, const dsssp_opts* o,
                      dsssp_pool** out);
void dsssp_pool_destroy(dsssp_pool* p);
/* The underlying engine graph (options, snapshots, statistics); owned by the pool. */
dsssp_graph* dsssp_pool_graph(dsssp_pool* p);
/* count + 1 offsets: offsets[i] = first id of graph i, offsets[count] = the end of the last
 * graph (graphs created with the pool are contiguous: graph i has offsets[i + 1] - offsets[i]
 * vertices; dsssp_pool_graph_range gives any graph's range). */
int dsssp_pool_offsets(const dsssp_pool* p, int64_t* offsets);
/* sources[i] = source of graph i (local id). */
int dsssp_pool_tree_compute(dsssp_pool* p, const int32_t* sources, dsssp_stats* st);
/* parent[i], dist[i] = tree of graph i (local ids, parent -1 = unreachable). */
int dsssp_pool_forest_load(dsssp_pool* p, const int32_t* const* parent, const int64_t* const* dist);
/* The union batch of nb batches (graphs[b] gets batches[b] of sizes[b] records) written to
 * out (cap records); *k = its size.  out may be NULL to validate and size it only. */
int dsssp_pool_union(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                     const int64_t* sizes, dsssp_change* out, int64_t cap, int64_t* k);
/* Applies the union batch of nb batches in one launch sequence and waits for it (returns what
 * dsssp_apply_batch returns, DSSSP_W_RECOMPUTED included). */
int dsssp_pool_apply(dsssp_pool* p, int32_t nb, const int32_t* graphs, const dsssp_change* const* batches,
                     const int64_t* sizes, dsssp_stats* st);
/* The tree of one graph (n[graph] entries, local ids). */
int dsssp_pool_tree_read(dsssp_pool* p, int32_t graph, int32_t* parent, int64_t* dist);
/* A pool with reserve_vertices spare vertex ids after its graphs (count may be 0 when the
 * reserve is not): room for graphs added later with dsssp_pool_add_graph. */
int dsssp_pool_create_reserved(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                               const int32_t* const* v, const int32_t* const* w, int64_t reserve_vertices,
                               const dsssp_opts* o, dsssp_pool** out);
/* Adds a graph (local ids, source src) in the lowest free id range of at least n ids: its source
 * becomes a new root and its edges go in as one insertion batch, whose relaxation builds its tree
 * (the other graphs are not touched).  *graph = its index.  DSSSP_E_OOM when no free range is
 * large enough (nothing changed). */
int dsssp_pool_add_graph(dsssp_pool* p, int32_t n, int64_t m, const int32_t* u, const int32_t* v,
                         const int32_t* w, int32_t src, int32_t* graph);
/* Removes graph `graph`: its edges become tombstones (dsssp_graph_compact reclaims them), its
 * vertices unreachable, its ids a free range for later graphs.  Its index is not reused. */
int dsssp_pool_remove_graph(dsssp_pool* p, int32_t graph);
/* First id and vertex count (0 once removed) of a graph in the pool's id space. */
int dsssp_pool_graph_range(const dsssp_pool* p, int32_t graph, int64_t* first, int32_t* n);
/* Vertex ids of the store, the free ones, and the largest free range; any may be NULL. */
int dsssp_pool_capacity(const dsssp_pool* p, int64_t* vertices, int64_t* free_vertices, int64_t* largest_free);
/* Device bytes the engine needs for a graph of n vertices and m undirected edges (admission). */
int64_t dsssp_estimate_footprint(int32_t n, int64_t m, int32_t slack_pct, int32_t slack_min);

/* ---- serving: a request loop with continuous batching ----------------------------
 * Tenants are admitted in order while their estimated footprint fits memory_budget and live
 * in one pool; a tenant that does not fit waits (its vertex ids are reserved) and is admitted
 * when a removal frees memory.  Tenants can also be added and removed while the server runs.
 * dsssp_submit validates a request, queues a copy of its batch and returns; a worker thread
 * runs epochs back to back, each taking the oldest waiting request of every admitted tenant
 * (oldest first, at most max_epoch_requests), copying their records once into a pinned buffer
 * (ids shifted into the pool's id space) and applying them as one union batch.  A tenant's
 * requests apply in arrival order and each result equals applying that batch alone.
 * Requests for a waiting or removed tenant are refused.  An epoch whose update kernel fails
 * is recovered on the device (DSSSP_W_RECOMPUTED, see dsssp_opts.recover): its requests are
 * served with that status and every tenant's tree stays exact.  While no request waits, the
 * worker compacts the store once its tombstones exceed compact_dead_frac of the live entries
 * (< 0: never) or its spare region is more than compact_spare_frac used.  Completed requests
 * are collected with dsssp_poll.  Submitting, polling, reading, adding and removing tenants
 * are thread-safe. */
typedef struct dsssp_server dsssp_server;
typedef struct {
    int64_t memory_budget;       /* device bytes for tenants; 0 = no limit */
    int32_t max_epoch_requests;  /* 0 = one request of every waiting tenant */
    int32_t record;              /* 1 = keep the tenant's tree after each request (dsssp_server_result) */
    double compact_dead_frac;    /* default 0.25 */
    double compact_spare_frac;   /* default 0.75 */
    int64_t reserve_vertices;    /* spare vertex ids for tenants added later (beyond the ids that
                                    tenants waiting at creation hold); default 0 */
    const char* tune_cache;      /* autotuner cache file (dsssp_autotune): each epoch runs with the
                                    cached options of its size class when there are any; NULL = the
                                    options given at creation throughout (default) */
} dsssp_server_opts;

#define DSSSP_REFUSED 1 /* request status: its tenant is not admitted (waiting, removed, unknown) */
/* request status DSSSP_W_RECOMPUTED (2): served; its epoch's update kernel failed and the trees
 * were recomputed (error says why) */

/* tenant states (dsssp_server_tenant_state) */
#define DSSSP_TENANT_WAITING 0  /* does not fit the memory budget or the free ids yet */
#define DSSSP_TENANT_ADMITTED 1
#define DSSSP_TENANT_REMOVED 2

typedef struct {
    int64_t id;
    int32_t tenant;
    int32_t status;      /* 0 served; DSSSP_REFUSED; a negative DSSSP_E_* code (error says why) */
    int64_t epoch;       /* epoch that served it, -1 if none */
    int64_t changes;     /* records in its batch */
    double arrival_us;   /* submission, microseconds since the server was created */
    double start_us;     /* its epoch's start */
    double done_us;      /* its epoch's end (the result is in the tree) */
    char error[96];
} dsssp_request_info;

void dsssp_default_server_opts(dsssp_server_opts* so);
/* Tenant t: graph (n[t], m[t], u[t], v[t], w[t]) with source sources[t]; trees of the admitted
 * tenants are computed on the device before the worker starts.  count may be 0 when
 * so->reserve_vertices is not (tenants then come with dsssp_server_add_tenant). */
int dsssp_server_create(int32_t count, const int32_t* n, const int64_t* m, const int32_t* const* u,
                        const int32_t* const* v, const int32_t* const* w, const int32_t* sources,
                        const dsssp_server_opts* so, const dsssp_opts* o, dsssp_server** out);
/* Finishes the queued requests, stops the worker and frees everything. */
void dsssp_server_destroy(dsssp_server* s);
/* Pool graph of a tenant, -1 if it is not admitted (waiting or removed). */
int dsssp_server_slot(const dsssp_server* s, int32_t tenant);
/* DSSSP_TENANT_WAITING / _ADMITTED / _REMOVED, or DSSSP_E_INVAL for no such tenant. */
int dsssp_server_tenant_state(const dsssp_server* s, int32_t tenant);
/* Adds a tenant (graph n, m, u, v, w with source src; the arrays are copied if it has to wait)
 * and returns its id in *tenant.  It is admitted at once (after the running epoch) when its
 * footprint fits the budget and a free range of n vertex ids exists -- its tree is built on the
 * device from its edges -- and waits otherwise. */
int dsssp_server_add_tenant(dsssp_server* s, int32_t n, int64_t m, const int32_t* u, const int32_t* v,
                            const int32_t* w, int32_t src, int32_t* tenant);
/* Removes a tenant after the running epoch: its queued requests are refused, its edges and ids
 * are released (the edges' slots at the next compaction), its footprint leaves the budget, and
 * waiting tenants that now fit are admitted in the order they came. */
int dsssp_server_remove_tenant(dsssp_server* s, int32_t tenant);
/* Epochs that were recovered by recomputing the trees (DSSSP_W_RECOMPUTED). */
int dsssp_server_recovered_epochs(dsssp_server* s, int64_t* epochs);
/* dsssp_debug_set on the pool's graph, between epochs (failure-detection tests). */
int dsssp_server_debug_set(dsssp_server* s, int32_t what, int64_t value);
/* Queues a copy of the batch; *id identifies the request in dsssp_poll. */
int dsssp_submit(dsssp_server* s, int32_t tenant, const dsssp_change* changes, int64_t k, int64_t* id);
/* Queues several requests at one instant (they can share an epoch). */
int dsssp_submit_many(dsssp_server* s, int32_t count, const int32_t* tenants,
                      const dsssp_change* const* batches, const int64_t* sizes, int64_t* ids);
/* Up to cap completed requests (waiting up to wait_ms for the first one). */
int dsssp_poll(dsssp_server* s, dsssp_request_info* out, int32_t cap, int32_t wait_ms, int32_t* count);
/* Waits until no request is queued or running; DSSSP_E_TIMEOUT after timeout_ms. */
int dsssp_server_drain(dsssp_server* s, int32_t timeout_ms);
/* Record mode: the tenant's tree right after request id (once per request). */
int dsssp_server_result(dsssp_server* s, int64_t id, int32_t* parent, int64_t* dist);
/* The tenant's current tree. */
int dsssp_server_tree_read(dsssp_server* s, int32_t tenant, int32_t* parent, int64_t* dist);
int dsssp_server_info(dsssp_server* s, int64_t* epochs, int64_t* compactions, double* compact_ms,
                      int64_t* pending);
dsssp_pool* dsssp_server_pool(dsssp_server* s);
/* Device certificate (dsssp_tree_validate) of every tenant's tree at once; *roots = one per
 * admitted tenant when all is well. */
int dsssp_server_validate(dsssp_server* s, int64_t* violations, int64_t* roots);
/* Switches record mode (0 also drops recorded trees not yet read). */
int dsssp_server_set_record(dsssp_server* s, int32_t on);

/* Vertex of maximum degree (lowest id on ties) of an edge list. */
int32_t dsssp_max_degree_vertex(int32_t n, int64_t m, const int32_t* u, const int32_t* v);

#ifdef __cplusplus
}
#endif
#endif /* DSSSP_H */
