/*
 * oracle.h -- CPU oracle for the dynamic SSSP batch update.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the dsssp library, its CLI,
 * the Python package) links, loads or calls this code.  It is used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 *
 * It restates, in plain C, three things of the reference (ArindamK92/DynamicSSSPv2):
 *   1. the graph that results from applying a change batch
 *      (all_structure_undir.cuh:106-117 appends insertions to the adjacency,
 *       gpuFunctions_undir.cuh:201-213 then removes every entry matching a deletion);
 *   2. the sequential Dijkstra of seqSSSPwithDist_undir.cpp:66-128 (lazy insertion,
 *      an inQ flag, dist initialised to 1000*N, parent = last strict improver);
 *   3. the reference GPU update of SSSPmainForUndirected.cu:196-281 with every kernel
 *      (gpuFunctions_undir.cuh:125-433) executed one thread at a time in index order,
 *      which is one legal interleaving of the reference's racy kernels.
 * plus a shortest-path-tree validator.
 *
 * Pinning: 2 and 3 are checked against the reference itself, compiled here from its own
 * sources (`make -C oracle ref` -> oracle/_ref/), through the golden fixtures in
 * tests/golden/ and the test tests/test_oracle.py.
 */
#ifndef DSSSP_ORACLE_H
#define DSSSP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Number of adjacency entries of the updated graph (for sizing the outputs of
 * orc_updated_graph).  Same arguments as orc_updated_graph without the outputs. */
int64_t orc_updated_graph_nnz(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                              const int32_t* ew, int64_t k, const int32_t* cu, const int32_t* cv,
                              const int32_t* cw, const int32_t* cop);

/* Adjacency (CSR, rows in line order) of the graph obtained by appending the insertions
 * (op==1) of the batch to the base edge list and then removing every line whose endpoint
 * pair {u,v} and weight equal those of a deletion (op==0).  Lines with other op values are
 * ignored (all_structure_undir.cuh:106-121).  off has n+1 entries; col/wt have
 * orc_updated_graph_nnz() entries.  If kept_lines is not NULL it receives, per line of the
 * concatenated list (m base lines, then the insertions), 1 if the line survives.
 * Returns the number of entries, or -1 if a vertex id is out of range. */
int64_t orc_updated_graph(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                          const int32_t* ew, int64_t k, const int32_t* cu, const int32_t* cv,
                          const int32_t* cw, const int32_t* cop, int64_t* off, int32_t* col,
                          int32_t* wt, uint8_t* kept_lines);

/* CSR of a plain edge list (line (a,b,w) adds b to row a and a to row b, in line order). */
int64_t orc_csr_from_edges(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev,
                           const int32_t* ew, int64_t* off, int32_t* col, int32_t* wt);

/* Sequential Dijkstra of seqSSSPwithDist_undir.cpp:66-128.  Distances start at inf_cap
 * (the reference uses 1000*N, seqSSSPwithDist_undir.cpp:69-73); a vertex whose distance is
 * never lowered below inf_cap keeps parent -1 and dist inf_cap.  Entries with a negative
 * weight are relaxed like any other (the reference does the same).
 * Returns the number of heap pops. */
int64_t orc_dijkstra(int32_t n, const int64_t* off, const int32_t* col, const int32_t* wt,
                     int32_t src, int64_t inf_cap, int64_t* dist, int32_t* parent);

/* Shortest-path-tree check of (dist, parent) on the graph in CSR form:
 *   dist[src]==0, parent[src]==src;
 *   parent[v]==-1  <=> v unreachable  (dist[v]==unreach);
 *   for reachable v != src there is a live entry (parent[v] -> v, w) with
 *   dist[parent[v]] + w == dist[v];
 *   no live entry (u -> c, w) with u reachable has dist[u] + w < dist[c];
 *   following parents from any reachable vertex ends at src (no cycle).
 * Entries with w < 0 are deleted (tombstoned) entries and are skipped.
 * Returns 0 if valid, else a positive code; msg (if not NULL) receives a description. */
int orc_validate_tree(int32_t n, const int64_t* off, const int32_t* col, const int32_t* wt,
                      int32_t src, const int64_t* dist, const int32_t* parent, int64_t unreach,
                      char* msg, int32_t msglen);

/* Sequential restatement of the reference GPU update, SSSPmainForUndirected.cu:42-281.
 *   in_parent/in_dist: the tree as read_SSSP (all_structure_undir.cuh:133-171) leaves it
 *   (callers pass the parsed file through orc_read_sssp_semantics first).
 *   out_dist/out_parent: RT_Vertex Dist / Parent after the update.
 * rounds_del / rounds_relax (optional) receive the host-loop iteration counts.
 * Returns 0, or -1 on an out-of-range vertex id. */
int orc_ref_update(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev, const int32_t* ew,
                   int64_t k, const int32_t* cu, const int32_t* cv, const int32_t* cw,
                   const int32_t* cop, const int32_t* in_parent, const int32_t* in_dist,
                   int32_t* out_dist, int32_t* out_parent, int64_t* rounds_del,
                   int64_t* rounds_relax);

/* read_SSSP (all_structure_undir.cuh:133-171) applied to already-split lines:
 * rows (node, parent, dist), in file order.  Gaps and trailing vertices get
 * Dist 9999999 / Parent -1; parent == -1 forces Dist 9999999. */
void orc_read_sssp_semantics(int32_t n, int64_t rows, const int32_t* node, const int32_t* par,
                             const int32_t* dist, int32_t* out_parent, int32_t* out_dist);

/* ---- seeded synthetic inputs (oracle_gen.c) ----------------------------------------
 * The same streams as the dsssp library's generators (include/dsssp.h dsssp_gen_er,
 * dsssp_gen_rmat, dsssp_gen_changes with DSSSP_INS_UNIFORM (0) or DSSSP_INS_RMAT (1),
 * dsssp_max_degree_vertex), restated so that the CPU reference arm of bench.py builds its
 * workload without the product library; tests check that the outputs are identical.
 * Outputs are caller arrays of m (edges) or n_ins + n_del (changes) entries; 0 or -1. */
int orc_gen_er(int32_t n, int64_t m, int32_t wlo, int32_t whi, uint64_t seed, int32_t* u, int32_t* v,
               int32_t* w);
int orc_gen_rmat(int32_t scale, int64_t m, double a, double b, double c, int32_t wlo, int32_t whi,
                 uint64_t seed, int32_t* u, int32_t* v, int32_t* w);
int32_t orc_max_degree_vertex(int32_t n, int64_t m, const int32_t* u, const int32_t* v);
int orc_gen_changes(int32_t n, int64_t m, const int32_t* eu, const int32_t* ev, const int32_t* ew,
                    int64_t n_ins, int64_t n_del, int32_t ins_kind, int32_t scale, double p0, double p1,
                    double p2, int32_t wlo, int32_t whi, uint64_t seed, int32_t* cu, int32_t* cv,
                    int32_t* cw, int32_t* cop);

#ifdef __cplusplus
}
#endif
#endif
