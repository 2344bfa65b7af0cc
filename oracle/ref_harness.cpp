/*
 * ref_harness.cpp -- runs the reference's own update path on the CPU (test infrastructure).
 *
 * Compiled by `make -C oracle ref` against the reference sources where they lie
 * (all_structure_undir.cuh, gpuFunctions_undir.cuh) with the host stand-ins of
 * oracle/ref_shim/ in place of the CUDA headers.  Every kernel launch of
 * SSSPmainForUndirected.cu:196-281 is replayed as a loop over (block, thread) in index order,
 * which is one legal interleaving of the reference's kernels.  The readers are the
 * reference's own (read_graphEdges, readin_changes, read_SSSP).
 *
 * usage: ref_update <graph> <N> <M> <SSSP> <cE>
 * prints one line "v Dist Parent" per vertex after the update, then
 * "rounds_del R1" and "rounds_relax R2".
 */
#include "gpuFunctions_undir.cuh"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

static const unsigned kBlock = THREADS_PER_BLOCK;

/* one launch <<<grid, kBlock>>> replayed thread by thread */
template <class F>
static void launch(unsigned grid, F&& body) {
    gridDim.x = grid;
    blockDim.x = kBlock;
    for (unsigned b = 0; b < grid; b++) {
        blockIdx.x = b;
        for (unsigned t = 0; t < kBlock; t++) {
            threadIdx.x = t;
            body();
        }
    }
}

int main(int argc, char* argv[]) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s graph N M SSSP cE\n", argv[0]);
        return 2;
    }
    int nodes = atoi(argv[2]);
    int totalInsertion = 0;
    std::vector<ColWtList> adj(nodes);
    read_graphEdges(adj, argv[1], &nodes);
    std::vector<changeEdge> ins, del;
    readin_changes(argv[5], ins, del, adj, totalInsertion);

    std::vector<int> tracker(nodes + 1, 0);
    std::vector<ColWt> full;
    for (int i = 0; i < nodes; i++) {
        tracker[i + 1] = tracker[i] + (int)adj[i].size();
        full.insert(full.end(), adj[i].begin(), adj[i].end());
    }
    full.push_back(ColWt{0, 0}); /* keeps .data() valid for an empty graph */

    std::vector<RT_Vertex> sssp(nodes, RT_Vertex{0, 0, 0, 0});
    read_SSSP(sssp.data(), argv[4], &nodes);

    /* the reference reads the lists past their counts before the bounds check
     * (gpuFunctions_undir.cuh:314); pad them so the replay stays in bounds */
    std::vector<int> list_del(nodes + 2 * kBlock, 0), list_all(nodes + 2 * kBlock, 0);
    std::vector<int> scratch(nodes + 2 * kBlock, 0);
    int counter_del = 0, counter = 0, updated_counter = 0, change = 0;
    RT_Vertex* S = sssp.data();
    ColWt* A = full.data();
    int* T = tracker.data();
    int nI = (int)ins.size(), nD = (int)del.size();

    if (nD > 0) launch(nD / kBlock + 1, [&] { deleteEdge(del.data(), S, nD, A, T); });
    if (nI > 0) launch(nI / kBlock + 1, [&] { insertEdge(ins.data(), S, nI, A, T); });

    long rounds_del = 0, rounds_relax = 0;
    long cap = 4L * nodes + 16;
    if (nD > 0) {
        launch(nodes / kBlock + 1, [&] { filterAffectedNodes(S, nodes, list_del.data(), &counter_del); });
        change = 1;
        while (change > 0 && rounds_del < cap) {
            change = 0;
            rounds_del++;
            launch(counter_del / kBlock + 1, [&] {
                updateNeighbors_del(S, &updated_counter, scratch.data(), list_del.data(),
                                    &counter_del, A, T, &change);
            });
            launch(1, [&] { if (threadIdx.x == 0) resetCounter(&counter_del); });
            launch(nodes / kBlock + 1, [&] { filterAffectedNodes(S, nodes, list_del.data(), &counter_del); });
        }
    }
    launch(nodes / kBlock + 1, [&] { filterAllAffected(S, list_all.data(), &counter, nodes); });
    change = 1;
    while (change == 1 && rounds_relax < cap) {
        change = 0;
        rounds_relax++;
        launch(counter / kBlock + 1, [&] { updateNeighbors(S, &counter, list_all.data(), A, T, &change); });
        launch(1, [&] { if (threadIdx.x == 0) resetCounter(&counter); });
        launch(nodes / kBlock + 1, [&] { filterAllAffected(S, list_all.data(), &counter, nodes); });
    }
    for (int i = 0; i < nodes; i++) printf("%d %d %d\n", i, S[i].Dist, S[i].Parent);
    printf("rounds_del %ld\nrounds_relax %ld\n", rounds_del, rounds_relax);
    return 0;
}
