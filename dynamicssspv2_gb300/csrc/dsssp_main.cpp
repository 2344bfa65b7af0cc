// dsssp_main.cpp -- drop-in command line for SSSPmainForUndirected.cu (README.md:13-18):
//
//   dsssp_main <graph> <N> <M> <SSSP> <changes> [--out FILE] [--json FILE] [--device D]
//              [--delta W] [--cache] [--autotune CACHE]
//
// --cache keeps a binary image of the graph and of the SSSP file next to them (<file>.dsssp.bin,
// include/dsssp.h binary cache) and reads it instead of the text when it is at least as new as
// the text; --delta sets the near-far bucket width of the relaxation rounds; --autotune takes
// the settings that the autotuner cache CACHE holds for this size class, or tunes them on the
// batch (on snapshots of the graph) and adds them to CACHE, before the batch is applied.
//
// Reads the three text formats, builds the device graph, loads the tree, applies the change
// batch through the C ABI and prints the reference's stdout lines (SSSPmainForUndirected.cu:
// 47-53, 58-64, 142-143, 153-159, 209-210, 258-259, 285-292, 296-312) with the same wording.
// Differences: the STEP timings are CUDA-event / device-timestamp times of the GPU work (the
// reference stops its STEP1 clock without a sync), "Total affected nodes" is the real number
// of cut-off vertices (the reference always prints 0), and --out writes the updated tree,
// which the reference never does.  Exit status is 0 on success, 1 on any error.
#include <sys/stat.h>

#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dsssp.h"

using clk = std::chrono::high_resolution_clock;

static long long us_since(clk::time_point t0) {
    return std::chrono::duration_cast<std::chrono::microseconds>(clk::now() - t0).count();
}

// true when `cache` exists and is not older than `text`
static bool cache_fresh(const std::string& cache, const char* text) {
    struct stat a, b;
    if (stat(cache.c_str(), &a) != 0 || stat(text, &b) != 0) return false;
    return a.st_mtime >= b.st_mtime;
}

// A whole decimal integer argument within [lo, hi] (atoi would accept "12abc" or wrap around).
static bool parse_int(const char* s, long long lo, long long hi, long long& out) {
    char* end = nullptr;
    errno = 0;
    const long long v = strtoll(s, &end, 10);
    if (errno != 0 || end == s || *end != '\0' || v < lo || v > hi) return false;
    out = v;
    return true;
}

static int die(const char* what, int rc) {
    fprintf(stderr, "dsssp_main: %s failed: %s (%s)\n", what, dsssp_strerror(rc), dsssp_last_error());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 6) {
        fprintf(stderr,
                "usage: %s <graph> <number_of_nodes> <number_of_edges> <SSSP> <change_edges> "
                "[--out FILE] [--json FILE] [--device D] [--delta W] [--cache] [--autotune CACHE]\n",
                argv[0]);
        return 2;
    }
    const char* out_path = nullptr;
    const char* json_path = nullptr;
    bool use_cache = false;
    const char* tune_path = nullptr;
    dsssp_opts opts;
    dsssp_default_opts(&opts);
    long long val = 0;
    for (int i = 6; i < argc; i++) {
        const bool has_value = i + 1 < argc;
        if (!strcmp(argv[i], "--out") && has_value) out_path = argv[++i];
        else if (!strcmp(argv[i], "--json") && has_value) json_path = argv[++i];
        else if (!strcmp(argv[i], "--device") && has_value && parse_int(argv[i + 1], 0, 1023, val)) opts.device = (int)val, i++;
        else if (!strcmp(argv[i], "--delta") && has_value && parse_int(argv[i + 1], -1, 2147483647, val)) opts.delta = (int)val, i++;
        else if (!strcmp(argv[i], "--cache")) use_cache = true;
        else if (!strcmp(argv[i], "--autotune") && has_value) tune_path = argv[++i];
        else {
            fprintf(stderr, "dsssp_main: bad option %s%s%s\n", argv[i], has_value ? " " : " (no value)",
                    has_value ? argv[i + 1] : "");
            return 2;
        }
    }
    long long nodes_arg = 0, edges_arg = 0;
    if (!parse_int(argv[2], 1, 2147483646, nodes_arg)) {
        fprintf(stderr, "dsssp_main: number_of_nodes must be an integer in 1..2147483646, not %s\n", argv[2]);
        return 2;
    }
    if (!parse_int(argv[3], 0, 9223372036854775807LL, edges_arg)) {
        fprintf(stderr, "dsssp_main: number_of_edges must be a non-negative integer, not %s\n", argv[3]);
        return 2;
    }
    const int nodes = (int)nodes_arg;

    printf("Reading input graph...\n");
    auto t0 = clk::now();
    int32_t *eu = nullptr, *ev = nullptr, *ew = nullptr;
    int64_t m = 0;
    const std::string gcache = std::string(argv[1]) + ".dsssp.bin";
    int rc = 1;
    if (use_cache && cache_fresh(gcache, argv[1])) {
        rc = dsssp_read_graph_binary(gcache.c_str(), nodes, &eu, &ev, &ew, &m);
        if (rc) fprintf(stderr, "dsssp_main: note: ignoring the graph cache: %s\n", dsssp_last_error());
    }
    if (rc) {
        rc = dsssp_read_graph_file(argv[1], nodes, &eu, &ev, &ew, &m);
        if (rc) return die("reading the graph", rc);
        if (use_cache && dsssp_write_graph_binary(gcache.c_str(), nodes, m, eu, ev, ew) != DSSSP_OK)
            fprintf(stderr, "dsssp_main: note: could not write the graph cache: %s\n", dsssp_last_error());
    }
    printf("Reading input graph completed\n");
    printf("Time taken to read input graph: %lld microseconds\n", us_since(t0));
    if (edges_arg < m)
        fprintf(stderr, "dsssp_main: note: the graph has %lld lines, more than number_of_edges=%lld\n",
                (long long)m, edges_arg);

    printf("Reading input changed edges data...\n");
    t0 = clk::now();
    dsssp_change* ch = nullptr;
    int64_t k = 0;
    rc = dsssp_read_changes_file(argv[5], nodes, &ch, &k);
    if (rc) return die("reading the change edges", rc);
    long long total_ins = 0;
    for (int64_t i = 0; i < k; i++) total_ins += ch[i].op == 1;
    printf("Reading input changed edges data completed. totalInsertion:%lld\n", total_ins);
    printf("Time taken to read input changed edges: %lld microseconds\n", us_since(t0));

    printf("creating 1D array from 2D to fit it in GPU\n");
    printf("creating 1D array from 2D completed\n");
    printf("Transferring graph data from CPU to GPU\n");
    t0 = clk::now();
    dsssp_graph* g = nullptr;
    rc = dsssp_graph_create(nodes, m, eu, ev, ew, &opts, &g);
    if (rc) return die("building the device graph", rc);
    printf("**Time taken to transfer graph data from CPU to GPU: %g milliseconds**\n", us_since(t0) / 1000.0);

    std::vector<int32_t> parent((size_t)nodes);
    std::vector<int64_t> dist((size_t)nodes);
    printf("Reading input SSSP tree data...\n");
    t0 = clk::now();
    int64_t lossy = 0;
    const std::string tcache = std::string(argv[4]) + ".dsssp.bin";
    rc = 1;
    if (use_cache && cache_fresh(tcache, argv[4])) {
        rc = dsssp_read_sssp_binary(tcache.c_str(), nodes, parent.data(), dist.data());
        if (rc) fprintf(stderr, "dsssp_main: note: ignoring the tree cache: %s\n", dsssp_last_error());
    }
    if (rc) {
        rc = dsssp_read_sssp_file(argv[4], nodes, parent.data(), dist.data(), &lossy);
        if (rc) return die("reading the SSSP tree", rc);
        if (use_cache && dsssp_write_sssp_binary(tcache.c_str(), nodes, parent.data(), dist.data()) != DSSSP_OK)
            fprintf(stderr, "dsssp_main: note: could not write the tree cache: %s\n", dsssp_last_error());
    }
    printf("Reading input SSSP tree data completed\n");
    printf("Time taken to read input input SSSP tree: %lld microseconds\n", us_since(t0));
    if (lossy)
        fprintf(stderr, "dsssp_main: warning: %lld distances were written in floating-point form and may have lost precision\n",
                (long long)lossy);
    rc = dsssp_tree_load(g, parent.data(), dist.data());
    if (rc) return die("loading the SSSP tree", rc);
    printf("reading input data completed\n");

    if (tune_path && k > 0) {  // settings of the cache for this size class, or tuned on this batch
        dsssp_tune_result tr;
        rc = dsssp_autotune(g, ch, k, tune_path, 2, 0, &tr);
        if (rc) return die("autotuning", rc);
        fprintf(stderr, "dsssp_main: autotune %s: %s (%.4f ms, %d candidates timed)\n", tr.key,
                tr.cached ? "cached settings" : "tuned", tr.ms, tr.trials);
    }
    dsssp_stats st;
    rc = dsssp_apply_batch(g, ch, k, nullptr, &st);
    if (rc < 0) return die("applying the change batch", rc);
    if (rc == DSSSP_W_RECOMPUTED)
        fprintf(stderr, "dsssp_main: note: %s (the updated tree is exact)\n", dsssp_last_error());
    printf("**Time taken for SSSP update STEP1: %g milliseconds**\n", st.t_step1_ms);
    printf("**Time taken for updateNeighbors_del: %g milliseconds**\n", st.t_inval_ms);
    printf("**Time taken for updateNeighbors: %g milliseconds**\n", st.t_relax_ms);
    printf("**Time taken for SSSP update STEP2: %g milliseconds**\n", st.t_update_ms);
    printf("****Total Time taken for SSSP update: %g milliseconds****\n", st.t_total_ms);
    printf("Total affected nodes by Delete edge only: %lld\n", (long long)st.n_invalidated);

    rc = dsssp_tree_read(g, parent.data(), dist.data());
    if (rc) return die("reading the tree back", rc);
    const int x = nodes < 40 ? nodes : 40;
    // unreachable vertices print the reference's "no path" sentinel of read_SSSP (9999999)
    printf("from GPU: \n[from GPU:\n[");
    for (int i = 0; i < x; i++)
        printf("%d:%lld:%d ", i, parent[(size_t)i] == -1 ? 9999999LL : (long long)dist[(size_t)i], parent[(size_t)i]);
    printf("]\n");
    printf("from CPU: \n[");
    for (int i = 0; i < x; i++) printf("%d:%lld ", i, parent[(size_t)i] == -1 ? 9999999LL : (long long)dist[(size_t)i]);
    printf("]\n");

    if (out_path) {
        rc = dsssp_write_sssp_file(out_path, nodes, parent.data(), dist.data());
        if (rc) return die("writing the updated tree", rc);
    }
    if (json_path) {
        FILE* f = fopen(json_path, "w");
        if (!f) return die("opening the json file", DSSSP_E_IO);
        const double t = st.t_total_ms > 0 ? st.t_total_ms : 1e-9;
        fprintf(f,
                "{\"changes\": %lld, \"insertions\": %lld, \"deletions\": %lld, \"invalidated\": %lld, "
                "\"rounds\": %lld, \"frontier_total\": %lld, \"edges_relaxed\": %lld, \"edges_inval\": %lld, "
                "\"updates\": %lld, \"repacks\": %lld, \"t_step1_ms\": %.6f, \"t_update_ms\": %.6f, "
                "\"t_total_ms\": %.6f, \"change_edges_per_s\": %.1f, \"bytes_alg\": %.0f, \"gb_per_s\": %.3f}\n",
                (long long)k, (long long)st.n_ins, (long long)st.n_del, (long long)st.n_invalidated,
                (long long)st.rounds, (long long)st.frontier_total, (long long)st.edges_relaxed,
                (long long)st.edges_inval, (long long)st.updates, (long long)st.repacks, st.t_step1_ms,
                st.t_update_ms, st.t_total_ms, (double)k / (t * 1e-3), st.bytes_alg, st.bytes_alg / (t * 1e-3) / 1e9);
        fclose(f);
    }
    dsssp_graph_destroy(g);
    dsssp_free(eu);
    dsssp_free(ev);
    dsssp_free(ew);
    dsssp_free(ch);
    return 0;
}
