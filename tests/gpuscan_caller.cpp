// A C++ program that calls the C++-linkage GPUScan() the way the reference's own program
// does (GPUSCAN++/main.cpp:20-123): load b_degree.bin / b_adj.bin into a graph_t with
// 32-bit offsets, compute the oriented edge list (getEidAndEdgeList's output), call
// GPUScan(&g, Edge_u, Edge_v, eps, miu), count the clusters as main.cpp:83-111 does and
// print "Cluster Number: N" to stderr, then free the result with free().
//
// Test infrastructure: tests/test_gpu_dropin_caller.py compiles it against the library and
// include/ and runs it on a GPU.  The reference's own main.cpp cannot be compiled on the
// GPU host (its sources are not there, and its Graph.cpp needs <x86intrin.h>); its link
// against the library is checked on x86_64 by tests/test_dropin_link.py.
//
//   gpuscan_caller <folder> <eps> <miu> [labels.bin]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gpuscan_compat.h"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "%s <Graph folder> <eps> <miu> [labels.bin]\n", argv[0]);
        return 1;
    }
    const double eps = std::atof(argv[2]);   // as main.cpp:26 reads it
    const int miu = std::atoi(argv[3]);
    scan_graph* sg = nullptr;
    if (scan_graph_load(argv[1], &sg) != SCAN_OK) {
        std::fprintf(stderr, "load: %s\n", scan_last_error());
        return 1;
    }
    const uint64_t n = scan_graph_num_vertices(sg), m = scan_graph_num_directed(sg);
    const uint64_t* off64 = scan_graph_offsets(sg);
    const uint32_t* adj32 = scan_graph_adjacency(sg);

    // graph_t as the reference's Graph loader fills it: malloc'd arrays, 32-bit offsets.
    graph_t g;
    g.n = (long)n;
    g.m = (long)m;
    g.adj = static_cast<vid_t*>(std::malloc(sizeof(vid_t) * (m ? m : 1)));
    g.num_edges = static_cast<eid_t*>(std::malloc(sizeof(eid_t) * (n + 1)));
    g.eid = static_cast<eid_t*>(std::malloc(sizeof(eid_t) * (m ? m : 1)));
    for (uint64_t v = 0; v <= n; ++v) g.num_edges[v] = (eid_t)off64[v];
    for (uint64_t j = 0; j < m; ++j) g.adj[j] = (vid_t)adj32[j];
    std::vector<int32_t> edge_u(m / 2 + 1), edge_v(m / 2 + 1);
    if (scan_orient_reference(sg, g.eid, edge_u.data(), edge_v.data()) != SCAN_OK) {
        std::fprintf(stderr, "orient: %s\n", scan_last_error());
        return 1;
    }
    std::fprintf(stderr, "node number and edge number: %ld, %ld\n", g.n, g.m);

    int* cluster = GPUScan(&g, edge_u.data(), edge_v.data(), eps, miu);
    if (!cluster) return 2;

    // main.cpp:83-111: mark every cluster id that occurs, then count the marks
    std::vector<char> seen(n, 0);
    for (uint64_t i = 0; i < n; ++i)
        if (cluster[i] >= 0) seen[cluster[i]] = 1;
    int sum = 0;
    for (uint64_t i = 0; i < n; ++i) sum += seen[i];
    std::fprintf(stderr, "Cluster Number: %d\n", sum);

    int rc = 0;
    if (argc > 4) {
        FILE* f = std::fopen(argv[4], "wb");
        if (!f || std::fwrite(cluster, sizeof(int), n, f) != n) rc = 3;
        if (f) std::fclose(f);
    }
    std::free(g.adj);
    std::free(g.num_edges);
    std::free(g.eid);
    std::free(cluster);
    scan_graph_free(sg);
    return rc;
}
