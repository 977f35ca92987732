// C entry point around the reference's host orientation, for pinning the oracle.
// TEST INFRASTRUCTURE ONLY.  Compiled together with GPUSCAN++/Graph.cpp (from the
// reference sources) by oracle/build.py; includes the reference's Graph.h for graph_t.
#include <cstdint>

#include "Graph.h"

extern "C" __attribute__((visibility("default"))) void ref_get_eid_and_edge_list(long n, long m, int* adj,
                                                                                 unsigned* num_edges, unsigned* eid,
                                                                                 int* edge_u, int* edge_v) {
    graph_t g;
    g.n = n;
    g.m = m;
    g.adj = adj;
    g.num_edges = num_edges;
    g.eid = nullptr;
    getEidAndEdgeList(&g, edge_u, edge_v);   // GPUSCAN++/Graph.cpp:52 (mallocs g.eid)
    for (long j = 0; j < m; ++j) eid[j] = g.eid[j];
    free(g.eid);
}
