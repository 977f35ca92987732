// C++-linkage GPUScan with the reference's signature (GPUSCAN++/GPUScan.h:7).
#include <cstdio>

#include "gpuscan_compat.h"

int* GPUScan(graph_t* g, int* Edge_u, int* Edge_v, double eps, int miu) {
    if (!g) {
        std::fprintf(stderr, "GPUScan: graph is null\n");
        return nullptr;
    }
    int32_t* out = scan_gpuscan_compat((int64_t)g->n, (int64_t)g->m, g->adj, g->num_edges, g->eid, Edge_u, Edge_v,
                                       eps, miu);
    if (!out) std::fprintf(stderr, "GPUScan: %s\n", scan_last_error());
    return out;
}
