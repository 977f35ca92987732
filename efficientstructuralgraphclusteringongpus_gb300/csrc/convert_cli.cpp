// scan-convert -- edge-list text to b_degree.bin / b_adj.bin, the arguments of the
// reference's converter (csr_convert/EdgeListToBinsConverter.cpp:123):
//
//   scan-convert <edge_list.txt> <output folder>
#include <cstdio>

#include "scan_gb300.h"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "%s <edge list file> <output folder>\n", argv[0]);
        return 1;
    }
    uint64_t n = 0, e = 0;
    scan_status st = scan_convert_edge_list(argv[1], argv[2], &n, &e);
    if (st != SCAN_OK) {
        std::fprintf(stderr, "convert failed (%s): %s\n", scan_status_string(st), scan_last_error());
        return 2;
    }
    std::printf("vertices %llu, undirected edges %llu\n", (unsigned long long)n, (unsigned long long)e);
    return 0;
}
