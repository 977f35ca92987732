// gpuscan -- command line with the reference's surface (GPUSCAN++/main.cpp:20-123):
//
//   gpuscan <folder> <eps> <miu> [--predicate ref-f64|exact] [--device N]
//           [--out labels.bin] [--out-text labels.txt] [--json]
//
// <folder> holds b_degree.bin / b_adj.bin.  Like the reference it prints the maximum
// degree on stdout, stage times and "Cluster Number: N" on stderr.  The default predicate
// is ref-f64, which reproduces the reference bit for bit; `exact` evaluates the eps test
// in integers.  --out writes label[n] as int32 (the reference's role array encoding:
// cluster id / -1 hub / -2 outlier); --out-text writes "vertex label role" lines.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "scan_gb300.h"

static int usage(const char* prog) {
    std::fprintf(stderr,
                 "%s <Graph folder> <eps> <miu> [--predicate ref-f64|exact] [--device N] [--out file] "
                 "[--out-text file] [--json]\n",
                 prog);
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 4) return usage(argv[0]);
    const char* dir = argv[1];
    const char* eps = argv[2];
    const int mu = std::atoi(argv[3]);
    scan_predicate pred = SCAN_PRED_REF_F64;
    int device = 0;
    const char* out_bin = nullptr;
    const char* out_txt = nullptr;
    bool json = false;
    for (int i = 4; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--predicate" && i + 1 < argc) {
            std::string p = argv[++i];
            if (p == "exact") pred = SCAN_PRED_EXACT;
            else if (p == "ref-f64") pred = SCAN_PRED_REF_F64;
            else return usage(argv[0]);
        } else if (a == "--device" && i + 1 < argc) {
            device = std::atoi(argv[++i]);
        } else if (a == "--out" && i + 1 < argc) {
            out_bin = argv[++i];
        } else if (a == "--out-text" && i + 1 < argc) {
            out_txt = argv[++i];
        } else if (a == "--json") {
            json = true;
        } else {
            return usage(argv[0]);
        }
    }
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    scan_graph* g = nullptr;
    scan_status st = scan_graph_load(dir, &g);
    if (st != SCAN_OK) {
        std::fprintf(stderr, "load failed (%s): %s\n", scan_status_string(st), scan_last_error());
        return 2;
    }
    auto t1 = clk::now();
    std::fprintf(stderr, "read graph time: %.3lf s\n", std::chrono::duration<double>(t1 - t0).count());
    std::printf("max degree: %u\n", scan_graph_max_degree(g));
    const uint64_t n = scan_graph_num_vertices(g);
    std::fprintf(stderr, "node number and edge number: %llu, %llu\n", (unsigned long long)n,
                 (unsigned long long)scan_graph_num_directed(g));
    std::vector<int32_t> label(n);
    std::vector<uint8_t> role(n);
    scan_stats s;
    std::fprintf(stderr, "Start GPUScan\n");
    auto t2 = clk::now();
    st = scan_run(g, device, eps, mu, pred, label.data(), role.data(), &s);
    auto t3 = clk::now();
    if (st != SCAN_OK) {
        std::fprintf(stderr, "scan failed (%s): %s\n", scan_status_string(st), scan_last_error());
        scan_graph_free(g);
        return 3;
    }
    std::fprintf(stderr, "Finish GPUScan\n");
    std::fprintf(stderr, "H2D time: %.3lf s\nOrient time: %.3lf s\nSimilarity time: %.3lf s\n", s.ms_h2d / 1e3,
                 s.ms_orient / 1e3, s.ms_similarity / 1e3);
    std::fprintf(stderr, "Cluster time: %.3lf s\nD2H time: %.3lf s\n", s.ms_cluster / 1e3, s.ms_d2h / 1e3);
    std::fprintf(stderr, "gpuscan time: %.3lf s\n", std::chrono::duration<double>(t3 - t2).count());
    std::fprintf(stderr, "core number: %llu\n", (unsigned long long)s.num_cores);
    std::fprintf(stderr, "Cluster Number: %llu\n", (unsigned long long)scan_count_clusters(label.data(), n));
    if (json) {
        std::printf(
            "{\"n\": %llu, \"edges\": %llu, \"cores\": %llu, \"clusters\": %llu, \"borders\": %llu, \"hubs\": %llu, "
            "\"outliers\": %llu, \"similar_edges\": %llu, \"predicate_disagreements\": %llu, "
            "\"ms_similarity\": %.4f, \"ms_cluster\": %.4f}\n",
            (unsigned long long)s.n, (unsigned long long)s.num_edges, (unsigned long long)s.num_cores,
            (unsigned long long)s.num_clusters, (unsigned long long)s.num_borders, (unsigned long long)s.num_hubs,
            (unsigned long long)s.num_outliers, (unsigned long long)s.num_similar_edges,
            (unsigned long long)s.pred_disagreements, s.ms_similarity, s.ms_cluster);
    }
    int rc = 0;
    if (out_bin) {
        FILE* f = std::fopen(out_bin, "wb");
        if (!f || std::fwrite(label.data(), 4, n, f) != n) { std::fprintf(stderr, "cannot write %s\n", out_bin); rc = 4; }
        if (f) std::fclose(f);
    }
    if (out_txt) {
        FILE* f = std::fopen(out_txt, "w");
        if (!f) { std::fprintf(stderr, "cannot write %s\n", out_txt); rc = 4; }
        else {
            for (uint64_t v = 0; v < n; ++v) std::fprintf(f, "%llu %d %u\n", (unsigned long long)v, label[v], role[v]);
            std::fclose(f);
        }
    }
    scan_graph_free(g);
    std::fprintf(stderr, "Work Complete!\n");
    return rc;
}
