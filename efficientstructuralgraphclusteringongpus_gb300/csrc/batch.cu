// Batched SCAN: many graphs with their own (eps, mu) in one pass.
//
// The graphs become one disjoint union on the device (vertex ids shifted by each graph's
// offset; no edge crosses graphs), so one set of similarity and cluster kernels covers all
// of them: the similarity kernels' persistent CTAs pull tasks of every graph from the same
// queues, and the predicate/core kernels read each graph's parameters through the vertex ->
// graph map.  Cluster ids come out as the smallest core id in union numbering and are
// shifted back per graph (components never cross graphs, so this is each graph's smallest
// core id).  The whole pass -- similarity stage and cluster stage -- is captured once into
// a CUDA graph and replayed per run, so a run is one graph launch plus the parameter and
// result copies.  An autotuner picks the task size and long-list threshold for the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <omp.h>

#include "device_graph.h"

using namespace scan;

struct scan_batch {
    int device = 0;
    uint32_t count = 0;
    std::vector<uint64_t> voff;          // count + 1 vertex offsets in the union
    DeviceGraph* d = nullptr;
    uint32_t* vgid = nullptr;            // device, n
    PredParams* gpp = nullptr;           // device, count
    int32_t* gmu = nullptr;              // device, count
    PredParams* sets = nullptr;          // device, kPruneSets: distinct parameter sets of a run
    uint32_t* nsets = nullptr;           // device
    uint32_t* np_tabs = nullptr;         // device, kPruneSets * kPruneTable prune thresholds
    PredParams* h_sets = nullptr;        // pinned, kPruneSets + 1 (the last: the count)
    PredParams* h_gpp = nullptr;         // pinned, count
    int32_t* h_gmu = nullptr;            // pinned, count
    int32_t* h_label = nullptr;          // pinned, n
    uint8_t* h_role = nullptr;           // pinned, n
    RunCounters* h_ctr = nullptr;        // pinned
    uint32_t* h_flag = nullptr;          // pinned
    cudaGraphExec_t exec = nullptr;
    uint32_t graph_launches = 0;         // kernels inside the captured graph
    float tuned_ms = 0.f;
    bool tune_pending = false;           // autotune at the first run, with its parameters
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

uint32_t jump_index(uint32_t n) { return jump_rounds(n) - 1; }

void batch_free_device(scan_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->vgid) cudaFree(b->vgid);
    if (b->gpp) cudaFree(b->gpp);
    if (b->gmu) cudaFree(b->gmu);
    for (void* p : {(void*)b->sets, (void*)b->nsets, (void*)b->np_tabs})
        if (p) cudaFree(p);
    if (b->h_sets) cudaFreeHost(b->h_sets);
    for (void* p : {(void*)b->h_gpp, (void*)b->h_gmu, (void*)b->h_label, (void*)b->h_role, (void*)b->h_ctr,
                    (void*)b->h_flag})
        if (p) cudaFreeHost(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->d) device_graph_free(b->d);
}

}  // namespace

#define B_CUDA(call)                                                                                  \
    do {                                                                                              \
        cudaError_t err_ = (call);                                                                    \
        if (err_ != cudaSuccess)                                                                      \
            return fail(SCAN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));        \
    } while (0)

extern "C" {

scan_status scan_batch_create(const scan_graph* const* graphs, uint32_t count, int device, int autotune,
                              scan_batch** out) {
    clear_error();
    if (!graphs || !out || count == 0 || device < 0) return fail(SCAN_ERR_INVALID_ARG, "bad batch arguments");
    *out = nullptr;
    std::unique_ptr<scan_batch, void (*)(scan_batch*)> b(new scan_batch(), [](scan_batch* x) {
        batch_free_device(x);
        delete x;
    });
    b->device = device;
    b->count = count;
    b->voff.assign(count + 1, 0);
    std::vector<uint64_t> eoff(count + 1, 0);
    for (uint32_t i = 0; i < count; ++i) {
        if (!graphs[i]) return fail(SCAN_ERR_INVALID_ARG, "null graph in the batch");
        b->voff[i + 1] = b->voff[i] + graphs[i]->n;
        eoff[i + 1] = eoff[i] + graphs[i]->m;
    }
    const uint64_t N = b->voff[count], M = eoff[count];
    if (N >= 0xFFFFFFF0ull || M >= 0xFFFFFFF0ull)
        return fail(SCAN_ERR_TOO_LARGE, "batch exceeds 2^32 vertices or directed entries");
    // the union CSR on the host (parallel over graphs)
    std::vector<uint64_t> off(N + 1);
    std::vector<uint32_t> adj(M);
    std::vector<uint32_t> vgid(N);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t i = 0; i < (int64_t)count; ++i) {
        const scan_graph* g = graphs[i];
        const uint64_t vb = b->voff[i], eb = eoff[i];
        for (uint64_t v = 0; v < g->n; ++v) {
            off[vb + v] = eb + g->off[v];
            vgid[vb + v] = (uint32_t)i;
        }
        for (uint64_t j = 0; j < g->m; ++j) adj[eb + j] = g->adj[j] + (uint32_t)vb;
    }
    off[N] = M;
    B_CUDA(cudaSetDevice(device));
    scan_status st = device_upload(device, N, M, off.data(), true, adj.data(), &b->d, nullptr);
    if (st != SCAN_OK) return st;
    B_CUDA(cudaMalloc(&b->vgid, N * sizeof(uint32_t)));
    B_CUDA(cudaMalloc(&b->gpp, count * sizeof(PredParams)));
    B_CUDA(cudaMalloc(&b->gmu, count * sizeof(int32_t)));
    B_CUDA(cudaMalloc(&b->sets, kPruneSets * sizeof(PredParams)));
    B_CUDA(cudaMalloc(&b->nsets, sizeof(uint32_t)));
    B_CUDA(cudaMalloc(&b->np_tabs, (size_t)kPruneSets * kPruneTable * sizeof(uint32_t)));
    B_CUDA(cudaHostAlloc(&b->h_sets, (kPruneSets + 1) * sizeof(PredParams), cudaHostAllocDefault));
    B_CUDA(cudaMemcpy(b->vgid, vgid.data(), N * sizeof(uint32_t), cudaMemcpyHostToDevice));
    B_CUDA(cudaHostAlloc(&b->h_gpp, count * sizeof(PredParams), cudaHostAllocDefault));
    B_CUDA(cudaHostAlloc(&b->h_gmu, count * sizeof(int32_t), cudaHostAllocDefault));
    B_CUDA(cudaHostAlloc(&b->h_label, N * sizeof(int32_t), cudaHostAllocDefault));
    B_CUDA(cudaHostAlloc(&b->h_role, N, cudaHostAllocDefault));
    B_CUDA(cudaHostAlloc(&b->h_ctr, sizeof(RunCounters), cudaHostAllocDefault));
    B_CUDA(cudaHostAlloc(&b->h_flag, sizeof(uint32_t), cudaHostAllocDefault));
    B_CUDA(cudaEventCreate(&b->ev0));
    B_CUDA(cudaEventCreate(&b->ev1));
    b->tune_pending = autotune != 0;
    *out = b.release();
    return SCAN_OK;
}

// One pass over the batch.  eps_decimal[i] / mu[i] are graph i's parameters; out_labels[i]
// (n_i entries) and out_roles[i] (may be NULL, or NULL entries) receive graph i's result
// in its own vertex ids.
scan_status scan_batch_run(scan_batch* b, const char* const* eps_decimal, const int32_t* mu,
                           scan_predicate predicate, int32_t* const* out_labels, uint8_t* const* out_roles,
                           scan_batch_stats* stats) {
    clear_error();
    if (!b || !eps_decimal || !mu || !out_labels) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t i = 0; i < b->count; ++i) {
        if (mu[i] < 1) return fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1 (graph " + std::to_string(i) + ")");
        scan_status st = make_pred(eps_decimal[i], &b->h_gpp[i], predicate);
        if (st != SCAN_OK) return st;
        b->h_gmu[i] = mu[i];
        if (!out_labels[i]) return fail(SCAN_ERR_INVALID_ARG, "null output for graph " + std::to_string(i));
    }
    // Distinct (eps, p, q) sets: each gets a prune-threshold table (the predicate mode does
    // not enter the thresholds); graphs past kPruneSets sets compute them per pivot.
    uint32_t nsets = 0;
    for (uint32_t i = 0; i < b->count; ++i) {
        PredParams& g = b->h_gpp[i];
        g.np_set = 0xFFFFFFFFu;
        for (uint32_t k = 0; k < nsets; ++k) {
            const PredParams& r = b->h_sets[k];
            if (std::memcmp(&r.eps, &g.eps, sizeof(double)) == 0 && r.p == g.p && r.q == g.q) {
                g.np_set = k;
                break;
            }
        }
        if (g.np_set == 0xFFFFFFFFu && nsets < kPruneSets) {
            b->h_sets[nsets] = g;
            g.np_set = nsets++;
        }
    }
    std::memcpy(&b->h_sets[kPruneSets], &nsets, sizeof(nsets));
    DeviceGraph* d = b->d;
    std::lock_guard<std::mutex> lock(d->mu);
    B_CUDA(cudaSetDevice(b->device));
    cudaStream_t s = d->stream;
    B_CUDA(cudaMemcpyAsync(b->gpp, b->h_gpp, b->count * sizeof(PredParams), cudaMemcpyHostToDevice, s));
    B_CUDA(cudaMemcpyAsync(b->gmu, b->h_gmu, b->count * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    B_CUDA(cudaMemcpyAsync(b->sets, b->h_sets, kPruneSets * sizeof(PredParams), cudaMemcpyHostToDevice, s));
    B_CUDA(cudaMemcpyAsync(b->nsets, &b->h_sets[kPruneSets], sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    BatchParams bp{b->vgid, b->gpp, b->gmu, b->sets, b->nsets, b->np_tabs};
    PredParams unused{};
    // The pass: with no split pivot, the one-shot path of a single run (degree prune, early
    // stop, the filter kernels, predicate fused into the counting), each pivot taking eps and
    // the predicate from its own graph; otherwise full counts, then the predicate per graph.
    auto similarity = [&](uint32_t* launches) -> scan_status {
        if (d->has_split) return launch_cn(d, launches);
        PredParams on{};   // "prune on"; every other parameter comes from the pivot's graph
        B_CUDA(cudaMemsetAsync(d->rs.sim, 0, d->E, s));
        B_CUDA(cudaMemsetAsync(d->rs.sd, 0, d->n * sizeof(int32_t), s));
        B_CUDA(cudaMemsetAsync(d->rs.ctr, 0, sizeof(RunCounters), s));
        return launch_cn(d, launches, &on, &d->rs, &bp);
    };
    auto queue = [&](uint32_t* launches) -> scan_status {
        scan_status st = similarity(launches);
        return st == SCAN_OK ? launch_cluster(d, d->rs, s, unused, 1, launches, &bp, !d->has_split) : st;
    };
    if (b->tune_pending) {
        // The plan is chosen on this run's parameters; the capture below then records it.
        scan_status st = autotune_similarity(d, &b->tuned_ms, similarity);
        if (st != SCAN_OK) return st;
        b->tune_pending = false;
    }
    if (!b->exec) {
        // First run: queue once directly (sets kernel attributes), then capture the same
        // sequence into a CUDA graph for every later run.
        uint32_t launches = 0;
        scan_status st = queue(&launches);
        if (st != SCAN_OK) return st;
        B_CUDA(cudaStreamSynchronize(s));
        cudaGraph_t graph = nullptr;
        B_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        launches = 0;
        st = queue(&launches);
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (st != SCAN_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ce != cudaSuccess) return fail(SCAN_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(SCAN_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
        b->graph_launches = launches;
    }
    B_CUDA(cudaEventRecord(b->ev0, s));
    B_CUDA(cudaGraphLaunch(b->exec, s));
    B_CUDA(cudaEventRecord(b->ev1, s));
    B_CUDA(cudaMemcpyAsync(b->h_label, d->rs.label, d->n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    B_CUDA(cudaMemcpyAsync(b->h_role, d->rs.role, d->n, cudaMemcpyDeviceToHost, s));
    B_CUDA(cudaMemcpyAsync(b->h_ctr, d->rs.ctr, sizeof(RunCounters), cudaMemcpyDeviceToHost, s));
    B_CUDA(cudaMemcpyAsync(b->h_flag, d->rs.jump_flags + jump_index(d->n), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    B_CUDA(cudaStreamSynchronize(s));
    if (b->h_ctr->error_flags || *b->h_flag) return fail(SCAN_ERR_DEVICE, "union-find did not finish within its limits");
    // split into per-graph outputs, cluster ids back to local numbering
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < (int64_t)b->count; ++i) {
        const uint64_t vb = b->voff[i], nv = b->voff[i + 1] - vb;
        int32_t* dst = out_labels[i];
        for (uint64_t v = 0; v < nv; ++v) {
            const int32_t l = b->h_label[vb + v];
            dst[v] = l >= 0 ? l - (int32_t)vb : l;
        }
        if (out_roles && out_roles[i]) std::memcpy(out_roles[i], b->h_role + vb, nv);
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        stats->ms_device = ms;
        stats->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->graph_kernels = b->graph_launches;
        stats->num_graphs = b->count;
        stats->num_vertices = d->n;
        stats->num_edges = d->E;
        stats->num_cores = b->h_ctr->cores;
        stats->num_clusters = b->h_ctr->clusters;
        stats->tuned_similarity_ms = b->tuned_ms;
        stats->long_words = d->long_words;
        stats->target_probes = d->plan.target_probes;
        stats->small_deg = d->plan.small_deg;
        stats->small_strategy = d->plan.small_strategy;
        stats->hub_min_deg = d->plan.bitmap_min_deg;
        stats->chunk_max = d->plan.chunk_max;
    }
    return SCAN_OK;
}

void scan_batch_free(scan_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    batch_free_device(b);
    delete b;
}

}  // extern "C"
