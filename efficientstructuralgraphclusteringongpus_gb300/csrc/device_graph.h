// Resident graph and per-run scratch, shared by the translation units that drive the
// kernels (scan_device.cu: single runs; server.cu: the serving loop).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "graph_internal.h"
#include "predicate.cuh"

namespace scan {
struct CnTask;

// Task sizing of the similarity stage (set by the planner; re-planned by the autotuner).
struct PlanParams {
    unsigned long long target_probes;          // probe work per hash-class task
    unsigned long long target_probes_bitmap;   // probe work per bitmap task
    uint32_t min_slice_edges;
    uint32_t chunk_max;                        // pivot entries per largest-class table (<= kChunkMaxCap)
    uint32_t small_deg;                        // pivots up to this degree: k_cn_small (<= kSmallDeg)
    uint32_t small_strategy;                   // k_cn_small: 0 serial hash, 1 batched hash, 2 batched search
    uint32_t bitmap_min_deg;                   // hubs: pivots above this degree (<= chunk_max)
};
}

// Working arrays of one SCAN pass over a resident graph (cluster stage).  One contiguous
// block, so a caller can place it anywhere (a plain allocation, or an arena slice in the
// serving loop); several passes over the same graph can run at once, each with its own.
struct RunScratch {
    uint32_t n = 0;
    uint64_t E = 0;
    uint8_t* sim = nullptr;        // E: predicate result
    int32_t* sd = nullptr;         // n: similar-neighbour count
    int32_t* parent = nullptr;     // n: union-find forest (cores), -1 for non-cores
    int32_t* bmin = nullptr;       // n: smallest / largest cluster a border is similar to
    int32_t* bmax = nullptr;
    int32_t* nmin = nullptr;       // n: smallest / largest label among an unattached vertex's neighbours
    int32_t* nmax = nullptr;
    int32_t* lab = nullptr;        // n: label after attachment
    int32_t* label = nullptr;      // n: final label
    uint8_t* role = nullptr;       // n: final role
    scan::RunCounters* ctr = nullptr;
    uint32_t* jump_flags = nullptr;   // kMaxJumpRounds
};

struct DeviceGraph {
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;   // the hub kernels of the similarity stage, beside the classes
    cudaStream_t aux = nullptr;    // upload: orientation passes beside the adjacency copy
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t chunk_ev[9] = {};  // upload: one per adjacency chunk, and the end of the aux stream
    uint32_t n = 0;
    uint64_t m = 0, E = 0;
    uint32_t* off = nullptr;
    uint32_t* adj = nullptr;
    uint32_t* lo_off = nullptr;
    uint32_t* lo_adj = nullptr;
    uint32_t* lo_src = nullptr;
    unsigned long long* work = nullptr;
    unsigned long long* cn_ctr = nullptr;
    uint32_t* task_queue = nullptr;        // launch_cn: one task counter per similarity kernel
    uint32_t* np_tab = nullptr;            // launch_cn: prune thresholds of pivot degrees < kPruneTable
    uint32_t* miss = nullptr;              // split pivots' lower edges: misses found so far (one-shot runs)
    uint32_t nmiss = 0, cap_miss = 0;
    bool has_split = false;                // the plan splits some pivot into chunks
    float* tau = nullptr;                  // served graphs: 2E similarity thresholds (k_tau)   // last launch_cn: [0] 16-byte list words read, [1] edges counted
    uint32_t* small_piv = nullptr;
    uint32_t nsmall = 0;
    scan::CnTask* big[scan::kNumBigClasses] = {};
    uint32_t nbig[scan::kNumBigClasses] = {};
    // bitmap path (null when off)
    uint32_t* hot = nullptr;       // n: hot id or kHotBits + v
    uint32_t* radj = nullptr;      // m + pad: adjacency mapped through hot[]
    uint32_t* tailc = nullptr;     // n: non-hot neighbours per vertex
    scan::CnTask* hubs = nullptr;  // hub tasks: hmid then bmp, one array
    scan::CnTask* hmid = nullptr;  // mid hubs (plan.bitmap_min_deg, kHubFilterMax]
    uint32_t nhmid = 0;
    scan::CnTask* bmp = nullptr;   // hubs above kHubFilterMax
    uint32_t nbmp = 0;
    uint32_t cap_small = 0, cap_big[scan::kNumBigClasses] = {}, cap_hubs = 0;   // task array capacities
    scan::PlanParams plan{};
    uint32_t long_words = 32;      // lists of >= long_words 16-byte words get a whole warp
    uint32_t* cn = nullptr;        // E: common-neighbour counts (the serving cache)
    bool cn_valid = false;
    bool cn_valid_before = false;
    RunScratch rs;                 // scratch of scan_run on this graph
    uint32_t* scratch = nullptr;   // scan tile sums, then dflags
    uint32_t* dflags = nullptr;    // [0] input checks, [1..8] planner counters, [16] long lists
    std::vector<std::pair<void*, size_t>> allocs;   // (pointer, bytes), returned to the cache on free
    uint64_t device_bytes = 0;     // device memory held by this graph
    uint32_t* adj_host = nullptr;  // streamed mode: pinned, GPU-mapped adjacency (adj points into it)
    cudaEvent_t ev[16] = {};       // 0-2 upload, 3-6 run stages, 7-12 and 15 similarity kernels
    std::mutex mu;                 // one run at a time per resident graph
};

namespace scan {

// Bytes of a RunScratch block for n vertices and E edges (256-byte aligned pieces).
size_t run_scratch_bytes(uint32_t n, uint64_t E);
// Point r's arrays into `base` (run_scratch_bytes(n, E) bytes of device memory).
void run_scratch_bind(RunScratch* r, void* base, uint32_t n, uint64_t E);

// Upload a CSR (32- or 64-bit offsets), check it and build the orientation and task plan.
// adj_in_host_memory: keep the adjacency in pinned, GPU-mapped host memory (the kernels read
// it over the host link) instead of HBM -- the streamed mode for graphs above a device budget.
scan_status device_upload(int device, uint64_t n, uint64_t m, const void* off_host, bool off64,
                          const uint32_t* adj_host, DeviceGraph** out, scan_stats* st,
                          bool adj_in_host_memory = false);
// cn for every edge on d->stream.
// cn for every edge; with `prune`, edges that the degree prune rules out at that eps are
// skipped and keep cn = 0 (a one-shot run; the result is not a reusable cache).
// With `fused` (a one-shot run whose plan splits no pivot), the kernels also run the
// predicate: sim, sd and the run counters must be zeroed before, and launch_cluster is
// then told so (predicate_done).
struct BatchParams;
// bp (batched runs, with prune and fused): each pivot takes eps and the predicate from its
// graph's entry of bp->gpp (prune then only supplies "on"); the one-shot fused path only.
scan_status launch_cn(DeviceGraph* d, uint32_t* launches, const PredParams* prune = nullptr,
                      const RunScratch* fused = nullptr, const BatchParams* bp = nullptr);
// Rebuild the similarity tasks for plan parameters pp.
scan_status plan_tasks(DeviceGraph* d, const PlanParams& pp);
// Time the similarity stage under plan settings (small-pivot strategy and degree cut, task
// size, chunk, long-list threshold, hub threshold; a coordinate search) and keep the
// fastest; returns its time in *best_ms.  stage (may be empty) queues the stage as the caller
// runs it (launch_cn with full counts when empty).
scan_status autotune_similarity(DeviceGraph* d, float* best_ms, const std::function<scan_status(uint32_t*)>& stage);
// Per-graph parameters of a batched run (many graphs as one disjoint union): the graph of
// each vertex and each graph's predicate parameters and mu (all device pointers).
struct BatchParams {
    const uint32_t* vgid;
    const PredParams* gpp;
    const int32_t* gmu;
    // prune-threshold tables: the distinct parameter sets (gpp[i].np_set indexes them; sets
    // beyond kPruneSets compute their thresholds per pivot), their number, the tables
    const PredParams* sets;
    const uint32_t* nsets;
    uint32_t* np_tabs;
};

// predicate -> cores -> union-find -> attach -> classify from d->cn into r, on stream s.
// No host synchronisation.  bp (may be null) gives per-graph parameters.
scan_status launch_cluster(const DeviceGraph* d, const RunScratch& r, cudaStream_t s, const PredParams& pp, int mu,
                           uint32_t* launches, const BatchParams* bp = nullptr, bool predicate_done = false);
// Cache the similarity threshold of every edge of a graph with full counts (served graphs).
scan_status compute_tau(DeviceGraph* d);
// eps text + mode -> predicate parameters.
scan_status make_pred(const char* eps_decimal, PredParams* pp, scan_predicate mode);

// Pointer-jumping rounds queued for n vertices: enough for any forest depth
// (ceil(log2(n + 1)) + 2, at most kMaxJumpRounds), or fewer under scan_set_loop_limits.
// Round r raises jump_flags[r] when it moved a pointer, so jump_flags[jump_rounds(n) - 1]
// != 0 means the flatten did not converge.
uint32_t jump_rounds(uint32_t n);
// CAS attempts a union may take before it gives up and raises kErrUnionFindLimit
// (1 << 20, or the value set by scan_set_loop_limits).
uint32_t union_find_limit();

}  // namespace scan
