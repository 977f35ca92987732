// Device side of the engine: resident graph, orientation, task planning, the SCAN
// pipeline and the C-ABI entry points that drive it.  One CUDA stream per resident graph;
// every stage is timed with CUDA events on that stream.
//
// Pipeline (reference stages in GPUSCAN++/GPUScan.cu:800-1009 for comparison):
//   upload     H2D of CSR, device-side input checks     (:836-851; checks of Graph.cpp:270-288)
//   orient     lower-list construction                   (host getEidAndEdgeList, Graph.cpp:52-141)
//   similarity cn for every edge (kernels_cn.cuh)        (__check_core + lazy intersect, :276-367)
//   predicate  eps test + similar-degree counts, fused    (__prep_edge/__check_core, :133-172)
//              into the counting in one-shot runs
//   cluster    cores, union-find, flatten                (__cluster_core1/2, __cluster_core, :479-652)
//   attach     borders                                   (__cluster_noncore, :654-730)
//   classify   hubs / outliers                           (__classify_others, :732-798)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <type_traits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "device_graph.h"
#include "graph_internal.h"
#include "kernels_cluster.cuh"
#include "kernels_cn.cuh"
#include "kernels_orient.cuh"

namespace scan {

#define SCAN_CUDA(call)                                                                               \
    do {                                                                                              \
        cudaError_t err_ = (call);                                                                    \
        if (err_ != cudaSuccess)                                                                      \
            return fail(SCAN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));        \
    } while (0)

#define SCAN_TRY(expr)                        \
    do {                                      \
        scan_status st_ = (expr);             \
        if (st_ != SCAN_OK) return st_;       \
    } while (0)

constexpr uint32_t kAdjPad = kGranuleEntries;   // zero entries past m: a granule's loads never leave the array

// Device-side input checks folded into the orientation count pass.
constexpr uint32_t kBadId = 1u, kBadSelfLoop = 2u, kBadOrder = 4u, kBadOffsets = 8u;

__global__ void k_offsets_from_u64(const uint64_t* __restrict__ in, uint64_t n1, uint32_t* __restrict__ out,
                                   uint32_t* __restrict__ bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n1; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t x = in[i];
        if (x > 0xFFFFFFFFull || (i > 0 && x < in[i - 1])) atomicOr(bad, kBadOffsets);
        out[i] = (uint32_t)x;
    }
}

__global__ void k_check_offsets32(const uint32_t* __restrict__ off, uint64_t n, uint64_t m, uint32_t* __restrict__ bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (off[i + 1] < off[i]) atomicOr(bad, kBadOffsets);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[n] != m)) atomicOr(bad, kBadOffsets);
}

__global__ void k_fill_u32(uint32_t* p, uint64_t n, uint32_t x) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = x;
}

// Reference edge order (GPUSCAN++/Graph.cpp:87-111): edge {u lower, v higher} has id
// P[u] + (rank of v among the higher neighbours of u), P = prefix of higher-neighbour
// counts.  Used to return cn[] in the order the reference's Edge_u/Edge_v use.
__global__ void k_higher_count(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ lo_off,
                               uint32_t* __restrict__ hcnt) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        hcnt[v] = (off[v + 1] - off[v]) - (lo_off[v + 1] - lo_off[v]);
}

__global__ void k_to_reference_order(uint64_t E, const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj,
                                     const uint32_t* __restrict__ lo_off, const uint32_t* __restrict__ lo_adj,
                                     const uint32_t* __restrict__ lo_src, const uint32_t* __restrict__ hpre,
                                     const uint32_t* __restrict__ cn, uint32_t* __restrict__ out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t u = lo_adj[e], v = lo_src[e];
        const uint32_t pos = lower_bound_u32(adj, off[u], off[u + 1], v) - off[u];        // v's index in N(u)
        const uint32_t lows = lower_bound_u32(lo_adj, lo_off[u], lo_off[u + 1], v) - lo_off[u];  // lower ones before v
        out[hpre[u] + (pos - lows)] = cn[e];
    }
}

}  // namespace scan

using namespace scan;

namespace scan {

// Device-memory cache: buffers of freed resident graphs are kept per device and handed to
// later uploads of similar size instead of cudaFree + cudaMalloc (cudaFree synchronises
// the whole device; both cost milliseconds at GB sizes).  At most g_cache_cap bytes per
// device are kept (8 GiB unless scan_set_cached_memory_limit says otherwise; the drop-in
// GPUScan() on R-MAT scale 22 uses about 2.6 GB); scan_release_cached_memory() frees them.
static std::mutex g_cache_mu;
static std::multimap<size_t, void*> g_cache[64];
static size_t g_cache_bytes[64] = {};
static size_t g_cache_cap = 8ull << 30;

static void* cache_take(int dev, size_t bytes, size_t* actual) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_cache_mu);
    auto it = g_cache[dev].lower_bound(bytes);
    if (it == g_cache[dev].end() || it->first > 2 * bytes + (1 << 20)) return nullptr;   // avoid large waste
    void* p = it->second;
    *actual = it->first;
    g_cache_bytes[dev] -= it->first;
    g_cache[dev].erase(it);
    return p;
}

extern "C" void scan_release_cached_memory(void) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    int prev = -1;
    cudaGetDevice(&prev);
    for (int dev = 0; dev < 64; ++dev) {
        if (g_cache[dev].empty()) continue;
        cudaSetDevice(dev);
        for (auto& kv : g_cache[dev]) cudaFree(kv.second);
        g_cache[dev].clear();
        g_cache_bytes[dev] = 0;
    }
    if (prev >= 0) cudaSetDevice(prev);
}

extern "C" void scan_set_cached_memory_limit(uint64_t bytes) {
    std::lock_guard<std::mutex> lock(g_cache_mu);
    g_cache_cap = bytes;
    int prev = -1;
    cudaGetDevice(&prev);
    for (int dev = 0; dev < 64; ++dev) {   // free the largest blocks until each device fits
        if (g_cache_bytes[dev] <= bytes) continue;
        cudaSetDevice(dev);
        while (g_cache_bytes[dev] > bytes && !g_cache[dev].empty()) {
            auto it = std::prev(g_cache[dev].end());
            cudaFree(it->second);
            g_cache_bytes[dev] -= it->first;
            g_cache[dev].erase(it);
        }
    }
    if (prev >= 0) cudaSetDevice(prev);
}

extern "C" uint64_t scan_cached_memory_bytes(int device) {
    if (device < 0 || device >= 64) return 0;
    std::lock_guard<std::mutex> lock(g_cache_mu);
    return g_cache_bytes[device];
}

static void cache_give(int dev, void* p, size_t bytes) {
    if (dev < 0 || dev >= 64) { cudaFree(p); return; }
    std::lock_guard<std::mutex> lock(g_cache_mu);
    if (g_cache_bytes[dev] + bytes > g_cache_cap) { cudaFree(p); return; }
    g_cache[dev].emplace(bytes, p);
    g_cache_bytes[dev] += bytes;
}

// Streams and events of a resident graph come from a per-device pool and go back to it
// when the graph is freed, so that a GPUScan() call (upload, run, free) creates and destroys
// none of its 3 streams and 29 events.
struct StreamSet {
    cudaStream_t stream, side, aux;
    cudaEvent_t fork, join, ev[16], chunk_ev[9];
};
static std::mutex g_ss_mu;
static std::vector<StreamSet> g_ss_pool[64];
constexpr size_t kStreamSetPool = 8;

static void destroy_streams(const StreamSet& x) {
    for (cudaStream_t st : {x.stream, x.side, x.aux})
        if (st) cudaStreamDestroy(st);
    for (cudaEvent_t e : {x.fork, x.join})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : x.ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : x.chunk_ev)
        if (e) cudaEventDestroy(e);
}

static StreamSet streams_of(const DeviceGraph* d) {
    StreamSet x{d->stream, d->side, d->aux, d->fork, d->join, {}, {}};
    std::copy(std::begin(d->ev), std::end(d->ev), x.ev);
    std::copy(std::begin(d->chunk_ev), std::end(d->chunk_ev), x.chunk_ev);
    return x;
}

// The current device must be d->device.
static scan_status take_streams(DeviceGraph* d) {
    StreamSet x{};
    bool pooled = false;
    if (d->device >= 0 && d->device < 64) {
        std::lock_guard<std::mutex> lock(g_ss_mu);
        auto& pool = g_ss_pool[d->device];
        if (!pool.empty()) {
            x = pool.back();
            pool.pop_back();
            pooled = true;
        }
    }
    if (!pooled) {
        auto make = [&]() -> cudaError_t {
            cudaError_t e = cudaSuccess;
            for (cudaStream_t* st : {&x.stream, &x.side, &x.aux})
                if (e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
            for (cudaEvent_t* ev : {&x.fork, &x.join})
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
            for (auto& ev : x.ev)
                if (e == cudaSuccess) e = cudaEventCreate(&ev);
            for (auto& ev : x.chunk_ev)
                if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            return e;
        };
        const cudaError_t e = make();
        if (e != cudaSuccess) {
            destroy_streams(x);
            return fail(SCAN_ERR_CUDA, std::string("stream/event creation: ") + cudaGetErrorString(e));
        }
    }
    d->stream = x.stream;
    d->side = x.side;
    d->aux = x.aux;
    d->fork = x.fork;
    d->join = x.join;
    std::copy(std::begin(x.ev), std::end(x.ev), d->ev);
    std::copy(std::begin(x.chunk_ev), std::end(x.chunk_ev), d->chunk_ev);
    return SCAN_OK;
}

void device_graph_free(DeviceGraph* d) {
    if (!d) return;
    int prev = -1;
    cudaGetDevice(&prev);
    if (d->device >= 0) cudaSetDevice(d->device);
    // the aux and side streams' last work is joined into the main stream
    const bool idle = d->stream && cudaStreamSynchronize(d->stream) == cudaSuccess;
    for (auto& a : d->allocs) cache_give(d->device, a.first, a.second);
    if (d->adj_host) cudaFreeHost(d->adj_host);
    const StreamSet x = streams_of(d);
    bool kept = false;
    if (idle && d->device >= 0 && d->device < 64 && x.stream && x.side && x.aux) {
        std::lock_guard<std::mutex> lock(g_ss_mu);
        if (g_ss_pool[d->device].size() < kStreamSetPool) {
            g_ss_pool[d->device].push_back(x);
            kept = true;
        }
    }
    if (!kept) destroy_streams(x);
    if (prev >= 0) cudaSetDevice(prev);
    delete d;
}

template <typename T>
static scan_status dalloc(DeviceGraph* d, T** p, uint64_t count) {
    const size_t want = std::max<uint64_t>(count, 1) * sizeof(T);
    const size_t bytes = (want + 255) & ~size_t(255);
    size_t got = bytes;                    // a cached block may be larger: keep its real size
    void* q = cache_take(d->device, bytes, &got);
    if (!q) {
        cudaError_t err = cudaMalloc(&q, bytes);
        if (err != cudaSuccess) {
            cudaGetLastError();
            // return cached blocks to the driver and try once more
            scan_release_cached_memory();
            err = cudaMalloc(&q, bytes);
        }
        if (err != cudaSuccess) {
            cudaGetLastError();
            return fail(SCAN_ERR_OUT_OF_MEMORY, "cudaMalloc of " + std::to_string(bytes) +
                                                    " bytes failed: " + cudaGetErrorString(err));
        }
    }
    d->allocs.emplace_back(q, got);
    d->device_bytes += bytes;
    *p = static_cast<T*>(q);
    return SCAN_OK;
}

static int grid_for(const DeviceGraph* d, uint64_t items, int threads, int per_sm = 8) {
    uint64_t g = (items + threads - 1) / threads;
    uint64_t cap = (uint64_t)d->num_sms * per_sm;
    if (g > cap) g = cap;
    return (int)std::max<uint64_t>(g, 1);
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t run_scratch_bytes(uint32_t n, uint64_t E) {
    return align256(E ? E : 1) + 8 * align256(4ull * n) + align256(n) + align256(sizeof(RunCounters)) +
           align256(4 * kMaxJumpRounds);
}

// The order is relied on: role follows label, and the round flags follow the counters
// (each padded to 256 bytes), so the serving loop copies each pair back in one transfer.
void run_scratch_bind(RunScratch* r, void* base, uint32_t n, uint64_t E) {
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) { char* q = p; p += align256(bytes); return q; };
    r->n = n;
    r->E = E;
    r->sim = reinterpret_cast<uint8_t*>(take(E ? E : 1));
    r->sd = reinterpret_cast<int32_t*>(take(4ull * n));
    r->parent = reinterpret_cast<int32_t*>(take(4ull * n));
    r->bmin = reinterpret_cast<int32_t*>(take(4ull * n));
    r->bmax = reinterpret_cast<int32_t*>(take(4ull * n));
    r->nmin = reinterpret_cast<int32_t*>(take(4ull * n));
    r->nmax = reinterpret_cast<int32_t*>(take(4ull * n));
    r->lab = reinterpret_cast<int32_t*>(take(4ull * n));
    r->label = reinterpret_cast<int32_t*>(take(4ull * n));
    r->role = reinterpret_cast<uint8_t*>(take(n));
    r->ctr = reinterpret_cast<RunCounters*>(take(sizeof(RunCounters)));
    r->jump_flags = reinterpret_cast<uint32_t*>(take(4 * kMaxJumpRounds));
}

// Limits of the bounded device loops.  Tests shrink them (scan_set_loop_limits) to make
// the loops give up and check that the error reaches the caller.
static std::atomic<uint32_t> g_union_limit{1u << 20};
static std::atomic<uint32_t> g_jump_cap{(uint32_t)kMaxJumpRounds};

uint32_t union_find_limit() { return g_union_limit.load(); }

uint32_t jump_rounds(uint32_t n) {
    uint32_t r = 2;
    while ((1ull << (r - 2)) < (uint64_t)n + 1 && r < (uint32_t)kMaxJumpRounds) ++r;
    return std::max(1u, std::min(r, g_jump_cap.load()));
}

static int grid_for_n(int num_sms, uint64_t items, int threads, int per_sm = 8) {
    uint64_t g = (items + threads - 1) / threads;
    uint64_t cap = (uint64_t)num_sms * per_sm;
    if (g > cap) g = cap;
    return (int)std::max<uint64_t>(g, 1);
}

// Exclusive scan of cnt[0..n) into out[0..n] on d->stream (out[n] = total); with popc,
// of the popcounts of cnt's words.  sums: one slot per kScanTile items.
static scan_status device_scan(DeviceGraph* d, const uint32_t* cnt, uint64_t n, uint32_t* out, uint32_t* sums,
                               bool popc = false) {
    const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles > 0) {
        if (popc)
            k_scan_tiles<true><<<(unsigned)tiles, kScanThreads, 0, d->stream>>>(cnt, n, out, sums);
        else
            k_scan_tiles<false><<<(unsigned)tiles, kScanThreads, 0, d->stream>>>(cnt, n, out, sums);
        k_scan_sums<<<1, kScanThreads, 0, d->stream>>>(sums, (uint32_t)tiles, out + n);
        k_scan_add<<<grid_for(d, n, 256), 256, 0, d->stream>>>(out, n, sums);
    } else {
        SCAN_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), d->stream));
    }
    SCAN_CUDA(cudaGetLastError());
    return SCAN_OK;
}

// Upload a CSR (32- or 64-bit offsets) and build the lower lists and the task plan.
// Build the similarity tasks for plan parameters pp (again on every call: the autotuner
// re-plans with other task sizes).  Needs the orientation (lo_off, work, tailc).
scan_status plan_tasks(DeviceGraph* d, const PlanParams& pp) {
    cudaStream_t s = d->stream;
    uint32_t* counts = d->dflags + 1;
    const unsigned pg = (unsigned)((d->n + 255) / 256);
    SCAN_CUDA(cudaMemsetAsync(counts, 0, (5 + kNumBigClasses) * sizeof(uint32_t), s));
    k_plan<<<pg, 256, 0, s>>>(d->n, d->off, d->lo_off, d->work, d->tailc, pp, counts, nullptr, nullptr, nullptr,
                              nullptr, nullptr, nullptr);
    uint32_t hc[5 + kNumBigClasses];
    SCAN_CUDA(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaStreamSynchronize(s));
    // task arrays: reuse the current ones when large enough
    auto ensure = [&](auto** p, uint32_t* cap, uint32_t need) -> scan_status {
        if (*p && *cap >= need) return SCAN_OK;
        SCAN_TRY(dalloc(d, p, need));
        *cap = need;
        return SCAN_OK;
    };
    d->nsmall = hc[0];
    SCAN_TRY(ensure(&d->small_piv, &d->cap_small, d->nsmall));
    for (int c = 0; c < kNumBigClasses; ++c) {
        d->nbig[c] = hc[1 + c];
        SCAN_TRY(ensure(&d->big[c], &d->cap_big[c], d->nbig[c]));
    }
    d->nbmp = hc[1 + kNumBigClasses];
    d->nhmid = hc[2 + kNumBigClasses];
    d->has_split = hc[3 + kNumBigClasses] > 0;
    d->nmiss = hc[4 + kNumBigClasses];               // lower edges of split pivots
    if (d->nmiss) SCAN_TRY(ensure(&d->miss, &d->cap_miss, d->nmiss));
    SCAN_TRY(ensure(&d->hubs, &d->cap_hubs, d->nhmid + d->nbmp));   // mid hubs, then the larger hubs
    d->hmid = d->hubs;
    d->bmp = d->hubs + d->nhmid;
    SCAN_CUDA(cudaMemsetAsync(counts, 0, sizeof(hc), s));
    k_plan<<<pg, 256, 0, s>>>(d->n, d->off, d->lo_off, d->work, d->tailc, pp, counts, d->small_piv, d->big[0],
                              d->big[1], d->big[2], d->bmp, d->hmid);
    SCAN_CUDA(cudaGetLastError());
    d->plan = pp;
    return SCAN_OK;
}

scan_status device_upload(int device, uint64_t n, uint64_t m, const void* off_host, bool off64,
                          const uint32_t* adj_host, DeviceGraph** out, scan_stats* st, bool adj_in_host_memory) {
    if (n == 0 || n >= 0xFFFFFFFFull) return fail(SCAN_ERR_INVALID_ARG, "vertex count must be in [1, 2^32-1)");
    if (m >= 0xFFFFFFF0ull) return fail(SCAN_ERR_TOO_LARGE, "m >= 2^32 directed entries");
    SCAN_CUDA(cudaSetDevice(device));
    std::unique_ptr<DeviceGraph, void (*)(DeviceGraph*)> d(new DeviceGraph(), device_graph_free);
    d->device = device;
    d->n = (uint32_t)n;
    d->m = m;
    SCAN_CUDA(cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, device));
    SCAN_TRY(take_streams(d.get()));
    cudaStream_t s = d->stream;

    SCAN_TRY(dalloc(d.get(), &d->off, n + 1));
    if (adj_in_host_memory) {
        SCAN_CUDA(cudaHostAlloc(&d->adj_host, (m + kAdjPad) * sizeof(uint32_t), cudaHostAllocMapped));
        SCAN_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&d->adj), d->adj_host, 0));
    } else {
        SCAN_TRY(dalloc(d.get(), &d->adj, m + kAdjPad));
    }
    SCAN_TRY(dalloc(d.get(), &d->lo_off, n + 1));
    SCAN_TRY(dalloc(d.get(), &d->work, n));
    const uint64_t tiles = (n + 1 + kScanTile - 1) / kScanTile;
    SCAN_TRY(dalloc(d.get(), &d->scratch, tiles + 64));
    uint32_t* flags = d->scratch + tiles;        // [0] input checks, [1..4] planner counters
    d->dflags = flags;
    uint32_t* cnt = nullptr;
    SCAN_TRY(dalloc(d.get(), &cnt, n));          // lower-neighbour counts (kept: reused below)

    SCAN_CUDA(cudaEventRecord(d->ev[0], s));
    SCAN_CUDA(cudaMemsetAsync(flags, 0, 64 * sizeof(uint32_t), s));
    if (off64) {
        uint64_t* tmp = nullptr;
        SCAN_CUDA(cudaMalloc(&tmp, (n + 1) * sizeof(uint64_t)));
        cudaError_t e1 = cudaMemcpyAsync(tmp, off_host, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
        if (e1 == cudaSuccess)
            k_offsets_from_u64<<<grid_for(d.get(), n + 1, 256), 256, 0, s>>>(tmp, n + 1, d->off, flags);
        cudaError_t e2 = cudaStreamSynchronize(s);
        cudaFree(tmp);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            return fail(SCAN_ERR_CUDA, std::string("offset upload: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    } else {
        SCAN_CUDA(cudaMemcpyAsync(d->off, off_host, (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    }
    // The offsets are checked first (every later kernel indexes lists by them), with the
    // degree histogram of the hot-id assignment; both need only the offsets, so the host
    // waits for those alone.
    k_check_offsets32<<<grid_for(d.get(), n, 256), 256, 0, s>>>(d->off, n, m, flags);

    // Hot ids for the bitmap path: the kHotBits highest-degree vertices (by degree bin).
    // On by default wherever it applies: its pivots are never split, so the early stop of
    // one-shot runs reaches the hubs too.  SCAN_GB300_BITMAP=off keeps the hash classes
    // only; "tails-free" turns it on only when every vertex with an edge gets a hot id.
    const char* knob = std::getenv("SCAN_GB300_BITMAP");
    const int mode = knob && !std::strcmp(knob, "off") ? 0 : knob && !std::strcmp(knob, "tails-free") ? 2 : 1;
    bool bitmap_path = mode != 0 && n + kHotBits < 0xFFFFFFF0ull && m > 0 && !adj_in_host_memory;
    uint32_t* hist = nullptr;
    std::vector<uint32_t> h(kDegBins, 0);
    if (bitmap_path) {
        SCAN_TRY(dalloc(d.get(), &hist, kDegBins + 1));
        SCAN_CUDA(cudaMemsetAsync(hist, 0, (kDegBins + 1) * sizeof(uint32_t), s));
        k_deg_hist<<<grid_for(d.get(), n, 256), 256, 0, s>>>(d->n, d->off, hist);
        SCAN_CUDA(cudaMemcpyAsync(h.data(), hist, kDegBins * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    }
    uint32_t bad = 0;
    SCAN_CUDA(cudaMemcpyAsync(&bad, flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaStreamSynchronize(s));
    if (bad) return fail(SCAN_ERR_FORMAT, "offsets are not a non-decreasing sequence from 0 to m");
    uint32_t min_bin = 1;                            // isolated vertices are never hot
    if (bitmap_path) {
        uint64_t acc = 0;
        for (uint32_t b = kDegBins; b-- > 1;) {
            if (acc + h[b] > kHotBits) { min_bin = b + 1; break; }
            acc += h[b];
        }
        if (mode == 2 && min_bin > 1) bitmap_path = false;   // some vertex would have a tail
    }
    const uint64_t fill_tiles = (m + kFillTile - 1) / kFillTile;
    uint32_t* tile_v = nullptr;                                // first vertex of each adjacency tile
    SCAN_TRY(dalloc(d.get(), &tile_v, fill_tiles + 1));
    uint32_t* lowbits = nullptr;                               // one bit per entry: lower neighbour
    SCAN_TRY(dalloc(d.get(), &lowbits, m / 32 + 2));
    if (bitmap_path) {
        SCAN_TRY(dalloc(d.get(), &d->hot, n));
        SCAN_TRY(dalloc(d.get(), &d->radj, m + kAdjPad));
        SCAN_TRY(dalloc(d.get(), &d->tailc, n));
    }

    // The adjacency arrives in chunks of whole vertex ranges; each chunk's entry checks,
    // hot-id mapping and orientation count (one pass, k_orient_tiles) run on a second stream
    // while the next chunk is copied.  The pass skips ids >= n, so no host check has to come
    // in between; the flags are read once, after the count.
    cudaStream_t s2 = d->aux;
    constexpr int kMaxChunks = 8;
    static_assert(kMaxChunks + 1 <= sizeof(d->chunk_ev) / sizeof(d->chunk_ev[0]), "one event per chunk and one more");
    cudaEvent_t* ev_chunk = d->chunk_ev;
    const int chunks = (adj_in_host_memory || m < (16ull << 20)) ? 1 : kMaxChunks;
    std::vector<uint32_t> vcut(chunks + 1, 0);
    vcut[chunks] = (uint32_t)n;
    auto off_at = [&](uint64_t v) -> uint64_t {
        return off64 ? static_cast<const uint64_t*>(off_host)[v] : static_cast<const uint32_t*>(off_host)[v];
    };
    for (int c = 1; c < chunks; ++c) {            // first vertex whose list starts at or after c*m/chunks
        uint64_t lo = vcut[c - 1], hi = n, target = m * (uint64_t)c / chunks;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) / 2;
            if (off_at(mid) < target) lo = mid + 1; else hi = mid;
        }
        vcut[c] = (uint32_t)lo;
    }
    scan_status ost = SCAN_OK;
    uint32_t orient_launches = 0;
    auto enqueue = [&]() -> scan_status {
        // on s2, needing only the offsets (already on the device)
        SCAN_CUDA(cudaMemsetAsync(lowbits, 0, (m / 32 + 2) * sizeof(uint32_t), s2));
        SCAN_CUDA(cudaMemsetAsync(cnt, 0, n * sizeof(uint32_t), s2));
        SCAN_CUDA(cudaMemsetAsync(d->work, 0, n * sizeof(unsigned long long), s2));
        if (bitmap_path) SCAN_CUDA(cudaMemsetAsync(d->tailc, 0, n * sizeof(uint32_t), s2));
        k_tile_map<<<grid_for(d.get(), n, 256), 256, 0, s2>>>(d->n, d->off, tile_v);
        if (bitmap_path)
            k_hot_assign<<<grid_for(d.get(), n, 256), 256, 0, s2>>>(d->n, d->off, min_bin, kHotBits, d->hot,
                                                                  hist + kDegBins);
        if (adj_in_host_memory) {
            std::memcpy(d->adj_host, adj_host, m * sizeof(uint32_t));
            std::memset(d->adj_host + m, 0, kAdjPad * sizeof(uint32_t));
        } else {
            SCAN_CUDA(cudaMemsetAsync(d->adj + m, 0, kAdjPad * sizeof(uint32_t), s));
        }
        for (int c = 0; c < chunks; ++c) {
            const uint64_t j0 = off_at(vcut[c]), j1 = off_at(vcut[c + 1]);
            if (!adj_in_host_memory && j1 > j0)
                SCAN_CUDA(cudaMemcpyAsync(d->adj + j0, adj_host + j0, (j1 - j0) * sizeof(uint32_t),
                                          cudaMemcpyHostToDevice, s));
            SCAN_CUDA(cudaEventRecord(ev_chunk[c], s));
            SCAN_CUDA(cudaStreamWaitEvent(s2, ev_chunk[c], 0));
            if (j1 > j0) {
                const uint64_t tiles = (j1 + kFillTile - 1) / kFillTile - j0 / kFillTile;
                k_orient_tiles<<<grid_for(d.get(), tiles * kFillThreads, kFillThreads), kFillThreads, 0, s2>>>(
                    j0, j1, d->n, m, d->off, d->adj, tile_v, d->hot, kHotBits, d->radj, cnt, d->work, d->tailc,
                    lowbits, flags, kBadId, kBadSelfLoop, kBadOrder);
                ++orient_launches;
            }
        }
        SCAN_CUDA(cudaEventRecord(d->ev[1], s));   // end of the copies
        if (bitmap_path) SCAN_CUDA(cudaMemsetAsync(d->radj + m, 0, kAdjPad * sizeof(uint32_t), s2));
        SCAN_CUDA(cudaEventRecord(ev_chunk[kMaxChunks], s2));
        SCAN_CUDA(cudaStreamWaitEvent(s, ev_chunk[kMaxChunks], 0));   // back to one stream
        return SCAN_OK;
    };
    ost = enqueue();
    if (ost != SCAN_OK) {
        cudaStreamSynchronize(s2);
        return ost;
    }
    SCAN_TRY(device_scan(d.get(), cnt, n, d->lo_off, d->scratch));
    uint32_t E32 = 0;
    SCAN_CUDA(cudaMemcpyAsync(&E32, d->lo_off + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaMemcpyAsync(&bad, flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaStreamSynchronize(s));
    if (bad & kBadId) return fail(SCAN_ERR_FORMAT, "neighbour id >= n");
    if (bad & kBadSelfLoop) return fail(SCAN_ERR_FORMAT, "self loop");
    if (bad & kBadOrder) return fail(SCAN_ERR_FORMAT, "neighbour list not sorted strictly ascending");
    d->E = E32;
    if (d->E * 2 != m) return fail(SCAN_ERR_FORMAT, "graph is not symmetric (lower entries * 2 != m)");
    SCAN_TRY(dalloc(d.get(), &d->lo_adj, d->E));
    SCAN_TRY(dalloc(d.get(), &d->lo_src, d->E));
    if (fill_tiles) {   // word prefix of the lower bits, then the fill
        const uint64_t nwords = (m + 31) / 32;
        uint32_t *wpre = nullptr, *wsums = nullptr;
        SCAN_TRY(dalloc(d.get(), &wpre, nwords + 1));
        SCAN_TRY(dalloc(d.get(), &wsums, (nwords + kScanTile - 1) / kScanTile + 1));
        SCAN_TRY(device_scan(d.get(), lowbits, nwords, wpre, wsums, true));
        k_fill_tiles<<<grid_for(d.get(), fill_tiles * kFillThreads, kFillThreads), kFillThreads, 0, s>>>(
            d->n, m, (uint32_t)d->E, d->off, d->adj, tile_v, lowbits, wpre, d->lo_adj, d->lo_src);
    }
    SCAN_CUDA(cudaGetLastError());

    // Task plan.
    PlanParams pp;
    pp.target_probes = 1ull << 22;
    pp.target_probes_bitmap = 1ull << 25;   // bitmap tasks: 8x, each pays a CTA-wide barrier
    pp.min_slice_edges = 64;
    pp.chunk_max = kChunkMax;
    pp.small_deg = kSmallDeg;
    pp.small_strategy = kSmallSerial;
    pp.bitmap_min_deg = kBitmapMinDeg;
    SCAN_TRY(plan_tasks(d.get(), pp));

    // Result and scratch arrays.
    SCAN_TRY(dalloc(d.get(), &d->cn, d->E));
    SCAN_TRY(dalloc(d.get(), &d->cn_ctr, 2));
    SCAN_TRY(dalloc(d.get(), &d->task_queue, 8));
    SCAN_TRY(dalloc(d.get(), &d->np_tab, kPruneTable));
    uint8_t* rs_mem = nullptr;
    SCAN_TRY(dalloc(d.get(), &rs_mem, run_scratch_bytes(d->n, d->E)));
    run_scratch_bind(&d->rs, rs_mem, d->n, d->E);
    SCAN_CUDA(cudaEventRecord(d->ev[2], s));
    SCAN_CUDA(cudaEventSynchronize(d->ev[2]));
    if (st) {
        st->ms_h2d = ev_ms(d->ev[0], d->ev[1]);
        st->ms_orient = ev_ms(d->ev[1], d->ev[2]);
        // offsets check (+ conversion), tile map, orientation passes, count scan, word scan +
        // fill, two planner passes; the bitmap path adds the degree histogram and hot ids
        st->kernel_launches += 2 + (off64 ? 1 : 0) + (bitmap_path ? 2 : 0) + orient_launches + (n ? 3 : 0) +
                               (fill_tiles ? 4 : 0) + 2;
    }
    *out = d.release();
    return SCAN_OK;
}

// Kernel attributes and occupancies, found once per device (so capturing launch_cn into a
// CUDA graph queries nothing).  [g] is 1 for the instantiations with per-graph parameters.
static bool g_attr_set[64] = {};
static bool g_attr_bitmap[64][2] = {};
static bool g_attr_filter[64][2][2] = {};   // [g][mid hubs]
static int g_per_sm[64][kNumBigClasses] = {};               // k_cn_big, each hash class
static int g_per_sm_hub_filter[64][2] = {};                 // k_cn_filter on the mid hubs
static int g_per_sm_filter[64][2][kNumBigClasses][2] = {};  // k_cn_filter, [g][class][largest class 2
                                                            // at the default chunk, or at the cap]

// A stride coprime to n near n / golden ratio: i * stride mod n visits 0..n-1 once each,
// consecutive draws far apart in the array (k_cn_big's order for split pivots).
static uint32_t spread_stride(uint32_t n) {
    if (n < 3) return 0;
    uint64_t st = (uint64_t)(n * 0.6180339887);
    auto gcd = [](uint64_t a, uint64_t b) { while (b) { const uint64_t r = a % b; a = b; b = r; } return a; };
    while (gcd(st, n) != 1) ++st;
    return (uint32_t)st;
}

template <bool kPerGraph>
static scan_status launch_cn_impl(DeviceGraph* d, uint32_t* launches, const CnPrune& pr, const FusedPred& fp) {
    cudaStream_t s = d->stream;
    const int g = kPerGraph ? 1 : 0;
    SCAN_CUDA(cudaEventRecord(d->ev[7], s));
    if (!g_attr_set[d->device]) {
        SCAN_CUDA(cudaFuncSetAttribute(k_cn_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(big_class_slots(kNumBigClasses - 1) * sizeof(uint32_t))));
        g_attr_set[d->device] = true;
    }
    // One-shot fused runs (every pivot unsplit) decide most edges from an upper bound on
    // their count (k_cn_filter); full counts and split plans use the bucketed table.
    const bool filter = fp.sim != nullptr;
    if (filter && !g_attr_filter[d->device][g][0]) {
        SCAN_CUDA(cudaFuncSetAttribute(k_cn_filter_classes<kPerGraph>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)filter_smem_bytes(kChunkMaxCap)));
        SCAN_CUDA(cudaFuncSetAttribute(k_cn_filter<kPerGraph>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)filter_smem_bytes(kHubFilterMax)));
        g_attr_filter[d->device][g][0] = true;
    }
    // The hub kernels run on the side stream (larger hubs, then mid hubs) while the hash
    // classes and the small pivots run on the main one, longest tasks first.  Every kernel is
    // persistent over its own task queue and writes its own edges' counts, so none waits on
    // another, and the CTAs of one fill the SMs that another's last tasks leave idle.  Run one
    // after the other, those tails added up (R-MAT s22 over the stage: 14.56 ms in sequence,
    // 13.3 ms on two streams; the larger hubs first: eps 0.2, mu 2 30.6 -> 29.8 ms).
    cudaStream_t sh = d->side;
    SCAN_CUDA(cudaEventRecord(d->fork, s));
    SCAN_CUDA(cudaStreamWaitEvent(sh, d->fork, 0));
    // Hubs.  The mid hubs of a one-shot run go to k_cn_filter like the hash classes; the
    // larger hubs, and every hub when counting in full, to the hot-id bitmap kernel (full
    // counts: one launch over both task lists, d->hmid being followed by d->bmp in one array).
    // Hubs above kHubFilterMax stay off k_cn_filter: edges between two hubs of degree above
    // 46,339 have no early-stop threshold (the reference's int square may wrap), so the
    // filter would end in an exact recount by binary search over the whole list.
    uint32_t nbitmap = d->nbmp;
    const CnTask* bitmap_tasks = d->bmp;
    const bool mid_on_filter = filter && d->nhmid;
    if (!mid_on_filter) {
        nbitmap += d->nhmid;
        bitmap_tasks = d->hmid;
    }
    if (nbitmap) {
        const size_t smem = (kHotBits / 32 + kTailSlots) * sizeof(uint32_t);
        if (!g_attr_bitmap[d->device][g]) {
            SCAN_CUDA(cudaFuncSetAttribute(k_cn_bitmap<kPerGraph>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
            g_attr_bitmap[d->device][g] = true;
        }
        const uint64_t grid = std::min<uint64_t>(nbitmap, (uint64_t)d->num_sms);
        k_cn_bitmap<kPerGraph><<<(unsigned)grid, kBitmapThreads, smem, sh>>>(
            bitmap_tasks, nbitmap, d->task_queue + 3, d->off, d->radj, d->lo_adj, d->cn, d->long_words, pr,
            d->cn_ctr, fp, pr.on);
        ++*launches;
    }
    if (mid_on_filter) {
        const int threads = 512;
        const size_t smem = filter_smem_bytes(kHubFilterMax);
        int& per_sm = g_per_sm_hub_filter[d->device][g];
        if (per_sm == 0) {
            SCAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cn_filter<kPerGraph>, threads, smem));
            per_sm = std::max(per_sm, 1);
        }
        const uint64_t grid = std::min<uint64_t>(d->nhmid, (uint64_t)d->num_sms * per_sm);
        k_cn_filter<kPerGraph><<<(unsigned)grid, threads, smem, sh>>>(
            d->hmid, d->nhmid, kHubFilterMax, d->task_queue + 4, d->off, d->adj,
            d->lo_adj, d->cn, d->long_words, pr, d->cn_ctr, fp, 1u);   // hubs: strided batches
        ++*launches;
    }
    for (int c = kNumBigClasses - 1; c >= 0; --c) {   // longest tasks first
        if (d->nbig[c]) {
            const int threads = c == 0 ? 128 : 512;   // class 0: many small pivots, measured fastest
            if (filter) {
                // unsplit: class 2 pivots hold up to the plan's chunk size
                const uint32_t entries = c == kNumBigClasses - 1 ? d->plan.chunk_max : big_class_entries(c);
                const size_t smem = filter_smem_bytes(entries);
                int& per_sm = g_per_sm_filter[d->device][g][c][entries > kChunkMax ? 1 : 0];
                if (per_sm == 0) {
                    SCAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cn_filter_classes<kPerGraph>,
                                                                            threads, smem));
                    per_sm = std::max(per_sm, 1);
                }
                const uint64_t grid = std::min<uint64_t>(d->nbig[c], (uint64_t)d->num_sms * per_sm);
                k_cn_filter_classes<kPerGraph><<<(unsigned)grid, threads, smem, s>>>(
                    d->big[c], d->nbig[c], entries, d->task_queue + c, d->off, d->adj,
                    d->lo_adj, d->cn, d->long_words, pr, d->cn_ctr, fp, 0u);
            } else {
                const size_t smem = big_class_slots(c) * sizeof(uint32_t);
                int& per_sm = g_per_sm[d->device][c];
                if (per_sm == 0) {
                    SCAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cn_big, threads, smem));
                    per_sm = std::max(per_sm, 1);
                }
                const uint64_t grid = std::min<uint64_t>(d->nbig[c], (uint64_t)d->num_sms * per_sm);
                k_cn_big<<<(unsigned)grid, threads, smem, s>>>(d->big[c], d->nbig[c], big_class_slots(c),
                                                                d->task_queue + c, d->off,
                                                                d->adj, d->lo_adj, d->cn, d->long_words, pr,
                                                                d->cn_ctr, pr.on ? d->miss : nullptr, d->nmiss,
                                                                pr.on && d->nmiss ? spread_stride(d->nbig[c]) : 0u);
            }
            ++*launches;
        }
        SCAN_CUDA(cudaEventRecord(d->ev[9 + c], s));
    }
    if (d->nsmall) {
        constexpr int kWpb = 8;
        const unsigned grid = (unsigned)grid_for(d, (uint64_t)d->nsmall * 32, kWpb * 32, 16);
        auto launch_small = [&](auto strategy) {
            k_cn_small<kWpb, kPerGraph, decltype(strategy)::value><<<grid, kWpb * 32, 0, s>>>(
                d->small_piv, d->nsmall, d->off, d->adj, d->lo_off, d->lo_adj, d->cn, d->long_words, pr, d->cn_ctr, fp,
                d->task_queue + 5);
        };
        if (d->plan.small_strategy == kSmallBatched) launch_small(std::integral_constant<int, kSmallBatched>());
        else if (d->plan.small_strategy == kSmallSearch) launch_small(std::integral_constant<int, kSmallSearch>());
        else launch_small(std::integral_constant<int, kSmallSerial>());
        ++*launches;
    }
    SCAN_CUDA(cudaEventRecord(d->ev[8], s));
    SCAN_CUDA(cudaEventRecord(d->ev[15], sh));
    SCAN_CUDA(cudaEventRecord(d->join, sh));
    SCAN_CUDA(cudaStreamWaitEvent(s, d->join, 0));
    SCAN_CUDA(cudaEventRecord(d->ev[12], s));
    SCAN_CUDA(cudaGetLastError());
    return SCAN_OK;
}

// cn for every edge (the similarity stage); events 7..12 bracket its kernels.
scan_status launch_cn(DeviceGraph* d, uint32_t* launches, const PredParams* prune, const RunScratch* fused,
                      const BatchParams* bp) {
    if (d->device < 0 || d->device >= 64) return fail(SCAN_ERR_INVALID_ARG, "device index must be < 64");
    CnPrune pr{0.0, 0, 1, 0u, 0, nullptr, nullptr, 0.0, 0.f, nullptr};
    if (prune) pr = CnPrune{prune->eps, prune->p, prune->q, 1u, prune->mode, nullptr, nullptr, prune->pq2,
                            prune->eps2_floor, nullptr};
    const bool per_graph = prune && bp;
    if (per_graph) {
        pr.gpp = bp->gpp;
        pr.vgid = bp->vgid;
    }
    FusedPred fp{nullptr, nullptr, nullptr};
    if (fused && prune && !d->has_split) fp = FusedPred{fused->sim, fused->sd, fused->ctr};
    if (per_graph && !fp.sim) return fail(SCAN_ERR_INVALID_ARG, "per-graph parameters need the fused one-shot path");
    cudaStream_t s = d->stream;
    SCAN_CUDA(cudaMemsetAsync(d->cn, 0, d->E * sizeof(uint32_t), s));
    SCAN_CUDA(cudaMemsetAsync(d->cn_ctr, 0, 2 * sizeof(unsigned long long), s));
    SCAN_CUDA(cudaMemsetAsync(d->task_queue, 0, 8 * sizeof(uint32_t), s));
    if (prune && d->nmiss) SCAN_CUDA(cudaMemsetAsync(d->miss, 0, (size_t)d->nmiss * sizeof(uint32_t), s));
    if (prune && !per_graph) {
        k_prune_table<<<kPruneTable / 256, 256, 0, s>>>(pr, d->np_tab);
        pr.np_tab = d->np_tab;
        ++*launches;
    } else if (per_graph && bp->np_tabs) {   // one table per parameter set of the batch
        k_prune_tables<<<dim3(kPruneTable / 256, kPruneSets), 256, 0, s>>>(bp->sets, bp->nsets, bp->np_tabs);
        pr.np_tab = bp->np_tabs;
        ++*launches;
    }
    return per_graph ? launch_cn_impl<true>(d, launches, pr, fp) : launch_cn_impl<false>(d, launches, pr, fp);
}

// Autotuner: a coordinate search over the plan, each setting timed on this graph with
// `stage` (the similarity stage as the caller runs it; null: full counts).  In order:
//   1. the small-pivot strategy (serial or batched lists) x the small-pivot degree cut;
//   2. the task size x the largest hash class's chunk;
//   3. the long-list threshold (lists of at least that many 16-byte words take a warp);
//   4. with the bitmap path on, the hub threshold (4,096 or 6,144 entries).
// Each step keeps the fastest setting found so far; the plan ends at the overall best.
scan_status autotune_similarity(DeviceGraph* d, float* best_ms, const std::function<scan_status(uint32_t*)>& stage) {
    auto run = [&](uint32_t* launches) -> scan_status {
        return stage ? stage(launches) : launch_cn(d, launches);
    };
    auto time_plan = [&](const PlanParams& pp, uint32_t lw, float* ms) -> scan_status {
        SCAN_TRY(plan_tasks(d, pp));
        d->long_words = lw;
        uint32_t launches = 0;
        SCAN_TRY(run(&launches));   // warm
        SCAN_CUDA(cudaEventRecord(d->ev[13], d->stream));
        SCAN_TRY(run(&launches));
        SCAN_CUDA(cudaEventRecord(d->ev[14], d->stream));
        SCAN_CUDA(cudaEventSynchronize(d->ev[14]));
        *ms = ev_ms(d->ev[13], d->ev[14]);
        return SCAN_OK;
    };
    PlanParams best_pp = d->plan;
    uint32_t best_lw = d->long_words;
    float best = 3.4e38f;
    auto consider = [&](const PlanParams& pp, uint32_t lw) -> scan_status {
        float ms = 0.f;
        SCAN_TRY(time_plan(pp, lw, &ms));
        if (ms < best) { best = ms; best_pp = pp; best_lw = lw; }
        return SCAN_OK;
    };
    for (uint32_t strategy : {(uint32_t)kSmallSerial, (uint32_t)kSmallBatched, (uint32_t)kSmallSearch})
        for (uint32_t sdeg : {64u, kSmallDeg}) {
            PlanParams pp = best_pp;
            pp.small_strategy = strategy;
            pp.small_deg = sdeg;
            SCAN_TRY(consider(pp, best_lw));
        }
    {
        const PlanParams base = best_pp;
        for (unsigned long long probes : {1ull << 20, 1ull << 22, 1ull << 24})
            for (uint32_t chunk : {kChunkMax, kChunkMaxCap}) {
                PlanParams pp = base;
                pp.target_probes = probes;
                pp.target_probes_bitmap = 8 * probes;
                pp.chunk_max = chunk;
                SCAN_TRY(consider(pp, best_lw));
            }
    }
    for (uint32_t lw : {16u, 32u, 64u}) SCAN_TRY(consider(best_pp, lw));
    if (d->tailc) {
        const PlanParams base = best_pp;
        for (uint32_t hub : {4096u, kBitmapMinDeg}) {
            PlanParams pp = base;
            pp.bitmap_min_deg = hub;
            SCAN_TRY(consider(pp, best_lw));
        }
    }
    SCAN_TRY(plan_tasks(d, best_pp));
    d->long_words = best_lw;
    d->cn_valid = false;
    if (best_ms) *best_ms = best;
    return SCAN_OK;
}

// Main stream: ev[7] (stage start), class 2 -> ev[11], class 1 -> ev[10], class 0 -> ev[9],
// small pivots -> ev[8]; side stream: the hubs from ev[7] to ev[15].
static void cn_kernel_times(DeviceGraph* d, scan_stats* st) {
    st->ms_cn_kernel[0] = ev_ms(d->ev[9], d->ev[8]);
    for (int c = 0; c < kNumBigClasses; ++c)
        st->ms_cn_kernel[1 + c] = ev_ms(c == kNumBigClasses - 1 ? d->ev[7] : d->ev[10 + c], d->ev[9 + c]);
    st->ms_cn_kernel[4] = ev_ms(d->ev[7], d->ev[15]);
    st->cn_work_items[0] = d->nsmall;
    for (int c = 0; c < kNumBigClasses; ++c) st->cn_work_items[1 + c] = d->nbig[c];
    st->cn_work_items[4] = d->nbmp + d->nhmid;
}

// predicate -> cores -> union-find -> attach -> classify, on cached cn.  Queued on s with
// no host synchronisation.
scan_status launch_cluster(const DeviceGraph* d, const RunScratch& r, cudaStream_t s, const PredParams& pp, int mu,
                           uint32_t* launches, const BatchParams* bp, bool predicate_done) {
    const uint64_t E = d->E;
    const uint32_t n = d->n;
    const int sms = d->num_sms, T = 256;
    const int ge = grid_for_n(sms, E, T), gn = grid_for_n(sms, n, T);
    k_cluster_reset<<<gn, T, 0, s>>>(n, predicate_done ? nullptr : r.sd, predicate_done ? nullptr : r.ctr,
                                     r.jump_flags, kMaxJumpRounds);
    ++*launches;
    const uint32_t* vgid = bp ? bp->vgid : nullptr;
    if (!predicate_done) {
        if (d->tau && !bp && d->cn_valid)
            k_predicate_tau<<<ge, T, 0, s>>>(E, d->lo_adj, d->lo_src, d->off, d->cn, d->tau, pp, r.sim, r.sd, r.ctr);
        else
            k_predicate<<<ge, T, 0, s>>>(E, d->lo_adj, d->lo_src, d->off, d->cn, pp, vgid, bp ? bp->gpp : nullptr,
                                         r.sim, r.sd, r.ctr);
        ++*launches;
    }
    k_core_init<<<gn, T, 0, s>>>(n, r.sd, mu, vgid, bp ? bp->gmu : nullptr, r.parent, r.bmin, r.bmax, r.nmin, r.nmax,
                                 r.ctr);
    k_union<<<ge, T, 0, s>>>(E, d->lo_adj, d->lo_src, r.sim, r.parent, r.ctr, union_find_limit());
    const uint32_t rounds = jump_rounds(n);
    if (n <= kJumpBlockMax) {
        k_jump_block<<<1, 1024, 0, s>>>(n, r.parent, r.jump_flags, rounds);
        ++*launches;
    } else {
        for (uint32_t i = 0; i < rounds; ++i) k_jump_round<<<gn, T, 0, s>>>(n, r.parent, r.jump_flags, i);
        *launches += rounds;
    }
    k_attach<<<ge, T, 0, s>>>(E, d->lo_adj, d->lo_src, r.sim, r.parent, r.bmin, r.bmax, r.ctr);
    k_label<<<gn, T, 0, s>>>(n, r.parent, r.bmin, r.lab, r.ctr);
    k_neighbour_labels<<<ge, T, 0, s>>>(E, d->lo_adj, d->lo_src, r.lab, r.nmin, r.nmax, r.ctr);
    k_finalize<<<gn, T, 0, s>>>(n, r.parent, r.bmin, r.bmax, r.nmin, r.nmax, r.label, r.role, r.ctr);
    *launches += 6;
    SCAN_CUDA(cudaGetLastError());
    return SCAN_OK;
}

scan_status compute_tau(DeviceGraph* d) {
    if (!d->tau) SCAN_TRY(dalloc(d, &d->tau, 2 * std::max<uint64_t>(d->E, 1)));
    if (d->E) k_tau<<<grid_for(d, d->E, 256), 256, 0, d->stream>>>(d->E, d->lo_adj, d->lo_src, d->off, d->cn, d->tau);
    SCAN_CUDA(cudaStreamSynchronize(d->stream));
    SCAN_CUDA(cudaGetLastError());
    return SCAN_OK;
}

scan_status make_pred(const char* eps_decimal, PredParams* pp, scan_predicate mode) {
    if (!eps_decimal) return fail(SCAN_ERR_INVALID_ARG, "eps text is null");
    uint64_t p = 0, q = 1;
    double e = 0;
    if (!parse_decimal(eps_decimal, &p, &q, &e))
        return fail(SCAN_ERR_INVALID_ARG, std::string("cannot read eps from '") + eps_decimal + "'");
    if (mode == SCAN_PRED_EXACT && p <= q && q > (1ull << 30))
        return fail(SCAN_ERR_INVALID_ARG, "exact predicate: eps needs a denominator <= 2^30 (at most 9 decimals)");
    if (mode != SCAN_PRED_EXACT && mode != SCAN_PRED_REF_F64) return fail(SCAN_ERR_INVALID_ARG, "unknown predicate");
    pp->eps = e;
    pp->p = p;
    pp->q = q;
    pp->mode = mode == SCAN_PRED_REF_F64 ? 1 : 0;
    if (pp->p > pp->q) { pp->p = 1; pp->q = 0; }   // eps > 1: exact predicate is never true
    pred_derive(pp);
    return SCAN_OK;
}

static scan_status ensure_device(scan_graph* g, int device, scan_stats* st) {
    if (device < 0) return fail(SCAN_ERR_INVALID_ARG, "device must be >= 0");
    if (g->dev && g->dev->device == device) return SCAN_OK;
    if (g->dev) { device_graph_free(g->dev); g->dev = nullptr; }
    return device_upload(device, g->n, g->m, g->off.data(), true, g->adj.data(), &g->dev, st);
}

// Full run on a resident graph: cn (unless cached and reuse_cn), then the cluster stages,
// then D2H of labels/roles.  Counts computed here skip the edges the degree prune rules
// out at this eps, so they do not fill the cache: cn_valid is left false.
// One write per 4 KB: the pages are mapped before a device-to-host copy lands in them.
static void touch_pages(void* p, size_t bytes) {
    if (!p) return;
    volatile char* c = static_cast<volatile char*>(p);
    for (size_t i = 0; i < bytes; i += 4096) c[i] = 0;
}

static scan_status run_resident(DeviceGraph* d, const PredParams& pp, int mu, bool reuse_cn, int32_t* out_label,
                                uint8_t* out_role, scan_stats* st) {
    std::lock_guard<std::mutex> lock(d->mu);
    SCAN_CUDA(cudaSetDevice(d->device));
    cudaStream_t s = d->stream;
    uint32_t launches = 0;
    SCAN_CUDA(cudaEventRecord(d->ev[3], s));
    d->cn_valid_before = d->cn_valid;
    const bool count = !(reuse_cn && d->cn_valid);
    // With no split pivot, the counting kernels also run the predicate (each count is final
    // in the lane that computes it).
    const bool fused = count && !d->has_split;
    if (count) {
        d->cn_valid = false;
        if (fused) {
            SCAN_CUDA(cudaMemsetAsync(d->rs.sim, 0, d->E, s));
            SCAN_CUDA(cudaMemsetAsync(d->rs.sd, 0, d->n * sizeof(int32_t), s));
            SCAN_CUDA(cudaMemsetAsync(d->rs.ctr, 0, sizeof(RunCounters), s));
        }
        SCAN_TRY(launch_cn(d, &launches, &pp, fused ? &d->rs : nullptr));
    }
    SCAN_CUDA(cudaEventRecord(d->ev[4], s));
    SCAN_TRY(launch_cluster(d, d->rs, s, pp, mu, &launches, nullptr, fused));
    SCAN_CUDA(cudaEventRecord(d->ev[5], s));
    // A copy into host pages the process has never touched costs far more than the copy
    // (R-MAT scale 22: 11 ms against 0.13 ms for 16 MB of labels into fresh malloc'd
    // memory), so the result's pages are touched here, while the kernels run.
    touch_pages(out_label, d->n * sizeof(int32_t));
    touch_pages(out_role, d->n);
    RunCounters hc;
    uint32_t last_round = 0;
    if (out_label) SCAN_CUDA(cudaMemcpyAsync(out_label, d->rs.label, d->n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (out_role) SCAN_CUDA(cudaMemcpyAsync(out_role, d->rs.role, d->n, cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaMemcpyAsync(&hc, d->rs.ctr, sizeof(hc), cudaMemcpyDeviceToHost, s));
    unsigned long long cn_ctr[2] = {0, 0};
    if (count) SCAN_CUDA(cudaMemcpyAsync(cn_ctr, d->cn_ctr, sizeof(cn_ctr), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaMemcpyAsync(&last_round, d->rs.jump_flags + jump_rounds(d->n) - 1, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaEventRecord(d->ev[6], s));
    SCAN_CUDA(cudaEventSynchronize(d->ev[6]));
    if (hc.error_flags) return fail(SCAN_ERR_DEVICE, "union-find exceeded its iteration limit");
    if (last_round) return fail(SCAN_ERR_DEVICE, "union-find flattening did not converge");
    if (st) {
        st->n = d->n;
        st->num_edges = d->E;
        st->num_cores = hc.cores;
        st->num_clusters = hc.clusters;
        st->num_hubs = hc.hubs;
        st->num_outliers = hc.outliers;
        st->num_borders = hc.borders;
        st->num_similar_edges = hc.similar_edges;
        st->pred_disagreements = hc.disagreements;
        st->multi_cluster_borders = hc.multi_borders;
        st->ms_similarity = ev_ms(d->ev[3], d->ev[4]);
        st->ms_cluster = ev_ms(d->ev[4], d->ev[5]);
        st->ms_d2h = ev_ms(d->ev[5], d->ev[6]);
        st->ms_total = ev_ms(d->ev[3], d->ev[6]);
        if (count) {
            cn_kernel_times(d, st);
            st->cn_words = cn_ctr[0];
            st->cn_edges_counted = cn_ctr[1];
        }
        st->kernel_launches += launches;
    }
    return SCAN_OK;
}

}  // namespace scan

extern "C" {

scan_status scan_graph_upload(scan_graph* g, int device) {
    clear_error();
    if (!g) return fail(SCAN_ERR_INVALID_ARG, "graph is null");
    return ensure_device(g, device, nullptr);
}

scan_status scan_graph_upload_streamed(scan_graph* g, int device, uint64_t device_budget_bytes,
                                       uint64_t* device_bytes_used) {
    clear_error();
    if (!g || device < 0) return fail(SCAN_ERR_INVALID_ARG, "graph is null or device < 0");
    if (g->dev) { device_graph_free(g->dev); g->dev = nullptr; }
    // device footprint: offsets, orientation, cn, run scratch, tasks (the adjacency stays on the host)
    const uint64_t E = g->m / 2;
    const uint64_t est = 4 * (g->n + 1) * 2 + 8 * g->n + 4 * g->n + 12 * E + run_scratch_bytes((uint32_t)g->n, E) +
                         (16ull << 20);
    if (device_budget_bytes && est > device_budget_bytes)
        return fail(SCAN_ERR_OUT_OF_MEMORY, "streamed graph needs about " + std::to_string(est >> 20) +
                                                " MiB of device memory, above the budget of " +
                                                std::to_string(device_budget_bytes >> 20) + " MiB");
    SCAN_TRY(device_upload(device, g->n, g->m, g->off.data(), true, g->adj.data(), &g->dev, nullptr, true));
    if (device_bytes_used) *device_bytes_used = g->dev->device_bytes;
    if (device_budget_bytes && g->dev->device_bytes > device_budget_bytes) {
        const uint64_t used = g->dev->device_bytes;
        device_graph_free(g->dev);
        g->dev = nullptr;
        return fail(SCAN_ERR_OUT_OF_MEMORY, "streamed graph used " + std::to_string(used >> 20) +
                                                " MiB of device memory, above the budget");
    }
    return SCAN_OK;
}

uint64_t scan_graph_device_bytes(const scan_graph* g) { return g && g->dev ? g->dev->device_bytes : 0; }

scan_status scan_graph_release_device(scan_graph* g) {
    clear_error();
    if (!g) return fail(SCAN_ERR_INVALID_ARG, "graph is null");
    if (g->dev) { device_graph_free(g->dev); g->dev = nullptr; }
    return SCAN_OK;
}

scan_status scan_run(scan_graph* g, int device, const char* eps_decimal, int mu, scan_predicate predicate,
                     int32_t* out_label, uint8_t* out_role, scan_stats* stats) {
    clear_error();
    if (!g || !out_label) return fail(SCAN_ERR_INVALID_ARG, "graph and out_label must be non-null");
    if (mu < 1) return fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1");
    PredParams pp;
    SCAN_TRY(make_pred(eps_decimal, &pp, predicate));
    if (stats) std::memset(stats, 0, sizeof(*stats));
    SCAN_TRY(ensure_device(g, device, stats));
    return run_resident(g->dev, pp, mu, false, out_label, out_role, stats);
}

scan_status scan_graph_autotune(scan_graph* g, int device, double* best_similarity_ms, uint32_t* long_words,
                                uint64_t* target_probes) {
    clear_error();
    if (!g) return fail(SCAN_ERR_INVALID_ARG, "graph is null");
    SCAN_TRY(ensure_device(g, device, nullptr));
    DeviceGraph* d = g->dev;
    std::lock_guard<std::mutex> lock(d->mu);
    SCAN_CUDA(cudaSetDevice(d->device));
    float ms = 0.f;
    SCAN_TRY(autotune_similarity(d, &ms, nullptr));
    if (best_similarity_ms) *best_similarity_ms = ms;
    if (long_words) *long_words = d->long_words;
    if (target_probes) *target_probes = d->plan.target_probes;
    return SCAN_OK;
}

scan_status scan_graph_plan(const scan_graph* g, uint32_t* small_deg, uint32_t* small_strategy, uint32_t* hub_min_deg,
                            uint32_t* chunk_max) {
    clear_error();
    if (!g || !g->dev) return fail(SCAN_ERR_INVALID_ARG, "graph is null or not resident");
    const PlanParams& pp = g->dev->plan;
    if (small_deg) *small_deg = pp.small_deg;
    if (small_strategy) *small_strategy = pp.small_strategy;
    if (hub_min_deg) *hub_min_deg = pp.bitmap_min_deg;
    if (chunk_max) *chunk_max = pp.chunk_max;
    return SCAN_OK;
}

scan_status scan_graph_set_plan(scan_graph* g, int device, uint32_t small_deg, uint32_t small_strategy,
                                uint32_t hub_min_deg, uint32_t chunk_max) {
    clear_error();
    if (!g) return fail(SCAN_ERR_INVALID_ARG, "graph is null");
    if (small_deg < 1 || small_deg > kSmallDeg || small_strategy > 2 || hub_min_deg < small_deg ||
        (chunk_max != kChunkMax && chunk_max != kChunkMaxCap))
        return fail(SCAN_ERR_INVALID_ARG, "plan: small_deg in [1, 128], small_strategy 0-2, hub_min_deg >= small_deg, "
                                          "chunk_max 6144 or 12288");
    SCAN_TRY(ensure_device(g, device, nullptr));
    DeviceGraph* d = g->dev;
    std::lock_guard<std::mutex> lock(d->mu);
    SCAN_CUDA(cudaSetDevice(d->device));
    PlanParams pp = d->plan;
    pp.small_deg = small_deg;
    pp.small_strategy = small_strategy;
    pp.bitmap_min_deg = hub_min_deg;
    pp.chunk_max = chunk_max;
    SCAN_TRY(plan_tasks(d, pp));
    d->cn_valid = false;
    return SCAN_OK;
}

scan_status scan_common_neighbors(scan_graph* g, int device, uint32_t* out_cn, scan_stats* stats) {
    clear_error();
    if (!g || !out_cn) return fail(SCAN_ERR_INVALID_ARG, "graph and out_cn must be non-null");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    SCAN_TRY(ensure_device(g, device, stats));
    DeviceGraph* d = g->dev;
    std::lock_guard<std::mutex> lock(d->mu);
    SCAN_CUDA(cudaSetDevice(d->device));
    cudaStream_t s = d->stream;
    uint32_t launches = 0;
    SCAN_CUDA(cudaEventRecord(d->ev[3], s));
    SCAN_TRY(launch_cn(d, &launches));
    SCAN_CUDA(cudaEventRecord(d->ev[4], s));
    d->cn_valid = true;
    // Reorder to the reference's edge ids.
    uint32_t *hcnt = nullptr, *hpre = nullptr, *sums = nullptr, *ref = nullptr;
    SCAN_CUDA(cudaMallocAsync(&hcnt, d->n * sizeof(uint32_t), s));
    SCAN_CUDA(cudaMallocAsync(&hpre, (d->n + 1) * sizeof(uint32_t), s));
    SCAN_CUDA(cudaMallocAsync(&sums, ((d->n + kScanTile) / kScanTile + 1) * sizeof(uint32_t), s));
    SCAN_CUDA(cudaMallocAsync(&ref, std::max<uint64_t>(d->E, 1) * sizeof(uint32_t), s));
    k_higher_count<<<grid_for(d, d->n, 256), 256, 0, s>>>(d->n, d->off, d->lo_off, hcnt);
    scan_status st = device_scan(d, hcnt, d->n, hpre, sums);
    if (st == SCAN_OK) {
        k_to_reference_order<<<grid_for(d, d->E, 256), 256, 0, s>>>(d->E, d->off, d->adj, d->lo_off, d->lo_adj,
                                                                    d->lo_src, hpre, d->cn, ref);
        touch_pages(out_cn, d->E * sizeof(uint32_t));   // while the kernels run (see run_resident)
        cudaMemcpyAsync(out_cn, ref, d->E * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    }
    cudaFreeAsync(hcnt, s);
    cudaFreeAsync(hpre, s);
    cudaFreeAsync(sums, s);
    cudaFreeAsync(ref, s);
    SCAN_CUDA(cudaStreamSynchronize(s));
    SCAN_CUDA(cudaGetLastError());
    if (st) return st;
    if (stats) {
        stats->n = d->n;
        stats->num_edges = d->E;
        stats->ms_similarity = ev_ms(d->ev[3], d->ev[4]);
        cn_kernel_times(d, stats);
        stats->kernel_launches += launches + 5;
    }
    return SCAN_OK;
}

scan_status scan_memberships(scan_graph* g, int device, const char* eps_decimal, int mu, scan_predicate predicate,
                             int32_t* out_cluster, int32_t* out_vertex, uint64_t capacity, uint64_t* num_pairs) {
    clear_error();
    if (!g || !num_pairs) return fail(SCAN_ERR_INVALID_ARG, "graph and num_pairs must be non-null");
    if (mu < 1) return fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1");
    PredParams pp;
    SCAN_TRY(make_pred(eps_decimal, &pp, predicate));
    SCAN_TRY(ensure_device(g, device, nullptr));
    DeviceGraph* d = g->dev;
    std::vector<int32_t> label(d->n);
    std::vector<uint8_t> role(d->n);
    SCAN_TRY(run_resident(d, pp, mu, true, label.data(), role.data(), nullptr));
    std::lock_guard<std::mutex> lock(d->mu);
    cudaStream_t s = d->stream;
    // Border pairs: count, then collect.
    unsigned long long* cnt = nullptr;
    SCAN_CUDA(cudaMallocAsync(&cnt, sizeof(unsigned long long), s));
    SCAN_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
    k_border_pairs<<<grid_for(d, d->E, 256), 256, 0, s>>>(d->E, d->lo_adj, d->lo_src, d->rs.sim, d->rs.parent, cnt,
                                                          nullptr, 0);
    unsigned long long nb = 0;
    SCAN_CUDA(cudaMemcpyAsync(&nb, cnt, sizeof(nb), cudaMemcpyDeviceToHost, s));
    SCAN_CUDA(cudaStreamSynchronize(s));
    std::vector<unsigned long long> keys(nb);
    if (nb) {
        unsigned long long* buf = nullptr;
        SCAN_CUDA(cudaMallocAsync(&buf, nb * sizeof(unsigned long long), s));
        SCAN_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        k_border_pairs<<<grid_for(d, d->E, 256), 256, 0, s>>>(d->E, d->lo_adj, d->lo_src, d->rs.sim, d->rs.parent, cnt,
                                                              buf, nb);
        SCAN_CUDA(cudaMemcpyAsync(keys.data(), buf, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        SCAN_CUDA(cudaFreeAsync(buf, s));
    }
    SCAN_CUDA(cudaFreeAsync(cnt, s));
    SCAN_CUDA(cudaStreamSynchronize(s));
    // Output formatting: add the cores, order by (cluster, vertex), drop repeats.
    for (uint32_t v = 0; v < d->n; ++v)
        if (role[v] == SCAN_ROLE_CORE) keys.push_back(((unsigned long long)(uint32_t)label[v] << 32) | v);
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    *num_pairs = keys.size();
    if (keys.size() > capacity || (!keys.empty() && (!out_cluster || !out_vertex)))
        return fail(SCAN_ERR_INVALID_ARG, "capacity too small for " + std::to_string(keys.size()) + " pairs");
    for (size_t i = 0; i < keys.size(); ++i) {
        out_cluster[i] = (int32_t)(keys[i] >> 32);
        out_vertex[i] = (int32_t)(uint32_t)keys[i];
    }
    return SCAN_OK;
}

void scan_set_loop_limits(int64_t union_find_iterations, int32_t jump_rounds_cap) {
    g_union_limit.store(union_find_iterations < 0 ? (1u << 20)
                                                  : (uint32_t)std::min<int64_t>(union_find_iterations, 1u << 30));
    g_jump_cap.store(jump_rounds_cap < 0 ? (uint32_t)kMaxJumpRounds
                                         : std::max<uint32_t>(1u, std::min<uint32_t>(jump_rounds_cap, kMaxJumpRounds)));
}

int32_t* scan_gpuscan_compat(int64_t n, int64_t m, const int32_t* adj, const uint32_t* num_edges, const uint32_t* eid,
                             const int32_t* edge_u, const int32_t* edge_v, double eps, int mu) {
    (void)eid;
    (void)edge_u;
    (void)edge_v;
    clear_error();
    if (n <= 0 || m < 0 || !num_edges || (!adj && m > 0)) {
        fail(SCAN_ERR_INVALID_ARG, "bad graph_t");
        return nullptr;
    }
    if (mu < 1) {
        fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1");
        return nullptr;
    }
    char text[48];
    if (scan_eps_to_decimal(eps, text, sizeof(text)) != SCAN_OK) return nullptr;
    PredParams pp;
    if (make_pred(text, &pp, SCAN_PRED_REF_F64) != SCAN_OK) return nullptr;
    pp.eps = eps;   // the double itself, exactly as the caller computed it
    pred_derive(&pp);
    const size_t bytes = (size_t)n * sizeof(int32_t);
    int32_t* out = static_cast<int32_t*>(std::malloc(bytes));
    if (!out) {
        fail(SCAN_ERR_OUT_OF_MEMORY, "malloc of the result failed");
        return nullptr;
    }
    DeviceGraph* d = nullptr;
    if (device_upload(0, (uint64_t)n, (uint64_t)m, num_edges, false, reinterpret_cast<const uint32_t*>(adj), &d,
                      nullptr) != SCAN_OK) {
        std::free(out);
        return nullptr;
    }
    scan_status st = run_resident(d, pp, mu, false, out, nullptr, nullptr);
    device_graph_free(d);
    if (st != SCAN_OK) {
        std::free(out);
        return nullptr;
    }
    return out;
}

}  // extern "C"
