// scan_cores_noalloc: the core check of SCAN without any device allocation.
//
// Who needs this: code that is handed its device buffers and may not allocate any of its
// own.  Examples: a plugin or custom-call inside a host framework that owns every byte of
// device memory and only passes buffers in; a serving process that has already committed
// nearly all HBM to resident graphs; code that must not call cudaMalloc/cudaFree because
// those calls synchronise the device and would stall other work on it.  The regular entry
// points (scan_run and friends) allocate their working arrays; this one does not.
//
// What it computes: for every vertex, whether it is a core for (eps, mu) -- at least mu of
// its neighbours are eps-similar -- from the caller's CSR offsets, undirected edge list and
// common-neighbour counts (for instance those returned by scan_common_neighbors, with the
// edges of scan_orient_reference).  The result equals role == SCAN_ROLE_CORE of scan_run.
//
// Scratch: one counter per vertex, held in a fixed array compiled into the library
// (g_similar_degree below, kNoAllocMaxVertices entries = 4 MiB).  Every GPU that loads the
// library keeps that array until the process exits.  Graphs with more vertices are
// rejected with SCAN_ERR_TOO_LARGE.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "graph_internal.h"
#include "predicate.cuh"

namespace {

constexpr uint32_t kNoAllocMaxVertices = 1u << 20;

// The fixed scratch.  Host code must not use this name as an address: on the host it only
// names a stand-in object, so its device address is looked up once per device below.
static __device__ __align__(256) int32_t g_similar_degree[kNoAllocMaxVertices];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
int32_t* g_scratch[kMaxDevices] = {};   // device address of g_similar_degree, per device

__global__ void k_noalloc_zero(int32_t* sd, uint32_t n) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) sd[v] = 0;
}

// Same test and counting as the engine's predicate stage; either orientation of an edge
// is accepted (the lower-degree endpoint is picked here).  Edges naming a vertex >= n are
// skipped.
__global__ void k_noalloc_count(uint64_t E, uint32_t n, const uint32_t* __restrict__ off,
                                const uint32_t* __restrict__ eu, const uint32_t* __restrict__ ev,
                                const uint32_t* __restrict__ cn, double eps, uint64_t p, uint64_t q, int mode,
                                int32_t* sd) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = eu[e], v = ev[e];
        if (u >= n || v >= n) continue;
        uint32_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v];
        if (du > dv) {
            const uint32_t t = u; u = v; v = t;
            const uint32_t dt = du; du = dv; dv = dt;
        }
        const uint32_t t = cn[e];
        const bool s = mode ? scan::ref_f64_similar(t, du, dv, eps) : scan::exact_similar(t, du, dv, p, q);
        if (s) {
            atomicAdd(&sd[u], 1);
            atomicAdd(&sd[v], 1);
        }
    }
}

__global__ void k_noalloc_flags(uint32_t n, const int32_t* __restrict__ sd, int mu, uint8_t* __restrict__ is_core) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        is_core[v] = sd[v] >= mu ? 1 : 0;
}

// Device address of the scratch array on the current device.  Looked up with that device
// current on the first call for it, and again on every call whose stream is not being
// captured (the lookup allocates nothing; after a cudaDeviceReset the library's module is
// loaded anew and the array's address can change).  A captured call uses the address found
// last, so the first call on a device has to come before any capture.
scan_status scratch_for_current_device(cudaStream_t s, int32_t** out) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return scan::fail(SCAN_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
    if (dev < 0 || dev >= kMaxDevices) return scan::fail(SCAN_ERR_INVALID_ARG, "device index must be < 64");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    err = cudaStreamIsCapturing(s, &cap);
    if (err != cudaSuccess)
        return scan::fail(SCAN_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(err));
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        int32_t* ptr = nullptr;
        err = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_similar_degree);
        if (err != cudaSuccess || !ptr)
            return scan::fail(SCAN_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(err));
        g_scratch[dev] = ptr;
    } else if (!g_scratch[dev]) {
        return scan::fail(SCAN_ERR_INVALID_ARG,
                          "scan_cores_noalloc: make the first call on a device before any stream capture");
    }
    *out = g_scratch[dev];
    return SCAN_OK;
}

}  // namespace

extern "C" scan_status scan_cores_noalloc(const uint32_t* d_offsets, uint32_t n, const uint32_t* d_edge_u,
                                          const uint32_t* d_edge_v, const uint32_t* d_cn, uint64_t num_edges,
                                          const char* eps_decimal, int mu, scan_predicate predicate,
                                          uint8_t* d_is_core, void* stream) {
    scan::clear_error();
    if (!d_offsets || !d_is_core || (num_edges && (!d_edge_u || !d_edge_v || !d_cn)))
        return scan::fail(SCAN_ERR_INVALID_ARG, "scan_cores_noalloc: null buffer");
    if (n == 0) return scan::fail(SCAN_ERR_INVALID_ARG, "scan_cores_noalloc: n must be >= 1");
    if (n > kNoAllocMaxVertices)
        return scan::fail(SCAN_ERR_TOO_LARGE, "scan_cores_noalloc handles at most " +
                                                  std::to_string(kNoAllocMaxVertices) +
                                                  " vertices (its fixed scratch); use scan_run for larger graphs");
    if (mu < 1) return scan::fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1");
    if (predicate != SCAN_PRED_EXACT && predicate != SCAN_PRED_REF_F64)
        return scan::fail(SCAN_ERR_INVALID_ARG, "unknown predicate");
    uint64_t p = 0, q = 1;
    double eps = 0;
    if (!scan::parse_decimal(eps_decimal, &p, &q, &eps))
        return scan::fail(SCAN_ERR_INVALID_ARG, std::string("cannot read eps from '") +
                                                    (eps_decimal ? eps_decimal : "(null)") + "'");
    if (predicate == SCAN_PRED_EXACT && p <= q && q > (1ull << 30))
        return scan::fail(SCAN_ERR_INVALID_ARG, "exact predicate: eps needs a denominator <= 2^30");
    if (p > q) { p = 1; q = 0; }   // eps > 1: the exact test never holds
    cudaGetLastError();   // an earlier, unrelated launch error is not this call's
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int32_t* sd = nullptr;
    scan_status st = scratch_for_current_device(s, &sd);
    if (st != SCAN_OK) return st;
    const int T = 256;
    const unsigned gv = (unsigned)std::min<uint64_t>((n + T - 1) / T, 4096);
    const unsigned ge = (unsigned)std::min<uint64_t>((num_edges + T - 1) / T + 1, 8192);
    k_noalloc_zero<<<gv, T, 0, s>>>(sd, n);                 // the array keeps the last call's counts
    if (num_edges)
        k_noalloc_count<<<ge, T, 0, s>>>(num_edges, n, d_offsets, d_edge_u, d_edge_v, d_cn, eps, p, q,
                                          predicate == SCAN_PRED_REF_F64 ? 1 : 0, sd);
    k_noalloc_flags<<<gv, T, 0, s>>>(n, sd, mu, d_is_core);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return scan::fail(SCAN_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(err));
    return SCAN_OK;
}
