// Orientation of the undirected edges and the exclusive scan used to lay them out.
//
// Every undirected edge {u, v} is stored once, under its higher endpoint v in
// (degree, id) order -- the "pivot" whose neighbour list the similarity kernel stages in
// shared memory.  The lower endpoint u is the same vertex the reference stores as
// Edge_u (GPUSCAN++/Graph.cpp:66-111); only the grouping differs (the reference groups
// edge ids by the lower endpoint, this layout by the higher one).
//
// HBM layout built here (all uint32):
//   lo_off[n+1]  edges of pivot v are e in [lo_off[v], lo_off[v+1])
//   lo_adj[E]    lower endpoint u of edge e (ascending id within a pivot)
//   lo_src[E]    pivot v of edge e
//   work[n]      sum of deg(u) over the lower neighbours of v (probe count of pivot v), u64
#pragma once

#include "device_common.cuh"

namespace scan {

// Warp per vertex: number of lower neighbours and their total degree; with hot ids
// (may be null), also the number of non-hot neighbours ("tail", bitmap path).
// Vertices with more than kBigList entries are left to the CTA-per-vertex kernels below
// (appended to big[] here), so one long list does not hold a warp for the whole pass.
constexpr uint32_t kBigList = 2048;

// Vertices [v_begin, v_end) (the upload runs it chunk by chunk as the adjacency arrives).
// Ids >= n are skipped here (the entry checks reject the graph before anything uses it).
// lowbits gets one bit per adjacency entry, set for the lower neighbours, so the fill
// pass reads the decision instead of gathering both degrees again.
__device__ __forceinline__ void set_low_bits(uint32_t* bits, uint32_t j0, uint32_t mask) {
    if (!mask) return;
    const uint32_t sh = j0 & 31u;
    atomicOr(&bits[j0 >> 5], mask << sh);
    if (sh) atomicOr(&bits[(j0 >> 5) + 1], mask >> (32u - sh));
}

__global__ void k_count_lower(uint32_t n, uint32_t v_begin, uint32_t v_end, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ adj,
                              uint32_t* __restrict__ cnt, unsigned long long* __restrict__ work,
                              const uint32_t* __restrict__ hot, uint32_t hot_bits, uint32_t* __restrict__ tail,
                              uint32_t* __restrict__ big, uint32_t* __restrict__ nbig, uint32_t* __restrict__ lowbits) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    for (uint64_t v = v_begin + warp; v < v_end; v += nwarps) {
        const uint32_t b = off[v], e = off[v + 1], dv = e - b;
        if (dv > kBigList) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = (uint32_t)v;
            continue;
        }
        uint32_t c = 0, tl = 0;
        unsigned long long w = 0;
        for (uint32_t j0 = b; j0 < e; j0 += 32) {
            const uint32_t j = j0 + lane;
            bool low = false;
            if (j < e) {
                const uint32_t u = adj[j];
                if (u < n) {
                    const uint32_t du = off[u + 1] - off[u];
                    low = precedes(du, u, dv, (uint32_t)v);
                    if (low) { ++c; w += du; }
                    if (hot) tl += hot[u] >= hot_bits;
                }
            }
            const uint32_t mask = __ballot_sync(0xFFFFFFFFu, low);
            if (lane == 0) set_low_bits(lowbits, j0, mask);
        }
        c = __reduce_add_sync(0xFFFFFFFFu, c);
        tl = __reduce_add_sync(0xFFFFFFFFu, tl);
        for (int s = 16; s > 0; s >>= 1) w += __shfl_xor_sync(0xFFFFFFFFu, w, s);
        if (lane == 0) {
            cnt[v] = c;
            work[v] = w;
            if (hot) tail[v] = tl;
        }
    }
}

// CTA per long list (vertices collected by k_count_lower): the same counts with a block
// reduction.
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long x, unsigned long long* sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = x;
    __syncthreads();
    unsigned long long t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0ull;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    }
    __syncthreads();
    return t;   // valid in thread 0
}

__global__ void k_count_lower_big(const uint32_t* __restrict__ big, const uint32_t* __restrict__ nbig,
                                  const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj,
                                  uint32_t* __restrict__ cnt, unsigned long long* __restrict__ work,
                                  const uint32_t* __restrict__ hot, uint32_t hot_bits, uint32_t* __restrict__ tail,
                                  uint32_t n, uint32_t* __restrict__ lowbits) {
    __shared__ unsigned long long sh[32];
    const uint32_t nb = *nbig;
    for (uint32_t i = blockIdx.x; i < nb; i += gridDim.x) {
        const uint32_t v = big[i];
        const uint32_t b = off[v], e = off[v + 1], dv = e - b;
        unsigned long long c = 0, w = 0, tl = 0;
        for (uint32_t j0 = b + (threadIdx.x & ~31u); j0 < e; j0 += blockDim.x) {   // warp-uniform bounds
            const uint32_t j = j0 + (threadIdx.x & 31u);
            bool low = false;
            if (j < e) {
                const uint32_t u = adj[j];
                if (u < n) {                 // ids >= n: rejected by the entry checks
                    const uint32_t du = off[u + 1] - off[u];
                    low = precedes(du, u, dv, v);
                    if (low) { ++c; w += du; }
                    if (hot) tl += hot[u] >= hot_bits;
                }
            }
            const uint32_t mask = __ballot_sync(0xFFFFFFFFu, low);
            if ((threadIdx.x & 31u) == 0) set_low_bits(lowbits, j0, mask);
        }
        c = block_sum_u64(c, sh);
        w = block_sum_u64(w, sh);
        tl = block_sum_u64(tl, sh);
        if (threadIdx.x == 0) {
            cnt[v] = (uint32_t)c;
            work[v] = w;
            if (hot) tail[v] = (uint32_t)tl;
        }
    }
}

// ---- input checks, entry-parallel -----------------------------------------------------------
// starts: one bit per adjacency position, set where a non-empty list begins.
// tile_v[k]: the vertex whose list holds entry k * kFillTile (the fill pass's tile map).
constexpr uint32_t kFillTile = 2048;
__global__ void k_mark_starts(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ starts,
                              uint32_t* __restrict__ tile_v) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = off[v], e = off[v + 1];
        if (e > b) {
            atomicOr(&starts[b >> 5], 1u << (b & 31u));
            for (uint64_t k = (b + (uint64_t)kFillTile - 1) / kFillTile; k * kFillTile < e; ++k)
                tile_v[k] = (uint32_t)v;
        }
    }
}

// Tile of kFillTile entries per CTA iteration: write the lower neighbours (bit set in
// lowbits) in adjacency order.  Entry j goes to wpre[j / 32] + (lower bits before j in its
// word), wpre being the exclusive scan of the words' popcounts; in adjacency order the
// lower entries of v are exactly lo_adj[lo_off[v], lo_off[v+1]).  The pivot of each
// entry comes from the tile's owner map: the list starts inside the tile are scattered
// into shared memory and an inclusive max-scan spreads each vertex over its entries.
// Entry-parallel, so a hub list costs what any other entries cost.
constexpr int kFillThreads = 256;
__device__ __forceinline__ uint32_t fill_slot(uint32_t i) { return i + (i >> 5); }   // bank skew

__global__ void __launch_bounds__(kFillThreads) k_fill_tiles(uint32_t n, uint64_t m, uint32_t E,
                                                             const uint32_t* __restrict__ off,
                                                             const uint32_t* __restrict__ adj,
                                                             const uint32_t* __restrict__ tile_v,
                                                             const uint32_t* __restrict__ lowbits,
                                                             const uint32_t* __restrict__ wpre,
                                                             uint32_t* __restrict__ lo_adj, uint32_t* __restrict__ lo_src) {
    constexpr int kPer = kFillTile / kFillThreads;
    __shared__ uint32_t owner[kFillTile + kFillTile / 32];
    __shared__ uint32_t warp_max[kFillThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint64_t ntiles = (m + kFillTile - 1) / kFillTile;
    for (uint64_t k = blockIdx.x; k < ntiles; k += gridDim.x) {
        const uint64_t j0 = k * kFillTile;
        const uint32_t len = (uint32_t)min((uint64_t)kFillTile, m - j0);
        const uint32_t v0 = tile_v[k];
        const uint32_t v1 = k + 1 < ntiles ? tile_v[k + 1] : n - 1;   // owner of the next tile's first entry
#pragma unroll
        for (int q = 0; q < kPer; ++q) owner[fill_slot(q * kFillThreads + tid)] = 0;
        __syncthreads();
        if (tid == 0) owner[0] = v0;
        // Every list that starts inside the tile belongs to a vertex in (v0, v1].
        for (uint64_t v = (uint64_t)v0 + 1 + tid; v <= v1; v += kFillThreads) {
            const uint32_t b = off[v];
            if (b < j0 + len && off[v + 1] > b) owner[fill_slot((uint32_t)(b - j0))] = (uint32_t)v;
        }
        __syncthreads();
        uint32_t x[kPer], run = 0;
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            run = max(run, owner[fill_slot(tid * kPer + q)]);
            x[q] = run;
        }
        uint32_t incl = run;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, s);
            if (lane >= (uint32_t)s) incl = max(incl, y);
        }
        uint32_t pre = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
        if (lane == 0) pre = 0;
        if (lane == 31) warp_max[wid] = incl;
        __syncthreads();
        for (uint32_t w = 0; w < wid; ++w) pre = max(pre, warp_max[w]);
#pragma unroll
        for (int q = 0; q < kPer; ++q) owner[fill_slot(tid * kPer + q)] = max(pre, x[q]);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = q * kFillThreads + tid;
            if (i < len) {
                const uint64_t j = j0 + i;
                const uint32_t word = lowbits[j >> 5], bit = (uint32_t)j & 31u;
                const uint32_t p = wpre[j >> 5] + __popc(word & ((1u << bit) - 1u));
                if (((word >> bit) & 1u) && p < E) {   // p < E always: the bits are the counted entries
                    lo_adj[p] = adj[j];
                    lo_src[p] = owner[fill_slot(i)];
                }
            }
        }
        __syncthreads();   // the owner map is reset for the next tile
    }
}

// Entry j of some list: its value w is < n; j is not inside w's own list (that would be a
// self-loop); unless j starts a list, w is above the previous entry.
// Entries [j_begin, j_end).
__global__ void k_check_entries(uint64_t j_begin, uint64_t j_end, uint32_t n, const uint32_t* __restrict__ off,
                                const uint32_t* __restrict__ adj, const uint32_t* __restrict__ starts,
                                uint32_t* __restrict__ bad, uint32_t bad_id, uint32_t bad_loop, uint32_t bad_order) {
    uint32_t flags = 0;
    for (uint64_t j = j_begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < j_end;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = adj[j];
        if (w >= n) { flags |= bad_id; continue; }
        if (off[w] <= j && j < off[w + 1]) flags |= bad_loop;
        const bool start = (starts[j >> 5] >> (j & 31u)) & 1u;
        if (!start && j > 0 && w <= adj[j - 1]) flags |= bad_order;
    }
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    if (flags && (threadIdx.x & 31) == 0) atomicOr(bad, flags);
}

// ---- hot ids for the bitmap path -----------------------------------------------------------
// Degree histogram with exact bins below 1024 and 256-wide bins above (monotone in degree).
constexpr uint32_t kDegBins = 2048;
__host__ __device__ __forceinline__ uint32_t deg_bin(uint32_t d) {
    return d < 1024u ? d : 1024u + min((d - 1024u) >> 8, 1023u);
}

__global__ void k_deg_hist(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kDegBins];
    for (uint32_t i = threadIdx.x; i < kDegBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[deg_bin(off[v + 1] - off[v])], 1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kDegBins; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// hot[v] in [0, hot_bits) for vertices whose degree bin is >= min_bin (at most hot_bits of
// them), hot_bits + v otherwise.  The order among hot ids is whatever the atomics give:
// counts do not depend on it.
__global__ void k_hot_assign(uint32_t n, const uint32_t* __restrict__ off, uint32_t min_bin, uint32_t hot_bits,
                             uint32_t* __restrict__ hot, uint32_t* __restrict__ counter) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t v0 = blockIdx.x * (uint64_t)blockDim.x; v0 < n; v0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = v0 + threadIdx.x;
        bool is_hot = false;
        if (v < n) {
            const uint32_t d = off[v + 1] - off[v];
            is_hot = d > 0 && deg_bin(d) >= min_bin;
        }
        const uint32_t mask = __ballot_sync(0xFFFFFFFFu, is_hot);
        uint32_t base = 0;
        if (lane == 0 && mask) base = atomicAdd(counter, __popc(mask));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (v < n) hot[v] = is_hot ? base + __popc(mask & ((1u << lane) - 1u)) : hot_bits + (uint32_t)v;
    }
}

// Entries [j_begin, j_end); ids >= n (rejected by the entry checks) map to 0xFFFFFFFF.
__global__ void k_map_adj(uint64_t j_begin, uint64_t j_end, uint32_t n, const uint32_t* __restrict__ adj,
                          const uint32_t* __restrict__ hot, uint32_t* __restrict__ radj) {
    for (uint64_t j = j_begin + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < j_end;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t w = adj[j];
        radj[j] = w < n ? hot[w] : 0xFFFFFFFFu;
    }
}

// ---- exclusive scan of uint32 counts (n items) into out[0..n], out[n] = total ----------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = x;
    for (int s = 1; s < 32; s <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, s);
        if (lane >= s) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t ws = lane < nw ? warp_sums[lane] : 0;
        uint32_t wi = ws;
        for (int s = 1; s < 32; s <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, s);
            if (lane >= s) wi += y;
        }
        if (lane < nw) warp_sums[lane] = wi - ws;
        if (lane == nw - 1) *total = wi;
    }
    __syncthreads();
    const uint32_t r = warp_sums[wid] + incl - x;
    __syncthreads();
    return r;
}

// kPopc: the items are the popcounts of the input words (the fill pass's word prefix).
template <bool kPopc>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ in, uint64_t n,
                                                             uint32_t* __restrict__ out, uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t total;
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t t = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? (kPopc ? (uint32_t)__popc(in[base + i]) : in[base + i]) : 0u;
        t += v[i];
    }
    uint32_t ex = block_exclusive_scan(t, warp_sums, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = ex;
        ex += v[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of the tile sums in place; writes the grand total to *grand.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* __restrict__ sums, uint32_t ntiles,
                                                            uint32_t* __restrict__ grand) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t total;
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < ntiles; b0 += kScanThreads) {
        const uint32_t i = b0 + threadIdx.x;
        const uint32_t x = i < ntiles ? sums[i] : 0u;
        const uint32_t ex = block_exclusive_scan(x, warp_sums, &total);
        if (i < ntiles) sums[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand = carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint64_t n, const uint32_t* __restrict__ sums) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] += sums[i / kScanTile];
}

}  // namespace scan
