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

// ---- entry-parallel tiles ---------------------------------------------------------------------
// The adjacency is cut into tiles of kFillTile entries.  tile_v[k] is the vertex whose list
// holds entry k * kFillTile.  A CTA working on tile k rebuilds the tile's owner map in shared
// memory: the lists that start inside the tile belong to the vertices in (tile_v[k],
// tile_v[k+1]]; their starts are scattered into the map and an inclusive max-scan spreads
// each vertex over its entries.  Every pass over the adjacency below is entry-parallel, so a
// hub list costs what any other entries cost.
constexpr uint32_t kFillTile = 2048;
constexpr int kFillThreads = 256;
__device__ __forceinline__ uint32_t fill_slot(uint32_t i) { return i + (i >> 5); }   // bank skew

__global__ void k_tile_map(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ tile_v) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = off[v], e = off[v + 1];
        for (uint64_t k = (b + (uint64_t)kFillTile - 1) / kFillTile; k * kFillTile < e; ++k) tile_v[k] = (uint32_t)v;
    }
}

// Owner map of tile k (entries [t0, t0 + len)): owner[fill_slot(i)] = key of the vertex whose
// list holds entry t0 + i.  Key = uint64: (v << 32) | degree of v; Key = uint32: v.  Keys
// grow with v, so the max-scan spreads them.  *first = off of the tile's first owner.  Ends
// with __syncthreads().
template <typename Key>
__device__ __forceinline__ Key owner_key(uint32_t v, uint32_t b, uint32_t e) {
    if constexpr (sizeof(Key) == 8) return ((unsigned long long)v << 32) | (e - b);
    else return v;
}

template <typename Key>
__device__ __forceinline__ void tile_owner_map(uint64_t k, uint64_t t0, uint32_t len, uint64_t ntiles, uint32_t n,
                                               const uint32_t* __restrict__ off, const uint32_t* __restrict__ tile_v,
                                               Key* owner, Key* warp_max, uint32_t* first) {
    constexpr int kPer = kFillTile / kFillThreads;
    const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t v0 = tile_v[k];
    const uint32_t v1 = k + 1 < ntiles ? tile_v[k + 1] : n - 1;   // owner of the next tile's first entry
#pragma unroll
    for (int q = 0; q < kPer; ++q) owner[fill_slot(q * kFillThreads + tid)] = 0;
    __syncthreads();
    if (tid == 0) {
        const uint32_t b = off[v0];
        owner[0] = owner_key<Key>(v0, b, off[v0 + 1]);
        *first = b;
    }
    for (uint64_t v = (uint64_t)v0 + 1 + tid; v <= v1; v += kFillThreads) {
        const uint32_t b = off[v], e = off[v + 1];
        if (b < t0 + len && e > b)
            owner[fill_slot((uint32_t)(b - t0))] = owner_key<Key>((uint32_t)v, b, e);
    }
    __syncthreads();
    Key x[kPer], run = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        run = max(run, owner[fill_slot(tid * kPer + q)]);
        x[q] = run;
    }
    Key incl = run;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        const Key y = __shfl_up_sync(0xFFFFFFFFu, incl, s);
        if (lane >= (uint32_t)s) incl = max(incl, y);
    }
    Key pre = __shfl_up_sync(0xFFFFFFFFu, incl, 1);
    if (lane == 0) pre = 0;
    if (lane == 31) warp_max[wid] = incl;
    __syncthreads();
    for (uint32_t w = 0; w < wid; ++w) pre = max(pre, warp_max[w]);
#pragma unroll
    for (int q = 0; q < kPer; ++q) owner[fill_slot(tid * kPer + q)] = max(pre, x[q]);
    __syncthreads();
}

// Entries [j_begin, j_end) of whole lists (one chunk of the upload): the input checks, the
// hot-id mapping and the orientation count in one read of the adjacency.  Per entry j of
// the list of v: w = adj[j] must be < n, differ from v (no self loop) and, unless j starts
// the list, exceed adj[j-1]; radj[j] = hot[w] (ids >= n: 0xFFFFFFFF) when hot is given;
// w is a lower neighbour when precedes(deg w, w, deg v, v), recorded as a bit of lowbits.
// Per vertex, added with one atomic per warp segment (the arrays start zeroed): cnt = the
// lower neighbours, work = the sum of their degrees, tail = the neighbours without a hot id.
__global__ void __launch_bounds__(kFillThreads) k_orient_tiles(
    uint64_t j_begin, uint64_t j_end, uint32_t n, uint64_t m, const uint32_t* __restrict__ off,
    const uint32_t* __restrict__ adj, const uint32_t* __restrict__ tile_v, const uint32_t* __restrict__ hot,
    uint32_t hot_bits, uint32_t* __restrict__ radj, uint32_t* __restrict__ cnt, unsigned long long* __restrict__ work,
    uint32_t* __restrict__ tail, uint32_t* __restrict__ lowbits, uint32_t* __restrict__ bad, uint32_t bad_id,
    uint32_t bad_loop, uint32_t bad_order) {
    constexpr int kPer = kFillTile / kFillThreads;
    __shared__ unsigned long long owner[kFillTile + kFillTile / 32];
    __shared__ unsigned long long warp_max[kFillThreads / 32];
    __shared__ uint32_t first;
    const uint32_t tid = threadIdx.x, lane = tid & 31;
    const uint64_t ntiles = (m + kFillTile - 1) / kFillTile;
    const uint64_t k_end = (j_end + kFillTile - 1) / kFillTile;
    uint32_t flags = 0;
    for (uint64_t k = j_begin / kFillTile + blockIdx.x; k < k_end; k += gridDim.x) {
        const uint64_t t0 = k * kFillTile;
        const uint32_t len = (uint32_t)min((uint64_t)kFillTile, m - t0);
        tile_owner_map(k, t0, len, ntiles, n, off, tile_v, owner, warp_max, &first);
#pragma unroll 2
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = q * kFillThreads + tid;
            const uint64_t j = t0 + i;
            const unsigned long long ow = owner[fill_slot(i)];
            const uint32_t v = (uint32_t)(ow >> 32), dv = (uint32_t)ow;
            bool low = false;
            uint32_t c = 0, tl = 0;
            unsigned long long ws = 0;
            if (j >= j_begin && j < j_end) {
                const uint32_t w = adj[j];
                if (w >= n) {
                    flags |= bad_id;
                    if (hot) radj[j] = 0xFFFFFFFFu;
                } else {
                    if (w == v) flags |= bad_loop;
                    const bool start = i == 0 ? j == first : (uint32_t)(owner[fill_slot(i - 1)] >> 32) != v;
                    if (!start && w <= adj[j - 1]) flags |= bad_order;
                    const uint32_t du = off[w + 1] - off[w];
                    low = precedes(du, w, dv, v);
                    if (low) { c = 1; ws = du; }
                    if (hot) {
                        const uint32_t h = hot[w];
                        radj[j] = h;
                        tl = h >= hot_bits;
                    }
                }
            }
            const uint32_t mask = __ballot_sync(0xFFFFFFFFu, low);
            if (lane == 0 && mask) atomicOr(&lowbits[j >> 5], mask);   // lane 0's j is 32-aligned
            // segmented sums over the warp's runs of one vertex (v is non-decreasing in lane)
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, v);
            const int lo = __ffs(peers) - 1, hi = 31 - __clz(peers);
#pragma unroll
            for (int s = 1; s < 32; s <<= 1) {
                const uint32_t yc = __shfl_up_sync(0xFFFFFFFFu, c, s), yt = __shfl_up_sync(0xFFFFFFFFu, tl, s);
                const unsigned long long yw = __shfl_up_sync(0xFFFFFFFFu, ws, s);
                if ((int)lane - s >= lo) { c += yc; tl += yt; ws += yw; }
            }
            if ((int)lane == hi && (c | tl)) {
                if (c) {
                    atomicAdd(&cnt[v], c);
                    atomicAdd(&work[v], ws);
                }
                if (tl) atomicAdd(&tail[v], tl);
            }
        }
        __syncthreads();   // the owner map is rebuilt for the next tile
    }
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    if (flags && lane == 0) atomicOr(bad, flags);
}

// Tile of kFillTile entries per CTA iteration: write the lower neighbours (bit set in
// lowbits) in adjacency order.  Entry j goes to wpre[j / 32] + (lower bits before j in its
// word), wpre being the exclusive scan of the words' popcounts; in adjacency order the
// lower entries of v are exactly lo_adj[lo_off[v], lo_off[v+1]).  The pivot of each entry
// comes from the tile's owner map.
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
    __shared__ uint32_t first;
    const uint32_t tid = threadIdx.x;
    const uint64_t ntiles = (m + kFillTile - 1) / kFillTile;
    for (uint64_t k = blockIdx.x; k < ntiles; k += gridDim.x) {
        const uint64_t j0 = k * kFillTile;
        const uint32_t len = (uint32_t)min((uint64_t)kFillTile, m - j0);
        tile_owner_map(k, j0, len, ntiles, n, off, tile_v, owner, warp_max, &first);
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
        __syncthreads();   // the owner map is rebuilt for the next tile
    }
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
