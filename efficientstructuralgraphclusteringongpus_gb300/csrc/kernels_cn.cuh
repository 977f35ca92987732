// Common-neighbour counting: cn[e] = |N(u) ∩ N(v)| for every undirected edge e = {u, v}.
//
// The reference counts each edge with a warp whose lanes binary-search the shorter list
// in the longer one (GPUSCAN++/GPUScan.cu:174-222), once per edge and again lazily in
// the link and attach phases (:579-584, :701-706).  Here every edge is counted exactly
// once, grouped by its higher endpoint v (the pivot):
//   1. the pivot's list N(v) (or one id-range chunk of it) is staged in shared memory: a
//      per-warp hash table for small pivots, and per CTA task a hashed bitmap plus a sorted
//      copy (one-shot runs, k_cn_filter), a bucketed hash table (full counts, k_cn_big) or
//      a bitmap of hot ids (hubs, k_cn_bitmap);
//   2. warps stream the lower endpoints' lists N(u) with 16-byte loads and probe each
//      element against it; ballots and warp reductions give the counts;
//   3. in one-shot runs the degree prune, the early stop and the predicate skip use integer
//      and float thresholds per pivot (predicate.cuh: pivot_tests, count_floor); only a
//      count that may be similar takes the two predicates in double and 128-bit integers.
// Per edge this reads deg(u) <= deg(v) entries, the shorter list, once; the longer
// list is read once per task, not once per edge.
//
// Work is cut into tasks (pivot, chunk of N(v), slice of the pivot's edges) by k_plan:
//   * small pivots (degree <= the plan's small_deg): one warp per pivot (k_cn_small);
//   * larger pivots: one CTA per task, by size class; hubs above the plan's hub threshold
//     take the hub task list;
//   * with the bitmap path off, pivots above the plan's chunk are split into id-range
//     chunks, each probed by the matching sub-range of N(u) (binary search), and the
//     partial counts are added atomically.
#pragma once

#include "device_common.cuh"
#include "device_graph.h"

namespace scan {

constexpr uint32_t kSmallDeg = 128;        // largest pivot degree handled by a single warp (the
                                           // plan's small_deg may be lower)
constexpr uint32_t kSmallSlots = 256;      // per-warp table slots (load <= 1/2)
constexpr uint32_t kChunkMax = 6144;       // default max pivot entries staged by one CTA (load 1/4)
constexpr uint32_t kChunkMaxCap = 12288;   // largest allowed (load 1/2 in the same table)
// Bitmap path: the kHotBits highest-degree vertices get ids in [0, kHotBits) ("hot");
// every other vertex x is kHotBits + x.  A pivot's hot neighbours go into a shared-memory
// bitmap (one bit per hot id, 128 KB), the rest (its "tail") into a bucketed table.
constexpr uint32_t kHotBits = 1u << 20;
constexpr uint32_t kTailSlots = 24576;     // 96 KB; tails up to kTailMax entries (load <= 1/2)
constexpr uint32_t kTailMax = kTailSlots / 2;
// Pivots above kBitmapMinDeg (the default of the plan's bitmap_min_deg) use the bitmap path
// (when it is on): those the largest hash table would split.  Smaller pivots stay on the hash classes, which run several CTAs per
// SM: a bitmap task of a mid-size pivot leaves most of its 32 warps waiting at the task
// barrier (R-MAT s22, eps 0.5: 33.0 ms against 38.3 ms with the threshold at 1024).
constexpr uint32_t kBitmapMinDeg = kChunkMax;
// Hubs up to kHubFilterMax entries (the "mid hubs") get their own task list: one-shot runs
// count them with k_cn_filter (a 2^19-bit filter, <= 1/42 false positives, plus the sorted
// copy: 112 KB, two CTAs per SM), full counts with k_cn_bitmap like the larger hubs.
constexpr uint32_t kHubFilterMax = kChunkMaxCap;
constexpr int kBitmapThreads = 1024;
__host__ __device__ constexpr uint32_t big_class_entries(int c) { return c == 0 ? 1024u : c == 1 ? 4096u : kChunkMax; }
__host__ __device__ constexpr uint32_t big_class_slots(int c) { return 4u * big_class_entries(c); }   // load <= 1/4
                                                                                                   // (class 2: <= 1/2)

struct CnTask {
    uint32_t v;      // pivot
    uint32_t cb;     // chunk of N(v): adjacency positions [cb, ce)
    uint32_t ce;
    uint32_t e0;     // edge slice [e0, e1) of the pivot
    uint32_t e1;
    uint32_t chunked;  // 1 when N(v) is split (partial counts are added atomically)
    uint32_t mofs;     // chunked: edge k's slot in the miss counters is k + mofs (mod 2^32)
    uint32_t pad1;
};

// Insert w into a table of `cap` slots (never full: load <= 1/4).
__device__ __forceinline__ void table_insert(uint32_t* tab, uint32_t cap, uint32_t w) {
    uint32_t s = hash_slot(w, cap);
    for (uint32_t it = 0; it < cap; ++it) {
        const uint32_t old = atomicCAS(&tab[s], kEmpty, w);
        if (old == kEmpty || old == w) return;
        s = (s + 1 == cap) ? 0 : s + 1;
    }
}

__device__ __forceinline__ uint32_t table_has(const uint32_t* tab, uint32_t cap, uint32_t w) {
    uint32_t s = hash_slot(w, cap);
    for (uint32_t it = 0; it < cap; ++it) {
        const uint32_t k = tab[s];
        if (k == w) return 1u;
        if (k == kEmpty) return 0u;
        s = (s + 1 == cap) ? 0 : s + 1;
    }
    return 0u;
}

// Bucketed table for the CTA-wide kernel: buckets of 4 slots (one 16-byte shared load),
// linear probing over buckets.  Insertion fills a bucket's slots in order, so a bucket
// whose last slot is empty ends every probe sequence through it.
__device__ __forceinline__ void bucket_insert(uint32_t* tab, uint32_t nb, uint32_t w) {
    uint32_t b = hash_slot(w, nb);
    for (uint32_t it = 0; it < nb; ++it) {
        uint32_t* s = tab + 4 * b;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t old = atomicCAS(&s[i], kEmpty, w);
            if (old == kEmpty || old == w) return;
        }
        b = (b + 1 == nb) ? 0 : b + 1;
    }
}

__device__ __forceinline__ uint32_t bucket_has(const uint32_t* tab, uint32_t nb, uint32_t w) {
    uint32_t b = hash_slot(w, nb);
    uint4 q = *reinterpret_cast<const uint4*>(tab + 4 * b);
    uint32_t hit = (q.x == w) | (q.y == w) | (q.z == w) | (q.w == w);
    if (hit || q.w == kEmpty) return hit;
    for (uint32_t it = 1; it < nb; ++it) {   // the home bucket is full: rare at load <= 1/4
        b = (b + 1 == nb) ? 0 : b + 1;
        q = *reinterpret_cast<const uint4*>(tab + 4 * b);
        hit = (q.x == w) | (q.y == w) | (q.z == w) | (q.w == w);
        if (hit || q.w == kEmpty) return hit;
    }
    return 0u;
}

// Degree prune of a one-shot run at a fixed eps: an edge that neither predicate can call
// similar whatever its count (ref_f64_never and exact_never both hold) is not counted;
// its cn stays 0, which both predicates still reject.  Off (on = 0) for the cached counts.
struct CnPrune {
    double eps;
    uint64_t p, q;
    uint32_t on;
    int mode;        // the run's predicate (PredParams::mode), for the fused predicate
    // batched runs: each graph's parameters and the graph of each vertex (device memory);
    // null for a single graph
    const PredParams* gpp;
    const uint32_t* vgid;
    double pq2;          // PredParams::pq2, eps2_floor (see pred_derive)
    float eps2_floor;
    const uint32_t* np_tab;   // single-graph runs: pivot_tests(d).np for d < kPruneTable (k_prune_table)
};

// The parameters for pivot v in a batched run: eps and the predicate of v's graph (the
// graphs of a batch are one disjoint union, so both endpoints of an edge share it).
// Kernels bind `const CnPrune& P = kPerGraph ? graph_copy : pr`, so single runs read
// the kernel parameter itself.
__device__ __forceinline__ CnPrune prune_of_graph(const CnPrune& pr, uint32_t v) {
    const PredParams g = pr.gpp[pr.vgid[v]];
    CnPrune r = pr;
    r.eps = g.eps;
    r.p = g.p;
    r.q = g.q;
    r.mode = g.mode;
    r.pq2 = g.pq2;
    r.eps2_floor = g.eps2_floor;
    r.np_tab = pr.np_tab && g.np_set < kPruneSets ? pr.np_tab + (size_t)g.np_set * kPruneTable : nullptr;
    return r;
}


__device__ __forceinline__ PivotTests pivot_tests(uint32_t dv, const CnPrune& P) {
    if (P.np_tab && dv < kPruneTable) {
        PivotTests t;
        t.np = P.np_tab[dv];
        t.tscale = P.eps2_floor * (float)(dv + 1ull);
        return t;
    }
    return pivot_tests(dv, P.on != 0, P.eps, P.p, P.q, P.pq2, P.eps2_floor);
}

// np_tab[d] = pivot_tests(d).np for every d < kPruneTable (capped at 2^32 - 1, above every
// du + 1 of a graph with fewer than 2^32 - 16 adjacency entries).
__device__ __forceinline__ uint32_t prune_threshold(uint32_t d, bool on, double eps, uint64_t p, uint64_t q,
                                                    double pq2) {
    const PivotTests t = pivot_tests(d, on, eps, p, q, pq2, 0.f);
    return t.np > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)t.np;
}

__global__ void k_prune_table(CnPrune pr, uint32_t* __restrict__ np_tab) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < kPruneTable) np_tab[d] = prune_threshold(d, pr.on != 0, pr.eps, pr.p, pr.q, pr.pq2);
}

// Batches: table y (blockIdx.y) for parameter set y < *nsets, pruning on.
__global__ void k_prune_tables(const PredParams* __restrict__ sets, const uint32_t* __restrict__ nsets,
                               uint32_t* __restrict__ np_tabs) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (y >= *nsets || d >= kPruneTable) return;
    const PredParams g = sets[y];
    np_tabs[(size_t)y * kPruneTable + d] = prune_threshold(d, true, g.eps, g.p, g.q, g.pq2);
}

// Predicate fused into the counting kernels of a one-shot run whose plan splits no pivot:
// the count of edge k is final when its lane holds it, so the eps test, the
// similar-degree counts and the run counters are done there instead of in k_predicate
// (which would read every edge, its endpoints and both degrees once more).  sim null:
// counts only.  sim must start zeroed (pruned edges of k_cn_small are not written).
struct FusedPred {
    uint8_t* sim;
    int32_t* sd;
    RunCounters* ctr;
};

// Warp-wide (holds a ballot): every lane calls it; lanes with valid set test edge k
// {u lower, v pivot} with count t.  v is the same for every lane of the call.  decided: both
// predicates reject the edge (pruned, or t below count_floor), so neither is evaluated.
// sim starts zeroed, so only similar edges are written.
__device__ __forceinline__ void fused_predicate(const FusedPred& fp, const CnPrune& pr, bool valid, bool decided,
                                                uint32_t k, uint32_t u, uint32_t v, uint32_t du, uint32_t dv,
                                                uint32_t t, uint32_t lane, unsigned long long& nsim,
                                                unsigned long long& ndis) {
    bool s = false;
    if (valid && !decided) {
        const bool r = ref_f64_similar(t, du, dv, pr.eps);
        const bool x = exact_similar(t, du, dv, pr.p, pr.q);
        s = pr.mode ? r : x;
        ndis += (r != x);
        nsim += s;
        if (s) {
            fp.sim[k] = 1;
            atomicAdd(&fp.sd[u], 1);
        }
    }
    const uint32_t nv = __popc(__ballot_sync(0xFFFFFFFFu, s));
    if (lane == 0 && nv) atomicAdd(&fp.sd[v], (int32_t)nv);
}

// End of a fused kernel: the warp's similar-edge and disagreement totals to the counters.
__device__ __forceinline__ void fused_totals(const FusedPred& fp, uint32_t lane, unsigned long long nsim,
                                             unsigned long long ndis) {
    if (!fp.sim) return;
    for (int o = 16; o > 0; o >>= 1) {
        nsim += __shfl_xor_sync(0xFFFFFFFFu, nsim, o);
        ndis += __shfl_xor_sync(0xFFFFFFFFu, ndis, o);
    }
    if (lane == 0) {
        if (nsim) atomicAdd(&fp.ctr->similar_edges, nsim);
        if (ndis) atomicAdd(&fp.ctr->disagreements, ndis);
    }
}

// First position in adj[b, e) whose value is >= key (scalar, uniform across the warp).
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* __restrict__ adj, uint32_t b, uint32_t e,
                                                    uint32_t key) {
    while (b < e) {
        const uint32_t mid = b + ((e - b) >> 1);
        if (__ldg(adj + mid) < key) b = mid + 1; else e = mid;
    }
    return b;
}

// Larger pivots: one CTA per task; a bucketed table of `cap` slots (cap/4 buckets) in
// dynamic shared memory.
//
// Warps fetch batches of 32 edges from a shared counter.  Lane i loads edge i's list
// bounds (narrowed to the task's id chunk when the pivot is split), so the dependent
// loads of 32 edges overlap.  Then
//   * lists of at least kLongWords 16-byte words are streamed one at a time by the whole
//     warp, two words in flight per lane, and counted with one warp reduction;
//   * the shorter lists, each widened to 32-byte boundaries, form one stream of 8-entry
//     granules; every round each lane takes one granule (a binary search over the batch's
//     prefix sums names its list), loads it and probes its valid entries, and each edge's
//     owner lane adds the hits that fell in its list from four ballots of the per-lane
//     counts (0..8).
constexpr uint32_t kLongWordsDefault = 32;   // lists of >= 128 entries take the whole warp (tunable)
constexpr int kWordsInFlight = 2;        // hash and class kernels (48+ registers would cost occupancy)
constexpr int kWordsInFlightMidHub = 3;  // k_cn_filter on mid hubs: two CTAs per SM by shared memory, so 64
                                         // registers cost nothing (R-MAT s22: 11.87 -> 11.73 ms; 3 in the
                                         // class kernels too: 12.11 ms)
constexpr int kWordsInFlightBitmap = 6;  // bitmap kernel: one CTA per SM, 64 registers at 6 (s22: -0.6 ms against 4)

__device__ __forceinline__ uint32_t lane_range_mask(int lo, int hi) {
    if (hi <= lo) return 0u;
    const uint32_t upto = hi >= 32 ? 0xFFFFFFFFu : ((1u << hi) - 1u);
    return upto & ~((1u << lo) - 1u);
}

__device__ __forceinline__ uint32_t probe_word(const uint4 x, uint32_t p, uint32_t lb, uint32_t le,
                                               const uint32_t* tab, uint32_t nb) {
    uint32_t c = 0;
    if (p >= lb && p < le) c += bucket_has(tab, nb, x.x);
    if (p + 1 >= lb && p + 1 < le) c += bucket_has(tab, nb, x.y);
    if (p + 2 >= lb && p + 2 < le) c += bucket_has(tab, nb, x.z);
    if (p + 3 >= lb && p + 3 < le) c += bucket_has(tab, nb, x.w);
    return c;
}

// Entries of a list of du that must be examined, given h hits so far, before the early
// stop can decide it: past du - tlo + h, hits + unexamined entries < tlo.  du when tlo = 0.
__device__ __forceinline__ uint32_t needed_entries(uint32_t du, uint32_t tlo, uint32_t h) {
    if (tlo == 0) return du;
    const int64_t need = (int64_t)du - (int64_t)tlo + (int64_t)h + 1;
    return need <= 0 ? 0u : need >= (int64_t)du ? du : (uint32_t)need;
}

// One list adj[b, e) streamed by the whole warp, W words in flight per lane; returns the
// warp's total (the same in every lane).  With tlo > 0 it stops once the list is decided
// (see needed_entries).  Every lane runs the same masked probe: measured faster than a
// separate unmasked interior path, whose head and tail words serialise.
template <int W, typename Probe>
__device__ __forceinline__ uint32_t warp_list(const uint32_t* __restrict__ adj, uint32_t b, uint32_t e, uint32_t tlo,
                                              uint32_t lane, uint32_t& words, Probe probe) {
    uint32_t h = 0;
    for (uint32_t base = b & ~3u; base < e; base += 128u * W) {
        words += min(32u * W, (e - base + 3u) >> 2);
        uint4 x[W];
#pragma unroll
        for (int q = 0; q < W; ++q) {
            const uint32_t pq = base + 4u * lane + 128u * q;
            x[q] = pq < e ? __ldg(reinterpret_cast<const uint4*>(adj + pq)) : make_uint4(0, 0, 0, 0);
        }
        uint32_t c = 0;
#pragma unroll
        for (int q = 0; q < W; ++q) c += probe(x[q], base + 4u * lane + 128u * q, b, e);
        h += __reduce_add_sync(0xFFFFFFFFu, c);
        if (tlo && min(e, base + 128u * W) - b >= needed_entries(e - b, tlo, h)) break;
    }
    return h;
}

// The short lists of a batch as one stream of granules, kGranuleWords 16-byte words each
// (8 entries, 32-byte aligned).  Lane i's list covers granules [excl_i, incl_i) of the
// stream; each round every lane takes one granule (a binary search over the inclusive
// prefixes names its list), loads its words, probes the valid entries, and the hits are
// credited to the owning lanes from four ballots of the per-granule counts (0..8).  Returns
// this lane's own count.  Two words per granule halve the search and the crediting per
// entry (R-MAT s22: 14.78 -> 14.56 ms over the stage); four words measured no faster (the
// lists' rounding wastes more), and one granule of two separate rounds costs more registers.
constexpr uint32_t kGranuleWords = 2;
constexpr uint32_t kGranuleEntries = 4u * kGranuleWords;   // adjacency arrays carry this many entries of padding

template <typename Probe>
__device__ __forceinline__ uint32_t short_stream(const uint32_t* __restrict__ adj, uint32_t lane, uint32_t ga,
                                                 uint32_t ub, uint32_t ue, uint32_t incl, uint32_t excl,
                                                 uint32_t total, Probe probe) {
    constexpr int kHitBits = 4;   // hits per granule <= 8
    uint32_t cnt = 0;
    for (uint32_t y0 = 0; y0 < total; y0 += 32u) {
        const uint32_t y = y0 + lane;
        uint32_t j = 0;   // owner: first lane whose inclusive prefix exceeds y
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
            const uint32_t pj = __shfl_sync(0xFFFFFFFFu, incl, j + st - 1);
            if (pj <= y) j += st;
        }
        j &= 31u;
        const uint32_t aj = __shfl_sync(0xFFFFFFFFu, ga, j);
        const uint32_t ej = __shfl_sync(0xFFFFFFFFu, excl, j);
        const uint32_t lb = __shfl_sync(0xFFFFFFFFu, ub, j);
        const uint32_t le = __shfl_sync(0xFFFFFFFFu, ue, j);
        const uint32_t p = aj + kGranuleEntries * (y - ej);
        uint32_t h = 0;
        if (y < total) {
            uint4 x[kGranuleWords];
#pragma unroll
            for (uint32_t q = 0; q < kGranuleWords; ++q) x[q] = __ldg(reinterpret_cast<const uint4*>(adj + p + 4u * q));
#pragma unroll
            for (uint32_t q = 0; q < kGranuleWords; ++q) h += probe(x[q], p + 4u * q, lb, le);
        }
        // this lane's granules within the round (stream positions below 2^31)
        const int lo = min(max((int)excl - (int)y0, 0), 32);
        const int hi = min(max((int)incl - (int)y0, 0), 32);
        const uint32_t m = lane_range_mask(lo, hi);
#pragma unroll
        for (int bit = 0; bit < kHitBits; ++bit)
            cnt += (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, (h >> bit) & 1u) & m) << bit;
    }
    return cnt;
}

// Counts for one batch of 32 edges; lane i holds list adj[ub, ue) of its lower endpoint
// (ue = ub for a pruned edge) and tlo, the early-stop threshold (0: count everything).
// Lists of at least long_words words of their needed prefix go to warp_list one at a
// time; the rest are streamed together by short_stream in phases: first each list's
// needed prefix at zero hits, then the extension its hits require, until every list is
// complete or decided.  Returns lane i's count (partial when decided early); adds the
// 16-byte words the warp read to `words` (the same in every lane).
template <int W, typename Probe>
__device__ __forceinline__ uint32_t count_batch(const uint32_t* __restrict__ adj, uint32_t lane, uint32_t ub,
                                                uint32_t ue, uint32_t tlo, uint32_t long_words, uint32_t& words,
                                                Probe probe) {
    const uint32_t du = ue - ub;
    uint32_t end = ub + needed_entries(du, tlo, 0);
    const uint32_t nwords = end > ub ? (((end + 3u) & ~3u) - (ub & ~3u)) >> 2 : 0u;
    uint32_t cnt = 0;
    uint32_t longs = __ballot_sync(0xFFFFFFFFu, nwords >= long_words);
    while (longs) {
        const int j = __ffs(longs) - 1;
        longs &= longs - 1;
        const uint32_t b = __shfl_sync(0xFFFFFFFFu, ub, j), e = __shfl_sync(0xFFFFFFFFu, ue, j);
        const uint32_t t = __shfl_sync(0xFFFFFFFFu, tlo, j);
        const uint32_t c = warp_list<W>(adj, b, e, t, lane, words, probe);
        if ((int)lane == j) cnt = c;
    }
    const bool done_long = nwords >= long_words;          // counted by the warp above
    uint32_t cur = ub;
    if (done_long) end = ub;
    for (;;) {
        const uint32_t ga = cur & ~(kGranuleEntries - 1u);
        const uint32_t sw = end > cur ? (((end + kGranuleEntries - 1u) & ~(kGranuleEntries - 1u)) - ga) / kGranuleEntries
                                      : 0u;
        if (__ballot_sync(0xFFFFFFFFu, sw != 0) == 0) break;
        uint32_t incl = sw;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, s);
            if ((int)lane >= s) incl += y;
        }
        const uint32_t excl = incl - sw;
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        words += total * kGranuleWords;
        cnt += short_stream(adj, lane, ga, cur, end, incl, excl, total, probe);
        // the next phase: what the hits found so far require (at least 8 words more)
        const uint32_t need = needed_entries(du, tlo, cnt);
        const uint32_t next = (!done_long && ub + need > end) ? min(ue, max(ub + need, end + 32u)) : end;
        cur = end;
        end = next;
    }
    return cnt;
}

// Small pivots: one warp per pivot.  Three ways to count a batch of 32 lower edges (lane i
// loads edge i's endpoint and list bounds, so the dependent loads of the 32 edges overlap);
// the planner picks one per graph (the autotuner times them):
//   * kSmallSerial: the pivot's list in a per-warp hash table; the warp counts the lists one
//     at a time, lanes over a list, one warp reduction per list;
//   * kSmallBatched: the same table; the 32 lists are streamed together by count_batch (one
//     stream of 8-entry granules, hits credited by ballot and popc), with the early stop of a
//     one-shot run.  The loads of different lists overlap: it pays where most edges are
//     counted (dense graphs), and costs where the degree prune leaves few;
//   * kSmallSearch: as kSmallBatched, but the pivot's list is kept sorted and each entry is
//     found by binary search (a galloping intersection, the reference's own method,
//     GPUSCAN++/GPUScan.cu:174-222, inside the warp-cooperative stream): no table to clear
//     or fill, log2(deg) dependent probes per entry.
// Warps draw pivots from a queue counter (`queue`, zeroed before the launch): pivots differ
// widely in cost, and a fixed stride left a tail (R-MAT s22: 1.40 -> 0.99 ms).
constexpr int kSmallSerial = 0, kSmallBatched = 1, kSmallSearch = 2;

__device__ __forceinline__ uint32_t sorted_has(const uint32_t* list, uint32_t n, uint32_t w) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (list[mid] < w) lo = mid + 1; else hi = mid;
    }
    return (lo < n && list[lo] == w) ? 1u : 0u;
}

__device__ __forceinline__ uint32_t search_probe_word(const uint4 x, uint32_t p, uint32_t lb, uint32_t le,
                                                      const uint32_t* list, uint32_t n) {
    uint32_t c = 0;
    if (p >= lb && p < le) c += sorted_has(list, n, x.x);
    if (p + 1 >= lb && p + 1 < le) c += sorted_has(list, n, x.y);
    if (p + 2 >= lb && p + 2 < le) c += sorted_has(list, n, x.z);
    if (p + 3 >= lb && p + 3 < le) c += sorted_has(list, n, x.w);
    return c;
}

__device__ __forceinline__ uint32_t small_probe_word(const uint4 x, uint32_t p, uint32_t lb, uint32_t le,
                                                     const uint32_t* tab) {
    uint32_t c = 0;
    if (p >= lb && p < le) c += table_has(tab, kSmallSlots, x.x);
    if (p + 1 >= lb && p + 1 < le) c += table_has(tab, kSmallSlots, x.y);
    if (p + 2 >= lb && p + 2 < le) c += table_has(tab, kSmallSlots, x.z);
    if (p + 3 >= lb && p + 3 < le) c += table_has(tab, kSmallSlots, x.w);
    return c;
}

template <int kWarpsPerBlock, bool kPerGraph, int kStrategy>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_cn_small(const uint32_t* __restrict__ pivots, uint32_t npiv, const uint32_t* __restrict__ off,
           const uint32_t* __restrict__ adj, const uint32_t* __restrict__ lo_off,
           const uint32_t* __restrict__ lo_adj, uint32_t* __restrict__ cn, uint32_t long_words, CnPrune pr,
           unsigned long long* __restrict__ ctr, FusedPred fp, uint32_t* queue) {
    __shared__ uint32_t tabs[kWarpsPerBlock][kSmallSlots];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* tab = tabs[wib];
    unsigned long long nsim = 0, ndis = 0;
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(queue, 1u);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        if (t >= npiv) break;
        const uint32_t v = pivots[t];
        CnPrune Pg;
        if constexpr (kPerGraph) Pg = prune_of_graph(pr, v);
        const CnPrune& P = kPerGraph ? Pg : pr;
        const uint32_t b = off[v], e = off[v + 1];
        const PivotTests pt = pivot_tests(e - b, P);
        if constexpr (kStrategy == kSmallSearch) {
            for (uint32_t j = b + lane; j < e; j += 32) tab[j - b] = adj[j];   // sorted copy (e - b <= 128)
        } else {
#pragma unroll
            for (uint32_t i = lane; i < kSmallSlots; i += 32) tab[i] = kEmpty;
            __syncwarp();
            for (uint32_t j = b + lane; j < e; j += 32) table_insert(tab, kSmallSlots, adj[j]);
        }
        __syncwarp();
        const uint32_t k0 = lo_off[v], k1 = lo_off[v + 1];
        uint32_t words = 0, counted = 0;
        for (uint32_t kb = k0; kb < k1; kb += 32) {
            const uint32_t kk = kb + lane;
            const bool vk = kk < k1;
            uint32_t u = 0, ub = 0, ue = 0, du = 0, mc = 0;
            bool pruned = false;
            if (vk) {
                u = lo_adj[kk];
                ub = off[u];
                ue = off[u + 1];
                du = ue - ub;
                pruned = edge_pruned(du, pt);
                if (pruned) ue = ub;   // cn stays 0
            }
            if constexpr (kStrategy != kSmallSerial) {
                const uint32_t tlo = (P.on && ue > ub) ? count_floor(du, e - b, pt, P.eps) : 0u;
                mc = count_batch<kWordsInFlight>(adj, lane, ub, ue, tlo, long_words, words,
                                                 [&](uint4 x, uint32_t p, uint32_t lb, uint32_t le) {
                                                     if constexpr (kStrategy == kSmallSearch)
                                                         return search_probe_word(x, p, lb, le, tab, e - b);
                                                     else
                                                         return small_probe_word(x, p, lb, le, tab);
                                                 });
                counted += __popc(__ballot_sync(0xFFFFFFFFu, ue > ub));
            } else {
                const uint32_t nk = min(32u, k1 - kb);
                for (uint32_t i = 0; i < nk; ++i) {
                    const uint32_t lb = __shfl_sync(0xFFFFFFFFu, ub, i), le = __shfl_sync(0xFFFFFFFFu, ue, i);
                    if (le == lb) continue;
                    words += (le - lb + 3u) >> 2;
                    ++counted;
                    uint32_t c = 0;
                    for (uint32_t j = lb + lane; j < le; j += 32) c += table_has(tab, kSmallSlots, __ldg(adj + j));
                    c = __reduce_add_sync(0xFFFFFFFFu, c);
                    if (lane == i) mc = c;
                }
            }
            if (vk) cn[kk] = mc;
            if (fp.sim)
                fused_predicate(fp, P, vk, pruned || mc < count_floor(du, e - b, pt, P.eps), kk, u, v, du, e - b, mc, lane, nsim,
                                ndis);
        }
        if (lane == 0 && counted) {
            atomicAdd(&ctr[0], (unsigned long long)words);
            atomicAdd(&ctr[1], (unsigned long long)counted);
        }
        __syncwarp();
    }
    fused_totals(fp, lane, nsim, ndis);
}

// Next task of a persistent CTA: from the launch's queue counter (dynamic: a CTA that drew
// short tasks takes more), or blockIdx-strided when queue is null.  Every thread calls it;
// it holds a CTA barrier.
__device__ __forceinline__ uint32_t next_task(uint32_t* queue, uint32_t prev, bool first, uint32_t* slot) {
    if (!queue) return first ? blockIdx.x : prev + gridDim.x;
    if (threadIdx.x == 0) *slot = atomicAdd(queue, 1u);
    __syncthreads();
    return *slot;
}

__global__ void k_cn_big(const CnTask* __restrict__ tasks, uint32_t ntasks, uint32_t cap, uint32_t* queue,
                         const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj,
                         const uint32_t* __restrict__ lo_adj, uint32_t* __restrict__ cn, uint32_t long_words,
                         CnPrune pr, unsigned long long* __restrict__ ctr, uint32_t* __restrict__ miss,
                         uint32_t nmiss, uint32_t stride) {
    extern __shared__ __align__(16) uint32_t tab[];
    __shared__ uint32_t next_batch, task_slot;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nb = cap / 4;
    for (uint32_t t = next_task(queue, 0, true, &task_slot); t < ntasks;
         t = next_task(queue, t, false, &task_slot)) {
        // stride (coprime to ntasks, 0: in order): the i-th task drawn is i * stride mod ntasks,
        // so the chunks of one split pivot, adjacent in the array, run spread over the launch
        // and the misses of the early ones can decide edges for the later ones
        const CnTask tk = tasks[stride ? (uint32_t)((uint64_t)t * stride % ntasks) : t];
        for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x)
            reinterpret_cast<uint4*>(tab)[i] = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
        if (threadIdx.x == 0) next_batch = 0;
        __syncthreads();
        for (uint32_t j = tk.cb + threadIdx.x; j < tk.ce; j += blockDim.x) bucket_insert(tab, nb, adj[j]);
        __syncthreads();
        const uint32_t vb = off[tk.v], ve = off[tk.v + 1];
        const PivotTests pt = pivot_tests(ve - vb, pr);   // np = 0 when counting in full
        const uint32_t lo_id = (tk.cb > vb) ? adj[tk.cb] : 0u;          // chunk id range
        const uint32_t hi_id = (tk.ce < ve) ? adj[tk.ce - 1] : kEmpty;
        for (;;) {
            uint32_t bidx = 0;
            if (lane == 0) bidx = atomicAdd(&next_batch, 1u);
            const uint32_t kb = tk.e0 + 32u * __shfl_sync(0xFFFFFFFFu, bidx, 0);
            if (kb >= tk.e1) break;
            const uint32_t k = kb + lane;
            const bool valid = k < tk.e1;
            uint32_t ub = 0, ue = 0, u = 0, du = 0, tlo = 0, mi = 0xFFFFFFFFu;
            bool counted = false;
            if (valid) {
                u = lo_adj[k];
                ub = off[u];
                ue = off[u + 1];
                du = ue - ub;
                if (edge_pruned(du, pt)) ue = ub;
                counted = ue > ub && tk.cb == vb;               // once per edge: in its first chunk
                if (pr.on && ue > ub) tlo = count_floor(du, ve - vb, pt, pr.eps);
                if (tk.chunked && ue > ub) {
                    // One-shot runs: the misses found by the edge's other chunks so far bound
                    // its count by du - misses; once that is below tlo the edge is decided and
                    // its other chunks skip it.  Stale reads only weaken the bound.
                    uint32_t pot = du;
                    if (tlo && miss && k + tk.mofs < nmiss) {
                        mi = k + tk.mofs;
                        const uint32_t m = __ldcg(miss + mi);
                        pot = m >= du ? 0u : du - m;
                    }
                    if (pot < tlo) {
                        ue = ub;
                    } else {
                        if (lo_id) ub = lower_bound_u32(adj, ub, ue, lo_id);
                        if (hi_id != kEmpty) ue = lower_bound_u32(adj, ub, ue, hi_id + 1);
                        // hits this chunk must still find for the edge to reach tlo; 0: none
                        // decides it here, so the chunk counts its sub-list in full
                        const uint64_t outside = (uint64_t)pot - (ue - ub);
                        tlo = mi != 0xFFFFFFFFu && tlo > outside ? (uint32_t)(tlo - outside) : 0u;
                    }
                }
            }
            uint32_t words = 0;
            const uint32_t cnt = count_batch<kWordsInFlight>(adj, lane, ub, ue, tlo, long_words, words,
                                                             [&](uint4 x, uint32_t p, uint32_t lb, uint32_t le) {
                                                                 return probe_word(x, p, lb, le, tab, nb);
                                                             });
            const uint32_t nc = __popc(__ballot_sync(0xFFFFFFFFu, counted));
            if (lane == 0 && (words | nc)) {
                atomicAdd(&ctr[0], (unsigned long long)words);
                atomicAdd(&ctr[1], (unsigned long long)nc);
            }
            if (valid) {
                if (!tk.chunked) {
                    cn[k] = cnt;
                } else {
                    if (cnt) atomicAdd(&cn[k], cnt);            // cn was zeroed before the launch
                    if (mi != 0xFFFFFFFFu && ue > ub) {
                        // below its threshold the chunk decided the edge (stopped early, or read
                        // in full with too few hits); otherwise it read all ue - ub entries
                        if (tlo && cnt < tlo) atomicMax(miss + mi, du);
                        else if (ue - ub > cnt) atomicAdd(miss + mi, ue - ub - cnt);
                    }
                }
            }
        }
        __syncthreads();
    }
}

// One-shot runs on the hash classes (no split pivot, predicate fused): nearly every counted
// edge ends not similar, so an upper bound on its count decides it.  The pivot's list is
// staged twice in shared memory: as a hashed bitmap of 2^log2bits bits (at least 32 bits
// per entry, so a probe of a non-neighbour finds its bit set with probability <= 1/32) and
// as a sorted copy.  Streaming a lower list counts the entries whose bit is set; every
// common neighbour's bit is set, so the bit count B over the examined prefix plus the
// unexamined entries bounds cn, and the early stop (needed_entries) runs on B.  A list
// decided that way stores B < tlo, which both predicates reject like the true count.  Lists
// whose bound reaches tlo (or with tlo = 0: any count may be similar) are recounted exactly,
// one at a time by the whole warp, each entry binary-searched in the sorted copy.
// A probe is one 4-byte shared load of a random word, against one 16-byte bucket load for
// the bucketed table of k_cn_big.  The bit is taken with a wrapping funnel shift (its shift
// count uses the low five bits), and a word wholly inside the list skips the bound tests
// (R-MAT s22: both together 17.5 -> 16.6 ms over the stage).
__device__ __forceinline__ uint32_t filter_bit(uint32_t w, uint32_t log2bits) {
    return (w * 0x9E3779B1u) >> (32u - log2bits);
}

__device__ __forceinline__ uint32_t filter_probe_word(const uint4 x, uint32_t p, uint32_t lb, uint32_t le,
                                                      const uint32_t* bits, uint32_t log2bits) {
    const uint32_t w[4] = {x.x, x.y, x.z, x.w};
    uint32_t c = 0;
#pragma unroll
    if (p >= lb && p + 4u <= le) {            // the whole word lies in the list
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t x32 = w[i] * 0x9E3779B1u;
            const uint32_t word = bits[x32 >> (37u - log2bits)];
            c += __funnelshift_r(word, word, x32 >> (32u - log2bits)) & 1u;
        }
        return c;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t x32 = w[i] * 0x9E3779B1u;
        const uint32_t word = bits[x32 >> (37u - log2bits)];
        const uint32_t b = __funnelshift_r(word, word, x32 >> (32u - log2bits)) & 1u;
        c += (p + i >= lb && p + i < le) ? b : 0u;
    }
    return c;
}

// |adj[b, e) ∩ list[0, dv)|, list sorted ascending: warp-wide, the result in every lane.
__device__ __forceinline__ uint32_t sorted_count(const uint32_t* list, uint32_t dv, const uint32_t* __restrict__ adj,
                                                 uint32_t b, uint32_t e, uint32_t lane) {
    uint32_t c = 0;
    for (uint32_t j = b + lane; j < e; j += 32) {
        const uint32_t w = __ldg(adj + j);
        uint32_t lo = 0, hi = dv;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (list[mid] < w) lo = mid + 1; else hi = mid;
        }
        c += (lo < dv && list[lo] == w) ? 1u : 0u;
    }
    return __reduce_add_sync(0xFFFFFFFFu, c);
}

// Shared memory of k_cn_filter for a class of up to `entries` pivot entries.
__host__ __device__ constexpr uint32_t filter_log2bits(uint32_t entries) {
    uint32_t l = 10;
    while ((1u << l) < 32u * entries) ++l;
    return l;
}
__host__ __device__ constexpr size_t filter_smem_bytes(uint32_t entries) {
    return (size_t(1) << filter_log2bits(entries)) / 8 + size_t(entries) * 4;
}

// list_entries: capacity of the shared sorted copy (pivots hold at most that many entries);
// the bitmap size follows from it in the kernel (R-MAT s22: passing the bit count as a
// kernel parameter instead measured 0.9 ms slower over the stage).
// strided: lane i of batch j takes edge e0 + j + i * nbatch instead of e0 + 32 j + i, so
// every batch samples the whole slice.  Lower edges are stored in id order, and a hub's
// expensive lower lists (those of high-degree neighbours, the ones the degree prune leaves)
// have low ids in R-MAT-like graphs: contiguous batches would hand them to a few warps while
// the rest finish the cheap batches and wait at the task barrier.
// Two entry points share the body: k_cn_filter_classes (hash classes) is launch-bounded to
// three 512-thread CTAs per SM, which holds it to 40 registers (R-MAT s22: the 4,096-entry
// class 4.67 -> 4.25 ms; two CTAs at 60 registers: slower again); k_cn_filter (mid hubs,
// held to two CTAs per SM by their 112 KB of shared memory) is left unbounded and streams
// three words per lane (64 registers; a bound measured slower there).
template <bool kPerGraph, int W>
__device__ __forceinline__ void cn_filter_body(const CnTask* __restrict__ tasks, uint32_t ntasks, uint32_t list_entries,
                            uint32_t* queue, const uint32_t* __restrict__ off,
                            const uint32_t* __restrict__ adj, const uint32_t* __restrict__ lo_adj,
                            uint32_t* __restrict__ cn, uint32_t long_words, CnPrune pr,
                            unsigned long long* __restrict__ ctr, FusedPred fp, uint32_t strided) {
    extern __shared__ __align__(16) uint32_t smem[];
    const uint32_t log2bits = filter_log2bits(list_entries);
    const uint32_t nwords = (1u << log2bits) >> 5;
    uint32_t* bits = smem;
    uint32_t* list = smem + nwords;
    __shared__ uint32_t next_batch, task_slot;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long nsim = 0, ndis = 0;
    for (uint32_t t = next_task(queue, 0, true, &task_slot); t < ntasks;
         t = next_task(queue, t, false, &task_slot)) {
        const CnTask tk = tasks[t];
        CnPrune Pg;
        if constexpr (kPerGraph) Pg = prune_of_graph(pr, tk.v);
        const CnPrune& P = kPerGraph ? Pg : pr;
        const uint32_t vb = off[tk.v], ve = off[tk.v + 1], dv = ve - vb;   // dv <= list_entries (no split)
        const PivotTests pt = pivot_tests(dv, P);
        for (uint32_t i = threadIdx.x; i < nwords / 4; i += blockDim.x)
            reinterpret_cast<uint4*>(bits)[i] = make_uint4(0, 0, 0, 0);
        if (threadIdx.x == 0) next_batch = 0;
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < dv; j += blockDim.x) {
            const uint32_t w = adj[vb + j];
            list[j] = w;
            const uint32_t h = filter_bit(w, log2bits);
            atomicOr(&bits[h >> 5], 1u << (h & 31u));
        }
        __syncthreads();
        for (;;) {
            uint32_t bidx = 0;
            if (lane == 0) bidx = atomicAdd(&next_batch, 1u);
            const uint32_t nbatch = (tk.e1 - tk.e0 + 31u) >> 5;
            const uint32_t j = __shfl_sync(0xFFFFFFFFu, bidx, 0);
            if (j >= nbatch) break;
            const uint32_t k = strided ? tk.e0 + j + lane * nbatch : tk.e0 + 32u * j + lane;
            const bool valid = k < tk.e1;
            uint32_t ub = 0, ue = 0, u = 0, du = 0, tlo = 0;
            bool pruned = false;
            if (valid) {
                u = lo_adj[k];
                ub = off[u];
                ue = off[u + 1];
                du = ue - ub;
                pruned = edge_pruned(du, pt);
                if (pruned) ue = ub;
                if (ue > ub) tlo = count_floor(du, dv, pt, P.eps);
            }
            // tlo = 0: any count may be similar, so the bound decides nothing; count exactly
            const bool bound_scan = ue > ub && tlo > 0;
            uint32_t words = 0;
            uint32_t cnt = count_batch<W>(adj, lane, ub, bound_scan ? ue : ub, tlo, long_words, words,
                                                       [&](uint4 x, uint32_t p, uint32_t lb, uint32_t le) {
                                                           return filter_probe_word(x, p, lb, le, bits, log2bits);
                                                       });
            uint32_t exact = __ballot_sync(0xFFFFFFFFu, ue > ub && cnt >= tlo);
            while (exact) {
                const int j = __ffs(exact) - 1;
                exact &= exact - 1;
                const uint32_t b = __shfl_sync(0xFFFFFFFFu, ub, j), e = __shfl_sync(0xFFFFFFFFu, ue, j);
                words += ((e + 3u) >> 2) - (b >> 2);
                const uint32_t c = sorted_count(list, dv, adj, b, e, lane);
                if ((int)lane == j) cnt = c;
            }
            const uint32_t nc = __popc(__ballot_sync(0xFFFFFFFFu, ue > ub));
            if (lane == 0 && (words | nc)) {
                atomicAdd(&ctr[0], (unsigned long long)words);
                atomicAdd(&ctr[1], (unsigned long long)nc);
            }
            if (valid) cn[k] = cnt;
            fused_predicate(fp, P, valid, pruned || cnt < tlo, k, u, tk.v, du, dv, cnt, lane, nsim, ndis);
        }
        __syncthreads();
    }
    fused_totals(fp, lane, nsim, ndis);
}


template <bool kPerGraph>
__global__ void __launch_bounds__(512, 3) k_cn_filter_classes(const CnTask* __restrict__ tasks, uint32_t ntasks, uint32_t list_entries,
                            uint32_t* queue, const uint32_t* __restrict__ off,
                            const uint32_t* __restrict__ adj, const uint32_t* __restrict__ lo_adj,
                            uint32_t* __restrict__ cn, uint32_t long_words, CnPrune pr,
                            unsigned long long* __restrict__ ctr, FusedPred fp, uint32_t strided) {
    cn_filter_body<kPerGraph, kWordsInFlight>(tasks, ntasks, list_entries, queue, off, adj, lo_adj, cn, long_words, pr, ctr, fp,
                              strided);
}

template <bool kPerGraph>
__global__ void k_cn_filter(const CnTask* __restrict__ tasks, uint32_t ntasks, uint32_t list_entries,
                            uint32_t* queue, const uint32_t* __restrict__ off,
                            const uint32_t* __restrict__ adj, const uint32_t* __restrict__ lo_adj,
                            uint32_t* __restrict__ cn, uint32_t long_words, CnPrune pr,
                            unsigned long long* __restrict__ ctr, FusedPred fp, uint32_t strided) {
    cn_filter_body<kPerGraph, kWordsInFlightMidHub>(tasks, ntasks, list_entries, queue, off, adj, lo_adj, cn, long_words, pr, ctr, fp,
                              strided);
}

// Bitmap path: one CTA of kBitmapThreads per task (pivot, edge slice), one CTA per SM.
// Shared memory: the hot bitmap (zeroed once; each task sets its pivot's bits and clears
// them again) and the tail table.  Probing an entry is one 4-byte shared load for hot ids.
__device__ __forceinline__ uint32_t bitmap_probe_word(const uint4 x, uint32_t p, uint32_t lb, uint32_t le,
                                                      const uint32_t* bits, const uint32_t* tail, uint32_t ntb) {
    const uint32_t w[4] = {x.x, x.y, x.z, x.w};
    uint32_t c = 0, tails = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t pos = p + i;
        if (pos >= lb && pos < le) {
            if (w[i] < kHotBits) c += (bits[w[i] >> 5] >> (w[i] & 31u)) & 1u;
            else tails |= 1u << i;
        }
    }
    while (tails) {
        const int i = __ffs(tails) - 1;
        tails &= tails - 1;
        c += bucket_has(tail, ntb, w[i]);
    }
    return c;
}

// task.cb carries the pivot's tail size.
template <bool kPerGraph>
__global__ void __launch_bounds__(kBitmapThreads, 1)
k_cn_bitmap(const CnTask* __restrict__ tasks, uint32_t ntasks, uint32_t* queue, const uint32_t* __restrict__ off,
            const uint32_t* __restrict__ radj, const uint32_t* __restrict__ lo_adj, uint32_t* __restrict__ cn,
            uint32_t long_words, CnPrune pr, unsigned long long* __restrict__ ctr, FusedPred fp,
            uint32_t strided) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* bits = smem;                              // kHotBits / 32 words
    uint32_t* tail = smem + kHotBits / 32;              // kTailSlots words
    __shared__ uint32_t next_batch, task_slot;
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long nsim = 0, ndis = 0;
    for (uint32_t i = threadIdx.x; i < kHotBits / 128; i += blockDim.x)
        reinterpret_cast<uint4*>(bits)[i] = make_uint4(0, 0, 0, 0);
    for (uint32_t t = next_task(queue, 0, true, &task_slot); t < ntasks;
         t = next_task(queue, t, false, &task_slot)) {
        const CnTask tk = tasks[t];
        CnPrune Pg;
        if constexpr (kPerGraph) Pg = prune_of_graph(pr, tk.v);
        const CnPrune& P = kPerGraph ? Pg : pr;
        const uint32_t vb = off[tk.v], ve = off[tk.v + 1];
        const PivotTests pt = pivot_tests(ve - vb, P);
        uint32_t ntb = 8;                                // tail buckets: >= tail size (load <= 1/4),
        while (ntb < tk.cb) ntb <<= 1;                   // capped at the table (load <= 1/2 there)
        ntb = min(ntb, kTailSlots / 4);
        for (uint32_t i = threadIdx.x; i < ntb; i += blockDim.x)
            reinterpret_cast<uint4*>(tail)[i] = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
        if (threadIdx.x == 0) next_batch = 0;
        __syncthreads();
        for (uint32_t j = vb + threadIdx.x; j < ve; j += blockDim.x) {
            const uint32_t w = radj[j];
            if (w < kHotBits) atomicOr(&bits[w >> 5], 1u << (w & 31u));
            else bucket_insert(tail, ntb, w);
        }
        __syncthreads();
        for (;;) {
            uint32_t bidx = 0;
            if (lane == 0) bidx = atomicAdd(&next_batch, 1u);
            const uint32_t nbatch = (tk.e1 - tk.e0 + 31u) >> 5;
            const uint32_t j = __shfl_sync(0xFFFFFFFFu, bidx, 0);
            if (j >= nbatch) break;
            // one-shot runs: strided, as k_cn_filter's hub launch; full counts (every edge
            // counted, no pruned majority): contiguous, measured faster
            const uint32_t k = strided ? tk.e0 + j + lane * nbatch : tk.e0 + 32u * j + lane;
            const bool valid = k < tk.e1;
            uint32_t ub = 0, ue = 0, u = 0, du = 0;
            bool pruned = false;
            if (valid) {
                u = lo_adj[k];
                ub = off[u];
                ue = off[u + 1];
                du = ue - ub;
                pruned = edge_pruned(du, pt);
                if (pruned) ue = ub;
            }
            const uint32_t tlo = (P.on && ue > ub) ? count_floor(du, ve - vb, pt, P.eps) : 0u;
            uint32_t words = 0;
            const uint32_t cnt = count_batch<kWordsInFlightBitmap>(radj, lane, ub, ue, tlo, long_words, words,
                                                                   [&](uint4 x, uint32_t p, uint32_t lb, uint32_t le) {
                                                                       return bitmap_probe_word(x, p, lb, le, bits,
                                                                                                tail, ntb);
                                                                   });
            const uint32_t nc = __popc(__ballot_sync(0xFFFFFFFFu, ue > ub));
            if (lane == 0 && (words | nc)) {
                atomicAdd(&ctr[0], (unsigned long long)words);
                atomicAdd(&ctr[1], (unsigned long long)nc);
            }
            if (valid) cn[k] = cnt;
            if (fp.sim) fused_predicate(fp, P, valid, pruned || cnt < tlo, k, u, tk.v, du, ve - vb, cnt, lane, nsim, ndis);
        }
        __syncthreads();
        for (uint32_t j = vb + threadIdx.x; j < ve; j += blockDim.x) {   // clear this pivot's bits
            const uint32_t w = radj[j];
            if (w < kHotBits) bits[w >> 5] = 0u;
        }
        __syncthreads();
    }
    fused_totals(fp, lane, nsim, ndis);
}

// Task planner.  Pass 1 (outputs null) counts tasks per class; pass 2 writes them.
// counts[0] small pivots, counts[1 + c] tasks of hash class c, counts[4] bitmap tasks of
// hubs above kHubFilterMax, counts[5] bitmap tasks of the mid hubs, counts[6] (pass 1 only)
// pivots split into chunks.
// tail (may be null: bitmap path off) holds each vertex's count of non-hot neighbours.
// (PlanParams: device_graph.h.)

__global__ void k_plan(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ lo_off,
                       const unsigned long long* __restrict__ work, const uint32_t* __restrict__ tail,
                       PlanParams pp, uint32_t* __restrict__ counts, uint32_t* __restrict__ small_out,
                       CnTask* __restrict__ big0, CnTask* __restrict__ big1, CnTask* __restrict__ big2,
                       CnTask* __restrict__ bmp, CnTask* __restrict__ hmid) {
    constexpr int kClasses = 3 + kNumBigClasses;   // small, hash classes, big hubs, mid hubs
    __shared__ uint32_t blk[kClasses];
    __shared__ uint32_t base[kClasses];
    if (threadIdx.x < kClasses) blk[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    int cls = -1;
    uint32_t ntask = 0, nch = 0, nsl = 0, L = 0, dv = 0;
    if (v < n) {
        L = lo_off[v + 1] - lo_off[v];
        dv = off[v + 1] - off[v];
        if (L > 0) {
            if (dv <= pp.small_deg) {
                cls = 0;
                ntask = 1;
            } else if (tail && dv > pp.bitmap_min_deg && tail[v] <= kTailMax) {
                cls = dv <= kHubFilterMax ? 2 + kNumBigClasses : 1 + kNumBigClasses;
                nch = 1;
                unsigned long long s = (work[v] + pp.target_probes_bitmap - 1) / pp.target_probes_bitmap;
                const uint32_t smax = (L + pp.min_slice_edges - 1) / pp.min_slice_edges;
                nsl = (uint32_t)(s < 1 ? 1 : (s > smax ? smax : s));
                ntask = nsl;
            } else {
                nch = (dv + pp.chunk_max - 1) / pp.chunk_max;
                const uint32_t ce = (dv + nch - 1) / nch;
                cls = 1 + (ce <= big_class_entries(0) ? 0 : ce <= big_class_entries(1) ? 1 : 2);
                unsigned long long w = work[v] / nch;   // probes per chunk (ids spread evenly)
                unsigned long long s = (w + pp.target_probes - 1) / pp.target_probes;
                const uint32_t smax = (L + pp.min_slice_edges - 1) / pp.min_slice_edges;
                nsl = (uint32_t)(s < 1 ? 1 : (s > smax ? smax : s));
                ntask = nch * nsl;
                if (nch > 1 && small_out == nullptr) {
                    atomicAdd(&counts[kClasses], 1u);       // split pivots
                    atomicAdd(&counts[kClasses + 1], L);    // ... and their lower edges (miss counters)
                }
            }
        }
    }
    uint32_t mine = 0;
    if (cls >= 0) mine = atomicAdd(&blk[cls], ntask);
    __syncthreads();
    if (threadIdx.x < kClasses) base[threadIdx.x] = atomicAdd(&counts[threadIdx.x], blk[threadIdx.x]);
    __syncthreads();
    if (cls < 0 || (small_out == nullptr)) return;
    const uint32_t pos = base[cls] + mine;
    if (cls == 0) {
        small_out[pos] = v;
        return;
    }
    CnTask* out = cls == 1 ? big0 : cls == 2 ? big1 : cls == 3 ? big2 : cls == 4 ? bmp : hmid;
    const uint32_t vb = off[v], e0 = lo_off[v];
    const uint32_t mbase = nch > 1 ? atomicAdd(&counts[kClasses + 1], L) : 0u;   // this pivot's miss counters
    uint32_t i = 0;
    for (uint32_t c = 0; c < nch; ++c) {
        const uint32_t cb = vb + (uint32_t)((uint64_t)dv * c / nch);
        const uint32_t cend = vb + (uint32_t)((uint64_t)dv * (c + 1) / nch);
        for (uint32_t s = 0; s < nsl; ++s, ++i) {
            CnTask t;
            t.v = v;
            t.cb = cls >= 1 + kNumBigClasses ? tail[v] : cb;
            t.ce = cend;
            t.e0 = e0 + (uint32_t)((uint64_t)L * s / nsl);
            t.e1 = e0 + (uint32_t)((uint64_t)L * (s + 1) / nsl);
            t.chunked = nch > 1;
            t.mofs = mbase - e0;
            t.pad1 = 0;
            out[pos + i] = t;
        }
    }
}

}  // namespace scan
