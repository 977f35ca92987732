// From common-neighbour counts to clusters: predicate, cores, union-find, attachment,
// hub/outlier classification.  All passes are edge-parallel over the E undirected edges
// (lo_adj/lo_src) or vertex-parallel; per-vertex arrays (n x 4 B) stay L2-resident.
#pragma once

#include "device_common.cuh"
#include "predicate.cuh"

namespace scan {

// sim[e] and the similar-degree count sd[] of both endpoints (core rule: a vertex is a
// core when at least mu of its neighbours are similar, GPUSCAN++/GPUScan.cu:147-165).
// Edges of one pivot are contiguous, so the pivot side is summed per warp segment.
// Batched runs (many graphs as one disjoint union) pass vgid[] (graph of each vertex) and
// per-graph parameters gpp[]; single runs pass null and use pp.
__global__ void k_predicate(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                            const uint32_t* __restrict__ off, const uint32_t* __restrict__ cn, PredParams pp,
                            const uint32_t* __restrict__ vgid, const PredParams* __restrict__ gpp,
                            uint8_t* __restrict__ sim, int32_t* __restrict__ sd, RunCounters* __restrict__ ctr) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long nsim = 0, ndis = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e0 = (uint64_t)blockIdx.x * blockDim.x; e0 < E; e0 += stride) {
        const uint64_t e = e0 + threadIdx.x;
        bool s = false;
        uint32_t v = kEmpty;
        if (e < E) {
            const uint32_t u = lo_adj[e];
            v = lo_src[e];
            const uint32_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v];
            const uint32_t t = cn[e];
            const PredParams P = vgid ? gpp[vgid[u]] : pp;
            const bool r = ref_f64_similar(t, du, dv, P.eps);
            const bool x = exact_similar(t, du, dv, P.p, P.q);
            s = P.mode ? r : x;
            ndis += (r != x);
            nsim += s;
            sim[e] = s;
            if (s) atomicAdd(&sd[u], 1);
        }
        // pivot side: one atomic per run of equal pivots within the warp
        const uint32_t key = s ? v : kEmpty;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (s && (__ffs(peers) - 1) == (int)lane) atomicAdd(&sd[v], __popc(peers));
    }
    for (int o = 16; o > 0; o >>= 1) {
        nsim += __shfl_xor_sync(0xFFFFFFFFu, nsim, o);
        ndis += __shfl_xor_sync(0xFFFFFFFFu, ndis, o);
    }
    if (lane == 0) {
        if (nsim) atomicAdd(&ctr->similar_edges, nsim);
        if (ndis) atomicAdd(&ctr->disagreements, ndis);
    }
}

// Served queries on cached counts: each edge's similarity threshold, precomputed once per
// graph, so the predicate is one compare per edge.  Edge e is similar at eps exactly when
// eps^2 <= tau(e): tau_x = (t+2)^2 / ((du+1)(dv+1)) for the exact test, tau_r =
// min((du+1)/(dv+1), max(4, t2)/((du+1)(dv+1))) for the reference's doubles: its 'N' prune,
// then its 'Y' prune or its intersect test (t2 the int square, which can wrap negative; the
// 'Y' threshold 4/((du+1)(dv+1)) still holds then).  Both are monotone in eps because IEEE
// products are.  Stored as floats; an edge whose tau lies within a relative kTauBand of
// eps^2 (float rounding is 6e-8) is decided by the predicate itself.
constexpr double kTauBand = 1e-6;

__global__ void k_tau(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                      const uint32_t* __restrict__ off, const uint32_t* __restrict__ cn, float* __restrict__ tau) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t u = lo_adj[e], v = lo_src[e];
        const uint32_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v], t = cn[e];
        const double du1 = (double)(du + 1u), dv1 = (double)(dv + 1u);
        const double a = (double)(t + 2u);
        tau[e] = (float)(a * a / (du1 * dv1));
        const int32_t t2 = (int32_t)((t + 2u) * (t + 2u));
        tau[E + e] = (float)fmin(du1 / dv1, fmax(4.0, (double)t2) / (du1 * dv1));
    }
}

// k_predicate for a served graph: the cached thresholds decide every edge outside the
// band; the disagreement counter is not kept (the server does not report it).
__global__ void k_predicate_tau(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                                const uint32_t* __restrict__ off, const uint32_t* __restrict__ cn,
                                const float* __restrict__ tau, PredParams pp, uint8_t* __restrict__ sim,
                                int32_t* __restrict__ sd, RunCounters* __restrict__ ctr) {
    const uint32_t lane = threadIdx.x & 31;
    const float* tm = tau + (pp.mode ? E : 0);
    double theta;
    if (pp.mode) theta = pp.eps * pp.eps;
    else theta = pp.q == 0 ? 2.0 : ((double)pp.p / (double)pp.q) * ((double)pp.p / (double)pp.q);
    const double hi = theta * (1.0 + kTauBand), lo = theta * (1.0 - kTauBand);
    unsigned long long nsim = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e0 = (uint64_t)blockIdx.x * blockDim.x; e0 < E; e0 += stride) {
        const uint64_t e = e0 + threadIdx.x;
        bool s = false;
        uint32_t v = kEmpty;
        if (e < E) {
            const double tv = (double)tm[e];
            if (tv >= hi) {
                s = true;
            } else if (tv > lo || (theta == 0.0 && tv == 0.0)) {
                const uint32_t u = lo_adj[e], w = lo_src[e];
                const uint32_t du = off[u + 1] - off[u], dw = off[w + 1] - off[w];
                s = pp.mode ? ref_f64_similar(cn[e], du, dw, pp.eps) : exact_similar(cn[e], du, dw, pp.p, pp.q);
            }
            sim[e] = s;
            if (s) {
                v = lo_src[e];
                atomicAdd(&sd[lo_adj[e]], 1);
                ++nsim;
            }
        }
        const uint32_t key = s ? v : kEmpty;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        if (s && (__ffs(peers) - 1) == (int)lane) atomicAdd(&sd[v], __popc(peers));
    }
    for (int o = 16; o > 0; o >>= 1) nsim += __shfl_xor_sync(0xFFFFFFFFu, nsim, o);
    if (lane == 0 && nsim) atomicAdd(&ctr->similar_edges, nsim);
}

// parent[v] = v for cores, -1 otherwise; border/neighbour label ranges reset.  Batched
// runs pass vgid[] and per-graph gmu[].
__global__ void k_core_init(uint32_t n, const int32_t* __restrict__ sd, int mu, const uint32_t* __restrict__ vgid,
                            const int32_t* __restrict__ gmu, int32_t* __restrict__ parent, int32_t* __restrict__ bmin,
                            int32_t* __restrict__ bmax, int32_t* __restrict__ nmin, int32_t* __restrict__ nmax,
                            RunCounters* __restrict__ ctr) {
    bool core = false;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const int m = vgid ? gmu[vgid[v]] : mu;
        const bool c = sd[v] >= m;
        core |= c;
        parent[v] = c ? (int32_t)v : -1;
        bmin[v] = 0x7FFFFFFF;
        bmax[v] = -1;
        nmin[v] = 0x7FFFFFFF;
        nmax[v] = -1;
    }
    if (__any_sync(0xFFFFFFFFu, core) && (threadIdx.x & 31) == 0) atomicOr(&ctr->any_core, 1u);
}

// Root of x with path halving.  parent[y] < y for every non-root y, so every write keeps
// the forest acyclic and the walk terminates.
__device__ __forceinline__ int32_t uf_find(volatile int32_t* parent, int32_t x) {
    int32_t p = parent[x];
    while (p != x) {
        const int32_t g = parent[p];
        if (g != p) parent[x] = g;
        x = p;
        p = g;
    }
    return x;
}

// Lock-free union by smaller root id: the root of a component is its smallest core id,
// which is the reference's cluster id (GPUSCAN++/GPUScan.cu:500-523 hooks the larger
// root under the smaller one).  At most `limit` CAS attempts; false if they all lost.
__device__ __forceinline__ bool uf_union(int32_t* parent, int32_t a, int32_t b, uint32_t limit) {
    volatile int32_t* vp = parent;
    for (uint32_t it = 0; it < limit; ++it) {
        a = uf_find(vp, a);
        b = uf_find(vp, b);
        if (a == b) return true;
        if (a < b) { const int32_t t = a; a = b; b = t; }   // a > b: hang a under b
        if (atomicCAS(&parent[a], a, b) == a) return true;
    }
    return false;
}

__global__ void k_union(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                        const uint8_t* __restrict__ sim, int32_t* parent, RunCounters* ctr, uint32_t limit) {
    if (!*(volatile uint32_t*)&ctr->any_core) return;   // no core: nothing to join
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        if (!sim[e]) continue;
        const int32_t u = (int32_t)lo_adj[e], v = (int32_t)lo_src[e];
        if (parent[u] < 0 || parent[v] < 0) continue;   // core-core only (cores never change)
        if (!uf_union(parent, u, v, limit)) atomicOr(&ctr->error_flags, kErrUnionFindLimit);
    }
}

// Flatten by pointer jumping: round r sets parent[v] = parent[parent[v]] for every core and
// raises flags[r] if any pointer moved.  The host queues enough rounds for any depth
// (ceil(log2 n) + 2); a round whose predecessor moved nothing returns at once, so the pass
// needs no host synchronisation.  Every value stored is an ancestor of v in the final
// forest and only v's own thread writes parent[v], so concurrent jumps never undo one
// another.  (A find with path halving would not be safe here: its halving store can
// overwrite a vertex whose root another thread has just written with an intermediate
// ancestor.)
__global__ void k_jump_round(uint32_t n, int32_t* parent, uint32_t* flags, uint32_t round) {
    if (round > 0 && *(volatile uint32_t*)&flags[round - 1] == 0) return;
    volatile int32_t* vp = parent;
    uint32_t ch = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t p = vp[v];
        if (p < 0) continue;
        const int32_t g = vp[p];
        if (g != p) {
            vp[v] = g;
            ch = 1;
        }
    }
    if (__any_sync(0xFFFFFFFFu, ch) && (threadIdx.x & 31) == 0) atomicOr(&flags[round], 1u);
}

// The same rounds in one CTA, for graphs of up to kJumpBlockMax vertices: a block barrier
// separates the rounds, so one launch replaces the chain of k_jump_round launches (the
// launch count matters for the many small queries of the serving loop).  flags follow the
// chain's convention: flags[i] != 0 when round i moved a pointer, so flags[rounds - 1] == 0
// means converged.
constexpr uint32_t kJumpBlockMax = 1u << 16;

__global__ void __launch_bounds__(1024) k_jump_block(uint32_t n, int32_t* parent, uint32_t* flags, uint32_t rounds) {
    volatile int32_t* vp = parent;
    for (uint32_t round = 0; round < rounds; ++round) {
        int ch = 0;
        for (uint32_t v = threadIdx.x; v < n; v += blockDim.x) {
            const int32_t p = vp[v];
            if (p < 0) continue;
            const int32_t g = vp[p];
            if (g != p) {
                vp[v] = g;
                ch = 1;
            }
        }
        ch = __syncthreads_or(ch);
        if (threadIdx.x == 0) flags[round] = ch ? 1u : 0u;
        if (!ch) break;
    }
}

// Zeroes a run's similar-degree counts (sd may be null: already done), counters and
// round flags in one launch.
__global__ void k_cluster_reset(uint32_t n, int32_t* sd, RunCounters* ctr, uint32_t* flags, uint32_t nflags) {
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if (sd)
        for (uint64_t v = i0; v < n; v += stride) sd[v] = 0;
    if (i0 < nflags) flags[i0] = 0;
    if (ctr && i0 == 0) *ctr = RunCounters{};
}

// Border attachment: a non-core similar to a core joins that core's cluster.  The
// reference keeps the last write among several clusters (GPUSCAN++/GPUScan.cu:716,722);
// here the smallest cluster id wins, and bmin != bmax marks a multi-cluster border.
__global__ void k_attach(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                         const uint8_t* __restrict__ sim, const int32_t* __restrict__ parent,
                         int32_t* __restrict__ bmin, int32_t* __restrict__ bmax, const RunCounters* ctr) {
    if (!*(const volatile uint32_t*)&ctr->any_core) return;   // no core: no border
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        if (!sim[e]) continue;
        const uint32_t u = lo_adj[e], v = lo_src[e];
        const int32_t pu = parent[u], pv = parent[v];
        if (pu >= 0 && pv < 0) { atomicMin(&bmin[v], pu); atomicMax(&bmax[v], pu); }
        else if (pv >= 0 && pu < 0) { atomicMin(&bmin[u], pv); atomicMax(&bmax[u], pv); }
    }
}

// Label after attachment: cluster id for cores and borders, -2 for the rest.
__global__ void k_label(uint32_t n, const int32_t* __restrict__ parent, const int32_t* __restrict__ bmin,
                        int32_t* __restrict__ lab, RunCounters* __restrict__ ctr) {
    bool member = false;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t p = parent[v];
        const int32_t l = p >= 0 ? p : (bmin[v] != 0x7FFFFFFF ? bmin[v] : -2);
        lab[v] = l;
        member |= l >= 0;
    }
    if (__any_sync(0xFFFFFFFFu, member) && (threadIdx.x & 31) == 0) atomicOr(&ctr->any_member, 1u);
}

// Hub test inputs: for each unlabelled vertex, the smallest and largest label among its
// neighbours.  Two distinct labels make it a hub (GPUSCAN++/GPUScan.cu:757-780 looks for a
// second neighbour label different from the first).
__global__ void k_neighbour_labels(uint64_t E, const uint32_t* __restrict__ lo_adj,
                                   const uint32_t* __restrict__ lo_src, const int32_t* __restrict__ lab,
                                   int32_t* __restrict__ nmin, int32_t* __restrict__ nmax, const RunCounters* ctr) {
    if (!*(const volatile uint32_t*)&ctr->any_member) return;   // no cluster: every other vertex is an outlier
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t u = lo_adj[e], v = lo_src[e];
        const int32_t lu = lab[u], lv = lab[v];
        if (lu < 0 && lv >= 0) { atomicMin(&nmin[u], lv); atomicMax(&nmax[u], lv); }
        else if (lv < 0 && lu >= 0) { atomicMin(&nmin[v], lu); atomicMax(&nmax[v], lu); }
    }
}

// Final labels, roles and counters.
__global__ void k_finalize(uint32_t n, const int32_t* __restrict__ parent, const int32_t* __restrict__ bmin,
                           const int32_t* __restrict__ bmax, const int32_t* __restrict__ nmin,
                           const int32_t* __restrict__ nmax, int32_t* __restrict__ label,
                           uint8_t* __restrict__ role, RunCounters* __restrict__ ctr) {
    unsigned long long c_core = 0, c_clu = 0, c_hub = 0, c_out = 0, c_bor = 0, c_multi = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t p = parent[v];
        int32_t l;
        uint8_t r;
        if (p >= 0) {
            l = p; r = kRoleCore; ++c_core; c_clu += (p == (int32_t)v);
        } else if (bmin[v] != 0x7FFFFFFF) {
            l = bmin[v]; r = kRoleBorder; ++c_bor; c_multi += (bmin[v] != bmax[v]);
        } else if (nmin[v] < nmax[v]) {
            l = -1; r = kRoleHub; ++c_hub;
        } else {
            l = -2; r = kRoleOutlier; ++c_out;
        }
        label[v] = l;
        if (role) role[v] = r;
    }
    for (int o = 16; o > 0; o >>= 1) {
        c_core += __shfl_xor_sync(0xFFFFFFFFu, c_core, o);
        c_clu += __shfl_xor_sync(0xFFFFFFFFu, c_clu, o);
        c_hub += __shfl_xor_sync(0xFFFFFFFFu, c_hub, o);
        c_out += __shfl_xor_sync(0xFFFFFFFFu, c_out, o);
        c_bor += __shfl_xor_sync(0xFFFFFFFFu, c_bor, o);
        c_multi += __shfl_xor_sync(0xFFFFFFFFu, c_multi, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c_core) atomicAdd(&ctr->cores, c_core);
        if (c_clu) atomicAdd(&ctr->clusters, c_clu);
        if (c_hub) atomicAdd(&ctr->hubs, c_hub);
        if (c_out) atomicAdd(&ctr->outliers, c_out);
        if (c_bor) atomicAdd(&ctr->borders, c_bor);
        if (c_multi) atomicAdd(&ctr->multi_borders, c_multi);
    }
}

// Memberships: every (cluster, border) pair from similar core-border edges.
__global__ void k_border_pairs(uint64_t E, const uint32_t* __restrict__ lo_adj, const uint32_t* __restrict__ lo_src,
                               const uint8_t* __restrict__ sim, const int32_t* __restrict__ parent,
                               unsigned long long* __restrict__ count, unsigned long long* __restrict__ out,
                               unsigned long long cap) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        if (!sim[e]) continue;
        const uint32_t u = lo_adj[e], v = lo_src[e];
        const int32_t pu = parent[u], pv = parent[v];
        unsigned long long key;
        if (pu >= 0 && pv < 0) key = ((unsigned long long)(uint32_t)pu << 32) | v;
        else if (pv >= 0 && pu < 0) key = ((unsigned long long)(uint32_t)pv << 32) | u;
        else continue;
        const unsigned long long i = atomicAdd(count, 1ull);
        if (i < cap) out[i] = key;
    }
}

}  // namespace scan
