/*
 * scan_oracle.c -- CPU restatement of GPUSCAN++'s SCAN semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle for the CUDA engine: only tests/,
 * __graft_entry__.smoke(), bench.py's CPU-baseline leg and bench.py's CPU reference arm load
 * it, always as the checker or the CPU baseline.  The product library (libscan_gb300.so)
 * never links, loads or calls it.
 *
 * Pinning: the reference ships no tests or golden vectors.  This restatement is pinned
 * (a) against the reference's own host orientation (GPUSCAN++/Graph.cpp:52-141, compiled
 *     from the reference sources by oracle/build.py) on the CPU, and
 * (b) against the reference's own kernels (GPUSCAN++/GPUScan.cu, compiled to a cubin by
 *     oracle/build.py and driven in the reference's launch order by
 *     oracle/ref_harness.cu) on the GPU.
 *
 * Semantics restated (reference file:line):
 *   orientation   lower/higher endpoint by (degree, id)          GPUSCAN++/Graph.cpp:66-111
 *   count         T = |N(u) ∩ N(v)| (open neighbourhoods)         GPUSCAN++/GPUScan.cu:174-219
 *   predicate     ref-f64: 'N' prune :145, 'Y' prune :156, test :220-221 (int (T+2)^2)
 *                 exact:   (T+2)^2 q^2 >= p^2 (du+1)(dv+1), eps = p/q
 *   core          #similar neighbours >= mu                       GPUSCAN++/GPUScan.cu:122-128,147-165,319-361
 *   clusters      components of core-core similar edges, id = smallest core id
 *                                                                  GPUSCAN++/GPUScan.cu:479-652
 *   borders       non-core similar to a core takes that core's cluster; of several, the
 *                 smallest id (the reference keeps the last write)  GPUSCAN++/GPUScan.cu:654-730
 *   hub/outlier   unattached vertex whose labelled neighbours carry >= 2 distinct labels
 *                 is a hub (-1), else an outlier (-2)              GPUSCAN++/GPUScan.cu:732-798
 * The intersection here is a two-pointer merge, or a binary search of the shorter list in
 * the longer one for skewed pairs (both different methods from the engine's shared-memory
 * hash probes), over OpenMP threads when available.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

static inline uint64_t deg_of(const uint64_t* off, uint64_t v) { return off[v + 1] - off[v]; }

/* u precedes v: smaller degree, ties by smaller id (GPUSCAN++/Graph.cpp:75-83). */
static inline int precedes(const uint64_t* off, uint32_t u, uint32_t v) {
    uint64_t du = deg_of(off, u), dv = deg_of(off, v);
    return du < dv || (du == dv && u < v);
}

/* Reference edge order (GPUSCAN++/Graph.cpp:66-111): ids grouped by the lower endpoint in
 * vertex order, then by the higher endpoint's position in the lower endpoint's list.
 * Writes edge_u/edge_v (E entries each); returns E, or -1 if the graph is not symmetric. */
ORACLE_API int64_t oracle_orient(uint64_t n, const uint64_t* off, const uint32_t* adj, uint32_t* edge_u,
                                 uint32_t* edge_v) {
    uint64_t e = 0;
    for (uint64_t u = 0; u < n; ++u) {
        for (uint64_t j = off[u]; j < off[u + 1]; ++j) {
            uint32_t v = adj[j];
            if (precedes(off, (uint32_t)u, v)) {
                edge_u[e] = (uint32_t)u;
                edge_v[e] = v;
                ++e;
            }
        }
    }
    if (2 * e != off[n]) return -1;
    return (int64_t)e;
}

/* |N(u) ∩ N(v)| of two sorted lists.  Lists of similar length: a two-pointer merge.  When
 * one list is more than 16 times longer, each entry of the shorter one is binary-searched in
 * the longer one, as the reference's intersect does (GPUSCAN++/GPUScan.cu:174-222); the
 * search window starts after the previous hit position, since both lists ascend. */
static inline uint32_t merge_count(const uint64_t* off, const uint32_t* adj, uint32_t u, uint32_t v) {
    uint64_t i = off[u], ie = off[u + 1], j = off[v], je = off[v + 1];
    uint32_t c = 0;
    if (ie - i > 16 * (je - j) || je - j > 16 * (ie - i)) {
        if (ie - i > je - j) { uint64_t t = i; i = j; j = t; t = ie; ie = je; je = t; }
        for (; i < ie && j < je; ++i) {
            const uint32_t x = adj[i];
            uint64_t lo = j, hi = je;
            while (lo < hi) {
                const uint64_t mid = lo + (hi - lo) / 2;
                if (adj[mid] < x) lo = mid + 1; else hi = mid;
            }
            j = lo;
            if (j < je && adj[j] == x) { ++c; ++j; }
        }
        return c;
    }
    while (i < ie && j < je) {          /* branch-free step: advance the smaller side (both on a hit) */
        const uint32_t a = adj[i], b = adj[j];
        c += a == b;
        i += a <= b;
        j += b <= a;
    }
    return c;
}

/* cn[e] for the E edges (edge_u[e], edge_v[e]). */
ORACLE_API void oracle_common_neighbors(const uint64_t* off, const uint32_t* adj, uint64_t E,
                                        const uint32_t* edge_u, const uint32_t* edge_v, uint32_t* cn) {
    int64_t i;
#pragma omp parallel for schedule(dynamic, 256)
    for (i = 0; i < (int64_t)E; ++i) cn[i] = merge_count(off, adj, edge_u[i], edge_v[i]);
}

/* ref-f64 predicate, operand order of GPUSCAN++/GPUScan.cu:145,156,220-221. */
ORACLE_API int oracle_ref_f64_similar(uint32_t t, uint32_t du, uint32_t dv, double eps) {
    double deg_u = (double)(du + 1u), deg_v = (double)(dv + 1u);
    if (deg_u < deg_v * eps * eps) return 0;                 /* 'N' */
    if (eps * eps * deg_u * deg_v <= 4.0) return 1;          /* 'Y' */
    int32_t sq = (int32_t)((t + 2u) * (t + 2u));             /* int product, wraps */
    return !((double)sq < eps * eps * (double)(int32_t)(du + 1u) * (double)(int32_t)(dv + 1u));
}

/* exact predicate: (t+2)^2 q^2 >= p^2 (du+1)(dv+1), p <= q <= 2^30; eps > 1 never holds. */
ORACLE_API int oracle_exact_similar(uint32_t t, uint32_t du, uint32_t dv, uint64_t p, uint64_t q) {
    if (p > q) return 0;
    unsigned __int128 a = (unsigned __int128)(t + 2ull) * q;
    unsigned __int128 lhs = a * a;
    unsigned __int128 rhs = (unsigned __int128)(p * p) * ((unsigned __int128)(du + 1ull) * (dv + 1ull));
    return lhs >= rhs;
}

static int32_t uf_root(int32_t* parent, int32_t x) {
    while (parent[x] != x) {
        parent[x] = parent[parent[x]];
        x = parent[x];
    }
    return x;
}

/* The reference's 'N' degree prune (GPUSCAN++/GPUScan.cu:145, in __prep_edge): with the
 * lower endpoint's degree du, deg_u < deg_v*eps*eps marks the edge not similar before any
 * intersection.  The exact counterpart, (du+1) q^2 < p^2 (dv+1), holds exactly when no count
 * can pass the exact test (T <= du - 1, so (T+2)^2 <= (du+1)^2).  An edge for which both
 * hold is rejected by both predicates whatever its count. */
static int pruned_both(uint32_t du, uint32_t dv, double eps, uint64_t p, uint64_t q) {
    double deg_u = (double)(du + 1u), deg_v = (double)(dv + 1u);
    if (!(deg_u < deg_v * eps * eps)) return 0;
    if (p > q) return 1;                                   /* eps > 1: exact never holds */
    return (unsigned __int128)(du + 1ull) * ((unsigned __int128)q * q) <
           (unsigned __int128)(p * p) * (dv + 1ull);
}

#define ORACLE_PRUNE 1u

/* cn of the edges e = stripe, stripe + nstripes, ... (the reference edge order given by
 * edge_u/edge_v), with the degree prune when flags & ORACLE_PRUNE (pruned edges get 0).
 * The stripes of one nstripes together cover every edge once, so a caller can split one
 * pass into bounded steps and finish it with oracle_scan_ex(cn_in = cn). */
ORACLE_API void oracle_count_stripe(const uint64_t* off, const uint32_t* adj, uint64_t E, const uint32_t* edge_u,
                                    const uint32_t* edge_v, uint64_t stripe, uint64_t nstripes, double eps,
                                    uint64_t p, uint64_t q, unsigned flags, uint32_t* cn) {
    if (nstripes == 0 || stripe >= nstripes || stripe >= E) return;
    const int64_t k = (int64_t)((E - 1 - stripe) / nstripes + 1);
    int64_t i;
#pragma omp parallel for schedule(dynamic, 256)
    for (i = 0; i < k; ++i) {
        const uint64_t e = stripe + (uint64_t)i * nstripes;
        const uint32_t u = edge_u[e], v = edge_v[e];
        cn[e] = (flags & ORACLE_PRUNE) && pruned_both((uint32_t)deg_of(off, u), (uint32_t)deg_of(off, v), eps, p, q)
                    ? 0u : merge_count(off, adj, u, v);
    }
}

/* Full SCAN.  mode 0 = exact (p/q), 1 = ref-f64 (eps).  Outputs label[n] (cluster id /
 * -1 hub / -2 outlier) and role[n] (0 outlier, 1 hub, 2 border, 3 core).
 * flags & ORACLE_PRUNE: edges both predicates reject by degree alone (pruned_both, the
 * reference's __prep_edge 'N' prune) are not intersected; their cn is left 0, which both
 * predicates reject too, so labels, roles and counts are unchanged.
 * cn_in (may be NULL): cn of every edge in the reference edge order, used instead of
 * intersecting.  cn_out (may be NULL) receives the counts used (0 for pruned edges).
 * counts (may be NULL) receives
 * {cores, clusters, borders, hubs, outliers, similar_edges, disagreements, multi_borders}.
 * Returns 0, or -1 on allocation failure / asymmetric input. */
ORACLE_API int oracle_scan_ex(uint64_t n, const uint64_t* off, const uint32_t* adj, int mode, double eps,
                              uint64_t p, uint64_t q, int mu, unsigned flags, const uint32_t* cn_in, int32_t* label,
                              uint8_t* role, uint32_t* cn_out, uint64_t* counts) {
    uint64_t E = off[n] / 2;
    uint32_t* eu = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* ev = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* cn = cn_out ? cn_out : (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint8_t* sim = (uint8_t*)malloc(E ? E : 1);
    int32_t* sd = (int32_t*)calloc(n, sizeof(int32_t));
    int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * n);
    int32_t* bmin = (int32_t*)malloc(sizeof(int32_t) * n);
    int32_t* bmax = (int32_t*)malloc(sizeof(int32_t) * n);
    int32_t* nmin = (int32_t*)malloc(sizeof(int32_t) * n);
    int32_t* nmax = (int32_t*)malloc(sizeof(int32_t) * n);
    int rc = -1;
    uint64_t c_sim = 0, c_dis = 0;
    if (!eu || !ev || !cn || !sim || !sd || !parent || !bmin || !bmax || !nmin || !nmax) goto done;
    if (oracle_orient(n, off, adj, eu, ev) < 0) goto done;
    if (cn_in) {
        memcpy(cn, cn_in, sizeof(uint32_t) * E);
    } else if (flags & ORACLE_PRUNE) {
        int64_t i;
#pragma omp parallel for schedule(dynamic, 256)
        for (i = 0; i < (int64_t)E; ++i)
            cn[i] = pruned_both((uint32_t)deg_of(off, eu[i]), (uint32_t)deg_of(off, ev[i]), eps, p, q)
                        ? 0u : merge_count(off, adj, eu[i], ev[i]);
    } else {
        oracle_common_neighbors(off, adj, E, eu, ev, cn);
    }
    for (uint64_t e = 0; e < E; ++e) {
        uint32_t du = (uint32_t)deg_of(off, eu[e]), dv = (uint32_t)deg_of(off, ev[e]);
        int r = oracle_ref_f64_similar(cn[e], du, dv, eps);
        int x = oracle_exact_similar(cn[e], du, dv, p, q);
        int s = mode ? r : x;
        c_dis += (r != x);
        c_sim += s;
        sim[e] = (uint8_t)s;
        if (s) { sd[eu[e]]++; sd[ev[e]]++; }
    }
    for (uint64_t v = 0; v < n; ++v) {
        parent[v] = sd[v] >= mu ? (int32_t)v : -1;
        bmin[v] = INT32_MAX; bmax[v] = -1; nmin[v] = INT32_MAX; nmax[v] = -1;
    }
    for (uint64_t e = 0; e < E; ++e) {
        if (!sim[e] || parent[eu[e]] < 0 || parent[ev[e]] < 0) continue;
        int32_t a = uf_root(parent, (int32_t)eu[e]), b = uf_root(parent, (int32_t)ev[e]);
        if (a == b) continue;
        if (a < b) parent[b] = a; else parent[a] = b;   /* root stays the smallest id */
    }
    for (uint64_t v = 0; v < n; ++v)
        if (parent[v] >= 0) parent[v] = uf_root(parent, (int32_t)v);
    for (uint64_t e = 0; e < E; ++e) {
        if (!sim[e]) continue;
        int32_t pu = parent[eu[e]], pv = parent[ev[e]];
        uint32_t x;
        int32_t c;
        if (pu >= 0 && pv < 0) { x = ev[e]; c = pu; }
        else if (pv >= 0 && pu < 0) { x = eu[e]; c = pv; }
        else continue;
        if (c < bmin[x]) bmin[x] = c;
        if (c > bmax[x]) bmax[x] = c;
    }
    for (uint64_t v = 0; v < n; ++v)
        label[v] = parent[v] >= 0 ? parent[v] : (bmin[v] != INT32_MAX ? bmin[v] : -2);
    for (uint64_t e = 0; e < E; ++e) {
        int32_t lu = label[eu[e]], lv = label[ev[e]];
        uint32_t x;
        int32_t c;
        if (lu < 0 && lv >= 0) { x = eu[e]; c = lv; }
        else if (lv < 0 && lu >= 0) { x = ev[e]; c = lu; }
        else continue;
        if (c < nmin[x]) nmin[x] = c;
        if (c > nmax[x]) nmax[x] = c;
    }
    uint64_t k[8] = {0, 0, 0, 0, 0, c_sim, c_dis, 0};
    for (uint64_t v = 0; v < n; ++v) {
        uint8_t r;
        if (parent[v] >= 0) { r = 3; k[0]++; k[1] += parent[v] == (int32_t)v; }
        else if (bmin[v] != INT32_MAX) { r = 2; k[2]++; k[7] += bmin[v] != bmax[v]; }
        else if (nmin[v] < nmax[v]) { r = 1; label[v] = -1; k[3]++; }
        else { r = 0; label[v] = -2; k[4]++; }
        if (role) role[v] = r;
    }
    if (counts) memcpy(counts, k, sizeof(k));
    rc = 0;
done:
    free(eu); free(ev); if (!cn_out) free(cn); free(sim); free(sd); free(parent);
    free(bmin); free(bmax); free(nmin); free(nmax);
    return rc;
}

/* oracle_scan_ex with every edge intersected (no prune, no given counts). */
ORACLE_API int oracle_scan(uint64_t n, const uint64_t* off, const uint32_t* adj, int mode, double eps, uint64_t p,
                           uint64_t q, int mu, int32_t* label, uint8_t* role, uint32_t* cn_out, uint64_t* counts) {
    return oracle_scan_ex(n, off, adj, mode, eps, p, q, mu, 0u, NULL, label, role, cn_out, counts);
}

/* All (cluster, vertex) memberships: cores once, borders once per cluster they are
 * similar to, sorted by (cluster, vertex).  Returns the pair count; writes at most cap. */
static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

ORACLE_API int64_t oracle_memberships(uint64_t n, const uint64_t* off, const uint32_t* adj, int mode, double eps,
                                      uint64_t p, uint64_t q, int mu, int32_t* out_cluster, int32_t* out_vertex,
                                      uint64_t cap) {
    int32_t* label = (int32_t*)malloc(sizeof(int32_t) * n);
    uint8_t* role = (uint8_t*)malloc(n);
    uint64_t E = off[n] / 2;
    uint32_t* cn = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* eu = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* ev = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (n + 2 * E + 1));
    int64_t cnt = -1;
    if (!label || !role || !cn || !eu || !ev || !keys) goto out;
    if (oracle_scan(n, off, adj, mode, eps, p, q, mu, label, role, cn, NULL) < 0) goto out;
    oracle_orient(n, off, adj, eu, ev);
    uint64_t k = 0;
    for (uint64_t v = 0; v < n; ++v)
        if (role[v] == 3) keys[k++] = ((uint64_t)(uint32_t)label[v] << 32) | v;
    for (uint64_t e = 0; e < E; ++e) {
        uint32_t du = (uint32_t)deg_of(off, eu[e]), dv = (uint32_t)deg_of(off, ev[e]);
        int s = mode ? oracle_ref_f64_similar(cn[e], du, dv, eps) : oracle_exact_similar(cn[e], du, dv, p, q);
        if (!s) continue;
        uint8_t ru = role[eu[e]], rv = role[ev[e]];
        if (ru == 3 && rv != 3) keys[k++] = ((uint64_t)(uint32_t)label[eu[e]] << 32) | ev[e];
        else if (rv == 3 && ru != 3) keys[k++] = ((uint64_t)(uint32_t)label[ev[e]] << 32) | eu[e];
    }
    qsort(keys, k, sizeof(uint64_t), cmp_u64);
    uint64_t w = 0;
    for (uint64_t i = 0; i < k; ++i)
        if (i == 0 || keys[i] != keys[i - 1]) keys[w++] = keys[i];
    for (uint64_t i = 0; i < w && i < cap; ++i) {
        out_cluster[i] = (int32_t)(keys[i] >> 32);
        out_vertex[i] = (int32_t)(uint32_t)keys[i];
    }
    cnt = (int64_t)w;
out:
    free(label); free(role); free(cn); free(eu); free(ev); free(keys);
    return cnt;
}

/* Admissibility of a reference-style output `cand` (label only, cores not marked) against
 * the oracle's memberships: the reference chooses among several clusters for a border by
 * write order (GPUSCAN++/GPUScan.cu:716,722), so any such choice is admissible, and its hub
 * test (:732-798) then runs on those choices.  viol receives
 *   [0] cores whose label differs from the oracle's cluster id
 *   [1] borders whose label is not one of their clusters
 *   [2] non-members labelled >= 0 (or members labelled < 0)
 *   [3] hub/outlier decisions that disagree with the hub rule applied to cand's own labels
 * cn_in (may be NULL): every edge's cn in the reference edge order, instead of intersecting.
 * Returns 0, or -1 on allocation failure. */
ORACLE_API int oracle_check_admissible_ex(uint64_t n, const uint64_t* off, const uint32_t* adj, int mode,
                                          double eps, uint64_t p, uint64_t q, int mu, const uint32_t* cn_in,
                                          const int32_t* cand, uint64_t* viol) {
    int32_t* label = (int32_t*)malloc(sizeof(int32_t) * n);
    uint8_t* role = (uint8_t*)malloc(n);
    uint64_t E = off[n] / 2;
    uint32_t* cn = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* eu = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint32_t* ev = (uint32_t*)malloc(sizeof(uint32_t) * (E ? E : 1));
    uint8_t* ok = (uint8_t*)calloc(n, 1);
    int rc = -1;
    viol[0] = viol[1] = viol[2] = viol[3] = 0;
    if (!label || !role || !cn || !eu || !ev || !ok) goto out2;
    if (oracle_scan_ex(n, off, adj, mode, eps, p, q, mu, 0u, cn_in, label, role, cn, NULL) < 0) goto out2;
    oracle_orient(n, off, adj, eu, ev);
    /* ok[v] = 1 when cand[v] is one of v's memberships */
    for (uint64_t v = 0; v < n; ++v) if (role[v] == 3 && cand[v] == label[v]) ok[v] = 1;
    for (uint64_t e = 0; e < E; ++e) {
        uint32_t du = (uint32_t)deg_of(off, eu[e]), dv = (uint32_t)deg_of(off, ev[e]);
        int s = mode ? oracle_ref_f64_similar(cn[e], du, dv, eps) : oracle_exact_similar(cn[e], du, dv, p, q);
        if (!s) continue;
        uint32_t a = eu[e], b = ev[e];
        if (role[a] == 3 && role[b] != 3 && cand[b] == label[a]) ok[b] = 1;
        if (role[b] == 3 && role[a] != 3 && cand[a] == label[b]) ok[a] = 1;
    }
    for (uint64_t v = 0; v < n; ++v) {
        if (role[v] == 3 && !ok[v]) viol[0]++;
        else if (role[v] == 2 && !ok[v]) viol[1]++;
        else if (role[v] < 2 && cand[v] >= 0) viol[2]++;
        if (role[v] >= 2 && cand[v] < 0) viol[2]++;
    }
    /* hub rule on cand's own labels */
    for (uint64_t v = 0; v < n; ++v) {
        if (cand[v] >= 0) continue;
        int32_t first = -1;
        int hub = 0;
        for (uint64_t j = off[v]; j < off[v + 1]; ++j) {
            int32_t l = cand[adj[j]];
            if (l < 0) continue;
            if (first < 0) first = l;
            else if (l != first) { hub = 1; break; }
        }
        if ((hub ? -1 : -2) != cand[v]) viol[3]++;
    }
    rc = 0;
out2:
    free(label); free(role); free(cn); free(eu); free(ev); free(ok);
    return rc;
}

ORACLE_API int oracle_check_admissible(uint64_t n, const uint64_t* off, const uint32_t* adj, int mode, double eps,
                                       uint64_t p, uint64_t q, int mu, const int32_t* cand, uint64_t* viol) {
    return oracle_check_admissible_ex(n, off, adj, mode, eps, p, q, mu, NULL, cand, viol);
}

/* eid[m] for every directed entry in the reference's edge order (GPUSCAN++/Graph.cpp:95-111):
 * both directions of an edge get the id oracle_orient assigns to it.  Returns 0, or -1 if
 * a reverse entry is missing (asymmetric graph). */
ORACLE_API int oracle_eid(uint64_t n, const uint64_t* off, const uint32_t* adj, uint32_t* eid) {
    uint64_t m = off[n];
    uint32_t* hr = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));   /* higher-rank before j */
    uint64_t* pre = (uint64_t*)malloc(sizeof(uint64_t) * (n + 1));
    int rc = -1;
    if (!hr || !pre) goto out3;
    pre[0] = 0;
    for (uint64_t u = 0; u < n; ++u) {
        uint32_t r = 0;
        for (uint64_t j = off[u]; j < off[u + 1]; ++j) {
            hr[j] = r;
            if (precedes(off, (uint32_t)u, adj[j])) ++r;
        }
        pre[u + 1] = pre[u] + r;
    }
    for (uint64_t u = 0; u < n; ++u) {
        for (uint64_t j = off[u]; j < off[u + 1]; ++j) {
            uint32_t v = adj[j];
            if (precedes(off, (uint32_t)u, v)) {
                eid[j] = (uint32_t)(pre[u] + hr[j]);
            } else {
                uint64_t lo = off[v], hi = off[v + 1];
                while (lo < hi) { uint64_t mid = lo + (hi - lo) / 2; if (adj[mid] < u) lo = mid + 1; else hi = mid; }
                if (lo == off[v + 1] || adj[lo] != (uint32_t)u) goto out3;
                eid[j] = (uint32_t)(pre[v] + hr[lo]);
            }
        }
    }
    rc = 0;
out3:
    free(hr); free(pre);
    return rc;
}

/* ---- seeded R-MAT graphs ------------------------------------------------------------------
 * The same graphs the engine's generator (scan_gen_rmat) builds, so that the CPU reference
 * path and the tests can make the benchmark inputs without loading the engine.  Both are
 * pinned by the same checksums (tests/golden/rmat_checksums.json).  Pair i draws `scale`
 * quadrant choices from its own splitmix64 stream (Steele, Lea, Flood 2014): a 64-bit draw
 * r picks the top-left quadrant below a*2^64, top-right below (a+b)*2^64, bottom-left below
 * (a+b+c)*2^64, else bottom-right.  The pairs are then symmetrised, self-loops dropped,
 * each list sorted and repeats merged. */
static inline uint64_t sm_mix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t prob_threshold(double x) { return x >= 1.0 ? ~0ull : (uint64_t)ldexp(x, 63) * 2; }

ORACLE_API void oracle_rmat_pairs(int scale, uint64_t num_pairs, double a, double b, double c, uint64_t seed,
                                  uint64_t* pairs) {
    const uint64_t ta = prob_threshold(a), tab = prob_threshold(a + b), tabc = prob_threshold(a + b + c);
    int64_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (int64_t)num_pairs; ++i) {
        uint64_t s = sm_mix(seed * 0x9E3779B97F4A7C15ull + sm_mix((uint64_t)i + 0x632BE59BD9B4E019ull));
        uint32_t u = 0, v = 0;
        for (int l = 0; l < scale; ++l) {
            s += 0x9E3779B97F4A7C15ull;
            const uint64_t r = sm_mix(s);
            u = (u << 1) | (uint32_t)(r >= tab);
            v = (v << 1) | (uint32_t)((r >= ta && r < tab) || r >= tabc);
        }
        pairs[i] = ((uint64_t)u << 32) | v;
    }
}

static int cmp_u32(const void* x, const void* y) {
    uint32_t a = *(const uint32_t*)x, b = *(const uint32_t*)y;
    return a < b ? -1 : a > b;
}

/* Symmetric CSR from vertex pairs (u << 32 | v): self-loops and ids >= n dropped, lists
 * sorted ascending without repeats.  off[n+1]; adj needs room for 2*num_pairs entries.
 * Returns m (directed entries), or -1 on allocation failure. */
ORACLE_API int64_t oracle_csr_from_pairs(uint64_t n, const uint64_t* pairs, uint64_t num_pairs, uint64_t* off,
                                         uint32_t* adj) {
    uint32_t* cnt = (uint32_t*)calloc(n ? n : 1, sizeof(uint32_t));
    uint64_t* cur = (uint64_t*)malloc(sizeof(uint64_t) * (n + 1));
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * (2 * num_pairs + 1));
    int64_t m = -1, i;
    if (!cnt || !cur || !tmp) goto out;
#pragma omp parallel for schedule(static)
    for (i = 0; i < (int64_t)num_pairs; ++i) {
        const uint32_t u = (uint32_t)(pairs[i] >> 32), v = (uint32_t)pairs[i];
        if (u == v || u >= n || v >= n) continue;
#pragma omp atomic
        cnt[u]++;
#pragma omp atomic
        cnt[v]++;
    }
    cur[0] = 0;
    for (uint64_t x = 0; x < n; ++x) cur[x + 1] = cur[x] + cnt[x];
    memcpy(off, cur, sizeof(uint64_t) * (n + 1));          /* raw list starts, for now */
#pragma omp parallel for schedule(static)
    for (i = 0; i < (int64_t)num_pairs; ++i) {
        const uint32_t u = (uint32_t)(pairs[i] >> 32), v = (uint32_t)pairs[i];
        uint64_t pu, pv;
        if (u == v || u >= n || v >= n) continue;
#pragma omp atomic capture
        pu = cur[u]++;
#pragma omp atomic capture
        pv = cur[v]++;
        tmp[pu] = v;
        tmp[pv] = u;
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (i = 0; i < (int64_t)n; ++i) {                        /* sort, merge repeats; cnt = new degree */
        uint32_t* l = tmp + off[i];
        const uint64_t len = off[i + 1] - off[i];
        if (len > 1) qsort(l, len, sizeof(uint32_t), cmp_u32);
        uint64_t k = 0;
        for (uint64_t j = 0; j < len; ++j)
            if (k == 0 || l[j] != l[k - 1]) l[k++] = l[j];
        cnt[i] = (uint32_t)k;
    }
    memcpy(cur, off, sizeof(uint64_t) * (n + 1));           /* cur = raw starts */
    off[0] = 0;
    for (uint64_t x = 0; x < n; ++x) off[x + 1] = off[x] + cnt[x];
#pragma omp parallel for schedule(dynamic, 1024)
    for (i = 0; i < (int64_t)n; ++i) memcpy(adj + off[i], tmp + cur[i], sizeof(uint32_t) * cnt[i]);
    m = (int64_t)off[n];
out:
    free(cnt); free(cur); free(tmp);
    return m;
}
