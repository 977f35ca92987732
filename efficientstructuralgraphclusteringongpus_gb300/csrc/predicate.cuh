// The epsilon predicate, shared by every kernel that tests similarity.
#pragma once

#include <cmath>
#include <cstdint>

namespace scan {

// ---- the epsilon predicate -------------------------------------------------------------
// u is the lower endpoint in (degree, id) order, v the higher; t = |N(u) ∩ N(v)|.
//
// ref-f64 reproduces, with the same operand order, the reference's three double tests:
//   'N' prune  deg_u < deg_v * eps * eps                      GPUSCAN++/GPUScan.cu:145
//   'Y' prune  eps * eps * deg_u * deg_v <= 4.0               GPUSCAN++/GPUScan.cu:156
//   intersect  (T+2)*(T+2) < eps * eps * (du+1) * (dv+1)      GPUSCAN++/GPUScan.cu:220-221
// with deg_x = d_x + 1 and (T+2)*(T+2) an int product (wraps past 46340).  The 'Y' prune
// agrees with the intersect test whenever the square does not wrap ((T+2)^2 >= 4), but not
// when it wraps negative (both degrees above 46339 and eps below about 4e-5): there 'Y'
// says similar and the intersect test would say not, so it is evaluated in its own right.
// Only IEEE multiplies and compares are used: no contraction, identical bits on any host.
// The 'N' prune alone: true when the degrees rule the edge out whatever t is.
__host__ __device__ __forceinline__ bool ref_f64_never(uint32_t du, uint32_t dv, double eps) {
    const double du1 = (double)(du + 1u), dv1 = (double)(dv + 1u);
    return du1 < dv1 * eps * eps;
}

__host__ __device__ __forceinline__ bool ref_f64_always(uint32_t du, uint32_t dv, double eps) {
    const double du1 = (double)(du + 1u), dv1 = (double)(dv + 1u);
    return eps * eps * du1 * dv1 <= 4.0;
}

__host__ __device__ __forceinline__ bool ref_f64_similar(uint32_t t, uint32_t du, uint32_t dv, double eps) {
    if (ref_f64_never(du, dv, eps)) return false;
    if (ref_f64_always(du, dv, eps)) return true;
    const int32_t t2 = (int32_t)((t + 2u) * (t + 2u));
    return !((double)t2 < eps * eps * (double)(int32_t)(du + 1u) * (double)(int32_t)(dv + 1u));
}

// exact: (t+2)^2 * q^2 >= p^2 * (du+1) * (dv+1) with eps = p/q, p <= q <= 2^30.
// (t+2)*q < 2^63 and p^2 < 2^60, so both sides fit 128 bits.
__host__ __device__ __forceinline__ bool exact_similar(uint32_t t, uint32_t du, uint32_t dv, uint64_t p, uint64_t q) {
    if (p > q) return false;  // sigma <= 1 < eps
    const uint64_t a = (uint64_t)(t + 2ull) * q;
    const unsigned __int128 lhs = (unsigned __int128)a * a;
    const unsigned __int128 rhs = (unsigned __int128)(p * p) * ((uint64_t)(du + 1ull) * (uint64_t)(dv + 1ull));
    return lhs >= rhs;
}

// True when no t the degrees allow can satisfy the exact test.  u's open neighbourhood
// holds v, which N(v) does not, so t <= du - 1 and t + 2 <= du + 1; then
// (t+2)^2 q^2 <= (du+1)^2 q^2 < (du+1) p^2 (dv+1) whenever (du+1) q^2 < p^2 (dv+1).
// Both sides are below 2^93 (q^2, p^2 <= 2^60; du+1, dv+1 <= 2^32).
__host__ __device__ __forceinline__ bool exact_never(uint32_t du, uint32_t dv, uint64_t p, uint64_t q) {
    if (p > q) return true;
    return (unsigned __int128)(q * q) * (du + 1ull) < (unsigned __int128)(p * p) * (dv + 1ull);
}

// Smallest count each predicate accepts, for the early stop of a one-shot run: a count
// below it can never be similar, so a list whose hits so far plus its unexamined entries
// fall below it is decided.  kNoCount when no count qualifies.
constexpr uint32_t kNoCount = 0xFFFFFFFFu;

// exact: the least a = t + 2 >= 2 with (a q)^2 >= p^2 (du+1)(dv+1).  a q < 2^63 as in
// exact_similar; the double square root lands within one of a, the loops settle it.
__host__ __device__ inline uint32_t exact_min_count(uint32_t du, uint32_t dv, uint64_t p, uint64_t q) {
    if (p > q) return kNoCount;
    const unsigned __int128 x = (unsigned __int128)(p * p) * ((uint64_t)(du + 1ull) * (uint64_t)(dv + 1ull));
    auto ok = [&](uint64_t a) { return (unsigned __int128)(a * q) * (a * q) >= x; };
    uint64_t a = (uint64_t)(sqrt((double)x) / (double)q);
    if (a < 2) a = 2;
    while (a > 2 && ok(a - 1)) --a;
    while (!ok(a)) ++a;
    return a - 2 >= kNoCount ? kNoCount - 1 : (uint32_t)(a - 2);
}

// ref-f64, for counts whose square does not wrap (t + 2 <= 46340): the least a = t + 2
// with !((double)(a*a) < eps*eps*(du+1)*(dv+1)), the expression of ref_f64_similar.
__host__ __device__ inline uint32_t ref_min_count(uint32_t du, uint32_t dv, double eps) {
    if (ref_f64_never(du, dv, eps)) return kNoCount;
    if (ref_f64_always(du, dv, eps)) return 0u;
    const double thr = eps * eps * (double)(int32_t)(du + 1u) * (double)(int32_t)(dv + 1u);
    auto ok = [&](uint32_t a) { return !((double)(int32_t)(a * a) < thr); };
    const double r = sqrt(thr);
    if (!(r < 46341.0)) return kNoCount;
    uint32_t a = (uint32_t)r;
    if (a < 2) a = 2;
    while (a > 2 && ok(a - 1)) --a;
    while (a <= 46340 && !ok(a)) ++a;
    return a > 46340 ? kNoCount : a - 2;
}

// Per-pivot constants of a one-shot run's per-edge tests.  GB300 issues double arithmetic at
// a small fraction of its integer and float rate: with every edge taking the prune, the
// early-stop threshold (a double square root) and both predicates in double, the FP64 pipe
// was 74% busy in the 1,024-entry class.  So each pivot's 'never' tests are reduced once to
// an integer threshold on du, the early-stop threshold is a float lower bound, and an edge
// takes the double tests only when the count can still be similar.
struct PivotTests {
    uint64_t np;     // the edge is pruned (both predicates' 'never' test holds) iff du + 1 < np
    float tscale;    // eps2_floor * (dv + 1), for count_floor
};

__host__ __device__ inline PivotTests pivot_tests(uint32_t dv, bool on, double eps, uint64_t p, uint64_t q,
                                                double pq2, float eps2_floor) {
    constexpr uint64_t kAll = 1ull << 33;      // above every du + 1
    const uint64_t dv1 = dv + 1ull;
    PivotTests t;
    t.tscale = eps2_floor * (float)dv1;
    t.np = 0;
    if (!on) return t;
    // ref-f64 'never', (double)du1 < dv1 * eps * eps: true exactly below ceil(dv1 * eps * eps)
    const double rn = (double)dv1 * eps * eps;
    const uint64_t n_ref = !(rn > 0.0) ? 0ull : rn >= (double)kAll ? kAll : (uint64_t)ceil(rn);
    // exact 'never', q^2 du1 < p^2 dv1: true exactly below ceil(p^2 dv1 / q^2); the double
    // estimate is within one of it (relative error < 2^-50 on a value below 2^33)
    uint64_t n_ex = kAll;
    if (p <= q) {
        const unsigned __int128 num = (unsigned __int128)(p * p) * dv1;
        const uint64_t q2 = q * q;
        const double est = pq2 * (double)dv1;
        uint64_t c = !(est > 0.0) ? 0ull : est >= (double)kAll ? kAll : (uint64_t)est;
        for (int i = 0; i < 4 && c > 0 && (unsigned __int128)q2 * (c - 1) >= num; ++i) --c;
        for (int i = 0; i < 4 && c < kAll && (unsigned __int128)q2 * c < num; ++i) ++c;
        const bool ok = (unsigned __int128)q2 * c >= num && (c == 0 || (unsigned __int128)q2 * (c - 1) < num);
        if (!ok) return t;                     // cannot happen; prune nothing rather than guess
        n_ex = c;
    }
    t.np = n_ref < n_ex ? n_ref : n_ex;
    return t;
}

// The kernels take a pivot's prune threshold for a degree below kPruneTable from a table
// filled once per run (k_prune_table; a batch fills one per distinct parameter set, up to
// kPruneSets, k_prune_tables): its double arithmetic (about ten FP64 instructions, 16 issue
// cycles each per warp on GB300) would otherwise be paid by every small pivot, most of
// which have few lower edges.
constexpr uint32_t kPruneTable = 4096;
constexpr uint32_t kPruneSets = 64;

__host__ __device__ __forceinline__ bool edge_pruned(uint32_t du, const PivotTests& pt) { return du + 1ull < pt.np; }

// A lower bound of the least count either predicate accepts (exact_min_count and
// ref_min_count): floor(sqrt(eps2_floor (du+1)(dv+1)) (1 - 1e-6)) - 2.  The float roundings
// (eps2_floor, two products, the square root, the scaling) stay below 4e-7 relative, and the
// reference's double threshold is at least eps^2 (du+1)(dv+1)(1 - 2^-51), so every count
// below the bound is rejected by both.  0 where any count may be similar.
// Where the reference's int square of the count can wrap (du + 1 > 46340), its test is not
// monotone in the count, but only counts above 46338 wrap: the bound is capped at 46339,
// below which the square is exact.  When the reference's threshold is 2^31 or more, no
// square, wrapped or not, reaches it, and the bound is left uncapped (its double threshold
// is evaluated for these edges only).
// Out of line, so that the compiler does not evaluate its double products for every edge
// (if-converted, they kept GB300's FP64 pipe 8.5% busy in the 1,024-entry class).
static __host__ __device__ __noinline__ uint32_t wrap_zone_floor(uint32_t l, uint32_t du, uint32_t dv, double eps) {
    const double thr = eps * eps * (double)(int32_t)(du + 1u) * (double)(int32_t)(dv + 1u);
    return thr >= 2147483648.0 ? l : (l < 46339u ? l : 46339u);
}

__host__ __device__ __forceinline__ uint32_t count_floor(uint32_t du, uint32_t dv, const PivotTests& pt, double eps) {
    float s = sqrtf(pt.tscale * (float)(du + 1u)) * 0.999999f;
    s = s < 4.0e9f ? s : 4.0e9f;                       // eps > 1: keep the conversion defined
    const uint32_t a = (uint32_t)s;
    const uint32_t l = a > 2u ? a - 2u : 0u;
    if (du + 1u <= 46340u) return l;
    return wrap_zone_floor(l, du, dv, eps);
}

struct PredParams {
    double eps;          // ref-f64 value (strtod of the decimal text, like atof in main.cpp:26)
    uint64_t p, q;       // exact value p/q
    int mode;            // 0 exact, 1 ref-f64
    // derived by pred_derive from the three above:
    double pq2;          // p^2 / q^2 rounded (an estimate only; infinity when p > q)
    float eps2_floor;    // min(p^2/q^2, eps*eps) as a float: within 2^-24 of a lower bound
                         // on the eps^2 of both predicates (count_floor's margin covers it)
    uint32_t np_set;     // batched runs: the graph's prune-threshold table (its parameter set)
};

// Fill the derived fields; call after eps, p or q change.
inline void pred_derive(PredParams* pp) {
    pp->pq2 = pp->p > pp->q ? INFINITY : ((double)pp->p * (double)pp->p) / ((double)pp->q * (double)pp->q);
    const double e2 = pp->eps * pp->eps;
    double m = pp->pq2 < e2 ? pp->pq2 : e2;
    if (!(m > 0.0)) m = 0.0;                 // eps = 0 (or not a number): no early stop
    pp->eps2_floor = m > 3.0e38 ? 3.0e38f : (float)m;
}

}  // namespace scan
