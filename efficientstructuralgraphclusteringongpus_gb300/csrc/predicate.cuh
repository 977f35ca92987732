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

struct PredParams {
    double eps;          // ref-f64 value (strtod of the decimal text, like atof in main.cpp:26)
    uint64_t p, q;       // exact value p/q
    int mode;            // 0 exact, 1 ref-f64
};

}  // namespace scan
