// The epsilon predicate, shared by every kernel that tests similarity.
#pragma once

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
// agrees with the intersect test whenever it fires ((T+2)^2 >= 4), so it is implied.
// Only IEEE multiplies and compares are used: no contraction, identical bits on any host.
__host__ __device__ __forceinline__ bool ref_f64_similar(uint32_t t, uint32_t du, uint32_t dv, double eps) {
    const double du1 = (double)(du + 1u), dv1 = (double)(dv + 1u);
    if (du1 < dv1 * eps * eps) return false;
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

struct PredParams {
    double eps;          // ref-f64 value (strtod of the decimal text, like atof in main.cpp:26)
    uint64_t p, q;       // exact value p/q
    int mode;            // 0 exact, 1 ref-f64
};

}  // namespace scan
