// Host check of the per-pivot tests of predicate.cuh (pivot_tests, edge_pruned, count_floor)
// against the per-edge double and 128-bit tests they replace in the counting kernels:
//   * edge_pruned(du) == ref_f64_never(du, dv) && exact_never(du, dv)   for every du checked;
//   * count_floor(du) <= exact_min_count and <= ref_min_count, and no count below it passes
//     either predicate (ref_f64_similar, exact_similar); where the reference's int square of
//     the count can wrap (du + 1 > 46340), every count below the bound is tried.
// The same source is compiled for the device; host and device give the same bits here (IEEE
// products, a correctly rounded sqrtf, no additions to contract).
//
// Test infrastructure: tests/test_predicate_bounds.py compiles and runs it on the CPU.
//   predicate_check            prints "ok <checks> <floor gap histogram>" or the first failure
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define __host__
#define __device__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#include "predicate.cuh"

using namespace scan;

namespace {

struct Eps {
    std::string text;
    double eps;
    uint64_t p, q;
};

// "0.123" -> p = 123, q = 1000, eps = strtod (the decimal form make_pred reads)
Eps eps_of(const char* text) {
    Eps e{text, std::strtod(text, nullptr), 0, 1};
    const char* dot = std::strchr(text, '.');
    std::string digits = text;
    if (dot) {
        digits = std::string(text, dot) + std::string(dot + 1);
        for (const char* c = dot + 1; *c; ++c) e.q *= 10;
    }
    e.p = std::strtoull(digits.c_str(), nullptr, 10);
    if (e.p > e.q) { e.p = 1; e.q = 0; }   // as make_pred: eps > 1, the exact test never holds
    return e;
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

int main() {
    const char* texts[] = {"0", "0.00001", "0.00005", "0.05", "0.1", "0.2", "0.25", "0.3", "0.333333333",
                           "0.4", "0.5", "0.6", "0.7", "0.75", "0.8", "0.9", "0.95", "0.999999999", "1",
                           "1.5", "0.123456789", "0.707106781"};
    std::vector<uint32_t> dvs;
    for (uint32_t d = 0; d < 600; ++d) dvs.push_back(d);
    for (uint32_t d = 600; d < 200000; d = d * 17 / 16 + 1) dvs.push_back(d);
    // degrees up to 2^31 - 9: each edge is stored twice in m < 2^32 - 16, so no vertex has more
    // (the reference's int degree never wraps)
    for (uint32_t d : {46339u, 46340u, 46341u, 65535u, 65536u, 163088u, 1151662u, 4000000u, 100000000u,
                       2000000000u, 2147483639u})
        dvs.push_back(d);
    uint64_t checks = 0, gap[4] = {0, 0, 0, 0};   // exact minimum - count_floor: 0, 1, 2, more
    uint64_t rng = 12345;
    for (const char* t : texts) {
        const Eps e = eps_of(t);
        PredParams pp{e.eps, e.p, e.q, 1, 0.0, 0.f};
        pred_derive(&pp);
        for (uint32_t dv : dvs) {
            const PivotTests pt = pivot_tests(dv, true, pp.eps, pp.p, pp.q, pp.pq2, pp.eps2_floor);
            // du: every value up to 2000 and around the thresholds, then a random sample
            std::vector<uint32_t> dus;
            for (uint32_t du = 0; du < 2000 && du <= dv; ++du) dus.push_back(du);
            for (int64_t k = -3; k <= 3; ++k) {
                const int64_t a = (int64_t)pt.np - 1 + k;
                if (a >= 0 && a <= (int64_t)dv) dus.push_back((uint32_t)a);
            }
            for (int i = 0; i < 300 && dv > 0; ++i) dus.push_back((uint32_t)(splitmix(rng) % ((uint64_t)dv + 1)));
            for (uint32_t du : dus) {
                ++checks;
                const bool want = ref_f64_never(du, dv, pp.eps) && exact_never(du, dv, pp.p, pp.q);
                if (edge_pruned(du, pt) != want) {
                    std::printf("FAIL prune eps=%s dv=%u du=%u np=%llu want=%d\n", t, dv, du,
                                (unsigned long long)pt.np, (int)want);
                    return 1;
                }
                if (want || du + 1u > 46340u) continue;
                const uint32_t fl = count_floor(du, dv, pt, pp.eps);
                const uint32_t mx = exact_min_count(du, dv, pp.p, pp.q);
                const uint32_t mr = ref_min_count(du, dv, pp.eps);
                const uint32_t m = mx < mr ? mx : mr;
                if (fl > m) {
                    std::printf("FAIL floor eps=%s dv=%u du=%u floor=%u exact_min=%u ref_min=%u\n", t, dv, du, fl,
                                mx, mr);
                    return 1;
                }
                for (uint32_t c = fl >= 3 ? fl - 3 : 0; c < fl; ++c) {
                    if (ref_f64_similar(c, du, dv, pp.eps) || exact_similar(c, du, dv, pp.p, pp.q)) {
                        std::printf("FAIL similar below floor eps=%s dv=%u du=%u count=%u floor=%u\n", t, dv, du, c,
                                    fl);
                        return 1;
                    }
                }
                if (m != kNoCount) ++gap[m - fl >= 3 ? 3 : m - fl];
            }
        }
    }
    // The wrap zone: lower degree above 46339.  Every count below the bound must fail both
    // predicates, the wrapped squares included.
    uint64_t wrap_checks = 0;
    for (const char* t : {"0.2", "0.4", "0.5", "0.9", "0.00005", "1"}) {
        const Eps e = eps_of(t);
        PredParams pp{e.eps, e.p, e.q, 1, 0.0, 0.f};
        pred_derive(&pp);
        for (uint32_t dv : {46340u, 50000u, 120000u, 290000u, 1151662u, 2000000000u}) {
            const PivotTests pt = pivot_tests(dv, true, pp.eps, pp.p, pp.q, pp.pq2, pp.eps2_floor);
            for (uint32_t du : {46340u, 46341u, 47000u, 60000u, 115000u, 290000u, 1151662u}) {
                if (du > dv || edge_pruned(du, pt)) continue;
                const uint32_t fl = count_floor(du, dv, pt, pp.eps);
                const uint32_t top = fl < du ? fl : du;      // counts are below du
                for (uint32_t c = 0; c < top; ++c) {
                    ++wrap_checks;
                    if (ref_f64_similar(c, du, dv, pp.eps) || exact_similar(c, du, dv, pp.p, pp.q)) {
                        std::printf("FAIL wrap eps=%s dv=%u du=%u count=%u floor=%u\n", t, dv, du, c, fl);
                        return 1;
                    }
                }
            }
        }
    }
    checks += wrap_checks;

    // eps with more than 9 decimals (ref-f64 runs only; GPUScan() passes the caller's double as
    // its shortest decimal): p^2 and q^2 wrap in 64 bits, so the exact side is not a test of
    // anything.  What the labels rest on must still hold: a pruned edge fails the reference's
    // 'never' test, and no count below count_floor passes the reference's predicate.
    for (const char* t : {"0.30000000000000004", "0.1234567890123", "0.7071067811865476", "0.49999999999"}) {
        const Eps e = eps_of(t);
        PredParams pp{e.eps, e.p, e.q, 1, 0.0, 0.f};
        pred_derive(&pp);
        for (uint32_t dv : dvs) {
            const PivotTests pt = pivot_tests(dv, true, pp.eps, pp.p, pp.q, pp.pq2, pp.eps2_floor);
            for (uint32_t du = 0; du < 3000 && du <= dv; du += 1 + du / 64) {
                ++checks;
                if (edge_pruned(du, pt) && !ref_f64_never(du, dv, pp.eps)) {
                    std::printf("FAIL long prune eps=%s dv=%u du=%u\n", t, dv, du);
                    return 1;
                }
                if (edge_pruned(du, pt)) continue;
                const uint32_t fl = count_floor(du, dv, pt, pp.eps);
                if (fl > ref_min_count(du, dv, pp.eps) || (fl > 0 && ref_f64_similar(fl - 1, du, dv, pp.eps))) {
                    std::printf("FAIL long floor eps=%s dv=%u du=%u floor=%u\n", t, dv, du, fl);
                    return 1;
                }
            }
        }
    }
    std::printf("ok %llu %llu %llu %llu %llu\n", (unsigned long long)checks, (unsigned long long)gap[0],
                (unsigned long long)gap[1], (unsigned long long)gap[2], (unsigned long long)gap[3]);
    return 0;
}
