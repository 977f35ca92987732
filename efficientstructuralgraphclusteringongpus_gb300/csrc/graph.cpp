// Host side of the engine: CSR files, validation, generators, reference-compatible
// orientation and error reporting.  Plain C++17 + OpenMP; no CUDA here.
//
// File format (written by csr_convert/EdgeListToBinsConverter.cpp:85-121, read by
// GPUSCAN++/Graph.cpp:157-223):
//   b_degree.bin : int32 int_size (=4), uint32 n, uint32 m (= directed entries), int32 deg[n]
//   b_adj.bin    : the n neighbour lists concatenated, uint32 each, sorted ascending
// 64-bit extension (int_size = 8): uint64 n, uint64 m, int64 deg[n]; b_adj.bin unchanged.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include <omp.h>

#include "graph_internal.h"

namespace scan {

static thread_local std::string g_last_error;

scan_status fail(scan_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

void clear_error() { g_last_error.clear(); }

void finish_graph(scan_graph* g) {
    uint32_t mx = 0;
    const int64_t n = (int64_t)g->n;
#pragma omp parallel for reduction(max : mx) schedule(static)
    for (int64_t v = 0; v < n; ++v) {
        uint64_t d = g->off[v + 1] - g->off[v];
        if (d > mx) mx = (uint32_t)d;
    }
    g->max_deg = mx;
}

// Exclusive prefix sum of counts[0..n) into off[0..n], done in parallel blocks.
static void exclusive_scan(const uint32_t* counts, uint64_t n, uint64_t* off) {
    const int nt = omp_get_max_threads();
    std::vector<uint64_t> part(nt + 1, 0);
#pragma omp parallel num_threads(nt)
    {
        int t = omp_get_thread_num();
        int T = omp_get_num_threads();
        uint64_t lo = n * t / T, hi = n * (t + 1) / T, s = 0;
        for (uint64_t i = lo; i < hi; ++i) s += counts[i];
        part[t + 1] = s;
#pragma omp barrier
#pragma omp single
        for (int i = 0; i < T; ++i) part[i + 1] += part[i];
        uint64_t run = part[t];
        for (uint64_t i = lo; i < hi; ++i) {
            off[i] = run;
            run += counts[i];
        }
    }
    off[n] = part[nt];
}

scan_status build_from_pairs(uint64_t n, std::vector<uint64_t>& pairs, scan_graph* g) {
    if (n == 0 || n > 0xFFFFFFFFull) return fail(SCAN_ERR_INVALID_ARG, "vertex count must be in [1, 2^32)");
    std::unique_ptr<std::atomic<uint32_t>[]> cnt(new std::atomic<uint32_t>[n]);
    const int64_t np = (int64_t)pairs.size();
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) cnt[v].store(0, std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < np; ++i) {
        uint32_t u = (uint32_t)(pairs[i] >> 32), v = (uint32_t)pairs[i];
        if (u == v || u >= n || v >= n) continue;
        cnt[u].fetch_add(1, std::memory_order_relaxed);
        cnt[v].fetch_add(1, std::memory_order_relaxed);
    }
    std::vector<uint32_t> raw(n);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) raw[v] = cnt[v].load(std::memory_order_relaxed);
    std::vector<uint64_t> roff(n + 1);
    exclusive_scan(raw.data(), n, roff.data());
    std::vector<uint32_t> tmp(roff[n]);
    std::unique_ptr<std::atomic<uint64_t>[]> cur(new std::atomic<uint64_t>[n]);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < (int64_t)n; ++v) cur[v].store(roff[v], std::memory_order_relaxed);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < np; ++i) {
        uint32_t u = (uint32_t)(pairs[i] >> 32), v = (uint32_t)pairs[i];
        if (u == v || u >= n || v >= n) continue;
        tmp[cur[u].fetch_add(1, std::memory_order_relaxed)] = v;
        tmp[cur[v].fetch_add(1, std::memory_order_relaxed)] = u;
    }
    std::vector<uint64_t>().swap(pairs);
    cnt.reset();
    cur.reset();
    std::vector<uint32_t> deg(n);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; ++v) {
        uint32_t* b = tmp.data() + roff[v];
        uint32_t* e = tmp.data() + roff[v + 1];
        std::sort(b, e);
        deg[v] = (uint32_t)(std::unique(b, e) - b);
    }
    g->n = n;
    g->off.assign(n + 1, 0);
    exclusive_scan(deg.data(), n, g->off.data());
    g->m = g->off[n];
    g->adj.resize(g->m);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < (int64_t)n; ++v)
        std::memcpy(g->adj.data() + g->off[v], tmp.data() + roff[v], sizeof(uint32_t) * deg[v]);
    finish_graph(g);
    return SCAN_OK;
}

bool parse_decimal(const char* text, uint64_t* p_out, uint64_t* q_out, double* as_double) {
    if (!text) return false;
    const char* s = text;
    while (*s == ' ' || *s == '\t') ++s;
    if (*s == '+' || *s == '-') ++s;  // the sign is irrelevant: both predicates square eps
    unsigned __int128 p = 0;
    int frac_digits = 0, digits = 0;
    bool dot = false;
    for (; *s; ++s) {
        if (*s >= '0' && *s <= '9') {
            p = p * 10 + (unsigned)(*s - '0');
            if (p > (unsigned __int128)1e30) return false;
            ++digits;
            if (dot) ++frac_digits;
        } else if (*s == '.' && !dot) {
            dot = true;
        } else {
            break;
        }
    }
    if (digits == 0) return false;
    int exp10 = 0;
    if (*s == 'e' || *s == 'E') {
        ++s;
        int sign = 1;
        if (*s == '+' || *s == '-') { sign = (*s == '-') ? -1 : 1; ++s; }
        if (!(*s >= '0' && *s <= '9')) return false;
        int e = 0;
        for (; *s >= '0' && *s <= '9'; ++s) { e = e * 10 + (*s - '0'); if (e > 60) return false; }
        exp10 = sign * e;
    }
    while (*s == ' ' || *s == '\t' || *s == '\n') ++s;
    if (*s) return false;
    int scale = frac_digits - exp10;  // value = p / 10^scale
    unsigned __int128 q = 1;
    while (scale > 0) { q *= 10; --scale; if (q > (unsigned __int128)1e36) return false; }
    while (scale < 0) { p *= 10; ++scale; if (p > (unsigned __int128)1e36) return false; }
    // reduce
    unsigned __int128 a = p, b = q;
    while (b) { unsigned __int128 t = a % b; a = b; b = t; }
    if (a > 1) { p /= a; q /= a; }
    if (p == 0) q = 1;
    if (p > (unsigned __int128)1000000000000000000ull || q > (unsigned __int128)1000000000000000000ull)
        return false;
    *p_out = (uint64_t)p;
    *q_out = (uint64_t)q;
    if (as_double) *as_double = std::strtod(text, nullptr);
    return true;
}

// splitmix64 finaliser: a bijective 64-bit mixer (Steele, Lea, Flood 2014).
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t stream_start(uint64_t seed, uint64_t index) {
    return mix64(seed * 0x9E3779B97F4A7C15ull + mix64(index + 0x632BE59BD9B4E019ull));
}
static inline uint64_t next64(uint64_t& s) {
    s += 0x9E3779B97F4A7C15ull;
    return mix64(s);
}
static inline uint64_t bounded(uint64_t r, uint64_t n) {
    return (uint64_t)(((unsigned __int128)r * n) >> 64);
}

}  // namespace scan

using namespace scan;

extern "C" {

const char* scan_last_error(void) { return g_last_error.c_str(); }

const char* scan_status_string(scan_status s) {
    switch (s) {
        case SCAN_OK: return "ok";
        case SCAN_ERR_INVALID_ARG: return "invalid argument";
        case SCAN_ERR_IO: return "i/o error";
        case SCAN_ERR_FORMAT: return "bad graph format";
        case SCAN_ERR_CUDA: return "cuda error";
        case SCAN_ERR_OUT_OF_MEMORY: return "out of memory";
        case SCAN_ERR_TOO_LARGE: return "graph too large";
        case SCAN_ERR_DEVICE: return "device-side check failed";
    }
    return "unknown status";
}

const char* scan_version(void) { return "0.1.0"; }

static scan_status read_exact(FILE* f, void* dst, size_t bytes, const std::string& what) {
    if (bytes && std::fread(dst, 1, bytes, f) != bytes)
        return fail(SCAN_ERR_IO, "short read in " + what);
    return SCAN_OK;
}

scan_status scan_graph_validate(const scan_graph* g, int check_symmetry) {
    if (!g) return fail(SCAN_ERR_INVALID_ARG, "graph is null");
    if (g->off.size() != g->n + 1 || g->off[0] != 0 || g->off[g->n] != g->m || g->adj.size() != g->m)
        return fail(SCAN_ERR_FORMAT, "offsets do not describe the adjacency array");
    std::atomic<int> bad{0};
    std::atomic<uint64_t> bad_v{0};
    const int64_t n = (int64_t)g->n;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < n; ++v) {
        if (bad.load(std::memory_order_relaxed)) continue;
        uint64_t b = g->off[v], e = g->off[v + 1];
        if (e < b) { bad = 1; bad_v = v; continue; }
        for (uint64_t j = b; j < e; ++j) {
            uint32_t w = g->adj[j];
            int code = 0;
            if (w >= g->n) code = 2;
            else if (w == (uint32_t)v) code = 3;  // CheckInputGraph: "Self loop"
            else if (j > b && w <= g->adj[j - 1]) code = 4;  // "not sorted in increasing id order"
            else if (check_symmetry &&
                     !std::binary_search(g->adj.begin() + g->off[w], g->adj.begin() + g->off[w + 1],
                                         (uint32_t)v))
                code = 5;
            if (code) { int z = 0; if (bad.compare_exchange_strong(z, code)) bad_v = v; break; }
        }
    }
    int code = bad.load();
    if (code) {
        const char* why = code == 2 ? "neighbour id >= n" : code == 3 ? "self loop"
                        : code == 4 ? "neighbour list not sorted strictly ascending"
                        : code == 5 ? "graph is not symmetric" : "offsets decrease";
        return fail(SCAN_ERR_FORMAT, std::string(why) + " at vertex " + std::to_string(bad_v.load()));
    }
    if (g->m % 2) return fail(SCAN_ERR_FORMAT, "odd number of directed entries (graph not symmetric)");
    if (g->m >= (1ull << 32)) return fail(SCAN_ERR_TOO_LARGE, "m >= 2^32 directed entries");
    return SCAN_OK;
}

scan_status scan_graph_load(const char* dir, scan_graph** out) {
    clear_error();
    if (!dir || !out) return fail(SCAN_ERR_INVALID_ARG, "dir and out must be non-null");
    *out = nullptr;
    std::string d(dir);
    FILE* fd = std::fopen((d + "/b_degree.bin").c_str(), "rb");
    if (!fd) return fail(SCAN_ERR_IO, "cannot open " + d + "/b_degree.bin: " + std::strerror(errno));
    std::unique_ptr<FILE, int (*)(FILE*)> fd_guard(fd, std::fclose);
    int32_t int_size = 0;
    scan_status st = read_exact(fd, &int_size, 4, "b_degree.bin header");
    if (st) return st;
    uint64_t n = 0, m = 0;
    if (int_size == 4) {
        uint32_t n32, m32;
        if ((st = read_exact(fd, &n32, 4, "b_degree.bin header"))) return st;
        if ((st = read_exact(fd, &m32, 4, "b_degree.bin header"))) return st;
        n = n32; m = m32;
    } else if (int_size == 8) {
        if ((st = read_exact(fd, &n, 8, "b_degree.bin header"))) return st;
        if ((st = read_exact(fd, &m, 8, "b_degree.bin header"))) return st;
    } else {
        return fail(SCAN_ERR_FORMAT, "b_degree.bin: int_size must be 4 or 8, got " + std::to_string(int_size));
    }
    if (n == 0 || n > 0xFFFFFFFFull) return fail(SCAN_ERR_FORMAT, "b_degree.bin: vertex count out of range");
    std::unique_ptr<scan_graph> g(new scan_graph());
    g->n = n;
    try {
        g->off.assign(n + 1, 0);
    } catch (...) { return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot allocate offsets"); }
    uint64_t sum = 0;
    if (int_size == 4) {
        std::vector<int32_t> deg(n);
        if ((st = read_exact(fd, deg.data(), 4 * n, "b_degree.bin degrees"))) return st;
        for (uint64_t v = 0; v < n; ++v) {
            if (deg[v] < 0) return fail(SCAN_ERR_FORMAT, "negative degree at vertex " + std::to_string(v));
            sum += (uint64_t)deg[v];
            g->off[v + 1] = sum;
        }
    } else {
        std::vector<int64_t> deg(n);
        if ((st = read_exact(fd, deg.data(), 8 * n, "b_degree.bin degrees"))) return st;
        for (uint64_t v = 0; v < n; ++v) {
            if (deg[v] < 0) return fail(SCAN_ERR_FORMAT, "negative degree at vertex " + std::to_string(v));
            sum += (uint64_t)deg[v];
            g->off[v + 1] = sum;
        }
    }
    if (sum != m)
        return fail(SCAN_ERR_FORMAT, "b_degree.bin: degrees sum to " + std::to_string(sum) +
                                         " but the header says m = " + std::to_string(m));
    g->m = m;
    FILE* fa = std::fopen((d + "/b_adj.bin").c_str(), "rb");
    if (!fa) return fail(SCAN_ERR_IO, "cannot open " + d + "/b_adj.bin: " + std::strerror(errno));
    std::unique_ptr<FILE, int (*)(FILE*)> fa_guard(fa, std::fclose);
    try {
        g->adj.resize(m);
    } catch (...) { return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot allocate adjacency"); }
    if ((st = read_exact(fa, g->adj.data(), 4 * m, "b_adj.bin"))) return st;
    if ((st = scan_graph_validate(g.get(), 0))) return st;
    finish_graph(g.get());
    *out = g.release();
    return SCAN_OK;
}

scan_status scan_graph_save(const scan_graph* g, const char* dir) {
    clear_error();
    if (!g || !dir) return fail(SCAN_ERR_INVALID_ARG, "graph and dir must be non-null");
    std::string d(dir);
    FILE* fd = std::fopen((d + "/b_degree.bin").c_str(), "wb");
    if (!fd) return fail(SCAN_ERR_IO, "cannot create " + d + "/b_degree.bin: " + std::strerror(errno));
    bool wide = g->n > 0xFFFFFFFFull || g->m > 0xFFFFFFFFull || g->max_deg > 0x7FFFFFFFu;
    bool ok = true;
    if (!wide) {
        int32_t hdr[3] = {4, (int32_t)(uint32_t)g->n, (int32_t)(uint32_t)g->m};
        ok &= std::fwrite(hdr, 4, 3, fd) == 3;
        std::vector<int32_t> deg(g->n);
        for (uint64_t v = 0; v < g->n; ++v) deg[v] = (int32_t)(g->off[v + 1] - g->off[v]);
        ok &= std::fwrite(deg.data(), 4, g->n, fd) == g->n;
    } else {
        int32_t isz = 8;
        ok &= std::fwrite(&isz, 4, 1, fd) == 1;
        ok &= std::fwrite(&g->n, 8, 1, fd) == 1;
        ok &= std::fwrite(&g->m, 8, 1, fd) == 1;
        std::vector<int64_t> deg(g->n);
        for (uint64_t v = 0; v < g->n; ++v) deg[v] = (int64_t)(g->off[v + 1] - g->off[v]);
        ok &= std::fwrite(deg.data(), 8, g->n, fd) == g->n;
    }
    ok &= std::fclose(fd) == 0;
    if (!ok) return fail(SCAN_ERR_IO, "write failed for b_degree.bin");
    FILE* fa = std::fopen((d + "/b_adj.bin").c_str(), "wb");
    if (!fa) return fail(SCAN_ERR_IO, "cannot create " + d + "/b_adj.bin: " + std::strerror(errno));
    ok = std::fwrite(g->adj.data(), 4, g->m, fa) == g->m;
    ok &= std::fclose(fa) == 0;
    if (!ok) return fail(SCAN_ERR_IO, "write failed for b_adj.bin");
    return SCAN_OK;
}

scan_status scan_graph_from_csr(const uint64_t* offsets, const uint32_t* adj, uint64_t n, uint64_t m,
                                scan_graph** out) {
    clear_error();
    if (!offsets || (!adj && m) || !out || n == 0) return fail(SCAN_ERR_INVALID_ARG, "null array or n == 0");
    *out = nullptr;
    std::unique_ptr<scan_graph> g(new scan_graph());
    g->n = n;
    g->m = m;
    try {
        g->off.assign(offsets, offsets + n + 1);
        g->adj.assign(adj, adj + m);
    } catch (...) { return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot copy the CSR arrays"); }
    scan_status st = scan_graph_validate(g.get(), 0);
    if (st) return st;
    finish_graph(g.get());
    *out = g.release();
    return SCAN_OK;
}

scan_status scan_graph_from_csr32(const uint32_t* offsets, const uint32_t* adj, uint64_t n, uint64_t m,
                                  scan_graph** out) {
    clear_error();
    if (!offsets || !out || n == 0) return fail(SCAN_ERR_INVALID_ARG, "null array or n == 0");
    std::vector<uint64_t> off(offsets, offsets + n + 1);
    return scan_graph_from_csr(off.data(), adj, n, m, out);
}

void scan_graph_free(scan_graph* g) {
    if (!g) return;
    if (g->dev) device_graph_free(g->dev);
    delete g;
}

uint64_t scan_graph_num_vertices(const scan_graph* g) { return g ? g->n : 0; }
uint64_t scan_graph_num_directed(const scan_graph* g) { return g ? g->m : 0; }
uint32_t scan_graph_max_degree(const scan_graph* g) { return g ? g->max_deg : 0; }
const uint64_t* scan_graph_offsets(const scan_graph* g) { return g ? g->off.data() : nullptr; }
const uint32_t* scan_graph_adjacency(const scan_graph* g) { return g ? g->adj.data() : nullptr; }

scan_status scan_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                          scan_graph** out) {
    clear_error();
    if (!out || scale < 1 || scale > 31 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return fail(SCAN_ERR_INVALID_ARG, "bad R-MAT parameters");
    *out = nullptr;
    const uint64_t n = 1ull << scale;
    const uint64_t ne = (uint64_t)edge_factor * n;
    // Quadrant thresholds on a uniform 64-bit draw: [0,a) top-left, [a,a+b) top-right,
    // [a+b,a+b+c) bottom-left, rest bottom-right.
    auto thr = [](double x) { return x >= 1.0 ? ~0ull : (uint64_t)std::ldexp(x, 63) * 2; };
    const uint64_t ta = thr(a), tab = thr(a + b), tabc = thr(a + b + c);
    std::vector<uint64_t> pairs;
    try { pairs.resize(ne); } catch (...) { return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot allocate edge pairs"); }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)ne; ++i) {
        uint64_t s = stream_start(seed, (uint64_t)i);
        uint32_t u = 0, v = 0;
        for (int l = 0; l < scale; ++l) {
            uint64_t r = next64(s);
            uint32_t bu = r >= tab, bv = (r >= ta && r < tab) || r >= tabc;
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        pairs[i] = ((uint64_t)u << 32) | v;
    }
    std::unique_ptr<scan_graph> g(new scan_graph());
    scan_status st = build_from_pairs(n, pairs, g.get());
    if (st) return st;
    *out = g.release();
    return SCAN_OK;
}

scan_status scan_gen_chung_lu(uint64_t n, double exponent, uint64_t target_edges, uint64_t max_degree,
                              uint64_t seed, scan_graph** out) {
    clear_error();
    if (!out || n < 2 || n > 0xFFFFFFFFull || exponent <= 1.0 || target_edges == 0 || max_degree == 0)
        return fail(SCAN_ERR_INVALID_ARG, "bad Chung-Lu parameters");
    *out = nullptr;
    // Expected-degree weights w_i = (i+1)^(-1/(exponent-1)), scaled so sum w = 2*target
    // and capped at max_degree (re-scaling the uncapped part a few times).
    std::vector<double> w(n);
    const double alpha = 1.0 / (exponent - 1.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) w[i] = std::pow((double)(i + 1), -alpha);
    const double want = 2.0 * (double)target_edges;
    for (int it = 0; it < 8; ++it) {
        double capped = 0, free_sum = 0;
        for (uint64_t i = 0; i < n; ++i) {
            if (w[i] >= (double)max_degree) capped += (double)max_degree; else free_sum += w[i];
        }
        double k = (want - capped) / free_sum;
        if (!(k > 0)) break;
        for (uint64_t i = 0; i < n; ++i) w[i] = std::min(w[i] * k, (double)max_degree);
        if (std::fabs(k - 1.0) < 1e-9) break;
    }
    // Vose alias table over the weights.
    double total = 0;
    for (uint64_t i = 0; i < n; ++i) total += w[i];
    std::vector<uint64_t> prob(n);
    std::vector<uint32_t> alias(n);
    {
        std::vector<double> sc(n);
        std::vector<uint32_t> small, large;
        for (uint64_t i = 0; i < n; ++i) {
            sc[i] = w[i] * (double)n / total;
            (sc[i] < 1.0 ? small : large).push_back((uint32_t)i);
        }
        while (!small.empty() && !large.empty()) {
            uint32_t s = small.back(); small.pop_back();
            uint32_t l = large.back();
            prob[s] = sc[s] >= 1.0 ? ~0ull : (uint64_t)std::ldexp(sc[s], 63) * 2;
            alias[s] = l;
            sc[l] = (sc[l] + sc[s]) - 1.0;
            if (sc[l] < 1.0) { large.pop_back(); small.push_back(l); }
        }
        for (uint32_t i : large) { prob[i] = ~0ull; alias[i] = i; }
        for (uint32_t i : small) { prob[i] = ~0ull; alias[i] = i; }
    }
    std::vector<uint64_t> pairs;
    try { pairs.resize(target_edges); } catch (...) { return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot allocate edge pairs"); }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)target_edges; ++i) {
        uint64_t s = stream_start(seed, (uint64_t)i);
        uint32_t ends[2];
        for (int k = 0; k < 2; ++k) {
            uint64_t slot = bounded(next64(s), n);
            uint64_t coin = next64(s);
            ends[k] = coin < prob[slot] ? (uint32_t)slot : alias[slot];
        }
        pairs[i] = ((uint64_t)ends[0] << 32) | ends[1];
    }
    std::unique_ptr<scan_graph> g(new scan_graph());
    scan_status st = build_from_pairs(n, pairs, g.get());
    if (st) return st;
    *out = g.release();
    return SCAN_OK;
}

scan_status scan_gen_sbm(uint64_t n, uint32_t blocks, double p_in, double p_out, double max_avg_degree,
                         uint64_t seed, scan_graph** out) {
    clear_error();
    if (!out || n < 2 || n > 0xFFFFFFFFull || blocks == 0 || blocks > n || p_in < 0 || p_out < 0 ||
        p_in > 1 || p_out > 1 || max_avg_degree <= 0)
        return fail(SCAN_ERR_INVALID_ARG, "bad SBM parameters");
    *out = nullptr;
    const double s = (double)n / blocks;
    double avg = p_in * (s - 1) + p_out * ((double)n - s);
    if (avg > max_avg_degree) {
        double k = max_avg_degree / avg;
        p_in *= k;
        p_out *= k;
    }
    // Blocks are contiguous id ranges; block k holds [n*k/blocks, n*(k+1)/blocks).
    std::vector<uint64_t> bstart(blocks + 1);
    for (uint32_t k = 0; k <= blocks; ++k) bstart[k] = n * k / blocks;
    std::vector<uint64_t> cnt(blocks + 1, 0);
    uint64_t intra_total = 0;
    for (uint32_t k = 0; k < blocks; ++k) {
        double sz = (double)(bstart[k + 1] - bstart[k]);
        cnt[k] = (uint64_t)std::llround(p_in * sz * (sz - 1) / 2);
        intra_total += cnt[k];
    }
    double all_pairs = (double)n * (double)(n - 1) / 2, intra_pairs = 0;
    for (uint32_t k = 0; k < blocks; ++k) {
        double sz = (double)(bstart[k + 1] - bstart[k]);
        intra_pairs += sz * (sz - 1) / 2;
    }
    const uint64_t inter = (uint64_t)std::llround(p_out * (all_pairs - intra_pairs));
    std::vector<uint64_t> first(blocks + 1, 0);
    for (uint32_t k = 0; k < blocks; ++k) first[k + 1] = first[k] + cnt[k];
    std::vector<uint64_t> pairs(intra_total + inter);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < (int64_t)blocks; ++k) {
        uint64_t lo = bstart[k], sz = bstart[k + 1] - bstart[k];
        for (uint64_t i = 0; i < cnt[k]; ++i) {
            uint64_t st = stream_start(seed, first[k] + i);
            uint64_t u = lo + bounded(next64(st), sz), v = lo + bounded(next64(st), sz);
            pairs[first[k] + i] = (u << 32) | v;
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)inter; ++i) {
        uint64_t st = stream_start(seed ^ 0x5BD1E995ull, (uint64_t)i);
        uint64_t u = bounded(next64(st), n);
        uint64_t v = bounded(next64(st), n);
        pairs[intra_total + i] = (u << 32) | v;  // may land inside a block: a small p_in bump
    }
    std::unique_ptr<scan_graph> g(new scan_graph());
    scan_status st = build_from_pairs(n, pairs, g.get());
    if (st) return st;
    *out = g.release();
    return SCAN_OK;
}

scan_status scan_orient_reference(const scan_graph* g, uint32_t* eid, int32_t* edge_u, int32_t* edge_v) {
    clear_error();
    if (!g || !eid || !edge_u || !edge_v) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    const int64_t n = (int64_t)g->n;
    // hrank[j] = 1-based rank of entry j among u's "higher" neighbours, 0 if the
    // neighbour is lower.  Higher = larger degree, ties broken by larger id
    // (GPUSCAN++/Graph.cpp:66-85).
    std::vector<uint32_t> hrank(g->m);
    std::vector<uint32_t> hcount(n);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < n; ++u) {
        uint64_t du = g->off[u + 1] - g->off[u];
        uint32_t r = 0;
        for (uint64_t j = g->off[u]; j < g->off[u + 1]; ++j) {
            uint32_t v = g->adj[j];
            uint64_t dv = g->off[v + 1] - g->off[v];
            bool higher = dv > du || (dv == du && v > (uint32_t)u);
            hrank[j] = higher ? ++r : 0;
        }
        hcount[u] = r;
    }
    std::vector<uint64_t> pre(n + 1);
    exclusive_scan(hcount.data(), (uint64_t)n, pre.data());
    if (pre[n] * 2 != g->m) return fail(SCAN_ERR_FORMAT, "graph is not symmetric");
    std::atomic<int> bad{0};
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t u = 0; u < n; ++u) {
        for (uint64_t j = g->off[u]; j < g->off[u + 1]; ++j) {
            uint32_t v = g->adj[j];
            if (hrank[j]) {
                uint64_t e = pre[u] + hrank[j] - 1;
                eid[j] = (uint32_t)e;
                edge_u[e] = (int32_t)u;
                edge_v[e] = (int32_t)v;
            } else {
                auto b = g->adj.begin() + g->off[v], en = g->adj.begin() + g->off[v + 1];
                auto it = std::lower_bound(b, en, (uint32_t)u);
                if (it == en || *it != (uint32_t)u) { bad = 1; continue; }
                uint64_t pos = (uint64_t)(it - g->adj.begin());
                eid[j] = (uint32_t)(pre[v] + hrank[pos] - 1);
            }
        }
    }
    if (bad.load()) return fail(SCAN_ERR_FORMAT, "graph is not symmetric");
    return SCAN_OK;
}

scan_status scan_convert_edge_list(const char* edge_list_path, const char* out_dir, uint64_t* num_vertices,
                                   uint64_t* num_edges) {
    clear_error();
    if (!edge_list_path || !out_dir) return fail(SCAN_ERR_INVALID_ARG, "null path");
    FILE* f = std::fopen(edge_list_path, "rb");
    if (!f) return fail(SCAN_ERR_IO, std::string("cannot open ") + edge_list_path + ": " + std::strerror(errno));
    std::unique_ptr<FILE, int (*)(FILE*)> guard(f, std::fclose);
    std::vector<uint64_t> pairs;
    uint64_t max_second = 0;
    bool any = false;
    std::vector<char> buf(1 << 20);
    std::string carry;
    auto parse_line = [&](const char* b, const char* e) -> bool {
        // "# ..." comment lines are skipped; otherwise two integers.  Lines with
        // first >= second are dropped (self-loops, and the second copy of each edge),
        // exactly as csr_convert/EdgeListToBinsConverter.cpp:28-46 does.
        while (b < e && (*b == ' ' || *b == '\t')) ++b;
        if (b == e || *b == '#' || *b == '\r') return true;
        uint64_t v[2];
        for (int k = 0; k < 2; ++k) {
            while (b < e && (*b == ' ' || *b == '\t' || *b == ',')) ++b;
            if (b == e || *b < '0' || *b > '9') return false;
            uint64_t x = 0;
            while (b < e && *b >= '0' && *b <= '9') {
                x = x * 10 + (uint64_t)(*b - '0');
                if (x > 0x7FFFFFFEull) return false;
                ++b;
            }
            v[k] = x;
        }
        if (v[0] >= v[1]) return true;
        pairs.push_back((v[0] << 32) | v[1]);
        if (v[1] > max_second) max_second = v[1];
        any = true;
        return true;
    };
    uint64_t line_no = 0;
    size_t got;
    while ((got = std::fread(buf.data(), 1, buf.size(), f)) > 0) {
        const char* p = buf.data();
        const char* end = p + got;
        while (p < end) {
            const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
            if (!nl) { carry.append(p, end); break; }
            ++line_no;
            bool ok;
            if (!carry.empty()) {
                carry.append(p, nl);
                ok = parse_line(carry.data(), carry.data() + carry.size());
                carry.clear();
            } else {
                ok = parse_line(p, nl);
            }
            if (!ok) return fail(SCAN_ERR_FORMAT, "edge list line " + std::to_string(line_no) + " is not two vertex ids");
            p = nl + 1;
        }
    }
    if (!carry.empty() && !parse_line(carry.data(), carry.data() + carry.size()))
        return fail(SCAN_ERR_FORMAT, "last edge list line is not two vertex ids");
    if (!any) return fail(SCAN_ERR_FORMAT, "edge list has no edge with first < second");
    const uint64_t n = max_second + 1;   // the converter's vertex count (largest second id + 1)
    scan_graph g;
    scan_status st = build_from_pairs(n, pairs, &g);
    if (st) return st;
    st = scan_graph_save(&g, out_dir);
    if (st) return st;
    if (num_vertices) *num_vertices = g.n;
    if (num_edges) *num_edges = g.m / 2;
    return SCAN_OK;
}

uint64_t scan_count_clusters(const int32_t* label, uint64_t n) {
    if (!label || n == 0) return 0;
    std::vector<uint8_t> seen(n, 0);
    for (uint64_t i = 0; i < n; ++i)
        if (label[i] >= 0 && (uint64_t)label[i] < n) seen[label[i]] = 1;
    uint64_t c = 0;
    for (uint64_t i = 0; i < n; ++i) c += seen[i];
    return c;
}

scan_status scan_eps_to_decimal(double eps, char* buf, size_t buflen) {
    if (!buf || buflen < 32 || !std::isfinite(eps)) return fail(SCAN_ERR_INVALID_ARG, "bad eps or buffer");
    for (int prec = 1; prec <= 17; ++prec) {
        std::snprintf(buf, buflen, "%.*g", prec, eps);
        if (std::strtod(buf, nullptr) == eps) return SCAN_OK;
    }
    return SCAN_OK;
}

}  // extern "C"
