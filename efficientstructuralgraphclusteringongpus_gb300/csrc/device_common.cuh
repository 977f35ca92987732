// Shared device helpers and the resident-graph layout.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace scan {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;   // empty hash slot / "no label"
constexpr int kWarp = 32;

// Per-vertex role codes used on the device (same values as scan_role).
constexpr uint8_t kRoleOutlier = 0, kRoleHub = 1, kRoleBorder = 2, kRoleCore = 3;

// Degree-order relation used for orientation: u precedes v when it has the smaller degree,
// ties broken by the smaller id.  The same relation decides Edge_u (lower) and Edge_v
// (higher) in the reference (GPUSCAN++/Graph.cpp:75-83).
__device__ __forceinline__ bool precedes(uint32_t du, uint32_t u, uint32_t dv, uint32_t v) {
    return du < dv || (du == dv && u < v);
}

// Fibonacci multiply then multiply-high range reduction: a slot in [0, cap) for any cap.
__device__ __forceinline__ uint32_t hash_slot(uint32_t w, uint32_t cap) {
    return __umulhi(w * 0x9E3779B1u, cap);
}

constexpr int kNumBigClasses = 3;           // hash-table classes of the similarity kernel
constexpr int kMaxJumpRounds = 40;          // pointer-jumping rounds of the union-find flatten

// Error flags written by bounded device loops.
constexpr uint32_t kErrUnionFindLimit = 1u;
constexpr uint32_t kErrHashFull = 2u;

// Device counters gathered by the final per-vertex pass (copied back with the labels).
struct RunCounters {
    unsigned long long cores, clusters, hubs, outliers, borders;
    unsigned long long similar_edges, disagreements, multi_borders;
    uint32_t error_flags;
    uint32_t any_core;      // set by k_core_init: the edge passes after it return at once when 0
    uint32_t any_member;    // set by k_label: the hub test's edge pass returns at once when 0
    uint32_t pad;
};

}  // namespace scan
