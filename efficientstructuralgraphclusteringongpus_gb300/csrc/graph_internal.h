// Internal host-side declarations shared by the C++ and CUDA translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "scan_gb300.h"

struct DeviceGraph;  // defined in scan_device.cu

struct scan_graph {
    uint64_t n = 0;
    uint64_t m = 0;                 // directed adjacency entries (2 * undirected edges)
    std::vector<uint64_t> off;      // n + 1
    std::vector<uint32_t> adj;      // m, each list sorted strictly ascending
    uint32_t max_deg = 0;
    DeviceGraph* dev = nullptr;     // resident device copy, or null
};

namespace scan {

// Records `msg` as the calling thread's last error and returns `s`.
scan_status fail(scan_status s, const std::string& msg);
void clear_error();

// Builds a validated graph from undirected pairs: drops self-loops, symmetrises,
// deduplicates and sorts each list.  `pairs` holds (u << 32 | v) and is consumed.
scan_status build_from_pairs(uint64_t n, std::vector<uint64_t>& pairs, scan_graph* g);

// Recomputes max_deg from the offsets.
void finish_graph(scan_graph* g);

// Frees the device-side state of a graph (defined in scan_device.cu).
void device_graph_free(DeviceGraph* d);

// Decimal text -> reduced fraction p/q with q <= 10^18 (no rounding); false on bad text.
bool parse_decimal(const char* text, uint64_t* p, uint64_t* q, double* as_double);

}  // namespace scan
