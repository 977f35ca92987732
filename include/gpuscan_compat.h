/*
 * gpuscan_compat.h -- the reference's own entry point, with C++ linkage, so a program
 * written against GPUSCAN++/GPUScan.h:7 links against libscan_gb300.so unchanged.
 *
 *   int* GPUScan(graph_t* g, int* Edge_u, int* Edge_v, double eps, int miu);
 *
 * graph_t has the layout of GPUSCAN++/Graph.h:20-27 (same members, same order), so the
 * mangled symbol is identical.  Semantics follow GPUSCAN++/GPUScan.cu:800-1009: device 0,
 * the reference's double-precision eps test, a malloc'd int[n] the caller releases with
 * free().  Differences: Edge_u, Edge_v and g->eid are accepted but not read (the engine
 * orients the graph on the device); on error it prints the reason to stderr and returns
 * NULL instead of calling exit(); mu must be >= 1.
 */
#ifndef GPUSCAN_COMPAT_H
#define GPUSCAN_COMPAT_H

#include "scan_gb300.h"

#ifndef SCAN_GRAPH_T_DEFINED
#define SCAN_GRAPH_T_DEFINED
typedef int vid_t;
typedef unsigned int eid_t;
typedef struct {
    long n;
    long m;
    vid_t* adj;
    eid_t* num_edges;
    eid_t* eid;
} graph_t;
#endif

int* GPUScan(graph_t* g, int* Edge_u, int* Edge_v, double eps, int miu);

#endif /* GPUSCAN_COMPAT_H */
