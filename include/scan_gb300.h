/*
 * scan_gb300.h -- C-ABI of the GB300-native SCAN structural graph clustering engine.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns a
 * scan_status (never calls exit()), and records a message for scan_last_error().
 *
 * Reference interfaces replaced (paths are inside the GPUSCAN++ project):
 *   Graph::Graph(char*)            GPUSCAN++/Graph.cpp:147-153   -> scan_graph_load
 *   Graph::ReadDegree/ReadAdj...   GPUSCAN++/Graph.cpp:157-223   -> scan_graph_load
 *   Graph::CheckInputGraph         GPUSCAN++/Graph.cpp:270-288   -> scan_graph_validate
 *   getEidAndEdgeList              GPUSCAN++/Graph.cpp:52-141    -> scan_orient_reference
 *   GPUScan(graph_t*,int*,int*,double,int)
 *                                  GPUSCAN++/GPUScan.h:7,
 *                                  GPUSCAN++/GPUScan.cu:800-1009 -> scan_run / scan_gpuscan_compat
 *                                                                   (and the C++-linkage GPUScan
 *                                                                   symbol in gpuscan_compat.h)
 *   main's cluster count           GPUSCAN++/main.cpp:83-111     -> scan_count_clusters
 *   csr_convert output format      csr_convert/EdgeListToBinsConverter.cpp:85-121
 *                                                                -> scan_graph_save
 *
 * Output encoding of label[] follows the reference's role array (GPUSCAN++/GPUScan.cu:124-127,
 * 780, 986): label >= 0 is a cluster id (the smallest core id of the cluster), -1 a hub,
 * -2 an outlier.  role[] adds what the reference array cannot show: core vs border.
 */
#ifndef SCAN_GB300_H
#define SCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum scan_status {
    SCAN_OK = 0,
    SCAN_ERR_INVALID_ARG = 1,   /* null pointer, eps/mu out of range, bad option            */
    SCAN_ERR_IO = 2,            /* file missing, short read, write failure                  */
    SCAN_ERR_FORMAT = 3,        /* header/size mismatch, self-loop, unsorted or duplicate    */
    SCAN_ERR_CUDA = 4,          /* a CUDA runtime call failed                                */
    SCAN_ERR_OUT_OF_MEMORY = 5, /* host or device allocation failed, or over the budget      */
    SCAN_ERR_TOO_LARGE = 6,     /* graph exceeds the engine's index width (m >= 2^32)        */
    SCAN_ERR_DEVICE = 7         /* a device-side check failed (bounded wait ran out, etc.)   */
} scan_status;

/* epsilon-similarity predicate.
 * SCAN_PRED_REF_F64 reproduces the reference's IEEE double expressions with their operand
 * order (GPUSCAN++/GPUScan.cu:145, 156, 220-221), so results are bit-identical to it.
 * SCAN_PRED_EXACT evaluates (cn+2)^2 * q^2 >= p^2 * (du+1) * (dv+1) in 128-bit integers,
 * with eps = p/q read exactly from the decimal string. */
typedef enum scan_predicate {
    SCAN_PRED_EXACT = 0,
    SCAN_PRED_REF_F64 = 1
} scan_predicate;

/* Per-vertex role (out_role).  Core and border both carry a cluster id in label[]. */
typedef enum scan_role {
    SCAN_ROLE_OUTLIER = 0,
    SCAN_ROLE_HUB = 1,
    SCAN_ROLE_BORDER = 2,
    SCAN_ROLE_CORE = 3
} scan_role;

typedef struct scan_graph scan_graph;   /* host CSR, optionally resident on the device */

/* Per-run statistics; every time is device time from CUDA events on the run's stream. */
typedef struct scan_stats {
    uint64_t n;                 /* vertices                                                  */
    uint64_t num_edges;         /* undirected edges E (= m/2)                                */
    uint64_t num_cores;
    uint64_t num_clusters;
    uint64_t num_hubs;
    uint64_t num_outliers;
    uint64_t num_borders;
    uint64_t num_similar_edges; /* undirected edges with sigma >= eps                        */
    uint64_t pred_disagreements;/* edges where the exact and ref-f64 predicates differ        */
    uint64_t multi_cluster_borders; /* border vertices similar to cores of >= 2 clusters      */
    double ms_h2d;              /* host->device copies (0 when the graph is already resident) */
    double ms_orient;           /* lower-list construction                                    */
    double ms_similarity;       /* common-neighbour counting + predicate (the hot kernel)     */
    double ms_cluster;          /* core flags, union-find, attach, hub/outlier                */
    double ms_d2h;              /* result copies                                              */
    double ms_total;            /* first event to last event of the run                       */
    double ms_cn_kernel[5];     /* similarity-stage kernels: small pivots; the three hash-table
                                   classes (1024 / 4096 / chunk entries); the hubs (mid hubs
                                   and larger hubs together).  The hubs run on a second stream
                                   beside the others, so these intervals overlap: each is its
                                   kernel's span on its own stream                             */
    uint64_t cn_work_items[5];  /* pivots (small class) or tasks (the others) of each           */
    uint32_t kernel_launches;   /* kernels this library launched for the run                  */
    uint32_t reserved;
    uint64_t cn_words;          /* 16-byte list words the similarity kernels read (0 when the
                                   cached counts were used)                                  */
    uint64_t cn_edges_counted;  /* edges whose lower list was read: all of them for the cached
                                   counts, those the degree prune leaves in a one-shot run   */
} scan_stats;

/* ---- errors ------------------------------------------------------------------------- */
/* Message of the last failing call on this host thread ("" if none). */
const char* scan_last_error(void);
const char* scan_status_string(scan_status s);
/* Library version as "major.minor.patch". */
const char* scan_version(void);

/* ---- graphs ------------------------------------------------------------------------- */
/* Read <dir>/b_degree.bin and <dir>/b_adj.bin (format written by csr_convert; a header
 * int_size of 8 selects the 64-bit extension with uint64 n and m), then validate them. */
scan_status scan_graph_load(const char* dir, scan_graph** out);
/* Write the graph in the same two-file format (int_size 4 when n and m fit 32 bits). */
scan_status scan_graph_save(const scan_graph* g, const char* dir);
/* Build from caller CSR arrays (offsets n+1 entries, adjacency m entries).  The arrays
 * are copied.  The graph is validated (sorted strictly ascending, no self-loops, ids < n). */
scan_status scan_graph_from_csr(const uint64_t* offsets, const uint32_t* adj,
                                uint64_t n, uint64_t m, scan_graph** out);
/* Same, with 32-bit offsets as in the reference's graph_t (GPUSCAN++/Graph.h:20-27). */
scan_status scan_graph_from_csr32(const uint32_t* offsets, const uint32_t* adj,
                                  uint64_t n, uint64_t m, scan_graph** out);
void scan_graph_free(scan_graph* g);
uint64_t scan_graph_num_vertices(const scan_graph* g);
uint64_t scan_graph_num_directed(const scan_graph* g);      /* m = 2E */
uint32_t scan_graph_max_degree(const scan_graph* g);
/* Borrow the host CSR arrays (valid until scan_graph_free). */
const uint64_t* scan_graph_offsets(const scan_graph* g);
const uint32_t* scan_graph_adjacency(const scan_graph* g);
/* Re-run the input checks of CheckInputGraph; check_symmetry adds an O(m log d) check. */
scan_status scan_graph_validate(const scan_graph* g, int check_symmetry);

/* Copy the CSR to device `device` and keep it there (plus the lower-list orientation),
 * so later scan_run calls start with inputs resident in HBM. */
scan_status scan_graph_upload(scan_graph* g, int device);
/* Streamed residency for graphs above a device-memory budget: the adjacency (the only
 * O(m) array the kernels gather from) stays in pinned, GPU-mapped host memory and is read
 * over the host link; offsets, orientation, counts and run scratch go to the device.  Fails
 * with SCAN_ERR_OUT_OF_MEMORY if the device part exceeds device_budget_bytes (0: no cap).
 * Later scan_run / scan_common_neighbors calls use this copy.  This is the GB300 form of the
 * reference's managed-memory and out-of-core variants (GPUSCAN++UVM/SCANum.cu:725-741,
 * GPUSCAN++O/SCANoffload.cu:976-1438). */
scan_status scan_graph_upload_streamed(scan_graph* g, int device, uint64_t device_budget_bytes,
                                       uint64_t* device_bytes_used);
/* Device memory held by the graph's resident copy (0 if none). */
uint64_t scan_graph_device_bytes(const scan_graph* g);
/* Drop the device copy (the host copy stays). */
scan_status scan_graph_release_device(scan_graph* g);
/* Device buffers of freed graphs (and of each drop-in GPUScan() call) are kept per device,
 * up to a limit, and reused by later uploads of similar size: cudaMalloc and cudaFree cost
 * milliseconds at GB sizes and cudaFree synchronises the whole device.  The memory stays
 * allocated to this process while cached.  The limit is 8 GiB per device by default.
 * scan_release_cached_memory returns every cached buffer to the driver;
 * scan_set_cached_memory_limit sets the limit (0 disables the cache) and frees cached buffers
 * above it; scan_cached_memory_bytes reports what is cached on `device`. */
void scan_release_cached_memory(void);
void scan_set_cached_memory_limit(uint64_t bytes);
uint64_t scan_cached_memory_bytes(int device);

/* ---- generators (deterministic for a seed on every platform) ------------------------ */
/* R-MAT: 2^scale vertices, edge_factor*2^scale sampled pairs with quadrant probabilities
 * a, b, c (d = 1-a-b-c); symmetrised, deduplicated, self-loops removed, lists sorted. */
scan_status scan_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                          uint64_t seed, scan_graph** out);
/* Chung-Lu: power-law expected degrees w_i ~ (i+1)^(-1/(exponent-1)), scaled to
 * ~target_edges undirected edges and capped at max_degree. */
scan_status scan_gen_chung_lu(uint64_t n, double exponent, uint64_t target_edges,
                              uint64_t max_degree, uint64_t seed, scan_graph** out);
/* Stochastic block model with `blocks` equal communities, edge probabilities p_in/p_out,
 * scaled down so the expected average degree is at most max_avg_degree. */
scan_status scan_gen_sbm(uint64_t n, uint32_t blocks, double p_in, double p_out,
                         double max_avg_degree, uint64_t seed, scan_graph** out);

/* ---- reference-compatible orientation ------------------------------------------------ */
/* getEidAndEdgeList (GPUSCAN++/Graph.cpp:52-141): eid[m] gives both directions of an
 * undirected edge the same id; edge_u[E]/edge_v[E] hold the lower/higher endpoint in
 * (degree, id) order; ids are grouped by the lower endpoint. */
scan_status scan_orient_reference(const scan_graph* g, uint32_t* eid, int32_t* edge_u,
                                  int32_t* edge_v);

/* ---- the SCAN pipeline ------------------------------------------------------------- */
/* Run SCAN(eps, mu) on device `device` (the graph is uploaded first if it is not resident
 * there).  eps_decimal is the decimal text of epsilon ("0.5"), mu >= 1.
 * out_label[n]: cluster id (smallest core id of the cluster) / -1 hub / -2 outlier.
 * out_role[n] (may be NULL): scan_role values.  stats (may be NULL).
 * Border vertices similar to cores of several clusters get the smallest such cluster id
 * (the reference keeps whichever write lands last, GPUSCAN++/GPUScan.cu:716,722). */
scan_status scan_run(scan_graph* g, int device, const char* eps_decimal, int mu,
                     scan_predicate predicate, int32_t* out_label, uint8_t* out_role,
                     scan_stats* stats);

/* Autotune the similarity stage of the resident graph (uploading it first), timing full
 * counts: a coordinate search over the small-pivot intersection strategy (lists counted one
 * at a time through a hash table, a batch's lists streamed through it, or streamed with
 * binary search in the sorted list) and degree cut, the task size
 * and largest table chunk, the long-list threshold, and the degree above which pivots take
 * the hub path.  The fastest plan is kept for later runs.  Outputs may be NULL. */
scan_status scan_graph_autotune(scan_graph* g, int device, double* best_similarity_ms,
                                uint32_t* long_words, uint64_t* target_probes);

/* The plan the similarity stage of a resident graph uses (after scan_graph_autotune, the
 * tuned one): small-pivot degree cut, small-pivot strategy (0 serial hash table, 1 batched
 * hash table, 2 batched binary search), hub degree threshold, largest table chunk.  Outputs
 * may be NULL. */
scan_status scan_graph_plan(const scan_graph* g, uint32_t* small_deg, uint32_t* small_strategy,
                            uint32_t* hub_min_deg, uint32_t* chunk_max);
/* Set that plan explicitly (uploading the graph first), e.g. to pin a plan tuned earlier:
 * small_deg in [1, 128], small_strategy 0-2, hub_min_deg >= small_deg, chunk_max 6144 or
 * 12288.  Every plan gives the same results. */
scan_status scan_graph_set_plan(scan_graph* g, int device, uint32_t small_deg, uint32_t small_strategy,
                                uint32_t hub_min_deg, uint32_t chunk_max);

/* Exact common-neighbour count of every undirected edge, in the reference's edge order
 * (the eid / edge_u / edge_v order of scan_orient_reference): out_cn[E]. */
scan_status scan_common_neighbors(scan_graph* g, int device, uint32_t* out_cn,
                                  scan_stats* stats);

/* Every (cluster, vertex) membership pair: cores once, borders once per cluster they are
 * similar to.  Pairs are sorted by (cluster, vertex).  *num_pairs receives the count; if
 * capacity is smaller, nothing is written past it and SCAN_ERR_INVALID_ARG is returned. */
scan_status scan_memberships(scan_graph* g, int device, const char* eps_decimal, int mu,
                             scan_predicate predicate, int32_t* out_cluster,
                             int32_t* out_vertex, uint64_t capacity, uint64_t* num_pairs);

/* Drop-in for GPUScan (GPUSCAN++/GPUScan.h:7): host CSR in, malloc'd int[n] out that the
 * caller frees with free().  eid/edge_u/edge_v are accepted for signature parity and not
 * read (the engine orients the graph on the device).  Uses the ref-f64 predicate on
 * device 0.  Returns NULL on failure (see scan_last_error()). */
int32_t* scan_gpuscan_compat(int64_t n, int64_t m, const int32_t* adj,
                             const uint32_t* num_edges, const uint32_t* eid,
                             const int32_t* edge_u, const int32_t* edge_v, double eps,
                             int mu);

/* ---- batched SCAN: many graphs with their own (eps, mu) in one pass ------------------
 * No counterpart in the reference (it runs one graph per process).  The graphs become one
 * disjoint union on the device; one set of kernels covers all of them, captured once into a
 * CUDA graph and replayed per run.  When no pivot is split, the pass is a single run's
 * one-shot path (degree prune, early stop, predicate fused into the counting), each pivot
 * taking eps and the predicate from its own graph.  With autotune != 0 the first run times
 * the plan settings of scan_graph_autotune on this batch with its parameters and keeps the
 * fastest before it captures the pass.  Results equal scan_run per graph. */
typedef struct scan_batch scan_batch;

typedef struct scan_batch_stats {
    double ms_device;           /* the graph launch (similarity + cluster stages), CUDA events */
    double ms_total;            /* host wall time of the call, copies and split included       */
    uint64_t num_graphs, num_vertices, num_edges, num_cores, num_clusters;
    uint32_t graph_kernels;     /* kernels inside the captured graph                          */
    uint32_t long_words;        /* tuned long-list threshold (16-byte words)                  */
    uint64_t target_probes;     /* tuned probe work per task                                  */
    double tuned_similarity_ms; /* similarity time of the chosen setting (0 if not tuned)     */
    uint32_t small_deg;         /* plan: small-pivot degree cut                                 */
    uint32_t small_strategy;    /* plan: small-pivot intersection, 0 serial hash table, 1 a
                                   batch's lists streamed through the table, 2 streamed with
                                   binary search in the sorted list                            */
    uint32_t hub_min_deg;       /* plan: pivots above this degree take the hub path              */
    uint32_t chunk_max;         /* plan: entries per table of the largest hash class             */
} scan_batch_stats;

scan_status scan_batch_create(const scan_graph* const* graphs, uint32_t count, int device,
                              int autotune, scan_batch** out);
/* eps_decimal[i], mu[i]: graph i's parameters.  out_labels[i] (n_i entries) and out_roles[i]
 * (may be NULL) receive graph i's result in its own vertex ids. */
scan_status scan_batch_run(scan_batch* b, const char* const* eps_decimal, const int32_t* mu,
                           scan_predicate predicate, int32_t* const* out_labels,
                           uint8_t* const* out_roles, scan_batch_stats* stats);
void scan_batch_free(scan_batch* b);

/* ---- serving: queries on resident graphs with cached common-neighbour counts ---------
 * A request loop over resident graphs; the reference has no serving loop.  Each graph
 * added is uploaded once and its exact cn[] computed once; a query (graph, eps, mu) then runs
 * only the cluster stage.  Queries are admitted in arrival order when one of max_in_flight
 * stream slots is free and their scratch fits memory_budget_bytes (reserved on the device at
 * creation); admitted queries run concurrently on their own streams.  Results are identical
 * to scan_run on the same graph and parameters, alone or in any mix. */
typedef struct scan_server scan_server;

typedef struct scan_query_result {
    uint64_t ticket;
    int32_t status;             /* scan_status of the query                                 */
    uint32_t graph_id;
    double queue_ms;            /* submitted -> admitted                                    */
    double latency_ms;          /* submitted -> result in the caller's buffers               */
    double device_ms;           /* cluster stage and result copy on the device (CUDA events)  */
    uint64_t num_cores;
    uint64_t num_clusters;
    uint64_t num_similar_edges;
} scan_query_result;

typedef struct scan_server_counters {
    uint64_t submitted, admitted, completed, failed;
    uint64_t pending, in_flight, graphs, budget_bytes;
    uint64_t kernel_launches;
} scan_server_counters;

scan_status scan_server_create(int device, uint64_t memory_budget_bytes, uint32_t max_in_flight,
                               scan_server** out);
/* Upload g and compute its common-neighbour counts; g may be freed afterwards.  Safe from
 * several threads and while queries run: a graph larger than any before it grows the pinned
 * result staging, which pauses admission until the running queries finish (one grow at a
 * time). */
scan_status scan_server_add_graph(scan_server* s, const scan_graph* g, uint32_t* graph_id);
/* Queue a query; out_label[n] (and out_role[n], may be NULL) are written before the ticket
 * completes.  Returns at once. */
scan_status scan_server_submit(scan_server* s, uint32_t graph_id, const char* eps_decimal, int mu,
                               scan_predicate predicate, int32_t* out_label, uint8_t* out_role,
                               uint64_t* ticket);
/* Block until the ticket completes; returns its status and releases the ticket. */
scan_status scan_server_wait(scan_server* s, uint64_t ticket, scan_query_result* result);
scan_status scan_server_poll(scan_server* s, uint64_t ticket, int* done);
scan_status scan_server_get_counters(scan_server* s, scan_server_counters* out);
/* Load replay: submits query i at arrival_ms[i] after the call starts (one thread sleeps and
 * spins to the arrival times) while this thread collects results in order.  Fills
 * latency_ms[i] (submit -> result) and status[i]; *wall_ms (may be NULL) is first arrival ->
 * last result.  Labels go to internal per-graph buffers: this measures time, not output. */
scan_status scan_server_replay(scan_server* s, uint64_t num_queries, const uint32_t* graph_id,
                               const char* const* eps_decimal, const int32_t* mu,
                               const int32_t* predicate, const double* arrival_ms,
                               double* latency_ms, int32_t* status, double* wall_ms);
/* Finishes queued and running queries, then frees everything. */
void scan_server_destroy(scan_server* s);

/* ---- core check without device allocation ------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device memory
 * themselves: a plugin or custom call whose host framework owns all device memory and only
 * hands buffers in, a process whose HBM is already committed to resident graphs, or code
 * that must avoid cudaMalloc/cudaFree because they synchronise the whole device.
 * Every buffer is the caller's device memory: d_offsets[n+1]; the undirected edges
 * d_edge_u/d_edge_v[num_edges] (each edge once, either orientation) with their common-
 * neighbour counts d_cn[num_edges], e.g. from scan_common_neighbors and
 * scan_orient_reference.  d_is_core[n] receives 1 for a core and 0 otherwise -- the same
 * answer as role == SCAN_ROLE_CORE from scan_run.  Work is queued on `stream` (a
 * cudaStream_t; NULL is the default stream) of the current device and the call returns
 * before it completes.  The per-vertex scratch is a fixed array built into the library
 * (4 MiB on every GPU that loads it, held until the process exits), so n above 2^20
 * returns SCAN_ERR_TOO_LARGE.  The first call on a device looks up that array's address:
 * make it before any stream capture (a captured first call returns SCAN_ERR_INVALID_ARG).
 * Calls on a stream that is not being captured look the address up again, so a
 * cudaDeviceReset between calls is harmless.  All calls share the one array and it keeps the last
 * call's contents (each call clears what it needs): calls that overlap on the GPU -- other
 * streams, other host threads -- race and give wrong results, so serialise them. */
scan_status scan_cores_noalloc(const uint32_t* d_offsets, uint32_t n, const uint32_t* d_edge_u,
                               const uint32_t* d_edge_v, const uint32_t* d_cn,
                               uint64_t num_edges, const char* eps_decimal, int mu,
                               scan_predicate predicate, uint8_t* d_is_core, void* stream);

/* Edge-list text -> <out_dir>/b_degree.bin + b_adj.bin, as csr_convert does
 * (csr_convert/EdgeListToBinsConverter.cpp:22-121): lines starting with '#' are skipped,
 * lines "first second" with first >= second are dropped (so each edge is taken from its
 * first < second copy), n = largest second id + 1, lists sorted and symmetric.  Unlike the
 * converter, repeated lines are merged (its output would fail its own loader's check). */
scan_status scan_convert_edge_list(const char* edge_list_path, const char* out_dir,
                                   uint64_t* num_vertices, uint64_t* num_edges);

/* Number of distinct labels >= 0, as printed by the reference CLI (main.cpp:83-111). */
uint64_t scan_count_clusters(const int32_t* label, uint64_t n);

/* Shortest decimal text that reads back as `eps` (so 0.4 -> "0.4"); buf >= 32 bytes. */
scan_status scan_eps_to_decimal(double eps, char* buf, size_t buflen);

/* ---- testing -------------------------------------------------------------------------
 * No counterpart in the reference.  Shrinks the limits of the engine's bounded device loops
 * so that tests can make them give up: union_find_iterations CAS attempts per union (default
 * 1 << 20; 0 makes every core-core union fail), and at most jump_rounds_cap pointer-jumping
 * rounds in the flatten (default enough for any depth; at least 1).  A negative value
 * restores the default.  A run whose loop gives up returns SCAN_ERR_DEVICE (a served query
 * completes with that status); the device stays usable.  Applies to work queued after the
 * call, process-wide; a batch keeps the rounds it was captured with. */
void scan_set_loop_limits(int64_t union_find_iterations, int32_t jump_rounds_cap);

#ifdef __cplusplus
}
#endif

#endif /* SCAN_GB300_H */
