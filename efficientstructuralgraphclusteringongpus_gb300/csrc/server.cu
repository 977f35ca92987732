// Serving loop: (graph, eps, mu) queries on resident graphs with cached common-neighbour
// counts, continuously batched.
//
// Each graph added to a server is uploaded once and its exact cn[] computed once (eps- and
// mu-independent).  A query then needs only the cluster stage (predicate, cores,
// union-find, attach, classify: kernels_cluster.cuh), a few milliseconds at most, instead
// of the full recompute whose similarity kernel dominates.
//
// Continuous batching: a scheduler thread admits queued queries in arrival order whenever
// a stream slot is free and the query's scratch fits the memory budget (an arena carved
// out of one device allocation made at creation; no allocation while serving).  Admitted
// queries run on their own streams, so their kernels overlap on the device; a host
// callback queued after each query's result copy wakes the scheduler, which hands the
// result to the caller, returns the arena block and admits the next queries.  Queries
// that arrive while others run are admitted as slots and memory free up.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device_graph.h"

using namespace scan;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// First-fit allocator over [0, size) with coalescing; 256-byte granules.
class Arena {
  public:
    void reset(uint64_t size) {
        free_.clear();
        if (size) free_[0] = size;
        size_ = size;
    }
    bool alloc(uint64_t bytes, uint64_t* off) {
        bytes = (bytes + 255) & ~uint64_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const uint64_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                return true;
            }
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = (bytes + 255) & ~uint64_t(255);
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t size() const { return size_; }

  private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t size_ = 0;
};

struct Query {
    uint64_t ticket = 0;
    uint32_t gid = 0;
    DeviceGraph* graph = nullptr;    // captured under the lock at submission
    PredParams pp{};
    int mu = 0;
    int32_t* out_label = nullptr;
    uint8_t* out_role = nullptr;
    Clock::time_point submitted, admitted, finished;
    bool done = false;
    scan_status status = SCAN_OK;
    std::string error;
    RunCounters counters{};
    float device_ms = 0.f;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;
    Query* q = nullptr;
    uint64_t arena_off = 0, arena_bytes = 0;
    // Pinned staging.  The run scratch keeps label[n] and role[n] adjacent (label padded
    // to 256 bytes), and the counters next to the round flags, so each pair comes back in
    // one copy: h_res holds label then role at res_role_offset(n); h_tail the counters
    // then the flags at kTailFlags.
    char* h_res = nullptr;           // capacity for n_cap vertices
    char* h_tail = nullptr;
    uint32_t n_cap = 0;
    std::atomic<bool> gpu_done{false};
    bool launching = false;          // assigned to q, CUDA work being queued (outside the lock)
    bool finishing = false;          // results being copied out (outside the lock)
};

}  // namespace

struct scan_server {
    int device = 0;
    char* arena_base = nullptr;
    Arena arena;
    std::vector<DeviceGraph*> graphs;
    std::vector<Slot> slots;
    std::deque<Query*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Query>> queries;
    uint64_t next_ticket = 1;
    std::mutex mu;
    std::condition_variable cv_work;   // scheduler: new query or a slot finished
    std::condition_variable cv_done;   // waiters: a query finished
    std::thread worker;                // the scheduler
    // Workers queue each admitted query's CUDA work and copy finished results out, several
    // at a time: one thread issuing a dozen CUDA calls per query capped the served rate.
    std::vector<std::thread> workers;
    std::deque<std::pair<bool, Slot*>> jobs;   // (launch, slot): launch, or copy out and free
    std::condition_variable cv_jobs;
    bool stop_workers = false;
    bool stop = false;
    bool mem_blocked = false;          // the queue head waits for arena space to be returned
    bool pause_admission = false;      // a graph is being added
    bool growing = false;              // one add_graph call is reallocating the result staging
    scan_server_counters totals{};
};

namespace {

// Runs on the CUDA callback thread.  It only flips an atomic flag and wakes the scheduler;
// the brief lock makes the wake-up race-free (the scheduler tests its predicate under the
// lock).  No thread holds the lock while it is inside a CUDA call, so this never waits on
// a thread that is itself waiting for the device.
void CUDART_CB on_slot_done(void* arg) {
    auto* pair = static_cast<std::pair<scan_server*, Slot*>*>(arg);
    scan_server* s = pair->first;
    pair->second->gpu_done.store(true);
    { std::lock_guard<std::mutex> lock(s->mu); }
    s->cv_work.notify_one();
    delete pair;
}

size_t pad256(size_t x) { return (x + 255) & ~size_t(255); }
size_t res_role_offset(uint32_t n) { return pad256(4ull * n); }
size_t res_bytes(uint32_t n) { return res_role_offset(n) + n; }
const size_t kTailFlags = pad256(sizeof(RunCounters));
const size_t kTailBytes = kTailFlags + 4 * kMaxJumpRounds;

uint32_t jump_flag_index(uint32_t n) { return jump_rounds(n) - 1; }

// Queue q's work on slot sl (scheduler thread, lock NOT held: CUDA calls only here).
// Returns the number of kernels launched.
uint32_t launch_query(scan_server* s, Slot& sl, Query* q) {
    DeviceGraph* g = q->graph;
    RunScratch r;
    run_scratch_bind(&r, s->arena_base + sl.arena_off, g->n, g->E);
    uint32_t launches = 0;
    cudaStream_t st = sl.stream;
    cudaEventRecord(sl.ev_start, st);
    scan_status rc = launch_cluster(g, r, st, q->pp, q->mu, &launches);
    cudaMemcpyAsync(sl.h_res, r.label, res_bytes(g->n), cudaMemcpyDeviceToHost, st);       // label, role
    cudaMemcpyAsync(sl.h_tail, r.ctr, kTailBytes, cudaMemcpyDeviceToHost, st);            // counters, flags
    cudaEventRecord(sl.ev_end, st);
    cudaError_t err = cudaLaunchHostFunc(st, on_slot_done, new std::pair<scan_server*, Slot*>(s, &sl));
    if (rc != SCAN_OK || err != cudaSuccess) {
        q->status = rc != SCAN_OK ? rc : SCAN_ERR_CUDA;
        q->error = rc != SCAN_OK ? scan_last_error() : cudaGetErrorString(err);
        if (err != cudaSuccess) sl.gpu_done.store(true);   // no callback will come
    }
    return launches;
}

bool slot_finished(const Slot& sl) { return sl.q && !sl.launching && !sl.finishing && sl.gpu_done.load(); }

// Copy a finished slot's results to the caller's buffers (lock not held).
void copy_out(Slot* sl) {
    Query* q = sl->q;
    DeviceGraph* g = q->graph;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, sl->ev_start, sl->ev_end);
    q->device_ms = ms;
    std::memcpy(&q->counters, sl->h_tail, sizeof(RunCounters));
    uint32_t last_flag = 0;
    std::memcpy(&last_flag, sl->h_tail + kTailFlags + 4 * jump_flag_index(g->n), sizeof(uint32_t));
    if (q->status == SCAN_OK && (q->counters.error_flags || last_flag)) {
        q->status = SCAN_ERR_DEVICE;
        q->error = "union-find did not finish within its limits";
    }
    if (q->status == SCAN_OK) {
        std::memcpy(q->out_label, sl->h_res, g->n * sizeof(int32_t));
        if (q->out_role) std::memcpy(q->out_role, sl->h_res + res_role_offset(g->n), g->n);
    }
}

// A worker: launches admitted queries and retires finished ones.  CUDA calls and result
// copies happen with the lock released; the bookkeeping that follows takes it briefly.
void worker_loop(scan_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::pair<bool, Slot*> job;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_jobs.wait(lock, [&] { return !s->jobs.empty() || s->stop_workers; });
            if (s->jobs.empty()) return;
            job = s->jobs.front();
            s->jobs.pop_front();
        }
        Slot* sl = job.second;
        if (job.first) {
            const uint32_t launches = launch_query(s, *sl, sl->q);
            std::lock_guard<std::mutex> lock(s->mu);
            sl->launching = false;
            s->totals.kernel_launches += launches;
        } else {
            copy_out(sl);
            std::lock_guard<std::mutex> lock(s->mu);
            Query* q = sl->q;
            s->arena.release(sl->arena_off, sl->arena_bytes);
            s->mem_blocked = false;
            sl->q = nullptr;
            sl->finishing = false;
            q->finished = Clock::now();
            q->done = true;
            ++s->totals.completed;
            if (q->status != SCAN_OK) ++s->totals.failed;
        }
        s->cv_work.notify_one();
        s->cv_done.notify_all();
    }
}

// The scheduler.  It only does bookkeeping under the lock: which slots finished (handed to
// the workers to copy out and free), which queries to admit (arena blocks, slots; handed
// to the workers to launch).  No thread calls into CUDA or copies results while holding
// the lock, so a device-wide synchronisation elsewhere in the process (cudaMalloc/cudaFree
// by another thread) can always drain the host callbacks it waits for.
void scheduler(scan_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        s->cv_work.wait(lock, [&] {
            bool any_busy = false;
            for (Slot& sl : s->slots) {
                if (slot_finished(sl)) return true;
                any_busy |= sl.q != nullptr;
            }
            if (s->stop && !any_busy && s->pending.empty()) return true;
            if (s->pending.empty() || s->mem_blocked || s->pause_admission) return false;
            for (Slot& sl : s->slots)
                if (!sl.q) return true;
            return false;
        });
        bool any_busy = false;
        for (Slot& sl : s->slots) any_busy |= sl.q != nullptr;
        if (s->stop && !any_busy && s->pending.empty()) return;
        bool queued = false;
        for (Slot& sl : s->slots)
            if (slot_finished(sl)) {
                sl.finishing = true;
                s->jobs.emplace_back(false, &sl);
                queued = true;
            }
        bool failed_any = false;
        // admit in arrival order while a slot is free and the scratch fits
        while (!s->pending.empty() && !s->pause_admission) {
            Query* q = s->pending.front();
            DeviceGraph* g = q->graph;
            const uint64_t need = run_scratch_bytes(g->n, g->E);
            if (need > s->arena.size()) {   // can never fit
                s->pending.pop_front();
                q->status = SCAN_ERR_OUT_OF_MEMORY;
                q->error = "query scratch exceeds the server's memory budget";
                q->finished = Clock::now();
                q->done = true;
                ++s->totals.completed;
                ++s->totals.failed;
                failed_any = true;
                continue;
            }
            Slot* free_slot = nullptr;
            for (Slot& sl : s->slots)
                if (!sl.q) { free_slot = &sl; break; }
            if (!free_slot) break;
            uint64_t off = 0;
            if (!s->arena.alloc(need, &off)) {
                s->mem_blocked = true;   // admitted again once a running query returns its block
                break;
            }
            s->pending.pop_front();
            free_slot->q = q;
            free_slot->arena_off = off;
            free_slot->arena_bytes = need;
            free_slot->gpu_done.store(false);
            free_slot->launching = true;
            q->admitted = Clock::now();
            ++s->totals.admitted;
            s->jobs.emplace_back(true, free_slot);
            queued = true;
        }
        if (queued) s->cv_jobs.notify_all();
        if (failed_any) s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

scan_status scan_server_create(int device, uint64_t memory_budget_bytes, uint32_t max_in_flight, scan_server** out) {
    clear_error();
    if (!out || device < 0 || max_in_flight == 0 || max_in_flight > 256 || memory_budget_bytes < 4096)
        return fail(SCAN_ERR_INVALID_ARG, "bad server parameters");
    *out = nullptr;
    cudaError_t err = cudaSetDevice(device);
    if (err != cudaSuccess) return fail(SCAN_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(err));
    std::unique_ptr<scan_server> s(new scan_server());
    s->device = device;
    err = cudaMalloc(&s->arena_base, memory_budget_bytes);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return fail(SCAN_ERR_OUT_OF_MEMORY, "cannot reserve the server's memory budget: " +
                                                std::string(cudaGetErrorString(err)));
    }
    s->arena.reset(memory_budget_bytes);
    s->slots = std::vector<Slot>(max_in_flight);   // Slot holds an atomic: built in place, never moved
    for (Slot& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&sl.ev_start) != cudaSuccess || cudaEventCreate(&sl.ev_end) != cudaSuccess ||
            cudaHostAlloc(&sl.h_tail, kTailBytes, cudaHostAllocDefault) != cudaSuccess) {
            scan_server_destroy(s.release());
            return fail(SCAN_ERR_CUDA, "cannot create the server's streams");
        }
    }
    const unsigned hw = std::max(2u, std::thread::hardware_concurrency());
    const unsigned nworkers = std::min<unsigned>(max_in_flight, std::min(8u, hw / 2));
    for (unsigned i = 0; i < std::max(1u, nworkers); ++i) s->workers.emplace_back(worker_loop, s.get());
    s->worker = std::thread(scheduler, s.get());
    *out = s.release();
    return SCAN_OK;
}

scan_status scan_server_add_graph(scan_server* s, const scan_graph* g, uint32_t* graph_id) {
    clear_error();
    if (!s || !g || !graph_id) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    DeviceGraph* d = nullptr;
    scan_status st = device_upload(s->device, g->n, g->m, g->off.data(), true, g->adj.data(), &d, nullptr);
    if (st != SCAN_OK) return st;
    uint32_t launches = 0;
    st = launch_cn(d, &launches);
    if (st == SCAN_OK && cudaStreamSynchronize(d->stream) != cudaSuccess)
        st = fail(SCAN_ERR_CUDA, "similarity stage failed while adding a graph");
    if (st == SCAN_OK) st = compute_tau(d);   // queries then test each edge with one compare
    if (st != SCAN_OK) {
        device_graph_free(d);
        return st;
    }
    d->cn_valid = true;
    std::unique_lock<std::mutex> lock(s->mu);
    // Result staging must hold the largest graph.  Growing it pauses admission and waits for
    // the slots to drain, then reallocates with the lock released (no CUDA call under it).
    // One grower at a time: a concurrent add_graph waits for the current grow step to end,
    // then checks again whether the staging already holds its graph.
    s->cv_done.wait(lock, [&] { return !s->growing; });
    bool grow = false;
    for (Slot& sl : s->slots) grow |= sl.n_cap < d->n;
    scan_status grow_status = SCAN_OK;
    if (grow) {
        s->growing = true;
        s->pause_admission = true;
        s->cv_done.wait(lock, [&] {
            for (Slot& sl : s->slots)
                if (sl.q) return false;
            return true;
        });
        lock.unlock();
        for (Slot& sl : s->slots) {
            if (sl.n_cap >= d->n) continue;
            if (sl.h_res) cudaFreeHost(sl.h_res);
            sl.h_res = nullptr;
            sl.n_cap = 0;
            if (cudaHostAlloc(&sl.h_res, res_bytes(d->n), cudaHostAllocDefault) != cudaSuccess) {
                grow_status = fail(SCAN_ERR_OUT_OF_MEMORY, "cannot allocate pinned result staging");
                break;
            }
            sl.n_cap = d->n;
        }
        lock.lock();
        s->pause_admission = false;
        s->growing = false;
        s->cv_done.notify_all();
    }
    if (grow_status != SCAN_OK) {
        lock.unlock();
        s->cv_work.notify_one();
        device_graph_free(d);
        return grow_status;
    }
    *graph_id = (uint32_t)s->graphs.size();
    s->graphs.push_back(d);
    lock.unlock();
    s->cv_work.notify_one();
    return SCAN_OK;
}

scan_status scan_server_submit(scan_server* s, uint32_t graph_id, const char* eps_decimal, int mu,
                               scan_predicate predicate, int32_t* out_label, uint8_t* out_role, uint64_t* ticket) {
    clear_error();
    if (!s || !out_label || !ticket) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    if (mu < 1) return fail(SCAN_ERR_INVALID_ARG, "mu must be >= 1");
    PredParams pp;
    scan_status st = make_pred(eps_decimal, &pp, predicate);
    if (st != SCAN_OK) return st;
    std::unique_ptr<Query> q(new Query());
    q->gid = graph_id;
    q->pp = pp;
    q->mu = mu;
    q->out_label = out_label;
    q->out_role = out_role;
    q->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (graph_id >= s->graphs.size()) return fail(SCAN_ERR_INVALID_ARG, "unknown graph id");
        q->graph = s->graphs[graph_id];
        if (s->stop) return fail(SCAN_ERR_INVALID_ARG, "server is shutting down");
        q->ticket = s->next_ticket++;
        *ticket = q->ticket;
        s->pending.push_back(q.get());
        s->queries.emplace(q->ticket, std::move(q));
        ++s->totals.submitted;
    }
    s->cv_work.notify_one();
    return SCAN_OK;
}

scan_status scan_server_wait(scan_server* s, uint64_t ticket, scan_query_result* result) {
    clear_error();
    if (!s) return fail(SCAN_ERR_INVALID_ARG, "null server");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(SCAN_ERR_INVALID_ARG, "unknown ticket");
    Query* q = it->second.get();
    s->cv_done.wait(lock, [&] { return q->done; });
    if (result) {
        std::memset(result, 0, sizeof(*result));
        result->ticket = q->ticket;
        result->status = q->status;
        result->graph_id = q->gid;
        result->queue_ms = q->status == SCAN_OK ? ms_between(q->submitted, q->admitted) : 0.0;
        result->latency_ms = ms_between(q->submitted, q->finished);
        result->device_ms = q->device_ms;
        result->num_cores = q->counters.cores;
        result->num_clusters = q->counters.clusters;
        result->num_similar_edges = q->counters.similar_edges;
    }
    scan_status st = q->status;
    std::string err = q->error;
    s->queries.erase(it);
    if (st != SCAN_OK) return fail(st, err);
    return SCAN_OK;
}

scan_status scan_server_poll(scan_server* s, uint64_t ticket, int* done) {
    clear_error();
    if (!s || !done) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(SCAN_ERR_INVALID_ARG, "unknown ticket");
    *done = it->second->done ? 1 : 0;
    return SCAN_OK;
}

scan_status scan_server_get_counters(scan_server* s, scan_server_counters* out) {
    clear_error();
    if (!s || !out) return fail(SCAN_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->totals;
    out->pending = s->pending.size();
    out->in_flight = 0;
    for (Slot& sl : s->slots) out->in_flight += sl.q != nullptr;
    out->graphs = s->graphs.size();
    out->budget_bytes = s->arena.size();
    return SCAN_OK;
}

scan_status scan_server_replay(scan_server* s, uint64_t num_queries, const uint32_t* graph_id,
                               const char* const* eps_decimal, const int32_t* mu, const int32_t* predicate,
                               const double* arrival_ms, double* latency_ms, int32_t* status, double* wall_ms) {
    clear_error();
    if (!s || (num_queries && (!graph_id || !eps_decimal || !mu || !predicate || !arrival_ms || !latency_ms ||
                               !status)))
        return fail(SCAN_ERR_INVALID_ARG, "null argument");
    // one output buffer per graph, shared by that graph's queries (the trace measures time)
    std::vector<std::vector<int32_t>> out;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        out.resize(s->graphs.size());
        for (size_t g = 0; g < s->graphs.size(); ++g) out[g].resize(s->graphs[g]->n);
    }
    for (uint64_t i = 0; i < num_queries; ++i)
        if (graph_id[i] >= out.size()) return fail(SCAN_ERR_INVALID_ARG, "unknown graph id in the trace");
    std::vector<uint64_t> tickets(num_queries, 0);
    std::vector<int32_t> submit_status(num_queries, SCAN_OK);
    std::mutex tmu;
    std::condition_variable tcv;
    uint64_t submitted = 0;
    const Clock::time_point t0 = Clock::now();
    std::thread submitter([&] {
        for (uint64_t i = 0; i < num_queries; ++i) {
            const auto due = t0 + std::chrono::duration_cast<Clock::duration>(
                                      std::chrono::duration<double, std::milli>(arrival_ms[i]));
            while (Clock::now() < due) {
                const auto left = due - Clock::now();
                if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
            }
            uint64_t t = 0;
            scan_status st = scan_server_submit(s, graph_id[i], eps_decimal[i], mu[i], (scan_predicate)predicate[i],
                                                out[graph_id[i]].data(), nullptr, &t);
            {
                std::lock_guard<std::mutex> lock(tmu);
                tickets[i] = t;
                submit_status[i] = st;
                submitted = i + 1;
            }
            tcv.notify_one();
        }
    });
    for (uint64_t i = 0; i < num_queries; ++i) {
        {
            std::unique_lock<std::mutex> lock(tmu);
            tcv.wait(lock, [&] { return submitted > i; });
        }
        if (submit_status[i] != SCAN_OK) {
            status[i] = submit_status[i];
            latency_ms[i] = 0;
            continue;
        }
        scan_query_result r;
        status[i] = scan_server_wait(s, tickets[i], &r);
        latency_ms[i] = r.latency_ms;
    }
    submitter.join();
    if (wall_ms) *wall_ms = ms_between(t0, Clock::now());
    clear_error();
    return SCAN_OK;
}

void scan_server_destroy(scan_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();   // returns once every slot is idle
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop_workers = true;
    }
    s->cv_jobs.notify_all();
    for (std::thread& w : s->workers)
        if (w.joinable()) w.join();
    cudaSetDevice(s->device);
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.ev_start) cudaEventDestroy(sl.ev_start);
        if (sl.ev_end) cudaEventDestroy(sl.ev_end);
        if (sl.h_res) cudaFreeHost(sl.h_res);
        if (sl.h_tail) cudaFreeHost(sl.h_tail);
    }
    for (DeviceGraph* d : s->graphs) device_graph_free(d);
    if (s->arena_base) cudaFree(s->arena_base);
    delete s;
}

}  // extern "C"
