// ref_harness.cu -- runs the reference's own SCAN kernels on the GPU, for parity pinning.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle; the product never loads it).
//
// The kernels come from GPUSCAN++/GPUScan.cu compiled unmodified into a cubin
// (oracle/build.py writes oracle/_ref/gpuscan_ref.cubin).  This file replays the host
// sequence of GPUScan() (GPUSCAN++/GPUScan.cu:800-1009): the same allocations and copies,
// the same eight kernel launches in the same order with the same grid shapes
// (TOTALTHDCOUNT = 65536 threads; 512-thread "ii" and 128-thread "cc" blocks, :18-21,
// :860-861).  The Thrust count/compaction glue between launches (:873, :906, :920,
// :978-982) is done on the host from a copy of role[], which yields the same core list
// (ascending ids, copy_if is stable) and the same "others" list (ascending ids,
// remove_if is stable).
//
// One deliberate difference: the adjacency buffer gets 32 zeroed entries past m, because
// __classify_others reads gpuadj[end] for the last vertex (:760), one entry past the
// reference's allocation; with the padding that read stays in bounds.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace {

std::string g_err;

bool ck(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return false;
}
bool ck(cudaError_t r, const char* what) {
    if (r == cudaSuccess) return true;
    g_err = std::string(what) + ": " + cudaGetErrorString(r);
    return false;
}

struct Mod {
    CUmodule mod = nullptr;
    CUfunction init_input, prep_edge, check_core, cluster_core1, cluster_core2, cluster_core, cluster_noncore,
        classify_others;
};

// Mangled names of the reference's kernels (signatures at GPUSCAN++/GPUScan.cu:116, 134,
// 277, 480, 531, 633, 655, 733).
bool load(const char* path, Mod* m) {
    if (!ck(cuModuleLoad(&m->mod, path), "cuModuleLoad")) return false;
    struct { CUfunction* f; const char* name; } t[] = {
        {&m->init_input, "_Z12__init_inputPiS_S_Pjil"},
        {&m->prep_edge, "_Z11__prep_edgePcPjPiS1_dilS1_S1_S1_"},
        {&m->check_core, "_Z12__check_coredillPKjPKiS2_S2_PcPiS4_S4_"},
        {&m->cluster_core1, "_Z15__cluster_core1PKjPKiS0_PcPiS2_i"},
        {&m->cluster_core2, "_Z15__cluster_core2dPKjPKiS0_PcPiS2_i"},
        {&m->cluster_core, "_Z14__cluster_corePiS_i"},
        {&m->cluster_noncore, "_Z17__cluster_noncoredPjPiS_PcS0_S0_i"},
        {&m->classify_others, "_Z17__classify_othersPiPjS_S_i"},
    };
    for (auto& e : t)
        if (!ck(cuModuleGetFunction(e.f, m->mod, e.name), e.name)) return false;
    return true;
}

bool launch(CUfunction f, unsigned grid, unsigned block, void** args, const char* what) {
    if (!ck(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr), what)) return false;
    return ck(cuCtxSynchronize(), what);
}

}  // namespace

extern "C" __attribute__((visibility("default"))) const char* ref_harness_error() { return g_err.c_str(); }

// Runs the reference pipeline; out_role[n] receives the reference's result array.
// ms_kernels (may be null) receives the summed kernel time (CUDA events).
extern "C" __attribute__((visibility("default"))) int ref_gpuscan(const char* cubin, int64_t n, int64_t m,
                                                                  const uint32_t* num_edges, const int32_t* adj,
                                                                  const uint32_t* eid, const int32_t* edge_u,
                                                                  const int32_t* edge_v, double eps, int miu,
                                                                  int32_t* out_role, float* ms_kernels) {
    g_err.clear();
    if (!ck(cudaSetDevice(0), "cudaSetDevice") || !ck(cudaFree(nullptr), "context")) return -1;
    Mod md;
    if (!load(cubin, &md)) return -1;
    const uint64_t TOTALTHDCOUNT = 65536;
    const unsigned ii_block = 512, cc_block = 128;
    const unsigned ii_grid = (unsigned)(TOTALTHDCOUNT / ii_block), cc_grid = (unsigned)(TOTALTHDCOUNT / cc_block);
    int *gpuadj = nullptr, *role = nullptr, *sd = nullptr, *ed = nullptr, *rawE_u = nullptr, *rawE_v = nullptr;
    unsigned *gpunum_edges = nullptr, *gpuEid = nullptr;
    char* similar = nullptr;
    int *core_node = nullptr, *others_node = nullptr;
    int rc = -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float total = 0.f;
    const int64_t half = m / 2;
    std::vector<int32_t> h_role(n);
    long vlength = (long)n, elength = (long)m;
    int core_number = 0, others_number = 0;
    if (!ck(cudaMalloc(&gpuadj, (m + 32) * sizeof(int)), "malloc adj")) goto out;
    if (!ck(cudaMalloc(&gpunum_edges, (n + 1) * sizeof(unsigned)), "malloc off")) goto out;
    if (!ck(cudaMalloc(&gpuEid, (m + 1) * sizeof(unsigned)), "malloc eid")) goto out;
    if (!ck(cudaMalloc(&similar, half + 1), "malloc similar")) goto out;
    if (!ck(cudaMalloc(&role, n * sizeof(int)), "malloc role")) goto out;
    if (!ck(cudaMalloc(&sd, n * sizeof(int)), "malloc sd")) goto out;
    if (!ck(cudaMalloc(&ed, n * sizeof(int)), "malloc ed")) goto out;
    if (!ck(cudaMalloc(&rawE_u, (half + 1) * sizeof(int)), "malloc eu")) goto out;
    if (!ck(cudaMalloc(&rawE_v, (half + 1) * sizeof(int)), "malloc ev")) goto out;
    if (!ck(cudaMemset(gpuadj, 0, (m + 32) * sizeof(int)), "memset adj")) goto out;
    if (!ck(cudaMemcpy(gpuadj, adj, m * sizeof(int), cudaMemcpyHostToDevice), "h2d adj")) goto out;
    if (!ck(cudaMemcpy(gpunum_edges, num_edges, (n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice), "h2d off")) goto out;
    if (!ck(cudaMemcpy(gpuEid, eid, m * sizeof(unsigned), cudaMemcpyHostToDevice), "h2d eid")) goto out;
    if (!ck(cudaMemcpy(rawE_u, edge_u, half * sizeof(int), cudaMemcpyHostToDevice), "h2d eu")) goto out;
    if (!ck(cudaMemcpy(rawE_v, edge_v, half * sizeof(int), cudaMemcpyHostToDevice), "h2d ev")) goto out;
    {
        float ms = 0.f;
        void* a_init[] = {&role, &sd, &ed, &gpunum_edges, &miu, &vlength};
        cudaEventRecord(e0);
        if (!launch(md.init_input, ii_grid, ii_block, a_init, "__init_input")) goto out;
        void* a_prep[] = {&similar, &gpunum_edges, &rawE_u, &rawE_v, &eps, &miu, &elength, &ed, &sd, &role};
        if (!launch(md.prep_edge, ii_grid, ii_block, a_prep, "__prep_edge")) goto out;
        void* a_cc[] = {&eps, &miu, &vlength, &elength, &gpunum_edges, &gpuadj, &rawE_u, &rawE_v, &similar, &role, &sd, &ed};
        if (!launch(md.check_core, cc_grid, cc_block, a_cc, "__check_core")) goto out;
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        // core list: thrust::copy_if(role >= 0), stable (GPUScan.cu:906, 920)
        if (!ck(cudaMemcpy(h_role.data(), role, n * sizeof(int), cudaMemcpyDeviceToHost), "d2h role")) goto out;
        std::vector<int32_t> cores;
        for (int64_t v = 0; v < n; ++v) if (h_role[v] >= 0) cores.push_back((int32_t)v);
        core_number = (int)cores.size();
        if (!ck(cudaMalloc(&core_node, (cores.size() + 1) * sizeof(int)), "malloc cores")) goto out;
        if (!cores.empty() &&
            !ck(cudaMemcpy(core_node, cores.data(), cores.size() * sizeof(int), cudaMemcpyHostToDevice), "h2d cores"))
            goto out;
        cudaEventRecord(e0);
        void* a_c1[] = {&gpunum_edges, &gpuadj, &gpuEid, &similar, &role, &core_node, &core_number};
        if (!launch(md.cluster_core1, cc_grid, cc_block, a_c1, "__cluster_core1")) goto out;
        void* a_c2[] = {&eps, &gpunum_edges, &gpuadj, &gpuEid, &similar, &role, &core_node, &core_number};
        if (!launch(md.cluster_core2, cc_grid, cc_block, a_c2, "__cluster_core2")) goto out;
        void* a_c[] = {&core_node, &role, &core_number};
        if (!launch(md.cluster_core, ii_grid, ii_block, a_c, "__cluster_core")) goto out;
        void* a_nc[] = {&eps, &gpunum_edges, &gpuadj, &gpuEid, &similar, &role, &core_node, &core_number};
        if (!launch(md.cluster_noncore, cc_grid, cc_block, a_nc, "__cluster_noncore")) goto out;
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        // others: count(role == -2) and remove_if(sequence, role >= 0) (GPUScan.cu:978-982)
        if (!ck(cudaMemcpy(h_role.data(), role, n * sizeof(int), cudaMemcpyDeviceToHost), "d2h role")) goto out;
        std::vector<int32_t> others;
        others_number = 0;
        for (int64_t v = 0; v < n; ++v) {
            if (h_role[v] == -2) ++others_number;
            if (h_role[v] < 0) others.push_back((int32_t)v);
        }
        if (!ck(cudaMalloc(&others_node, (n + 1) * sizeof(int)), "malloc others")) goto out;
        if (!others.empty() &&
            !ck(cudaMemcpy(others_node, others.data(), others.size() * sizeof(int), cudaMemcpyHostToDevice), "h2d others"))
            goto out;
        cudaEventRecord(e0);
        void* a_cl[] = {&role, &gpunum_edges, &gpuadj, &others_node, &others_number};
        if (!launch(md.classify_others, ii_grid, ii_block, a_cl, "__classify_others")) goto out;
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
        if (!ck(cudaMemcpy(out_role, role, n * sizeof(int), cudaMemcpyDeviceToHost), "d2h result")) goto out;
    }
    if (ms_kernels) *ms_kernels = total;
    rc = 0;
out:
    cudaFree(gpuadj); cudaFree(gpunum_edges); cudaFree(gpuEid); cudaFree(similar); cudaFree(role);
    cudaFree(sd); cudaFree(ed); cudaFree(rawE_u); cudaFree(rawE_v); cudaFree(core_node); cudaFree(others_node);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (md.mod) cuModuleUnload(md.mod);
    return rc;
}
