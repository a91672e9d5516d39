// Host-side engine: owns device buffers and runs the pipeline.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.cuh"
#include "pbig2.h"

namespace pbig {

// grow-only device allocation
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need, bool zero, cudaStream_t st);
    void release();
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct HostPinned {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need);
    void release();
};

struct SceneIn {
    uint64_t box_off, n;
    uint32_t shift;   // chosen cell shift
};

// cell-size autotuner (host): cost model over candidate shifts, fed from a
// sample of boxes. `words` = 2*dims+1.
struct TuneResult {
    uint32_t shift;
    double est_entries, est_tests, est_cells;
};
TuneResult tune_shift_sample(const uint32_t* boxes, uint64_t n_avail, uint64_t n_true, int dims, uint32_t range,
                             uint64_t max_sample);
uint32_t nrc_for(uint32_t range, uint32_t shift);
// records `msg` as the calling thread's pbig2_last_error() and returns code
int api_fail(int code, const char* msg);

}  // namespace pbig

struct pbig2_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evp[9] = {};
    pbig::DevBuf d_merged;  // merged mode: cell -> root table
    bool merged_mode = false;
    bool rice_mode = false;      // record mode (PBIG2_OPT_RICE)
    bool result_records = false; // the last result is a record stream
    uint64_t rice_words = 0;     // words of the last record stream
    uint64_t last_ncells = 0, last_entries = 0;
    uint32_t merged_blocks = 0;  // merged blocks of the last query
    uint32_t last_err = 0;       // error bits of the last pipeline pass
    pbig::DevBuf d_boxes, d_counts, d_entries, d_lists, d_tasks, d_state, d_out, d_out2, d_ctr,
        d_scenes, d_scene_off, d_scene_pair, d_scene_cursor, d_dims, d_scene_tab, d_tune;
    pbig::HostPinned h_ctr, h_stage;
    // caller's pair buffer for self/bipartite queries (pbig2_set_pair_output)
    uint2* ext_out = nullptr;
    uint64_t ext_cap = 0;
    bool ext_host = false;    // ext_out is page-locked host memory
    // pairs to host memory: SMs of the small-cell and block kernels beside
    // the medium-cell kernel (PBIG2_OPT_HOST_SPLIT; 0 = automatic, < 0 = off)
    int host_split = 0;
    cudaStream_t side_stream = nullptr;
    // page-locked host input of the running query, uploaded by the count
    // kernel (device-mapped addresses; null: the boxes are on the device)
    const uint32_t* up_red = nullptr;
    const uint32_t* up_blue = nullptr;
    uint64_t up_split = 0;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool result_ext = false;  // the last result went to ext_out
    // last result
    const uint2* result = nullptr;
    uint64_t npairs = 0;
    std::vector<uint64_t> scene_pair_off;
    std::vector<uint32_t> scene_shifts;  // cell-size shift of every scene of the last query
    pbig2_stats stats{};
    // capacity hints carried between queries
    uint64_t out_hint = 0;
    // captured batched pipeline (CUDA graph) and the capacities it serves
    bool use_graph = true;
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        const uint32_t* boxes = nullptr;
        int dims = 0;
        uint32_t range = 0, split = 0;
        uint64_t nboxes_cap = 0, ncells_cap = 0, nscenes_cap = 0, entry_cap = 0, out_cap = 0;
        unsigned long long class_map = 0;
        uintptr_t buffers = 0;  // buffers_sig() at capture: any reallocation invalidates the graph
        int launches = 0;
    } graph;
    uintptr_t buffers_sig() const {
        uintptr_t h = 0;
        for (const pbig::DevBuf* b : {&d_counts, &d_entries, &d_lists, &d_tasks, &d_state, &d_out, &d_out2,
                                      &d_ctr, &d_scenes, &d_scene_off, &d_scene_pair, &d_scene_cursor, &d_dims,
                                      &d_scene_tab})
            h = h * 1000003u + (uintptr_t)b->p;
        return h * 1000003u + (uintptr_t)h_ctr.p;
    }
    void drop_graph() {
        if (graph.exec) cudaGraphExecDestroy(graph.exec);
        graph = Graph();
    }
    // one-launch queries of small scenes (PBIG2_OPT_ONE_LAUNCH): the grid
    // barriers' arrival counter and its value before the next launch, and
    // the entry capacity the last one needed
    bool use_fused = true;
    pbig::DevBuf d_bar, d_fctr;  // barrier arrivals; two slots of run counters (a launch zeroes the other)
    unsigned int bar_base = 0;
    int fused_slot = 0;
    bool fused_dirty = true;     // the counters may hold values another pipeline left (or are new)
    uint64_t fused_entry_hint = 0;
    bool fused_stall_test = false;  // the next launch's barriers never complete (test of the bounded wait)
    // work-list class map of later queries (PBIG2_OPT_CLASS_MAP; 0: automatic)
    unsigned long long class_map = 0;
    uint32_t merge_limit = 256;  // merged mode's block limit (PBIG2_OPT_MERGE_LIMIT)
    // autotuner memo: (n, dims, range, mean extent) -> shift
    struct TuneMemo { uint64_t n; int dims; uint32_t range; double ext; uint32_t shift; double est_e; };
    std::vector<TuneMemo> memo;
};
