// Host orchestration of the pair-detection pipeline and the C ABI (pbig2.h).
//
// One query = one pass of count -> scan -> expand -> scatter -> pairs on the
// context's stream, after the cell size has been chosen by the autotuner.
// The reference runs the same phases with host round trips in between
// (plan_phase / map_phase / sched_phase / match_phase, src/pbig/pbig.cu:1361,
// 1429, 1592, 1694); here every phase stays on the device and the host reads
// back one small counter block per query.
#include "engine.h"

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>

namespace pbig {

static thread_local std::string g_last_error;

static int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int api_fail(int code, const char* msg) { return fail(code, "%s", msg); }

#define CK(expr)                                                                                   \
    do {                                                                                           \
        cudaError_t _e = (expr);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return fail(_e == cudaErrorMemoryAllocation ? PBIG2_ENOMEM : PBIG2_ECUDA, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(_e), __FILE__, __LINE__);                        \
    } while (0)

cudaError_t DevBuf::ensure(size_t need, bool zero, cudaStream_t st) {
    if (need == 0) need = 256;
    if (need <= bytes) return cudaSuccess;
    release();
    size_t b = need + need / 8;
    b = (b + 255) & ~size_t(255);
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
        p = nullptr;
        return e;
    }
    bytes = b;
    if (zero) return cudaMemsetAsync(p, 0, b, st);
    return cudaSuccess;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

cudaError_t HostPinned::ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    release();
    cudaError_t e = cudaMallocHost(&p, need);
    if (e != cudaSuccess) {
        p = nullptr;
        return e;
    }
    bytes = need;
    return cudaSuccess;
}

void HostPinned::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
}

uint32_t nrc_for(uint32_t range, uint32_t shift) {
    return (uint32_t)(((uint64_t)range + (1ull << shift) - 1) >> shift);
}

// --------------------------------------------------------------------------
// autotuner: cost(s) = kCell*C(s) + kEntry*E(s) + kTest*T(s) in seconds
// (C cells, E box-in-cell entries, T pair tests; tune_cost in kernels.cuh),
// estimated from a sample. T is counted exactly on the sample (cell
// occupancy by hashing) and scaled by (n/m)^2, since a pair of boxes
// survives sampling with probability (m/n)^2. A test costs more once the
// tests sit in cells beyond the medium-cell kernel's reach: with the
// entry-weighted mean occupancy m = 2T/E + 1, kTest is scaled by
// max(1, m / kOccTest). The constants are fitted on GB300 cell-size sweeps
// (2-D/3-D, uniform/clustered, single scenes and a 4096-scene batch), where
// they pick the fastest size or one within 2%; per unit, an entry costs
// ~16 ps in the count and scatter plus its fetch and sweep in the pair
// kernels, a test ~1 ps in the medium-cell kernel and ~2 ps in the block
// kernel. Batched queries run the same model on the device, one warp per
// scene, with T = E^2 / 2C (k_tune_scenes).
// --------------------------------------------------------------------------

// pair tests of the sample at one cell size: occupancy of the sample's cells
// counted in an open-addressing hash table (key = cell id + 1)
static double tests_in_sample(const uint32_t* boxes, const std::vector<uint64_t>& idx, int dims, uint32_t shift,
                              uint32_t nrc, uint64_t nkeys, std::vector<uint64_t>& keys, std::vector<uint32_t>& cnt) {
    const int W = 2 * dims + 1;
    uint64_t cap = 64;
    while (cap < 2 * nkeys) cap <<= 1;
    keys.assign(cap, 0);
    cnt.assign(cap, 0);
    const uint64_t mask = cap - 1;
    double t = 0;
    for (uint64_t i : idx) {
        const uint32_t* b = boxes + i * W;
        uint32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        for (int d = 0; d < dims; d++) {
            lo[d] = b[2 * d] >> shift;
            hi[d] = b[2 * d + 1] >> shift;
        }
        for (uint32_t k = lo[2]; k <= hi[2]; k++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t x = lo[0]; x <= hi[0]; x++) {
                    const uint64_t key = ((uint64_t)k * nrc + j) * nrc + x + 1;
                    uint64_t h = (key * 0x9e3779b97f4a7c15ULL) >> 20;
                    for (;; h++) {
                        uint64_t& slot = keys[h & mask];
                        if (slot == key) break;
                        if (slot == 0) { slot = key; break; }
                    }
                    t += cnt[h & mask]++;  // a new member pairs with every earlier one
                }
    }
    return t;
}

static bool box_ok(const uint32_t* b, int dims, uint32_t range) {
    for (int d = 0; d < dims; d++)
        if (b[2 * d] > b[2 * d + 1] || b[2 * d + 1] >= range) return false;
    return true;
}

// n is the number of boxes the sample idx stands for
static TuneResult tune_impl(const uint32_t* boxes, const std::vector<uint64_t>& idx, uint64_t n, int dims,
                            uint32_t range) {
    const int W = 2 * dims + 1;
    TuneResult best{0, 0, 0, 0};
    if (idx.empty()) {
        best.shift = 31;
        while (best.shift > 0 && nrc_for(range, best.shift - 1) <= 1) best.shift--;
        return best;
    }
    uint64_t ext_sum = 0, good = 0;  // exact: the device tuner sums the same integers
    for (uint64_t i : idx) {
        const uint32_t* b = boxes + i * W;
        if (!box_ok(b, dims, range)) continue;
        for (int d = 0; d < dims; d++) ext_sum += (uint64_t)(b[2 * d + 1] - b[2 * d]) + 1;
        good++;
    }
    const int s0 = tune_s0(ext_sum, (good ? good : 1) * (uint64_t)dims);
    const double scale = (double)n / (double)idx.size();
    std::vector<uint64_t> keys;
    std::vector<uint32_t> cnts;
    double best_cost = 1e300;
    // candidates: s0-2 .. s0+3; only when none of those qualifies (a few
    // huge boxes in the sample can disqualify them all), every coarser size,
    // the cheapest by the cost model
    const int s_win = std::min(31, s0 + 3);
    for (int s = std::max(0, s0 - 2); s <= 31; s++) {
        if (s == s_win + 1 && best_cost < 1e300) break;
        const uint32_t nrc = nrc_for(range, (uint32_t)s);
        const double C = tune_cells(nrc, dims);
        if (C > 4.0e9) continue;
        if (s > s_win && C > std::max(4096.0, 64.0 * (double)n)) continue;  // widened: grids in proportion to n
        double E = 0, cmax = 0;
        for (uint64_t i : idx) {
            const uint32_t* b = boxes + i * W;
            if (!box_ok(b, dims, range)) continue;
            double c = 1;
            for (int d = 0; d < dims; d++) c *= (double)((b[2 * d + 1] >> s) - (b[2 * d] >> s) + 1);
            E += c;
            cmax = std::max(cmax, c);
        }
        if (E / (double)idx.size() > 64.0) continue;  // replication too high to be a candidate
        if (cmax >= (double)(1u << 26)) continue;     // a sampled box would not fit (2^26 cells or more)
        const double Es = E;
        E *= scale;
        const double T = tests_in_sample(boxes, idx, dims, (uint32_t)s, nrc, (uint64_t)Es, keys, cnts) * scale * scale;
        const double cost = tune_cost(C, E, T);
        if (cost < best_cost) {
            best_cost = cost;
            best = TuneResult{(uint32_t)s, E, T, C};
        }
    }
    if (best_cost == 1e300) {  // fall back to the coarsest grid that is not a single cell
        uint32_t s = 31;
        while (s > 0 && nrc_for(range, s - 1) <= 1) s--;
        best.shift = s;
        best.est_cells = tune_cells(nrc_for(range, s), dims);
        best.est_entries = (double)n;
        best.est_tests = (double)n * n / 2;
    }
    return best;
}

// boxes: n_avail records standing for n_true boxes (a sample when smaller)
TuneResult tune_shift_sample(const uint32_t* boxes, uint64_t n_avail, uint64_t n_true, int dims, uint32_t range,
                             uint64_t max_sample) {
    std::vector<uint64_t> idx;
    const uint64_t m = std::min<uint64_t>(n_avail, std::max<uint64_t>(1, max_sample));
    idx.reserve(m);
    for (uint64_t i = 0; i < m; i++) idx.push_back((uint64_t)((unsigned __int128)i * n_avail / m));
    return tune_impl(boxes, idx, n_true, dims, range);
}


// --------------------------------------------------------------------------
// pipeline
// --------------------------------------------------------------------------
struct GridScene {
    uint64_t box_off, n;
    uint32_t shift;
    int grid_of;  // index of the scene whose grid this one shares (self for its own)
};

// device buffers of one query; fills the matching Params fields
static int ensure_query_buffers(pbig2_ctx* c, Params& p, uint64_t entry_cap, uint64_t out_cap, uint64_t task_cap,
                                uint32_t nsc, bool grouped, cudaStream_t st) {
    CK(c->d_entries.ensure(entry_cap * 4, false, st));
    // list regions: a cell of class c holds at least lo_c boxes, so with
    // E <= entry capacity no list can overflow
    const uint64_t ecap = c->d_entries.bytes / 4;
    const unsigned long long map = p.class_map ? p.class_map : kClassMapDefault;
    uint64_t loff = 0;
    for (int k = 0; k < kNumLists; k++) {
        const uint64_t lo = class_map_min(map, k);  // 0: the map sends no cell there
        p.list_off[k] = loff;
        p.list_cap[k] = lo ? ecap / lo + 1 : 1;
        loff += p.list_cap[k];
    }
    CK(c->d_lists.ensure(loff * 8, false, st));
    CK(c->d_tasks.ensure(task_cap * 16, false, st));
    CK(c->d_out.ensure(out_cap * 8, false, st));
    if (grouped) {
        CK(c->d_out2.ensure(c->d_out.bytes, false, st));
        CK(c->d_scene_pair.ensure((nsc + 1) * 8, false, st));
        CK(c->d_scene_cursor.ensure((nsc + 1) * 8, false, st));
    }
    p.counts = c->d_counts.as<uint32_t>();
    p.entries = c->d_entries.as<uint32_t>();
    p.entry_cap = ecap;
    p.lists = c->d_lists.as<uint2>();
    p.tasks = c->d_tasks.as<uint4>();
    p.task_cap = c->d_tasks.bytes / 16;
    p.out = c->d_out.as<uint2>();
    p.out_cap = c->d_out.bytes / 8;
    return PBIG2_OK;
}

// the launches of one pipeline pass (also what a graph captures): counters
// and scan state reset, count, scan, expand, scatter, the three pair
// kernels and, for batches, grouping of the pairs by scene
static int g_record_line = 0;  // line of the call that failed in record_pipeline

static cudaError_t record_pipeline(pbig2_ctx* c, const Params& p, int dims, bool grouped, uint32_t nsc,
                                   bool full, cudaStream_t st) {
    cudaError_t e;
    (void)cudaGetLastError();  // launch checks below must not see older, unrelated errors
    // inside a stream capture an event record must be an external node to be timed
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(st, &cap)) != cudaSuccess) return e;
    const unsigned evf = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
#define R(x)                          \
    if ((e = (x)) != cudaSuccess) {   \
        g_record_line = __LINE__;     \
        return e;                     \
    }
    if (full) {
        R(cudaMemsetAsync(p.ctr, 0, sizeof(Ctr), st));
        if (p.scene_table) R(launch_scene_table(p, st));
        R(cudaEventRecordWithFlags(c->evp[0], st, evf));
        R(launch_count(p, dims, st));
        R(cudaEventRecordWithFlags(c->evp[1], st, evf));
        R(launch_scan(p, st));
        R(cudaEventRecordWithFlags(c->evp[2], st, evf));
        R(launch_expand(p, st));
        R(cudaEventRecordWithFlags(c->evp[3], st, evf));
        R(launch_scatter(p, dims, st));
        R(cudaEventRecordWithFlags(c->evp[4], st, evf));
    } else {
        // keep the grid and lists; clear the pair count and error word
        R(cudaMemsetAsync(&p.ctr->pairs, 0, sizeof(unsigned long long), st));
        R(cudaMemsetAsync(&p.ctr->err, 0, sizeof(unsigned int), st));
        R(cudaMemsetAsync(&p.ctr->med_next, 0, sizeof(unsigned int), st));
        R(cudaEventRecordWithFlags(c->evp[4], st, evf));
    }
    // pairs stored over the host link: the lighter pair kernels run beside
    // the medium-cell kernel (two fifths of the SMs unless set)
    PairOverlap ov{c->side_stream, c->ev_fork, c->ev_join,
                   c->host_split > 0 ? c->host_split : (2 * c->sm_count + 2) / 5};
    const bool overlap = c->ext_host && p.out == c->ext_out && c->host_split >= 0 && !p.records;
    R(launch_pairs(p, dims, c->sm_count, st, &c->evp[7], evf, overlap ? &ov : nullptr));  // records evp[7], evp[8]
    R(cudaEventRecordWithFlags(c->evp[5], st, evf));
    if (grouped) {
        unsigned long long* hist = c->d_scene_cursor.as<unsigned long long>();
        unsigned long long* offs = c->d_scene_pair.as<unsigned long long>();
        R(cudaMemsetAsync(hist, 0, (nsc + 1) * 8, st));
        R(launch_scene_hist(p, hist, st));
        R(launch_scene_offsets(p, hist, offs, nsc, st));
        R(cudaMemsetAsync(hist, 0, (nsc + 1) * 8, st));
        R(launch_group_by_scene(p, offs, hist, c->d_out2.as<uint2>(), st));
    }
    R(cudaEventRecordWithFlags(c->ev1, st, evf));
#undef R
    return cudaSuccess;
}

// result bookkeeping after a pass: pair count, per-scene offsets, stats
static int finish_query(pbig2_ctx* c, const Ctr& h, uint64_t nboxes, uint64_t ncells, uint32_t nsc,
                        const std::vector<GridScene>& scenes, bool grouped, int launches, cudaStream_t st,
                        bool phases = true) {
    c->result_records = c->rice_mode && !grouped;
    c->rice_words = c->result_records ? h.pairs : 0;
    c->npairs = c->result_records ? h.rec_pairs : h.pairs;
    c->last_ncells = ncells;
    c->last_entries = h.entries;
    c->result = grouped ? c->d_out2.as<uint2>() : c->result_ext ? c->ext_out : c->d_out.as<uint2>();
    if (grouped) {
        CK(c->h_stage.ensure((nsc + 1) * 8));
        CK(cudaMemcpyAsync(c->h_stage.p, c->d_scene_pair.p, (nsc + 1) * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        c->scene_pair_off.assign((const uint64_t*)c->h_stage.p, (const uint64_t*)c->h_stage.p + nsc + 1);
    } else {
        c->scene_pair_off.assign(1, 0);
        c->scene_pair_off.push_back(c->npairs);
    }
    float ms = 0;
    if (phases) cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    double phase[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 5 && phases; k++) {
        float x = 0;
        if (cudaEventElapsedTime(&x, c->evp[k], c->evp[k + 1]) == cudaSuccess) phase[k] = x;
    }
    if (phases) {
        float x = 0;
        if (grouped && cudaEventElapsedTime(&x, c->evp[5], c->ev1) == cudaSuccess) phase[5] = x;
        // (the pair kernels may overlap: a phase that ends before the
        // previous one reads 0)
        if (cudaEventElapsedTime(&x, c->evp[4], c->evp[7]) == cudaSuccess) phase[6] = std::max(0.f, x);
        if (cudaEventElapsedTime(&x, c->evp[7], c->evp[8]) == cudaSuccess) phase[7] = std::max(0.f, x);
        if (cudaEventElapsedTime(&x, c->evp[8], c->evp[5]) == cudaSuccess) phase[8] = std::max(0.f, x);
    }
    c->last_err = h.err;
    pbig2_stats& s = c->stats;
    s.boxes = nboxes;
    s.bad_boxes = h.bad;
    s.cells = ncells;
    s.entries = h.entries;
    s.pair_tests = h.tests;
    s.comp_pairs = h.comp_pairs;
    s.jobs = h.jobs;
    s.max_cell = h.max_cell ? h.max_cell : (h.entries ? 1u : 0u);
    s.merged_blocks = c->merged_blocks;
    s.merge_limit = c->merge_limit;
    s.pairs = c->npairs;
    s.cell_shift = scenes.empty() ? 0 : scenes[0].shift;
    s.scenes = nsc;
    s.kernels = (uint32_t)launches;
    s.grid_retries = 0;  // set by the caller after a coarser-grid rerun
    s.device_ms = ms;
    for (int k = 0; k < 9; k++) s.phase_ms[k] = phase[k];
    (void)cudaGetLastError();  // a timing query on an unrecorded event is not an error of the query
    if (h.bad) return fail(PBIG2_EINPUT, "%u boxes violate the input contract (error bits 0x%x) and were skipped",
                           h.bad, h.err);
    return PBIG2_OK;
}

// capture the pipeline of a batched query (sizes read from device memory,
// grids and buffers sized for this query) into a graph for later batches
static int capture_graph(pbig2_ctx* c, const Params& p0, const uint32_t* d_boxes, uint64_t nboxes, uint64_t ncells,
                         uint32_t nsc, int dims, uint32_t range, uint32_t split, uint64_t entry_cap,
                         cudaStream_t st) {
    (void)entry_cap;
    CK(cudaStreamSynchronize(st));
    Params p = p0;
    p.dyn = c->d_dims.as<RunDims>();
    p.nboxes = nboxes;
    p.ncells = ncells;
    p.nscenes = nsc;
    cudaStream_t cs = c->own_stream;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = record_pipeline(c, p, dims, true, nsc, true, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_ctr.p, p.ctr, sizeof(Ctr), cudaMemcpyDeviceToHost, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(PBIG2_ECUDA, "graph capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(PBIG2_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    c->drop_graph();
    pbig2_ctx::Graph& G = c->graph;
    G.exec = ex;
    G.boxes = d_boxes;
    G.dims = dims;
    G.range = range;
    G.split = split;
    G.nboxes_cap = nboxes;
    G.ncells_cap = ncells;
    G.nscenes_cap = nsc;
    G.entry_cap = p.entry_cap;
    G.out_cap = p.out_cap;
    G.class_map = c->class_map;  // the option (0: automatic), as graph_fits compares it
    G.launches = 13;  // scene table, count (2), scan (2), expand, scatter, pairs (3), scene grouping (3)
    G.buffers = c->buffers_sig();
    return PBIG2_OK;
}

// Merged mode, the reference's h_merge_grids (src/pbig/pbig.cu:1066-1251) on
// the counts of a first pass: cells in id order; a cell that is in no block
// grows a block from itself along +x, +y (and +z), one slab at a time, while
// the new slab holds no merged cell and the block's running count (the sum of
// the first pass's per-cell counts) stays <= 256. merged[c] = the block root
// of every cell of a block of two or more cells (the root included), else
// kUnmerged. Returns the number of such blocks.
static uint32_t merge_cells(std::vector<uint32_t>& nrs, std::vector<uint32_t>& merged, uint32_t nrc, int dims,
                            uint32_t limit) {
    const uint64_t C = nrs.size();
    const uint64_t kLimit = limit;  // NTPB of the shipped build by default (256)
    merged.assign(C, kUnmerged);
    const uint64_t nrc2 = (uint64_t)nrc * nrc;
    uint32_t blocks = 0;
    // try to add the slab next to block (root, h x v x u) along axis dir
    auto grow = [&](uint64_t root, int dir, uint32_t& h, uint32_t& v, uint32_t& u) -> int {
        uint64_t step1, step2, n1, n2, base;
        if (dims == 2) {
            step1 = 0;
            n1 = 1;
            step2 = dir == 0 ? nrc : 1;
            n2 = dir == 0 ? v : h;
            base = dir == 0 ? root + h : root + (uint64_t)v * nrc;
        } else if (dir == 0) {
            step1 = nrc2; step2 = nrc; n1 = u; n2 = v; base = root + h;
        } else if (dir == 1) {
            step1 = nrc2; step2 = 1; n1 = u; n2 = h; base = root + (uint64_t)v * nrc;
        } else {
            step1 = nrc; step2 = 1; n1 = v; n2 = h; base = root + (uint64_t)u * nrc2;
        }
        for (uint64_t a = 0; a < n1; a++)
            for (uint64_t b = 0; b < n2; b++)
                if (merged[base + a * step1 + b * step2] != kUnmerged) return 0;
        uint64_t acc = nrs[root];
        for (uint64_t a = 0; a < n1; a++)
            for (uint64_t b = 0; b < n2; b++) {
                acc += nrs[base + a * step1 + b * step2];
                if (acc > kLimit) return 0;
            }
        for (uint64_t a = 0; a < n1; a++)
            for (uint64_t b = 0; b < n2; b++) merged[base + a * step1 + b * step2] = (uint32_t)root;
        merged[root] = (uint32_t)root;
        nrs[root] = (uint32_t)acc;
        if (dir == 0) h++;
        else if (dir == 1) v++;
        else u++;
        return 1;
    };
    for (uint64_t i = 0; i < C; i++) {
        if (merged[i] != kUnmerged) continue;
        const uint64_t gx = i % nrc;
        const uint64_t gy = dims == 3 ? (i % nrc2) / nrc : i / nrc;
        const uint64_t gz = dims == 3 ? i / nrc2 : 0;
        uint32_t h = 1, v = 1, u = 1;
        int progress;
        do {
            progress = 0;
            if (gx + h < nrc) progress += grow(i, 0, h, v, u);
            if (gy + v < nrc) progress += grow(i, 1, h, v, u);
            if (dims == 3 && gz + u < nrc) progress += grow(i, 2, h, v, u);
        } while (progress != 0);
        if (merged[i] == (uint32_t)i) blocks++;
    }
    return blocks;
}

static int run_pipeline(pbig2_ctx* c, const uint32_t* d_boxes, uint64_t nboxes, int dims, uint32_t range,
                        const std::vector<GridScene>& scenes, uint32_t split, double est_entries,
                        cudaStream_t st, bool group) {
    const uint32_t nsc = (uint32_t)scenes.size();
    c->last_err = 0;
    c->fused_dirty = true;  // this pipeline leaves cell starts in the counters
    if (nboxes > (uint64_t)kIdMask + 1)
        return fail(PBIG2_EINVAL, "a query holds at most 2^29 boxes (got %llu)", (unsigned long long)nboxes);
    // scene table
    std::vector<Scene> tab(nsc);
    std::vector<uint32_t> box_off(nsc + 1);
    uint64_t ncells = 0;
    for (uint32_t i = 0; i < nsc; i++) {
        const GridScene& g = scenes[i];
        Scene& s = tab[i];
        s.box_off = (uint32_t)g.box_off;
        s.n = (uint32_t)g.n;
        s.shift = g.shift;
        s.nrc = nrc_for(range, g.shift);
        s.range = range;
        s.pad = 0;
        if (g.grid_of == (int)i) {
            s.cell_off = ncells;
            const uint64_t cc = grid_cells(range, g.shift, dims);  // saturating
            ncells = cc > ~0ull - ncells ? ~0ull : ncells + cc;
        } else {
            s.cell_off = tab[g.grid_of].cell_off;
        }
        box_off[i] = (uint32_t)g.box_off;
    }
    box_off[nsc] = (uint32_t)nboxes;
    if (ncells >= (1ull << 32) - 1)
        return fail(PBIG2_EINVAL, "grid too fine: %llu cells (limit 2^32)", (unsigned long long)ncells);
    const bool grouped = group && nsc > 1;

    // a captured graph serves this query if the buffers it was captured with
    // are large enough and the fixed arguments match
    pbig2_ctx::Graph& G = c->graph;
    const bool graph_fits = c->use_graph && grouped && G.exec && G.boxes == d_boxes && G.dims == dims &&
                            G.range == range && G.split == split && nboxes <= G.nboxes_cap &&
                            ncells <= G.ncells_cap && nsc <= G.nscenes_cap && G.buffers == c->buffers_sig() &&
                            G.class_map == c->class_map;

    // tables -> pinned staging -> device (before the pipeline or graph)
    const size_t tab_bytes = nsc * sizeof(Scene), off_bytes = (nsc + 1) * sizeof(uint32_t);
    CK(c->h_stage.ensure(tab_bytes + off_bytes + sizeof(RunDims) + 64));
    CK(cudaStreamSynchronize(st));  // staging buffer reuse
    RunDims rd{};
    rd.nboxes = nboxes;
    rd.ncells = ncells;
    rd.nscenes = nsc;
    memcpy(c->h_stage.p, tab.data(), tab_bytes);
    memcpy((char*)c->h_stage.p + tab_bytes, box_off.data(), off_bytes);
    memcpy((char*)c->h_stage.p + tab_bytes + off_bytes, &rd, sizeof rd);
    if (!graph_fits) {
        CK(c->d_scenes.ensure(tab_bytes, false, st));
        CK(c->d_scene_off.ensure(off_bytes, false, st));
    }
    CK(c->d_dims.ensure(sizeof(RunDims), false, st));
    CK(cudaMemcpyAsync(c->d_scenes.p, c->h_stage.p, tab_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_scene_off.p, (char*)c->h_stage.p + tab_bytes, off_bytes, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->d_dims.p, (char*)c->h_stage.p + tab_bytes + off_bytes, sizeof rd, cudaMemcpyHostToDevice,
                       st));

    Ctr h{};
    int launches = 0;
    if (graph_fits) {
        CK(cudaEventRecord(c->ev0, st));
        CK(cudaGraphLaunch(G.exec, st));
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            return fail(PBIG2_ECUDA, "pipeline failed: %s", cudaGetErrorString(e));
        }
        memcpy(&h, c->h_ctr.p, sizeof(Ctr));
        launches = G.launches;
        const bool over = (h.err & (kErrEntryOvf | kErrTaskOvf | kErrOutOvf)) || h.entries > G.entry_cap ||
                          h.pairs > G.out_cap;
        if (h.err & kErrWait) {
            return fail(PBIG2_ETIMEOUT, "a bounded device wait gave up (scan bulk copy)");
        }
        if (over) {
            // redo eagerly with larger buffers
            // and capture again next time
            c->drop_graph();
            c->out_hint = std::max<uint64_t>(c->out_hint, h.pairs + h.pairs / 8);
            est_entries = std::max(est_entries, (double)h.entries * 1.1);
        } else {
            const int rf = finish_query(c, h, nboxes, ncells, nsc, scenes, grouped, launches, st);
            c->stats.class_map = c->class_map ? c->class_map : kClassMapDefault;
            return rf;
        }
    }

    // ---- eager run (retries on capacity) ----
    CK(c->d_counts.ensure(ncells * 4 + 16, false, st));  // zeroed by every pass
    CK(c->d_state.ensure(scan_state_bytes(ncells), false, st));
    CK(c->d_ctr.ensure(sizeof(Ctr), false, st));
    CK(c->h_ctr.ensure(sizeof(Ctr)));

    uint64_t entry_cap = (uint64_t)(est_entries * 1.25) + 4096;
    entry_cap = std::max<uint64_t>(entry_cap, c->d_entries.bytes / 4);
    uint64_t out_cap = std::max<uint64_t>({c->out_hint, nboxes * 4, 1u << 16});
    out_cap = std::max<uint64_t>(out_cap, c->d_out.bytes / 8);
    uint64_t task_cap = std::max<uint64_t>(c->d_tasks.bytes / 16, 4096);

    Params p{};
    p.boxes = d_boxes;
    p.nboxes = nboxes;
    if (c->up_red || c->up_blue) {  // the count uploads the boxes (self and red/blue queries)
        p.up_red = c->up_red;
        p.up_blue = c->up_blue;
        p.up_split = c->up_split;
        p.box_copy = const_cast<uint32_t*>(d_boxes);
    }
    p.scenes = c->d_scenes.as<Scene>();
    p.scene_box_off = c->d_scene_off.as<uint32_t>();
    if (grouped) {  // many scenes: the scene of every 256th box, for the scene lookups of the kernels
        CK(c->d_scene_tab.ensure(scene_table_entries(nboxes) * 4, false, st));
        p.scene_table = c->d_scene_tab.as<uint32_t>();
    }
    p.nscenes = nsc;
    p.split = split;
    p.max_range = range;
    p.ncells = ncells;
    p.tile_state = c->d_state.as<unsigned long long>();
    p.ctr = c->d_ctr.as<Ctr>();
    p.dyn = nullptr;
    p.class_map = c->class_map ? c->class_map : kClassMapDefault;
    c->merged_blocks = 0;
    bool one_grid = true;  // a single scene, or red and blue sharing one grid
    for (uint32_t i = 0; i < nsc; i++) one_grid = one_grid && scenes[i].grid_of == 0;
    if (c->merged_mode && one_grid && !grouped) {
        // first pass: plain counts; merge on the host; the pass below then
        // counts, bins and tests per merged block
        Params p0 = p;
        p0.counts = c->d_counts.as<uint32_t>();
        CK(cudaMemsetAsync(p.ctr, 0, sizeof(Ctr), st));
        CK(launch_count(p0, dims, st));
        std::vector<uint32_t> nrs(ncells), merged;
        CK(cudaMemcpyAsync(nrs.data(), p0.counts, ncells * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        c->merged_blocks = merge_cells(nrs, merged, tab[0].nrc, dims, c->merge_limit);
        CK(c->d_merged.ensure(ncells * 4, false, st));
        CK(cudaMemcpyAsync(c->d_merged.p, merged.data(), ncells * 4, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));  // `merged` goes out of scope
        p.merged = c->d_merged.as<uint32_t>();
    }
    bool need_full = true;
    // self/bipartite pairs go straight to the caller's buffer when one is set;
    // a result that does not fit is redone into the context's buffer
    p.records = (c->rice_mode && !grouped) ? 1u : 0u;
    if (p.records && split != kNoSplit) return fail(PBIG2_EINVAL, "record mode serves self queries only");
    bool use_ext = c->ext_out != nullptr && !grouped && !p.records;
    c->result_ext = false;
    for (int attempt = 0; attempt < 6; attempt++) {
        int rc = ensure_query_buffers(c, p, entry_cap, use_ext ? 1 : out_cap, task_cap, nsc, grouped, st);
        if (rc) return rc;
        if (use_ext) {
            p.out = c->ext_out;
            p.out_cap = c->ext_cap;
        }
        if (attempt == 0) CK(cudaEventRecord(c->ev0, st));
        {
            const cudaError_t re = record_pipeline(c, p, dims, grouped, nsc, need_full, st);
            if (re != cudaSuccess)
                return fail(PBIG2_ECUDA, "pipeline launch (engine.cu:%d): %s", g_record_line, cudaGetErrorString(re));
        }
        launches += need_full ? 6 : 0;  // count, scan (3), expand, scatter
        launches += 3 + (grouped ? 3 : 0) + (p.records ? 1 : 0) + (need_full && p.scene_table ? 1 : 0);
        CK(cudaMemcpyAsync(c->h_ctr.p, p.ctr, sizeof(Ctr), cudaMemcpyDeviceToHost, st));
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            return fail(PBIG2_ECUDA, "pipeline failed: %s", cudaGetErrorString(e));
        }
        memcpy(&h, c->h_ctr.p, sizeof(Ctr));
        if (h.err & kErrWait) {
            return fail(PBIG2_ETIMEOUT, "a bounded device wait gave up (scan bulk copy)");
        }
        if (h.err & kErrRecCell)
            return fail(PBIG2_ECAPACITY, "a cell of 65536 boxes or more cannot be written as records");
        if (h.err & kErrIndex) {
            return fail(PBIG2_ECUDA, "inconsistent cell lists (error bits 0x%x)", h.err);
        }
        if ((h.err & kErrEntryOvf) || h.entries > p.entry_cap) {
            if (h.entries >= (1ull << 32))
                return fail(PBIG2_ENOMEM, "%llu cell entries exceed the 2^32 limit of one query",
                            (unsigned long long)h.entries);
            entry_cap = h.entries + h.entries / 16 + 4096;
            need_full = true;
            continue;
        }
        if (h.err & kErrTaskOvf) {
            task_cap = (uint64_t)h.need_tasks + 1024;
            need_full = true;
            continue;
        }
        if ((h.err & kErrOutOvf) || h.pairs > p.out_cap) {
            out_cap = std::max<uint64_t>(out_cap, h.pairs + h.pairs / 8 + 1024);
            use_ext = false;
            need_full = false;
            continue;
        }
        break;
    }
    c->result_ext = use_ext;
    if (h.err & (kErrEntryOvf | kErrTaskOvf | kErrOutOvf)) return fail(PBIG2_ENOMEM, "capacity retries exhausted");
    c->out_hint = std::max<uint64_t>(c->out_hint, h.pairs + h.pairs / 8);
    int rc = finish_query(c, h, nboxes, ncells, nsc, scenes, grouped, launches, st);
    c->stats.class_map = p.class_map;
    if (rc != PBIG2_OK && rc != PBIG2_EINPUT) return rc;
    // capture this query's pipeline for later batches of the same shape
    if (G.exec && G.buffers != c->buffers_sig()) c->drop_graph();
    if (c->use_graph && grouped && !G.exec) {
        int rg = capture_graph(c, p, d_boxes, nboxes, ncells, nsc, dims, range, split, entry_cap, st);
        if (rg) return rg;
    }
    return rc;
}

// One-launch query of a small scene (kernels.cuh: launch_fused). Returns
// kFusedRedo when the result did not fit the buffers it was given (the
// caller then runs the regular pipeline, and the hints grow for next time).
constexpr int kFusedRedo = -1000;

static bool fused_eligible(const pbig2_ctx* c, uint64_t n, int dims, uint32_t range, uint32_t cell_shift) {
    if (!c->use_fused || fused_blocks() <= 0 || c->merged_mode || c->rice_mode) return false;
    if (n == 0 || n > kFusedMaxBoxes) return false;
    return cell_shift == PBIG2_AUTO || grid_cells(range, cell_shift, dims) <= kFusedMaxCells;
}

static int fused_query(pbig2_ctx* c, const uint32_t* d_boxes, uint64_t n, int dims, uint32_t range,
                       uint32_t cell_shift, cudaStream_t st) {
    c->last_err = 0;
    const uint64_t cells_cap = cell_shift == PBIG2_AUTO ? kFusedMaxCells : grid_cells(range, cell_shift, dims);
    void* counts_before = c->d_counts.p;
    CK(c->d_counts.ensure(cells_cap * 4 + 16, false, st));
    if (c->d_counts.p != counts_before) c->fused_dirty = true;
    CK(c->d_state.ensure(kFusedMaxCells / 512 * 4 + 8192 * 4, false, st));  // chunk totals, then small-grid cell ends
    CK(c->h_ctr.ensure(sizeof(Ctr)));
    CK(c->d_scenes.ensure(sizeof(Scene), false, st));
    if (!c->d_bar.p || !c->d_fctr.p) {
        CK(c->d_bar.ensure(sizeof(unsigned int), true, st));
        CK(c->d_fctr.ensure(2 * sizeof(Ctr), true, st));
        c->bar_base = 0;
        c->fused_slot = 0;
    }
    const uint64_t entry_cap = std::max<uint64_t>({c->fused_entry_hint, 8 * n + 4096, c->d_entries.bytes / 4});
    const uint64_t out_cap = std::max<uint64_t>({c->out_hint, n * 4, 1u << 16, c->d_out.bytes / 8});
    const uint64_t task_cap = std::max<uint64_t>(c->d_tasks.bytes / 16, 4096);
    const bool use_ext = c->ext_out != nullptr;
    Ctr* slots = c->d_fctr.as<Ctr>();
    Params p{};
    p.boxes = d_boxes;
    p.nboxes = n;
    p.scenes = c->d_scenes.as<Scene>();
    p.nscenes = 1;
    p.split = kNoSplit;
    p.max_range = range;
    p.tile_state = c->d_state.as<unsigned long long>();
    p.class_map = c->class_map ? c->class_map : kClassMapOneLaunch;
    int rc = ensure_query_buffers(c, p, entry_cap, use_ext ? 1 : out_cap, task_cap, 1, false, st);
    if (rc) return rc;
    p.ctr = slots + c->fused_slot;
    if (use_ext) {
        p.out = c->ext_out;
        p.out_cap = c->ext_cap;
    }
    FusedArgs a{};
    a.bar = c->d_bar.as<unsigned int>();
    // (test of the bounded wait: a count far ahead of every arrival)
    a.bar_base = c->fused_stall_test ? c->bar_base + (1u << 24) : c->bar_base;
    c->fused_stall_test = false;
    a.chunk_sum = c->d_state.as<uint32_t>();
    a.ends = c->d_state.as<uint32_t>() + kFusedMaxCells / 512;
    a.scenes = c->d_scenes.as<Scene>();
    a.ctr_next = slots + (c->fused_slot ^ 1);
    a.zero_cells = c->fused_dirty ? std::min<uint64_t>(kFusedMaxCells, c->d_counts.bytes / 4) : 0;
    a.shift = cell_shift == PBIG2_AUTO ? kFusedTune : cell_shift;
    // the kernel's last block writes the counters to h_ctr (page-locked);
    // `barriers` stays at this mark when the launch gave up before that
    Ctr* hc = static_cast<Ctr*>(c->h_ctr.p);
    hc->barriers = 0xffffffffu;
    a.ctr_host = hc;
    CK(launch_fused(p, a, dims, st));
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(PBIG2_ECUDA, "one-launch query failed: %s", cudaGetErrorString(e));
    Ctr h{};
    memcpy(&h, hc, sizeof(Ctr));
    if (h.barriers == 0xffffffffu) {  // no block copied the counters: read them
        CK(cudaMemcpy(&h, p.ctr, sizeof(Ctr), cudaMemcpyDeviceToHost));
        h.err |= kErrWait;
    }
    if (h.err & kErrWait) {
        // the barriers' count and the counters are unknown now: start again from zero
        CK(cudaMemsetAsync(c->d_bar.p, 0, sizeof(unsigned int), st));
        CK(cudaMemsetAsync(c->d_fctr.p, 0, 2 * sizeof(Ctr), st));
        CK(cudaStreamSynchronize(st));
        c->bar_base = 0;
        c->fused_slot = 0;
        c->fused_dirty = true;
        return fail(PBIG2_ETIMEOUT, "a bounded device wait gave up (grid barrier of a one-launch query)");
    }
    c->bar_base += h.barriers * (unsigned int)fused_blocks();
    c->fused_slot ^= 1;
    c->fused_dirty = false;
    if (h.err & kErrIndex) return fail(PBIG2_ECUDA, "inconsistent cell lists (error bits 0x%x)", h.err);
    if ((h.err & (kErrEntryOvf | kErrTaskOvf | kErrOutOvf)) || h.entries > p.entry_cap || h.pairs > p.out_cap) {
        c->fused_entry_hint = std::max<uint64_t>(c->fused_entry_hint, h.entries + h.entries / 8 + 4096);
        if (!use_ext || h.pairs <= p.out_cap) c->out_hint = std::max<uint64_t>(c->out_hint, h.pairs + h.pairs / 8);
        return kFusedRedo;
    }
    c->result_ext = use_ext;
    c->out_hint = std::max<uint64_t>(c->out_hint, h.pairs + h.pairs / 8);
    c->merged_blocks = 0;
    std::vector<GridScene> sc{{0, n, h.shift, 0}};
    rc = finish_query(c, h, n, h.cells, 1, sc, false, 1, st, false);
    c->stats.class_map = p.class_map;
    c->stats.device_ms = h.t_end > h.t_start ? (double)(h.t_end - h.t_start) * 1e-6 : 0.0;  // the kernel's own clock
    return rc;
}

static cudaStream_t pick_stream(pbig2_ctx* c, void* stream) {
    return stream ? (cudaStream_t)stream : c->own_stream;
}

// strided sample of device-resident boxes (host copy) for the autotuner
static int sample_device_boxes(pbig2_ctx* c, const uint32_t* d_boxes, uint64_t n, int dims, uint64_t m,
                               cudaStream_t st, std::vector<uint32_t>& out) {
    const int W = 2 * dims + 1;
    m = std::min<uint64_t>(m, n);
    out.resize(m * W);
    if (m == 0) return PBIG2_OK;
    CK(c->h_stage.ensure(m * W * 4));
    const uint64_t stride = n / m;
    CK(cudaMemcpy2DAsync(c->h_stage.p, W * 4, d_boxes, stride * W * 4, W * 4, m, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    memcpy(out.data(), c->h_stage.p, m * W * 4);
    return PBIG2_OK;
}

// device-mapped address of page-locked host memory, or null (pageable memory)
static const uint32_t* mapped_host(const uint32_t* h) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? static_cast<const uint32_t*>(a.devicePointer) : nullptr;
}

static int stage_boxes_in(pbig2_ctx* c, const uint32_t* boxes, uint64_t words, int loc, cudaStream_t st,
                          const uint32_t** d_boxes) {
    if (loc == PBIG2_DEVICE) {
        *d_boxes = boxes;
        return PBIG2_OK;
    }
    CK(c->d_boxes.ensure(words * 4, false, st));
    CK(cudaMemcpyAsync(c->d_boxes.p, boxes, words * 4, cudaMemcpyHostToDevice, st));
    *d_boxes = c->d_boxes.as<uint32_t>();
    return PBIG2_OK;
}

}  // namespace pbig

using namespace pbig;

extern "C" {

PBIG2_API const char* pbig2_last_error(void) { return g_last_error.c_str(); }

PBIG2_API int pbig2_version(void) { return 1; }

PBIG2_API int pbig2_create(int device, pbig2_ctx** out) {
    if (!out) return fail(PBIG2_EINVAL, "out is null");
    *out = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(PBIG2_EINVAL, "device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));
    pbig2_ctx* c = new pbig2_ctx();
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    for (int k = 0; k < 9 && e == cudaSuccess; k++) e = cudaEventCreate(&c->evp[k]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = kernels_init();
    if (e != cudaSuccess) {
        pbig2_destroy(c);
        return fail(PBIG2_ECUDA, "context setup: %s", cudaGetErrorString(e));
    }
    *out = c;
    return PBIG2_OK;
}

PBIG2_API int pbig2_destroy(pbig2_ctx* c) {
    if (!c) return PBIG2_OK;
    cudaSetDevice(c->device);
    if (c->own_stream) cudaStreamSynchronize(c->own_stream);
    c->drop_graph();
    for (DevBuf* b : {&c->d_boxes, &c->d_counts, &c->d_entries, &c->d_bar, &c->d_fctr,
                      &c->d_lists, &c->d_tasks, &c->d_state,
                      &c->d_out, &c->d_out2, &c->d_ctr, &c->d_scenes, &c->d_scene_off, &c->d_scene_pair,
                      &c->d_scene_cursor, &c->d_dims, &c->d_scene_tab, &c->d_tune})
        b->release();
    c->h_ctr.release();
    c->h_stage.release();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (cudaEvent_t ev : c->evp)
        if (ev) cudaEventDestroy(ev);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side_stream) cudaStreamDestroy(c->side_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return PBIG2_OK;
}

PBIG2_API uint64_t pbig2_class_map_auto(uint32_t one_launch) {
    return one_launch ? kClassMapOneLaunch : kClassMapDefault;
}

PBIG2_API uint32_t pbig2_class_map_check(uint64_t map) { return class_map_check(map); }

PBIG2_API uint64_t pbig2_grid_cells(uint32_t range, uint32_t shift, uint32_t dims) {
    return grid_cells(range, shift, (int)dims);
}

PBIG2_API int pbig2_tune_shift(const uint32_t* boxes, uint64_t n, uint32_t dims, uint32_t range, uint64_t sample,
                               uint32_t* shift) {
    if (!boxes || !shift || (dims != 2 && dims != 3) || range == 0) return fail(PBIG2_EINVAL, "bad arguments");
    *shift = tune_shift_sample(boxes, n, n, (int)dims, range, sample ? sample : 4096).shift;
    return PBIG2_OK;
}

// autotuner with a per-context memo: a query whose size, dims, range and
// mean box extent (over 256 strided boxes) match an earlier one within 5%
// reuses that choice
constexpr uint64_t kMemoRows = 256;

static double mean_extent(const uint32_t* boxes, uint64_t n_avail, int dims) {
    const int W = 2 * dims + 1;
    const uint64_t m = std::min<uint64_t>(n_avail, kMemoRows);
    double ext = 0;
    for (uint64_t i = 0; i < m; i++) {
        const uint32_t* b = boxes + (uint64_t)((unsigned __int128)i * n_avail / m) * W;
        for (int d = 0; d < dims; d++) ext += (double)b[2 * d + 1] - (double)b[2 * d];
    }
    return m ? ext / (double)(m * dims) : 0;
}

static bool memo_find(pbig2_ctx* c, uint64_t n, int dims, uint32_t range, double ext, TuneResult& tr) {
    for (const auto& e : c->memo)
        if (e.dims == dims && e.range == range && std::fabs((double)e.n - (double)n) <= 0.05 * (double)n &&
            std::fabs(e.ext - ext) <= 0.05 * std::max(1.0, e.ext)) {
            tr = TuneResult{e.shift, e.est_e * (double)n / std::max(1.0, (double)e.n), 0, 0};
            return true;
        }
    return false;
}

static void memo_put(pbig2_ctx* c, uint64_t n, int dims, uint32_t range, double ext, const TuneResult& tr) {
    if (c->memo.size() >= 64) c->memo.erase(c->memo.begin());
    c->memo.push_back({n, dims, range, ext, tr.shift, tr.est_entries});
}

static TuneResult memo_tune(pbig2_ctx* c, const uint32_t* boxes, uint64_t n_avail, uint64_t n, int dims,
                            uint32_t range, uint64_t sample) {
    const double ext = mean_extent(boxes, n_avail, dims);
    TuneResult tr{};
    if (memo_find(c, n, dims, range, ext, tr)) return tr;
    tr = tune_shift_sample(boxes, n_avail, n, dims, range, sample);
    memo_put(c, n, dims, range, ext, tr);
    return tr;
}

// A box outside the tuner's sample can cover 2^26 cells or more at the cell
// size chosen from the sample; the count kernel then skips it as an input
// error (kErrCellOvf). A query whose cell sizes were chosen automatically is
// then run again on grids twice as coarse per axis, until every box fits.
static bool coarser_grid_helps(const pbig2_ctx* c, int rc) {
    return rc == PBIG2_EINPUT && (c->last_err & kErrCellOvf) != 0;
}

// later queries of a remembered scene start at the cell size that fitted
static void memo_raise(pbig2_ctx* c, uint64_t n, int dims, uint32_t range, uint32_t from, uint32_t to) {
    for (auto& e : c->memo)
        if (e.n == n && e.dims == dims && e.range == range && e.shift == from) e.shift = to;
}

static int self_or_bip(pbig2_ctx* c, const uint32_t* red, uint64_t n_red, const uint32_t* blue, uint64_t n_blue,
                       uint32_t dims, uint32_t range, uint32_t cell_shift, int loc, void* stream, uint64_t* npairs) {
    if (!c || !npairs || (dims != 2 && dims != 3) || range == 0) return fail(PBIG2_EINVAL, "bad arguments");
    if ((n_red && !red) || (n_blue && !blue)) return fail(PBIG2_EINVAL, "null box pointer");
    if (cell_shift != PBIG2_AUTO && cell_shift > 31) return fail(PBIG2_EINVAL, "cell_shift %u > 31", cell_shift);
    *npairs = 0;
    CK(cudaSetDevice(c->device));
    cudaStream_t st = pick_stream(c, stream);
    const int W = 2 * (int)dims + 1;
    const bool bip = blue != nullptr;
    const uint64_t n = n_red + n_blue;
    const uint32_t* d_boxes = nullptr;
    if (!bip && fused_eligible(c, n, (int)dims, range, cell_shift)) {
        int rc = stage_boxes_in(c, red, n * W, loc, st, &d_boxes);
        if (rc) return rc;
        rc = fused_query(c, d_boxes, n, (int)dims, range, cell_shift, st);
        if (rc != kFusedRedo) {
            c->scene_shifts.assign(1, c->stats.cell_shift);
            *npairs = c->npairs;
            return rc;
        }
    }
    // page-locked host input needs no copy before the pipeline: the count
    // kernel reads it over the host link and writes the device copy
    const uint32_t* m_red = loc == PBIG2_HOST && n_red ? mapped_host(red) : nullptr;
    const uint32_t* m_blue = loc == PBIG2_HOST && bip && n_blue ? mapped_host(blue) : nullptr;
    const bool fused = loc == PBIG2_HOST && n > 0 && (n_red == 0 || m_red) && (!bip || n_blue == 0 || m_blue);
    if (fused) {
        CK(c->d_boxes.ensure(n * W * 4 + 16, false, st));
        d_boxes = c->d_boxes.as<uint32_t>();
    } else if (!bip) {
        int rc = stage_boxes_in(c, red, n_red * W, loc, st, &d_boxes);
        if (rc) return rc;
    } else {
        CK(c->d_boxes.ensure(n * W * 4 + 16, false, st));
        const cudaMemcpyKind k = loc == PBIG2_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        if (n_red) CK(cudaMemcpyAsync(c->d_boxes.p, red, n_red * W * 4, k, st));
        if (n_blue) CK(cudaMemcpyAsync(c->d_boxes.as<uint32_t>() + n_red * W, blue, n_blue * W * 4, k, st));
        d_boxes = c->d_boxes.as<uint32_t>();
    }
    // choose the cell size (from a sample of the union for red/blue)
    TuneResult tr{};
    std::vector<uint32_t> smp;
    const uint64_t kSample = 4096;
    if (cell_shift != PBIG2_AUTO) {
        tr.shift = cell_shift;
    } else if (loc == PBIG2_HOST && !bip) {
        tr = memo_tune(c, red, n, n, (int)dims, range, kSample);
    } else {
        if (loc == PBIG2_HOST) {
            const uint64_t m = std::min<uint64_t>(n, kSample);
            smp.resize(m * W);
            for (uint64_t i = 0; i < m; i++) {
                const uint64_t g = (uint64_t)((unsigned __int128)i * n / m);
                const uint32_t* src = g < n_red ? red + g * W : blue + (g - n_red) * W;
                memcpy(&smp[i * W], src, W * 4);
            }
            tr = memo_tune(c, smp.data(), smp.size() / W, n, (int)dims, range, kSample);
        } else {
            // device-resident boxes: 256 rows recognise a remembered scene;
            // the full sample crosses to the host only when none matches
            int rc = sample_device_boxes(c, d_boxes, n, (int)dims, kMemoRows, st, smp);
            if (rc) return rc;
            const double ext = mean_extent(smp.data(), smp.size() / W, (int)dims);
            if (!memo_find(c, n, (int)dims, range, ext, tr)) {
                rc = sample_device_boxes(c, d_boxes, n, (int)dims, kSample, st, smp);
                if (rc) return rc;
                tr = tune_shift_sample(smp.data(), smp.size() / W, n, (int)dims, range, kSample);
                memo_put(c, n, (int)dims, range, ext, tr);
            }
        }
    }
    std::vector<GridScene> sc;
    if (!bip) {
        sc.push_back({0, n, tr.shift, 0});
    } else {
        sc.push_back({0, n_red, tr.shift, 0});
        sc.push_back({n_red, n_blue, tr.shift, 0});
    }
    if (fused) {
        c->up_red = m_red;
        c->up_blue = m_blue;
        c->up_split = n_red;
    }
    int rc = run_pipeline(c, d_boxes, n, (int)dims, range, sc, bip ? (uint32_t)n_red : kNoSplit,
                          std::max(tr.est_entries, (double)n), st, false);
    if (cell_shift == PBIG2_AUTO && coarser_grid_helps(c, rc)) {
        const uint32_t first = tr.shift;
        while (coarser_grid_helps(c, rc) && tr.shift < 31) {
            tr.shift++;
            for (auto& g : sc) g.shift = tr.shift;
            rc = run_pipeline(c, d_boxes, n, (int)dims, range, sc, bip ? (uint32_t)n_red : kNoSplit,
                              std::max(tr.est_entries, (double)n), st, false);
        }
        memo_raise(c, n, (int)dims, range, first, tr.shift);
        c->stats.grid_retries = tr.shift - first;
    }
    c->up_red = c->up_blue = nullptr;
    c->scene_shifts.assign(1, tr.shift);
    *npairs = c->npairs;
    return rc;
}

PBIG2_API int pbig2_self_intersect(pbig2_ctx* c, const uint32_t* boxes, uint64_t n, uint32_t dims, uint32_t range,
                                   uint32_t cell_shift, int boxes_loc, void* stream, uint64_t* npairs) {
    return self_or_bip(c, boxes, n, nullptr, 0, dims, range, cell_shift, boxes_loc, stream, npairs);
}

PBIG2_API int pbig2_bipartite_intersect(pbig2_ctx* c, const uint32_t* red, uint64_t n_red, const uint32_t* blue,
                                        uint64_t n_blue, uint32_t dims, uint32_t range, uint32_t cell_shift,
                                        int boxes_loc, void* stream, uint64_t* npairs) {
    if (!blue && n_blue == 0) {
        static const uint32_t dummy[8] = {0};
        blue = dummy;
    }
    return self_or_bip(c, red, n_red, blue, n_blue, dims, range, cell_shift, boxes_loc, stream, npairs);
}

PBIG2_API int pbig2_batch_intersect(pbig2_ctx* c, const uint32_t* boxes, const uint64_t* scene_offsets,
                                    uint32_t n_scenes, uint32_t dims, uint32_t range, const uint32_t* cell_shifts,
                                    int boxes_loc, void* stream, uint64_t* npairs) {
    if (!c || !npairs || !scene_offsets || (dims != 2 && dims != 3) || range == 0 || n_scenes == 0)
        return fail(PBIG2_EINVAL, "bad arguments");
    *npairs = 0;
    CK(cudaSetDevice(c->device));
    cudaStream_t st = pick_stream(c, stream);
    const int W = 2 * (int)dims + 1;
    const uint64_t n = scene_offsets[n_scenes];
    for (uint32_t i = 0; i < n_scenes; i++)
        if (scene_offsets[i + 1] < scene_offsets[i]) return fail(PBIG2_EINVAL, "scene offsets must not decrease");
    if (n && !boxes) return fail(PBIG2_EINVAL, "null boxes");
    const uint32_t* d_boxes = nullptr;
    int rc = stage_boxes_in(c, boxes, n * W, boxes_loc, st, &d_boxes);
    if (rc) return rc;
    // per-scene cell sizes: given, or chosen on the device (k_tune_scenes,
    // one warp per scene on up to 64 of its boxes); one small copy back
    std::vector<GridScene> sc(n_scenes);
    double est_e = 0;
    const SceneTune* tuned = nullptr;
    if (!cell_shifts) {
        const size_t off_bytes = ((size_t)n_scenes + 1) * 8, tune_bytes = (size_t)n_scenes * sizeof(SceneTune);
        CK(c->h_stage.ensure(off_bytes + tune_bytes));
        CK(cudaStreamSynchronize(st));  // staging buffer reuse
        CK(c->d_tune.ensure(off_bytes + tune_bytes, false, st));
        memcpy(c->h_stage.p, scene_offsets, off_bytes);
        const unsigned long long* d_offs = c->d_tune.as<unsigned long long>();
        SceneTune* d_res = reinterpret_cast<SceneTune*>(c->d_tune.as<char>() + off_bytes);
        CK(cudaMemcpyAsync(c->d_tune.p, c->h_stage.p, off_bytes, cudaMemcpyHostToDevice, st));
        CK(launch_tune_scenes(d_boxes, d_offs, n_scenes, (int)dims, range, d_res, st));
        CK(cudaMemcpyAsync((char*)c->h_stage.p + off_bytes, d_res, tune_bytes, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        tuned = reinterpret_cast<const SceneTune*>((const char*)c->h_stage.p + off_bytes);
    }
    for (uint32_t i = 0; i < n_scenes; i++) {
        const uint64_t a = scene_offsets[i], b = scene_offsets[i + 1], ns = b - a;
        uint32_t shift;
        double e = (double)ns;
        if (cell_shifts) {
            shift = cell_shifts[i];
            if (shift > 31) return fail(PBIG2_EINVAL, "cell_shifts[%u] > 31", i);
        } else {
            shift = tuned[i].shift;
            e = std::max(e, tuned[i].est_entries);
        }
        sc[i] = GridScene{a, ns, shift, (int)i};
        est_e += e;
    }
    rc = run_pipeline(c, d_boxes, n, (int)dims, range, sc, kNoSplit, est_e, st, true);
    // automatic cell sizes: coarser grids for every scene while a box does
    // not fit (the failing scene is not known)
    uint32_t retries = 0;
    while (!cell_shifts && coarser_grid_helps(c, rc)) {
        bool raised = false;
        for (auto& g : sc)
            if (g.shift < 31) {
                g.shift++;
                raised = true;
            }
        if (!raised) break;
        rc = run_pipeline(c, d_boxes, n, (int)dims, range, sc, kNoSplit, est_e, st, true);
        retries++;
    }
    c->stats.grid_retries = retries;
    c->scene_shifts.resize(n_scenes);
    for (uint32_t i = 0; i < n_scenes; i++) c->scene_shifts[i] = sc[i].shift;
    *npairs = c->npairs;
    return rc;
}

PBIG2_API int pbig2_result_pairs(pbig2_ctx* c, const uint32_t** dev_pairs, uint64_t* npairs) {
    if (!c || !dev_pairs || !npairs) return fail(PBIG2_EINVAL, "bad arguments");
    *dev_pairs = reinterpret_cast<const uint32_t*>(c->result);
    *npairs = c->npairs;
    return PBIG2_OK;
}

PBIG2_API int pbig2_copy_pairs(pbig2_ctx* c, uint32_t* dst, uint64_t first, uint64_t count, int dst_loc,
                               void* stream) {
    if (!c || (count && !dst)) return fail(PBIG2_EINVAL, "bad arguments");
    if (c->result_records) return fail(PBIG2_EINVAL, "the last result is a record stream (pbig2_result_records)");
    if (first > c->npairs || count > c->npairs - first) return fail(PBIG2_EINVAL, "range beyond the result");
    if (count == 0) return PBIG2_OK;
    CK(cudaSetDevice(c->device));
    cudaStream_t st = pick_stream(c, stream);
    if ((const void*)dst == (const void*)(c->result + first)) return PBIG2_OK;  // already there
    // the result is in device memory or in the caller's page-locked buffer
    CK(cudaMemcpyAsync(dst, c->result + first, count * 8, cudaMemcpyDefault, st));
    if (dst_loc != PBIG2_DEVICE) CK(cudaStreamSynchronize(st));
    return PBIG2_OK;
}

PBIG2_API int pbig2_copy_pairs_async(pbig2_ctx* c, uint32_t* dst, uint64_t first, uint64_t count, int dst_loc,
                                     void* stream) {
    if (!c || (count && !dst)) return fail(PBIG2_EINVAL, "bad arguments");
    if (c->result_records) return fail(PBIG2_EINVAL, "the last result is a record stream (pbig2_result_records)");
    if (first > c->npairs || count > c->npairs - first) return fail(PBIG2_EINVAL, "range beyond the result");
    if (count == 0) return PBIG2_OK;
    CK(cudaSetDevice(c->device));
    (void)dst_loc;
    if ((const void*)dst == (const void*)(c->result + first)) return PBIG2_OK;  // already there
    CK(cudaMemcpyAsync(dst, c->result + first, count * 8, cudaMemcpyDefault, pick_stream(c, stream)));
    return PBIG2_OK;
}

PBIG2_API int pbig2_result_records(pbig2_ctx* c, const uint64_t** words, uint64_t* nwords, const uint32_t** start_i,
                                   uint64_t* ncells, const uint32_t** recs, uint64_t* nentries) {
    if (!c || !words || !nwords || !start_i || !ncells || !recs || !nentries) return fail(PBIG2_EINVAL, "bad arguments");
    if (!c->result_records) return fail(PBIG2_EINVAL, "the last result is not a record stream (PBIG2_OPT_RICE)");
    *words = reinterpret_cast<const uint64_t*>(c->result);
    *nwords = c->rice_words;
    *start_i = c->d_counts.as<uint32_t>();
    *ncells = c->last_ncells;
    *recs = c->d_entries.as<uint32_t>();
    *nentries = c->last_entries;
    return PBIG2_OK;
}

PBIG2_API int pbig2_copy_records(pbig2_ctx* c, uint64_t* words, uint32_t* start_i, uint32_t* recs) {
    if (!c || (!words && !start_i && !recs)) return fail(PBIG2_EINVAL, "bad arguments");
    if (!c->result_records) return fail(PBIG2_EINVAL, "the last result is not a record stream (PBIG2_OPT_RICE)");
    CK(cudaSetDevice(c->device));
    cudaStream_t st = c->own_stream;
    if (words && c->rice_words) CK(cudaMemcpyAsync(words, c->result, c->rice_words * 8, cudaMemcpyDefault, st));
    if (start_i && c->last_ncells) CK(cudaMemcpyAsync(start_i, c->d_counts.p, c->last_ncells * 4, cudaMemcpyDefault, st));
    if (recs && c->last_entries) CK(cudaMemcpyAsync(recs, c->d_entries.p, c->last_entries * 4, cudaMemcpyDefault, st));
    CK(cudaStreamSynchronize(st));
    return PBIG2_OK;
}

// the reference's decode() (src/pbig/decode.cc:26-138) for the Rice records,
// with the column bytes read where the writer puts them (record + 6 + k;
// the reference reads record + 10 + k, decode.cc:80 against pbig.cu:851)
PBIG2_API int pbig2_decode_records(const uint64_t* w, uint64_t nwords, const uint32_t* start_i, uint64_t ncells,
                                   const uint32_t* recs, uint64_t nentries, uint32_t* pairs, uint64_t cap,
                                   uint64_t* npairs) {
    if (!npairs || (nwords && (!w || !start_i || !recs)) || (cap && !pairs)) return fail(PBIG2_EINVAL, "bad arguments");
    const uint64_t kUnused = 0x0fffff11ull;
    uint64_t np = 0, i = 0;
    while (i < nwords) {
        if (w[i] != kUnused || i + 1 >= nwords) return fail(PBIG2_EINPUT, "record stream: block header expected at word %llu", (unsigned long long)i);
        const uint64_t gid = w[i + 1];
        if (gid >= ncells) return fail(PBIG2_EINPUT, "record stream: cell %llu out of range", (unsigned long long)gid);
        i += 2;
        while (i < nwords && w[i] != kUnused) {
            const unsigned char* r = reinterpret_cast<const unsigned char*>(w + i);
            const uint32_t seg1 = r[0], seg2 = r[1];
            const uint32_t lrow = (uint32_t)r[2] | ((uint32_t)r[3] << 8);
            const uint32_t nh = (uint32_t)r[4] | ((uint32_t)r[5] << 8);
            const uint64_t len = (6u + nh + 7u) >> 3;
            if (i + len > nwords) return fail(PBIG2_EINPUT, "record stream: record past the end");
            const uint64_t base1 = (uint64_t)start_i[gid] + (seg1 << 8), base2 = (uint64_t)start_i[gid] + (seg2 << 8);
            if (base1 + lrow >= nentries) return fail(PBIG2_EINPUT, "record stream: row past the entries");
            const uint32_t a = recs[base1 + lrow];
            for (uint32_t k = 0; k < nh; k++) {
                const uint64_t e = base2 + r[6 + k];
                if (e >= nentries) return fail(PBIG2_EINPUT, "record stream: column past the entries");
                const uint32_t b = recs[e];
                if (np < cap) {
                    pairs[2 * np] = a < b ? a : b;
                    pairs[2 * np + 1] = a < b ? b : a;
                }
                np++;
            }
            i += len;
        }
    }
    *npairs = np;
    return np <= cap ? PBIG2_OK : fail(PBIG2_ECAPACITY, "pair buffer too small; *npairs holds the pair count");
}

PBIG2_API int pbig2_set_pair_output(pbig2_ctx* c, uint32_t* dst, uint64_t cap_pairs) {
    if (!c || (dst && cap_pairs == 0)) return fail(PBIG2_EINVAL, "bad arguments");
    if (dst) {
        // the pair kernels store into dst: it must be device memory or
        // page-locked host memory mapped into the device's address space
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, dst) != cudaSuccess || a.type == cudaMemoryTypeUnregistered ||
            a.devicePointer == nullptr) {
            (void)cudaGetLastError();
            return fail(PBIG2_EINVAL, "pair output must be device memory or page-locked (pbig2_host_alloc) host memory");
        }
        if (((uintptr_t)dst & 7u) != 0) return fail(PBIG2_EINVAL, "pair output must be 8-byte aligned");
        c->ext_out = reinterpret_cast<uint2*>(a.devicePointer);
        c->ext_host = a.type == cudaMemoryTypeHost;
    } else {
        c->ext_out = nullptr;
        c->ext_host = false;
    }
    c->ext_cap = dst ? cap_pairs : 0;
    return PBIG2_OK;
}

PBIG2_API int pbig2_sync(pbig2_ctx* c, void* stream) {
    if (!c) return fail(PBIG2_EINVAL, "bad arguments");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(pick_stream(c, stream)));
    return PBIG2_OK;
}

PBIG2_API int pbig2_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(PBIG2_EINVAL, "bad arguments");
    *ptr = nullptr;
    CK(cudaMallocHost(ptr, bytes ? bytes : 1));
    return PBIG2_OK;
}

PBIG2_API int pbig2_host_free(void* ptr) {
    if (ptr) CK(cudaFreeHost(ptr));
    return PBIG2_OK;
}

PBIG2_API int pbig2_result_scene_offsets(pbig2_ctx* c, uint64_t* offsets, uint32_t n_scenes) {
    if (!c || !offsets) return fail(PBIG2_EINVAL, "bad arguments");
    if (c->scene_pair_off.size() != (size_t)n_scenes + 1)
        return fail(PBIG2_EINVAL, "last result has %zu scenes", c->scene_pair_off.size() - 1);
    memcpy(offsets, c->scene_pair_off.data(), (n_scenes + 1) * 8);
    return PBIG2_OK;
}

PBIG2_API int pbig2_result_scene_shifts(pbig2_ctx* c, uint32_t* shifts, uint32_t n_scenes) {
    if (!c || !shifts) return fail(PBIG2_EINVAL, "bad arguments");
    if (c->scene_shifts.size() != (size_t)n_scenes)
        return fail(PBIG2_EINVAL, "last query has %zu scenes", c->scene_shifts.size());
    memcpy(shifts, c->scene_shifts.data(), (size_t)n_scenes * 4);
    return PBIG2_OK;
}

PBIG2_API int pbig2_set_option(pbig2_ctx* c, int option, int64_t value) {
    if (!c) return fail(PBIG2_EINVAL, "bad arguments");
    if (option == PBIG2_OPT_GRAPH) {
        c->use_graph = value != 0;
        if (!c->use_graph) c->drop_graph();
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_MERGED) {
        c->merged_mode = value != 0;
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_RICE) {
        c->rice_mode = value != 0;
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_CLASS_MAP) {
        const unsigned long long map = (unsigned long long)value;
        if (map) {
            const uint32_t bad = class_map_check(map);
            if (bad)
                return fail(PBIG2_EINVAL, "class map 0x%llx: bucket %u names a list that cannot hold its cells", map,
                            bad);
        }
        c->class_map = map;
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_MERGE_LIMIT) {
        if (value < 0 || value > (1 << 30)) return fail(PBIG2_EINVAL, "merge limit %lld", (long long)value);
        c->merge_limit = value ? (uint32_t)value : 256u;
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_ONE_LAUNCH) {
        if (value == 2) {  // test of the bounded wait: the next launch's barriers never complete
            c->fused_stall_test = true;
            return PBIG2_OK;
        }
        c->use_fused = value != 0;
        return PBIG2_OK;
    }
    if (option == PBIG2_OPT_HOST_SPLIT) {
        if (value >= c->sm_count) return fail(PBIG2_EINVAL, "host split of %lld SMs (the device has %d)",
                                              (long long)value, c->sm_count);
        c->host_split = value < 0 ? -1 : (int)value;
        return PBIG2_OK;
    }
    return fail(PBIG2_EINVAL, "unknown option %d", option);
}

PBIG2_API int pbig2_get_stats(pbig2_ctx* c, pbig2_stats* s) {
    if (!c || !s) return fail(PBIG2_EINVAL, "bad arguments");
    *s = c->stats;
    return PBIG2_OK;
}

}  // extern "C"
