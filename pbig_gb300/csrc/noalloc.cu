// Allocation-free self-intersection entry point (pbig2_self_intersect_noalloc).
//
// Some callers cannot allocate device memory while they run this query: a
// process whose device memory is owned entirely by another allocator (for
// example a caching allocator that has reserved the whole GPU), or a
// latency-critical loop that cannot afford cudaMalloc/cudaFree, which may
// synchronize the whole device. For them this entry point runs the same
// kernels as pbig2_self_intersect but keeps every intermediate buffer (cell
// counts, cell entries, work lists, tile tasks, scan state,
// counters) in one fixed scratch array that is part of the library image.
// The caller passes device-resident boxes and a device output buffer; the
// call allocates nothing.
//
// The scratch array is a file-scope __device__ array of kScratchBytes
// (16 MiB): every GPU that loads the library holds it until the process
// exits. Every call shares it and it keeps the last call's contents, so the
// call clears what must start at zero; calls that overlap on the GPU (two
// host threads, or two streams) race on it and must be serialized by the
// caller.
//
// The first call on a device does that device's set-up (the scratch
// address via cudaGetSymbolAddress and the kernels' shared-memory limits);
// make that first call before any stream capture.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "kernels.cuh"
#include "pbig2.h"

namespace pbig {

static constexpr size_t kScratchBytes = 16u << 20;

// limits of one allocation-free query (so that everything fits the scratch)
static constexpr uint64_t kNaMaxBoxes = 1u << 18;    // 262,144 boxes
static constexpr uint64_t kNaMaxCells = 1u << 20;    // grid cells
static constexpr uint64_t kNaMaxEntries = 1u << 19;  // box-in-cell entries
static constexpr uint64_t kNaMaxTasks = 1u << 16;    // tile tasks of cells above kBigMax

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

static constexpr int kMaxDevices = 64;
static void* g_scratch_ptr[kMaxDevices];
static bool g_scratch_ready[kMaxDevices];
static std::mutex g_setup_mutex;
static thread_local char g_na_error[256];

static int na_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess) snprintf(g_na_error, sizeof g_na_error, "%s: %s", msg, cudaGetErrorString(e));
    else snprintf(g_na_error, sizeof g_na_error, "%s", msg);
    return code;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace pbig

using namespace pbig;

extern "C" {

// Error text of the last failing pbig2_self_intersect_noalloc call on this thread.
PBIG2_API const char* pbig2_noalloc_last_error(void) { return g_na_error; }

PBIG2_API int pbig2_self_intersect_noalloc(const uint32_t* d_boxes, uint64_t n, uint32_t dims, uint32_t range,
                                           uint32_t cell_shift, uint32_t* d_pairs, uint64_t pair_cap,
                                           uint64_t* npairs, void* stream) {
    if (!npairs || (dims != 2 && dims != 3) || range == 0 || (n && !d_boxes) || (pair_cap && !d_pairs))
        return na_fail(PBIG2_EINVAL, "bad arguments");
    *npairs = 0;
    // the pair kernels store 8- and 16-byte units into the pair buffer
    if (((uintptr_t)d_pairs & 7u) != 0) return na_fail(PBIG2_EINVAL, "d_pairs must be 8-byte aligned");
    if (n > kNaMaxBoxes) return na_fail(PBIG2_ECAPACITY, "more than 262144 boxes: use pbig2_self_intersect");
    if (cell_shift != PBIG2_AUTO && cell_shift > 31) return na_fail(PBIG2_EINVAL, "cell_shift > 31");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_fail(PBIG2_ECUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return na_fail(PBIG2_EINVAL, "device index beyond 63");
    {
        std::lock_guard<std::mutex> lk(g_setup_mutex);
        if (!g_scratch_ready[dev]) {
            // the symbol's host-side name is not a device address: ask the runtime
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return na_fail(PBIG2_ECUDA, "cudaGetSymbolAddress", e);
            e = kernels_init();
            if (e != cudaSuccess) return na_fail(PBIG2_ECUDA, "kernel set-up", e);
            g_scratch_ptr[dev] = ptr;
            g_scratch_ready[dev] = true;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int W = 2 * (int)dims + 1;

    // cell size: caller's, or from the mean extent of up to 256 boxes copied
    // into a stack buffer, coarsened until the grid fits the scratch
    uint32_t shift = cell_shift;
    if (shift == PBIG2_AUTO) {
        uint32_t smp[256 * 7];
        const uint64_t m = n < 256 ? n : 256;
        double ext = 1.0;
        if (m) {
            const uint64_t stride = n / m;
            e = cudaMemcpy2DAsync(smp, W * 4, d_boxes, stride * W * 4, W * 4, m, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return na_fail(PBIG2_ECUDA, "sampling boxes", e);
            double s = 0;
            for (uint64_t i = 0; i < m; i++)
                for (int d = 0; d < (int)dims; d++) s += (double)smp[i * W + 2 * d + 1] - (double)smp[i * W + 2 * d] + 1.0;
            ext = s / (double)(m * dims);
        }
        shift = 0;
        while (shift < 31 && (double)(1u << (shift + 1)) <= ext) shift++;
    }
    // grid_cells saturates: a fine grid over a wide range (3-D, shift 0,
    // range 2^24: 2^72 cells) must not wrap to a small count
    while (shift < 31 && grid_cells(range, shift, (int)dims) > kNaMaxCells) shift++;
    const uint64_t ncells = grid_cells(range, shift, (int)dims);
    if (ncells > kNaMaxCells) return na_fail(PBIG2_ECAPACITY, "grid does not fit the scratch");
    // with at most 2^20 cells in the grid no box can cover the 2^26 cells at
    // which the count skips it, so unlike pbig2_self_intersect this entry
    // point never needs a coarser retry

    // carve the scratch
    unsigned char* base = (unsigned char*)g_scratch_ptr[dev];
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += align256(bytes);
        return p;
    };
    Params p{};
    Scene* scene = (Scene*)take(sizeof(Scene));
    uint32_t* scene_off = (uint32_t*)take(2 * sizeof(uint32_t));
    p.ctr = (Ctr*)take(sizeof(Ctr));
    p.counts = (uint32_t*)take(ncells * 4 + 16);
    const uint64_t tiles = scan_tiles(ncells);
    p.tile_state = (unsigned long long*)take(scan_state_bytes(ncells));
    p.entries = (uint32_t*)take(kNaMaxEntries * 4);
    p.entry_cap = kNaMaxEntries;
    const uint64_t lo[kNumLists] = {2, 5, 9, 17, 33, kMedMax + 1, kBigMax + 1};
    uint64_t loff = 0;
    for (int k = 0; k < kNumLists; k++) {
        p.list_off[k] = loff;
        p.list_cap[k] = kNaMaxEntries / lo[k] + 1;
        loff += p.list_cap[k];
    }
    p.lists = (uint2*)take(loff * 8);
    p.tasks = (uint4*)take(kNaMaxTasks * 16);
    p.task_cap = kNaMaxTasks;
    if (off > kScratchBytes) return na_fail(PBIG2_ECAPACITY, "scratch layout exceeds 16 MiB");

    Scene sc{};
    sc.box_off = 0;
    sc.n = (uint32_t)n;
    sc.shift = shift;
    sc.nrc = (uint32_t)(((uint64_t)range + (1ull << shift) - 1) >> shift);
    sc.cell_off = 0;
    sc.range = range;
    const uint32_t offs[2] = {0u, (uint32_t)n};
    p.boxes = d_boxes;
    p.nboxes = n;
    p.scenes = scene;
    p.scene_box_off = scene_off;
    p.nscenes = 1;
    p.split = kNoSplit;
    p.max_range = range;
    p.ncells = ncells;
    p.out = reinterpret_cast<uint2*>(d_pairs);
    p.out_cap = pair_cap;

    // the scratch keeps the previous call's contents: zero what must start at zero
    e = cudaMemcpyAsync(scene, &sc, sizeof(Scene), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(scene_off, offs, sizeof offs, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.ctr, 0, sizeof(Ctr), st);
    if (e == cudaSuccess) e = launch_count(p, (int)dims, st);
    if (e == cudaSuccess) e = launch_scan(p, st);
    if (e == cudaSuccess) e = launch_expand(p, st);
    if (e == cudaSuccess) e = launch_scatter(p, (int)dims, st);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = launch_pairs(p, (int)dims, sms, st);
    Ctr h{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, p.ctr, sizeof(Ctr), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(PBIG2_ECUDA, "pipeline", e);
    // an entry or task overflow leaves the pair count meaningless: *npairs stays 0
    if (h.err & (kErrEntryOvf | kErrTaskOvf)) return na_fail(PBIG2_ECAPACITY, "scene needs more cell entries than the scratch holds (limit 524288)");
    *npairs = h.pairs;
    if (h.err & kErrWait) return na_fail(PBIG2_ETIMEOUT, "a bounded device wait gave up (scan bulk copy)");
    if (h.err & kErrIndex) return na_fail(PBIG2_ECUDA, "inconsistent cell lists");
    if (h.pairs > pair_cap) return na_fail(PBIG2_ECAPACITY, "pair buffer too small; *npairs holds the pair count");
    if (h.bad) return na_fail(PBIG2_EINPUT, "some boxes violate the input contract and were skipped");
    return PBIG2_OK;
}

}  // extern "C"
