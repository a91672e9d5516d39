// Device-side data structures and kernel launchers of the pair-detection
// pipeline (count -> scan -> expand -> scatter -> pair test).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pbig {

// error bits accumulated in Ctr::err
enum : uint32_t {
    kErrRange = 1u,       // a coordinate >= range
    kErrInverted = 2u,    // min > max on some axis
    kErrRid = 4u,         // rid != index within the scene
    kErrEntryOvf = 8u,    // entry buffer too small (E > capacity)
    kErrOutOvf = 16u,     // pair buffer too small
    kErrWait = 32u,       // a bounded spin-wait gave up
    kErrTaskOvf = 64u,    // tile-task buffer too small
    kErrCellOvf = 128u,   // one box covers >= 2^31 cells
    kErrIndex = 256u,     // more than 2^29 boxes in one launch
    kErrRecCell = 512u    // record mode: a cell of 65536 boxes or more (the record format's limit)
};

constexpr uint32_t kNoSplit = 0xffffffffu;
constexpr int kIdBits = 29;
constexpr uint32_t kIdMask = (1u << kIdBits) - 1u;

// class lists built by the scan, one {start, n} record per cell: cells with
// 2..4, 5..8, 9..16, 17..32 boxes (several per warp), 33..kMedMax (one per
// warp, staged whole), kMedMax+1..kBigMax (one block, staged whole) and
// larger (32x32 tile tasks)
constexpr int kNumLists = 7;
constexpr int kListMed = 4, kListBig = 5, kListHuge = 6;
constexpr uint32_t kMedMax = 128;   // largest cell staged by one warp
constexpr uint32_t kBigMax = 512;   // largest cell staged by one block

// Which list a cell goes to is a class map: nibble L (L = ceil(log2 n), 1..15;
// 15 also for larger cells) holds the list of cells of n in (2^(L-1), 2^L].
// A list takes cells up to its capacity: 4, 8, 16, 32 boxes (lists 0..3, a
// lane group of that width per cell), kMedMax (4), kBigMax (5), any (6). The
// default sends each bucket to the smallest list that holds it.
constexpr unsigned long long kClassMapDefault = 0x6666665544321000ull;
constexpr unsigned long long kClassMapOneLaunch = 0x6666665544444000ull;  // 5..32 to the one-warp pass
__host__ __device__ inline uint32_t class_map_list(unsigned long long map, uint32_t L) {
    return (uint32_t)(map >> (4u * (L < 15u ? L : 15u))) & 15u;
}
// 0 when every bucket L = 1..15 names a list that holds it, else the first bad bucket
__host__ __device__ inline uint32_t class_map_check(unsigned long long map) {
    const uint64_t cap[kNumLists] = {4, 8, 16, 32, kMedMax, kBigMax, ~0ull};
    for (uint32_t L = 1; L <= 15; L++) {
        const uint32_t k = class_map_list(map, L);
        if (k >= (uint32_t)kNumLists || (L < 15 && (1ull << L) > cap[k]) || (L == 15 && k != (uint32_t)kListHuge))
            return L;
    }
    return 0;
}
// smallest cell a list can receive under the map (0: none), for list capacities
__host__ __device__ inline uint64_t class_map_min(unsigned long long map, int list) {
    for (uint32_t L = 1; L <= 15; L++)
        if (class_map_list(map, L) == (uint32_t)list) return L == 1 ? 2 : (1ull << (L - 1)) + 1;
    return 0;
}

// cells of a dims-D grid with ceil(range / 2^shift) cells per axis,
// saturating at UINT64_MAX (in 3-D a fine grid over a wide range has more
// than 2^64 cells: range 2^32 at shift 0 gives 2^96)
__host__ __device__ inline uint64_t grid_cells(uint32_t range, uint32_t shift, int dims) {
    const uint64_t nrc = shift >= 32 ? (range ? 1u : 0u) : (((uint64_t)range + (1ull << shift) - 1) >> shift);
    uint64_t c = nrc;
    for (int d = 1; d < dims; d++) {
        if (nrc && c > ~0ull / nrc) return ~0ull;
        c *= nrc;
    }
    return c;
}

// Cell-size cost model shared by the host tuner and the per-scene device
// tuner of batched queries: cost(s) = kCell*C + kEntry*E + kTest*T seconds
// (C cells, E box-in-cell entries, T pair tests), with kTest scaled by
// max(1, m / kOccTest) for the entry-weighted mean occupancy m = 2T/E + 1.
// The products are rounded one at a time (no fused multiply-add), so that
// host and device compute the same costs.
constexpr double kTuneCell = 2.4e-12, kTuneEntry = 80.0e-12, kTuneTest = 0.9e-12, kTuneOcc = 96.0;

__host__ __device__ inline double tune_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ inline double tune_add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ inline double tune_cost(double C, double E, double T) {
    const double occ = tune_add(tune_mul(2.0, T) / (E > 1.0 ? E : 1.0), 1.0);
    const double f = occ / kTuneOcc > 1.0 ? occ / kTuneOcc : 1.0;
    return tune_add(tune_add(tune_mul(kTuneCell, C), tune_mul(kTuneEntry, E)), tune_mul(tune_mul(kTuneTest, f), T));
}
// C = nrc^dims in double (rounded product; exact below 2^53)
__host__ __device__ inline double tune_cells(uint64_t nrc, int dims) {
    double c = (double)nrc;
    for (int d = 1; d < dims; d++) c = tune_mul(c, (double)nrc);
    return c;
}
// floor(log2(mean box extent)), at least 0, from the exact integer sum of
// the sampled extents (sum of (max - min + 1) over boxes and axes)
__host__ __device__ inline int tune_s0(uint64_t ext_sum, uint64_t nvals) {
    const double mean = (double)ext_sum / (double)(nvals ? nvals : 1);
    if (!(mean >= 2.0)) return 0;
    const uint64_t f = (uint64_t)mean;  // floor; log2 of a real >= 1 floors to that of its floor
    int k = 0;
    while ((f >> (k + 1)) != 0) k++;
    return k;
}

// result of the per-scene device tuner (batched queries)
struct SceneTune {
    uint32_t shift;
    uint32_t pad;
    double est_entries;
};

struct Scene {
    uint32_t box_off;   // first box of the scene (global index)
    uint32_t n;         // boxes in the scene
    uint32_t shift;     // log2(cell size)
    uint32_t nrc;       // cells per axis: ceil(range / 2^shift)
    uint64_t cell_off;  // first cell of the scene's grid (global cell id)
    uint32_t range;     // coordinate bound
    uint32_t pad;
};

// device-resident counters of one run (zeroed before the run)
struct Ctr {
    unsigned int err;
    unsigned int bad;
    unsigned int ticket;                // scan tile ticket
    unsigned int n_list[kNumLists];     // class list sizes
    unsigned int n_tasks;               // tile tasks written for huge cells
    unsigned int need_tasks;            // tile tasks needed
    unsigned int max_cell;              // largest cell (or merged block) of two or more boxes
    unsigned int med_next;              // next medium-cell item (items are taken one at a time)
    unsigned long long entries;         // E
    unsigned long long pairs;           // pairs found (may exceed capacity)
    unsigned long long tests;           // sum of n(n-1)/2 over cells
    unsigned long long comp_pairs;      // sum of n*n/2 over cells of n >= 2 (the reference's numCompPairs)
    unsigned long long jobs;            // sum of ceil(n/256) over cells of n >= 2 (its 256-row jobs)
    unsigned long long rec_pairs;       // record mode: pairs in the records (pairs counts 8-byte words)
    unsigned long long cells;           // one-launch queries: cells of the grid the kernel chose
    unsigned int shift;                 // one-launch queries: its cell shift
    unsigned int barriers;              // one-launch queries: grid barriers the launch passed
    unsigned long long t_start, t_end;  // one-launch queries: device time (ns) at the start and the end
};

// query sizes read from device memory (graph replays: one captured graph
// serves every batch up to the capacities it was captured with)
struct RunDims {
    unsigned long long nboxes;
    unsigned long long ncells;
    unsigned int nscenes;
    unsigned int pad;
};

struct Params {
    const uint32_t* boxes;        // RectInfo records, 2*D+1 words each
    uint64_t nboxes;              // boxes over all scenes
    const Scene* scenes;          // scene table (device)
    const uint32_t* scene_box_off;// nscenes+1 box offsets (device)
    uint32_t* scene_table;        // batched queries: scene of box 256*b, per b (built by launch_scene_table)
    uint32_t nscenes;
    uint32_t split;               // bipartite: global index of the first blue box
    uint32_t max_range;           // largest scene range (selects the pair-test arithmetic)
    uint32_t* counts;             // [ncells] per-cell counts; cell ends after the scan, starts after the scatter
    uint64_t ncells;
    uint32_t* entries;            // [entry_cap]: flags<<29 | global box index
    uint64_t entry_cap;
    uint2* lists;                 // kNumLists regions of {start, n}
    uint64_t list_off[kNumLists]; // region offsets into lists
    uint64_t list_cap[kNumLists];
    uint4* tasks;                 // huge-cell tile tasks {start, n, r, x0}
    uint64_t task_cap;
    unsigned long long* tile_state; // scan tile records (128 bytes per 4096 cells)
    uint2* out;                   // pairs
    uint64_t out_cap;
    Ctr* ctr;
    const RunDims* dyn;           // when set, overrides nboxes / ncells / nscenes
    const uint32_t* merged;       // merged mode (one scene): cell -> root of its merged block, or kUnmerged
    uint32_t records;             // record mode: work lists hold {cell id, n}; the pair kernels write the
                                  // reference's Rice record stream (8-byte words) instead of pairs
    unsigned long long class_map; // cell size -> work list (0: kClassMapDefault)
    // upload fused into the count: when box_copy is set, the count reads the
    // boxes from page-locked host memory (boxes [0, up_split) at up_red, the
    // rest at up_blue, device-mapped addresses) and writes them to box_copy,
    // the device copy (== boxes) that the later kernels read
    const uint32_t* up_red;
    const uint32_t* up_blue;
    uint64_t up_split;
    uint32_t* box_copy;
};

constexpr uint32_t kUnmerged = 0x0fffff11u;  // a cell outside every merged block

// launchers (all asynchronous on `st`); dims is 2 or 3
// grids: sized from p.nboxes / p.ncells (which must then be upper bounds
// of the device-side sizes when p.dyn is set)
cudaError_t launch_count(const Params& p, int dims, cudaStream_t st);
cudaError_t launch_scan(const Params& p, cudaStream_t st);
cudaError_t launch_expand(const Params& p, cudaStream_t st);
cudaError_t launch_scatter(const Params& p, int dims, cudaStream_t st);
// exclusive scan of nscenes+1 per-scene pair counts (one block)
// per-scene cell sizes of a batched query (one warp per scene, a strided
// sample of up to 64 boxes of each scene, T estimated as E^2 / 2C); offs:
// nscenes+1 box offsets in device memory
cudaError_t launch_tune_scenes(const uint32_t* boxes, const unsigned long long* offs, uint32_t nscenes, int dims,
                               uint32_t range, SceneTune* out, cudaStream_t st);
cudaError_t launch_scene_offsets(const Params& p, const unsigned long long* hist, unsigned long long* off,
                                 uint32_t nscenes_cap, cudaStream_t st);
// Pairs bound for page-locked host memory are limited by the host link, not
// by the kernels: with an overlap the small-cell and block kernels run on
// `side` over side_sms SMs while the medium-cell kernel runs on the others,
// so the link stays busy while the lighter kernels compute. `fork` and
// `join` are events owned by the caller.
struct PairOverlap {
    cudaStream_t side;
    cudaEvent_t fork, join;
    int side_sms;
};

// ev (optional, 2 events) is recorded after the small-cell and after the
// medium-cell kernel (with an overlap: after the small-cell kernel on the side
// stream and after the medium-cell kernel on st)
cudaError_t launch_pairs(const Params& p, int dims, int sm_count, cudaStream_t st, cudaEvent_t* ev = nullptr,
                         unsigned ev_flags = cudaEventRecordDefault, const PairOverlap* ov = nullptr);
cudaError_t launch_group_by_scene(const Params& p, const unsigned long long* scene_pair_off,
                                  unsigned long long* scene_cursor, uint2* dst, cudaStream_t st);
cudaError_t launch_scene_hist(const Params& p, unsigned long long* hist, cudaStream_t st);
// p.scene_table for p.nboxes boxes (scene_table_entries of them)
cudaError_t launch_scene_table(const Params& p, cudaStream_t st);
uint64_t scene_table_entries(uint64_t nboxes);
uint64_t scan_tiles(uint64_t ncells);
size_t scan_state_bytes(uint64_t ncells);  // scan tile records
size_t pair_smem_bytes();
cudaError_t kernels_init();

// ---- one-launch queries of small scenes -----------------------------------
// A self query of at most kFusedMaxBoxes boxes runs as one cooperative
// launch: the cell size (chosen on the device when `shift` is kFusedTune,
// grids of at most kFusedMaxCells cells), the count, the scan, the scatter
// and every pair pass, separated by grid barriers whose waits are bounded
// (kErrWait). p must carry the device boxes, counts (kFusedMaxCells or the
// given grid), entries, lists, tasks, out and ctr, whose counters must be
// zero at launch; the kernel zeroes ctr_next for the launch after it, writes
// the chosen grid (ctr->cells, ctr->shift) and the scene table for the host,
// leaves the counters of its grid zero, and its last block to finish copies
// the run counters to ctr_host with the number of barrier arrivals per block
// the launch made (ctr_host->barriers; unchanged when a wait gave up). Counters that may hold anything else (another pipeline
// used them, or they are new) are zeroed first when zero_cells says so.
constexpr uint64_t kFusedMaxBoxes = 1u << 18;
constexpr uint64_t kFusedMaxCells = 1u << 20;
constexpr uint32_t kFusedTune = 0xffffffffu;

struct FusedArgs {
    unsigned int* bar;        // arrival counter of the grid barriers (only ever increases)
    unsigned int bar_base;    // its value when the launch starts
    uint32_t* chunk_sum;      // entry totals of 512-cell chunks (kFusedMaxCells / 512 words)
    uint32_t* ends;           // cell ends of grids of at most 8192 cells (8192 words)
    Scene* scenes;            // the scene table for the host, written by the kernel
    Ctr* ctr_next;            // the run counters of the next launch (zeroed by this one)
    Ctr* ctr_host;            // page-locked host copy of the final counters, written by the last block
    uint64_t zero_cells;      // counters to zero before the count (0: they are zero)
    uint32_t shift;           // the cell shift, or kFusedTune
};
// blocks of a one-launch query (0: not available on this device)
int fused_blocks();
cudaError_t launch_fused(const Params& p, const FusedArgs& a, int dims, cudaStream_t st);

}  // namespace pbig
