// Kernels of the GB300 pairwise box-intersection pipeline.
//
//   k_count    boxes -> per-cell counts                (src/pbig/pbig.cu:174-221)
//   k_scan     counts -> cell starts + cell work lists (host thrust scan, pbig.cu:1497-1505,
//              and the job list of sched_phase, pbig.cu:1586-1688)
//   k_expand   tile tasks for cells too big for shared memory (sched_phase's 256-row jobs)
//   k_scatter  boxes -> cell entry lists               (d_mapping, pbig.cu:321-427)
//   k_pairs    per-cell all-pairs test with the reference-cell rule and compacted output
//              (d_matching + prefix_scan, pbig.cu:429-543, 562-603, 641-932)
//
// Box records are the reference's RectInfo (rect.h): 2*D+1 unsigned words.
// Cell ids follow the reference linearisation gid = (k*nrc + j)*nrc + i.
// An entry stores the box index and three "starts here" bits: bit d is set
// when the box's minimum along axis d lies in this cell. The reference-cell
// rule of calcRightToWrite (pbig.cu:579-603) -- a pair is reported in the
// cell holding the minimum corner of the two boxes' intersection -- is then
// exactly (flags_a | flags_b) == 7: along each axis max(min_a, min_b) falls
// in this cell iff one of the two minima does (both boxes cover the cell).
#include "kernels.cuh"

#include <cstdio>

namespace pbig {

#define FULL_MASK 0xffffffffu

__host__ __device__ __forceinline__ unsigned long long mn64(unsigned long long a, unsigned long long b) {
    return a < b ? a : b;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(FULL_MASK, v, o);
        if (lane_id() >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

// kernels take their sizes from device memory when p.dyn is set
__device__ __forceinline__ Params resolve(const Params& in) {
    Params p = in;
    if (p.dyn) {
        p.nboxes = p.dyn->nboxes;
        p.ncells = p.dyn->ncells;
        p.nscenes = p.dyn->nscenes;
    }
    return p;
}

// the last scene s in [lo, hi) with scene_box_off[s] <= gi
__device__ __forceinline__ uint32_t search_scene(const Params& p, uint64_t gi, uint32_t lo, uint32_t hi) {
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (p.scene_box_off[mid] <= gi) lo = mid;
        else hi = mid;
    }
    return lo;
}

// scene of global box gi: with the scene table (scene of every 256th box)
// the search covers only the scenes that start inside gi's 256-box block
constexpr uint32_t kSceneTableShift = 8;
__device__ __forceinline__ uint32_t find_scene(const Params& p, uint64_t gi) {
    if (p.nscenes <= 1) return 0;
    if (p.scene_table) {
        const uint64_t b = gi >> kSceneTableShift;
        const uint32_t s0 = p.scene_table[b];
        const uint32_t s1 = ((b + 1) << kSceneTableShift) < p.nboxes ? p.scene_table[b + 1] : p.nscenes - 1;
        return search_scene(p, gi, s0, s1 + 1);
    }
    return search_scene(p, gi, 0, p.nscenes);
}

__global__ void k_scene_table(Params pin) {
    const Params p = resolve(pin);
    const uint64_t n = (p.nboxes + (1u << kSceneTableShift) - 1) >> kSceneTableShift;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += (uint64_t)gridDim.x * blockDim.x)
        p.scene_table[b] = p.nscenes <= 1 ? 0u : search_scene(p, b << kSceneTableShift, 0, p.nscenes);
}

// ---------------------------------------------------------------------------
// per-scene cell sizes of a batched query: one warp per scene runs the host
// tuner's analytic model (tune_impl with T = E^2 / 2C) on the rows
// a + floor(k * n / m), k < m = min(n, 64), of the scene [a, a + n). Every
// sum is of integers (exact in any order), so the choice equals the host
// model's on the same rows.
// ---------------------------------------------------------------------------
constexpr uint32_t kTuneRows = 64;

__device__ __forceinline__ uint32_t nrc_dev(uint32_t range, int s) {
    return (uint32_t)(((uint64_t)range + (1ull << s) - 1) >> s);
}

// one warp: the cell shift of the scene of n boxes at row a (grids of at
// most max_cells cells)
__device__ __forceinline__ SceneTune tune_scene_warp(const uint32_t* boxes, uint64_t a, uint64_t n, int dims,
                                                     uint32_t range, double max_cells) {
    const uint32_t lane = lane_id();
    const uint32_t W = 2 * (uint32_t)dims + 1;
    {
        const uint64_t m = n < kTuneRows ? n : kTuneRows;
        uint32_t lo[2][3] = {{0, 0, 0}, {0, 0, 0}}, hi[2][3] = {{0, 0, 0}, {0, 0, 0}};
        bool ok[2] = {false, false};
        uint64_t ext = 0, good = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const uint64_t k = lane + 32u * j;
            if (k >= m) continue;
            const uint32_t* b = boxes + (a + k * n / m) * W;
            bool v = true;
            for (int d = 0; d < dims; d++) {
                lo[j][d] = b[2 * d];
                hi[j][d] = b[2 * d + 1];
                v = v && lo[j][d] <= hi[j][d] && hi[j][d] < range;
            }
            ok[j] = v;
            if (v) {
                for (int d = 0; d < dims; d++) ext += (uint64_t)(hi[j][d] - lo[j][d]) + 1;
                good++;
            }
        }
        ext = warp_sum_u64(ext);
        good = warp_sum_u64(good);
        SceneTune best{0u, 0u, 0.0};
        if (m == 0) {
            uint32_t s = 31;
            while (s > 0 && nrc_dev(range, (int)s - 1) <= 1) s--;
            best.shift = s;
        } else {
            const int s0 = tune_s0(ext, (good ? good : 1) * (uint64_t)dims);
            const double scale = (double)n / (double)m;
            const int s_win = s0 + 3 < 31 ? s0 + 3 : 31;
            double best_cost = 1e300;
            for (int s = s0 - 2 > 0 ? s0 - 2 : 0; s <= 31; s++) {
                if (s == s_win + 1 && best_cost < 1e300) break;
                const double C = tune_cells(nrc_dev(range, s), dims);
                if (C > max_cells) continue;
                if (s > s_win && C > fmax(4096.0, 64.0 * (double)n)) continue;
                double e = 0, cm = 0;
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    if (!ok[j]) continue;
                    double c = 1;
                    for (int d = 0; d < dims; d++) c = tune_mul(c, (double)((hi[j][d] >> s) - (lo[j][d] >> s) + 1));
                    e = tune_add(e, c);
                    cm = fmax(cm, c);
                }
#pragma unroll
                for (int o = 16; o; o >>= 1) {
                    e = tune_add(e, __shfl_xor_sync(FULL_MASK, e, o));
                    cm = fmax(cm, __shfl_xor_sync(FULL_MASK, cm, o));
                }
                if (e / (double)m > 64.0) continue;
                if (cm >= (double)(1u << 26)) continue;
                const double E = tune_mul(e, scale);
                const double T = tune_mul(E, E) / tune_mul(2.0, C);
                const double cost = tune_cost(C, E, T);
                if (cost < best_cost) {
                    best_cost = cost;
                    best.shift = (uint32_t)s;
                    best.est_entries = E;
                }
            }
            if (best_cost == 1e300) {  // the coarsest grid that is not a single cell
                uint32_t s = 31;
                while (s > 0 && nrc_dev(range, (int)s - 1) <= 1) s--;
                best.shift = s;
                best.est_entries = (double)n;
            }
        }
        return best;
    }
}

__global__ void k_tune_scenes(const uint32_t* boxes, const unsigned long long* offs, uint32_t nsc, int dims,
                              uint32_t range, SceneTune* out) {
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t sc = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; sc < nsc; sc += nw) {
        const uint64_t a = offs[sc];
        const SceneTune best = tune_scene_warp(boxes, a, offs[sc + 1] > a ? offs[sc + 1] - a : 0, dims, range, 4.0e9);
        if (lane_id() == 0) out[sc] = best;
    }
}

// ---------------------------------------------------------------------------
// count / scatter: one thread per box, boxes staged through shared memory with
// 16-byte vector loads; the cells of the 32 boxes of a warp are enumerated
// cooperatively (lane q handles cell q of the warp's concatenated cell list),
// so a box spanning many cells does not stall its warp.
// ---------------------------------------------------------------------------
constexpr int kBoxThreads = 256;

template <int D>
__device__ __forceinline__ void stage_boxes(const Params& p, uint64_t b0, uint32_t nb, uint32_t* sbox) {
    constexpr uint32_t W = 2 * D + 1;
    const uint32_t* src = p.boxes + b0 * W;
    const uint32_t nwords = nb * W;
    if (((reinterpret_cast<uintptr_t>(src) & 15u) == 0) && (nwords & 3u) == 0) {
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(sbox);
        for (uint32_t k = threadIdx.x; k < nwords / 4; k += blockDim.x) d4[k] = __ldg(s4 + k);
    } else {
        for (uint32_t k = threadIdx.x; k < nwords; k += blockDim.x) sbox[k] = __ldg(src + k);
    }
}

__device__ __forceinline__ void copy_words(const uint32_t* src, uint32_t* dst, uint32_t nwords) {
    if ((((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) && (nwords & 3u) == 0) {
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (uint32_t k = threadIdx.x; k < nwords / 4; k += blockDim.x) d4[k] = __ldg(s4 + k);
    } else {
        for (uint32_t k = threadIdx.x; k < nwords; k += blockDim.x) dst[k] = __ldg(src + k);
    }
}

// the count's upload: a tile of boxes from page-locked host memory into
// shared memory (the host link is the bound, so the count's own work hides
// under it), then on to the device copy
template <int D>
__device__ __forceinline__ void stage_upload(const Params& p, uint64_t b0, uint32_t nb, uint32_t* sbox) {
    constexpr uint32_t W = 2 * D + 1;
    const uint64_t split = p.up_split;
    if (b0 + nb <= split || b0 >= split) {
        copy_words(b0 < split ? p.up_red + b0 * W : p.up_blue + (b0 - split) * W, sbox, nb * W);
    } else {  // the tile straddles red and blue
        const uint64_t sw = split * W;
        for (uint32_t k = threadIdx.x; k < nb * W; k += blockDim.x) {
            const uint64_t gw = b0 * W + k;
            sbox[k] = gw < sw ? __ldg(p.up_red + gw) : __ldg(p.up_blue + (gw - sw));
        }
    }
    __syncthreads();
    uint32_t* dst = p.box_copy + b0 * W;
    if (((reinterpret_cast<uintptr_t>(dst) & 15u) == 0) && ((nb * W) & 3u) == 0) {
        const uint4* s4 = reinterpret_cast<const uint4*>(sbox);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (uint32_t k = threadIdx.x; k < nb * W / 4; k += blockDim.x) d4[k] = s4[k];
    } else {
        for (uint32_t k = threadIdx.x; k < nb * W; k += blockDim.x) dst[k] = sbox[k];
    }
}

// n / d (d >= 1) by a multiply-high with the divisor's multiplier m =
// magic_of(d) = ceil(2^32 / d) (0 for d = 1): for n < 2^31 the estimate is
// exact or one too large, which one compare fixes
__device__ __forceinline__ uint32_t magic_of(uint32_t d) { return d > 1u ? 0xffffffffu / d + 1u : 0u; }
__device__ __forceinline__ uint32_t div_magic(uint32_t n, uint32_t d, uint32_t m) {
    if (m == 0u) return n;
    const uint32_t q = __umulhi(n, m);
    return q * d > n ? q - 1u : q;
}

template <int D, bool SCATTER, bool MERGED>
__device__ __forceinline__ void enumerate_cells(const Params& p, const uint32_t* sbox, uint64_t b0,
                                                uint32_t nb) {
    constexpr uint32_t W = 2 * D + 1;
    const uint32_t t = threadIdx.x, lane = t & 31u;
    const uint64_t gi = b0 + t;
    uint32_t cnt = 0, sx = 1, sy = 1, nrc = 0;
    uint64_t base = 0;
    if (t < nb) {
        const uint32_t* b = sbox + t * W;
        const Scene sc = p.scenes[find_scene(p, gi)];
        uint32_t err = 0;
#pragma unroll
        for (int d = 0; d < D; d++) {
            if (b[2 * d] >= sc.range || b[2 * d + 1] >= sc.range) err |= kErrRange;
            if (b[2 * d] > b[2 * d + 1]) err |= kErrInverted;
        }
        if (b[2 * D] != (uint32_t)(gi - sc.box_off)) err |= kErrRid;
        if (gi > kIdMask) err |= kErrIndex;
        if (!err) {
            const uint32_t sh = sc.shift;
            const uint32_t lo0 = b[0] >> sh, lo1 = b[2] >> sh, lo2 = D == 3 ? (b[4] >> sh) : 0u;
            sx = (b[1] >> sh) - lo0 + 1;
            sy = (b[3] >> sh) - lo1 + 1;
            const uint32_t sz = D == 3 ? (b[5] >> sh) - lo2 + 1 : 1u;
            const uint64_t c64 = (uint64_t)sx * sy * sz;
            if (c64 >= (1ull << 26)) {
                err |= kErrCellOvf;
            } else {
                cnt = (uint32_t)c64;
                nrc = sc.nrc;
                base = sc.cell_off + ((uint64_t)lo2 * nrc + lo1) * nrc + lo0;
            }
        }
        if (err && !SCATTER) {
            atomicOr(&p.ctr->err, err);
            atomicAdd(&p.ctr->bad, 1u);
        }
    }
    const uint32_t incl = warp_incl_scan(cnt);
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    const uint32_t excl = incl - cnt;
    const uint64_t wbox0 = b0 + (t & ~31u);
    const uint32_t mx = magic_of(sx), my = magic_of(sy);  // one division per box, none per cell
    for (uint32_t q0 = 0; q0 < total; q0 += 32) {
        const uint32_t q = q0 + lane;
        uint32_t o = 0;  // owner lane: number of lanes whose inclusive count <= q
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1) {
            const uint32_t v = __shfl_sync(FULL_MASK, incl, o + step - 1);
            if (v <= q) o += step;
        }
        const uint32_t o_excl = __shfl_sync(FULL_MASK, excl, o);
        const uint32_t o_sx = __shfl_sync(FULL_MASK, sx, o);
        const uint32_t o_sy = __shfl_sync(FULL_MASK, sy, o);
        const uint32_t o_nrc = __shfl_sync(FULL_MASK, nrc, o);
        const uint64_t o_base = __shfl_sync(FULL_MASK, base, o);
        const uint32_t o_mx = __shfl_sync(FULL_MASK, mx, o);
        const uint32_t o_my = __shfl_sync(FULL_MASK, my, o);
        if (q < total) {
            const uint32_t lq = q - o_excl;  // < 2^26
            const uint32_t rr = div_magic(lq, o_sx, o_mx), i = lq - rr * o_sx;
            const uint32_t k = div_magic(rr, o_sy, o_my), j = rr - k * o_sy;
            uint64_t gid = o_base + ((uint64_t)k * o_nrc + j) * o_nrc + i;
            uint32_t f = (i == 0 ? 1u : 0u) | (j == 0 ? 2u : 0u) | ((D == 2 || k == 0) ? 4u : 0u);
            bool take = true;
            if (MERGED) {
                // merged mode: a cell of a merged block stands for the block's
                // root, and a box enters the block once, at the minimum corner of
                // (box range x block) -- the first-visit rule of d_postcounting,
                // pbig.cu:223-318; "starts here" is then per axis "the box's
                // first cell is inside the block"
                const uint32_t m = p.merged[gid];
                if (m != kUnmerged) {
                    const uint64_t nr = o_nrc;
                    const uint32_t ci = (uint32_t)(gid % nr), cj = (uint32_t)((gid / nr) % nr);
                    const uint32_t ck = D == 3 ? (uint32_t)(gid / (nr * nr)) : 0u;
                    const uint32_t lx = ci - i, ly = cj - j, lz = ck - k;
                    const uint32_t rx = (uint32_t)(m % nr), ry = (uint32_t)((m / nr) % nr);
                    const uint32_t rz = D == 3 ? (uint32_t)(m / (nr * nr)) : 0u;
                    take = ci == max(lx, rx) && cj == max(ly, ry) && ck == max(lz, rz);
                    gid = m;
                    f = (lx >= rx ? 1u : 0u) | (ly >= ry ? 2u : 0u) | ((D == 2 || lz >= rz) ? 4u : 0u);
                }
            }
            if (!take) {
            } else if (SCATTER) {
                // after the scan a cell's counter holds its end: counting it
                // down hands out the cell's slots (and leaves its start)
                const uint64_t pos = (uint64_t)(atomicSub(&p.counts[gid], 1u) - 1u);
                if (pos < p.entry_cap) p.entries[pos] = (f << kIdBits) | (uint32_t)(wbox0 + o);
                else atomicOr(&p.ctr->err, kErrEntryOvf);
            } else {
                atomicAdd(&p.counts[gid], 1u);
            }
        }
    }
}

// counts = 0 before a pass (the scatter leaves every cell's start there)
__global__ void k_zero_counts(Params pin) {
    const Params p = resolve(pin);
    const uint64_t n4 = p.ncells / 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint4* c4 = reinterpret_cast<uint4*>(p.counts);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) c4[i] = make_uint4(0, 0, 0, 0);
    for (uint64_t i = 4 * n4 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.ncells; i += stride) p.counts[i] = 0;
}

// tiles of TILE boxes: blk, blk + nblk, ... (blockDim.x == TILE)
template <int D, bool SCATTER, bool MERGED, uint32_t TILE = kBoxThreads>
__device__ __forceinline__ void box_pass(const Params& p, uint32_t* sbox, uint64_t blk, uint64_t nblk) {
    for (uint64_t b0 = blk * TILE; b0 < p.nboxes; b0 += nblk * TILE) {
        const uint32_t nb = (uint32_t)mn64(TILE, p.nboxes - b0);
        if (!SCATTER && p.box_copy) stage_upload<D>(p, b0, nb, sbox);
        else stage_boxes<D>(p, b0, nb, sbox);
        __syncthreads();
        enumerate_cells<D, SCATTER, MERGED>(p, sbox, b0, nb);
        __syncthreads();
    }
}

template <int D, bool MERGED>
__global__ void __launch_bounds__(kBoxThreads) k_count(Params pin) {
    __shared__ __align__(16) uint32_t sbox[kBoxThreads * (2 * D + 1)];
    box_pass<D, false, MERGED>(resolve(pin), sbox, blockIdx.x, gridDim.x);
}

template <int D, bool MERGED>
__global__ void __launch_bounds__(kBoxThreads) k_scatter(Params pin) {
    __shared__ __align__(16) uint32_t sbox[kBoxThreads * (2 * D + 1)];
    box_pass<D, true, MERGED>(resolve(pin), sbox, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// scan: counts -> cell starts and the work lists of the pair kernels, in
// two launches without inter-block waits.
//
// A tile is 4096 cells, a chunk 512 of them; every warp works on whole
// chunks with no block barrier, so the loads of all resident warps are in
// flight together. Tile records (64 bytes, zeroed before the scan) collect
// per-chunk entry sums and per-tile totals.
//
//   k_scan_reduce  chunk entry total (stored per chunk, added to the tile);
//                  two chunks per warp iteration, so eight 16-byte loads
//                  per lane are in flight together. The last block to
//                  finish turns the tile entry totals into exclusive
//                  prefixes; the entry total goes to the counters.
//   k_scan_cells   the same chunks again: starts from the tile prefix, the
//                  tile's earlier chunks and a warp scan; every cell of two
//                  or more boxes goes to its work list, a chunk reserving
//                  its places with one atomic per list (list order is free);
//                  each warp sums the work statistics of its cells (pair
//                  tests, numCompPairs, 256-row jobs, largest cell) and adds
//                  them to the counters once.
//
// Lane l of a warp owns the 4 cells at 4l of each of the chunk's 4 rows of
// 128 cells, so each 16-byte load or store of a warp covers 512 contiguous
// bytes. The work list of a cell of n >= 2 boxes is 2..4, 5..8, 9..16,
// 17..32, 33..128, 129..512 or more boxes; per-lane list counts travel
// packed in 10-bit fields (a chunk has at most 512 cells per list).
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 16;
constexpr int kScanChunk = 32 * kScanPerThread;              // cells per warp item
constexpr int kScanChunks = 8;                               // chunks per tile
constexpr int kScanTile = kScanChunk * kScanChunks;

struct TileRec {                         // 64 bytes per tile
    unsigned long long sum;              // entries; exclusive prefix after k_scan_reduce
    uint32_t chunk[kScanChunks];         // entries per chunk
    uint32_t pad[6];
};
static_assert(sizeof(TileRec) == 64, "tile record layout");

static_assert(kMedMax == 128 && kBigMax == 512, "list bounds are powers of two (the class map's buckets)");
// the work list of a cell of n >= 2 boxes under the class map
__device__ __forceinline__ uint32_t class_of(uint32_t n, unsigned long long map) {
    const uint32_t lg = 32u - __clz(n - 1u);  // ceil(log2 n) for n >= 2
    return (uint32_t)(map >> (4u * min(lg, 15u))) & 15u;
}

__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long v) {
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(FULL_MASK, v, o);
        if (lane_id() >= o) v += t;
    }
    return v;
}

// cell r*128 + 4*lane of chunk `chunk`, chunks of Q rows of 128 cells
template <int Q = 4>
__device__ __forceinline__ uint64_t chunk_cell(uint64_t chunk, int r) {
    return chunk * (128u * Q) + (uint64_t)r * 128 + lane_id() * 4;
}

// the 4*Q counts of this lane's cells of the chunk (zeros past the end);
// PAST_L1: counts written by other blocks of the same launch
template <int Q = 4, bool PAST_L1 = false>
__device__ __forceinline__ void scan_load(const Params& p, uint64_t chunk, uint32_t (&v)[4 * Q]) {
    const bool full = chunk * (128u * Q) + 128u * Q <= p.ncells;
#pragma unroll
    for (int r = 0; r < Q; r++) {
        const uint64_t c = chunk_cell<Q>(chunk, r);
        if (full) {
            const uint4* a = reinterpret_cast<const uint4*>(p.counts + c);
            const uint4 q = PAST_L1 ? __ldcg(a) : *a;
            v[4 * r] = q.x; v[4 * r + 1] = q.y; v[4 * r + 2] = q.z; v[4 * r + 3] = q.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                v[4 * r + k] = c + k < p.ncells ? (PAST_L1 ? __ldcg(p.counts + c + k) : p.counts[c + k]) : 0u;
        }
    }
}

__device__ __forceinline__ void reduce_chunk(TileRec* rec, uint64_t ch, const uint32_t v[kScanPerThread]) {
    const uint32_t lane = lane_id();
    uint32_t lsum = 0;  // < 2^32 while the entry total is
#pragma unroll
    for (int k = 0; k < kScanPerThread; k++) lsum += v[k];
    lsum = __reduce_add_sync(FULL_MASK, lsum);
    TileRec& r = rec[ch / kScanChunks];
    if (lane == 0) {
        r.chunk[ch % kScanChunks] = lsum;
        if (lsum) atomicAdd(&r.sum, (unsigned long long)lsum);
    }
}

// tile entry totals -> exclusive prefixes; the entry total goes to the
// counters. Run by one block of kReduceThreads threads, kPrefixPer tiles per
// thread per round (4096 tiles in two rounds).
constexpr int kReduceThreads = kScanThreads;
constexpr int kPrefixPer = 8;
__device__ __forceinline__ void scan_prefix_block(const Params& p) {
    __shared__ unsigned long long s_part[kReduceThreads / 32];
    __shared__ unsigned long long s_carry;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint64_t tiles = (p.ncells + kScanTile - 1) / kScanTile;
    TileRec* rec = reinterpret_cast<TileRec*>(p.tile_state);
    if (t == 0) s_carry = 0;
    // rounds of kPrefixPer tiles per thread: all loads of a round in flight
    // together; the records were written through L2 by other blocks (read
    // past L1)
    for (uint64_t r0 = 0; r0 < tiles; r0 += kPrefixPer * kReduceThreads) {
        unsigned long long x[kPrefixPer], sx = 0;
#pragma unroll
        for (int k = 0; k < kPrefixPer; k++) {
            const uint64_t i = r0 + kPrefixPer * (uint64_t)t + k;
            x[k] = i < tiles ? __ldcg(&rec[i].sum) : 0ull;
            sx += x[k];
        }
        const unsigned long long ix = warp_incl_scan64(sx);
        if (lane == 31) s_part[warp] = ix;
        __syncthreads();
        unsigned long long wo = s_carry, tot = 0;
        for (int w = 0; w < kReduceThreads / 32; w++) {
            const unsigned long long a = s_part[w];
            if (w < (int)warp) wo += a;
            tot += a;
        }
        unsigned long long run = wo + (ix - sx);
#pragma unroll
        for (int k = 0; k < kPrefixPer; k++) {
            const uint64_t i = r0 + kPrefixPer * (uint64_t)t + k;
            if (i < tiles) rec[i].sum = run;
            run += x[k];
        }
        __syncthreads();
        if (t == 0) s_carry += tot;
        __syncthreads();
    }
    if (t == 0) {
        p.ctr->entries = s_carry;
        if (s_carry >= (1ull << 32)) atomicOr(&p.ctr->err, kErrEntryOvf);
    }
}

// the last block to finish (a ticket taken after a fence, no waiting) runs
// the tile prefix, so no separate launch is needed for it
__global__ void __launch_bounds__(kReduceThreads, 4) k_scan_reduce(Params pin) {
    __shared__ uint32_t s_last;
    const Params p = resolve(pin);
    const uint32_t warp = threadIdx.x >> 5;
    const uint64_t chunks = (p.ncells + kScanChunk - 1) / kScanChunk;
    TileRec* rec = reinterpret_cast<TileRec*>(p.tile_state);
    const uint64_t nw = (uint64_t)gridDim.x * (kReduceThreads / 32);
    for (uint64_t ch = 2 * ((uint64_t)blockIdx.x * (kReduceThreads / 32) + warp); ch < chunks; ch += 2 * nw) {
        uint32_t v[kScanPerThread], w[kScanPerThread];
        scan_load(p, ch, v);
        const bool two = ch + 1 < chunks;
        if (two) scan_load(p, ch + 1, w);
        reduce_chunk(rec, ch, v);
        if (two) reduce_chunk(rec, ch + 1, w);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&p.ctr->ticket, 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (s_last == 0u) return;
    __threadfence();
    scan_prefix_block(p);
    if (threadIdx.x == 0) p.ctr->ticket = 0;  // the next scan needs no reset
}

// ---- bulk asynchronous copies (global -> shared) completing on an mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// arm the barrier for `bytes` and copy them (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase of parity `parity`; false when it gave up
constexpr uint32_t kBulkWaitLimit = 1u << 20;
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    for (uint32_t i = 0; i < kBulkWaitLimit; i++)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// the cells of chunk ch (counts v; `base` entries before the chunk): each
// non-empty cell's end (start + count) into its counter (an empty cell's is
// never read: the scatter and the work lists touch cells with entries only,
// and skipping those stores, most of a fine grid, saves the scatter the
// write-backs of their lines), each cell of two or more boxes into its work
// list (one atomic per list and chunk), and the work statistics into ws
struct ScanStats {
    unsigned long long tests = 0;
    uint32_t half = 0, jobs = 0, max = 0;
};

// (pl: the kernel's own parameters, for the list tables: indexing a local
// copy of Params with a run-time list number would move it to local memory)
template <int Q = 4>
__device__ __forceinline__ void scan_chunk(const Params& p, const Params& pl, uint64_t ch, bool full,
                                           const uint32_t (&v)[4 * Q], unsigned long long base, ScanStats& ws) {
    constexpr int kPer = 4 * Q;
    const uint32_t lane = lane_id();
    const unsigned long long cmap = p.class_map ? p.class_map : kClassMapDefault;
    uint32_t big = 0;
#pragma unroll
    for (int k = 0; k < kPer; k++) big |= v[k] >> 1;
    // row scans: the cells of row q before this lane's, and rows < q whole
    uint32_t st[kPer];
    unsigned long long wtot = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const uint32_t rs = v[4 * q] + v[4 * q + 1] + v[4 * q + 2] + v[4 * q + 3];
        const uint32_t inc = warp_incl_scan(rs);  // < 2^32 while the entry total is
        unsigned long long run = base + wtot + (inc - rs);
        wtot += __shfl_sync(FULL_MASK, inc, 31);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            st[4 * q + k] = (uint32_t)run;
            run += v[4 * q + k];
        }
        // a non-empty cell's counter becomes its end (start + count), in place
        const uint64_t c = chunk_cell<Q>(ch, q);
        if (full) {
            if (rs != 0u)
                *reinterpret_cast<uint4*>(p.counts + c) = make_uint4(
                    st[4 * q] + v[4 * q], st[4 * q + 1] + v[4 * q + 1], st[4 * q + 2] + v[4 * q + 2], st[4 * q + 3] + v[4 * q + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (c + k < p.ncells && v[4 * q + k] != 0u) p.counts[c + k] = st[4 * q + k] + v[4 * q + k];
        }
    }
    if (__any_sync(FULL_MASK, big != 0)) {
        // per-lane list counts: lists 0..5 in 10-bit fields of pk, list 6 in pk6
        unsigned long long pk = 0;
        uint32_t pk6 = 0;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            if (v[k] >= 2u) {
                const uint32_t c = class_of(v[k], cmap);
                if (c < 6u) pk += 1ull << (10u * c);
                else pk6 += 1u;
            }
        }
        const unsigned long long pinc = warp_incl_scan64(pk);
        const uint32_t p6inc = warp_incl_scan(pk6);
        unsigned long long pk_excl = pinc - pk;
        uint32_t pk6_excl = p6inc - pk6;
        // lane c < 7: this chunk's first place in list c
        const unsigned long long ptot = __shfl_sync(FULL_MASK, pinc, 31);
        const uint32_t p6tot = __shfl_sync(FULL_MASK, p6inc, 31);
        uint32_t lbase = 0;
        if (lane < kNumLists) {
            const uint32_t x = lane < 6u ? (uint32_t)(ptot >> (10u * lane)) & 1023u : p6tot;
            if (x) lbase = atomicAdd(&p.ctr->n_list[lane], x);
        }
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const uint32_t c = v[k] >= 2u ? class_of(v[k], cmap) : 0u;
            const uint32_t b = __shfl_sync(FULL_MASK, lbase, c);
            if (v[k] >= 2u) {
                uint32_t rk;
                if (c < 6u) {
                    rk = (uint32_t)(pk_excl >> (10u * c)) & 1023u;
                    pk_excl += 1ull << (10u * c);
                } else {
                    rk = pk6_excl++;
                }
                const uint64_t idx = (uint64_t)b + rk;
                const uint32_t key = p.records ? (uint32_t)(chunk_cell<Q>(ch, k >> 2) + (k & 3)) : st[k];
                if (idx < pl.list_cap[c]) p.lists[pl.list_off[c] + idx] = make_uint2(key, v[k]);
                ws.tests += (unsigned long long)v[k] * (v[k] - 1u) / 2u;
                ws.half += v[k] >> 1;  // n*n/2 = n(n-1)/2 + n/2, rounded down
                ws.jobs += (v[k] + 255u) >> 8;
                ws.max = max(ws.max, v[k]);
            }
        }
    }
}

// the work statistics of a warp's cells (pair tests, and the reference's
// numCompPairs, 256-row jobs and largest cell) into the counters
__device__ __forceinline__ void scan_stats_flush(const Params& p, const ScanStats& st) {
    const unsigned long long tests = warp_sum_u64(st.tests);
    const unsigned long long half = warp_sum_u64(st.half), jobs = warp_sum_u64(st.jobs);
    const uint32_t mx = __reduce_max_sync(FULL_MASK, st.max);
    if (lane_id() == 0 && mx) {
        atomicAdd(&p.ctr->tests, tests);
        atomicAdd(&p.ctr->comp_pairs, tests + half);
        atomicAdd(&p.ctr->jobs, jobs);
        atomicMax(&p.ctr->max_cell, mx);
    }
}

// k_scan_cells: each warp keeps its next chunk's counts in flight as a bulk
// copy into one of two shared-memory buffers while it works on the current
// one. A partial chunk (only the grid's last) is read with plain loads.
__global__ void __launch_bounds__(kScanThreads, 4) k_scan_cells(Params pin) {
    __shared__ __align__(128) uint32_t s_buf[kScanThreads / 32][2][kScanChunk];
    __shared__ __align__(8) unsigned long long s_bar[kScanThreads / 32][2];
    const Params p = resolve(pin);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint64_t chunks = (p.ncells + kScanChunk - 1) / kScanChunk;
    const uint64_t full_chunks = p.ncells / kScanChunk;
    const TileRec* rec = reinterpret_cast<const TileRec*>(p.tile_state);
    const uint64_t nw = (uint64_t)gridDim.x * (kScanThreads / 32);
    const uint64_t first = (uint64_t)blockIdx.x * (kScanThreads / 32) + warp;
    if (lane == 0) {
        mbar_init(&s_bar[warp][0], 1);
        mbar_init(&s_bar[warp][1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    auto issue = [&](uint64_t i) {  // chunk i of this warp into buffer i & 1
        const uint64_t ch = first + i * nw;
        if (lane == 0 && ch < full_chunks)
            bulk_load(s_buf[warp][i & 1], p.counts + ch * kScanChunk, kScanChunk * 4, &s_bar[warp][i & 1]);
    };
    issue(0);
    issue(1);
    ScanStats stats;
    for (uint64_t i = 0;; i++) {
        const uint64_t ch = first + i * nw;
        if (ch >= chunks) break;
        uint32_t v[kScanPerThread];
        if (ch < full_chunks) {
            if (!mbar_wait(&s_bar[warp][i & 1], (uint32_t)(i >> 1) & 1u)) {
                // give up: report, wait (bounded) for the copy still in flight, stop
                if (lane == 0) atomicOr(&p.ctr->err, kErrWait);
                mbar_wait(&s_bar[warp][i & 1], (uint32_t)(i >> 1) & 1u);
                if (first + (i + 1) * nw < full_chunks)
                    mbar_wait(&s_bar[warp][(i + 1) & 1], (uint32_t)((i + 1) >> 1) & 1u);
                return;
            }
            const uint32_t* b = s_buf[warp][i & 1];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint4 x = *reinterpret_cast<const uint4*>(b + q * 128 + lane * 4);
                v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
            }
            __syncwarp();
            // the buffer's reads are done: it can take the chunk after next
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(i + 2);
        } else {
            scan_load(p, ch, v);
        }
        const TileRec& r = rec[ch / kScanChunks];
        const uint32_t ci = (uint32_t)(ch % kScanChunks);
        // entries before this chunk: tile prefix + the tile's earlier chunks
        unsigned long long base = lane == 0 ? r.sum : 0ull;
        if (lane > 0 && lane <= ci) base = r.chunk[lane - 1];
        base = warp_sum_u64(base);
        scan_chunk(p, pin, ch, ch < full_chunks, v, base, stats);
    }
    scan_stats_flush(p, stats);
}

// ---------------------------------------------------------------------------
// expand: cells larger than kBigMax get tile tasks {cell, row tile r, column
// tiles [x0,x1)} with 32-box tiles, x >= r, at most 8 column tiles a task.
// ---------------------------------------------------------------------------
constexpr uint32_t kTaskCols = 8;

// a run counter that a pass reads: FRESH (one-launch queries, where phases
// of the same kernel change the counters) reads it past L1; the separate
// kernels of the regular pipeline read it plainly (a load past L1 there
// measured 20 % slower medium-cell and twice slower block passes)
template <bool FRESH>
__device__ __forceinline__ uint32_t ctr_read(const unsigned int* a) { return FRESH ? __ldcg(a) : *a; }

// huge cells i0, i0 + stride, ...
template <bool FRESH = false>
__device__ __forceinline__ void expand_cells(const Params& p, uint32_t i0, uint32_t stride) {
    const uint32_t nh = mn64(ctr_read<FRESH>(&p.ctr->n_list[kListHuge]), p.list_cap[kListHuge]);
    for (uint32_t i = i0; i < nh; i += stride) {
        const uint2 sn = p.lists[p.list_off[kListHuge] + i];
        const uint32_t n = sn.y;
        const uint32_t R = (n + 31) >> 5;
        uint32_t cnt = 0;
        for (uint32_t r = 0; r < R; r++) cnt += (R - r + kTaskCols - 1) / kTaskCols;
        const uint32_t b = atomicAdd(&p.ctr->need_tasks, cnt);
        uint32_t k = 0;
        for (uint32_t r = 0; r < R; r++)
            for (uint32_t x0 = r; x0 < R; x0 += kTaskCols, k++)
                if ((uint64_t)b + k < p.task_cap) p.tasks[b + k] = make_uint4(sn.x, n, r, x0);
        if ((uint64_t)b + cnt > p.task_cap) atomicOr(&p.ctr->err, kErrTaskOvf);
    }
}

__global__ void k_expand(Params p) { expand_cells(p, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x); }

// ---------------------------------------------------------------------------
// pair test
//
// Three kernels share the per-pair test and the sweeps:
//   k_pairs_small  cells of 2..32 boxes, 32/WG cells per warp item
//   k_pairs_med    cells of 33..kMedMax boxes, one cell per warp item,
//                  staged whole in the warp's shared memory
//   k_pairs_block  cells of kMedMax+1..kBigMax boxes staged whole by a
//                  block, and 32x32 tile tasks of larger cells
// The warp items of the small- and medium-cell kernels run independently (no
// block barriers); each warp compacts its pairs into its own shared-memory
// buffer and flushes it to the pair array with one global reservation per
// flush (the block kernel does the same per block).
//
// The test of one (row box, column box) pair is branch free: with every
// coordinate < 2^29 the six differences max-min are non-negative exactly
// when the closed intervals overlap, and a negative difference sets bits
// 29..31; the reference-cell rule adds the "does not start here" bits of
// both boxes in bits 29..31, so the pair is reported iff the OR of all of
// them is < 2^29. Wider coordinates use plain comparisons.
// ---------------------------------------------------------------------------
constexpr int kPairThreads = 256;
constexpr int kPairWarps = kPairThreads / 32;
constexpr uint32_t kMissShift = 29;
constexpr uint32_t kWarpOut = 256;          // per-warp output buffer (pairs), small cells
constexpr uint32_t kMedOut = 512;           // per-warp output buffer (pairs), medium cells: above the
                                            // typical output of one emission step, so it rarely spills
constexpr uint32_t kSmallSlots = 64;        // per-warp staging, small cells (each cell twice in a row)
constexpr uint32_t kMedSlots = kMedMax;     // per-warp staging, medium cells
constexpr uint32_t kBlockSlots = kBigMax;   // per-block staging, big cells
constexpr uint32_t kBlockOut = 2048;        // per-block output buffer (pairs)
// big cells per block task: two, so the few hundred big cells of a large
// scene spread over the blocks (eight per task kept 60 of 304 blocks busy on
// the clustered 4M-box scene: 0.060 ms; one per task 0.028, two 0.024 ms)
constexpr uint32_t kBigCellsPerTask = 2;

struct Box {
    uint32_t x0, x1, y0, y1, z0, z1, f, id;  // f: axes where the box does not start in this cell, << 29
};

// staging arrays in shared memory: slot i = (a[i], b[i])
struct Slots {
    uint4* a;  // x0 x1 y0 y1
    uint4* b;  // z0 z1 f id
};

__device__ __forceinline__ void slot_put(const Slots& s, uint32_t i, const Box& x) {
    s.a[i] = make_uint4(x.x0, x.x1, x.y0, x.y1);
    s.b[i] = make_uint4(x.z0, x.z1, x.f, x.id);
}
__device__ __forceinline__ Box slot_get(const Slots& s, uint32_t i) {
    const uint4 a = s.a[i], b = s.b[i];
    Box x;
    x.x0 = a.x; x.x1 = a.y; x.y0 = a.z; x.y1 = a.w;
    x.z0 = b.x; x.z1 = b.y; x.f = b.z; x.id = b.w;
    return x;
}
__device__ __forceinline__ uint32_t slot_id(const Slots& s, uint32_t i) { return s.b[i].w; }

// a box that overlaps nothing (pads tiles to multiples of 8 and idle lanes)
template <bool NARROW>
__device__ __forceinline__ Box dummy_box() {
    Box x;
    x.x0 = x.y0 = x.z0 = NARROW ? (1u << 30) : 0xffffffffu;
    x.x1 = x.y1 = x.z1 = 0u;
    x.f = 7u << kMissShift;
    x.id = 0;
    return x;
}

template <int D, bool NARROW>
__device__ __forceinline__ Box load_box(const Params& p, uint32_t raw) {
    Box x;
    x.id = raw & kIdMask;
    x.f = (~(raw >> kIdBits) & 7u) << kMissShift;
    if (x.id >= p.nboxes) {  // cannot happen with a consistent grid; never read past the box buffer
        atomicOr(&p.ctr->err, kErrIndex);
        return dummy_box<NARROW>();
    }
    const uint32_t* b = p.boxes + (uint64_t)x.id * (2 * D + 1);
    x.x0 = __ldg(b); x.x1 = __ldg(b + 1); x.y0 = __ldg(b + 2); x.y1 = __ldg(b + 3);
    if (D == 3) { x.z0 = __ldg(b + 4); x.z1 = __ldg(b + 5); }
    else { x.z0 = 0; x.z1 = 0; }
    return x;
}

// closed-interval overlap on every axis (calcOverlaps, pbig.cu:562-577) and
// the reference-cell rule (calcRightToWrite, pbig.cu:579-603); 1 or 0
template <int D, bool BIP, bool NARROW>
__device__ __forceinline__ uint32_t hit_bit(const Box& a, const Box& b, uint32_t split) {
    uint32_t ok;
    if (NARROW) {
        uint32_t t = (b.x1 - a.x0) | (a.x1 - b.x0) | (b.y1 - a.y0) | (a.y1 - b.y0) | (a.f & b.f);
        if (D == 3) t |= (b.z1 - a.z0) | (a.z1 - b.z0);
        ok = t < (1u << kMissShift) ? 1u : 0u;
    } else {
        ok = ((a.x0 <= b.x1) & (b.x0 <= a.x1) & (a.y0 <= b.y1) & (b.y0 <= a.y1) & ((a.f & b.f) == 0u)) ? 1u : 0u;
        if (D == 3) ok &= ((a.z0 <= b.z1) & (b.z0 <= a.z1)) ? 1u : 0u;
    }
    if (BIP) ok &= ((a.id < split) != (b.id < split)) ? 1u : 0u;
    return ok;
}

// circular half sweep over the m boxes in slots [base, base+m): lane l < m
// tests box l against boxes l+1 .. l+floor(m/2) (mod m), lanes past m/2 one
// fewer when m is even (the BALANCE=1 sweep of d_matching, pbig.cu:804-825),
// so each unordered pair is tested once. Bit d of the result: partner l+d.
template <int D, bool BIP, bool NARROW>
__device__ __forceinline__ uint32_t sweep_diag(const Slots& s, const Box& me, uint32_t lane, uint32_t base,
                                               uint32_t m, uint32_t split) {
    const uint32_t l = lane < m ? lane : 0u;
    const uint32_t nelm = lane < m ? (lane < (m >> 1) ? (m >> 1) : ((m - 1) >> 1)) : 0u;
    const uint32_t dmax = m >> 1;
    uint32_t mask = 0;
#pragma unroll 4
    for (uint32_t d = 1; d <= dmax; d++) {
        uint32_t pr = l + d;
        if (pr >= m) pr -= m;
        mask |= (hit_bit<D, BIP, NARROW>(me, slot_get(s, base + pr), split) & (d <= nelm ? 1u : 0u)) << d;
    }
    return mask;
}

// row box against the column boxes in slots [base, base+cols8), cols8 a
// multiple of 8 (padding slots hold dummy boxes); bit j: column j
template <int D, bool BIP, bool NARROW>
__device__ __forceinline__ uint32_t sweep_cols(const Slots& s, const Box& me, uint32_t base, uint32_t cols8,
                                               uint32_t split) {
    uint32_t mask = 0;
    if (cols8 == 32) {
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) mask |= hit_bit<D, BIP, NARROW>(me, slot_get(s, base + j), split) << j;
    } else {
        for (uint32_t j0 = 0; j0 < cols8; j0 += 8) {
#pragma unroll
            for (uint32_t jj = 0; jj < 8; jj++)
                mask |= hit_bit<D, BIP, NARROW>(me, slot_get(s, base + j0 + jj), split) << (j0 + jj);
        }
    }
    return mask;
}

// ---- output: warp-private buffer ------------------------------------------
struct WarpOut {
    uint2* buf;
    uint32_t n;    // warp-uniform fill
    uint32_t cap;  // buffer capacity (pairs)
    unsigned long long hits = 0;  // record mode: pairs written by this lane
};

// copy n pairs (8-byte words) from shared memory to p.out[base, base + n):
// thread t of nt (a multiple of 32) stores 16-byte units laid on the
// destination's 128-byte lines, so a warp store covers whole lines and only
// the first and last line of a run are partial. The pair array may be
// page-locked host memory, where partial lines cost a large share of the
// link's write bandwidth.
__device__ __forceinline__ void store_run(const Params& p, unsigned long long base, const uint2* src, uint32_t n,
                                          uint32_t t, uint32_t nt) {
    if (base + n > p.out_cap) {
        for (uint32_t k = t; k < n; k += nt) {
            const unsigned long long g = base + k;
            if (g < p.out_cap) p.out[g] = src[k];
            else atomicOr(&p.ctr->err, kErrOutOvf);
        }
        return;
    }
    // pairs of base's line before base (the pair array is 8-byte aligned)
    const uint32_t lead = (uint32_t)(((reinterpret_cast<uintptr_t>(p.out) >> 3) + base) & 15u);
    const uint32_t units = (lead + n + 1) >> 1;
    uint2* dst = p.out + base;
    for (uint32_t u = t; u < units; u += nt) {
        const int r = 2 * (int)u - (int)lead;  // first pair of the unit, relative to base
        if (r >= 0 && r + 1 < (int)n) {
            const uint2 a = src[r], b = src[r + 1];
            *reinterpret_cast<uint4*>(dst + r) = make_uint4(a.x, a.y, b.x, b.y);
        } else {
            if (r >= 0 && r < (int)n) dst[r] = src[r];
            if (r + 1 >= 0 && r + 1 < (int)n) dst[r + 1] = src[r + 1];
        }
    }
}

__device__ __forceinline__ void wflush(const Params& p, WarpOut& o) {
    if (o.n == 0) return;
    const uint32_t lane = lane_id();
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&p.ctr->pairs, (unsigned long long)o.n);
    base = __shfl_sync(FULL_MASK, base, 0);
    __syncwarp();
    store_run(p, base, o.buf, o.n, lane, 32);
    __syncwarp();
    o.n = 0;
}

// compaction of the set bits of two masks (ranks from one warp scan of the
// per-lane popcounts) into the warp buffer, or straight to the pair array
// when the batch is larger than the buffer
template <bool BIP, class PA, class PB>
__device__ __forceinline__ void wemit(const Params& p, WarpOut& o, uint32_t ma, PA pa, uint32_t mb, PB pb,
                                      uint32_t myid) {
    const uint32_t lane = lane_id();
    const uint32_t k = __popc(ma) + __popc(mb);
    const uint32_t incl = warp_incl_scan(k);
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    if (total == 0) return;
    bool direct = false;
    unsigned long long gbase = 0;
    if (o.n + total > o.cap) {
        wflush(p, o);
        if (total > o.cap) {
            direct = true;
            if (lane == 0) gbase = atomicAdd(&p.ctr->pairs, (unsigned long long)total);
            gbase = __shfl_sync(FULL_MASK, gbase, 0);
        }
    }
    uint32_t w = incl - k;
    auto pair = [&](uint32_t q) {
        uint2 pr = make_uint2(min(myid, q), max(myid, q));
        if (BIP) pr.y -= p.split;
        return pr;
    };
    if (!direct) {  // (warp-uniform: the loops below carry no per-pair branch)
        uint2* dst = o.buf + o.n + w;
        while (ma) {
            const uint32_t bit = 31u - __clz(ma);  // highest set bit first
            ma ^= 1u << bit;
            *dst++ = pair(pa(bit));
        }
        while (mb) {
            const uint32_t bit = 31u - __clz(mb);
            mb ^= 1u << bit;
            *dst++ = pair(pb(bit));
        }
        __syncwarp();
        o.n += total;
        return;
    }
    auto put = [&](uint32_t q) {
        const unsigned long long g = gbase + w;
        if (g < p.out_cap) p.out[g] = pair(q);
        else atomicOr(&p.ctr->err, kErrOutOvf);
        w++;
    };
    while (ma) {
        const uint32_t bit = __ffs(ma) - 1;
        ma &= ma - 1;
        put(pa(bit));
    }
    while (mb) {
        const uint32_t bit = __ffs(mb) - 1;
        mb &= mb - 1;
        put(pb(bit));
    }
    __syncwarp();
}

// ---- record mode: the reference's Rice stream ------------------------------
// (RICE_COMPRESSION with 8-byte OTYPE: writer src/pbig/pbig.cu:788-920, reader
// src/pbig/decode.cc:38-131). A block is the header {UNUSED, cell id} followed
// by records; a record is one row box's hits in one 256-column tile of the
// cell: byte 0 row tile (row >> 8), byte 1 column tile, bytes 2-3 the row's
// index in its tile, bytes 4-5 the hit count, then one byte per hit (the
// column's index in its tile), padded to 8 bytes. Rows and columns are
// indices into the cell's entry list. Here a block is written per emission
// step (a cell may have several blocks, as the reference's cells of several
// jobs do), and a record covers one 32-column tile or the diagonal sweep.
constexpr unsigned long long kRiceUnused = 0x0fffff11ull;  // UNUSED, the block marker

__device__ __forceinline__ uint32_t rec_words(uint32_t hits) { return hits ? (6u + hits + 7u) >> 3 : 0u; }

// one record: `row` and the columns loc(bit) of the set bits of m (all in one
// 256-column tile) into dst, or nowhere when `keep` is false
template <class L>
__device__ __forceinline__ void rec_write(unsigned long long* dst, bool keep, uint32_t row, uint32_t m, L loc) {
    const uint32_t nh = __popc(m);
    unsigned long long word = (unsigned long long)(row >> 8) | ((unsigned long long)(loc(__ffs(m) - 1) >> 8) << 8) |
                              ((unsigned long long)(row & 255u) << 16) | ((unsigned long long)nh << 32);
    uint32_t byte = 6, wi = 0;
    while (m) {
        const uint32_t b = __ffs(m) - 1;
        m &= m - 1;
        word |= (unsigned long long)(loc(b) & 255u) << (8 * byte);
        if (++byte == 8) {
            if (keep) dst[wi] = word;
            wi++;
            word = 0;
            byte = 0;
        }
    }
    if (byte && keep) dst[wi] = word;
}

// warp step: lane records for ma (columns la) and mb (columns lb), one block
// header per cell before its first record; gmask: the lanes of this lane's
// cell (the whole warp, or a lane group of the small-cell kernel)
template <class LA, class LB>
__device__ __forceinline__ void remit(const Params& p, WarpOut& o, uint32_t ma, LA la, uint32_t mb, LB lb,
                                      uint32_t row, uint32_t gid, uint32_t gmask) {
    const uint32_t lane = lane_id();
    const uint32_t wa = rec_words(__popc(ma)), wb = rec_words(__popc(mb));
    const uint32_t gany = __ballot_sync(FULL_MASK, (wa | wb) != 0u) & gmask;
    const bool hdr = gany != 0u && lane == (uint32_t)(__ffs(gany) - 1);
    const uint32_t k = wa + wb + (hdr ? 2u : 0u);
    const uint32_t incl = warp_incl_scan(k);
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    if (total == 0) return;
    o.hits += __popc(ma) + __popc(mb);
    bool direct = false;
    unsigned long long gbase = 0;
    if (o.n + total > o.cap) {
        wflush(p, o);
        if (total > o.cap) {
            direct = true;
            if (lane == 0) gbase = atomicAdd(&p.ctr->pairs, (unsigned long long)total);
            gbase = __shfl_sync(FULL_MASK, gbase, 0);
        }
    }
    const bool keep = !direct || gbase + total <= p.out_cap;
    if (direct && !keep && lane == 0) atomicOr(&p.ctr->err, kErrOutOvf);
    unsigned long long* dst = direct ? reinterpret_cast<unsigned long long*>(p.out) + gbase
                                     : reinterpret_cast<unsigned long long*>(o.buf + o.n);
    uint32_t w = incl - k;
    if (hdr && keep) {
        dst[w] = kRiceUnused;
        dst[w + 1] = gid;
    }
    if (hdr) w += 2;
    if (wa) rec_write(dst + w, keep, row, ma, la);
    if (wb) rec_write(dst + w + wa, keep, row, mb, lb);
    __syncwarp();
    if (!direct) o.n += total;
}

// row tile r of a cell staged at slots [off, off + n8): the diagonal tile and
// every column tile x > r, emitted two tiles at a time
template <int D, bool BIP, bool NARROW, bool REC, class Emit>
__device__ __forceinline__ void row_unit(const Params& p, const Slots& s, uint32_t off, uint32_t n, uint32_t r,
                                         Emit emit) {
    const uint32_t lane = lane_id();
    const uint32_t R = (n + 31) >> 5;
    const uint32_t rows = min(32u, n - 32 * r);
    const uint32_t rbase = off + 32 * r;
    const Box me = lane < rows ? slot_get(s, rbase + lane) : dummy_box<NARROW>();
    const uint32_t md = sweep_diag<D, BIP, NARROW>(s, me, lane, rbase, rows, p.split);
    if constexpr (REC) {  // records: cell-local row and column indices
        const uint32_t row = 32 * r + lane;
        auto ldiag = [&](uint32_t d) {
            uint32_t pr = lane + d;
            if (pr >= rows) pr -= rows;
            return 32 * r + pr;
        };
        uint32_t x = r + 1;
        if (x >= R) {
            emit(md, ldiag, 0u, ldiag, row);
            return;
        }
        {
            const uint32_t cb = off + 32 * x, c8 = (min(32u, n - 32 * x) + 7) & ~7u;
            const uint32_t mc = sweep_cols<D, BIP, NARROW>(s, me, cb, c8, p.split);
            emit(md, ldiag, mc, [&](uint32_t j) { return 32 * x + j; }, row);
        }
        for (x = r + 2; x < R; x += 2) {
            const uint32_t cb1 = off + 32 * x, c81 = (min(32u, n - 32 * x) + 7) & ~7u;
            const uint32_t m1 = sweep_cols<D, BIP, NARROW>(s, me, cb1, c81, p.split);
            uint32_t m2 = 0;
            if (x + 1 < R)
                m2 = sweep_cols<D, BIP, NARROW>(s, me, off + 32 * (x + 1), (min(32u, n - 32 * (x + 1)) + 7) & ~7u,
                                                p.split);
            emit(m1, [&](uint32_t j) { return 32 * x + j; }, m2, [&](uint32_t j) { return 32 * (x + 1) + j; }, row);
        }
        return;
    }
    auto pdiag = [&](uint32_t d) {
        uint32_t pr = lane + d;
        if (pr >= rows) pr -= rows;
        return slot_id(s, rbase + pr);
    };
    uint32_t x = r + 1;
    if (x >= R) {
        emit(md, pdiag, 0u, pdiag, me.id);
        return;
    }
    {
        const uint32_t cb = off + 32 * x, c8 = (min(32u, n - 32 * x) + 7) & ~7u;
        const uint32_t mc = sweep_cols<D, BIP, NARROW>(s, me, cb, c8, p.split);
        emit(md, pdiag, mc, [&](uint32_t j) { return slot_id(s, cb + j); }, me.id);
    }
    for (x = r + 2; x < R; x += 2) {
        const uint32_t cb1 = off + 32 * x, c81 = (min(32u, n - 32 * x) + 7) & ~7u;
        const uint32_t m1 = sweep_cols<D, BIP, NARROW>(s, me, cb1, c81, p.split);
        uint32_t m2 = 0, cb2 = cb1;
        if (x + 1 < R) {
            cb2 = off + 32 * (x + 1);
            m2 = sweep_cols<D, BIP, NARROW>(s, me, cb2, (min(32u, n - 32 * (x + 1)) + 7) & ~7u, p.split);
        }
        emit(m1, [&](uint32_t j) { return slot_id(s, cb1 + j); }, m2, [&](uint32_t j) { return slot_id(s, cb2 + j); },
             me.id);
    }
}

// Medium-cell staging. With coordinates < 2^29 a slot holds its box as the
// six signed terms (-x1, x0, -y1, y0, -z1, z0) (then f and the index), and a
// row box is taken as the partner terms (x0-1, -x1-1, y0-1, -y1-1, z0-1,
// -z1-1). Each sum row_k + col_k is the gap between the two boxes along one
// axis and side minus one (a.x0 - c.x1 - 1, c.x0 - a.x1 - 1, ...), so the
// closed boxes overlap iff the largest of the six sums is negative: one add
// and five add-max instructions per test, the result's sign bit the hit.
// Wider coordinates keep the plain layout and comparisons.
struct SepRow {
    int t0, t1, t2, t3, t4, t5;
};
template <bool NARROW> struct MedRowT { using type = Box; };
template <> struct MedRowT<true> { using type = SepRow; };

// (with narrow coordinates the b array's space holds the z terms,
// uint2[kMedSlots], then {f, id}, uint2[kMedSlots]: 8-byte loads of
// consecutive slots take two wavefronts a warp, not four)
__device__ __forceinline__ uint2* med_z(const Slots& s) { return reinterpret_cast<uint2*>(s.b); }
__device__ __forceinline__ uint2* med_fi(const Slots& s) { return reinterpret_cast<uint2*>(s.b) + kMedSlots; }

template <bool NARROW>
__device__ __forceinline__ void med_slot_put(const Slots& s, uint32_t i, const Box& x) {
    if constexpr (NARROW) {
        s.a[i] = make_uint4(0u - x.x1, x.x0, 0u - x.y1, x.y0);
        med_z(s)[i] = make_uint2(0u - x.z1, x.z0);
        med_fi(s)[i] = make_uint2(x.f, x.id);
    } else {
        slot_put(s, i, x);
    }
}

// a staged medium-cell box in slot_get's form
template <bool NARROW>
__device__ __forceinline__ Box med_slot_get(const Slots& s, uint32_t i) {
    if constexpr (NARROW) {
        const uint4 a = s.a[i];
        const uint2 z = med_z(s)[i], fi = med_fi(s)[i];
        Box x;
        x.x0 = a.x; x.x1 = a.y; x.y0 = a.z; x.y1 = a.w;
        x.z0 = z.x; x.z1 = z.y; x.f = fi.x; x.id = fi.y;
        return x;
    } else {
        return slot_get(s, i);
    }
}

template <bool NARROW>
__device__ __forceinline__ uint32_t med_slot_id(const Slots& s, uint32_t i) {
    if constexpr (NARROW) return med_fi(s)[i].y;
    else return slot_id(s, i);
}

// the row form of a staged box (st: slot_get of its slot)
template <bool NARROW>
__device__ __forceinline__ typename MedRowT<NARROW>::type med_row(const Box& st) {
    if constexpr (NARROW) {  // slot_get maps (-x1, x0, -y1, y0, -z1, z0) to (x0, x1, y0, y1, z0, z1)
        return SepRow{(int)st.x1 - 1, (int)st.x0 - 1, (int)st.y1 - 1, (int)st.y0 - 1, (int)st.z1 - 1, (int)st.z0 - 1};
    } else {
        return st;
    }
}

// bit 31 set iff row box r and column box (ca, cz) overlap
template <int D>
__device__ __forceinline__ uint32_t sep_hit(const SepRow& r, const uint4& ca, const uint2& cz) {
    int m = r.t0 + (int)ca.x;
    m = __viaddmax_s32(r.t1, (int)ca.y, m);
    m = __viaddmax_s32(r.t2, (int)ca.z, m);
    m = __viaddmax_s32(r.t3, (int)ca.w, m);
    if (D == 3) {
        m = __viaddmax_s32(r.t4, (int)cz.x, m);
        m = __viaddmax_s32(r.t5, (int)cz.y, m);
    }
    return (uint32_t)m;
}

// ---- small cells ------------------------------------------------------------
// lane group g (WG lanes) holds cell item*G+g of the class list, lane r its
// box r; the circular half sweep runs inside the group.
template <int D, int WG, bool NARROW, bool REC>
__device__ __forceinline__ Box small_fetch(const Params& p, int list, uint64_t nl, uint64_t ci, uint32_t r,
                                           uint32_t& n, uint32_t& gid) {
    n = 0;
    gid = 0;
    uint32_t start = 0;
    if (ci < nl) {
        const uint2 sn = p.lists[p.list_off[list] + ci];
        start = sn.x;
        n = sn.y;
        if (REC) {  // the list holds the cell id; its start is in the counters after the scatter
            gid = sn.x;
            start = gid < p.ncells ? p.counts[gid] : 0xffffffffu;
        }
        if (n > WG || (uint64_t)start + n > p.entry_cap) n = 0;  // inconsistent grid: skip
    }
    return r < n ? load_box<D, NARROW>(p, p.entries[start + r]) : dummy_box<NARROW>();
}

template <int D, int WG, bool BIP, bool NARROW, bool REC>
__device__ __forceinline__ void small_sweep(const Params& p, const Slots& s, WarpOut& o, const Box& me, uint32_t n,
                                            uint32_t lane, uint32_t g, uint32_t r, uint32_t gid) {
    if constexpr (NARROW && !REC) {
        // the medium-cell test: boxes staged as separation terms, one add and
        // add-max instructions per test; the group's cell staged twice in a
        // row, so partner r+d needs no wrap; the reference-cell and red/blue
        // rules applied once per cell from ballots. Slot i: s.a[i] the x and y
        // terms, then in s.b's space the z terms (8 bytes per slot, so a
        // warp's loads take two wavefronts) and the box index.
        const uint32_t gb = g * (2 * WG);
        uint2* zz = reinterpret_cast<uint2*>(s.b);
        uint32_t* ids = reinterpret_cast<uint32_t*>(s.b) + 2 * kSmallSlots;
        if (r < n) {
            const uint4 xa = make_uint4(0u - me.x1, me.x0, 0u - me.y1, me.y0);
            s.a[gb + r] = xa;
            s.a[gb + n + r] = xa;
            if (D == 3) {
                const uint2 zt = make_uint2(0u - me.z1, me.z0);
                zz[gb + r] = zt;
                zz[gb + n + r] = zt;
            }
            ids[gb + r] = me.id;
            ids[gb + n + r] = me.id;
        }
        __syncwarp();
        const uint32_t nelm = r < n ? (r < (n >> 1) ? (n >> 1) : ((n - 1) >> 1)) : 0u;
        const uint32_t dlim = __reduce_max_sync(FULL_MASK, nelm);
        // bit j: group lane j is a partner the rules exclude
        const uint32_t sh = WG == 32 ? 0u : g * WG;
        const uint32_t nm = n >= 32u ? FULL_MASK : ((1u << n) - 1u);
        const uint32_t fa = me.f >> kMissShift;
        const uint32_t m0 = (__ballot_sync(FULL_MASK, (fa & 1u) != 0u) >> sh) & nm;
        const uint32_t m1 = (__ballot_sync(FULL_MASK, (fa & 2u) != 0u) >> sh) & nm;
        const uint32_t m2 = (__ballot_sync(FULL_MASK, (fa & 4u) != 0u) >> sh) & nm;
        uint32_t deny = ((fa & 1u) ? m0 : 0u) | ((fa & 2u) ? m1 : 0u) | ((fa & 4u) ? m2 : 0u);
        if (BIP) {
            const uint32_t red = (__ballot_sync(FULL_MASK, me.id < p.split) >> sh) & nm;
            deny |= me.id < p.split ? red : (~red & nm);
        }
        // bit d: partner (r + d) mod n
        uint32_t rot = 0;
        if (r < n) rot = n >= 32u ? __funnelshift_r(deny, deny, r) : (((deny >> r) | (deny << (n - r))) & nm);
        const SepRow row{(int)me.x0 - 1, -(int)me.x1 - 1, (int)me.y0 - 1, -(int)me.y1 - 1, (int)me.z0 - 1,
                         -(int)me.z1 - 1};
        uint32_t mask = 0;
#pragma unroll
        for (uint32_t d = 1; d <= WG / 2; d++) {
            if (d > dlim) break;
            const uint32_t i = gb + r + d;
            const uint4 ca = s.a[i];
            const uint2 cz = D == 3 ? zz[i] : make_uint2(0u, 0u);
            mask |= (sep_hit<D>(row, ca, cz) >> 31) << d;
        }
        mask &= ~rot & ((2u << nelm) - 2u);
        auto pid = [&](uint32_t d) { return ids[gb + r + d]; };
        wemit<BIP>(p, o, mask, pid, 0u, pid, me.id);
        return;
    }
    slot_put(s, lane, me);
    __syncwarp();
    const uint32_t gb = g * WG;
    const uint32_t nelm = r < n ? (r < (n >> 1) ? (n >> 1) : ((n - 1) >> 1)) : 0u;
    // partners a lane of the warp needs at most: the sweep stops there rather
    // than at WG/2 (a cell of 17 boxes in a 32-lane group needs 8, not 16)
    const uint32_t dlim = __reduce_max_sync(FULL_MASK, nelm);
    uint32_t mask = 0;
#pragma unroll
    for (uint32_t d = 1; d <= WG / 2; d++) {
        if (d > dlim) break;
        uint32_t pr = r + d;
        if (pr >= n) pr -= n;
        if (pr >= WG) pr = 0;  // idle lanes (n = 0) stay inside the group
        mask |= (hit_bit<D, BIP, NARROW>(me, slot_get(s, gb + pr), p.split) & (d <= nelm ? 1u : 0u)) << d;
    }
    if constexpr (REC) {
        auto ploc = [&](uint32_t d) {
            uint32_t pr = r + d;
            if (pr >= n) pr -= n;
            return pr;
        };
        const uint32_t gmask = WG == 32 ? FULL_MASK : (((1u << WG) - 1u) << (g * WG));
        remit(p, o, mask, ploc, 0u, ploc, r, gid, gmask);
    } else {
        auto pid = [&](uint32_t d) {
            uint32_t pr = r + d;
            if (pr >= n) pr -= n;
            return slot_id(s, gb + pr);
        };
        wemit<BIP>(p, o, mask, pid, 0u, pid, me.id);
    }
}

template <int D, int WG, bool BIP, bool NARROW, bool REC, bool FRESH = false>
__device__ __forceinline__ void small_items(const Params& p, const Slots& s, WarpOut& o, int list, uint64_t first,
                                            uint64_t stride) {
    constexpr uint32_t G = 32 / WG;
    const uint32_t lane = lane_id(), g = lane / WG, r = lane % WG;
    const uint64_t nl = mn64(ctr_read<FRESH>(&p.ctr->n_list[list]), p.list_cap[list]);
    const uint64_t nitems = (nl + G - 1) / G;
    for (uint64_t item = first; item < nitems; item += stride) {
        uint32_t n1, gid;
        const Box a = small_fetch<D, WG, NARROW, REC>(p, list, nl, item * G + g, r, n1, gid);
        small_sweep<D, WG, BIP, NARROW, REC>(p, s, o, a, n1, lane, g, r, gid);
    }
}

// hits of a warp's records, added to the query's pair count
__device__ __forceinline__ void rec_hits(const Params& p, const WarpOut& o) {
    const unsigned long long h = warp_sum_u64(o.hits);
    if (lane_id() == 0 && h) atomicAdd(&p.ctr->rec_pairs, h);
}

// the four small-cell lists, warp gw of nw; per-warp staging in s_a, s_b
// (kSmallSlots each) and an output buffer of kWarpOut pairs
template <int D, bool BIP, bool NARROW, bool REC, bool FRESH = false>
__device__ __forceinline__ void small_pass(const Params& p, uint4* s_a, uint4* s_b, uint2* s_out, uint64_t gw,
                                           uint64_t nw) {
    const Slots s{s_a, s_b};
    WarpOut o{s_out, 0, kWarpOut};
    // classes interleaved over the warps so every warp gets a similar mix
    small_items<D, 32, BIP, NARROW, REC, FRESH>(p, s, o, 3, gw, nw);
    small_items<D, 16, BIP, NARROW, REC, FRESH>(p, s, o, 2, (gw + nw / 4) % nw, nw);
    small_items<D, 8, BIP, NARROW, REC, FRESH>(p, s, o, 1, (gw + nw / 2) % nw, nw);
    small_items<D, 4, BIP, NARROW, REC, FRESH>(p, s, o, 0, (gw + 3 * nw / 4) % nw, nw);
    wflush(p, o);
    if (REC) rec_hits(p, o);
}

template <int D, bool BIP, bool NARROW, bool REC = false>
__global__ void __launch_bounds__(kPairThreads, 5) k_pairs_small(Params p) {
    __shared__ uint4 s_a[kPairWarps][kSmallSlots], s_b[kPairWarps][kSmallSlots];
    __shared__ uint2 s_out[kPairWarps][kWarpOut];
    const uint32_t warp = threadIdx.x >> 5;
    small_pass<D, BIP, NARROW, REC>(p, s_a[warp], s_b[warp], s_out[warp], (uint64_t)blockIdx.x * kPairWarps + warp,
                                    (uint64_t)gridDim.x * kPairWarps);
}

// ---- medium cells: one per warp item, staged whole ---------------------------
// The reference-cell rule and the red/blue rule are applied per 32-column
// tile with ballots (bit j: column j may pair with this lane's row box), so
// the per-pair work is the overlap test alone: six differences whose OR has
// bit 31 set iff some pair of intervals is disjoint, pushed into the hit
// mask with one funnel shift (mask = mask << 1 | hit).

// columns [c0, c0 + ncol) of the staged cell that row box `me` may pair with
template <bool BIP, bool NARROW>
__device__ __forceinline__ uint32_t tile_allow(const Params& p, const Slots& s, uint32_t c0, uint32_t ncol,
                                               const Box& me) {
    const uint32_t lane = lane_id();
    const bool v = lane < ncol;
    uint32_t bf, bid;
    if constexpr (NARROW) {
        const uint2 fi = med_fi(s)[c0 + (v ? lane : 0u)];
        bf = fi.x;
        bid = fi.y;
    } else {
        const uint4 b = s.b[c0 + (v ? lane : 0u)];
        bf = b.z;
        bid = b.w;
    }
    const uint32_t f = v ? bf >> kMissShift : 0u;
    const uint32_t vm = __ballot_sync(FULL_MASK, v);
    const uint32_t m0 = __ballot_sync(FULL_MASK, (f & 1u) != 0u);
    const uint32_t m1 = __ballot_sync(FULL_MASK, (f & 2u) != 0u);
    const uint32_t m2 = __ballot_sync(FULL_MASK, (f & 4u) != 0u);
    const uint32_t fa = me.f >> kMissShift;
    uint32_t allow = vm & ~(((fa & 1u) ? m0 : 0u) | ((fa & 2u) ? m1 : 0u) | ((fa & 4u) ? m2 : 0u));
    if (BIP) {
        const uint32_t red = __ballot_sync(FULL_MASK, v && bid < p.split);
        allow &= (me.id < p.split) ? ~red : red;
    }
    return allow;
}

// bit 31 set iff row box a and column box (ca, cz) are disjoint on some axis
template <int D, bool NARROW>
__device__ __forceinline__ uint32_t miss_word(const Box& a, const uint4& ca, const uint2& cz) {
    if (NARROW) {
        uint32_t t = (ca.y - a.x0) | (a.x1 - ca.x) | (ca.w - a.y0) | (a.y1 - ca.z);
        if (D == 3) t |= (cz.y - a.z0) | (a.z1 - cz.x);
        return t;
    }
    bool ok = (a.x0 <= ca.y) & (ca.x <= a.x1) & (a.y0 <= ca.w) & (ca.z <= a.y1);
    if (D == 3) ok &= (a.z0 <= cz.y) & (cz.x <= a.z1);
    return ok ? 0u : 0x80000000u;
}

__device__ __forceinline__ uint32_t push_hit(uint32_t mask, uint32_t miss) { return __funnelshift_l(~miss, mask, 1); }

template <int D, bool NARROW, class Row>
__device__ __forceinline__ uint32_t test_slot(const Slots& s, const Row& me, uint32_t mask, uint32_t i) {
    const uint4 ca = s.a[i];
    const uint2 cz = D == 3 ? (NARROW ? med_z(s)[i] : *reinterpret_cast<const uint2*>(&s.b[i])) : make_uint2(0u, 0u);
    if constexpr (NARROW) return __funnelshift_l(sep_hit<D>(me, ca, cz), mask, 1);
    else return push_hit(mask, miss_word<D, false>(me, ca, cz));
}

// row box against columns [c0, c0 + cnt), cnt a multiple of 8 up to 32;
// bit cnt-1-j of the result: column j
template <int D, bool NARROW, class Row>
__device__ __forceinline__ uint32_t sweep_tile(const Slots& s, const Row& me, uint32_t c0, uint32_t cnt) {
    uint32_t mask = 0;
    if (cnt == 32) {
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) mask = test_slot<D, NARROW>(s, me, mask, c0 + j);
    } else {
        for (uint32_t j0 = 0; j0 < cnt; j0 += 8) {
#pragma unroll
            for (uint32_t jj = 0; jj < 8; jj++) mask = test_slot<D, NARROW>(s, me, mask, c0 + j0 + jj);
        }
    }
    return mask;
}

// circular half sweep of the m rows staged at [rb, rb + m): lane l < m tests
// partners l+1 .. l+floor(m/2) (mod m), lanes past m/2 one fewer when m is
// even (the BALANCE=1 sweep of d_matching, pbig.cu:804-825), so each
// unordered pair is tested once; bit dmax-d of the result: partner l+d
template <int D, bool NARROW, class Row>
__device__ __forceinline__ uint32_t sweep_diag2(const Slots& s, const Row& me, uint32_t l, uint32_t rb, uint32_t m) {
    uint32_t mask = 0;
    if (m == 32) {
#pragma unroll
        for (uint32_t d = 1; d <= 16; d++) mask = test_slot<D, NARROW>(s, me, mask, rb + ((l + d) & 31u));
    } else {
        const uint32_t dmax = m >> 1;
#pragma unroll 4
        for (uint32_t d = 1; d <= dmax; d++) {
            uint32_t pr = l + d;
            if (pr >= m) pr -= m;
            mask = test_slot<D, NARROW>(s, me, mask, rb + pr);
        }
    }
    return mask;
}

// the allow mask of the diagonal tile in sweep_diag2's bit order, with the
// half-sweep limit applied
__device__ __forceinline__ uint32_t diag_allow(uint32_t allow, uint32_t lane, uint32_t m) {
    if (lane >= m) return 0u;
    const uint32_t dmax = m >> 1;
    if (dmax == 0) return 0u;
    uint32_t rot;  // bit d: partner (lane + d) mod m
    if (m == 32) rot = __funnelshift_r(allow, allow, lane);
    else rot = ((allow >> lane) | (allow << (m - lane))) & ((1u << m) - 1u);
    uint32_t a = (__brev(rot) >> (31u - dmax)) & ((1u << dmax) - 1u);
    if ((m & 1u) == 0u && lane >= dmax) a &= ~1u;  // even m: the opposite partner once
    return a;
}

// the medium-cell list, warp gw of nw (the one-launch kernel: items in a
// fixed stride; the medium-cell kernel: every warp takes items from one
// counter); wsm: the warp's kMedWarpBytes of shared memory (staging slots,
// then the output buffer)
constexpr uint32_t kMedWarpBytes = kMedSlots * 2 * sizeof(uint4) + kMedOut * sizeof(uint2);

template <int D, bool BIP, bool NARROW, bool REC, bool FRESH = false>
__device__ __forceinline__ void med_pass(const Params& p, unsigned char* wsm, uint64_t gw, uint64_t nw) {
    const uint32_t lane = lane_id();
    uint4* base = reinterpret_cast<uint4*>(wsm);
    const Slots s{base, base + kMedSlots};
    WarpOut o{reinterpret_cast<uint2*>(base + 2 * kMedSlots), 0, kMedOut};
    const uint64_t nl = mn64(ctr_read<FRESH>(&p.ctr->n_list[kListMed]), p.list_cap[kListMed]);
    auto cell = [&](uint64_t item) {
        const uint2 sn = p.lists[p.list_off[kListMed] + item];
        const uint32_t gid = sn.x;  // record mode: the cell id (its start is in the counters)
        const uint32_t start = REC ? (gid < p.ncells ? p.counts[gid] : 0xffffffffu) : sn.x;
        const uint32_t n = sn.y;
        if (n > kMedMax || (uint64_t)start + n > p.entry_cap) return;  // inconsistent grid: skip
        const uint32_t R = (n + 31) >> 5;
        // stage: all entry ids first, then all boxes (loads in flight together)
        uint32_t raw[kMedSlots / 32];
#pragma unroll
        for (uint32_t k = 0; k < kMedSlots / 32; k++) {
            const uint32_t e = lane + 32 * k;
            raw[k] = e < n ? p.entries[start + e] : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < kMedSlots / 32; k++) {
            const uint32_t e = lane + 32 * k;
            if (e < 32 * R) med_slot_put<NARROW>(s, e, e < n ? load_box<D, NARROW>(p, raw[k]) : dummy_box<NARROW>());
        }
        __syncwarp();
        for (uint32_t r = 0; r < R; r++) {
            const uint32_t rows = min(32u, n - 32 * r), rb = 32 * r;
            const Box me = med_slot_get<NARROW>(s, rb + lane);  // lanes >= rows hold a padding box, masked below
            const auto row = med_row<NARROW>(me);
            const uint32_t l = lane < rows ? lane : 0u;
            const uint32_t dm = sweep_diag2<D, NARROW>(s, row, l, rb, rows) &
                                diag_allow(tile_allow<BIP, NARROW>(p, s, rb, rows, me), lane, rows);
            const uint32_t dmax = rows >> 1;
            auto pdiag = [&](uint32_t k) {
                uint32_t pr = l + dmax - k;
                if (pr >= rows) pr -= rows;
                return med_slot_id<NARROW>(s, rb + pr);
            };
            uint32_t pend = dm;  // the diagonal's hits wait for the first column tile
            bool have = true;
            for (uint32_t x = r + 1; x < R; x++) {
                const uint32_t c0 = 32 * x, ncol = min(32u, n - c0);
                uint32_t allow = tile_allow<BIP, NARROW>(p, s, c0, ncol, me);
                if (lane >= rows) allow = 0u;
                uint32_t mc = 0;
                const uint32_t cnt = (ncol + 7) & ~7u;
                if (__any_sync(FULL_MASK, allow != 0u))
                    mc = sweep_tile<D, NARROW>(s, row, c0, cnt) & (__brev(allow) >> (32u - cnt));
                auto pcol = [&](uint32_t k) { return med_slot_id<NARROW>(s, c0 + cnt - 1 - k); };
                if constexpr (REC) {
                    auto lcol = [&](uint32_t k) { return c0 + cnt - 1 - k; };
                    auto ldiag = [&](uint32_t k) {
                        uint32_t pr = l + dmax - k;
                        if (pr >= rows) pr -= rows;
                        return rb + pr;
                    };
                    if (have) remit(p, o, pend, ldiag, mc, lcol, rb + lane, gid, FULL_MASK);
                    else remit(p, o, mc, lcol, 0u, lcol, rb + lane, gid, FULL_MASK);
                    have = false;
                } else if (have) {
                    wemit<BIP>(p, o, pend, pdiag, mc, pcol, me.id);
                    have = false;
                } else {
                    wemit<BIP>(p, o, mc, pcol, 0u, pcol, me.id);
                }
            }
            if (have) {
                if constexpr (REC) {
                    auto ldiag = [&](uint32_t k) {
                        uint32_t pr = l + dmax - k;
                        if (pr >= rows) pr -= rows;
                        return rb + pr;
                    };
                    remit(p, o, pend, ldiag, 0u, ldiag, rb + lane, gid, FULL_MASK);
                } else {
                    wemit<BIP>(p, o, pend, pdiag, 0u, pdiag, me.id);
                }
            }
        }
        __syncwarp();
    };
    // items taken one at a time from a counter, so warps whose cells were
    // larger end no later than the others (on the clustered 4M-box scene
    // 0.444 ms, against 0.499 ms for a fixed stride over the list and
    // 0.455-0.50 ms for a fixed stride over its first half to seven eighths).
    // A one-launch query's warps take one or two cells each: there the
    // counter's round trip costs more than the balance gains.
    if constexpr (FRESH) {
        for (uint64_t item = gw; item < nl; item += nw) cell(item);
    } else {
        for (;;) {
            uint64_t item = 0;
            if (lane == 0) item = atomicAdd(&p.ctr->med_next, 1u);
            item = __shfl_sync(FULL_MASK, item, 0);
            if (item >= nl) break;
            cell(item);
        }
    }
    wflush(p, o);
    if (REC) rec_hits(p, o);
}

template <int D, bool BIP, bool NARROW, bool REC = false>
__global__ void __launch_bounds__(kPairThreads, 3) k_pairs_med(Params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t warp = threadIdx.x >> 5;
    med_pass<D, BIP, NARROW, REC>(p, smem_raw + warp * kMedWarpBytes, (uint64_t)blockIdx.x * kPairWarps + warp,
                                  (uint64_t)gridDim.x * kPairWarps);
}

// ---- big cells (block staged) and huge cells (tiles) -----------------------
// a barrier of the whole block, or (SUB) of its first kPairThreads threads
template <bool SUB>
__device__ __forceinline__ void block_sync() {
    if constexpr (SUB) asm volatile("bar.sync 1, %0;" ::"n"(kPairThreads) : "memory");
    else __syncthreads();
}

struct BlockSmem {
    uint4 a[kBlockSlots];
    uint4 b[kBlockSlots];
    uint2 out[kBlockOut];
    uint32_t out_n, first_ovf;
    unsigned long long gbase;
    uint32_t cell_start[kBigCellsPerTask], cell_n[kBigCellsPerTask], cell_off[kBigCellsPerTask + 1];
    uint32_t unit_pref[kBigCellsPerTask + 1];
    uint32_t k, tot, units;
    unsigned long long nbt[2];
    uint32_t cell_gid[kBigCellsPerTask];  // record mode: cell ids
    unsigned long long hits;              // record mode: pairs written by the block
};

// block-buffer compaction (shared reservation per warp call); when the
// buffer is full the warp reserves global space itself
template <bool BIP, class PA, class PB>
__device__ __forceinline__ void bemit(const Params& p, BlockSmem& s, uint32_t ma, PA pa, uint32_t mb, PB pb,
                                      uint32_t myid) {
    const uint32_t lane = lane_id();
    const uint32_t k = __popc(ma) + __popc(mb);
    const uint32_t incl = warp_incl_scan(k);
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    if (total == 0) return;
    uint32_t pos = 0;
    unsigned long long gbase = 0;
    if (lane == 0) {
        pos = atomicAdd(&s.out_n, total);
        if (pos + total > kBlockOut) {
            atomicMin(&s.first_ovf, pos);
            gbase = atomicAdd(&p.ctr->pairs, (unsigned long long)total);
        }
    }
    pos = __shfl_sync(FULL_MASK, pos, 0);
    gbase = __shfl_sync(FULL_MASK, gbase, 0);
    const bool direct = pos + total > kBlockOut;
    uint32_t w = incl - k;
    auto put = [&](uint32_t q) {
        uint2 pr = make_uint2(min(myid, q), max(myid, q));
        if (BIP) pr.y -= p.split;
        if (!direct) {
            s.out[pos + w] = pr;
        } else {
            const unsigned long long g = gbase + w;
            if (g < p.out_cap) p.out[g] = pr;
            else atomicOr(&p.ctr->err, kErrOutOvf);
        }
        w++;
    };
    while (ma) {
        const uint32_t bit = __ffs(ma) - 1;
        ma &= ma - 1;
        put(pa(bit));
    }
    while (mb) {
        const uint32_t bit = __ffs(mb) - 1;
        mb &= mb - 1;
        put(pb(bit));
    }
}

// block-buffer record step (the words of a warp step go to the block buffer
// or, when it is full, straight to global memory)
template <class LA, class LB>
__device__ __forceinline__ void bremit(const Params& p, BlockSmem& s, uint32_t ma, LA la, uint32_t mb, LB lb,
                                       uint32_t row, uint32_t gid) {
    const uint32_t lane = lane_id();
    const uint32_t wa = rec_words(__popc(ma)), wb = rec_words(__popc(mb));
    const uint32_t any = __ballot_sync(FULL_MASK, (wa | wb) != 0u);
    const bool hdr = any != 0u && lane == (uint32_t)(__ffs(any) - 1);
    const uint32_t k = wa + wb + (hdr ? 2u : 0u);
    const uint32_t incl = warp_incl_scan(k);
    const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
    if (total == 0) return;
    const unsigned long long hits = warp_sum_u64(__popc(ma) + __popc(mb));
    uint32_t pos = 0;
    unsigned long long gbase = 0;
    if (lane == 0) {
        atomicAdd(&s.hits, hits);
        pos = atomicAdd(&s.out_n, total);
        if (pos + total > kBlockOut) {
            atomicMin(&s.first_ovf, pos);
            gbase = atomicAdd(&p.ctr->pairs, (unsigned long long)total);
        }
    }
    pos = __shfl_sync(FULL_MASK, pos, 0);
    gbase = __shfl_sync(FULL_MASK, gbase, 0);
    const bool direct = pos + total > kBlockOut;
    const bool keep = !direct || gbase + total <= p.out_cap;
    if (direct && !keep && lane == 0) atomicOr(&p.ctr->err, kErrOutOvf);
    unsigned long long* dst = direct ? reinterpret_cast<unsigned long long*>(p.out) + gbase
                                     : reinterpret_cast<unsigned long long*>(s.out + pos);
    uint32_t w = incl - k;
    if (hdr && keep) {
        dst[w] = kRiceUnused;
        dst[w + 1] = gid;
    }
    if (hdr) w += 2;
    if (wa) rec_write(dst + w, keep, row, ma, la);
    if (wb) rec_write(dst + w + wa, keep, row, mb, lb);
}

template <int D, bool BIP, bool NARROW, bool REC, bool FRESH = false, bool SUB = false>
__device__ void big_task(const Params& p, BlockSmem& s, uint64_t task) {
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const Slots sl{s.a, s.b};
    auto emit = [&](uint32_t ma, auto pa, uint32_t mb, auto pb, uint32_t myid) { bemit<BIP>(p, s, ma, pa, mb, pb, myid); };
    const uint64_t nl = mn64(ctr_read<FRESH>(&p.ctr->n_list[kListBig]), p.list_cap[kListBig]);
    uint64_t cur = task * kBigCellsPerTask;
    const uint64_t end = mn64(cur + kBigCellsPerTask, nl);
    while (cur < end) {
        if (warp == 0) {
            uint32_t n = 0, st = 0;
            const bool v = lane < kBigCellsPerTask && cur + lane < end;
            uint32_t gid = 0;
            if (v) {
                const uint2 sn = p.lists[p.list_off[kListBig] + cur + lane];
                st = sn.x;
                n = sn.y;
                if (REC) {  // the list holds the cell id; its start is in the counters
                    gid = sn.x;
                    st = gid < p.ncells ? p.counts[gid] : 0xffffffffu;
                }
                if (n > kBigMax || (uint64_t)st + n > p.entry_cap) n = 0;  // inconsistent grid: skip
            }
            const uint32_t n8 = (n + 7) & ~7u;
            const uint32_t inc = warp_incl_scan(n8);
            const uint32_t fits = __ballot_sync(FULL_MASK, v && inc <= kBlockSlots);
            const uint32_t k = __popc(fits);  // fits is a run of low bits
            const uint32_t units = lane < k ? (n + 31) >> 5 : 0u;
            const uint32_t uinc = warp_incl_scan(units);
            if (lane < k) {
                s.cell_start[lane] = st;
                s.cell_gid[lane] = gid;
                s.cell_n[lane] = n;
                s.cell_off[lane] = inc - n8;
                s.unit_pref[lane + 1] = uinc;
            }
            if (lane == 0) {
                s.unit_pref[0] = 0;
                if (k == 0) s.k = s.tot = s.units = 0;
            }
            if (k > 0 && lane == k - 1) {
                s.cell_off[k] = inc;
                s.k = k;
                s.tot = inc;
                s.units = uinc;
            }
        }
        block_sync<SUB>();
        const uint32_t K = s.k, tot = s.tot, U = s.units;
        if (K == 0) break;  // uniform: every thread read the same K
        for (uint32_t e = t; e < tot; e += kPairThreads) {
            uint32_t c = 0;  // last cell whose slots start at or before e
#pragma unroll
            for (uint32_t step = 4; step; step >>= 1)
                if (c + step < K && s.cell_off[c + step] <= e) c += step;
            const uint32_t local = e - s.cell_off[c];
            slot_put(sl, e, local < s.cell_n[c] ? load_box<D, NARROW>(p, p.entries[s.cell_start[c] + local])
                                                : dummy_box<NARROW>());
        }
        block_sync<SUB>();
        for (uint32_t u = warp; u < U; u += kPairWarps) {
            uint32_t c = 0;
#pragma unroll
            for (uint32_t step = 4; step; step >>= 1)
                if (c + step < K && s.unit_pref[c + step] <= u) c += step;
            if constexpr (REC) {
                const uint32_t gid = s.cell_gid[c];
                auto remit_b = [&](uint32_t ma, auto la, uint32_t mb, auto lb, uint32_t row) {
                    bremit(p, s, ma, la, mb, lb, row, gid);
                };
                row_unit<D, BIP, NARROW, true>(p, sl, s.cell_off[c], s.cell_n[c], u - s.unit_pref[c], remit_b);
            } else {
                row_unit<D, BIP, NARROW, false>(p, sl, s.cell_off[c], s.cell_n[c], u - s.unit_pref[c], emit);
            }
        }
        block_sync<SUB>();
        cur += K;
    }
}

// huge cells: one tile task {start, n, r, x0} per warp; boxes gathered per
// tile into the warp's 64 slots (32 rows, 32 columns)
template <int D, bool BIP, bool NARROW, bool REC, bool FRESH = false>
__device__ __forceinline__ void huge_item(const Params& p, BlockSmem& s, uint64_t item, uint32_t slot0) {
    const uint32_t lane = lane_id();
    const Slots sl{s.a, s.b};
    const uint64_t nt = mn64(ctr_read<FRESH>(&p.ctr->need_tasks), p.task_cap);
    if (item >= nt) return;
    const uint4 tk = p.tasks[item];
    const uint32_t gid = tk.x;  // record mode: the cell id; its start is in the counters
    const uint32_t start = REC ? (gid < p.ncells ? p.counts[gid] : 0xffffffffu) : tk.x;
    const uint32_t n = tk.y, r = tk.z, x0 = tk.w;
    if (REC && n >= 65536u) {  // beyond the record format (u8 row tile)
        if (lane == 0) atomicOr(&p.ctr->err, kErrRecCell);
        return;
    }
    const uint32_t R = (n + 31) >> 5;
    const uint32_t x1 = min(x0 + kTaskCols, R);
    if ((uint64_t)start + n > p.entry_cap || r >= R || x0 >= R) return;
    const uint32_t rows = min(32u, n - 32 * r);
    const Box me = lane < rows ? load_box<D, NARROW>(p, p.entries[start + 32 * r + lane]) : dummy_box<NARROW>();
    slot_put(sl, slot0 + lane, me);
    __syncwarp();
    for (uint32_t x = x0; x < x1; x++) {
        if (x == r) {
            const uint32_t md = sweep_diag<D, BIP, NARROW>(sl, me, lane, slot0, rows, p.split);
            if constexpr (REC) {
                auto ld = [&](uint32_t d) {
                    uint32_t pr = lane + d;
                    if (pr >= rows) pr -= rows;
                    return 32 * r + pr;
                };
                bremit(p, s, md, ld, 0u, ld, 32 * r + lane, gid);
            } else {
                auto pd = [&](uint32_t d) {
                    uint32_t pr = lane + d;
                    if (pr >= rows) pr -= rows;
                    return slot_id(sl, slot0 + pr);
                };
                bemit<BIP>(p, s, md, pd, 0u, pd, me.id);
            }
        } else {
            const uint32_t cols = min(32u, n - 32 * x);
            slot_put(sl, slot0 + 32 + lane,
                     lane < cols ? load_box<D, NARROW>(p, p.entries[start + 32 * x + lane]) : dummy_box<NARROW>());
            __syncwarp();
            const uint32_t mc = sweep_cols<D, BIP, NARROW>(sl, me, slot0 + 32, (cols + 7) & ~7u, p.split);
            if constexpr (REC) {
                auto lc = [&](uint32_t j) { return 32 * x + j; };
                bremit(p, s, mc, lc, 0u, lc, 32 * r + lane, gid);
            } else {
                auto pc = [&](uint32_t j) { return slot_id(sl, slot0 + 32 + j); };
                bemit<BIP>(p, s, mc, pc, 0u, pc, me.id);
            }
        }
        __syncwarp();
    }
}

// big-cell tasks and huge-cell tile tasks, block blk of nblk (SUB: run by
// the block's first kPairThreads threads alone)
template <int D, bool BIP, bool NARROW, bool REC, bool FRESH = false, bool SUB = false>
__device__ __forceinline__ void block_pass(const Params& p, BlockSmem& s, uint64_t blk, uint64_t nblk) {
    const uint32_t t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        s.out_n = 0;
        s.first_ovf = kBlockOut;
        s.hits = 0;
        const uint64_t nb = mn64(ctr_read<FRESH>(&p.ctr->n_list[kListBig]), p.list_cap[kListBig]);
        const uint64_t nt = mn64(ctr_read<FRESH>(&p.ctr->need_tasks), p.task_cap);
        s.nbt[0] = (nb + kBigCellsPerTask - 1) / kBigCellsPerTask;
        s.nbt[1] = (nt + kPairWarps - 1) / kPairWarps;
    }
    block_sync<SUB>();
    const uint64_t total = s.nbt[0] + s.nbt[1];
    for (uint64_t bt = blk; bt < total; bt += nblk) {
        if (bt < s.nbt[0]) big_task<D, BIP, NARROW, REC, FRESH, SUB>(p, s, bt);
        else huge_item<D, BIP, NARROW, REC, FRESH>(p, s, (bt - s.nbt[0]) * kPairWarps + warp, warp * 64);
        block_sync<SUB>();
        const uint32_t on = s.out_n, ovf = s.first_ovf;
        const uint32_t nv = min(on, ovf);
        const bool last = bt + nblk >= total;
        if (nv >= kBlockOut / 2 || on > nv || (last && on > 0)) {
            if (t == 0) s.gbase = nv ? atomicAdd(&p.ctr->pairs, (unsigned long long)nv) : 0ull;
            block_sync<SUB>();
            store_run(p, s.gbase, s.out, nv, t, kPairThreads);
            block_sync<SUB>();
            if (t == 0) {
                s.out_n = 0;
                s.first_ovf = kBlockOut;
            }
            block_sync<SUB>();
        }
    }
    if (REC && t == 0 && s.hits) atomicAdd(&p.ctr->rec_pairs, s.hits);
}

template <int D, bool BIP, bool NARROW, bool REC = false>
__global__ void __launch_bounds__(kPairThreads, 2) k_pairs_block(Params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    block_pass<D, BIP, NARROW, REC>(p, *reinterpret_cast<BlockSmem*>(smem_raw), blockIdx.x, gridDim.x);
}

// record mode, after the pair kernels: entries become the plain box indices
// the record decoder reads (the reference's Recs array)
__global__ void k_strip_entries(Params pin) {
    const Params p = resolve(pin);
    const uint64_t n = mn64(p.ctr->entries, p.entry_cap);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p.entries[i] &= kIdMask;
}

// ---------------------------------------------------------------------------
// group pairs by scene (batched queries): a pair's scene is the scene of its
// first box; pairs are written to their scene's range with scene-local ids.
// ---------------------------------------------------------------------------
// lanes of a warp holding pairs of the same scene share one atomic (pairs
// come out of the pair kernels in runs of one scene)
__device__ __forceinline__ unsigned long long warp_scene_reserve(unsigned long long* ctr, uint32_t sc, bool valid,
                                                                  uint32_t& rank) {
    const uint32_t lane = lane_id();
    const uint32_t key = valid ? sc : 0xffffffffu;
    const uint32_t same = __match_any_sync(FULL_MASK, key);
    const uint32_t leader = __ffs(same) - 1;
    rank = __popc(same & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (valid && lane == leader) base = atomicAdd(&ctr[sc], (unsigned long long)__popc(same));
    return __shfl_sync(FULL_MASK, base, leader);
}

__global__ void k_group_by_scene(Params pin, const unsigned long long* scene_pair_off,
                                 unsigned long long* scene_cursor, uint2* dst, unsigned long long n) {
    const Params p = resolve(pin);
    n = mn64(p.ctr->pairs, p.out_cap);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long n32 = (n + 31) & ~31ull;  // whole warps iterate together
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n32; i += stride) {
        const bool valid = i < n;
        const uint2 pr = valid ? p.out[i] : make_uint2(0u, 0u);
        const uint32_t sc = valid ? find_scene(p, pr.x) : 0u;
        uint32_t rank;
        const unsigned long long base = warp_scene_reserve(scene_cursor, sc, valid, rank);
        if (valid) {
            const uint32_t off = p.scene_box_off[sc];
            dst[scene_pair_off[sc] + base + rank] = make_uint2(pr.x - off, pr.y - off);
        }
    }
}

__global__ void k_scene_hist(Params pin, unsigned long long* hist, unsigned long long n) {
    const Params p = resolve(pin);
    n = mn64(p.ctr->pairs, p.out_cap);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long n32 = (n + 31) & ~31ull;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n32; i += stride) {
        const bool valid = i < n;
        const uint32_t sc = valid ? find_scene(p, p.out[i].x) : 0u;
        uint32_t rank;
        warp_scene_reserve(hist, sc, valid, rank);
    }
}

// exclusive scan of the per-scene pair counts: off[s] = sum of hist[< s],
// off[nscenes] = total; one block, 1024 threads, chunks of 1024 scenes
__global__ void __launch_bounds__(1024) k_scene_offsets(Params pin, const unsigned long long* hist,
                                                        unsigned long long* off) {
    const Params p = resolve(pin);
    __shared__ unsigned long long s_w[32];
    __shared__ unsigned long long s_carry;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    if (t == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 <= p.nscenes; c0 += 1024) {
        const uint32_t i = c0 + t;
        const unsigned long long v = i < p.nscenes ? hist[i] : 0ull;
        unsigned long long x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(FULL_MASK, w, o);
                if (lane >= (uint32_t)o) w += y;
            }
            s_w[lane] = w;
        }
        __syncthreads();
        const unsigned long long incl = x + (warp ? s_w[warp - 1] : 0ull) + s_carry;
        if (i <= p.nscenes) off[i] = incl - v;
        __syncthreads();
        if (t == 1023) s_carry = incl;
        __syncthreads();
    }
}


// ---------------------------------------------------------------------------
// one-launch queries of small scenes: a cooperative launch whose blocks run
// the whole pipeline, phase after phase, separated by grid barriers
//   P0   every block: the cell size (warp 0 runs the tuner's model on 64
//        sampled boxes: the same choice in every block) and the scene in
//        shared memory; block 0 the chosen grid for the host and the next
//        launch's zeroed run counters; the counters are zeroed first only
//        when they may hold anything else (one more barrier)
//   P1   count
//   P2   entry totals of chunks -- a small grid's (128-cell chunks)
//        computed by every block itself, a larger one's (512-cell chunks) by
//        all blocks (one more barrier) -- then the chunk prefixes in shared
//        memory, and each warp's chunks' cell ends, work lists, statistics;
//        a small grid's cell ends go to a buffer of their own, since other
//        blocks may still be reading the counters
//   P3   expand and scatter
//   P4   small, medium and block pair passes; the grid's counters zeroed for
//        the next launch; the last block to finish copies the run counters
//        to the host
// Data written in one phase and read in a later one is read past L1. A
// barrier's wait is bounded: a block that gives up sets kErrWait and leaves,
// and the others give up at their next barrier.
// ---------------------------------------------------------------------------
constexpr uint32_t kFusedThreads = 2 * kPairThreads;
constexpr uint32_t kFusedWarps = kFusedThreads / 32;
constexpr uint32_t kFusedChunks = (uint32_t)(kFusedMaxCells / kScanChunk);
constexpr uint32_t kFusedLocalCells = 8192;  // grids of up to 8192 cells: 128-cell chunks, totals per block
constexpr uint32_t kGridWaitLimit = 1u << 20;  // polls of 64 ns or more: the wait ends after a second at most
constexpr uint32_t kSmallWarpBytes = 2 * kSmallSlots * sizeof(uint4) + kWarpOut * sizeof(uint2);
static_assert(kFusedChunks % kFusedThreads == 0, "chunk prefixes per thread");
static_assert(2 * kMedSlots * sizeof(uint2) <= kMedSlots * sizeof(uint4), "medium-cell z terms and {f, id} in the b array");
static_assert(kSmallSlots * sizeof(uint2) + kSmallSlots * sizeof(uint32_t) <= kSmallSlots * sizeof(uint4), "small-cell z terms and indices in the b array");

// barrier number k of this launch (k counts the barriers passed so far)
__device__ __forceinline__ bool grid_barrier(const FusedArgs& a, uint32_t k) {
    __shared__ uint32_t s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.add.u32 [%0], 1;" ::"l"(a.bar) : "memory");
        const uint32_t target = (k + 1) * gridDim.x;
        uint32_t ok = 0;
        for (uint32_t i = 0; i < kGridWaitLimit; i++) {
            uint32_t v;
            asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(a.bar) : "memory");
            if ((int32_t)(v - a.bar_base) >= (int32_t)target) {
                ok = 1;
                break;
            }
            if (i >= 64) __nanosleep(64);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0u;
}

// the tuner's model (k_tune_scenes) for one scene of n boxes at row 0, in
// single precision over exact integer sums: the one-launch path cannot wait
// for double-precision divisions. Grids of at most max_cells cells, so a
// box covers at most max_cells cells and every per-box product fits 32 bits.
__device__ __forceinline__ uint32_t tune_scene_fast(const uint32_t* boxes, uint64_t n, int dims, uint32_t range,
                                                    uint64_t max_cells) {
    const uint32_t lane = lane_id();
    const uint32_t W = 2 * (uint32_t)dims + 1;
    const uint64_t m = n < kTuneRows ? n : kTuneRows;
    uint32_t lo[2][3] = {{0, 0, 0}, {0, 0, 0}}, hi[2][3] = {{0, 0, 0}, {0, 0, 0}};
    bool ok[2] = {false, false};
    unsigned long long ext = 0, good = 0;
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const uint64_t k = lane + 32u * j;
        if (k >= m) continue;
        const uint32_t* b = boxes + (k * n / m) * W;
        bool v = true;
        for (int d = 0; d < dims; d++) {
            lo[j][d] = __ldg(b + 2 * d);
            hi[j][d] = __ldg(b + 2 * d + 1);
            v = v && lo[j][d] <= hi[j][d] && hi[j][d] < range;
        }
        ok[j] = v;
        if (v) {
            for (int d = 0; d < dims; d++) ext += (unsigned long long)(hi[j][d] - lo[j][d]) + 1;
            good++;
        }
    }
    ext = warp_sum_u64(ext);
    good = warp_sum_u64(good);
    // s0 = floor(log2(mean extent)), 0 below 2
    const unsigned long long mean = ext / ((good ? good : 1ull) * (unsigned long long)dims);
    const int s0 = mean < 2 ? 0 : 63 - __clzll(mean);
    const int s_win = s0 + 3 < 31 ? s0 + 3 : 31;
    const float scale = (float)n / (float)(m ? m : 1);
    const uint64_t far_cap = n * 64 > 4096 ? n * 64 : 4096;
    float best_cost = 3.0e38f;
    uint32_t best = 0xffffffffu;
    for (int s = s0 - 2 > 0 ? s0 - 2 : 0; s <= 31 && m > 0; s++) {
        if (s == s_win + 1 && best != 0xffffffffu) break;
        const uint64_t nrc = nrc_dev(range, s);
        if (nrc > max_cells) continue;
        const uint64_t C = dims == 3 ? nrc * nrc * nrc : nrc * nrc;  // nrc <= 2^20: no overflow in 64 bits
        if (C > max_cells) continue;
        if (s > s_win && C > far_cap) continue;
        uint32_t e = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            if (!ok[j]) continue;
            uint32_t c = 1;
            for (int d = 0; d < dims; d++) c *= (hi[j][d] >> s) - (lo[j][d] >> s) + 1;
            e += c;  // <= 2 * max_cells
        }
        e = __reduce_add_sync(FULL_MASK, e);
        if (e > 64u * (uint32_t)m) continue;
        const float E = (float)e * scale, Cf = (float)C;
        const float T = E * E / (2.0f * Cf);
        const float occ = 2.0f * T / (E > 1.0f ? E : 1.0f) + 1.0f;
        const float f = occ / (float)kTuneOcc > 1.0f ? occ / (float)kTuneOcc : 1.0f;
        const float cost = (float)kTuneCell * Cf + (float)kTuneEntry * E + (float)kTuneTest * f * T;
        if (cost < best_cost) {
            best_cost = cost;
            best = (uint32_t)s;
        }
    }
    if (best == 0xffffffffu) {  // the coarsest grid that is not a single cell
        uint32_t s = 31;
        while (s > 0 && nrc_dev(range, (int)s - 1) <= 1) s--;
        best = s;
    }
    return best;
}

template <int D, bool NARROW>
__global__ void __launch_bounds__(kFusedThreads, 1) k_fused(Params pin, FusedArgs a) {
    Params p = pin;  // the grid's size is set below
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_shift;
    __shared__ Scene s_scene;
    __shared__ unsigned long long s_wsum[kFusedWarps];
    __shared__ uint32_t s_csum[kFusedLocalCells / 128];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint64_t blk = blockIdx.x, nblk = gridDim.x;
    const uint64_t gw = blk * kFusedWarps + warp, nw = nblk * kFusedWarps;
    const uint64_t gt = blk * kFusedThreads + t, nt = nblk * kFusedThreads;
    const uint32_t range = p.max_range;
    uint32_t nbar = 0;
    if (blk == 0 && t == 0) {
        unsigned long long now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        p.ctr->t_start = now;
    }
#define FUSED_BARRIER()                                        \
    if (!grid_barrier(a, nbar++)) {                            \
        if (t == 0) atomicOr(&p.ctr->err, (unsigned)kErrWait); \
        return;                                                \
    }
    // P0
    if (warp == 0) {
        uint32_t sh = a.shift;
        if (sh == kFusedTune) sh = tune_scene_fast(p.boxes, p.nboxes, D, range, kFusedMaxCells);
        if (lane == 0) s_shift = sh;
    }
    __syncthreads();
    const uint32_t shift = s_shift, nrc = nrc_dev(range, (int)shift);
    p.ncells = D == 3 ? (uint64_t)nrc * nrc * nrc : (uint64_t)nrc * nrc;
    if (t == 0) s_scene = Scene{0u, (uint32_t)p.nboxes, shift, nrc, 0ull, range, 0u};
    if (blk == 0 && t == 0) {
        *a.ctr_next = Ctr{};
        p.ctr->cells = p.ncells;
        p.ctr->shift = shift;
        a.scenes[0] = Scene{0u, (uint32_t)p.nboxes, shift, nrc, 0ull, range, 0u};
    }
    __syncthreads();
    p.scenes = &s_scene;  // the count and the scatter read the scene from shared memory
    if (a.zero_cells) {
        uint4* c4 = reinterpret_cast<uint4*>(p.counts);
        for (uint64_t i = gt; i < a.zero_cells / 4; i += nt) c4[i] = make_uint4(0u, 0u, 0u, 0u);
        for (uint64_t i = 4 * (a.zero_cells / 4) + gt; i < a.zero_cells; i += nt) p.counts[i] = 0u;
        FUSED_BARRIER()
    }
    // P1: count
    uint32_t* sbox = reinterpret_cast<uint32_t*>(smem_raw);
    box_pass<D, false, false, kFusedThreads>(p, sbox, blk, nblk);
    FUSED_BARRIER()
    // P2: chunk entry totals and prefixes, then the cells
    uint32_t* pre = reinterpret_cast<uint32_t*>(smem_raw);
    unsigned long long total = 0;
    bool fits;
    if (p.ncells <= kFusedLocalCells) {
        const uint32_t nch = (uint32_t)((p.ncells + 127) / 128);
        for (uint32_t ch = warp; ch < nch; ch += kFusedWarps) {
            uint32_t v[4];
            scan_load<1, true>(p, ch, v);
            s_csum[ch] = __reduce_add_sync(FULL_MASK, v[0] + v[1] + v[2] + v[3]);  // < 2^32 (at most 2^25)
        }
        __syncthreads();
        if (t == 0) {
            unsigned long long run = 0;
            for (uint32_t ch = 0; ch < nch; ch++) {
                pre[ch] = (uint32_t)run;  // < entry_cap when it is used
                run += s_csum[ch];
            }
            s_wsum[0] = run;
        }
        __syncthreads();
        total = s_wsum[0];
        fits = total <= p.entry_cap;
        if (fits) {
            // the cell ends go to a buffer of their own: other blocks may
            // still be summing the counters
            Params pe = p;
            pe.counts = a.ends;
            ScanStats ws;
            const uint64_t full = p.ncells / 128;
            for (uint64_t ch = gw; ch < nch; ch += nw) {
                uint32_t v[4];
                scan_load<1, true>(p, ch, v);
                scan_chunk<1>(pe, pin, ch, ch < full, v, pre[ch], ws);
            }
            scan_stats_flush(p, ws);
        }
    } else {
        const uint64_t nch = (p.ncells + kScanChunk - 1) / kScanChunk;
        for (uint64_t ch = gw; ch < nch; ch += nw) {
            uint32_t v[kScanPerThread];
            scan_load<4, true>(p, ch, v);
            uint32_t sum = 0;  // < 2^32: a chunk holds at most 512 cells of at most kFusedMaxBoxes entries
#pragma unroll
            for (int k = 0; k < kScanPerThread; k++) sum += v[k];
            sum = __reduce_add_sync(FULL_MASK, sum);
            if (lane == 0) a.chunk_sum[ch] = sum;
        }
        FUSED_BARRIER()
        constexpr uint32_t kPer = kFusedChunks / kFusedThreads;
        uint32_t x[kPer];
        unsigned long long sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint64_t i = (uint64_t)t * kPer + k;
            x[k] = i < nch ? __ldcg(a.chunk_sum + i) : 0u;
            sum += x[k];
        }
        const unsigned long long incl = warp_incl_scan64(sum);
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        unsigned long long run = incl - sum;
#pragma unroll
        for (uint32_t w = 0; w < kFusedWarps; w++) {
            if (w < warp) run += s_wsum[w];
            total += s_wsum[w];
        }
#pragma unroll
        for (uint32_t k = 0; k < kPer; k++) {
            const uint64_t i = (uint64_t)t * kPer + k;
            if (i < nch) pre[i] = (uint32_t)run;  // < entry_cap when it is used
            run += x[k];
        }
        __syncthreads();
        fits = total <= p.entry_cap;
        if (fits) {
            ScanStats ws;
            const uint64_t full = p.ncells / kScanChunk;
            for (uint64_t ch = gw; ch < nch; ch += nw) {
                uint32_t v[kScanPerThread];
                scan_load<4, true>(p, ch, v);
                scan_chunk(p, pin, ch, ch < full, v, pre[ch], ws);
            }
            scan_stats_flush(p, ws);
        }
    }
    if (blk == 0 && t == 0) {
        p.ctr->entries = total;
        if (!fits) atomicOr(&p.ctr->err, (unsigned)kErrEntryOvf);
    }
    FUSED_BARRIER()
    // P3: tile tasks of huge cells, scatter (against the cell ends)
    if (fits) {
        expand_cells<true>(p, (uint32_t)gt, (uint32_t)nt);
        Params pe = p;
        if (p.ncells <= kFusedLocalCells) pe.counts = a.ends;
        box_pass<D, true, false, kFusedThreads>(pe, sbox, blk, nblk);
    }
    FUSED_BARRIER()
#undef FUSED_BARRIER
    // P4: the counters zeroed for the next launch (the pair passes read the
    // work lists, not the counters), then the pairs
    {
        uint4* c4 = reinterpret_cast<uint4*>(p.counts);
        for (uint64_t i = gt; i < p.ncells / 4; i += nt) c4[i] = make_uint4(0u, 0u, 0u, 0u);
        for (uint64_t i = 4 * (p.ncells / 4) + gt; i < p.ncells; i += nt) p.counts[i] = 0u;
    }
    if (fits) {
        unsigned char* ws = smem_raw + warp * kSmallWarpBytes;
        uint4* sa = reinterpret_cast<uint4*>(ws);
        small_pass<D, false, NARROW, false, true>(p, sa, sa + kSmallSlots, reinterpret_cast<uint2*>(sa + 2 * kSmallSlots),
                                            gw, nw);
        __syncthreads();
        med_pass<D, false, NARROW, false, true>(p, smem_raw + warp * kMedWarpBytes, gw, nw);
        __syncthreads();
        if (t < kPairThreads)  // (the block pass is laid out for kPairThreads threads)
            block_pass<D, false, NARROW, false, true, true>(p, *reinterpret_cast<BlockSmem*>(smem_raw), blk, nblk);
    }
    // the last block to finish copies the run counters to the host (one
    // more arrival per block on the barriers' count)
    __syncthreads();
    if (t == 0) {
        __threadfence();
        uint32_t old;
        asm volatile("atom.acq_rel.gpu.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(a.bar) : "memory");
        if ((int32_t)(old - a.bar_base) == (int32_t)((nbar + 1) * nblk - 1)) {
            __threadfence();
            constexpr uint32_t kWords = sizeof(Ctr) / sizeof(unsigned long long);
            static_assert(sizeof(Ctr) % sizeof(unsigned long long) == 0, "run counters in 8-byte words");
            const unsigned long long* src = reinterpret_cast<const unsigned long long*>(p.ctr);
            unsigned long long w[kWords];
#pragma unroll
            for (uint32_t k = 0; k < kWords; k++) w[k] = __ldcg(src + k);
            Ctr* h = a.ctr_host;
            unsigned long long* dst = reinterpret_cast<unsigned long long*>(h);
#pragma unroll
            for (uint32_t k = 0; k < kWords; k++) dst[k] = w[k];
            h->barriers = nbar + 1;
            unsigned long long now;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
            h->t_end = now;
            __threadfence_system();
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int g_blocks_small = 1, g_blocks_med = 1, g_blocks_block = 1;
static int g_sm_count = 0;

static size_t med_smem() { return (size_t)kPairWarps * kMedWarpBytes; }

size_t pair_smem_bytes() { return sizeof(BlockSmem); }

template <int D, bool B, bool N, bool R = false>
static cudaError_t init_variant() {
    cudaError_t e = cudaFuncSetAttribute(k_pairs_med<D, B, N, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)med_smem());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_pairs_block<D, B, N, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BlockSmem));
    return e;
}

static int g_fused_blocks = 0;

static size_t fused_smem() {
    size_t b = (size_t)kFusedWarps * kMedWarpBytes;
    b = b > sizeof(BlockSmem) ? b : sizeof(BlockSmem);
    b = b > (size_t)kFusedWarps * kSmallWarpBytes ? b : (size_t)kFusedWarps * kSmallWarpBytes;
    b = b > (size_t)kFusedChunks * 4 ? b : (size_t)kFusedChunks * 4;
    b = b > (size_t)kFusedThreads * 7 * 4 ? b : (size_t)kFusedThreads * 7 * 4;
    return b;
}

int fused_blocks() { return g_fused_blocks; }

template <int D, bool N>
static cudaError_t launch_fused_t(const Params& p, const FusedArgs& a, cudaStream_t st) {
    Params pp = p;
    FusedArgs aa = a;
    void* args[] = {&pp, &aa};
    return cudaLaunchCooperativeKernel((const void*)k_fused<D, N>, dim3((unsigned)g_fused_blocks), dim3(kFusedThreads),
                                      args, fused_smem(), st);
}

cudaError_t launch_fused(const Params& p, const FusedArgs& a, int dims, cudaStream_t st) {
    if (g_fused_blocks <= 0) return cudaErrorNotSupported;
    const bool narrow = p.max_range <= (1u << kMissShift);
    if (narrow) return dims == 2 ? launch_fused_t<2, true>(p, a, st) : launch_fused_t<3, true>(p, a, st);
    return dims == 2 ? launch_fused_t<2, false>(p, a, st) : launch_fused_t<3, false>(p, a, st);
}

template <int D, bool N>
static cudaError_t init_fused() {
    return cudaFuncSetAttribute(k_fused<D, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_smem());
}

cudaError_t kernels_init() {
    cudaError_t e;
    {
        int dev = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    }
    if ((e = init_variant<2, false, true>()) != cudaSuccess) return e;
    if ((e = init_variant<3, false, true>()) != cudaSuccess) return e;
    if ((e = init_variant<2, true, true>()) != cudaSuccess) return e;
    if ((e = init_variant<3, true, true>()) != cudaSuccess) return e;
    if ((e = init_variant<2, false, false>()) != cudaSuccess) return e;
    if ((e = init_variant<3, false, false>()) != cudaSuccess) return e;
    if ((e = init_variant<2, true, false>()) != cudaSuccess) return e;
    if ((e = init_variant<3, true, false>()) != cudaSuccess) return e;
    if ((e = init_variant<2, false, true, true>()) != cudaSuccess) return e;
    if ((e = init_variant<3, false, true, true>()) != cudaSuccess) return e;
    if ((e = init_variant<2, false, false, true>()) != cudaSuccess) return e;
    if ((e = init_variant<3, false, false, true>()) != cudaSuccess) return e;
    int nb = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pairs_small<3, false, true>, kPairThreads, 0)) != cudaSuccess) return e;
    g_blocks_small = nb > 0 ? nb : 1;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pairs_med<3, false, true>, kPairThreads, med_smem())) != cudaSuccess) return e;
    g_blocks_med = nb > 0 ? nb : 1;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_pairs_block<3, false, true>, kPairThreads, sizeof(BlockSmem))) != cudaSuccess) return e;
    g_blocks_block = nb > 0 ? nb : 1;
    // one-launch queries: one block per SM, all resident (cooperative launch)
    if ((e = init_fused<2, true>()) != cudaSuccess) return e;
    if ((e = init_fused<3, true>()) != cudaSuccess) return e;
    if ((e = init_fused<2, false>()) != cudaSuccess) return e;
    if ((e = init_fused<3, false>()) != cudaSuccess) return e;
    {
        int dev = 0, coop = 0, nf = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nf, k_fused<3, true>, kFusedThreads, fused_smem())) !=
            cudaSuccess)
            return e;
        g_fused_blocks = coop && nf >= 1 ? g_sm_count : 0;
    }
    return cudaSuccess;
}

cudaError_t launch_scene_hist(const Params& p, unsigned long long* hist, cudaStream_t st) {
    // the pair count is read on the device
    k_scene_hist<<<(unsigned)((g_sm_count > 0 ? g_sm_count : 152) * 8), 256, 0, st>>>(p, hist, 0);
    return cudaGetLastError();
}

uint64_t scan_tiles(uint64_t ncells) { return (ncells + kScanTile - 1) / kScanTile; }

uint64_t scene_table_entries(uint64_t nboxes) { return (nboxes >> kSceneTableShift) + 2; }

cudaError_t launch_scene_table(const Params& p, cudaStream_t st) {
    const uint64_t n = scene_table_entries(p.nboxes);
    const uint64_t cap = (uint64_t)(g_sm_count > 0 ? g_sm_count : 152) * 4;
    const uint64_t g = (n + 255) / 256;
    k_scene_table<<<(unsigned)(g < cap ? g : cap), 256, 0, st>>>(p);
    return cudaGetLastError();
}

static unsigned box_grid(uint64_t nboxes) {
    const uint64_t nb = (nboxes + kBoxThreads - 1) / kBoxThreads;
    const uint64_t cap = (uint64_t)(g_sm_count > 0 ? g_sm_count : 152) * 8;
    return (unsigned)(nb < cap ? nb : cap);
}

cudaError_t launch_count(const Params& p, int dims, cudaStream_t st) {
    k_zero_counts<<<(unsigned)((g_sm_count > 0 ? g_sm_count : 152) * 4), 512, 0, st>>>(p);
    const unsigned g = box_grid(p.nboxes);
    if (g == 0) return cudaSuccess;
    if (p.merged) {
        if (dims == 2) k_count<2, true><<<g, kBoxThreads, 0, st>>>(p);
        else k_count<3, true><<<g, kBoxThreads, 0, st>>>(p);
    } else {
        if (dims == 2) k_count<2, false><<<g, kBoxThreads, 0, st>>>(p);
        else k_count<3, false><<<g, kBoxThreads, 0, st>>>(p);
    }
    return cudaGetLastError();
}

cudaError_t launch_scatter(const Params& p, int dims, cudaStream_t st) {
    const unsigned g = box_grid(p.nboxes);
    if (g == 0) return cudaSuccess;
    if (p.merged) {
        if (dims == 2) k_scatter<2, true><<<g, kBoxThreads, 0, st>>>(p);
        else k_scatter<3, true><<<g, kBoxThreads, 0, st>>>(p);
    } else {
        if (dims == 2) k_scatter<2, false><<<g, kBoxThreads, 0, st>>>(p);
        else k_scatter<3, false><<<g, kBoxThreads, 0, st>>>(p);
    }
    return cudaGetLastError();
}

cudaError_t launch_scan(const Params& p, cudaStream_t st) {
    const uint64_t chunks = (p.ncells + kScanChunk - 1) / kScanChunk;
    const uint64_t blocks = (chunks + kScanThreads / 32 - 1) / (kScanThreads / 32);
    const uint64_t sms = (uint64_t)(g_sm_count > 0 ? g_sm_count : 152);
    const uint64_t cap = sms * 4;  // resident: 4 blocks per SM
    const unsigned g = (unsigned)(blocks < cap ? (blocks ? blocks : 1) : cap);
    // reduce: two chunks per warp item, 4 resident blocks per SM
    const uint64_t rblocks = (chunks + 2 * (kReduceThreads / 32) - 1) / (2 * (kReduceThreads / 32));
    const unsigned g2 = (unsigned)(rblocks < cap ? (rblocks ? rblocks : 1) : cap);
    cudaError_t e = cudaMemsetAsync(p.tile_state, 0, scan_state_bytes(p.ncells), st);
    if (e != cudaSuccess) return e;
    k_scan_reduce<<<g2, kReduceThreads, 0, st>>>(p);
    k_scan_cells<<<g, kScanThreads, 0, st>>>(p);
    return cudaGetLastError();
}

size_t scan_state_bytes(uint64_t ncells) { return scan_tiles(ncells) * sizeof(TileRec); }

cudaError_t launch_scene_offsets(const Params& p, const unsigned long long* hist, unsigned long long* off,
                                 uint32_t nscenes_cap, cudaStream_t st) {
    (void)nscenes_cap;
    k_scene_offsets<<<1, 1024, 0, st>>>(p, hist, off);
    return cudaGetLastError();
}

cudaError_t launch_tune_scenes(const uint32_t* boxes, const unsigned long long* offs, uint32_t nscenes, int dims,
                               uint32_t range, SceneTune* out, cudaStream_t st) {
    if (nscenes == 0) return cudaSuccess;
    const uint64_t blocks = ((uint64_t)nscenes + 7) / 8;  // 8 warps (scenes) per block
    const uint64_t cap = (uint64_t)(g_sm_count > 0 ? g_sm_count : 152) * 16;
    k_tune_scenes<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(boxes, offs, nscenes, dims, range, out);
    return cudaGetLastError();
}

cudaError_t launch_expand(const Params& p, cudaStream_t st) {
    k_expand<<<64, 256, 0, st>>>(p);
    return cudaGetLastError();
}

template <int D, bool B, bool N, bool R = false>
static cudaError_t launch_pairs_t(const Params& p, int sm_count, cudaStream_t st, cudaEvent_t* ev, unsigned evf,
                                  const PairOverlap* ov) {
    if (ov && !R && ov->side_sms > 0 && ov->side_sms < sm_count) {
        cudaError_t e;
        if ((e = cudaEventRecord(ov->fork, st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(ov->side, ov->fork, 0)) != cudaSuccess) return e;
        k_pairs_small<D, B, N, R><<<ov->side_sms * g_blocks_small, kPairThreads, 0, ov->side>>>(p);
        if (ev) cudaEventRecordWithFlags(ev[0], ov->side, evf);
        k_pairs_block<D, B, N, R><<<ov->side_sms * g_blocks_block, kPairThreads, sizeof(BlockSmem), ov->side>>>(p);
        k_pairs_med<D, B, N, R><<<(sm_count - ov->side_sms) * g_blocks_med, kPairThreads, med_smem(), st>>>(p);
        if (ev) cudaEventRecordWithFlags(ev[1], st, evf);
        if ((e = cudaEventRecord(ov->join, ov->side)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st, ov->join, 0)) != cudaSuccess) return e;
        return cudaGetLastError();
    }
    k_pairs_small<D, B, N, R><<<sm_count * g_blocks_small, kPairThreads, 0, st>>>(p);
    if (ev) cudaEventRecordWithFlags(ev[0], st, evf);
    k_pairs_med<D, B, N, R><<<sm_count * g_blocks_med, kPairThreads, med_smem(), st>>>(p);
    if (ev) cudaEventRecordWithFlags(ev[1], st, evf);
    k_pairs_block<D, B, N, R><<<sm_count * g_blocks_block, kPairThreads, sizeof(BlockSmem), st>>>(p);
    if (R) k_strip_entries<<<(unsigned)(sm_count * 4), 512, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pairs(const Params& p, int dims, int sm_count, cudaStream_t st, cudaEvent_t* ev, unsigned evf,
                         const PairOverlap* ov) {
    const bool bip = p.split != kNoSplit;
    const bool narrow = p.max_range <= (1u << kMissShift);
    if (p.records) {  // record mode: self queries
        if (bip) return cudaErrorInvalidValue;
        if (narrow) return dims == 2 ? launch_pairs_t<2, false, true, true>(p, sm_count, st, ev, evf, ov)
                                     : launch_pairs_t<3, false, true, true>(p, sm_count, st, ev, evf, ov);
        return dims == 2 ? launch_pairs_t<2, false, false, true>(p, sm_count, st, ev, evf, ov)
                         : launch_pairs_t<3, false, false, true>(p, sm_count, st, ev, evf, ov);
    }
    if (narrow) {
        if (dims == 2) return bip ? launch_pairs_t<2, true, true>(p, sm_count, st, ev, evf, ov) : launch_pairs_t<2, false, true>(p, sm_count, st, ev, evf, ov);
        return bip ? launch_pairs_t<3, true, true>(p, sm_count, st, ev, evf, ov) : launch_pairs_t<3, false, true>(p, sm_count, st, ev, evf, ov);
    }
    if (dims == 2) return bip ? launch_pairs_t<2, true, false>(p, sm_count, st, ev, evf, ov) : launch_pairs_t<2, false, false>(p, sm_count, st, ev, evf, ov);
    return bip ? launch_pairs_t<3, true, false>(p, sm_count, st, ev, evf, ov) : launch_pairs_t<3, false, false>(p, sm_count, st, ev, evf, ov);
}

cudaError_t launch_group_by_scene(const Params& p, const unsigned long long* scene_pair_off,
                                  unsigned long long* scene_cursor, uint2* dst, cudaStream_t st) {
    // the pair count is read on the device
    k_group_by_scene<<<(unsigned)((g_sm_count > 0 ? g_sm_count : 152) * 8), 256, 0, st>>>(p, scene_pair_off,
                                                                                          scene_cursor, dst, 0);
    return cudaGetLastError();
}

}  // namespace pbig
