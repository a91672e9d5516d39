// Resident scenes and incremental updates (pbig2_scene_*).
//
// A scene keeps its boxes, a grid and its full pair list on the device. The
// grid gives every cell a capacity above its count (slack), so that moving a
// few boxes re-bins only those boxes: their old entries become tombstones and
// their new entries go into the slack of their new cells. The pairs that
// involve moved boxes are found by testing each moved box against the entries
// of its own cells -- before the move (the pairs it had) and after it (the
// pairs it has) -- with the same closed-interval test and reference-cell rule
// as the full query (src/pbig/pbig.cu:562-603); a pair of two moved boxes is
// reported once, from the box with the smaller index. The full list follows
// as (old list minus every pair touching a moved box) plus the pairs after.
// Every slot of the grid holds the box's coordinates next to its index (32
// bytes), so testing a cell reads it contiguously with no gather, and a new
// entry first takes a tombstone of its cell. A cell whose slack runs out
// rebuilds the grid from the current boxes.
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine.h"

namespace pbig {

constexpr uint32_t kDead = 0xffffffffu;

struct ResCtr {
    unsigned int err;                // kErr* bits
    unsigned int overflow;           // a cell ran out of slack
    unsigned long long out;          // pairs written by a query (may exceed capacity)
    unsigned long long kept;         // pairs kept by the filter
    unsigned long long dead;         // tombstones made by a removal
};

struct ResGrid {
    const uint32_t* boxes;
    uint64_t nboxes;
    uint32_t shift, nrc, range;
    uint64_t ncells;
    uint32_t* start;     // [ncells + 1] capacity region of each cell
    uint32_t* used;      // [ncells] slots used (live entries and tombstones)
    uint4* entries;      // two per slot: {x0, x1, y0, y1}, {z0, z1, start bits << 29 | box index (kDead: free), 0}
    ResCtr* ctr;
};

// slack of a cell of n boxes
__host__ __device__ __forceinline__ uint32_t res_cap(uint32_t n) { return n + (n >> 1) + 4u; }

template <int D>
__device__ __forceinline__ void res_range(const uint32_t* b, uint32_t sh, uint32_t lo[3], uint32_t hi[3]) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
        lo[d] = d < D ? b[2 * d] >> sh : 0u;
        hi[d] = d < D ? b[2 * d + 1] >> sh : 0u;
    }
}

__device__ __forceinline__ uint64_t res_gid(const ResGrid& g, uint32_t i, uint32_t j, uint32_t k) {
    return ((uint64_t)k * g.nrc + j) * g.nrc + i;
}

// one thread per listed box (idx == nullptr: boxes 0..k-1): count its cells
template <int D>
__global__ void k_res_count(ResGrid g, uint32_t* cnt) {
    constexpr int W = 2 * D + 1;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.nboxes; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo[3], hi[3];
        res_range<D>(g.boxes + t * W, g.shift, lo, hi);
        for (uint32_t k = lo[2]; k <= hi[2]; k++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t i = lo[0]; i <= hi[0]; i++) atomicAdd(&cnt[res_gid(g, i, j, k)], 1u);
    }
}

__global__ void k_res_caps(const uint32_t* cnt, uint32_t* cap, uint64_t ncells) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (uint64_t)gridDim.x * blockDim.x)
        cap[c] = res_cap(cnt[c]);
}

// ends (in place of the capacities, after the scan) -> starts; used = 0
__global__ void k_res_starts(const uint32_t* cnt, const uint32_t* ends, ResGrid g) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.ncells; c += (uint64_t)gridDim.x * blockDim.x) {
        g.start[c] = ends[c] - res_cap(cnt[c]);
        g.used[c] = 0;
        if (c == g.ncells - 1) g.start[g.ncells] = ends[c];
    }
}

// the slot pair of a box in one cell
template <int D>
__device__ __forceinline__ void res_slot(const uint32_t* b, uint32_t idw, uint4& e0, uint4& e1) {
    e0 = make_uint4(b[0], b[1], b[2], b[3]);
    e1 = make_uint4(D == 3 ? b[4] : 0u, D == 3 ? b[5] : 0u, idw, 0u);
}

// build: every box (one thread each) appended to its cells
template <int D>
__global__ void k_res_fill(ResGrid g) {
    constexpr int W = 2 * D + 1;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.nboxes; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t* b = g.boxes + t * W;
        uint32_t lo[3], hi[3];
        res_range<D>(b, g.shift, lo, hi);
        for (uint32_t kk = lo[2]; kk <= hi[2]; kk++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t i = lo[0]; i <= hi[0]; i++) {
                    const uint64_t c = res_gid(g, i, j, kk);
                    const uint32_t f = (i == lo[0] ? 1u : 0u) | (j == lo[1] ? 2u : 0u) | (kk == lo[2] ? 4u : 0u);
                    const uint32_t slot = atomicAdd(&g.used[c], 1u);
                    if (slot < g.start[c + 1] - g.start[c]) {
                        uint4 e0, e1;
                        res_slot<D>(b, (f << kIdBits) | (uint32_t)t, e0, e1);
                        g.entries[2 * (uint64_t)(g.start[c] + slot)] = e0;
                        g.entries[2 * (uint64_t)(g.start[c] + slot) + 1] = e1;
                    } else {
                        atomicOr(&g.ctr->overflow, 1u);
                    }
                }
    }
}

// moves: one warp per listed box; in each of its cells it takes a tombstone
// (claimed with a compare-and-swap on the index word) or else appends
template <int D>
__global__ void k_res_insert(ResGrid g, const uint32_t* idx, uint64_t k) {
    constexpr int W = 2 * D + 1;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < k; t += nw) {
        const uint32_t id = idx[t];
        const uint32_t* b = g.boxes + (uint64_t)id * W;
        uint32_t lo[3], hi[3];
        res_range<D>(b, g.shift, lo, hi);
        for (uint32_t kk = lo[2]; kk <= hi[2]; kk++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t i = lo[0]; i <= hi[0]; i++) {
                    const uint64_t c = res_gid(g, i, j, kk);
                    const uint32_t f = (i == lo[0] ? 1u : 0u) | (j == lo[1] ? 2u : 0u) | (kk == lo[2] ? 4u : 0u);
                    const uint32_t idw = (f << kIdBits) | id;
                    const uint32_t s0 = g.start[c], cap = g.start[c + 1] - s0, n = min(g.used[c], cap);
                    int64_t slot = -1;  // warp-uniform once found
                    for (uint32_t e0 = 0; e0 < n && slot < 0; e0 += 32) {
                        const uint32_t e = e0 + lane;
                        unsigned int* w = e < n ? &g.entries[2 * (uint64_t)(s0 + e) + 1].z : nullptr;
                        uint32_t cand = __ballot_sync(0xffffffffu, w && *w == kDead);
                        while (cand && slot < 0) {  // claim one tombstone, nearest first
                            const uint32_t l = __ffs(cand) - 1;
                            uint32_t won = 0;
                            if (lane == l) won = atomicCAS(w, kDead, idw) == kDead;
                            if (__shfl_sync(0xffffffffu, won, l)) slot = e0 + l;
                            cand &= cand - 1;
                        }
                    }
                    if (slot < 0) {  // no tombstone: append
                        uint32_t sl = 0;
                        if (lane == 0) sl = atomicAdd(&g.used[c], 1u);
                        sl = __shfl_sync(0xffffffffu, sl, 0);
                        if (sl < cap) slot = sl;
                        else if (lane == 0) atomicOr(&g.ctr->overflow, 1u);
                    }
                    if (slot >= 0 && lane == 0) {
                        uint4 e0, e1;
                        res_slot<D>(b, idw, e0, e1);
                        g.entries[2 * (uint64_t)(s0 + slot)] = e0;
                        g.entries[2 * (uint64_t)(s0 + slot) + 1] = e1;
                    }
                }
    }
}

// one warp per listed box: its entries (at the box's current coordinates) become tombstones
template <int D>
__global__ void k_res_remove(ResGrid g, const uint32_t* idx, uint64_t k) {
    constexpr int W = 2 * D + 1;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t t = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < k; t += nw) {
        const uint32_t id = idx[t];
        uint32_t lo[3], hi[3];
        res_range<D>(g.boxes + (uint64_t)id * W, g.shift, lo, hi);
        uint32_t removed = 0;
        for (uint32_t kk = lo[2]; kk <= hi[2]; kk++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t i = lo[0]; i <= hi[0]; i++) {
                    const uint64_t c = res_gid(g, i, j, kk);
                    const uint32_t s0 = g.start[c], n = min(g.used[c], g.start[c + 1] - s0);
                    for (uint32_t e0 = 0; e0 < n; e0 += 128) {
                        uint32_t v[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const uint32_t e = e0 + 32 * u + lane;
                            v[u] = e < n ? g.entries[2 * (uint64_t)(s0 + e) + 1].z : kDead;
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            if (v[u] != kDead && (v[u] & kIdMask) == id) {
                                g.entries[2 * (uint64_t)(s0 + e0 + 32 * u + lane) + 1].z = kDead;
                                removed++;
                            }
                    }
                }
        removed = __reduce_add_sync(0xffffffffu, removed);
        if (lane == 0 && removed) atomicAdd(&g.ctr->dead, (unsigned long long)removed);
    }
}

__device__ __forceinline__ bool res_moved(const uint32_t* bits, uint32_t id) { return (bits[id >> 5] >> (id & 31u)) & 1u; }

// one warp per listed box m: every pair (m, o) of the box with another box o
// that shares a cell with it, reported in the cell of the minimum corner of
// their intersection; a pair of two listed boxes is reported from the smaller
// index. Pairs are compacted per warp through shared memory.
constexpr int kResThreads = 256;
constexpr uint32_t kResBuf = 256;  // pairs per warp buffer

template <int D>
__global__ void __launch_bounds__(kResThreads) k_res_query(ResGrid g, const uint32_t* idx, uint64_t k,
                                                           const uint32_t* moved, uint2* out, uint64_t out_cap) {
    constexpr int W = 2 * D + 1;
    __shared__ uint2 s_buf[kResThreads / 32][kResBuf];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint2* buf = s_buf[warp];
    uint32_t nbuf = 0;
    auto flush = [&]() {
        unsigned long long base = 0;
        if (lane == 0 && nbuf) base = atomicAdd(&g.ctr->out, (unsigned long long)nbuf);
        base = __shfl_sync(0xffffffffu, base, 0);
        __syncwarp();
        for (uint32_t q = lane; q < nbuf; q += 32)
            if (base + q < out_cap) out[base + q] = buf[q];
        __syncwarp();
        nbuf = 0;
    };
    const uint64_t nw = (uint64_t)gridDim.x * (kResThreads / 32);
    for (uint64_t t = (uint64_t)blockIdx.x * (kResThreads / 32) + warp; t < k; t += nw) {
        const uint32_t m = idx[t];
        const uint32_t* bm = g.boxes + (uint64_t)m * W;
        uint32_t a[6];
#pragma unroll
        for (int d = 0; d < 6; d++) a[d] = d < 2 * D ? bm[d] : 0u;
        uint32_t lo[3], hi[3];
        res_range<D>(bm, g.shift, lo, hi);
        for (uint32_t kk = lo[2]; kk <= hi[2]; kk++)
            for (uint32_t j = lo[1]; j <= hi[1]; j++)
                for (uint32_t i = lo[0]; i <= hi[0]; i++) {
                    const uint64_t c = res_gid(g, i, j, kk);
                    const uint32_t fm = (i == lo[0] ? 1u : 0u) | (j == lo[1] ? 2u : 0u) | (kk == lo[2] ? 4u : 0u);
                    const uint32_t s0 = g.start[c], n = min(g.used[c], g.start[c + 1] - s0);
                    // 128 slots per step: four slot pairs per lane in flight together
                    for (uint32_t e0 = 0; e0 < n; e0 += 128) {
                        uint4 c0[4], c1[4];
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const uint32_t e = e0 + 32 * u + lane;
                            if (e < n) {
                                const uint64_t sl = 2 * (uint64_t)(s0 + e);
                                c0[u] = g.entries[sl];
                                c1[u] = g.entries[sl + 1];
                            } else {
                                c1[u].z = kDead;
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const uint32_t v = c1[u].z, o = v & kIdMask;
                            bool hit = false;
                            if (v != kDead && o != m && !(res_moved(moved, o) && o < m) && ((fm | (v >> kIdBits)) == 7u)) {
                                hit = a[0] <= c0[u].y && c0[u].x <= a[1] && a[2] <= c0[u].w && c0[u].z <= a[3];
                                if (D == 3) hit = hit && a[4] <= c1[u].y && c1[u].x <= a[5];
                            }
                            const uint32_t hm = __ballot_sync(0xffffffffu, hit);
                            if (nbuf + __popc(hm) > kResBuf) flush();
                            if (hit) buf[nbuf + __popc(hm & ((1u << lane) - 1u))] = make_uint2(min(m, o), max(m, o));
                            nbuf += __popc(hm);
                            __syncwarp();
                        }
                    }
                }
    }
    flush();
}

// pairs of `in` without a moved box go to `out`: each thread takes 4 pairs
// (two 16-byte loads), one reservation per block and round
constexpr int kFilterThreads = 512;
constexpr int kFilterPer = 4;
__global__ void __launch_bounds__(kFilterThreads) k_res_filter(const uint2* in, uint64_t n, const uint32_t* moved,
                                                               uint2* out, ResCtr* ctr) {
    __shared__ uint32_t s_w[kFilterThreads / 32];
    __shared__ unsigned long long s_base;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint64_t round = (uint64_t)kFilterThreads * kFilterPer;
    for (uint64_t b0 = (uint64_t)blockIdx.x * round; b0 < n; b0 += (uint64_t)gridDim.x * round) {
        const uint64_t i0 = b0 + (uint64_t)t * kFilterPer;
        uint2 pr[kFilterPer];
        uint32_t keep = 0;
        if (i0 + kFilterPer <= n) {
            const uint4* q = reinterpret_cast<const uint4*>(in + i0);
            const uint4 a = q[0], b = q[1];
            pr[0] = make_uint2(a.x, a.y); pr[1] = make_uint2(a.z, a.w);
            pr[2] = make_uint2(b.x, b.y); pr[3] = make_uint2(b.z, b.w);
        } else {
#pragma unroll
            for (int k = 0; k < kFilterPer; k++) pr[k] = i0 + k < n ? in[i0 + k] : make_uint2(0u, 0u);
        }
#pragma unroll
        for (int k = 0; k < kFilterPer; k++)
            if (i0 + k < n && !res_moved(moved, pr[k].x) && !res_moved(moved, pr[k].y)) keep |= 1u << k;
        const uint32_t cnt = __popc(keep);
        uint32_t incl = cnt;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += x;
        }
        if (lane == 31) s_w[warp] = incl;
        __syncthreads();
        if (t == 0) {
            uint32_t tot = 0;
            for (int w = 0; w < kFilterThreads / 32; w++) {
                const uint32_t x = s_w[w];
                s_w[w] = tot;
                tot += x;
            }
            s_base = tot ? atomicAdd(&ctr->kept, (unsigned long long)tot) : 0ull;
        }
        __syncthreads();
        uint64_t pos = s_base + s_w[warp] + (incl - cnt);
#pragma unroll
        for (int k = 0; k < kFilterPer; k++)
            if (keep & (1u << k)) out[pos++] = pr[k];
        __syncthreads();
    }
}

// mark (set) or unmark the listed boxes; an index listed twice is an error
__global__ void k_res_bits(uint32_t* bits, const uint32_t* idx, uint64_t k, int set, ResCtr* ctr) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < k; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t id = idx[t], bit = 1u << (id & 31u);
        if (set) {
            if (atomicOr(&bits[id >> 5], bit) & bit) atomicOr(&ctr->err, kErrIndex);
        } else {
            atomicAnd(&bits[id >> 5], ~bit);
        }
    }
}

// validate the new records (rid = listed index < n, coordinates < range,
// min <= max) and copy them over the boxes
template <int D>
__global__ void k_res_check(const uint32_t* nb, const uint32_t* idx, uint64_t k, uint64_t n, uint32_t range,
                            ResCtr* ctr) {
    constexpr int W = 2 * D + 1;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < k; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t* b = nb + t * W;
        uint32_t err = 0;
        if (idx[t] >= n || b[2 * D] != idx[t]) err |= kErrRid;
#pragma unroll
        for (int d = 0; d < D; d++) {
            if (b[2 * d] >= range || b[2 * d + 1] >= range) err |= kErrRange;
            if (b[2 * d] > b[2 * d + 1]) err |= kErrInverted;
        }
        if (err) atomicOr(&ctr->err, err);
    }
}

template <int D>
__global__ void k_res_write(uint32_t* boxes, const uint32_t* nb, const uint32_t* idx, uint64_t k) {
    constexpr int W = 2 * D + 1;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < k; t += (uint64_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int w = 0; w < W; w++) boxes[(uint64_t)idx[t] * W + w] = nb[t * W + w];
}

}  // namespace pbig

using namespace pbig;

struct pbig2_scene {
    pbig2_ctx* ctx = nullptr;
    int dims = 3;
    uint32_t range = 0, shift = 0, nrc = 0;
    uint64_t n = 0, ncells = 0;
    DevBuf boxes, start, used, entries, cnt, tmp, state, ctrbuf, rctr, lists, moved, idx, nb;
    DevBuf full[2], rem, add;
    int cur = 0;  // full[cur] holds the current list
    bool keep_full = true;  // maintain the full pair list on every move
    uint64_t nfull = 0, nrem = 0, nadd = 0, slots = 0, dead = 0;
    uint64_t rebuilds = 0;

    ResGrid grid() {
        ResGrid g{};
        g.boxes = boxes.as<uint32_t>();
        g.nboxes = n;
        g.shift = shift;
        g.nrc = nrc;
        g.range = range;
        g.ncells = ncells;
        g.start = start.as<uint32_t>();
        g.used = used.as<uint32_t>();
        g.entries = entries.as<uint4>();
        g.ctr = rctr.as<ResCtr>();
        return g;
    }
};

namespace {

#define SCK(expr)                                                                                      \
    do {                                                                                               \
        cudaError_t _e = (expr);                                                                       \
        if (_e != cudaSuccess) {                                                                       \
            char _m[256];                                                                              \
            snprintf(_m, sizeof _m, "%s: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, __LINE__); \
            return api_fail(_e == cudaErrorMemoryAllocation ? PBIG2_ENOMEM : PBIG2_ECUDA, _m);        \
        }                                                                                              \
    } while (0)

unsigned grid_for(uint64_t items, unsigned per_block, int sms) {
    uint64_t b = (items + per_block - 1) / per_block;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 152) * 16;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

ResCtr read_ctr(pbig2_scene* s, cudaStream_t st, cudaError_t* e) {
    ResCtr h{};
    *e = cudaMemcpyAsync(&h, s->rctr.p, sizeof h, cudaMemcpyDeviceToHost, st);
    if (*e == cudaSuccess) *e = cudaStreamSynchronize(st);
    return h;
}

// the grid of the scene's current boxes: counts, capacities with slack,
// starts (the engine's scan), then every box inserted
int build_grid(pbig2_scene* s, cudaStream_t st) {
    const int sms = s->ctx->sm_count;
    SCK(s->cnt.ensure(s->ncells * 4 + 16, false, st));
    SCK(s->tmp.ensure(s->ncells * 4 + 16, false, st));
    SCK(s->start.ensure((s->ncells + 1) * 4, false, st));
    SCK(s->used.ensure(s->ncells * 4, false, st));
    SCK(s->state.ensure(scan_state_bytes(s->ncells), false, st));
    SCK(s->ctrbuf.ensure(sizeof(Ctr), false, st));
    SCK(s->lists.ensure(256, false, st));
    SCK(cudaMemsetAsync(s->cnt.p, 0, s->ncells * 4, st));
    SCK(cudaMemsetAsync(s->rctr.p, 0, sizeof(ResCtr), st));
    ResGrid g = s->grid();
    if (s->dims == 2) k_res_count<2><<<grid_for(s->n, 256, sms), 256, 0, st>>>(g, s->cnt.as<uint32_t>());
    else k_res_count<3><<<grid_for(s->n, 256, sms), 256, 0, st>>>(g, s->cnt.as<uint32_t>());
    SCK(cudaGetLastError());
    k_res_caps<<<grid_for(s->ncells, 256, sms), 256, 0, st>>>(s->cnt.as<uint32_t>(), s->tmp.as<uint32_t>(), s->ncells);
    SCK(cudaGetLastError());
    // exclusive scan of the capacities with the engine's scan kernels (the
    // cell ends replace the capacities in place; no work lists)
    Params p{};
    p.counts = s->tmp.as<uint32_t>();
    p.ncells = s->ncells;
    p.tile_state = s->state.as<unsigned long long>();
    p.ctr = s->ctrbuf.as<Ctr>();
    p.lists = s->lists.as<uint2>();
    SCK(cudaMemsetAsync(p.ctr, 0, sizeof(Ctr), st));
    SCK(launch_scan(p, st));
    k_res_starts<<<grid_for(s->ncells, 256, sms), 256, 0, st>>>(s->cnt.as<uint32_t>(), s->tmp.as<uint32_t>(), g);
    SCK(cudaGetLastError());
    uint32_t total = 0;
    SCK(cudaMemcpyAsync(&total, s->start.as<uint32_t>() + s->ncells, 4, cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    SCK(s->entries.ensure((uint64_t)total * 32 + 32, false, st));
    g = s->grid();
    if (s->dims == 2) k_res_fill<2><<<grid_for(s->n, 256, sms), 256, 0, st>>>(g);
    else k_res_fill<3><<<grid_for(s->n, 256, sms), 256, 0, st>>>(g);
    SCK(cudaGetLastError());
    cudaError_t e;
    const ResCtr h = read_ctr(s, st, &e);
    SCK(e);
    if (h.overflow) return api_fail(PBIG2_ECUDA, "resident grid: a cell overflowed its own count");
    s->dead = 0;
    s->slots = total;
    s->rebuilds++;
    return PBIG2_OK;
}

// pairs of the listed boxes (at their current coordinates) into buf; grows
// the buffer and repeats when it was too small
int query_listed(pbig2_scene* s, uint64_t k, DevBuf& buf, uint64_t& count, cudaStream_t st) {
    const int sms = s->ctx->sm_count;
    for (int attempt = 0; attempt < 3; attempt++) {
        SCK(buf.ensure(256 * 8, false, st));
        const uint64_t cap = buf.bytes / 8;
        SCK(cudaMemsetAsync(&s->rctr.as<ResCtr>()->out, 0, 8, st));
        const ResGrid g = s->grid();
        const unsigned blocks = grid_for(k, kResThreads / 32, sms);
        if (s->dims == 2)
            k_res_query<2><<<blocks, kResThreads, 0, st>>>(g, s->idx.as<uint32_t>(), k, s->moved.as<uint32_t>(),
                                                           buf.as<uint2>(), cap);
        else
            k_res_query<3><<<blocks, kResThreads, 0, st>>>(g, s->idx.as<uint32_t>(), k, s->moved.as<uint32_t>(),
                                                           buf.as<uint2>(), cap);
        SCK(cudaGetLastError());
        cudaError_t e;
        const ResCtr h = read_ctr(s, st, &e);
        SCK(e);
        count = h.out;
        if (count <= cap) return PBIG2_OK;
        SCK(buf.ensure(count * 8 + count / 4 + 1024, false, st));
    }
    return api_fail(PBIG2_ENOMEM, "pair buffer retries exhausted");
}

}  // namespace

extern "C" {

PBIG2_API int pbig2_scene_create(pbig2_ctx* c, const uint32_t* boxes, uint64_t n, uint32_t dims, uint32_t range,
                                 uint32_t cell_shift, int boxes_loc, uint32_t flags, pbig2_scene** out,
                                 uint64_t* npairs) {
    if (!c || !out || !npairs || (dims != 2 && dims != 3) || range == 0 || (n && !boxes))
        return api_fail(PBIG2_EINVAL, "bad arguments");
    *out = nullptr;
    *npairs = 0;
    if (n == 0 || n > (uint64_t)kIdMask + 1) return api_fail(PBIG2_EINVAL, "a scene holds 1 .. 2^29 boxes");
    // the full query first: its pairs, its cell size, and the input checks
    uint64_t np = 0;
    int rc = pbig2_self_intersect(c, boxes, n, dims, range, cell_shift, boxes_loc, nullptr, &np);
    if (rc != PBIG2_OK) return rc == PBIG2_EINPUT ? api_fail(PBIG2_EINPUT, "a scene's boxes must all be valid") : rc;
    pbig2_stats st{};
    pbig2_get_stats(c, &st);
    pbig2_scene* s = new pbig2_scene();
    s->ctx = c;
    s->dims = (int)dims;
    s->range = range;
    s->shift = st.cell_shift;
    s->nrc = nrc_for(range, s->shift);
    s->n = n;
    s->ncells = grid_cells(range, s->shift, (int)dims);  // below 2^32: the query above ran on this grid
    cudaStream_t sm = c->own_stream;
    const int W = 2 * (int)dims + 1;
    auto bail = [&](int code) {
        pbig2_scene_destroy(s);
        return code;
    };
    if (s->boxes.ensure(n * W * 4 + 16, false, sm) != cudaSuccess ||
        s->rctr.ensure(sizeof(ResCtr), false, sm) != cudaSuccess ||
        s->moved.ensure(((n + 31) / 32) * 4 + 16, true, sm) != cudaSuccess ||
        s->full[0].ensure(np * 8 + 16, false, sm) != cudaSuccess)
        return bail(api_fail(PBIG2_ENOMEM, "scene allocation failed"));
    if (cudaMemcpyAsync(s->boxes.p, boxes, n * W * 4, cudaMemcpyDefault, sm) != cudaSuccess)
        return bail(api_fail(PBIG2_ECUDA, "copying the scene's boxes failed"));
    if (np && pbig2_copy_pairs(c, s->full[0].as<uint32_t>(), 0, np, PBIG2_DEVICE, sm) != PBIG2_OK) return bail(PBIG2_ECUDA);
    s->nfull = np;
    s->keep_full = (flags & PBIG2_SCENE_DELTA_ONLY) == 0;
    rc = build_grid(s, sm);
    if (rc != PBIG2_OK) return bail(rc);
    *out = s;
    *npairs = np;
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_destroy(pbig2_scene* s) {
    if (!s) return PBIG2_OK;
    for (DevBuf* b : {&s->boxes, &s->start, &s->used, &s->entries, &s->cnt, &s->tmp, &s->state, &s->ctrbuf, &s->rctr,
                      &s->lists, &s->moved, &s->idx, &s->nb, &s->full[0], &s->full[1], &s->rem, &s->add})
        b->release();
    delete s;
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_move(pbig2_scene* s, const uint32_t* idx, uint64_t k, const uint32_t* new_boxes, int loc,
                               uint64_t* n_removed, uint64_t* n_added) {
    if (!s || !n_removed || !n_added || (k && (!idx || !new_boxes))) return api_fail(PBIG2_EINVAL, "bad arguments");
    *n_removed = *n_added = 0;
    if (k == 0) {
        s->nrem = s->nadd = 0;
        return PBIG2_OK;
    }
    if (k > s->n) return api_fail(PBIG2_EINVAL, "more moved boxes than the scene holds");
    SCK(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->own_stream;
    const int sms = s->ctx->sm_count;
    const int W = 2 * s->dims + 1;
    (void)loc;  // copies below read host or device memory alike
    SCK(s->idx.ensure(k * 4 + 16, false, st));
    SCK(s->nb.ensure(k * W * 4 + 16, false, st));
    SCK(cudaMemcpyAsync(s->idx.p, idx, k * 4, cudaMemcpyDefault, st));
    SCK(cudaMemcpyAsync(s->nb.p, new_boxes, k * W * 4, cudaMemcpyDefault, st));
    SCK(cudaMemsetAsync(s->rctr.p, 0, sizeof(ResCtr), st));
    const unsigned gk = grid_for(k, 256, sms);
    const uint32_t* d_idx = s->idx.as<uint32_t>();
    if (s->dims == 2) k_res_check<2><<<gk, 256, 0, st>>>(s->nb.as<uint32_t>(), d_idx, k, s->n, s->range, s->rctr.as<ResCtr>());
    else k_res_check<3><<<gk, 256, 0, st>>>(s->nb.as<uint32_t>(), d_idx, k, s->n, s->range, s->rctr.as<ResCtr>());
    SCK(cudaGetLastError());
    cudaError_t e;
    ResCtr h = read_ctr(s, st, &e);
    SCK(e);
    if (h.err)
        return api_fail(PBIG2_EINVAL, "moved boxes must keep rid = their index, coordinates < range and min <= max");
    k_res_bits<<<gk, 256, 0, st>>>(s->moved.as<uint32_t>(), d_idx, k, 1, s->rctr.as<ResCtr>());
    SCK(cudaGetLastError());
    h = read_ctr(s, st, &e);
    SCK(e);
    if (h.err) {
        k_res_bits<<<gk, 256, 0, st>>>(s->moved.as<uint32_t>(), d_idx, k, 0, s->rctr.as<ResCtr>());
        SCK(cudaStreamSynchronize(st));
        return api_fail(PBIG2_EINVAL, "a box is listed twice");
    }
    // 1. pairs of the moved boxes before the move
    int rc = query_listed(s, k, s->rem, s->nrem, st);
    if (rc) return rc;
    // 2. their entries become tombstones, 3. new coordinates, 4. new entries
    const ResGrid g = s->grid();
    const unsigned gw = grid_for(k, 8, sms);
    if (s->dims == 2) k_res_remove<2><<<gw, 256, 0, st>>>(g, d_idx, k);
    else k_res_remove<3><<<gw, 256, 0, st>>>(g, d_idx, k);
    SCK(cudaGetLastError());
    if (s->dims == 2) k_res_write<2><<<gk, 256, 0, st>>>(s->boxes.as<uint32_t>(), s->nb.as<uint32_t>(), d_idx, k);
    else k_res_write<3><<<gk, 256, 0, st>>>(s->boxes.as<uint32_t>(), s->nb.as<uint32_t>(), d_idx, k);
    SCK(cudaGetLastError());
    if (s->dims == 2) k_res_insert<2><<<gw, 256, 0, st>>>(g, d_idx, k);
    else k_res_insert<3><<<gw, 256, 0, st>>>(g, d_idx, k);
    SCK(cudaGetLastError());
    h = read_ctr(s, st, &e);
    SCK(e);
    s->dead += h.dead;
    if (h.overflow) {
        rc = build_grid(s, st);  // a cell ran out of slack
        if (rc) return rc;
    }
    // 5. pairs of the moved boxes after the move
    rc = query_listed(s, k, s->add, s->nadd, st);
    if (rc) return rc;
    // 6. the full list: the old one without the moved boxes' pairs, then the new ones
    if (!s->keep_full) {
        k_res_bits<<<gk, 256, 0, st>>>(s->moved.as<uint32_t>(), d_idx, k, 0, s->rctr.as<ResCtr>());
        SCK(cudaGetLastError());
        SCK(cudaStreamSynchronize(st));
        *n_removed = s->nrem;
        *n_added = s->nadd;
        return PBIG2_OK;
    }
    const int nxt = s->cur ^ 1;
    SCK(s->full[nxt].ensure((s->nfull + s->nadd) * 8 + 16, false, st));
    SCK(cudaMemsetAsync(&s->rctr.as<ResCtr>()->kept, 0, 8, st));
    if (s->nfull)
        k_res_filter<<<grid_for(s->nfull, kFilterThreads * kFilterPer, sms), kFilterThreads, 0, st>>>(
            s->full[s->cur].as<uint2>(), s->nfull, s->moved.as<uint32_t>(), s->full[nxt].as<uint2>(), s->rctr.as<ResCtr>());
    SCK(cudaGetLastError());
    h = read_ctr(s, st, &e);
    SCK(e);
    if (s->nadd)
        SCK(cudaMemcpyAsync(s->full[nxt].as<uint2>() + h.kept, s->add.p, s->nadd * 8, cudaMemcpyDeviceToDevice, st));
    k_res_bits<<<gk, 256, 0, st>>>(s->moved.as<uint32_t>(), d_idx, k, 0, s->rctr.as<ResCtr>());
    SCK(cudaGetLastError());
    SCK(cudaStreamSynchronize(st));
    s->cur = nxt;
    s->nfull = h.kept + s->nadd;
    *n_removed = s->nrem;
    *n_added = s->nadd;
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_delta(pbig2_scene* s, const uint32_t** removed, uint64_t* n_removed, const uint32_t** added,
                                uint64_t* n_added) {
    if (!s || !removed || !n_removed || !added || !n_added) return api_fail(PBIG2_EINVAL, "bad arguments");
    *removed = s->rem.as<uint32_t>();
    *n_removed = s->nrem;
    *added = s->add.as<uint32_t>();
    *n_added = s->nadd;
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_pairs(pbig2_scene* s, const uint32_t** pairs, uint64_t* npairs) {
    if (!s || !pairs || !npairs) return api_fail(PBIG2_EINVAL, "bad arguments");
    if (!s->keep_full) return api_fail(PBIG2_EINVAL, "the scene keeps no full pair list (PBIG2_SCENE_DELTA_ONLY)");
    *pairs = s->full[s->cur].as<uint32_t>();
    *npairs = s->nfull;
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_copy(pbig2_scene* s, int which, uint32_t* dst, uint64_t count) {
    if (!s || (count && !dst) || which < 0 || which > 2) return api_fail(PBIG2_EINVAL, "bad arguments");
    if (which == 0 && !s->keep_full) return api_fail(PBIG2_EINVAL, "the scene keeps no full pair list (PBIG2_SCENE_DELTA_ONLY)");
    const uint64_t have = which == 0 ? s->nfull : which == 1 ? s->nrem : s->nadd;
    if (count > have) return api_fail(PBIG2_EINVAL, "more pairs asked for than the list holds");
    if (count == 0) return PBIG2_OK;
    const void* src = which == 0 ? s->full[s->cur].p : which == 1 ? s->rem.p : s->add.p;
    SCK(cudaSetDevice(s->ctx->device));
    SCK(cudaMemcpyAsync(dst, src, count * 8, cudaMemcpyDefault, s->ctx->own_stream));
    SCK(cudaStreamSynchronize(s->ctx->own_stream));
    return PBIG2_OK;
}

PBIG2_API int pbig2_scene_boxes(pbig2_scene* s, const uint32_t** boxes, uint64_t* n) {
    if (!s || !boxes || !n) return api_fail(PBIG2_EINVAL, "bad arguments");
    *boxes = s->boxes.as<uint32_t>();
    *n = s->n;
    return PBIG2_OK;
}

}  // extern "C"
