// One step of the serving loop in native code (pbig2_serve_batch).
//
// The request loop (pbig_gb300/serve.py) decides which pending requests form
// a batch and where each scene lives on the device; everything a batch then
// does on the host and the device runs here, in one call that holds no
// interpreter lock: the cell size of new scenes (the autotuner on a sample of
// the host rows), the moved rows of updates (into the host copy, and into
// the device copy by one scatter kernel), uploads of scenes that are not on
// the device, the concatenation of the batch's scenes, the batched query,
// and the copy of the pairs into the caller's page-locked buffer.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine.h"
#include "kernels.cuh"
#include "pbig2.h"

namespace {

constexpr uint32_t kRowWords = 7;    // RectInfo, 3-D
constexpr uint32_t kStageWords = 8;  // a staged update row: 7 words, then the box index

// staged rows -> their boxes' rows in a scene's device copy
__global__ void k_put_rows(uint32_t* dst, const uint32_t* rows, uint64_t k, uint64_t n) {
    const uint64_t words = k * kRowWords;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = i / kRowWords, w = i % kRowWords;
        const uint64_t box = rows[r * kStageWords + kRowWords];
        if (box < n) dst[box * kRowWords + w] = rows[r * kStageWords + w];
    }
}

double ms_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

int fail(int code, const char* fmt, ...) {
    char msg[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    return pbig::api_fail(code, msg);
}

}  // namespace

extern "C" {

PBIG2_API int pbig2_serve_batch(pbig2_ctx* c, pbig2_batch_item* items, uint32_t n_items, uint32_t range,
                                uint32_t* cat_dev, uint64_t cat_rows, uint32_t* stage_host, uint32_t* stage_dev,
                                uint64_t stage_rows, void* stream, uint32_t* pairs_host, uint64_t pairs_cap,
                                uint64_t* npairs, uint64_t* scene_pair_off, double* phase_ms) {
    if (!c || !items || n_items == 0 || range == 0 || !npairs || !scene_pair_off)
        return fail(PBIG2_EINVAL, "serve_batch: bad arguments");
    *npairs = 0;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(PBIG2_ECUDA, "serve_batch: cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->own_stream;
    double ph[4] = {0, 0, 0, 0};
    auto t = std::chrono::steady_clock::now();
#define SCK(x)                                                                                          \
    do {                                                                                                \
        cudaError_t e_ = (x);                                                                           \
        if (e_ != cudaSuccess) return fail(PBIG2_ECUDA, "serve_batch: %s", cudaGetErrorString(e_));  \
    } while (0)

    // 1. cell sizes, moved rows (host copy first, so that an upload carries
    //    them), uploads, then the staged rows of resident scenes
    uint64_t staged = 0, total = 0;
    for (uint32_t i = 0; i < n_items; i++) {
        pbig2_batch_item& it = items[i];
        if (!it.dev || !it.host || (it.k && (!it.rows || !it.idx)))
            return fail(PBIG2_EINVAL, "serve_batch: item %u: missing buffers", i);
        total += it.n;
        if (it.shift == PBIG2_AUTO) it.shift = pbig::tune_shift_sample(it.host, it.n, it.n, 3, range, 256).shift;
        for (uint64_t r = 0; r < it.k; r++) {
            if (it.idx[r] >= it.n) return fail(PBIG2_EINVAL, "serve_batch: item %u: row index out of range", i);
            memcpy(it.host + (uint64_t)it.idx[r] * kRowWords, it.rows + r * kRowWords, kRowWords * 4);
        }
        if (it.upload) {
            SCK(cudaMemcpyAsync(it.dev, it.host, it.n * kRowWords * 4, cudaMemcpyHostToDevice, st));
        } else if (it.k) {
            if (staged + it.k > stage_rows || !stage_host || !stage_dev)
                return fail(PBIG2_ECAPACITY, "serve_batch: %llu staged rows exceed the staging buffer",
                                      (unsigned long long)(staged + it.k));
            for (uint64_t r = 0; r < it.k; r++) {
                uint32_t* s = stage_host + (staged + r) * kStageWords;
                memcpy(s, it.rows + r * kRowWords, kRowWords * 4);
                s[kRowWords] = it.idx[r];
            }
            staged += it.k;
        }
    }
    if (staged) {
        SCK(cudaMemcpyAsync(stage_dev, stage_host, staged * kStageWords * 4, cudaMemcpyHostToDevice, st));
        uint64_t off = 0;
        for (uint32_t i = 0; i < n_items; i++) {
            const pbig2_batch_item& it = items[i];
            if (it.upload || !it.k) continue;
            const uint64_t blocks = (it.k * kRowWords + 255) / 256;
            k_put_rows<<<(unsigned)(blocks < 1024 ? blocks : 1024), 256, 0, st>>>(it.dev, stage_dev + off * kStageWords,
                                                                                 it.k, it.n);
            SCK(cudaGetLastError());
            off += it.k;
        }
    }
    ph[0] = ms_since(t);
    t = std::chrono::steady_clock::now();

    // 2. the batch's scenes side by side
    const uint32_t* boxes = items[0].dev;
    if (n_items > 1) {
        if (!cat_dev || total > cat_rows)
            return fail(PBIG2_ECAPACITY, "serve_batch: %llu rows exceed the concatenation buffer",
                                  (unsigned long long)total);
        uint64_t off = 0;
        for (uint32_t i = 0; i < n_items; i++) {
            SCK(cudaMemcpyAsync(cat_dev + off * kRowWords, items[i].dev, items[i].n * kRowWords * 4,
                                cudaMemcpyDeviceToDevice, st));
            off += items[i].n;
        }
        boxes = cat_dev;
    }
    ph[1] = ms_since(t);
    t = std::chrono::steady_clock::now();

    // 3. the batched query (per-scene grids at the chosen cell sizes)
    std::vector<uint64_t> offs(n_items + 1, 0);
    std::vector<uint32_t> shifts(n_items);
    for (uint32_t i = 0; i < n_items; i++) {
        offs[i + 1] = offs[i] + items[i].n;
        shifts[i] = items[i].shift;
    }
    int rc = pbig2_batch_intersect(c, boxes, offs.data(), n_items, 3, range, shifts.data(), PBIG2_DEVICE, st, npairs);
    if (rc != PBIG2_OK) return rc;
    rc = pbig2_result_scene_offsets(c, scene_pair_off, n_items);
    if (rc != PBIG2_OK) return rc;
    ph[2] = ms_since(t);
    t = std::chrono::steady_clock::now();

    // 4. the pairs into the caller's page-locked buffer
    if (*npairs > pairs_cap || (*npairs && !pairs_host)) {
        if (phase_ms) memcpy(phase_ms, ph, sizeof ph);
        return fail(PBIG2_ECAPACITY, "serve_batch: %llu pairs exceed the pair buffer",
                              (unsigned long long)*npairs);
    }
    if (*npairs) {
        rc = pbig2_copy_pairs_async(c, pairs_host, 0, *npairs, PBIG2_HOST, st);
        if (rc != PBIG2_OK) return rc;
    }
    SCK(cudaStreamSynchronize(st));
    ph[3] = ms_since(t);
    if (phase_ms) memcpy(phase_ms, ph, sizeof ph);
#undef SCK
    return PBIG2_OK;
}

}  // extern "C"
