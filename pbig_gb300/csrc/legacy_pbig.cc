// The PBIG library API (pbig.h) on top of the pbig2 C ABI.
//
// Compiled together with the caller's report.h (it must be first on the
// include path): pbig_check inlines report::operator() exactly as the
// reference's decode() does (src/pbig/decode.cc:26-138, src/pbig/report.h:10),
// so any report type a client defines keeps working. The pair kernels store
// the pairs straight into a page-locked host buffer (pbig2_set_pair_output),
// so the callbacks start as soon as the query returns; a result larger than
// that buffer is streamed from the device in chunks instead, the copy of
// chunk k+1 overlapping the callbacks of chunk k (the reference's two-buffer
// match_phase pipeline, src/pbig/pbig.cu:1694-1960, reduced to its output
// half), and the buffer grows for the next query.
//
// Errors follow the reference: CUDA failures print a message and exit(-1)
// (src/pbig/log.h:4-12); boxes that break the input contract (coordinate >=
// range, min > max, rid != index) are skipped with a warning, the pairs of
// the valid boxes are still reported.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "rect.h"
#include "report.h"
#include "pbig.h"
#include "pbig2.h"

static_assert(sizeof(RectInfo) == (2 * DIMS + 1) * sizeof(unsigned int), "RectInfo must be packed u32 words");

namespace {

struct LegacyState {
    pbig2_ctx* ctx = nullptr;
    unsigned num = 0, range = 0;
    uint32_t shift = PBIG2_AUTO;
    uint32_t* chunk[2] = {nullptr, nullptr};
    uint32_t* out = nullptr;  // direct pair output (page-locked)
    uint64_t out_cap = 0;
    bool warned = false;
};
LegacyState g_state;
const uint64_t kChunkPairs = 1u << 22;  // 32 MiB per buffer

void die(const char* where) {
    printf("ERROR:%s: %s\n", where, pbig2_last_error());
    exit(-1);
}

}  // namespace

// device_init / cuda_finalize: the two other symbols the reference library
// exports for its harness (src/pbig/pbig.cu:2087, 129; declared by the
// harness itself, src/pbig/hybrid.cc:16). The reference maps every device
// symbol to device 0.
int device_init(unsigned int deviceSymbol) {
    (void)deviceSymbol;
    return 0;
}

void pbig_finalize();

void cuda_finalize() { pbig_finalize(); }

static void set_out(uint64_t cap) {
    if (g_state.out) {
        pbig2_set_pair_output(g_state.ctx, nullptr, 0);
        pbig2_host_free(g_state.out);
        g_state.out = nullptr;
        g_state.out_cap = 0;
    }
    if (pbig2_host_alloc(cap * 8, (void**)&g_state.out) != PBIG2_OK) die("pbig_init");
    g_state.out_cap = cap;
    if (pbig2_set_pair_output(g_state.ctx, g_state.out, cap) != PBIG2_OK) die("pbig_init");
}

void pbig_finalize() {
    for (auto& c : g_state.chunk) {
        if (c) pbig2_host_free(c);
        c = nullptr;
    }
    if (g_state.ctx && g_state.out) pbig2_set_pair_output(g_state.ctx, nullptr, 0);
    if (g_state.out) pbig2_host_free(g_state.out);
    g_state.out = nullptr;
    g_state.out_cap = 0;
    if (g_state.ctx) pbig2_destroy(g_state.ctx);
    g_state.ctx = nullptr;
}

void pbig_init(unsigned int num, unsigned int range, unsigned int cs, unsigned int deviceID,
               unsigned int hasProfSteps) {
    (void)hasProfSteps;
    if (g_state.ctx) pbig_finalize();
    if (pbig2_create((int)deviceID, &g_state.ctx) != PBIG2_OK) die("pbig_init");
    g_state.num = num;
    g_state.range = range;
    g_state.shift = PBIG2_AUTO;
    if (cs != 0 && (cs & (cs - 1)) == 0) {
        uint32_t s = 0;
        while ((1u << s) < cs) s++;
        g_state.shift = s;
    }
    for (auto& c : g_state.chunk)
        if (pbig2_host_alloc(kChunkPairs * 8, (void**)&c) != PBIG2_OK) die("pbig_init");
    set_out(kChunkPairs);
}

void pbig_check(struct RectInfo* input, struct report* r) {
    if (!g_state.ctx) {
        printf("ERROR:pbig_check called before pbig_init\n");
        exit(-1);
    }
    uint64_t np = 0;
    int rc = pbig2_self_intersect(g_state.ctx, reinterpret_cast<const uint32_t*>(input), g_state.num, DIMS,
                                  g_state.range, g_state.shift, PBIG2_HOST, nullptr, &np);
    if (rc == PBIG2_EINPUT) {
        if (!g_state.warned) printf("WARNING:pbig_check: %s\n", pbig2_last_error());
        g_state.warned = true;
    } else if (rc != PBIG2_OK) {
        die("pbig_check");
    }
    if (np == 0) return;
    const uint32_t* res = nullptr;
    uint64_t rn = 0;
    if (pbig2_result_pairs(g_state.ctx, &res, &rn) != PBIG2_OK) die("pbig_check");
    if (res == g_state.out) {  // already in host memory
        for (uint64_t k = 0; k < np; k++) (*r)(res[2 * k], res[2 * k + 1]);
        return;
    }
    uint64_t first = 0;
    int cur = 0;
    uint64_t cnt = np < kChunkPairs ? np : kChunkPairs;
    if (pbig2_copy_pairs_async(g_state.ctx, g_state.chunk[cur], 0, cnt, PBIG2_HOST, nullptr) != PBIG2_OK)
        die("pbig_check");
    while (first < np) {
        if (pbig2_sync(g_state.ctx, nullptr) != PBIG2_OK) die("pbig_check");
        const uint64_t next = first + cnt;
        const uint64_t ncnt = np - next < kChunkPairs ? np - next : kChunkPairs;
        if (next < np &&
            pbig2_copy_pairs_async(g_state.ctx, g_state.chunk[cur ^ 1], next, ncnt, PBIG2_HOST, nullptr) != PBIG2_OK)
            die("pbig_check");
        const uint32_t* p = g_state.chunk[cur];
        for (uint64_t k = 0; k < cnt; k++) (*r)(p[2 * k], p[2 * k + 1]);
        first = next;
        cnt = ncnt;
        cur ^= 1;
    }
    set_out(np + np / 4);  // the next query's pairs go straight to the host
}
