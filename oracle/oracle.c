/*
 * ORACLE — test infrastructure only. This is a CPU restatement of PBIG's
 * pairwise box-intersection path (awatch/pbig v0.2), used by tests/ to check
 * the CUDA engine and by bench.py as the timed CPU baseline. It is never
 * linked into or called by the product library.
 *
 * Parity pin: the grid restatement reproduces the reference's published pair
 * counts for its own harness generator (benchmarks/test1/filter_file:7 and
 * benchmarks/test3/filter_file:40), see tests/test_oracle_golden.py.
 *
 * Everything follows the reference's unsigned 32-bit arithmetic; each
 * function cites the reference source it restates (paths relative to the
 * reference project root).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_UNUSED 0x0fffff11u  /* src/pbig/cuda_comm.h:10 */
#define ORC_NTPB 256u            /* src/pbig/config.cmake:2 */
#define ORC_MAX_BATCH_RECS (480u * ORC_NTPB) /* src/pbig/pbig_internal.h:16 */

typedef struct {
    uint32_t cs, shift, nrc, ncells;
    uint64_t entries;     /* E: total cell entries (MAX_Grid_Recs) */
    uint64_t jobs;        /* number of (cell, 256-row tile) jobs */
    uint64_t batches;     /* number of match batches */
    uint64_t comp_pairs;  /* numCompPairs statistic */
    uint64_t pairs;       /* pairs emitted */
    uint32_t max_cell;    /* largest cell (after merging) */
    uint32_t would_abort; /* 1 if the reference would abort (cell >= MaxBatchRecs) */
    uint64_t tests;       /* pair tests actually executed */
} orc_stats;

/* ------------------------------------------------------------------ */
/* glibc random()/rand() (TYPE_3 additive feedback, degree 31, sep 3)  */
/* restated from its published description; used by the reference's   */
/* harness generator (src/pbig/main.cc:223 srand(100), rand()).        */
/* ------------------------------------------------------------------ */
typedef struct { uint32_t r[34]; int idx; } orc_rand_state;

void orc_srand(orc_rand_state* s, uint32_t seed) {
    int32_t r[344];
    if (seed == 0) seed = 1;
    r[0] = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
        int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
        int64_t w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        r[i] = (int32_t)w;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 34; i < 344; i++) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
    for (int i = 0; i < 34; i++) s->r[i] = (uint32_t)r[310 + i];
    s->idx = 0; /* ring over the last 34 values */
}

int32_t orc_rand(orc_rand_state* s) {
    /* r[k] = r[k-31] + r[k-3]; ring of 34 holds r[k-34..k-1] */
    int k = s->idx;
    uint32_t v = s->r[(k + 3) % 34] + s->r[(k + 31) % 34];
    s->r[k] = v;
    s->idx = (k + 1) % 34;
    return (int32_t)(v >> 1);
}

/* The reference harness generator, src/pbig/main.cc:223-335:
 * per box: 3 sizes ('U': rand()%S, 'N': normal(S, S*0.2)), then
 * 3 positions ('U': rand()%range, 'N': normal(range/2, range/2*0.2)),
 * xmin = pos, xmax = Inc(pos, size, range) (main.cc:220).
 * 3-D layout, rid = index. sim = "UU", "UN", "NU" or "NN". */
static double harness_normal(orc_rand_state* s, unsigned mean, unsigned stdv) {
    /* main.cc:209-217 */
    double u = orc_rand(s) / (double)2147483647;
    double v = orc_rand(s) / (double)2147483647;
    return sqrt(-2 * log(u)) * cos(2 * M_PI * v) * stdv + mean;
}

int orc_gen_harness(uint32_t n, uint32_t S, uint32_t range, const char* sim, uint32_t seed,
                    int dims, uint32_t* out) {
    orc_rand_state st;
    orc_srand(&st, seed);
    int W = 2 * dims + 1;
    for (uint32_t i = 0; i < n; i++) {
        int sz[3], pos[3];
        for (int d = 0; d < dims; d++) {
            if (sim[0] == 'U') sz[d] = (int)(double)((uint32_t)orc_rand(&st) % S);
            else sz[d] = (int)harness_normal(&st, S, (unsigned)(S * 0.2));
        }
        for (int d = 0; d < dims; d++) {
            if (sim[1] == 'U') pos[d] = (int)(double)((uint32_t)orc_rand(&st) % range);
            else pos[d] = (int)harness_normal(&st, range / 2, (unsigned)((range / 2) * 0.2));
        }
        uint32_t* b = out + (uint64_t)i * W;
        for (int d = 0; d < dims; d++) {
            int sum = pos[d] + sz[d];
            b[2 * d] = (uint32_t)pos[d];
            b[2 * d + 1] = ((uint32_t)sum >= range) ? range - 1 : (uint32_t)sum;
        }
        b[2 * dims] = i;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* decideCellSize: src/pbig/pbig.cu:1285-1357 (avg functors :1256-1281) */
/* The averages sum the first min(1000,N) extents with an int          */
/* accumulator and float adds (thrust::transform_reduce with int init) */
/* then integer-divide by the sample count.                            */
/* ------------------------------------------------------------------ */
uint32_t orc_decide_cell_size(const uint32_t* b, uint32_t n, int dims, uint32_t range,
                              uint64_t free_bytes) {
    int W = 2 * dims + 1;
    int nSamples = 1000 > (int)n ? (int)n : 1000;
    if (nSamples <= 0) nSamples = 1;
    float avg[3] = {0, 0, 0};
    for (int d = 0; d < dims; d++) {
        int acc = 0;
        for (int i = 0; i < nSamples && (uint32_t)i < n; i++) {
            float v = (float)(b[(uint64_t)i * W + 2 * d + 1] - b[(uint64_t)i * W + 2 * d]);
            acc = (int)((float)acc + v);
        }
        avg[d] = (float)(acc / nSamples);
    }
    int cs = 1;
    while ((uint32_t)(cs * 2) < range) cs *= 2;
    for (;;) {
        long long nrc = (range + (uint32_t)cs - 1) / (uint32_t)cs;
        long long nc = nrc * nrc;
        double nmr = (float)(1 + avg[0] / cs) * (float)(1 + avg[1] / cs);
        if (dims == 3) {
            nc *= nrc;
            nmr *= (float)(1 + avg[2] / cs);
        }
        int nRecsPerCell = (int)(nmr * n / nc);
        if (cs < avg[0]) break;
        if (nRecsPerCell < 32 || nmr > (dims == 3 ? 8 : 4)) break;
        if (cs == 1) break;
        uint32_t nrc32 = (range + (uint32_t)cs - 1) / (uint32_t)cs;
        uint32_t cells32 = dims == 3 ? nrc32 * nrc32 * nrc32 : nrc32 * nrc32;
        uint64_t need = (uint64_t)cells32 * sizeof(uint32_t) * 3;
        if (need >= free_bytes) break;
        cs /= 2;
    }
    return (uint32_t)(cs * 2);
}

/* ------------------------------------------------------------------ */
/* Grid geometry and cell enumeration                                   */
/* ------------------------------------------------------------------ */
typedef struct {
    int dims, merged;
    uint32_t shift, nrc, ncells;
    const uint32_t* boxes;
    uint32_t n;
    uint32_t *NRs, *StartI, *Merged, *Recs;
} grid_t;

/* Visit every cell of box `rid` (src/pbig/pbig.cu:174-221 precount,
 * :223-318 postcount, :321-427 mapping). With merging, a cell that belongs
 * to a merged block is replaced by the block root and counted only on the
 * first visit rule of the reference. `fn` receives the final cell id. */
typedef void (*visit_fn)(grid_t* g, uint32_t gid, uint32_t rid, void* ctx);

static void visit_cells(grid_t* g, uint32_t box, int use_merge, visit_fn fn, void* ctx) {
    const int W = 2 * g->dims + 1;
    const uint32_t* b = g->boxes + (uint64_t)box * W;
    const uint32_t rid = b[2 * g->dims];
    const uint32_t s = g->shift, nrc = g->nrc, nrc2 = nrc * nrc;
    uint32_t f_l = b[0] >> s, f_u = b[1] >> s, s_l = b[2] >> s, s_u = b[3] >> s;
    uint32_t t_l = 0, t_u = 0;
    if (g->dims == 3) { t_l = b[4] >> s; t_u = b[5] >> s; }
    int64_t zmin = -1;
    for (uint64_t k = t_l; k <= t_u; k++) {
        uint32_t product = (g->dims == 3) ? nrc2 * (uint32_t)k : 0u;
        int64_t ymin = -1;
        for (uint64_t j = s_l; j <= s_u; j++) {
            uint32_t m_gid = product + nrc * (uint32_t)j;
            int64_t xmin = -1;
            for (uint64_t i = f_l; i <= f_u; i++) {
                uint32_t gid = m_gid + (uint32_t)i;
                if (gid >= g->ncells) continue;
                if (use_merge && g->Merged[gid] != ORC_UNUSED) {
                    uint32_t mg = g->Merged[gid];
                    int64_t gx = (int32_t)(mg % nrc);
                    int64_t gy = g->dims == 3 ? (int32_t)((mg % nrc2) / nrc) : (int32_t)(mg / nrc);
                    int64_t gz = g->dims == 3 ? (int32_t)(mg / nrc2) : 0;
                    int ok = gx > xmin && gy > ymin && (g->dims == 2 || gz > zmin);
                    if (!ok) continue;
                    gid = mg;
                }
                xmin = (int64_t)i;
                fn(g, gid, rid, ctx);
            }
            ymin = (int64_t)j;
        }
        zmin = (int64_t)k;
    }
}

static void fn_count(grid_t* g, uint32_t gid, uint32_t rid, void* ctx) {
    (void)rid; (void)ctx;
    g->NRs[gid]++;
}
static void fn_map(grid_t* g, uint32_t gid, uint32_t rid, void* ctx) {
    uint32_t* cursor = (uint32_t*)ctx;
    g->Recs[cursor[gid]++] = rid;
}

/* ------------------------------------------------------------------ */
/* Cell merging: try_merge / h_merge_grids, src/pbig/pbig.cu:1066-1251   */
/* ------------------------------------------------------------------ */
static int try_merge(grid_t* g, uint32_t gid, int dir, uint32_t* h, uint32_t* v, uint32_t* u) {
    const uint32_t nrc = g->nrc, lim = ORC_NTPB;
    uint32_t acc = g->NRs[gid];
    uint32_t step1, step2, n1, n2, base;
    if (g->dims == 2) {
        step1 = 0; n1 = 1;
        step2 = dir == 0 ? nrc : 1;
        n2 = dir == 0 ? *v : *h;
        base = dir == 0 ? gid + *h : gid + (*v) * nrc;
    } else {
        if (dir == 0) { step1 = nrc * nrc; step2 = nrc; n1 = *u; n2 = *v; base = gid + *h; }
        else if (dir == 1) { step1 = nrc * nrc; step2 = 1; n1 = *u; n2 = *h; base = gid + (*v) * nrc; }
        else { step1 = nrc; step2 = 1; n1 = *v; n2 = *h; base = gid + (*u) * nrc * nrc; }
    }
    for (uint32_t a = 0; a < n1; a++)
        for (uint32_t c = 0; c < n2; c++)
            if (g->Merged[base + a * step1 + c * step2] != ORC_UNUSED) return 0;
    for (uint32_t a = 0; a < n1; a++)
        for (uint32_t c = 0; c < n2; c++) {
            acc += g->NRs[base + a * step1 + c * step2];
            if (acc > lim) return 0;
        }
    for (uint32_t a = 0; a < n1; a++)
        for (uint32_t c = 0; c < n2; c++) g->Merged[base + a * step1 + c * step2] = gid;
    g->Merged[gid] = gid;
    g->NRs[gid] = acc;
    if (dir == 0) (*h)++;
    else if (dir == 1) (*v)++;
    else (*u)++;
    return 1;
}

static void merge_grids(grid_t* g) {
    const uint32_t nrc = g->nrc;
    for (uint32_t i = 0; i < g->ncells; i++) {
        uint32_t h = 1, v = 1, u = 1;
        if (g->Merged[i] != ORC_UNUSED) continue;
        uint32_t gx = i % nrc;
        uint32_t gy = g->dims == 3 ? (i % (nrc * nrc)) / nrc : i / nrc;
        uint32_t gz = g->dims == 3 ? i / (nrc * nrc) : 0;
        int progress;
        do {
            progress = 0;
            if (gx + h < nrc) progress = try_merge(g, i, 0, &h, &v, &u);
            if (gy + v < nrc) progress += try_merge(g, i, 1, &h, &v, &u);
            if (g->dims == 3 && gz + u < nrc) progress += try_merge(g, i, 2, &h, &v, &u);
        } while (progress != 0);
    }
}

/* ------------------------------------------------------------------ */
/* Matching: d_matching with BALANCE=1, src/pbig/pbig.cu:641-932;        */
/* calcOverlaps :562-577 (closed intervals); calcRightToWrite :579-603. */
/* ------------------------------------------------------------------ */
typedef struct { uint32_t gid, seg_s; } job_t;  /* struct Job, pbig.cu:115-121 */

typedef struct {
    uint32_t* data;
    uint64_t n, cap;
} pairbuf;

static void pb_push(pairbuf* p, uint32_t a, uint32_t b) {
    if (p->n == p->cap) {
        uint64_t nc = p->cap ? p->cap * 2 : 4096;
        uint32_t* nd = (uint32_t*)realloc(p->data, nc * 2 * sizeof(uint32_t));
        if (!nd) return;
        p->data = nd;
        p->cap = nc;
    }
    p->data[2 * p->n] = a;
    p->data[2 * p->n + 1] = b;
    p->n++;
}

static inline int overlaps(const uint32_t* c1, const uint32_t* c2, int dims) {
    int r = (c1[0] <= c2[1]) + (c2[0] <= c1[1]) + (c1[2] <= c2[3]) + (c2[2] <= c1[3]);
    if (dims == 3) r += (c1[4] <= c2[5]) + (c2[4] <= c1[5]);
    return r;
}

static inline int right_to_write(const grid_t* g, uint32_t gid, const uint32_t* c1, const uint32_t* c2) {
    uint32_t s = g->shift, nrc = g->nrc;
    uint32_t f = (c1[0] > c2[0] ? c1[0] : c2[0]) >> s;
    uint32_t sl = (c1[2] > c2[2] ? c1[2] : c2[2]) >> s;
    uint32_t cid;
    if (g->dims == 3) {
        uint32_t t = (c1[4] > c2[4] ? c1[4] : c2[4]) >> s;
        cid = nrc * nrc * t + nrc * sl + f;
    } else {
        cid = nrc * sl + f;
    }
    if (g->merged && cid < g->ncells && g->Merged[cid] != ORC_UNUSED) cid = g->Merged[cid];
    return cid == gid;
}

typedef struct {
    grid_t* g;
    const job_t* jobs;
    uint64_t njobs;
    uint64_t* next;     /* shared job counter */
    int count_only;
    pairbuf out;
    uint64_t npairs, tests;
} match_ctx;

static void match_job(match_ctx* m, const job_t* jb) {
    grid_t* g = m->g;
    const int dims = g->dims, W = 2 * dims + 1, MATCHED = 2 * dims + 1;
    const uint32_t gid = jb->gid, n = g->NRs[gid], first = g->StartI[gid];
    const uint32_t seg = jb->seg_s, area_y = seg / ORC_NTPB;
    for (uint32_t t = 0; t < ORC_NTPB; t++) {
        if (seg + t >= n) break;
        uint32_t rid1 = g->Recs[first + seg + t];
        const uint32_t* c1 = g->boxes + (uint64_t)rid1 * W;
        for (uint32_t i = 0; i < n; i += ORC_NTPB) {
            uint32_t area_x = i / ORC_NTPB;
            int type;
            if (area_x == area_y) type = 1;
            else if ((area_y > area_x && ((area_x + area_y) & 1) == 1) ||
                     (area_y < area_x && ((area_x + area_y) & 1) == 0)) type = 2;
            else continue;
            uint32_t nx = (i + ORC_NTPB >= n) ? n - i : ORC_NTPB; /* Incr */
            uint32_t k, nElm;
            if (type == 1) {
                k = t + 1;
                nElm = (t < (nx >> 1)) ? (nx >> 1) : ((nx - 1) >> 1);
            } else {
                k = 0;
                nElm = nx;
            }
            for (uint32_t e = 0; e < nElm; e++, k++) {
                if (k >= nx) k = 0;
                uint32_t rid2 = g->Recs[first + i + k];
                const uint32_t* c2 = g->boxes + (uint64_t)rid2 * W;
                m->tests++;
                int res = overlaps(c1, c2, dims) + right_to_write(g, gid, c1, c2);
                if (res == MATCHED) {
                    m->npairs++;
                    if (!m->count_only) pb_push(&m->out, rid1 < rid2 ? rid1 : rid2, rid1 < rid2 ? rid2 : rid1);
                }
            }
        }
    }
}

static void* match_thread(void* arg) {
    match_ctx* m = (match_ctx*)arg;
    for (;;) {
        uint64_t j = __atomic_fetch_add(m->next, 16, __ATOMIC_RELAXED);
        if (j >= m->njobs) break;
        uint64_t e = j + 16 < m->njobs ? j + 16 : m->njobs;
        for (; j < e; j++) match_job(m, &m->jobs[j]);
    }
    return 0;
}

static int collect(match_ctx* ms, int threads, uint32_t* out, uint64_t cap, uint64_t* total) {
    uint64_t t = 0;
    for (int i = 0; i < threads; i++) t += ms[i].npairs;
    *total = t;
    if (out) {
        uint64_t o = 0;
        for (int i = 0; i < threads; i++) {
            uint64_t k = ms[i].out.n;
            if (o + k > cap) k = cap > o ? cap - o : 0;
            if (k) memcpy(out + 2 * o, ms[i].out.data, k * 2 * sizeof(uint32_t));
            o += k;
        }
    }
    for (int i = 0; i < threads; i++) free(ms[i].out.data);
    return (out && t > cap) ? 1 : 0;
}

/* Full reference pipeline on the CPU: plan (cell size), map (count, scan,
 * scatter), optional merge, sched (jobs of 256-row tiles) and match.
 * cs_in = 0 selects the reference heuristic. Returns 0, or 1 if `out` was
 * too small (stats->pairs still holds the full count), or -1 on error. */
int orc_grid_pairs(const uint32_t* boxes, uint32_t n, int dims, uint32_t range, uint32_t cs_in,
                   int merged, uint64_t free_bytes, int threads, uint32_t* out, uint64_t cap,
                   orc_stats* st) {
    memset(st, 0, sizeof *st);
    if (dims != 2 && dims != 3) return -1;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    grid_t g;
    memset(&g, 0, sizeof g);
    g.dims = dims; g.merged = merged; g.boxes = boxes; g.n = n;
    uint32_t cs = cs_in ? cs_in : orc_decide_cell_size(boxes, n, dims, range, free_bytes);
    g.shift = (uint32_t)log2((float)cs);          /* pbig.cu:1446 */
    g.nrc = (range + cs - 1) / cs;                /* pbig.cu:1368 */
    g.ncells = dims == 3 ? g.nrc * g.nrc * g.nrc : g.nrc * g.nrc;
    st->cs = cs; st->shift = g.shift; st->nrc = g.nrc; st->ncells = g.ncells;
    if (g.ncells == 0) return -1;

    g.NRs = (uint32_t*)calloc(g.ncells, 4);
    g.StartI = (uint32_t*)calloc(g.ncells, 4);
    g.Merged = (uint32_t*)malloc((uint64_t)g.ncells * 4);
    if (!g.NRs || !g.StartI || !g.Merged) return -1;
    for (uint32_t i = 0; i < g.ncells; i++) g.Merged[i] = ORC_UNUSED;

    /* map_phase, pbig.cu:1429-1584 */
    for (uint32_t r = 0; r < n; r++) visit_cells(&g, r, 0, fn_count, 0);
    if (merged) {
        merge_grids(&g);
        memset(g.NRs, 0, (uint64_t)g.ncells * 4);
        for (uint32_t r = 0; r < n; r++) visit_cells(&g, r, 1, fn_count, 0);
    }
    uint32_t acc = 0;
    for (uint32_t i = 0; i < g.ncells; i++) { g.StartI[i] = acc; acc += g.NRs[i]; }
    st->entries = acc;
    g.Recs = (uint32_t*)malloc((uint64_t)(acc ? acc : 1) * 4);
    uint32_t* cursor = (uint32_t*)malloc((uint64_t)g.ncells * 4);
    memcpy(cursor, g.StartI, (uint64_t)g.ncells * 4);
    for (uint32_t r = 0; r < n; r++) visit_cells(&g, r, merged, fn_map, cursor);
    free(cursor);

    /* sched_phase, pbig.cu:1586-1688 */
    uint64_t njobs = 0, accRecs = 0;
    for (uint32_t i = 0; i < g.ncells; i++) {
        uint32_t c = g.NRs[i];
        if (c > st->max_cell) st->max_cell = c;
        if (c <= 1) { accRecs += c; continue; }
        if (c >= ORC_MAX_BATCH_RECS) st->would_abort = 1;
        if (accRecs + c <= ORC_MAX_BATCH_RECS) accRecs += c;
        else { st->batches++; accRecs = c; }
        st->comp_pairs += (uint64_t)c * c / 2;
        njobs += (c + ORC_NTPB - 1) / ORC_NTPB;
    }
    st->batches++;
    st->jobs = njobs;
    job_t* jobs = (job_t*)malloc((njobs ? njobs : 1) * sizeof(job_t));
    uint64_t ji = 0;
    for (uint32_t i = 0; i < g.ncells; i++) {
        uint32_t c = g.NRs[i];
        if (c <= 1) continue;
        for (uint32_t s = 0; s < c; s += ORC_NTPB) { jobs[ji].gid = i; jobs[ji].seg_s = s; ji++; }
    }

    /* match_phase, pbig.cu:1694-1960 (work split over host threads) */
    match_ctx* ms = (match_ctx*)calloc(threads, sizeof(match_ctx));
    pthread_t* tid = (pthread_t*)calloc(threads, sizeof(pthread_t));
    uint64_t next = 0;
    for (int t = 0; t < threads; t++) {
        ms[t].g = &g; ms[t].jobs = jobs; ms[t].njobs = njobs; ms[t].next = &next;
        ms[t].count_only = out == 0;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tid[t], 0, match_thread, &ms[t]);
    match_thread(&ms[0]);
    for (int t = 1; t < threads; t++) pthread_join(tid[t], 0);
    for (int t = 0; t < threads; t++) st->tests += ms[t].tests;
    int rc = collect(ms, threads, out, cap, &st->pairs);
    free(ms); free(tid); free(jobs);
    free(g.NRs); free(g.StartI); free(g.Merged); free(g.Recs);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Independent checker: all-pairs brute force with the closed-interval  */
/* test of calcOverlaps (pbig.cu:562-577) and the soundness/uniqueness  */
/* semantics of checkOverlaps (pbig.cu:988-1023): a box never pairs     */
/* with itself; pairs are unordered.                                    */
/* ------------------------------------------------------------------ */
typedef struct {
    const uint32_t* boxes;
    uint32_t n;
    int dims;
    uint64_t* next;
    int count_only;
    pairbuf out;
    uint64_t npairs, tests;
} brute_ctx;

static void* brute_thread(void* arg) {
    brute_ctx* m = (brute_ctx*)arg;
    const int W = 2 * m->dims + 1;
    for (;;) {
        uint64_t a0 = __atomic_fetch_add(m->next, 64, __ATOMIC_RELAXED);
        if (a0 >= m->n) break;
        uint64_t a1 = a0 + 64 < m->n ? a0 + 64 : m->n;
        for (uint64_t a = a0; a < a1; a++) {
            const uint32_t* c1 = m->boxes + a * W;
            for (uint64_t b = a + 1; b < m->n; b++) {
                const uint32_t* c2 = m->boxes + b * W;
                if (overlaps(c1, c2, m->dims) == 2 * m->dims) {
                    m->npairs++;
                    if (!m->count_only) pb_push(&m->out, (uint32_t)a, (uint32_t)b);
                }
            }
        }
    }
    return 0;
}

int orc_brute_pairs(const uint32_t* boxes, uint32_t n, int dims, int threads, uint32_t* out,
                    uint64_t cap, uint64_t* npairs) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    brute_ctx* ms = (brute_ctx*)calloc(threads, sizeof(brute_ctx));
    pthread_t* tid = (pthread_t*)calloc(threads, sizeof(pthread_t));
    uint64_t next = 0;
    for (int t = 0; t < threads; t++) {
        ms[t].boxes = boxes; ms[t].n = n; ms[t].dims = dims; ms[t].next = &next;
        ms[t].count_only = out == 0;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tid[t], 0, brute_thread, &ms[t]);
    brute_thread(&ms[0]);
    for (int t = 1; t < threads; t++) pthread_join(tid[t], 0);
    match_ctx* mc = (match_ctx*)calloc(threads, sizeof(match_ctx));
    for (int t = 0; t < threads; t++) { mc[t].out = ms[t].out; mc[t].npairs = ms[t].npairs; }
    int rc = collect(mc, threads, out, cap, npairs);
    free(mc); free(ms); free(tid);
    return rc;
}

/* Sort canonical pairs (a<b) lexicographically, in place (radix sort on
 * the 64-bit key a<<32|b), so that outputs compare with memcmp. */
void orc_sort_pairs(uint32_t* pairs, uint64_t n) {
    if (n < 2) return;
    uint64_t* k = (uint64_t*)malloc(n * 8);
    uint64_t* t = (uint64_t*)malloc(n * 8);
    for (uint64_t i = 0; i < n; i++) k[i] = ((uint64_t)pairs[2 * i] << 32) | pairs[2 * i + 1];
    for (int pass = 0; pass < 4; pass++) {
        uint64_t cnt[65537];
        memset(cnt, 0, sizeof cnt);
        int sh = pass * 16;
        for (uint64_t i = 0; i < n; i++) cnt[((k[i] >> sh) & 0xffff) + 1]++;
        for (int b = 0; b < 65536; b++) cnt[b + 1] += cnt[b];
        for (uint64_t i = 0; i < n; i++) t[cnt[(k[i] >> sh) & 0xffff]++] = k[i];
        uint64_t* s = k; k = t; t = s;
    }
    for (uint64_t i = 0; i < n; i++) { pairs[2 * i] = (uint32_t)(k[i] >> 32); pairs[2 * i + 1] = (uint32_t)k[i]; }
    free(k); free(t);
}

/* ------------------------------------------------------------------ */
/* decode() of the Rice records, src/pbig/decode.cc:26-138 (RICE_COMPRESSION,
 * 8-byte words), with the column bytes read where the writer puts them:
 * record + 6 + k (the reference reads ((i+1)<<3)+2+k = record + 10 + k,
 * decode.cc:80, against the writer's overcnt = 6, pbig.cu:790, 851). The loop
 * follows the reference's; it stops at the end of the stream instead of
 * reading the word after it. Pairs come out as (min, max); returns the pair
 * count (out may be NULL to count), or -1 on a malformed stream.           */
/* ------------------------------------------------------------------ */
int64_t orc_decode_rice(const uint64_t* p, uint64_t cnt, const uint32_t* StartI, uint64_t ncells,
                        const uint32_t* Recs, uint64_t nrecs, uint32_t* out, uint64_t cap) {
    const uint64_t UNUSED = 0x0fffff11ull;
    const unsigned char* bytes = (const unsigned char*)p;
    const unsigned short* shorts = (const unsigned short*)p;
    uint64_t np = 0;
    for (uint64_t i = 2; i < cnt; i += 2) {
        if (p[i - 2] != UNUSED) return -1;
        uint64_t gid = p[i - 1];
        if (gid >= ncells) return -1;
        do {
            uint32_t seg1 = bytes[(i << 3) + 0];
            uint32_t seg2 = bytes[(i << 3) + 1];
            uint32_t l_rid = shorts[(i << 2) + 1];
            uint32_t nlaps = shorts[(i << 2) + 2];
            uint64_t base1 = (uint64_t)StartI[gid] + (seg1 << 8);
            uint64_t base2 = (uint64_t)StartI[gid] + (seg2 << 8);
            if (base1 + l_rid >= nrecs) return -1;
            uint32_t rid1 = Recs[base1 + l_rid];
            for (uint32_t k = 0; k < nlaps; k++) {
                uint32_t t = bytes[(i << 3) + 6 + k];
                if (base2 + t >= nrecs) return -1;
                uint32_t rid2 = Recs[base2 + t];
                if (out && np < cap) {
                    out[2 * np] = rid1 < rid2 ? rid1 : rid2;
                    out[2 * np + 1] = rid1 < rid2 ? rid2 : rid1;
                }
                np++;
            }
            i = i + ((6 + nlaps + sizeof(uint64_t) - 1) >> 3);
        } while (i < cnt && p[i] != UNUSED);
    }
    return (int64_t)np;
}
