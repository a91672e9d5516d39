/*
 * Seeded scene generators for the pair-detection workloads.
 *
 * Every variate is a pure function of (seed, stream, index): a counter-based
 * splitmix64 hash, so a box's coordinates do not depend on thread count or
 * on the machine. The transcendental functions below (log, exp, cos) are
 * written with IEEE-754 basic operations only (+ - * / sqrt, exact frexp and
 * ldexp) and this file is compiled with -ffp-contract=off, so x86-64 and
 * aarch64 hosts produce identical bytes.
 *
 * Boxes are produced in fp32 in [0,1) and quantised to the unsigned-int
 * coordinates of the PBIG API (rect.h: CType = unsigned int) with
 * maxRange R = 2^24:  q(f) = min(floor(f * 2^24), 2^24 - 1).
 * Output layout is PBIG's RectInfo: {xmin,xmax,ymin,ymax[,zmin,zmax],rid},
 * i.e. 2*dims+1 words per box, rid = index within the scene.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <pthread.h>
#include <stdlib.h>

#define QSCALE 16777216.0 /* 2^24 */
#define QMAX 16777215u

static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

/* counter-based hash: one 64-bit variate per (seed, stream, index) */
static inline uint64_t rng_u64(uint64_t seed, uint64_t stream, uint64_t idx) {
    uint64_t k = mix64(seed * 0x9e3779b97f4a7c15ULL + 0x632be59bd9b4e019ULL);
    k = mix64(k ^ (stream * 0xd1b54a32d192ed03ULL + 0x8cb92ba72f3d8dd7ULL));
    return mix64(k + (idx + 1) * 0x9e3779b97f4a7c15ULL);
}

/* uniform in [0,1) with 53 random bits */
static inline double u01(uint64_t seed, uint64_t stream, uint64_t idx) {
    return (double)(rng_u64(seed, stream, idx) >> 11) * (1.0 / 9007199254740992.0);
}

static const double LN2 = 0.6931471805599453094;
static const double TWO_PI = 6.283185307179586477;

/* natural log for x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
 * log m = 2 atanh(z), z = (m-1)/(m+1), |z| < 0.1716 -> 14 odd terms. */
double pbig_gen_log(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double z = (m - 1.0) / (m + 1.0);
    double z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 0; k < 14; k++) {
        sum = sum + term / (double)(2 * k + 1);
        term = term * z2;
    }
    return 2.0 * sum + (double)e * LN2;
}

/* exp(x) for |x| < 700: x = k ln2 + r, |r| <= ln2/2, Taylor to 22 terms */
double pbig_gen_exp(double x) {
    double kf = floor(x / LN2 + 0.5);
    double r = x - kf * LN2;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 22; k++) {
        term = term * r / (double)k;
        sum = sum + term;
    }
    return ldexp(sum, (int)kf);
}

/* cos(2*pi*u) for u in [0,1): reduce to t in [-1/2,1/2), a = 2*pi*t,
 * Taylor series of cos to a^36 (|a| <= pi). */
double pbig_gen_cos2pi(double u) {
    double t = u - floor(u + 0.5);
    double a = TWO_PI * t;
    double a2 = a * a;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 18; k++) {
        term = -term * a2 / (double)((2 * k - 1) * (2 * k));
        sum = sum + term;
    }
    return sum;
}

/* standard normal by Box-Muller (cosine branch) from two uniforms */
static inline double normal(uint64_t seed, uint64_t stream, uint64_t idx) {
    double u1 = 1.0 - u01(seed, stream, 2 * idx);     /* (0,1] */
    double u2 = u01(seed, stream, 2 * idx + 1);
    return sqrt(-2.0 * pbig_gen_log(u1)) * pbig_gen_cos2pi(u2);
}

static inline float clip01f(float f) {
    const float hi = 0x1.fffffep-1f; /* largest float below 1 */
    if (!(f > 0.0f)) return 0.0f;  /* also maps NaN to 0 */
    if (f > hi) return hi;
    return f;
}

static inline uint32_t quant(float f) {
    double v = floor((double)clip01f(f) * QSCALE);
    uint32_t q = (uint32_t)v;
    return q > QMAX ? QMAX : q;
}

/* write one box given its fp64 low/high corner per axis */
static inline void put_box(uint32_t* out, int dims, uint32_t rid, const double* lo, const double* hi) {
    for (int d = 0; d < dims; d++) {
        uint32_t a = quant((float)lo[d]);
        uint32_t b = quant((float)hi[d]);
        out[2 * d] = a;
        out[2 * d + 1] = b;
    }
    out[2 * dims] = rid;
}

/* ---- streams (one per kind of variate) ---- */
enum { S_LO = 1, S_SIDE = 2, S_COMP = 3, S_MEAN = 4, S_NORM = 5, S_LSIDE = 6,
       S_LARGE = 7, S_CENTRE = 8, S_SCENE = 9, S_MOVE = 10, S_PICK = 11 };

typedef struct {
    int kind;
    uint64_t seed;
    uint32_t* out;
    uint64_t begin, end;
    double p0, p1;           /* kind-specific parameters */
    const double* means;     /* mixture means (kind 2) */
} gen_job;

/* kind 1: 2-D, lower corner U[0,1)^2, side U[p0, p1] per axis */
static void gen_k1(const gen_job* j) {
    for (uint64_t i = j->begin; i < j->end; i++) {
        double lo[2], hi[2];
        for (int d = 0; d < 2; d++) {
            lo[d] = u01(j->seed, S_LO, 2 * i + d);
            double s = j->p0 + (j->p1 - j->p0) * u01(j->seed, S_SIDE, 2 * i + d);
            hi[d] = lo[d] + s;
        }
        put_box(j->out + i * 5, 2, (uint32_t)i, lo, hi);
    }
}

/* kind 2: 3-D Gaussian mixture (64 components, sigma p0), lognormal sides
 * exp(N(ln 0.002, p1^2)); centres clipped to [0,1). */
static void gen_k2(const gen_job* j) {
    const double mu = pbig_gen_log(0.002);
    for (uint64_t i = j->begin; i < j->end; i++) {
        uint32_t comp = (uint32_t)(rng_u64(j->seed, S_COMP, i) & 63u);
        double lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            double c = j->means[3 * comp + d] + j->p0 * normal(j->seed, S_NORM, 3 * i + d);
            if (c < 0.0) c = 0.0;
            if (c >= 1.0) c = 0x1.fffffffffffffp-1;
            double s = pbig_gen_exp(mu + j->p1 * normal(j->seed, S_LSIDE, 3 * i + d));
            lo[d] = c - 0.5 * s;
            hi[d] = c + 0.5 * s;
        }
        put_box(j->out + i * 7, 3, (uint32_t)i, lo, hi);
    }
}

/* kind 3: 3-D uniform centres, side U[0.001,0.004]; a box is large with
 * probability p0 (side U[0.02,0.1]). */
static void gen_k3(const gen_job* j) {
    for (uint64_t i = j->begin; i < j->end; i++) {
        int large = u01(j->seed, S_LARGE, i) < j->p0;
        double lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            double c = u01(j->seed, S_CENTRE, 3 * i + d);
            double u = u01(j->seed, S_SIDE, 3 * i + d);
            double s = large ? 0.02 + 0.08 * u : 0.001 + 0.003 * u;
            lo[d] = c - 0.5 * s;
            hi[d] = c + 0.5 * s;
        }
        put_box(j->out + i * 7, 3, (uint32_t)i, lo, hi);
    }
}

/* kind 4: one batched/serving scene of n = p1 boxes: uniform centres,
 * side U[0.5,2.0] * n^(-1/3) * 0.5 per axis. */
static void gen_k4(const gen_job* j) {
    double scale = 0.5 * pbig_gen_exp(-pbig_gen_log(j->p1) / 3.0);
    for (uint64_t i = j->begin; i < j->end; i++) {
        double lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            double c = u01(j->seed, S_CENTRE, 3 * i + d);
            double s = (0.5 + 1.5 * u01(j->seed, S_SIDE, 3 * i + d)) * scale;
            lo[d] = c - 0.5 * s;
            hi[d] = c + 0.5 * s;
        }
        put_box(j->out + i * 7, 3, (uint32_t)i, lo, hi);
    }
}

static void* gen_thread(void* arg) {
    const gen_job* j = (const gen_job*)arg;
    switch (j->kind) {
        case 1: gen_k1(j); break;
        case 2: gen_k2(j); break;
        case 3: gen_k3(j); break;
        case 4: gen_k4(j); break;
    }
    return 0;
}

static int run_jobs(gen_job proto, uint64_t n, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    if ((uint64_t)threads > n / 4096 + 1) threads = (int)(n / 4096 + 1);
    pthread_t tid[64];
    gen_job jobs[64];
    for (int t = 0; t < threads; t++) {
        jobs[t] = proto;
        jobs[t].begin = n * t / threads;
        jobs[t].end = n * (t + 1) / threads;
    }
    for (int t = 1; t < threads; t++) pthread_create(&tid[t], 0, gen_thread, &jobs[t]);
    gen_thread(&jobs[0]);
    for (int t = 1; t < threads; t++) pthread_join(tid[t], 0);
    return 0;
}

/* 2-D self-intersection scene: lower corners U[0,1)^2, sides U[lo,hi] */
int pbig_gen_uniform2d(uint64_t n, uint64_t seed, double side_lo, double side_hi,
                       uint32_t* out, int threads) {
    gen_job j; memset(&j, 0, sizeof j);
    j.kind = 1; j.seed = seed; j.out = out; j.p0 = side_lo; j.p1 = side_hi;
    return run_jobs(j, n, threads);
}

/* 3-D clustered scene: 64 Gaussian components, means U[0.1,0.9]^3 */
int pbig_gen_clustered3d(uint64_t n, uint64_t seed, double sigma, double log_sigma,
                         uint32_t* out, int threads) {
    double means[64 * 3];
    for (int m = 0; m < 64 * 3; m++) means[m] = 0.1 + 0.8 * u01(seed, S_MEAN, (uint64_t)m);
    gen_job j; memset(&j, 0, sizeof j);
    j.kind = 2; j.seed = seed; j.out = out; j.p0 = sigma; j.p1 = log_sigma; j.means = means;
    return run_jobs(j, n, threads);
}

/* 3-D uniform scene with a fraction of large boxes (one colour of the
 * red/blue bipartite workload) */
int pbig_gen_mixed3d(uint64_t n, uint64_t seed, double large_frac, uint32_t* out, int threads) {
    gen_job j; memset(&j, 0, sizeof j);
    j.kind = 3; j.seed = seed; j.out = out; j.p0 = large_frac;
    return run_jobs(j, n, threads);
}

/* 3-D uniform scene whose side scale follows its size (batched scenes) */
int pbig_gen_scene3d(uint64_t n, uint64_t seed, uint32_t* out, int threads) {
    gen_job j; memset(&j, 0, sizeof j);
    j.kind = 4; j.seed = seed; j.out = out; j.p1 = (double)n;
    return run_jobs(j, n, threads);
}

/* log-uniform integer in [lo, hi]: floor(lo * (hi/lo)^u), u = U[0,1) */
uint64_t pbig_gen_loguniform(uint64_t seed, uint64_t idx, double lo, double hi) {
    double u = u01(seed, S_SCENE, idx);
    double v = lo * pbig_gen_exp(u * pbig_gen_log(hi / lo));
    uint64_t r = (uint64_t)floor(v);
    if (r < (uint64_t)lo) r = (uint64_t)lo;
    if (r > (uint64_t)hi) r = (uint64_t)hi;
    return r;
}

/* uniform double in [0,1) / standard normal on a named stream: used by
 * the serving-loop arrival process and incremental-update generator */
double pbig_gen_uniform(uint64_t seed, uint64_t stream, uint64_t idx) {
    return u01(seed, stream, idx);
}
double pbig_gen_normal(uint64_t seed, uint64_t stream, uint64_t idx) {
    return normal(seed, stream, idx);
}

/* k distinct indices in [0, n), sorted: one per stratum -- index j is drawn
 * uniformly from [j*n/k, (j+1)*n/k) -- so no sort is needed. */
int pbig_gen_pick(uint64_t n, uint64_t k, uint64_t seed, uint32_t* out) {
    if (n == 0 || k == 0 || k > n) return -1;
    for (uint64_t j = 0; j < k; j++) {
        const uint64_t lo = (uint64_t)(((unsigned __int128)j * n) / k);
        const uint64_t hi = (uint64_t)(((unsigned __int128)(j + 1) * n) / k);
        out[j] = (uint32_t)(lo + rng_u64(seed, S_PICK, j) % (hi - lo));
    }
    return 0;
}

/* Move boxes of a resident 3-D scene: for each listed box, shift it by
 * N(0, sigma) per axis (in [0,1) units), keeping its extent, and
 * re-quantise. idx[] are box indices, k of them. */
/* Division-free variants of the log and cos2pi series above for the update
 * stream (same expansions; the reciprocal coefficients are compile-time
 * constants, so results differ from pbig_gen_log/cos2pi by rounding only). */
static const double INV_ODD[14] = {1.0, 1.0 / 3, 1.0 / 5, 1.0 / 7, 1.0 / 9, 1.0 / 11, 1.0 / 13,
                                   1.0 / 15, 1.0 / 17, 1.0 / 19, 1.0 / 21, 1.0 / 23, 1.0 / 25, 1.0 / 27};
static const double COS_C[18] = {1.0 / 2, 1.0 / 12, 1.0 / 30, 1.0 / 56, 1.0 / 90, 1.0 / 132,
                                 1.0 / 182, 1.0 / 240, 1.0 / 306, 1.0 / 380, 1.0 / 462, 1.0 / 552,
                                 1.0 / 650, 1.0 / 756, 1.0 / 870, 1.0 / 992, 1.0 / 1122, 1.0 / 1260};

static double log_nodiv(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double z = (m - 1.0) / (m + 1.0);
    double z2 = z * z, acc = 0.0;
    for (int k = 13; k >= 0; k--) acc = acc * z2 + INV_ODD[k];
    return 2.0 * z * acc + (double)e * LN2;
}

static double cos2pi_nodiv(double u) {
    double t = u - floor(u + 0.5);
    double a = TWO_PI * t;
    double a2 = a * a, acc = 1.0;
    /* cos a = 1 - a2/(1*2) (1 - a2/(3*4) (1 - ...)) */
    for (int k = 17; k >= 0; k--) acc = 1.0 - a2 * COS_C[k] * acc;
    return acc;
}

static inline double normal_nodiv(uint64_t seed, uint64_t stream, uint64_t idx) {
    double u1 = 1.0 - u01(seed, stream, 2 * idx);
    double u2 = u01(seed, stream, 2 * idx + 1);
    return sqrt(-2.0 * log_nodiv(u1)) * cos2pi_nodiv(u2);
}

int pbig_gen_move3d(uint32_t* boxes, const uint32_t* idx, uint64_t k, uint64_t seed, double sigma) {
    for (uint64_t t = 0; t < k; t++) {
        uint32_t* b = boxes + (uint64_t)idx[t] * 7;
        double lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            double dx = sigma * normal_nodiv(seed, S_MOVE, 3 * t + d);
            double a = (double)b[2 * d] / QSCALE, c = (double)b[2 * d + 1] / QSCALE;
            lo[d] = a + dx;
            hi[d] = c + dx;
        }
        put_box(b, 3, b[6], lo, hi);
    }
    return 0;
}

double pbig_gen_log_nodiv(double x) { return log_nodiv(x); }
double pbig_gen_cos2pi_nodiv(double u) { return cos2pi_nodiv(u); }
