/*
 * oracle.c -- CPU restatement of ParAGraph's per-epoch growth step (C99 + OpenMP).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine and the timed CPU baseline.  The
 * product never calls it.  Parity against the reference is unpinned (the reference has no tests
 * or fixed seeds and cannot be built here); see oracle.h.
 *
 * Built with -O2 -ffp-contract=off and no fast-math so every floating-point operation rounds once,
 * exactly as the device code does.
 *
 * What each part restates:
 *   og_load           Graph::ParseEdgelist/AddEdge set semantics (src/graph.cu:376-447,820-826):
 *                     duplicate edges collapse, self-loops stay; rows kept sorted like std::set.
 *   weights / CDF     the per-epoch score preparation of execute() (src/kernel.cu:1698-1706,
 *                     src/abm.cu:112-208,324-338), with the baseline weight functor
 *                     w_j = f_j^g (indeg_j+1)^a exp(-(t-t_j)/tau) instead of the linear mix.
 *   neighbourhood     the 2-hop undirected ball of GetOneAndTwoHopNeighborhood
 *                     (src/abm.cu:577-682): forward and backward rows of the anchors and of their
 *                     neighbours.
 *   sampling          weighted sampling without replacement with weights w_j beta^[j in N_a].
 *                     The reference draws Efraimidis-Spirakis keys log(u)/score and keeps a top-k
 *                     heap (src/abm.cu:461-565, gpu-std/device_min_heap.cuh:71-145).  Two
 *                     restatements of that law, each consuming its own Philox streams:
 *                     sample_agent_thin (default): one Poisson event stream with rate beta w_j,
 *                       each event global (kept) with probability 1/beta or boost (kept iff the
 *                       node is in the ball); the first k distinct kept nodes are the sample;
 *                     sample_agent (enumeration): a global race of sequential inverse-CDF draws
 *                       without replacement merged with a neighbourhood race over the enumerated
 *                       ball (keys E/w_j, k smallest).
 *   edge emit         ABMKernelStage4 (src/abm.cu:958-994): one (agent, cited) edge per choice.
 *   CSR append        the host edge insert and updateNodeInDegreeOutDegree
 *                     (src/kernel.cu:1766-1815, src/graph.cu:537-618).
 *   ER                G(n,p) against pre-epoch nodes, as recorded in
 *                     results/slurm-8634746.out:60-73, by geometric skips.
 */
#include "oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ Philox4x32-10 */
/* Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11. */
void og_philox(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]) {
    uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
    uint32_t key0 = k[0], key1 = k[1];
    for (int round = 0; round < 10; round++) {
        if (round) {
            key0 += 0x9E3779B9u;
            key1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ key0;
        uint32_t y1 = (uint32_t)p1;
        uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ key1;
        uint32_t y3 = (uint32_t)p0;
        x0 = y0;
        x1 = y1;
        x2 = y2;
        x3 = y3;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
}

enum { S_OUTDEG = 1, S_ANCHOR = 2, S_GLOBAL = 3, S_BOOST = 4, S_FIT = 5, S_ER = 6 };

static void rng(uint64_t seed, uint32_t stream, uint32_t aux, uint32_t epoch, uint32_t unit,
                uint32_t i, uint32_t out[4]) {
    uint32_t c[4] = {i, unit, epoch, (stream << 24) | (aux & 0xFFFFFFu)};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    og_philox(c, k, out);
}

static float unif_f(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }
static double unif_d(uint32_t lo, uint32_t hi) {
    uint64_t v = ((((uint64_t)hi) << 32) | lo) >> 11;
    return (double)(v + 1u) * 0x1p-53;
}
static uint64_t join64(uint32_t lo, uint32_t hi) { return (((uint64_t)hi) << 32) | lo; }
static uint64_t hi_mul64(uint64_t a, uint64_t b) {
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
}

/* ------------------------------------------------------------------ elementary functions */
/* exp: Cody-Waite reduction + Taylor series; log: atanh series on the mantissa.  Same published
 * methods and the same rounded series coefficients as the engine, written out independently. */
static float f_from_bits(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static uint32_t bits_of_f(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static double d_from_bits(uint64_t u) {
    double d;
    memcpy(&d, &u, 8);
    return d;
}
static uint64_t bits_of_d(double d) {
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
}

float og_expf(float x) {
    if (isnan(x)) return x;
    if (x > 88.0f) return INFINITY;
    if (x < -87.0f) return 0.0f;
    float k = rintf(x * 0x1.715476p+0f);
    float r = fmaf(-k, 0x1.62e430p-1f, x);
    r = fmaf(-k, -0x1.05c610p-29f, r);
    static const float c[8] = {0x1.a01a02p-13f, 0x1.6c16c2p-10f, 0x1.111112p-7f, 0x1.555556p-5f,
                               0x1.555556p-3f,  0x1.0p-1f,       1.0f,           1.0f};
    float p = c[0];
    for (int i = 1; i < 8; i++) p = fmaf(p, r, c[i]);
    int ki = (int)k;
    return p * f_from_bits((uint32_t)(ki + 127) << 23);
}

float og_logf(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int adj = 0;
    if (x < 0x1p-126f) {
        x *= 0x1p23f;
        adj = -23;
    }
    uint32_t b = bits_of_f(x);
    int e = (int)(b >> 23) - 127 + adj;
    float m = f_from_bits((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 0x1.6a09e6p+0f) {
        m *= 0.5f;
        e++;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    static const float c[4] = {0x1.c71c72p-4f, 0x1.24924ap-3f, 0x1.99999ap-3f, 0x1.555556p-2f};
    float p = c[0];
    for (int i = 1; i < 4; i++) p = fmaf(p, z, c[i]);
    float t = s + s;
    float lm = fmaf(t * z, p, t);
    float ef = (float)e;
    return fmaf(ef, 0x1.62e430p-1f, fmaf(ef, -0x1.05c610p-29f, lm));
}

double og_logf_max_ulp(float lo, float hi) {
    uint32_t a = bits_of_f(lo), b = bits_of_f(hi);
    double worst = 0.0;
#pragma omp parallel for schedule(static) reduction(max : worst)
    for (int64_t i = (int64_t)a; i <= (int64_t)b; i++) {
        const float x = f_from_bits((uint32_t)i);
        const double t = log((double)x);
        const float tf = (float)t;
        if (tf == 0.0f) continue;
        const double ulp = fabs((double)nextafterf(tf, 0.0f) - (double)tf);
        const double e = fabs((double)og_logf(x) - t) / ulp;
        if (e > worst) worst = e;
    }
    return worst;
}

double og_exp(double x) {
    if (isnan(x)) return x;
    if (x > 709.0) return INFINITY;
    if (x < -708.0) return 0.0;
    double k = rint(x * 0x1.71547652b82fep+0);
    double r = fma(-k, 0x1.62e42fefa39efp-1, x);
    r = fma(-k, 0x1.abc9e3b39803fp-56, r);
    static const double c[14] = {
        0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26, 0x1.27e4fb7789f5cp-22,
        0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10,
        0x1.1111111111111p-7,  0x1.5555555555555p-5,  0x1.5555555555555p-3,  0x1.0p-1,
        1.0,                   1.0};
    double p = c[0];
    for (int i = 1; i < 14; i++) p = fma(p, r, c[i]);
    int64_t ki = (int64_t)k;
    return p * d_from_bits((uint64_t)(ki + 1023) << 52);
}

double og_log(double x) {
    if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int adj = 0;
    if (x < 0x1p-1022) {
        x *= 0x1p52;
        adj = -52;
    }
    uint64_t b = bits_of_d(x);
    int e = (int)(b >> 52) - 1023 + adj;
    double m = d_from_bits((b & 0xFFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
    if (m > 0x1.6a09e667f3bcdp+0) {
        m *= 0.5;
        e++;
    }
    double s = (m - 1.0) / (m + 1.0);
    double z = s * s;
    static const double c[11] = {0x1.642c8590b2164p-5, 0x1.8618618618618p-5, 0x1.af286bca1af28p-5,
                                 0x1.e1e1e1e1e1e1ep-5, 0x1.1111111111111p-4, 0x1.3b13b13b13b14p-4,
                                 0x1.745d1745d1746p-4, 0x1.c71c71c71c71cp-4, 0x1.2492492492492p-3,
                                 0x1.999999999999ap-3, 0x1.5555555555555p-2};
    double p = c[0];
    for (int i = 1; i < 11; i++) p = fma(p, z, c[i]);
    double t = s + s;
    double lm = fma(t * z, p, t);
    double ef = (double)e;
    return fma(ef, 0x1.62e42fefa39efp-1, fma(ef, 0x1.abc9e3b39803fp-56, lm));
}

#define OG_TABLE 257 /* out-degrees 0..256 */
#define OG_RC_FIT_MAX 1000 /* peak fitness values 1..1000 */

/* Poisson(lambda) CDF * 2^64, saturating; the out-degree law of the baseline configs. */
void og_poisson_table(double lambda, uint64_t* table) {
    double p = og_exp(-lambda), cdf = p;
    for (int i = 0; i < OG_TABLE; i++) {
        if (i > 0) {
            p = p * lambda / (double)i;
            cdf = cdf + p;
        }
        if (cdf >= 1.0 || i == OG_TABLE - 1)
            table[i] = UINT64_MAX;
        else
            table[i] = (uint64_t)(cdf * 0x1p64);
    }
}

/* lognormal(0,1) by the Marsaglia polar method */
float og_fitness(uint64_t seed, uint32_t replica, uint32_t epoch, uint32_t unit) {
    for (uint32_t i = 0; i < 32; i++) {
        uint32_t r[4];
        rng(seed, S_FIT, replica, epoch, unit, i, r);
        for (int h = 0; h < 2; h++) {
            float v1 = 2.0f * unif_f(r[2 * h]) - 1.0f;
            float v2 = 2.0f * unif_f(r[2 * h + 1]) - 1.0f;
            float s = v1 * v1 + v2 * v2;
            if (s < 1.0f && s > 0.0f) return og_expf(v1 * sqrtf(-2.0f * og_logf(s) / s));
        }
    }
    return 1.0f;
}

/* ------------------------------------------------------------------ graph state */
struct og_graph {
    uint64_t seed;
    uint32_t replica;
    int64_t epoch;
    /* params */
    float alpha_f, gamma_f, tau_f;
    double beta_m1, p_global, lambda, growth_rate;
    int64_t fixed_new;
    int anchors;
    int sampler; /* 0 thinning, 1 neighbourhood enumeration */
    int64_t hub_thr; /* degree from which a node is a hub this epoch (thinning counters) */
    uint64_t table[OG_TABLE];
    /* nodes */
    int64_t n;
    int32_t* pub;
    float* fit;
    int32_t* indeg;
    /* CSR */
    int64_t m;
    int64_t* fwd_off;
    int32_t* fwd_col;
    int64_t* bwd_off;
    int32_t* bwd_col;
    /* last epoch */
    int64_t last_first, last_count;
    int32_t* arrivals;
    int64_t stats[6];
    float* w;
    uint64_t* cdf;
    int64_t w_n;
    int32_t shift;
    /* refcompat functor (og_rc_configure) */
    int rc;
    double rc_w[3], rc_alpha, rc_frc, rc_sy, rc_growth;
    int rc_gamma, rc_decay;
    uint64_t rc_bag[OG_TABLE];
    uint64_t rc_fit_table[OG_RC_FIT_MAX];
    double* rc_rec;
    int rc_rec_len;
    int32_t* rc_lag; /* per node: fitness lag and peak duration (the peak value is fit[]) */
    int32_t* rc_dur;
    double* rc_agents; /* last epoch, per agent: pa, rec, fit weights, alpha, generator, out-degree */
};

og_graph* og_create(uint64_t seed, uint32_t replica) {
    og_graph* g = (og_graph*)calloc(1, sizeof(og_graph));
    g->seed = seed;
    g->replica = replica;
    og_set_params(g, 1.0, 5.0, 1.0, 4.0, 15.0, 0.0, 0, 3);
    return g;
}

void og_destroy(og_graph* g) {
    if (!g) return;
    free(g->pub);
    free(g->fit);
    free(g->indeg);
    free(g->fwd_off);
    free(g->fwd_col);
    free(g->bwd_off);
    free(g->bwd_col);
    free(g->arrivals);
    free(g->w);
    free(g->cdf);
    free(g->rc_rec);
    free(g->rc_lag);
    free(g->rc_dur);
    free(g->rc_agents);
    free(g);
}

int og_set_params(og_graph* g, double alpha, double tau, double gamma, double beta, double lambda,
                  double growth_rate, int64_t fixed_new, int32_t num_anchors) {
    if (!(tau > 0) || !(beta >= 1.0) || num_anchors < 1 || num_anchors > 4 || !(lambda >= 0))
        return 3;
    g->alpha_f = (float)alpha;
    g->gamma_f = (float)gamma;
    g->tau_f = (float)tau;
    g->beta_m1 = beta - 1.0;
    g->p_global = 1.0 / beta;
    g->lambda = lambda;
    g->growth_rate = growth_rate;
    g->fixed_new = fixed_new;
    g->anchors = num_anchors;
    og_poisson_table(lambda, g->table);
    return 0;
}

void og_set_epoch(og_graph* g, int64_t epoch) { g->epoch = epoch; }
void og_set_sampler(og_graph* g, int sampler) { g->sampler = sampler; }
int64_t og_epoch(const og_graph* g) { return g->epoch; }

static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

typedef struct {
    int32_t a, b;
} pair32;
static int cmp_pair(const void* x, const void* y) {
    const pair32* p = (const pair32*)x;
    const pair32* q = (const pair32*)y;
    if (p->a != q->a) return (p->a > q->a) - (p->a < q->a);
    return (p->b > q->b) - (p->b < q->b);
}

/* Build CSR (sorted rows, duplicates collapsed) from an edge list. */
static void build_csr(int64_t n, int64_t m, const int32_t* src, const int32_t* dst, int64_t** off_out,
                      int32_t** col_out, int64_t* m_out) {
    pair32* e = (pair32*)malloc(sizeof(pair32) * (size_t)(m > 0 ? m : 1));
    for (int64_t i = 0; i < m; i++) {
        e[i].a = src[i];
        e[i].b = dst[i];
    }
    qsort(e, (size_t)m, sizeof(pair32), cmp_pair);
    int64_t u = 0;
    for (int64_t i = 0; i < m; i++)
        if (i == 0 || e[i].a != e[i - 1].a || e[i].b != e[i - 1].b) e[u++] = e[i];
    int64_t* off = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int32_t* col = (int32_t*)malloc(sizeof(int32_t) * (size_t)(u > 0 ? u : 1));
    for (int64_t i = 0; i < u; i++) off[e[i].a + 1]++;
    for (int64_t i = 0; i < n; i++) off[i + 1] += off[i];
    for (int64_t i = 0; i < u; i++) col[i] = e[i].b;
    free(e);
    *off_out = off;
    *col_out = col;
    *m_out = u;
}

int og_load(og_graph* g, int64_t n, const int32_t* pub, const float* fitness, int64_t m,
            const int32_t* src, const int32_t* dst) {
    if (n <= 0) return 3;
    for (int64_t i = 0; i < m; i++)
        if (src[i] < 0 || src[i] >= n || dst[i] < 0 || dst[i] >= n) return 3;
    g->n = n;
    g->pub = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    g->fit = (float*)malloc(sizeof(float) * (size_t)n);
    g->indeg = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    memcpy(g->pub, pub, sizeof(int32_t) * (size_t)n);
    memcpy(g->fit, fitness, sizeof(float) * (size_t)n);
    build_csr(n, m, src, dst, &g->fwd_off, &g->fwd_col, &g->m);
    int64_t mb;
    build_csr(n, m, dst, src, &g->bwd_off, &g->bwd_col, &mb);
    for (int64_t i = 0; i < n; i++) g->indeg[i] = (int32_t)(g->bwd_off[i + 1] - g->bwd_off[i]);
    return 0;
}

/* ------------------------------------------------------------------ CSR append */
/* Appends rows for `delta` new nodes (their forward rows given in agent order, each sorted) and
 * the matching backward entries; the appended part of every backward row is in agent order, which
 * is ascending source id.  Restates the host insert of execute() (src/kernel.cu:1766-1815) and
 * updateNodeInDegreeOutDegree (src/graph.cu:537-618). */
static void append_rows(og_graph* g, int64_t delta, const int64_t* row_off, const int32_t* rows,
                        int32_t new_pub, const float* new_fit) {
    int64_t n = g->n, n2 = n + delta;
    int64_t e_new = row_off[delta];
    /* forward */
    int64_t* fo = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n2 + 1));
    memcpy(fo, g->fwd_off, sizeof(int64_t) * (size_t)(n + 1));
    for (int64_t a = 0; a < delta; a++) fo[n + a + 1] = g->m + row_off[a + 1];
    int32_t* fc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->m + e_new + 1));
    memcpy(fc, g->fwd_col, sizeof(int32_t) * (size_t)g->m);
    memcpy(fc + g->m, rows, sizeof(int32_t) * (size_t)e_new);
    /* backward */
    int64_t* inc = (int64_t*)calloc((size_t)n2, sizeof(int64_t));
    for (int64_t i = 0; i < e_new; i++) inc[rows[i]]++;
    int64_t* bo = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n2 + 1));
    bo[0] = 0;
    for (int64_t j = 0; j < n2; j++) {
        int64_t old = j < n ? g->bwd_off[j + 1] - g->bwd_off[j] : 0;
        bo[j + 1] = bo[j] + old + inc[j];
    }
    int32_t* bc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(bo[n2] + 1));
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)n2);
    for (int64_t j = 0; j < n2; j++) {
        int64_t old = j < n ? g->bwd_off[j + 1] - g->bwd_off[j] : 0;
        if (old) memcpy(bc + bo[j], g->bwd_col + g->bwd_off[j], sizeof(int32_t) * (size_t)old);
        cur[j] = bo[j] + old;
    }
    for (int64_t a = 0; a < delta; a++)
        for (int64_t i = row_off[a]; i < row_off[a + 1]; i++) bc[cur[rows[i]]++] = (int32_t)(n + a);
    /* nodes */
    g->pub = (int32_t*)realloc(g->pub, sizeof(int32_t) * (size_t)n2);
    g->fit = (float*)realloc(g->fit, sizeof(float) * (size_t)n2);
    g->indeg = (int32_t*)realloc(g->indeg, sizeof(int32_t) * (size_t)n2);
    for (int64_t a = 0; a < delta; a++) {
        g->pub[n + a] = new_pub;
        g->fit[n + a] = new_fit[a];
        g->indeg[n + a] = 0;
    }
    for (int64_t j = 0; j < n2; j++) g->indeg[j] += (int32_t)inc[j];
    free(g->fwd_off);
    free(g->fwd_col);
    free(g->bwd_off);
    free(g->bwd_col);
    g->fwd_off = fo;
    g->fwd_col = fc;
    g->bwd_off = bo;
    g->bwd_col = bc;
    g->last_first = g->m;
    g->last_count = e_new;
    g->m += e_new;
    g->n = n2;
    free(inc);
    free(cur);
}

/* ------------------------------------------------------------------ PA epoch */
typedef struct {
    float key;
    int32_t id;
} keyed;
static int keyed_less(keyed x, keyed y) { return x.key < y.key || (x.key == y.key && x.id < y.id); }
static int cmp_keyed(const void* a, const void* b) {
    keyed x = *(const keyed*)a, y = *(const keyed*)b;
    return keyed_less(x, y) ? -1 : (keyed_less(y, x) ? 1 : 0);
}

typedef struct {
    keyed* v;
    int64_t n, cap;
} keyvec;
static void kv_push(keyvec* kv, keyed x) {
    if (kv->n == kv->cap) {
        kv->cap = kv->cap ? kv->cap * 2 : 1024;
        kv->v = (keyed*)realloc(kv->v, sizeof(keyed) * (size_t)kv->cap);
    }
    kv->v[kv->n++] = x;
}

/* Sample one agent; writes k sorted citations to out_sorted and the arrival order to out_arr.
 * Returns k.  Counters: cnt[0] rows expanded, cnt[1] elements keyed. */
static int sample_agent(const og_graph* g, int64_t a, const float* w, const uint64_t* cdf,
                        int shift, int64_t npos, int32_t* out_sorted, int32_t* out_arr,
                        int64_t* cnt, keyvec* kv) {
    const int64_t n = g->n;
    const uint32_t ep = (uint32_t)g->epoch, rep = g->replica, unit = (uint32_t)a;
    uint32_t r[4];
    /* out-degree: Poisson via the CDF table, clipped to [1, min(n, npos)] */
    rng(g->seed, S_OUTDEG, rep, ep, unit, 0, r);
    uint64_t u = join64(r[0], r[1]);
    int kraw = OG_TABLE - 1;
    for (int i = 0; i < OG_TABLE; i++)
        if (u < g->table[i]) {
            kraw = i;
            break;
        }
    int64_t k = kraw < 1 ? 1 : kraw;
    if (k > n) k = n;
    if (k > npos) k = npos;
    /* anchors: uniform over existing nodes (getGeneratorNode, src/abm.cu:567-574) */
    int32_t anchor[4];
    rng(g->seed, S_ANCHOR, rep, ep, unit, 0, r);
    for (int i = 0; i < g->anchors; i++) anchor[i] = (int32_t)(((uint64_t)r[i] * (uint64_t)n) >> 32);

    /* global race: k sequential inverse-CDF draws without replacement */
    int32_t g_id[256];
    double g_t[256];
    int32_t c_id[256];   /* chosen ids, ascending */
    uint64_t c_q[256];   /* their quantised weights */
    int nc = 0;
    uint64_t R = cdf[n - 1];
    double t = 0.0;
    const double unit_scale = d_from_bits((uint64_t)(1023 - shift) << 52); /* 2^-shift */
    for (int64_t i = 0; i < k; i++) {
        if (R == 0) break;
        rng(g->seed, S_GLOBAL, rep, ep, unit, (uint32_t)i, r);
        double E = -og_log(unif_d(r[0], r[1]));
        double Rd = (double)R * unit_scale;
        t = t + E / Rd;
        uint64_t y = hi_mul64(join64(r[2], r[3]), R);
        /* smallest j with cdf[j] - C(j) > y; C(j) = sum of chosen q with id <= j */
        int64_t lo = 0, hi = n - 1;
        while (lo < hi) {
            int64_t mid = lo + (hi - lo) / 2;
            uint64_t cm = 0;
            for (int c = 0; c < nc && c_id[c] <= mid; c++) cm += c_q[c];
            if (cdf[mid] - cm > y)
                hi = mid;
            else
                lo = mid + 1;
        }
        int32_t j = (int32_t)lo;
        uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
        g_id[i] = j;
        g_t[i] = t;
        int pos = nc;
        while (pos > 0 && c_id[pos - 1] > j) {
            c_id[pos] = c_id[pos - 1];
            c_q[pos] = c_q[pos - 1];
            pos--;
        }
        c_id[pos] = j;
        c_q[pos] = qj;
        nc++;
        R -= qj;
    }
    int ng = nc;

    /* neighbourhood race over the 2-hop undirected ball (multiset; duplicates share a key) */
    keyed b[256];
    int nb = 0;
    if (g->beta_m1 > 0.0) {
        kv->n = 0;
#define OG_KEY(node)                                                        \
    do {                                                                    \
        int32_t nd_ = (node);                                               \
        cnt[1]++;                                                           \
        if (w[nd_] > 0.0f) {                                                \
            uint32_t rb_[4];                                                \
            rng(g->seed, S_BOOST, rep, ep, unit, (uint32_t)nd_, rb_);       \
            keyed kk_ = {-og_logf(unif_f(rb_[0])) / w[nd_], nd_};           \
            kv_push(kv, kk_);                                               \
        }                                                                   \
    } while (0)
        for (int i = 0; i < g->anchors; i++) OG_KEY(anchor[i]);
        for (int i = 0; i < g->anchors; i++) {
            int32_t x = anchor[i];
            cnt[0]++;
            for (int dir = 0; dir < 2; dir++) {
                const int64_t* off = dir ? g->bwd_off : g->fwd_off;
                const int32_t* col = dir ? g->bwd_col : g->fwd_col;
                for (int64_t p = off[x]; p < off[x + 1]; p++) {
                    int32_t y1 = col[p];
                    OG_KEY(y1);
                    cnt[0]++;
                    for (int dir2 = 0; dir2 < 2; dir2++) {
                        const int64_t* off2 = dir2 ? g->bwd_off : g->fwd_off;
                        const int32_t* col2 = dir2 ? g->bwd_col : g->fwd_col;
                        for (int64_t p2 = off2[y1]; p2 < off2[y1 + 1]; p2++) OG_KEY(col2[p2]);
                    }
                }
            }
        }
#undef OG_KEY
        qsort(kv->v, (size_t)kv->n, sizeof(keyed), cmp_keyed);
        for (int64_t i = 0; i < kv->n && nb < k; i++)
            if (i == 0 || kv->v[i].id != kv->v[i - 1].id || kv->v[i].key != kv->v[i - 1].key)
                b[nb++] = kv->v[i];
    }

    /* merge the two races: first k distinct nodes by (time, id) */
    int taken = 0, gi = 0, bi = 0;
    while (taken < k && (gi < ng || bi < nb)) {
        int32_t id;
        double tb = bi < nb ? (double)b[bi].key / g->beta_m1 : 0.0;
        int take_g = bi >= nb || (gi < ng && (g_t[gi] < tb || (g_t[gi] == tb && g_id[gi] <= b[bi].id)));
        if (take_g)
            id = g_id[gi++];
        else
            id = b[bi++].id;
        int dup = 0;
        for (int q = 0; q < taken; q++)
            if (out_arr[q] == id) {
                dup = 1;
                break;
            }
        if (!dup) out_arr[taken++] = id;
    }
    memcpy(out_sorted, out_arr, sizeof(int32_t) * (size_t)taken);
    qsort(out_sorted, (size_t)taken, sizeof(int32_t), cmp_i32);
    return taken;
}

/* ------------------------------------------------------------------ thinning sampler */
static int bsearch32(const int32_t* a, int64_t n, int32_t v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo < n && a[lo] == v;
}

/* j in the 2-hop undirected ball of the anchors <=> j in Z = anchors U adj(anchors), or an
 * adjacency row of j meets Z.  Pure set membership: any evaluation order gives the same answer.
 * *examined counts the adjacency entries of j looked at in order (forward row, then backward row)
 * up to and including the first hit; it is 0 when j is in Z or is a hub (degree >= hub_thr), whose
 * membership the engine answers from a bit mask. */
static int in_ball(const og_graph* g, const int32_t* Z, int64_t nz, int32_t j, int64_t* examined) {
    *examined = 0;
    if (bsearch32(Z, nz, j)) return 1;
    const int64_t deg = (g->fwd_off[j + 1] - g->fwd_off[j]) + (g->bwd_off[j + 1] - g->bwd_off[j]);
    const int hub = deg >= g->hub_thr;
    int64_t seen = 0;
    for (int dir = 0; dir < 2; dir++) {
        const int64_t* off = dir ? g->bwd_off : g->fwd_off;
        const int32_t* col = dir ? g->bwd_col : g->fwd_col;
        for (int64_t p = off[j]; p < off[j + 1]; p++) {
            seen++;
            if (bsearch32(Z, nz, col[p])) {
                if (!hub) *examined = seen;
                return 1;
            }
        }
    }
    if (!hub) *examined = seen;
    return 0;
}

/* Hub threshold of the epoch: at most 256 nodes, those in the highest log2-degree bins (>= 2^10). */
static int64_t hub_threshold(const og_graph* g) {
    int64_t hist[24] = {0};
    for (int64_t v = 0; v < g->n; v++) {
        int64_t d = (g->fwd_off[v + 1] - g->fwd_off[v]) + (g->bwd_off[v + 1] - g->bwd_off[v]);
        if (d >= 1024) {
            int b = 63 - __builtin_clzll((unsigned long long)d) - 10;
            if (b > 23) b = 23;
            hist[b]++;
        }
    }
    int64_t thr = INT64_MAX, cum = 0;
    for (int b = 23; b >= 0; b--) {
        cum += hist[b];
        if (cum > 256) break;
        if (hist[b]) thr = (int64_t)1 << (b + 10);
    }
    return thr;
}

enum { S_FALLBACK = 9 };

/* Thinning sampler.  One Poisson event stream over all nodes with rate beta*w_j: each event picks
 * j from the global CDF and is "global" with probability 1/beta (always accepted) or "boost"
 * (accepted iff j is in the ball).  Node j's accepted events have rate w_j beta^[j in ball], so the
 * first k distinct accepted nodes are a successive-sampling draw with those weights.  After
 * 64k+256 events the remaining draws continue without replacement from the CDF minus the chosen
 * weight (exact by memorylessness), which bounds the work when a few nodes hold most weight. */
static int sample_agent_thin(const og_graph* g, int64_t a, const uint64_t* cdf, int64_t npos,
                             int32_t* out_sorted, int32_t* out_arr, int64_t* cnt, int32_t** zbuf,
                             int64_t* zcap) {
    const int64_t n = g->n;
    const uint32_t ep = (uint32_t)g->epoch, rep = g->replica, unit = (uint32_t)a;
    uint32_t r[4];
    rng(g->seed, S_OUTDEG, rep, ep, unit, 0, r);
    uint64_t u = join64(r[0], r[1]);
    int kraw = OG_TABLE - 1;
    for (int i = 0; i < OG_TABLE; i++)
        if (u < g->table[i]) {
            kraw = i;
            break;
        }
    int64_t k = kraw < 1 ? 1 : kraw;
    if (k > n) k = n;
    if (k > npos) k = npos;
    int32_t anchor[4];
    rng(g->seed, S_ANCHOR, rep, ep, unit, 0, r);
    for (int i = 0; i < g->anchors; i++) anchor[i] = (int32_t)(((uint64_t)r[i] * (uint64_t)n) >> 32);
    /* Z = sorted unique anchors U their forward and backward rows (only needed when beta > 1) */
    const int nanch = g->p_global < 1.0 ? g->anchors : 0;
    int64_t nz = nanch;
    for (int i = 0; i < nanch; i++)
        nz += (g->fwd_off[anchor[i] + 1] - g->fwd_off[anchor[i]]) +
              (g->bwd_off[anchor[i] + 1] - g->bwd_off[anchor[i]]);
    cnt[0] += nz;
    if (nz + 1 > *zcap) {
        *zcap = nz + 1;
        *zbuf = (int32_t*)realloc(*zbuf, sizeof(int32_t) * (size_t)(nz + 1));
    }
    int32_t* Z = *zbuf;
    int64_t w = 0;
    for (int i = 0; i < nanch; i++) {
        Z[w++] = anchor[i];
        for (int64_t p = g->fwd_off[anchor[i]]; p < g->fwd_off[anchor[i] + 1]; p++) Z[w++] = g->fwd_col[p];
        for (int64_t p = g->bwd_off[anchor[i]]; p < g->bwd_off[anchor[i] + 1]; p++) Z[w++] = g->bwd_col[p];
    }
    qsort(Z, (size_t)nz, sizeof(int32_t), cmp_i32);
    int64_t uz = 0;
    for (int64_t i = 0; i < nz; i++)
        if (i == 0 || Z[i] != Z[i - 1]) Z[uz++] = Z[i];
    nz = uz;

    const uint64_t Wq = cdf[n - 1];
    int taken = 0;
    const int64_t maxev = 64 * k + 256;
    int64_t events = 0, tests = 0, scanned = 0;
    for (int64_t i = 0; i < maxev && taken < k; i++) {
        rng(g->seed, S_GLOBAL, rep, ep, unit, (uint32_t)i, r);
        uint64_t y = hi_mul64(join64(r[0], r[1]), Wq);
        int64_t lo = 0, hi = n - 1;
        while (lo < hi) {
            int64_t mid = lo + (hi - lo) / 2;
            if (cdf[mid] > y)
                hi = mid;
            else
                lo = mid + 1;
        }
        int32_t j = (int32_t)lo;
        events++;
        int glob = unif_d(r[2], r[3]) <= g->p_global;
        int dup = 0;
        for (int q = 0; q < taken; q++)
            if (out_arr[q] == j) {
                dup = 1;
                break;
            }
        if (dup) continue; /* an arrived node gains nothing from another event */
        if (!glob) {
            int64_t ex;
            tests++;
            int mem = in_ball(g, Z, nz, j, &ex);
            scanned += ex;
            if (!mem) continue;
        }
        out_arr[taken++] = j;
    }
    if (taken < k) {
        /* exact continuation without replacement over the unchosen nodes */
        int32_t c_id[256];
        uint64_t c_q[256];
        int nc = 0;
        uint64_t R = Wq;
        for (int q = 0; q < taken; q++) {
            int32_t j = out_arr[q];
            uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
            int pos = nc;
            while (pos > 0 && c_id[pos - 1] > j) {
                c_id[pos] = c_id[pos - 1];
                c_q[pos] = c_q[pos - 1];
                pos--;
            }
            c_id[pos] = j;
            c_q[pos] = qj;
            nc++;
            R -= qj;
        }
        for (uint32_t f = 0; taken < k && R > 0 && f < (1u << 24); f++) {
            rng(g->seed, S_FALLBACK, rep, ep, unit, f, r);
            uint64_t y = hi_mul64(join64(r[0], r[1]), R);
            int64_t lo = 0, hi = n - 1;
            while (lo < hi) {
                int64_t mid = lo + (hi - lo) / 2;
                uint64_t cm = 0;
                for (int c = 0; c < nc && c_id[c] <= mid; c++) cm += c_q[c];
                if (cdf[mid] - cm > y)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            int32_t j = (int32_t)lo;
            events++;
            int glob = unif_d(r[2], r[3]) <= g->p_global;
            if (!glob) {
                int64_t ex;
                tests++;
                int mem = in_ball(g, Z, nz, j, &ex);
                scanned += ex;
                if (!mem) continue;
            }
            uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
            int pos = nc;
            while (pos > 0 && c_id[pos - 1] > j) {
                c_id[pos] = c_id[pos - 1];
                c_q[pos] = c_q[pos - 1];
                pos--;
            }
            c_id[pos] = j;
            c_q[pos] = qj;
            nc++;
            R -= qj;
            out_arr[taken++] = j;
        }
    }
    cnt[1] += tests;
    cnt[2] += events;
    cnt[3] += scanned;
    memcpy(out_sorted, out_arr, sizeof(int32_t) * (size_t)taken);
    qsort(out_sorted, (size_t)taken, sizeof(int32_t), cmp_i32);
    return taken;
}

static void compute_weights(og_graph* g, int64_t* npos_out) {
    int64_t n = g->n;
    free(g->w);
    free(g->cdf);
    g->w = (float*)malloc(sizeof(float) * (size_t)n);
    g->cdf = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)n);
    g->w_n = n;
    float wmax = 0.0f;
    for (int64_t j = 0; j < n; j++) {
        float a = og_logf(g->fit[j]);
        float b = og_logf((float)(g->indeg[j] + 1));
        float c = (float)(int32_t)(g->epoch - g->pub[j]) / g->tau_f;
        float w = og_expf(fmaf(g->gamma_f, a, fmaf(g->alpha_f, b, -c)));
        g->w[j] = w;
        if (w > wmax) wmax = w;
    }
    /* fixed-point shift: q_j = floor(w_j 2^s) < 2^(62 - ceil(log2 n)) */
    int ex = (int)((bits_of_f(wmax) >> 23) & 0xFF) - 126;
    int cl = 0;
    while (cl < 63 && ((uint64_t)1 << cl) < (uint64_t)n) cl++;
    int s = 62 - ex - cl;
    g->shift = s;
    double scale = d_from_bits((uint64_t)(s + 1023) << 52);
    uint64_t acc = 0;
    int64_t npos = 0;
    for (int64_t j = 0; j < n; j++) {
        uint64_t q = 0;
        if (g->w[j] > 0.0f) {
            q = (uint64_t)((double)g->w[j] * scale);
            if (q == 0) q = 1;
            npos++;
        }
        acc += q;
        g->cdf[j] = acc;
    }
    *npos_out = npos;
}

int og_pa_epoch(og_graph* g, int threads) {
    if (g->n <= 0) return 6;
    int64_t n = g->n;
    int64_t delta = g->growth_rate > 0 ? (int64_t)ceil((double)n * g->growth_rate) : g->fixed_new;
    if (delta <= 0) return 3;
    int64_t npos;
    compute_weights(g, &npos);
    if (npos == 0) return 3;
    int32_t* rows = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta * 256);
    int32_t* arr = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta * 256);
    int32_t* kk = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta);
    int64_t rows_exp = 0, elems = 0, draws = 0, scanned = 0;
    g->hub_thr = g->sampler == 0 ? hub_threshold(g) : INT64_MAX;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : rows_exp, elems, draws, scanned)
    {
        keyvec kv = {0, 0, 0};
        int32_t* zbuf = NULL;
        int64_t zcap = 0;
#pragma omp for schedule(dynamic, 16)
        for (int64_t a = 0; a < delta; a++) {
            int64_t cnt[4] = {0, 0, 0, 0};
            if (g->sampler == 0) {
                kk[a] = sample_agent_thin(g, a, g->cdf, npos, rows + a * 256, arr + a * 256, cnt,
                                          &zbuf, &zcap);
            } else {
                kk[a] = sample_agent(g, a, g->w, g->cdf, g->shift, npos, rows + a * 256,
                                     arr + a * 256, cnt, &kv);
                cnt[2] = kk[a];
            }
            rows_exp += cnt[0];
            elems += cnt[1];
            draws += cnt[2];
            scanned += cnt[3];
        }
        free(kv.v);
        free(zbuf);
    }
    int64_t* row_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(delta + 1));
    row_off[0] = 0;
    for (int64_t a = 0; a < delta; a++) row_off[a + 1] = row_off[a] + kk[a];
    int64_t e_new = row_off[delta];
    int32_t* flat = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e_new + 1));
    free(g->arrivals);
    g->arrivals = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e_new + 1));
    for (int64_t a = 0; a < delta; a++) {
        memcpy(flat + row_off[a], rows + a * 256, sizeof(int32_t) * (size_t)kk[a]);
        memcpy(g->arrivals + row_off[a], arr + a * 256, sizeof(int32_t) * (size_t)kk[a]);
    }
    float* nf = (float*)malloc(sizeof(float) * (size_t)delta);
    for (int64_t a = 0; a < delta; a++)
        nf[a] = og_fitness(g->seed, g->replica, (uint32_t)g->epoch, (uint32_t)a);
    append_rows(g, delta, row_off, flat, (int32_t)g->epoch, nf);
    g->stats[0] = n;
    g->stats[1] = rows_exp;
    g->stats[2] = elems;
    g->stats[3] = draws;
    g->stats[4] = e_new;
    g->stats[5] = scanned;
    g->epoch++;
    free(rows);
    free(arr);
    free(kk);
    free(row_off);
    free(flat);
    free(nf);
    return 0;
}

/* ------------------------------------------------------------------ ER epoch */
#define OG_ER_CHUNK 65536

/* Geometric-skip walk of one (new node, 2^16-id chunk) task.  Emits into out (may be NULL) and
 * returns the number of successes. */
static int64_t er_task(const og_graph* g, int64_t i, int64_t c, int64_t n, double inv_l,
                       int32_t* out) {
    int64_t lo = c * OG_ER_CHUNK, hi = lo + OG_ER_CHUNK < n ? lo + OG_ER_CHUNK : n;
    int64_t pos = lo - 1, cnt = 0;
    uint32_t r[4];
    for (uint32_t d = 0;; d++) {
        if ((d & 1u) == 0) rng(g->seed, S_ER, (uint32_t)c, (uint32_t)g->epoch, (uint32_t)i, d >> 1, r);
        double u = (d & 1u) ? unif_d(r[2], r[3]) : unif_d(r[0], r[1]);
        double sk = floor(og_log(u) * inv_l);
        if (sk >= (double)(hi - pos - 1)) break;
        pos = pos + 1 + (int64_t)sk;
        if (out) out[cnt] = (int32_t)pos;
        cnt++;
    }
    return cnt;
}

int og_er_epoch(og_graph* g, int64_t delta, double p, int threads) {
    if (g->n <= 0) return 6;
    if (delta <= 0 || isnan(p)) return 3;
    if (p > 1.0) p = 1.0;
    int64_t n = g->n;
    int64_t chunks = (n + OG_ER_CHUNK - 1) / OG_ER_CHUNK;
    int64_t tasks = delta * chunks;
    int64_t* cnt = (int64_t*)calloc((size_t)tasks + 1, sizeof(int64_t));
    double inv_l = 1.0 / og_log(1.0 - p);
    if (threads > 0) omp_set_num_threads(threads);
    if (p > 0.0) {
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t t = 0; t < tasks; t++) cnt[t + 1] = er_task(g, t / chunks, t % chunks, n, inv_l, NULL);
    }
    for (int64_t t = 0; t < tasks; t++) cnt[t + 1] += cnt[t];
    int32_t* flat = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cnt[tasks] + 1));
    if (p > 0.0) {
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t t = 0; t < tasks; t++) er_task(g, t / chunks, t % chunks, n, inv_l, flat + cnt[t]);
    }
    int64_t* row_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(delta + 1));
    for (int64_t a = 0; a <= delta; a++) row_off[a] = cnt[a * chunks];
    float* nf = (float*)malloc(sizeof(float) * (size_t)delta);
    for (int64_t a = 0; a < delta; a++)
        nf[a] = og_fitness(g->seed, g->replica, (uint32_t)g->epoch, (uint32_t)a);
    free(g->arrivals);
    g->arrivals = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cnt[tasks] + 1));
    memcpy(g->arrivals, flat, sizeof(int32_t) * (size_t)cnt[tasks]);
    append_rows(g, delta, row_off, flat, (int32_t)g->epoch, nf);
    memset(g->stats, 0, sizeof(g->stats));
    g->stats[3] = 0;
    g->stats[4] = cnt[tasks];
    g->epoch++;
    free(cnt);
    free(flat);
    free(row_off);
    free(nf);
    return 0;
}

/* ------------------------------------------------------------------ readers */
int64_t og_num_nodes(const og_graph* g) { return g->n; }
int64_t og_num_edges(const og_graph* g) { return g->m; }
void og_copy_csr(const og_graph* g, int which, int64_t* off, int32_t* col) {
    const int64_t* o = which ? g->bwd_off : g->fwd_off;
    const int32_t* c = which ? g->bwd_col : g->fwd_col;
    memcpy(off, o, sizeof(int64_t) * (size_t)(g->n + 1));
    memcpy(col, c, sizeof(int32_t) * (size_t)g->m);
}
void og_copy_degrees(const og_graph* g, int32_t* indeg, int32_t* outdeg) {
    for (int64_t i = 0; i < g->n; i++) {
        if (indeg) indeg[i] = g->indeg[i];
        if (outdeg) outdeg[i] = (int32_t)(g->fwd_off[i + 1] - g->fwd_off[i]);
    }
}
void og_copy_nodes(const og_graph* g, int32_t* pub, float* fitness) {
    memcpy(pub, g->pub, sizeof(int32_t) * (size_t)g->n);
    memcpy(fitness, g->fit, sizeof(float) * (size_t)g->n);
}
void og_epoch_edges(const og_graph* g, int64_t* first, int64_t* count) {
    *first = g->last_first;
    *count = g->last_count;
}
void og_copy_arrivals(const og_graph* g, int32_t* cited) {
    if (g->arrivals) memcpy(cited, g->arrivals, sizeof(int32_t) * (size_t)g->last_count);
}
void og_stats(const og_graph* g, int64_t* out6) { memcpy(out6, g->stats, sizeof(g->stats)); }
int64_t og_copy_weights(const og_graph* g, float* w, uint64_t* cdf, int32_t* shift) {
    if (w) memcpy(w, g->w, sizeof(float) * (size_t)g->w_n);
    if (cdf) memcpy(cdf, g->cdf, sizeof(uint64_t) * (size_t)g->w_n);
    if (shift) *shift = g->shift;
    return g->w_n;
}

/* ------------------------------------------------------------------ anchors of an epoch's agents */
void og_agent_anchors(uint64_t seed, uint32_t replica, uint32_t epoch, int64_t n, int64_t agents,
                      int num_anchors, int32_t* out) {
    for (int64_t a = 0; a < agents; a++) {
        uint32_t r[4];
        rng(seed, S_ANCHOR, replica, epoch, (uint32_t)a, 0, r);
        for (int i = 0; i < 4; i++)
            out[a * 4 + i] = i < num_anchors ? (int32_t)(((uint64_t)r[i] * (uint64_t)n) >> 32) : -1;
    }
}

/* ------------------------------------------------------------------ log-likelihood of a trace
 *
 * No counterpart in the reference: the model the samplers above draw from, written as a density.
 * Agent a of trace epoch e is node n_0 + a; it drew c_1..c_k in this order by successive sampling
 * without replacement over the nodes j < n_e that existed when the epoch began, with weights
 *   W_j = f_j^gamma (indeg_e(j)+1)^alpha exp(-(t_e - t_j)/tau) beta^[j in N_a],
 * indeg_e the in-degree in the epoch-start graph and N_a the undirected 2-hop ball of the agent's
 * anchors in that graph.  Then
 *   log L = sum_a sum_i [ log W_{c_i} - log(Z_a - sum_{l<i} W_{c_l}) ],  Z_a = sum_{j<n_e} W_j.
 * The out-degree and the anchors do not depend on theta = (alpha, tau, gamma, beta).  The gradient
 * is the direct derivative:  d/dtheta log W_j = g_j = (log(indeg+1), (t_e-t_j)/tau^2, log f_j,
 * [j in N_a]/beta),  dZ_a = sum_j W_j g_j.  All arithmetic is FP64 with libm exp and log.
 */
static int64_t upper_bound64(const int32_t* a, int64_t lo, int64_t hi, int32_t v) {
    /* first index in [lo, hi) with a[i] > v */
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        if (a[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

int og_loglik(const og_trace* T, int batch, const double* theta, double* ll, double* grad,
              int threads) {
    const int64_t n = T->num_nodes;
    const int E = T->num_epochs;
    if (n <= 0 || E < 1 || batch < 1) return 3;
    const int64_t n0 = T->epoch_nodes[0];
    const int64_t agents = n - n0;
    if (T->epoch_nodes[E] != n) return 3;
    const int64_t mc = T->cite_off[agents];
    /* final graph: seed edges plus every agent's citations */
    const int64_t m = T->num_seed_edges + mc;
    int32_t* src = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int32_t* dst = (int32_t*)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    memcpy(src, T->seed_src, sizeof(int32_t) * (size_t)T->num_seed_edges);
    memcpy(dst, T->seed_dst, sizeof(int32_t) * (size_t)T->num_seed_edges);
    for (int64_t a = 0; a < agents; a++)
        for (int64_t p = T->cite_off[a]; p < T->cite_off[a + 1]; p++) {
            src[T->num_seed_edges + p] = (int32_t)(n0 + a);
            dst[T->num_seed_edges + p] = T->cites[p];
        }
    int64_t *fo, *bo, mf, mb;
    int32_t *fc, *bc;
    build_csr(n, m, src, dst, &fo, &fc, &mf);
    build_csr(n, m, dst, src, &bo, &bc, &mb);
    free(src);
    free(dst);
    /* theta-independent node features of every epoch */
    double* lf = (double*)malloc(sizeof(double) * (size_t)n);
    double* ld = (double*)malloc(sizeof(double) * (size_t)n * (size_t)E);
    for (int64_t j = 0; j < n; j++) lf[j] = log((double)T->fitness[j]);
    for (int e = 0; e < E; e++) {
        const int64_t ne = T->epoch_nodes[e];
        for (int64_t j = 0; j < ne; j++) {
            const int64_t d = upper_bound64(bc, bo[j], bo[j + 1], (int32_t)(ne - 1)) - bo[j];
            ld[(size_t)e * (size_t)n + (size_t)j] = log((double)d + 1.0);
        }
    }
    /* per epoch and theta: Z_glob = sum_j w_j and G_glob = sum_j w_j g_j (alpha, tau, gamma) */
    double* zg = (double*)calloc((size_t)E * (size_t)batch * 4, sizeof(double));
    for (int e = 0; e < E; e++) {
        const int64_t ne = T->epoch_nodes[e];
        const double te = (double)T->epoch_t[e];
        for (int b = 0; b < batch; b++) {
            const double al = theta[b * 4], tau = theta[b * 4 + 1], ga = theta[b * 4 + 2];
            double z = 0, g0 = 0, g1 = 0, g2 = 0;
            for (int64_t j = 0; j < ne; j++) {
                const double dl = ld[(size_t)e * (size_t)n + (size_t)j], dt = te - (double)T->pub[j];
                const double w = exp(ga * lf[j] + al * dl - dt / tau);
                z += w;
                g0 += w * dl;
                g1 += w * dt;
                g2 += w * lf[j];
            }
            double* o = zg + ((size_t)e * (size_t)batch + (size_t)b) * 4;
            o[0] = z;
            o[1] = g0;
            o[2] = g1 / (tau * tau);
            o[3] = g2;
        }
    }
    for (int b = 0; b < batch; b++) {
        ll[b] = 0;
        if (grad)
            for (int k = 0; k < 4; k++) grad[b * 4 + k] = 0;
    }
    if (threads > 0) omp_set_num_threads(threads);
    int bad = 0;
#pragma omp parallel
    {
        int32_t* stamp = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        int32_t* ball = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
        double* acc = (double*)calloc((size_t)batch * 5, sizeof(double));
        for (int64_t j = 0; j < n; j++) stamp[j] = -1;
#pragma omp for schedule(dynamic, 32)
        for (int64_t a = 0; a < agents; a++) {
            const int64_t v = n0 + a;
            int e = 0;
            while (e + 1 < E && T->epoch_nodes[e + 1] <= v) e++;
            const int64_t ne = T->epoch_nodes[e];
            const double te = (double)T->epoch_t[e];
            const double* lde = ld + (size_t)e * (size_t)n;
            /* the 2-hop ball in the epoch-start graph (rows restricted to nodes j < n_e) */
            int64_t nb = 0;
            const int32_t mark = (int32_t)a;
#define OG_BALL_ADD(x)                       \
    do {                                     \
        const int32_t x_ = (x);              \
        if (stamp[x_] != mark) {             \
            stamp[x_] = mark;                \
            ball[nb++] = x_;                 \
        }                                    \
    } while (0)
            for (int i = 0; i < T->num_anchors; i++) {
                const int32_t x = T->anchors[a * 4 + i];
                if (x < 0) continue;
                OG_BALL_ADD(x);
            }
            const int64_t n1 = nb;
            /* 1-hop: neighbours of the anchors */
            int64_t h1 = nb;
            for (int64_t q = 0; q < n1; q++) {
                const int32_t x = ball[q];
                for (int64_t p = fo[x]; p < fo[x + 1]; p++) OG_BALL_ADD(fc[p]);
                const int64_t be = upper_bound64(bc, bo[x], bo[x + 1], (int32_t)(ne - 1));
                for (int64_t p = bo[x]; p < be; p++) OG_BALL_ADD(bc[p]);
            }
            h1 = nb;
            /* 2-hop: neighbours of the 1-hop nodes */
            for (int64_t q = n1; q < h1; q++) {
                const int32_t x = ball[q];
                for (int64_t p = fo[x]; p < fo[x + 1]; p++) OG_BALL_ADD(fc[p]);
                const int64_t be = upper_bound64(bc, bo[x], bo[x + 1], (int32_t)(ne - 1));
                for (int64_t p = bo[x]; p < be; p++) OG_BALL_ADD(bc[p]);
            }
#undef OG_BALL_ADD
            const int64_t c0 = T->cite_off[a], c1 = T->cite_off[a + 1];
            for (int b = 0; b < batch; b++) {
                const double al = theta[b * 4], tau = theta[b * 4 + 1], ga = theta[b * 4 + 2],
                             be = theta[b * 4 + 3];
                const double itau2 = 1.0 / (tau * tau), lbe = log(be);
                double s = 0, t0 = 0, t1 = 0, t2 = 0;
                for (int64_t q = 0; q < nb; q++) {
                    const int32_t j = ball[q];
                    const double dl = lde[j], dt = te - (double)T->pub[j];
                    const double w = exp(ga * lf[j] + al * dl - dt / tau);
                    s += w;
                    t0 += w * dl;
                    t1 += w * dt;
                    t2 += w * lf[j];
                }
                const double* gg = zg + ((size_t)e * (size_t)batch + (size_t)b) * 4;
                const double z = gg[0] + (be - 1.0) * s;
                const double dz[4] = {gg[1] + (be - 1.0) * t0, gg[2] + (be - 1.0) * t1 * itau2,
                                      gg[3] + (be - 1.0) * t2, s};
                double p = 0, dp[4] = {0, 0, 0, 0}, l = 0, gsum[4] = {0, 0, 0, 0};
                for (int64_t i = c0; i < c1; i++) {
                    const int32_t c = T->cites[i];
                    const int in = stamp[c] == mark;
                    const double dl = lde[c], dt = te - (double)T->pub[c];
                    const double x = ga * lf[c] + al * dl - dt / tau + (in ? lbe : 0.0);
                    const double W = exp(x);
                    const double D = z - p;
                    if (!(D > 0)) bad = 1;
                    l += x - log(D);
                    const double g[4] = {dl, dt * itau2, lf[c], in ? 1.0 / be : 0.0};
                    for (int k = 0; k < 4; k++) {
                        gsum[k] += g[k] - (dz[k] - dp[k]) / D;
                        dp[k] += W * g[k];
                    }
                    p += W;
                }
                acc[b * 5] += l;
                for (int k = 0; k < 4; k++) acc[b * 5 + 1 + k] += gsum[k];
            }
        }
#pragma omp critical
        for (int b = 0; b < batch; b++) {
            ll[b] += acc[b * 5];
            if (grad)
                for (int k = 0; k < 4; k++) grad[b * 4 + k] += acc[b * 5 + 1 + k];
        }
        free(stamp);
        free(ball);
        free(acc);
    }
    free(fo);
    free(fc);
    free(bo);
    free(bc);
    free(lf);
    free(ld);
    free(zg);
    return bad ? 4 : 0;
}

/* ------------------------------------------------------------------ refcompat functor
 *
 * ParAGraph's own per-paper model (the drop-in semantics of its abm driver), on the same graph
 * state.  Per epoch t with n nodes and delta = ceil(n * growth_rate) new papers:
 *   scores (ABM::FillInDegreeArr / FillFitnessArr / FillRecencyArr / CalculateScores,
 *   src/abm.cu:112-208,324-338):
 *     f_j   = 1 before pub+lag, the peak value up to pub+lag+dur, then (int)(peak/(t-pub-lag-dur+1)^decay)
 *     pa_j  = (indeg_j^gamma + 1) / sum,  fit_j = (f_j^gamma + 1) / sum   (integer sums, exact)
 *     rec_j = P(t-pub_j) / (count(t-pub_j) * sum of P over the distinct ages present)
 *     score_aj = w_pa pa_j + w_rec rec_j + w_fit fit_j (per-agent weights, normalised)
 *   agent a (budget split src/kernel.cu:230-402; citations src/abm.cu:376-565):
 *     d from the out-degree bag, clipped to [1, min(256, n-1)]; generator g uniform over [0, n);
 *     sy = 1 for exactly floor(delta * same_year) agents, citing paper n + U[0, delta);
 *     rsv = floor(fully_random d);  in = min(ceil((d-1-sy-rsv) alpha), |N1|) from the 1-hop set
 *     of g;  out = min(d-1-sy-rsv-in, |N2|) from the 2-hop set (minus the 1-hop set and g), both
 *     by Efraimidis-Spirakis keys (k smallest E_j/score_j, E_j exponential, keyed by (agent, j));
 *     the remaining d-1-sy-in-out uniformly from [0, n-1) without g and earlier choices.
 * Arrival order: g, the same-year paper, 1-hop picks, 2-hop picks (key order), uniform picks.
 */
enum { S_SAMEYEAR = 7, S_FILL = 8, S_RCAGENT = 10, S_RCKEY = 11, S_RCFIT = 12 };
#define OG_RC_FILL_BLOCKS (1u << 20) /* Philox blocks a uniform fill may use (then an error) */

static double u128_to_d(unsigned __int128 v) {
    return (double)(uint64_t)(v >> 64) * 0x1p64 + (double)(uint64_t)v;
}

void og_rc_bag_table(const int32_t* bag, int64_t len, uint64_t* table) {
    int64_t cnt[OG_TABLE];
    memset(cnt, 0, sizeof(cnt));
    for (int64_t i = 0; i < len; i++) {
        int32_t v = bag[i] < 0 ? 0 : (bag[i] > OG_TABLE - 1 ? OG_TABLE - 1 : bag[i]);
        cnt[v]++;
    }
    int64_t cum = 0;
    for (int v = 0; v < OG_TABLE; v++) {
        cum += cnt[v];
        table[v] = (cum >= len || v == OG_TABLE - 1)
                       ? ~(uint64_t)0
                       : (uint64_t)((((unsigned __int128)cum) << 64) / (unsigned __int128)len);
    }
}

/* Peak-fitness distribution of ABM::AssignPeakFitnessValues (includes/abm.cuh:469-484):
 * P(v) proportional to v^-1.634 for v in 1..1000, as 2^64-scaled CDF thresholds. */
void og_rc_fitness_table(uint64_t* table) {
    double p[OG_RC_FIT_MAX], tot = 0.0;
    for (int i = 0; i < OG_RC_FIT_MAX; i++) {
        p[i] = og_exp(-1.634 * og_log((double)(i + 1)));
        tot += p[i];
    }
    double cum = 0.0;
    for (int i = 0; i < OG_RC_FIT_MAX; i++) {
        cum += p[i];
        double q = cum / tot;
        table[i] = (q >= 1.0 || i == OG_RC_FIT_MAX - 1) ? ~(uint64_t)0 : (uint64_t)(q * 0x1p64);
    }
}

int og_rc_configure(og_graph* g, const double* prm, const int32_t* bag, int64_t bag_len,
                    const double* rec, int32_t rec_len) {
    /* prm: pa, rec, fit weights, alpha, fully_random, same_year, growth_rate, gamma, decay */
    if (bag_len <= 0 || rec_len < 0 || !(prm[6] > 0.0)) return 3;
    int fixed = prm[0] >= 0.0 && prm[1] >= 0.0 && prm[2] >= 0.0;
    if (fixed && !(prm[0] + prm[1] + prm[2] > 0.0)) return 3;
    g->rc = 1;
    for (int i = 0; i < 3; i++) g->rc_w[i] = fixed ? prm[i] : -1.0;
    g->rc_alpha = prm[3] > 1.0 ? 1.0 : prm[3];
    g->rc_frc = prm[4];
    g->rc_sy = prm[5];
    g->rc_growth = prm[6];
    g->rc_gamma = (int)prm[7];
    g->rc_decay = (int)prm[8];
    og_rc_bag_table(bag, bag_len, g->rc_bag);
    og_rc_fitness_table(g->rc_fit_table);
    free(g->rc_rec);
    g->rc_rec_len = rec_len;
    g->rc_rec = (double*)malloc(sizeof(double) * (size_t)(rec_len > 0 ? rec_len : 1));
    if (rec_len) memcpy(g->rc_rec, rec, sizeof(double) * (size_t)rec_len);
    free(g->rc_lag);
    free(g->rc_dur);
    g->rc_lag = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->n > 0 ? g->n : 1));
    g->rc_dur = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->n > 0 ? g->n : 1));
    for (int64_t j = 0; j < g->n; j++) {
        g->rc_lag[j] = 0;
        g->rc_dur[j] = 1000;
    }
    return 0;
}

void og_rc_set_nodes(og_graph* g, int64_t first, int64_t count, const int32_t* lag,
                     const int32_t* peak, const int32_t* dur) {
    for (int64_t i = 0; i < count; i++) {
        g->rc_lag[first + i] = lag[i];
        g->fit[first + i] = (float)peak[i];
        g->rc_dur[first + i] = dur[i];
    }
}

static int64_t ipow_i64(int64_t x, int e) {
    int64_t r = 1;
    for (int i = 0; i < e; i++) r *= x;
    return r;
}

/* fitness of node j at epoch t (ABM::FillFitnessArr, src/abm.cu:152-176) */
static int32_t rc_fitness_at(const og_graph* g, int64_t j, int64_t t) {
    int64_t pub = g->pub[j], lag = g->rc_lag[j], dur = g->rc_dur[j];
    int64_t peak = (int64_t)g->fit[j];
    if (pub + lag > t) return 1;
    if (pub + lag + dur >= t) return (int32_t)peak;
    double den = (double)ipow_i64(t - pub - lag - dur + 1, g->rc_decay);
    return (int32_t)((double)peak / den);
}

static void rc_scores(const og_graph* g, double* pa, double* rec, double* fit) {
    int64_t n = g->n, t = g->epoch;
    unsigned __int128 spa = 0, sfit = 0;
    int64_t* cnt = (int64_t*)calloc((size_t)(g->rc_rec_len > 0 ? g->rc_rec_len : 1), sizeof(int64_t));
    for (int64_t j = 0; j < n; j++) {
        unsigned __int128 a = 1, f = 1, x = (unsigned __int128)(uint32_t)g->indeg[j];
        unsigned __int128 y = (unsigned __int128)(uint32_t)rc_fitness_at(g, j, t);
        for (int e = 0; e < g->rc_gamma; e++) {
            a *= x;
            f *= y;
        }
        spa += a + 1;
        sfit += f + 1;
        pa[j] = u128_to_d(a + 1);
        fit[j] = u128_to_d(f + 1);
        int64_t dy = t - g->pub[j];
        if (dy >= 0 && dy < g->rc_rec_len) cnt[dy]++;
    }
    double U = 0.0;
    for (int i = 0; i < g->rc_rec_len; i++)
        if (cnt[i]) U += g->rc_rec[i];
    double dpa = u128_to_d(spa), dfit = u128_to_d(sfit);
    for (int64_t j = 0; j < n; j++) {
        pa[j] = pa[j] / dpa;
        fit[j] = fit[j] / dfit;
        int64_t dy = t - g->pub[j];
        rec[j] = (dy >= 0 && dy < g->rc_rec_len && U > 0.0) ? g->rc_rec[dy] / ((double)cnt[dy] * U) : 0.0;
    }
    free(cnt);
}

/* bijection of [0, 2^bits): three rounds of xor-key, odd multiply, xorshift */
static uint32_t rc_perm(uint32_t x, int bits, const uint32_t key[4]) {
    uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    int h = bits / 2 + 1;
    for (int r = 0; r < 3; r++) {
        x = (x ^ key[r]) & mask;
        x = (x * (key[(r + 1) & 3] | 1u)) & mask;
        if (h < bits) x ^= x >> h;
    }
    return x;
}

/* 1 when agent a is one of the floor(delta * same_year) same-year citers; its target in *tgt */
static int rc_same_year(const og_graph* g, int64_t a, int64_t delta, int32_t* tgt) {
    int64_t S = (int64_t)floor((double)delta * g->rc_sy);
    if (S <= 0) return 0;
    int bits = 1;
    while (bits < 31 && ((int64_t)1 << bits) < delta) bits++;
    uint32_t key[4];
    rng(g->seed, S_SAMEYEAR, g->replica, (uint32_t)g->epoch, 0xFFFFFFFFu, 0, key);
    uint32_t x = (uint32_t)a;
    do {
        x = rc_perm(x, bits, key);
    } while ((int64_t)x >= delta);
    if ((int64_t)x >= S) return 0;
    uint32_t r[4];
    rng(g->seed, S_SAMEYEAR, g->replica, (uint32_t)g->epoch, (uint32_t)a, 0, r);
    *tgt = (int32_t)(g->n + (int64_t)(((uint64_t)r[0] * (uint64_t)delta) >> 32));
    return 1;
}

static float rc_key(const og_graph* g, int64_t a, int32_t j, double score) {
    if (!(score > 0.0)) return INFINITY;
    uint32_t r[4];
    rng(g->seed, S_RCKEY, g->replica, (uint32_t)g->epoch, (uint32_t)a, (uint32_t)j, r);
    double E = -og_log(unif_d(r[0], r[1]));
    return (float)(E / score);
}

/* k smallest distinct (key, id) of a keyed multiset (duplicates share a key) */
static int rc_topk(keyvec* kv, int k, int32_t* out) {
    qsort(kv->v, (size_t)kv->n, sizeof(keyed), cmp_keyed);
    int c = 0;
    for (int64_t i = 0; i < kv->n && c < k; i++)
        if (i == 0 || kv->v[i].id != kv->v[i - 1].id) out[c++] = kv->v[i].id;
    return c;
}

static int rc_in_row(const og_graph* g, int32_t x, int32_t v) {
    return bsearch32(g->fwd_col + g->fwd_off[x], g->fwd_off[x + 1] - g->fwd_off[x], v) ||
           bsearch32(g->bwd_col + g->bwd_off[x], g->bwd_off[x + 1] - g->bwd_off[x], v);
}

/* Per-agent parameters: weights (normalised), alpha, generator. */
static void rc_agent_params(const og_graph* g, int64_t a, double* w3, double* alpha, int32_t* gen) {
    uint32_t r0[4], r1[4], r2[4];
    rng(g->seed, S_RCAGENT, g->replica, (uint32_t)g->epoch, (uint32_t)a, 0, r0);
    rng(g->seed, S_RCAGENT, g->replica, (uint32_t)g->epoch, (uint32_t)a, 1, r1);
    rng(g->seed, S_RCAGENT, g->replica, (uint32_t)g->epoch, (uint32_t)a, 2, r2);
    double wp = g->rc_w[0] >= 0.0 ? g->rc_w[0] : unif_d(r0[0], r0[1]);
    double wr = g->rc_w[1] >= 0.0 ? g->rc_w[1] : unif_d(r0[2], r0[3]);
    double wf = g->rc_w[2] >= 0.0 ? g->rc_w[2] : unif_d(r1[0], r1[1]);
    double sum = wp + wr + wf;
    w3[0] = wp / sum;
    w3[1] = wr / sum;
    w3[2] = wf / sum;
    *alpha = g->rc_alpha >= 0.0 ? g->rc_alpha : unif_d(r1[2], r1[3]);
    *gen = (int32_t)(((uint64_t)r2[0] * (uint64_t)g->n) >> 32);
}

static int rc_agent(const og_graph* g, int64_t a, int64_t delta, int d, const double* pa,
                    const double* rec, const double* fit, int32_t* out_sorted, int32_t* out_arr,
                    int64_t* cnt, keyvec* kv, double* info) {
    const int64_t n = g->n;
    double w3[3], alpha;
    int32_t gen;
    rc_agent_params(g, a, w3, &alpha, &gen);
#define RC_SCORE(j) (w3[0] * pa[j] + w3[1] * rec[j] + w3[2] * fit[j])
    int c = 0;
    out_arr[c++] = gen;
    int32_t tgt;
    int sy = d >= 2 ? rc_same_year(g, a, delta, &tgt) : 0; /* an agent of out-degree 1 cites g only */
    if (sy) out_arr[c++] = tgt;
    int rsv = (int)floor(g->rc_frc * (double)d);
    int rem1 = d - 1 - sy - rsv;
    int in_t = rem1 > 0 ? (int)ceil((double)rem1 * alpha) : 0;
    if (in_t > rem1) in_t = rem1 > 0 ? rem1 : 0;
    /* 1-hop set of the generator (streamed when it has a budget) */
    kv->n = 0;
    cnt[0]++;
    for (int dir = 0; dir < 2 && in_t > 0; dir++) {
        const int64_t* off = dir ? g->bwd_off : g->fwd_off;
        const int32_t* col = dir ? g->bwd_col : g->fwd_col;
        for (int64_t p = off[gen]; p < off[gen + 1]; p++) {
            int32_t y = col[p];
            if (y == gen) continue;
            cnt[1]++;
            keyed kk = {rc_key(g, a, y, RC_SCORE(y)), y};
            kv_push(kv, kk);
        }
    }
    int in = in_t > 0 ? rc_topk(kv, in_t, out_arr + c) : 0;
    c += in;
    int rem2 = d - 1 - sy - rsv - in;
    int out = 0;
    if (rem2 > 0) {
        kv->n = 0;
        for (int dir = 0; dir < 2; dir++) {
            const int64_t* off = dir ? g->bwd_off : g->fwd_off;
            const int32_t* col = dir ? g->bwd_col : g->fwd_col;
            for (int64_t p = off[gen]; p < off[gen + 1]; p++) {
                int32_t y = col[p];
                if (y == gen) continue;
                cnt[0]++;
                for (int dir2 = 0; dir2 < 2; dir2++) {
                    const int64_t* off2 = dir2 ? g->bwd_off : g->fwd_off;
                    const int32_t* col2 = dir2 ? g->bwd_col : g->fwd_col;
                    for (int64_t p2 = off2[y]; p2 < off2[y + 1]; p2++) {
                        int32_t z = col2[p2];
                        if (z == gen || rc_in_row(g, gen, z)) continue;
                        cnt[1]++;
                        keyed kk = {rc_key(g, a, z, RC_SCORE(z)), z};
                        kv_push(kv, kk);
                    }
                }
            }
        }
        out = rc_topk(kv, rem2, out_arr + c);
        c += out;
    }
    int rnd = d - 1 - sy - in - out;
    /* uniform fill over [0, n-1) without the generator and earlier choices */
    for (uint32_t i = 0; rnd > 0; i++) {
        uint32_t r[4];
        if (i >= OG_RC_FILL_BLOCKS) return -1;
        rng(g->seed, S_FILL, g->replica, (uint32_t)g->epoch, (uint32_t)a, i, r);
        for (int q = 0; q < 4 && rnd > 0; q++) {
            int32_t v = (int32_t)(((uint64_t)r[q] * (uint64_t)(n - 1)) >> 32);
            cnt[2]++;
            int dup = 0;
            for (int z = 0; z < c; z++)
                if (out_arr[z] == v) {
                    dup = 1;
                    break;
                }
            if (dup) continue;
            out_arr[c++] = v;
            rnd--;
        }
    }
#undef RC_SCORE
    info[0] = w3[0];
    info[1] = w3[1];
    info[2] = w3[2];
    info[3] = alpha;
    info[4] = (double)gen;
    info[5] = (double)d;
    memcpy(out_sorted, out_arr, sizeof(int32_t) * (size_t)c);
    qsort(out_sorted, (size_t)c, sizeof(int32_t), cmp_i32);
    return c;
}

int og_rc_epoch(og_graph* g, int threads) {
    if (!g->rc || g->n < 2) return 6;
    const int64_t n = g->n;
    const int64_t delta = (int64_t)ceil((double)n * g->rc_growth);
    if (delta <= 0) return 3;
    double* pa = (double*)malloc(sizeof(double) * (size_t)n);
    double* rec = (double*)malloc(sizeof(double) * (size_t)n);
    double* fit = (double*)malloc(sizeof(double) * (size_t)n);
    rc_scores(g, pa, rec, fit);
    int32_t* rows = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta * 256);
    int32_t* arr = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta * 256);
    int32_t* kk = (int32_t*)malloc(sizeof(int32_t) * (size_t)delta);
    free(g->rc_agents);
    g->rc_agents = (double*)malloc(sizeof(double) * 6 * (size_t)delta);
    int64_t rows_exp = 0, elems = 0, draws = 0;
    int failed = 0;
    /* the reference's per-paper citation capacity (src/kernel.cu:1151) */
    int dmax = n - 1 < 250 ? (int)(n - 1) : 250;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : rows_exp, elems, draws) reduction(| : failed)
    {
        keyvec kv = {0, 0, 0};
#pragma omp for schedule(dynamic, 16)
        for (int64_t a = 0; a < delta; a++) {
            uint32_t r[4];
            rng(g->seed, S_OUTDEG, g->replica, (uint32_t)g->epoch, (uint32_t)a, 0, r);
            uint64_t u = join64(r[0], r[1]);
            int d = OG_TABLE - 1;
            for (int i = 0; i < OG_TABLE; i++)
                if (u < g->rc_bag[i]) {
                    d = i;
                    break;
                }
            if (d < 1) d = 1;
            if (d > dmax) d = dmax;
            int64_t cnt[3] = {0, 0, 0};
            int c = rc_agent(g, a, delta, d, pa, rec, fit, rows + a * 256, arr + a * 256, cnt, &kv,
                             g->rc_agents + 6 * a);
            if (c < 0) {
                failed = 1;
                c = 0;
            }
            kk[a] = c;
            rows_exp += cnt[0];
            elems += cnt[1];
            draws += cnt[2];
        }
        free(kv.v);
    }
    if (failed) {
        free(pa);
        free(rec);
        free(fit);
        free(rows);
        free(arr);
        free(kk);
        return 4;
    }
    int64_t* row_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(delta + 1));
    row_off[0] = 0;
    for (int64_t a = 0; a < delta; a++) row_off[a + 1] = row_off[a] + kk[a];
    int64_t e_new = row_off[delta];
    int32_t* flat = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e_new + 1));
    free(g->arrivals);
    g->arrivals = (int32_t*)malloc(sizeof(int32_t) * (size_t)(e_new + 1));
    for (int64_t a = 0; a < delta; a++) {
        memcpy(flat + row_off[a], rows + a * 256, sizeof(int32_t) * (size_t)kk[a]);
        memcpy(g->arrivals + row_off[a], arr + a * 256, sizeof(int32_t) * (size_t)kk[a]);
    }
    /* new papers: peak fitness from the power-law table, static window (lag 0, duration 1000) */
    float* nf = (float*)malloc(sizeof(float) * (size_t)delta);
    for (int64_t a = 0; a < delta; a++) {
        uint32_t r[4];
        rng(g->seed, S_RCFIT, g->replica, (uint32_t)g->epoch, (uint32_t)a, 0, r);
        uint64_t u = join64(r[0], r[1]);
        int v = OG_RC_FIT_MAX;
        for (int i = 0; i < OG_RC_FIT_MAX; i++)
            if (u < g->rc_fit_table[i]) {
                v = i + 1;
                break;
            }
        nf[a] = (float)v;
    }
    append_rows(g, delta, row_off, flat, (int32_t)g->epoch, nf);
    g->rc_lag = (int32_t*)realloc(g->rc_lag, sizeof(int32_t) * (size_t)g->n);
    g->rc_dur = (int32_t*)realloc(g->rc_dur, sizeof(int32_t) * (size_t)g->n);
    for (int64_t j = n; j < g->n; j++) {
        g->rc_lag[j] = 0;
        g->rc_dur[j] = 1000;
    }
    g->stats[0] = n;
    g->stats[1] = rows_exp;
    g->stats[2] = elems;
    g->stats[3] = draws;
    g->stats[4] = e_new;
    g->stats[5] = 0;
    g->epoch++;
    free(pa);
    free(rec);
    free(fit);
    free(rows);
    free(arr);
    free(kk);
    free(row_off);
    free(flat);
    free(nf);
    return 0;
}

void og_rc_copy_agents(const og_graph* g, double* out6) {
    /* agents of the last epoch = nodes added by it */
    if (g->rc_agents) memcpy(out6, g->rc_agents, sizeof(double) * 6 * (size_t)(g->n - g->stats[0]));
}
