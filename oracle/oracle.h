/*
 * oracle.h -- CPU restatement of ParAGraph's per-epoch graph-growth step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine and the timed CPU
 * baseline; the product (paragraph_gb300) never links, loads or calls it.  Only tests/, the
 * smoke() entry of __graft_entry__.py and bench.py's CPU legs use it.
 *
 * Parity status: the reference ships no tests, golden vectors or fixed seeds, and it cannot be
 * built here (it needs cuCollections, which is absent), so this restatement is pinned by the
 * published Philox4x32-10 known-answer vectors, by libm error bounds for the elementary functions,
 * and by distribution-level checks against independent samplers; its choice-level agreement with
 * the reference itself is unpinned.
 */
#ifndef PG_ORACLE_H
#define PG_ORACLE_H
#include <stdint.h>

typedef struct og_graph og_graph;

/* elementary building blocks (independent restatements) */
void og_philox(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]);
float og_logf(float x);
/* Largest error of og_logf over every float in [lo, hi] (0 < lo <= hi), in units in the last place
 * of the correctly rounded result; the ER skip's fp32 estimate relies on it being below 2. */
double og_logf_max_ulp(float lo, float hi);
float og_expf(float x);
double og_log(double x);
double og_exp(double x);
void og_poisson_table(double lambda, uint64_t* table); /* 257 entries */
float og_fitness(uint64_t seed, uint32_t replica, uint32_t epoch, uint32_t unit);

/* graph state */
og_graph* og_create(uint64_t seed, uint32_t replica);
void og_destroy(og_graph* g);
int og_load(og_graph* g, int64_t n, const int32_t* pub, const float* fitness, int64_t m,
            const int32_t* src, const int32_t* dst);
int og_set_params(og_graph* g, double alpha, double tau, double gamma, double beta,
                  double mean_out_degree, double growth_rate, int64_t fixed_new_nodes,
                  int32_t num_anchors);
void og_set_epoch(og_graph* g, int64_t epoch);
/* 0: thinning sampler (default), 1: full 2-hop neighbourhood enumeration */
void og_set_sampler(og_graph* g, int sampler);
int64_t og_epoch(const og_graph* g);

/* one step; threads <= 0 uses every OpenMP thread.  Returns 0 on success. */
int og_pa_epoch(og_graph* g, int threads);
int og_er_epoch(og_graph* g, int64_t delta, double p, int threads);

/* readers */
int64_t og_num_nodes(const og_graph* g);
int64_t og_num_edges(const og_graph* g);
void og_copy_csr(const og_graph* g, int which, int64_t* off, int32_t* col);
void og_copy_degrees(const og_graph* g, int32_t* indeg, int32_t* outdeg);
void og_copy_nodes(const og_graph* g, int32_t* pub, float* fitness);
/* last epoch: first edge index (forward-CSR order) and count; arrivals in arrival order */
void og_epoch_edges(const og_graph* g, int64_t* first, int64_t* count);
void og_copy_arrivals(const og_graph* g, int32_t* cited);
/* last epoch counters: nodes_weighted, rows_expanded, elems_streamed, draws, new_edges, adj_scanned */
void og_stats(const og_graph* g, int64_t* out6);
/* last epoch weights w0 (float, n_pre entries) and CDF (uint64) for unit tests */
int64_t og_copy_weights(const og_graph* g, float* w, uint64_t* cdf, int32_t* shift);

/* anchors of an epoch's agents: [agents][4], unused slots -1 (uniform over the n existing nodes) */
void og_agent_anchors(uint64_t seed, uint32_t replica, uint32_t epoch, int64_t n, int64_t agents,
                      int num_anchors, int32_t* out);

/* A growth trace: the seed graph, then epochs of agents (agent a is node epoch_nodes[0] + a) with
 * their anchors and their citations in draw order. */
typedef struct {
    int64_t num_nodes;          /* nodes at the end of the trace */
    const int32_t* pub;         /* [num_nodes] publication epoch */
    const float* fitness;       /* [num_nodes] */
    int64_t num_seed_edges;
    const int32_t* seed_src;
    const int32_t* seed_dst;
    int32_t num_epochs;
    int32_t num_anchors;
    const int64_t* epoch_nodes; /* [num_epochs + 1] nodes when each epoch began; last = num_nodes */
    const int32_t* epoch_t;     /* [num_epochs] epoch index t of each trace epoch */
    const int32_t* anchors;     /* [agents][4] */
    const int64_t* cite_off;    /* [agents + 1] */
    const int32_t* cites;       /* citations of each agent in draw order */
} og_trace;

/* FP64 log-likelihood of the trace at each theta[b] = (alpha, tau, gamma, beta); grad ([batch][4])
 * may be NULL.  Returns 0, or 4 when a normaliser was not positive. */
int og_loglik(const og_trace* trace, int batch, const double* theta, double* ll, double* grad,
              int threads);

/* ---- refcompat functor: ParAGraph's own per-paper model ----
 * prm: pa, rec, fit weights (all >= 0: fixed, normalised; else drawn per agent), alpha (< 0: per
 * agent), fully_random, same_year, growth_rate, gamma, decay.  bag: out-degree bag; rec[dy]:
 * recency probability of age dy in [0, rec_len).  Returns 0 or 3. */
int og_rc_configure(og_graph* g, const double* prm, const int32_t* bag, int64_t bag_len,
                    const double* rec, int32_t rec_len);
void og_rc_bag_table(const int32_t* bag, int64_t len, uint64_t* table);    /* 257 entries */
void og_rc_fitness_table(uint64_t* table);                                  /* 1000 entries */
/* fitness window of nodes [first, first+count): lag, peak value, duration */
void og_rc_set_nodes(og_graph* g, int64_t first, int64_t count, const int32_t* lag,
                     const int32_t* peak, const int32_t* dur);
int og_rc_epoch(og_graph* g, int threads);
/* last refcompat epoch, per agent: pa, rec, fit weights, alpha, generator, out-degree */
void og_rc_copy_agents(const og_graph* g, double* out6);

#endif
