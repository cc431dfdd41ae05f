/*
 * paragraph_gb300.h -- C ABI of the GB300 (sm_103a) per-epoch graph-growth engine.
 *
 * One context owns one CUDA device stream and one device arena holding R >= 1 citation graphs
 * ("replicas").  R == 1 is the plain drop-in for ParAGraph's per-epoch growth step; R > 1 is the
 * batched ensemble.  Every entry point returns a pg_status; pg_last_error() gives the message.
 * No C++ exception crosses this boundary and no entry point takes a torch or CUDA type.
 *
 * Reference interfaces replaced (paths are inside the ParAGraph project):
 *   pg_load_graph / pg_load_replicas <- Graph::ParseNodelist / ParseEdgelist / AddEdge and the
 *                                       per-epoch host CSR rebuild prepareGraph
 *                                       (src/graph.cu:336-447, src/graph.cu:820-826,
 *                                        src/utils.cu:75-142)
 *   pg_grow_epoch                    <- buildOneNodeConnections_timed (src/kernel.cu:1125-1586) plus
 *                                       the host edge insert and in-degree update that follow it in
 *                                       execute() (src/kernel.cu:1766-1815, src/graph.cu:537-618)
 *   pg_rc_configure + pg_grow_epoch  <- the same step with the reference's own model (context
 *     (weight_model REFCOMPAT)          created with PG_WEIGHTS_REFCOMPAT): its linear score mix
 *                                       (src/abm.cu:112-208,324-338), budget split, same-year,
 *                                       1-hop / 2-hop picks and uniform fill (src/kernel.cu:196-402,
 *                                       src/abm.cu:376-565)
 *   pg_er_epoch                      <- the G(n,p) growth step of the reference's ER model, whose
 *                                       semantics are recorded in results/slurm-8634746.out:60-73
 *   pg_copy_edges / pg_epoch_edges   <- append_device_to_host (includes/utils.cuh:151-200) and the
 *                                       new_edges_vec the step appends to
 *   pg_copy_degrees                  <- Graph::GetInDegree / GetOutDegree (src/graph.cu:537-618)
 *   pg_get_stats                     <- EpochTiming / print_epoch_report
 *                                       (includes/epoch_profiler.cuh:56-242)
 */
#ifndef PARAGRAPH_GB300_H
#define PARAGRAPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PG_OK = 0,
    PG_ERR_CUDA = 1,      /* a CUDA runtime call failed */
    PG_ERR_CAPACITY = 2,  /* a node/edge/agent capacity would be exceeded */
    PG_ERR_ARG = 3,       /* invalid argument (bad id, size or parameter) */
    PG_ERR_TIMEOUT = 4,   /* a bounded device wait ran out (status read back from the device) */
    PG_ERR_IO = 5,        /* file input/output failed */
    PG_ERR_STATE = 6      /* call made in the wrong state (e.g. grow before load) */
} pg_status;

/* Weight functors for the preferential-attachment step. */
enum {
    PG_WEIGHTS_BASELINE = 0,  /* w_j = f_j^gamma (indeg_j+1)^alpha exp(-(t-t_j)/tau) beta^[j in N_a] */
    PG_WEIGHTS_REFCOMPAT = 1  /* ParAGraph's pa/rec/fit linear mix with its budget split */
};

/* Largest out-degree a single agent may draw; the Poisson table saturates here. */
#define PG_MAX_OUT_DEGREE 256
/* Most anchors a baseline agent may use for its neighbourhood. */
#define PG_MAX_ANCHORS 4

typedef struct pg_ctx pg_ctx;

typedef struct {
    int32_t device;        /* CUDA device ordinal */
    int32_t num_replicas;  /* R >= 1 */
    uint64_t seed;         /* Philox key */
    int32_t weight_model;  /* PG_WEIGHTS_* */
    int32_t record_trace;  /* 1: keep each epoch's arrival-ordered citations for pg_loglik_* */
    int32_t sampler;       /* PG_SAMPLER_* */
    int32_t replica_base;  /* RNG index of replica 0 (replica r draws as replica_base + r), so a
                              single-replica context can reproduce replica i of a batched one */
} pg_config;

/* How an agent draws its citations; both give the same law (weighted sampling without
 * replacement with weights w_j beta^[j in 2-hop ball]) from different random streams. */
enum {
    PG_SAMPLER_THINNING = 0,  /* Poisson thinning against ball membership; cost independent of the
                                 ball's size (default) */
    PG_SAMPLER_ENUMERATE = 1  /* warp-cooperative streaming of the whole 2-hop ball with per-node
                                 exponential keys */
};

/* Per-replica model parameters (baseline functor). */
typedef struct {
    double alpha;            /* exponent on (indeg+1) */
    double tau;              /* recency time constant, epochs */
    double gamma;            /* exponent on fitness */
    double beta;             /* neighbourhood boost, >= 1 */
    double mean_out_degree;  /* Poisson mean of the out-degree, clipped to [1, n] */
    double growth_rate;      /* > 0: new nodes per epoch = ceil(n * growth_rate) */
    int64_t fixed_new_nodes; /* used when growth_rate <= 0 */
    int32_t num_anchors;     /* 1..PG_MAX_ANCHORS */
    int32_t reserved;
} pg_pa_params;

/* One replica's seed graph and capacities.  Ids are dense in [0, num_nodes). */
typedef struct {
    int64_t num_nodes;
    const int32_t* pub_epoch;  /* [num_nodes] publication epoch (may be negative) */
    const float* fitness;      /* [num_nodes] > 0 */
    int64_t num_edges;
    const int32_t* src;        /* [num_edges] citing node */
    const int32_t* dst;        /* [num_edges] cited node */
    int64_t node_capacity;     /* >= num_nodes; 0 derives it from params and planned_epochs */
    int64_t edge_capacity;     /* 0 derives it */
    int32_t planned_epochs;    /* epochs the capacities must cover when derived */
    int32_t reserved;
    pg_pa_params params;
} pg_replica_desc;

/* Counters of the last epoch (summed over replicas) and per-kernel device times. */
typedef struct {
    int64_t epoch;             /* index of the last epoch run */
    int64_t new_nodes;
    int64_t new_edges;
    int64_t nodes_weighted;    /* nodes whose weight and CDF entry were computed */
    int64_t rows_expanded;     /* adjacency rows (fwd+bwd pairs) read by the neighbourhood stage */
    int64_t elems_streamed;    /* neighbourhood elements keyed (with multiplicity) */
    int64_t draws;             /* global-race draws */
    int64_t bwd_moved;         /* old backward entries copied because their row outgrew its room */
    int64_t bytes_alg;         /* algorithmic bytes of the epoch (per-stage byte model of the engine) */
    int64_t bytes_alg_agents;  /* algorithmic bytes of the agent kernel alone */
    double ms_total;           /* device time of the whole epoch, CUDA events */
    double ms_weights;         /* weights + quantise + CDF scan */
    double ms_setup;           /* out-degree draw + edge-offset scan */
    double ms_agents;          /* the agent kernel(s) */
    double ms_csr;             /* CSR append */
    double ms_er;              /* ER count + emit (ER epochs) */
    /* totals of the last pg_run_epochs call (every epoch of the run) */
    int64_t run_epochs;
    int64_t run_new_nodes;
    int64_t run_new_edges;
    int64_t run_rows_expanded;
    int64_t run_elems_streamed;
    int64_t run_draws;
    int64_t run_bwd_moved;
    int64_t run_nodes_weighted;
    int64_t run_bytes_alg;
    int64_t run_bytes_alg_agents;
    double run_ms_weights;     /* sums over the run's epochs, CUDA events on the context stream */
    double run_ms_setup;
    double run_ms_agents;
    double run_ms_csr;
    int64_t run_kernel_launches; /* kernels the run enqueued (graph nodes when captured) */
    int64_t adj_scanned;       /* adjacency entries examined by ball-membership tests (thinning) */
    int64_t run_adj_scanned;
    /* last pg_loglik_fwd: ball elements summed over agents, adjacency entries read to build the
     * balls, citations; device milliseconds of the last pg_loglik_fwd and pg_loglik_bwd calls */
    int64_t lik_ball_elems;
    int64_t lik_adj_entries;
    int64_t lik_citations;
    double lik_ms_fwd;
    double lik_ms_bwd;
} pg_stats;

/* ---- lifecycle ---- */
pg_status pg_create(pg_ctx** out, const pg_config* cfg);
void pg_destroy(pg_ctx* ctx);
const char* pg_last_error(const pg_ctx* ctx);
const char* pg_status_string(pg_status s);

/* ---- graph input ---- */
/* Replica 0 of a context created with num_replicas == 1, default parameters, capacities derived
 * from planned_epochs.  Edge semantics follow Graph::AddEdge: duplicates collapse, self-loops stay. */
pg_status pg_load_graph(pg_ctx* ctx, int64_t n, const int32_t* pub_epoch, const float* fitness,
                        int64_t m, const int32_t* src, const int32_t* dst);
/* Set all replicas at once (required before the first epoch when R > 1). */
pg_status pg_load_replicas(pg_ctx* ctx, const pg_replica_desc* descs, int32_t num);
pg_status pg_set_params(pg_ctx* ctx, int32_t replica, const pg_pa_params* params);
pg_status pg_default_params(pg_pa_params* out);
/* Current epoch index (publication epoch of the next cohort); default 0. */
pg_status pg_set_epoch(pg_ctx* ctx, int64_t epoch);

/* ---- growth ---- */
/* One preferential-attachment epoch over every replica.  Synchronous: on return new_nodes /
 * new_edges hold the totals over replicas (either pointer may be NULL). */
pg_status pg_grow_epoch(pg_ctx* ctx, int64_t* new_nodes, int64_t* new_edges);
/* num_epochs PA epochs without host synchronisation between them; use_graph != 0 captures the
 * whole run in one CUDA graph the first time and replays it afterwards. */
pg_status pg_run_epochs(pg_ctx* ctx, int32_t num_epochs, int32_t use_graph, int64_t* new_edges);
/* pg_run_epochs that also delivers every new citation (source, target) into src/dst (capacity
 * entries each), epoch by epoch and, within an epoch, replica by replica in forward-CSR order; the
 * per-epoch, per-replica counts go to counts[epoch * num_replicas + r] (may be NULL).  Page-locked
 * buffers (cudaHostAlloc / cudaHostRegister) are written by the device while the next epoch runs,
 * so the copy-out overlaps the growth; other buffers are filled after the run.  An epoch whose
 * citations do not fit the remaining capacity is grown but not written: the call then returns
 * PG_ERR_CAPACITY with *new_edges = the citations written (the context stays usable).  Replaces the
 * reference's per-agent cudaMemcpy of the edges back to the host (includes/utils.cuh:151-200). */
pg_status pg_run_epochs_out(pg_ctx* ctx, int32_t num_epochs, int32_t use_graph, int32_t* src, int32_t* dst,
                            int64_t capacity, int64_t* counts, int64_t* new_edges);
/* One Erdos-Renyi G(n,p) epoch on replica 0: delta new nodes, each linking to every pre-epoch node
 * with probability p, by geometric skips. */
pg_status pg_er_epoch(pg_ctx* ctx, int64_t delta, double p, int64_t* new_edges);
/* num_epochs ER epochs of delta new nodes each, enqueued without host synchronisation between them
 * (the node counts of every epoch are known in advance; the arena is sized for the run from an
 * 8-sigma bound on its edges, and a device check stops the run with PG_ERR_CAPACITY if it is
 * exceeded).  Edges and graph equal num_epochs calls of pg_er_epoch. */
pg_status pg_run_er_epochs(pg_ctx* ctx, int32_t num_epochs, int64_t delta, double p, int64_t* new_edges);
/* Grow a single-replica context to hold at least n_cap nodes and m_cap citations before its
 * epochs run (ER epochs, whose edge count a PA plan does not cover, otherwise grow the arena
 * through the host when they outrun it).  No-op when the capacity suffices; growing the arena
 * drops a checkpoint and a captured run graph (both refer to the old buffers). */
pg_status pg_reserve(pg_ctx* ctx, int64_t n_cap, int64_t m_cap);

/* ---- refcompat functor: ParAGraph's own per-paper model (the abm driver's options) ---- */
typedef struct {
    double pa_weight;     /* --preferential-weight; all three >= 0: fixed (normalised to sum 1), */
    double rec_weight;    /* --recency-weight        else each agent draws three U(0,1) weights   */
    double fit_weight;    /* --fitness-weight        and normalises them (ABM::PopulateWeightArrs) */
    double alpha;         /* --alpha: share of the neighbourhood budget taken from the 1-hop set;
                             < 0: U(0,1) per agent (ABM::PopulateAlphaArr) */
    double fully_random;  /* --fully-random-citations: out-degree fraction reserved for uniform picks */
    double same_year;     /* --same-year-proportion: fraction of each epoch's agents citing a paper
                             of their own epoch */
    double growth_rate;   /* --growth-rate: new papers per epoch = ceil(n * growth_rate) */
    int32_t gamma;        /* exponent of the in-degree and fitness scores, 1..4 (reference: 3) */
    int32_t decay;        /* fitness decay exponent after the peak window, 0..8 (reference: 3) */
} pg_rc_params;
/* Configures replica `replica` of a PG_WEIGHTS_REFCOMPAT context after pg_load_graph (whose
 * fitness values are the seed papers' peak fitness; lag 0, duration 1000): the parameters, the
 * out-degree bag (ABM::ReadOutDegreeBag, src/abm.cu:70-89; values clipped to [0, 256], out-degrees
 * to [1, min(250, n-1)], 250 being the reference's per-paper citation capacity, src/kernel.cu:1151) and the recency probabilities rec[age] for age 0..rec_len-1, rec_len <= 1024
 * (ABM::ReadRecencyProbabilities, src/abm.cu:91-110).  pg_grow_epoch / pg_run_epochs then run the
 * reference's per-paper rule on the device. */
pg_status pg_rc_configure(pg_ctx* ctx, int32_t replica, const pg_rc_params* params, const int32_t* bag,
                          int64_t bag_len, const double* rec, int32_t rec_len);
/* Fitness windows of papers [first, first+count): lag, peak value (>= 1), peak duration -- the
 * planted papers of ABM::PlantNodes (includes/abm.cuh:486-504). */
pg_status pg_rc_set_nodes(pg_ctx* ctx, int32_t replica, int64_t first, int64_t count, const int32_t* lag,
                          const int32_t* peak, const int32_t* dur);
/* Per-paper draws of the last refcompat epoch, [new_nodes][6]: pa, rec and fit weights, alpha,
 * generator node, out-degree (the agent columns of Graph::WriteAttributes, src/graph.cu:1057-1211). */
pg_status pg_rc_copy_agents(pg_ctx* ctx, int32_t replica, double* out);
/* Host tables shared with tests: the bag's 257-entry CDF and the 1000-entry peak-fitness CDF (2^64). */
pg_status pg_rc_bag_table(const int32_t* bag, int64_t len, uint64_t* table);
pg_status pg_rc_fitness_table(uint64_t* table);

/* ---- output ---- */
pg_status pg_get_counts(const pg_ctx* ctx, int32_t replica, int64_t* n, int64_t* m);
/* Range [first, first+count) of the last epoch's edges in forward-CSR order. */
pg_status pg_epoch_edges(const pg_ctx* ctx, int32_t replica, int64_t* first, int64_t* count);
/* Edges [first, first+count) in forward-CSR order (source ascending, then target ascending). */
pg_status pg_copy_edges(pg_ctx* ctx, int32_t replica, int64_t first, int64_t count,
                        int32_t* src, int32_t* dst);
pg_status pg_copy_degrees(pg_ctx* ctx, int32_t replica, int32_t* indeg, int32_t* outdeg);
pg_status pg_copy_nodes(pg_ctx* ctx, int32_t replica, int32_t* pub_epoch, float* fitness);
/* which: 0 forward (out-edges), 1 backward (in-edges).  off has n+1 entries, col m.  The backward
 * rows are kept with room to grow in the device arena; this returns them compacted in node order. */
pg_status pg_copy_csr(pg_ctx* ctx, int32_t replica, int32_t which, int64_t* off, int32_t* col);
/* Citations of the last epoch in arrival order ([count] as from pg_epoch_edges); needs
 * record_trace. */
pg_status pg_copy_arrivals(pg_ctx* ctx, int32_t replica, int32_t* cited);
/* Anchors of the last PA epoch's agents, [new_nodes][4] with unused slots -1; needs record_trace.
 * (The reference draws one generator node per paper, getGeneratorNode, src/abm.cu:567-574.) */
pg_status pg_copy_anchors(pg_ctx* ctx, int32_t replica, int32_t* anchors);

/* The replica's edge list as text, one "source,target\n" line per edge in forward-CSR order (the
 * rows of Graph::WriteGraph, src/graph.cu:909-1003, without its "#source,target" header), node v
 * printed as ids[v] (n_ids = the replica's node count); formatted on the device.  out == NULL only
 * reports the size in *bytes; a buffer smaller than the text gives PG_ERR_CAPACITY. */
pg_status pg_format_edges(pg_ctx* ctx, int32_t replica, const int64_t* ids, int64_t n_ids, char* out,
                          int64_t cap, int64_t* bytes);

/* The rows of the attribute file (Graph::WriteAttributes, src/graph.cu:1057-1218, without its
 * header line), formatted on the device, one line per node v of the replica:
 *   id,type,year,pa_weight,rec_weight,fit_weight,fit_lag_duration,fit_peak_value,
 *   fit_peak_duration,alpha,in_degree,out_degree,assigned_out_degree,planted_line,generators
 * The weights and alpha print as C's "%.10g", the peak as "%d" of the fitness (peak_integer != 0,
 * the refcompat model's integer peaks) or "%.9g" of the fp32 fitness; nodes v < num_seed are
 * typed "seed" with generators "no_generators", the rest "agent" with their generator ids joined
 * by ';' ("-1" when none).  Year, fitness and degrees are the replica's own; the caller gives the
 * printed ids and the per-paper columns.  out == NULL only reports the size in *bytes; a smaller
 * buffer gives PG_ERR_CAPACITY. */
typedef struct {
    int64_t num_nodes;         /* the replica's node count */
    int64_t num_seed;          /* nodes typed "seed" (the loaded graph) */
    const int64_t* ids;        /* [num_nodes] printed node ids */
    const double* draws;       /* [num_nodes][4] pa, rec, fit weight, alpha (-1 where absent) */
    const int32_t* ints;       /* [num_nodes][4] fitness lag, peak duration, assigned out-degree,
                                  planted-papers line (-1 where absent) */
    const int64_t* generators; /* [num_nodes][4] printed ids of each agent's generators, -1 unused */
    int32_t peak_integer;      /* 1: the peak column is "%d" of the fitness; 0: "%.9g" */
    int32_t reserved;
} pg_attr_rows;
pg_status pg_format_attributes(pg_ctx* ctx, int32_t replica, const pg_attr_rows* rows, char* out,
                               int64_t cap, int64_t* bytes);

/* ---- measurement ---- */
/* enable != 0 records CUDA events around every kernel group of each epoch (default on). */
pg_status pg_set_timing(pg_ctx* ctx, int32_t enable);
pg_status pg_get_stats(const pg_ctx* ctx, pg_stats* out);
pg_status pg_sync(pg_ctx* ctx);
/* Reads the device error word; PG_OK when no kernel reported a fault. */
pg_status pg_check_device(pg_ctx* ctx);
/* Stream-ordered timer on the context's stream: stop waits for the stream and returns the
 * milliseconds between the two CUDA events. */
pg_status pg_timer_start(pg_ctx* ctx);
pg_status pg_timer_stop(pg_ctx* ctx, double* ms);

/* ---- checkpoint / resume ---- */
/* Save the whole graph state (nodes, both CSRs, epoch counter) in device memory; pg_restore puts
 * it back, so a run can be repeated or resumed bit-exactly (the RNG is counter-based). */
pg_status pg_checkpoint(pg_ctx* ctx);
pg_status pg_restore(pg_ctx* ctx);

/* ---- launch tuning (no counterpart in the reference; results never depend on it) ---- */
typedef struct {
    int32_t agent_ctas_per_sm; /* CTAs per SM of the k <= 64 agent kernel; 0 = occupancy limit */
    int32_t small_hash;        /* shape of that kernel: 0 a 2048-slot frontier hash per warp and
                                  512-entry stage buffers; 1 1024 slots, 1024-entry stages */
    int32_t copy_ctas_per_sm;  /* CTAs per SM of the copy of moved backward rows; 0 = default (8) */
    int32_t lik_chunk_agents;  /* > 0: pg_trace_load keeps at most this many agents' neighbourhood
                                  balls per chunk, so every likelihood pass rebuilds them chunk by
                                  chunk; 0: as many as fit in a quarter of free device memory (one
                                  chunk = built once and reused by every pass) */
    int32_t epoch_kernel;      /* 1: each epoch of the thinning sampler with the baseline weights is
                                  ONE persistent cooperative kernel over all replicas (every stage
                                  a phase, grid barriers between them); 0: the sequence of stage
                                  kernels.  Ignored (0) where the device cannot launch it. */
    int32_t er_slot_sigmas;    /* ER: each (new node, 2^16-id chunk) walk writes its edges into slots
                                  reserved for mean + this many standard deviations + 8 of its
                                  binomial count (0 = default 8); a walk with more edges finishes in
                                  an overflow pass.  Small values send many walks there (tests). */
} pg_tuning;
pg_status pg_set_tuning(pg_ctx* ctx, const pg_tuning* tuning);
pg_status pg_get_tuning(const pg_ctx* ctx, pg_tuning* tuning);
/* Times every candidate tuning on the next num_epochs epochs of the loaded replicas and keeps the
 * fastest (written to best, its time in milliseconds to best_ms; either may be NULL).  The graph is
 * saved before and put back after every candidate, so the context is left exactly as it was; a
 * checkpoint taken earlier with pg_checkpoint is kept.  Every candidate must produce the same edge
 * count, else PG_ERR_STATE. */
pg_status pg_autotune(pg_ctx* ctx, int32_t num_epochs, pg_tuning* best, double* best_ms);

/* ---- failure-path hook (no counterpart in the reference, which turns any CUDA error into exit
 * status 1, src/kernel.cu:1761-1764) ----
 * The thinning agent kernel stages candidate rows with asynchronous bulk copies and waits for each
 * on an mbarrier with a bounded number of polls (default 2^22).  This sets the bound of the FIRST
 * wait on each staged chunk; polls = 0 makes every first wait give up at once, negative restores
 * the default.  A wait that gives up sets the device error word (the epoch then returns
 * PG_ERR_TIMEOUT and the context refuses growth until pg_restore or a reload); the warp then waits
 * again, with the full bound, for its copies in flight, so none is left running when it stops.
 * For tests of that path; results of epochs that succeed do not depend on it. */
pg_status pg_set_wait_limit(pg_ctx* ctx, int64_t polls);

/* ---- log-likelihood of a growth trace and its adjoint (no counterpart in the reference) ----
 * A trace is a seed graph followed by epochs of agents; agent a (node epoch_nodes[0] + a, in the
 * epoch whose node range holds it) drew its citations c_1..c_k in the recorded order by
 * successive sampling without replacement over the nodes j < n_e that existed when the epoch
 * began, with weights
 *   W_j = fitness_j^gamma (indeg_e(j)+1)^alpha exp(-(t_e - t_j)/tau) beta^[j in N_a],
 * indeg_e the in-degree in the epoch-start graph and N_a the undirected 2-hop ball of the agent's
 * anchors in that graph.  log L(theta) = sum_a sum_i [log W_{c_i} - log(Z_a - sum_{l<i} W_{c_l})],
 * Z_a = sum_{j < n_e} W_j, theta = (alpha, tau, gamma, beta).  Weights are fp32; Z_a, the prefix
 * sums and the log-sums are FP64. */
typedef struct {
    int64_t num_nodes;          /* nodes at the end of the trace */
    const int32_t* pub_epoch;   /* [num_nodes] */
    const float* fitness;       /* [num_nodes] > 0 */
    int64_t num_seed_edges;     /* edges among the seed nodes (set semantics) */
    const int32_t* seed_src;
    const int32_t* seed_dst;
    int32_t num_epochs;
    int32_t num_anchors;        /* anchors per agent, 1..PG_MAX_ANCHORS */
    const int64_t* epoch_nodes; /* [num_epochs + 1] nodes when each epoch began; last = num_nodes */
    const int32_t* epoch_t;     /* [num_epochs] epoch index t_e (recency origin) */
    const int32_t* anchors;     /* [agents][4], unused slots -1 */
    const int64_t* cite_off;    /* [agents + 1], at most PG_MAX_OUT_DEGREE citations per agent */
    const int32_t* cites;       /* citations of every agent in draw order */
} pg_trace_desc;
/* Copies the trace to the device (a trace and the growth state coexist in one context). */
pg_status pg_trace_load(pg_ctx* ctx, const pg_trace_desc* trace);
/* Arithmetic of the next forward passes (and of the adjoint passes that follow them): exact = 0
 * (the default, fastest) takes 2^x from the GPU's special-function unit (relative error < 2^-22)
 * of an exponent rounded once per node; exact = 1 carries the exponent and log f without rounding
 * of their own, takes 2^x from fp32 arithmetic accurate to about 2 ulp and sums every ball weight
 * and product on its own into compensated sums.  The per-node roundings of exact = 0 do not
 * average out and leave about 1e-5 of the gradient's norm where the gradient nearly vanishes (at a
 * trace's generating parameters; 1e-7 elsewhere); exact = 1 keeps the gradient within 1e-6 of the
 * FP64 value there too, at about a third of the throughput. */
pg_status pg_lik_set_exact_exp2(pg_ctx* ctx, int32_t exact);
/* log L at each of batch points theta[b] = (alpha, tau, gamma, beta) (row-major [batch][4]).  Saves
 * the per-agent normalisers Z_a for pg_loglik_bwd. */
pg_status pg_loglik_fwd(pg_ctx* ctx, int32_t batch, const double* theta, double* loglik);
/* Adjoint: grad[b][k] = dloglik[b] * d log L / d theta_k at the points of the last pg_loglik_fwd
 * (theta must be the same; dloglik NULL means all ones).  Weights are recomputed, not stored. */
pg_status pg_loglik_bwd(pg_ctx* ctx, int32_t batch, const double* theta, const double* dloglik,
                        double* grad);

/* ---- allocation-free generation ---- */
/* Largest delta * ceil(n_existing / 65536) that pg_er_generate_noalloc accepts. */
#define PG_NOALLOC_MAX_TASKS (1 << 18)
/* No counterpart in the reference: an Erdos-Renyi epoch's edge list written into device buffers
 * the caller owns, without allocating device memory.  It is for callers that must not call
 * cudaMalloc/cudaFree at this point -- e.g. a program timing other device work, or a runtime that
 * only hands out pre-sized buffers.  The edges equal those pg_er_epoch appends for
 * the same seed, epoch, n_existing (pre-epoch nodes), delta and p: sources n_existing + i, targets
 * in [0, n_existing), ordered by (source, target).  Scratch is a fixed 4 MiB device array inside
 * the library (held by every GPU that loads it until the process exits); delta *
 * ceil(n_existing/65536) above PG_NOALLOC_MAX_TASKS is rejected with PG_ERR_CAPACITY.  The first
 * call on a device looks up that array's device address, so make it before any stream capture.
 * Calls share the array: calls that overlap on the GPU (other streams or threads) race.  The call
 * synchronises `stream` (a cudaStream_t, NULL for the legacy default stream); *num_edges receives
 * the edge count, and when it exceeds `capacity` nothing is written and PG_ERR_CAPACITY is
 * returned. */
pg_status pg_er_generate_noalloc(uint64_t seed, int64_t epoch, int64_t n_existing, int64_t delta,
                                 double p, int32_t* d_src, int32_t* d_dst, int64_t capacity,
                                 int64_t* num_edges, void* stream);

/* ---- host-side building blocks shared with tests ---- */
/* Philox4x32-10 block (Salmon et al., SC'11) for counter c[4] and key k[2]. */
void pg_philox4x32_10(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]);
/* Poisson(lambda) CDF thresholds scaled to 2^64, PG_MAX_OUT_DEGREE+1 entries. */
pg_status pg_poisson_table(double lambda, uint64_t* table);
/* The library's own elementary functions (identical on host and device). */
float pg_logf_host(float x);
float pg_expf_host(float x);
double pg_log_host(double x);
double pg_exp_host(double x);
/* Version string of the build. */
const char* pg_version(void);
/* C's "%.<precision>g" of x (precision 1..13) into out (at least 32 bytes), returning the length:
 * the conversion pg_format_attributes runs on the device, compiled for the host. */
int32_t pg_format_g_host(double x, int32_t precision, char* out);

#ifdef __cplusplus
}
#endif
#endif /* PARAGRAPH_GB300_H */
