// pg_api.cu -- host side of the C ABI: context, device arena, epoch sequencing.
//
// Replaces the host orchestration around buildOneNodeConnections_timed (src/kernel.cu:1125-1586):
// the reference allocates and frees all device memory per call and per mini-batch, rebuilds the
// CSR on the host every epoch and copies edges back per agent.  Here the graph stays resident in
// one arena sized once (capacities planned from the growth rule), an epoch is a fixed sequence of
// kernels on one stream, and a multi-epoch run can be captured once as a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/paragraph_gb300.h"
#include "pg_engine.cuh"
#include "pg_lik.cuh"
#include "pg_rc.cuh"

using namespace pg;

namespace {

struct HostRep {
    int64_t nbase, obase, ebase, n_cap, m_cap, n, m;
    int64_t bbase = 0, b_cap = 0, b_top = 0;  // backward region (b_top: as laid out at load)
    int32_t tbase, ntiles;
    pg_pa_params prm;
    // refcompat functor (pg_rc_configure)
    bool rc = false;
    pg_rc_params rcp{};
    int32_t kmax = 0;                  // largest out-degree of the bag (clipped to [1, 256])
    std::vector<uint64_t> bag_table;   // [kTableEntries]
    std::vector<double> rtab;          // [kRcAgeMax]
};

template <typename T>
struct DBuf {
    T* p = nullptr;
    int64_t n = 0;
};

// A loaded growth trace and the buffers of the likelihood passes.
struct LikState {
    bool loaded = false;
    int64_t n = 0, n0 = 0, agents = 0;
    int epochs = 0, num_anchors = 0, words = 0, chunks = 0, ball_grid = 0, eval_grid[2] = {0, 0};
    int64_t chunk_agents = 0;  // > 0: at most this many agents' balls per chunk (pg_tuning)
    DBuf<int64_t> epoch_nodes, fo, bo, coff, boff, bcnt, badj;
    DBuf<int32_t> epoch_t, fc, bc, pub, anchors, cites, agent_epoch, bids;
    DBuf<uint8_t> cflag;
    DBuf<float> fit;
    DBuf<float4> feat;
    DBuf<double> theta, pp, zglob, gglob, gpart, zagent, out, res;
    DBuf<uint32_t> err;
    std::vector<int64_t> hboff;              // ball offsets on the host
    std::vector<std::pair<int64_t, int64_t>> ball_chunks;  // agent ranges whose balls fit in bids
    bool balls_cached = false;               // one chunk: built at load, reused by every pass
    int64_t ball_elems = 0, adj_entries = 0, citations = 0;
    std::vector<double> fwd_theta;  // points of the last forward pass
    int32_t exact_exp2 = 0;         // pg_lik_set_exact_exp2
    int32_t fwd_exact_exp2 = 0;     // the mode of the last forward pass (the adjoint reuses it)
    int32_t feat_exact = 0;         // the layout of the feature rows (the mode they were built for)
};

struct Checkpoint {
    bool valid = false;
    int64_t epoch = 0;
    std::vector<HostRep> hrep;
    std::vector<int64_t> b_top;  // backward entries in use per replica
    DBuf<int32_t> pub, indeg, fwd_col, bcol, bcap, rc_lag, rc_dur;
    DBuf<float> fit;
    DBuf<int64_t> fwd_off;
    DBuf<BRow> brow;
    DBuf<Replica> rep;
};

}  // namespace

struct pg_ctx {
    pg_config cfg{};
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;        // the hub index of an epoch, beside the weights
    cudaEvent_t fork = nullptr, join = nullptr;
    int R = 1;
    bool loaded = false;
    bool poisoned = false;  // a kernel reported an error mid-epoch; reload before growing again
    int64_t epoch = 0;
    std::vector<HostRep> hrep;
    int64_t S = 0, T = 0, M = 0;  // slots, tiles, edge slots
    int64_t B = 0;                // backward-region entries (all replicas)
    int64_t agent_cap = 0, edge_cap = 0, blocks_cap = 0;
    // device buffers
    DBuf<Replica> rep;
    DBuf<EpochState> st;
    DBuf<int32_t> tile_rep, pub, indeg, inc, kk, big_list, heavy_list, heavy_mark, e_dst, e_rank, arrivals, hlist, anchors,
        hub_rem, hub_add, hub_cand;
    DBuf<int16_t> hslot;
    DBuf<uint64_t> hub2;
    DBuf<uint32_t> hub_need;
    DBuf<int32_t> zbig;
    DBuf<uint64_t> hmask;
    DBuf<float> fit, w;
    DBuf<uint64_t> cdf, tilesum, tileoff, tables;
    DBuf<int32_t> guide;
    DBuf<int64_t> fwd_off, new_start, sort_small, sort_large, sort_large_off, eoff, blocksum, er_cnt, er_toff;
    DBuf<int32_t> fwd_col, bcol, bcap;
    DBuf<BRow> brow;
    DBuf<longlong2> reloc;  // copy tasks of the backward rows that move in an epoch
    DBuf<int2> er_slots, er_ov;  // ER walks: (position, rank) slots of every task, overflow area
    DBuf<int64_t> er_ovb;        // ER walks: start of each overflowing task's block
    DBuf<int32_t> src_tmp;  // sources of an edge range being copied out
    // refcompat functor
    DBuf<double> rc_pa, rc_rec, rc_fit, rc_rtab, rc_agent;
    DBuf<int32_t> rc_big_id;
    DBuf<long long> rc_big_meta;
    DBuf<int32_t> rc_lag, rc_dur, rc_cnt;
    DBuf<uint64_t> rc_ftab;
    DBuf<unsigned long long> rc_acc;
    // host mirror of the last epoch
    EpochState h_st{};
    std::vector<Replica> h_rep;
    pg_stats stats{};
    int64_t last_first = 0, last_count = 0;  // replica 0 bookkeeping is per replica below
    std::vector<int64_t> rep_last_first, rep_last_count;
    bool timing = true;
    cudaEvent_t ev[6] = {};
    std::vector<cudaEvent_t> run_ev;  // 5 per epoch of a pg_run_epochs call
    cudaEvent_t tev[2] = {};          // pg_timer_start / pg_timer_stop
    cudaEvent_t lev[2] = {};          // around each likelihood pass
    int64_t launches = 0;             // kernels enqueued by the last run
    // CUDA graph of a multi-epoch run
    cudaGraphExec_t gexec = nullptr;
    int64_t g_epoch0 = -1;
    int g_epochs = 0;
    const void* g_out = nullptr;  // the output buffers a captured run writes to (baked into it)
    // citation output of the current pg_run_epochs_out call (device-visible pointers; null otherwise)
    int32_t* out_src = nullptr;
    int32_t* out_dst = nullptr;
    int64_t out_cap = 0, out_epochs = 0;
    DBuf<int64_t> out_counts;
    DBuf<int32_t> out_stage_src, out_stage_dst;  // staging when the caller's buffers are pageable
    Checkpoint ckpt;
    LikState lik;
    pg_tuning tune{};
    uint32_t first_wait_polls = kWaitPolls;  // pg_set_wait_limit (failure-path tests)
    std::string err;
};

namespace {

pg_status fail(pg_ctx* c, pg_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

#define PG_CUDA(ctx, call)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(ctx, PG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

template <typename T>
cudaError_t dalloc(DBuf<T>& b, int64_t n) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    if (n <= 0) n = 1;
    cudaError_t e = cudaMalloc((void**)&b.p, sizeof(T) * (size_t)n);
    if (e == cudaSuccess) b.n = n;
    return e;
}

template <typename T>
void dfree(DBuf<T>& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

// Temporaries of a load (raw edges, sort scratch, offset-form CSR) come from a stream-ordered pool
// owned by the library: freeing them does not synchronise the device, and a later load in the same
// process reuses the memory instead of mapping it again.  The pool keeps what it holds (release
// threshold: unlimited) until the process ends: at most one load's temporaries, about 40 bytes per
// raw edge.
cudaMemPool_t temp_pool(int device) {
    static cudaMemPool_t pools[64] = {};
    if (device < 0 || device >= 64) return nullptr;
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        pools[device] = p;
    }
    return pools[device];
}

template <typename T>
cudaError_t talloc(DBuf<T>& b, int64_t n, int device, cudaStream_t s) {
    if (n <= 0) n = 1;
    b.p = nullptr;
    b.n = 0;
    cudaMemPool_t pool = temp_pool(device);
    cudaError_t e = pool ? cudaMallocFromPoolAsync((void**)&b.p, sizeof(T) * (size_t)n, pool, s)
                         : cudaMalloc((void**)&b.p, sizeof(T) * (size_t)n);
    if (e == cudaSuccess) b.n = n;
    return e;
}

template <typename T>
void tfree(DBuf<T>& b, int device, cudaStream_t s) {
    if (b.p) {
        if (temp_pool(device))
            cudaFreeAsync(b.p, s);
        else
            cudaFree(b.p);
    }
    b.p = nullptr;
    b.n = 0;
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

int64_t delta_of(const pg_pa_params& p, int64_t n) {
    if (p.growth_rate > 0.0) return (int64_t)std::ceil((double)n * p.growth_rate);
    return p.fixed_new_nodes > 0 ? p.fixed_new_nodes : 0;
}

// Upper bound on one epoch's edges for d agents (Poisson(lambda) out-degree clipped to
// [1, min(256, n)]): mean + 8 standard deviations, never above the hard bound.
int64_t edge_bound(int64_t d, double lambda, int64_t n, int32_t kmax = 0) {
    if (d <= 0) return 0;
    if (kmax > 0) return d * std::min<int64_t>(std::min<int64_t>(kmax, kKMax), std::max<int64_t>(n - 1, 1));
    const double mu = (double)d * (lambda + 1.0);
    const int64_t stat = (int64_t)std::ceil(mu + 8.0 * std::sqrt(mu) + 64.0);
    const int64_t hard = d * std::min<int64_t>(kKMax, std::max<int64_t>(n, 1));
    return std::min(stat, hard);
}

Arena make_arena(pg_ctx* c) {
    Arena A{};
    A.rep = c->rep.p;
    A.R = c->R;
    A.ntiles = (int32_t)c->T;
    A.tile_rep = c->tile_rep.p;
    A.pub = c->pub.p;
    A.fit = c->fit.p;
    A.indeg = c->indeg.p;
    A.w = c->w.p;
    A.cdf = c->cdf.p;
    A.guide = c->guide.p;
    A.inc = c->inc.p;
    A.fwd_off = c->fwd_off.p;
    A.fwd_col = c->fwd_col.p;
    A.brow = c->brow.p;
    A.bcap = c->bcap.p;
    A.bcol = c->bcol.p;
    A.reloc = c->reloc.p;
    A.reloc_cap = c->reloc.n;
    A.tables = c->tables.p;
    A.kk = c->kk.p;
    A.eoff = c->eoff.p;
    A.e_dst = c->e_dst.p;
    A.e_rank = c->e_rank.p;
    A.arrivals = c->cfg.record_trace ? c->arrivals.p : nullptr;
    A.anchors_out = c->cfg.record_trace ? c->anchors.p : nullptr;
    A.big_list = c->big_list.p;
    A.heavy_list = c->heavy_list.p;
    A.heavy_mark = c->heavy_mark.p;
    A.new_start = c->new_start.p;
    A.tilesum = c->tilesum.p;
    A.tileoff = c->tileoff.p;
    A.blocksum = c->blocksum.p;
    A.sort_small = c->sort_small.p;
    A.sort_large = c->sort_large.p;
    A.sort_large_off = c->sort_large_off.p;
    A.st = c->st.p;
    A.agent_cap = c->agent_cap;
    A.edge_cap = c->edge_cap;
    A.seed = c->cfg.seed;
    A.record_trace = c->cfg.record_trace;
    A.hslot = c->hslot.p;
    A.hmask = c->hmask.p;
    A.hub2 = c->hub2.p;
    A.hub_need = c->hub_need.p;
    A.zbig = c->zbig.p;
    A.hlist = c->hlist.p;
    A.hub_rem = c->hub_rem.p;
    A.hub_add = c->hub_add.p;
    A.hub_cand = c->hub_cand.p;
    A.out_src = c->out_src;
    A.out_dst = c->out_dst;
    A.out_cap = c->out_cap;
    A.out_counts = c->out_counts.p;
    A.out_epochs = c->out_epochs;
    A.sampler = c->cfg.sampler;
    A.tune_agent_ctas = c->tune.agent_ctas_per_sm;
    A.tune_small_hash = c->tune.small_hash;
    A.tune_copy_ctas = c->tune.copy_ctas_per_sm;
    A.rep_base = c->cfg.replica_base;
    A.first_wait_polls = c->first_wait_polls;
    A.weight_model = c->cfg.weight_model;
    A.rc_pa = c->rc_pa.p;
    A.rc_rec = c->rc_rec.p;
    A.rc_fit = c->rc_fit.p;
    A.rc_lag = c->rc_lag.p;
    A.rc_dur = c->rc_dur.p;
    A.rc_rtab = c->rc_rtab.p;
    A.rc_ftab = c->rc_ftab.p;
    A.rc_acc = c->rc_acc.p;
    A.rc_cnt = c->rc_cnt.p;
    A.rc_agent = c->rc_agent.p;
    A.rc_big_id = c->rc_big_id.p;
    A.rc_big_meta = c->rc_big_meta.p;
    return A;
}

Replica to_device_rep(const HostRep& h) {
    Replica r{};
    r.nbase = h.nbase;
    r.obase = h.obase;
    r.ebase = h.ebase;
    r.n_cap = h.n_cap;
    r.m_cap = h.m_cap;
    r.bbase = h.bbase;
    r.b_cap = h.b_cap;
    r.b_top = (unsigned long long)h.b_top;
    r.n = h.n;
    r.m = h.m;
    r.tbase = h.tbase;
    r.ntiles = h.ntiles;
    r.alpha = (float)h.prm.alpha;
    r.gamma = (float)h.prm.gamma;
    r.tau = (float)h.prm.tau;
    r.beta_m1 = h.prm.beta - 1.0;
    r.growth_rate = h.prm.growth_rate;
    r.fixed_new = h.prm.fixed_new_nodes;
    r.anchors = h.prm.num_anchors;
    r.p_global = 1.0 / h.prm.beta;
    r.glob_thr = global_threshold(r.p_global);
    r.heavy_thr = 0x7fffffff;
    if (h.rc) {
        const bool fixed = h.rcp.pa_weight >= 0.0 && h.rcp.rec_weight >= 0.0 && h.rcp.fit_weight >= 0.0;
        r.rc_w[0] = fixed ? h.rcp.pa_weight : -1.0;
        r.rc_w[1] = fixed ? h.rcp.rec_weight : -1.0;
        r.rc_w[2] = fixed ? h.rcp.fit_weight : -1.0;
        r.rc_alpha = h.rcp.alpha > 1.0 ? 1.0 : h.rcp.alpha;
        r.rc_frc = h.rcp.fully_random;
        r.rc_sy = h.rcp.same_year;
        r.rc_gamma = h.rcp.gamma;
        r.rc_decay = h.rcp.decay;
        r.rc_rec_len = (int32_t)h.rtab.size();
    }
    return r;
}

pg_status check_params(pg_ctx* c, const pg_pa_params& p) {
    if (!(p.tau > 0.0)) return fail(c, PG_ERR_ARG, "tau must be > 0");
    if (!(p.beta >= 1.0) || p.beta > 1000.0) return fail(c, PG_ERR_ARG, "beta must be in [1, 1000]");
    if (!(p.mean_out_degree >= 0.0) || p.mean_out_degree > 200.0)
        return fail(c, PG_ERR_ARG, "mean_out_degree must be in [0, 200]");
    if (p.num_anchors < 1 || p.num_anchors > PG_MAX_ANCHORS)
        return fail(c, PG_ERR_ARG, "num_anchors must be in [1, 4]");
    if (!(p.growth_rate > 0.0) && p.fixed_new_nodes <= 0)
        return fail(c, PG_ERR_ARG, "need growth_rate > 0 or fixed_new_nodes > 0");
    if (!std::isfinite(p.alpha) || !std::isfinite(p.gamma))
        return fail(c, PG_ERR_ARG, "alpha and gamma must be finite");
    return PG_OK;
}

void free_checkpoint(Checkpoint& k) {
    dfree(k.pub);
    dfree(k.indeg);
    dfree(k.fwd_col);
    dfree(k.bcol);
    dfree(k.fit);
    dfree(k.fwd_off);
    dfree(k.brow);
    dfree(k.bcap);
    dfree(k.rep);
    dfree(k.rc_lag);
    dfree(k.rc_dur);
    k.valid = false;
}

void free_lik(LikState& L) {
    DBuf<int64_t>* i64[] = {&L.epoch_nodes, &L.fo, &L.bo, &L.coff, &L.boff, &L.bcnt, &L.badj};
    for (auto* b : i64) dfree(*b);
    DBuf<int32_t>* i32[] = {&L.epoch_t, &L.fc, &L.bc, &L.pub, &L.anchors, &L.cites, &L.agent_epoch, &L.bids};
    for (auto* b : i32) dfree(*b);
    DBuf<double>* f64[] = {&L.theta, &L.pp, &L.zglob, &L.gglob, &L.gpart, &L.zagent, &L.out, &L.res};
    for (auto* b : f64) dfree(*b);
    dfree(L.cflag);
    dfree(L.fit);
    dfree(L.feat);
    dfree(L.err);
    L.hboff.clear();
    L.ball_chunks.clear();
    L.balls_cached = false;
    L.loaded = false;
    L.fwd_theta.clear();
}

void destroy_graph_exec(pg_ctx* c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->g_epoch0 = -1;
}

pg_status alloc_epoch_buffers(pg_ctx* c, int64_t agent_cap, int64_t edge_cap, int64_t tasks) {
    const int64_t scan_n = std::max<int64_t>(std::max<int64_t>(agent_cap, tasks), 1);
    const int64_t blocks = scan_blocks_needed(scan_n) + 2;
    // buffers that must grow grow by half again, so a run of growing epochs reallocates rarely
    if (agent_cap > c->agent_cap) agent_cap = std::max<int64_t>(agent_cap, c->agent_cap + c->agent_cap / 2);
    if (edge_cap > c->edge_cap) edge_cap = std::max<int64_t>(edge_cap, c->edge_cap + c->edge_cap / 2);
    // a captured run carries the buffers' addresses: any reallocation retires it
    if (agent_cap > c->agent_cap || edge_cap > c->edge_cap || blocks > c->blocks_cap) destroy_graph_exec(c);
    if (agent_cap > c->agent_cap) {
        PG_CUDA(c, dalloc(c->kk, agent_cap));
        PG_CUDA(c, dalloc(c->big_list, agent_cap));
        PG_CUDA(c, dalloc(c->heavy_list, agent_cap));
        PG_CUDA(c, dalloc(c->heavy_mark, agent_cap));
        PG_CUDA(c, dalloc(c->eoff, agent_cap + 1));
        if (c->cfg.record_trace) PG_CUDA(c, dalloc(c->anchors, 4 * agent_cap));
        if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) PG_CUDA(c, dalloc(c->rc_agent, 6 * agent_cap));
        c->agent_cap = agent_cap;
    }
    if (edge_cap > c->edge_cap) {
        PG_CUDA(c, dalloc(c->e_dst, edge_cap));
        PG_CUDA(c, dalloc(c->e_rank, edge_cap));
        if (c->cfg.record_trace) PG_CUDA(c, dalloc(c->arrivals, edge_cap));
        c->edge_cap = edge_cap;
    }
    if (blocks > c->blocks_cap) {
        PG_CUDA(c, dalloc(c->blocksum, blocks));
        c->blocks_cap = blocks;
    }
    // copy tasks of the backward rows that move in one epoch: a moved row is a cited one (at most
    // one per edge); its old entries (at most the replica's m) and forward row copy (at most m + 3 n
    // over all rows) split into kRelocChunk chunks
    const int64_t reloc = c->edge_cap + (2 * c->M + 3 * c->S) / kRelocChunk + c->R + 1;
    if (reloc > c->reloc.n) {
        destroy_graph_exec(c);
        PG_CUDA(c, dalloc(c->reloc, reloc + reloc / 2));
    }
    return PG_OK;
}

// (Re)build the whole arena from host CSRs.  Used at load and when an R == 1 context grows.
struct HostGraph {
    std::vector<int32_t> pub, indeg;
    std::vector<float> fit;
    std::vector<int64_t> fo, bo;
    std::vector<int32_t> fc, bc;
    std::vector<int32_t> lag, dur;  // refcompat fitness windows (empty: lag 0, duration 1000)
};

// raw != nullptr: the replicas' CSRs are built on the device from raw[r].src / raw[r].dst (h.m is
// an upper bound on entry and the unique edge count on return); else hg holds host CSRs.
pg_status upload_arena(pg_ctx* c, std::vector<HostRep>& reps, const std::vector<HostGraph>& hg,
                       const pg_replica_desc* raw = nullptr) {
    const int R = (int)reps.size();
    int64_t S = 0, T = 0, M = 0, B = 0;
    for (int r = 0; r < R; ++r) {
        HostRep& h = reps[r];
        h.n_cap = round_up(std::max<int64_t>(h.n_cap, h.n + 1), kTile);
        h.nbase = S;
        h.obase = S + r;
        h.ebase = M;
        h.tbase = (int32_t)T;
        h.ntiles = (int32_t)(h.n_cap / kTile);
        S += h.n_cap;
        T += h.ntiles;
        // edge regions are multiples of 4 entries, so every 16-byte-aligned window around a row
        // (the agent kernel's bulk copies) starts and ends inside its replica's region
        h.m_cap = round_up(std::max<int64_t>(h.m_cap, h.m + 1), 4);
        M += h.m_cap;
        // backward region: growable rows (BRow), 16-byte aligned; bregion_entries bounds every
        // span the rows can take while the replica stays within n_cap nodes and m_cap edges
        h.bbase = B;
        h.b_cap = bregion_entries(h.n_cap, h.m_cap);
        B += h.b_cap;
        if (h.b_cap > kBRegionMax) return fail(c, PG_ERR_CAPACITY, "replica too large for the backward region");
    }
    // every replica's raw edges are uploaded (each at its offset in one staging buffer) and checked
    // on the device before the arena is touched, so a bad edge list leaves the loaded graph intact;
    // the builds below read the staged edges
    DBuf<int32_t> raw_src, raw_dst;
    std::vector<int64_t> raw_off((size_t)R + 1, 0);
    if (raw) {
        for (int r = 0; r < R; ++r) raw_off[(size_t)r + 1] = raw_off[(size_t)r] + std::max<int64_t>(raw[r].num_edges, 0);
        const int64_t tot = raw_off[(size_t)R];
        DBuf<unsigned long long> first;
        auto drop = [&]() {
            tfree(raw_src, c->device, c->stream);
            tfree(raw_dst, c->device, c->stream);
            tfree(first, c->device, c->stream);
        };
        cudaError_t e = talloc(raw_src, std::max<int64_t>(tot, 1), c->device, c->stream);
        if (e == cudaSuccess) e = talloc(raw_dst, std::max<int64_t>(tot, 1), c->device, c->stream);
        if (e == cudaSuccess) e = talloc(first, R, c->device, c->stream);
        // edge lists in page-locked host memory (mapped into the device's address space) are read by
        // the gather kernel directly; any other list is copied into the staging arrays first
        auto mapped = [](const void* p) -> const void* {
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
        };
        // the gather's table: list offsets (R + 1), node counts (R), source / target arrays (2 R)
        std::vector<int64_t> chk_h(raw_off);
        for (int r = 0; r < R; ++r) chk_h.push_back(raw[r].num_nodes);
        for (int r = 0; r < R && e == cudaSuccess; ++r) {
            const pg_replica_desc& d = raw[r];
            const size_t o = (size_t)raw_off[(size_t)r];
            const void* ms = d.num_edges > 0 ? mapped(d.src) : nullptr;
            const void* md = d.num_edges > 0 ? mapped(d.dst) : nullptr;
            if (d.num_edges > 0 && !(ms && md)) {
                e = cudaMemcpyAsync(raw_src.p + o, d.src, 4 * (size_t)d.num_edges, cudaMemcpyHostToDevice, c->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(raw_dst.p + o, d.dst, 4 * (size_t)d.num_edges, cudaMemcpyHostToDevice, c->stream);
                ms = raw_src.p + o;
                md = raw_dst.p + o;
            }
            chk_h.push_back((int64_t)(uintptr_t)ms);
            chk_h.push_back((int64_t)(uintptr_t)md);
        }
        DBuf<int64_t> chk;
        if (e == cudaSuccess) e = talloc(chk, (int64_t)chk_h.size(), c->device, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(chk.p, chk_h.data(), 8 * chk_h.size(), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            launch_gather_edges(tot, chk.p, chk.p + R + 1, chk.p + 2 * R + 1, R, raw_src.p, raw_dst.p, first.p,
                                c->stream);
        std::vector<unsigned long long> bad((size_t)R, ~0ull);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(bad.data(), first.p, sizeof(unsigned long long) * (size_t)R, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        tfree(first, c->device, c->stream);
        tfree(chk, c->device, c->stream);
        if (e != cudaSuccess) {
            drop();
            return fail(c, PG_ERR_CUDA, std::string("edge upload: ") + cudaGetErrorString(e));
        }
        for (int r = 0; r < R; ++r)
            if (bad[(size_t)r] != ~0ull) {
                drop();
                return fail(c, PG_ERR_ARG, "edge endpoint out of range at index " + std::to_string(bad[(size_t)r]) +
                                               (R > 1 ? " of replica " + std::to_string(r) : std::string()));
            }
    }
    c->S = S;
    c->T = T;
    c->M = M;
    c->B = B;
    destroy_graph_exec(c);
    c->ckpt.valid = false;
    PG_CUDA(c, dalloc(c->rep, R));
    PG_CUDA(c, dalloc(c->tile_rep, T));
    PG_CUDA(c, dalloc(c->tilesum, std::max<int64_t>(T, R) + 1));
    PG_CUDA(c, dalloc(c->tileoff, T + 1));
    PG_CUDA(c, dalloc(c->pub, S));
    PG_CUDA(c, dalloc(c->fit, S));
    PG_CUDA(c, dalloc(c->indeg, S));
    PG_CUDA(c, dalloc(c->inc, S));
    PG_CUDA(c, dalloc(c->w, S));
    PG_CUDA(c, dalloc(c->cdf, S));
    PG_CUDA(c, dalloc(c->guide, S));
    PG_CUDA(c, dalloc(c->new_start, S));
    PG_CUDA(c, dalloc(c->sort_small, S));
    PG_CUDA(c, dalloc(c->sort_large, S));
    PG_CUDA(c, dalloc(c->sort_large_off, S));
    PG_CUDA(c, dalloc(c->fwd_off, S + R));
    PG_CUDA(c, dalloc(c->fwd_col, M));
    PG_CUDA(c, dalloc(c->brow, S));
    PG_CUDA(c, dalloc(c->bcap, S));
    PG_CUDA(c, dalloc(c->bcol, B));
    PG_CUDA(c, dalloc(c->tables, (int64_t)R * kTableEntries));
    PG_CUDA(c, dalloc(c->hslot, S));
    PG_CUDA(c, dalloc(c->hmask, S * kMaskWords));
    PG_CUDA(c, dalloc(c->hub2, (int64_t)R * kHeavyMax * kMaskWords));
    PG_CUDA(c, dalloc(c->hub_need, (int64_t)R * (kHeavyMax / 32)));
    PG_CUDA(c, dalloc(c->hlist, (int64_t)R * kHeavyMax));
    PG_CUDA(c, dalloc(c->hub_rem, (int64_t)R * kHeavyMax));
    PG_CUDA(c, dalloc(c->hub_add, (int64_t)R * kHeavyMax));
    PG_CUDA(c, dalloc(c->hub_cand, (int64_t)R * kHeavyMax));
    if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) {
        PG_CUDA(c, dalloc(c->rc_pa, S));
        if (!c->rc_big_id.p) {
            PG_CUDA(c, dalloc(c->rc_big_id, (int64_t)kRcBigCap * kKMax));
            PG_CUDA(c, dalloc(c->rc_big_meta, (int64_t)kRcBigCap * 3));
        }
        PG_CUDA(c, dalloc(c->rc_rec, S));
        PG_CUDA(c, dalloc(c->rc_fit, S));
        PG_CUDA(c, dalloc(c->rc_lag, S));
        PG_CUDA(c, dalloc(c->rc_dur, S));
        PG_CUDA(c, dalloc(c->rc_acc, 4 * (int64_t)R));
        PG_CUDA(c, dalloc(c->rc_cnt, (int64_t)R * kRcAgeMax));
        PG_CUDA(c, dalloc(c->rc_rtab, (int64_t)R * kRcAgeMax));
        if (!c->rc_ftab.p) {
            std::vector<uint64_t> ft(kRcFitMax);
            rc_fitness_table_host(ft.data());
            PG_CUDA(c, dalloc(c->rc_ftab, kRcFitMax));
            PG_CUDA(c, cudaMemcpyAsync(c->rc_ftab.p, ft.data(), 8 * ft.size(), cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaStreamSynchronize(c->stream));
        }
        std::vector<double> rt((size_t)R * kRcAgeMax, 0.0);
        for (int r = 0; r < R; ++r)
            std::copy(reps[r].rtab.begin(), reps[r].rtab.end(), rt.begin() + (size_t)r * kRcAgeMax);
        PG_CUDA(c, cudaMemcpyAsync(c->rc_rtab.p, rt.data(), 8 * rt.size(), cudaMemcpyHostToDevice, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    PG_CUDA(c, cudaMemsetAsync(c->hslot.p, 0xFF, 2 * (size_t)S, c->stream));
    PG_CUDA(c, cudaMemsetAsync(c->inc.p, 0, sizeof(int32_t) * (size_t)S, c->stream));
    PG_CUDA(c, cudaMemsetAsync(c->w.p, 0, sizeof(float) * (size_t)S, c->stream));
    // empty rows everywhere: slots of nodes not yet born hold {0, 0, 0} until their first citation
    PG_CUDA(c, cudaMemsetAsync(c->brow.p, 0, sizeof(BRow) * (size_t)S, c->stream));
    PG_CUDA(c, cudaMemsetAsync(c->bcap.p, 0, sizeof(int32_t) * (size_t)S, c->stream));
    std::vector<int32_t> trep((size_t)T);
    std::vector<Replica> drep((size_t)R);
    std::vector<uint64_t> tabs((size_t)R * kTableEntries);
    // scratch of the device CSR build: raw edges of one replica and the sort buffers; the
    // offset-form backward CSR each replica is built or uploaded in before its rows are laid out
    // (every replica is enqueued without a host synchronisation: unique-edge counts, row-layout
    // sizes and error words per replica stay on the device and are read back once at the end)
    DBuf<char> scratch;
    DBuf<uint32_t> berr;
    DBuf<int64_t> t_bo, t_caps, t_begs, t_bsum, t_u, t_laid;
    DBuf<int32_t> t_bc;
    DBuf<int64_t> t_ro;
    DBuf<int32_t> t_fsrc, t_btgt;  // one replica's raw build: every entry's row, for the row layout
    struct Temps {
        std::vector<std::function<void()>> f;
        ~Temps() {
            for (auto& g : f) g();
        }
    } temps;
    temps.f.push_back([&]() {
        tfree(t_bo, c->device, c->stream);
        tfree(t_caps, c->device, c->stream);
        tfree(t_begs, c->device, c->stream);
        tfree(t_bsum, c->device, c->stream);
        tfree(t_bc, c->device, c->stream);
        tfree(t_u, c->device, c->stream);
        tfree(t_laid, c->device, c->stream);
        tfree(scratch, c->device, c->stream);
        tfree(raw_src, c->device, c->stream);
        tfree(raw_dst, c->device, c->stream);
        tfree(berr, c->device, c->stream);
    });
    {
        int64_t nn = 1, mm = 1;
        for (int r = 0; r < R; ++r) {
            nn = std::max<int64_t>(nn, reps[r].n);
            mm = std::max<int64_t>(mm, raw ? raw[r].num_edges : reps[r].m);
        }
        PG_CUDA(c, talloc(t_bo, nn + 1, c->device, c->stream));
        PG_CUDA(c, talloc(t_caps, nn + 1, c->device, c->stream));
        PG_CUDA(c, talloc(t_begs, nn + 1, c->device, c->stream));
        PG_CUDA(c, talloc(t_bsum, scan_blocks_needed(nn + 1) + 2, c->device, c->stream));
        PG_CUDA(c, talloc(t_bc, mm, c->device, c->stream));
        PG_CUDA(c, talloc(t_u, R, c->device, c->stream));
        PG_CUDA(c, talloc(t_laid, R, c->device, c->stream));
        PG_CUDA(c, cudaMemsetAsync(t_laid.p, 0, 8 * (size_t)R, c->stream));
    }
    // several replicas' seeds are built as one graph over the arena's slots (launch_build_all); one
    // replica's by the build per replica below
    const bool batched = raw && R > 1;
    temps.f.push_back([&]() { tfree(t_ro, c->device, c->stream); });
    temps.f.push_back([&]() {
        tfree(t_fsrc, c->device, c->stream);
        tfree(t_btgt, c->device, c->stream);
    });
    if (raw) {
        int64_t mm = 1, nn = 1;
        for (int r = 0; r < R; ++r) {
            mm = std::max<int64_t>(mm, raw[r].num_edges);
            nn = std::max<int64_t>(nn, raw[r].num_nodes);
        }
        const size_t sb = batched ? build_all_scratch_bytes(raw_off[(size_t)R], S) : build_scratch_bytes(mm, nn);
        PG_CUDA(c, talloc(scratch, (int64_t)sb, c->device, c->stream));
        if (!batched) {
            PG_CUDA(c, talloc(t_fsrc, mm, c->device, c->stream));
            PG_CUDA(c, talloc(t_btgt, mm, c->device, c->stream));
        }
        PG_CUDA(c, talloc(berr, R, c->device, c->stream));
        PG_CUDA(c, cudaMemsetAsync(berr.p, 0, 4 * (size_t)R, c->stream));
    }
    if (batched) {
        // the tile map and the replicas' bases first: the build cuts its result by them
        for (int r = 0; r < R; ++r) {
            for (int t = 0; t < reps[r].ntiles; ++t) trep[(size_t)reps[r].tbase + t] = r;
            drep[(size_t)r] = to_device_rep(reps[r]);
        }
        PG_CUDA(c, talloc(t_ro, R + 1, c->device, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(t_ro.p, raw_off.data(), 8 * (size_t)(R + 1), cudaMemcpyHostToDevice, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(c->tile_rep.p, trep.data(), 4 * (size_t)T, cudaMemcpyHostToDevice, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(c->rep.p, drep.data(), sizeof(Replica) * (size_t)R, cudaMemcpyHostToDevice, c->stream));
        cudaGetLastError();
        launch_build_all(raw_src.p, raw_dst.p, raw_off[(size_t)R], t_ro.p, R, S, c->tile_rep.p, c->rep.p, scratch.p,
                         c->fwd_off.p, c->fwd_col.p, c->brow.p, c->bcap.p, c->bcol.p, c->indeg.p, t_u.p, t_laid.p,
                         berr.p, c->stream);
        PG_CUDA(c, cudaGetLastError());
    }
    for (int r = 0; r < R; ++r) {
        HostRep& h = reps[r];
        for (int t = 0; t < h.ntiles; ++t) trep[(size_t)h.tbase + t] = r;
        if (h.rc)
            std::copy(h.bag_table.begin(), h.bag_table.end(), tabs.begin() + (size_t)r * kTableEntries);
        else
            poisson_table(h.prm.mean_out_degree, tabs.data() + (size_t)r * kTableEntries, kTableEntries);
        const HostGraph& g = hg[(size_t)r];
        const size_t n = (size_t)h.n, m = (size_t)h.m;
        if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) {
            std::vector<int32_t> lag(n, 0), dur(n, 1000);
            const std::vector<int32_t>& L = g.lag.size() == n ? g.lag : lag;
            const std::vector<int32_t>& D = g.dur.size() == n ? g.dur : dur;
            PG_CUDA(c, cudaMemcpyAsync(c->rc_lag.p + h.nbase, L.data(), 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(c->rc_dur.p + h.nbase, D.data(), 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaStreamSynchronize(c->stream));
        }
        if (raw) {
            const pg_replica_desc& d = raw[r];
            PG_CUDA(c, cudaMemcpyAsync(c->pub.p + h.nbase, d.pub_epoch, 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(c->fit.p + h.nbase, d.fitness, 4 * n, cudaMemcpyHostToDevice, c->stream));
            if (batched) continue;
            cudaGetLastError();
            const size_t o = (size_t)raw_off[(size_t)r];
            launch_build_csr(raw_src.p + o, raw_dst.p + o, d.num_edges, (int64_t)n, scratch.p, c->fwd_off.p + h.obase,
                             c->fwd_col.p + h.ebase, t_bo.p, t_bc.p, c->indeg.p + h.nbase, t_u.p + r, berr.p + r,
                             c->stream, t_fsrc.p, t_btgt.p);
            PG_CUDA(c, cudaGetLastError());
        } else {
            PG_CUDA(c, cudaMemcpyAsync(c->pub.p + h.nbase, g.pub.data(), 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(c->fit.p + h.nbase, g.fit.data(), 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(c->indeg.p + h.nbase, g.indeg.data(), 4 * n, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(c->fwd_off.p + h.obase, g.fo.data(), 8 * (n + 1), cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(t_bo.p, g.bo.data(), 8 * (n + 1), cudaMemcpyHostToDevice, c->stream));
            if (m) {
                PG_CUDA(c, cudaMemcpyAsync(c->fwd_col.p + h.ebase, g.fc.data(), 4 * m, cudaMemcpyHostToDevice, c->stream));
                PG_CUDA(c, cudaMemcpyAsync(t_bc.p, g.bc.data(), 4 * m, cudaMemcpyHostToDevice, c->stream));
            }
        }
        // the backward rows with room to grow (h.m bounds the entries; the layout reads the count)
        if (n) {
            launch_brow_layout(t_bo.p, t_bc.p, c->fwd_off.p + h.obase, c->fwd_col.p + h.ebase, (int64_t)n, h.m,
                               t_caps.p, t_begs.p, t_bsum.p, c->brow.p + h.nbase, c->bcap.p + h.nbase,
                               c->bcol.p + h.bbase, c->stream, raw ? t_fsrc.p : nullptr, raw ? t_btgt.p : nullptr);
            PG_CUDA(c, cudaGetLastError());
            PG_CUDA(c, cudaMemcpyAsync(t_laid.p + r, t_begs.p + n, 8, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    {
        std::vector<int64_t> us((size_t)R, 0), laid((size_t)R, 0);
        std::vector<uint32_t> be((size_t)R, 0);
        if (raw) {
            PG_CUDA(c, cudaMemcpyAsync(us.data(), t_u.p, 8 * (size_t)R, cudaMemcpyDeviceToHost, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(be.data(), berr.p, 4 * (size_t)R, cudaMemcpyDeviceToHost, c->stream));
        }
        PG_CUDA(c, cudaMemcpyAsync(laid.data(), t_laid.p, 8 * (size_t)R, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (raw) {
            tfree(scratch, c->device, c->stream);
            tfree(raw_src, c->device, c->stream);
            tfree(raw_dst, c->device, c->stream);
            tfree(berr, c->device, c->stream);
        }
        for (int r = 0; r < R; ++r) {
            HostRep& h = reps[r];
            if (raw) {
                if (be[(size_t)r]) return fail(c, PG_ERR_ARG, "edge endpoint out of range in replica " + std::to_string(r));
                // at most the raw edge count; anything else means the sequence above failed
                if (us[(size_t)r] < 0 || us[(size_t)r] > raw[r].num_edges)
                    return fail(c, PG_ERR_CUDA, "seed CSR build failed in replica " + std::to_string(r));
                h.m = us[(size_t)r];
            }
            if (laid[(size_t)r] < 0 || laid[(size_t)r] > h.b_cap)
                return fail(c, PG_ERR_CUDA, "backward row layout out of range");
            h.b_top = laid[(size_t)r];
            drep[(size_t)r] = to_device_rep(h);
        }
    }
    PG_CUDA(c, cudaMemcpyAsync(c->tile_rep.p, trep.data(), 4 * (size_t)T, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(c->rep.p, drep.data(), sizeof(Replica) * (size_t)R, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(c->tables.p, tabs.data(), 8 * tabs.size(), cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemsetAsync(c->st.p, 0, sizeof(EpochState), c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->hrep = reps;
    c->R = R;
    c->loaded = true;
    c->poisoned = false;
    c->rep_last_first.assign((size_t)R, 0);
    c->rep_last_count.assign((size_t)R, 0);
    return PG_OK;
}

// Replica r's backward CSR in offset form on the host (off: n + 1 entries, col: m): the rows and
// the used part of the region read back, then compacted in node order.  Either output may be null.
pg_status backward_offset_form(pg_ctx* c, int r, int64_t* off, int32_t* col) {
    const HostRep& h = c->hrep[(size_t)r];
    const size_t n = (size_t)h.n;
    Replica dr{};
    PG_CUDA(c, cudaMemcpyAsync(&dr, c->rep.p + r, sizeof(Replica), cudaMemcpyDeviceToHost, c->stream));
    std::vector<BRow> rows(n);
    if (n) PG_CUDA(c, cudaMemcpyAsync(rows.data(), c->brow.p + h.nbase, sizeof(BRow) * n, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    const int64_t top = (int64_t)dr.b_top;
    if (top < 0 || top > h.b_cap) return fail(c, PG_ERR_STATE, "backward region state out of range");
    std::vector<int32_t> reg;
    if (col && top) {
        reg.resize((size_t)top);
        PG_CUDA(c, cudaMemcpyAsync(reg.data(), c->bcol.p + h.bbase, 4 * (size_t)top, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    int64_t o = 0;
    for (size_t v = 0; v < n; ++v) {
        const BRow& w = rows[v];
        const int64_t beg = (int64_t)w.beg4 << 2;
        if (w.len < 0 || beg + w.len > top || o + w.len > h.m) return fail(c, PG_ERR_STATE, "backward row out of range");
        if (off) off[v] = o;
        if (col && w.len) std::memcpy(col + o, reg.data() + beg, 4 * (size_t)w.len);
        o += w.len;
    }
    if (off) off[n] = o;
    return PG_OK;
}

// Host copy of replica r's current graph (used when an R == 1 context grows).
pg_status download_graph(pg_ctx* c, int r, HostGraph& g) {
    const HostRep& h = c->hrep[(size_t)r];
    const size_t n = (size_t)h.n, m = (size_t)h.m;
    g.pub.resize(n);
    g.fit.resize(n);
    g.indeg.resize(n);
    g.fo.resize(n + 1);
    g.bo.resize(n + 1);
    g.fc.resize(std::max<size_t>(m, 1));
    g.bc.resize(std::max<size_t>(m, 1));
    PG_CUDA(c, cudaMemcpyAsync(g.pub.data(), c->pub.p + h.nbase, 4 * n, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(g.fit.data(), c->fit.p + h.nbase, 4 * n, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(g.indeg.data(), c->indeg.p + h.nbase, 4 * n, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(g.fo.data(), c->fwd_off.p + h.obase, 8 * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (m) PG_CUDA(c, cudaMemcpyAsync(g.fc.data(), c->fwd_col.p + h.ebase, 4 * m, cudaMemcpyDeviceToHost, c->stream));
    if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) {
        g.lag.resize(n);
        g.dur.resize(n);
        PG_CUDA(c, cudaMemcpyAsync(g.lag.data(), c->rc_lag.p + h.nbase, 4 * n, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(g.dur.data(), c->rc_dur.p + h.nbase, 4 * n, cudaMemcpyDeviceToHost, c->stream));
    }
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return backward_offset_form(c, r, g.bo.data(), g.bc.data());
}

// Make sure an R == 1 context can hold `need_n` nodes and `need_m` edges.
pg_status ensure_capacity(pg_ctx* c, int64_t need_n, int64_t need_m) {
    HostRep& h = c->hrep[0];
    if (need_n <= h.n_cap && need_m <= h.m_cap) return PG_OK;
    if (c->R != 1) return fail(c, PG_ERR_CAPACITY, "replica capacity exceeded (plan more epochs)");
    HostGraph g;
    pg_status s = download_graph(c, 0, g);
    if (s != PG_OK) return s;
    std::vector<HostRep> reps = c->hrep;
    reps[0].n_cap = std::max<int64_t>(need_n, h.n_cap + h.n_cap / 2);
    reps[0].m_cap = std::max<int64_t>(need_m, h.m_cap + h.m_cap / 2);
    std::vector<HostGraph> hg(1);
    hg[0] = std::move(g);
    return upload_arena(c, reps, hg);
}

pg_status read_back(pg_ctx* c) {
    PG_CUDA(c, cudaMemcpyAsync(&c->h_st, c->st.p, sizeof(EpochState), cudaMemcpyDeviceToHost, c->stream));
    c->h_rep.resize((size_t)c->R);
    PG_CUDA(c, cudaMemcpyAsync(c->h_rep.data(), c->rep.p, sizeof(Replica) * (size_t)c->R,
                               cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status device_error(pg_ctx* c) {
    const uint32_t e = c->h_st.error;
    if (!e) return PG_OK;
    c->poisoned = true;
    std::string msg = "device reported:";
    if (e & kErrCapacity) msg += " capacity exceeded;";
    if (e & kErrBadWeight) msg += " non-finite or all-zero weights;";
    if (e & kErrArg) msg += " inconsistent agent draw;";
    if (e & kErrTimeout) msg += " bounded wait on an asynchronous copy ran out;";
    return fail(c, (e & kErrCapacity) ? PG_ERR_CAPACITY : ((e & kErrTimeout) ? PG_ERR_TIMEOUT : PG_ERR_ARG), msg);
}

float ms_between(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();  // an unavailable timing must not surface as a later launch error
        return 0.0f;
    }
    return ms;
}

// Record a timing event.  Inside a stream capture a plain record only expresses a dependency; the
// external flag turns it into an event-record node, so captured runs are timed as well.
void record_event(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else
        cudaEventRecord(e, s);
}

// Enqueue one PA epoch (no synchronisation).  agents = total new nodes of the epoch.  Returns the
// first launch error with the stage that raised it.
pg_status enqueue_pa_epoch(pg_ctx* c, int64_t epoch, int64_t agents, cudaEvent_t* ev) {
    const bool events = ev != nullptr;
    Arena A = make_arena(c);
    cudaStream_t s = c->stream;
    cudaError_t e;
#define PG_STAGE(name)                                                                          \
    if ((e = cudaPeekAtLastError()) != cudaSuccess) {                                           \
        cudaGetLastError();                                                                     \
        return fail(c, PG_ERR_CUDA, std::string("launch error in ") + name + ": " + cudaGetErrorString(e)); \
    }
    if (events) record_event(ev[0], s);
    if (c->cfg.weight_model == PG_WEIGHTS_BASELINE && c->cfg.sampler == PG_SAMPLER_THINNING && c->tune.epoch_kernel &&
        epoch_kernel_ctas() > 0) {
        // the whole epoch as one persistent cooperative kernel (its stages are phases; the stage
        // events all fall on its two ends, so the epoch counts as agent time)
        PG_CUDA(c, cudaMemsetAsync(&c->st.p->gbar_count, 0, sizeof(unsigned int), s));
        if (events) {
            record_event(ev[1], s);
            record_event(ev[2], s);
        }
        e = launch_epoch_kernel(A, epoch, agents, s);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(c, PG_ERR_CUDA, std::string("launch error in the epoch kernel: ") + cudaGetErrorString(e));
        }
        if (events) {
            record_event(ev[3], s);
            record_event(ev[4], s);
        }
        c->launches += 1;
        return PG_OK;
    }
    launch_epoch_begin(A, epoch, 1, s);
    PG_STAGE("epoch begin");
    if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) {
        // ParAGraph's own model: score components, out-degrees, the per-paper rule, CSR append
        launch_rc_scores(A, s);
        PG_STAGE("refcompat scores");
        if (events) record_event(ev[1], s);
        launch_agent_setup(A, agents, s);
        PG_STAGE("agent setup");
        if (events) record_event(ev[2], s);
        launch_rc_big(A, c->num_sms, s);
        launch_rc_agents(A, agents, c->num_sms, s);
        PG_STAGE("refcompat agents");
        if (events) record_event(ev[3], s);
        launch_bwd_append(A, agents, c->num_sms, s, c->side, c->fork, c->join);
        PG_STAGE("backward append");
        if (events) record_event(ev[4], s);
        c->launches += kPaEpochKernels - 4 - 2 + kRcScoreKernels + 2 + (c->out_src ? 1 : 0);
        return PG_OK;
    }
    // the hub index reads only the CSR and the weights and guide table only node attributes: the
    // hub kernels run on a side stream forked here and joined before the agent setup (the same
    // dependencies inside a captured graph)
    const bool thin = c->cfg.sampler == PG_SAMPLER_THINNING;
    if (thin) {
        PG_CUDA(c, cudaEventRecord(c->fork, s));
        PG_CUDA(c, cudaStreamWaitEvent(c->side, c->fork, 0));
        launch_hubs(A, c->num_sms, c->side);
        PG_STAGE("hub index");
        PG_CUDA(c, cudaEventRecord(c->join, c->side));
    }
    launch_weights(A, s);
    PG_STAGE("weights");
    if (thin) {
        launch_guide(A, s);
        PG_STAGE("guide table");
        PG_CUDA(c, cudaStreamWaitEvent(s, c->join, 0));
        c->launches += kThinKernels;
    }
    if (events) record_event(ev[1], s);
    launch_agent_setup(A, agents, s);
    PG_STAGE("agent setup");
    if (c->cfg.sampler == PG_SAMPLER_THINNING) {
        launch_hub_pairs(A, s);  // for the hubs the setup found among the anchors
        PG_STAGE("hub pairs");
    }
    if (events) record_event(ev[2], s);
    launch_agents(A, agents, c->num_sms, s);
    PG_STAGE("agents");
    if (events) record_event(ev[3], s);
    launch_bwd_append(A, agents, c->num_sms, s, c->side, c->fork, c->join);
    PG_STAGE("backward append");
    if (events) record_event(ev[4], s);
#undef PG_STAGE
    c->launches += kPaEpochKernels + (c->out_src ? 1 : 0);
    return PG_OK;
}

// Planned agents of the next epoch and the node/edge needs of every replica.
int64_t plan_epoch(pg_ctx* c, std::vector<int64_t>* deltas) {
    int64_t tot = 0;
    if (deltas) deltas->assign((size_t)c->R, 0);
    for (int r = 0; r < c->R; ++r) {
        const int64_t d = delta_of(c->hrep[(size_t)r].prm, c->hrep[(size_t)r].n);
        if (deltas) (*deltas)[(size_t)r] = d;
        tot += d;
    }
    return tot;
}

// Algorithmic bytes of the PA epoch (the minimum traffic of the algorithm, not what a given
// implementation moves):
//   agents, thinning sampler: per frontier entry gathered 36 B (its int32 id and its 256-bit hub
//            mask), per membership test 16 B (the candidate's row offsets), per adjacency entry the
//            test examined 4 B, per event 32 B (one CDF sector), per edge 16 B (forward column,
//            in-degree counter, rank, destination)
//   agents, enumeration sampler: per adjacency row read 32 B (fwd and bwd begin/end, int64), per
//            streamed neighbour 8 B (its int32 id and its fp32 weight), per draw 32 B, per edge 16 B
//   weights: per node 44 B (fitness, in-degree, publication epoch, weight write, weight read, CDF
//            write, CDF read+write in the tile-offset pass)
//   csr    : 8 B per moved backward entry, 12 B per new edge (place + sort), 24 B per node
//            (old and new backward offsets, length)
int64_t agent_bytes(bool thin, int64_t rows, int64_t elems, int64_t draws, int64_t edges,
                    int64_t scanned) {
    if (thin) return 36 * rows + 16 * elems + 4 * scanned + 32 * draws + 16 * edges;
    return 32 * rows + 8 * elems + 32 * draws + 16 * edges;
}
int64_t weight_bytes(int64_t nodes) { return 44 * nodes; }
// backward append: 8 B per entry of a row that moved (read and written), 32 B per new edge (its
// target and rank read by the grow and place passes, its row's start of new entries read, the entry
// written, its cited row's length, room and in-degree updated at most once per edge), 40 B per new
// node (its hub mask and slot, its row)
int64_t csr_bytes(int64_t moved, int64_t edges, int64_t new_nodes) { return 8 * moved + 32 * edges + 40 * new_nodes; }

void fill_stats(pg_ctx* c, int64_t new_nodes, bool er) {
    pg_stats& S = c->stats;
    const EpochState& st = c->h_st;
    S.epoch = st.epoch;
    S.new_nodes = new_nodes;
    S.new_edges = st.edges;
    S.nodes_weighted = (int64_t)st.nodes_weighted;
    S.rows_expanded = (int64_t)st.rows_expanded;
    S.elems_streamed = (int64_t)st.elems_streamed;
    S.draws = (int64_t)st.draws;
    S.bwd_moved = (int64_t)st.bwd_moved;
    S.adj_scanned = (int64_t)st.adj_scanned;
    const int64_t E = st.edges;
    const int64_t ab = agent_bytes(c->cfg.sampler == PG_SAMPLER_THINNING, S.rows_expanded,
                                   S.elems_streamed, S.draws, E, S.adj_scanned);
    S.bytes_alg_agents = er ? 0 : ab;
    // ER: per edge 8 B edge-list write + 12 B CSR append; per new node 32 B (count + offsets)
    S.bytes_alg = er ? (8 * E + 12 * E + 32 * new_nodes + 8 * S.bwd_moved)
                     : ab + weight_bytes(S.nodes_weighted) +
                           csr_bytes(S.bwd_moved, E, new_nodes);
}

pg_status finish_epoch(pg_ctx* c, const std::vector<int64_t>& deltas, bool er) {
    pg_status s = read_back(c);
    if (s != PG_OK) return s;
    s = device_error(c);
    if (s != PG_OK) return s;
    int64_t nn = 0;
    for (int r = 0; r < c->R; ++r) {
        HostRep& h = c->hrep[(size_t)r];
        c->rep_last_first[(size_t)r] = h.m;
        h.n = c->h_rep[(size_t)r].n;
        h.m = c->h_rep[(size_t)r].m;
        c->rep_last_count[(size_t)r] = h.m - c->rep_last_first[(size_t)r];
        nn += deltas[(size_t)r];
    }
    c->epoch += 1;
    fill_stats(c, nn, er);
    return PG_OK;
}

pg_status check_rc_ready(pg_ctx* c) {
    if (c->cfg.weight_model != PG_WEIGHTS_REFCOMPAT) return PG_OK;
    for (int r = 0; r < c->R; ++r) {
        if (!c->hrep[(size_t)r].rc)
            return fail(c, PG_ERR_STATE, "refcompat context: call pg_rc_configure for every replica first");
        if (c->hrep[(size_t)r].n < 2) return fail(c, PG_ERR_STATE, "refcompat growth needs at least 2 nodes");
    }
    return PG_OK;
}

pg_status prepare_pa(pg_ctx* c, std::vector<int64_t>& deltas, int64_t& agents) {
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (check_rc_ready(c) != PG_OK) return PG_ERR_STATE;
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    agents = plan_epoch(c, &deltas);
    if (agents <= 0) return fail(c, PG_ERR_ARG, "epoch adds no nodes");
    int64_t ebound = 0;
    for (int r = 0; r < c->R; ++r) {
        const HostRep& h = c->hrep[(size_t)r];
        const int64_t eb = edge_bound(deltas[(size_t)r], h.prm.mean_out_degree, h.n, h.rc ? h.kmax : 0);
        ebound += eb;
        if (c->R == 1) {
            pg_status s = ensure_capacity(c, h.n + deltas[(size_t)r], h.m + eb);
            if (s != PG_OK) return s;
        }
    }
    return alloc_epoch_buffers(c, agents, ebound, 0);
}

}  // namespace

// ===================================================================== C ABI
extern "C" {

const char* pg_version(void) { return "paragraph_gb300 0.1 (sm_103a)"; }

const char* pg_status_string(pg_status s) {
    switch (s) {
        case PG_OK: return "ok";
        case PG_ERR_CUDA: return "CUDA error";
        case PG_ERR_CAPACITY: return "capacity exceeded";
        case PG_ERR_ARG: return "invalid argument";
        case PG_ERR_TIMEOUT: return "device wait timed out";
        case PG_ERR_IO: return "I/O error";
        case PG_ERR_STATE: return "invalid state";
    }
    return "unknown status";
}

const char* pg_last_error(const pg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

pg_status pg_default_params(pg_pa_params* out) {
    if (!out) return PG_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    out->alpha = 1.0;
    out->tau = 5.0;
    out->gamma = 1.0;
    out->beta = 4.0;
    out->mean_out_degree = 15.0;
    out->growth_rate = 0.0;
    out->fixed_new_nodes = 5000;
    out->num_anchors = 3;
    return PG_OK;
}

pg_status pg_create(pg_ctx** out, const pg_config* cfg) {
    if (!out || !cfg) return PG_ERR_ARG;
    *out = nullptr;
    if (cfg->num_replicas < 1 || cfg->replica_base < 0) return PG_ERR_ARG;
    if (cfg->weight_model != PG_WEIGHTS_BASELINE && cfg->weight_model != PG_WEIGHTS_REFCOMPAT) return PG_ERR_ARG;
    pg_ctx* c = new (std::nothrow) pg_ctx();
    if (!c) return PG_ERR_CAPACITY;
    c->cfg = *cfg;
    c->R = cfg->num_replicas;
    c->device = cfg->device;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(c->st, 1);
    if (e == cudaSuccess) e = init_agent_kernels();
    if (e == cudaSuccess) e = init_csr_kernels();
    if (e == cudaSuccess && cfg->weight_model == PG_WEIGHTS_BASELINE && cfg->sampler == PG_SAMPLER_THINNING)
        e = init_epoch_kernel(c->num_sms);
    if (e == cudaSuccess && cfg->weight_model == PG_WEIGHTS_REFCOMPAT) e = init_rc_kernels();
    // one global hash per resident agent warp, for anchors whose rows overflow the shared one
    if (e == cudaSuccess && cfg->weight_model == PG_WEIGHTS_BASELINE && cfg->sampler == PG_SAMPLER_THINNING)
        e = dalloc(c->zbig, agent_warp_slots(c->num_sms) << kGBits);
    for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->tev[i]);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->lev[i]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        c->err = std::string("CUDA initialisation failed: ") + cudaGetErrorString(e);
        *out = c;
        return PG_ERR_CUDA;
    }
    *out = c;
    return PG_OK;
}

void pg_destroy(pg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    destroy_graph_exec(c);
    DBuf<int32_t>* i32[] = {&c->tile_rep, &c->pub, &c->indeg, &c->inc, &c->kk, &c->big_list, &c->heavy_list, &c->heavy_mark,
                            &c->e_dst, &c->e_rank, &c->arrivals, &c->anchors, &c->fwd_col, &c->bcol, &c->bcap};
    for (auto* b : i32) dfree(*b);
    dfree(c->brow);
    dfree(c->reloc);
    dfree(c->er_slots);
    dfree(c->out_counts);
    dfree(c->out_stage_src);
    dfree(c->out_stage_dst);
    dfree(c->er_ov);
    dfree(c->er_ovb);
    DBuf<int64_t>* i64[] = {&c->fwd_off, &c->new_start,
                            &c->sort_small, &c->sort_large, &c->sort_large_off, &c->eoff,
                            &c->blocksum, &c->er_cnt, &c->er_toff};
    for (auto* b : i64) dfree(*b);
    free_checkpoint(c->ckpt);
    free_lik(c->lik);
    dfree(c->fit);
    dfree(c->w);
    dfree(c->cdf);
    dfree(c->guide);
    dfree(c->rc_pa);
    dfree(c->rc_rec);
    dfree(c->rc_fit);
    dfree(c->rc_rtab);
    dfree(c->rc_agent);
    dfree(c->rc_big_id);
    dfree(c->rc_big_meta);
    dfree(c->rc_lag);
    dfree(c->rc_dur);
    dfree(c->rc_cnt);
    dfree(c->rc_ftab);
    dfree(c->rc_acc);
    dfree(c->tilesum);
    dfree(c->tileoff);
    dfree(c->tables);
    dfree(c->hlist);
    dfree(c->hub_rem);
    dfree(c->hub_add);
    dfree(c->hub_cand);
    dfree(c->hslot);
    dfree(c->hmask);
    dfree(c->hub2);
    dfree(c->hub_need);
    dfree(c->zbig);
    dfree(c->src_tmp);
    dfree(c->rep);
    dfree(c->st);
    for (int i = 0; i < 6; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < 2; ++i) {
        if (c->tev[i]) cudaEventDestroy(c->tev[i]);
        if (c->lev[i]) cudaEventDestroy(c->lev[i]);
    }
    for (cudaEvent_t e : c->run_ev) cudaEventDestroy(e);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

pg_status pg_load_replicas(pg_ctx* c, const pg_replica_desc* descs, int32_t num) {
    if (!c) return PG_ERR_ARG;
    if (!descs || num != c->cfg.num_replicas) return fail(c, PG_ERR_ARG, "need one descriptor per replica");
    PG_CUDA(c, cudaSetDevice(c->device));
    std::vector<HostRep> reps((size_t)num);
    std::vector<HostGraph> hg((size_t)num);
    int64_t max_agents = 0, max_edges = 0;
    const int max_plan = 1 << 20;
    std::vector<int64_t> plan_agents, plan_edges;
    for (int r = 0; r < num; ++r) {
        const pg_replica_desc& d = descs[r];
        pg_status s = check_params(c, d.params);
        if (s != PG_OK) return s;
        if (d.num_nodes <= 0 || d.num_nodes > (int64_t)INT32_MAX / 2) return fail(c, PG_ERR_ARG, "num_nodes out of range");
        if (d.num_edges < 0 || (d.num_edges > 0 && (!d.src || !d.dst))) return fail(c, PG_ERR_ARG, "bad edge arrays");
        if (!d.pub_epoch || !d.fitness) return fail(c, PG_ERR_ARG, "pub_epoch and fitness are required");
        // the endpoints are checked on the device after the upload the build needs anyway, before
        // the arena is touched (upload_arena)
    }
    // the CSRs are built on the device from the raw edges (upload_arena); the plan below uses the
    // raw edge count, an upper bound on the unique edges
    for (int r = 0; r < num; ++r) {
        const pg_replica_desc& d = descs[r];
        HostRep& h = reps[(size_t)r];
        h.prm = d.params;
        h.n = d.num_nodes;
        h.m = d.num_edges;
        // capacity plan
        int64_t n = h.n, m = h.m;
        const int epochs = std::max(1, std::min(d.planned_epochs, max_plan));
        if ((int)plan_agents.size() < epochs) {
            plan_agents.resize((size_t)epochs, 0);
            plan_edges.resize((size_t)epochs, 0);
        }
        for (int e = 0; e < epochs; ++e) {
            const int64_t dl = delta_of(h.prm, n);
            const int64_t eb = edge_bound(dl, h.prm.mean_out_degree, n, h.rc ? h.kmax : 0);
            plan_agents[(size_t)e] += dl;
            plan_edges[(size_t)e] += eb;
            n += dl;
            m += eb;
        }
        h.n_cap = std::max<int64_t>(d.node_capacity, n);
        h.m_cap = std::max<int64_t>(d.edge_capacity, m);
    }
    for (size_t e = 0; e < plan_agents.size(); ++e) {
        max_agents = std::max(max_agents, plan_agents[e]);
        max_edges = std::max(max_edges, plan_edges[e]);
    }
    pg_status s = upload_arena(c, reps, hg, descs);
    if (s != PG_OK) return s;
    c->epoch = 0;
    return alloc_epoch_buffers(c, max_agents, max_edges, 0);
}

pg_status pg_load_graph(pg_ctx* c, int64_t n, const int32_t* pub_epoch, const float* fitness,
                        int64_t m, const int32_t* src, const int32_t* dst) {
    if (!c) return PG_ERR_ARG;
    if (c->cfg.num_replicas != 1) return fail(c, PG_ERR_ARG, "pg_load_graph needs num_replicas == 1");
    pg_replica_desc d{};
    d.num_nodes = n;
    d.pub_epoch = pub_epoch;
    d.fitness = fitness;
    d.num_edges = m;
    d.src = src;
    d.dst = dst;
    d.planned_epochs = 1;
    pg_default_params(&d.params);
    if (c->loaded) d.params = c->hrep[0].prm;
    return pg_load_replicas(c, &d, 1);
}

pg_status pg_set_params(pg_ctx* c, int32_t replica, const pg_pa_params* p) {
    if (!c || !p) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "load a graph first");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    pg_status s = check_params(c, *p);
    if (s != PG_OK) return s;
    HostRep& h = c->hrep[(size_t)replica];
    h.prm = *p;
    if (h.rc) h.prm.growth_rate = h.rcp.growth_rate;  // the refcompat growth rate stays in force
    destroy_graph_exec(c);
    std::vector<uint64_t> tab(kTableEntries);
    if (h.rc)
        tab = h.bag_table;
    else
        poisson_table(p->mean_out_degree, tab.data(), kTableEntries);
    PG_CUDA(c, cudaMemcpyAsync(c->tables.p + (size_t)replica * kTableEntries, tab.data(), 8 * tab.size(),
                               cudaMemcpyHostToDevice, c->stream));
    // refresh the parameter fields of the device replica
    Replica dr;
    PG_CUDA(c, cudaMemcpyAsync(&dr, c->rep.p + replica, sizeof(Replica), cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    const Replica fresh = to_device_rep(h);
    dr.alpha = fresh.alpha;
    dr.gamma = fresh.gamma;
    dr.tau = fresh.tau;
    dr.beta_m1 = fresh.beta_m1;
    dr.p_global = fresh.p_global;
    dr.glob_thr = fresh.glob_thr;
    dr.growth_rate = fresh.growth_rate;
    dr.fixed_new = fresh.fixed_new;
    dr.anchors = fresh.anchors;
    PG_CUDA(c, cudaMemcpyAsync(c->rep.p + replica, &dr, sizeof(Replica), cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_set_epoch(pg_ctx* c, int64_t epoch) {
    if (!c) return PG_ERR_ARG;
    c->epoch = epoch;
    destroy_graph_exec(c);
    return PG_OK;
}

pg_status pg_grow_epoch(pg_ctx* c, int64_t* new_nodes, int64_t* new_edges) {
    if (!c) return PG_ERR_ARG;
    PG_CUDA(c, cudaSetDevice(c->device));
    std::vector<int64_t> deltas;
    int64_t agents = 0;
    pg_status s = prepare_pa(c, deltas, agents);
    if (s != PG_OK) return s;
    cudaGetLastError();  // errors of earlier, unrelated calls are not this epoch's
    s = enqueue_pa_epoch(c, c->epoch, agents, c->timing ? c->ev : nullptr);
    if (s != PG_OK) {
        cudaStreamSynchronize(c->stream);
        c->poisoned = true;
        return s;
    }
    s = finish_epoch(c, deltas, false);
    if (s != PG_OK) return s;
    if (c->timing) {
        c->stats.ms_weights = ms_between(c->ev[0], c->ev[1]);
        c->stats.ms_setup = ms_between(c->ev[1], c->ev[2]);
        c->stats.ms_agents = ms_between(c->ev[2], c->ev[3]);
        c->stats.ms_csr = ms_between(c->ev[3], c->ev[4]);
        c->stats.ms_total = ms_between(c->ev[0], c->ev[4]);
        c->stats.ms_er = 0.0;
    }
    if (new_nodes) *new_nodes = c->stats.new_nodes;
    if (new_edges) *new_edges = c->stats.new_edges;
    return PG_OK;
}

namespace {

// Plans num_epochs PA epochs on the host mirror (agents per epoch, largest agent and edge counts)
// and makes sure the arena and per-epoch buffers hold the whole run: a single-replica arena grows,
// a multi-replica one must already be large enough.
pg_status plan_run(pg_ctx* c, int num_epochs, std::vector<int64_t>& agents, int64_t& max_agents,
                   int64_t& max_edges) {
    std::vector<HostRep> planned = c->hrep;
    agents.assign((size_t)num_epochs, 0);
    max_agents = max_edges = 0;
    for (int e = 0; e < num_epochs; ++e) {
        int64_t tot = 0, eb = 0;
        for (int r = 0; r < c->R; ++r) {
            HostRep& h = planned[(size_t)r];
            const int64_t d = delta_of(h.prm, h.n);
            const int64_t b = edge_bound(d, h.prm.mean_out_degree, h.n, h.rc ? h.kmax : 0);
            tot += d;
            eb += b;
            h.n += d;
            h.m += b;
        }
        agents[(size_t)e] = tot;
        max_agents = std::max(max_agents, tot);
        max_edges = std::max(max_edges, eb);
    }
    if (c->R == 1) {
        const pg_status s = ensure_capacity(c, planned[0].n, planned[0].m);
        if (s != PG_OK) return s;
    } else {
        for (int r = 0; r < c->R; ++r)
            if (planned[(size_t)r].n > c->hrep[(size_t)r].n_cap || planned[(size_t)r].m > c->hrep[(size_t)r].m_cap)
                return fail(c, PG_ERR_CAPACITY, "run exceeds the planned capacity of replica " + std::to_string(r));
    }
    return alloc_epoch_buffers(c, max_agents, max_edges, 0);
}

}  // namespace

pg_status pg_run_epochs(pg_ctx* c, int32_t num_epochs, int32_t use_graph, int64_t* new_edges) {
    if (!c) return PG_ERR_ARG;
    if (num_epochs < 1) return fail(c, PG_ERR_ARG, "num_epochs must be >= 1");
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    if (check_rc_ready(c) != PG_OK) return PG_ERR_STATE;
    PG_CUDA(c, cudaSetDevice(c->device));
    std::vector<int64_t> agents;
    int64_t max_agents = 0, max_edges = 0;
    pg_status s = plan_run(c, num_epochs, agents, max_agents, max_edges);
    if (s != PG_OK) return s;
    const int64_t e0 = c->epoch;
    const bool events = c->timing;
    if (events && (int64_t)c->run_ev.size() < 5 * (int64_t)num_epochs) {
        const size_t have = c->run_ev.size();
        c->run_ev.resize((size_t)num_epochs * 5, nullptr);
        for (size_t i = have; i < c->run_ev.size(); ++i) PG_CUDA(c, cudaEventCreate(&c->run_ev[i]));
        destroy_graph_exec(c);
    }
    auto enqueue_all = [&]() -> pg_status {
        pg_status es = PG_OK;
        c->launches = 0;
        // clear the run totals (captured as a memset node, so every replay clears them too)
        const size_t cum0 = offsetof(EpochState, cum_rows_expanded);
        cudaMemsetAsync(reinterpret_cast<char*>(c->st.p) + cum0, 0, sizeof(EpochState) - cum0, c->stream);
        for (int e = 0; e < num_epochs && es == PG_OK; ++e)
            es = enqueue_pa_epoch(c, e0 + e, agents[(size_t)e], events ? &c->run_ev[(size_t)e * 5] : nullptr);
        return es;
    };
    cudaGetLastError();  // errors of earlier, unrelated calls are not this run's
    if (use_graph) {
        if (!(c->gexec && c->g_epoch0 == e0 && c->g_epochs == num_epochs && c->g_out == (const void*)c->out_src)) {
            destroy_graph_exec(c);
            cudaGraph_t graph;
            PG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            const pg_status es = enqueue_all();
            cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
            if (es != PG_OK) {
                if (ce == cudaSuccess) cudaGraphDestroy(graph);
                return es;
            }
            if (ce != cudaSuccess) return fail(c, PG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
            ce = cudaGraphInstantiate(&c->gexec, graph, 0);
            cudaGraphDestroy(graph);
            if (ce != cudaSuccess) return fail(c, PG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
            c->g_epoch0 = e0;
            c->g_epochs = num_epochs;
            c->g_out = c->out_src;
        }
        PG_CUDA(c, cudaGraphLaunch(c->gexec, c->stream));
    } else {
        const pg_status es = enqueue_all();
        if (es != PG_OK) {
            cudaStreamSynchronize(c->stream);
            c->poisoned = true;
            return es;
        }
    }
    PG_CUDA(c, cudaGetLastError());
    s = read_back(c);
    if (s != PG_OK) return s;
    s = device_error(c);
    if (s != PG_OK) return s;
    int64_t total = 0, nn = 0;
    for (int r = 0; r < c->R; ++r) {
        HostRep& h = c->hrep[(size_t)r];
        total += c->h_rep[(size_t)r].m - h.m;
        nn += c->h_rep[(size_t)r].n - h.n;
        h.n = c->h_rep[(size_t)r].n;
        h.m = c->h_rep[(size_t)r].m;
    }
    c->epoch = e0 + num_epochs;
    fill_stats(c, nn, false);
    pg_stats& S = c->stats;
    const EpochState& hs = c->h_st;
    S.run_epochs = (int64_t)hs.cum_epochs;
    S.run_new_nodes = (int64_t)hs.cum_new_nodes;
    S.run_new_edges = (int64_t)hs.cum_edges;
    S.run_rows_expanded = (int64_t)hs.cum_rows_expanded;
    S.run_elems_streamed = (int64_t)hs.cum_elems_streamed;
    S.run_draws = (int64_t)hs.cum_draws;
    S.run_bwd_moved = (int64_t)hs.cum_bwd_moved;
    S.run_nodes_weighted = (int64_t)hs.cum_nodes_weighted;
    S.run_adj_scanned = (int64_t)hs.cum_adj_scanned;
    S.run_bytes_alg_agents = agent_bytes(c->cfg.sampler == PG_SAMPLER_THINNING, S.run_rows_expanded,
                                         S.run_elems_streamed, S.run_draws, S.run_new_edges,
                                         S.run_adj_scanned);
    S.run_bytes_alg = S.run_bytes_alg_agents + weight_bytes(S.run_nodes_weighted) +
                      csr_bytes(S.run_bwd_moved, S.run_new_edges, S.run_new_nodes);
    S.run_kernel_launches = c->launches;
    S.run_ms_weights = S.run_ms_setup = S.run_ms_agents = S.run_ms_csr = 0.0;
    if (events) {
        for (int e = 0; e < num_epochs; ++e) {
            cudaEvent_t* ev = &c->run_ev[(size_t)e * 5];
            S.run_ms_weights += ms_between(ev[0], ev[1]);
            S.run_ms_setup += ms_between(ev[1], ev[2]);
            S.run_ms_agents += ms_between(ev[2], ev[3]);
            S.run_ms_csr += ms_between(ev[3], ev[4]);
        }
        cudaEvent_t* last = &c->run_ev[(size_t)(num_epochs - 1) * 5];
        S.ms_total = ms_between(c->run_ev[0], last[4]);
        S.ms_weights = ms_between(last[0], last[1]);
        S.ms_setup = ms_between(last[1], last[2]);
        S.ms_agents = ms_between(last[2], last[3]);
        S.ms_csr = ms_between(last[3], last[4]);
    }
    S.new_edges = total;
    if (new_edges) *new_edges = total;
    return PG_OK;
}

pg_status pg_run_epochs_out(pg_ctx* c, int32_t num_epochs, int32_t use_graph, int32_t* src, int32_t* dst,
                            int64_t capacity, int64_t* counts, int64_t* new_edges) {
    if (!c) return PG_ERR_ARG;
    if (!src || !dst || capacity < 0) return fail(c, PG_ERR_ARG, "output buffers required");
    if (num_epochs < 1) return fail(c, PG_ERR_ARG, "num_epochs must be >= 1");
    PG_CUDA(c, cudaSetDevice(c->device));
    // page-locked buffers mapped into the device's address space are written by the device during
    // the run; any other buffers get a device staging copy, read back after the run
    auto mapped = [&](void* p) -> void* {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
    };
    int32_t* ds = static_cast<int32_t*>(mapped(src));
    int32_t* dd = static_cast<int32_t*>(mapped(dst));
    const bool staged = !(ds && dd);
    const int64_t cap = std::max<int64_t>(capacity, 1);
    if (staged) {
        if (c->out_stage_src.n < cap) PG_CUDA(c, dalloc(c->out_stage_src, cap));
        if (c->out_stage_dst.n < cap) PG_CUDA(c, dalloc(c->out_stage_dst, cap));
        ds = c->out_stage_src.p;
        dd = c->out_stage_dst.p;
    }
    const int64_t nc = (int64_t)num_epochs * c->R;
    if (c->out_counts.n < nc) {
        destroy_graph_exec(c);
        PG_CUDA(c, dalloc(c->out_counts, nc));
    }
    PG_CUDA(c, cudaMemsetAsync(c->out_counts.p, 0, 8 * (size_t)nc, c->stream));  // epochs not written stay 0
    c->out_src = ds;
    c->out_dst = dd;
    c->out_cap = capacity;
    c->out_epochs = num_epochs;
    int64_t ne = 0;
    pg_status s = pg_run_epochs(c, num_epochs, use_graph, &ne);
    c->out_src = c->out_dst = nullptr;
    c->out_cap = c->out_epochs = 0;
    if (s != PG_OK) return s;
    // epochs whose citations did not fit the buffers were grown all the same; the caller learns of it
    const bool short_out = c->h_st.out_short != 0;
    if (short_out) ne = (int64_t)c->h_st.out_count;
    if (staged && ne > 0) {
        PG_CUDA(c, cudaMemcpyAsync(src, ds, 4 * (size_t)ne, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(dst, dd, 4 * (size_t)ne, cudaMemcpyDeviceToHost, c->stream));
    }
    if (counts)
        PG_CUDA(c, cudaMemcpyAsync(counts, c->out_counts.p, 8 * (size_t)nc, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (new_edges) *new_edges = ne;
    if (short_out)
        return fail(c, PG_ERR_CAPACITY, "output buffers hold " + std::to_string(capacity) + " citations; the run made " +
                                            std::to_string(c->h_st.out_count + c->h_st.out_short) +
                                            " (the graph grew; the epochs that did not fit were not written)");
    return PG_OK;
}

namespace {
// Buffers of ER epochs with at most `tasks` walks and `slots` reserved slots.
pg_status ensure_er_buffers(pg_ctx* c, int64_t tasks, int64_t slots) {
    if (c->er_cnt.n < tasks + 1) PG_CUDA(c, dalloc(c->er_cnt, tasks + 1));
    if (c->er_toff.n < tasks + 1) PG_CUDA(c, dalloc(c->er_toff, tasks + 1));
    if (c->er_ovb.n < tasks) PG_CUDA(c, dalloc(c->er_ovb, std::max<int64_t>(tasks, 1)));
    if (c->er_slots.n < slots) PG_CUDA(c, dalloc(c->er_slots, std::max<int64_t>(slots, 1)));
    const int64_t ov = std::max<int64_t>(slots, 1 << 16);
    if (c->er_ov.n < ov) PG_CUDA(c, dalloc(c->er_ov, ov));
    return PG_OK;
}
ErBuffers er_buffers(pg_ctx* c) {
    ErBuffers B;
    B.cnt = c->er_cnt.p;
    B.toff = c->er_toff.p;
    B.slots = c->er_slots.p;
    B.ov = c->er_ov.p;
    B.ov_cap = c->er_ov.n;
    B.ovb = c->er_ovb.p;
    return B;
}
}  // namespace

pg_status pg_er_epoch(pg_ctx* c, int64_t delta, double p, int64_t* new_edges) {
    if (!c) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->R != 1) return fail(c, PG_ERR_ARG, "ER epochs run on single-replica contexts");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    if (delta <= 0 || std::isnan(p)) return fail(c, PG_ERR_ARG, "need delta > 0 and a numeric p");
    if (p > 1.0) p = 1.0;
    PG_CUDA(c, cudaSetDevice(c->device));
    HostRep& h = c->hrep[0];
    const int64_t n = h.n;
    const int64_t chunks = (n + kErChunk - 1) / kErChunk;
    const int64_t tasks = delta * chunks;
    const double pe = p > 0.0 ? p : 0.0;
    const double mu = (double)delta * (double)n * pe;
    int64_t eb = (int64_t)std::ceil(mu + 8.0 * std::sqrt(mu) + 1024.0);
    eb = std::min<int64_t>(eb, delta * n);
    pg_status s = ensure_capacity(c, n + delta, h.m + eb);
    if (s != PG_OK) return s;
    s = alloc_epoch_buffers(c, delta, eb, tasks);
    if (s != PG_OK) return s;
    const ErPlan plan = er_plan(n, delta, p, c->tune.er_slot_sigmas);
    s = ensure_er_buffers(c, plan.tasks, delta * plan.per_node);
    if (s != PG_OK) return s;
    Arena A = make_arena(c);
    cudaStream_t st = c->stream;
    if (c->timing) cudaEventRecord(c->ev[0], st);
    launch_epoch_begin_delta(A, c->epoch, delta, st);
    launch_er_epoch(A, delta, p, plan, er_buffers(c), c->num_sms, st);
    if (c->timing) cudaEventRecord(c->ev[1], st);
    launch_bwd_append(A, delta, c->num_sms, st, c->side, c->fork, c->join);
    if (c->timing) cudaEventRecord(c->ev[2], st);
    PG_CUDA(c, cudaGetLastError());
    std::vector<int64_t> deltas(1, delta);
    s = finish_epoch(c, deltas, true);
    if (s != PG_OK) return s;
    if (c->timing) {
        c->stats.ms_er = ms_between(c->ev[0], c->ev[1]);
        c->stats.ms_csr = ms_between(c->ev[1], c->ev[2]);
        c->stats.ms_total = ms_between(c->ev[0], c->ev[2]);
        c->stats.ms_weights = c->stats.ms_setup = c->stats.ms_agents = 0.0;
    }
    if (new_edges) *new_edges = c->stats.new_edges;
    return PG_OK;
}

pg_status pg_run_er_epochs(pg_ctx* c, int32_t num_epochs, int64_t delta, double p, int64_t* new_edges) {
    if (!c) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->R != 1) return fail(c, PG_ERR_ARG, "ER epochs run on single-replica contexts");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    if (num_epochs < 1 || delta <= 0 || std::isnan(p)) return fail(c, PG_ERR_ARG, "need num_epochs >= 1, delta > 0 and a numeric p");
    if (p > 1.0) p = 1.0;
    PG_CUDA(c, cudaSetDevice(c->device));
    const int64_t n0 = c->hrep[0].n, m0 = c->hrep[0].m;
    const double pe = p > 0.0 ? p : 0.0;
    // every epoch's node count is known; edges are bounded per epoch by mean + 8 sigma
    int64_t need_m = m0, max_eb = 0, max_tasks = 0, max_slots = 0;
    std::vector<ErPlan> plans((size_t)num_epochs);
    for (int e = 0; e < num_epochs; ++e) {
        const int64_t n = n0 + (int64_t)e * delta;
        const double mu = (double)delta * (double)n * pe;
        const int64_t eb = std::min<int64_t>((int64_t)std::ceil(mu + 8.0 * std::sqrt(mu) + 1024.0), delta * n);
        need_m += eb;
        max_eb = std::max(max_eb, eb);
        plans[(size_t)e] = er_plan(n, delta, p, c->tune.er_slot_sigmas);
        max_tasks = std::max(max_tasks, plans[(size_t)e].tasks);
        max_slots = std::max(max_slots, delta * plans[(size_t)e].per_node);
    }
    pg_status s = ensure_capacity(c, n0 + (int64_t)num_epochs * delta, need_m);
    if (s != PG_OK) return s;
    s = alloc_epoch_buffers(c, delta, max_eb, max_tasks);
    if (s != PG_OK) return s;
    s = ensure_er_buffers(c, max_tasks, max_slots);
    if (s != PG_OK) return s;
    cudaStream_t st = c->stream;
    const size_t cum0 = offsetof(EpochState, cum_rows_expanded);
    PG_CUDA(c, cudaMemsetAsync(reinterpret_cast<char*>(c->st.p) + cum0, 0, sizeof(EpochState) - cum0, st));
    cudaGetLastError();
    if (c->timing) cudaEventRecord(c->ev[0], st);
    for (int e = 0; e < num_epochs; ++e) {
        Arena A = make_arena(c);
        launch_epoch_begin_delta(A, c->epoch + e, delta, st);
        launch_er_epoch(A, delta, p, plans[(size_t)e], er_buffers(c), c->num_sms, st);
        launch_bwd_append(A, delta, c->num_sms, st, c->side, c->fork, c->join);
    }
    if (c->timing) cudaEventRecord(c->ev[1], st);
    PG_CUDA(c, cudaGetLastError());
    s = read_back(c);
    if (s != PG_OK) return s;
    s = device_error(c);
    if (s != PG_OK) return s;
    HostRep& h = c->hrep[0];
    h.n = c->h_rep[0].n;
    h.m = c->h_rep[0].m;
    c->epoch += num_epochs;
    c->rep_last_first[0] = h.m - (int64_t)c->h_st.edges;  // the last epoch's edges
    c->rep_last_count[0] = (int64_t)c->h_st.edges;
    fill_stats(c, delta, true);
    c->stats.run_epochs = num_epochs;
    c->stats.run_new_nodes = (int64_t)num_epochs * delta;
    c->stats.run_new_edges = h.m - m0;
    if (c->timing) {
        c->stats.ms_er = c->stats.ms_total = ms_between(c->ev[0], c->ev[1]);
        c->stats.ms_weights = c->stats.ms_setup = c->stats.ms_agents = c->stats.ms_csr = 0.0;
    }
    if (new_edges) *new_edges = h.m - m0;
    return PG_OK;
}

pg_status pg_reserve(pg_ctx* c, int64_t n_cap, int64_t m_cap) {
    if (!c) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->R != 1) return fail(c, PG_ERR_ARG, "capacity reservations apply to single-replica contexts");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    if (n_cap < 0 || m_cap < 0) return fail(c, PG_ERR_ARG, "negative capacity");
    PG_CUDA(c, cudaSetDevice(c->device));
    return ensure_capacity(c, n_cap, m_cap);
}

pg_status pg_get_counts(const pg_ctx* c, int32_t replica, int64_t* n, int64_t* m) {
    if (!c || replica < 0 || replica >= c->R || !c->loaded) return PG_ERR_ARG;
    if (n) *n = c->hrep[(size_t)replica].n;
    if (m) *m = c->hrep[(size_t)replica].m;
    return PG_OK;
}

pg_status pg_epoch_edges(const pg_ctx* c, int32_t replica, int64_t* first, int64_t* count) {
    if (!c || replica < 0 || replica >= c->R || !c->loaded) return PG_ERR_ARG;
    if (first) *first = c->rep_last_first[(size_t)replica];
    if (count) *count = c->rep_last_count[(size_t)replica];
    return PG_OK;
}

pg_status pg_copy_edges(pg_ctx* c, int32_t replica, int64_t first, int64_t count, int32_t* src,
                        int32_t* dst) {
    if (!c) return PG_ERR_ARG;
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    const HostRep& h = c->hrep[(size_t)replica];
    if (first < 0 || count < 0 || first + count > h.m) return fail(c, PG_ERR_ARG, "edge range out of bounds");
    PG_CUDA(c, cudaSetDevice(c->device));
    if (dst && count)
        PG_CUDA(c, cudaMemcpyAsync(dst, c->fwd_col.p + h.ebase + first, 4 * (size_t)count,
                                   cudaMemcpyDeviceToHost, c->stream));
    if (src && count) {
        // sources expanded from the forward offsets on the device (rows are contiguous in edge
        // order), then one copy
        if (c->src_tmp.n < count) PG_CUDA(c, dalloc(c->src_tmp, count));
        launch_edge_sources(c->fwd_off.p + h.obase, h.n, first, count, c->src_tmp.p, c->num_sms, c->stream);
        PG_CUDA(c, cudaGetLastError());
        PG_CUDA(c, cudaMemcpyAsync(src, c->src_tmp.p, 4 * (size_t)count, cudaMemcpyDeviceToHost, c->stream));
    }
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_copy_degrees(pg_ctx* c, int32_t replica, int32_t* indeg, int32_t* outdeg) {
    if (!c) return PG_ERR_ARG;
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    const HostRep& h = c->hrep[(size_t)replica];
    PG_CUDA(c, cudaSetDevice(c->device));
    if (indeg)
        PG_CUDA(c, cudaMemcpyAsync(indeg, c->indeg.p + h.nbase, 4 * (size_t)h.n, cudaMemcpyDeviceToHost, c->stream));
    if (outdeg) {
        std::vector<int64_t> off((size_t)h.n + 1);
        PG_CUDA(c, cudaMemcpyAsync(off.data(), c->fwd_off.p + h.obase, 8 * off.size(), cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int64_t v = 0; v < h.n; ++v) outdeg[v] = (int32_t)(off[(size_t)v + 1] - off[(size_t)v]);
    }
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_copy_nodes(pg_ctx* c, int32_t replica, int32_t* pub_epoch, float* fitness) {
    if (!c) return PG_ERR_ARG;
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    const HostRep& h = c->hrep[(size_t)replica];
    PG_CUDA(c, cudaSetDevice(c->device));
    if (pub_epoch)
        PG_CUDA(c, cudaMemcpyAsync(pub_epoch, c->pub.p + h.nbase, 4 * (size_t)h.n, cudaMemcpyDeviceToHost, c->stream));
    if (fitness)
        PG_CUDA(c, cudaMemcpyAsync(fitness, c->fit.p + h.nbase, 4 * (size_t)h.n, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_copy_csr(pg_ctx* c, int32_t replica, int32_t which, int64_t* off, int32_t* col) {
    if (!c) return PG_ERR_ARG;
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    if (which != 0 && which != 1) return fail(c, PG_ERR_ARG, "which must be 0 or 1");
    const HostRep& h = c->hrep[(size_t)replica];
    PG_CUDA(c, cudaSetDevice(c->device));
    if (which) return backward_offset_form(c, replica, off, col);
    if (off)
        PG_CUDA(c, cudaMemcpyAsync(off, c->fwd_off.p + h.obase, 8 * (size_t)(h.n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (col && h.m)
        PG_CUDA(c, cudaMemcpyAsync(col, c->fwd_col.p + h.ebase, 4 * (size_t)h.m, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_copy_arrivals(pg_ctx* c, int32_t replica, int32_t* cited) {
    if (!c || !cited) return PG_ERR_ARG;
    if (!c->cfg.record_trace) return fail(c, PG_ERR_STATE, "context created without record_trace");
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    // epoch edge index of the replica's first edge = sum of earlier replicas' counts
    int64_t base = 0;
    for (int r = 0; r < replica; ++r) base += c->rep_last_count[(size_t)r];
    const int64_t cnt = c->rep_last_count[(size_t)replica];
    if (cnt)
        PG_CUDA(c, cudaMemcpyAsync(cited, c->arrivals.p + base, 4 * (size_t)cnt, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_copy_anchors(pg_ctx* c, int32_t replica, int32_t* anchors) {
    if (!c || !anchors) return PG_ERR_ARG;
    if (!c->cfg.record_trace) return fail(c, PG_ERR_STATE, "context created without record_trace");
    if (replica < 0 || replica >= c->R || !c->loaded) return fail(c, PG_ERR_ARG, "bad replica");
    if (c->h_rep.size() != (size_t)c->R || c->stats.epoch < 0 || c->rep_last_count.empty())
        return fail(c, PG_ERR_STATE, "no PA epoch has run");
    const Replica& h = c->h_rep[(size_t)replica];
    if (h.delta > 0)
        PG_CUDA(c, cudaMemcpyAsync(anchors, c->anchors.p + 4 * h.abase, 16 * (size_t)h.delta,
                                   cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_set_timing(pg_ctx* c, int32_t enable) {
    if (!c) return PG_ERR_ARG;
    c->timing = enable != 0;
    destroy_graph_exec(c);
    return PG_OK;
}

pg_status pg_get_stats(const pg_ctx* c, pg_stats* out) {
    if (!c || !out) return PG_ERR_ARG;
    *out = c->stats;
    return PG_OK;
}

pg_status pg_sync(pg_ctx* c) {
    if (!c) return PG_ERR_ARG;
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_check_device(pg_ctx* c) {
    if (!c) return PG_ERR_ARG;
    pg_status s = read_back(c);
    if (s != PG_OK) return s;
    return device_error(c);
}

pg_status pg_timer_start(pg_ctx* c) {
    if (!c) return PG_ERR_ARG;
    PG_CUDA(c, cudaEventRecord(c->tev[0], c->stream));
    return PG_OK;
}

pg_status pg_timer_stop(pg_ctx* c, double* ms) {
    if (!c || !ms) return PG_ERR_ARG;
    PG_CUDA(c, cudaEventRecord(c->tev[1], c->stream));
    PG_CUDA(c, cudaEventSynchronize(c->tev[1]));
    float f = 0.0f;
    PG_CUDA(c, cudaEventElapsedTime(&f, c->tev[0], c->tev[1]));
    *ms = f;
    return PG_OK;
}

pg_status pg_checkpoint(pg_ctx* c) {
    if (!c) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "state is inconsistent after a device error");
    Checkpoint& k = c->ckpt;
    cudaStream_t s = c->stream;
    if (k.pub.n != c->S) {
        PG_CUDA(c, dalloc(k.pub, c->S));
        PG_CUDA(c, dalloc(k.indeg, c->S));
        PG_CUDA(c, dalloc(k.fit, c->S));
        PG_CUDA(c, dalloc(k.fwd_off, c->S + c->R));
        PG_CUDA(c, dalloc(k.brow, c->S));
        PG_CUDA(c, dalloc(k.bcap, c->S));
        PG_CUDA(c, dalloc(k.rep, c->R));
    }
    if (k.fwd_col.n != c->M) PG_CUDA(c, dalloc(k.fwd_col, c->M));
    if (k.bcol.n != c->B) PG_CUDA(c, dalloc(k.bcol, c->B));
    // the backward entries in use per replica (the device bump pointers)
    std::vector<Replica> dr((size_t)c->R);
    PG_CUDA(c, cudaMemcpyAsync(dr.data(), c->rep.p, sizeof(Replica) * (size_t)c->R, cudaMemcpyDeviceToHost, s));
    PG_CUDA(c, cudaStreamSynchronize(s));
    k.b_top.assign((size_t)c->R, 0);
    for (int r = 0; r < c->R; ++r) {
        const int64_t top = (int64_t)dr[(size_t)r].b_top;
        if (top < 0 || top > c->hrep[(size_t)r].b_cap) return fail(c, PG_ERR_STATE, "backward region state out of range");
        k.b_top[(size_t)r] = top;
    }
    const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
    if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT) {
        if (k.rc_lag.n != c->S) {
            PG_CUDA(c, dalloc(k.rc_lag, c->S));
            PG_CUDA(c, dalloc(k.rc_dur, c->S));
        }
        PG_CUDA(c, cudaMemcpyAsync(k.rc_lag.p, c->rc_lag.p, 4 * (size_t)c->S, d2d, s));
        PG_CUDA(c, cudaMemcpyAsync(k.rc_dur.p, c->rc_dur.p, 4 * (size_t)c->S, d2d, s));
    }
    PG_CUDA(c, cudaMemcpyAsync(k.pub.p, c->pub.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.indeg.p, c->indeg.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.fit.p, c->fit.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.fwd_off.p, c->fwd_off.p, 8 * (size_t)(c->S + c->R), d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.brow.p, c->brow.p, sizeof(BRow) * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.bcap.p, c->bcap.p, sizeof(int32_t) * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(k.rep.p, c->rep.p, sizeof(Replica) * (size_t)c->R, d2d, s));
    for (int r = 0; r < c->R; ++r) {
        const HostRep& h = c->hrep[(size_t)r];
        if (h.m) PG_CUDA(c, cudaMemcpyAsync(k.fwd_col.p + h.ebase, c->fwd_col.p + h.ebase, 4 * (size_t)h.m, d2d, s));
        const int64_t top = k.b_top[(size_t)r];
        if (top) PG_CUDA(c, cudaMemcpyAsync(k.bcol.p + h.bbase, c->bcol.p + h.bbase, 4 * (size_t)top, d2d, s));
    }
    PG_CUDA(c, cudaStreamSynchronize(s));
    k.epoch = c->epoch;
    k.hrep = c->hrep;
    k.valid = true;
    return PG_OK;
}

pg_status pg_restore(pg_ctx* c) {
    if (!c) return PG_ERR_ARG;
    Checkpoint& k = c->ckpt;
    if (!k.valid || k.pub.n != c->S || k.fwd_col.n != c->M || k.bcol.n != c->B)
        return fail(c, PG_ERR_STATE, "no checkpoint matches the current arena");
    cudaStream_t s = c->stream;
    const cudaMemcpyKind d2d = cudaMemcpyDeviceToDevice;
    if (c->cfg.weight_model == PG_WEIGHTS_REFCOMPAT && k.rc_lag.n == c->S) {
        PG_CUDA(c, cudaMemcpyAsync(c->rc_lag.p, k.rc_lag.p, 4 * (size_t)c->S, d2d, s));
        PG_CUDA(c, cudaMemcpyAsync(c->rc_dur.p, k.rc_dur.p, 4 * (size_t)c->S, d2d, s));
    }
    PG_CUDA(c, cudaMemcpyAsync(c->pub.p, k.pub.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->indeg.p, k.indeg.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->fit.p, k.fit.p, 4 * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->fwd_off.p, k.fwd_off.p, 8 * (size_t)(c->S + c->R), d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->brow.p, k.brow.p, sizeof(BRow) * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->bcap.p, k.bcap.p, sizeof(int32_t) * (size_t)c->S, d2d, s));
    PG_CUDA(c, cudaMemcpyAsync(c->rep.p, k.rep.p, sizeof(Replica) * (size_t)c->R, d2d, s));
    // the hub index is not part of the checkpoint: the next epoch rebuilds it
    PG_CUDA(c, cudaMemset2DAsync(reinterpret_cast<char*>(c->rep.p) + offsetof(Replica, hub_valid), sizeof(Replica), 0,
                                 sizeof(int32_t), (size_t)c->R, s));
    for (size_t r = 0; r < k.hrep.size(); ++r) {
        const HostRep& h = k.hrep[r];
        if (h.m) PG_CUDA(c, cudaMemcpyAsync(c->fwd_col.p + h.ebase, k.fwd_col.p + h.ebase, 4 * (size_t)h.m, d2d, s));
        const int64_t top = k.b_top[r];
        if (top) PG_CUDA(c, cudaMemcpyAsync(c->bcol.p + h.bbase, k.bcol.p + h.bbase, 4 * (size_t)top, d2d, s));
    }
    PG_CUDA(c, cudaMemsetAsync(c->inc.p, 0, 4 * (size_t)c->S, s));
    // the saved state is consistent: clear the error word a failed epoch left set
    PG_CUDA(c, cudaMemsetAsync(reinterpret_cast<char*>(c->st.p) + offsetof(EpochState, error), 0,
                               sizeof(uint32_t), s));
    PG_CUDA(c, cudaStreamSynchronize(s));
    c->epoch = k.epoch;
    c->hrep = k.hrep;
    c->poisoned = false;
    return PG_OK;
}

pg_status pg_set_tuning(pg_ctx* c, const pg_tuning* t) {
    if (!c) return PG_ERR_ARG;
    if (!t || t->agent_ctas_per_sm < 0 || t->agent_ctas_per_sm > 32 || t->copy_ctas_per_sm < 0 ||
        t->copy_ctas_per_sm > 64 || (t->small_hash != 0 && t->small_hash != 1) || t->lik_chunk_agents < 0 ||
        (t->epoch_kernel != 0 && t->epoch_kernel != 1) || t->er_slot_sigmas < 0 || t->er_slot_sigmas > 64)
        return fail(c, PG_ERR_ARG, "tuning out of range");
    if (std::memcmp(&c->tune, t, sizeof(pg_tuning)) != 0) {
        c->tune = *t;
        destroy_graph_exec(c);  // captured launches carry the old grid sizes
    }
    return PG_OK;
}

pg_status pg_lik_set_exact_exp2(pg_ctx* c, int32_t exact) {
    if (!c) return PG_ERR_ARG;
    if (exact != 0 && exact != 1) return fail(c, PG_ERR_ARG, "exact must be 0 or 1");
    c->lik.exact_exp2 = exact;
    return PG_OK;
}

pg_status pg_set_wait_limit(pg_ctx* c, int64_t polls) {
    if (!c) return PG_ERR_ARG;
    const uint32_t v = polls < 0 ? kWaitPolls : (uint32_t)std::min<int64_t>(polls, kWaitPolls);
    if (v != c->first_wait_polls) {
        c->first_wait_polls = v;
        destroy_graph_exec(c);  // captured launches carry the old bound
    }
    return PG_OK;
}

pg_status pg_get_tuning(const pg_ctx* c, pg_tuning* t) {
    if (!c || !t) return PG_ERR_ARG;
    *t = c->tune;
    return PG_OK;
}

// Coordinate search: agent-kernel shape (frontier hash capacity x CTAs per SM) first, then the
// backward-copy grid, then the whole epoch as one persistent kernel.  Each candidate runs the same
// epochs from the same saved state twice, as a captured graph (the second run, a replay, is the
// one timed).
pg_status pg_autotune(pg_ctx* c, int32_t num_epochs, pg_tuning* best, double* best_ms) {
    if (!c) return PG_ERR_ARG;
    if (num_epochs < 1) return fail(c, PG_ERR_ARG, "num_epochs must be >= 1");
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (c->poisoned) return fail(c, PG_ERR_STATE, "an earlier epoch failed on the device; reload the graph");
    PG_CUDA(c, cudaSetDevice(c->device));
    {
        // size the arena for the run first: a single-replica arena that grew afterwards would no
        // longer match the saved state
        std::vector<int64_t> agents;
        int64_t ma = 0, me = 0;
        const pg_status ps = plan_run(c, num_epochs, agents, ma, me);
        if (ps != PG_OK) return ps;
    }
    Checkpoint user = c->ckpt;  // the caller's checkpoint stays aside, untouched
    c->ckpt = Checkpoint{};
    const pg_tuning start = c->tune;
    pg_status s = PG_OK;
    int64_t ref_edges = -1;
    double best_t = 1e300;
    pg_tuning best_cfg = start;
    auto trial = [&](const pg_tuning& t) -> pg_status {
        pg_status ts = pg_set_tuning(c, &t);
        double ms = 0.0;
        int64_t e1 = 0, e2 = 0;
        if (ts == PG_OK) ts = pg_restore(c);
        if (ts == PG_OK) ts = pg_run_epochs(c, num_epochs, 1, &e1);
        if (ts == PG_OK) ts = pg_restore(c);
        if (ts == PG_OK) ts = pg_timer_start(c);
        if (ts == PG_OK) ts = pg_run_epochs(c, num_epochs, 1, &e2);
        if (ts == PG_OK) ts = pg_timer_stop(c, &ms);
        if (ts != PG_OK) return ts;
        if (ref_edges < 0) ref_edges = e1;
        if (e1 != ref_edges || e2 != ref_edges)
            return fail(c, PG_ERR_STATE, "tuning candidates disagree on the edge count");
        if (ms < best_t) {
            best_t = ms;
            best_cfg = c->tune;
        }
        return PG_OK;
    };
    s = pg_checkpoint(c);
    const int thin = c->cfg.sampler == PG_SAMPLER_THINNING ? 1 : 0;
    for (int hs = 0; hs <= thin && s == PG_OK; ++hs) {
        const int occ = agent_occupancy(thin, hs);
        std::vector<int> vals;
        for (int v : {0, std::max(1, (occ * 3) / 4), std::max(1, occ / 2)}) {
            if (v >= occ) v = 0;
            if (std::find(vals.begin(), vals.end(), v) == vals.end()) vals.push_back(v);
        }
        for (int v : vals) {
            if (s != PG_OK) break;
            pg_tuning t = start;
            t.agent_ctas_per_sm = v;
            t.small_hash = hs;
            s = trial(t);
        }
    }
    const int copies[3] = {4, 8, 16};
    const pg_tuning agent_best = best_cfg;
    for (int i = 0; i < 3 && s == PG_OK; ++i) {
        pg_tuning t = agent_best;
        t.copy_ctas_per_sm = copies[i];
        if (t.copy_ctas_per_sm == (agent_best.copy_ctas_per_sm ? agent_best.copy_ctas_per_sm : 8)) continue;
        s = trial(t);
    }
    // the whole epoch as one persistent kernel (its own launch shape: two CTAs of 8 warps per SM)
    if (s == PG_OK && thin && c->cfg.weight_model == PG_WEIGHTS_BASELINE && epoch_kernel_ctas() > 0) {
        pg_tuning t = start;
        t.epoch_kernel = 1;
        s = trial(t);
    }
    // leave the graph as it was and the best tuning in force
    if (c->ckpt.valid) {
        const pg_status rs = pg_restore(c);
        if (s == PG_OK) s = rs;
    }
    free_checkpoint(c->ckpt);
    c->ckpt = user;
    if (s != PG_OK) {
        pg_set_tuning(c, &start);
        return s;
    }
    s = pg_set_tuning(c, &best_cfg);
    if (best) *best = best_cfg;
    if (best_ms) *best_ms = best_t;
    return s;
}

void pg_philox4x32_10(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]) {
    const u32x4 r = philox(c[0], c[1], c[2], c[3], k[0], k[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.x[i];
}

pg_status pg_poisson_table(double lambda, uint64_t* table) {
    if (!table || !(lambda >= 0.0)) return PG_ERR_ARG;
    poisson_table(lambda, table, kTableEntries);
    return PG_OK;
}

float pg_logf_host(float x) { return logf_pg(x); }
float pg_expf_host(float x) { return expf_pg(x); }
double pg_log_host(double x) { return log_pg(x); }
double pg_exp_host(double x) { return exp_pg(x); }


// ---------------------------------------------------------------- refcompat functor
pg_status pg_rc_bag_table(const int32_t* bag, int64_t len, uint64_t* table) {
    if (!bag || len <= 0 || !table) return PG_ERR_ARG;
    rc_bag_table_host(bag, len, table);
    return PG_OK;
}

pg_status pg_rc_fitness_table(uint64_t* table) {
    if (!table) return PG_ERR_ARG;
    rc_fitness_table_host(table);
    return PG_OK;
}

pg_status pg_rc_configure(pg_ctx* c, int32_t replica, const pg_rc_params* p, const int32_t* bag,
                          int64_t bag_len, const double* rec, int32_t rec_len) {
    if (!c || !p) return PG_ERR_ARG;
    if (c->cfg.weight_model != PG_WEIGHTS_REFCOMPAT)
        return fail(c, PG_ERR_STATE, "the context was not created with PG_WEIGHTS_REFCOMPAT");
    if (!c->loaded) return fail(c, PG_ERR_STATE, "load a graph first");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    if (!bag || bag_len <= 0) return fail(c, PG_ERR_ARG, "the out-degree bag is empty");
    if (rec_len < 0 || rec_len > kRcAgeMax || (rec_len > 0 && !rec))
        return fail(c, PG_ERR_ARG, "recency table must have 0..1024 entries");
    if (!(p->growth_rate > 0.0)) return fail(c, PG_ERR_ARG, "growth_rate must be > 0");
    if (!(p->fully_random >= 0.0 && p->fully_random <= 1.0)) return fail(c, PG_ERR_ARG, "fully_random must be in [0, 1]");
    if (!(p->same_year >= 0.0 && p->same_year <= 1.0)) return fail(c, PG_ERR_ARG, "same_year must be in [0, 1]");
    if (p->gamma < 1 || p->gamma > 4 || p->decay < 0 || p->decay > 8)
        return fail(c, PG_ERR_ARG, "gamma must be in [1, 4] and decay in [0, 8]");
    const bool fixed = p->pa_weight >= 0.0 && p->rec_weight >= 0.0 && p->fit_weight >= 0.0;
    if (fixed && !(p->pa_weight + p->rec_weight + p->fit_weight > 0.0))
        return fail(c, PG_ERR_ARG, "the three score weights sum to zero");
    for (int i = 0; i < rec_len; ++i)
        if (!(rec[i] >= 0.0) || !std::isfinite(rec[i])) return fail(c, PG_ERR_ARG, "recency probabilities must be finite and >= 0");
    PG_CUDA(c, cudaSetDevice(c->device));
    HostRep& h = c->hrep[(size_t)replica];
    h.rc = true;
    h.rcp = *p;
    h.prm.growth_rate = p->growth_rate;
    h.prm.fixed_new_nodes = 0;
    h.bag_table.assign(kTableEntries, 0);
    rc_bag_table_host(bag, bag_len, h.bag_table.data());
    int32_t kmax = 1;
    for (int64_t i = 0; i < bag_len; ++i) kmax = std::max(kmax, std::min<int32_t>(bag[i], kRcMaxOutDegree));
    h.kmax = kmax;
    h.rtab.assign(rec, rec + rec_len);
    destroy_graph_exec(c);
    std::vector<double> rt(kRcAgeMax, 0.0);
    std::copy(h.rtab.begin(), h.rtab.end(), rt.begin());
    PG_CUDA(c, cudaMemcpyAsync(c->rc_rtab.p + (size_t)replica * kRcAgeMax, rt.data(), 8 * rt.size(),
                               cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(c->tables.p + (size_t)replica * kTableEntries, h.bag_table.data(),
                               8 * h.bag_table.size(), cudaMemcpyHostToDevice, c->stream));
    Replica dr;
    PG_CUDA(c, cudaMemcpyAsync(&dr, c->rep.p + replica, sizeof(Replica), cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    const Replica fresh = to_device_rep(h);
    for (int i = 0; i < 3; ++i) dr.rc_w[i] = fresh.rc_w[i];
    dr.rc_alpha = fresh.rc_alpha;
    dr.rc_frc = fresh.rc_frc;
    dr.rc_sy = fresh.rc_sy;
    dr.rc_gamma = fresh.rc_gamma;
    dr.rc_decay = fresh.rc_decay;
    dr.rc_rec_len = fresh.rc_rec_len;
    dr.growth_rate = fresh.growth_rate;
    dr.fixed_new = fresh.fixed_new;
    PG_CUDA(c, cudaMemcpyAsync(c->rep.p + replica, &dr, sizeof(Replica), cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_rc_set_nodes(pg_ctx* c, int32_t replica, int64_t first, int64_t count, const int32_t* lag,
                          const int32_t* peak, const int32_t* dur) {
    if (!c || !lag || !peak || !dur) return PG_ERR_ARG;
    if (c->cfg.weight_model != PG_WEIGHTS_REFCOMPAT)
        return fail(c, PG_ERR_STATE, "the context was not created with PG_WEIGHTS_REFCOMPAT");
    if (!c->loaded) return fail(c, PG_ERR_STATE, "load a graph first");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    const HostRep& h = c->hrep[(size_t)replica];
    if (first < 0 || count < 0 || first + count > h.n) return fail(c, PG_ERR_ARG, "node range out of bounds");
    if (count == 0) return PG_OK;
    std::vector<float> pk((size_t)count);
    for (int64_t i = 0; i < count; ++i) {
        if (peak[i] < 1 || lag[i] < 0 || dur[i] < 0) return fail(c, PG_ERR_ARG, "peak must be >= 1, lag and duration >= 0");
        pk[(size_t)i] = (float)peak[i];
    }
    PG_CUDA(c, cudaSetDevice(c->device));
    PG_CUDA(c, cudaMemcpyAsync(c->rc_lag.p + h.nbase + first, lag, 4 * (size_t)count, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(c->rc_dur.p + h.nbase + first, dur, 4 * (size_t)count, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(c->fit.p + h.nbase + first, pk.data(), 4 * (size_t)count, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_rc_copy_agents(pg_ctx* c, int32_t replica, double* out) {
    if (!c || !out) return PG_ERR_ARG;
    if (c->cfg.weight_model != PG_WEIGHTS_REFCOMPAT)
        return fail(c, PG_ERR_STATE, "the context was not created with PG_WEIGHTS_REFCOMPAT");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    if (c->h_rep.size() != (size_t)c->R || !c->rc_agent.p) return fail(c, PG_ERR_STATE, "no refcompat epoch has run");
    const Replica& r = c->h_rep[(size_t)replica];
    PG_CUDA(c, cudaSetDevice(c->device));
    PG_CUDA(c, cudaMemcpyAsync(out, c->rc_agent.p + 6 * r.abase, 8 * 6 * (size_t)r.delta, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}


// ---------------------------------------------------------------- text output
pg_status pg_format_edges(pg_ctx* c, int32_t replica, const int64_t* ids, int64_t n_ids, char* out,
                          int64_t cap, int64_t* bytes) {
    if (!c || !ids || !bytes) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    const HostRep& h = c->hrep[(size_t)replica];
    if (n_ids != h.n) return fail(c, PG_ERR_ARG, "ids must hold one id per node");
    PG_CUDA(c, cudaSetDevice(c->device));
    const int64_t n = h.n, m = h.m;
    struct Tmp {
        DBuf<int64_t> did, off, bs;
        DBuf<int32_t> len;
        DBuf<char> txt;
        ~Tmp() {
            dfree(did);
            dfree(off);
            dfree(bs);
            dfree(len);
            dfree(txt);
        }
    } t;
    PG_CUDA(c, dalloc(t.did, n));
    PG_CUDA(c, dalloc(t.len, std::max<int64_t>(m, 1)));
    PG_CUDA(c, dalloc(t.off, m + 1));
    PG_CUDA(c, dalloc(t.bs, scan_blocks_needed(std::max<int64_t>(m, 1)) + 2));
    PG_CUDA(c, cudaMemcpyAsync(t.did.p, ids, 8 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    const int64_t* fo = c->fwd_off.p + h.obase;
    const int32_t* fc = c->fwd_col.p + h.ebase;
    cudaGetLastError();
    launch_text_len(fo, fc, n, m, t.did.p, t.len.p, c->num_sms, c->stream);
    launch_scan_i32_to_i64(t.len.p, t.off.p, m, t.bs.p, c->stream);
    PG_CUDA(c, cudaGetLastError());
    int64_t total = 0;
    PG_CUDA(c, cudaMemcpyAsync(&total, t.off.p + m, 8, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    *bytes = total;
    if (!out) return PG_OK;
    if (cap < total)
        return fail(c, PG_ERR_CAPACITY, "the output buffer holds " + std::to_string(cap) + " bytes, the text needs " +
                                            std::to_string(total));
    PG_CUDA(c, dalloc(t.txt, std::max<int64_t>(total, 1)));
    launch_text_write(fo, fc, n, m, t.did.p, t.off.p, t.txt.p, c->num_sms, c->stream);
    PG_CUDA(c, cudaGetLastError());
    PG_CUDA(c, cudaMemcpyAsync(out, t.txt.p, (size_t)total, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

pg_status pg_format_attributes(pg_ctx* c, int32_t replica, const pg_attr_rows* rows, char* out, int64_t cap,
                               int64_t* bytes) {
    if (!c || !rows || !bytes) return PG_ERR_ARG;
    if (!c->loaded) return fail(c, PG_ERR_STATE, "no graph loaded");
    if (replica < 0 || replica >= c->R) return fail(c, PG_ERR_ARG, "replica out of range");
    const HostRep& h = c->hrep[(size_t)replica];
    const int64_t n = h.n;
    if (rows->num_nodes != n) return fail(c, PG_ERR_ARG, "rows must describe every node of the replica");
    if (rows->num_seed < 0 || rows->num_seed > n) return fail(c, PG_ERR_ARG, "num_seed out of range");
    if (!rows->ids || !rows->draws || !rows->ints || (!rows->generators && rows->num_seed < n))
        return fail(c, PG_ERR_ARG, "ids, draws, ints and generators are required");
    PG_CUDA(c, cudaSetDevice(c->device));
    struct Tmp {
        DBuf<int64_t> did, gen, off, bs;
        DBuf<double> draws;
        DBuf<int32_t> ints, len;
        DBuf<char> txt;
        ~Tmp() {
            dfree(did);
            dfree(gen);
            dfree(off);
            dfree(bs);
            dfree(draws);
            dfree(ints);
            dfree(len);
            dfree(txt);
        }
    } t;
    const size_t nn = (size_t)std::max<int64_t>(n, 1);
    PG_CUDA(c, dalloc(t.did, n));
    PG_CUDA(c, dalloc(t.draws, 4 * n));
    PG_CUDA(c, dalloc(t.ints, 4 * n));
    PG_CUDA(c, dalloc(t.gen, 4 * n));
    PG_CUDA(c, dalloc(t.len, n));
    PG_CUDA(c, dalloc(t.off, n + 1));
    PG_CUDA(c, dalloc(t.bs, scan_blocks_needed(std::max<int64_t>(n, 1)) + 2));
    PG_CUDA(c, cudaMemcpyAsync(t.did.p, rows->ids, 8 * nn, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(t.draws.p, rows->draws, 32 * nn, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(t.ints.p, rows->ints, 16 * nn, cudaMemcpyHostToDevice, c->stream));
    if (rows->num_seed < n) {
        const int64_t k = n - rows->num_seed;  // only the agents' generator rows are read
        PG_CUDA(c, cudaMemcpyAsync(t.gen.p + 4 * rows->num_seed, rows->generators + 4 * rows->num_seed,
                                   32 * (size_t)k, cudaMemcpyHostToDevice, c->stream));
    }
    AttrCols C{};
    C.n = n;
    C.n_seed = rows->num_seed;
    C.ids = t.did.p;
    C.draws = t.draws.p;
    C.ints = t.ints.p;
    C.gens = t.gen.p;
    C.pub = c->pub.p + h.nbase;
    C.fit = c->fit.p + h.nbase;
    C.indeg = c->indeg.p + h.nbase;
    C.fo = c->fwd_off.p + h.obase;
    C.peak_int = rows->peak_integer ? 1 : 0;
    cudaGetLastError();
    launch_attr_text(C, t.len.p, nullptr, nullptr, c->num_sms, c->stream);
    launch_scan_i32_to_i64(t.len.p, t.off.p, n, t.bs.p, c->stream);
    PG_CUDA(c, cudaGetLastError());
    int64_t total = 0;
    PG_CUDA(c, cudaMemcpyAsync(&total, t.off.p + n, 8, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    *bytes = total;
    if (!out) return PG_OK;
    if (cap < total)
        return fail(c, PG_ERR_CAPACITY, "the output buffer holds " + std::to_string(cap) + " bytes, the text needs " +
                                            std::to_string(total));
    PG_CUDA(c, dalloc(t.txt, std::max<int64_t>(total, 1)));
    launch_attr_text(C, nullptr, t.off.p, t.txt.p, c->num_sms, c->stream);
    PG_CUDA(c, cudaGetLastError());
    PG_CUDA(c, cudaMemcpyAsync(out, t.txt.p, (size_t)total, cudaMemcpyDeviceToHost, c->stream));
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- trace log-likelihood
namespace {

template <typename T>
pg_status upload(pg_ctx* c, DBuf<T>& d, const T* h, int64_t n) {
    PG_CUDA(c, dalloc(d, n));
    if (n > 0) PG_CUDA(c, cudaMemcpyAsync(d.p, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    return PG_OK;
}

LikTrace make_trace(const pg_ctx* c) {
    const LikState& L = c->lik;
    LikTrace T{};
    T.n = L.n;
    T.agents = L.agents;
    T.epochs = L.epochs;
    T.num_anchors = L.num_anchors;
    T.bitmap_words = L.words;
    T.chunks = L.chunks;
    T.epoch_nodes = L.epoch_nodes.p;
    T.epoch_t = L.epoch_t.p;
    T.fo = L.fo.p;
    T.fc = L.fc.p;
    T.bo = L.bo.p;
    T.bc = L.bc.p;
    T.fit = L.fit.p;
    T.pub = L.pub.p;
    T.feat = L.feat.p;
    T.anchors = L.anchors.p;
    T.coff = L.coff.p;
    T.cites = L.cites.p;
    T.agent_epoch = L.agent_epoch.p;
    return T;
}

pg_status check_theta(pg_ctx* c, int32_t batch, const double* theta) {
    if (batch < 1 || !theta) return fail(c, PG_ERR_ARG, "need batch >= 1 parameter points");
    for (int b = 0; b < batch; ++b) {
        const double* t = theta + 4 * b;
        if (!std::isfinite(t[0]) || !std::isfinite(t[2]) || !(t[1] > 0.0) || !std::isfinite(t[1]) ||
            !(t[3] > 0.0) || !std::isfinite(t[3]))
            return fail(c, PG_ERR_ARG, "theta " + std::to_string(b) + ": need finite alpha, gamma and tau, beta > 0");
    }
    return PG_OK;
}

LikBalls make_balls(const LikState& L, int64_t a0) {
    LikBalls Bl{};
    Bl.boff = L.boff.p;
    Bl.base = L.hboff.empty() ? 0 : L.hboff[(size_t)a0];
    Bl.ids = L.bids.p;
    Bl.cflag = L.cflag.p;
    Bl.cnt = L.bcnt.p;
    Bl.adj = L.badj.p;
    return Bl;
}

// One pass (forward or adjoint) over every group of <= 64 points; results[b * K + k].
pg_status run_lik(pg_ctx* c, int32_t batch, const double* theta, int adjoint, double* results) {
    LikState& L = c->lik;
    if (!adjoint) {
        L.fwd_exact_exp2 = L.exact_exp2;
        if (L.feat_exact != L.exact_exp2) {  // the rows follow the mode; the adjoint keeps the forward's
            cudaGetLastError();
            launch_lik_features(make_trace(c), L.exact_exp2, c->num_sms, c->stream);
            PG_CUDA(c, cudaGetLastError());
            L.feat_exact = L.exact_exp2;
        }
    }
    const int groups = (batch + kLikMaxB - 1) / kLikMaxB;
    const int K = adjoint ? 4 : 1;
    const int64_t zneed = (int64_t)groups * std::max<int64_t>(L.agents, 1) * kLikMaxB;
    if (L.theta.n < 4 * (int64_t)groups * kLikMaxB) PG_CUDA(c, dalloc(L.theta, 4 * (int64_t)groups * kLikMaxB));
    if (L.pp.n < 8 * (int64_t)groups * kLikMaxB) PG_CUDA(c, dalloc(L.pp, 8 * (int64_t)groups * kLikMaxB));
    if (L.zagent.n < zneed) {
        if (adjoint) return fail(c, PG_ERR_STATE, "run pg_loglik_fwd first");
        PG_CUDA(c, dalloc(L.zagent, zneed));
    }
    if (L.zglob.n < (int64_t)groups * L.epochs * kLikMaxB) {
        if (adjoint) return fail(c, PG_ERR_STATE, "run pg_loglik_fwd first");
        PG_CUDA(c, dalloc(L.zglob, (int64_t)groups * L.epochs * kLikMaxB));
    }
    if (L.gglob.n < (int64_t)L.epochs * kLikMaxB * 3) PG_CUDA(c, dalloc(L.gglob, (int64_t)L.epochs * kLikMaxB * 3));
    if (L.gpart.n < (int64_t)L.epochs * L.chunks * kLikMaxB * 4)
        PG_CUDA(c, dalloc(L.gpart, (int64_t)L.epochs * L.chunks * kLikMaxB * 4));
    if (L.out.n < std::max<int64_t>(1, L.agents) * kLikMaxB * 4)
        PG_CUDA(c, dalloc(L.out, std::max<int64_t>(1, L.agents) * kLikMaxB * 4));
    if (L.res.n < kLikMaxB * 4) PG_CUDA(c, dalloc(L.res, kLikMaxB * 4));
    // per point: alpha, 1/tau, gamma, beta, log beta, 1/beta, 1/tau^2, tau
    std::vector<double> pp((size_t)batch * 8);
    for (int b = 0; b < batch; ++b) {
        const double* t = theta + 4 * b;
        double* q = pp.data() + 8 * b;
        q[0] = t[0];
        q[1] = 1.0 / t[1];
        q[2] = t[2];
        q[3] = t[3];
        q[4] = log_pg(t[3]);
        q[5] = 1.0 / t[3];
        q[6] = 1.0 / (t[1] * t[1]);
        q[7] = t[1];
    }
    PG_CUDA(c, cudaMemcpyAsync(L.theta.p, theta, sizeof(double) * 4 * (size_t)batch, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemcpyAsync(L.pp.p, pp.data(), sizeof(double) * 8 * (size_t)batch, cudaMemcpyHostToDevice, c->stream));
    PG_CUDA(c, cudaMemsetAsync(L.err.p, 0, sizeof(uint32_t), c->stream));
    const LikTrace T = make_trace(c);
    if (c->timing) record_event(c->lev[0], c->stream);
    std::vector<double> h((size_t)kLikMaxB * 4);
    cudaGetLastError();
    for (int g = 0; g < groups; ++g) {
        LikBatch P{};
        P.B = std::min(kLikMaxB, batch - g * kLikMaxB);
        P.BE = 1;
        while (P.BE < P.B) P.BE <<= 1;
        P.BW = std::min(P.BE, 32);
        P.exact_exp2 = adjoint ? L.fwd_exact_exp2 : L.exact_exp2;
        P.theta = L.theta.p + 4 * (int64_t)g * kLikMaxB;
        P.pp = L.pp.p + 8 * (int64_t)g * kLikMaxB;
        P.zglob = L.zglob.p + (int64_t)g * L.epochs * kLikMaxB;
        P.gglob = L.gglob.p;
        P.gpart = L.gpart.p;
        P.zagent = L.zagent.p + (int64_t)g * L.agents * kLikMaxB;
        P.out = L.out.p;
        P.res = L.res.p;
        P.error = L.err.p;
        launch_lik_global(T, P, adjoint, c->stream);
        for (const auto& ch : L.ball_chunks) {
            const LikBalls Bl = make_balls(L, ch.first);
            if (!L.balls_cached) launch_lik_ball(T, Bl, 1, ch.first, ch.second, L.ball_grid, c->stream);
            launch_lik_eval(T, P, Bl, adjoint, ch.first, ch.second, L.eval_grid[adjoint], c->stream);
        }
        launch_lik_sum(T, P, adjoint, c->stream);
        PG_CUDA(c, cudaGetLastError());
        PG_CUDA(c, cudaMemcpyAsync(h.data(), L.res.p, sizeof(double) * (size_t)P.B * K, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
        std::memcpy(results + (int64_t)g * kLikMaxB * K, h.data(), sizeof(double) * (size_t)P.B * K);
    }
    if (c->timing) {
        record_event(c->lev[1], c->stream);
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
        (adjoint ? c->stats.lik_ms_bwd : c->stats.lik_ms_fwd) = ms_between(c->lev[0], c->lev[1]);
    }
    uint32_t err = 0;
    PG_CUDA(c, cudaMemcpy(&err, L.err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (err) return fail(c, PG_ERR_ARG, "a per-agent normaliser was not positive (weights underflow at this theta)");
    return PG_OK;
}

}  // namespace

pg_status pg_trace_load(pg_ctx* c, const pg_trace_desc* t) {
    if (!c) return PG_ERR_ARG;
    if (!t || !t->pub_epoch || !t->fitness || !t->epoch_nodes || !t->epoch_t || !t->cite_off)
        return fail(c, PG_ERR_ARG, "incomplete trace descriptor");
    const int64_t n = t->num_nodes;
    const int E = t->num_epochs;
    if (n <= 0 || n > (int64_t)INT32_MAX / 2 || E < 1) return fail(c, PG_ERR_ARG, "trace size out of range");
    if (t->num_anchors < 1 || t->num_anchors > PG_MAX_ANCHORS) return fail(c, PG_ERR_ARG, "num_anchors must be in [1, 4]");
    const int64_t n0 = t->epoch_nodes[0];
    if (n0 < 1 || t->epoch_nodes[E] != n) return fail(c, PG_ERR_ARG, "epoch_nodes must run from the seed size to num_nodes");
    for (int e = 0; e < E; ++e)
        if (t->epoch_nodes[e + 1] < t->epoch_nodes[e]) return fail(c, PG_ERR_ARG, "epoch_nodes must not decrease");
    const int64_t agents = n - n0;
    if (agents > 0 && (!t->anchors || !t->cites)) return fail(c, PG_ERR_ARG, "anchors and cites are required");
    if (t->num_seed_edges < 0 || (t->num_seed_edges > 0 && (!t->seed_src || !t->seed_dst)))
        return fail(c, PG_ERR_ARG, "bad seed edge arrays");
    for (int64_t i = 0; i < t->num_seed_edges; ++i)
        if (t->seed_src[i] < 0 || t->seed_src[i] >= n0 || t->seed_dst[i] < 0 || t->seed_dst[i] >= n0)
            return fail(c, PG_ERR_ARG, "seed edge " + std::to_string(i) + " leaves the seed");
    if (t->cite_off[0] != 0) return fail(c, PG_ERR_ARG, "cite_off[0] must be 0");
    std::vector<int32_t> aep((size_t)std::max<int64_t>(agents, 1));
    {
        int e = 0;
        for (int64_t a = 0; a < agents; ++a) {
            const int64_t v = n0 + a;
            while (t->epoch_nodes[e + 1] <= v) ++e;
            aep[(size_t)a] = e;
            const int64_t ne = t->epoch_nodes[e];
            const int64_t k = t->cite_off[a + 1] - t->cite_off[a];
            if (k < 0 || k > PG_MAX_OUT_DEGREE)
                return fail(c, PG_ERR_ARG, "agent " + std::to_string(a) + ": 0..256 citations");
            for (int64_t p = t->cite_off[a]; p < t->cite_off[a + 1]; ++p)
                if (t->cites[p] < 0 || t->cites[p] >= ne)
                    return fail(c, PG_ERR_ARG, "agent " + std::to_string(a) + " cites a node that did not exist yet");
            for (int i = 0; i < 4; ++i) {
                const int32_t x = t->anchors[a * 4 + i];
                if (x < -1 || x >= ne || (i < t->num_anchors && x < 0) || (i >= t->num_anchors && x != -1))
                    return fail(c, PG_ERR_ARG, "agent " + std::to_string(a) + ": bad anchor");
            }
        }
    }
    PG_CUDA(c, cudaSetDevice(c->device));
    // final graph = seed edges + every agent's citations (assembled on the device below)
    const int64_t mc = t->cite_off[agents];
    const int64_t ns = t->num_seed_edges;
    const int64_t m = ns + mc;
    LikState& L = c->lik;
    free_lik(L);
    L.n = n;
    L.n0 = n0;
    L.agents = agents;
    L.epochs = E;
    L.num_anchors = t->num_anchors;
    int64_t nmax = 1;
    for (int e = 0; e < E; ++e) nmax = std::max(nmax, t->epoch_nodes[e]);
    L.words = (int)std::min<int64_t>((nmax + 31) / 32, kLikMaxWords);
    L.words = (L.words + 3) / 4 * 4;
    L.chunks = (int)((nmax + kLikChunk - 1) / kLikChunk);
    pg_status s = PG_OK;
    if ((s = upload(c, L.epoch_nodes, t->epoch_nodes, (int64_t)E + 1)) != PG_OK) return s;
    if ((s = upload(c, L.epoch_t, t->epoch_t, (int64_t)E)) != PG_OK) return s;
    if ((s = upload(c, L.coff, t->cite_off, agents + 1)) != PG_OK) return s;
    if ((s = upload(c, L.cites, t->cites, mc)) != PG_OK) return s;
    // the final graph's forward and backward CSR, built on the device from the edge list: the seed
    // edges, then every agent's citations (rows ascending, duplicate edges collapsed)
    {
        PG_CUDA(c, dalloc(L.fo, n + 1));
        PG_CUDA(c, dalloc(L.fc, std::max<int64_t>(m, 1)));
        PG_CUDA(c, dalloc(L.bo, n + 1));
        PG_CUDA(c, dalloc(L.bc, std::max<int64_t>(m, 1)));
        DBuf<int32_t> t_src, t_dst, t_indeg;
        DBuf<int64_t> t_u;
        DBuf<uint32_t> t_err;
        DBuf<char> t_scratch;
        struct Temps {  // released on every path
            pg_ctx* c;
            DBuf<int32_t>*a, *b, *d;
            DBuf<int64_t>* u;
            DBuf<uint32_t>* e;
            DBuf<char>* s;
            ~Temps() {
                tfree(*a, c->device, c->stream);
                tfree(*b, c->device, c->stream);
                tfree(*d, c->device, c->stream);
                tfree(*u, c->device, c->stream);
                tfree(*e, c->device, c->stream);
                tfree(*s, c->device, c->stream);
            }
        } temps{c, &t_src, &t_dst, &t_indeg, &t_u, &t_err, &t_scratch};
        PG_CUDA(c, talloc(t_src, std::max<int64_t>(m, 1), c->device, c->stream));
        PG_CUDA(c, talloc(t_dst, std::max<int64_t>(m, 1), c->device, c->stream));
        PG_CUDA(c, talloc(t_indeg, n, c->device, c->stream));
        PG_CUDA(c, talloc(t_u, 1, c->device, c->stream));
        PG_CUDA(c, talloc(t_err, 1, c->device, c->stream));
        PG_CUDA(c, talloc(t_scratch, (int64_t)build_scratch_bytes(m, n), c->device, c->stream));
        PG_CUDA(c, cudaMemsetAsync(t_err.p, 0, sizeof(uint32_t), c->stream));
        if (ns) {
            PG_CUDA(c, cudaMemcpyAsync(t_src.p, t->seed_src, 4 * (size_t)ns, cudaMemcpyHostToDevice, c->stream));
            PG_CUDA(c, cudaMemcpyAsync(t_dst.p, t->seed_dst, 4 * (size_t)ns, cudaMemcpyHostToDevice, c->stream));
        }
        cudaGetLastError();
        launch_trace_edges(L.coff.p, L.cites.p, agents, n0, ns, t_src.p, t_dst.p, c->num_sms, c->stream);
        launch_build_csr(t_src.p, t_dst.p, m, n, t_scratch.p, L.fo.p, L.fc.p, L.bo.p, L.bc.p, t_indeg.p, t_u.p,
                         t_err.p, c->stream);
        PG_CUDA(c, cudaGetLastError());
        uint32_t berr = 0;
        PG_CUDA(c, cudaMemcpyAsync(&berr, t_err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (berr) return fail(c, PG_ERR_ARG, "trace edge endpoint out of range");
    }
    if ((s = upload(c, L.fit, t->fitness, n)) != PG_OK) return s;
    if ((s = upload(c, L.pub, t->pub_epoch, n)) != PG_OK) return s;
    if ((s = upload(c, L.anchors, t->anchors, 4 * std::max<int64_t>(agents, 1) * (agents > 0))) != PG_OK) return s;
    if ((s = upload(c, L.agent_epoch, aep.data(), agents)) != PG_OK) return s;
    PG_CUDA(c, dalloc(L.feat, (int64_t)E * n));
    PG_CUDA(c, dalloc(L.err, 1));
    int ball_sm = 1, eval_sm[2] = {1, 1};
    PG_CUDA(c, init_lik_kernels(L.words, &ball_sm, eval_sm));
    L.ball_grid = c->num_sms * ball_sm;
    L.eval_grid[0] = c->num_sms * eval_sm[0];
    L.eval_grid[1] = c->num_sms * eval_sm[1];
    cudaGetLastError();
    launch_lik_features(make_trace(c), L.exact_exp2, c->num_sms, c->stream);
    PG_CUDA(c, cudaGetLastError());
    L.feat_exact = L.exact_exp2;
    // balls: sizes first, then as many agents' balls per chunk as memory allows
    const int64_t na = std::max<int64_t>(agents, 1);
    PG_CUDA(c, dalloc(L.bcnt, na));
    PG_CUDA(c, dalloc(L.badj, na));
    PG_CUDA(c, dalloc(L.cflag, std::max<int64_t>(mc, 1)));
    // the count pass keeps every agent's bitmaps when they fit an eighth of free memory, so that
    // the emit pass reads them back instead of walking the rows a second time
    DBuf<uint32_t> bmap;
    struct BmapGuard {
        pg_ctx* c;
        DBuf<uint32_t>* b;
        ~BmapGuard() { tfree(*b, c->device, c->stream); }
    } bmap_guard{c, &bmap};
    const int64_t pass_ids = (int64_t)L.words * 32;
    const int64_t bstride = (nmax + pass_ids - 1) / pass_ids * L.words;
    {
        size_t free0 = 0, total0 = 0;
        PG_CUDA(c, cudaMemGetInfo(&free0, &total0));
        if ((double)std::max<int64_t>(agents, 1) * (double)bstride * 4.0 <= (double)free0 / 8.0 &&
            talloc(bmap, std::max<int64_t>(agents, 1) * bstride, c->device, c->stream) != cudaSuccess) {
            cudaGetLastError();  // no room after all: the emit pass walks the rows
            bmap.p = nullptr;
        }
    }
    LikBalls count_balls = make_balls(L, 0);
    count_balls.bmap = bmap.p;
    count_balls.bmap_stride = bstride;
    launch_lik_ball(make_trace(c), count_balls, 0, 0, agents, L.ball_grid, c->stream);
    PG_CUDA(c, cudaGetLastError());
    std::vector<int64_t> cnt((size_t)na, 0), adj((size_t)na, 0);
    if (agents > 0) {
        PG_CUDA(c, cudaMemcpyAsync(cnt.data(), L.bcnt.p, 8 * (size_t)agents, cudaMemcpyDeviceToHost, c->stream));
        PG_CUDA(c, cudaMemcpyAsync(adj.data(), L.badj.p, 8 * (size_t)agents, cudaMemcpyDeviceToHost, c->stream));
    }
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    L.hboff.assign((size_t)agents + 1, 0);
    int64_t biggest = 1;
    L.adj_entries = 0;
    for (int64_t a = 0; a < agents; ++a) {
        L.hboff[(size_t)a + 1] = L.hboff[(size_t)a] + cnt[(size_t)a];
        biggest = std::max(biggest, cnt[(size_t)a]);
        L.adj_entries += adj[(size_t)a];
    }
    L.ball_elems = L.hboff[(size_t)agents];
    L.citations = mc;
    if ((s = upload(c, L.boff, L.hboff.data(), agents + 1)) != PG_OK) return s;
    size_t free_b = 0, total_b = 0;
    PG_CUDA(c, cudaMemGetInfo(&free_b, &total_b));
    const int64_t budget = std::max<int64_t>(biggest, (int64_t)(free_b / 4) / 4);  // ids in a quarter of free memory
    int64_t a = 0;
    while (a < agents) {
        int64_t b = a;
        while (b < agents && L.hboff[(size_t)b + 1] - L.hboff[(size_t)a] <= budget &&
               (c->tune.lik_chunk_agents <= 0 || b - a < c->tune.lik_chunk_agents))
            ++b;
        if (b == a) b = a + 1;
        L.ball_chunks.emplace_back(a, b);
        a = b;
    }
    int64_t chunk_max = 1;
    for (const auto& ch : L.ball_chunks)
        chunk_max = std::max(chunk_max, L.hboff[(size_t)ch.second] - L.hboff[(size_t)ch.first]);
    PG_CUDA(c, dalloc(L.bids, chunk_max));
    L.balls_cached = L.ball_chunks.size() == 1;
    if (L.balls_cached) {
        LikBalls emit_balls = make_balls(L, 0);
        emit_balls.bmap = bmap.p;
        emit_balls.bmap_stride = bstride;
        launch_lik_ball(make_trace(c), emit_balls, 1, 0, agents, L.ball_grid, c->stream);
        PG_CUDA(c, cudaGetLastError());
    }
    PG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->stats.lik_ball_elems = L.ball_elems;
    c->stats.lik_adj_entries = L.adj_entries;
    c->stats.lik_citations = L.citations;
    L.loaded = true;
    return PG_OK;
}

pg_status pg_loglik_fwd(pg_ctx* c, int32_t batch, const double* theta, double* loglik) {
    if (!c) return PG_ERR_ARG;
    if (!c->lik.loaded) return fail(c, PG_ERR_STATE, "no trace loaded");
    if (!loglik) return fail(c, PG_ERR_ARG, "loglik is NULL");
    pg_status s = check_theta(c, batch, theta);
    if (s != PG_OK) return s;
    PG_CUDA(c, cudaSetDevice(c->device));
    c->lik.fwd_theta.clear();
    s = run_lik(c, batch, theta, 0, loglik);
    if (s == PG_OK) c->lik.fwd_theta.assign(theta, theta + 4 * (size_t)batch);
    return s;
}

pg_status pg_loglik_bwd(pg_ctx* c, int32_t batch, const double* theta, const double* dloglik,
                        double* grad) {
    if (!c) return PG_ERR_ARG;
    if (!c->lik.loaded) return fail(c, PG_ERR_STATE, "no trace loaded");
    if (!grad) return fail(c, PG_ERR_ARG, "grad is NULL");
    pg_status s = check_theta(c, batch, theta);
    if (s != PG_OK) return s;
    if (c->lik.fwd_theta.size() != 4 * (size_t)batch ||
        std::memcmp(c->lik.fwd_theta.data(), theta, sizeof(double) * 4 * (size_t)batch) != 0)
        return fail(c, PG_ERR_STATE, "pg_loglik_bwd needs the points of the last pg_loglik_fwd");
    PG_CUDA(c, cudaSetDevice(c->device));
    s = run_lik(c, batch, theta, 1, grad);
    if (s != PG_OK) return s;
    if (dloglik)
        for (int b = 0; b < batch; ++b)
            for (int k = 0; k < 4; ++k) grad[4 * b + k] *= dloglik[b];
    return PG_OK;
}
