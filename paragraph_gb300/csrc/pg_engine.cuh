// pg_engine.cuh -- device data layout and shared primitives of the growth engine.
//
// Layout in HBM (one arena per context, R replicas):
//   node slot arrays (pub, fitness, indeg, w, cdf, inc) are indexed nbase_r + v, v < n_cap_r; every
//   nbase_r is a multiple of kTile so a scan tile never spans two replicas;
//   forward offsets (fwd_off) hold n_cap_r + 1 int64 entries at obase_r = nbase_r + r and are LOCAL
//   to the replica's edge region; forward columns (fwd_col) hold replica-local int32 node ids at
//   ebase_r + offset (rows appended in node order, never moved);
//   backward rows (brow, one 8-byte BRow per node slot, and bcap, the room of each) point into the
//   replica's backward region (bcol at bbase_r, b_cap_r entries): a row holds `len` entries from
//   its 16-byte-aligned start and grows in place until its room is full, when it moves to twice
//   its length at the region's bump pointer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_core.cuh"

namespace pg {

constexpr int kTile = 1024;          // slots per scan tile
constexpr int kTileThreads = 256;    // threads per tile CTA (4 slots each)
constexpr int kKSmall = 64;          // agents with k <= 64 use the small-capacity path
constexpr int kKMax = 256;           // PG_MAX_OUT_DEGREE
constexpr int kRcMaxOutDegree = 250; // refcompat: the reference's per-paper citation capacity (src/kernel.cu:1151)
constexpr int kTableEntries = kKMax + 1;
constexpr int kAgentWarps = 4;       // warps per CTA in the agent kernel
constexpr int kErChunk = 65536;      // ids per ER Philox stream
constexpr int kSortMid = 256;        // appended segments up to this length sort in one warp's registers
constexpr int kBitmapWords = 40960;  // 160 KiB of shared bitmap in the large-segment sort
#define PG_MAX_ANCHORS_DEV 4
constexpr int kRcBigGd = 32;         // refcompat generators with this many row entries: a CTA per 2-hop stream
constexpr int kRcBigStream = 1024;  // ... or a 2-hop stream (the rows of the generator's rows) this long
constexpr int kRcBigCap = 16384;     // such agents per epoch (the rest keep the one-warp path)
constexpr int kGBits = 13;           // per-warp global hash for anchor rows too large for shared memory
constexpr int kZCap = 1024;          // 1-hop frontier entries kept in shared memory per warp
constexpr int kRelocChunk = 4096;    // backward entries per copy task of a moved row
constexpr int kHeavyMax = 256;       // hubs per replica with a bit in the per-node hub mask
constexpr int kMaskWords = kHeavyMax / 64;
constexpr int kHeavyMinLog = 10;     // only nodes with degree >= 2^10 can be hubs
constexpr int kHeavyBins = 24;       // log2-degree histogram bins 10..33
constexpr int kRcAgeMax = 1024;      // recency probabilities by age 0..1023 (refcompat)
constexpr int kRcFitMax = 1000;      // peak fitness values 1..1000 (refcompat)
constexpr uint32_t kRcFillBlocks = 1u << 20;  // Philox blocks a uniform fill may use
constexpr uint32_t kWaitPolls = 1u << 22;     // polls of a bounded wait on an asynchronous copy

enum Sampler : int32_t {
    kSamplerThinning = 0,   // Poisson thinning against ball membership (default)
    kSamplerEnumerate = 1,  // stream the whole 2-hop ball and key every element
};

// Device error word bits.
enum : uint32_t {
    kErrCapacity = 1u,
    kErrBadWeight = 2u,
    kErrArg = 4u,
    kErrTimeout = 8u,  // a bounded wait on an asynchronous copy ran out
};

// Backward row of a node: entries bcol[bbase + 4 beg4, bbase + 4 beg4 + len), so every row starts on
// a 16-byte boundary; its room (a multiple of 4 entries, 0 for an empty row) is kept apart in bcap,
// which only the append reads, so the record the samplers load per node is 8 bytes.
//
// A node's span in the region, once the node has been cited (len > 0):
//   [ pad | forward row copy (o entries) | backward entries (len) | room ]
//   ^ span start (16-byte aligned)        ^ 4 beg4 (16-byte aligned)
// where o is the node's out-degree and pad + o = fwd_prefix(o).  The copy makes the node's
// forward and backward rows one contiguous window, so the thinning sampler stages a tested
// candidate with one bulk copy instead of two.  A node never cited has no span (len = 0, beg4 = 0,
// room 0): its forward row is read from the forward CSR.
struct __align__(8) BRow {
    uint32_t beg4;
    int32_t len;
};
constexpr int64_t kBRegionMax = (int64_t)1 << 34;  // entries a backward region may span (beg4 is 32-bit)

// Room given to a backward row that must hold L >= 1 entries: 2L rounded up to a multiple of 4.
PG_HD int64_t brow_cap(int64_t L) { return (2 * L + 3) & ~3ll; }
// Entries before 4 beg4 that hold the forward row copy of a node of out-degree o.
PG_HD int64_t fwd_prefix(int64_t o) { return (o + 3) & ~3ll; }
// Span of a cited row of L >= 1 backward entries and prefix P: brow_cap(L + P); its room (entries
// from 4 beg4) is the span minus P, at least 2 L + P.  A row that outgrows its room moves to a new
// span, so the totals T_k = L_k + P of its spans c_k = brow_cap(T_k) satisfy
// c_k < T_(k+1) <= c_(k+1) / 2: together the spans take less than 2 c_K <= 4 (L + P) + 6 entries (L
// the final length).  Over all rows (sum of L <= m, sum of P <= m + 3 n) a region of 8 m + 18 n + 4
// entries never runs out; each entry moves O(1) times amortised.
PG_HD int64_t brow_span(int64_t L, int64_t P) { return brow_cap(L + P); }
PG_HD int64_t bregion_entries(int64_t n_cap, int64_t m_cap) { return 8 * m_cap + 18 * n_cap + 4; }

struct Replica {
    // static layout
    int64_t nbase, obase, ebase;
    int64_t n_cap, m_cap;
    int64_t bbase, b_cap;           // backward region: first entry and size
    unsigned long long b_top;       // backward region: entries handed out (bump pointer)
    // state
    int64_t n, m;
    // this epoch
    int64_t delta;
    int64_t abase;      // first agent (global agent index) of this replica
    int64_t npos;       // nodes with positive weight
    uint64_t wq_total;  // quantised total weight
    uint32_t wmax_bits;
    int32_t shift;
    int32_t tbase;      // first slot tile of the replica
    int32_t ntiles;     // slot tiles of the replica (n_cap / kTile)
    // parameters
    float alpha, gamma, tau, pad0;
    double beta_m1;
    double p_global;  // 1 / beta: probability that a thinning event is a global (always kept) one
    uint64_t glob_thr;  // u01d(lo, hi) <= p_global  <=>  (hi:lo >> 11) + 1 <= glob_thr (global_threshold)
    double growth_rate;
    int64_t fixed_new;
    int32_t anchors;
    // hub index of the epoch: nodes with degree >= heavy_thr get one of <= kHeavyMax mask bits; the
    // bits and masks carry over from epoch to epoch while hub_valid (cleared by a load or restore)
    int32_t heavy_thr;
    int32_t heavy_count;  // highest bit in use + 1
    int32_t hub_valid;
    int32_t hub_full;     // this epoch rebuilds the index from scratch
    int32_t hub_nadd;     // nodes that become hubs this epoch
    int32_t hub_pad;
    int32_t heavy_hist[kHeavyBins];
    // refcompat functor (weight model PG_WEIGHTS_REFCOMPAT)
    double rc_w[3];   // pa, rec, fit weights, normalised; rc_w[0] < 0: drawn per agent
    double rc_alpha;  // share of the neighbourhood budget from the 1-hop set; < 0: per agent
    double rc_frc;    // fraction of the out-degree reserved for uniform citations
    double rc_sy;     // fraction of agents citing a paper of their own epoch
    double rc_dpa, rc_dfit, rc_U;  // this epoch: score normalisers and the recency denominator
    int32_t rc_gamma, rc_decay, rc_rec_len, rc_pad;
};

// Per-epoch device scalars; reset by the epoch-begin kernel.
struct EpochState {
    int64_t epoch;
    int64_t agents;       // total agents this epoch
    int64_t edges;        // total new edges this epoch
    uint32_t error;
    uint32_t pad;
    unsigned long long queue_small;
    unsigned long long queue_big;
    unsigned long long big_count;
    unsigned long long heavy_count;  // agents the small thinning kernel takes first
    unsigned long long rc_big_count, rc_big_queue;  // refcompat agents with a CTA-wide 2-hop pass
    unsigned long long sort_small_count;
    unsigned long long sort_large_count;
    unsigned long long sort_scratch;
    // counters of the byte model
    unsigned long long rows_expanded;
    unsigned long long elems_streamed;
    unsigned long long draws;
    unsigned long long bwd_moved;
    unsigned long long nodes_weighted;
    unsigned long long reloc_count; // copy tasks of the backward rows that moved this epoch
    unsigned long long er_ov_count; // ER: overflow-area entries taken this epoch
    unsigned long long adj_scanned; // adjacency entries examined by membership tests
    // run totals, accumulated by the epoch-end kernel and cleared by the host at run start
    unsigned long long cum_rows_expanded;
    unsigned long long cum_elems_streamed;
    unsigned long long cum_draws;
    unsigned long long cum_bwd_moved;
    unsigned long long cum_nodes_weighted;
    unsigned long long cum_edges;
    unsigned long long cum_new_nodes;
    unsigned long long cum_epochs;
    unsigned long long cum_adj_scanned;
    unsigned long long out_count;   // citations streamed to the run's output buffers so far
    unsigned long long out_short;   // citations that did not fit them (the run goes on; nothing is written past them)
    // grid barrier of the persistent epoch kernel: arrivals (back to 0 after every barrier, reset
    // by the host before each launch) and generation
    unsigned int gbar_count;
    unsigned int gbar_gen;
};

// Device pointers of the arena (passed by value to kernels).
struct Arena {
    Replica* rep;
    int32_t R;
    int32_t ntiles;            // total slot tiles
    const int32_t* tile_rep;   // [ntiles]
    int32_t* pub;
    float* fit;
    int32_t* indeg;
    float* w;
    uint64_t* cdf;
    int32_t* guide;            // [slots] guide table of the CDF (thinning sampler)
    int32_t* inc;
    int64_t* fwd_off;
    int32_t* fwd_col;
    BRow* brow;                // [slots] backward row of each node
    int32_t* bcap;             // [slots] room of each backward row (entries)
    int32_t* bcol;             // backward regions of all replicas
    const uint64_t* tables;    // [R][kTableEntries]
    // per-epoch buffers
    int32_t* kk;               // [agent cap] out-degree per agent
    int64_t* eoff;             // [agent cap + 1] edge offsets
    int32_t* e_dst;            // [edge cap]
    int32_t* e_rank;           // [edge cap]
    int32_t* arrivals;         // [edge cap] or null
    int32_t* anchors_out;      // [agent cap][4] anchors of each agent, or null (record_trace)
    int32_t* big_list;         // [agent cap]
    int32_t* heavy_list;       // [agent cap] agents with a hub or a large frontier (k <= kKSmall)
    int32_t* heavy_mark;       // [agent cap] 1 when the agent is on heavy_list
    int32_t* zbig;             // [agent-kernel warp slots][1 << kGBits] rows of anchors too large for H
    int32_t* rc_big_id;        // [kRcBigCap][kKMax] sorted top of each listed refcompat agent's 2-hop stream
    long long* rc_big_meta;    // [kRcBigCap][3] entries, rows, elements of that stream
    longlong2* reloc;          // [reloc_cap] moved-row copy tasks: (source, destination << 16 | length)
    int64_t reloc_cap;
    int64_t* new_start;        // [slots] where a row's new entries of the epoch start
    uint64_t* tilesum;         // [ntiles]
    uint64_t* tileoff;         // [ntiles]
    int64_t* blocksum;         // [scan blocks]
    int64_t* sort_small;       // [slots] packed (slot << 9 | new entries)
    int64_t* sort_large;       // [slots] slot
    int64_t* sort_large_off;   // [slots] packed (scratch offset << 32 | new entries)
    int16_t* hslot;            // [slots] hub bit of the node or -1
    uint64_t* hmask;           // [slots][kMaskWords] bit b set when hub b is adjacent to the node
    uint64_t* hub2;            // [R][kHeavyMax][kMaskWords] hubs sharing a neighbour with hub b
    uint32_t* hub_need;        // [R][kHeavyMax / 32] hubs some agent of the epoch has as anchor
    int32_t* hlist;            // [R][kHeavyMax] hub node of each bit, -1 when the bit is free
    int32_t* hub_rem;          // [R][kHeavyMax] node leaving bit b this epoch, or -1
    int32_t* hub_add;          // [R][kHeavyMax] node taking bit b this epoch, or -1
    int32_t* hub_cand;         // [R][kHeavyMax] nodes that become hubs this epoch
    // refcompat functor (null unless the context uses PG_WEIGHTS_REFCOMPAT)
    double* rc_pa;             // [slots] score components of the epoch
    double* rc_rec;
    double* rc_fit;
    int32_t* rc_lag;           // [slots] fitness window: lag and peak duration (peak = fit)
    int32_t* rc_dur;
    const double* rc_rtab;     // [R][kRcAgeMax] recency probability by age
    const uint64_t* rc_ftab;   // [kRcFitMax] peak-fitness CDF thresholds (2^64 scale)
    unsigned long long* rc_acc;  // [R][4] 128-bit sums of the pa and fit numerators (lo, hi)
    int32_t* rc_cnt;           // [R][kRcAgeMax] nodes per age
    double* rc_agent;          // [agent cap][6] pa, rec, fit weights, alpha, generator, out-degree
    int32_t weight_model;      // PG_WEIGHTS_*
    int32_t pad_wm;
    EpochState* st;
    int64_t agent_cap, edge_cap;
    uint64_t seed;
    int32_t record_trace;
    int32_t sampler;
    // launch tuning (results do not depend on it)
    int32_t tune_agent_ctas;   // agent-kernel CTAs per SM, 0 = occupancy limit
    int32_t tune_small_hash;   // 1: 1024-slot frontier hash in the k <= 64 kernel, 0: 2048
    int32_t tune_copy_ctas;    // moved-row copy CTAs per SM
    int32_t rep_base;          // RNG replica index of replica 0 (pg_config.replica_base)
    uint32_t first_wait_polls; // polls of the first bounded wait on each staged copy (pg_set_wait_limit)
    uint32_t pad_wp;
    // citation output of a run (pg_run_epochs_out), null otherwise: every epoch's new citations,
    // (source, target) replica by replica, written from the device at out_count; per-epoch,
    // per-replica counts at out_counts[epoch of the run * R + r]
    int32_t* out_src;
    int32_t* out_dst;
    int64_t out_cap;
    int64_t* out_counts;
    int64_t out_epochs;
};

// u01d(lo, hi) <= p compared in integers: u = (v + 1) 2^-53 with v the draw's top 53 bits, and
// p 2^53 is exact in double, so u <= p  <=>  v + 1 <= floor(p 2^53) (every draw for p >= 1).
PG_HD uint64_t global_threshold(double p) { return p >= 1.0 ? (1ull << 53) : (p > 0.0 ? (uint64_t)(p * 0x1p53) : 0ull); }
PG_HD bool u01d_at_most(uint32_t lo, uint32_t hi, uint64_t thr) { return (u64of(lo, hi) >> 11) + 1u <= thr; }

// Guide table of a replica's CDF (total Wq over n nodes): bucket g covers [g 2^gs, (g+1) 2^gs),
// with gs the smallest shift that leaves at most n buckets, so there are more than n/2 of them and
// a draw's answer lies between two adjacent guide entries a few CDF entries apart on average.
PG_HD int bitlen_u64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return x ? 64 - __clzll((long long)x) : 0;
#else
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
#endif
}
PG_HD int guide_shift(uint64_t Wq, int64_t n) {
    if (Wq <= 1) return 0;
    const uint64_t top = Wq - 1, lim = (uint64_t)(n > 1 ? n - 1 : 0);
    const int bt = bitlen_u64(top), bl = bitlen_u64(lim);
    int s = bt > bl ? bt - bl : 0;
    if ((top >> s) > lim) ++s;
    return s;
}

// ---------------------------------------------------------------- warp helpers
#if defined(__CUDACC__)
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Bounds [b, e) of backward row x (one 8-byte load), relative to the replica's region.
__device__ __forceinline__ void bspan(const BRow* br, int64_t x, int64_t& b, int64_t& e) {
    const uint2 q = *reinterpret_cast<const uint2*>(br + x);
    b = (int64_t)q.x << 2;
    e = b + (int64_t)(int32_t)q.y;
}
__device__ __forceinline__ int64_t blen(const BRow* br, int64_t x) { return br[x].len; }

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    const int l = lane_id();
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T o = __shfl_up_sync(0xffffffffu, v, d);
        if (l >= d) v += o;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// Bitonic network over R registers per lane: element i of lane l has index 32 i + l; partners
// 32 or more apart sit in the same lane (register compare), nearer ones in another lane (shuffle).
template <int R>
__device__ __forceinline__ void warp_bitonic(int (&v)[R], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    const int ip = i ^ (j >> 5);
                    if (ip > i) {
                        const bool up = ((i * 32 + lane) & k) == 0;
                        const int a = v[i], b = v[ip];
                        const bool sw = (a > b) == up;
                        v[i] = sw ? b : a;
                        v[ip] = sw ? a : b;
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    const int o = __shfl_xor_sync(0xffffffffu, v[i], j);
                    const bool up = ((i * 32 + lane) & k) == 0;
                    const bool lower = (lane & j) == 0;
                    v[i] = (lower == up) ? min(v[i], o) : max(v[i], o);
                }
            }
        }
    }
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024, multiple of 32).
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* smem_warp, T* total) {
    const int l = lane_id(), wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T incl = warp_incl_scan(v);
    if (l == 31) smem_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        T x = l < nw ? smem_warp[l] : T(0);
        T xi = warp_incl_scan(x);
        if (l < nw) smem_warp[l] = xi - x;
        if (l == nw - 1) smem_warp[32] = xi;
    }
    __syncthreads();
    T out = smem_warp[wid] + incl - v;
    if (total) *total = smem_warp[32];
    __syncthreads();
    return out;
}

// Geometric skip of one ER draw, floor(log_pg(u) * inv_l) exactly, u = u01d(lo, hi), inv_l =
// 1 / log(1 - p) <= 0.  An fp32 estimate y = logf_pg(u) * inv_l decides it unless an integer lies
// within its error bound: |y - y64| <= |inv_l| 2^-24 (u rounded to fp32 moves log u by at most
// 2^-24) + |y| 3 2^-23 (logf_pg is within 2 ulp on [2^-60, 1] -- checked there exhaustively --
// plus the fp32 roundings of inv_l and of the product) + |y64| 2^-50 (the FP64 expression's own
// error).  The bound used, d = |inv_l| 2^-23 + |y| 2^-20, is at least twice that and also covers
// the roundings of y - d and y + d.  Only when floor(y - d) != floor(y + d) is the FP64 expression
// evaluated (for about 2 d of the draws: under 0.3 % at p = 1e-3); a skip known to reach `cap` (the
// chunk's remaining length) ends the walk whatever its exact value.  GB300's FP64 rate is a small
// fraction of its FP32 rate, so the fp32 estimate is what makes the walk cheap.
struct ErSkip {
    double inv_l;  // 1 / log(1 - p)
    float inv_f;   // inv_l rounded to fp32
    float dabs;    // |inv_l| 2^-23, rounded up
};
__device__ __forceinline__ double er_skip(const ErSkip& K, uint32_t lo, uint32_t hi, float cap) {
    const double u = u01d(lo, hi);
    const float y = logf_pg((float)u) * K.inv_f;
    const float d = __fmaf_rn(y, 0x1p-20f, K.dabs);
    const float a = floorf(y - d);
    if (a >= cap || a == floorf(y + d)) return (double)a;
    return floor(log_pg(u) * K.inv_l);
}

// The device error word as one value for the whole CTA (a barrier and an OR of every thread's
// read): a body that synchronises its CTA must not let some threads return on an error bit another
// CTA set a moment later while the rest go on to a barrier.
__device__ __forceinline__ bool cta_error(const Arena& A) { return __syncthreads_or(A.st->error != 0u) != 0; }

// Replica of a global agent index: largest r with abase_r <= a.
__device__ __forceinline__ int replica_of_agent(const Replica* rep, int R, int64_t a) {
    int lo = 0, hi = R - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rep[mid].abase <= a)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}
#endif

// ---------------------------------------------------------------- host launchers
// Kernels one PA epoch enqueues: epoch begin (1), weights + CDF (4), agent setup + offset scan +
// check (5), agent kernels (2), backward append incl. epoch end (6: grow, moved-row copy, place,
// two sorts, end).
constexpr int kPaEpochKernels = 18;
// Extra kernels of the thinning sampler: the CDF's guide table (1) and the hub index (histogram,
// pick, collect, bit assignment, mask clears, mask sets, hub pairs).
constexpr int kThinKernels = 8;
void launch_epoch_begin(const Arena& A, int64_t epoch, int pa_mode, cudaStream_t s);
void launch_epoch_begin_delta(const Arena& A, int64_t epoch, int64_t delta, cudaStream_t s);
void launch_weights(const Arena& A, cudaStream_t s);
void launch_hubs(const Arena& A, int num_sms, cudaStream_t s);
void launch_hub_pairs(const Arena& A, cudaStream_t s);
void launch_guide(const Arena& A, cudaStream_t s);
void launch_agent_setup(const Arena& A, int64_t agents, cudaStream_t s);
void launch_agents(const Arena& A, int64_t agents, int num_sms, cudaStream_t s);
// The whole thinning PA epoch (baseline weights) as one cooperative persistent kernel: every stage
// above as a phase, grid barriers between dependent phases.  epoch_kernel_ctas() is its grid (0
// when the device cannot run it); launch_epoch_kernel returns the launch's error.
cudaError_t init_epoch_kernel(int num_sms);
int epoch_kernel_ctas();
cudaError_t launch_epoch_kernel(const Arena& A, int64_t epoch, int64_t agents, cudaStream_t s);
// side/fork/join (optional): the old-entry copy runs on `side` beside the new-entry placement and sorts
void launch_bwd_append(const Arena& A, int64_t agents, int num_sms, cudaStream_t s, cudaStream_t side = nullptr,
                       cudaEvent_t fork = nullptr, cudaEvent_t join = nullptr);
// refcompat functor: score components of the epoch (4 kernels) and the agent kernel
constexpr int kRcScoreKernels = 4;
void launch_rc_scores(const Arena& A, cudaStream_t s);
void launch_rc_big(const Arena& A, int num_sms, cudaStream_t s);
void launch_rc_agents(const Arena& A, int64_t agents, int num_sms, cudaStream_t s);
cudaError_t init_rc_kernels();
// ER epoch plan: tasks are (new node, 2^16-id chunk) pairs over n existing nodes; each task owns
// s_full slots (s_last for the last chunk), laid out per_node apart
struct ErPlan {
    int64_t n, chunks, tasks;
    int64_t s_full, s_last, per_node;
};
ErPlan er_plan(int64_t n, int64_t delta, double p, int sigmas);
struct ErBuffers {
    int64_t* cnt;    // [tasks + 1] successes per task
    int64_t* toff;   // [tasks + 1] their exclusive scan
    int2* slots;     // [delta * per_node] (position, rank) of each task's first successes
    int2* ov;        // [ov_cap] the excess of the tasks that overflowed
    int64_t ov_cap;
    int64_t* ovb;    // [tasks] start of a task's overflow block
};
void launch_er_epoch(const Arena& A, int64_t delta, double p, const ErPlan& P, const ErBuffers& B, int num_sms,
                     cudaStream_t s);
// the skip constants of probability p (host)
ErSkip er_skip_constants(double p);
// generic exclusive scan of n values; out has n+1 entries (out[n] = total)
void launch_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* blocksum, cudaStream_t s);
void launch_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* blocksum,
                            cudaStream_t s);
int scan_blocks_needed(int64_t n);
cudaError_t init_agent_kernels();
// the edge list as text on the device (pg_text.cu)
void launch_text_len(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m, const int64_t* ids, int32_t* len,
                     int num_sms, cudaStream_t s);
void launch_text_write(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m, const int64_t* ids,
                       const int64_t* off, char* out, int num_sms, cudaStream_t s);
// the attribute file as text on the device (pg_text.cu); out == nullptr: line lengths into len
struct AttrCols {  // columns of the attribute file (device pointers)
    int64_t n, n_seed;
    const int64_t* ids;     // [n]
    const double* draws;    // [n][4] pa, rec, fit weight, alpha
    const int32_t* ints;    // [n][4] lag, duration, assigned out-degree, planted line
    const int64_t* gens;    // [n][4] generator ids, -1 unused
    const int32_t* pub;
    const float* fit;
    const int32_t* indeg;
    const int64_t* fo;      // forward offsets: the out-degree of v is fo[v + 1] - fo[v]
    int32_t peak_int;
};
void launch_attr_text(const AttrCols& C, int32_t* len, const int64_t* off, char* out, int num_sms,
                      cudaStream_t s);
// the source of every edge in [first, first + count) of a forward CSR, from its offsets
void launch_edge_sources(const int64_t* fo, int64_t n, int64_t first, int64_t count, int32_t* out,
                         int num_sms, cudaStream_t s);
// device CSR construction from a raw edge list (pg_build.cu)
void launch_first_bad_edge(const int32_t* src, const int32_t* dst, int64_t m, int64_t n, unsigned long long* first,
                           cudaStream_t s);
// R edge lists gathered into the staging arrays src/dst and checked in one launch (list r at
// [off[r], off[r + 1]), m = off[R], ids below nodes[r], read from ptr[2 r] / ptr[2 r + 1]: mapped
// page-locked host memory or the staging arrays; off, nodes and ptr in device memory); first[r]
// relative to off[r]
void launch_gather_edges(int64_t m, const int64_t* off, const int64_t* nodes, const int64_t* ptr, int R, int32_t* src,
                         int32_t* dst, unsigned long long* first, cudaStream_t s);
size_t build_scratch_bytes(int64_t m, int64_t n);
// fsrc / btgt (may be null): the source of every unique forward edge, the target of every backward
// entry (m entries each)
void launch_build_csr(const int32_t* src, const int32_t* dst, int64_t m, int64_t n, void* scratch,
                      int64_t* fo, int32_t* fc, int64_t* bo, int32_t* bc, int32_t* indeg, int64_t* u_dev,
                      uint32_t* err, cudaStream_t s, int32_t* fsrc = nullptr, int32_t* btgt = nullptr);
// growable backward rows from an offset-form backward CSR (pg_build.cu), with the forward row copies
// in front of them (fo/fc: the replica's forward CSR): caps n, begs n + 1 (begs[n] = entries laid
// out), blocksum scan_blocks_needed(n) + 2 entries of scratch; brow/bcol: the replica's rows and
// region
// (fsrc / btgt, when not null: every forward entry's and backward entry's row, from launch_build_csr)
void launch_brow_layout(const int64_t* bo, const int32_t* bc, const int64_t* fo, const int32_t* fc, int64_t n,
                        int64_t m, int64_t* caps, int64_t* begs, int64_t* blocksum, BRow* brow, int32_t* bcap,
                        int32_t* bcol, cudaStream_t s, const int32_t* fsrc = nullptr, const int32_t* btgt = nullptr);
// the seeds of all replicas as one build over the arena's node slots (pg_build.cu): raw edges
// src/dst (replica r's at [raw_off[r], raw_off[r+1]), rewritten in place to slot ids), the device
// Replica array and tile map already uploaded; u/laid receive each replica's unique edges and
// backward entries laid out
size_t build_all_scratch_bytes(int64_t m, int64_t S);
void launch_build_all(int32_t* src, int32_t* dst, int64_t m, const int64_t* raw_off, int R, int64_t S,
                      const int32_t* tile_rep, const Replica* rep, void* scratch, int64_t* fwd_off, int32_t* fwd_col,
                      BRow* brow, int32_t* bcap, int32_t* bcol, int32_t* indeg, int64_t* u, int64_t* laid, uint32_t* err,
                      cudaStream_t s);
// resident CTAs per SM of the k <= 64 agent kernel (after init_agent_kernels)
int agent_occupancy(int thin, int small_hash);
int64_t agent_warp_slots(int num_sms);
cudaError_t init_csr_kernels();

}  // namespace pg
