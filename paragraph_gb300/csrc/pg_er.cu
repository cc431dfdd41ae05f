// pg_er.cu -- Erdos-Renyi G(n,p) growth by geometric skips (stage d).
//
// The reference's ER model lives on a branch that is not in the tree; its behaviour is recorded in
// results/slurm-8634746.out:60-73: every new node links to each pre-epoch node independently with
// probability p (724,781 edges for 14,746 new x 491,532 existing x 1e-4).
//
// Work is O(edges): the gap to the next success is floor(log(u) / log(1-p)).  The id range of each
// new node is cut into 2^16-id chunks with their own Philox stream, so a (node, chunk) task is
// independent of how tasks are spread over threads; where a chunk expects several successes a
// group of lanes walks it, drawing consecutive gaps together.  Every skip is walked once: each task
// owns a block of slots sized for its binomial count (mean + sigmas standard deviations + 8, laid
// out in closed form: all full chunks have the same size), the walk writes each success's position
// and in-degree rank there and counts exactly; a task with more successes than slots (with the
// default 8 sigmas, about never) is walked again by the overflow pass, which writes only its excess
// into an overflow area.  A scan of the counts and a compaction pass then write the edges in
// (source, target) order with no sort.
// The skip is floor(log(u) / log(1 - p)) with the library's own fp64 log, so the edge list is
// bit-identical to the CPU oracle; an fp32 estimate with a proven error bound decides almost every
// skip and the FP64 expression runs only when an integer lies within that bound (er_skip).
#include "pg_engine.cuh"

namespace pg {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int64_t er_slots_of(const ErPlan& P, int64_t c) { return c == P.chunks - 1 ? P.s_last : P.s_full; }
__device__ __forceinline__ int64_t er_base_of(const ErPlan& P, int64_t i, int64_t c) { return i * P.per_node + c * P.s_full; }

// One success of a task: its k-th edge at position pos, with its rank among the node's new entries.
// Edges k < S go to the task's slots (pass 1), the others to its overflow block (overflow pass).
__device__ __forceinline__ void er_put(const Arena& A, int64_t k, int64_t pos, int64_t S, int2* slots, int64_t sbase,
                                       int2* ov, int64_t obase) {
    if (slots && k < S)
        slots[sbase + k] = make_int2((int32_t)pos, atomicAdd(&A.inc[A.rep[0].nbase + pos], 1));
    else if (ov && k >= S)
        ov[obase + k - S] = make_int2((int32_t)pos, atomicAdd(&A.inc[A.rep[0].nbase + pos], 1));
}

// One thread walks task (i, c): returns its successes.
__device__ __forceinline__ int64_t er_walk(const Arena& A, int64_t i, int64_t c, int64_t n, const ErSkip& K,
                                           int64_t S, int2* slots, int64_t sbase, int2* ov, int64_t obase) {
    const int64_t lo = c * kErChunk;
    const int64_t hi = lo + kErChunk < n ? lo + kErChunk : n;
    int64_t pos = lo - 1, cnt = 0;
    const uint32_t ep = (uint32_t)A.st->epoch;
    u32x4 x;
    x.x[0] = x.x[1] = x.x[2] = x.x[3] = 0;
    for (uint32_t d = 0;; ++d) {
        if ((d & 1u) == 0) x = draw(A.seed, kStreamEr, (uint32_t)c, ep, (uint32_t)i, d >> 1);
        const double rem = (double)(hi - pos - 1);
        const double sk = (d & 1u) ? er_skip(K, x.x[2], x.x[3], (float)rem) : er_skip(K, x.x[0], x.x[1], (float)rem);
        if (sk >= rem) break;
        pos = pos + 1 + (int64_t)sk;
        er_put(A, cnt, pos, S, slots, sbase, ov, obase);
        ++cnt;
    }
    return cnt;
}

__global__ void __launch_bounds__(256) k_er_setup(Arena A, int64_t delta) {
    if (A.st->error) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= delta) return;
    const Replica& rp = A.rep[0];
    const int64_t slot = rp.nbase + rp.n + i;
    const uint32_t ep = (uint32_t)A.st->epoch;
    A.pub[slot] = (int32_t)A.st->epoch;
    A.fit[slot] = lognormal_fitness(A.seed, 0u, ep, (uint32_t)i);
    A.indeg[slot] = 0;
}

__global__ void __launch_bounds__(256) k_er_walk(Arena A, ErPlan P, ErSkip K, int64_t* cnt, int2* slots) {
    if (A.st->error) return;
    const int64_t n = A.rep[0].n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < P.tasks;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / P.chunks, c = t % P.chunks;
        cnt[t] = er_walk(A, i, c, n, K, er_slots_of(P, c), slots, er_base_of(P, i, c), nullptr, 0);
    }
}

__global__ void k_er_check(Arena A, const int64_t* toff, int64_t tasks) {
    if (A.st->error) return;
    const int64_t E = toff[tasks];
    const Replica& rp = A.rep[0];
    A.st->edges = E;
    if (E > A.edge_cap || rp.m + E > rp.m_cap) atomicOr(&A.st->error, kErrCapacity);
}

// The tasks with more successes than slots walk again (one thread each: they are rare) and write
// only their excess, into blocks of the overflow area reserved here.
__global__ void __launch_bounds__(256) k_er_overflow(Arena A, ErPlan P, ErSkip K, const int64_t* cnt, int2* ov,
                                                     int64_t ov_cap, int64_t* ovb) {
    if (A.st->error) return;
    const int64_t n = A.rep[0].n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < P.tasks;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t % P.chunks, S = er_slots_of(P, c);
        if (cnt[t] <= S) continue;
        const int64_t ob = (int64_t)atomicAdd(&A.st->er_ov_count, (unsigned long long)(cnt[t] - S));
        if (ob + cnt[t] - S > ov_cap) {
            atomicOr(&A.st->error, kErrCapacity);
            continue;
        }
        ovb[t] = ob;
        er_walk(A, t / P.chunks, c, n, K, S, nullptr, 0, ov, ob);
    }
}

// The same walk by a group of G lanes: the gaps of a task are independent draws, so the group
// draws G of them at once (lane l takes draw d0 + l), turns them into positions with a prefix sum
// of 1 + gap, keeps the prefix that lies below the chunk end and continues from its last position.
// The positions, their order and the draws consumed are those of er_walk.  Every lane of the warp
// stays in the loop until all of its groups are done (the shuffles span the warp).
template <int G>
__device__ __forceinline__ int64_t er_walk_group(const Arena& A, bool live, int64_t i, int64_t c, int64_t n,
                                                 const ErSkip& K, int64_t S, int2* slots, int64_t sbase) {
    const int lane = lane_id(), gl = lane & (G - 1);
    const unsigned gm = G == 32 ? kFull : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const int64_t lo = c * kErChunk;
    const int64_t hi = lo + kErChunk < n ? lo + kErChunk : n;
    const uint32_t ep = (uint32_t)A.st->epoch;
    int64_t pos = lo - 1, cnt = 0;
    bool act = live;
    for (uint32_t d0 = 0; __any_sync(kFull, act); d0 += G) {
        int64_t step = 0;
        if (act) {
            const uint32_t d = d0 + (uint32_t)gl;
            const u32x4 x = draw(A.seed, kStreamEr, (uint32_t)c, ep, (uint32_t)i, d >> 1);
            const double sk = (d & 1u) ? er_skip(K, x.x[2], x.x[3], (float)kErChunk)
                                       : er_skip(K, x.x[0], x.x[1], (float)kErChunk);
            step = sk < 1099511627776.0 ? (int64_t)sk + 1 : ((int64_t)1 << 40);  // 2^40: past any chunk
        }
        int64_t incl = step;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const int64_t y = __shfl_up_sync(kFull, incl, o, G);
            if (gl >= o) incl += y;
        }
        const int64_t q = pos + incl;
        const bool ok = act && q < hi;  // a prefix of the group: positions increase along it
        const int nok = __popc(__ballot_sync(kFull, ok) & gm);
        if (ok) er_put(A, cnt + gl, q, S, slots, sbase, nullptr, 0);
        cnt += nok;
        pos = __shfl_sync(kFull, q, G - 1, G);
        if (nok < G) act = false;
    }
    return cnt;
}

template <int G>
__global__ void __launch_bounds__(256) k_er_walk_g(Arena A, ErPlan P, ErSkip K, int64_t* cnt, int2* slots) {
    if (A.st->error) return;
    const int64_t n = A.rep[0].n;
    constexpr int per = 32 / G;  // tasks per warp and round
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = warp * per; b < P.tasks; b += nwarps * per) {
        const int64_t t = b + (lane_id() / G);
        const bool live = t < P.tasks;
        const int64_t tt = live ? t : 0;
        const int64_t i = tt / P.chunks, c = tt % P.chunks;
        const int64_t c0 = er_walk_group<G>(A, live, i, c, n, K, er_slots_of(P, c), slots, er_base_of(P, i, c));
        if (live && (lane_id() & (G - 1)) == 0) cnt[t] = c0;
    }
}

// The edges of every task at their place in the epoch's edge list and the new forward rows, G lanes
// per task (G = 1: one thread), from its slots and, past them, its overflow block.
template <int G>
__global__ void __launch_bounds__(256) k_er_place(Arena A, ErPlan P, const int64_t* cnt, const int64_t* toff,
                                                  const int2* slots, const int2* ov, const int64_t* ovb) {
    if (A.st->error) return;
    const Replica& rp = A.rep[0];
    const int64_t n = rp.n;
    int32_t* fcol = A.fwd_col + rp.ebase + rp.m;
    constexpr int per = 32 / G;
    const int gl = lane_id() & (G - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = warp * per; b < P.tasks; b += nwarps * per) {
        const int64_t t = b + (lane_id() / G);
        if (t >= P.tasks) continue;
        const int64_t i = t / P.chunks, c = t % P.chunks;
        const int64_t S = er_slots_of(P, c), sb = er_base_of(P, i, c), k1 = cnt[t], e0 = toff[t];
        const int64_t ob = k1 > S ? ovb[t] : 0;
        for (int64_t k = gl; k < k1; k += G) {
            const int2 v = k < S ? slots[sb + k] : ov[ob + k - S];
            const int64_t e = e0 + k;
            A.e_dst[e] = v.x;
            A.e_rank[e] = v.y;
            fcol[e] = v.x;
            if (A.arrivals) A.arrivals[e] = v.x;
        }
        if (gl == 0 && c == P.chunks - 1) A.fwd_off[rp.obase + n + i + 1] = rp.m + e0 + k1;
    }
}

__global__ void __launch_bounds__(256) k_er_eoff(Arena A, const int64_t* toff, int64_t delta,
                                                 int64_t chunks) {
    if (A.st->error) return;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= delta) A.eoff[i] = toff[i * chunks];
}

ErSkip er_skip_constants(double p) {
    ErSkip K;
    K.inv_l = 1.0 / log_pg(1.0 - (p < 1.0 ? p : 1.0));
    K.inv_f = (float)K.inv_l;
    const float a = (float)(fabs(K.inv_l) * 0x1p-23);
    K.dabs = nextafterf(a, INFINITY);  // rounded up
    return K;
}

ErPlan er_plan(int64_t n, int64_t delta, double p, int sigmas) {
    ErPlan P;
    P.n = n;
    P.chunks = n > 0 ? (n + kErChunk - 1) / kErChunk : 0;
    P.tasks = delta * P.chunks;
    const int sg = sigmas > 0 ? sigmas : 8;
    const double q = p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p);
    auto slots = [&](int64_t len) -> int64_t {
        const double mu = (double)len * q;
        const double sd = sqrt(mu * (1.0 - q));
        int64_t s = (int64_t)ceil(mu + sg * sd) + 8;
        return s < len ? s : len;
    };
    P.s_full = slots(kErChunk);
    P.s_last = P.chunks > 0 ? slots(n - (P.chunks - 1) * kErChunk) : 0;
    P.per_node = P.chunks > 0 ? (P.chunks - 1) * P.s_full + P.s_last : 0;
    return P;
}

// Walk (counts and slots), scan, overflow, placement; the caller then runs the backward append.
void launch_er_epoch(const Arena& A, int64_t delta, double p, const ErPlan& P, const ErBuffers& B, int num_sms,
                     cudaStream_t s) {
    k_er_setup<<<(unsigned)((delta + 255) / 256), 256, 0, s>>>(A, delta);
    if (!(p > 0.0) || P.tasks == 0) {  // no edges: zero offsets keep the CSR append consistent
        cudaMemsetAsync(B.toff, 0, sizeof(int64_t) * (size_t)(P.tasks + 1), s);
        k_er_check<<<1, 32, 0, s>>>(A, B.toff, P.tasks);
        k_er_eoff<<<(unsigned)((delta + 256) / 256), 256, 0, s>>>(A, B.toff, delta, P.chunks);
        return;
    }
    const ErSkip K = er_skip_constants(p);
    // lanes per task: about the expected successes of a full chunk (1: one thread walks a task)
    const double mu = (double)(P.n < kErChunk ? P.n : kErChunk) * (p < 1.0 ? p : 1.0);
    int G = 1;
    while (G < 32 && G < mu) G <<= 1;
    int64_t g = (P.tasks * G + 255) / 256;
    if (g > (int64_t)num_sms * 32) g = (int64_t)num_sms * 32;
    if (g < 1) g = 1;
    switch (G) {
        case 1: k_er_walk<<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
        case 2: k_er_walk_g<2><<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
        case 4: k_er_walk_g<4><<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
        case 8: k_er_walk_g<8><<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
        case 16: k_er_walk_g<16><<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
        default: k_er_walk_g<32><<<(unsigned)g, 256, 0, s>>>(A, P, K, B.cnt, B.slots); break;
    }
    launch_scan_i64(B.cnt, B.toff, P.tasks, A.blocksum, s);
    k_er_check<<<1, 32, 0, s>>>(A, B.toff, P.tasks);
    int64_t go = (P.tasks + 255) / 256;
    if (go > (int64_t)num_sms * 8) go = (int64_t)num_sms * 8;
    k_er_overflow<<<(unsigned)go, 256, 0, s>>>(A, P, K, B.cnt, B.ov, B.ov_cap, B.ovb);
    switch (G) {
        case 1: k_er_place<1><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
        case 2: k_er_place<2><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
        case 4: k_er_place<4><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
        case 8: k_er_place<8><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
        case 16: k_er_place<16><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
        default: k_er_place<32><<<(unsigned)g, 256, 0, s>>>(A, P, B.cnt, B.toff, B.slots, B.ov, B.ovb); break;
    }
    k_er_eoff<<<(unsigned)((delta + 256) / 256), 256, 0, s>>>(A, B.toff, delta, P.chunks);
}

}  // namespace pg
