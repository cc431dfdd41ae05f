// pg_er.cu -- Erdos-Renyi G(n,p) growth by geometric skips (stage d).
//
// The reference's ER model lives on a branch that is not in the tree; its behaviour is recorded in
// results/slurm-8634746.out:60-73: every new node links to each pre-epoch node independently with
// probability p (724,781 edges for 14,746 new x 491,532 existing x 1e-4).
//
// Work is O(edges): the gap to the next success is floor(log(u) / log(1-p)).  The id range of each
// new node is cut into 2^16-id chunks with their own Philox stream, so a (node, chunk) task is
// independent of how tasks are spread over threads; where a chunk expects several successes a
// group of lanes walks it, drawing consecutive gaps together.  A count pass, an exclusive scan and
// an emit pass that replays the same streams write the edges in (source, target) order with no
// sort.
// The skip is floor(log(u) / log(1 - p)) with the library's own fp64 log, so the edge list is
// bit-identical to the CPU oracle; an fp32 estimate with a proven error bound decides almost every
// skip and the FP64 expression runs only when an integer lies within that bound (er_skip).
#include "pg_engine.cuh"

namespace pg {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int64_t er_walk(const Arena& A, int64_t i, int64_t c, int64_t n,
                                           const ErSkip& K, int32_t* out, int64_t out_base,
                                           int32_t* col_out, int64_t col_base) {
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
        if (out) {
            out[out_base + cnt] = (int32_t)pos;
            col_out[col_base + cnt] = (int32_t)pos;
            A.e_rank[out_base + cnt] = atomicAdd(&A.inc[A.rep[0].nbase + pos], 1);
        }
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

__global__ void __launch_bounds__(256) k_er_count(Arena A, int64_t tasks, int64_t chunks,
                                                  ErSkip K, int64_t* cnt) {
    if (A.st->error) return;
    const int64_t n = A.rep[0].n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tasks;
         t += (int64_t)gridDim.x * blockDim.x)
        cnt[t] = er_walk(A, t / chunks, t % chunks, n, K, nullptr, 0, nullptr, 0);
}

__global__ void k_er_check(Arena A, const int64_t* toff, int64_t tasks) {
    if (A.st->error) return;
    const int64_t E = toff[tasks];
    const Replica& rp = A.rep[0];
    A.st->edges = E;
    if (E > A.edge_cap || rp.m + E > rp.m_cap) atomicOr(&A.st->error, kErrCapacity);
}

__global__ void __launch_bounds__(256) k_er_emit(Arena A, int64_t tasks, int64_t chunks,
                                                 ErSkip K, const int64_t* toff) {
    if (A.st->error) return;
    const Replica& rp = A.rep[0];
    const int64_t n = rp.n;
    int32_t* fcol = A.fwd_col + rp.ebase;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tasks;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / chunks, c = t % chunks;
        const int64_t e0 = toff[t];
        const int64_t cnt = er_walk(A, i, c, n, K, A.e_dst, e0, fcol, rp.m + e0);
        if (A.arrivals)
            for (int64_t q = 0; q < cnt; ++q) A.arrivals[e0 + q] = A.e_dst[e0 + q];
        if (c == chunks - 1) A.fwd_off[rp.obase + n + i + 1] = rp.m + e0 + cnt;
    }
}

// The same walk by a group of G lanes: the gaps of a task are independent draws, so the group
// draws G of them at once (lane l takes draw d0 + l), turns them into positions with a prefix sum
// of 1 + gap, keeps the prefix that lies below the chunk end and continues from its last position.
// The positions, their order and the draws consumed are those of er_walk.  Every lane of the warp
// stays in the loop until all of its groups are done (the shuffles span the warp).
template <int G>
__device__ __forceinline__ int64_t er_walk_group(const Arena& A, bool live, int64_t i, int64_t c, int64_t n,
                                                 const ErSkip& K, int32_t* out, int64_t out_base,
                                                 int32_t* col_out, int64_t col_base) {
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
        if (ok && out) {
            const int64_t e = out_base + cnt + gl;
            out[e] = (int32_t)q;
            col_out[col_base + cnt + gl] = (int32_t)q;
            A.e_rank[e] = atomicAdd(&A.inc[A.rep[0].nbase + q], 1);
            if (A.arrivals) A.arrivals[e] = (int32_t)q;
        }
        cnt += nok;
        pos = __shfl_sync(kFull, q, G - 1, G);
        if (nok < G) act = false;
    }
    return cnt;
}

template <int G>
__global__ void __launch_bounds__(256) k_er_count_g(Arena A, int64_t tasks, int64_t chunks, ErSkip K,
                                                    int64_t* cnt) {
    if (A.st->error) return;
    const int64_t n = A.rep[0].n;
    constexpr int per = 32 / G;  // tasks per warp and round
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = warp * per; b < tasks; b += nwarps * per) {
        const int64_t t = b + (lane_id() / G);
        const bool live = t < tasks;
        const int64_t tt = live ? t : 0;
        const int64_t c0 = er_walk_group<G>(A, live, tt / chunks, tt % chunks, n, K, nullptr, 0, nullptr, 0);
        if (live && (lane_id() & (G - 1)) == 0) cnt[t] = c0;
    }
}

template <int G>
__global__ void __launch_bounds__(256) k_er_emit_g(Arena A, int64_t tasks, int64_t chunks, ErSkip K,
                                                   const int64_t* toff) {
    if (A.st->error) return;
    const Replica& rp = A.rep[0];
    const int64_t n = rp.n;
    int32_t* fcol = A.fwd_col + rp.ebase;
    constexpr int per = 32 / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = warp * per; b < tasks; b += nwarps * per) {
        const int64_t t = b + (lane_id() / G);
        const bool live = t < tasks;
        const int64_t tt = live ? t : 0;
        const int64_t i = tt / chunks, c = tt % chunks;
        const int64_t e0 = toff[tt];
        const int64_t cnt = er_walk_group<G>(A, live, i, c, n, K, A.e_dst, e0, fcol, rp.m + e0);
        if (live && (lane_id() & (G - 1)) == 0 && c == chunks - 1) A.fwd_off[rp.obase + n + i + 1] = rp.m + e0 + cnt;
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

// Count, scan and emit; the caller then runs the backward append.
void launch_er_epoch(const Arena& A, int64_t delta, double p, int64_t n, int64_t* cnt,
                     int64_t* toff, int num_sms, cudaStream_t s) {
    const int64_t chunks = (n + kErChunk - 1) / kErChunk;
    const int64_t tasks = delta * chunks;
    k_er_setup<<<(unsigned)((delta + 255) / 256), 256, 0, s>>>(A, delta);
    if (!(p > 0.0)) {  // no edges: zero offsets keep the CSR append consistent
        cudaMemsetAsync(toff, 0, sizeof(int64_t) * (size_t)(tasks + 1), s);
        k_er_check<<<1, 32, 0, s>>>(A, toff, tasks);
        k_er_eoff<<<(unsigned)((delta + 256) / 256), 256, 0, s>>>(A, toff, delta, chunks);
        return;
    }
    const ErSkip K = er_skip_constants(p);
    // lanes per task: about the expected successes of a full chunk (1: one thread walks a task)
    const double mu = (double)(n < kErChunk ? n : kErChunk) * (p < 1.0 ? p : 1.0);
    int G = 1;
    while (G < 32 && G < mu) G <<= 1;
    int64_t g = (tasks * G + 255) / 256;
    if (g > (int64_t)num_sms * 32) g = (int64_t)num_sms * 32;
    if (g < 1) g = 1;
    switch (G) {
        case 1: k_er_count<<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
        case 2: k_er_count_g<2><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
        case 4: k_er_count_g<4><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
        case 8: k_er_count_g<8><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
        case 16: k_er_count_g<16><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
        default: k_er_count_g<32><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, cnt); break;
    }
    launch_scan_i64(cnt, toff, tasks, A.blocksum, s);
    k_er_check<<<1, 32, 0, s>>>(A, toff, tasks);
    switch (G) {
        case 1: k_er_emit<<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
        case 2: k_er_emit_g<2><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
        case 4: k_er_emit_g<4><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
        case 8: k_er_emit_g<8><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
        case 16: k_er_emit_g<16><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
        default: k_er_emit_g<32><<<(unsigned)g, 256, 0, s>>>(A, tasks, chunks, K, toff); break;
    }
    k_er_eoff<<<(unsigned)((delta + 256) / 256), 256, 0, s>>>(A, toff, delta, chunks);
}

}  // namespace pg
