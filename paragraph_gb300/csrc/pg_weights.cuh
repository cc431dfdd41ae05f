// pg_weights.cuh -- epoch start, per-node weights and the segmented fixed-point CDF.
//
// Restates the per-epoch score preparation of execute() (src/kernel.cu:1698-1706;
// FillInDegreeArr/FillFitnessArr/FillRecencyArr/CalculateScores, src/abm.cu:112-208,324-338),
// which the reference runs on the host every epoch, with the baseline weight functor
//   w_j = exp(gamma log f_j + alpha log(indeg_j + 1) - (t - t_j) / tau).
//
// The CDF is a per-replica inclusive prefix sum of q_j = floor(w_j 2^s) in uint64 ("segmented":
// segments are replicas; tiles never span two).  Integer sums are exact and associative, so the CDF
// is identical for any tile decomposition and any search order -- which is what lets the GPU's
// 32-ary warp search and the CPU oracle's binary search pick the same node for the same uniform.
//
// HBM roofline per node: read fitness, indeg, pub (12 B), write w (4 B); read w (4 B), write cdf
// (8 B); cdf read+write in the offset pass (16 B).
#pragma once
#include "pg_engine.cuh"

namespace pg {

__device__ __forceinline__ void d_epoch_begin(const Arena& A, int64_t epoch, int64_t delta_override) {
    __shared__ int64_t sw[33];
    __shared__ int64_t carry;
    EpochState* st = A.st;
    if (threadIdx.x == 0) {
        carry = 0;
        st->reloc_count = 0;
        st->er_ov_count = 0;
        st->epoch = epoch;
        st->edges = 0;
        st->queue_small = 0;
        st->queue_big = 0;
        st->big_count = 0;
        st->heavy_count = 0;
        st->rc_big_count = 0;
        st->rc_big_queue = 0;
        st->sort_small_count = 0;
        st->sort_large_count = 0;
        st->sort_scratch = 0;
        st->rows_expanded = 0;
        st->elems_streamed = 0;
        st->draws = 0;
        st->bwd_moved = 0;
        st->nodes_weighted = 0;
        st->adj_scanned = 0;
    }
    __syncthreads();
    for (int base = 0; base < A.R; base += blockDim.x) {
        const int r = base + threadIdx.x;
        int64_t d = 0;
        if (r < A.R) {
            Replica& rp = A.rep[r];
            if (delta_override >= 0)
                d = (r == 0) ? delta_override : 0;
            else if (rp.growth_rate > 0.0)
                d = (int64_t)ceil((double)rp.n * rp.growth_rate);
            else
                d = rp.fixed_new;
            if (d < 0) d = 0;
            if (rp.n + d > rp.n_cap) atomicOr(&st->error, kErrCapacity);
            rp.delta = d;
            rp.wmax_bits = 0;
            rp.npos = 0;
            rp.wq_total = 0;
            for (int b = 0; b < kHeavyBins; ++b) rp.heavy_hist[b] = 0;
            rp.heavy_count = 0;
        }
        int64_t tot;
        const int64_t ex = block_excl_scan<int64_t>(d, sw, &tot);
        if (r < A.R) A.rep[r].abase = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->agents = carry;
        if (carry > A.agent_cap) atomicOr(&st->error, kErrCapacity);
    }
}

__global__ void __launch_bounds__(1024) k_epoch_begin(Arena A, int64_t epoch, int64_t delta_override) { d_epoch_begin(A, epoch, delta_override); }

// w_j for active nodes; per-replica max (as float bits, valid for non-negative floats) and count
// of positive weights.
__device__ __forceinline__ void d_weights(const Arena& A, int vb) {
    __shared__ uint32_t s_max[kTileThreads / 32];
    __shared__ int s_cnt[kTileThreads / 32], s_act[kTileThreads / 32];
    if (cta_error(A)) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const int64_t n = rp.n;
    const int32_t ep = (int32_t)A.st->epoch;
    constexpr int kPer = kTile / kTileThreads;
    // every input of the thread's nodes is loaded before any weight is stored (the stores could
    // otherwise alias the later loads and serialise them)
    float fv[kPer];
    int32_t iv[kPer], pv[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        const int64_t slot = rp.nbase + (v < n ? v : 0);
        fv[i] = A.fit[slot];
        iv[i] = A.indeg[slot];
        pv[i] = A.pub[slot];
    }
    uint32_t wmax = 0;
    int cnt = 0, act = 0;
    bool bad = false;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        if (v < n) {
            const float w = weight0(fv[i], iv[i], ep - pv[i], rp.alpha, rp.gamma, rp.tau);
            A.w[rp.nbase + v] = w;
            ++act;
            if (!(w <= 3.0e38f)) bad = true;  // inf or NaN
            if (w > 0.0f) {
                ++cnt;
                const uint32_t b = fbits(w);
                wmax = b > wmax ? b : wmax;
            }
        }
    }
    // one set of replica atomics per CTA
    wmax = __reduce_max_sync(0xffffffffu, wmax);
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    act = __reduce_add_sync(0xffffffffu, act);
    if (__any_sync(0xffffffffu, bad) && lane_id() == 0) atomicOr(&A.st->error, kErrBadWeight);
    const int wid = threadIdx.x >> 5;
    if (lane_id() == 0) {
        s_max[wid] = wmax;
        s_cnt[wid] = cnt;
        s_act[wid] = act;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kTileThreads / 32; ++w) {
            wmax = s_max[w] > wmax ? s_max[w] : wmax;
            cnt += s_cnt[w];
            act += s_act[w];
        }
        if (wmax) atomicMax(&A.rep[r].wmax_bits, wmax);
        if (cnt) atomicAdd((unsigned long long*)&A.rep[r].npos, (unsigned long long)cnt);
        if (act) atomicAdd(&A.st->nodes_weighted, (unsigned long long)act);
    }
}

__global__ void __launch_bounds__(kTileThreads) k_weights(Arena A) { d_weights(A, blockIdx.x); }

// q_j = quantise(w_j, s_r); tile-local inclusive scan into cdf, tile total into tilesum.
__device__ __forceinline__ void d_cdf_tiles(const Arena& A, int vb) {
    __shared__ uint64_t sw[33];
    const int t = vb;
    if (cta_error(A)) return;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) {
        if (threadIdx.x == 0) A.tilesum[t] = 0;
        return;
    }
    const uint32_t wb = rp.wmax_bits;
    if (wb == 0) {
        if (threadIdx.x == 0) atomicOr(&A.st->error, kErrBadWeight);
        return;
    }
    const int s = cdf_shift(bitsf(wb), rp.n);
    const int64_t n = rp.n;
    const int64_t vt = v0 + (int64_t)threadIdx.x * 4;
    const float4 w4 = *reinterpret_cast<const float4*>(A.w + rp.nbase + vt);
    uint64_t q[4];
    q[0] = vt + 0 < n ? quantise(w4.x, s) : 0;
    q[1] = vt + 1 < n ? quantise(w4.y, s) : 0;
    q[2] = vt + 2 < n ? quantise(w4.z, s) : 0;
    q[3] = vt + 3 < n ? quantise(w4.w, s) : 0;
    q[1] += q[0];
    q[2] += q[1];
    q[3] += q[2];
    uint64_t tot;
    const uint64_t ex = block_excl_scan<uint64_t>(q[3], sw, &tot);
    ulonglong2* dst = reinterpret_cast<ulonglong2*>(A.cdf + rp.nbase + vt);
    dst[0] = make_ulonglong2(ex + q[0], ex + q[1]);
    dst[1] = make_ulonglong2(ex + q[2], ex + q[3]);
    *reinterpret_cast<int4*>(A.guide + rp.nbase + vt) = make_int4(0, 0, 0, 0);  // marks start at 0
    if (threadIdx.x == 0) A.tilesum[t] = tot;
}

__global__ void __launch_bounds__(kTileThreads) k_cdf_tiles(Arena A) { d_cdf_tiles(A, blockIdx.x); }

// One CTA: tileoff[t] = sum of tilesum over the earlier tiles of the same replica (mod 2^64, which
// is exact because every replica's own total is below 2^63); each replica's total goes to wq_total.
__device__ __forceinline__ void d_tile_scan(const Arena& A) {
    __shared__ uint64_t sw[33];
    __shared__ uint64_t carry;
    if (cta_error(A)) return;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int T = A.ntiles;
    for (int base = 0; base < T; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const uint64_t v = i < T ? A.tilesum[i] : 0;
        uint64_t tot;
        const uint64_t ex = block_excl_scan<uint64_t>(v, sw, &tot);
        if (i < T) A.tileoff[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    // per-replica base and total; tilesum[] is free now and holds the bases
    for (int r = threadIdx.x; r < A.R; r += blockDim.x) {
        const Replica& rp = A.rep[r];
        const uint64_t b = A.tileoff[rp.tbase];
        const int e = rp.tbase + rp.ntiles;
        const uint64_t end = e < T ? A.tileoff[e] : carry;
        A.tilesum[r] = b;
        A.rep[r].wq_total = end - b;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < T; i += blockDim.x) A.tileoff[i] -= A.tilesum[A.tile_rep[i]];
}

__global__ void __launch_bounds__(1024) k_tile_scan(Arena A) { d_tile_scan(A); }

// Tile offsets into the CDF, and the guide table's marks: node v whose CDF interval
// [cdf[v-1], cdf[v]) contains bucket starts g 2^gs marks the first of them, guide[g] = v.
__device__ __forceinline__ void d_cdf_add(const Arena& A, int vb) {
    if (cta_error(A)) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const uint64_t off = A.tileoff[t];
    const int64_t vt = v0 + (int64_t)threadIdx.x * 4;
    ulonglong2* p = reinterpret_cast<ulonglong2*>(A.cdf + rp.nbase + vt);
    ulonglong2 a = p[0], b = p[1];
    // the tile-local value before this thread's first slot (written by k_cdf_tiles, read before
    // any thread of the tile adds the offset)
    const uint64_t before = threadIdx.x == 0 ? 0 : A.cdf[rp.nbase + vt - 1];
    __syncthreads();
    a.x += off;
    a.y += off;
    b.x += off;
    b.y += off;
    if (off) {
        p[0] = a;
        p[1] = b;
    }
    const int gs = guide_shift(rp.wq_total, rp.n);
    const uint64_t c[5] = {before + off, a.x, a.y, b.x, b.y};
    int32_t* guide = A.guide + rp.nbase;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint64_t lo = c[i], hi = c[i + 1];
        if (vt + i < rp.n && hi > lo) {
            const uint64_t g0 = (lo + ((1ull << gs) - 1)) >> gs, g1 = (hi - 1) >> gs;
            if (g0 <= g1) guide[g0] = (int32_t)(vt + i);
        }
    }
}

__global__ void __launch_bounds__(kTileThreads) k_cdf_add(Arena A) { d_cdf_add(A, blockIdx.x); }

// Guide table fill: guide[g] = smallest v with cdf[v] > g 2^gs, for g < used(Wq, n).  Each tile of
// buckets takes the running maximum of its marks, starting from the node that owns its first
// bucket (one binary search per tile), so no tile waits for another.
__device__ __forceinline__ void d_guide_fill(const Arena& A, int vb) {
    __shared__ int32_t wmax[kTileThreads / 32];
    __shared__ int32_t carry;
    if (cta_error(A)) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const uint64_t Wq = rp.wq_total;
    if (Wq == 0 || rp.n <= 0) return;
    const int gs = guide_shift(Wq, rp.n);
    const int64_t used = (int64_t)((Wq - 1) >> gs) + 1;
    const int64_t g0 = (int64_t)(t - rp.tbase) * kTile;
    if (g0 >= used) return;
    const uint64_t* cdf = A.cdf + rp.nbase;
    if (threadIdx.x == 0) {
        int32_t v = 0;
        if (g0 > 0) {
            const uint64_t y = (uint64_t)g0 << gs;
            int64_t lo = 0, hi = rp.n - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (cdf[mid] > y)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            v = (int32_t)lo;
        }
        carry = v;
    }
    int4* gp = reinterpret_cast<int4*>(A.guide + rp.nbase + g0) + threadIdx.x;
    int4 m = *gp;
    m.y = max(m.y, m.x);
    m.z = max(m.z, m.y);
    m.w = max(m.w, m.z);
    // block-wide inclusive running maximum of the threads' last values
    int32_t x = m.w;
    const int lane = lane_id(), wid = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t o = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x = max(x, o);
    }
    if (lane == 31) wmax[wid] = x;
    __syncthreads();
    int32_t pre = carry;
    for (int w = 0; w < wid; ++w) pre = max(pre, wmax[w]);
    const int32_t prev = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane > 0) pre = max(pre, prev);
    m.x = max(m.x, pre);
    m.y = max(m.y, pre);
    m.z = max(m.z, pre);
    m.w = max(m.w, pre);
    *gp = m;
}

__global__ void __launch_bounds__(kTileThreads) k_guide_fill(Arena A) { d_guide_fill(A, blockIdx.x); }

// ---------------------------------------------------------------- hub index
// Ball membership of a high-degree node j needs adj(j) intersected with the agent's 1-hop
// frontier, which is expensive when j has millions of neighbours.  Each epoch the nodes of degree
// >= heavy_thr become hubs (at most kHeavyMax per replica, the highest log2-degree bins); each holds
// one bit, and hmask[v] has bit b set when hub b is adjacent to v, so an agent ORs hmask over its
// frontier once and answers "hub b in my ball?" with one bit test.  Which nodes are hubs only changes
// speed, never a result.
// The index is kept from epoch to epoch.  Adjacency only grows by new nodes' edges, and a new node
// is never a hub, so the placement of an epoch's edges writes each new node's mask from the hubs it
// cites; the next epoch then only moves the hubs that changed: a node that left the hub set clears
// its bit on its neighbours, a node that joined takes a free bit and sets it on its neighbours.  A
// load or restore clears hub_valid and the next epoch rebuilds the whole index.
__device__ __forceinline__ int64_t degree_of(const Arena& A, const Replica& rp, int64_t v) {
    const int64_t* fo = A.fwd_off + rp.obase;
    return (fo[v + 1] - fo[v]) + blen(A.brow + rp.nbase, v);
}

__device__ __forceinline__ void d_hub_hist(const Arena& A, int vb) {
    if (A.st->error) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const bool full = !rp.hub_valid;
    constexpr int kPer = kTile / kTileThreads;
    int64_t dg[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        dg[i] = v < rp.n ? degree_of(A, rp, v) : 0;
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        if (v >= rp.n) continue;
        if (full) {  // the degrees were loaded first: these stores could otherwise delay them
            const int64_t slot = rp.nbase + v;
            A.hslot[slot] = -1;
            static_assert(kMaskWords == 4, "hub mask row of 32 bytes");
            ulonglong2* hm = reinterpret_cast<ulonglong2*>(A.hmask + slot * kMaskWords);
            hm[0] = make_ulonglong2(0ull, 0ull);
            hm[1] = make_ulonglong2(0ull, 0ull);
        }
        const int64_t d = dg[i];
        if (d >= (1 << kHeavyMinLog)) {
            int b = 63 - __clzll((unsigned long long)d) - kHeavyMinLog;
            if (b >= kHeavyBins) b = kHeavyBins - 1;
            atomicAdd(&rp.heavy_hist[b], 1);
        }
    }
}

__global__ void __launch_bounds__(kTileThreads) k_hub_hist(Arena A) { d_hub_hist(A, blockIdx.x); }

__device__ __forceinline__ void d_hub_pick(const Arena& A) {
    if (cta_error(A)) return;
    for (int r = threadIdx.x; r < A.R; r += blockDim.x) {
        Replica& rp = A.rep[r];
        int thr = 0x7fffffff, cum = 0;
        for (int b = kHeavyBins - 1; b >= 0; --b) {
            cum += rp.heavy_hist[b];
            if (cum > kHeavyMax) break;
            if (rp.heavy_hist[b]) thr = 1 << (b + kHeavyMinLog);
        }
        rp.heavy_thr = thr;
        rp.hub_nadd = 0;
        rp.hub_full = !rp.hub_valid;
        rp.hub_valid = 1;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < (int64_t)A.R * kHeavyMax; i += blockDim.x) {
        A.hub_rem[i] = -1;
        A.hub_add[i] = -1;
        if (A.rep[i / kHeavyMax].hub_full) A.hlist[i] = -1;
    }
    // hub-pair masks are OR-accumulated by k_hub_pairs, for the hubs the agent setup flags
    const int64_t words = (int64_t)A.R * kHeavyMax * kMaskWords;
    for (int64_t i = threadIdx.x; i < words; i += blockDim.x) A.hub2[i] = 0;
    for (int64_t i = threadIdx.x; i < (int64_t)A.R * (kHeavyMax / 32); i += blockDim.x) A.hub_need[i] = 0u;
}

__global__ void k_hub_pick(Arena A) { d_hub_pick(A); }

// Nodes leaving the hub set give up their bit (hub_rem), nodes joining it are listed (hub_cand).
__device__ __forceinline__ void d_hub_collect(const Arena& A, int vb) {
    if (A.st->error) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const int64_t thr = rp.heavy_thr;
    constexpr int kPer = kTile / kTileThreads;
    int64_t dg[kPer];
    int hs[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        dg[i] = v < rp.n ? degree_of(A, rp, v) : 0;
        hs[i] = v < rp.n ? A.hslot[rp.nbase + v] : -1;
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        if (v >= rp.n) continue;
        const bool want = dg[i] >= thr;
        if (hs[i] >= 0 && !want) {
            A.hub_rem[(int64_t)r * kHeavyMax + hs[i]] = (int32_t)v;
            A.hslot[rp.nbase + v] = -1;
        } else if (hs[i] < 0 && want) {
            const int q = atomicAdd(&rp.hub_nadd, 1);
            if (q < kHeavyMax) A.hub_cand[(int64_t)r * kHeavyMax + q] = (int32_t)v;
        }
    }
}

__global__ void __launch_bounds__(kTileThreads) k_hub_collect(Arena A) { d_hub_collect(A, blockIdx.x); }

// Bits of the epoch, one warp per replica: the bits given up are freed, and the q-th joining node
// takes the q-th free bit.  (At most kHeavyMax nodes have degree >= heavy_thr, so there are always
// enough free bits.)
__device__ __forceinline__ void d_hub_assign(const Arena& A) {
    if (A.st->error) return;
    const int lane = lane_id();
    for (int r = threadIdx.x >> 5; r < A.R; r += blockDim.x >> 5) {
        Replica& rp = A.rep[r];
        int32_t* hl = A.hlist + (int64_t)r * kHeavyMax;
        const int32_t* rem = A.hub_rem + (int64_t)r * kHeavyMax;
        unsigned freew[kHeavyMax / 32];
#pragma unroll
        for (int w = 0; w < kHeavyMax / 32; ++w) {
            const int b = w * 32 + lane;
            const bool fr = hl[b] < 0 || rem[b] >= 0;
            if (rem[b] >= 0) hl[b] = -1;
            freew[w] = __ballot_sync(0xffffffffu, fr);
        }
        const int nadd = rp.hub_nadd < kHeavyMax ? rp.hub_nadd : kHeavyMax;
        for (int q = lane; q < nadd; q += 32) {
            // the q-th free bit
            int left = q, b = -1;
#pragma unroll
            for (int w = 0; w < kHeavyMax / 32; ++w) {
                const int c = __popc(freew[w]);
                if (b < 0 && left < c) {
                    unsigned m = freew[w];
                    for (int k = 0; k < left; ++k) m &= m - 1u;
                    b = w * 32 + __ffs(m) - 1;
                }
                if (b < 0) left -= c;
            }
            if (b >= 0) {
                const int32_t v = A.hub_cand[(int64_t)r * kHeavyMax + q];
                hl[b] = v;
                A.hub_add[(int64_t)r * kHeavyMax + b] = v;
                A.hslot[rp.nbase + v] = (int16_t)b;
            } else {
                atomicOr(&A.st->error, kErrCapacity);  // cannot happen: see above
            }
        }
        __syncwarp();
        int top = 0;
#pragma unroll
        for (int w = 0; w < kHeavyMax / 32; ++w) {
            const unsigned used = __ballot_sync(0xffffffffu, hl[w * 32 + lane] >= 0);
            if (used) top = w * 32 + 32 - __clz((int)used);
        }
        if (lane == 0) rp.heavy_count = top;
    }
}

__global__ void __launch_bounds__(256) k_hub_assign(Arena A) { d_hub_assign(A); }

// G CTAs per (replica, hub bit) split a hub's neighbours.  SET = false: the node that left bit b
// clears it on its neighbours; SET = true: the node that took bit b sets it (the clears of an epoch
// all finish before its sets, so a bit freed and taken again in one epoch ends up right).
template <bool SET>
__device__ __forceinline__ void d_hub_mask(const Arena& A, int G, int vb) {
    if (A.st->error) return;
    const int item = vb / G, g = vb % G;
    const int r = item / kHeavyMax, b = item % kHeavyMax;
    if (r >= A.R) return;
    const Replica& rp = A.rep[r];
    const int64_t h = (SET ? A.hub_add : A.hub_rem)[(int64_t)r * kHeavyMax + b];
    if (h < 0) return;
    const unsigned long long bit = 1ull << (b & 63);
    const int64_t stride = (int64_t)G * blockDim.x;
    for (int dir = 0; dir < 2; ++dir) {
        int64_t p0, p1;
        const int32_t* col;
        if (dir) {
            bspan(A.brow + rp.nbase, h, p0, p1);
            col = A.bcol + rp.bbase;
        } else {
            p0 = A.fwd_off[rp.obase + h];
            p1 = A.fwd_off[rp.obase + h + 1];
            col = A.fwd_col + rp.ebase;
        }
        for (int64_t p = p0 + (int64_t)g * blockDim.x + threadIdx.x; p < p1; p += stride) {
            unsigned long long* w = (unsigned long long*)&A.hmask[(rp.nbase + col[p]) * kMaskWords + (b >> 6)];
            if (SET)
                atomicOr(w, bit);
            else
                atomicAnd(w, ~bit);
        }
    }
}

template <bool SET>
__global__ void __launch_bounds__(256) k_hub_mask(Arena A, int G) { d_hub_mask<SET>(A, G, blockIdx.x); }

// hub2[b] = OR of hmask over the hub's neighbours: the hubs sharing a neighbour with hub b.
__device__ __forceinline__ void d_hub_pairs(const Arena& A, int G, int vb) {
    __shared__ unsigned long long acc[kMaskWords];
    if (cta_error(A)) return;
    const int item = vb / G, g = vb % G;
    const int r = item / kHeavyMax, b = item % kHeavyMax;
    if (r >= A.R) return;
    const Replica& rp = A.rep[r];
    const int64_t h = A.hlist[(int64_t)r * kHeavyMax + b];
    if (h < 0) return;
    // only an agent whose anchor is hub b reads its row
    if (!((A.hub_need[(int64_t)r * (kHeavyMax / 32) + (b >> 5)] >> (b & 31)) & 1u)) return;
    if (threadIdx.x < kMaskWords) acc[threadIdx.x] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)G * blockDim.x;
    unsigned long long m[kMaskWords];
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) m[w] = 0;
    for (int dir = 0; dir < 2; ++dir) {
        int64_t p0, p1;
        const int32_t* col;
        if (dir) {
            bspan(A.brow + rp.nbase, h, p0, p1);
            col = A.bcol + rp.bbase;
        } else {
            p0 = A.fwd_off[rp.obase + h];
            p1 = A.fwd_off[rp.obase + h + 1];
            col = A.fwd_col + rp.ebase;
        }
        for (int64_t p = p0 + (int64_t)g * blockDim.x + threadIdx.x; p < p1; p += stride) {
            const uint64_t* hm = A.hmask + (rp.nbase + col[p]) * kMaskWords;
#pragma unroll
            for (int w = 0; w < kMaskWords; ++w) m[w] |= hm[w];
        }
    }
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) {
        unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)m[w]);
        unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(m[w] >> 32));
        if (lane_id() == 0 && (lo | hi)) atomicOr(&acc[w], ((unsigned long long)hi << 32) | lo);
    }
    __syncthreads();
    if (threadIdx.x < kMaskWords && acc[threadIdx.x])
        atomicOr((unsigned long long*)&A.hub2[((int64_t)r * kHeavyMax + b) * kMaskWords + threadIdx.x],
                 acc[threadIdx.x]);
}

__global__ void __launch_bounds__(256) k_hub_pairs(Arena A, int G) { d_hub_pairs(A, G, blockIdx.x); }

void launch_hubs(const Arena& A, int num_sms, cudaStream_t s) {
    (void)num_sms;
    const int G = A.R >= 64 ? 1 : 64 / A.R;  // CTAs per hub
    k_hub_hist<<<A.ntiles, kTileThreads, 0, s>>>(A);
    k_hub_pick<<<1, 256, 0, s>>>(A);
    k_hub_collect<<<A.ntiles, kTileThreads, 0, s>>>(A);
    k_hub_assign<<<1, 256, 0, s>>>(A);
    k_hub_mask<false><<<(unsigned)(A.R * kHeavyMax * G), 256, 0, s>>>(A, G);
    k_hub_mask<true><<<(unsigned)(A.R * kHeavyMax * G), 256, 0, s>>>(A, G);
}

void launch_hub_pairs(const Arena& A, cudaStream_t s) {
    const int G = A.R >= 64 ? 1 : 64 / A.R;
    k_hub_pairs<<<(unsigned)(A.R * kHeavyMax * G), 256, 0, s>>>(A, G);
}

void launch_epoch_begin(const Arena& A, int64_t epoch, int pa_mode, cudaStream_t s) {
    (void)pa_mode;
    k_epoch_begin<<<1, 1024, 0, s>>>(A, epoch, -1);
}

void launch_epoch_begin_delta(const Arena& A, int64_t epoch, int64_t delta, cudaStream_t s) {
    k_epoch_begin<<<1, 1024, 0, s>>>(A, epoch, delta);
}

void launch_weights(const Arena& A, cudaStream_t s) {
    k_weights<<<A.ntiles, kTileThreads, 0, s>>>(A);
    k_cdf_tiles<<<A.ntiles, kTileThreads, 0, s>>>(A);
    k_tile_scan<<<1, 1024, 0, s>>>(A);
    k_cdf_add<<<A.ntiles, kTileThreads, 0, s>>>(A);
}

void launch_guide(const Arena& A, cudaStream_t s) { k_guide_fill<<<A.ntiles, kTileThreads, 0, s>>>(A); }

}  // namespace pg
