// pg_csr.cuh -- device CSR append of one epoch's edges (stage e; part of the epoch translation unit,
// pg_agents.cu).
//
// Replaces the reference's per-epoch host work: sorting new_edges_vec, inserting into
// std::map<int, std::set<int>> adjacency (src/kernel.cu:1766-1810), updating in-degrees
// (src/graph.cu:537-618) and rebuilding int32 CSRs with prepareGraph (src/utils.cu:75-142).
//
// Forward rows of new nodes were written by the agent kernel (append-only, sorted).  Backward rows
// grow in place (BRow: room for cap entries, len used), so an epoch touches only the rows it
// appends to:
//   grow : one thread per edge; each cited node is handled once, by its edge of rank 0 (the agent
//          kernel's in-degree increment returned each edge's rank among the node's new entries):
//          new length = old + inc; a row without room for it takes a new span of
//          brow_span(new, P) entries from the region's bump pointer (one reservation per warp step,
//          P = fwd_prefix(out-degree)) and lists for the copy, in chunks of kRelocChunk, its old
//          span's forward row copy and entries -- or, at its first citation, its forward row from
//          the forward CSR; where the epoch's entries start goes to new_start; indeg += inc; rows
//          with two or more new entries are listed for the sort
//   copy : the listed chunks moved in 16-byte vectors, forward rows entry by entry (on a side
//          stream, beside place and sort)
//   place: each new edge at its row's start of new entries + rank
//   sort : the appended part of a row holds distinct new-node ids in atomic order; rows with up to
//          256 new entries are sorted by a register bitonic network in one warp, longer ones by a
//          shared-memory bitmap over the epoch's new-id range.  Rows end up ascending, like the
//          reference's std::set rows, and bit-identical run to run.
// Which span a row occupies depends on the order of the reservations; its entries do not.
#pragma once
#include "pg_engine.cuh"

namespace pg {

constexpr unsigned kFullMask = 0xffffffffu;

// Replica of epoch edge e: the last replica whose edges start at or before e.
__device__ __forceinline__ int replica_of_edge(const Arena& A, int64_t e) {
    int lo = 0, hi = A.R - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.eoff[A.rep[mid].abase] <= e)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// One thread per epoch edge, 32 consecutive edges per warp step; the edge of rank 0 handles its row.
__device__ __forceinline__ void d_bwd_grow(const Arena& A, int64_t agents) {
    if (A.st->error) return;
    const int lane = lane_id();
    const unsigned below = (1u << lane) - 1u;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t E = A.eoff[agents];
    unsigned long long moved = 0;
    for (int64_t eb = warp * 32; eb < E; eb += nwarps * 32) {
        const int64_t e = eb + lane;
        const int r = A.R == 1 ? 0 : replica_of_edge(A, e < E ? e : E - 1);
        Replica& rp = A.rep[r];
        bool mine = e < E && A.e_rank[e] == 0;
        int64_t slot = 0, nl = 0, need = 0, nch = 0, f0 = 0, o = 0, P = 0, mv = 0;
        int ic = 0;
        BRow rw{0u, 0};
        if (mine) {
            const int32_t v = A.e_dst[e];
            slot = rp.nbase + v;
            ic = A.inc[slot];
            rw = A.brow[slot];
            nl = (int64_t)rw.len + ic;
            if (nl > A.bcap[slot]) {
                const int64_t* fo = A.fwd_off + rp.obase;
                f0 = fo[v];
                o = fo[v + 1] - f0;
                P = fwd_prefix(o);
                need = brow_span(nl, P);
                // a row with a span moves its prefix and entries; a first span copies the forward row
                mv = rw.len > 0 ? P + rw.len : o;
                nch = (mv + kRelocChunk - 1) / kRelocChunk;
            }
        }
        // the step's reservations, one atomic each where the warp lies in one replica: region
        // spans, copy tasks, sort-list entries and large-sort scratch
        const bool uni = __all_sync(kFullMask, r == __shfl_sync(kFullMask, r, 0));
        const int64_t incl = warp_incl_scan<int64_t>(need);
        const int64_t tot = __shfl_sync(kFullMask, incl, 31);
        const int64_t cincl = warp_incl_scan<int64_t>(nch);
        const int64_t ctot = __shfl_sync(kFullMask, cincl, 31);
        const bool small = mine && ic >= 2 && ic <= kSortMid, large = mine && ic > kSortMid;
        const unsigned bs = __ballot_sync(kFullMask, small), bl = __ballot_sync(kFullMask, large);
        const int64_t sincl = warp_incl_scan<int64_t>(large ? ic : 0);
        const int64_t stot = __shfl_sync(kFullMask, sincl, 31);
        int64_t base = 0, cbase = 0, sbase = 0, lbase = 0, scbase = 0;
        if (lane == 0) {
            if (uni && tot) base = (int64_t)atomicAdd(&rp.b_top, (unsigned long long)tot);
            if (ctot) cbase = (int64_t)atomicAdd(&A.st->reloc_count, (unsigned long long)ctot);
            if (bs) sbase = (int64_t)atomicAdd(&A.st->sort_small_count, (unsigned long long)__popc(bs));
            if (bl) {
                lbase = (int64_t)atomicAdd(&A.st->sort_large_count, (unsigned long long)__popc(bl));
                scbase = (int64_t)atomicAdd(&A.st->sort_scratch, (unsigned long long)stot);
            }
        }
        base = __shfl_sync(kFullMask, base, 0);
        cbase = __shfl_sync(kFullMask, cbase, 0);
        sbase = __shfl_sync(kFullMask, sbase, 0);
        lbase = __shfl_sync(kFullMask, lbase, 0);
        scbase = __shfl_sync(kFullMask, scbase, 0);
        int64_t nb = base + incl - need;
        if (!uni && need) nb = (int64_t)atomicAdd(&rp.b_top, (unsigned long long)need);
        // the region and the task list are sized so that neither can run out
        const bool room = (uni ? base + tot : (need ? nb + need : 0)) <= rp.b_cap && cbase + ctot <= A.reloc_cap;
        if (!room) atomicOr(&A.st->error, kErrCapacity);
        if (!mine || !room) continue;
        const int64_t old = rw.len;
        int64_t beg = (int64_t)rw.beg4 << 2;
        if (need) {
            // moves: from the old span's start (4 beg4 - P), both spans 16-byte aligned; first spans:
            // from the forward CSR (a negative source, -1 - index) to the o entries before 4 beg4
            const int64_t q = cbase + cincl - nch;
            const int64_t src0 = old > 0 ? rp.bbase + beg - P : -1 - (rp.ebase + f0);
            const int64_t dst0 = rp.bbase + nb + (old > 0 ? 0 : P - o);
            for (int64_t c = 0; c < nch; ++c) {
                const int64_t off = c * kRelocChunk;
                const int64_t len = mv - off < kRelocChunk ? mv - off : kRelocChunk;
                A.reloc[q + c] = make_longlong2(old > 0 ? src0 + off : src0 - off, ((dst0 + off) << 16) | len);
            }
            moved += (unsigned long long)mv;
            beg = nb + P;
            rw.beg4 = (uint32_t)(beg >> 2);
            A.bcap[slot] = (int32_t)(need - P);
        }
        A.new_start[slot] = beg + old;
        rw.len = (int32_t)nl;
        A.brow[slot] = rw;
        A.indeg[slot] += ic;
        A.inc[slot] = 0;
        if (small) A.sort_small[sbase + __popc(bs & below)] = (slot << 9) | (int64_t)ic;
        if (large) {
            const int64_t q = lbase + __popc(bl & below);
            A.sort_large[q] = slot;
            A.sort_large_off[q] = ((scbase + sincl - ic) << 32) | (int64_t)ic;
        }
    }
    moved = warp_sum(moved);
    if (lane == 0 && moved) atomicAdd(&A.st->bwd_moved, moved);
}

__global__ void __launch_bounds__(256) k_bwd_grow(Arena A, int64_t agents) { d_bwd_grow(A, agents); }

// The old spans of the rows that moved (forward row copy and entries), one listed chunk (at most
// kRelocChunk entries) per warp: source and destination are 16-byte aligned, the copy goes in int4
// vectors with eight of them per lane in flight, and the chunk's last (len mod 4) entries one by
// one -- the vector past them would overwrite the row's first new entries, which the placement
// writes at the same time.  A chunk with a negative source (-1 - index) is a first span's forward
// row, copied entry by entry from the forward CSR (no alignment in common).
__device__ __forceinline__ void d_bwd_reloc(const Arena& A) {
    if (A.st->error) return;
    const int lane = lane_id();
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t cnt = (int64_t)A.st->reloc_count;
    constexpr int kU = 8;
    for (int64_t i = warp; i < cnt; i += nwarps) {
        const longlong2 t = A.reloc[i];
        const int64_t src = t.x, dst = t.y >> 16;
        const int len = (int)(t.y & 0xffff);
        if (src < 0) {
            const int32_t* f = A.fwd_col + (-1 - src);
            for (int j = lane; j < len; j += 32) A.bcol[dst + j] = f[j];
            continue;
        }
        const int nv = len >> 2;
        const int4* s4 = reinterpret_cast<const int4*>(A.bcol + src);
        int4* d4 = reinterpret_cast<int4*>(A.bcol + dst);
        for (int v0 = 0; v0 < nv; v0 += 32 * kU) {
            int4 x[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int v = v0 + 32 * u + lane;
                if (v < nv) x[u] = s4[v];
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int v = v0 + 32 * u + lane;
                if (v < nv) d4[v] = x[u];
            }
        }
        if (lane < (len & 3)) A.bcol[dst + 4 * nv + lane] = A.bcol[src + 4 * nv + lane];
    }
}

__global__ void __launch_bounds__(256) k_bwd_reloc(Arena A) { d_bwd_reloc(A); }

// One warp per agent: each edge at its row's start of new entries + rank.  The agent is a new node:
// its hub-index entry is written here (no hub bit, and a mask of the hubs it cites), so the next
// epoch's hub index only has to move the hubs that changed.
__device__ __forceinline__ void d_bwd_place(const Arena& A, int64_t agents) {
    if (A.st->error) return;
    const int lane = lane_id();
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a = warp; a < agents; a += nwarps) {
        const int r = replica_of_agent(A.rep, A.R, a);
        const Replica& rp = A.rep[r];
        const int32_t src = (int32_t)(rp.n + (a - rp.abase));
        const int64_t e0 = A.eoff[a], e1 = A.eoff[a + 1];
        int32_t* bc = A.bcol + rp.bbase;
        const int64_t* st = A.new_start + rp.nbase;
        unsigned hm[2 * kMaskWords] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        for (int64_t e = e0 + lane; e < e1; e += 32) {
            const int32_t j = A.e_dst[e];
            bc[st[j] + A.e_rank[e]] = src;
            const int hs = A.hslot[rp.nbase + j];
            if (hs >= 0) {
#pragma unroll
                for (int w = 0; w < 2 * kMaskWords; ++w)
                    if ((hs >> 5) == w) hm[w] |= 1u << (hs & 31);
            }
        }
#pragma unroll
        for (int w = 0; w < 2 * kMaskWords; ++w) hm[w] = __reduce_or_sync(kFullMask, hm[w]);
        if (lane < kMaskWords) {
            const int64_t slot = rp.nbase + src;
            unsigned lo = hm[0], hi = hm[1];
#pragma unroll
            for (int w = 1; w < kMaskWords; ++w)
                if (lane == w) {
                    lo = hm[2 * w];
                    hi = hm[2 * w + 1];
                }
            A.hmask[slot * kMaskWords + lane] = ((unsigned long long)hi << 32) | lo;
            if (lane == 0) A.hslot[slot] = -1;
        }
    }
}

__global__ void __launch_bounds__(256) k_bwd_place(Arena A, int64_t agents) { d_bwd_place(A, agents); }

// A run's citation output (pg_run_epochs_out): the epoch's citations, (source, target), at the
// run's running count, written in whole lines -- the writes cross the host link, where a partial
// line costs as much as a full one.  Each CTA takes kCopyTile consecutive edges: the targets are
// copied straight through; the sources (the citing agents' node ids, one run per agent) are first
// laid out in `stage` (kCopyTile ints of shared memory) from the agents whose edges meet the tile.
// The first CTA records the epoch's count per replica.  The targets are read from the epoch's edge
// list, which the next epoch overwrites, so the stream order puts this before the epoch end.
constexpr int kCopyTile = 2048;
__device__ __forceinline__ void d_copy_out(const Arena& A, int64_t agents, int32_t* stage) {
    if (!A.out_src || A.st->error) return;
    const int64_t base = (int64_t)A.st->out_count;
    const int64_t E = A.eoff[agents];
    if (base + E > A.out_cap) {  // the buffers are full: the growth goes on, the host reports it
        if (blockIdx.x == 0 && threadIdx.x == 0) A.st->out_short += (unsigned long long)E;
        return;
    }
    if (blockIdx.x == 0) {
        const int64_t k = (int64_t)A.st->cum_epochs;
        for (int r = threadIdx.x; r < A.R && k < A.out_epochs; r += blockDim.x) {
            const Replica& rp = A.rep[r];
            A.out_counts[k * A.R + r] = A.eoff[rp.abase + rp.delta] - A.eoff[rp.abase];
        }
    }
    __shared__ int64_t span[2];  // the tile's first and last agent
    // the last agent whose edges start at or before edge e
    auto agent_of = [&](int64_t e) -> int64_t {
        int64_t lo = 0, hi = agents - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (A.eoff[mid] <= e)
                lo = mid;
            else
                hi = mid - 1;
        }
        return lo;
    };
    for (int64_t t0 = (int64_t)blockIdx.x * kCopyTile; t0 < E; t0 += (int64_t)gridDim.x * kCopyTile) {
        const int64_t t1 = E < t0 + kCopyTile ? E : t0 + kCopyTile;
        if (threadIdx.x == 0) {
            span[0] = agent_of(t0);
            span[1] = agent_of(t1 - 1);
        }
        __syncthreads();
        for (int64_t a = span[0] + threadIdx.x; a <= span[1]; a += blockDim.x) {
            const int r = replica_of_agent(A.rep, A.R, a);
            const Replica& rp = A.rep[r];
            const int32_t src = (int32_t)(rp.n + (a - rp.abase));
            const int64_t lo = A.eoff[a] > t0 ? A.eoff[a] : t0, hi = A.eoff[a + 1] < t1 ? A.eoff[a + 1] : t1;
            for (int64_t e = lo; e < hi; ++e) stage[e - t0] = src;
        }
        __syncthreads();
        for (int64_t e = t0 + threadIdx.x; e < t1; e += blockDim.x) {
            A.out_src[base + e] = stage[e - t0];
            A.out_dst[base + e] = A.e_dst[e];
        }
        __syncthreads();  // the stage is rewritten by the next tile
    }
}

__global__ void __launch_bounds__(256) k_copy_out(Arena A, int64_t agents) {
    __shared__ int32_t stage[kCopyTile];
    d_copy_out(A, agents, stage);
}

// The epoch's `added` entries of the row in `slot` (the row's last ones): replica and first entry.
__device__ __forceinline__ void seg_bounds(const Arena& A, int64_t slot, int64_t added, const Replica*& rpp,
                                           int64_t& start) {
    const int r = A.tile_rep[slot / kTile];
    const Replica& rp = A.rep[r];
    rpp = &rp;
    const BRow rw = A.brow[slot];
    start = rp.bbase + ((int64_t)rw.beg4 << 2) + rw.len - added;
}

template <int R>
__device__ __forceinline__ void warp_sort_segment(int32_t* seg, int64_t len, int lane) {
    int v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = i * 32 + lane < len ? seg[i * 32 + lane] : 0x7fffffff;
    warp_bitonic<R>(v, lane);
#pragma unroll
    for (int i = 0; i < R; ++i)
        if (i * 32 + lane < len) seg[i * 32 + lane] = v[i];
}

// Rows with 2..kSortMid appended entries: one warp, bitonic network in registers (1, 2, 4 or 8
// entries per lane).
__device__ __forceinline__ void d_sort_small(const Arena& A) {
    if (A.st->error) return;
    const int lane = lane_id();
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t cnt = (int64_t)A.st->sort_small_count;
    for (int64_t i = warp; i < cnt; i += nwarps) {
        const int64_t slot = A.sort_small[i] >> 9;
        const int64_t len = A.sort_small[i] & 511;
        const Replica* rp;
        int64_t start;
        seg_bounds(A, slot, len, rp, start);
        int32_t* seg = A.bcol + start;
        if (len <= 32)
            warp_sort_segment<1>(seg, len, lane);
        else if (len <= 64)
            warp_sort_segment<2>(seg, len, lane);
        else if (len <= 128)
            warp_sort_segment<4>(seg, len, lane);
        else
            warp_sort_segment<8>(seg, len, lane);
    }
}

__global__ void __launch_bounds__(256) k_sort_small(Arena A) { d_sort_small(A); }

// Rows with more than kSortMid appended entries: one CTA, shared bitmap bm of bm_words words over
// [n, n + delta), in chunks when the range is longer.
__device__ __forceinline__ void d_sort_large(const Arena& A, uint32_t* bm, int64_t bm_words) {
    __shared__ int64_t sw[33];
    __shared__ int64_t outpos;
    if (cta_error(A)) return;
    const int64_t cnt = (int64_t)A.st->sort_large_count;
    const int64_t kBits = bm_words * 32;
    for (int64_t i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int64_t slot = A.sort_large[i];
        const int64_t len = A.sort_large_off[i] & 0xffffffffll;
        const Replica* rp;
        int64_t start;
        seg_bounds(A, slot, len, rp, start);
        int32_t* seg = A.bcol + start;
        const int64_t lo = rp->n, range = rp->delta;
        const int32_t* srcv = seg;
        if (range > kBits) {  // several chunks: keep the input in the spent rank buffer
            int32_t* scratch = A.e_rank + (A.sort_large_off[i] >> 32);
            for (int64_t q = threadIdx.x; q < len; q += blockDim.x) scratch[q] = seg[q];
            __syncthreads();
            srcv = scratch;
        }
        if (threadIdx.x == 0) outpos = 0;
        for (int64_t cb = 0; cb < range; cb += kBits) {
            const int64_t bits = range - cb < kBits ? range - cb : kBits;
            const int nw = (int)((bits + 31) >> 5);
            for (int q = threadIdx.x; q < nw; q += blockDim.x) bm[q] = 0;
            __syncthreads();
            for (int64_t q = threadIdx.x; q < len; q += blockDim.x) {
                const int64_t x = (int64_t)srcv[q] - lo - cb;
                if (x >= 0 && x < bits) atomicOr(&bm[x >> 5], 1u << (x & 31));
            }
            __syncthreads();
            const int per = (nw + (int)blockDim.x - 1) / (int)blockDim.x;
            const int w0 = threadIdx.x * per;
            int64_t c = 0;
            for (int q = w0; q < w0 + per && q < nw; ++q) c += __popc(bm[q]);
            int64_t tot;
            int64_t ex = block_excl_scan<int64_t>(c, sw, &tot) + outpos;
            for (int q = w0; q < w0 + per && q < nw; ++q) {
                uint32_t word = bm[q];
                while (word) {
                    const int b = __ffs(word) - 1;
                    word &= word - 1;
                    seg[ex++] = (int32_t)(lo + cb + (int64_t)q * 32 + b);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) outpos += tot;
            __syncthreads();
        }
    }
}

// bm_words: the bitmap of this launch (dynamic shared memory), enough for the epoch's new-id range
// where that fits, so two CTAs share an SM.  1024 threads per CTA: a hub's row can take tens of
// thousands of new entries in one epoch, and that one row sets the kernel's length.
__global__ void __launch_bounds__(1024) k_sort_large(Arena A, int64_t bm_words) {
    extern __shared__ uint32_t bm[];
    d_sort_large(A, bm, bm_words);
}

__device__ __forceinline__ void d_epoch_end(const Arena& A, int64_t agents) {
    EpochState* st = A.st;
    if (st->error) return;
    for (int r = threadIdx.x; r < A.R; r += blockDim.x) {
        Replica& rp = A.rep[r];
        const int64_t er = A.eoff[rp.abase + rp.delta] - A.eoff[rp.abase];
        rp.m += er;
        rp.n += rp.delta;
    }
    if (threadIdx.x == 0) {
        st->cum_rows_expanded += st->rows_expanded;
        st->cum_elems_streamed += st->elems_streamed;
        st->cum_draws += st->draws;
        st->cum_bwd_moved += st->bwd_moved;
        st->cum_nodes_weighted += st->nodes_weighted;
        st->cum_edges += (unsigned long long)A.eoff[agents];
        st->cum_new_nodes += (unsigned long long)agents;
        st->cum_epochs += 1;
        st->cum_adj_scanned += st->adj_scanned;
        if (A.out_src && st->out_count + (unsigned long long)A.eoff[agents] <= (unsigned long long)A.out_cap)
            st->out_count += (unsigned long long)A.eoff[agents];
    }
}

__global__ void k_epoch_end(Arena A, int64_t agents) { d_epoch_end(A, agents); }

// The large-segment sort uses 160 KiB of dynamic shared memory; called once per process.
cudaError_t init_csr_kernels() {
    return cudaFuncSetAttribute(k_sort_large, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kBitmapWords * 4);
}

void launch_bwd_append(const Arena& A, int64_t agents, int num_sms, cudaStream_t s, cudaStream_t side,
                       cudaEvent_t fork, cudaEvent_t join) {
    int64_t ga = (agents + 7) / 8;
    if (ga > (int64_t)num_sms * 16) ga = (int64_t)num_sms * 16;
    if (ga < 1) ga = 1;
    k_bwd_grow<<<(unsigned)ga, 256, 0, s>>>(A, agents);
    const int copy_per_sm = A.tune_copy_ctas > 0 ? A.tune_copy_ctas : 8;
    // the moved rows' old entries and the new entries' placement and sorts write disjoint
    // positions: with a side stream they overlap
    const bool two = side && fork && join;
    if (two) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
    }
    k_bwd_reloc<<<(unsigned)(num_sms * copy_per_sm), 256, 0, two ? side : s>>>(A);
    // one CTA per SM: the copy is bound by the host link, and the placement and sorts beside it
    // keep the rest of the SMs
    if (A.out_src) k_copy_out<<<(unsigned)num_sms, 256, 0, two ? side : s>>>(A, agents);
    if (two) cudaEventRecord(join, side);
    k_bwd_place<<<(unsigned)ga, 256, 0, s>>>(A, agents);
    k_sort_small<<<(unsigned)num_sms * 8, 256, 0, s>>>(A);
    // a replica's new ids span at most the epoch's agents
    int64_t words = (agents + 31) / 32 + 1;
    if (words > kBitmapWords) words = kBitmapWords;
    k_sort_large<<<(unsigned)num_sms * 2, 1024, (size_t)words * 4, s>>>(A, words);
    if (two) cudaStreamWaitEvent(s, join, 0);
    k_epoch_end<<<1, 256, 0, s>>>(A, agents);
}

}  // namespace pg
