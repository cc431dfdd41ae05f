// pg_csr.cuh -- device CSR append of one epoch's edges (stage e; part of the epoch translation unit,
// pg_agents.cu).
//
// Replaces the reference's per-epoch host work: sorting new_edges_vec, inserting into
// std::map<int, std::set<int>> adjacency (src/kernel.cu:1766-1810), updating in-degrees
// (src/graph.cu:537-618) and rebuilding int32 CSRs with prepareGraph (src/utils.cu:75-142).
//
// Forward rows of new nodes were written by the agent kernel (append-only, sorted).  Backward rows
// are rebuilt into the other buffer:
//   len  : new_len = old_len + inc (inc = in-degree histogram of the epoch, filled by atomics in
//          the agent kernel, which also returned each edge's rank); indeg += inc; the rows whose
//          span starts a copy tile are recorded
//   scan : per-replica exclusive scan of new_len -> new int64 offsets
//   copy : old entries moved in tiles of kCopyTile positions (on a side stream, beside place/sort)
//   place: each new edge at new_off + old_len + rank
//   sort : the appended part of a row holds distinct new-node ids in atomic order; rows with up to
//          256 new entries are sorted by a register bitonic network in one warp, longer ones by a
//          shared-memory bitmap over the epoch's new-id range.  Rows end up ascending, like the
//          reference's std::set rows, and bit-identical run to run.
#pragma once
#include "pg_engine.cuh"

namespace pg {

constexpr unsigned kFullMask = 0xffffffffu;

__device__ __forceinline__ void d_bwd_len(const Arena& A, int vb) {
    __shared__ uint64_t sw[33];
    if (cta_error(A)) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    const int64_t nact = rp.n + rp.delta;
    if (v0 >= nact) {
        if (threadIdx.x == 0) A.tilesum[t] = 0;
        return;
    }
    const int64_t* off = A.bwd_off_cur + rp.obase;
    int64_t sum = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t v = v0 + (int64_t)threadIdx.x * 4 + i;
        const int64_t slot = rp.nbase + v;
        int64_t len = 0;
        if (v < nact) {
            const int64_t old = v < rp.n ? off[v + 1] - off[v] : 0;
            if (old > 0) {
                // the copy tiles whose first position lies in this row start their row search here
                for (int64_t ct = (off[v] + kCopyTile - 1) / kCopyTile; ct * kCopyTile < off[v + 1]; ++ct)
                    A.tile_row[rp.ctbase + ct] = (int32_t)v;
            }
            const int ic = A.inc[slot];
            len = old + ic;
            if (ic) {
                A.indeg[slot] += ic;
                A.inc[slot] = 0;
                if (ic >= 2) {
                    if (ic <= kSortMid) {
                        const unsigned long long q = atomicAdd(&A.st->sort_small_count, 1ull);
                        A.sort_small[q] = (slot << 9) | (int64_t)ic;
                    } else {
                        const unsigned long long q = atomicAdd(&A.st->sort_large_count, 1ull);
                        A.sort_large[q] = slot;
                        A.sort_large_off[q] =
                            (int64_t)atomicAdd(&A.st->sort_scratch, (unsigned long long)ic);
                    }
                }
            }
        }
        A.len_tmp[slot] = len;
        sum += len;
    }
    uint64_t tot;
    block_excl_scan<uint64_t>((uint64_t)sum, sw, &tot);
    if (threadIdx.x == 0) A.tilesum[t] = tot;
}

__global__ void __launch_bounds__(kTileThreads) k_bwd_len(Arena A) { d_bwd_len(A, blockIdx.x); }

__device__ __forceinline__ void d_bwd_off(const Arena& A, int vb) {
    __shared__ int64_t sw[33];
    if (cta_error(A)) return;
    const int t = vb;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    const int64_t nact = rp.n + rp.delta;
    if (v0 >= nact) return;
    int64_t len[4], s = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t v = v0 + (int64_t)threadIdx.x * 4 + i;
        len[i] = v < nact ? A.len_tmp[rp.nbase + v] : 0;
        s += len[i];
    }
    int64_t tot;
    int64_t ex = block_excl_scan<int64_t>(s, sw, &tot) + (int64_t)A.tileoff[t];
    int64_t* off = A.bwd_off_nxt + rp.obase;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t v = v0 + (int64_t)threadIdx.x * 4 + i;
        if (v < nact) off[v] = ex;
        ex += len[i];
        if (v == nact - 1) off[nact] = ex;
    }
}

__global__ void __launch_bounds__(kTileThreads) k_bwd_off(Arena A) { d_bwd_off(A, blockIdx.x); }

// Largest v in [lo, hi] with off[v] <= p (the row holding position p).
__device__ __forceinline__ int64_t row_of(const int64_t* off, int64_t lo, int64_t hi, int64_t p) {
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= p)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Old backward entries moved to their new positions, in tiles of kCopyTile consecutive positions
// (not rows), so a hub row with millions of entries is spread over many CTAs.  Reads and writes are
// coalesced.  The tile's row offsets and per-row shifts (new - old start) are staged in shared
// memory once, with the row holding the first position of every 32-position block, so each
// position searches only the rows between its block's row and the next block's (usually one or
// two); a tile spanning more than kCopyRows rows (long runs of empty rows) searches the global
// offsets instead.
constexpr int kCopyRows = 2048;
constexpr int kCopyBlocks = kCopyTile / 32;

// s_oc [kCopyRows + 1]: old offsets of the tile's rows, and the next one; s_sh [kCopyRows]: new minus
// old offset of the tile's rows; s_blk [kCopyBlocks]: row (tile-relative) holding each block's first
// position -- shared memory of the calling CTA (kCopySmemBytes in all)
// KU positions per thread are in flight at once (their loads issued before any is placed): 8 in
// the stage kernel, more in the epoch kernel, whose CTAs are fewer per SM.
template <int KU>
__device__ __forceinline__ void d_bwd_copy(const Arena& A, int64_t* s_oc, int64_t* s_sh, int16_t* s_blk) {
    if (cta_error(A)) return;
    const int64_t total = (int64_t)A.st->copy_tiles;
    unsigned long long moved = 0;
    for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
        int lo = 0, hi = A.R - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.rep[mid].ctbase <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        const Replica& rp = A.rep[lo];
        const int64_t p0 = (t - rp.ctbase) * kCopyTile;
        const int64_t p1 = p0 + kCopyTile < rp.m ? p0 + kCopyTile : rp.m;
        const int64_t* oc = A.bwd_off_cur + rp.obase;
        const int64_t* on = A.bwd_off_nxt + rp.obase;
        const int32_t* cc = A.bwd_col_cur + rp.ebase;
        int32_t* cn = A.bwd_col_nxt + rp.ebase;
        // rows holding the tile's first position and the next tile's first position (recorded by
        // k_bwd_len); the tile's last position lies in a row between them
        const int64_t tl = t - rp.ctbase;
        const int64_t r0 = A.tile_row[t];
        const int64_t r1 = (tl + 1) * kCopyTile < rp.m ? (int64_t)A.tile_row[t + 1] : rp.n - 1;
        if (threadIdx.x == 0) moved += (unsigned long long)(p1 - p0);
        const int64_t nr = r1 - r0 + 1;
        if (nr <= kCopyRows) {
            for (int64_t i = threadIdx.x; i < nr; i += blockDim.x) {
                const int64_t o = oc[r0 + i];
                s_oc[i] = o;
                s_sh[i] = on[r0 + i] - o;
            }
            if (threadIdx.x == 0) s_oc[nr] = oc[r1 + 1];
            __syncthreads();
            // block b starts at p0 + 32 b; the non-empty row holding it marks it
            for (int64_t i = threadIdx.x; i < nr; i += blockDim.x) {
                const int64_t a = s_oc[i] - p0, e = s_oc[i + 1] - p0;
                int64_t b0 = a > 0 ? (a + 31) >> 5 : 0;
                const int64_t b1 = e > 0 ? ((e - 1) >> 5) : -1;
                for (; b0 <= b1 && b0 < kCopyBlocks; ++b0) s_blk[b0] = (int16_t)i;
            }
            __syncthreads();
            const int last = (int)nr - 1;
            const int nblk = (int)((p1 - p0 + 31) >> 5);
            constexpr int kU = KU;
            for (int64_t pb = p0 + threadIdx.x; pb < p1; pb += kU * (int64_t)blockDim.x) {
                int32_t val[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int64_t p = pb + u * (int64_t)blockDim.x;
                    val[u] = p < p1 ? cc[p] : 0;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int64_t p = pb + u * (int64_t)blockDim.x;
                    if (p >= p1) break;
                    const int b = (int)((p - p0) >> 5);
                    int l = s_blk[b], h = b + 1 < nblk ? s_blk[b + 1] : last;
                    while (l < h) {
                        const int mid = (l + h + 1) >> 1;
                        if (s_oc[mid] <= p)
                            l = mid;
                        else
                            h = mid - 1;
                    }
                    cn[p + s_sh[l]] = val[u];
                }
            }
        } else {
            for (int64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
                const int64_t v = row_of(oc, r0, r1, p);
                cn[on[v] + (p - oc[v])] = cc[p];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && moved) atomicAdd(&A.st->bwd_moved, moved);
}

constexpr int kCopySmemBytes = 8 * (kCopyRows + 1) + 8 * kCopyRows + 2 * kCopyBlocks;

__global__ void __launch_bounds__(256) k_bwd_copy(Arena A) {
    __shared__ int64_t s_oc[kCopyRows + 1];
    __shared__ int64_t s_sh[kCopyRows];
    __shared__ int16_t s_blk[kCopyBlocks];
    d_bwd_copy<8>(A, s_oc, s_sh, s_blk);
}

// One warp per agent: place its edges at new_off[dst] + old_len(dst) + rank.
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
        const int64_t* oc = A.bwd_off_cur + rp.obase;
        const int64_t* on = A.bwd_off_nxt + rp.obase;
        int32_t* cn = A.bwd_col_nxt + rp.ebase;
        for (int64_t e = e0 + lane; e < e1; e += 32) {
            const int32_t j = A.e_dst[e];
            const int64_t old = j < rp.n ? oc[j + 1] - oc[j] : 0;
            cn[on[j] + old + A.e_rank[e]] = src;
        }
    }
}

__global__ void __launch_bounds__(256) k_bwd_place(Arena A, int64_t agents) { d_bwd_place(A, agents); }

__device__ __forceinline__ void seg_bounds(const Arena& A, int64_t slot, const Replica*& rpp,
                                           int64_t& start, int64_t& len) {
    const int r = A.tile_rep[slot / kTile];
    const Replica& rp = A.rep[r];
    rpp = &rp;
    const int64_t v = slot - rp.nbase;
    const int64_t* oc = A.bwd_off_cur + rp.obase;
    const int64_t* on = A.bwd_off_nxt + rp.obase;
    const int64_t old = v < rp.n ? oc[v + 1] - oc[v] : 0;
    start = rp.ebase + on[v] + old;
    len = on[v + 1] - on[v] - old;
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
        const Replica* rp;
        int64_t start, len;
        seg_bounds(A, slot, rp, start, len);
        int32_t* seg = A.bwd_col_nxt + start;
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
        const Replica* rp;
        int64_t start, len;
        seg_bounds(A, slot, rp, start, len);
        int32_t* seg = A.bwd_col_nxt + start;
        const int64_t lo = rp->n, range = rp->delta;
        const int32_t* srcv = seg;
        if (range > kBits) {  // several chunks: keep the input in the spent rank buffer
            int32_t* scratch = A.e_rank + A.sort_large_off[i];
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

__global__ void __launch_bounds__(1024) k_sort_large(Arena A) {
    extern __shared__ uint32_t bm[];
    d_sort_large(A, bm, kBitmapWords);
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
    k_bwd_len<<<A.ntiles, kTileThreads, 0, s>>>(A);
    launch_tile_scan(A, 1, s);
    k_bwd_off<<<A.ntiles, kTileThreads, 0, s>>>(A);
    const int copy_per_sm = A.tune_copy_ctas > 0 ? A.tune_copy_ctas : 8;
    // the old entries' copy and the new entries' placement and sorts write disjoint positions of
    // the next backward CSR: with a side stream they overlap
    const bool two = side && fork && join;
    if (two) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(side, fork, 0);
    }
    k_bwd_copy<<<(unsigned)(num_sms * copy_per_sm), 256, 0, two ? side : s>>>(A);
    if (two) cudaEventRecord(join, side);
    int64_t ga = (agents + 7) / 8;
    if (ga > (int64_t)num_sms * 16) ga = (int64_t)num_sms * 16;
    if (ga < 1) ga = 1;
    k_bwd_place<<<(unsigned)ga, 256, 0, s>>>(A, agents);
    k_sort_small<<<(unsigned)num_sms * 8, 256, 0, s>>>(A);
    k_sort_large<<<(unsigned)num_sms, 1024, kBitmapWords * 4, s>>>(A);
    if (two) cudaStreamWaitEvent(s, join, 0);
    k_epoch_end<<<1, 256, 0, s>>>(A, agents);
}

}  // namespace pg
