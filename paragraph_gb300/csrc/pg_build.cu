// pg_build.cu -- device construction of a replica's forward and backward CSR from a raw edge list.
//
// Replaces the reference's seed load (Graph::ParseEdgelist / AddEdge into std::map<int,
// std::set<int>>, src/graph.cu:376-447,820-826, then prepareGraph's int32 CSR, src/utils.cu:75-142)
// with a device pipeline, so a load costs one upload of the raw (source, target) arrays:
//   k_edge_keys     key = source << b | target (b = bits of n - 1), ids checked against [0, n)
//   radix passes    stable LSD radix sort of the keys, 8-bit digits over the 2b key bits
//                   (per pass: tile histograms, one scan over [digit][tile], stable scatter)
//   k_unique_*      duplicates collapse (Graph::AddEdge set semantics), forward columns and
//                   per-source counts; counts -> int64 offsets by the engine's scan
//   radix passes    the keys stably re-sorted on the target field only, which orders the unique
//                   ones by (target, source) and puts the duplicates (marked) last: backward
//                   columns and in-degrees.
// Nothing is read back on the way: the unique count stays on the device (u_dev) and bounds the
// later kernels there, so the replicas of a context are built one after another without a host
// synchronisation.
// Rows come out ascending, as the reference's std::set rows.  Every step is integer work, so the
// result equals the host construction bit for bit.
#include <algorithm>

#include "pg_engine.cuh"

namespace pg {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortTile = kSortThreads * 16;  // keys per CTA

__global__ void __launch_bounds__(256) k_edge_keys(const int32_t* src, const int32_t* dst, int64_t m,
                                                   int64_t n, int bits, unsigned long long* keys,
                                                   uint32_t* err) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = src[i], d = dst[i];
        if (s < 0 || s >= n || d < 0 || d >= n) {
            atomicOr(err, kErrArg);
            keys[i] = 0ull;
            continue;
        }
        keys[i] = ((unsigned long long)s << bits) | (unsigned long long)d;
    }
}

// Digit histogram of each tile, written digit-major: hist[d * tiles + t].
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const unsigned long long* keys, int64_t m, int shift,
                                                             int dmask, int64_t tiles, int64_t* hist) {
    __shared__ int h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += kSortThreads) h[i] = 0;
    __syncthreads();
    const int64_t t = blockIdx.x;
    const int64_t base = t * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        const int64_t k = base + i;
        if (k < m) atomicAdd(&h[(int)((keys[k] >> shift) & dmask)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kSortThreads) hist[(int64_t)d * tiles + t] = h[d];
}

// Stable scatter: key k of tile t with digit d goes to off[d * tiles + t] + (number of earlier keys
// of the tile with digit d).  Each warp owns a contiguous segment of the tile (kSortPerLane keys per
// lane, walked 32 at a time in order).  First pass: the warp counts its segment's digits (match:
// the leader of each group of equal digits adds the group's size).  After one barrier the counts
// become each (warp, digit) run's start in the tile's digit order (the exclusive scan of the tile's
// digit counts, then the earlier warps').  Second pass: the warp walks its segment again (the keys
// come from L1/L2) and places each key at its run's running position plus its place in the group,
// in shared memory.  The runs are then written out in tile order, consecutive threads writing
// consecutive keys of a run (coalesced).
constexpr int kSortPerLane = kSortTile / kSortThreads;  // 16
static_assert(kSortThreads == kRadix, "one thread per digit in the run-start scan");
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned long long* keys, int64_t m,
                                                                int shift, int dmask, int64_t tiles,
                                                                const int64_t* off, unsigned long long* out) {
    constexpr int W = kSortThreads / 32;
    __shared__ unsigned long long tile[kSortTile];  // the tile's keys in digit order
    __shared__ int64_t gbase[kRadix];               // global position of the digit's run minus its start
    __shared__ int wcnt[W][kRadix];                 // per warp: digit counts, then running positions
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t t = blockIdx.x;
    const int64_t base = t * kSortTile;
    const int cnt = (int)(m - base < kSortTile ? m - base : kSortTile);
    const int seg = warp * 32 * kSortPerLane;
    const unsigned below = (1u << lane) - 1u;
    for (int i = threadIdx.x; i < W * kRadix; i += kSortThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    for (int j = 0; j < kSortPerLane; ++j) {
        const int q = seg + 32 * j + lane;
        const int d = q < cnt ? (int)((keys[base + q] >> shift) & dmask) : kRadix;  // kRadix: no digit
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (d < kRadix && lane == __ffs(peers) - 1) wcnt[warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // run starts: digit d's run of warp w begins at (keys of digits < d) + (keys of digit d in warps
    // < w); one thread per digit, the digits' totals scanned by the first warp's shuffles
    {
        const int d = threadIdx.x;  // kSortThreads == kRadix
        int tot = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) tot += wcnt[w][d];
        // exclusive scan of tot over the 256 digits: per-warp shuffle scan, then the warps' sums
        int incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        __shared__ int wsum[W];
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        int prior = 0;
        for (int w = 0; w < warp; ++w) prior += wsum[w];
        int acc = prior + incl - tot;  // this digit's start in the tile's digit order
        gbase[d] = off[(int64_t)d * tiles + t] - acc;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            const int c = wcnt[w][d];
            wcnt[w][d] = acc;
            acc += c;
        }
    }
    __syncthreads();
    for (int j = 0; j < kSortPerLane; ++j) {
        const int q = seg + 32 * j + lane;
        const bool valid = q < cnt;
        const unsigned long long key = valid ? keys[base + q] : 0ull;
        const int d = valid ? (int)((key >> shift) & dmask) : kRadix;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        int pos = 0;
        if (valid && lane == leader) {
            pos = wcnt[warp][d];
            wcnt[warp][d] = pos + __popc(peers);
        }
        pos = __shfl_sync(0xffffffffu, pos, leader);
        if (valid) tile[pos + __popc(peers & below)] = key;
        __syncwarp();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < cnt; i += kSortThreads) {
        const unsigned long long key = tile[i];
        out[gbase[(int)((key >> shift) & dmask)] + i] = key;
    }
}

// flag[i] = 1 when key i differs from key i-1 (the first of a run of duplicates)
__global__ void __launch_bounds__(256) k_unique_flags(const unsigned long long* keys, int64_t m, int32_t* flag) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// The unique keys (sorted by source, then target) as forward columns, and the edges of every source.
// fsrc (may be null): the source of every unique edge, for the callers that lay rows out per entry.
__global__ void __launch_bounds__(256) k_unique_compact(const unsigned long long* keys, int64_t m, const int32_t* flag,
                                                        const int64_t* pos, int bits, int32_t* fcol, int32_t* fcnt,
                                                        int32_t* fsrc) {
    const unsigned long long mask = (1ull << bits) - 1ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[i]) continue;
        const unsigned long long k = keys[i];
        const int64_t p = pos[i];
        fcol[p] = (int32_t)(k & mask);
        if (fsrc) fsrc[p] = (int32_t)(k >> bits);
        atomicAdd(&fcnt[(int64_t)(k >> bits)], 1);
    }
}

// Keys for the backward sort, one per sorted key: a unique edge as source << (bits + 1) | target,
// a duplicate as all ones, whose low bits + 1 bits exceed every target, so it sorts last.
__global__ void __launch_bounds__(256) k_backward_keys(const unsigned long long* keys, int64_t m, const int32_t* flag,
                                                       int bits, unsigned long long* bkeys) {
    const unsigned long long mask = (1ull << bits) - 1ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        bkeys[i] = flag[i] ? (((k >> bits) << (bits + 1)) | (k & mask)) : ~0ull;
    }
}

// Keys sorted by (target, source), the u_dev unique ones first: backward columns (sources) and
// per-target counts; btgt (may be null): the target of every backward entry.
__global__ void __launch_bounds__(256) k_backward_cols(const unsigned long long* keys, const int64_t* u_dev, int bits,
                                                       int32_t* bcol, int32_t* bcnt, int32_t* btgt) {
    const unsigned long long mask = (1ull << (bits + 1)) - 1ull;
    const int64_t u = *u_dev;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < u; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[i];
        bcol[i] = (int32_t)(k >> (bits + 1));
        if (btgt) btgt[i] = (int32_t)(k & mask);
        atomicAdd(&bcnt[(int64_t)(k & mask)], 1);
    }
}

// Index of the first edge with an endpoint outside [0, n) (atomic minimum; ~0 when none).
__global__ void __launch_bounds__(256) k_first_bad_edge(const int32_t* src, const int32_t* dst, int64_t m, int64_t n,
                                                        unsigned long long* first) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        if ((uint32_t)src[i] >= (uint32_t)n || (uint32_t)dst[i] >= (uint32_t)n) atomicMin(first, (unsigned long long)i);
}

void launch_first_bad_edge(const int32_t* src, const int32_t* dst, int64_t m, int64_t n, unsigned long long* first,
                           cudaStream_t s) {
    cudaMemsetAsync(first, 0xFF, sizeof(unsigned long long), s);
    if (m <= 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>((m + 255) / 256, 152 * 16);
    k_first_bad_edge<<<grid, 256, 0, s>>>(src, dst, m, n, first);
}

// Many edge lists at once: list r is [off[r], off[r + 1]) of the staging arrays src/dst, with ids
// below nodes[r]; its source and target arrays are at ptr[2 r] and ptr[2 r + 1] -- page-locked host
// memory mapped into the device's address space (read here directly, over the host link) or the
// staging arrays themselves (already copied there).  Every edge is written to the staging arrays
// and its endpoints are checked; first[r] receives the first bad index of list r, relative to
// off[r] (~0 when none).
__global__ void __launch_bounds__(256) k_gather_edges(const int64_t* off, const int64_t* nodes, const int64_t* ptr,
                                                      int R, int32_t* src, int32_t* dst, unsigned long long* first) {
    const int64_t m = off[R];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = R - 1;  // the last list starting at or before i
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= i)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int64_t j = i - off[lo];
        const int32_t s = reinterpret_cast<const int32_t*>(ptr[2 * lo])[j];
        const int32_t d = reinterpret_cast<const int32_t*>(ptr[2 * lo + 1])[j];
        src[i] = s;
        dst[i] = d;
        const uint32_t n = (uint32_t)nodes[lo];
        if ((uint32_t)s >= n || (uint32_t)d >= n) atomicMin(&first[lo], (unsigned long long)j);
    }
}

void launch_gather_edges(int64_t m, const int64_t* off, const int64_t* nodes, const int64_t* ptr, int R, int32_t* src,
                         int32_t* dst, unsigned long long* first, cudaStream_t s) {
    cudaMemsetAsync(first, 0xFF, sizeof(unsigned long long) * (size_t)R, s);
    if (m <= 0) return;
    const unsigned grid = (unsigned)std::min<int64_t>((m + 255) / 256, 152 * 16);
    k_gather_edges<<<grid, 256, 0, s>>>(off, nodes, ptr, R, src, dst, first);
}

int64_t build_radix_tiles(int64_t m) { return (m + kSortTile - 1) / kSortTile; }
int64_t build_scan_entries(int64_t m) { return build_radix_tiles(m) * kRadix; }

// One stable pass on the `width` (<= 8) key bits from `shift`; `hist`/`off` hold kRadix * tiles
// (+1) entries.
static void radix_pass(const unsigned long long* in, unsigned long long* out, int64_t m, int shift, int width,
                       int64_t* hist, int64_t* off, int64_t* blocksum, cudaStream_t s) {
    const int64_t tiles = build_radix_tiles(m);
    const int dmask = (1 << width) - 1;
    k_radix_hist<<<(unsigned)tiles, kSortThreads, 0, s>>>(in, m, shift, dmask, tiles, hist);
    launch_scan_i64(hist, off, tiles * kRadix, blocksum, s);
    k_radix_scatter<<<(unsigned)tiles, kSortThreads, 0, s>>>(in, m, shift, dmask, tiles, off, out);
}

// Sorts keys[0..m) stably on bits [lo, hi) (8-bit digits from lo); tmp is a second buffer of m keys.
// Returns the buffer holding the result (keys or tmp).
static unsigned long long* radix_sort(unsigned long long* keys, unsigned long long* tmp, int64_t m, int lo, int hi,
                                      int64_t* hist, int64_t* off, int64_t* blocksum, cudaStream_t s) {
    unsigned long long* a = keys;
    unsigned long long* b = tmp;
    for (int sh = lo; sh < hi; sh += kRadixBits) {
        // the last digit stops at bit hi: the bits above it belong to another field of the key
        radix_pass(a, b, m, sh, hi - sh < kRadixBits ? hi - sh : kRadixBits, hist, off, blocksum, s);
        unsigned long long* t = a;
        a = b;
        b = t;
    }
    return a;
}

// The scratch the build needs for m raw edges (bytes), for the caller's allocation.
size_t build_scratch_bytes(int64_t m, int64_t n) {
    const int64_t e = m > 0 ? m : 1;
    const int64_t scan = build_scan_entries(e) + 1;
    return (size_t)(3 * e) * 8 + (size_t)e * 4 + (size_t)(e + 1) * 8 + (size_t)(2 * scan) * 8 +
           (size_t)(n + 1) * 4 * 2 + (size_t)(scan_blocks_needed(std::max<int64_t>(std::max<int64_t>(scan, e + 1), n + 1)) + 2) * 8 +
           16 * 256;
}

// Builds replica CSRs on the device.  src/dst: m raw device edges; outputs: fo/fc/bo/bc (the
// replica's regions), indeg (n entries), the number of unique edges in *u_dev (device memory; bo[n]
// holds it too).  Scratch layout is carved from `scratch`.
void launch_build_csr(const int32_t* src, const int32_t* dst, int64_t m, int64_t n, void* scratch,
                      int64_t* fo, int32_t* fc, int64_t* bo, int32_t* bc, int32_t* indeg, int64_t* u_dev,
                      uint32_t* err, cudaStream_t s, int32_t* fsrc, int32_t* btgt) {
    const int64_t e = m > 0 ? m : 1;
    const int64_t scan = build_scan_entries(e) + 1;
    char* p = reinterpret_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        char* q = p;
        p += (bytes + 255) & ~(size_t)255;
        return q;
    };
    unsigned long long* k0 = reinterpret_cast<unsigned long long*>(take((size_t)e * 8));
    unsigned long long* k1 = reinterpret_cast<unsigned long long*>(take((size_t)e * 8));
    unsigned long long* uk = reinterpret_cast<unsigned long long*>(take((size_t)e * 8));
    int32_t* flag = reinterpret_cast<int32_t*>(take((size_t)e * 4));
    int64_t* pos = reinterpret_cast<int64_t*>(take((size_t)(e + 1) * 8));
    int64_t* hist = reinterpret_cast<int64_t*>(take((size_t)scan * 8));
    int64_t* off = reinterpret_cast<int64_t*>(take((size_t)scan * 8));
    int32_t* fcnt = reinterpret_cast<int32_t*>(take((size_t)(n + 1) * 4));
    int32_t* bcnt = reinterpret_cast<int32_t*>(take((size_t)(n + 1) * 4));
    int64_t* blocksum = reinterpret_cast<int64_t*>(
        take((size_t)(scan_blocks_needed(std::max<int64_t>(std::max<int64_t>(scan, e + 1), n + 1)) + 2) * 8));
    int bits = 1;
    while (bits < 31 && ((int64_t)1 << bits) < n) ++bits;
    cudaMemsetAsync(fcnt, 0, (size_t)(n + 1) * 4, s);
    cudaMemsetAsync(bcnt, 0, (size_t)(n + 1) * 4, s);
    const unsigned grid = (unsigned)std::min<int64_t>((e + 255) / 256, 152 * 16);
    if (m > 0) {
        k_edge_keys<<<grid, 256, 0, s>>>(src, dst, m, n, bits, k0, err);
        unsigned long long* sorted = radix_sort(k0, k1, m, 0, 2 * bits, hist, off, blocksum, s);
        k_unique_flags<<<grid, 256, 0, s>>>(sorted, m, flag);
        launch_scan_i32_to_i64(flag, pos, m, blocksum, s);
        k_unique_compact<<<grid, 256, 0, s>>>(sorted, m, flag, pos, bits, fc, fcnt, fsrc);
        cudaMemcpyAsync(u_dev, pos + m, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);  // unique edges
        k_backward_keys<<<grid, 256, 0, s>>>(sorted, m, flag, bits, uk);
        unsigned long long* other = sorted == k0 ? k1 : k0;
        unsigned long long* bsorted = radix_sort(uk, other, m, 0, bits + 1, hist, off, blocksum, s);
        k_backward_cols<<<grid, 256, 0, s>>>(bsorted, u_dev, bits, bc, bcnt, btgt);
    } else {
        cudaMemsetAsync(u_dev, 0, sizeof(int64_t), s);
    }
    launch_scan_i32_to_i64(fcnt, fo, n, blocksum, s);
    launch_scan_i32_to_i64(bcnt, bo, n, blocksum, s);
    cudaMemcpyAsync(indeg, bcnt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
}

// ---------------------------------------------------------------- growable backward rows
// The engine keeps backward rows with room to grow (BRow).  From a backward CSR in offset form
// (bo: n + 1 offsets, bc: its columns) and the forward offsets fo, row v of length L > 0 gets a span
// of brow_span(L, P) entries, P = fwd_prefix(out-degree), at the exclusive scan of the spans: its
// forward row copy ends at the span start + P (= 4 beg4), its backward entries follow.  A row with
// no backward entry gets no span.
__global__ void __launch_bounds__(256) k_brow_caps(const int64_t* bo, const int64_t* fo, int64_t n, int64_t* caps) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t len = bo[v + 1] - bo[v];
        caps[v] = len > 0 ? brow_span(len, fwd_prefix(fo[v + 1] - fo[v])) : 0;
    }
}

__global__ void __launch_bounds__(256) k_brow_rows(const int64_t* bo, const int64_t* fo, const int64_t* begs, int64_t n,
                                                   BRow* brow, int32_t* bcap) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t len = bo[v + 1] - bo[v];
        const int64_t P = len > 0 ? fwd_prefix(fo[v + 1] - fo[v]) : 0;
        BRow r;
        r.beg4 = len > 0 ? (uint32_t)((begs[v] + P) >> 2) : 0u;
        r.len = (int32_t)len;
        brow[v] = r;
        bcap[v] = (int32_t)(len > 0 ? begs[v + 1] - begs[v] - P : 0);
    }
}

// entry p of the offset form goes to its row's span: the row is the last v with bo[v] <= p (bo[n],
// the entry count, is read on the device; m only bounds it)
__global__ void __launch_bounds__(256) k_brow_cols(const int64_t* bo, const int32_t* bc, const BRow* brow,
                                                   int64_t n, int64_t m, int32_t* out) {
    const int64_t mm = bo[n] < m ? bo[n] : m;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < mm; p += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = n - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (bo[mid] <= p)
                lo = mid;
            else
                hi = mid - 1;
        }
        out[((int64_t)brow[lo].beg4 << 2) + (p - bo[lo])] = bc[p];
    }
}

// the forward row copies in front of the laid-out rows: one warp per node with a span
__global__ void __launch_bounds__(256) k_brow_prefix(const int64_t* fo, const int32_t* fc, const BRow* brow, int64_t n,
                                                     int32_t* out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < n; v += nwarps) {
        const BRow r = brow[v];
        if (r.len <= 0) continue;
        const int64_t f0 = fo[v], o = fo[v + 1] - f0;
        int32_t* dst = out + ((int64_t)r.beg4 << 2) - o;
        for (int64_t i = lane; i < o; i += 32) dst[i] = fc[f0 + i];
    }
}

// the same two copies when the CSR build gave every entry its row: backward entry i belongs to row
// btgt[i], forward entry p to row fsrc[p] (no search)
__global__ void __launch_bounds__(256) k_brow_cols_rows(const int64_t* bo, const int32_t* bc, const int32_t* btgt,
                                                        const BRow* brow, int64_t n, int64_t m, int32_t* out) {
    const int64_t u = bo[n] < m ? bo[n] : m;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < u; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = btgt[i];
        out[((int64_t)brow[v].beg4 << 2) + (i - bo[v])] = bc[i];
    }
}

__global__ void __launch_bounds__(256) k_brow_prefix_rows(const int64_t* fo, const int32_t* fc, const int32_t* fsrc,
                                                          const BRow* brow, int64_t n, int64_t m, int32_t* out) {
    const int64_t u = fo[n] < m ? fo[n] : m;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < u; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = fsrc[p];
        const BRow r = brow[v];
        if (r.len <= 0) continue;
        const int64_t f0 = fo[v], o = fo[v + 1] - f0;
        out[((int64_t)r.beg4 << 2) - o + (p - f0)] = fc[p];
    }
}

void launch_brow_layout(const int64_t* bo, const int32_t* bc, const int64_t* fo, const int32_t* fc, int64_t n,
                        int64_t m, int64_t* caps, int64_t* begs, int64_t* blocksum, BRow* brow, int32_t* bcap,
                        int32_t* bcol, cudaStream_t s, const int32_t* fsrc, const int32_t* btgt) {
    if (n <= 0) return;
    const unsigned gn = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
    k_brow_caps<<<gn, 256, 0, s>>>(bo, fo, n, caps);
    launch_scan_i64(caps, begs, n, blocksum, s);
    k_brow_rows<<<gn, 256, 0, s>>>(bo, fo, begs, n, brow, bcap);
    if (m > 0) {
        const unsigned gm = (unsigned)std::min<int64_t>((m + 255) / 256, 152 * 16);
        if (btgt)
            k_brow_cols_rows<<<gm, 256, 0, s>>>(bo, bc, btgt, brow, n, m, bcol);
        else
            k_brow_cols<<<gm, 256, 0, s>>>(bo, bc, brow, n, m, bcol);
        if (fsrc) {
            k_brow_prefix_rows<<<gm, 256, 0, s>>>(fo, fc, fsrc, brow, n, m, bcol);
        } else {
            const unsigned gw = (unsigned)std::min<int64_t>((n + 7) / 8, 152 * 16);
            k_brow_prefix<<<gw, 256, 0, s>>>(fo, fc, brow, n, bcol);
        }
    }
}

// ---------------------------------------------------------------- all replicas in one build
// A context of many replicas builds its seeds as ONE graph over the arena's node slots: every raw
// edge is rewritten to slot ids (replica base + node), the whole edge list goes through the build
// above once (keys of slot ids never collide across replicas), and the result is cut into the
// replicas' regions: forward offsets relative to each replica's first slot, forward columns at the
// replica's edge region, backward rows laid out per replica region (each replica's rows packed from
// the start of its region, as a build per replica would), in-degrees straight into the slot array.
// A few dozen launches in all instead of a few dozen per replica.

// raw edges [off[r], off[r+1]) belong to replica r: ids += the replica's first slot
__global__ void __launch_bounds__(256) k_raw_to_slots(int32_t* src, int32_t* dst, int64_t m, const int64_t* off, int R,
                                                      const Replica* rep) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < m; g += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = R - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= g)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int32_t nb = (int32_t)rep[lo].nbase;
        src[g] += nb;
        dst[g] += nb;
    }
}

// forward offsets of every replica from the slot-wide ones
__global__ void __launch_bounds__(256) k_fwd_offsets(const int64_t* go, int64_t S, const int32_t* tile_rep,
                                                     const Replica* rep, int64_t* fwd_off) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (int64_t)gridDim.x * blockDim.x) {
        const Replica& rp = rep[tile_rep[s / kTile]];
        const int64_t v = s - rp.nbase;
        if (v <= rp.n) fwd_off[rp.obase + v] = go[s] - go[rp.nbase];
    }
}

// forward columns: unique edge p (slot-wide order) to its replica's edge region, as a local id
__global__ void __launch_bounds__(256) k_fwd_columns(const int64_t* go, const int32_t* gc, int64_t S, int64_t m,
                                                     const int32_t* tile_rep, const Replica* rep, int32_t* fwd_col) {
    const int64_t u = go[S] < m ? go[S] : m;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < u; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = gc[p];
        const Replica& rp = rep[tile_rep[d / kTile]];
        fwd_col[rp.ebase + (p - go[rp.nbase])] = d - (int32_t)rp.nbase;
    }
}

// backward rows of every slot: the span starts relative to the replica's first slot's, the forward
// row copy (prefix P) first
__global__ void __launch_bounds__(256) k_brow_rows_all(const int64_t* bo, const int64_t* go, const int64_t* gbeg,
                                                       int64_t S, const int32_t* tile_rep, const Replica* rep,
                                                       BRow* brow, int32_t* bcap) {
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < S; s += (int64_t)gridDim.x * blockDim.x) {
        const Replica& rp = rep[tile_rep[s / kTile]];
        const int64_t len = bo[s + 1] - bo[s];
        const int64_t P = len > 0 ? fwd_prefix(go[s + 1] - go[s]) : 0;
        BRow r;
        r.beg4 = len > 0 ? (uint32_t)((gbeg[s] - gbeg[rp.nbase] + P) >> 2) : 0u;
        r.len = (int32_t)len;
        brow[s] = r;
        bcap[s] = (int32_t)(len > 0 ? gbeg[s + 1] - gbeg[s] - P : 0);
    }
}

// forward row copies of every slot with a span, one thread per unique forward edge p (slot-wide
// order; fsrc[p] its source slot, gc[p] its target slot, made local)
__global__ void __launch_bounds__(256) k_brow_prefix_all(const int64_t* go, const int32_t* gc, const int32_t* fsrc,
                                                         const BRow* brow, int64_t S, int64_t m,
                                                         const int32_t* tile_rep, const Replica* rep, int32_t* bcol) {
    const int64_t u = go[S] < m ? go[S] : m;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < u; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sl = fsrc[p];
        const BRow r = brow[sl];
        if (r.len <= 0) continue;
        const Replica& rp = rep[tile_rep[sl / kTile]];
        const int64_t f0 = go[sl], o = go[sl + 1] - f0;
        bcol[rp.bbase + ((int64_t)r.beg4 << 2) - o + (p - f0)] = gc[p] - (int32_t)rp.nbase;
    }
}

// backward entry i (slot-wide order) of the row of slot btgt[i]
__global__ void __launch_bounds__(256) k_brow_cols_all(const int64_t* bo, const int32_t* bc, const int32_t* btgt,
                                                       const BRow* brow, int64_t S, int64_t m, const int32_t* tile_rep,
                                                       const Replica* rep, int32_t* bcol) {
    const int64_t u = bo[S] < m ? bo[S] : m;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < u; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sl = btgt[i];
        const Replica& rp = rep[tile_rep[sl / kTile]];
        bcol[rp.bbase + ((int64_t)brow[sl].beg4 << 2) + (i - bo[sl])] = bc[i] - (int32_t)rp.nbase;
    }
}

// per replica: unique edges and backward entries laid out
__global__ void k_rep_totals(const int64_t* go, const int64_t* gbeg, int R, const Replica* rep, int64_t* u,
                             int64_t* laid) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const Replica& rp = rep[r];
        u[r] = go[rp.nbase + rp.n_cap] - go[rp.nbase];
        laid[r] = gbeg[rp.nbase + rp.n_cap] - gbeg[rp.nbase];
    }
}

size_t build_all_scratch_bytes(int64_t m, int64_t S) {
    // the pieces launch_build_all carves, each rounded up to 256 bytes
    return build_scratch_bytes(m, S) + (size_t)(S + 1) * 8 * 4 + (size_t)(m > 0 ? m : 1) * 4 * 4 + 8 +
           (size_t)(scan_blocks_needed(S + 1) + 2) * 8 + 256 * 12;
}

void launch_build_all(int32_t* src, int32_t* dst, int64_t m, const int64_t* raw_off, int R, int64_t S,
                      const int32_t* tile_rep, const Replica* rep, void* scratch, int64_t* fwd_off, int32_t* fwd_col,
                      BRow* brow, int32_t* bcap, int32_t* bcol, int32_t* indeg, int64_t* u, int64_t* laid, uint32_t* err,
                      cudaStream_t s) {
    char* p = reinterpret_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        char* q = p;
        p += (bytes + 255) & ~(size_t)255;
        return q;
    };
    const int64_t e = m > 0 ? m : 1;
    int64_t* go = reinterpret_cast<int64_t*>(take((size_t)(S + 1) * 8));
    int64_t* bo = reinterpret_cast<int64_t*>(take((size_t)(S + 1) * 8));
    int64_t* caps = reinterpret_cast<int64_t*>(take((size_t)(S + 1) * 8));
    int64_t* gbeg = reinterpret_cast<int64_t*>(take((size_t)(S + 1) * 8));
    int32_t* gc = reinterpret_cast<int32_t*>(take((size_t)e * 4));
    int32_t* bc = reinterpret_cast<int32_t*>(take((size_t)e * 4));
    int32_t* fsrc = reinterpret_cast<int32_t*>(take((size_t)e * 4));
    int32_t* btgt = reinterpret_cast<int32_t*>(take((size_t)e * 4));
    int64_t* ucount = reinterpret_cast<int64_t*>(take(8));
    void* inner = take(build_scratch_bytes(m, S));
    int64_t* blocksum = reinterpret_cast<int64_t*>(take((size_t)(scan_blocks_needed(S + 1) + 2) * 8));
    const unsigned gm = (unsigned)std::min<int64_t>((e + 255) / 256, 152 * 16);
    const unsigned gs = (unsigned)std::min<int64_t>((S + 255) / 256, 152 * 16);
    if (m > 0) k_raw_to_slots<<<gm, 256, 0, s>>>(src, dst, m, raw_off, R, rep);
    launch_build_csr(src, dst, m, S, inner, go, gc, bo, bc, indeg, ucount, err, s, fsrc, btgt);
    k_fwd_offsets<<<gs, 256, 0, s>>>(go, S, tile_rep, rep, fwd_off);
    if (m > 0) k_fwd_columns<<<gm, 256, 0, s>>>(go, gc, S, m, tile_rep, rep, fwd_col);
    k_brow_caps<<<gs, 256, 0, s>>>(bo, go, S, caps);
    launch_scan_i64(caps, gbeg, S, blocksum, s);
    k_brow_rows_all<<<gs, 256, 0, s>>>(bo, go, gbeg, S, tile_rep, rep, brow, bcap);
    if (m > 0) {
        k_brow_cols_all<<<gm, 256, 0, s>>>(bo, bc, btgt, brow, S, m, tile_rep, rep, bcol);
        k_brow_prefix_all<<<gm, 256, 0, s>>>(go, gc, fsrc, brow, S, m, tile_rep, rep, bcol);
    }
    k_rep_totals<<<1, 256, 0, s>>>(go, gbeg, R, rep, u, laid);
}

}  // namespace pg
