// pg_text.cu -- the edge list as text, formatted on the device (the output writer of the growth
// step).
//
// Restates Graph::WriteGraph (src/graph.cu:909-1003): one "source,target\n" line per edge, sources
// in ascending sequence id, targets ascending within a source, both printed as the caller's
// original ids.  The reference formats on the host threads with std::to_chars; here one pass
// computes every line's length, the engine's scan turns lengths into offsets, and a second pass
// writes the digits, so a 60M-edge graph becomes text in a few milliseconds and leaves the device
// in one copy.
#include "pg_engine.cuh"

namespace pg {

__device__ __forceinline__ int dec_len(int64_t v) {
    uint64_t u = v < 0 ? (uint64_t)(-(v + 1)) + 1u : (uint64_t)v;
    int n = v < 0 ? 1 : 0;
    do {
        ++n;
        u /= 10u;
    } while (u);
    return n;
}

// writes the decimal text of v into p[0, len)
__device__ __forceinline__ void dec_write(char* p, int64_t v, int len) {
    uint64_t u = v < 0 ? (uint64_t)(-(v + 1)) + 1u : (uint64_t)v;
    int i = len - 1;
    do {
        p[i--] = (char)('0' + (int)(u % 10u));
        u /= 10u;
    } while (u);
    if (v < 0) p[0] = '-';
}

// source of edge e: the last row whose start is at or before e
__device__ __forceinline__ int64_t edge_source(const int64_t* fo, int64_t n, int64_t e) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (fo[mid] <= e)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_text_len(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m,
                                                  const int64_t* ids, int32_t* len) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = edge_source(fo, n, e);
        len[e] = dec_len(ids[s]) + dec_len(ids[fc[e]]) + 2;
    }
}

__global__ void __launch_bounds__(256) k_text_write(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m,
                                                    const int64_t* ids, const int64_t* off, char* out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = edge_source(fo, n, e);
        const int64_t a = ids[s], b = ids[fc[e]];
        const int la = dec_len(a), lb = dec_len(b);
        char* p = out + off[e];
        dec_write(p, a, la);
        p[la] = ',';
        dec_write(p + la + 1, b, lb);
        p[la + 1 + lb] = '\n';
    }
}

// Sources of the edges [first, first + count): one thread per row writes the row's part of the
// range (rows are contiguous in edge order, so the writes of neighbouring rows are adjacent).
__global__ void __launch_bounds__(256) k_edge_sources(const int64_t* fo, int64_t n, int64_t first, int64_t count,
                                                      int32_t* out) {
    const int64_t last = first + count;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        int64_t p0 = fo[v], p1 = fo[v + 1];
        if (p1 <= first || p0 >= last) continue;
        p0 = p0 > first ? p0 : first;
        p1 = p1 < last ? p1 : last;
        for (int64_t p = p0; p < p1; ++p) out[p - first] = (int32_t)v;
    }
}

void launch_edge_sources(const int64_t* fo, int64_t n, int64_t first, int64_t count, int32_t* out,
                         int num_sms, cudaStream_t s) {
    if (count <= 0 || n <= 0) return;
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)num_sms * 16) g = (int64_t)num_sms * 16;
    k_edge_sources<<<(unsigned)g, 256, 0, s>>>(fo, n, first, count, out);
}

void launch_text_len(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m, const int64_t* ids, int32_t* len,
                     int num_sms, cudaStream_t s) {
    if (m <= 0) return;
    int64_t g = (m + 255) / 256;
    if (g > (int64_t)num_sms * 16) g = (int64_t)num_sms * 16;
    k_text_len<<<(unsigned)g, 256, 0, s>>>(fo, fc, n, m, ids, len);
}

void launch_text_write(const int64_t* fo, const int32_t* fc, int64_t n, int64_t m, const int64_t* ids,
                       const int64_t* off, char* out, int num_sms, cudaStream_t s) {
    if (m <= 0) return;
    int64_t g = (m + 255) / 256;
    if (g > (int64_t)num_sms * 16) g = (int64_t)num_sms * 16;
    k_text_write<<<(unsigned)g, 256, 0, s>>>(fo, fc, n, m, ids, off, out);
}

}  // namespace pg
