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
#include "pg_fmt.cuh"

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


// ---------------------------------------------------------------- the attribute file
// Restates Graph::WriteAttributes (src/graph.cu:1057-1218): one line per node,
//   id,type,year,pa_weight,rec_weight,fit_weight,fit_lag_duration,fit_peak_value,
//   fit_peak_duration,alpha,in_degree,out_degree,assigned_out_degree,planted_line,generators
// with the weights and alpha as "%.10g", the peak as "%d" (refcompat's integer peak) or "%.9g" of
// the fp32 fitness, seeds typed "seed" with "no_generators", agents typed "agent" with their
// generator ids joined by ';' ("-1" when there is none).  Year, fitness and degrees come from the
// arena; the per-paper draws, printed ids and generators from the caller.  Pass 1 measures every
// line (no output buffer), the scan places them, pass 2 writes them.

struct LineOut {
    char* p;  // null: count only
    int n;
    __device__ __forceinline__ void put(char c) {
        if (p) p[n] = c;
        ++n;
    }
    __device__ __forceinline__ void str(const char* s) {
        while (*s) put(*s++);
    }
    __device__ __forceinline__ void dec(int64_t v) {
        const int l = dec_len(v);
        if (p) dec_write(p + n, v, l);
        n += l;
    }
    __device__ __forceinline__ void g(double x, int prec) {
        char b[32];
        const int l = fmt_g(x, prec, b);
        for (int i = 0; i < l; ++i) put(b[i]);
    }
};

__device__ int attr_line(const AttrCols& C, int64_t v, char* p) {
    LineOut o{p, 0};
    const bool seed = v < C.n_seed;
    const double* d = C.draws + v * 4;
    const int32_t* q = C.ints + v * 4;
    o.dec(C.ids[v]);
    o.str(seed ? ",seed," : ",agent,");
    o.dec(C.pub[v]);
    for (int i = 0; i < 3; ++i) {
        o.put(',');
        o.g(d[i], 10);
    }
    o.put(',');
    o.dec(q[0]);
    o.put(',');
    if (C.peak_int)
        o.dec((int64_t)(int32_t)C.fit[v]);
    else
        o.g((double)C.fit[v], 9);
    o.put(',');
    o.dec(q[1]);
    o.put(',');
    o.g(d[3], 10);
    o.put(',');
    o.dec(C.indeg[v]);
    o.put(',');
    o.dec(C.fo[v + 1] - C.fo[v]);
    o.put(',');
    o.dec(q[2]);
    o.put(',');
    o.dec(q[3]);
    o.put(',');
    if (seed) {
        o.str("no_generators");
    } else {
        int k = 0;
        for (int i = 0; i < 4; ++i) {
            const int64_t gid = C.gens[v * 4 + i];
            if (gid < 0) continue;
            if (k++) o.put(';');
            o.dec(gid);
        }
        if (!k) o.str("-1");
    }
    o.put('\n');
    return o.n;
}

__global__ void __launch_bounds__(128) k_attr_len(AttrCols C, int32_t* len) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < C.n; v += (int64_t)gridDim.x * blockDim.x)
        len[v] = attr_line(C, v, nullptr);
}

__global__ void __launch_bounds__(128) k_attr_write(AttrCols C, const int64_t* off, char* out) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < C.n; v += (int64_t)gridDim.x * blockDim.x)
        attr_line(C, v, out + off[v]);
}

void launch_attr_text(const AttrCols& C, int32_t* len, const int64_t* off, char* out, int num_sms,
                      cudaStream_t s) {
    if (C.n <= 0) return;
    int64_t g = (C.n + 127) / 128;
    if (g > (int64_t)num_sms * 16) g = (int64_t)num_sms * 16;
    if (out)
        k_attr_write<<<(unsigned)g, 128, 0, s>>>(C, off, out);
    else
        k_attr_len<<<(unsigned)g, 128, 0, s>>>(C, len);
}

}  // namespace pg

// C's "%.<precision>g" of x (the device attribute writer's conversion, compiled for the host).
extern "C" int32_t pg_format_g_host(double x, int32_t precision, char* out) {
    if (precision < 1) precision = 1;
    if (precision > 13) precision = 13;
    return pg::fmt_g(x, precision, out);
}
