// pg_noalloc.cu -- G(n,p) edge generation that allocates no device memory.
//
// Some callers cannot allocate device memory when they call this library -- for instance a host
// program that must not call cudaMalloc while other work on the device is being timed or captured,
// or a runtime that hands out pre-sized buffers and forbids allocation inside its callbacks.  For
// them this file provides one entry point that generates an Erdos-Renyi epoch's edge list into
// buffers the caller already owns.  Its only scratch (per-task edge counts, their exclusive scan
// and the scan's block sums, each in its own region) lives in a fixed file-scope __device__ array,
// so no cudaMalloc, cudaFree or allocating library routine is ever called.
//
// The edges are the ones pg_er_epoch appends for the same (seed, epoch, n_existing, delta, p):
// the same Philox streams, the same 2^16-id chunks, the same library log, the same
// (source, target) order.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>

#include "../../include/paragraph_gb300.h"
#include "pg_engine.cuh"

namespace pg {
namespace {

constexpr int64_t kNoAllocMaxTasks = PG_NOALLOC_MAX_TASKS;
constexpr int64_t kNoAllocBlocks = (kNoAllocMaxTasks + 1023) / 1024 + 2;

// Three regions: per-task counts [kNoAllocMaxTasks], their exclusive scan [kNoAllocMaxTasks + 1]
// (entry [tasks] = total) and the scan's block sums.  Every GPU that loads the library holds this
// array (about 4 MiB) until the process exits.
constexpr int64_t kNoAllocWords = 2 * kNoAllocMaxTasks + 1 + kNoAllocBlocks;
static __device__ __align__(256) int64_t g_noalloc_scratch[kNoAllocWords];

// Device address of the array, looked up once per device; several host threads may call.
std::atomic<int64_t*> g_scratch_addr[64] = {};

__device__ __forceinline__ int64_t walk(uint64_t seed, uint32_t ep, int64_t i, int64_t c, int64_t n,
                                        const ErSkip& K, int64_t src, int32_t* out_src,
                                        int32_t* out_dst, int64_t base) {
    const int64_t lo = c * kErChunk;
    const int64_t hi = lo + kErChunk < n ? lo + kErChunk : n;
    int64_t pos = lo - 1, cnt = 0;
    u32x4 x;
    x.x[0] = x.x[1] = x.x[2] = x.x[3] = 0;
    for (uint32_t d = 0;; ++d) {
        if ((d & 1u) == 0) x = draw(seed, kStreamEr, (uint32_t)c, ep, (uint32_t)i, d >> 1);
        const double rem = (double)(hi - pos - 1);
        const double sk = (d & 1u) ? er_skip(K, x.x[2], x.x[3], (float)rem) : er_skip(K, x.x[0], x.x[1], (float)rem);
        if (sk >= rem) break;
        pos = pos + 1 + (int64_t)sk;
        if (out_dst) {
            out_src[base + cnt] = (int32_t)src;
            out_dst[base + cnt] = (int32_t)pos;
        }
        ++cnt;
    }
    return cnt;
}

__global__ void __launch_bounds__(256) k_na_count(uint64_t seed, uint32_t ep, int64_t n,
                                                  int64_t tasks, int64_t chunks, ErSkip K,
                                                  int64_t* cnt) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tasks;
         t += (int64_t)gridDim.x * blockDim.x)
        cnt[t] = walk(seed, ep, t / chunks, t % chunks, n, K, 0, nullptr, nullptr, 0);
}

__global__ void __launch_bounds__(256) k_na_emit(uint64_t seed, uint32_t ep, int64_t n,
                                                 int64_t tasks, int64_t chunks, ErSkip K,
                                                 const int64_t* off, int32_t* src, int32_t* dst) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < tasks;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / chunks;
        walk(seed, ep, i, t % chunks, n, K, n + i, src, dst, off[t]);
    }
}

// Device address of the scratch array for the current device (set up once per device).
pg_status scratch_for_current_device(int64_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PG_ERR_CUDA;
    int64_t* a = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!a) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PG_ERR_CUDA;
        a = static_cast<int64_t*>(p);
        g_scratch_addr[dev].store(a, std::memory_order_release);  // every thread stores the same value
    }
    *out = a;
    return PG_OK;
}

}  // namespace
}  // namespace pg

extern "C" pg_status pg_er_generate_noalloc(uint64_t seed, int64_t epoch, int64_t n_existing,
                                            int64_t delta, double p, int32_t* d_src,
                                            int32_t* d_dst, int64_t capacity, int64_t* num_edges,
                                            void* stream) {
    using namespace pg;
    if (!num_edges) return PG_ERR_ARG;
    *num_edges = 0;
    if (n_existing <= 0 || n_existing > (int64_t)INT32_MAX / 2 || delta <= 0 || std::isnan(p) ||
        capacity < 0 || (capacity > 0 && (!d_src || !d_dst)))
        return PG_ERR_ARG;
    if (n_existing + delta > (int64_t)INT32_MAX) return PG_ERR_ARG;
    const int64_t chunks = (n_existing + kErChunk - 1) / kErChunk;
    if (delta > kNoAllocMaxTasks / chunks) return PG_ERR_CAPACITY;  // scratch holds one count per task
    const int64_t tasks = delta * chunks;
    if (!(p > 0.0)) return PG_OK;  // no edges
    const ErSkip K = er_skip_constants(p);
    int64_t* scratch = nullptr;
    pg_status s = scratch_for_current_device(&scratch);
    if (s != PG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int64_t* cnt = scratch;                          // [tasks]
    int64_t* off = scratch + kNoAllocMaxTasks;        // [tasks + 1], exclusive scan of cnt
    int64_t* blocksum = off + kNoAllocMaxTasks + 1;   // [scan blocks + 1]
    const uint32_t ep = (uint32_t)epoch;
    int64_t g = (tasks + 255) / 256;
    if (g > 4096) g = 4096;
    k_na_count<<<(unsigned)g, 256, 0, st>>>(seed, ep, n_existing, tasks, chunks, K, cnt);
    launch_scan_i64(cnt, off, tasks, blocksum, st);
    if (cudaGetLastError() != cudaSuccess) return PG_ERR_CUDA;  // *num_edges stays 0
    int64_t total = 0;
    if (cudaMemcpyAsync(&total, off + tasks, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PG_ERR_CUDA;
    *num_edges = total;
    if (total > capacity) return PG_ERR_CAPACITY;  // nothing written
    k_na_emit<<<(unsigned)g, 256, 0, st>>>(seed, ep, n_existing, tasks, chunks, K, off, d_src, d_dst);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) return PG_ERR_CUDA;
    return PG_OK;
}
