// pg_scan.cuh -- exclusive scans used by the growth step (part of the epoch translation unit,
// pg_agents.cu).
//
// Reduce-then-scan in three steps (tile sums, one CTA scans the sums, tiles rescan with their
// offset), as three launches or as three phases of the persistent epoch kernel.  Integer sums are
// exact, so the result does not depend on the tile decomposition.
#pragma once
#include "pg_engine.cuh"

namespace pg {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

int scan_blocks_needed(int64_t n) { return (int)((n + kScanBlock - 1) / kScanBlock); }

// block vb of the reduce step (kScanThreads threads)
template <typename TIn>
__device__ __forceinline__ void d_scan_reduce(const TIn* __restrict__ in, int64_t n, int64_t* __restrict__ blocksum,
                                              int vb) {
    __shared__ int64_t sw[33];
    const int64_t base = (int64_t)vb * kScanBlock;
    int64_t v = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + threadIdx.x + (int64_t)i * kScanThreads;
        if (idx < n) v += (int64_t)in[idx];
    }
    v = warp_sum(v);
    if (lane_id() == 0) sw[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += sw[w];
        blocksum[vb] = t;
    }
}

template <typename TIn>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const TIn* __restrict__ in, int64_t n,
                                                              int64_t* __restrict__ blocksum) {
    d_scan_reduce<TIn>(in, n, blocksum, blockIdx.x);
}

// One CTA (any multiple of 32 threads up to 1024): exclusive scan of blocksum[0..nb) in place;
// blocksum[nb] = total.
__device__ __forceinline__ void d_scan_blocksums(int64_t* __restrict__ blocksum, int nb) {
    __shared__ int64_t sw[33];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int64_t v = i < nb ? blocksum[i] : 0;
        int64_t tot;
        const int64_t ex = block_excl_scan<int64_t>(v, sw, &tot);
        if (i < nb) blocksum[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) blocksum[nb] = carry;
}

__global__ void __launch_bounds__(1024) k_scan_blocksums(int64_t* __restrict__ blocksum, int nb) {
    d_scan_blocksums(blocksum, nb);
}

// block vb of the apply step (kScanThreads threads)
template <typename TIn>
__device__ __forceinline__ void d_scan_apply(const TIn* __restrict__ in, int64_t n, const int64_t* __restrict__ blocksum,
                                             int nb, int64_t* __restrict__ out, int vb) {
    __shared__ int64_t sw[33];
    const int64_t base = (int64_t)vb * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i;
        v[i] = idx < n ? (int64_t)in[idx] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t ex = block_excl_scan<int64_t>(s, sw, &tot) + blocksum[vb];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const int64_t idx = base + i;
        if (idx < n) out[idx] = ex;
        ex += v[i];
    }
    if (vb == nb - 1 && threadIdx.x == 0) out[n] = blocksum[nb];
}

template <typename TIn>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const TIn* __restrict__ in, int64_t n,
                                                             const int64_t* __restrict__ blocksum,
                                                             int nb, int64_t* __restrict__ out) {
    d_scan_apply<TIn>(in, n, blocksum, nb, out, blockIdx.x);
}

template <typename TIn>
static void scan_impl(const TIn* in, int64_t* out, int64_t n, int64_t* blocksum, cudaStream_t s) {
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int64_t), s);
        return;
    }
    const int nb = scan_blocks_needed(n);
    k_scan_reduce<TIn><<<nb, kScanThreads, 0, s>>>(in, n, blocksum);
    k_scan_blocksums<<<1, 1024, 0, s>>>(blocksum, nb);
    k_scan_apply<TIn><<<nb, kScanThreads, 0, s>>>(in, n, blocksum, nb, out);
}

void launch_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* blocksum, cudaStream_t s) {
    scan_impl<int64_t>(in, out, n, blocksum, s);
}
void launch_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* blocksum,
                            cudaStream_t s) {
    scan_impl<int32_t>(in, out, n, blocksum, s);
}

}  // namespace pg
