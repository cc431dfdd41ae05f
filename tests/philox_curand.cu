// Test helper (built by tests/test_gpu_philox.py on the GPU machine): the library's device Philox4x32-10
// next to cuRAND's device generator of the same name, block for block.
//
// cuRAND's curand_init(seed, subsequence, offset) keys its Philox4x32-10 with the seed (low, high
// 32 bits) and starts the 128-bit counter at (offset / 4 as a 64-bit low half, subsequence as the
// high half); curand4 returns that counter's block.  So block q of subsequence s under seed K is
// philox(counter = (q_lo, q_hi, s_lo, s_hi), key = (K_lo, K_hi)).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "../paragraph_gb300/csrc/pg_core.cuh"

namespace {

// entry i: seed, subsequence and block index; out_c: cuRAND's block, out_p: the library's
__global__ void k_xcheck(int n, const unsigned long long* seed, const unsigned long long* sub,
                         const unsigned long long* blk, uint4* out_c, uint4* out_p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed[i], sub[i], 4ull * blk[i], &st);
    out_c[i] = curand4(&st);
    const pg::u32x4 x = pg::philox((uint32_t)blk[i], (uint32_t)(blk[i] >> 32), (uint32_t)sub[i],
                                   (uint32_t)(sub[i] >> 32), (uint32_t)seed[i], (uint32_t)(seed[i] >> 32));
    out_p[i] = make_uint4(x.x[0], x.x[1], x.x[2], x.x[3]);
}

// the library's device Philox on raw (counter, key) pairs: ck[6 i ..] = c0..c3, k0, k1
__global__ void k_raw(int n, const uint32_t* ck, uint4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* q = ck + 6 * i;
    const pg::u32x4 x = pg::philox(q[0], q[1], q[2], q[3], q[4], q[5]);
    out[i] = make_uint4(x.x[0], x.x[1], x.x[2], x.x[3]);
}

template <typename T>
int upload(T** d, const T* h, int n) {
    if (cudaMalloc(reinterpret_cast<void**>(d), sizeof(T) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) return 1;
    return cudaMemcpy(*d, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess;
}

}  // namespace

// 0 on success; out_c / out_p: 4 n words each
extern "C" int philox_xcheck(int n, const unsigned long long* seed, const unsigned long long* sub,
                             const unsigned long long* blk, unsigned int* out_c, unsigned int* out_p) {
    unsigned long long *ds = nullptr, *du = nullptr, *db = nullptr;
    uint4 *dc = nullptr, *dp = nullptr;
    int rc = upload(&ds, seed, n) || upload(&du, sub, n) || upload(&db, blk, n) ||
             cudaMalloc(reinterpret_cast<void**>(&dc), sizeof(uint4) * (size_t)n) != cudaSuccess ||
             cudaMalloc(reinterpret_cast<void**>(&dp), sizeof(uint4) * (size_t)n) != cudaSuccess;
    if (!rc) {
        k_xcheck<<<(n + 255) / 256, 256>>>(n, ds, du, db, dc, dp);
        rc = cudaDeviceSynchronize() != cudaSuccess ||
             cudaMemcpy(out_c, dc, sizeof(uint4) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess ||
             cudaMemcpy(out_p, dp, sizeof(uint4) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess;
    }
    cudaFree(ds);
    cudaFree(du);
    cudaFree(db);
    cudaFree(dc);
    cudaFree(dp);
    return rc;
}

extern "C" int philox_raw(int n, const unsigned int* ck, unsigned int* out) {
    uint32_t* d = nullptr;
    uint4* o = nullptr;
    int rc = upload(&d, ck, 6 * n) || cudaMalloc(reinterpret_cast<void**>(&o), sizeof(uint4) * (size_t)n) != cudaSuccess;
    if (!rc) {
        k_raw<<<(n + 255) / 256, 256>>>(n, d, o);
        rc = cudaDeviceSynchronize() != cudaSuccess ||
             cudaMemcpy(out, o, sizeof(uint4) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess;
    }
    cudaFree(d);
    cudaFree(o);
    return rc;
}
