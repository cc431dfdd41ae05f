// pg_refcompat.cu -- per-epoch score components of the refcompat functor on the device.
//
// Replaces the host score preparation the reference runs every epoch (FillInDegreeArr,
// FillFitnessArr, FillRecencyArr, CalculateScores, src/abm.cu:112-208,324-338, called from
// src/kernel.cu:1698-1706):
//   k_rc_begin   clear each replica's 128-bit sums and age histogram
//   k_rc_node    per node: fitness at t, the numerators indeg^gamma + 1 and f^gamma + 1 (128-bit
//                integers, added exactly into the replica's sums), the node's age in the histogram
//   k_rc_norm    per replica: the two normalisers and the recency denominator (ages ascending)
//   k_rc_scores  per node: pa, rec and fit components in FP64
// HBM per node: read pub, indeg, fit, lag, dur (20 B), write three doubles twice (48 B) and read
// them back once (16 B).
#include "pg_rc.cuh"

namespace pg {

__global__ void __launch_bounds__(1024) k_rc_begin(Arena A) {
    if (A.st->error) return;
    for (int64_t i = threadIdx.x; i < (int64_t)A.R * 4; i += blockDim.x) A.rc_acc[i] = 0ull;
    for (int64_t i = threadIdx.x; i < (int64_t)A.R * kRcAgeMax; i += blockDim.x) A.rc_cnt[i] = 0;
}

__device__ __forceinline__ void add128(uint64_t& hi, uint64_t& lo, uint64_t h2, uint64_t l2) {
    const uint64_t l = lo + l2;
    hi += h2 + (l < lo ? 1ull : 0ull);
    lo = l;
}

__global__ void __launch_bounds__(kTileThreads) k_rc_node(Arena A) {
    // The age histogram and the 128-bit sums are gathered per CTA in shared memory, then added
    // to the replica's totals once per CTA (integer sums: the order does not change them).
    __shared__ int s_age[kRcAgeMax];
    __shared__ unsigned long long s_sum[kTileThreads / 32][4];
    if (A.st->error) return;
    const int t = blockIdx.x;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const int64_t ep = A.st->epoch;
    const int rec_len = rp.rc_rec_len;
    for (int i = threadIdx.x; i < rec_len; i += kTileThreads) s_age[i] = 0;
    __syncthreads();
    uint64_t sph = 0, spl = 0, sfh = 0, sfl = 0;
#pragma unroll
    for (int i = 0; i < kTile / kTileThreads; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        if (v >= rp.n) continue;
        const int64_t slot = rp.nbase + v;
        const int32_t f = rc_fitness_at(A.pub[slot], A.rc_lag[slot], A.rc_dur[slot],
                                        (int64_t)A.fit[slot], ep, rp.rc_decay);
        uint64_t ah, alo, fh, flo;
        pow1_u128((uint64_t)(uint32_t)A.indeg[slot], rp.rc_gamma, &ah, &alo);
        pow1_u128((uint64_t)(uint32_t)f, rp.rc_gamma, &fh, &flo);
        A.rc_pa[slot] = u128_to_d(ah, alo);
        A.rc_fit[slot] = u128_to_d(fh, flo);
        add128(sph, spl, ah, alo);
        add128(sfh, sfl, fh, flo);
        const int64_t age = ep - A.pub[slot];
        if (age >= 0 && age < rec_len) atomicAdd(&s_age[age], 1);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const uint64_t a = __shfl_xor_sync(0xffffffffu, sph, d), b = __shfl_xor_sync(0xffffffffu, spl, d);
        const uint64_t c = __shfl_xor_sync(0xffffffffu, sfh, d), e = __shfl_xor_sync(0xffffffffu, sfl, d);
        add128(sph, spl, a, b);
        add128(sfh, sfl, c, e);
    }
    if (lane_id() == 0) {
        unsigned long long* w = s_sum[threadIdx.x >> 5];
        w[0] = spl;
        w[1] = sph;
        w[2] = sfl;
        w[3] = sfh;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kTileThreads / 32; ++w) {
            add128(sph, spl, s_sum[w][1], s_sum[w][0]);
            add128(sfh, sfl, s_sum[w][3], s_sum[w][2]);
        }
        unsigned long long* acc = A.rc_acc + (int64_t)r * 4;
        const unsigned long long o0 = atomicAdd(&acc[0], (unsigned long long)spl);
        if (o0 + spl < o0) atomicAdd(&acc[1], 1ull);
        atomicAdd(&acc[1], (unsigned long long)sph);
        const unsigned long long o2 = atomicAdd(&acc[2], (unsigned long long)sfl);
        if (o2 + sfl < o2) atomicAdd(&acc[3], 1ull);
        atomicAdd(&acc[3], (unsigned long long)sfh);
    }
    for (int i = threadIdx.x; i < rec_len; i += kTileThreads)
        if (s_age[i]) atomicAdd(&A.rc_cnt[(int64_t)r * kRcAgeMax + i], s_age[i]);
}

__global__ void k_rc_norm(Arena A) {
    if (A.st->error) return;
    for (int r = threadIdx.x; r < A.R; r += blockDim.x) {
        Replica& rp = A.rep[r];
        const unsigned long long* acc = A.rc_acc + (int64_t)r * 4;
        rp.rc_dpa = u128_to_d(acc[1], acc[0]);
        rp.rc_dfit = u128_to_d(acc[3], acc[2]);
        double U = 0.0;
        const int32_t* cnt = A.rc_cnt + (int64_t)r * kRcAgeMax;
        const double* P = A.rc_rtab + (int64_t)r * kRcAgeMax;
        for (int i = 0; i < rp.rc_rec_len; ++i)
            if (cnt[i]) U += P[i];
        rp.rc_U = U;
    }
}

__global__ void __launch_bounds__(kTileThreads) k_rc_scores(Arena A) {
    if (A.st->error) return;
    const int t = blockIdx.x;
    const int r = A.tile_rep[t];
    const Replica& rp = A.rep[r];
    const int64_t v0 = (int64_t)(t - rp.tbase) * kTile;
    if (v0 >= rp.n) return;
    const int64_t ep = A.st->epoch;
    const int32_t* cnt = A.rc_cnt + (int64_t)r * kRcAgeMax;
    const double* P = A.rc_rtab + (int64_t)r * kRcAgeMax;
    unsigned act = 0;
#pragma unroll
    for (int i = 0; i < kTile / kTileThreads; ++i) {
        const int64_t v = v0 + threadIdx.x + i * kTileThreads;
        if (v >= rp.n) continue;
        const int64_t slot = rp.nbase + v;
        A.rc_pa[slot] = A.rc_pa[slot] / rp.rc_dpa;
        A.rc_fit[slot] = A.rc_fit[slot] / rp.rc_dfit;
        const int64_t age = ep - A.pub[slot];
        A.rc_rec[slot] = (age >= 0 && age < rp.rc_rec_len && rp.rc_U > 0.0)
                             ? P[age] / ((double)cnt[age] * rp.rc_U)
                             : 0.0;
        ++act;
    }
    act = __reduce_add_sync(0xffffffffu, act);
    if (lane_id() == 0 && act) atomicAdd(&A.st->nodes_weighted, (unsigned long long)act);
}

void launch_rc_scores(const Arena& A, cudaStream_t s) {
    k_rc_begin<<<1, 1024, 0, s>>>(A);
    k_rc_node<<<A.ntiles, kTileThreads, 0, s>>>(A);
    k_rc_norm<<<1, 256, 0, s>>>(A);
    k_rc_scores<<<A.ntiles, kTileThreads, 0, s>>>(A);
}

}  // namespace pg
