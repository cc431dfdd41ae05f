// pg_lik.cu -- log-likelihood of a growth trace under theta = (alpha, tau, gamma, beta), and its
// adjoint, batched over up to 64 parameter points per launch.  No counterpart in the reference:
// this is the density of the sampling law the growth step draws from
// (w_j beta^[j in N_a], successive sampling without replacement).
//
// Per launch (forward or adjoint):
//   k_lik_global      per epoch: sum_{j<n_e} w_j (forward) or sum_j w_j g_j (adjoint), one CTA per
//                     4096-node chunk; fp32 weights, compensated fp32 sums per thread, FP64 across
//                     threads and chunks (fixed order, so results are reproducible).
//   k_lik_global_sum  chunks -> one FP64 value per (epoch, point).
//   k_lik_agents      one CTA per agent (static assignment): builds the agent's 2-hop ball as a
//                     bitmap over [0, n_e) in shared memory (passes of 786,432 ids), compacts it
//                     into windows of ids, and every point sums its ball weights S_a (adjoint: also
//                     sum w g) -- the ball is built once for all points of the batch.  Then one
//                     warp per point walks the agent's citations in draw order with FP64 prefix
//                     scans: D_i = Z_a - sum_{l<i} W_{c_l}, log-likelihood sum x_i - log D_i, and
//                     in the adjoint g_i - (dZ_a - dP_i) / D_i.  The adjoint recomputes every
//                     weight and reads only the forward's per-agent Z_a.
//   k_lik_sum         agents -> totals per point (fixed order).
#include "pg_lik.cuh"

namespace pg {

namespace {

struct Kahan {
    float s = 0.f, c = 0.f;
};

// Compensated summation (Kahan 1965); the build has no FMA contraction and no reassociation.
__device__ __forceinline__ void kadd(Kahan& k, float v) {
    const float y = v - k.c;
    const float t = k.s + y;
    k.c = (t - k.s) - y;
    k.s = t;
}
__device__ __forceinline__ double kval(const Kahan& k) { return (double)k.s - (double)k.c; }

// First position of x's backward row whose source is >= ne (rows ascending).
__device__ __forceinline__ int64_t bwd_cut(const LikTrace& T, int64_t x, int64_t ne) {
    int64_t lo = T.bo[x], hi = T.bo[x + 1];
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)T.bc[mid] < ne)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ float lik_x(const float4 f, float al, float ga, float itau) {
    return ga * f.x + al * f.y - f.z * itau;
}

}  // namespace

__global__ void __launch_bounds__(256) k_lik_features(LikTrace T) {
    const int e = blockIdx.y;
    const int64_t ne = T.epoch_nodes[e];
    const int32_t te = T.epoch_t[e];
    float4* F = T.feat + (int64_t)e * T.n;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ne;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = bwd_cut(T, j, ne) - T.bo[j];
        float4 f;
        f.x = logf_pg(T.fit[j]);
        f.y = logf_pg((float)(d + 1));
        f.z = (float)(te - T.pub[j]);
        f.w = 0.f;
        F[j] = f;
    }
}

template <bool ADJ>
__global__ void __launch_bounds__(kLikThreads) k_lik_global(LikTrace T, LikBatch P) {
    __shared__ double red[kLikThreads * 4];
    const int e = blockIdx.y, tid = threadIdx.x;
    const int64_t ne = T.epoch_nodes[e];
    const int64_t lo = (int64_t)blockIdx.x * kLikChunk;
    const int BE = P.BE, B = P.B;
    const int b = tid & (BE - 1), sub = tid / BE, nsub = kLikThreads / BE;
    Kahan s, t0, t1, t2;
    if (b < B && lo < ne) {
        const float al = (float)P.theta[b * 4], itau = (float)(1.0 / P.theta[b * 4 + 1]),
                    ga = (float)P.theta[b * 4 + 2];
        const int64_t hi = ne < lo + kLikChunk ? ne : lo + kLikChunk;
        const float4* F = T.feat + (int64_t)e * T.n;
        for (int64_t j = lo + sub; j < hi; j += nsub) {
            const float4 f = F[j];
            const float w = expf_pg(lik_x(f, al, ga, itau));
            kadd(s, w);
            if (ADJ) {
                kadd(t0, w * f.y);
                kadd(t1, w * f.z);
                kadd(t2, w * f.x);
            }
        }
    }
    red[tid * 4 + 0] = kval(s);
    red[tid * 4 + 1] = kval(t0);
    red[tid * 4 + 2] = kval(t1);
    red[tid * 4 + 3] = kval(t2);
    __syncthreads();
    if (sub == 0 && b < B) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < nsub; ++q)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += red[(q * BE + b) * 4 + k];
        double* o = P.gpart + (((int64_t)e * T.chunks + blockIdx.x) * B + b) * 4;
#pragma unroll
        for (int k = 0; k < 4; ++k) o[k] = acc[k];
    }
}

template <bool ADJ>
__global__ void k_lik_global_sum(LikTrace T, LikBatch P) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= T.epochs * P.B) return;
    const int e = idx / P.B, b = idx % P.B;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < T.chunks; ++c) {
        const double* g = P.gpart + (((int64_t)e * T.chunks + c) * P.B + b) * 4;
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] += g[k];
    }
    if (!ADJ) {
        P.zglob[e * P.B + b] = acc[0];
    } else {
        const double tau = P.theta[b * 4 + 1];
        double* o = P.gglob + ((int64_t)e * P.B + b) * 3;
        o[0] = acc[1];
        o[1] = acc[2] * (1.0 / (tau * tau));
        o[2] = acc[3];
    }
}

template <bool ADJ>
__global__ void __launch_bounds__(kLikThreads) k_lik_agents(LikTrace T, LikBatch P) {
    extern __shared__ __align__(16) unsigned char lik_smem[];
    double* red = reinterpret_cast<double*>(lik_smem);     // [256][4]
    double* sums = red + kLikThreads * 4;                  // [64][4]
    int32_t* list = reinterpret_cast<int32_t*>(sums + kLikMaxB * 4);  // [kLikList]
    int32_t* cid = list + kLikList;                        // [kKMax]
    uint32_t* bits = reinterpret_cast<uint32_t*>(cid + kKMax);        // [bitmap_words]
    uint8_t* flag = reinterpret_cast<uint8_t*>(bits + T.bitmap_words);  // [kKMax]
    __shared__ int64_t seg[2 * PG_MAX_ANCHORS_DEV + 1];  // prefix of the anchors' row lengths
    __shared__ int64_t rowb[2 * PG_MAX_ANCHORS_DEV];     // first entry of each anchor row
    __shared__ int32_t anc[PG_MAX_ANCHORS_DEV];
    __shared__ int32_t nanc;
    __shared__ int32_t scan_ws[33];
    __shared__ unsigned long long adj_read;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int BE = P.BE, B = P.B;
    const int b = tid & (BE - 1), sub = tid / BE, nsub = kLikThreads / BE;
    float al = 0.f, ga = 0.f, itau = 0.f;
    if (b < B) {
        al = (float)P.theta[b * 4];
        itau = (float)(1.0 / P.theta[b * 4 + 1]);
        ga = (float)P.theta[b * 4 + 2];
    }
    const int64_t pass_ids = (int64_t)T.bitmap_words * 32;
    for (int64_t a = blockIdx.x; a < T.agents; a += gridDim.x) {
        const int e = T.agent_epoch[a];
        const int64_t ne = T.epoch_nodes[e];
        const float4* F = T.feat + (int64_t)e * T.n;
        const int64_t c0 = T.coff[a];
        const int k = (int)(T.coff[a + 1] - c0);
        for (int i = tid; i < k; i += kLikThreads) {
            cid[i] = T.cites[c0 + i];
            flag[i] = 0;
        }
        if (tid == 0) {
            int na = 0;
            for (int i = 0; i < T.num_anchors; ++i) {
                const int32_t x = T.anchors[a * 4 + i];
                if (x >= 0) anc[na++] = x;
            }
            nanc = na;
            int64_t acc = 0;
            for (int i = 0; i < na; ++i) {
                const int64_t x = anc[i];
                rowb[2 * i] = T.fo[x];
                seg[2 * i] = acc;
                acc += T.fo[x + 1] - T.fo[x];
                rowb[2 * i + 1] = T.bo[x];
                seg[2 * i + 1] = acc;
                acc += bwd_cut(T, x, ne) - T.bo[x];
            }
            seg[2 * na] = acc;
            adj_read = (unsigned long long)acc;
        }
        unsigned long long ball_elems = 0;
        Kahan s, t0, t1, t2;
        __syncthreads();
        const int na = nanc;
        const int64_t L1 = seg[2 * na];
        for (int64_t lo = 0; lo < ne; lo += pass_ids) {
            const int64_t hi = ne < lo + pass_ids ? ne : lo + pass_ids;
            const int nw = (int)((hi - lo + 31) >> 5);
            for (int w = tid; w < nw; w += kLikThreads) bits[w] = 0u;
            __syncthreads();
            auto mark = [&](int64_t v) {
                if (v >= lo && v < hi) {
                    const int64_t o = v - lo;
                    atomicOr(&bits[o >> 5], 1u << (o & 31));
                }
            };
            if (tid < na) mark(anc[tid]);
            // every 1-hop node y (one warp each) and the rows of y
            for (int64_t q = warp; q < L1; q += kLikThreads / 32) {
                int sg = 0;
                while (seg[sg + 1] <= q) ++sg;
                const int32_t* col = (sg & 1) ? T.bc : T.fc;
                const int64_t y = col[rowb[sg] + (q - seg[sg])];
                if (lane == 0) mark(y);
                const int64_t f1 = T.fo[y + 1];
                for (int64_t p = T.fo[y] + lane; p < f1; p += 32) mark(T.fc[p]);
                const int64_t b1 = bwd_cut(T, y, ne);
                for (int64_t p = T.bo[y] + lane; p < b1; p += 32) mark(T.bc[p]);
                if (!ADJ && P.counters && lane == 0 && lo == 0)
                    atomicAdd(&adj_read, (unsigned long long)((f1 - T.fo[y]) + (b1 - T.bo[y])));
            }
            __syncthreads();
            for (int i = tid; i < k; i += kLikThreads) {
                const int64_t c = cid[i];
                if (c >= lo && c < hi) {
                    const int64_t o = c - lo;
                    if ((bits[o >> 5] >> (o & 31)) & 1u) flag[i] = 1;
                }
            }
            // compact the set bits into windows of ids; every point sums the window's weights
            const int wpt = (nw + kLikThreads - 1) / kLikThreads;
            const int w0 = tid * wpt < nw ? tid * wpt : nw;
            const int w1 = w0 + wpt < nw ? w0 + wpt : nw;
            int cnt = 0;
            for (int w = w0; w < w1; ++w) cnt += __popc(bits[w]);
            int total = 0;
            const int off = block_excl_scan<int>(cnt, scan_ws, &total);
            ball_elems += (unsigned long long)total;
            for (int base = 0; base < total; base += kLikList) {
                if (cnt > 0 && off + cnt > base && off < base + kLikList) {
                    int r = off;
                    for (int w = w0; w < w1 && r < base + kLikList; ++w) {
                        uint32_t m = bits[w];
                        while (m) {
                            const int bit = __ffs(m) - 1;
                            m &= m - 1u;
                            if (r >= base && r < base + kLikList)
                                list[r - base] = (int32_t)(lo + ((int64_t)w << 5) + bit);
                            ++r;
                        }
                    }
                }
                __syncthreads();
                const int cw = total - base < kLikList ? total - base : kLikList;
                if (b < B) {
                    for (int i = sub; i < cw; i += nsub) {
                        const float4 f = F[list[i]];
                        const float w = expf_pg(lik_x(f, al, ga, itau));
                        kadd(s, w);
                        if (ADJ) {
                            kadd(t0, w * f.y);
                            kadd(t1, w * f.z);
                            kadd(t2, w * f.x);
                        }
                    }
                }
                __syncthreads();
            }
        }
        red[tid * 4 + 0] = kval(s);
        red[tid * 4 + 1] = kval(t0);
        red[tid * 4 + 2] = kval(t1);
        red[tid * 4 + 3] = kval(t2);
        __syncthreads();
        if (!ADJ && P.counters && tid == 0) {
            atomicAdd(&P.counters[0], ball_elems);
            atomicAdd(&P.counters[1], adj_read);
            atomicAdd(&P.counters[2], (unsigned long long)k);
        }
        if (tid < B) {
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            for (int q = 0; q < nsub; ++q)
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) acc[kk] += red[(q * BE + tid) * 4 + kk];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) sums[tid * 4 + kk] = acc[kk];
        }
        __syncthreads();
        // citations in draw order, one warp per point
        for (int bb = warp; bb < B; bb += kLikThreads / 32) {
            const double beta = P.theta[bb * 4 + 3], tau = P.theta[bb * 4 + 1];
            const float alb = (float)P.theta[bb * 4], gab = (float)P.theta[bb * 4 + 2],
                        itb = (float)(1.0 / tau);
            const double lbe = log_pg(beta), ibe = 1.0 / beta, itau2 = 1.0 / (tau * tau);
            const double S = sums[bb * 4];
            double Z;
            double dz[4] = {0.0, 0.0, 0.0, 0.0};
            if (!ADJ) {
                Z = P.zglob[e * B + bb] + (beta - 1.0) * S;
                if (lane == 0) P.zagent[a * B + bb] = Z;
            } else {
                Z = P.zagent[a * B + bb];
                const double* gg = P.gglob + ((int64_t)e * B + bb) * 3;
                dz[0] = gg[0] + (beta - 1.0) * sums[bb * 4 + 1];
                dz[1] = gg[1] + (beta - 1.0) * (sums[bb * 4 + 2] * itau2);
                dz[2] = gg[2] + (beta - 1.0) * sums[bb * 4 + 3];
                dz[3] = S;
            }
            double carry = 0.0, l = 0.0;
            double dcarry[4] = {0.0, 0.0, 0.0, 0.0}, g[4] = {0.0, 0.0, 0.0, 0.0};
            for (int i0 = 0; i0 < k; i0 += 32) {
                const int i = i0 + lane;
                const bool v = i < k;
                double W = 0.0, x64 = 0.0;
                double gk[4] = {0.0, 0.0, 0.0, 0.0};
                if (v) {
                    const float4 f = F[cid[i]];
                    const float x = lik_x(f, alb, gab, itb);
                    const float w = expf_pg(x);
                    const bool in = flag[i] != 0;
                    W = in ? (double)w * beta : (double)w;
                    x64 = in ? (double)x + lbe : (double)x;
                    gk[0] = f.y;
                    gk[1] = (double)f.z * itau2;
                    gk[2] = f.x;
                    gk[3] = in ? ibe : 0.0;
                }
                const double incl = warp_incl_scan(W);
                double excl = __shfl_up_sync(0xffffffffu, incl, 1);
                if (lane == 0) excl = 0.0;
                double D = Z - (carry + excl);
                if (D < W) D = W;
                if (v && !(D > 0.0)) {
                    atomicOr(P.error, 2u);
                    D = 1.0;
                }
                if (v) l += x64 - log_pg(D);
                if (ADJ) {
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const double ik = warp_incl_scan(W * gk[kk]);
                        double ek = __shfl_up_sync(0xffffffffu, ik, 1);
                        if (lane == 0) ek = 0.0;
                        if (v) g[kk] += gk[kk] - (dz[kk] - (dcarry[kk] + ek)) / D;
                        dcarry[kk] += __shfl_sync(0xffffffffu, ik, 31);
                    }
                }
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (!ADJ) {
                l = warp_sum(l);
                if (lane == 0) P.out[a * B + bb] = l;
            } else {
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) g[kk] = warp_sum(g[kk]);
                if (lane == 0)
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) P.out[(a * B + bb) * 4 + kk] = g[kk];
            }
        }
        __syncthreads();  // shared buffers are reused by the next agent
    }
}

// Totals over agents, one CTA per (point, component), fixed summation order.
__global__ void __launch_bounds__(256) k_lik_sum(const double* out, int64_t agents, int B, int K,
                                                 double* res) {
    __shared__ double r[256];
    const int b = blockIdx.x / K, kk = blockIdx.x % K;
    double acc = 0.0;
    for (int64_t a = threadIdx.x; a < agents; a += 256) acc += out[(a * B + b) * K + kk];
    r[threadIdx.x] = acc;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) r[threadIdx.x] += r[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) res[b * K + kk] = r[0];
}

size_t lik_agent_smem(int bitmap_words) {
    return sizeof(double) * (kLikThreads * 4 + kLikMaxB * 4) + sizeof(int32_t) * (kLikList + kKMax) +
           sizeof(uint32_t) * (size_t)bitmap_words + kKMax;
}

cudaError_t init_lik_kernels(int bitmap_words, int* blocks_per_sm) {
    const int smem = (int)lik_agent_smem(bitmap_words);
    cudaError_t e = cudaFuncSetAttribute(k_lik_agents<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lik_agents<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int b0 = 1, b1 = 1;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_lik_agents<false>, kLikThreads, smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_lik_agents<true>, kLikThreads, smem);
    const int b = b0 < b1 ? b0 : b1;
    *blocks_per_sm = b < 1 ? 1 : b;
    return e;
}

void launch_lik_features(const LikTrace& T, int num_sms, cudaStream_t s) {
    int64_t gx = (T.n + 255) / 256;
    if (gx > (int64_t)num_sms * 8) gx = (int64_t)num_sms * 8;
    if (gx < 1) gx = 1;
    k_lik_features<<<dim3((unsigned)gx, (unsigned)T.epochs), 256, 0, s>>>(T);
}

void launch_lik(const LikTrace& T, const LikBatch& P, int adjoint, int agent_grid, cudaStream_t s) {
    const dim3 gg((unsigned)T.chunks, (unsigned)T.epochs);
    const unsigned gs = (unsigned)((T.epochs * P.B + 127) / 128);
    const size_t smem = lik_agent_smem(T.bitmap_words);
    int64_t ga = T.agents < agent_grid ? T.agents : agent_grid;
    if (ga < 1) ga = 1;
    const int K = adjoint ? 4 : 1;
    if (adjoint) {
        k_lik_global<true><<<gg, kLikThreads, 0, s>>>(T, P);
        k_lik_global_sum<true><<<gs, 128, 0, s>>>(T, P);
        k_lik_agents<true><<<(unsigned)ga, kLikThreads, smem, s>>>(T, P);
    } else {
        k_lik_global<false><<<gg, kLikThreads, 0, s>>>(T, P);
        k_lik_global_sum<false><<<gs, 128, 0, s>>>(T, P);
        k_lik_agents<false><<<(unsigned)ga, kLikThreads, smem, s>>>(T, P);
    }
    k_lik_sum<<<(unsigned)(P.B * K), 256, 0, s>>>(P.out, T.agents, P.B, K, P.res);
}

}  // namespace pg
