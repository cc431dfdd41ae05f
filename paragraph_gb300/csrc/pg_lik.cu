// pg_lik.cu -- log-likelihood of a growth trace under theta = (alpha, tau, gamma, beta), and its
// adjoint, batched over up to 64 parameter points per launch.  No counterpart in the reference:
// this is the density of the sampling law the growth step draws from
// (w_j beta^[j in N_a], successive sampling without replacement).
//
// Weights: w_j = 2^(x2_j), x2_j = log2(e) (gamma log f_j + alpha log(indeg_j+1) - (t-t_j)/tau), the
// exponent carried as an unevaluated fp32 pair h + l: the per-point constants are split into fp32
// high and low parts and log(indeg+1) is stored as a high/low pair.  A feature or constant rounded
// once to fp32 is a fixed error of every node that shares it -- it does not average out over the
// trace and moves the gradient by the Hessian times a 2^-24 shift of the data or of theta, which
// shows where the gradient nearly vanishes (the generating point of a trace).  Two arithmetic
// modes:
//   default     h by one FMA chain (its roundings are dropped), log f in fp32, 2^h from the
//               special-function unit (PTX ex2.approx.ftz.f32, relative error < 2^-22; results
//               below 2^-126 flush to zero) scaled by 1 + l ln 2, ball sums pairwise over four
//               weights: ~1e-5 of the gradient's norm at the generating point of a 200k-node trace,
//               1e-7 elsewhere;
//   exact_exp2  every product and sum of the exponent keeps its rounding error, log f is an FP64 log
//               carried as high part plus packed remainder, 2^(h + l) from exp2_exact (fp32
//               arithmetic, about 2 ulp), and every ball weight and product is summed on its own
//               (BallSum): ~3e-7 of the gradient's norm there, at about a third of the throughput.
// The same weight function feeds every sum below, so the normalisers and the citations' prefix
// sums agree: an error that is a smooth function of the weight (such as the unit's) largely
// cancels between them.  The per-epoch sums over all nodes are shared by every agent of the epoch, so they are
// accumulated in FP64 (an fp32 partial's rounding would be common to all of the epoch's
// citations); the per-agent ball sums use compensated fp32.
//
// Per launch (forward or adjoint):
//   k_lik_global      per epoch: sum_{j<n_e} w_j (forward) or sum_j w_j g_j (adjoint), one CTA per
//                     4096-node chunk; compensated fp32 sums per thread, FP64 across threads and
//                     chunks (fixed order, so results are reproducible).
//   k_lik_global_sum  chunks -> one FP64 value per (epoch, point).
//   k_lik_ball        (once per trace, or per chunk of agents and pass) the agent's 2-hop ball as
//                     a bitmap over [0, n_e) in shared memory, compacted to ascending ids.
//   k_lik_eval        one warp per agent and group of points: every point sums its ball weights
//                     S_a (adjoint: also sum w g), reading each ball element once for all the
//                     warp's points.  Then the citations are walked in draw order with FP64 running
//                     sums: D_i = Z_a - sum_{l<i} W_{c_l}, log-likelihood sum x_i - log D_i, and in
//                     the adjoint g_i - (dZ_a - dP_i) / D_i.  The adjoint recomputes every weight and
//                     reads only the forward's per-agent Z_a.
//   k_lik_sum         agents -> totals per point (fixed order).
#include "pg_lik.cuh"

#include <cuda_fp16.h>

namespace pg {

namespace {

constexpr double kLn2d = 0x1.62e42fefa39efp-1;
constexpr float kLn2f = 0x1.62e430p-1f;

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

// A ball's sums for one point: S = sum w (and, in the adjoint, sum w g for the three continuous
// features).  Default: four weights summed pairwise, products in FMA chains, then compensated fp32.
// EXACT: every weight and every rounded product enters the compensated sums on its own and the
// products' rounding errors (FMA residuals) are summed beside them, so a ball sum keeps no
// rounding of its own above the compensated sum's (these per-agent errors otherwise reach ~3e-6
// of the gradient where it nearly vanishes).
template <bool ADJ, bool EXACT>
struct BallSum {
    Kahan s, t0, t1, t2;
    float r0 = 0.f, r1 = 0.f, r2 = 0.f;
    __device__ __forceinline__ void add1(const float w, const float4 f) {
        kadd(s, w);
        if (ADJ) {
            const float p0 = w * f.y, p1 = w * f.z, p2 = w * f.x;
            kadd(t0, p0);
            kadd(t1, p1);
            kadd(t2, p2);
            if (EXACT) {
                r0 += __fmaf_rn(w, f.y, -p0);
                r1 += __fmaf_rn(w, f.z, -p1);
                r2 += __fmaf_rn(w, f.x, -p2);
            }
        }
    }
    __device__ __forceinline__ void add4(const float w0, const float w1, const float w2, const float w3,
                                         const float4 f0, const float4 f1, const float4 f2, const float4 f3) {
        if (EXACT) {
            add1(w0, f0);
            add1(w1, f1);
            add1(w2, f2);
            add1(w3, f3);
            return;
        }
        kadd(s, (w0 + w1) + (w2 + w3));
        if (ADJ) {
            kadd(t0, __fmaf_rn(w3, f3.y, __fmaf_rn(w2, f2.y, __fmaf_rn(w1, f1.y, w0 * f0.y))));
            kadd(t1, __fmaf_rn(w3, f3.z, __fmaf_rn(w2, f2.z, __fmaf_rn(w1, f1.z, w0 * f0.z))));
            kadd(t2, __fmaf_rn(w3, f3.x, __fmaf_rn(w2, f2.x, __fmaf_rn(w1, f1.x, w0 * f0.x))));
        }
    }
    __device__ __forceinline__ double S() const { return kval(s); }
    __device__ __forceinline__ double T0() const { return kval(t0) + (double)r0; }
    __device__ __forceinline__ double T1() const { return kval(t1) + (double)r1; }
    __device__ __forceinline__ double T2() const { return kval(t2) + (double)r2; }
};

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

// Per-point constants of the weight exponent in base 2, each as an fp32 high part and the fp32
// remainder of its FP64 value; al2s and ga2s scale the exact layout's packed low parts (stored
// times 2^24) back.
struct LikC {
    float al2, ga2, it2;     // alpha log2 e, gamma log2 e, log2 e / tau (high parts)
    float al2l, ga2l, it2l;  // their remainders
    float al2s, ga2s;        // al2 2^-24, ga2 2^-24 (exact)
};
__device__ __forceinline__ LikC lik_c(const double* pp) {
    LikC c;
    const double a = pp[0] * kLog2e, g = pp[2] * kLog2e, t = pp[1] * kLog2e;
    c.al2 = (float)a;
    c.ga2 = (float)g;
    c.it2 = (float)t;
    c.al2l = (float)(a - (double)c.al2);
    c.ga2l = (float)(g - (double)c.ga2);
    c.it2l = (float)(t - (double)c.it2);
    c.al2s = c.al2 * 0x1p-24f;
    c.ga2s = c.ga2 * 0x1p-24f;
    return c;
}

// The exact layout's fourth word: the fp32 remainders of log(d+1) (low half) and of log f (high
// half), each times 2^24 as an IEEE half.  A remainder is at most 2^-25 of its high part, so 11 bits
// of it carry the pair to about 2^-35.
__device__ __forceinline__ float lik_pack_lows(float ly_rem24, float lx_rem24) {
    const uint32_t y = __half_as_ushort(__float2half_rn(ly_rem24));
    const uint32_t x = __half_as_ushort(__float2half_rn(lx_rem24));
    return __uint_as_float(y | (x << 16));
}
__device__ __forceinline__ void lik_unpack_lows(float w, float& ly_rem24, float& lx_rem24) {
    const uint32_t b = __float_as_uint(w);
    ly_rem24 = __half2float(__ushort_as_half((unsigned short)(b & 0xFFFFu)));
    lx_rem24 = __half2float(__ushort_as_half((unsigned short)(b >> 16)));
}
// 2^x on the special-function unit (PTX ex2.approx.ftz.f32).
__device__ __forceinline__ float ex2_sfu(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// log2 of the weight, ga2 log f + al2 log(d+1) - it2 (t - t_j), as h + l.  Features: f.y = log(d+1)
// (fp32 high part), f.z = t - t_j (an exact integer); default layout: f.x = log f in fp32 (logf_pg),
// f.w = the remainder of log(d+1); exact layout: f.x = the fp32 high part of the FP64 log f,
// f.w = both logs' remainders, packed (lik_pack_lows).
struct X2 {
    float h, l;
};
// a + b = s + err exactly (Knuth's two-sum; the build neither contracts nor reassociates)
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
    const float s = a + b;
    const float bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}
// the low-order terms of the exponent: the constants' remainders times the features' high parts,
// the constants times the features' remainders (the exact layout also carries log f's)
template <bool EXACT>
__device__ __forceinline__ float lik_tail(const float4 f, const LikC& c) {
    const float base = __fmaf_rn(c.al2l, f.y, __fmaf_rn(c.ga2l, f.x, -(c.it2l * f.z)));
    if (!EXACT) return __fmaf_rn(c.al2, f.w, base);
    float ly, lx;
    lik_unpack_lows(f.w, ly, lx);
    return __fmaf_rn(c.al2s, ly, __fmaf_rn(c.ga2s, lx, base));
}
template <bool EXACT>
__device__ __forceinline__ X2 lik_x2(const float4 f, const LikC& c) {
    X2 x;
    if (EXACT) {
        // every product and sum keeps its rounding error (FMA residuals, two-sums): h + l is the
        // exponent to about 2^-40, so no node's weight carries a fixed error of its own
        const float p3 = c.ga2 * f.x, e3 = __fmaf_rn(c.ga2, f.x, -p3);
        const float p1 = c.al2 * f.y, e1 = __fmaf_rn(c.al2, f.y, -p1);
        const float p2 = -c.it2 * f.z, e2 = __fmaf_rn(-c.it2, f.z, -p2);
        float r1, r2;
        const float s1 = two_sum(p3, p1, r1);
        x.h = two_sum(s1, p2, r2);
        x.l = ((e1 + e2) + (e3 + (r1 + r2))) + lik_tail<true>(f, c);
    } else {
        x.h = __fmaf_rn(c.al2, f.y, __fmaf_rn(-c.it2, f.z, c.ga2 * f.x));
        x.l = lik_tail<false>(f, c);
    }
    return x;
}
// 2^(h + l) for |l| < 2^-18 in fp32 arithmetic: n = rint(h), f = h - n (exact), t = (f + l) ln 2
// in [-0.35, 0.35], e^t by its Taylor series through t^7/7! (truncation below 5e-9 relative), times
// 2^n built in the exponent field: about 2 ulp, with rounding errors that vary from node to node.
__device__ __forceinline__ float exp2_exact(const X2 x) {
    const float n = rintf(x.h);
    const int ni = (int)n;
    if (ni < -126) return 0.0f;
    const float t = __fmaf_rn(x.h - n, kLn2f, x.l * kLn2f);
    float p = 1.0f / 5040.0f;
    p = __fmaf_rn(p, t, 1.0f / 720.0f);
    p = __fmaf_rn(p, t, 1.0f / 120.0f);
    p = __fmaf_rn(p, t, 1.0f / 24.0f);
    p = __fmaf_rn(p, t, 1.0f / 6.0f);
    p = __fmaf_rn(p, t, 0.5f);
    p = __fmaf_rn(p, t, 1.0f);
    p = __fmaf_rn(p, t, 1.0f);
    return p * __int_as_float((ni > 127 ? 255 : ni + 127) << 23);
}
// the weight 2^(h + l): EXACT selects exp2_exact, else the special-function unit's 2^h scaled by
// 1 + l ln 2 + O(l^2)
template <bool EXACT>
__device__ __forceinline__ float lik_w(const X2 x) {
    if (EXACT) return exp2_exact(x);
    const float e = ex2_sfu(x.h);
    return __fmaf_rn(e, x.l * kLn2f, e);
}

// Double-float numbers (a pair of fp32, h + l with |l| <= ulp(h) / 2; Dekker 1971, Knuth's two-sum):
// about 44 significant bits from fp32 arithmetic.  The citation loops run in them: GB300's FP64
// rate is a small fraction of its fp32 rate, and FP64 there cost as much as the ball sums.
struct DF {
    float h, l;
};
__device__ __forceinline__ DF df_of(double x) {
    DF r;
    r.h = (float)x;
    r.l = (float)(x - (double)r.h);
    return r;
}
__device__ __forceinline__ double df_val(const DF a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ DF df_norm(float s, float e) {  // s + e as a pair, any magnitudes
    float r;
    const float h = two_sum(s, e, r);
    return DF{h, r};
}
__device__ __forceinline__ DF df_add(const DF a, const DF b) {
    float e;
    const float s = two_sum(a.h, b.h, e);
    return df_norm(s, e + (a.l + b.l));
}
__device__ __forceinline__ DF df_neg(const DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_mul(const DF a, const DF b) {
    const float p = a.h * b.h;
    const float e = __fmaf_rn(a.h, b.h, -p);
    return df_norm(p, __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e)));
}
__device__ __forceinline__ DF df_mulf(const DF a, float b) {
    const float p = a.h * b;
    const float e = __fmaf_rn(a.h, b, -p);
    return df_norm(p, __fmaf_rn(a.l, b, e));
}
__device__ __forceinline__ bool df_gt(const DF a, const DF b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
// 1/a for a > 0: the fp32 reciprocal r, then one Newton step r + r (1 - a r) in double-float
__device__ __forceinline__ DF df_recip(const DF a) {
    const float r = 1.0f / a.h;
    const DF e = df_add(DF{1.0f, 0.0f}, df_neg(df_mulf(a, r)));
    return df_add(DF{r, 0.0f}, df_mulf(e, r));
}

// log(1 - u) for u in [0, 0.5): -2 atanh(t), t = u / (2 - u) in [0, 1/3), by the odd Taylor series
// of atanh, t + t^3/3 + ... + t^17/17 (truncation below 1e-9 relative at t = 1/3).
__device__ __forceinline__ float log1m_pg(float u) {
    const float t = u / (2.0f - u);
    const float s = t * t;
    float p = 1.0f / 17.0f;
    p = p * s + 1.0f / 15.0f;
    p = p * s + 1.0f / 13.0f;
    p = p * s + 1.0f / 11.0f;
    p = p * s + 1.0f / 9.0f;
    p = p * s + 1.0f / 7.0f;
    p = p * s + 1.0f / 5.0f;
    p = p * s + 1.0f / 3.0f;
    p = p * s + 1.0f;
    return -2.0f * t * p;
}

}  // namespace

// EXACT selects the exact layout (see lik_x2)
template <bool EXACT>
__global__ void __launch_bounds__(256) k_lik_features(LikTrace T) {
    const int e = blockIdx.y;
    const int64_t ne = T.epoch_nodes[e];
    const int32_t te = T.epoch_t[e];
    float4* F = T.feat + (int64_t)e * T.n;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ne;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = bwd_cut(T, j, ne) - T.bo[j];
        const double ly = log_pg((double)(d + 1));
        float4 f;
        f.y = (float)ly;
        f.z = (float)(te - T.pub[j]);
        if (EXACT) {
            const double lx = log_pg((double)T.fit[j]);
            f.x = (float)lx;
            f.w = lik_pack_lows((float)((ly - (double)f.y) * 0x1p24), (float)((lx - (double)f.x) * 0x1p24));
        } else {
            f.x = logf_pg(T.fit[j]);
            f.w = (float)(ly - (double)f.y);
        }
        F[j] = f;
    }
}

template <bool ADJ, bool EXACT>
__global__ void __launch_bounds__(kLikThreads) k_lik_global(LikTrace T, LikBatch P) {
    __shared__ double red[kLikThreads * 4];
    const int e = blockIdx.y, tid = threadIdx.x;
    const int64_t ne = T.epoch_nodes[e];
    const int64_t lo = (int64_t)blockIdx.x * kLikChunk;
    const int BE = P.BE, B = P.B;
    const int b = tid & (BE - 1), sub = tid / BE, nsub = kLikThreads / BE;
    double s = 0.0, t0 = 0.0, t1 = 0.0, t2 = 0.0;
    if (b < B && lo < ne) {
        const LikC c = lik_c(P.pp + b * 8);
        const int64_t hi = ne < lo + kLikChunk ? ne : lo + kLikChunk;
        const float4* F = T.feat + (int64_t)e * T.n;
        for (int64_t j = lo + sub; j < hi; j += nsub) {
            const float4 f = F[j];
            const double w = (double)lik_w<EXACT>(lik_x2<EXACT>(f, c));
            s += w;
            if (ADJ) {
                t0 = __fma_rn(w, (double)f.y, t0);
                t1 = __fma_rn(w, (double)f.z, t1);
                t2 = __fma_rn(w, (double)f.x, t2);
            }
        }
    }
    red[tid * 4 + 0] = s;
    red[tid * 4 + 1] = t0;
    red[tid * 4 + 2] = t1;
    red[tid * 4 + 3] = t2;
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

// The 2-hop ball of agents [a0, a1) in the epoch-start graph, one CTA per agent, as a bitmap over
// [0, n_e) in shared memory (passes of bitmap_words * 32 ids).  EMIT = false: ball sizes (and the
// adjacency entries read) into Bl.cnt; EMIT = true: the ids, ascending, at Bl.ids[boff[a] - base]
// and the ball membership of each citation into Bl.cflag.
template <bool EMIT>
__global__ void __launch_bounds__(kLikThreads) k_lik_ball(LikTrace T, LikBalls Bl, int64_t a0, int64_t a1) {
    extern __shared__ __align__(16) unsigned char lik_smem[];
    uint32_t* bits = reinterpret_cast<uint32_t*>(lik_smem);  // [bitmap_words]
    __shared__ int64_t seg[2 * PG_MAX_ANCHORS_DEV + 1];       // prefix of the anchors' row lengths
    __shared__ int64_t rowb[2 * PG_MAX_ANCHORS_DEV];          // first entry of each anchor row
    __shared__ int32_t anc[PG_MAX_ANCHORS_DEV];
    __shared__ int32_t nanc;
    __shared__ int32_t scan_ws[33];
    __shared__ unsigned long long adj_read;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t pass_ids = (int64_t)T.bitmap_words * 32;
    for (int64_t a = a0 + blockIdx.x; a < a1; a += gridDim.x) {
        const int e = T.agent_epoch[a];
        const int64_t ne = T.epoch_nodes[e];
        const int64_t c0 = T.coff[a];
        const int k = (int)(T.coff[a + 1] - c0);
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
        __syncthreads();
        const int na = nanc;
        const int64_t L1 = seg[2 * na];
        int64_t written = EMIT ? Bl.boff[a] - Bl.base : 0;
        unsigned long long ball = 0;
        for (int64_t lo = 0; lo < ne; lo += pass_ids) {
            const int64_t hi = ne < lo + pass_ids ? ne : lo + pass_ids;
            const int nw = (int)((hi - lo + 31) >> 5);
            uint32_t* cache = Bl.bmap ? Bl.bmap + a * Bl.bmap_stride + (lo / pass_ids) * T.bitmap_words : nullptr;
            if (EMIT && cache) {
                // the count pass left this agent's bitmap: no row walk
                for (int w = tid; w < nw; w += kLikThreads) bits[w] = cache[w];
                __syncthreads();
            } else {
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
                    if (!EMIT && lane == 0 && lo == 0)
                        atomicAdd(&adj_read, (unsigned long long)((f1 - T.fo[y]) + (b1 - T.bo[y])));
                }
                __syncthreads();
                if (!EMIT && cache)
                    for (int w = tid; w < nw; w += kLikThreads) cache[w] = bits[w];
            }
            if (EMIT) {
                for (int i = tid; i < k; i += kLikThreads) {
                    const int64_t c = T.cites[c0 + i];
                    if (c >= lo && c < hi) {
                        const int64_t o = c - lo;
                        Bl.cflag[c0 + i] = (uint8_t)((bits[o >> 5] >> (o & 31)) & 1u);
                    }
                }
            }
            // each thread owns a contiguous run of words; a block scan of their popcounts places
            // its ids so the ball comes out ascending
            const int wpt = (nw + kLikThreads - 1) / kLikThreads;
            const int w0 = tid * wpt < nw ? tid * wpt : nw;
            const int w1 = w0 + wpt < nw ? w0 + wpt : nw;
            int cnt = 0;
            for (int w = w0; w < w1; ++w) cnt += __popc(bits[w]);
            int total = 0;
            const int off = block_excl_scan<int>(cnt, scan_ws, &total);
            if (EMIT && cnt > 0) {
                int32_t* out = Bl.ids + written + off;
                int r = 0;
                for (int w = w0; w < w1; ++w) {
                    uint32_t m = bits[w];
                    while (m) {
                        const int bit = __ffs(m) - 1;
                        m &= m - 1u;
                        out[r++] = (int32_t)(lo + ((int64_t)w << 5) + bit);
                    }
                }
            }
            written += total;
            ball += (unsigned long long)total;
            __syncthreads();  // the bitmap is cleared by the next pass
        }
        if (!EMIT && tid == 0) {
            Bl.cnt[a] = (int64_t)ball;
            Bl.adj[a] = (int64_t)adj_read;
        }
        __syncthreads();
    }
}

// Forward (ADJ = false) or adjoint pass over agents [a0, a1) whose balls are in Bl.  One warp per
// (agent, group of points).  NP = 2 (33..64 points): lane l holds points l and l + 32, and every lane
// walks the whole ball, so each ball element is read once for all points.  NP = 1 (<= 32 points):
// lane = point p + BW * slice; the slices split the ball, so a single point spreads its ball over
// the whole warp.  Ball sums: fp32 weights, four elements summed pairwise, then compensated fp32
// per lane, FP64 across slices.  The citations are then walked in draw order by the slice-0 lane
// of each point with FP64 running sums:  D_i = Z_a - P_i,  log D_i = log Z_a + log(1 - P_i / Z_a),
// and in the adjoint g_i - (dZ_a - dP_i) / D_i.
template <bool ADJ, int NP, bool EXACT>
__global__ void __launch_bounds__(kLikThreads, ADJ ? 2 : 3) k_lik_eval(LikTrace T, LikBatch P, LikBalls Bl,
                                                          int64_t a0, int64_t a1) {
    __shared__ float4 lik_stage[kLikThreads / 32][32];
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int BW = NP == 2 ? 32 : P.BW, SL = 32 / BW;
    const int groups = NP == 2 ? 1 : (P.B + BW - 1) / BW;
    const int pl = lane & (BW - 1), sl = lane / BW;
    const int64_t items = (a1 - a0) * groups;
    for (int64_t it = wid; it < items; it += nwarps) {
        const int64_t a = a0 + it / groups;
        int bq[NP];
        bool act[NP];
        LikC cq[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            bq[p] = NP == 2 ? lane + 32 * p : (int)(it % groups) * BW + pl;
            act[p] = bq[p] < P.B;
            cq[p] = lik_c(P.pp + (act[p] ? bq[p] : 0) * 8);
        }
        const int e = T.agent_epoch[a];
        const float4* F = T.feat + (int64_t)e * T.n;
        const int64_t j0 = Bl.boff[a] - Bl.base, j1 = Bl.boff[a + 1] - Bl.base;
        BallSum<ADJ, EXACT> acc[NP];
        if constexpr (NP == 2) {
            // the ball in batches of 32: lane l loads element l's id and feature row, the next
            // batch's loads are issued before this batch is summed, and the rows are read back
            // from the warp's shared buffer in the same groups of four (same sums) as below
            float4* buf = lik_stage[threadIdx.x >> 5];
            float4 cur = make_float4(0.f, 0.f, 0.f, 0.f);
            if (j0 + lane < j1) cur = F[Bl.ids[j0 + lane]];
            for (int64_t b0 = j0; b0 < j1; b0 += 32) {
                const int cnt = j1 - b0 < 32 ? (int)(j1 - b0) : 32;
                float4 nxt = make_float4(0.f, 0.f, 0.f, 0.f);
                if (b0 + 32 + lane < j1) nxt = F[Bl.ids[b0 + 32 + lane]];
                __syncwarp();
                buf[lane] = cur;
                __syncwarp();
                int i = 0;
                for (; i + 3 < cnt; i += 4) {
                    const float4 f0 = buf[i], f1 = buf[i + 1], f2 = buf[i + 2], f3 = buf[i + 3];
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        const float w0 = lik_w<EXACT>(lik_x2<EXACT>(f0, cq[p])), w1 = lik_w<EXACT>(lik_x2<EXACT>(f1, cq[p])),
                                    w2 = lik_w<EXACT>(lik_x2<EXACT>(f2, cq[p])), w3 = lik_w<EXACT>(lik_x2<EXACT>(f3, cq[p]));
                        acc[p].add4(w0, w1, w2, w3, f0, f1, f2, f3);
                    }
                }
                for (; i < cnt; ++i) {
                    const float4 f = buf[i];
#pragma unroll
                    for (int p = 0; p < NP; ++p) acc[p].add1(lik_w<EXACT>(lik_x2<EXACT>(f, cq[p])), f);
                }
                cur = nxt;
            }
        }
        int64_t q = NP == 2 ? j1 : j0 + sl;
        for (; q + 3 * SL < j1; q += 4 * SL) {
            const int32_t i0 = Bl.ids[q], i1 = Bl.ids[q + SL], i2 = Bl.ids[q + 2 * SL], i3 = Bl.ids[q + 3 * SL];
            const float4 f0 = F[i0], f1 = F[i1], f2 = F[i2], f3 = F[i3];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float w0 = lik_w<EXACT>(lik_x2<EXACT>(f0, cq[p])), w1 = lik_w<EXACT>(lik_x2<EXACT>(f1, cq[p])),
                            w2 = lik_w<EXACT>(lik_x2<EXACT>(f2, cq[p])), w3 = lik_w<EXACT>(lik_x2<EXACT>(f3, cq[p]));
                acc[p].add4(w0, w1, w2, w3, f0, f1, f2, f3);
            }
        }
        for (; q < j1; q += SL) {
            const float4 f = F[Bl.ids[q]];
#pragma unroll
            for (int p = 0; p < NP; ++p) acc[p].add1(lik_w<EXACT>(lik_x2<EXACT>(f, cq[p])), f);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            double S = acc[p].S(), T0 = 0.0, T1 = 0.0, T2 = 0.0;
            if (ADJ) {
                T0 = acc[p].T0();
                T1 = acc[p].T1();
                T2 = acc[p].T2();
            }
            for (int o = BW; o < 32; o <<= 1) {
                S += __shfl_xor_sync(0xffffffffu, S, o);
                if (ADJ) {
                    T0 += __shfl_xor_sync(0xffffffffu, T0, o);
                    T1 += __shfl_xor_sync(0xffffffffu, T1, o);
                    T2 += __shfl_xor_sync(0xffffffffu, T2, o);
                }
            }
            if (!act[p] || sl != 0) continue;
            const int b = bq[p];
            const LikC c = cq[p];
            const double* pp = P.pp + b * 8;
            const double beta = pp[3], lbe = pp[4], ibe = pp[5], itau2 = pp[6];
            const int64_t c0 = T.coff[a];
            const int k = (int)(T.coff[a + 1] - c0);
            double Z;
            double dz[4] = {0.0, 0.0, 0.0, 0.0};
            if (!ADJ) {
                Z = P.zglob[e * P.B + b] + (beta - 1.0) * S;
                P.zagent[a * P.B + b] = Z;
            } else {
                Z = P.zagent[a * P.B + b];
                const double* gg = P.gglob + ((int64_t)e * P.B + b) * 3;
                dz[0] = gg[0] + (beta - 1.0) * T0;
                dz[1] = gg[1] + (beta - 1.0) * (T1 * itau2);
                dz[2] = gg[2] + (beta - 1.0) * T2;
                dz[3] = S;
            }
            if (!(Z > 0.0)) {
                atomicOr(P.error, 2u);
                continue;
            }
            // the citations in draw order, in fp32 / double-float arithmetic (FP64 only per agent
            // and in the rare u >= 1/2 case): W_i = w_i beta^[in ball], P the weight drawn before
            if (!ADJ) {
                // l_a = ln2 sum x_i + n_in log beta - (k log Z_a + sum log(1 - u_i)), u_i = P_i / Z_a;
                // the sums of x_i (its two parts), of log(1 - u_i) and of P compensated in fp32
                const double logZ = log_pg(Z);
                const float invZ = 1.0f / (float)Z, betaf = (float)beta;
                Kahan sh, sl, slr, pc;
                double lr_far = 0.0;
                int n_in = 0;
                for (int i = 0; i < k; ++i) {
                    const bool in = Bl.cflag[c0 + i] != 0;
                    const float4 f = F[T.cites[c0 + i]];
                    const X2 x2 = lik_x2<EXACT>(f, c);
                    const float w = lik_w<EXACT>(x2);
                    const float W = in ? w * betaf : w;
                    const float u = (pc.s - pc.c) * invZ;
                    if (u < 0.5f)
                        kadd(slr, log1m_pg(u));
                    else  // 1 - u is small: log(Z - P) - log Z from the FP64 difference
                        lr_far += log_pg(Z - kval(pc)) - logZ;
                    kadd(sh, x2.h);
                    kadd(sl, x2.l);
                    n_in += in ? 1 : 0;
                    kadd(pc, W);
                }
                const double l = (kval(sh) + kval(sl)) * kLn2d + (double)n_in * lbe -
                                 ((double)k * logZ + kval(slr) + lr_far);
                P.out[a * P.B + b] = l;
            } else {
                // g_k = sum_i [gk_i - (dZ_k - dP_k,i) / D_i],  D_i = Z_a - P_i,  dP_k,i = sum_{j<i} W_j gk_j
                const DF Zd = df_of(Z), betad = df_of(beta), itau2d = df_of(itau2), ibed = df_of(ibe);
                DF dzd[4], dP[4], g[4];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    dzd[kk] = df_of(dz[kk]);
                    dP[kk] = DF{0.0f, 0.0f};
                    g[kk] = DF{0.0f, 0.0f};
                }
                DF Pc{0.0f, 0.0f};
                for (int i = 0; i < k; ++i) {
                    const bool in = Bl.cflag[c0 + i] != 0;
                    const float4 f = F[T.cites[c0 + i]];
                    const X2 x2 = lik_x2<EXACT>(f, c);
                    const float w = lik_w<EXACT>(x2);
                    const DF W = in ? df_mulf(betad, w) : DF{w, 0.0f};
                    const DF D = df_add(Zd, df_neg(Pc));
                    const DF id = df_recip(df_gt(D, W) ? D : W);
                    const DF gk[4] = {DF{f.y, 0.0f}, df_mulf(itau2d, f.z), DF{f.x, 0.0f}, in ? ibed : DF{0.0f, 0.0f}};
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const DF t = df_mul(df_add(dzd[kk], df_neg(dP[kk])), id);
                        g[kk] = df_add(g[kk], df_add(gk[kk], df_neg(t)));
                        dP[kk] = df_add(dP[kk], df_mul(W, gk[kk]));
                    }
                    Pc = df_add(Pc, W);
                }
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) P.out[(a * P.B + b) * 4 + kk] = df_val(g[kk]);
            }
        }
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

size_t lik_ball_smem(int bitmap_words) { return sizeof(uint32_t) * (size_t)bitmap_words; }

cudaError_t init_lik_kernels(int bitmap_words, int* ball_per_sm, int* eval_per_sm) {
    // eval_per_sm[0]: forward, [1]: adjoint
    const int smem = (int)lik_ball_smem(bitmap_words);
    cudaError_t e = cudaFuncSetAttribute(k_lik_ball<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lik_ball<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int b0 = 1, b1 = 1, v0 = 1, v1 = 1;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, k_lik_ball<false>, kLikThreads, smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_lik_ball<true>, kLikThreads, smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v0, k_lik_eval<false, 2, false>, kLikThreads, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v1, k_lik_eval<true, 2, false>, kLikThreads, 0);
    *ball_per_sm = b0 < b1 ? (b0 < 1 ? 1 : b0) : (b1 < 1 ? 1 : b1);
    eval_per_sm[0] = v0 < 1 ? 1 : v0;
    eval_per_sm[1] = v1 < 1 ? 1 : v1;
    return e;
}

void launch_lik_ball(const LikTrace& T, const LikBalls& Bl, int emit, int64_t a0, int64_t a1, int grid,
                     cudaStream_t s) {
    if (a1 <= a0) return;
    int64_t g = a1 - a0 < grid ? a1 - a0 : grid;
    const size_t smem = lik_ball_smem(T.bitmap_words);
    if (emit)
        k_lik_ball<true><<<(unsigned)g, kLikThreads, smem, s>>>(T, Bl, a0, a1);
    else
        k_lik_ball<false><<<(unsigned)g, kLikThreads, smem, s>>>(T, Bl, a0, a1);
}

void launch_lik_global(const LikTrace& T, const LikBatch& P, int adjoint, cudaStream_t s) {
    const dim3 gg((unsigned)T.chunks, (unsigned)T.epochs);
    const unsigned gs = (unsigned)((T.epochs * P.B + 127) / 128);
    const bool x = P.exact_exp2 != 0;
    if (adjoint) {
        if (x)
            k_lik_global<true, true><<<gg, kLikThreads, 0, s>>>(T, P);
        else
            k_lik_global<true, false><<<gg, kLikThreads, 0, s>>>(T, P);
        k_lik_global_sum<true><<<gs, 128, 0, s>>>(T, P);
    } else {
        if (x)
            k_lik_global<false, true><<<gg, kLikThreads, 0, s>>>(T, P);
        else
            k_lik_global<false, false><<<gg, kLikThreads, 0, s>>>(T, P);
        k_lik_global_sum<false><<<gs, 128, 0, s>>>(T, P);
    }
}

void launch_lik_eval(const LikTrace& T, const LikBatch& P, const LikBalls& Bl, int adjoint, int64_t a0,
                     int64_t a1, int grid, cudaStream_t s) {
    if (a1 <= a0) return;
    const bool two = P.B > 32;
    const int groups = two ? 1 : (P.B + P.BW - 1) / P.BW;
    const int64_t warps = (a1 - a0) * groups;
    int64_t g = (warps + kLikThreads / 32 - 1) / (kLikThreads / 32);
    if (g > grid) g = grid;
    const unsigned gu = (unsigned)g;
    const bool x = P.exact_exp2 != 0;
#define PG_LIK_EVAL(ADJ, NP, EX) k_lik_eval<ADJ, NP, EX><<<gu, kLikThreads, 0, s>>>(T, P, Bl, a0, a1)
    if (adjoint) {
        if (two)
            x ? PG_LIK_EVAL(true, 2, true) : PG_LIK_EVAL(true, 2, false);
        else
            x ? PG_LIK_EVAL(true, 1, true) : PG_LIK_EVAL(true, 1, false);
    } else {
        if (two)
            x ? PG_LIK_EVAL(false, 2, true) : PG_LIK_EVAL(false, 2, false);
        else
            x ? PG_LIK_EVAL(false, 1, true) : PG_LIK_EVAL(false, 1, false);
    }
#undef PG_LIK_EVAL
}

void launch_lik_sum(const LikTrace& T, const LikBatch& P, int adjoint, cudaStream_t s) {
    const int K = adjoint ? 4 : 1;
    k_lik_sum<<<(unsigned)(P.B * K), 256, 0, s>>>(P.out, T.agents, P.B, K, P.res);
}

// one warp per agent
__global__ void __launch_bounds__(256) k_trace_edges(const int64_t* coff, const int32_t* cites, int64_t agents,
                                                     int64_t n0, int64_t ns, int32_t* src, int32_t* dst) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a = warp; a < agents; a += nwarps) {
        const int64_t p1 = coff[a + 1];
        for (int64_t p = coff[a] + lane; p < p1; p += 32) {
            src[ns + p] = (int32_t)(n0 + a);
            dst[ns + p] = cites[p];
        }
    }
}

void launch_trace_edges(const int64_t* coff, const int32_t* cites, int64_t agents, int64_t n0, int64_t ns,
                        int32_t* src, int32_t* dst, int num_sms, cudaStream_t s) {
    if (agents <= 0) return;
    int64_t g = (agents + 7) / 8;
    if (g > (int64_t)num_sms * 16) g = (int64_t)num_sms * 16;
    k_trace_edges<<<(unsigned)g, 256, 0, s>>>(coff, cites, agents, n0, ns, src, dst);
}

void launch_lik_features(const LikTrace& T, int exact, int num_sms, cudaStream_t s) {
    int64_t gx = (T.n + 255) / 256;
    if (gx > (int64_t)num_sms * 8) gx = (int64_t)num_sms * 8;
    if (gx < 1) gx = 1;
    const dim3 grid((unsigned)gx, (unsigned)T.epochs);
    if (exact)
        k_lik_features<true><<<grid, 256, 0, s>>>(T);
    else
        k_lik_features<false><<<grid, 256, 0, s>>>(T);
}

}  // namespace pg
