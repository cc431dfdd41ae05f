// pg_core.cuh -- counter-based RNG and elementary functions shared by host and device code.
//
// Everything here is integer arithmetic or IEEE-754 operations with one rounding each (+, -, *, /,
// sqrt, fma), so the host build (-ffp-contract=off) and the device build (--fmad=false, no fast
// math) produce identical bits.  That is what makes the growth step's citation choices bit-exact
// between the GPU and the CPU oracle.
//
// RNG: Philox4x32-10, J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11.  It replaces the reference's per-agent cuRAND XORWOW states seeded from the clock
// (src/kernel.cu:233, src/abm.cu:355-374) and the host minstd_rand draws (src/abm.cu:242-290).
//
// exp: Cody & Waite argument reduction x = k ln2 + r, |r| <= ln2/2 (W. Cody, W. Waite, "Software
// Manual for the Elementary Functions", 1980) followed by the Taylor series of e^r.
// log: x = 2^e m, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m-1)/(m+1), summed as the
// odd series 2(s + s^3/3 + s^5/5 + ...) (J.-M. Muller, "Elementary Functions", ch. on table-free
// methods).  Coefficients are the exact series terms rounded to the working precision.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD static inline
#endif

namespace pg {

// ---------------------------------------------------------------- Philox4x32-10
struct u32x4 {
    uint32_t x[4];
};

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;  // golden ratio
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;  // sqrt(3) - 1

PG_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

PG_HD u32x4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += kPhiloxW0;
            k1 += kPhiloxW1;
        }
        const uint32_t hi0 = mulhi32(kPhiloxM0, c0), lo0 = kPhiloxM0 * c0;
        const uint32_t hi1 = mulhi32(kPhiloxM1, c2), lo1 = kPhiloxM1 * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    u32x4 o;
    o.x[0] = c0;
    o.x[1] = c1;
    o.x[2] = c2;
    o.x[3] = c3;
    return o;
}

// Stream ids (top 8 bits of counter word 3; the low 24 bits carry the replica or the ER chunk).
enum Stream : uint32_t {
    kStreamOutDegree = 1,
    kStreamAnchor = 2,
    kStreamGlobal = 3,
    kStreamBoost = 4,
    kStreamFitness = 5,
    kStreamEr = 6,
    kStreamSameYear = 7,
    kStreamUniformFill = 8,
    kStreamFallback = 9,
    kStreamRcAgent = 10,
    kStreamRcKey = 11,
    kStreamRcFitness = 12,
};

// Counter layout: (i, unit, epoch, stream << 24 | aux); key = (seed lo, seed hi).
PG_HD u32x4 draw(uint64_t seed, uint32_t stream, uint32_t aux, uint32_t epoch, uint32_t unit,
                 uint32_t i) {
    return philox(i, unit, epoch, (stream << 24) | (aux & 0xFFFFFFu), (uint32_t)seed,
                  (uint32_t)(seed >> 32));
}

// uniform in (0, 1], exact in fp32: ((x >> 8) + 1) * 2^-24
PG_HD float u01f(uint32_t x) { return (float)((x >> 8) + 1u) * 0x1p-24f; }
// uniform in (0, 1], exact in fp64: ((hi:lo >> 11) + 1) * 2^-53
PG_HD double u01d(uint32_t lo, uint32_t hi) {
    const uint64_t v = (((uint64_t)hi << 32) | lo) >> 11;
    return (double)(v + 1u) * 0x1p-53;
}
PG_HD uint64_t u64of(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }
// high 64 bits of a * b
PG_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
// uniform integer in [0, n) by multiply-shift
PG_HD uint32_t bounded32(uint32_t x, uint32_t n) { return (uint32_t)(((uint64_t)x * n) >> 32); }

// ---------------------------------------------------------------- bit casts
PG_HD uint32_t fbits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
PG_HD float bitsf(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
PG_HD uint64_t dbits(double d) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    __builtin_memcpy(&u, &d, 8);
    return u;
#endif
}
PG_HD double bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    __builtin_memcpy(&d, &u, 8);
    return d;
#endif
}
PG_HD float fmaf_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
PG_HD double fma_(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return __builtin_fma(a, b, c);
#endif
}
PG_HD float rintf_(float x) {
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return __builtin_rintf(x);
#endif
}
PG_HD double rint_(double x) {
#if defined(__CUDA_ARCH__)
    return rint(x);
#else
    return __builtin_rint(x);
#endif
}

// ---------------------------------------------------------------- fp32 exp / log
// The library's own elementary functions, the same code on host and device so that keys and
// weights are bit-identical in the oracle.  exp: Cody-Waite reduction x = k ln2 + r with ln 2 split
// into a high and a low part, then the Taylor series of e^r (coefficients 1/n!) by Horner's rule
// and the scale 2^k.  log: x = 2^e m with m in (sqrt(2)/2, sqrt(2)], then
// log m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...) with s = (m - 1)/(m + 1), plus e ln 2.
// The CPU tests hold them within 2 ulp of the correctly rounded values.
constexpr float kLog2eF = 0x1.715476p+0f;
constexpr float kLn2HiF = 0x1.62e430p-1f;
constexpr float kLn2LoF = -0x1.05c610p-29f;
constexpr float kSqrt2F = 0x1.6a09e6p+0f;

// e^x; returns +inf above 88 and 0 below -87 (no subnormal results).
PG_HD float expf_pg(float x) {
    if (x != x) return x;
    if (x > 88.0f) return bitsf(0x7F800000u);
    if (x < -87.0f) return 0.0f;
    const float k = rintf_(x * kLog2eF);
    float r = fmaf_(-k, kLn2HiF, x);
    r = fmaf_(-k, kLn2LoF, r);
    float p = 0x1.a01a02p-13f;      // 1/7!
    p = fmaf_(p, r, 0x1.6c16c2p-10f);  // 1/6!
    p = fmaf_(p, r, 0x1.111112p-7f);   // 1/5!
    p = fmaf_(p, r, 0x1.555556p-5f);   // 1/4!
    p = fmaf_(p, r, 0x1.555556p-3f);   // 1/3!
    p = fmaf_(p, r, 0x1.0p-1f);        // 1/2!
    p = fmaf_(p, r, 1.0f);
    p = fmaf_(p, r, 1.0f);
    const int ki = (int)k;  // in [-126, 127]
    return p * bitsf((uint32_t)(ki + 127) << 23);
}

// natural log; log(0) = -inf, log(x<0) = NaN.
PG_HD float logf_pg(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? bitsf(0xFF800000u) : bitsf(0x7FC00000u);
    if (x == bitsf(0x7F800000u)) return x;
    int eadj = 0;
    if (x < 0x1p-126f) {
        x = x * 0x1p23f;
        eadj = -23;
    }
    const uint32_t b = fbits(x);
    int e = (int)(b >> 23) - 127 + eadj;
    float m = bitsf((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > kSqrt2F) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (m + 1.0f);
    const float z = s * s;
    float p = 0x1.c71c72p-4f;         // 1/9
    p = fmaf_(p, z, 0x1.24924ap-3f);  // 1/7
    p = fmaf_(p, z, 0x1.99999ap-3f);  // 1/5
    p = fmaf_(p, z, 0x1.555556p-2f);  // 1/3
    const float t = s + s;
    const float lm = fmaf_(t * z, p, t);
    const float ef = (float)e;
    return fmaf_(ef, kLn2HiF, fmaf_(ef, kLn2LoF, lm));
}

// ---------------------------------------------------------------- fp64 exp / log
constexpr double kLog2e = 0x1.71547652b82fep+0;
constexpr double kLn2Hi = 0x1.62e42fefa39efp-1;
constexpr double kLn2Lo = 0x1.abc9e3b39803fp-56;
constexpr double kSqrt2 = 0x1.6a09e667f3bcdp+0;

// e^x; +inf above 709, 0 below -708 (no subnormal results).
PG_HD double exp_pg(double x) {
    if (x != x) return x;
    if (x > 709.0) return bitsd(0x7FF0000000000000ull);
    if (x < -708.0) return 0.0;
    const double k = rint_(x * kLog2e);
    double r = fma_(-k, kLn2Hi, x);
    r = fma_(-k, kLn2Lo, r);
    double p = 0x1.6124613a86d09p-33;  // 1/13!
    p = fma_(p, r, 0x1.1eed8eff8d898p-29);
    p = fma_(p, r, 0x1.ae64567f544e4p-26);
    p = fma_(p, r, 0x1.27e4fb7789f5cp-22);
    p = fma_(p, r, 0x1.71de3a556c734p-19);
    p = fma_(p, r, 0x1.a01a01a01a01ap-16);
    p = fma_(p, r, 0x1.a01a01a01a01ap-13);
    p = fma_(p, r, 0x1.6c16c16c16c17p-10);
    p = fma_(p, r, 0x1.1111111111111p-7);
    p = fma_(p, r, 0x1.5555555555555p-5);
    p = fma_(p, r, 0x1.5555555555555p-3);
    p = fma_(p, r, 0x1.0p-1);
    p = fma_(p, r, 1.0);
    p = fma_(p, r, 1.0);
    const int64_t ki = (int64_t)k;  // in [-1022, 1023]
    return p * bitsd((uint64_t)(ki + 1023) << 52);
}

PG_HD double log_pg(double x) {
    if (!(x > 0.0))
        return (x == 0.0) ? bitsd(0xFFF0000000000000ull) : bitsd(0x7FF8000000000000ull);
    if (x == bitsd(0x7FF0000000000000ull)) return x;
    int eadj = 0;
    if (x < 0x1p-1022) {
        x = x * 0x1p52;
        eadj = -52;
    }
    const uint64_t b = dbits(x);
    int e = (int)(b >> 52) - 1023 + eadj;
    double m = bitsd((b & 0xFFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
    if (m > kSqrt2) {
        m = m * 0.5;
        e += 1;
    }
    const double f = m - 1.0;
    const double s = f / (m + 1.0);
    const double z = s * s;
    double p = 0x1.642c8590b2164p-5;  // 1/23
    p = fma_(p, z, 0x1.8618618618618p-5);  // 1/21
    p = fma_(p, z, 0x1.af286bca1af28p-5);  // 1/19
    p = fma_(p, z, 0x1.e1e1e1e1e1e1ep-5);  // 1/17
    p = fma_(p, z, 0x1.1111111111111p-4);  // 1/15
    p = fma_(p, z, 0x1.3b13b13b13b14p-4);  // 1/13
    p = fma_(p, z, 0x1.745d1745d1746p-4);  // 1/11
    p = fma_(p, z, 0x1.c71c71c71c71cp-4);  // 1/9
    p = fma_(p, z, 0x1.2492492492492p-3);  // 1/7
    p = fma_(p, z, 0x1.999999999999ap-3);  // 1/5
    p = fma_(p, z, 0x1.5555555555555p-2);  // 1/3
    const double t = s + s;
    const double lm = fma_(t * z, p, t);
    const double ef = (double)e;
    return fma_(ef, kLn2Hi, fma_(ef, kLn2Lo, lm));
}

// ---------------------------------------------------------------- model helpers
// Baseline weight w0_j = exp(gamma log f + alpha log(indeg+1) - (t - t_j)/tau); the beta boost is
// applied per agent by the neighbourhood race.
PG_HD float weight0(float fitness, int32_t indeg, int32_t age, float alpha, float gamma,
                    float tau) {
    const float a = logf_pg(fitness);
    const float b = logf_pg((float)(indeg + 1));
    const float c = (float)age / tau;
    return expf_pg(fmaf_(gamma, a, fmaf_(alpha, b, -c)));
}

// Lognormal(0,1) fitness by the Marsaglia polar method; at most 32 Philox blocks, then 1.
PG_HD float lognormal_fitness(uint64_t seed, uint32_t aux, uint32_t epoch, uint32_t unit) {
    for (uint32_t i = 0; i < 32; ++i) {
        const u32x4 r = draw(seed, kStreamFitness, aux, epoch, unit, i);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float v1 = 2.0f * u01f(r.x[2 * h]) - 1.0f;
            const float v2 = 2.0f * u01f(r.x[2 * h + 1]) - 1.0f;
            const float s = v1 * v1 + v2 * v2;
            if (s < 1.0f && s > 0.0f) {
                const float g = v1 * sqrtf(-2.0f * logf_pg(s) / s);
                return expf_pg(g);
            }
        }
    }
    return 1.0f;
}

// Poisson(lambda) CDF scaled to 2^64 with saturation; table[i] = floor(P(X <= i) 2^64).
PG_HD void poisson_table(double lambda, uint64_t* table, int entries) {
    double p = exp_pg(-lambda);
    double cdf = p;
    for (int i = 0; i < entries; ++i) {
        if (i > 0) {
            p = p * lambda / (double)i;
            cdf = cdf + p;
        }
        table[i] = (cdf >= 1.0 || i == entries - 1) ? ~0ull : (uint64_t)(cdf * 0x1p64);
    }
}

PG_HD int poisson_draw(const uint64_t* table, int entries, uint64_t u) {
    for (int i = 0; i < entries; ++i)
        if (u < table[i]) return i;
    return entries - 1;
}

PG_HD int ceil_log2_u64(uint64_t n) {
    int c = 0;
    while (c < 63 && ((uint64_t)1 << c) < n) ++c;
    return c;
}

// Fixed-point shift for a replica: every q_j = floor(w_j 2^s) < 2^(62 - ceil_log2 n).
PG_HD int cdf_shift(float wmax, int64_t n) {
    const uint32_t b = fbits(wmax);
    const int ex = (int)((b >> 23) & 0xFF) - 126;  // wmax < 2^ex (wmax is a normal float here)
    return 62 - ex - ceil_log2_u64((uint64_t)(n > 0 ? n : 1));
}

PG_HD uint64_t quantise(float w, int s) {
    if (!(w > 0.0f)) return 0;
    const double v = (double)w * bitsd((uint64_t)(s + 1023) << 52);  // exact scaling by 2^s
    const uint64_t q = (uint64_t)v;
    return q > 0 ? q : 1;
}

}  // namespace pg
