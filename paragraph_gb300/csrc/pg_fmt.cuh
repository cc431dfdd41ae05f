// pg_fmt.cuh -- C's "%.<P>g" conversion of a double, exactly as the C library prints it, for host
// and device (the attribute writer formats its floating-point columns on the GPU).
//
// Method (exact, no table of powers): for v = m 2^e (m a 53-bit integer) and a decimal exponent
// guess k, the P significant digits are D = round_half_even(v 10^s), s = P - 1 - k.  A double
// estimate of v 10^s is within one of the true value (its relative error is ~1e-15 and D < 2^34),
// so D is decided among three neighbours by exact integer comparisons of v 10^s with D + 1/2:
//   2 m 2^e 10^s  <=>  (2D + 1)   becomes   m 2^max(e+1,0) 10^max(s,0)  <=>  (2D + 1) 2^max(-e-1,0) 10^max(-s,0),
// both sides multi-word integers (at most ~1170 bits for any finite double).  Equality is an exact
// tie, resolved to the even D as the C library does in its default rounding mode.  If D reaches
// 10^P the exponent guess was one low (and one high if D < 10^(P-1)); k is corrected and D redone.
// Then the %g rules: exponent X = k after rounding; fixed notation when -4 <= X < P, else
// d.ddde+XX (at least two exponent digits); trailing zeros and a bare decimal point are dropped.
#pragma once
#include <math.h>
#include <stdint.h>

#include "pg_core.cuh"

namespace pg {

constexpr int kBigLimbs = 40;  // 1280 bits

struct Big {
    uint32_t w[kBigLimbs];
    int n;  // limbs in use (w[n..] are zero)
};

PG_HD void big_set(Big& b, uint64_t v) {
    b.w[0] = (uint32_t)v;
    b.w[1] = (uint32_t)(v >> 32);
    b.n = b.w[1] ? 2 : (b.w[0] ? 1 : 0);
    for (int i = 2; i < kBigLimbs; ++i) b.w[i] = 0u;
}

// b *= x (x < 2^32)
PG_HD void big_mul_small(Big& b, uint32_t x) {
    uint64_t carry = 0;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t t = (uint64_t)b.w[i] * x + carry;
        b.w[i] = (uint32_t)t;
        carry = t >> 32;
    }
    if (carry && b.n < kBigLimbs) b.w[b.n++] = (uint32_t)carry;
}

// b *= 10^p
PG_HD void big_mul_pow10(Big& b, int p) {
    while (p >= 9) {
        big_mul_small(b, 1000000000u);
        p -= 9;
    }
    uint32_t r = 1;
    while (p-- > 0) r *= 10u;
    if (r > 1) big_mul_small(b, r);
}

// b <<= s
PG_HD void big_shl(Big& b, int s) {
    if (b.n == 0 || s <= 0) return;
    const int q = s >> 5, r = s & 31;
    int n = b.n + q + 1;
    if (n > kBigLimbs) n = kBigLimbs;
    for (int i = n - 1; i >= 0; --i) {
        const int j = i - q;
        uint32_t v = 0;
        if (j >= 0 && j < b.n) v = b.w[j] << r;
        if (r && j - 1 >= 0 && j - 1 < b.n) v |= b.w[j - 1] >> (32 - r);
        b.w[i] = v;
    }
    b.n = n;
    while (b.n > 0 && b.w[b.n - 1] == 0) --b.n;
}

PG_HD int big_cmp(const Big& a, const Big& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; --i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

// compare v 10^s with D + 1/2 (v = m 2^e > 0): -1, 0 (an exact tie) or 1
PG_HD int cmp_half(uint64_t m, int e, int s, uint64_t D) {
    Big L, R;
    big_set(L, m);
    big_shl(L, e + 1 > 0 ? e + 1 : 0);
    if (s > 0) big_mul_pow10(L, s);
    big_set(R, 2 * D + 1);
    big_shl(R, -e - 1 > 0 ? -e - 1 : 0);
    if (s < 0) big_mul_pow10(R, -s);
    return big_cmp(L, R);
}

// round_half_even(v 10^s) for v = m 2^e, from an estimate within one of v 10^s
PG_HD uint64_t round_scaled(uint64_t m, int e, int s, double est) {
    uint64_t D = est < 1.0 ? 0 : (uint64_t)est;  // floor of the estimate
    if (D > 0) --D;                              // true floor is D, D + 1 or D + 2 from here
    // smallest D with v 10^s < D + 1/2, or an exact tie
    for (int it = 0; it < 4; ++it) {
        const int c = cmp_half(m, e, s, D);
        if (c < 0) return D;
        if (c == 0) return (D & 1u) ? D + 1 : D;
        ++D;
    }
    return D;  // not reached for a valid estimate
}

// 10^p in double for |p| <= 170: exact powers 10^q (q <= 22) multiplied (p > 0) or divided (p < 0)
// in, so the relative error stays below (|p| / 22 + 1) ulp
PG_HD double pow10_dbl(int p) {
    int q = p >= 0 ? p : -p;
    double r = 1.0;
    while (q >= 22) {
        r = p >= 0 ? r * 1e22 : r / 1e22;
        q -= 22;
    }
    double t = 1.0;
    while (q-- > 0) t *= 10.0;
    return p >= 0 ? r * t : r / t;
}

// Writes "%.<prec>g" of x into out (at least 32 bytes); returns the length.  prec 1..13: the
// double estimate of v 10^s must stay within one of the truth for D < 10^(prec+1).
PG_HD int fmt_g(double x, int prec, char* out) {
    int len = 0;
    uint64_t bits;
#if defined(__CUDA_ARCH__)
    bits = (uint64_t)__double_as_longlong(x);
#else
    __builtin_memcpy(&bits, &x, 8);
#endif
    const bool neg = (bits >> 63) != 0;
    const int be = (int)((bits >> 52) & 0x7FF);
    uint64_t m = bits & ((1ull << 52) - 1);
    if (be == 0x7FF) {
        if (neg) out[len++] = '-';
        const char* t = m ? "nan" : "inf";
        for (int i = 0; i < 3; ++i) out[len++] = t[i];
        return len;
    }
    if (neg) out[len++] = '-';
    if (be == 0 && m == 0) {
        out[len++] = '0';
        return len;
    }
    int e;
    if (be == 0) {
        e = -1074;
    } else {
        m |= 1ull << 52;
        e = be - 1075;
    }
    const double ax = neg ? -x : x;
    // decimal exponent guess from the binary exponent (within one)
    int msb = 63;
    while (!((m >> msb) & 1ull)) --msb;
    const int b2 = e + msb;  // 2^b2 <= ax < 2^(b2+1)
    int k = (int)floor((double)b2 * 0.30102999566398120);
    uint64_t D = 0;
    uint64_t lo = 1;
    for (int i = 1; i < prec; ++i) lo *= 10u;
    const uint64_t hi = lo * 10u;
    for (int it = 0; it < 4; ++it) {
        const int s = prec - 1 - k;
        // v 10^s in double, scaled in two steps so neither factor overflows
        const int s1 = s / 2, s2 = s - s1;
        const double est = ax * pow10_dbl(s1) * pow10_dbl(s2);
        D = round_scaled(m, e, s, est);
        if (D >= hi) {
            ++k;
            continue;
        }
        if (D < lo) {
            --k;
            continue;
        }
        break;
    }
    char dg[20];
    for (int i = prec - 1; i >= 0; --i) {
        dg[i] = (char)('0' + (int)(D % 10u));
        D /= 10u;
    }
    int nd = prec;  // significant digits after dropping trailing zeros
    while (nd > 1 && dg[nd - 1] == '0') --nd;
    const int X = k;
    if (X >= -4 && X < prec) {
        if (X >= 0) {
            for (int i = 0; i <= X; ++i) out[len++] = dg[i];
            if (nd > X + 1) {
                out[len++] = '.';
                for (int i = X + 1; i < nd; ++i) out[len++] = dg[i];
            }
        } else {
            out[len++] = '0';
            out[len++] = '.';
            for (int i = 0; i < -X - 1; ++i) out[len++] = '0';
            for (int i = 0; i < nd; ++i) out[len++] = dg[i];
        }
    } else {
        out[len++] = dg[0];
        if (nd > 1) {
            out[len++] = '.';
            for (int i = 1; i < nd; ++i) out[len++] = dg[i];
        }
        out[len++] = 'e';
        int ax10 = X;
        out[len++] = ax10 < 0 ? '-' : '+';
        if (ax10 < 0) ax10 = -ax10;
        char ed[4];
        int ne = 0;
        while (ax10 > 0) {
            ed[ne++] = (char)('0' + ax10 % 10);
            ax10 /= 10;
        }
        while (ne < 2) ed[ne++] = '0';
        while (ne > 0) out[len++] = ed[--ne];
    }
    return len;
}

}  // namespace pg
