// pg_rc.cuh -- host/device helpers of the refcompat functor: ParAGraph's own per-paper model
// (linear pa/rec/fit score mix, budget split between the generator's 1-hop and 2-hop sets and a
// uniform fill, same-year citations), on the engine's graph state.
//
// Restated from the reference:
//   scores      ABM::FillInDegreeArr / FillFitnessArr / FillRecencyArr / CalculateScores
//               (src/abm.cu:112-208,324-338): pa_j = (indeg_j^gamma + 1) / sum,
//               fit_j = (f_j^gamma + 1) / sum, rec_j = P(age_j) / (count(age_j) * sum of P over the
//               ages present); score = w_pa pa + w_rec rec + w_fit fit.
//   fitness     f_j = 1 before pub+lag, the peak value until pub+lag+dur, then
//               (int)(peak / (t - pub - lag - dur + 1)^decay)  (src/abm.cu:152-176); new papers
//               draw the peak from P(v) ~ v^-1.634, v in 1..1000 (includes/abm.cuh:469-484).
//   budget      d from the out-degree bag; one citation of the generator; same-year citation for
//               floor(delta * same_year) agents; rsv = floor(fully_random d);
//               in = min(ceil((d-1-sy-rsv) alpha), |N1|); out = min(d-1-sy-rsv-in, |N2|);
//               the rest uniform (src/kernel.cu:230-273,320-343,377-401).
//   picks       Efraimidis-Spirakis top-k over N1 and over N2 by score (src/abm.cu:461-565), here in
//               exponential-clock form: the k smallest E_j / score_j, E_j exponential keyed by
//               (agent, j); the uniform fill rejects the generator and earlier picks
//               (src/abm.cu:386-432).
// Integer sums (128-bit) make the normalisers independent of the summation order, so the GPU and
// the CPU restatement compute identical scores.
#pragma once
#include "pg_engine.cuh"

namespace pg {

// (hi, lo) 128-bit integer to double, one fixed rounding sequence on host and device
PG_HD double u128_to_d(uint64_t hi, uint64_t lo) { return (double)hi * 0x1p64 + (double)lo; }

// x^e + 1 as a 128-bit integer (x < 2^31, e <= 4)
PG_HD void pow1_u128(uint64_t x, int e, uint64_t* hi, uint64_t* lo) {
    uint64_t h = 0, l = 1;
    for (int i = 0; i < e; ++i) {
        const uint64_t nl = l * x;
        h = h * x + mulhi64(l, x);
        l = nl;
    }
    l += 1;
    if (l == 0) ++h;
    *hi = h;
    *lo = l;
}

// fitness of a node at epoch t
PG_HD int32_t rc_fitness_at(int64_t pub, int64_t lag, int64_t dur, int64_t peak, int64_t t, int decay) {
    if (pub + lag > t) return 1;
    if (pub + lag + dur >= t) return (int32_t)peak;
    const int64_t b = t - pub - lag - dur + 1;
    int64_t den = 1;
    for (int i = 0; i < decay; ++i) den *= b;
    return (int32_t)((double)peak / (double)den);
}

// A bijection of [0, 2^bits): three rounds of xor with a key word, multiplication by an odd key
// word and a right xorshift.
PG_HD uint32_t rc_perm(uint32_t x, int bits, const u32x4& key) {
    const uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    const int h = bits / 2 + 1;
    for (int r = 0; r < 3; ++r) {
        x = (x ^ key.x[r]) & mask;
        x = (x * (key.x[(r + 1) & 3] | 1u)) & mask;
        if (h < bits) x ^= x >> h;
    }
    return x;
}

// 1 when agent al is one of exactly floor(delta * same_year) same-year citers (a keyed permutation
// of the epoch's agents, cycle-walked into [0, delta)); its target n + U[0, delta) in *tgt.
PG_HD int rc_same_year(uint64_t seed, uint32_t rep, uint32_t ep, int64_t al, int64_t delta,
                       double same_year, int64_t n, int32_t* tgt) {
    const int64_t S = (int64_t)floor((double)delta * same_year);
    if (S <= 0) return 0;
    int bits = 1;
    while (bits < 31 && ((int64_t)1 << bits) < delta) ++bits;
    const u32x4 key = draw(seed, kStreamSameYear, rep, ep, 0xFFFFFFFFu, 0);
    uint32_t x = (uint32_t)al;
    do {
        x = rc_perm(x, bits, key);
    } while ((int64_t)x >= delta);
    if ((int64_t)x >= S) return 0;
    const u32x4 r = draw(seed, kStreamSameYear, rep, ep, (uint32_t)al, 0);
    *tgt = (int32_t)(n + (int64_t)bounded32(r.x[0], (uint32_t)delta));
    return 1;
}

// Per-agent weights (normalised), alpha and generator.
PG_HD void rc_agent_params(uint64_t seed, uint32_t rep, uint32_t ep, uint32_t unit, int64_t n,
                           const double* w_fixed, double alpha_fixed, double* w3, double* alpha,
                           int32_t* gen) {
    const u32x4 r0 = draw(seed, kStreamRcAgent, rep, ep, unit, 0);
    const u32x4 r1 = draw(seed, kStreamRcAgent, rep, ep, unit, 1);
    const u32x4 r2 = draw(seed, kStreamRcAgent, rep, ep, unit, 2);
    const double wp = w_fixed[0] >= 0.0 ? w_fixed[0] : u01d(r0.x[0], r0.x[1]);
    const double wr = w_fixed[0] >= 0.0 ? w_fixed[1] : u01d(r0.x[2], r0.x[3]);
    const double wf = w_fixed[0] >= 0.0 ? w_fixed[2] : u01d(r1.x[0], r1.x[1]);
    const double sum = wp + wr + wf;
    w3[0] = wp / sum;
    w3[1] = wr / sum;
    w3[2] = wf / sum;
    *alpha = alpha_fixed >= 0.0 ? alpha_fixed : u01d(r1.x[2], r1.x[3]);
    *gen = (int32_t)bounded32(r2.x[0], (uint32_t)n);
}

// Efraimidis-Spirakis key of node j for agent unit: E / score, E = -log(U(0,1]); +inf when the
// score is not positive.
PG_HD float rc_key(uint64_t seed, uint32_t rep, uint32_t ep, uint32_t unit, int32_t j, double score) {
    if (!(score > 0.0)) return bitsf(0x7F800000u);
    const u32x4 r = draw(seed, kStreamRcKey, rep, ep, unit, (uint32_t)j);
    const double E = -log_pg(u01d(r.x[0], r.x[1]));
    return (float)(E / score);
}

// Peak fitness of a new paper: inversion of the 1000-entry CDF table.
PG_HD int32_t rc_peak_draw(const uint64_t* table, uint64_t u) {
    for (int i = 0; i < kRcFitMax; ++i)
        if (u < table[i]) return i + 1;
    return kRcFitMax;
}

// ---- host tables
// Out-degree bag as 257 CDF thresholds scaled to 2^64 (values clipped to [0, 256]); the reference
// draws a uniform index into the bag (ABM::PopulateOutDegreeArr, src/abm.cu:282-290), which has the
// same distribution.
inline void rc_bag_table_host(const int32_t* bag, int64_t len, uint64_t* table) {
    int64_t cnt[kTableEntries] = {0};
    for (int64_t i = 0; i < len; ++i) {
        const int32_t v = bag[i] < 0 ? 0 : (bag[i] > kTableEntries - 1 ? kTableEntries - 1 : bag[i]);
        ++cnt[v];
    }
    int64_t cum = 0;
    for (int v = 0; v < kTableEntries; ++v) {
        cum += cnt[v];
        table[v] = (cum >= len || v == kTableEntries - 1)
                       ? ~0ull
                       : (uint64_t)((((unsigned __int128)cum) << 64) / (unsigned __int128)len);
    }
}

// Peak-fitness distribution P(v) ~ v^-1.634, v in 1..1000, as CDF thresholds scaled to 2^64.
inline void rc_fitness_table_host(uint64_t* table) {
    double p[kRcFitMax], tot = 0.0;
    for (int i = 0; i < kRcFitMax; ++i) {
        p[i] = exp_pg(-1.634 * log_pg((double)(i + 1)));
        tot += p[i];
    }
    double cum = 0.0;
    for (int i = 0; i < kRcFitMax; ++i) {
        cum += p[i];
        const double q = cum / tot;
        table[i] = (q >= 1.0 || i == kRcFitMax - 1) ? ~0ull : (uint64_t)(q * 0x1p64);
    }
}

}  // namespace pg
