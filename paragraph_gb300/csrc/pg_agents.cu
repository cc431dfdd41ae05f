// pg_agents.cu -- per-agent citation sampling of the preferential-attachment epoch.
//
// Replaces kernelCallStage1/_warped/2/3/4 and the fused ABMKernel (src/kernel.cu:17-402,436-573;
// device bodies src/abm.cu:376-565,577-994).  One warp owns one agent (new paper) and does:
//   1. global race: k draws without replacement from the replica's quantised CDF.  Draw i picks the
//      smallest j with cdf[j] - C(j) > y, where C(j) sums the weights already chosen at ids <= j;
//      the warp searches 32-ary (32 probes per round, ballot), which gives the same j as any other
//      search because the function is monotone and integer.  Arrival times are exponential
//      increments E / R with R the remaining weight.
//   2. neighbourhood race: the 2-hop undirected ball of the anchors (forward and backward rows,
//      the reference's GetOneAndTwoHopNeighborhood semantics) is streamed with load-balanced
//      expansion (32 neighbours' rows at a time, owner found by a shuffle search).  Each element j
//      gets the key E_j / w_j with E_j drawn from Philox keyed by (agent, j), so duplicates in the
//      stream share a key and the k smallest distinct keys are found without deduplicating the
//      ball and without depending on traversal order -- the Efraimidis-Spirakis top-k of the
//      reference (src/abm.cu:529-564) in exponential-clock form.
//   3. merge: the first k distinct nodes of the two races by (time, id) are the agent's citations
//      (weights w_j beta^[j in ball]); they are sorted and appended to the forward CSR, and each
//      cited node's in-degree counter returns the edge's rank for the backward append.
// No per-agent O(n) state exists (the reference clears O(n) bitmaps per agent,
// includes/abm.cuh:178-184, src/abm.cu:722-726).
#include <type_traits>

#include "pg_engine.cuh"
#include "pg_rc.cuh"
#include "pg_scan.cuh"
#include "pg_weights.cuh"
#include "pg_csr.cuh"

namespace pg {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ bool key_less(float ka, int ia, float kb, int ib) {
    return ka < kb || (ka == kb && ia < ib);
}

template <int KCAP>
struct AgentSmem {
    double g_t[KCAP];
    uint64_t c_cq[KCAP];
    int32_t g_id[KCAP];
    int32_t c_id[KCAP];
    float bk[KCAP];
    int32_t bi[KCAP];
    int32_t out[KCAP];
};

// Offer one candidate per lane to the warp's sorted top-k list (bk, bi)[0..nb) of S.
template <typename SM>
__device__ __forceinline__ void topk_offer(bool valid, float key, int id, int k, int& nb, SM& S) {
    const int lane = lane_id();
    bool pass = valid && (nb < k || key_less(key, id, S.bk[k - 1], S.bi[k - 1]));
    unsigned mask = __ballot_sync(kFull, pass);
    while (mask) {
        const int leader = __ffs(mask) - 1;
        const float ck = __shfl_sync(kFull, key, leader);
        const int cid = __shfl_sync(kFull, id, leader);
        int less_cnt = 0;
        bool dup = false;
        for (int i = lane; i < nb; i += 32) {
            const int ii = S.bi[i];
            if (ii == cid) dup = true;
            if (key_less(S.bk[i], ii, ck, cid)) ++less_cnt;
        }
        if (!__any_sync(kFull, dup)) {
            const int pos = __reduce_add_sync(kFull, less_cnt);
            const int last = nb < k ? nb : k - 1;
            for (int hi = last; hi > pos; hi -= 32) {
                const int i = hi - 1 - lane;
                const bool act = i >= pos;
                float tk = 0.0f;
                int ti = 0;
                if (act) {
                    tk = S.bk[i];
                    ti = S.bi[i];
                }
                __syncwarp();
                if (act) {
                    S.bk[i + 1] = tk;
                    S.bi[i + 1] = ti;
                }
                __syncwarp();
            }
            if (lane == 0) {
                S.bk[pos] = ck;
                S.bi[pos] = cid;
            }
            __syncwarp();
            nb = nb < k ? nb + 1 : k;
        }
        pass = pass && lane != leader && (nb < k || key_less(key, id, S.bk[k - 1], S.bi[k - 1]));
        mask = __ballot_sync(kFull, pass);
    }
}

struct AgentCtx {
    const uint64_t* cdf;
    const float* w;
    const int64_t* fwd_off;
    const int32_t* fwd_col;
    const BRow* bwd_row;
    const int32_t* bwd_col;
    uint64_t seed;
    uint32_t rep, ep, unit;
    double beta_m1;
};

__device__ __forceinline__ void boost_key(const AgentCtx& C, bool valid, int z, float& key,
                                          bool& ok) {
    ok = false;
    key = 0.0f;
    if (valid) {
        const float wz = C.w[z];
        if (wz > 0.0f) {
            const u32x4 x = draw(C.seed, kStreamBoost, C.rep, C.ep, C.unit, (uint32_t)z);
            key = -logf_pg(u01f(x.x[0])) / wz;
            ok = true;
        }
    }
}

// The agent's targets sorted (bitonic network in registers, R entries per lane), written to its
// forward row and the edge list, and counted into the in-degree increments.
template <int R>
__device__ __forceinline__ void emit_sorted(const Arena& A, const Replica& rp, int64_t e0, int64_t row0,
                                            const int32_t* arr, int taken, int lane) {
    int v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = i * 32 + lane < taken ? arr[i * 32 + lane] : 0x7fffffff;
    warp_bitonic<R>(v, lane);
    int32_t* fcol = A.fwd_col + rp.ebase;
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int q = i * 32 + lane;
        if (q < taken) {
            const int d = v[i];
            fcol[row0 + q] = d;
            A.e_dst[e0 + q] = d;
            A.e_rank[e0 + q] = atomicAdd(&A.inc[rp.nbase + d], 1);
        }
    }
}

// Append one agent's citations: arrival order to the trace, the sorted row to the forward CSR and
// the epoch edge list, one in-degree increment (whose old value is the edge's rank in the cited
// node's new backward entries) per citation, and the byte-model counters.
template <int KCAP>
__device__ void emit_row(const Arena& A, const Replica& rp, int64_t a, int64_t al, int64_t n,
                         const int32_t* arr, int taken, long long rows, long long elems, long long draws) {
    const int lane = lane_id();
    const int64_t e0 = A.eoff[a];
    if (A.arrivals)
        for (int q = lane; q < taken; q += 32) A.arrivals[e0 + q] = arr[q];
    const int64_t row0 = rp.m + (e0 - A.eoff[rp.abase]);
    if (taken <= 32)
        emit_sorted<1>(A, rp, e0, row0, arr, taken, lane);
    else if (KCAP <= 64 || taken <= 64)
        emit_sorted<2>(A, rp, e0, row0, arr, taken, lane);
    else if (KCAP <= 128 || taken <= 128)
        emit_sorted<4>(A, rp, e0, row0, arr, taken, lane);
    else
        emit_sorted<8>(A, rp, e0, row0, arr, taken, lane);
    if (lane == 0) {
        A.fwd_off[rp.obase + n + al + 1] = row0 + taken;
        atomicAdd(&A.st->rows_expanded, (unsigned long long)rows);
        atomicAdd(&A.st->elems_streamed, (unsigned long long)elems);
        atomicAdd(&A.st->draws, (unsigned long long)draws);
    }
    __syncwarp();
}

template <int KCAP>
__device__ void process_agent(const Arena& A, int64_t a, int k, AgentSmem<KCAP>& S) {
    const int lane = lane_id();
    const int r = replica_of_agent(A.rep, A.R, a);
    const Replica& rp = A.rep[r];
    const int64_t n = rp.n;
    const int64_t al = a - rp.abase;
    AgentCtx C;
    C.cdf = A.cdf + rp.nbase;
    C.w = A.w + rp.nbase;
    C.fwd_off = A.fwd_off + rp.obase;
    C.fwd_col = A.fwd_col + rp.ebase;
    C.bwd_row = A.brow + rp.nbase;
    C.bwd_col = A.bcol + rp.bbase;
    C.seed = A.seed;
    C.rep = (uint32_t)(r + A.rep_base);
    C.ep = (uint32_t)A.st->epoch;
    C.unit = (uint32_t)al;
    C.beta_m1 = rp.beta_m1;
    const int s = cdf_shift(bitsf(rp.wmax_bits), n);
    const double scale = bitsd((uint64_t)(1023 - s) << 52);

    // ---------------------------------------------------------------- 1. global race
    uint64_t R = rp.wq_total;
    double t = 0.0;
    int nc = 0;
    for (int i = 0; i < k; ++i) {
        if (R == 0) break;
        const u32x4 x = draw(C.seed, kStreamGlobal, C.rep, C.ep, C.unit, (uint32_t)i);
        const double E = -log_pg(u01d(x.x[0], x.x[1]));
        t = t + E / ((double)R * scale);
        const uint64_t y = mulhi64(u64of(x.x[2], x.x[3]), R);
        // 32-ary search for the smallest j in [0, n) with F(j) = cdf[j] - C(j) > y
        int64_t lo = 0, hi = n;
        while (true) {
            const int64_t span = hi - lo;
            const int64_t step = span > 32 ? (span + 31) / 32 : 1;
            int64_t p = lo + (int64_t)(lane + 1) * step - 1;
            if (p > hi - 1) p = hi - 1;
            // C(p): chosen weight at ids <= p
            int cl = 0, ch = nc;
            while (cl < ch) {
                const int mid = (cl + ch) >> 1;
                if (S.c_id[mid] <= p)
                    cl = mid + 1;
                else
                    ch = mid;
            }
            const uint64_t cp = cl ? S.c_cq[cl - 1] : 0;
            const bool pred = (C.cdf[p] - cp) > y;
            const unsigned m = __ballot_sync(kFull, pred);
            if (m == 0) {  // F(hi-1) > y is an invariant; report instead of probing out of range
                if (lane == 0) atomicOr(&A.st->error, kErrArg);
                lo = 0;
                break;
            }
            const int L = __ffs(m) - 1;  // lane probing hi-1 is always true
            const int64_t pL = __shfl_sync(kFull, p, L);
            const int64_t pL1 = __shfl_sync(kFull, p, L > 0 ? L - 1 : 0);
            if (span <= 32) {
                lo = pL;
                break;
            }
            hi = pL + 1;
            lo = L > 0 ? pL1 + 1 : lo;
        }
        const int j = (int)lo;
        const uint64_t qj = C.cdf[j] - (j > 0 ? C.cdf[j - 1] : 0);
        // insert j into the sorted chosen list
        int below = 0;
        for (int q = lane; q < nc; q += 32) below += S.c_id[q] < j ? 1 : 0;
        const int pos = __reduce_add_sync(kFull, below);
        for (int top = nc; top > pos; top -= 32) {
            const int q = top - 1 - lane;
            const bool act = q >= pos;
            int tid = 0;
            uint64_t tq = 0;
            if (act) {
                tid = S.c_id[q];
                tq = S.c_cq[q];
            }
            __syncwarp();
            if (act) {
                S.c_id[q + 1] = tid;
                S.c_cq[q + 1] = tq + qj;
            }
            __syncwarp();
        }
        if (lane == 0) {
            S.c_id[pos] = j;
            S.c_cq[pos] = (pos > 0 ? S.c_cq[pos - 1] : 0) + qj;
            S.g_id[i] = j;
            S.g_t[i] = t;
        }
        __syncwarp();
        ++nc;
        R -= qj;
    }
    const int ng = nc;

    // ---------------------------------------------------------------- 2. neighbourhood race
    int nb = 0;
    long long rows = 0, elems = 0;
    if (C.beta_m1 > 0.0) {
        const int na = rp.anchors;
        const u32x4 xa = draw(C.seed, kStreamAnchor, C.rep, C.ep, C.unit, 0);
        uint32_t xr = xa.x[0];
        if (lane == 1) xr = xa.x[1];
        if (lane == 2) xr = xa.x[2];
        if (lane == 3) xr = xa.x[3];
        const int anchor = (int)bounded32(xr, (uint32_t)n);
        {
            float key;
            bool ok;
            boost_key(C, lane < na, anchor, key, ok);
            topk_offer(ok, key, anchor, k, nb, S);
        }
        rows += na;
        elems += na;
        for (int ai = 0; ai < na; ++ai) {
            const int x = __shfl_sync(kFull, anchor, ai);
            const int64_t fb = C.fwd_off[x], fe = C.fwd_off[x + 1];
            int64_t bb, be;
            bspan(C.bwd_row, x, bb, be);
            const int64_t lf = fe - fb;
            const int64_t deg1 = lf + (be - bb);
            rows += deg1;
            elems += deg1;
            for (int64_t base = 0; base < deg1; base += 32) {
                const int64_t idx = base + lane;
                const bool valid = idx < deg1;
                int y = 0;
                if (valid) y = idx < lf ? C.fwd_col[fb + idx] : C.bwd_col[bb + idx - lf];
                {
                    float key;
                    bool ok;
                    boost_key(C, valid, y, key, ok);
                    topk_offer(ok, key, y, k, nb, S);
                }
                int64_t yf = 0, yb = 0, ylf = 0, ylen = 0;
                if (valid) {
                    yf = C.fwd_off[y];
                    ylf = C.fwd_off[y + 1] - yf;
                    int64_t ye;
                    bspan(C.bwd_row, y, yb, ye);
                    ylen = ylf + (ye - yb);
                }
                const int64_t incl = warp_incl_scan<int64_t>(ylen);
                const int64_t total = __shfl_sync(kFull, incl, 31);
                elems += total;
                for (int64_t pb = 0; pb < total; pb += 32) {
                    const int64_t p = pb + lane;
                    const bool v2 = p < total;
                    int o = 0;
#pragma unroll
                    for (int b = 16; b >= 1; b >>= 1) {
                        const int64_t iv = __shfl_sync(kFull, incl, o + b - 1);
                        if (iv <= p) o += b;
                    }
                    const int64_t ex_o = __shfl_sync(kFull, incl - ylen, o);
                    const int64_t yf_o = __shfl_sync(kFull, yf, o);
                    const int64_t ylf_o = __shfl_sync(kFull, ylf, o);
                    const int64_t yb_o = __shfl_sync(kFull, yb, o);
                    int z = 0;
                    if (v2) {
                        const int64_t within = p - ex_o;
                        z = within < ylf_o ? C.fwd_col[yf_o + within]
                                           : C.bwd_col[yb_o + within - ylf_o];
                    }
                    float key;
                    bool ok;
                    boost_key(C, v2, z, key, ok);
                    topk_offer(ok, key, z, k, nb, S);
                }
            }
        }
    }

    // ---------------------------------------------------------------- 3. merge and emit
    int taken = 0, gi = 0, bj = 0;
    while (taken < k && (gi < ng || bj < nb)) {
        const double tb = bj < nb ? (double)S.bk[bj] / C.beta_m1 : 0.0;
        const bool take_g =
            bj >= nb || (gi < ng && (S.g_t[gi] < tb || (S.g_t[gi] == tb && S.g_id[gi] <= S.bi[bj])));
        const int id = take_g ? S.g_id[gi] : S.bi[bj];
        if (take_g)
            ++gi;
        else
            ++bj;
        bool dup = false;
        for (int q = lane; q < taken; q += 32) dup |= (S.out[q] == id);
        if (!__any_sync(kFull, dup)) {
            if (lane == 0) S.out[taken] = id;
            __syncwarp();
            ++taken;
        }
    }
    if (taken != k && lane == 0) atomicOr(&A.st->error, kErrArg);
    emit_row<KCAP>(A, rp, a, al, n, S.out, taken, rows, elems, ng);
}

#include "pg_thin.cuh"
#include "pg_rc_agent.cuh"

// ---------------------------------------------------------------- setup: out-degree + new nodes
__device__ __forceinline__ void d_agent_setup(const Arena& A, int64_t agents, int vb) {
    if (A.st->error) return;
    const int64_t a = (int64_t)vb * blockDim.x + threadIdx.x;
    if (a >= agents) return;
    const int r = replica_of_agent(A.rep, A.R, a);
    const Replica& rp = A.rep[r];
    const int64_t al = a - rp.abase;
    const uint32_t ep = (uint32_t)A.st->epoch;
    const bool rc = A.weight_model == 1;
    // out-degree: Poisson (baseline) or the out-degree bag (refcompat), both as a 257-entry CDF
    const u32x4 x = draw(A.seed, kStreamOutDegree, (uint32_t)(r + A.rep_base), ep, (uint32_t)al, 0);
    const int kraw = poisson_draw(A.tables + (int64_t)r * kTableEntries, kTableEntries,
                                  u64of(x.x[0], x.x[1]));
    int64_t k = kraw < 1 ? 1 : kraw;
    if (rc) {
        const int64_t kmax = rp.n - 1 < kRcMaxOutDegree ? rp.n - 1 : kRcMaxOutDegree;
        if (k > kmax) k = kmax;
    } else {
        if (k > rp.n) k = rp.n;
        if (k > rp.npos) k = rp.npos;
    }
    A.kk[a] = (int32_t)k;
    if (!rc && k > kKSmall) {
        const unsigned long long i = atomicAdd(&A.st->big_count, 1ull);
        A.big_list[i] = (int32_t)a;
    }
    const int64_t slot = rp.nbase + rp.n + al;
    A.pub[slot] = (int32_t)A.st->epoch;
    if (rc) {
        // peak fitness from the power-law table, static window (ABM::AssignPeakFitnessValues,
        // AssignFitnessLagDuration, AssignFitnessPeakDuration; includes/abm.cuh:447-484)
        const u32x4 xf = draw(A.seed, kStreamRcFitness, (uint32_t)(r + A.rep_base), ep, (uint32_t)al, 0);
        A.fit[slot] = (float)rc_peak_draw(A.rc_ftab, u64of(xf.x[0], xf.x[1]));
        A.rc_lag[slot] = 0;
        A.rc_dur[slot] = 1000;
    } else {
        A.fit[slot] = lognormal_fitness(A.seed, (uint32_t)(r + A.rep_base), ep, (uint32_t)al);
    }
    A.indeg[slot] = 0;
    int heavy = 0;
    if (rc && k >= 2) {
        // a generator with many row entries, or a few long ones, makes a long 2-hop stream: such
        // agents are listed for the CTA-wide pass (k_rc_big), mark = list slot + 1
        double w3[3], alpha;
        int32_t gen;
        rc_agent_params(A.seed, (uint32_t)(r + A.rep_base), ep, (uint32_t)al, rp.n, rp.rc_w, rp.rc_alpha, w3,
                        &alpha, &gen);
        const int64_t* fo = A.fwd_off + rp.obase;
        const BRow* br = A.brow + rp.nbase;
        int64_t gb0, gb1;
        bspan(br, gen, gb0, gb1);
        const int64_t gd = (fo[gen + 1] - fo[gen]) + (gb1 - gb0);
        bool big = gd >= kRcBigGd;
        if (!big) {
            const int32_t* fc = A.fwd_col + rp.ebase;
            const int32_t* bc = A.bcol + rp.bbase;
            int64_t len = 0;
            for (int64_t e = fo[gen]; e < fo[gen + 1]; ++e) {
                const int32_t y = fc[e];
                len += (fo[y + 1] - fo[y]) + blen(br, y);
            }
            for (int64_t e = gb0; e < gb1; ++e) {
                const int32_t y = bc[e];
                len += (fo[y + 1] - fo[y]) + blen(br, y);
            }
            big = len >= kRcBigStream;
        }
        if (big) {
            const unsigned long long q = atomicAdd(&A.st->rc_big_count, 1ull);
            if (q < (unsigned long long)kRcBigCap) {
                A.heavy_list[q] = (int32_t)a;
                heavy = (int)q + 1;
            }
        }
    }
    if (!rc && A.sampler == kSamplerThinning && rp.p_global < 1.0) {
        // the anchors (the same draw the agent kernel makes): flag the hubs among them, whose
        // hub-pair rows are the only ones read, and mark the agent heavy when an anchor is a hub or
        // the anchors' rows would not all fit the smaller shared frontier (the agent then tests
        // memberships against global rows); heavy agents are taken first, so none starts late
        const u32x4 xa = draw(A.seed, kStreamAnchor, (uint32_t)(r + A.rep_base), ep, (uint32_t)al, 0);
        const int64_t* fo = A.fwd_off + rp.obase;
        const BRow* br = A.brow + rp.nbase;
        int64_t zsize = rp.anchors;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i >= rp.anchors) break;
            const int64_t x = bounded32(xa.x[i], (uint32_t)rp.n);
            const int hs = A.hslot[rp.nbase + x];
            if (hs >= 0) {
                atomicOr(&A.hub_need[(int64_t)r * (kHeavyMax / 32) + (hs >> 5)], 1u << (hs & 31));
                heavy = 1;
            } else {
                zsize += (fo[x + 1] - fo[x]) + blen(br, x);
            }
        }
        if (zsize > kZCap / 2) heavy = 1;
        if (k > kKSmall) heavy = 0;  // the k <= 256 kernel has its own list
        if (heavy) A.heavy_list[atomicAdd(&A.st->heavy_count, 1ull)] = (int32_t)a;
    }
    A.heavy_mark[a] = heavy;
    if (A.anchors_out) {
        // the same draw the agent kernels make for the neighbourhood (recorded for traces)
        const u32x4 xa = draw(A.seed, kStreamAnchor, (uint32_t)(r + A.rep_base), ep, (uint32_t)al, 0);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            A.anchors_out[a * 4 + i] = i < rp.anchors ? (int32_t)bounded32(xa.x[i], (uint32_t)rp.n) : -1;
    }
}

__global__ void __launch_bounds__(256) k_agent_setup(Arena A, int64_t agents) { d_agent_setup(A, agents, blockIdx.x); }

// After the edge-offset scan: totals and capacity checks.
__device__ __forceinline__ void d_edges_check(const Arena& A, int64_t agents) {
    if (A.st->error) return;
    const int64_t E = A.eoff[agents];
    if (threadIdx.x == 0) {
        A.st->edges = E;
        if (E > A.edge_cap) atomicOr(&A.st->error, kErrCapacity);
    }
    for (int r = threadIdx.x; r < A.R; r += blockDim.x) {
        const Replica& rp = A.rep[r];
        const int64_t er = A.eoff[rp.abase + rp.delta] - A.eoff[rp.abase];
        if (rp.m + er > rp.m_cap) atomicOr(&A.st->error, kErrCapacity);
    }
}

__global__ void k_edges_check(Arena A, int64_t agents) { d_edges_check(A, agents); }

// Shapes of the k <= 64 thinning kernel (pg_tuning.small_hash = HS): 0 -- a 2048-slot frontier hash
// and 512-entry stage buffers; 1 -- 1024 slots and 1024-entry stages; both 4 CTAs per SM.  The
// k <= 256 kernel always has 1024 slots and 512-entry stages.  Shapes with more resident warps were
// measured on the PA workload and were slower: 1024 slots and 512-entry stages at 5 CTAs per SM (96
// registers) by 9 %, and 2048 slots and 256-entry stages at 5 CTAs per SM with the heavy agents'
// instance out of line (the lean one then fits 96 registers) by 8 %.
template <int KCAP, int HS>
struct ThinStage {
    static constexpr int value = (KCAP <= kKSmall && HS == 1) ? 1024 : 512;
};
template <int KCAP, int HS>
struct ThinHash {
    static constexpr int value = (KCAP <= kKSmall && HS == 0) ? 2 * kZCap : kZCap;
};
template <int KCAP, int HS>
__host__ __device__ constexpr size_t thin_smem_bytes() {
    return sizeof(ThinSmem<KCAP, ThinHash<KCAP, HS>::value, ThinStage<KCAP, HS>::value>) * kAgentWarps;
}

// The agent loop of one warp.  Thinning variants: the warp's shared memory is dsm + warp * stride
// (the calling kernel's dynamic shared memory; stride >= sizeof of this variant's ThinSmem); the
// enumeration variants use static shared memory.
template <int KCAP, bool BIG, bool THIN, int HS = 0>
__device__ __forceinline__ void d_agents(const Arena& A, int64_t agents, unsigned char* dsm, size_t stride) {
    constexpr int HCAP = ThinHash<KCAP, HS>::value;
    constexpr int STAGE = ThinStage<KCAP, HS>::value;
    using Smem = typename std::conditional<THIN, ThinSmem<KCAP, HCAP, STAGE>, AgentSmem<KCAP>>::type;
    Smem* sp;
    if constexpr (THIN) {
        sp = reinterpret_cast<Smem*>(dsm + (threadIdx.x >> 5) * stride);
    } else {
        __shared__ Smem agent_ssm[kAgentWarps];
        sp = &agent_ssm[threadIdx.x >> 5];
        (void)dsm;
        (void)stride;
    }
    if (A.st->error) return;
    Smem& S = *sp;
    const int lane = lane_id();
    // the small thinning kernel walks the heavy list, then every agent not on it
    constexpr bool kHeavyFirst = THIN && !BIG;
    const int64_t hc = kHeavyFirst ? (int64_t)A.st->heavy_count : 0;
    const int64_t limit = BIG ? (int64_t)A.st->big_count : agents + hc;
    uint32_t phase = 0;
    if constexpr (THIN) {
        if (lane == 0) {
            mbar_init(&S.bar[0], 1);
            mbar_init(&S.bar[1], 1);
        }
        fence_proxy_async();
        __syncwarp();
    }
    while (true) {
        long long q = 0;
        if (lane == 0)
            q = (long long)atomicAdd(BIG ? &A.st->queue_big : &A.st->queue_small, 1ull);
        q = __shfl_sync(kFull, q, 0);
        if (q >= limit) break;
        int64_t a;
        bool general = true;  // heavy-listed (or k > 64) agents take the general instance
        if (BIG)
            a = (int64_t)A.big_list[q];
        else if (q < hc)
            a = (int64_t)A.heavy_list[q];
        else {
            a = q - hc;
            if (kHeavyFirst && A.heavy_mark[a]) continue;
            general = !kHeavyFirst;
        }
        const int k = A.kk[a];
        if (!BIG && k > KCAP) continue;
        if constexpr (THIN) {
            const bool ok = general ? process_agent_thin<KCAP, HCAP, STAGE, true>(A, a, k, S, phase)
                                    : process_agent_thin<KCAP, HCAP, STAGE, false>(A, a, k, S, phase);
            if (!ok) break;
        } else
            process_agent<KCAP>(A, a, k, S);
    }
    if constexpr (THIN) {
        // every copy this warp issued has been waited for: the barriers' memory can be reused
        __syncwarp();
        if (lane == 0) {
            mbar_inval(&S.bar[0]);
            mbar_inval(&S.bar[1]);
        }
        __syncwarp();
    }
}

template <int KCAP, bool BIG, bool THIN, int HS = 0>
__global__ void __launch_bounds__(kAgentWarps * 32, 4) k_agents(Arena A, int64_t agents) {
    // the thinning variants hold two stage buffers per warp and go past 48 KiB: dynamic
    extern __shared__ __align__(16) unsigned char agent_dsm[];
    constexpr size_t stride = thin_smem_bytes<KCAP, HS>() / kAgentWarps;
    d_agents<KCAP, BIG, THIN, HS>(A, agents, agent_dsm, stride);
}

__global__ void __launch_bounds__(kAgentWarps * 32) k_agents_rc(Arena A, int64_t agents) {
    __shared__ RcSmem smem[kAgentWarps];
    if (A.st->error) return;
    RcSmem& S = smem[threadIdx.x >> 5];
    const int lane = lane_id();
    while (true) {
        long long q = 0;
        if (lane == 0) q = (long long)atomicAdd(&A.st->queue_small, 1ull);
        q = __shfl_sync(kFull, q, 0);
        if (q >= agents) break;
        process_agent_rc(A, q, A.kk[q], S);
    }
}

// The 2-hop streams of the refcompat agents the setup listed (long streams), one CTA per
// agent: the warps take the 32-entry chunks of every group's stream in turn, each keeping its own top
// min(k, kKMax) of its part of the stream with the keys, validity and duplicate rule of the
// one-warp path; the lists are merged pairwise (dropping entries that two warps both reached; the
// k smallest distinct (key, id) pairs do not depend on the merge order) and warp 0 stores
// the sorted ids and the stream's counters for k_agents_rc.
constexpr int kRcBigWarps = 8;

__global__ void __launch_bounds__(kRcBigWarps * 32) k_rc_big(Arena A) {
    __shared__ RcSmem sm[kRcBigWarps];
    __shared__ int s_nb[kRcBigWarps];
    __shared__ long long s_cnt[2];
    __shared__ long long s_item;
    if (cta_error(A)) return;
    const int warp = threadIdx.x >> 5, lane = lane_id();
    RcSmem& S = sm[warp];
    const long long listed = (long long)A.st->rc_big_count;
    const long long total = listed < kRcBigCap ? listed : kRcBigCap;
    while (true) {
        if (threadIdx.x == 0) s_item = (long long)atomicAdd(&A.st->rc_big_queue, 1ull);
        if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
        __syncthreads();
        const long long it = s_item;
        if (it >= total) break;
        const int64_t a = A.heavy_list[it];
        const int r = replica_of_agent(A.rep, A.R, a);
        const Replica& rp = A.rep[r];
        const int64_t al = a - rp.abase;
        RcCtx X;
        X.fo = A.fwd_off + rp.obase;
        X.fc = A.fwd_col + rp.ebase;
        X.br = A.brow + rp.nbase;
        X.bc = A.bcol + rp.bbase;
        X.pa = A.rc_pa + rp.nbase;
        X.rec = A.rc_rec + rp.nbase;
        X.fit = A.rc_fit + rp.nbase;
        X.seed = A.seed;
        X.rep = (uint32_t)(r + A.rep_base);
        X.ep = (uint32_t)A.st->epoch;
        X.unit = (uint32_t)al;
        double alpha;
        rc_agent_params(A.seed, X.rep, X.ep, X.unit, rp.n, rp.rc_w, rp.rc_alpha, X.w3, &alpha, &X.gen);
        X.gf0 = X.fo[X.gen];
        X.glf = X.fo[X.gen + 1] - X.gf0;
        int64_t gb1;
        bspan(X.br, X.gen, X.gb0, gb1);
        X.gd = X.glf + (gb1 - X.gb0);
        const int k = A.kk[a];
        const int kcap = k < kKMax ? k : kKMax;
        int nb = 0;
        long long rows = 0, elems = 0;
        rc_2hop_slice(X, 32 * warp, 32 * kRcBigWarps, warp == 0, kcap, nb, rows, elems, S);
        if (lane == 0) {
            s_nb[warp] = nb;
            atomicAdd((unsigned long long*)&s_cnt[0], (unsigned long long)rows);
            atomicAdd((unsigned long long*)&s_cnt[1], (unsigned long long)elems);
        }
        __syncthreads();
        // pairwise merges, log2(warps) rounds: warp w takes warp w + h's list when w % 2h == 0
        for (int h = 1; h < kRcBigWarps; h <<= 1) {
            if ((warp & (2 * h - 1)) == 0) {
                const int w = warp + h;
                const int nw = s_nb[w];
                for (int q0 = 0; q0 < nw; q0 += 32) {
                    const int q = q0 + lane;
                    const bool v = q < nw;
                    rc_topk_offer(v, v ? sm[w].bk[q] : 0.0f, v ? sm[w].bi[q] : 0, kcap, nb, S);
                }
                if (lane == 0) s_nb[warp] = nb;
            }
            __syncthreads();
        }
        if (warp == 0) {
            int32_t* ids = A.rc_big_id + it * kKMax;
            for (int q = lane; q < nb; q += 32) ids[q] = S.bi[q];
            if (lane == 0) {
                long long* meta = A.rc_big_meta + it * 3;
                meta[0] = nb;
                meta[1] = s_cnt[0];
                meta[2] = s_cnt[1];
            }
        }
        __syncthreads();  // the lists and counters are reused by the next agent
    }
}

void launch_rc_big(const Arena& A, int num_sms, cudaStream_t s) {
    k_rc_big<<<(unsigned)num_sms * 2, kRcBigWarps * 32, 0, s>>>(A);
}

static int g_blocks_rc = 0;

cudaError_t init_rc_kernels() {
    if (g_blocks_rc) return cudaSuccess;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_rc, k_agents_rc, kAgentWarps * 32, 0);
    if (g_blocks_rc < 1) g_blocks_rc = 1;
    return e;
}

void launch_rc_agents(const Arena& A, int64_t agents, int num_sms, cudaStream_t s) {
    if (agents <= 0) return;
    int64_t grid = (int64_t)num_sms * (g_blocks_rc ? g_blocks_rc : 1);
    const int64_t need = (agents + kAgentWarps - 1) / kAgentWarps;
    if (grid > need) grid = need;
    k_agents_rc<<<(unsigned)grid, kAgentWarps * 32, 0, s>>>(A, agents);
}

static int g_blocks[2][2] = {{0, 0}, {0, 0}};  // [thin][big]
static int g_blocks_hs[2] = {0, 0};             // thinning, k <= 64, by shape (small_hash)

void launch_agent_setup(const Arena& A, int64_t agents, cudaStream_t s) {
    if (agents <= 0) return;
    k_agent_setup<<<(unsigned)((agents + 255) / 256), 256, 0, s>>>(A, agents);
    launch_scan_i32_to_i64(A.kk, A.eoff, agents, A.blocksum, s);
    k_edges_check<<<1, 256, 0, s>>>(A, agents);
}

// Occupancy of the persistent agent kernels; called once per process before any capture.
cudaError_t init_agent_kernels() {
    if (g_blocks[0][0]) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    const int th = kAgentWarps * 32;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks[0][0], k_agents<kKSmall, false, false>, th, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks[0][1], k_agents<kKMax, true, false>, th, 0);
    constexpr size_t d0 = thin_smem_bytes<kKSmall, 0>(), d1 = thin_smem_bytes<kKSmall, 1>(),
                     db = thin_smem_bytes<kKMax, 0>();
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_agents<kKSmall, false, true, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d0);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_agents<kKSmall, false, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_agents<kKMax, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)db);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_hs[0], k_agents<kKSmall, false, true, 0>, th, d0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks_hs[1], k_agents<kKSmall, false, true, 1>, th, d1);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_blocks[1][1], k_agents<kKMax, true, true>, th, db);
    g_blocks[1][0] = g_blocks_hs[0];
    for (auto& row : g_blocks)
        for (int& b : row)
            if (b < 1) b = 1;
    for (int& b : g_blocks_hs)
        if (b < 1) b = 1;
    return e;
}

// Warps of the agent kernels that can be resident at once (the rows of the global anchor table).
int64_t agent_warp_slots(int num_sms) {
    int mb = 1;
    for (int b : g_blocks_hs) mb = b > mb ? b : mb;
    for (auto& row : g_blocks)
        for (int b : row) mb = b > mb ? b : mb;
    const int64_t sep = (int64_t)num_sms * mb * kAgentWarps;
    const int64_t per = (int64_t)(2 * num_sms) * 8;  // the epoch kernel: 2 CTAs of 8 warps per SM at most
    return sep > per ? sep : per;
}

int agent_occupancy(int thin, int small_hash) {
    if (!thin) return g_blocks[0][0];
    return g_blocks_hs[small_hash == 1 ? 1 : 0];
}

void launch_agents(const Arena& A, int64_t agents, int num_sms, cudaStream_t s) {
    if (agents <= 0) return;
    const int t = A.sampler == kSamplerThinning ? 1 : 0;
    const int hs = t && A.tune_small_hash == 1 ? 1 : 0;
    int per_sm = agent_occupancy(t, hs);
    if (A.tune_agent_ctas > 0 && A.tune_agent_ctas < per_sm) per_sm = A.tune_agent_ctas;
    int64_t need = (agents + kAgentWarps - 1) / kAgentWarps;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > need) grid = need;
    const unsigned gbig = (unsigned)num_sms * g_blocks[t][1];
    const int th = kAgentWarps * 32;
    if (t) {
        if (hs == 1)
            k_agents<kKSmall, false, true, 1><<<(unsigned)grid, th, thin_smem_bytes<kKSmall, 1>(), s>>>(A, agents);
        else
            k_agents<kKSmall, false, true, 0><<<(unsigned)grid, th, thin_smem_bytes<kKSmall, 0>(), s>>>(A, agents);
        k_agents<kKMax, true, true><<<gbig, th, thin_smem_bytes<kKMax, 0>(), s>>>(A, agents);
    } else {
        k_agents<kKSmall, false, false><<<(unsigned)grid, th, 0, s>>>(A, agents);
        k_agents<kKMax, true, false><<<gbig, th, 0, s>>>(A, agents);
    }
}


// ---------------------------------------------------------------- one persistent kernel per epoch
// The thinning epoch of every replica as ONE cooperative launch (one CTA pair per SM, all CTAs
// resident), instead of the two dozen launches above.  The phases are the same device bodies the
// separate kernels run -- tiles and blocks walked by the CTAs in turn, single-CTA steps on one CTA,
// grid-stride loops as they are -- so every result is bit-identical to the launch sequence.  A grid
// barrier separates dependent phases; independent stages share a phase (the hub index beside the
// weights and the CDF, the old-entry copy beside the placement of the new ones).  Each barrier
// wait is bounded: on expiry the CTA sets the timeout bit of the error word and goes on, and every
// later phase sees the bit and skips its work, so the launch always ends.
constexpr int kEpochThreads = 256;
constexpr int kEpochWarps = kEpochThreads / 32;
constexpr uint32_t kGridWaitPolls = 1u << 24;  // with a 64 ns back-off: about a second at least

__device__ __forceinline__ void grid_sync(const Arena& A) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = &A.st->gbar_gen;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(&A.st->gbar_count, 1u) == gridDim.x - 1) {
            atomicExch(&A.st->gbar_count, 0u);
            __threadfence();
            atomicAdd(&A.st->gbar_gen, 1u);
        } else {
            for (uint32_t i = 0; *gen == g; ++i) {
                if (i >= kGridWaitPolls) {
                    atomicOr(&A.st->error, kErrTimeout);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// per-warp shared memory of the agent phase: the larger of the two thinning variants it runs (the
// k <= 64 one with the 1024-slot frontier and 1024-entry stages)
constexpr size_t kEpochWarpSmem =
    thin_smem_bytes<kKSmall, 1>() > thin_smem_bytes<kKMax, 0>() ? thin_smem_bytes<kKSmall, 1>() / kAgentWarps
                                                                  : thin_smem_bytes<kKMax, 0>() / kAgentWarps;
constexpr size_t kEpochSmem = kEpochWarps * kEpochWarpSmem;

__global__ void __launch_bounds__(kEpochThreads, 2) k_epoch(Arena A, int64_t epoch, int64_t agents, int G) {
    extern __shared__ __align__(16) unsigned char ep_dsm[];
    const int T = A.ntiles;
    const int hub_items = A.R * kHeavyMax * G;
    // epoch start: new-node counts and agent offsets
    if (blockIdx.x == 0) d_epoch_begin(A, epoch, -1);
    grid_sync(A);
    // hub histogram and weights
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        d_hub_hist(A, t);
        d_weights(A, t);
        __syncthreads();
    }
    grid_sync(A);
    // hub threshold; tile-local CDF scans
    if (blockIdx.x == 0) d_hub_pick(A);
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        d_cdf_tiles(A, t);
        __syncthreads();
    }
    grid_sync(A);
    // hubs leaving and joining; tile offsets of the CDF (on the last CTA, so CTA 0 is not the only
    // one with extra work)
    for (int t = blockIdx.x; t < T; t += gridDim.x) d_hub_collect(A, t);
    if (blockIdx.x == gridDim.x - 1) d_tile_scan(A);
    grid_sync(A);
    // hub bits; CDF offsets and guide marks
    if (blockIdx.x == 0) d_hub_assign(A);
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        d_cdf_add(A, t);
        __syncthreads();
    }
    grid_sync(A);
    // bits cleared by the hubs that left; guide table; per-agent out-degrees, new nodes, heavy lists
    for (int i = blockIdx.x; i < hub_items; i += gridDim.x) d_hub_mask<false>(A, G, i);
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        d_guide_fill(A, t);
        __syncthreads();
    }
    const int setup_blocks = (int)((agents + 255) / 256);
    for (int b = blockIdx.x; b < setup_blocks; b += gridDim.x) d_agent_setup(A, agents, b);
    grid_sync(A);
    // bits set by the hubs that joined; edge offsets: exclusive scan of the out-degrees (reduce,
    // block sums, apply)
    for (int i = blockIdx.x; i < hub_items; i += gridDim.x) d_hub_mask<true>(A, G, i);
    const int nb = (int)((agents + kScanBlock - 1) / kScanBlock);
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        d_scan_reduce<int32_t>(A.kk, agents, A.blocksum, b);
        __syncthreads();
    }
    grid_sync(A);
    if (blockIdx.x == 0) d_scan_blocksums(A.blocksum, nb);
    grid_sync(A);
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        d_scan_apply<int32_t>(A.kk, agents, A.blocksum, nb, A.eoff, b);
        __syncthreads();
    }
    grid_sync(A);
    // capacity check; hub-pair rows for the hub anchors
    if (blockIdx.x == 0) d_edges_check(A, agents);
    for (int i = blockIdx.x; i < hub_items; i += gridDim.x) {
        d_hub_pairs(A, G, i);
        __syncthreads();
    }
    grid_sync(A);
    // the agents: k <= 256 queue, then the k <= 64 queue (heavy list first)
    d_agents<kKMax, true, true>(A, agents, ep_dsm, kEpochWarpSmem);
    d_agents<kKSmall, false, true, 1>(A, agents, ep_dsm, kEpochWarpSmem);
    grid_sync(A);
    // backward append: the cited rows' new lengths, new spans for the rows that outgrew theirs
    d_bwd_grow(A, agents);
    grid_sync(A);
    // the moved rows' old entries copied, new entries placed (disjoint positions)
    d_bwd_reloc(A);
    d_bwd_place(A, agents);
    d_copy_out(A, agents, reinterpret_cast<int32_t*>(ep_dsm));  // this phase uses no other shared memory
    grid_sync(A);
    // appended segments sorted
    d_sort_small(A);
    __syncthreads();
    d_sort_large(A, reinterpret_cast<uint32_t*>(ep_dsm), (int64_t)(kEpochSmem / 4));
    grid_sync(A);
    if (blockIdx.x == 0) d_epoch_end(A, agents);
}

static int g_epoch_ctas = 0;

cudaError_t init_epoch_kernel(int num_sms) {
    if (g_epoch_ctas) return cudaSuccess;
    int dev = 0, coop = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_epoch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEpochSmem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_epoch, kEpochThreads, kEpochSmem);
    if (e != cudaSuccess || !coop || per_sm < 1) {
        cudaGetLastError();
        g_epoch_ctas = -1;  // not available on this device: the launch sequence is used
        return cudaSuccess;
    }
    g_epoch_ctas = num_sms * (per_sm < 2 ? per_sm : 2);
    return cudaSuccess;
}

int epoch_kernel_ctas() { return g_epoch_ctas > 0 ? g_epoch_ctas : 0; }

cudaError_t launch_epoch_kernel(const Arena& A, int64_t epoch, int64_t agents, cudaStream_t s) {
    if (g_epoch_ctas <= 0) return cudaErrorNotSupported;
    Arena a = A;
    int G = A.R >= 64 ? 1 : 64 / A.R;
    void* args[] = {&a, &epoch, &agents, &G};
    return cudaLaunchCooperativeKernel((const void*)k_epoch, dim3((unsigned)g_epoch_ctas), dim3(kEpochThreads), args,
                                       kEpochSmem, s);
}

}  // namespace pg
