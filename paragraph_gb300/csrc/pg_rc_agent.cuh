// pg_rc_agent.cuh -- the refcompat agent: ParAGraph's own per-paper citation rule (included by
// pg_agents.cu after the top-k and emit helpers).
//
// One warp owns one agent (new paper) of out-degree d and, in arrival order, cites
//   its generator g (uniform over the existing papers; getGeneratorNode, src/abm.cu:567-574),
//   a paper of its own epoch when it is a same-year citer (MakeSameYearCitations, src/abm.cu:376-384),
//   the `in` best of the generator's 1-hop set N1 and the `out` best of its 2-hop set N2 (N2 without
//   N1 and g) by Efraimidis-Spirakis keys on the linear score (ABMKernelStage2/3 with
//   MakePopulateCitations, src/abm.cu:461-565; budget split src/kernel.cu:230-273,320-343),
//   and uniformly drawn papers from [0, n-1) that are neither g nor already cited
//   (MakeUniformRandomCitations, src/abm.cu:386-432).
// The 2-hop stream is load-balanced over the warp: 32 entries of N1 at a time, their rows
// concatenated and split evenly over the lanes.  Keys are functions of (agent, node), so the stream
// is never deduplicated and its order does not matter.

struct RcSmem {
    float bk[kKMax];    // top-k keys, ascending
    int32_t bi[kKMax];  // their ids
    int32_t arr[kKMax]; // citations in arrival order
    int32_t out[kKMax]; // sorted row (emit)
};

__device__ __forceinline__ bool rc_in_rows(const int64_t* fo, const int32_t* fc, const int64_t* bo,
                                           const int32_t* bc, int32_t g, int32_t v) {
    return contains(fc, fo[g], fo[g + 1], v) || contains(bc, bo[g], bo[g + 1], v);
}

__device__ void process_agent_rc(const Arena& A, int64_t a, int k, RcSmem& S) {
    const int lane = lane_id();
    const unsigned below = (1u << lane) - 1u;
    const int r = replica_of_agent(A.rep, A.R, a);
    const Replica& rp = A.rep[r];
    const int64_t n = rp.n, al = a - rp.abase;
    const uint32_t ep = (uint32_t)A.st->epoch, unit = (uint32_t)al, rep = (uint32_t)(r + A.rep_base);
    const int64_t* fo = A.fwd_off + rp.obase;
    const int32_t* fc = A.fwd_col + rp.ebase;
    const int64_t* bo = A.bwd_off_cur + rp.obase;
    const int32_t* bc = A.bwd_col_cur + rp.ebase;
    const double* pa = A.rc_pa + rp.nbase;
    const double* rec = A.rc_rec + rp.nbase;
    const double* fit = A.rc_fit + rp.nbase;
    double w3[3], alpha;
    int32_t gen;
    rc_agent_params(A.seed, rep, ep, unit, n, rp.rc_w, rp.rc_alpha, w3, &alpha, &gen);
    auto score = [&](int32_t j) { return w3[0] * pa[j] + w3[1] * rec[j] + w3[2] * fit[j]; };

    int c = 1;
    if (lane == 0) S.arr[0] = gen;
    int32_t tgt = 0;
    const int sy = k >= 2 ? rc_same_year(A.seed, rep, ep, al, rp.delta, rp.rc_sy, n, &tgt) : 0;
    if (sy) {
        if (lane == 0) S.arr[c] = tgt;
        ++c;
    }
    const int rsv = (int)floor(rp.rc_frc * (double)k);
    const int rem1 = k - 1 - sy - rsv;
    int in_t = rem1 > 0 ? (int)ceil((double)rem1 * alpha) : 0;
    if (in_t > rem1) in_t = rem1 > 0 ? rem1 : 0;
    long long rows = 1, elems = 0, draws = 0;
    const int64_t gf0 = fo[gen], glf = fo[gen + 1] - gf0, gb0 = bo[gen];
    const int64_t gd = glf + (bo[gen + 1] - gb0);

    // ---- the 1-hop set
    int in = 0;
    if (in_t > 0) {
        int nb = 0;
        for (int64_t q0 = 0; q0 < gd; q0 += 32) {
            const int64_t q = q0 + lane;
            bool valid = false;
            int32_t y = 0;
            float key = 0.0f;
            if (q < gd) {
                y = q < glf ? fc[gf0 + q] : bc[gb0 + (q - glf)];
                valid = y != gen;
                if (valid) key = rc_key(A.seed, rep, ep, unit, y, score(y));
            }
            elems += __popc(__ballot_sync(kFull, valid));
            topk_offer(valid, key, y, in_t, nb, S);
        }
        in = nb;
        __syncwarp();
        for (int q = lane; q < in; q += 32) S.arr[c + q] = S.bi[q];
        __syncwarp();
        c += in;
    }

    // ---- the 2-hop set (without N1 and g)
    const int rem2 = k - 1 - sy - rsv - in;
    int out = 0;
    if (rem2 > 0) {
        int nb = 0;
        for (int64_t q0 = 0; q0 < gd; q0 += 32) {
            const int64_t q = q0 + lane;
            int32_t y = -1;
            if (q < gd) {
                y = q < glf ? fc[gf0 + q] : bc[gb0 + (q - glf)];
                if (y == gen) y = -1;
            }
            rows += __popc(__ballot_sync(kFull, y >= 0));
            int64_t yf0 = 0, ylf = 0, yb0 = 0, yd = 0;
            if (y >= 0) {
                yf0 = fo[y];
                ylf = fo[y + 1] - yf0;
                yb0 = bo[y];
                yd = ylf + (bo[y + 1] - yb0);
            }
            const int64_t incl = warp_incl_scan(yd);
            const int64_t tot = __shfl_sync(kFull, incl, 31);
            const int64_t ys = incl - yd;
            for (int64_t t0 = 0; t0 < tot; t0 += 32) {
                const int64_t t = t0 + lane;
                const int64_t tt = t < tot ? t : tot - 1;
                int lo = 0, hi = 31;  // owner: the last lane whose rows start at or before tt
#pragma unroll
                for (int it = 0; it < 5; ++it) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (__shfl_sync(kFull, ys, mid) <= tt)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                const int64_t of0 = __shfl_sync(kFull, yf0, lo), olf = __shfl_sync(kFull, ylf, lo);
                const int64_t ob0 = __shfl_sync(kFull, yb0, lo), oys = __shfl_sync(kFull, ys, lo);
                bool valid = false;
                int32_t z = 0;
                float key = 0.0f;
                if (t < tot) {
                    const int64_t x = t - oys;
                    z = x < olf ? fc[of0 + x] : bc[ob0 + (x - olf)];
                    valid = z != gen && !rc_in_rows(fo, fc, bo, bc, gen, z);
                    if (valid) key = rc_key(A.seed, rep, ep, unit, z, score(z));
                }
                elems += __popc(__ballot_sync(kFull, valid));
                topk_offer(valid, key, z, rem2, nb, S);
            }
        }
        out = nb;
        __syncwarp();
        for (int q = lane; q < out; q += 32) S.arr[c + q] = S.bi[q];
        __syncwarp();
        c += out;
    }

    // ---- uniform fill over [0, n-1) without g and earlier choices; the 32 lanes draw the next 32
    // candidates (4 per Philox block) and take them in order, exactly as one at a time
    int rnd = k - 1 - sy - in - out;
    uint32_t cidx = 0;
    while (rnd > 0) {
        if (cidx >= 4u * kRcFillBlocks) {
            if (lane == 0) atomicOr(&A.st->error, kErrArg);
            break;
        }
        const uint32_t my = cidx + (uint32_t)lane;
        const u32x4 x = draw(A.seed, kStreamUniformFill, rep, ep, unit, my >> 2);
        const uint32_t xr = (my & 3u) == 0 ? x.x[0] : ((my & 3u) == 1 ? x.x[1] : ((my & 3u) == 2 ? x.x[2] : x.x[3]));
        const int32_t v = (int32_t)bounded32(xr, (uint32_t)(n - 1));
        bool pre = false;
        for (int q = 0; q < c; ++q) pre |= S.arr[q] == v;
        const unsigned grp = __match_any_sync(kFull, v);
        const unsigned gc = grp & __ballot_sync(kFull, !pre);
        const int first = gc ? __ffs(gc) - 1 : 32;
        const unsigned am = __ballot_sync(kFull, !pre && lane == first);
        unsigned consumed = kFull;
        if (__popc(am) >= rnd) {
            unsigned m = am;
            for (int q = 1; q < rnd; ++q) m &= m - 1u;
            const int L = __ffs(m) - 1;
            consumed = L == 31 ? kFull : ((1u << (L + 1)) - 1u);
        }
        draws += __popc(consumed);
        const unsigned took = am & consumed;
        __syncwarp();
        if ((took >> lane) & 1u) S.arr[c + __popc(took & below)] = v;
        __syncwarp();
        c += __popc(took);
        rnd -= __popc(took);
        cidx += 32;
    }
    if (c != k && lane == 0) atomicOr(&A.st->error, kErrArg);
    if (lane == 0 && A.rc_agent) {
        double* o = A.rc_agent + a * 6;
        o[0] = w3[0];
        o[1] = w3[1];
        o[2] = w3[2];
        o[3] = alpha;
        o[4] = (double)gen;
        o[5] = (double)k;
    }
    emit_row<kKMax>(A, rp, a, al, n, S.arr, c < k ? c : k, rows, elems, draws);
}
