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

__device__ __forceinline__ bool rc_in_rows(const int64_t* fo, const int32_t* fc, const BRow* br,
                                           const int32_t* bc, int32_t g, int32_t v) {
    if (contains(fc, fo[g], fo[g + 1], v)) return true;
    int64_t b0, b1;
    bspan(br, g, b0, b1);
    return contains(bc, b0, b1, v);
}

// Offer one candidate per lane to the top-k list.  When more than two pass the list's threshold
// they are merged as a batch: sorted across the lanes by (key, id), duplicates dropped (equal
// neighbours, or already listed), and list entries and candidates written at their merged ranks,
// the first k kept.  The result is the one candidate-by-candidate insertion gives: the k smallest
// distinct (key, id) pairs offered.  S.out is scratch.
__device__ __forceinline__ void rc_topk_offer(bool valid, float key, int id, int k, int& nb, RcSmem& S) {
    const int lane = lane_id();
    const bool pass = valid && (nb < k || key_less(key, id, S.bk[k - 1], S.bi[k - 1]));
    const unsigned pm = __ballot_sync(kFull, pass);
    if (!pm) return;
    if (__popc(pm) <= 2) {
        topk_offer(valid, key, id, k, nb, S);
        return;
    }
    float ck = pass ? key : __int_as_float(0x7f800000);  // not passing: +inf, sorted last
    int cid = pass ? id : 0x7fffffff;
#pragma unroll
    for (int w = 2; w <= 32; w <<= 1) {
#pragma unroll
        for (int j = w >> 1; j > 0; j >>= 1) {
            const float ok = __shfl_xor_sync(kFull, ck, j);
            const int oi = __shfl_xor_sync(kFull, cid, j);
            const bool up = (lane & w) == 0, lower = (lane & j) == 0;
            if ((lower == up) ? key_less(ok, oi, ck, cid) : key_less(ck, cid, ok, oi)) {
                ck = ok;
                cid = oi;
            }
        }
    }
    const int np = __popc(pm);
    const float pk = __shfl_up_sync(kFull, ck, 1);
    const int pi = __shfl_up_sync(kFull, cid, 1);
    bool keep = lane < np && !(lane > 0 && pk == ck && pi == cid);
    int below = 0;  // list entries ahead of the candidate
    if (lane < np) {
        int lo = 0, hi = nb;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (key_less(S.bk[mid], S.bi[mid], ck, cid))
                lo = mid + 1;
            else
                hi = mid;
        }
        below = lo;
        if (lo < nb && S.bk[lo] == ck && S.bi[lo] == cid) keep = false;
    }
    const unsigned km = __ballot_sync(kFull, keep);
    const int nk = __popc(km);
    if (!nk) return;
    const int rank = __popc(km & ((1u << lane) - 1u));
    if (keep) S.out[rank] = below;
    float tk[kKMax / 32];
    int ti[kKMax / 32];
#pragma unroll
    for (int j = 0; j < kKMax / 32; ++j) {
        const int i = lane + 32 * j;
        tk[j] = 0.0f;
        ti[j] = 0;
        if (i < nb) {
            tk[j] = S.bk[i];
            ti[j] = S.bi[i];
        }
    }
    __syncwarp();  // every read of the old list (and the scratch writes) done
#pragma unroll
    for (int j = 0; j < kKMax / 32; ++j) {
        const int i = lane + 32 * j;
        if (i < nb) {
            int lo = 0, hi = nk;  // kept candidates ahead of entry i: those with below <= i
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (S.out[mid] <= i)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            const int p = i + lo;
            if (p < k) {
                S.bk[p] = tk[j];
                S.bi[p] = ti[j];
            }
        }
    }
    if (keep && below + rank < k) {
        S.bk[below + rank] = ck;
        S.bi[below + rank] = cid;
    }
    __syncwarp();
    nb = nb + nk < k ? nb + nk : k;
}

// What the 2-hop stream of one refcompat agent needs.
struct RcCtx {
    const int64_t* fo;
    const int32_t* fc;
    const BRow* br;
    const int32_t* bc;
    const double* pa;
    const double* rec;
    const double* fit;
    double w3[3];
    uint64_t seed;
    uint32_t rep, ep, unit;
    int32_t gen;
    int64_t gf0, glf, gb0, gd;  // the generator's forward row start and length, backward start, degree
};

// The 2-hop stream (N2 without N1 and g) of the generator's 1-hop groups (32 entries of N1 each):
// every group's rows are concatenated, and the 32-entry chunks t0 = cfirst, cfirst + cstep, ... of
// that concatenation are split over the lanes, each valid entry keyed and offered to the warp's
// top-k list of capacity kcap.  One warp takes every chunk (cfirst 0, cstep 32); the warps of a
// CTA take every cstep-th.  rows (when count_rows) and elems count the byte model.
__device__ __forceinline__ void rc_2hop_slice(const RcCtx& X, int64_t cfirst, int64_t cstep, bool count_rows, int kcap,
                                              int& nb, long long& rows, long long& elems, RcSmem& S) {
    const int lane = lane_id();
    for (int64_t q0 = 0; q0 < X.gd; q0 += 32) {
        const int64_t q = q0 + lane;
        int32_t y = -1;
        if (q < X.gd) {
            y = q < X.glf ? X.fc[X.gf0 + q] : X.bc[X.gb0 + (q - X.glf)];
            if (y == X.gen) y = -1;
        }
        const int nrow = __popc(__ballot_sync(kFull, y >= 0));
        if (count_rows) rows += nrow;
        int64_t yf0 = 0, ylf = 0, yb0 = 0, yd = 0;
        if (y >= 0) {
            yf0 = X.fo[y];
            ylf = X.fo[y + 1] - yf0;
            int64_t yb1;
            bspan(X.br, y, yb0, yb1);
            yd = ylf + (yb1 - yb0);
        }
        const int64_t incl = warp_incl_scan(yd);
        const int64_t tot = __shfl_sync(kFull, incl, 31);
        const int64_t ys = incl - yd;
        for (int64_t t0 = cfirst; t0 < tot; t0 += cstep) {
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
                z = x < olf ? X.fc[of0 + x] : X.bc[ob0 + (x - olf)];
                valid = z != X.gen && !rc_in_rows(X.fo, X.fc, X.br, X.bc, X.gen, z);
                if (valid)
                    key = rc_key(X.seed, X.rep, X.ep, X.unit, z,
                                 X.w3[0] * X.pa[z] + X.w3[1] * X.rec[z] + X.w3[2] * X.fit[z]);
            }
            elems += __popc(__ballot_sync(kFull, valid));
            topk_offer(valid, key, z, kcap, nb, S);
        }
    }
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
    const BRow* br = A.brow + rp.nbase;
    const int32_t* bc = A.bcol + rp.bbase;
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
    const int64_t gf0 = fo[gen], glf = fo[gen + 1] - gf0;
    int64_t gb0, gb1;
    bspan(br, gen, gb0, gb1);
    const int64_t gd = glf + (gb1 - gb0);

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
        RcCtx X;
        X.fo = fo;
        X.fc = fc;
        X.br = br;
        X.bc = bc;
        X.pa = pa;
        X.rec = rec;
        X.fit = fit;
        X.w3[0] = w3[0];
        X.w3[1] = w3[1];
        X.w3[2] = w3[2];
        X.seed = A.seed;
        X.rep = rep;
        X.ep = ep;
        X.unit = unit;
        X.gen = gen;
        X.gf0 = gf0;
        X.glf = glf;
        X.gb0 = gb0;
        X.gd = gd;
        const int big = A.heavy_mark[a];
        if (big > 0) {
            // listed by the setup: k_rc_big has walked the stream with a whole CTA; its sorted
            // top min(k, kKMax) starts with this agent's top rem2
            const long long* meta = A.rc_big_meta + (int64_t)(big - 1) * 3;
            const int have = (int)meta[0];
            nb = have < rem2 ? have : rem2;
            for (int q = lane; q < nb; q += 32) S.bi[q] = A.rc_big_id[(int64_t)(big - 1) * kKMax + q];
            rows += meta[1];
            elems += meta[2];
            __syncwarp();
        } else {
            rc_2hop_slice(X, 0, 32, true, rem2, nb, rows, elems, S);
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
