// pg_thin.cuh -- the thinning sampler of the agent kernel (included by pg_agents.cu).
//
// One Poisson event stream over all nodes with rate beta * w_j: an event picks j from the global
// CDF and is global with probability 1/beta (always accepted) or a boost event (accepted iff j is
// in the agent's 2-hop ball).  Node j's accepted events then have rate w_j beta^[j in ball], so the
// first k distinct accepted nodes are the successive-sampling draw with those weights -- the law of
// the reference's ES top-k over the neighbourhood (src/abm.cu:461-565) -- at a cost that does not
// depend on the ball's size.  The 32 lanes evaluate 32 events at once (Philox + CDF search); the
// acceptances are then taken in event order, each boost candidate tested by the whole warp.
//
// Ball membership, the 2-hop BFS of GetOneAndTwoHopNeighborhood (src/abm.cu:577-682) answered on
// demand instead of materialised:
//   Z  = anchors U adj(x) for every non-hub anchor x   -- the 1-hop frontier, sorted in shared mem.
//   HA = hub bits of the anchors that are hubs          -- their (huge) rows stay implicit.
//   in_z(v)   <=> v in Z  or  hmask[v] & HA != 0        (v adjacent to a hub anchor)
//   member(j) <=> in_z(j)  or  some z in adj(j) has in_z(z)
// For a hub j, the second clause is one bit of HM = OR of hmask over Z | OR of hub2[b] over b in HA,
// where hub2[b] marks the hubs that share a neighbour with hub b.

template <int KCAP, int ZCAP>
struct ThinSmem {
    int32_t Z[ZCAP];
    int32_t arr[KCAP];
    int32_t out[KCAP];
    int32_t c_id[KCAP];
    uint64_t c_cq[KCAP];
};

struct Mask {
    unsigned long long w[kMaskWords];
};

struct Ball {
    const int64_t* fo;
    const int32_t* fc;
    const int64_t* bo;
    const int32_t* bc;
    const int16_t* hslot;       // hub bit of the node or -1
    const unsigned long long* hmask;  // [node][kMaskWords]
    const int32_t* Z;           // sorted unique (shared memory) when small
    int nz;
    bool small;
    int na;
    int anchors[PG_MAX_ANCHORS_DEV];
    bool big_anchor[PG_MAX_ANCHORS_DEV];  // non-hub anchor whose rows did not fit in Z
    Mask ha;                    // hub bits of hub anchors
    bool any_ha;
    Mask hm;                    // hubs in the ball through Z or a hub anchor
};

__device__ __forceinline__ bool contains(const int32_t* a, int64_t lo, int64_t hi, int32_t v) {
    int64_t l = lo, h = hi;
    while (l < h) {
        const int64_t mid = (l + h) >> 1;
        if (a[mid] < v)
            l = mid + 1;
        else
            h = mid;
    }
    return l < hi && a[l] == v;
}

__device__ __forceinline__ int hub_slot(const Ball& B, int32_t v) { return B.hslot[v]; }

__device__ __forceinline__ bool mask_bit(const Mask& m, int b) { return (m.w[b >> 6] >> (b & 63)) & 1ull; }

// v in Z (frontier) -- lane-level, any lane may call it with its own v
__device__ __forceinline__ bool in_z(const Ball& B, int32_t v) {
    if (B.small) {
        if (contains(B.Z, 0, B.nz, v)) return true;
    } else {
        for (int i = 0; i < B.na; ++i) {
            const int x = B.anchors[i];
            if (v == x) return true;
            if (B.big_anchor[i] &&
                (contains(B.fc, B.fo[x], B.fo[x + 1], v) || contains(B.bc, B.bo[x], B.bo[x + 1], v)))
                return true;
        }
        if (contains(B.Z, 0, B.nz, v)) return true;
    }
    if (B.any_ha) {
        const unsigned long long* m = B.hmask + (int64_t)v * kMaskWords;
#pragma unroll
        for (int w = 0; w < kMaskWords; ++w)
            if (m[w] & B.ha.w[w]) return true;
    }
    return false;
}

// Warp-cooperative membership of one node j (warp-uniform argument and result).
__device__ bool member_warp(const Ball& B, int32_t j) {
    const int lane = lane_id();
    if (in_z(B, j)) return true;  // every lane evaluates the same thing
    const int hs = hub_slot(B, j);
    if (hs >= 0) return mask_bit(B.hm, hs);
    for (int dir = 0; dir < 2; ++dir) {
        const int64_t* off = dir ? B.bo : B.fo;
        const int32_t* col = dir ? B.bc : B.fc;
        const int64_t p0 = off[j], p1 = off[j + 1];
        for (int64_t p = p0; p < p1; p += 32) {
            const bool hit = (p + lane < p1) && in_z(B, col[p + lane]);
            if (__any_sync(kFull, hit)) return true;
        }
    }
    return false;
}

template <int KCAP, int ZCAP>
__device__ void process_agent_thin(const Arena& A, int64_t a, int k, ThinSmem<KCAP, ZCAP>& S) {
    const int lane = lane_id();
    const int r = replica_of_agent(A.rep, A.R, a);
    const Replica& rp = A.rep[r];
    const int64_t n = rp.n;
    const int64_t al = a - rp.abase;
    const uint32_t ep = (uint32_t)A.st->epoch, unit = (uint32_t)al, rep = (uint32_t)r;
    const uint64_t* cdf = A.cdf + rp.nbase;
    Ball B;
    B.fo = A.fwd_off + rp.obase;
    B.fc = A.fwd_col + rp.ebase;
    B.bo = A.bwd_off_cur + rp.obase;
    B.bc = A.bwd_col_cur + rp.ebase;
    B.hslot = A.hslot + rp.nbase;
    B.hmask = reinterpret_cast<const unsigned long long*>(A.hmask) + rp.nbase * kMaskWords;
    B.Z = S.Z;
    B.nz = 0;
    B.small = true;
    B.na = 0;
    B.any_ha = false;
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) B.ha.w[w] = B.hm.w[w] = 0ull;
    const bool boost = rp.p_global < 1.0;
    long long rows = 0;

    // ---------------------------------------------------------------- frontier
    if (boost) {
        B.na = rp.anchors;
        const u32x4 xa = draw(A.seed, kStreamAnchor, rep, ep, unit, 0);
        int64_t zsize = B.na;
#pragma unroll
        for (int i = 0; i < PG_MAX_ANCHORS_DEV; ++i) {
            B.anchors[i] = (int)bounded32(xa.x[i], (uint32_t)n);
            B.big_anchor[i] = false;
        }
        for (int i = 0; i < B.na; ++i) {
            const int x = B.anchors[i];
            const int64_t d = (B.fo[x + 1] - B.fo[x]) + (B.bo[x + 1] - B.bo[x]);
            rows += d;
            const int hs = hub_slot(B, x);
            if (hs >= 0) {
                B.ha.w[hs >> 6] |= 1ull << (hs & 63);
                B.any_ha = true;
            } else {
                zsize += d;
            }
        }
        rows += B.na;
        // non-hub anchors whose rows would overflow the shared frontier stay implicit
        if (zsize > ZCAP) {
            B.small = false;
            zsize = B.na;
            for (int i = 0; i < B.na; ++i) {
                const int x = B.anchors[i];
                if (hub_slot(B, x) >= 0) continue;
                const int64_t d = (B.fo[x + 1] - B.fo[x]) + (B.bo[x + 1] - B.bo[x]);
                if (zsize + d <= ZCAP)
                    zsize += d;
                else
                    B.big_anchor[i] = true;
            }
        }
        int w = 0;
        for (int i = 0; i < B.na; ++i) {
            const int x = B.anchors[i];
            if (lane == 0) S.Z[w] = x;
            ++w;
            if (hub_slot(B, x) >= 0 || B.big_anchor[i]) continue;
            const int64_t lf = B.fo[x + 1] - B.fo[x], lb = B.bo[x + 1] - B.bo[x];
            for (int64_t q = lane; q < lf; q += 32) S.Z[w + q] = B.fc[B.fo[x] + q];
            w += (int)lf;
            for (int64_t q = lane; q < lb; q += 32) S.Z[w + q] = B.bc[B.bo[x] + q];
            w += (int)lb;
        }
        int P = 1;
        while (P < w) P <<= 1;
        for (int q = w + lane; q < P; q += 32) S.Z[q] = 0x7fffffff;
        __syncwarp();
        for (int kk = 2; kk <= P; kk <<= 1) {
            for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                for (int q = lane; q < P; q += 32) {
                    const int qx = q ^ jj;
                    if (qx > q) {
                        const int va = S.Z[q], vb = S.Z[qx];
                        if ((va > vb) == ((q & kk) == 0)) {
                            S.Z[q] = vb;
                            S.Z[qx] = va;
                        }
                    }
                }
                __syncwarp();
            }
        }
        // in-place unique; a chunk's predecessor is carried in a register because the previous
        // chunk's writes may have overwritten it
        int nz = 0, carry = -1;
        for (int base = 0; base < w; base += 32) {
            const int q = base + lane;
            const int v = q < w ? S.Z[q] : 0x7fffffff;
            int pv = __shfl_up_sync(kFull, v, 1);
            if (lane == 0) pv = carry;
            carry = __shfl_sync(kFull, v, 31);
            const bool keep = q < w && (q == 0 || pv != v);
            const unsigned m = __ballot_sync(kFull, keep);
            __syncwarp();
            if (keep) S.Z[nz + __popc(m & ((1u << lane) - 1))] = v;
            nz += __popc(m);
            __syncwarp();
        }
        B.nz = nz;
        // HM: hubs adjacent to the frontier, to a big anchor's rows, or sharing a neighbour with a
        // hub anchor
        Mask hm;
#pragma unroll
        for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] = 0ull;
        for (int q = lane; q < nz; q += 32) {
            const unsigned long long* m = B.hmask + (int64_t)S.Z[q] * kMaskWords;
#pragma unroll
            for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] |= m[ww];
        }
        for (int i = 0; i < B.na; ++i) {
            const int x = B.anchors[i];
            if (!B.big_anchor[i]) continue;
            for (int dir = 0; dir < 2; ++dir) {
                const int64_t* off = dir ? B.bo : B.fo;
                const int32_t* col = dir ? B.bc : B.fc;
                for (int64_t p = off[x] + lane; p < off[x + 1]; p += 32) {
                    const unsigned long long* m = B.hmask + (int64_t)col[p] * kMaskWords;
#pragma unroll
                    for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] |= m[ww];
                }
            }
        }
        if (B.any_ha) {
            const unsigned long long* hh = reinterpret_cast<const unsigned long long*>(A.hub2) +
                                           (int64_t)r * kHeavyMax * kMaskWords;
            for (int b = lane; b < kHeavyMax; b += 32)
                if (mask_bit(B.ha, b)) {
#pragma unroll
                    for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] |= hh[(int64_t)b * kMaskWords + ww];
                }
        }
#pragma unroll
        for (int ww = 0; ww < kMaskWords; ++ww) {
            unsigned lo = (unsigned)hm.w[ww], hi = (unsigned)(hm.w[ww] >> 32);
            lo = __reduce_or_sync(kFull, lo);
            hi = __reduce_or_sync(kFull, hi);
            B.hm.w[ww] = ((unsigned long long)hi << 32) | lo;
        }
    }

    // ---------------------------------------------------------------- events
    const uint64_t Wq = rp.wq_total;
    const double pg = rp.p_global;
    int nch = 0;
    long long events = 0, tests = 0;
    const int maxev = 64 * k + 256;
    for (int i0 = 0; i0 < maxev && nch < k; i0 += 32) {
        const u32x4 x = draw(A.seed, kStreamGlobal, rep, ep, unit, (uint32_t)(i0 + lane));
        const uint64_t y = mulhi64(u64of(x.x[0], x.x[1]), Wq);
        int64_t lo = 0, hi = n - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (cdf[mid] > y)
                hi = mid;
            else
                lo = mid + 1;
        }
        const int j = (int)lo;
        const bool glob = u01d(x.x[2], x.x[3]) <= pg;
        for (int l = 0; l < 32 && nch < k; ++l) {
            const int jl = __shfl_sync(kFull, j, l);
            const bool gl = __shfl_sync(kFull, glob, l);
            ++events;
            bool dup = false;
            for (int q = lane; q < nch; q += 32) dup |= (S.arr[q] == jl);
            if (__any_sync(kFull, dup)) continue;
            if (!gl) {
                ++tests;
                if (!member_warp(B, jl)) continue;
            }
            if (lane == 0) S.arr[nch] = jl;
            __syncwarp();
            ++nch;
        }
    }
    if (nch < k) {
        // exact continuation without replacement (memoryless): CDF minus the chosen weight
        uint64_t R = Wq;
        if (lane == 0) {
            int nc = 0;
            for (int q = 0; q < nch; ++q) {
                const int j = S.arr[q];
                const uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
                int pos = nc;
                while (pos > 0 && S.c_id[pos - 1] > j) {
                    S.c_id[pos] = S.c_id[pos - 1];
                    S.c_cq[pos] = S.c_cq[pos - 1];
                    --pos;
                }
                S.c_id[pos] = j;
                S.c_cq[pos] = qj;
                ++nc;
                R -= qj;
            }
            uint64_t acc = 0;
            for (int q = 0; q < nc; ++q) {
                acc += S.c_cq[q];
                S.c_cq[q] = acc;
            }
        }
        __syncwarp();
        int nc = nch;
        R = __shfl_sync(kFull, R, 0);
        for (uint32_t f = 0; nch < k && R > 0 && f < (1u << 24); ++f) {
            const u32x4 x = draw(A.seed, kStreamFallback, rep, ep, unit, f);
            const uint64_t y = mulhi64(u64of(x.x[0], x.x[1]), R);
            int64_t lo = 0, hi = n;
            while (true) {
                const int64_t span = hi - lo;
                const int64_t step = span > 32 ? (span + 31) / 32 : 1;
                int64_t p = lo + (int64_t)(lane + 1) * step - 1;
                if (p > hi - 1) p = hi - 1;
                int cl = 0, ch = nc;
                while (cl < ch) {
                    const int mid = (cl + ch) >> 1;
                    if (S.c_id[mid] <= p)
                        cl = mid + 1;
                    else
                        ch = mid;
                }
                const uint64_t cp = cl ? S.c_cq[cl - 1] : 0;
                const unsigned m = __ballot_sync(kFull, (cdf[p] - cp) > y);
                if (m == 0) {
                    if (lane == 0) atomicOr(&A.st->error, kErrArg);
                    lo = 0;
                    break;
                }
                const int L = __ffs(m) - 1;
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
            const bool glob = u01d(x.x[2], x.x[3]) <= pg;
            ++events;
            if (!glob) {
                ++tests;
                if (!member_warp(B, j)) continue;
            }
            const uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
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
                S.arr[nch] = j;
            }
            __syncwarp();
            ++nc;
            ++nch;
            R -= qj;
        }
    }
    if (nch != k && lane == 0) atomicOr(&A.st->error, kErrArg);
    emit_row<KCAP>(A, rp, a, al, n, S.arr, S.out, nch, rows, tests, events);
}
