// pg_thin.cuh -- the thinning sampler of the agent kernel (included by pg_agents.cu).
//
// One Poisson event stream over all nodes with rate beta * w_j: an event picks j from the global
// CDF and is global with probability 1/beta (always accepted) or a boost event (accepted iff j is
// in the agent's 2-hop ball).  Node j's accepted events then have rate w_j beta^[j in ball], so the
// first k distinct accepted nodes are the successive-sampling draw with those weights -- the law of
// the reference's ES top-k over the neighbourhood (src/abm.cu:461-565) -- at a cost that does not
// depend on the ball's size.  The 32 lanes evaluate 32 events at once (Philox + guide-table CDF
// search); the acceptances are then taken in event order.  The rows of all boost candidates of a
// batch are staged into shared memory by bulk copies and tested together: one copy per candidate,
// since a cited node's backward span carries a copy of its forward row in front of its backward
// entries (a node never cited is its forward row alone).
//
// Ball membership, the 2-hop BFS of GetOneAndTwoHopNeighborhood (src/abm.cu:577-682) answered on
// demand instead of materialised:
//   Z  = anchors U adj(x) for every non-hub anchor x   -- the 1-hop frontier, a hash set in shared
//                                                          memory (4-slot buckets, load <= 1/2);
//                                                          rows too large for it go to a per-warp
//                                                          global table or stay in the CSR.
//   HA = hub bits of the anchors that are hubs          -- their (huge) rows stay implicit.
//   in_z(v)   <=> v in Z  or  hmask[v] & HA != 0        (v adjacent to a hub anchor)
//   member(j) <=> in_z(j)  or  some z in adj(j) has in_z(z)
// For a hub j, the second clause is one bit of HM = OR of hmask over Z | OR of hub2[b] over b in HA,
// where hub2[b] marks the hubs that share a neighbour with hub b.  A test of a non-hub j scans
// adj(j) (forward row, then backward row) and keeps its first hit; the number of entries it
// examined (up to that hit) feeds the byte model.

// Per-warp shared-memory part of an agent's ball (kept out of registers: read only on the rare
// paths of hub anchors, oversized anchors and hub candidates).
struct BallAux {
    unsigned long long ha[kMaskWords];     // hub bits of hub anchors
    unsigned long long hm[kMaskWords];     // hubs in the ball through Z or a hub anchor
    int32_t anchors[PG_MAX_ANCHORS_DEV];
    int32_t big[PG_MAX_ANCHORS_DEV];       // non-hub anchor whose rows did not fit in H
    int32_t na;
};

constexpr uint32_t kWaitLimit = kWaitPolls;  // polls of a bulk-copy barrier before giving up
constexpr int kTestU = 4;                  // entries per lane and step of the membership scan

// STAGE: adjacency entries per stage buffer (two per warp); the struct lives in dynamic shared
// memory, one per warp.  The exact continuation's lists (chosen ids and their cumulative quantised
// weights) are only used after the event loop, when no copy is in flight, so they share the stage
// buffers' memory (a proxy fence orders them before the next agent's bulk copies).
template <int KCAP, int HCAP, int STAGE>
struct ThinSmem {
    static_assert(2 * STAGE * 4 >= KCAP * 12, "continuation lists must fit the stage buffers");
    __align__(16) int32_t stage[2][STAGE];  // candidate rows, two buffers filled by bulk copies
    int32_t H[HCAP];  // frontier hash set, -1 = empty
    int32_t arr[KCAP];
    BallAux aux;
    unsigned long long bar[2];  // mbarriers of the two stage buffers
    __device__ int32_t* c_id() { return &stage[0][0]; }
    __device__ uint64_t* c_cq() { return reinterpret_cast<uint64_t*>(&stage[0][0] + 2 * KCAP); }
};

// ---- bulk asynchronous copies (the TMA engine's cp.async.bulk) into shared memory
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity; false when `limit` polls ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// bytes (a multiple of 16, both addresses 16-byte aligned) from global to shared memory, counted
// on the barrier's transaction bytes.  The copied rows are read once per test, so they are marked
// first to leave L2 (evict-first policy): the per-node records, CDF and hub masks that every
// event reads stay resident instead.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
        : "memory");
}

struct Mask {
    unsigned long long w[kMaskWords];
};

struct Ball {
    const int64_t* fo;
    const int32_t* fc;
    const BRow* br;
    const int32_t* bc;
    const int16_t* hslot;             // hub bit of the node or -1
    const unsigned long long* hmask;  // [node][kMaskWords]
    const int32_t* H;                 // frontier hash set (shared memory)
    const int32_t* G;                 // rows of the anchors too large for H (global), or null
    const BallAux* X;                 // anchors and hub masks (shared memory)
    int hbits;                        // log2 of the hash capacity
    bool small;                       // every non-hub anchor's rows are in H
    bool any_ha;                      // some anchor is a hub
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

// The frontier set is an open-addressing table probed linearly from the first slot of a 4-slot
// bucket.  With no deletions a bucket always fills as a prefix, so a lookup reads a whole bucket
// with one 16-byte load and stops at the first bucket whose last slot is free.
__device__ __forceinline__ uint32_t hslot_of(int32_t v, int bits) {
    return (((uint32_t)v * 0x9E3779B1u) >> (34 - bits)) << 2;
}

// Insert v into the shared hash set (any lane, concurrently).
__device__ __forceinline__ void hash_insert(int32_t* H, int bits, int32_t v) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t s = hslot_of(v, bits);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int prev = atomicCAS(&H[s], -1, v);
        if (prev == -1 || prev == v) return;
        s = (s + 1u) & mask;
    }
}

__device__ __forceinline__ bool bucket_has(const int4& b, int32_t v) {
    return b.x == v || b.y == v || b.z == v || b.w == v;
}

__device__ __forceinline__ bool hash_contains(const int32_t* H, int bits, int32_t v) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t s = hslot_of(v, bits);
    for (uint32_t probe = 0; probe <= mask; probe += 4) {
        const int4 b = *reinterpret_cast<const int4*>(H + s);
        if (bucket_has(b, v)) return true;
        if (b.w == -1) return false;
        s = (s + 4u) & mask;
    }
    return false;
}

// The same set in global memory (the warp's own table of 1 << kGBits slots), for the rows of
// anchors that do not fit the shared one.  Lookups read through L2 (ld.global.cg): the table is
// cleared with stores and filled with L2 atomics in the same agent, so an L1 copy from an earlier
// agent must not answer.
__device__ __forceinline__ void ghash_insert(int32_t* G, int32_t v) {
    const uint32_t mask = (1u << kGBits) - 1u;
    uint32_t s = hslot_of(v, kGBits);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const int prev = atomicCAS(&G[s], -1, v);
        if (prev == -1 || prev == v) return;
        s = (s + 1u) & mask;
    }
}

__device__ __forceinline__ bool ghash_contains(const int32_t* G, int32_t v) {
    const uint32_t mask = (1u << kGBits) - 1u;
    uint32_t s = hslot_of(v, kGBits);
    for (uint32_t probe = 0; probe <= mask; probe += 4) {
        const int4 b = __ldcg(reinterpret_cast<const int4*>(G + s));
        if (bucket_has(b, v)) return true;
        if (b.w == -1) return false;
        s = (s + 4u) & mask;
    }
    return false;
}

__device__ __forceinline__ int hub_slot(const Ball& B, int32_t v) { return B.hslot[v]; }

__device__ __forceinline__ bool mask_bit(const Mask& m, int b) {
    const int w = b >> 6;  // a select, not an indexed load: the mask stays in registers
    const unsigned long long x = w == 0 ? m.w[0] : (w == 1 ? m.w[1] : (w == 2 ? m.w[2] : m.w[3]));
    return (x >> (b & 63)) & 1ull;
}

// v in Z (frontier) -- lane-level, any lane may call it with its own v
__device__ __forceinline__ bool in_z(const Ball& B, int32_t v) {
    if (hash_contains(B.H, B.hbits, v)) return true;
    if (B.G) {
        if (ghash_contains(B.G, v)) return true;
    } else if (!B.small) {
        const BallAux& X = *B.X;
        for (int i = 0; i < X.na; ++i) {
            if (!X.big[i]) continue;
            const int x = X.anchors[i];
            if (contains(B.fc, B.fo[x], B.fo[x + 1], v)) return true;
            int64_t b0, b1;
            bspan(B.br, x, b0, b1);
            if (contains(B.bc, b0, b1, v)) return true;
        }
    }
    if (B.any_ha) {
        const unsigned long long* m = B.hmask + (int64_t)v * kMaskWords;
#pragma unroll
        for (int w = 0; w < kMaskWords; ++w)
            if (m[w] & B.X->ha[w]) return true;
    }
    return false;
}

// Warp-cooperative row scan of a non-hub j outside Z (warp-uniform argument and result), 128
// entries per step.  `examined` gets the adjacency entries looked at, in order (forward row, then
// backward row), up to and including the first hit.
__device__ bool member_rows_warp(const Ball& B, int32_t j, long long& examined) {
    const int lane = lane_id();
    examined = 0;
    for (int dir = 0; dir < 2; ++dir) {
        const int32_t* col = dir ? B.bc : B.fc;
        int64_t p0, p1;
        if (dir) {
            bspan(B.br, j, p0, p1);
        } else {
            p0 = B.fo[j];
            p1 = B.fo[j + 1];
        }
        for (int64_t p = p0; p < p1; p += 128) {
            int32_t v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t x = p + 32 * u + lane;
                v[u] = x < p1 ? col[x] : -1;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const unsigned m = __ballot_sync(kFull, v[u] >= 0 && in_z(B, v[u]));
                if (m) {
                    examined += (p + 32 * u - p0) + __ffs(m);
                    return true;
                }
            }
        }
        examined += p1 - p0;
    }
    return false;
}

// Warp-cooperative membership of one node j (warp-uniform argument and result).
__device__ bool member_warp(const Ball& B, int32_t j, long long& examined) {
    examined = 0;
    if (in_z(B, j)) return true;  // every lane evaluates the same thing
    const int hs = hub_slot(B, j);
    if (hs >= 0) return (B.X->hm[hs >> 6] >> (hs & 63)) & 1ull;
    return member_rows_warp(B, j, examined);
}

// Returns false when a bounded wait ran out (the error word is set and the warp must stop).
// GENERAL = false is the lean instance for the agents the setup did not list as heavy: no hub
// anchor and anchor rows within the shared frontier, so membership in Z is the frontier hash alone.
template <int KCAP, int HCAP, int STAGE, bool GENERAL>
__device__ bool process_agent_thin(const Arena& A, int64_t a, int k, ThinSmem<KCAP, HCAP, STAGE>& S,
                                   uint32_t& phase) {
    constexpr int kStage = STAGE;
    constexpr int kHBits = HCAP == 4096 ? 12 : (HCAP == 2048 ? 11 : 10);
    static_assert(HCAP == (1 << kHBits), "hash capacity must be 1024, 2048 or 4096");
    constexpr int ZCAP = HCAP / 2;  // entries gathered into the frontier (with repeats)
    const int lane = lane_id();
    const int r = replica_of_agent(A.rep, A.R, a);
    const Replica& rp = A.rep[r];
    const int64_t n = rp.n;
    const int64_t al = a - rp.abase;
    const uint32_t ep = (uint32_t)A.st->epoch, unit = (uint32_t)al, rep = (uint32_t)(r + A.rep_base);
    const uint64_t* cdf = A.cdf + rp.nbase;
    Ball B;
    B.fo = A.fwd_off + rp.obase;
    B.fc = A.fwd_col + rp.ebase;
    B.br = A.brow + rp.nbase;
    B.bc = A.bcol + rp.bbase;
    B.hslot = A.hslot + rp.nbase;
    B.hmask = reinterpret_cast<const unsigned long long*>(A.hmask) + rp.nbase * kMaskWords;
    B.H = S.H;
    B.G = nullptr;
    B.X = &S.aux;
    B.hbits = kHBits;
    B.small = true;
    B.any_ha = false;
    const bool boost = rp.p_global < 1.0;
    long long rows = 0;

    // ---------------------------------------------------------------- frontier
    // Lane l < 2na owns one anchor row (anchor l >> 1; forward row for even l, backward for odd),
    // so the anchors' row bounds and hub slots load together; every lane then derives the same
    // anchor facts with shuffles, lane 0 stores them in the warp's BallAux, and the rows of the
    // non-hub anchors are gathered flat, each entry loaded and inserted independently.
    static_assert(kMaskWords == 4 && PG_MAX_ANCHORS_DEV == 4, "frontier layout");
    Mask ha;
#pragma unroll
    for (int w = 0; w < kMaskWords; ++w) ha.w[w] = 0ull;
    const int na = boost ? rp.anchors : 0;
    if (boost) {
        for (int q = lane; q < HCAP; q += 32) S.H[q] = -1;
        const u32x4 xa = draw(A.seed, kStreamAnchor, rep, ep, unit, 0);
        auto anchor = [&](int i) -> int {
            const uint32_t w = i == 0 ? xa.x[0] : (i == 1 ? xa.x[1] : (i == 2 ? xa.x[2] : xa.x[3]));
            return (int)bounded32(w, (uint32_t)n);
        };
        const int rl = (lane >> 1) & 3;
        const bool has_row = lane < 2 * na;
        const int xrow = anchor(rl);
        int64_t r_st = 0, r_len = 0;
        int r_hs = -1;
        if (has_row) {
            int64_t r_end;
            if (lane & 1) {
                bspan(B.br, xrow, r_st, r_end);
            } else {
                r_st = B.fo[xrow];
                r_end = B.fo[xrow + 1];
            }
            r_len = r_end - r_st;
            r_hs = hub_slot(B, xrow);
        }
        int64_t dd[PG_MAX_ANCHORS_DEV];
        int hh[PG_MAX_ANCHORS_DEV];
        int64_t zsize = 0;
#pragma unroll
        for (int i = 0; i < PG_MAX_ANCHORS_DEV; ++i) {
            dd[i] = __shfl_sync(kFull, r_len, 2 * i) + __shfl_sync(kFull, r_len, 2 * i + 1);
            hh[i] = __shfl_sync(kFull, r_hs, 2 * i);
            if (i < na) {
                rows += dd[i] + 1;
                if (hh[i] >= 0) {
#pragma unroll
                    for (int w = 0; w < kMaskWords; ++w)
                        if ((hh[i] >> 6) == w) ha.w[w] |= 1ull << (hh[i] & 63);
                    B.any_ha = true;
                } else {
                    zsize += dd[i];
                }
            }
        }
        // non-hub anchors whose rows would overflow the shared frontier stay implicit
        unsigned bigm = 0u;  // bit i: anchor i's rows are not in H
        if (zsize + na > ZCAP) {
            B.small = false;
            zsize = na;
#pragma unroll
            for (int i = 0; i < PG_MAX_ANCHORS_DEV; ++i) {
                if (i >= na || hh[i] >= 0) continue;
                if (zsize + dd[i] <= ZCAP)
                    zsize += dd[i];
                else
                    bigm |= 1u << i;
            }
        }
        // the general instance puts the rows of the anchors left out of H into the warp's global
        // table when they fit it at three-quarters load (otherwise membership in them is a binary
        // search of the rows)
        int32_t* G = nullptr;
        if (GENERAL && bigm && A.zbig) {
            int64_t tb = 0;
#pragma unroll
            for (int i = 0; i < PG_MAX_ANCHORS_DEV; ++i)
                if ((bigm >> i) & 1u) tb += dd[i];
            if (tb <= (3 << kGBits) / 4) {
                G = A.zbig + (((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) << kGBits);
                int4* g4 = reinterpret_cast<int4*>(G);
                for (int q = lane; q < (1 << kGBits) / 4; q += 32) g4[q] = make_int4(-1, -1, -1, -1);
                __syncwarp();
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < PG_MAX_ANCHORS_DEV; ++i) {
                S.aux.anchors[i] = anchor(i);
                S.aux.big[i] = (int)((bigm >> i) & 1u);
            }
            S.aux.na = na;
#pragma unroll
            for (int w = 0; w < kMaskWords; ++w) S.aux.ha[w] = ha.w[w];
        }
        Mask hm;
#pragma unroll
        for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] = 0ull;
        auto add_mask = [&](int32_t v) {
            const ulonglong2* m = reinterpret_cast<const ulonglong2*>(B.hmask + (int64_t)v * kMaskWords);
            const ulonglong2 m0 = m[0], m1 = m[1];
            hm.w[0] |= m0.x;
            hm.w[1] |= m0.y;
            hm.w[2] |= m1.x;
            hm.w[3] |= m1.y;
        };
        if (lane < na) {
            const int x = anchor(lane & 3);
            hash_insert(S.H, kHBits, x);
            add_mask(x);
        }
        // the non-hub anchors' rows, flat: entry p belongs to the last row lane whose exclusive
        // offset is at or below p (the rows are laid out in lane order)
        const bool row_in = has_row && r_hs < 0;
        const int64_t len_in = row_in ? r_len : 0;
        const int64_t incl = warp_incl_scan(len_in);
        const int64_t excl = incl - len_in;
        const int64_t T = __shfl_sync(kFull, incl, 31);
        // 1: into H; 2: into the global table; 0: neither (hub masks only)
        const int into = row_in ? (!((bigm >> rl) & 1u) ? 1 : (G ? 2 : 0)) : 0;
        for (int64_t p0 = 0; p0 < T; p0 += 64) {
            int32_t v[2];
            int ih[2];
            bool ok[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int64_t p = p0 + 32 * u + lane;
                int L = 0;
#pragma unroll
                for (int bb = 4; bb >= 1; bb >>= 1)
                    if (__shfl_sync(kFull, excl, L + bb) <= p) L += bb;
                const int64_t st = __shfl_sync(kFull, r_st, L), e0 = __shfl_sync(kFull, excl, L);
                ih[u] = __shfl_sync(kFull, into, L);
                ok[u] = p < T;
                // streaming load: the anchor rows are read once per agent
                v[u] = ok[u] ? __ldcs(&((L & 1) ? B.bc : B.fc)[st + (p - e0)]) : 0;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (!ok[u]) continue;
                if (ih[u] == 1)
                    hash_insert(S.H, kHBits, v[u]);
                else if (GENERAL && ih[u] == 2)
                    ghash_insert(G, v[u]);
                add_mask(v[u]);
            }
        }
        if (B.any_ha) {
            const unsigned long long* hh2 = reinterpret_cast<const unsigned long long*>(A.hub2) +
                                            (int64_t)r * kHeavyMax * kMaskWords;
            for (int bb = lane; bb < kHeavyMax; bb += 32)
                if (mask_bit(ha, bb)) {
#pragma unroll
                    for (int ww = 0; ww < kMaskWords; ++ww) hm.w[ww] |= hh2[(int64_t)bb * kMaskWords + ww];
                }
        }
#pragma unroll
        for (int ww = 0; ww < kMaskWords; ++ww) {
            unsigned lo = (unsigned)hm.w[ww], hi = (unsigned)(hm.w[ww] >> 32);
            lo = __reduce_or_sync(kFull, lo);
            hi = __reduce_or_sync(kFull, hi);
            if (lane == 0) S.aux.hm[ww] = ((unsigned long long)hi << 32) | lo;
        }
        __syncwarp();
        B.G = G;
    }

    if (!GENERAL && !(B.small && !B.any_ha)) {
        // the setup lists every agent with a hub anchor or anchor rows beyond 512 entries as
        // heavy, so the lean instance never gets one; a mismatch is reported, not guessed around
        if (lane == 0) atomicOr(&A.st->error, kErrArg);
        return false;
    }

    // ---------------------------------------------------------------- events
    // the previous agent's continuation lists were written over the stage buffers by the generic
    // proxy: order those writes before this agent's bulk copies into the same memory
    fence_proxy_async();
    __syncwarp();
    const uint64_t Wq = rp.wq_total;
    int nch = 0;
    long long events = 0, tests = 0, scanned = 0;
    const int maxev = 64 * k + 256;
    // guide table: the answer for y lies in [guide[g], guide[g + 1]], g = y >> gs
    const int32_t* guide = A.guide + rp.nbase;
    const int gs = guide_shift(Wq, n);
    const int64_t used = Wq ? (int64_t)((Wq - 1) >> gs) + 1 : 0;
    const unsigned below = (1u << lane) - 1u;
    for (int i0 = 0; i0 < maxev && nch < k; i0 += 32) {
        const u32x4 x = draw(A.seed, kStreamGlobal, rep, ep, unit, (uint32_t)(i0 + lane));
        const uint64_t y = mulhi64(u64of(x.x[0], x.x[1]), Wq);
        const int64_t g = (int64_t)(y >> gs);
        int64_t lo = guide[g], hi = g + 1 < used ? guide[g + 1] : n - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (cdf[mid] > y)
                hi = mid;
            else
                lo = mid + 1;
        }
        const int j = (int)lo;
        const bool glob = u01d_at_most(x.x[2], x.x[3], rp.glob_thr);
        // The 32 events of the batch are decided together, with the result of taking them one
        // at a time in event order: an event whose node was already chosen is skipped, a boost
        // event is tested for membership, and the first k acceptances end the draw.
        bool pre = false;  // node chosen by an earlier batch
        for (int q = 0; q < nch; ++q) pre |= S.arr[q] == j;
        // one membership test per distinct boost node, by the lowest lane holding it
        const unsigned grp = __match_any_sync(kFull, j);
        const unsigned bm = __ballot_sync(kFull, !glob);
        bool mem = false, scan = false;
        long long ex = 0;
        int64_t d = 0, W = 0;
        int lead = 0;                // entries of the window before the row's first
        const int32_t* wsrc = B.fc;  // the window's first entry
        if (lane == __ffs(grp) - 1 && !pre && (grp & bm)) {
            // the node's hub slot and row bounds are loaded before the frontier probe, so the
            // global loads overlap the shared-memory hash lookups
            const int hs = hub_slot(B, j);
            const int64_t jf0 = B.fo[j], jf1 = B.fo[j + 1];
            int64_t jb0, jb1;
            bspan(B.br, j, jb0, jb1);
            if (GENERAL ? in_z(B, j) : hash_contains(S.H, kHBits, j)) {
                mem = true;
            } else if (hs >= 0) {
                mem = (B.X->hm[hs >> 6] >> (hs & 63)) & 1ull;
            } else {
                const int64_t lf = jf1 - jf0, lb = jb1 - jb0;
                d = lf + lb;
                scan = d > 0;
                ex = d;  // a miss examines both rows
                if (lb > 0) {
                    // a cited node: its forward row copy ends where its backward entries begin
                    // (16-byte aligned), so both rows are one window of the backward region
                    const int64_t P = fwd_prefix(lf);
                    wsrc = B.bc + (jb0 - P);
                    lead = (int)(P - lf);
                    W = P + ((lb + 3) & ~3ll);
                } else if (lf > 0) {
                    // never cited: the forward row in the forward CSR (edge regions are multiples of
                    // 4 entries, so the aligned window stays inside the replica's)
                    const int64_t fa0 = jf0 & ~3ll;
                    wsrc = B.fc + fa0;
                    lead = (int)(jf0 - fa0);
                    W = ((jf0 + lf + 3) & ~3ll) - fa0;
                }
            }
        }
        // The rows of every node under test are staged into shared memory by bulk asynchronous
        // copies of their 16-byte-aligned windows (lane after lane), kStage entries per chunk; each
        // row keeps its first hit, and a row with a hit copies nothing more.
        const int64_t wincl = warp_incl_scan(W);
        const int64_t wx = wincl - W;
        const int64_t DW = __shfl_sync(kFull, wincl, 31);
        int64_t mp = d;  // first-hit position of this lane's node (d: none yet)
        // this lane's part of chunk c0 (empty once its row has a hit)
        auto part = [&](int64_t c0, int64_t& s0, int64_t& s1) {
            const int64_t c1 = c0 + kStage < DW ? c0 + kStage : DW;
            s0 = wx > c0 ? wx : c0;
            s1 = wx + W < c1 ? wx + W : c1;
            if (mp < d || s1 < s0) s1 = s0;
        };
        // issue the bulk copies of chunk c0 into buffer `buf`; false when nothing is copied
        auto issue = [&](int64_t c0, int buf) -> bool {
            int64_t s0, s1;
            part(c0, s0, s1);
            const uint32_t total = __reduce_add_sync(kFull, (uint32_t)(s1 - s0) * 4u);
            if (total == 0) return false;
            // the warp's reads of this buffer have completed (their values fed its ballots)
            __syncwarp();
            if (lane == 0) mbar_expect_tx(&S.bar[buf], total);
            __syncwarp();
            if (s1 > s0) bulk_g2s(&S.stage[buf][s0 - c0], wsrc + (s0 - wx), (uint32_t)(s1 - s0) * 4u, &S.bar[buf]);
            return true;
        };
        // chunks are double-buffered: chunk c+1 is in flight while chunk c is tested
        const bool simple = !GENERAL || (B.small && !B.any_ha);  // membership in Z: the hash alone
        const int64_t nchunk = (DW + kStage - 1) / kStage;
        uint32_t armed = 0;  // bit b: buffer b has copies in flight
        if (nchunk > 0 && issue(0, 0)) armed = 1u;
        for (int64_t c = 0; c < nchunk; ++c) {
            const int buf = (int)(c & 1);
            const int64_t c0 = c * kStage;
            if (c + 1 < nchunk && issue(c0 + kStage, buf ^ 1)) armed |= 2u >> buf;
            if (!((armed >> buf) & 1u)) continue;
            armed &= ~(1u << buf);
            const bool ok = mbar_wait(&S.bar[buf], (phase >> buf) & 1u, A.first_wait_polls);
            phase ^= 1u << buf;
            if (!__all_sync(kFull, ok)) {
                // give the copies in flight a second bounded wait (the full limit, whatever the
                // first wait's), then abandon the warp
                if (lane == 0) atomicOr(&A.st->error, kErrTimeout);
                mbar_wait(&S.bar[buf], ((phase >> buf) & 1u) ^ 1u);
                if (armed) mbar_wait(&S.bar[buf ^ 1], (phase >> (buf ^ 1)) & 1u);
                return false;
            }
            const int32_t* stg = S.stage[buf];
            // The chunk is tested flat, kTestU entries per lane and step, whatever row they belong
            // to; a hit is then given to the lane whose window holds it, which keeps it when its
            // row has no hit yet and the entry is the row's own (not window padding).  Entries of
            // a row whose hit came in an earlier chunk (copied before the hit was known) or of a
            // row not copied at all (stale) are tested too and their hits dropped.  Chunk
            // position q maps to row position q + x0 (forward row first, then backward).
            const int nq = (int)(DW - c0 < kStage ? DW - c0 : kStage);
            for (int i0 = 0; i0 < nq; i0 += 32 * kTestU) {
                bool hit[kTestU];
                if (simple) {
                    // the entries' first buckets are read together; a full bucket without
                    // the entry (rare at the frontier's load) continues the probe
                    int32_t v[kTestU];
                    int4 hb[kTestU];
#pragma unroll
                    for (int u = 0; u < kTestU; ++u) {
                        const int q = i0 + 32 * u + lane;
                        v[u] = stg[q];  // q < kStage: past nq the entry is stale and masked below
                        hb[u] = *reinterpret_cast<const int4*>(S.H + hslot_of(v[u], kHBits));
                    }
                    bool more[kTestU], anymore = false;
#pragma unroll
                    for (int u = 0; u < kTestU; ++u) {
                        const bool in = i0 + 32 * u + lane < nq;
                        hit[u] = in && bucket_has(hb[u], v[u]);
                        more[u] = in && !hit[u] && hb[u].w != -1;
                        anymore |= more[u];
                    }
                    if (__any_sync(kFull, anymore)) {
#pragma unroll
                        for (int u = 0; u < kTestU; ++u)
                            if (more[u]) hit[u] = hash_contains(S.H, kHBits, v[u]);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < kTestU; ++u) {
                        const int q = i0 + 32 * u + lane;
                        hit[u] = false;
                        if (q < nq) {  // stale entries may hold any value: only node ids reach the masks
                            const int32_t v = stg[q];
                            hit[u] = (uint32_t)v < (uint32_t)n && in_z(B, v);
                        }
                    }
                }
                // hits are rare: one vote skips the per-entry ballots of a step without any
                bool anyhit = false;
#pragma unroll
                for (int u = 0; u < kTestU; ++u) anyhit |= hit[u];
                if (!__any_sync(kFull, anyhit)) continue;
                // a step with hits: this lane's window in chunk coordinates (computed only here)
                const int64_t wlo64 = wx - c0, whi64 = wx + W - c0;
                const int wlo = (int)(wlo64 < -1 ? -1 : (wlo64 > kStage ? kStage : wlo64));
                const int whi = (int)(whi64 < -1 ? -1 : (whi64 > kStage ? kStage : whi64));
                const int x0 = (int)((c0 - wx) - lead);
                const int d32 = (int)d;
#pragma unroll
                for (int u = 0; u < kTestU; ++u) {
                    unsigned hm = __ballot_sync(kFull, hit[u]);
                    while (hm) {
                        const int qh = i0 + 32 * u + __ffs(hm) - 1;
                        hm &= hm - 1u;
                        if (qh >= wlo && qh < whi && mp == d) {
                            const int x = qh + x0;
                            if (x >= 0 && x < d32) mp = x;
                        }
                    }
                }
            }
        }
        if (scan && mp < d) {
            mem = true;
            ex = mp + 1;
        }
        const int leader = __ffs(grp) - 1;
        mem = __shfl_sync(kFull, mem, leader);
        ex = __shfl_sync(kFull, ex, leader);
        // acceptance: the first candidate lane of each node's group; the batch ends at the
        // acceptance that completes k
        const bool cand = !pre && (glob || mem);
        const unsigned gc = grp & __ballot_sync(kFull, cand);
        const int first = gc ? __ffs(gc) - 1 : 32;
        const unsigned am = __ballot_sync(kFull, cand && lane == first);
        const int R = k - nch;
        unsigned consumed = kFull;
        if (__popc(am) >= R) {
            unsigned m = am;
            for (int q = 1; q < R; ++q) m &= m - 1u;
            const int L = __ffs(m) - 1;
            consumed = L == 31 ? kFull : ((1u << (L + 1)) - 1u);
        }
        const bool tested = !glob && !pre && lane <= first && ((consumed >> lane) & 1u);
        events += __popc(consumed);
        tests += __popc(__ballot_sync(kFull, tested));
        scanned += warp_sum<long long>(tested ? ex : 0ll);
        const unsigned took = am & consumed;
        if ((took >> lane) & 1u) S.arr[nch + __popc(took & below)] = j;
        __syncwarp();
        nch += __popc(took);
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
                while (pos > 0 && S.c_id()[pos - 1] > j) {
                    S.c_id()[pos] = S.c_id()[pos - 1];
                    S.c_cq()[pos] = S.c_cq()[pos - 1];
                    --pos;
                }
                S.c_id()[pos] = j;
                S.c_cq()[pos] = qj;
                ++nc;
                R -= qj;
            }
            uint64_t acc = 0;
            for (int q = 0; q < nc; ++q) {
                acc += S.c_cq()[q];
                S.c_cq()[q] = acc;
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
                    if (S.c_id()[mid] <= p)
                        cl = mid + 1;
                    else
                        ch = mid;
                }
                const uint64_t cp = cl ? S.c_cq()[cl - 1] : 0;
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
            const bool glob = u01d_at_most(x.x[2], x.x[3], rp.glob_thr);
            ++events;
            if (!glob) {
                ++tests;
                long long ex;
                const bool mem = member_warp(B, j, ex);
                scanned += ex;
                if (!mem) continue;
            }
            const uint64_t qj = cdf[j] - (j > 0 ? cdf[j - 1] : 0);
            int below = 0;
            for (int q = lane; q < nc; q += 32) below += S.c_id()[q] < j ? 1 : 0;
            const int pos = __reduce_add_sync(kFull, below);
            for (int top = nc; top > pos; top -= 32) {
                const int q = top - 1 - lane;
                const bool act = q >= pos;
                int tid = 0;
                uint64_t tq = 0;
                if (act) {
                    tid = S.c_id()[q];
                    tq = S.c_cq()[q];
                }
                __syncwarp();
                if (act) {
                    S.c_id()[q + 1] = tid;
                    S.c_cq()[q + 1] = tq + qj;
                }
                __syncwarp();
            }
            if (lane == 0) {
                S.c_id()[pos] = j;
                S.c_cq()[pos] = (pos > 0 ? S.c_cq()[pos - 1] : 0) + qj;
                S.arr[nch] = j;
            }
            __syncwarp();
            ++nc;
            ++nch;
            R -= qj;
        }
    }
    if (nch != k && lane == 0) atomicOr(&A.st->error, kErrArg);
    if (lane == 0 && scanned) atomicAdd(&A.st->adj_scanned, (unsigned long long)scanned);
    emit_row<KCAP>(A, rp, a, al, n, S.arr, nch, rows, tests, events);
    return true;
}
