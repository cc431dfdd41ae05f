// pg_lik.cuh -- device layout of a growth trace and of one batch of parameter points for the
// log-likelihood forward pass and its adjoint.
//
// The trace lives in its own buffers beside the growth arena:
//   final graph as forward and backward CSR (rows sorted ascending), int64 offsets;
//   feat[e][j] = (log f_j, log(indeg_e(j)+1), t_e - t_j, low parts) for every trace epoch e and node j < n_e
//   in the layout of the arithmetic mode of the last forward pass,
//   one float4 per (epoch, node) so a weight is one 16-byte gather and one exp;
//   per agent: its epoch, anchors [4] and citations in draw order (cite offsets int64).
// indeg_e(j) is the number of in-edges of j from nodes < n_e: the prefix of j's backward row below
// n_e, because rows are sorted and node ids grow with time.
#pragma once
#include "pg_engine.cuh"

namespace pg {

constexpr int kLikMaxB = 64;         // parameter points per launch
constexpr int kLikThreads = 256;
constexpr int kLikList = 4096;       // ball ids staged in shared memory per window
constexpr int kLikChunk = 4096;      // nodes per CTA in the per-epoch global sums
constexpr int kLikMaxWords = 24576;  // ball bitmap words per pass (96 KiB, 786,432 ids)

struct LikTrace {
    int64_t n;                   // nodes at the end of the trace
    int64_t agents;
    int32_t epochs;
    int32_t num_anchors;
    int32_t bitmap_words;        // words of the shared ball bitmap per pass (multiple of 4)
    int32_t chunks;              // node chunks per epoch in the global pass
    const int64_t* epoch_nodes;  // [epochs + 1]
    const int32_t* epoch_t;      // [epochs]
    const int64_t* fo;
    const int32_t* fc;
    const int64_t* bo;
    const int32_t* bc;
    const float* fit;            // [n]
    const int32_t* pub;          // [n]
    float4* feat;                // [epochs][n]
    const int32_t* anchors;      // [agents][4]
    const int64_t* coff;         // [agents + 1]
    const int32_t* cites;
    const int32_t* agent_epoch;  // [agents]
};

struct LikBatch {
    int32_t B;           // points in this launch (<= kLikMaxB)
    int32_t BE;          // global pass: B rounded up to a power of two (threads per node slice)
    int32_t BW;          // agent pass: points per warp, min(32, B) rounded up to a power of two
    int32_t exact_exp2;  // 1: weights from exp2_exact (fp32, ~2 ulp), 0: the special-function unit
    const double* theta; // [B][4] alpha, tau, gamma, beta
    const double* pp;    // [B][8] alpha, 1/tau, gamma, beta, log beta, 1/beta, 1/tau^2, tau
    double* zglob;       // [epochs][B]      sum_{j<n_e} w_j          (forward writes)
    double* gglob;       // [epochs][B][3]   sum_j w_j dlog w_j/dtheta (adjoint writes)
    double* gpart;       // [epochs][chunks][B][4] partial sums of the global pass
    double* zagent;      // [agents][B]      per-agent normaliser Z_a (forward writes, adjoint reads)
    double* out;         // [agents][B][1|4] per-agent log-likelihood or gradient
    double* res;         // [B][1|4]         totals
    uint32_t* error;     // bit 2: a normaliser was not positive
};

// Agents' 2-hop balls, built once per trace when they fit in memory (else per chunk of agents and
// pass).  Ids of a ball are ascending.
struct LikBalls {
    const int64_t* boff;  // [agents + 1] offsets into the concatenation of all balls
    int64_t base;         // boff of the first agent whose ball is in ids
    int32_t* ids;         // ball ids of agents [a0, a1) at boff[a] - base
    uint8_t* cflag;       // [citations] 1 when the cited node is in the citing agent's ball
    int64_t* cnt;         // [agents] ball sizes (count pass)
    int64_t* adj;         // [agents] adjacency entries read to build each ball (count pass)
    // optional: every agent's bitmaps, written by the count pass and read by the emit pass instead
    // of walking the rows again (agent a's bitmap of pass i at bmap + a bmap_stride + i bitmap_words)
    uint32_t* bmap;
    int64_t bmap_stride;
};

size_t lik_ball_smem(int bitmap_words);
// resident CTAs per SM: ball kernels (*ball_per_sm), forward and adjoint pass (eval_per_sm[2])
cudaError_t init_lik_kernels(int bitmap_words, int* ball_per_sm, int* eval_per_sm);
// a trace's citations as edges: edge ns + p, for citation p of agent a (coff: agents + 1 offsets),
// is (n0 + a, cites[p]); the seed edges fill [0, ns) beforehand
void launch_trace_edges(const int64_t* coff, const int32_t* cites, int64_t agents, int64_t n0, int64_t ns,
                        int32_t* src, int32_t* dst, int num_sms, cudaStream_t s);
// the feature rows in the layout of the arithmetic mode (exact: packed low parts of both logs)
void launch_lik_features(const LikTrace& T, int exact, int num_sms, cudaStream_t s);
// emit = 0: ball sizes into Bl.cnt / Bl.adj; 1: ball ids and citation flags
void launch_lik_ball(const LikTrace& T, const LikBalls& Bl, int emit, int64_t a0, int64_t a1, int grid,
                     cudaStream_t s);
// per-epoch sums: forward Z_glob, adjoint dZ_glob
void launch_lik_global(const LikTrace& T, const LikBatch& P, int adjoint, cudaStream_t s);
// per-agent pass over agents [a0, a1) (their balls in Bl)
void launch_lik_eval(const LikTrace& T, const LikBatch& P, const LikBalls& Bl, int adjoint, int64_t a0,
                     int64_t a1, int grid, cudaStream_t s);
void launch_lik_sum(const LikTrace& T, const LikBatch& P, int adjoint, cudaStream_t s);

}  // namespace pg
