// Learned world-line proposals: per-spin features, the MLP's element-wise
// parts (the 64 x 64 layers run on the tensor cores through pq_tc_gemm_bf16),
// the Metropolis-Hastings world-line move, and the training kernels.
//
// Features of spin i of a replica (P slices, local fields f^k = h_i + sum_m J_m t_m^k
// from its neighbours m, which belong to other update classes; s^k, t_m^k = +-1):
//   x0 = mean_k f^k / (1 + sum_m |J_m| + |h_i|)   (normalised local field)
//   x1 = std_k f^k / (same scale)
//   x2 = mean_k s^k                                (world-line magnetisation)
//   x3 = #{k : s^k != s^{k+1}} / P                 (slice disagreements, periodic)
//   x4 = mean_k s^k f^k / (same scale)             (alignment; the flip costs 2 P x4 scale)
//   x5 = beta * (classical flip cost) / P, clipped to [-8, 8]
//   x6 = J-perp * beta / P, clipped to [0, 8]      (how stiff the world-lines are)
//   x7 = 1                                         (bias input)
// The slice sums come from popcounts of the packed world-lines (exact integers),
// combined in FP32 in the order spin_features writes them:
//   sum_k t_m^k = P - 2 popc(w_m),  sum_k s^k t_m^k = P - 2 popc(w_i ^ w_m),
//   sum_k t_m^k t_l^k = P - 2 popc(w_m ^ w_l).
// The flipped world-line (s -> -s in every slice) has x2, x4, x5 negated and the
// rest unchanged; both versions are scored in one pass.
#include <cuda_bf16.h>

#include "common.cuh"
#include "sweep_core.cuh"
#include "tc_gemm.cuh"

namespace {

using namespace pq;

constexpr int kFeat = 8;
constexpr int kLd = 64;  // padded feature / hidden width of the GEMM operands

__device__ __forceinline__ int popc_(uint32_t x) { return __popc(x); }
__device__ __forceinline__ int popc_(uint64_t x) { return __popcll(x); }

template <typename W>
__device__ __forceinline__ W slice_mask(int P) {
    return P >= (int)(8 * sizeof(W)) ? ~(W)0 : (((W)1 << P) - 1);
}

// Neighbour world-lines and couplings of spin i (padding entries point at i with coupling 0).
// Entries m >= maxdeg are zero couplings to i itself, so every loop below runs over all MAXD
// (>= maxdeg) entries, unrolled into registers.
template <typename W, int MAXD>
__device__ __forceinline__ void load_neighbourhood(const W* __restrict__ words_r, int i, int n, int maxdeg,
                                                   const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                                   W (&nbw)[MAXD], float (&J)[MAXD]) {
#pragma unroll
    for (int m = 0; m < MAXD; ++m) {
        J[m] = 0.0f;
        nbw[m] = words_r[i];
        if (m < maxdeg) {
            const int j = __ldg(nbr + (int64_t)m * n + i);
            J[m] = __ldg(cpl + (int64_t)m * n + i);
            nbw[m] = words_r[(unsigned)j < (unsigned)n ? j : i];
        }
    }
}

// sum_k s^k f^k of spin i's world-line: h (P - 2 popc(w_i)), then + J_m (P - 2 popc(w_i ^ w_m)) for m in order.
// Flipping every slice changes the classical energy by 2 * this.
template <typename W, int MAXD>
__device__ __forceinline__ float worldline_align(W wi, const W (&nbw)[MAXD], const float (&J)[MAXD], int deg,
                                                 float h, int P, W mask) {
    float sa = __fmul_rn(h, (float)(P - 2 * popc_(wi & mask)));
#pragma unroll
    for (int m = 0; m < MAXD; ++m)
        if (m < deg)
        sa = __fadd_rn(sa, __fmul_rn(J[m], (float)(P - 2 * popc_((wi ^ nbw[m]) & mask))));
    return sa;
}

// What the features of spin i read from memory: its world-line, its neighbours'
// world-lines and couplings, its field.
template <typename W, int MAXD>
struct SiteIn {
    W wi;
    W nbw[MAXD];
    float J[MAXD];
    float h;
};

template <typename W, int MAXD>
__device__ __forceinline__ void load_site_in(const W* __restrict__ words_r, int i, int n, int maxdeg,
                                             const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                             const float* __restrict__ field, SiteIn<W, MAXD>& s) {
    s.wi = words_r[i];
    s.h = __ldg(field + i);
    load_neighbourhood<W, MAXD>(words_r, i, n, maxdeg, nbr, cpl, s.nbw, s.J);
}

template <typename W, int MAXD>
__device__ __forceinline__ void site_features(const SiteIn<W, MAXD>& st, int P, int maxdeg, float beta, float jp,
                                              float (&x)[kFeat], float& dE) {
    const W mask = slice_mask<W>(P);
    const W wi = st.wi & mask;
    const float h = st.h;
    const int deg = maxdeg;
    const float Pf = (float)P;
    float scale = __fadd_rn(1.0f, fabsf(h));
    float s1 = __fmul_rn(Pf, h);                  // sum_k f^k
    float s2 = __fmul_rn(Pf, __fmul_rn(h, h));    // sum_k (f^k)^2
    const float h2 = __fmul_rn(2.0f, h);
#pragma unroll
    for (int m = 0; m < MAXD; ++m) {
        if (m >= deg) break;
        scale = __fadd_rn(scale, fabsf(st.J[m]));
        const float tm = (float)(P - 2 * popc_(st.nbw[m] & mask));
        s1 = __fadd_rn(s1, __fmul_rn(st.J[m], tm));
        s2 = __fadd_rn(s2, __fmul_rn(__fmul_rn(h2, st.J[m]), tm));
        s2 = __fadd_rn(s2, __fmul_rn(__fmul_rn(st.J[m], st.J[m]), Pf));
#pragma unroll
        for (int l = 0; l < MAXD; ++l) {
            if (l >= m) break;
            const float tml = (float)(P - 2 * popc_((st.nbw[m] ^ st.nbw[l]) & mask));
            s2 = __fadd_rn(s2, __fmul_rn(__fmul_rn(2.0f, __fmul_rn(st.J[m], st.J[l])), tml));
        }
    }
    const float sa = worldline_align<W, MAXD>(wi, st.nbw, st.J, deg, h, P, mask);
    const float inv = __fdiv_rn(1.0f, Pf);
    const float mean = __fmul_rn(s1, inv);
    const float var = fmaxf(__fsub_rn(__fmul_rn(s2, inv), __fmul_rn(mean, mean)), 0.0f);
    const W rot = ((wi >> 1) | (wi << (P - 1))) & mask;   // bit k = slice k + 1 (periodic)
    dE = __fmul_rn(2.0f, sa);
    x[0] = __fdiv_rn(mean, scale);
    x[1] = __fdiv_rn(__fsqrt_rn(var), scale);
    x[2] = __fmul_rn((float)(P - 2 * popc_(wi)), inv);
    x[3] = __fmul_rn((float)popc_(wi ^ rot), inv);
    x[4] = __fdiv_rn(__fmul_rn(sa, inv), scale);
    x[5] = fminf(fmaxf(__fmul_rn(__fmul_rn(beta, dE), inv), -8.0f), 8.0f);
    x[6] = fminf(fmaxf(__fmul_rn(__fmul_rn(jp, beta), inv), 0.0f), 8.0f);
    x[7] = 1.0f;
}

template <typename W, int MAXD>
__device__ __forceinline__ void spin_features(const W* __restrict__ words_r, int i, int n, int P, int maxdeg,
                                              const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                              const float* __restrict__ field, float beta, float jp,
                                              float (&x)[kFeat], float& dE) {
    SiteIn<W, MAXD> st;
    load_site_in<W, MAXD>(words_r, i, n, maxdeg, nbr, cpl, field, st);
    site_features<W, MAXD>(st, P, maxdeg, beta, jp, x, dE);
}

// Rows [0, M): features of the current world-lines of class `cls` (all replicas,
// row = r * csize + s); rows [M, 2M): the flipped versions.  dE[row] = classical
// flip cost of the current world-line.
template <typename W, int MAXD>
__global__ void features_kernel(const W* __restrict__ words, int n, int P, int R, int maxdeg,
                                const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                const float* __restrict__ field, int cls, int stride, int csize, float beta, float jp,
                                __nv_bfloat16* __restrict__ X, float* __restrict__ dE, int64_t Mpad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)R * csize;
    if (t >= M) return;
    const int r = (int)(t / csize), s = (int)(t % csize);
    const int i = cls * stride + s;
    float x[kFeat], de;
    spin_features<W, MAXD>(words + (int64_t)r * n, i, n, P, maxdeg, nbr, cpl, field, beta, jp, x, de);
    dE[t] = de;
    __nv_bfloat16* row = X + t * kLd;
    __nv_bfloat16* rowf = X + (Mpad + t) * kLd;
#pragma unroll
    for (int c = 0; c < kFeat; ++c) {
        const float xf = (c == 2 || c == 4 || c == 5) ? -x[c] : x[c];
        row[c] = __float2bfloat16_rn(x[c]);
        rowf[c] = __float2bfloat16_rn(xf);
    }
}

// H (FP32, ld kLd) -> relu -> BF16 (ld kLd), rows [0, rows).
__global__ void relu_bf16_kernel(const float* __restrict__ H, __nv_bfloat16* __restrict__ out, int64_t n) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = __float2bfloat16_rn(fmaxf(H[t], 0.0f));
}

// logit = relu(H2) . w3 + b3 per row.
__global__ void head_kernel(const float* __restrict__ H2, const float* __restrict__ w3, float b3,
                            float* __restrict__ logit, int64_t rows) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows) return;
    const float* h = H2 + t * kLd;
    float acc = b3;
#pragma unroll 16
    for (int c = 0; c < 64; ++c) acc = __fmaf_rn(fmaxf(h[c], 0.0f), w3[c], acc);
    logit[t] = acc;
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + expf(-z)); }

// Learned world-line move of every spin of class `cls` (all replicas, in global
// words): proposed with q = clamp(sigmoid(logit), qmin, 1), accepted with
// min(1, exp(-beta dE) q'/q), q' from the flipped features.  Uniforms:
// Philox(ctr = {i, move, replica, 3 << 24 | cls}) words 0 (propose) and 1 (accept).
template <typename W>
__global__ void propose_kernel(W* __restrict__ words, int n, int P, int R, int cls, int stride, int csize,
                               const float* __restrict__ logit, const float* __restrict__ dE, int64_t Mpad,
                               float qmin, float beta, uint32_t move, uint32_t key0, uint32_t key1,
                               uint32_t replica_base, unsigned long long* __restrict__ counters) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)R * csize;
    if (t >= M) return;
    const int r = (int)(t / csize), s = (int)(t % csize);
    const int i = cls * stride + s;
    const pq_u32x4 u = pq_philox(pq_u32x4{(uint32_t)i, move, replica_base + (uint32_t)r, (3u << 24) | (uint32_t)cls},
                                 key0, key1);
    const float q = fminf(fmaxf(sigmoidf_(logit[t]), qmin), 1.0f);
    const float qf = fminf(fmaxf(sigmoidf_(logit[Mpad + t]), qmin), 1.0f);
    const bool proposed = pq_u01(u.x) < q;
    bool acc = false;
    if (proposed) {
        // ratio = exp(-beta dE) q'/q; dE <= 0 with q' >= q accepts outright
        const float lr = -beta * dE[t] + logf(qf) - logf(q);
        acc = lr >= 0.0f || pq_u01(u.y) < expf(lr);
        if (acc) {
            const W mask = P >= (int)(8 * sizeof(W)) ? ~(W)0 : (((W)1 << P) - 1);
            words[(int64_t)r * n + i] ^= mask;
        }
    }
    if (counters) {
        if (proposed) atomicAdd(counters, 1ull);
        if (acc) atomicAdd(counters + 1, 1ull);
    }
}

// ---------------------------------------------------------------------------
// Pair world-line moves (no reference counterpart): the world-lines of the two
// spins i, j of a bond (total coupling J_b between them) flip together, in every
// slice.  Local sweeps and single world-line flips leave the anneal in states
// that are stable against single flips but not against flipping two coupled
// spins; this move reaches them.
//  * cost: dE = fl(fl(2 sa_i) + fl(2 sa_j)) - fl(4 fl(J_b c)), c = P - 2 popc(w_i ^ w_j),
//    sa = worldline_align (the bond's own term is unchanged by the move);
//  * bonds are visited class by class: no endpoint of a bond of a class is an
//    endpoint of, or a neighbour of an endpoint of, another bond of the class, so a
//    pair flip changes neither the cost nor the features of another bond of its class;
//  * decision with proposal probabilities q (current pair) and q' (flipped pair),
//    x = -fl(beta dE), u uniform: x <= 0 accepts iff fl(u q) < fl(q' expf_neg(x)),
//    x > 0 accepts iff fl(fl(u q) expf_neg(-x)) < q' -- the Metropolis-Hastings test
//    u < exp(x) q'/q; the uniform pass has q = q' = 1 (every bond tried);
//  * proposal: q = clamp(sigmoid(logit), qmin, 1), sigmoid(z) = 1 / (1 + expf_neg(-z))
//    for z >= 0 and e / (1 + e) with e = expf_neg(z) for z < 0;
//  * uniforms: Philox(ctr = {bond id, move, replica, 5 << 24 | class}), word 0 proposes,
//    word 1 accepts;
//  * features of a pair state (the reverse row is the same function of the flipped state):
//    x0, x1, x2 = beta dE / P, beta dE_i / P, beta dE_j / P clipped to [-8, 8] (dE_i = 2 sa_i,
//    the single world-line flip cost), x3 = (J_b c / P) / (1 + |J_b|),
//    x4 = (kinks_i + kinks_j) / (2 P), x5 = m_i m_j (world-line magnetisations),
//    x6 = clip(jp beta / P, 0, 8), x7 = 1.
// ---------------------------------------------------------------------------
template <typename W, int MAXD>
struct PairIn {
    int si, sj;                 // the bond's slots
    W wi, wj;
    W nbi[MAXD], nbj[MAXD];     // neighbour world-lines
    int ii[MAXD], ij[MAXD];     // neighbour slots
    float Ji[MAXD], Jj[MAXD];
    float hi, hj, Jb;
};

template <typename W, int MAXD>
__device__ __forceinline__ void load_side(const W* __restrict__ words_r, int s, int n, int maxdeg,
                                          const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                          W (&nb)[MAXD], int (&ix)[MAXD], float (&J)[MAXD], bool& bad) {
#pragma unroll
    for (int m = 0; m < MAXD; ++m) {
        J[m] = 0.0f;
        ix[m] = s;
        nb[m] = words_r[s];
        if (m < maxdeg) {
            int j = __ldg(nbr + (int64_t)m * n + s);
            if ((unsigned)j >= (unsigned)n) { bad = true; j = s; }
            ix[m] = j;
            J[m] = __ldg(cpl + (int64_t)m * n + s);
            nb[m] = words_r[j];
        }
    }
}

template <typename W, int MAXD>
__device__ __forceinline__ void load_pair(const W* __restrict__ words_r, int si, int sj, float Jb, int n, int maxdeg,
                                          const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                          const float* __restrict__ field, PairIn<W, MAXD>& p, bool& bad) {
    p.si = si; p.sj = sj; p.Jb = Jb;
    p.wi = words_r[si];
    p.wj = words_r[sj];
    p.hi = __ldg(field + si);
    p.hj = __ldg(field + sj);
    load_side<W, MAXD>(words_r, si, n, maxdeg, nbr, cpl, p.nbi, p.ii, p.Ji, bad);
    load_side<W, MAXD>(words_r, sj, n, maxdeg, nbr, cpl, p.nbj, p.ij, p.Jj, bad);
}

// The pair state after the move: both world-lines flipped, wherever they appear.
template <typename W, int MAXD>
__device__ __forceinline__ void flip_pair(PairIn<W, MAXD>& p, W mask) {
    const W fi = p.wi ^ mask, fj = p.wj ^ mask;
#pragma unroll
    for (int m = 0; m < MAXD; ++m) {
        p.nbi[m] = p.ii[m] == p.sj ? fj : (p.ii[m] == p.si ? fi : p.nbi[m]);
        p.nbj[m] = p.ij[m] == p.si ? fi : (p.ij[m] == p.sj ? fj : p.nbj[m]);
    }
    p.wi = fi;
    p.wj = fj;
}

template <typename W, int MAXD>
__device__ __forceinline__ float pair_cost(const PairIn<W, MAXD>& p, int P, int maxdeg, W mask, float& dEi,
                                           float& dEj, int& c) {
    dEi = __fmul_rn(2.0f, worldline_align<W, MAXD>(p.wi & mask, p.nbi, p.Ji, maxdeg, p.hi, P, mask));
    dEj = __fmul_rn(2.0f, worldline_align<W, MAXD>(p.wj & mask, p.nbj, p.Jj, maxdeg, p.hj, P, mask));
    c = P - 2 * popc_((p.wi ^ p.wj) & mask);
    return __fsub_rn(__fadd_rn(dEi, dEj), __fmul_rn(4.0f, __fmul_rn(p.Jb, (float)c)));
}

__device__ __forceinline__ float clip8(float v) { return fminf(fmaxf(v, -8.0f), 8.0f); }

template <typename W, int MAXD>
__device__ __forceinline__ float pair_features(const PairIn<W, MAXD>& p, int P, int maxdeg, float beta, float jp,
                                               float (&x)[kFeat]) {
    const W mask = slice_mask<W>(P);
    float dEi, dEj;
    int c;
    const float dE = pair_cost<W, MAXD>(p, P, maxdeg, mask, dEi, dEj, c);
    const float inv = __fdiv_rn(1.0f, (float)P);
    const W wi = p.wi & mask, wj = p.wj & mask;
    const W roti = ((wi >> 1) | (wi << (P - 1))) & mask, rotj = ((wj >> 1) | (wj << (P - 1))) & mask;
    x[0] = clip8(__fmul_rn(__fmul_rn(beta, dE), inv));
    x[1] = clip8(__fmul_rn(__fmul_rn(beta, dEi), inv));
    x[2] = clip8(__fmul_rn(__fmul_rn(beta, dEj), inv));
    x[3] = __fdiv_rn(__fmul_rn(__fmul_rn(p.Jb, (float)c), inv), __fadd_rn(1.0f, fabsf(p.Jb)));
    x[4] = __fdiv_rn((float)(popc_(wi ^ roti) + popc_(wj ^ rotj)), (float)(2 * P));
    x[5] = __fmul_rn(__fmul_rn((float)(P - 2 * popc_(wi)), inv), __fmul_rn((float)(P - 2 * popc_(wj)), inv));
    x[6] = fminf(fmaxf(__fmul_rn(__fmul_rn(jp, beta), inv), 0.0f), 8.0f);
    x[7] = 1.0f;
    return dE;
}

__device__ __forceinline__ float pair_sigmoid(float z) {
    if (z >= 0.0f) return __fdiv_rn(1.0f, __fadd_rn(1.0f, pq_expf_neg(-z)));
    const float e = pq_expf_neg(z);
    return __fdiv_rn(e, __fadd_rn(1.0f, e));
}

__device__ __forceinline__ bool pair_accept(float dE, float beta, float q, float qf, float u) {
    const float x = -__fmul_rn(beta, dE);
    const float uq = __fmul_rn(u, q);
    if (x <= 0.0f) return uq < __fmul_rn(qf, pq_expf_neg(x));
    return __fmul_rn(uq, pq_expf_neg(-x)) < qf;
}

template <typename W>
__device__ __forceinline__ void pair_apply(W* __restrict__ words_r, int si, int sj, int P) {
    const W mask = slice_mask<W>(P);
    words_r[si] ^= mask;
    words_r[sj] ^= mask;
}

// Rows [0, M): features of the current pairs of bonds [first, first + count) (all
// replicas, row = r * count + b); rows [Mpad, Mpad + M): of the flipped pairs;
// dE[row] = cost of the move.
template <typename W, int MAXD>
__global__ void pair_features_kernel(const W* __restrict__ words, int n, int P, int R, int maxdeg,
                                     const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                     const float* __restrict__ field, const int32_t* __restrict__ bi,
                                     const int32_t* __restrict__ bj, const float* __restrict__ bJ, int first,
                                     int count, float beta, float jp, __nv_bfloat16* __restrict__ X,
                                     float* __restrict__ dE, int64_t Mpad, int32_t* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)R * count;
    if (t >= M) return;
    const int r = (int)(t / count), b = first + (int)(t % count);
    const int si = bi[b], sj = bj[b];
    if ((unsigned)si >= (unsigned)n || (unsigned)sj >= (unsigned)n) {
        pq_set_status(status, PQ_ERR_BAD_INDEX);
        return;
    }
    bool bad = false;
    PairIn<W, MAXD> p;
    load_pair<W, MAXD>(words + (int64_t)r * n, si, sj, bJ[b], n, maxdeg, nbr, cpl, field, p, bad);
    float x[kFeat];
    dE[t] = pair_features<W, MAXD>(p, P, maxdeg, beta, jp, x);
    __nv_bfloat16* row = X + t * kLd;
#pragma unroll
    for (int k = 0; k < kFeat; ++k) row[k] = __float2bfloat16_rn(x[k]);
    flip_pair<W, MAXD>(p, slice_mask<W>(P));
    pair_features<W, MAXD>(p, P, maxdeg, beta, jp, x);
    __nv_bfloat16* rowf = X + (Mpad + t) * kLd;
#pragma unroll
    for (int k = 0; k < kFeat; ++k) rowf[k] = __float2bfloat16_rn(x[k]);
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
}

// The learned pair move of bonds [first, first + count), from the logits of the
// features rows (current at t, flipped at Mpad + t) and their costs.
template <typename W>
__global__ void pair_propose_kernel(W* __restrict__ words, int n, int P, int R, const int32_t* __restrict__ bi,
                                    const int32_t* __restrict__ bj, int first, int count, int cls,
                                    const float* __restrict__ logit, const float* __restrict__ dE, int64_t Mpad,
                                    float qmin, float beta, uint32_t move, uint32_t key0, uint32_t key1,
                                    uint32_t replica_base, unsigned long long* __restrict__ counters,
                                    int32_t* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)R * count;
    if (t >= M) return;
    const int r = (int)(t / count), b = first + (int)(t % count);
    const int si = bi[b], sj = bj[b];
    if ((unsigned)si >= (unsigned)n || (unsigned)sj >= (unsigned)n) {
        pq_set_status(status, PQ_ERR_BAD_INDEX);
        return;
    }
    const pq_u32x4 u = pq_philox(pq_u32x4{(uint32_t)b, move, replica_base + (uint32_t)r, (5u << 24) | (uint32_t)cls},
                                 key0, key1);
    const float q = fminf(fmaxf(pair_sigmoid(logit[t]), qmin), 1.0f);
    const float qf = fminf(fmaxf(pair_sigmoid(logit[Mpad + t]), qmin), 1.0f);
    const bool proposed = pq_u01(u.x) < q;
    const bool acc = proposed && pair_accept(dE[t], beta, q, qf, pq_u01(u.y));
    if (acc) pair_apply<W>(words + (int64_t)r * n, si, sj, P);
    if (counters) {
        if (proposed) atomicAdd(counters, 1ull);
        if (acc) atomicAdd(counters + 1, 1ull);
    }
}

// The uniform pair move (q = q' = 1) of bonds [first, first + count): cost and decision only.
template <typename W, int MAXD>
__global__ void pair_uniform_kernel(W* __restrict__ words, int n, int P, int R, int maxdeg,
                                    const int32_t* __restrict__ nbr, const float* __restrict__ cpl,
                                    const float* __restrict__ field, const int32_t* __restrict__ bi,
                                    const int32_t* __restrict__ bj, const float* __restrict__ bJ, int first,
                                    int count, int cls, float beta, uint32_t move, uint32_t key0, uint32_t key1,
                                    uint32_t replica_base, unsigned long long* __restrict__ counters,
                                    int32_t* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)R * count;
    if (t >= M) return;
    const int r = (int)(t / count), b = first + (int)(t % count);
    const int si = bi[b], sj = bj[b];
    if ((unsigned)si >= (unsigned)n || (unsigned)sj >= (unsigned)n) {
        pq_set_status(status, PQ_ERR_BAD_INDEX);
        return;
    }
    bool bad = false;
    PairIn<W, MAXD> p;
    W* words_r = words + (int64_t)r * n;
    load_pair<W, MAXD>(words_r, si, sj, bJ[b], n, maxdeg, nbr, cpl, field, p, bad);
    float dEi, dEj;
    int c;
    const float dE = pair_cost<W, MAXD>(p, P, maxdeg, slice_mask<W>(P), dEi, dEj, c);
    const pq_u32x4 u = pq_philox(pq_u32x4{(uint32_t)b, move, replica_base + (uint32_t)r, (5u << 24) | (uint32_t)cls},
                                 key0, key1);
    const bool acc = pair_accept(dE, beta, 1.0f, 1.0f, pq_u01(u.y));
    if (acc) pair_apply<W>(words_r, si, sj, P);
    if (counters) {
        atomicAdd(counters, 1ull);
        if (acc) atomicAdd(counters + 1, 1ull);
    }
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
}

// ---------------------------------------------------------------------------
// training: binary cross-entropy against soft targets y (the Metropolis
// acceptance probability of the recorded move), mean over the batch.
// ---------------------------------------------------------------------------

// dlogit = (sigmoid(l) - y) / B; dh2 = dlogit * w3 * [h2 > 0] in BF16, row-major and
// transposed ([64][B]); loss partial sums; grads of w3 and b3 accumulated.
__global__ void head_backward_kernel(const float* __restrict__ H2, const float* __restrict__ logit,
                                     const float* __restrict__ y, const float* __restrict__ w3, int B,
                                     __nv_bfloat16* __restrict__ dH2, __nv_bfloat16* __restrict__ dH2T,
                                     float* __restrict__ gw3, float* __restrict__ gb3, float* __restrict__ loss) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ float sg[64];
    __shared__ float sb, sl;
    if (threadIdx.x < 64) sg[threadIdx.x] = 0.0f;
    if (threadIdx.x == 0) { sb = 0.0f; sl = 0.0f; }
    __syncthreads();
    if (b < B) {
        const float z = logit[b];
        const float p = sigmoidf_(z);
        const float yt = y[b];
        const float dl = (p - yt) / (float)B;
        // BCE with logits, numerically stable
        const float l = fmaxf(z, 0.0f) - z * yt + log1pf(__expf(-fabsf(z)));
        atomicAdd(&sl, l / (float)B);
        atomicAdd(&sb, dl);
        const float* h = H2 + (int64_t)b * kLd;
        for (int c = 0; c < 64; ++c) {
            const float hc = fmaxf(h[c], 0.0f);
            atomicAdd(&sg[c], dl * hc);
            const float g = h[c] > 0.0f ? dl * w3[c] : 0.0f;
            const __nv_bfloat16 gb = __float2bfloat16_rn(g);
            dH2[(int64_t)b * kLd + c] = gb;
            dH2T[(int64_t)c * B + b] = gb;
        }
    }
    __syncthreads();
    if (threadIdx.x < 64) atomicAdd(gw3 + threadIdx.x, sg[threadIdx.x]);
    if (threadIdx.x == 0) { atomicAdd(gb3, sb); atomicAdd(loss, sl); }
}

// g (FP32 [B][64], the GEMM dH1 = dH2 W2) -> masked by [h1 > 0] -> BF16 transposed [64][B];
// bias grads accumulated.
__global__ void hidden_backward_kernel(const float* __restrict__ G, const float* __restrict__ H1, int B,
                                       __nv_bfloat16* __restrict__ dH1T, float* __restrict__ gb1) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ float sg[64];
    if (threadIdx.x < 64) sg[threadIdx.x] = 0.0f;
    __syncthreads();
    if (b < B) {
        for (int c = 0; c < 64; ++c) {
            const float g = H1[(int64_t)b * kLd + c] > 0.0f ? G[(int64_t)b * kLd + c] : 0.0f;
            dH1T[(int64_t)c * B + b] = __float2bfloat16_rn(g);
            atomicAdd(&sg[c], g);
        }
    }
    __syncthreads();
    if (threadIdx.x < 64) atomicAdd(gb1 + threadIdx.x, sg[threadIdx.x]);
}

// Column sums of a BF16 [64][B] matrix (bias gradient of layer 2 from dH2T).
__global__ void colsum_kernel(const __nv_bfloat16* __restrict__ T, int B, float* __restrict__ out) {
    const int c = blockIdx.x;
    float acc = 0.0f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) acc += __bfloat162float(T[(int64_t)c * B + b]);
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    __shared__ float part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        out[c] += s;
    }
}

// Row-major BF16 [B][64] -> transposed [64][B].
__global__ void transpose_bf16_kernel(const __nv_bfloat16* __restrict__ A, int B, __nv_bfloat16* __restrict__ AT) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)B * kLd) return;
    const int b = (int)(t / kLd), c = (int)(t % kLd);
    AT[(int64_t)c * B + b] = A[t];
}

// Adam on FP32 parameters.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}


// ---------------------------------------------------------------------------
// Fused learned move.  A persistent CTA of 4 warps takes tiles of 128 spins of
// the class; thread t owns spin t of the tile and TMEM lane t.  Per tile:
//   features of the current and flipped world-lines -> X, Xf (BF16, K = 16,
//   columns 8..15 zero) in shared memory;
//   layer 1: two tcgen05 MMAs (M = 128, N = 64, K = 16) into TMEM columns 0..63
//   (current) and 64..127 (flipped); bias + ReLU -> H, Hf (BF16) in shared memory;
//   layer 2: 2 x 4 MMAs (K = 64) into the same columns; bias + ReLU + head in
//   registers, so each thread holds both logits of its spin;
//   the MH decision as propose_kernel makes it.
// The epilogues round exactly as the unfused path does (relu(acc + b1) to
// BF16; head acc = b3 + sum_c relu(acc_c + b2) w3_c in column order), and the
// K = 16 layer 1 equals the unfused K = 64 one whose extra columns are zero.
// ---------------------------------------------------------------------------
constexpr int kTile = 128;
constexpr int kK1 = 16;
constexpr int kOffX = 0;                              // X, Xf: 2 x [128][16] BF16
constexpr int kOffH = kOffX + 2 * kTile * kK1 * 2;    // H, Hf: 2 x [128][64] BF16
constexpr int kOffW1 = kOffH + 2 * kTile * kLd * 2;   // W1: [64][16] BF16
constexpr int kOffW2 = kOffW1 + kLd * kK1 * 2;        // W2: [64][64] BF16
constexpr int kOffB = kOffW2 + kLd * kLd * 2;         // b1, b2, w3: 3 x 64 FP32
constexpr int kOffBar = kOffB + 3 * kLd * 4;          // mbarrier, TMEM slot
constexpr int kSmemMove = kOffBar + 16;
constexpr long long kMmaWait = 1ll << 24;
static_assert(kOffH % 16 == 0 && kOffW1 % 16 == 0 && kOffW2 % 16 == 0 && kOffBar % 8 == 0, "alignment");

struct MoveArgs {
    int n, P, R, maxdeg, cls, stride, csize;
    float beta, jp, qmin, b3;
    uint32_t move, key0, key1, replica_base;
    int64_t ntiles;
};

// Two floats rounded to BF16 (nearest even), the first in the low half (the lower address).
__device__ __forceinline__ uint32_t bf16x2_bits(float lo, float hi) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&b);
}

__device__ __forceinline__ float sigmoid_clamped(float z, float qmin) {
    return fminf(fmaxf(1.0f / (1.0f + expf(-z)), qmin), 1.0f);
}

template <typename W, int MAXD>
__global__ void __launch_bounds__(128) learned_move_kernel(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                                          const float* __restrict__ cpl,
                                                          const float* __restrict__ field,
                                                          const __nv_bfloat16* __restrict__ W1,
                                                          const __nv_bfloat16* __restrict__ W2,
                                                          const float* __restrict__ b1, const float* __restrict__ b2,
                                                          const float* __restrict__ w3, MoveArgs a,
                                                          float* __restrict__ logit_out,
                                                          unsigned long long* __restrict__ counters,
                                                          int32_t* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sX = smem + kOffX;
    unsigned char* sXf = sX + kTile * kK1 * 2;
    unsigned char* sH = smem + kOffH;
    unsigned char* sHf = sH + kTile * kLd * 2;
    unsigned char* sW1 = smem + kOffW1;
    unsigned char* sW2 = smem + kOffW2;
    float* sb1 = reinterpret_cast<float*>(smem + kOffB);
    float* sb2 = sb1 + kLd;
    float* sw3 = sb2 + kLd;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kOffBar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kOffBar + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t M = (int64_t)a.R * a.csize;

    // weights (W1 columns 0..15 of its padded 64) and the zero K padding of X, Xf
    for (int c = tid; c < kLd * (kK1 / 8); c += 128) {
        const int r = c / (kK1 / 8), kk = (c % (kK1 / 8)) * 8;
        *reinterpret_cast<uint4*>(sW1 + tc::tile_off(r, kk, kK1)) =
            *reinterpret_cast<const uint4*>(W1 + r * kLd + kk);
    }
    for (int c = tid; c < kLd * (kLd / 8); c += 128) {
        const int r = c / (kLd / 8), kk = (c % (kLd / 8)) * 8;
        *reinterpret_cast<uint4*>(sW2 + tc::tile_off(r, kk, kLd)) =
            *reinterpret_cast<const uint4*>(W2 + r * kLd + kk);
    }
    for (int c = tid; c < 2 * kTile * kK1 * 2 / 16; c += 128) reinterpret_cast<uint4*>(sX)[c] = make_uint4(0, 0, 0, 0);
    if (tid < kLd) { sb1[tid] = b1[tid]; sb2[tid] = b2[tid]; sw3[tid] = w3[tid]; }
    if (tid == 0) {
        tc::mbar_init(tc::smem_addr(mbar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(tslot), 2 * kLd);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t tlane = tmem + ((uint32_t)(32 * warp) << 16);
    constexpr uint32_t idesc = tc::idesc_bf16(kTile, kLd);
    const W mask = slice_mask<W>(a.P);
    uint32_t phase = 0;
    bool ok = true;

    // the inputs of the next tile's features are loaded while this tile's MMAs run
    SiteIn<W, MAXD> nxt;
    auto prefetch = [&](int64_t tile) {
        const int64_t t = tile * kTile + tid;
        if (tile < a.ntiles && t < M) {
            const int r = (int)(t / a.csize);
            const int i = a.cls * a.stride + (int)(t - (int64_t)r * a.csize);
            load_site_in<W, MAXD>(words + (int64_t)r * a.n, i, a.n, a.maxdeg, nbr, cpl, field, nxt);
        }
    };
    prefetch(blockIdx.x);
    for (int64_t tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        const int64_t t = tile * kTile + tid;
        const bool valid = t < M;
        int r = 0, i = 0;
        float de = 0.0f;
        {
            float x[kFeat] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (valid) {
                r = (int)(t / a.csize);
                i = a.cls * a.stride + (int)(t - (int64_t)r * a.csize);
                site_features<W, MAXD>(nxt, a.P, a.maxdeg, a.beta, a.jp, x, de);
            }
            // one 16-byte core-matrix row each: features 0..7 of the current and the flipped world-line
            uint32_t pc[4], pf[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = 2 * e;
                const float f0 = (c == 2 || c == 4) ? -x[c] : x[c];
                const float f1 = (c + 1 == 5) ? -x[c + 1] : x[c + 1];
                pc[e] = bf16x2_bits(x[c], x[c + 1]);
                pf[e] = bf16x2_bits(f0, f1);
            }
            *reinterpret_cast<uint4*>(sX + tc::tile_off(tid, 0, kK1)) = make_uint4(pc[0], pc[1], pc[2], pc[3]);
            *reinterpret_cast<uint4*>(sXf + tc::tile_off(tid, 0, kK1)) = make_uint4(pf[0], pf[1], pf[2], pf[3]);
        }
        // layer 1
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint64_t bd = tc::smem_desc(tc::smem_addr(sW1), 128, kK1 * 16);
            tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(sX), 128, kK1 * 16), bd, idesc, 0u);
            tc::mma_bf16(tmem + kLd, tc::smem_desc(tc::smem_addr(sXf), 128, kK1 * 16), bd, idesc, 0u);
            tc::mma_commit(tc::smem_addr(mbar));
        }
        // spins of the next tile are not touched by this tile's moves (one thread per spin)
        prefetch(tile + gridDim.x);
        if (!tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait)) { ok = false; break; }
        phase ^= 1u;
        tc::fence_after_sync();
#pragma unroll 1
        for (int half = 0; half < 2; ++half) {
            uint32_t u0[32], u1[32];
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd), u0);
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd + 32), u1);
            tc::tmem_wait_ld();
            unsigned char* dst = half ? sHf : sH;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t pk[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = 8 * q + 2 * e;
                    const float v0 = __uint_as_float(j < 32 ? u0[j & 31] : u1[j & 31]);
                    const float v1 = __uint_as_float(j + 1 < 32 ? u0[(j + 1) & 31] : u1[(j + 1) & 31]);
                    pk[e] = bf16x2_bits(fmaxf(__fadd_rn(v0, sb1[j]), 0.0f), fmaxf(__fadd_rn(v1, sb1[j + 1]), 0.0f));
                }
                *reinterpret_cast<uint4*>(dst + tc::tile_off(tid, 8 * q, kLd)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        // layer 2
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int st = 0; st < kLd / 16; ++st) {
                const uint64_t bd = tc::smem_desc(tc::smem_addr(sW2) + st * 256, 128, kLd * 16);
                tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(sH) + st * 256, 128, kLd * 16), bd, idesc,
                             st > 0 ? 1u : 0u);
                tc::mma_bf16(tmem + kLd, tc::smem_desc(tc::smem_addr(sHf) + st * 256, 128, kLd * 16), bd, idesc,
                             st > 0 ? 1u : 0u);
            }
            tc::mma_commit(tc::smem_addr(mbar));
        }
        if (!tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait)) { ok = false; break; }
        phase ^= 1u;
        tc::fence_after_sync();
        float lg0 = a.b3, lg1 = a.b3;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t u0[32], u1[32];
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd), u0);
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd + 32), u1);
            tc::tmem_wait_ld();
            float acc = a.b3;
#pragma unroll
            for (int j = 0; j < 32; ++j)
                acc = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(u0[j]), sb2[j]), 0.0f), sw3[j], acc);
#pragma unroll
            for (int j = 0; j < 32; ++j)
                acc = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(u1[j]), sb2[32 + j]), 0.0f), sw3[32 + j], acc);
            if (half == 0) lg0 = acc; else lg1 = acc;
        }
        const float lg[2] = {lg0, lg1};
        // MH decision: uniforms Philox(ctr = {i, move, replica, 3 << 24 | cls}) words 0 and 1
        bool proposed = false, accepted = false;
        if (valid) {
            if (logit_out) {
                logit_out[t] = lg[0];
                logit_out[M + t] = lg[1];
            }
            const pq_u32x4 u = pq_philox(
                pq_u32x4{(uint32_t)i, a.move, a.replica_base + (uint32_t)r, (3u << 24) | (uint32_t)a.cls}, a.key0,
                a.key1);
            const float q = sigmoid_clamped(lg[0], a.qmin), qf = sigmoid_clamped(lg[1], a.qmin);
            proposed = pq_u01(u.x) < q;
            if (proposed) {
                const float lr = -a.beta * de + logf(qf) - logf(q);
                accepted = lr >= 0.0f || pq_u01(u.y) < expf(lr);
                if (accepted) words[(int64_t)r * a.n + i] ^= mask;
            }
        }
        const unsigned bp = __ballot_sync(0xffffffffu, proposed), ba = __ballot_sync(0xffffffffu, accepted);
        if (counters && lane == 0) {
            if (bp) atomicAdd(counters, (unsigned long long)__popc(bp));
            if (ba) atomicAdd(counters + 1, (unsigned long long)__popc(ba));
        }
        tc::fence_before_sync();
    }
    if (!ok) {
        pq_set_status(status, PQ_ERR_TIMEOUT);
        // the MMAs of the phase that timed out get one more bounded chance to land before TMEM is freed
        tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, 2 * kLd);
}

// Fused learned pair move: the tile pipeline of learned_move_kernel with one
// (replica, bond) row per thread -- features of the current and the flipped pair
// (pair_features), both layers on the tensor cores, head, and the decision and
// flips of pair_propose_kernel.  Rows t = r * count + b of bonds [first, first +
// count) of class `cls`.  The inputs of the next tile are loaded while this
// tile's moves land: the bonds of a class are independent, so no move of the
// class changes them.
struct PairMoveArgs {
    int n, P, R, maxdeg, cls, first, count;
    float beta, jp, qmin, b3;
    uint32_t move, key0, key1, replica_base;
    int64_t ntiles;
};

template <typename W, int MAXD>
__global__ void __launch_bounds__(128) learned_pair_kernel(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                                          const float* __restrict__ cpl,
                                                          const float* __restrict__ field,
                                                          const int32_t* __restrict__ bi,
                                                          const int32_t* __restrict__ bj,
                                                          const float* __restrict__ bJ,
                                                          const __nv_bfloat16* __restrict__ W1,
                                                          const __nv_bfloat16* __restrict__ W2,
                                                          const float* __restrict__ b1, const float* __restrict__ b2,
                                                          const float* __restrict__ w3, PairMoveArgs a,
                                                          unsigned long long* __restrict__ counters,
                                                          int32_t* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char* sX = smem + kOffX;
    unsigned char* sXf = sX + kTile * kK1 * 2;
    unsigned char* sH = smem + kOffH;
    unsigned char* sHf = sH + kTile * kLd * 2;
    unsigned char* sW1 = smem + kOffW1;
    unsigned char* sW2 = smem + kOffW2;
    float* sb1 = reinterpret_cast<float*>(smem + kOffB);
    float* sb2 = sb1 + kLd;
    float* sw3 = sb2 + kLd;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kOffBar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kOffBar + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t M = (int64_t)a.R * a.count;

    for (int c = tid; c < kLd * (kK1 / 8); c += 128) {
        const int r = c / (kK1 / 8), kk = (c % (kK1 / 8)) * 8;
        *reinterpret_cast<uint4*>(sW1 + tc::tile_off(r, kk, kK1)) =
            *reinterpret_cast<const uint4*>(W1 + r * kLd + kk);
    }
    for (int c = tid; c < kLd * (kLd / 8); c += 128) {
        const int r = c / (kLd / 8), kk = (c % (kLd / 8)) * 8;
        *reinterpret_cast<uint4*>(sW2 + tc::tile_off(r, kk, kLd)) =
            *reinterpret_cast<const uint4*>(W2 + r * kLd + kk);
    }
    for (int c = tid; c < 2 * kTile * kK1 * 2 / 16; c += 128) reinterpret_cast<uint4*>(sX)[c] = make_uint4(0, 0, 0, 0);
    if (tid < kLd) { sb1[tid] = b1[tid]; sb2[tid] = b2[tid]; sw3[tid] = w3[tid]; }
    if (tid == 0) {
        tc::mbar_init(tc::smem_addr(mbar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(tslot), 2 * kLd);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t tlane = tmem + ((uint32_t)(32 * warp) << 16);
    constexpr uint32_t idesc = tc::idesc_bf16(kTile, kLd);
    const W mask = slice_mask<W>(a.P);
    uint32_t phase = 0;
    bool ok = true, bad = false;

    PairIn<W, MAXD> nxt;
    bool nxt_ok = false;
    auto prefetch = [&](int64_t tile) {
        const int64_t t = tile * kTile + tid;
        nxt_ok = false;
        if (tile < a.ntiles && t < M) {
            const int r = (int)(t / a.count);
            const int b = a.first + (int)(t - (int64_t)r * a.count);
            const int si = bi[b], sj = bj[b];
            if ((unsigned)si < (unsigned)a.n && (unsigned)sj < (unsigned)a.n) {
                load_pair<W, MAXD>(words + (int64_t)r * a.n, si, sj, bJ[b], a.n, a.maxdeg, nbr, cpl, field, nxt,
                                   bad);
                nxt_ok = true;
            } else {
                bad = true;
            }
        }
    };
    prefetch(blockIdx.x);
    for (int64_t tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        const int64_t t = tile * kTile + tid;
        const bool valid = t < M && nxt_ok;
        int r = 0, b = 0, si = 0, sj = 0;
        float de = 0.0f;
        {
            float x[kFeat] = {0, 0, 0, 0, 0, 0, 0, 0}, xf[kFeat] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (valid) {
                r = (int)(t / a.count);
                b = a.first + (int)(t - (int64_t)r * a.count);
                si = nxt.si;
                sj = nxt.sj;
                de = pair_features<W, MAXD>(nxt, a.P, a.maxdeg, a.beta, a.jp, x);
                flip_pair<W, MAXD>(nxt, mask);
                pair_features<W, MAXD>(nxt, a.P, a.maxdeg, a.beta, a.jp, xf);
            }
            uint32_t pc[4], pf[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                pc[e] = bf16x2_bits(x[2 * e], x[2 * e + 1]);
                pf[e] = bf16x2_bits(xf[2 * e], xf[2 * e + 1]);
            }
            *reinterpret_cast<uint4*>(sX + tc::tile_off(tid, 0, kK1)) = make_uint4(pc[0], pc[1], pc[2], pc[3]);
            *reinterpret_cast<uint4*>(sXf + tc::tile_off(tid, 0, kK1)) = make_uint4(pf[0], pf[1], pf[2], pf[3]);
        }
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint64_t bd = tc::smem_desc(tc::smem_addr(sW1), 128, kK1 * 16);
            tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(sX), 128, kK1 * 16), bd, idesc, 0u);
            tc::mma_bf16(tmem + kLd, tc::smem_desc(tc::smem_addr(sXf), 128, kK1 * 16), bd, idesc, 0u);
            tc::mma_commit(tc::smem_addr(mbar));
        }
        prefetch(tile + gridDim.x);
        if (!tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait)) { ok = false; break; }
        phase ^= 1u;
        tc::fence_after_sync();
#pragma unroll 1
        for (int half = 0; half < 2; ++half) {
            uint32_t u0[32], u1[32];
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd), u0);
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd + 32), u1);
            tc::tmem_wait_ld();
            unsigned char* dst = half ? sHf : sH;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                uint32_t pk[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = 8 * q + 2 * e;
                    const float v0 = __uint_as_float(j < 32 ? u0[j & 31] : u1[j & 31]);
                    const float v1 = __uint_as_float(j + 1 < 32 ? u0[(j + 1) & 31] : u1[(j + 1) & 31]);
                    pk[e] = bf16x2_bits(fmaxf(__fadd_rn(v0, sb1[j]), 0.0f), fmaxf(__fadd_rn(v1, sb1[j + 1]), 0.0f));
                }
                *reinterpret_cast<uint4*>(dst + tc::tile_off(tid, 8 * q, kLd)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            }
        }
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int st = 0; st < kLd / 16; ++st) {
                const uint64_t bd = tc::smem_desc(tc::smem_addr(sW2) + st * 256, 128, kLd * 16);
                tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(sH) + st * 256, 128, kLd * 16), bd, idesc,
                             st > 0 ? 1u : 0u);
                tc::mma_bf16(tmem + kLd, tc::smem_desc(tc::smem_addr(sHf) + st * 256, 128, kLd * 16), bd, idesc,
                             st > 0 ? 1u : 0u);
            }
            tc::mma_commit(tc::smem_addr(mbar));
        }
        if (!tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait)) { ok = false; break; }
        phase ^= 1u;
        tc::fence_after_sync();
        float lg[2] = {a.b3, a.b3};
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t u0[32], u1[32];
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd), u0);
            tc::tmem_ld32_async(tlane + (uint32_t)(half * kLd + 32), u1);
            tc::tmem_wait_ld();
            float acc = a.b3;
#pragma unroll
            for (int j = 0; j < 32; ++j)
                acc = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(u0[j]), sb2[j]), 0.0f), sw3[j], acc);
#pragma unroll
            for (int j = 0; j < 32; ++j)
                acc = __fmaf_rn(fmaxf(__fadd_rn(__uint_as_float(u1[j]), sb2[32 + j]), 0.0f), sw3[32 + j], acc);
            lg[half] = acc;
        }
        bool proposed = false, accepted = false;
        if (valid) {
            const pq_u32x4 u = pq_philox(
                pq_u32x4{(uint32_t)b, a.move, a.replica_base + (uint32_t)r, (5u << 24) | (uint32_t)a.cls}, a.key0,
                a.key1);
            const float q = fminf(fmaxf(pair_sigmoid(lg[0]), a.qmin), 1.0f);
            const float qf = fminf(fmaxf(pair_sigmoid(lg[1]), a.qmin), 1.0f);
            proposed = pq_u01(u.x) < q;
            accepted = proposed && pair_accept(de, a.beta, q, qf, pq_u01(u.y));
            if (accepted) pair_apply<W>(words + (int64_t)r * a.n, si, sj, a.P);
        }
        const unsigned bp = __ballot_sync(0xffffffffu, proposed), ba = __ballot_sync(0xffffffffu, accepted);
        if (counters && lane == 0) {
            if (bp) atomicAdd(counters, (unsigned long long)__popc(bp));
            if (ba) atomicAdd(counters + 1, (unsigned long long)__popc(ba));
        }
        tc::fence_before_sync();
    }
    if (!ok) {
        pq_set_status(status, PQ_ERR_TIMEOUT);
        tc::mbar_wait(tc::smem_addr(mbar), phase, kMmaWait);
    }
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, 2 * kLd);
}

// Uniform world-line move of every spin of class `cls` (the plain form the
// learned one is judged against): proposed always, accepted with
// min(1, exp(-beta dE)), dE = 2 worldline_align; the same uniforms and the same
// decision arithmetic as the learned move with q = q' = 1.
template <typename W, int MAXD>
__global__ void uniform_move_kernel(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                    const float* __restrict__ cpl, const float* __restrict__ field, MoveArgs a,
                                    unsigned long long* __restrict__ counters) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t M = (int64_t)a.R * a.csize;
    bool accepted = false;
    if (t < M) {
        const int r = (int)(t / a.csize);
        const int i = a.cls * a.stride + (int)(t - (int64_t)r * a.csize);
        const W* wr = words + (int64_t)r * a.n;
        const W mask = slice_mask<W>(a.P);
        W nbw[MAXD];
        float J[MAXD];
        load_neighbourhood<W, MAXD>(wr, i, a.n, a.maxdeg, nbr, cpl, nbw, J);
        const W wi = wr[i] & mask;
        const float de = __fmul_rn(2.0f, worldline_align<W, MAXD>(wi, nbw, J, a.maxdeg, __ldg(field + i), a.P, mask));
        const pq_u32x4 u = pq_philox(
            pq_u32x4{(uint32_t)i, a.move, a.replica_base + (uint32_t)r, (3u << 24) | (uint32_t)a.cls}, a.key0, a.key1);
        const float lr = -a.beta * de;
        accepted = lr >= 0.0f || pq_u01(u.y) < expf(lr);
        if (accepted) words[(int64_t)r * a.n + i] ^= mask;
    }
    const unsigned ba = __ballot_sync(0xffffffffu, accepted);
    const unsigned bp = __ballot_sync(0xffffffffu, t < M);
    if (counters && (threadIdx.x & 31) == 0) {
        if (bp) atomicAdd(counters, (unsigned long long)__popc(bp));
        if (ba) atomicAdd(counters + 1, (unsigned long long)__popc(ba));
    }
}

// Persistent grid: SMs x resident CTAs per SM.  The runtime's occupancy query
// reports one CTA per SM for this kernel (it cannot see the TMEM budget), so the
// residency is computed from the kernel's own resources: shared memory, registers
// and TMEM (4 x 128 columns per SM) -- four CTAs per SM.  One cache per kernel
// instantiation (the Tag), per device.
template <typename W, int MAXD, int KIND>
struct GridTag {};

template <typename Tag>
int tile_grid(const void* kernel, int64_t ntiles) {
    // per device: (context identity, SMs, resident CTAs per SM)
    static std::mutex mu;
    static unsigned long long ctx[kPqMaxDevices];
    static int nsm_dev[kPqMaxDevices], occ_dev[kPqMaxDevices];
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kPqMaxDevices) return -(int)cudaErrorInvalidDevice;   // callers read <= 0 as an error
    std::lock_guard<std::mutex> lock(mu);
    const unsigned long long id = pq_context_id();
    if (!id || ctx[dev] != id) {
        int nsm = 0, smem_sm = 0, regs_sm = 0, reserved = 0;
        PQ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        PQ_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        PQ_CUDA_TRY(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
        PQ_CUDA_TRY(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
        PQ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMove));
        PQ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
        cudaFuncAttributes fa;
        PQ_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
        const int by_smem = smem_sm / (kSmemMove + (int)fa.sharedSizeBytes + reserved);
        const int warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;    // allocated per warp in units of 256
        const int by_regs = regs_sm / (warp_regs * 4);
        const int by_tmem = 512 / (2 * kLd);
        int occ = by_smem < by_regs ? by_smem : by_regs;
        occ = occ < by_tmem ? occ : by_tmem;
        nsm_dev[dev] = nsm;
        occ_dev[dev] = occ < 1 ? 1 : occ;
        ctx[dev] = pq_context_id();
    }
    const int64_t g = (int64_t)nsm_dev[dev] * occ_dev[dev];
    return (int)(ntiles < g ? ntiles : g);
}

template <typename W, int MAXD>
int move_grid(int64_t ntiles) {
    return tile_grid<GridTag<W, MAXD, 0>>((const void*)learned_move_kernel<W, MAXD>, ntiles);
}

template <typename W, int MAXD>
int pair_grid(int64_t ntiles) {
    return tile_grid<GridTag<W, MAXD, 1>>((const void*)learned_pair_kernel<W, MAXD>, ntiles);
}

inline unsigned blocks_for(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

// Runs the statement given with W = the word type and D = the unrolled neighbour count (4 or 16).
#define PQ_WORD_DEG_DISPATCH(word_bits, maxdeg, ...)                  \
    if ((word_bits) == 32 && (maxdeg) <= 4) {                          \
        using W = uint32_t;                                            \
        constexpr int D = 4;                                           \
        __VA_ARGS__;                                                   \
    } else if ((word_bits) == 32) {                                    \
        using W = uint32_t;                                            \
        constexpr int D = 16;                                          \
        __VA_ARGS__;                                                   \
    } else if ((word_bits) == 64 && (maxdeg) <= 4) {                   \
        using W = uint64_t;                                            \
        constexpr int D = 4;                                           \
        __VA_ARGS__;                                                   \
    } else if ((word_bits) == 64) {                                    \
        using W = uint64_t;                                            \
        constexpr int D = 16;                                          \
        __VA_ARGS__;                                                   \
    } else {                                                           \
        return PQ_ERR_INVALID_ARG;                                     \
    }

}  // namespace

extern "C" {

int pq_mlp_features(const void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                    const float* cpl, const float* field, int cls, int stride, int csize, float beta, float jp,
                    void* X, float* dE, int64_t Mpad, void* stream) {
    if (!words || !field || !X || !dE || n <= 0 || P < 1 || R <= 0 || csize < 0 || maxdeg > 16 ||
        Mpad < (int64_t)R * csize)
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * csize;
    if (M == 0) return PQ_OK;
    cudaStream_t st = (cudaStream_t)stream;
    PQ_WORD_DEG_DISPATCH(word_bits, maxdeg,
                         (features_kernel<W, D><<<blocks_for(M), 256, 0, st>>>((const W*)words, n, P, R, maxdeg, nbr,
                                                                               cpl, field, cls, stride, csize, beta,
                                                                               jp, (__nv_bfloat16*)X, dE, Mpad)));
    return pq_launch_status();
}

int pq_mlp_relu_bf16(const float* H, void* out, int64_t n, void* stream) {
    if (!H || !out || n < 0) return PQ_ERR_INVALID_ARG;
    if (n == 0) return PQ_OK;
    relu_bf16_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(H, (__nv_bfloat16*)out, n);
    return pq_launch_status();
}

int pq_mlp_head(const float* H2, const float* w3, float b3, float* logit, int64_t rows, void* stream) {
    if (!H2 || !w3 || !logit || rows < 0) return PQ_ERR_INVALID_ARG;
    if (rows == 0) return PQ_OK;
    head_kernel<<<blocks_for(rows), 256, 0, (cudaStream_t)stream>>>(H2, w3, b3, logit, rows);
    return pq_launch_status();
}

int pq_mlp_propose(void* words, int word_bits, int n, int P, int R, int cls, int stride, int csize,
                   const float* logit, const float* dE, int64_t Mpad, float qmin, float beta, uint32_t move,
                   uint64_t seed, int replica_base, unsigned long long* counters, void* stream) {
    if (!words || !logit || !dE || n <= 0 || P < 1 || R <= 0 || csize < 0 || Mpad < (int64_t)R * csize ||
        !(qmin > 0.0f) || qmin > 1.0f)
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * csize;
    if (M == 0) return PQ_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    if (word_bits == 32)
        propose_kernel<uint32_t><<<blocks_for(M), 256, 0, st>>>((uint32_t*)words, n, P, R, cls, stride, csize, logit,
                                                                dE, Mpad, qmin, beta, move, k0, k1,
                                                                (uint32_t)replica_base, counters);
    else if (word_bits == 64)
        propose_kernel<uint64_t><<<blocks_for(M), 256, 0, st>>>((uint64_t*)words, n, P, R, cls, stride, csize, logit,
                                                                dE, Mpad, qmin, beta, move, k0, k1,
                                                                (uint32_t)replica_base, counters);
    else
        return PQ_ERR_INVALID_ARG;
    return pq_launch_status();
}

int pq_mlp_learned_move(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                        const float* cpl, const float* field, int cls, int stride, int csize, float beta, float jp,
                        const void* W1, const void* W2, const float* b1, const float* b2, const float* w3, float b3,
                        float qmin, uint32_t move, uint64_t seed, int replica_base, float* logit_out,
                        unsigned long long* counters, int32_t* status, void* stream) {
    if (!words || !nbr || !cpl || !field || !W1 || !W2 || !b1 || !b2 || !w3 || n <= 0 || P < 1 || R <= 0 ||
        csize < 0 || maxdeg < 0 || maxdeg > 16 || !(qmin > 0.0f) || qmin > 1.0f || ((uintptr_t)W1 & 15) ||
        ((uintptr_t)W2 & 15) || (word_bits == 32 && P > 32) || P > 64)
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * csize;
    if (M == 0) return PQ_OK;
    MoveArgs a{n, P, R, maxdeg, cls, stride, csize, beta, jp, qmin, b3, move, (uint32_t)seed,
               (uint32_t)(seed >> 32), (uint32_t)replica_base, (M + kTile - 1) / kTile};
    cudaStream_t st = (cudaStream_t)stream;
    const __nv_bfloat16* w1 = (const __nv_bfloat16*)W1;
    const __nv_bfloat16* w2 = (const __nv_bfloat16*)W2;
    PQ_WORD_DEG_DISPATCH(word_bits, maxdeg, {
        const int grid = move_grid<W, D>(a.ntiles);
        if (grid <= 0) return grid;   // a CUDA error, negated
        learned_move_kernel<W, D><<<grid, 128, kSmemMove, st>>>((W*)words, nbr, cpl, field, w1, w2, b1, b2, w3, a,
                                                                logit_out, counters, status);
    });
    return pq_launch_status();
}

int pq_worldline_move(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                      const float* cpl, const float* field, int cls, int stride, int csize, float beta, uint32_t move,
                      uint64_t seed, int replica_base, unsigned long long* counters, void* stream) {
    if (!words || !nbr || !cpl || !field || n <= 0 || P < 1 || R <= 0 || csize < 0 || maxdeg < 0 || maxdeg > 16 ||
        (word_bits == 32 && P > 32) || P > 64)
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * csize;
    if (M == 0) return PQ_OK;
    MoveArgs a{n, P, R, maxdeg, cls, stride, csize, beta, 0.0f, 1.0f, 0.0f, move, (uint32_t)seed,
               (uint32_t)(seed >> 32), (uint32_t)replica_base, 0};
    cudaStream_t st = (cudaStream_t)stream;
    PQ_WORD_DEG_DISPATCH(word_bits, maxdeg,
                         (uniform_move_kernel<W, D><<<blocks_for(M), 256, 0, st>>>((W*)words, nbr, cpl, field, a,
                                                                                   counters)));
    return pq_launch_status();
}

int pq_mlp_learned_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                        const float* cpl, const float* field, int nclass, int stride, const int32_t* class_size,
                        float beta, float jp, const void* W1, const void* W2, const float* b1, const float* b2,
                        const float* w3, float b3, float qmin, uint32_t move, uint64_t seed, int replica_base,
                        unsigned long long* counters, int32_t* status, void* stream) {
    if (!class_size || nclass < 0 || nclass > PQ_MAX_CLASSES) return PQ_ERR_INVALID_ARG;
    for (int c = 0; c < nclass; ++c) {
        const int rc = pq_mlp_learned_move(words, word_bits, n, P, R, maxdeg, nbr, cpl, field, c, stride, class_size[c],
                                           beta, jp, W1, W2, b1, b2, w3, b3, qmin, move, seed, replica_base, nullptr,
                                           counters, status, stream);
        if (rc != PQ_OK) return rc;
    }
    return PQ_OK;
}

int pq_worldline_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                      const float* cpl, const float* field, int nclass, int stride, const int32_t* class_size,
                      float beta, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                      void* stream) {
    if (!class_size || nclass < 0 || nclass > PQ_MAX_CLASSES) return PQ_ERR_INVALID_ARG;
    for (int c = 0; c < nclass; ++c) {
        const int rc = pq_worldline_move(words, word_bits, n, P, R, maxdeg, nbr, cpl, field, c, stride, class_size[c],
                                         beta, move, seed, replica_base, counters, stream);
        if (rc != PQ_OK) return rc;
    }
    return PQ_OK;
}

int pq_pair_features(const void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                     const float* cpl, const float* field, const int32_t* bond_i, const int32_t* bond_j,
                     const float* bond_J, int first, int count, float beta, float jp, void* X, float* dE,
                     int64_t Mpad, int32_t* status, void* stream) {
    if (!words || !field || !bond_i || !bond_j || !bond_J || !X || !dE || n <= 0 || P < 1 || P > 64 || R <= 0 ||
        first < 0 || count < 0 || maxdeg < 0 || maxdeg > 16 || (maxdeg > 0 && (!nbr || !cpl)) ||
        Mpad < (int64_t)R * count || (P > 32 && word_bits != 64))
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * count;
    if (M == 0) return PQ_OK;
    cudaStream_t st = (cudaStream_t)stream;
    PQ_WORD_DEG_DISPATCH(word_bits, maxdeg,
                         (pair_features_kernel<W, D><<<blocks_for(M), 256, 0, st>>>(
                             (const W*)words, n, P, R, maxdeg, nbr, cpl, field, bond_i, bond_j, bond_J, first, count,
                             beta, jp, (__nv_bfloat16*)X, dE, Mpad, status)));
    return pq_launch_status();
}

int pq_pair_propose(void* words, int word_bits, int n, int P, int R, const int32_t* bond_i, const int32_t* bond_j,
                    int first, int count, int cls, const float* logit, const float* dE, int64_t Mpad, float qmin,
                    float beta, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                    int32_t* status, void* stream) {
    if (!words || !bond_i || !bond_j || !logit || !dE || n <= 0 || P < 1 || P > 64 || R <= 0 || first < 0 ||
        count < 0 || Mpad < (int64_t)R * count || !(qmin > 0.0f) || qmin > 1.0f || (P > 32 && word_bits != 64))
        return PQ_ERR_INVALID_ARG;
    const int64_t M = (int64_t)R * count;
    if (M == 0) return PQ_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    if (word_bits == 32)
        pair_propose_kernel<uint32_t><<<blocks_for(M), 256, 0, st>>>((uint32_t*)words, n, P, R, bond_i, bond_j, first,
                                                                     count, cls, logit, dE, Mpad, qmin, beta, move, k0,
                                                                     k1, (uint32_t)replica_base, counters, status);
    else if (word_bits == 64)
        pair_propose_kernel<uint64_t><<<blocks_for(M), 256, 0, st>>>((uint64_t*)words, n, P, R, bond_i, bond_j, first,
                                                                     count, cls, logit, dE, Mpad, qmin, beta, move, k0,
                                                                     k1, (uint32_t)replica_base, counters, status);
    else
        return PQ_ERR_INVALID_ARG;
    return pq_launch_status();
}

int pq_pair_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr, const float* cpl,
                 const float* field, const int32_t* bond_i, const int32_t* bond_j, const float* bond_J,
                 const int32_t* class_start, int nclass, float beta, uint32_t move, uint64_t seed, int replica_base,
                 unsigned long long* counters, int32_t* status, void* stream) {
    if (!words || !field || !bond_i || !bond_j || !bond_J || !class_start || nclass < 0 || n <= 0 || P < 1 ||
        P > 64 || R <= 0 || maxdeg < 0 || maxdeg > 16 || (maxdeg > 0 && (!nbr || !cpl)) ||
        (P > 32 && word_bits != 64))
        return PQ_ERR_INVALID_ARG;
    for (int c = 0; c < nclass; ++c)
        if (class_start[c] < 0 || class_start[c + 1] < class_start[c]) return PQ_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (int c = 0; c < nclass; ++c) {
        const int first = class_start[c], count = class_start[c + 1] - class_start[c];
        const int64_t M = (int64_t)R * count;
        if (M == 0) continue;
        PQ_WORD_DEG_DISPATCH(word_bits, maxdeg,
                             (pair_uniform_kernel<W, D><<<blocks_for(M), 256, 0, st>>>(
                                 (W*)words, n, P, R, maxdeg, nbr, cpl, field, bond_i, bond_j, bond_J, first, count, c,
                                 beta, move, k0, k1, (uint32_t)replica_base, counters, status)));
        const int rc = pq_launch_status();
        if (rc != PQ_OK) return rc;
    }
    return PQ_OK;
}

int pq_pair_learned_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                         const float* cpl, const float* field, const int32_t* bond_i, const int32_t* bond_j,
                         const float* bond_J, const int32_t* class_start, int nclass, float beta, float jp,
                         const void* W1, const void* W2, const float* b1, const float* b2, const float* w3, float b3,
                         float qmin, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                         int32_t* status, void* stream) {
    if (!words || !field || !bond_i || !bond_j || !bond_J || !class_start || nclass < 0 || !W1 || !W2 || !b1 ||
        !b2 || !w3 || n <= 0 || P < 1 || P > 64 || R <= 0 || maxdeg < 0 || maxdeg > 16 ||
        (maxdeg > 0 && (!nbr || !cpl)) || !(qmin > 0.0f) || qmin > 1.0f || (P > 32 && word_bits != 64))
        return PQ_ERR_INVALID_ARG;
    for (int c = 0; c < nclass; ++c)
        if (class_start[c] < 0 || class_start[c + 1] < class_start[c]) return PQ_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    for (int c = 0; c < nclass; ++c) {
        PairMoveArgs a;
        a.n = n; a.P = P; a.R = R; a.maxdeg = maxdeg; a.cls = c; a.first = class_start[c];
        a.count = class_start[c + 1] - class_start[c];
        a.beta = beta; a.jp = jp; a.qmin = qmin; a.b3 = b3;
        a.move = move; a.key0 = (uint32_t)seed; a.key1 = (uint32_t)(seed >> 32); a.replica_base = (uint32_t)replica_base;
        const int64_t M = (int64_t)R * a.count;
        if (M == 0) continue;
        a.ntiles = (M + kTile - 1) / kTile;
        PQ_WORD_DEG_DISPATCH(word_bits, maxdeg, {
            const int grid = pair_grid<W, D>(a.ntiles);
            if (grid <= 0) return grid;
            learned_pair_kernel<W, D><<<grid, 128, kSmemMove, st>>>((W*)words, nbr, cpl, field, bond_i, bond_j,
                                                                    bond_J, (const __nv_bfloat16*)W1,
                                                                    (const __nv_bfloat16*)W2, b1, b2, w3, a, counters,
                                                                    status);
        });
        const int rc = pq_launch_status();
        if (rc != PQ_OK) return rc;
    }
    return PQ_OK;
}

int pq_mlp_head_backward(const float* H2, const float* logit, const float* y, const float* w3, int B, void* dH2,
                         void* dH2T, float* gw3, float* gb3, float* loss, void* stream) {
    if (!H2 || !logit || !y || !w3 || !dH2 || !dH2T || !gw3 || !gb3 || !loss || B <= 0) return PQ_ERR_INVALID_ARG;
    head_backward_kernel<<<blocks_for(B), 256, 0, (cudaStream_t)stream>>>(
        H2, logit, y, w3, B, (__nv_bfloat16*)dH2, (__nv_bfloat16*)dH2T, gw3, gb3, loss);
    return pq_launch_status();
}

int pq_mlp_hidden_backward(const float* G, const float* H1, int B, void* dH1T, float* gb1, void* stream) {
    if (!G || !H1 || !dH1T || !gb1 || B <= 0) return PQ_ERR_INVALID_ARG;
    hidden_backward_kernel<<<blocks_for(B), 256, 0, (cudaStream_t)stream>>>(G, H1, B, (__nv_bfloat16*)dH1T, gb1);
    return pq_launch_status();
}

int pq_mlp_colsum_bf16(const void* T, int cols, int B, float* out, void* stream) {
    if (!T || !out || B <= 0 || cols <= 0) return PQ_ERR_INVALID_ARG;
    colsum_kernel<<<cols, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)T, B, out);
    return pq_launch_status();
}

int pq_mlp_transpose_bf16(const void* A, int B, void* AT, void* stream) {
    if (!A || !AT || B <= 0) return PQ_ERR_INVALID_ARG;
    transpose_bf16_kernel<<<blocks_for((int64_t)B * kLd), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)A, B, (__nv_bfloat16*)AT);
    return pq_launch_status();
}

int pq_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps, int step,
            void* stream) {
    if (!p || !g || !m || !v || n <= 0 || step < 1) return PQ_ERR_INVALID_ARG;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    adam_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return pq_launch_status();
}

}  // extern "C"
