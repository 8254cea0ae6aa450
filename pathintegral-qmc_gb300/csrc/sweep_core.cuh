// The packed sweep of one work item (a few replicas of one instance), run by a
// group of warps that synchronises on its own barrier.  Shared by the
// single-instance kernel (fast.cu: one group = the whole CTA) and the
// persistent batched kernel (batch.cu: several groups per CTA).
//
// Physics: qmc.QuantumAnneal (reference piqmc/qmc.pyx:30-136) with its two
// quirks corrected -- the energy difference is recomputed for every spin, and
// slice k couples to slices k-1 and k+1 (periodic).  Acceptance follows the
// reference's convention: flip when ediff > 0, else when u < exp(ediff / T),
// with J-perp = -(P T / 2) ln tanh(G / (P T)).
//
// Order of one local sweep: the M update classes (independent sets) are
// visited in a per-(replica, sweep) random order (or 0..M-1); within a class
// every spin updates all slices of one slice class at once, then all slices of
// the other.  Spins of one class share no coupling and slices of one slice
// class are not Trotter neighbours, so the updates of a phase are independent
// and the sweep equals a sequential sweep in a definite order.  Slice classes:
// P even -> {even k}, {odd k}; P odd -> {even k < P-1}, {odd k}, {P-1};
// P = 1 -> {0} (no Trotter term).  For P even the random order also picks,
// per class, which slice class goes first.
//
// Arithmetic of one update (spin i of replica r, slice k), every op one IEEE
// FP32 rounding, in this order:
//   e = s_i h_i;  e += J_im s_i s_jm for m = 0..maxdeg-1 (table order);
//   t = (J-perp s_i s_{k-1}) + (J-perp s_i s_{k+1})      (exact);
//   ediff = -2 (e + t);  flip if ediff > 0 or u < expf_neg(ediff * beta),
// u = ((r >> 9) + 1/2) * 2^-23.  Uniforms: Philox4x32-10, key = seed.  Local update:
// counter = (device slot i, sweep, replica, q << 16 | m >> 2), word m & 3 for
// the m-th slice of class q.  World-line move: counter = (i, last sweep of the
// step, replica, 1 << 24 | gm << 16 | class), word 0.  Class order of a sweep:
// counter = (0xFFFFFFFF, sweep, replica, 2 << 24 | b); words w[0..] of blocks
// b = 0,1,..; Fisher-Yates for j = M-1..1 swaps order[j] with
// order[(w[M-1-j] * (j+1)) >> 32]; w[M-1] bit p = which slice class goes first
// for the p-th visited class.
#pragma once
#include "common.cuh"

namespace pq {

constexpr int kMaxClasses = PQ_MAX_CLASSES;

// Everything one work item needs; the tables are the instance's.
struct Item {
    const int32_t* nbr;       // [maxdeg][n] device slots
    const float* cpl;         // [maxdeg][n]
    const float* field;       // [n], or null when every field is zero
    const int32_t* csize;     // [nclass] class sizes (global or shared memory)
    const float* jperp;       // [nsched]
    const float* betas;       // [nsched] or null (then beta)
    void* words;              // [nrep][n] world-lines (uint32 or uint64)
    int n, P, maxdeg, nclass, stride, order_mode;
    int nrep;
    uint32_t replica0;        // RNG replica id of the first replica
    uint32_t key0, key1;
    int64_t sweep_base;
    int nsched, mcsteps, global_moves;
    float beta;
};

// A set of warps of one CTA working on one item.
struct Group {
    int tid;    // thread index within the group
    int nthr;   // threads in the group (a multiple of 32)
    int bar;    // named barrier id; 0 = __syncthreads (the group is the whole CTA)
};

// A one-warp group needs no CTA barrier: __syncwarp orders its shared-memory
// accesses as bar.sync would.
__device__ __forceinline__ void group_sync(const Group& g) {
    if (g.bar == 0) __syncthreads();
    else if (g.nthr == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(g.bar), "r"(g.nthr) : "memory");
}

template <typename W>
__device__ __forceinline__ uint32_t bit_to_sign(W d, int k) {
    return (uint32_t)(d >> k) << 31;
}

template <typename W>
__device__ __forceinline__ W full_mask(int P) {
    return P >= (int)(8 * sizeof(W)) ? ~(W)0 : (((W)1 << P) - 1);
}

// Bits k of the result: s^k xor s^{k-1} (left) and s^k xor s^{k+1} (right), periodic in P.
template <typename W>
__device__ __forceinline__ void trotter_diffs(W w, int P, W mask, W& dl, W& dr) {
    const W up = ((w << 1) | (w >> (P - 1))) & mask;   // bit k = s^{k-1}
    const W dn = ((w >> 1) | (w << (P - 1))) & mask;   // bit k = s^{k+1}
    dl = w ^ up;
    dr = w ^ dn;
}

__device__ __forceinline__ float flip_sign(float v, uint32_t signbit) {
    return __uint_as_float(__float_as_uint(v) ^ signbit);
}

__device__ __forceinline__ int slice_count(int P, int q) {
    if (P == 1) return 1;
    if ((P & 1) == 0) return P >> 1;
    return q == 2 ? 1 : (P - 1) >> 1;
}

__device__ __forceinline__ int slice_of(int P, int q, int m) { return q == 2 ? P - 1 : 2 * m + q; }

// Class visiting order of one (replica, sweep) and the slice-class parity word.
template <typename KS>
__device__ inline void class_order(int M, int order_mode, const KS& ks, uint32_t sweep, uint32_t replica,
                                   uint8_t* order, uint32_t* parity) {
    for (int c = 0; c < M; ++c) order[c] = (uint8_t)c;
    if (order_mode == 0) { *parity = 0; return; }
    uint32_t w[4] = {0, 0, 0, 0};
    int used = 4, blk = 0;
    for (int j = M - 1; j >= 0; --j) {
        if (used == 4) {
            const pq_u32x4 r = pq_philox_ks(pq_u32x4{0xFFFFFFFFu, sweep, replica, (2u << 24) | (uint32_t)blk++}, ks);
            w[0] = r.x; w[1] = r.y; w[2] = r.z; w[3] = r.w;
            used = 0;
        }
        const uint32_t x = w[used++];
        if (j == 0) { *parity = x; break; }
        const uint32_t k = (uint32_t)(((uint64_t)x * (uint32_t)(j + 1)) >> 32);
        const uint8_t t = order[j]; order[j] = order[k]; order[k] = t;
    }
}

// A site's field; an instance without fields passes no table (+0, exactly what a
// table of zeros would give).
__device__ __forceinline__ float site_field(const Item& it, int i) { return it.field ? __ldg(it.field + i) : 0.0f; }

template <typename W, int MAXDEG>
__device__ __forceinline__ void load_site(const W* rw, int i, int n, int maxdeg, const int32_t* __restrict__ nbr,
                                          const float* __restrict__ cpl, W wi, W (&d)[MAXDEG], float (&J)[MAXDEG],
                                          bool& bad) {
#pragma unroll
    for (int m = 0; m < MAXDEG; ++m) {
        if (m < maxdeg) {
            int j = __ldg(nbr + (int64_t)m * n + i);
            if ((unsigned)j >= (unsigned)n) { bad = true; j = i; }
            J[m] = __ldg(cpl + (int64_t)m * n + i);
            d[m] = wi ^ rw[j];
        } else {
            J[m] = 0.0f;
            d[m] = 0;
        }
    }
}

// Metropolis decision for sum = e + t (ediff = -2 sum): flip when sum < 0, else
// when u < expf_neg(fl(sum * m2beta)) with m2beta = -2 beta.  The hardware 2^x
// (argument fl(sum * m2blog2e), m2blog2e = fl(-2 beta log2 e)) settles it outside
// a 1e-4 relative guard band -- its error against expf_neg is under 5e-5 for every
// argument above -87 (checked exhaustively on the GPU; measured 3.6e-6), and the
// rounding of its argument adds under 1.7e-5 -- and expf_neg itself settles the
// rest, so the result is exactly the specification's.
__device__ __forceinline__ bool decide(float sum, float u, float m2beta, float m2blog2e) {
    if (sum < 0.0f) return true;
    const float pf = pq_ex2_approx(__fmul_rn(sum, m2blog2e));
    if (u > __fmul_rn(pf, 1.0001f)) return false;
    if (u < __fmul_rn(pf, 0.9999f) && pf > 1e-30f) return true;
    return u < pq_expf_neg(__fmul_rn(sum, m2beta));
}

// Core of the compile-time path: NQH slices m = 0..NQH-1 whose bits sit at
// positions 2m of the 32-bit (q-shifted) words wq, dq, dl, dr; the m-th uses
// word m & 3 of Philox block blk0 + (m >> 2).  Returns the flips at bits 2m.
//   calm: cleared unless every slice's sum is at least smin (a certain rejection,
// settle_threshold).
template <int NQH, int DEG, typename KS>
__device__ __forceinline__ uint32_t update_half(uint32_t wq, const uint32_t (&dq)[DEG], uint32_t dl, uint32_t dr,
                                                const float (&J)[DEG], float h, float jp, int q, int blk0, uint32_t i,
                                                uint32_t sweep, uint32_t rep, const KS& ks, float m2beta,
                                                float m2blog2e, float smin, bool& calm) {
    uint32_t flips = 0;
#pragma unroll
    for (int blk = 0; blk < (NQH + 3) / 4; ++blk) {
        const pq_u32x4 rnd = pq_philox_ks(pq_u32x4{i, sweep, rep, (uint32_t)((q << 16) | (blk0 + blk))}, ks);
        const uint32_t rw4[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int mm = blk * 4 + jj;
            if (mm < NQH) {
                const int sh = 31 - 2 * mm;  // bit 2*mm -> sign bit
                float e = flip_sign(h, (wq << sh) & 0x80000000u);
#pragma unroll
                for (int m = 0; m < DEG; ++m) e = __fadd_rn(e, flip_sign(J[m], (dq[m] << sh) & 0x80000000u));
                const float t = __fadd_rn(flip_sign(jp, (dl << sh) & 0x80000000u), flip_sign(jp, (dr << sh) & 0x80000000u));
                const float sum = __fadd_rn(e, t);
                calm = calm && sum >= smin;
                if (decide(sum, pq_u01(rw4[jj]), m2beta, m2blog2e)) flips |= 1u << (2 * mm);
            }
        }
    }
    return flips;
}

// One spin's local update over the slices of slice class q, P = 2 * NQ slices
// fixed at compile time (NQ <= 16 with 32-bit words, NQ = 32 with 64-bit words
// as two 32-bit halves), DEG couplings.  Same arithmetic and uniforms as the
// generic path.
// calm: cleared unless every slice of the class is a certain rejection (sum >= smin)
// whose Trotter partners are not both opposite to it (t = -2 J-perp would fall as
// J-perp grows; t = 2 J-perp or 0 does not).
template <int NQ, int DEG, typename W, typename KS>
__device__ __forceinline__ W update_fixed(W wi, const W (&d)[DEG], const float (&J)[DEG], float h, float jp, int q,
                                          uint32_t i, uint32_t sweep, uint32_t rep, const KS& ks, float m2beta,
                                          float m2blog2e, float smin, bool& calm) {
    constexpr int P = 2 * NQ;
    constexpr int BITS = 8 * sizeof(W);
    constexpr W MASK = P >= BITS ? ~(W)0 : (((W)1 << P) - 1);
    const W up = ((wi << 1) | (wi >> (P - 1))) & MASK;
    const W dn = ((wi >> 1) | (wi << (P - 1))) & MASK;
    const W dlw = wi ^ up, drw = wi ^ dn;
    W cm = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) cm |= (W)1 << (2 * k);
    calm = calm && (dlw & drw & (cm << q)) == 0;
    W flips = 0;
#pragma unroll
    for (int half = 0; half < (P + 31) / 32; ++half) {
        constexpr int NQH = NQ < 16 ? NQ : 16;
        uint32_t dq[DEG];
#pragma unroll
        for (int m = 0; m < DEG; ++m) dq[m] = (uint32_t)(d[m] >> (32 * half)) >> q;
        const uint32_t f = update_half<NQH, DEG, KS>((uint32_t)(wi >> (32 * half)) >> q, dq,
                                                     (uint32_t)(dlw >> (32 * half)) >> q,
                                                     (uint32_t)(drw >> (32 * half)) >> q, J, h, jp, q, 4 * half, i,
                                                     sweep, rep, ks, m2beta, m2blog2e, smin, calm);
        flips |= (W)f << (32 * half);
    }
    return flips << q;
}

// The share of lane t of L lanes (L a power of two) in update_fixed's work on slice
// class q: the Philox blocks b = t, t + L, ... of the class (4 slices each), with the
// same uniforms and arithmetic; the L lanes' flips together are update_fixed's.  Each
// block's words are shifted once so that its slices sit at fixed bit positions.  One
// block per loop pass: smaller code than update_fixed's unrolled classes (what the
// batched kernel, with a variant per instance shape, wants).
template <int NQ, int DEG, typename W, typename KS>
__device__ __forceinline__ W update_part(W wi, const W (&d)[DEG], const float (&J)[DEG], float h, float jp, int q,
                                         uint32_t i, uint32_t sweep, uint32_t rep, const KS& ks, float m2beta,
                                         float m2blog2e, float smin, bool& calm, int t, int L) {
    constexpr int P = 2 * NQ;
    constexpr int NB = (NQ + 3) / 4;
    constexpr int BITS = 8 * sizeof(W);
    constexpr W MASK = P >= BITS ? ~(W)0 : (((W)1 << P) - 1);
    const W up = ((wi << 1) | (wi >> (P - 1))) & MASK;
    const W dn = ((wi >> 1) | (wi << (P - 1))) & MASK;
    const W dlw = wi ^ up, drw = wi ^ dn;
    W cm = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) cm |= (W)1 << (2 * k);
    calm = calm && (dlw & drw & (cm << q)) == 0;
    W flips = 0;
#pragma unroll 1
    for (int b = t; b < NB; b += L) {
        const int sh = 8 * b + q;   // bit of the block's first slice
        const uint32_t wq = (uint32_t)(wi >> sh), dl = (uint32_t)(dlw >> sh), dr = (uint32_t)(drw >> sh);
        uint32_t dq[DEG];
#pragma unroll
        for (int m = 0; m < DEG; ++m) dq[m] = (uint32_t)(d[m] >> sh);
        const int nv = NQ - 4 * b;   // slices of this block (4, or fewer in the last)
        const pq_u32x4 rnd = pq_philox_ks(pq_u32x4{i, sweep, rep, (uint32_t)((q << 16) | b)}, ks);
        const uint32_t rw4[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
        uint32_t f = 0;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            if (jj < nv) {
                const int s2 = 31 - 2 * jj;  // bit 2 jj -> sign bit
                float e = flip_sign(h, (wq << s2) & 0x80000000u);
#pragma unroll
                for (int m = 0; m < DEG; ++m) e = __fadd_rn(e, flip_sign(J[m], (dq[m] << s2) & 0x80000000u));
                const float tt =
                    __fadd_rn(flip_sign(jp, (dl << s2) & 0x80000000u), flip_sign(jp, (dr << s2) & 0x80000000u));
                const float sum = __fadd_rn(e, tt);
                calm = calm && sum >= smin;
                if (decide(sum, pq_u01(rw4[jj]), m2beta, m2blog2e)) f |= 1u << (2 * jj);
            }
        }
        flips |= (W)f << sh;
    }
    return flips;
}

// One 32-bit half (bits 32*half .. 32*half+31) of update_fixed<32, DEG, uint64_t>:
// the same updates, uniforms and arithmetic for the slices of that half, so two
// lanes that take one half each and combine their flips reproduce it exactly.
template <int DEG, typename KS>
__device__ __forceinline__ uint64_t update_fixed_half64(uint64_t wi, const uint64_t (&d)[DEG], const float (&J)[DEG],
                                                        float h, float jp, int q, int half, uint32_t i,
                                                        uint32_t sweep, uint32_t rep, const KS& ks, float m2beta,
                                                        float m2blog2e, float smin, bool& calm) {
    const uint64_t up = (wi << 1) | (wi >> 63);
    const uint64_t dn = (wi >> 1) | (wi << 63);
    const uint64_t dlw = wi ^ up, drw = wi ^ dn;
    const int sh = 32 * half;
    calm = calm && ((uint32_t)((dlw & drw) >> sh) & (0x55555555u << q)) == 0;
    uint32_t dq[DEG];
#pragma unroll
    for (int m = 0; m < DEG; ++m) dq[m] = (uint32_t)(d[m] >> sh) >> q;
    const uint32_t f = update_half<16, DEG, KS>((uint32_t)(wi >> sh) >> q, dq, (uint32_t)(dlw >> sh) >> q,
                                                (uint32_t)(drw >> sh) >> q, J, h, jp, q, 4 * half, i, sweep, rep, ks,
                                                m2beta, m2blog2e, smin, calm);
    return ((uint64_t)f << sh) << q;
}

// Settled decisions.  The smallest uniform is 2^-24 (pq_u01), and expf_neg(x) <=
// 2^-24 for every FP32 x <= kSettledX = -16.63553237915039 (bit pattern 0xc1851592;
// checked over every float in [-87, kSettledX]; below -87 expf_neg is 0).  So an
// update with sum >= 0 and fl(sum * m2beta) <= kSettledX rejects whatever its
// uniform, and one with sum < 0 flips whatever its uniform.
__device__ __forceinline__ float settled_x() { return __uint_as_float(0xc1851592u); }

// Slice-class masks of P = 2 * NQ slices: bits of class 0 (even k), and the same
// without its top bit (the bits b whose class successor b + 2 is in the class).
template <typename W, int NQ>
struct ClassMasks {
    static constexpr W class0() {
        W m = 0;
        for (int k = 0; k < NQ; ++k) m |= (W)1 << (2 * k);
        return m;
    }
    static constexpr W CM0 = class0();
    static constexpr W IN0 = NQ > 0 ? (W)(CM0 & ~((W)1 << (NQ > 0 ? 2 * NQ - 2 : 0))) : (W)0;
    static constexpr W MASK = 2 * NQ >= (int)(8 * sizeof(W)) ? ~(W)0 : (((W)1 << (2 * NQ)) - 1);
};

// Outcome of one site's visit in a staged phase.
enum SiteVisit { kVisitKept = 0, kVisitQuiet = 1, kVisitChanged = 2 };

// The local update of one site in a staged phase (compile-time P = 2 * NQC), from
// one load of its neighbourhood.  A slice class all of whose slices see the same
// neighbourhood -- own bit, neighbour bits and both Trotter partners equal across
// the class -- has one energy sum for all of them; when that sum settles the class
// (flip all, or reject all, see settled_x) it is applied without random numbers,
// which is exactly what the per-slice update would do.  Classes are taken in the
// replica's parity order; from the first class left unsettled on, every slice
// draws its uniform and is decided on its own (update_fixed).  A flip of a whole
// class keeps every word straight on the other class, so the test of the second
// class uses the neighbour words loaded once.
//
// Returns kVisitQuiet when every slice of both classes is a rejection whatever its
// uniform and its sum s = e + t cannot fall as J-perp grows (t = 2 J-perp or 0, not
// -2 J-perp): either the site's own and neighbour world-lines are straight and the
// common sum s = e + 2 J-perp rejects, or every slice, decided on its own, had
// s >= smin and no slice had both Trotter partners opposite to it.  Such a site
// rejects again at every later visit for which nothing in its neighbourhood has
// changed, J-perp has not decreased and beta has not decreased (each s only grows
// with J-perp, and fl(s * -2 beta) only falls as s and beta grow).  kVisitChanged
// when the site's word changed.
//
// Lanes: `part` of the `nparts` lanes of part_mask that visit the site together
// (SPLIT: the lane pair, one 32-bit half each; COMPACT: a group of adjacent lanes
// that share its Philox blocks, update_part); otherwise one lane (part 0).
template <typename W, int MAXDEG, int NQC, typename KS, bool SPLIT, bool COMPACT>
__device__ __forceinline__ int site_visit(const Item& it, const KS& ks, W* rw, int i, uint32_t rep, uint32_t first,
                                          float jp, uint32_t sweep, float m2beta, float m2blog2e, float smin, int part,
                                          int nparts, unsigned part_mask, bool& bad, unsigned long long& nacc) {
    static_assert(NQC > 0, "staged phases need a compile-time slice count");
    using CMk = ClassMasks<W, NQC>;
    constexpr int P = 2 * NQC;
    const W w0 = rw[i];
    W wi = w0;
    W d[MAXDEG];
    float J[MAXDEG];
    load_site<W, MAXDEG>(rw, i, it.n, it.maxdeg, it.nbr, it.cpl, wi, d, J, bad);
    const float h = site_field(it, i);
    int qq = 0;
    if (((wi ^ (wi >> 2)) & (CMk::IN0 | (CMk::IN0 << 1))) == 0) {   // own world-line straight per class
        W full = wi ^ (wi >> 1);
#pragma unroll
        for (int m = 0; m < MAXDEG; ++m) full |= d[m] ^ (d[m] >> 1);
        if ((full & (CMk::MASK >> 1)) == 0) {
            // Every slice sees the same neighbourhood (own and neighbour world-lines
            // straight): one sum e serves both classes -- the second class has the same
            // own and neighbour bits, and Trotter partners that agree with it (t = jp + jp)
            // unless the first class flipped (t = -jp + -jp).
            float e = flip_sign(h, bit_to_sign<W>(wi, 0));
#pragma unroll
            for (int m = 0; m < MAXDEG; ++m) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], 0)));
            const float sum = __fadd_rn(e, __fadd_rn(jp, jp));
            if (sum >= 0.0f) {
                if (__fmul_rn(sum, m2beta) <= settled_x()) return kVisitQuiet;   // both classes reject
                // neither class settled: every slice on its own
            } else {
                const W fl = CMk::CM0 << first;
                const float mjp = flip_sign(jp, 0x80000000u);
                const float sum2 = __fadd_rn(e, __fadd_rn(mjp, mjp));
                W fl2 = 0;
                qq = 2;
                if (sum2 < 0.0f) fl2 = CMk::CM0 << (first ^ 1u);
                else if (!(__fmul_rn(sum2, m2beta) <= settled_x())) qq = 1;
                wi ^= fl | fl2;
#pragma unroll
                for (int m = 0; m < MAXDEG; ++m) d[m] ^= fl | fl2;
                if (part == 0)
                    nacc += sizeof(W) == 8 ? __popcll((unsigned long long)(fl | fl2)) : __popc((uint32_t)(fl | fl2));
            }
        } else {
            W nbx = 0;
#pragma unroll
            for (int m = 0; m < MAXDEG; ++m) nbx |= d[m] ^ (d[m] >> 2);
            for (; qq < 2; ++qq) {
                const int q = qq ^ (int)first;
                if (nbx & (CMk::IN0 << q)) break;
                const W up = ((wi << 1) | (wi >> (P - 1))) & CMk::MASK;   // bit k = s^{k-1}
                const W dn = ((wi >> 1) | (wi << (P - 1))) & CMk::MASK;   // bit k = s^{k+1}
                float e = flip_sign(h, bit_to_sign<W>(wi, q));
#pragma unroll
                for (int m = 0; m < MAXDEG; ++m) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], q)));
                const float t =
                    __fadd_rn(flip_sign(jp, bit_to_sign<W>(wi ^ up, q)), flip_sign(jp, bit_to_sign<W>(wi ^ dn, q)));
                const float sum = __fadd_rn(e, t);
                W fl;
                if (sum < 0.0f) fl = CMk::CM0 << q;
                else if (__fmul_rn(sum, m2beta) <= settled_x()) fl = 0;
                else break;
                wi ^= fl;
#pragma unroll
                for (int m = 0; m < MAXDEG; ++m) d[m] ^= fl;
                if (part == 0)
                    nacc += sizeof(W) == 8 ? __popcll((unsigned long long)fl) : __popc((uint32_t)fl);
            }
        }
    }
    bool calm = qq == 0;   // both classes decided slice by slice (none settled above)
#pragma unroll 1
    for (; qq < 2; ++qq) {
        const int q = qq ^ (int)first;
        W fl;
        if constexpr (SPLIT) {
            const W own = update_fixed_half64<MAXDEG, KS>(wi, d, J, h, jp, q, part, (uint32_t)i, sweep, rep, ks,
                                                         m2beta, m2blog2e, smin, calm);
            nacc += __popcll((unsigned long long)own);
            fl = own | (W)__shfl_xor_sync(part_mask, (unsigned long long)own, 1);
        } else if constexpr (COMPACT) {
            fl = update_part<NQC, MAXDEG, W, KS>(wi, d, J, h, jp, q, (uint32_t)i, sweep, rep, ks, m2beta, m2blog2e,
                                                 smin, calm, part, nparts);
            nacc += sizeof(W) == 8 ? __popcll((unsigned long long)fl) : __popc((uint32_t)fl);
            for (int off = 1; off < nparts; off <<= 1) fl |= (W)__shfl_xor_sync(part_mask, fl, off);
        } else {
            fl = update_fixed<NQC, MAXDEG, W, KS>(wi, d, J, h, jp, q, (uint32_t)i, sweep, rep, ks, m2beta, m2blog2e,
                                                  smin, calm);
            nacc += sizeof(W) == 8 ? __popcll((unsigned long long)fl) : __popc((uint32_t)fl);
        }
        // the neighbours are unchanged in this phase: only the spin's own bits move
        wi ^= fl;
#pragma unroll
        for (int m = 0; m < MAXDEG; ++m) d[m] ^= fl;
    }
    if (nparts > 1) calm = __all_sync(part_mask, calm);
    if (wi == w0) return calm ? kVisitQuiet : kVisitKept;
    if (part == 0) rw[i] = wi;
    return kVisitChanged;
}

// The smallest FP32 s >= 0 with fl(s * m2beta) <= settled_x() (m2beta = -2 beta < 0;
// the product falls as s grows, so s >= the result is exactly that test); +inf when
// m2beta >= 0.  Bisection over the bit patterns of the non-negative floats.
__device__ __forceinline__ float settle_threshold(float m2beta) {
    if (!(m2beta < 0.0f)) return __uint_as_float(0x7f800000u);
    uint32_t lo = 0u, hi = 0x7f800000u;   // fails at lo (+0), holds at hi (+inf)
#pragma unroll 1
    while (hi - lo > 1u) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (__fmul_rn(__uint_as_float(mid), m2beta) <= settled_x()) hi = mid;
        else lo = mid;
    }
    return __uint_as_float(hi);
}

// Quiet bits (one per device slot and replica, in shared memory after the parity
// words): bit i set = site i was quiet at its last visit (site_visit) and nothing
// in its neighbourhood has changed since.  A staged phase visits only the sites
// whose bit is clear; any change of a word clears the bits of the site and of its
// neighbours.
__host__ __device__ inline int quiet_words(int n) { return (n + 31) >> 5; }

__device__ __forceinline__ void quiet_set(uint32_t* quiet, int i) { atomicOr(quiet + (i >> 5), 1u << (i & 31)); }

__device__ __forceinline__ void quiet_clear(uint32_t* quiet, int i) { atomicAnd(quiet + (i >> 5), ~(1u << (i & 31))); }

// After site i of one replica changed: its neighbours are no longer known to be quiet
// (its own bit is clear: only sites with a clear bit are visited, and a world-line
// move clears it itself).
template <int MAXDEG>
__device__ __forceinline__ void quiet_clear_neighbours(const Item& it, uint32_t* quiet, int i) {
#pragma unroll
    for (int m = 0; m < MAXDEG; ++m) {
        if (m < it.maxdeg) {
            const int j = __ldg(it.nbr + (int64_t)m * it.n + i);
            if ((unsigned)j < (unsigned)it.n) quiet_clear(quiet, j);
        }
    }
}

// The per-slice local update of one site from slice class qq0 on (all classes when
// qq0 = 0): every slice draws its uniform and is decided on its own.
template <typename W, int MAXDEG, int NQC, typename KS, bool SPLIT>
__device__ __forceinline__ void site_update(const Item& it, const KS& ks, W* rw, int i, uint32_t rep, int qq0,
                                            uint32_t first, int nclass_q, float jp, uint32_t sweep, float m2beta,
                                            float m2blog2e, W mask, int half, unsigned pair_mask, bool& bad,
                                            unsigned long long& nacc) {
    const int P = it.P;
    W wi = rw[i];
    W d[MAXDEG];
    float J[MAXDEG];
    load_site<W, MAXDEG>(rw, i, it.n, it.maxdeg, it.nbr, it.cpl, wi, d, J, bad);
    const float h = site_field(it, i);
    for (int qq = qq0; qq < nclass_q; ++qq) {
        const int q = nclass_q == 2 ? (qq ^ (int)first) : qq;
        W fl;
        if constexpr (SPLIT) {
            bool calm = false;   // not used here
            const W own = update_fixed_half64<MAXDEG, KS>(wi, d, J, h, jp, q, half, (uint32_t)i, sweep, rep, ks,
                                                         m2beta, m2blog2e, 0.0f, calm);
            nacc += __popcll((unsigned long long)own);
            fl = own | (W)__shfl_xor_sync(pair_mask, (unsigned long long)own, 1);
        } else if constexpr (NQC > 0) {
            bool calm = false;   // not used here
            fl = update_fixed<NQC, MAXDEG, W, KS>(wi, d, J, h, jp, q, (uint32_t)i, sweep, rep, ks, m2beta, m2blog2e,
                                                  0.0f, calm);
        } else {
            W dl, dr;
            trotter_diffs<W>(wi, P, mask, dl, dr);
            fl = 0;
            const int nq = slice_count(P, q);
            for (int mb = 0; mb * 4 < nq; ++mb) {
                const pq_u32x4 rnd = pq_philox_ks(pq_u32x4{(uint32_t)i, sweep, rep, (uint32_t)((q << 16) | mb)}, ks);
                const uint32_t rw4[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const int mm = mb * 4 + jj;
                    if (mm < nq) {
                        const int k = slice_of(P, q, mm);
                        float e = flip_sign(h, bit_to_sign<W>(wi, k));
#pragma unroll
                        for (int m = 0; m < MAXDEG; ++m)
                            if (m < it.maxdeg) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], k)));
                        const float t = __fadd_rn(flip_sign(jp, bit_to_sign<W>(dl, k)),
                                                  flip_sign(jp, bit_to_sign<W>(dr, k)));
                        const bool acc = decide(__fadd_rn(e, t), pq_u01(rw4[jj]), m2beta, m2blog2e);
                        fl |= (W)acc << k;
                    }
                }
            }
        }
        // the neighbours are unchanged in this phase: only the spin's own bits move
        wi ^= fl;
#pragma unroll
        for (int m = 0; m < MAXDEG; ++m) d[m] ^= fl;
        if constexpr (!SPLIT) nacc += sizeof(W) == 8 ? __popcll((unsigned long long)fl) : __popc((uint32_t)fl);
    }
    if (half == 0) rw[i] = wi;
}

// One queued site of replica r in phase p: visit it (lane `part` of the `nparts`
// lanes of part_mask that visit it, site_visit), then record what the visit showed
// in the quiet bits.  fresh: the sweep visits every site and rewrites its
// bit (the bits read before it are not trusted); otherwise the site's bit is clear.
template <typename W, int MAXDEG, int NQC, typename KS, bool SPLIT, bool COMPACT>
__device__ __forceinline__ void visit_queued(const Item& it, const KS& ks, W* sw, uint32_t* quiet, int nwq,
                                             const uint32_t* parity, int p, int i, int r, bool fresh, float jp,
                                             uint32_t sweep, float m2beta, float m2blog2e, float smin, int part,
                                             int nparts, unsigned part_mask, bool& bad, unsigned long long& nacc) {
    const int v = site_visit<W, MAXDEG, NQC, KS, SPLIT, COMPACT>(it, ks, sw + r * it.n, i, it.replica0 + r,
                                                                 (parity[r] >> p) & 1u, jp, sweep, m2beta, m2blog2e,
                                                                 smin, part, nparts, part_mask, bad, nacc);
    if (part != 0) return;
    uint32_t* qr = quiet + r * nwq;
    if (v == kVisitQuiet) {
        quiet_set(qr, i);
    } else {
        if (fresh) quiet_clear(qr, i);
        if (v == kVisitChanged) quiet_clear_neighbours<MAXDEG>(it, qr, i);
    }
}

// Lanes that may share one visited site: the Philox blocks of a slice class (4
// slices each), rounded up to a power of two, at most 4.
template <int NQC>
__host__ __device__ constexpr int kVisitLanes() {
    return (NQC + 3) / 4 >= 3 ? 4 : ((NQC + 3) / 4 >= 2 ? 2 : 1);
}

// Queue of the sites a phase visits, per group: kQueuePerThread entries per thread
// of the group in shared memory, and two phase counters (used alternately).
constexpr int kQueuePerThread = 2;

struct SiteQueue {
    uint32_t* slots;   // cap entries
    int* count;        // [2]
    int cap;           // entries of slots
};

// Queue entries that hold every site of a phase (rounded up to whole 32-site words per
// replica), at least kQueuePerThread per thread: what the single-instance kernel
// takes when its shared memory allows, so that its word scan runs a phase in one chunk.
__host__ __device__ inline int whole_phase_queue(int threads, int rpc, int stride) {
    const int64_t phase = (int64_t)rpc * (((int64_t)stride + 31) / 32 + 1) * 32;
    const int64_t per_thread = (int64_t)kQueuePerThread * threads;
    return (int)(phase > per_thread ? phase : per_thread);
}

// The quiet bits of an item: after its parity words (item_smem_bytes).
__device__ __forceinline__ uint32_t* item_quiet(uint32_t* parity, int nrep) {
    return parity + ((((size_t)nrep * 4 + 15) & ~(size_t)15) >> 2);
}

// Anneal one item through its schedule.  sw: shared memory holding the item's
// nrep x n words (staged by the caller); order: nrep x kMaxClasses bytes;
// parity: nrep words, followed by the quiet bits; q: the group's queue.  Counts
// accepted local flips into nacc and out-of-range indices into bad.
//
// Compile-time P (NQC > 0): each phase runs in two stages.  The scan appends
// (warp-aggregated) the phase's sites whose quiet bit is clear to the group's queue
// as (slot, replica); after a group barrier, the visit stage runs site_visit on the
// queued sites, one per thread (lane pair), so the per-slice work fills whole warps.
// A quiet site is skipped: site_visit would reject both of its classes without
// drawing a uniform, so skipping it changes no result.  The first sweep of the item,
// and of a schedule step whose J-perp or beta is below the previous step's, visits
// every site and rewrites its bit.  Sites of one phase share no coupling, so which
// thread takes a site, and in which chunk, does not change any result.
//
// The single-instance kernel (INLINE) scans a 32-site word of quiet bits per lane
// into a queue that holds a whole phase (in chunks of words when it cannot); the
// batched kernel's items walk their sites one per lane, and a site that finds the
// small per-group queue full is visited at once by its own thread.
//
// SPLIT (64-bit words with P = 64 only): two adjacent lanes share each site, one
// 32-bit half of the world-line each, and exchange their flips after every slice
// class; the sweep's serial work per lane halves, its result is unchanged.
template <typename W, int MAXDEG, int NQC, bool INLINE, typename KS, bool SPLIT = false, bool STAGED = true>
__device__ __forceinline__ void run_item_body(const Item& it, const KS& ks, W* sw, uint8_t* order, uint32_t* parity,
                                              const SiteQueue& q, const Group& g, bool& bad,
                                              unsigned long long& nacc);

// Staged phases run for every compile-time P: only they skip quiet sites (measured
// on GB300: the 256-instance batched workload 2.35e11 -> 3.54e11 updates/s against
// per-site phases for items with under two sites per lane).  Run-time P takes
// per-site phases.
__host__ __device__ constexpr bool staged_phase(int nqc) { return nqc > 0; }

// The single-instance kernel inlines the item loop (INLINE: visits with the
// unrolled update_fixed); the batched kernel calls one out-of-line copy per variant,
// so each variant keeps its own register budget, and visits with the compact
// update_part (its many variants share the instruction cache; measured on GB300 the
// 256-instance workload ran 4.0-4.3e11 updates/s with it against 3.5e11, while the
// single-instance 80x80 kernel ran 202 ms per anneal unrolled against 228-370 ms).
template <typename W, int MAXDEG, int NQC, bool STAGED>
__device__ __forceinline__ void run_item(const Item& it, const PhiloxKeyTable& keys, W* sw, uint8_t* order,
                                         uint32_t* parity, const SiteQueue& q, const Group& g, bool& bad,
                                         unsigned long long& nacc) {
    run_item_body<W, MAXDEG, NQC, true, PhiloxKeysTab, false, STAGED>(it, PhiloxKeysTab{keys}, sw, order, parity, q,
                                                                      g, bad, nacc);
}

template <typename W, int MAXDEG, int NQC, bool SPLIT = false, bool STAGED = true>
__device__ __noinline__ void run_item_call(const Item& it, W* sw, uint8_t* order, uint32_t* parity,
                                           const SiteQueue& q, const Group& g, bool& bad, unsigned long long& nacc) {
    run_item_body<W, MAXDEG, NQC, false, PhiloxKeysReg, SPLIT, STAGED>(it, PhiloxKeysReg{it.key0, it.key1}, sw,
                                                                       order, parity, q, g, bad, nacc);
}

template <typename W, int MAXDEG, int NQC, bool INLINE, typename KS, bool SPLIT, bool STAGED>
__device__ __forceinline__ void run_item_body(const Item& it, const KS& ks, W* sw, uint8_t* order, uint32_t* parity,
                                              const SiteQueue& q, const Group& g, bool& bad,
                                              unsigned long long& nacc) {
    const int n = it.n, P = it.P, S = it.stride, nrep = it.nrep;
    const W mask = full_mask<W>(P);
    const int nclass_q = P == 1 ? 1 : ((P & 1) ? 3 : 2);
    static_assert(!SPLIT || (sizeof(W) == 8 && NQC == 32), "lane pairs split 64-slice world-lines only");
    // the batched kernel's out-of-line copies visit with update_part (compact code, lanes shared)
    constexpr bool COMPACT = !INLINE && !SPLIT;
    // site walk of the local updates: one lane per site, or a lane pair per site
    const int site_tid = SPLIT ? g.tid >> 1 : g.tid;
    const int site_nthr = SPLIT ? g.nthr >> 1 : g.nthr;
    const int half = SPLIT ? (g.tid & 1) : 0;
    const unsigned pair_mask = 3u << ((g.tid & 31) & ~1);
    const uint32_t lane = (uint32_t)(g.tid & 31);
    // queue rank below this site: lanes below this lane (below the pair's first lane for SPLIT)
    const uint32_t lanes_below = (1u << (SPLIT ? (lane & ~1u) : lane)) - 1u;
    const int qcap = q.cap;
    uint32_t phase = 0;   // running phase count: picks the phase's queue counter
    uint32_t* const quiet = item_quiet(parity, nrep);
    const int nwq = quiet_words(n);
    if (NQC > 0 && g.tid == 0) { q.count[0] = 0; q.count[1] = 0; }
    for (int gs = 0; gs < it.nsched; ++gs) {
        const float jp = P == 1 ? 0.0f : __ldg(it.jperp + gs);
        const float beta = it.betas ? __ldg(it.betas + gs) : it.beta;
        const float m2beta = __fmul_rn(-2.0f, beta);                          // exact
        const float m2blog2e = __fmul_rn(m2beta, 1.44269502162933349609375f);  // guard-band argument scale
        const float smin = NQC > 0 && STAGED ? settle_threshold(m2beta) : 0.0f;
        // quiet bits hold while J-perp and beta do not decrease (site_visit): the first
        // sweep of the item, or of a step where either decreased, visits every site
        // and rewrites its bit
        bool renew = true;
        if (gs > 0) {
            const float jp_prev = P == 1 ? 0.0f : __ldg(it.jperp + gs - 1);
            const float beta_prev = it.betas ? __ldg(it.betas + gs - 1) : it.beta;
            renew = !(jp >= jp_prev && beta >= beta_prev && beta_prev > 0.0f);
        }
        for (int step = 0; step < it.mcsteps; ++step) {
            const bool fresh = renew && step == 0;
            const uint32_t sweep = (uint32_t)(it.sweep_base + (int64_t)gs * it.mcsteps + step);
            if (g.tid < nrep)
                class_order<KS>(it.nclass, it.order_mode, ks, sweep, it.replica0 + g.tid,
                                order + g.tid * kMaxClasses, parity + g.tid);
            group_sync(g);
            // Phase = one update class.  Its spins share no coupling, so each thread takes
            // its spins one at a time through every slice class (in the replica's parity
            // order): the same result as slice class by slice class over all spins, with
            // one barrier and one load of the neighbourhood per spin and class.
            // The group's threads walk the phase's sites replica after replica, each
            // replica over the real size of the class it visits in this phase.
            for (int p = 0; p < it.nclass; ++p) {
                int rl = 0, s = site_tid;
                int cls = order[p], cs = it.csize[cls];
                while (s >= cs) {
                    s -= cs;
                    if (++rl == nrep) break;
                    cls = order[rl * kMaxClasses + p];
                    cs = it.csize[cls];
                }
                if constexpr (NQC > 0 && STAGED && INLINE) {
                    // scan by words (single-instance kernel): each lane takes one 32-site
                    // word of a replica's class range, and the warp queues the word's sites
                    // whose quiet bit is clear.  The phase's words go in chunks the queue
                    // can hold whole (one chunk when it holds every site of a phase), each
                    // chunk scanned, then visited: sites of one phase are independent.
                    int nwords = 0;
                    for (int r = 0; r < nrep; ++r) {
                        const int c2 = order[r * kMaxClasses + p], b2 = c2 * S, n2 = it.csize[c2];
                        nwords += n2 > 0 ? ((b2 + n2 - 1) >> 5) - (b2 >> 5) + 1 : 0;
                    }
                    const int chunk = qcap >> 5;
                    for (int c0 = 0; c0 < nwords; c0 += chunk) {
                        int* cnt = q.count + (phase & 1u);
                        const int c1 = min(nwords, c0 + chunk);
                        // this thread's first word of the chunk: replica wr, word wo of its range
                        int wr = 0, wo = c0 + site_tid;
                        int wb = order[p] * S, wcs = it.csize[order[p]];
                        int wn = wcs > 0 ? ((wb + wcs - 1) >> 5) - (wb >> 5) + 1 : 0;
                        int wi = c0 + site_tid;   // flattened word index
                        while (wo >= wn) {
                            wo -= wn;
                            if (++wr == nrep) break;
                            const int c2 = order[wr * kMaxClasses + p];
                            wb = c2 * S;
                            wcs = it.csize[c2];
                            wn = wcs > 0 ? ((wb + wcs - 1) >> 5) - (wb >> 5) + 1 : 0;
                        }
                        for (;;) {
                            const bool active = wi < c1;
                            if (!__any_sync(0xffffffffu, active)) break;
                            uint32_t bits = 0;
                            int w = 0;
                            if (active) {
                                w = (wb >> 5) + wo;
                                const int lo = wb - 32 * w;          // > 0 only in the range's first word
                                const int hi = wb + wcs - 32 * w;    // < 32 only in its last word (>= 1)
                                uint32_t m = lo > 0 ? (0xFFFFFFFFu << lo) : 0xFFFFFFFFu;
                                if (hi < 32) m &= (1u << hi) - 1u;
                                bits = (fresh ? 0xFFFFFFFFu : ~quiet[wr * nwq + w]) & m;
                            }
                            const int c = __popc(bits);
                            int incl = c;
#pragma unroll
                            for (int off = 1; off < 32; off <<= 1) {
                                const int t = __shfl_up_sync(0xffffffffu, incl, off);
                                if ((int)lane >= off) incl += t;
                            }
                            const int tot = __shfl_sync(0xffffffffu, incl, 31);
                            int base = 0;
                            if (lane == 31 && tot) base = atomicAdd(cnt, tot);
                            base = __shfl_sync(0xffffffffu, base, 31);
                            int pos = base + incl - c;   // < qcap: a chunk holds at most qcap sites
                            const uint32_t rtag = (uint32_t)wr << 22;
                            while (bits) {
                                const int bpos = __ffs(bits) - 1;
                                bits &= bits - 1u;
                                q.slots[pos++] = (uint32_t)(32 * w + bpos) | rtag;
                            }
                            if (active) {
                                wi += site_nthr;
                                wo += site_nthr;
                                while (wo >= wn) {
                                    wo -= wn;
                                    if (++wr == nrep) break;
                                    const int c2 = order[wr * kMaxClasses + p];
                                    wb = c2 * S;
                                    wcs = it.csize[c2];
                                    wn = wcs > 0 ? ((wb + wcs - 1) >> 5) - (wb >> 5) + 1 : 0;
                                }
                            }
                        }
                        // the other counter's last reader finished before this chunk began
                        if (g.tid == 0) q.count[(phase + 1u) & 1u] = 0;
                        group_sync(g);
                        // visits of the queued sites, one per thread
                        const int nq = *cnt;
                        for (int e = site_tid; e < nq; e += site_nthr) {
                            const uint32_t en = q.slots[e];
                            visit_queued<W, MAXDEG, NQC, KS, SPLIT, false>(
                                it, ks, sw, quiet, nwq, parity, p, (int)(en & 0x3FFFFFu), (int)((en >> 22) & 0xFFu),
                                fresh, jp, sweep, m2beta, m2blog2e, smin, 0, 1, 1u << lane, bad, nacc);
                        }
                        ++phase;
                        if (c1 < nwords) group_sync(g);   // the next chunk reuses the queue
                    }
                } else if constexpr (NQC > 0 && STAGED) {
                    int* cnt = q.count + (phase & 1u);
                    // scan: queue the sites whose quiet bit is clear
                    for (;;) {
                        const bool active = rl < nrep;
                        if (!__any_sync(0xffffffffu, active)) break;
                        bool pend = false;
                        uint32_t entry = 0;
                        int site_i = 0, site_r = 0;
                        if (active) {
                            site_i = cls * S + s;
                            site_r = rl;
                            pend = fresh || ((quiet[rl * nwq + (site_i >> 5)] >> (site_i & 31)) & 1u) == 0u;
                            entry = (uint32_t)site_i | ((uint32_t)rl << 22);
                            s += site_nthr;
                            while (s >= cs) {
                                s -= cs;
                                if (++rl == nrep) break;
                                cls = order[rl * kMaxClasses + p];
                                cs = it.csize[cls];
                            }
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, pend && half == 0);
                        if (bal) {
                            const int leader = __ffs(bal) - 1;
                            int base = 0;
                            if ((int)lane == leader) base = atomicAdd(cnt, __popc(bal));
                            base = __shfl_sync(0xffffffffu, base, leader);
                            const int slot = base + __popc(bal & lanes_below);
                            if (pend) {
                                if (slot < qcap) {
                                    if (half == 0) q.slots[slot] = entry;
                                } else {   // queue full: visit the site now
                                    visit_queued<W, MAXDEG, NQC, KS, SPLIT, COMPACT>(
                                        it, ks, sw, quiet, nwq, parity, p, site_i, site_r, fresh, jp, sweep, m2beta,
                                        m2blog2e, smin, half, SPLIT ? 2 : 1, SPLIT ? pair_mask : (1u << lane), bad,
                                        nacc);
                                }
                            }
                        }
                    }
                    // the other counter's last reader finished before this phase began
                    if (g.tid == 0) q.count[(phase + 1u) & 1u] = 0;
                    group_sync(g);
                    // visits of the queued sites, one per thread (lane pair); with COMPACT
                    // visits a short queue gives each site up to kVisitLanes adjacent lanes,
                    // which share its Philox blocks
                    const int nq = min(*cnt, qcap);
                    int nparts = 1;
                    if constexpr (COMPACT) {
                        while (nparts < kVisitLanes<NQC>() && nq * 2 * nparts <= site_nthr) nparts <<= 1;
                    }
                    const int part = SPLIT ? half : (site_tid & (nparts - 1));
                    const unsigned part_mask =
                        SPLIT ? pair_mask : ((0xFFFFFFFFu >> (32 - nparts)) << ((int)lane & ~(nparts - 1)));
                    const int groups = site_nthr / nparts;
                    for (int e = site_tid / nparts; e < nq; e += groups) {
                        const uint32_t en = q.slots[e];
                        visit_queued<W, MAXDEG, NQC, KS, SPLIT, COMPACT>(
                            it, ks, sw, quiet, nwq, parity, p, (int)(en & 0x3FFFFFu), (int)((en >> 22) & 0xFFu), fresh,
                            jp, sweep, m2beta, m2blog2e, smin, part, SPLIT ? 2 : nparts, part_mask, bad, nacc);
                    }
                    ++phase;
                } else {
                    for (; rl < nrep;) {
                        const uint32_t first = nclass_q == 2 ? (parity[rl] >> p) & 1u : 0u;
                        site_update<W, MAXDEG, NQC, KS, SPLIT>(it, ks, sw + rl * n, cls * S + s, it.replica0 + rl, 0,
                                                               first, nclass_q, jp, sweep, m2beta, m2blog2e, mask,
                                                               half, pair_mask, bad, nacc);
                        s += site_nthr;
                        while (s >= cs) {
                            s -= cs;
                            if (++rl == nrep) break;
                            cls = order[rl * kMaxClasses + p];
                            cs = it.csize[cls];
                        }
                    }
                }
                group_sync(g);
            }
        }
        // world-line moves: flip spin i in every slice at once, classes in order
        for (int gm = 0; gm < it.global_moves; ++gm) {
            const uint32_t sweep = (uint32_t)(it.sweep_base + (int64_t)gs * it.mcsteps + it.mcsteps - 1);
            for (int cls = 0; cls < it.nclass; ++cls) {
                const int csz = it.csize[cls];
                if (csz <= 0) continue;
                int rl = 0, s = g.tid;
                while (s >= csz) { s -= csz; ++rl; }
                for (; rl < nrep;) {
                    {
                        const int i = cls * S + s;
                        W* rw = sw + rl * n;
                        const W wi = rw[i];
                        W d[MAXDEG];
                        float J[MAXDEG];
                        load_site<W, MAXDEG>(rw, i, n, it.maxdeg, it.nbr, it.cpl, wi, d, J, bad);
                        const float h = site_field(it, i);
                        float E = 0.0f;
                        for (int k = 0; k < P; ++k) {
                            float e = flip_sign(h, bit_to_sign<W>(wi, k));
#pragma unroll
                            for (int m = 0; m < MAXDEG; ++m)
                                if (m < it.maxdeg) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], k)));
                            E = __fadd_rn(E, e);
                        }
                        const pq_u32x4 rnd = pq_philox_ks(
                            pq_u32x4{(uint32_t)i, sweep, it.replica0 + rl,
                                     (uint32_t)((1u << 24) | ((uint32_t)gm << 16) | (uint32_t)cls)},
                            ks);
                        if (decide(E, pq_u01(rnd.x), m2beta, m2blog2e)) {
                            rw[i] = wi ^ mask;
                            if constexpr (NQC > 0 && STAGED) {
                                quiet_clear(quiet + rl * nwq, i);
                                quiet_clear_neighbours<MAXDEG>(it, quiet + rl * nwq, i);
                            }
                        }
                    }
                    s += g.nthr;
                    while (s >= csz) { s -= csz; ++rl; }
                }
                group_sync(g);
            }
        }
    }
}

// Stage an item's words into shared memory / write them back (group-strided).
template <typename W>
__device__ __forceinline__ void stage_in(const Item& it, W* sw, const Group& g) {
    const W* src = reinterpret_cast<const W*>(it.words);
    for (int t = g.tid; t < it.nrep * it.n; t += g.nthr) sw[t] = src[t];
    group_sync(g);
}

template <typename W>
__device__ __forceinline__ void stage_out(const Item& it, const W* sw, const Group& g) {
    W* dst = reinterpret_cast<W*>(it.words);
    group_sync(g);
    for (int t = g.tid; t < it.nrep * it.n; t += g.nthr) dst[t] = sw[t];
}

// One item's compile-time variant, staged or per-site phases (staged_phase).
template <typename W, int MAXDEG, int NQC, bool SPLIT = false>
__device__ __forceinline__ void run_item_pick(const Item& it, W* sw, uint8_t* order, uint32_t* parity,
                                              const SiteQueue& q, const Group& g, bool& bad,
                                              unsigned long long& nacc) {
    if constexpr (staged_phase(NQC))
        run_item_call<W, MAXDEG, NQC, SPLIT, true>(it, sw, order, parity, q, g, bad, nacc);
    else
        run_item_call<W, MAXDEG, NQC, SPLIT, false>(it, sw, order, parity, q, g, bad, nacc);
}

// Word type / degree / compile-time P dispatch of one item (any degree up to four takes
// the four-coupling variants: the padded terms add +0 and change no decision).
__device__ inline void run_item_any(const Item& it, unsigned char* smem, const SiteQueue& q, const Group& g, bool& bad,
                                    unsigned long long& nacc, int lanes_per_site = 1) {
    // layout of the item's shared memory: words, then order bytes, then parity words
    const size_t wbytes = it.P <= 32 ? 4 : 8;
    const size_t words_bytes = ((size_t)it.nrep * it.n * wbytes + 15) & ~(size_t)15;
    uint8_t* order = smem + words_bytes;
    uint32_t* parity = reinterpret_cast<uint32_t*>(order + (((size_t)it.nrep * kMaxClasses + 15) & ~(size_t)15));
    if (it.P <= 32) {
        uint32_t* sw = reinterpret_cast<uint32_t*>(smem);
        stage_in<uint32_t>(it, sw, g);
        if (it.maxdeg <= 4 && it.P == 20) run_item_pick<uint32_t, 4, 10>(it, sw, order, parity, q, g, bad, nacc);
        else if (it.maxdeg <= 4 && it.P == 16) run_item_pick<uint32_t, 4, 8>(it, sw, order, parity, q, g, bad, nacc);
        else if (it.maxdeg <= 4 && it.P == 32) run_item_pick<uint32_t, 4, 16>(it, sw, order, parity, q, g, bad, nacc);
        else if (it.maxdeg <= 4) run_item_call<uint32_t, 4, 0>(it, sw, order, parity, q, g, bad, nacc);
        else run_item_call<uint32_t, 8, 0>(it, sw, order, parity, q, g, bad, nacc);
        stage_out<uint32_t>(it, sw, g);
    } else {
        uint64_t* sw = reinterpret_cast<uint64_t*>(smem);
        stage_in<uint64_t>(it, sw, g);
        if (it.maxdeg <= 4 && it.P == 64 && lanes_per_site == 2)
            run_item_pick<uint64_t, 4, 32, true>(it, sw, order, parity, q, g, bad, nacc);
        else if (it.maxdeg <= 4 && it.P == 64) run_item_pick<uint64_t, 4, 32>(it, sw, order, parity, q, g, bad, nacc);
        else if (it.maxdeg <= 4) run_item_call<uint64_t, 4, 0>(it, sw, order, parity, q, g, bad, nacc);
        else run_item_call<uint64_t, 8, 0>(it, sw, order, parity, q, g, bad, nacc);
        stage_out<uint64_t>(it, sw, g);
    }
}

// Shared memory one item needs (words + order bytes + parity words + quiet bits), 16-byte aligned.
__host__ __device__ inline size_t item_smem_bytes(int nrep, int n, int P) {
    const size_t wbytes = P <= 32 ? 4 : 8;
    return (((size_t)nrep * n * wbytes + 15) & ~(size_t)15) + (((size_t)nrep * kMaxClasses + 15) & ~(size_t)15) +
           (((size_t)nrep * 4 + 15) & ~(size_t)15) + (((size_t)nrep * quiet_words(n) * 4 + 15) & ~(size_t)15);
}

}  // namespace pq
