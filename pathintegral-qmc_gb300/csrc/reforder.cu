// Reference-order sweeps: the reference's own update order and arithmetic.
//
// One thread walks one replica through the schedule exactly as the Cython loop
// does (reference piqmc/qmc.pyx:93-136, piqmc/qmc.pyx:197-242,
// piqmc/sa.pyx:94-120): same spin order (the caller's permutations), same
// FP32 accumulator rounded after every FP64 term, same FP32 divide, libm-style
// FP64 exp, same uniforms (the caller's libc rand() stream, consumed only when
// the Metropolis test reaches its random branch).
//
// exp parity.  CUDA's exp() and the host libm's exp() are each within about
// one ulp of the true value, so they can differ in the last bit.  Such a
// difference can only change a decision when exp(x) lies within a couple of
// ulps of the uniform q.  Every such "close call" is checked: the kernel looks
// x up in an override table of host-libm values (sorted FP32 bit patterns),
// and records close calls that had no override, so the host can compare them
// with its own exp() and rerun the chunk with new overrides when one differs.
// A run that records no close call is bit-exact whatever the host libm is.
//
// Speed.  FP64 is a narrow pipe on this GPU, so the common path avoids it
// without changing a single decision:
//  * every sparse-sweep term is +-2 x (an FP32 value), exact in FP32, and
//    (float)((double)a + (double)b) equals the FP32 sum a + b for FP32 a, b
//    (double rounding through a format with 53 >= 2*24 + 2 bits is innocuous),
//    so the accumulator runs in FP32 (flag PQ_ACC_FP64 forces the FP64 form for
//    couplings near the FP32 overflow threshold, where 2J would overflow);
//  * the Metropolis test first compares an FP32 exp (max relative error 7.9e-8
//    over every FP32 input in [-87, 0], checked exhaustively) and an FP32
//    uniform (relative error < 2e-7) with a 2e-6 relative guard band; only
//    inside the band -- or for rand() == 0 -- does it evaluate the FP64 test.
#include <math.h>

#include "common.cuh"

namespace {

struct RefRng {
    const int32_t* rands;
    int64_t cap;
    int64_t used;
    bool dead;
};

struct ExpPatch {
    const uint32_t* ov_x;   // sorted FP32 bit patterns
    const double* ov_y;     // host libm exp of those inputs
    int ov_n;
    uint32_t* close_x;      // recorded close calls without an override
    double* close_y;        // the device exp value used for them
    int close_cap;
    int* close_cnt;
};

// Records a close call that had no override: x and the device exp value used.
__device__ __forceinline__ void record_close(const ExpPatch& ep, float xf, double e) {
    if (!ep.close_cnt) return;
    const int slot = atomicAdd(ep.close_cnt, 1);
    if (slot < ep.close_cap) { ep.close_x[slot] = __float_as_uint(xf); ep.close_y[slot] = e; }
}

// exp((double)xf) for the test against q, with the host-libm override for x when the
// two are close.  A close call without an override is recorded -- or, with deferred,
// only flagged there, for a caller that records it once the decision is known to stand.
__device__ __forceinline__ double patched_exp(float xf, double q, const ExpPatch& ep, bool* deferred = nullptr) {
    double e = exp((double)xf);
    const double d = fabs(e - q);
    const bool close = d <= 1e-15 * fmax(e, q) || (q == 0.0 && e < 1e-300);
    if (!close) return e;
    const uint32_t xb = __float_as_uint(xf);
    int lo = 0, hi = ep.ov_n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ep.ov_x[mid] < xb) lo = mid + 1; else hi = mid;
    }
    if (lo < ep.ov_n && ep.ov_x[lo] == xb) return ep.ov_y[lo];
    if (deferred) *deferred = true;
    else record_close(ep, xf, e);
    return e;
}

// Decision of exp(x) > rv / RAND_MAX when it is certain from FP32 values:
// 1 accept, 0 reject, -1 undecided (inside the guard band, rv == 0, x > 0 or NaN).
__device__ __forceinline__ int fp32_decide(float xf, int32_t rv) {
    if (rv <= 0 || !(xf <= 0.0f)) return -1;
    const float ef = pq_expf_neg(xf);
    const float qf = __fmul_rn((float)rv, 4.656612873077392578125e-10f);  // 2^-31; (rv/(2^31-1))(1 - 4.7e-10)
    if (ef > __fmul_rn(qf, 1.000002f)) return 1;
    if (ef < __fmul_rn(qf, 0.999998f)) return 0;
    return -1;
}

// The same decision from a cheaper estimate, for the warp-level kernels: x' = e * rl with
// rl = fl(fl(1 / T) * fl(log2 e)) (set once per temperature) and 2^x' by ex2.approx.
// Against exp((double)fl(e / T)) the estimate errs by under 8e-5 (relative) wherever
// exp > 1e-30: ex2.approx of a once-rounded argument is within 5e-5 of expf_neg there
// (pq_guard_band_probe checks every such FP32 input against that bound; measured
// 3.6e-6), the three extra roundings of the argument add under 2.1e-5 and the
// quotient's own rounding 5.2e-6.  Below that
// both sides are under about 1e-30, far below any nonzero uniform (>= 2^-31).  A 1e-4
// band around the FP32 uniform therefore leaves only decisions that the exact path
// would also find close -- including every close call it records -- to that path.
// 1 accept, 0 reject, -1 undecided (rv == 0, e > 0 or NaN, or inside the band).
__device__ __forceinline__ int quick_decide(float e, float rl, int32_t rv) {
    if (rv <= 0 || !(e <= 0.0f)) return -1;
    const float pf = pq_ex2_approx(__fmul_rn(e, rl));
    const float qf = __fmul_rn((float)rv, 4.656612873077392578125e-10f);  // 2^-31
    if (pf > __fmul_rn(qf, 1.0001f)) return 1;
    if (pf < __fmul_rn(qf, 0.9999f)) return 0;
    return -1;
}

// rl of quick_decide for temperature T, or 0 (quick path off) when T is not a
// normal positive FP32 value.
__device__ __forceinline__ float quick_scale(float temp) {
    if (!(temp >= 1.17549435e-38f && temp <= 3.4e38f)) return 0.0f;
    return __fmul_rn(__frcp_rn(temp), 1.44269502162933349609375f);
}

// The caller's uniform stream read by a warp in chunks of 32 values, the two chunks
// after the current one loaded ahead of use: a block of 32 positions consumes at
// most 32 values, so the values at used .. used + 63 are always in registers.
// Loads go to clamped, always valid addresses; values past the end of the stream
// are never used (the caller stops at cap).
__device__ const int32_t g_no_rands[1] = {0};

struct UniformRing {
    const int32_t* rr;
    int64_t last;       // index of the last value (0 for an empty stream, read from g_no_rands)
    int64_t k;          // chunk index of a
    int32_t a, b, c;    // this lane's values of chunks k, k + 1, k + 2
    __device__ __forceinline__ int32_t load(int64_t kk, int lane) const {
        const int64_t t = kk * 32 + lane;
        return __ldg(rr + (t < last ? t : last));
    }
    __device__ __forceinline__ void init(const int32_t* rr_, int64_t cap_, int lane) {
        rr = cap_ > 0 ? rr_ : g_no_rands;
        last = cap_ > 0 ? cap_ - 1 : 0;
        k = 0;
        a = load(0, lane); b = load(1, lane); c = load(2, lane);
    }
    // Value at stream index u, 32k <= u < 32k + 64 (every lane of the warp calls it).
    __device__ __forceinline__ int32_t get(int64_t u) const {
        const int32_t va = __shfl_sync(0xffffffffu, a, (int)(u & 31));
        const int32_t vb = __shfl_sync(0xffffffffu, b, (int)(u & 31));
        return (u >> 5) == k ? va : vb;
    }
    // The stream has advanced to index used.
    __device__ __forceinline__ void advance(int64_t used, int lane) {
        while ((used >> 5) > k) {
            a = b; b = c; ++k;
            c = load(k + 2, lane);
        }
    }
};

// Barrier of the two warps of a replica's CTA (named barrier 1, 64 threads).
__device__ __forceinline__ void pair_barrier() { asm volatile("bar.sync 1, 64;" ::: "memory"); }

// Metropolis test of reference piqmc/qmc.pyx:130-133 (ge = false) and
// piqmc/sa.pyx:114-117 (ge = true): deterministic accept on ediff > 0 (>= 0),
// otherwise exp((double)(ediff / temp)) > rand() / (double)RAND_MAX.
__device__ __forceinline__ bool ref_accept(float ediff, float temp, bool ge, RefRng& rng,
                                           const ExpPatch& ep, int32_t* status) {
    if (ge ? (ediff >= 0.0f) : (ediff > 0.0f)) return true;
    if (rng.used >= rng.cap) {
        pq_set_status(status, PQ_ERR_RAND_EXHAUSTED);
        rng.dead = true;
        return false;
    }
    const int32_t rv = rng.rands[rng.used++];
    const float xf = __fdiv_rn(ediff, temp);
    const int quick = fp32_decide(xf, rv);
    if (quick >= 0) return quick != 0;
    const double q = (double)rv / 2147483647.0;  // glibc RAND_MAX
    return patched_exp(xf, q, ep) > q;
}

// ediff = (float)((double)ediff + t): the generated C accumulates every FP64
// term into the FP32 variable this way (piqmc/qmc.c:2201, 2233, 2346, 2375).
__device__ __forceinline__ float acc(float ediff, double t) {
    return __double2float_rn(__dadd_rn((double)ediff, t));
}

// The same for a term -2 * s * v with v an FP32 value and s = +-1: the term is
// exact in FP32, and the double-rounded sum equals the FP32 sum (see above).
template <bool FP64>
__device__ __forceinline__ float acc2(float ediff, float s2, float v) {
    if (FP64) return acc(ediff, (double)s2 * (double)v);
    return __fadd_rn(ediff, __fmul_rn(s2, v));
}

// One CTA (one warp) per replica; lane 0 walks the replica.  The replica's
// spins are staged in shared memory when they fit (SMEM), and for MAXNB > 0 the
// neighbour row is read with all its loads issued before the (ordered) sums.
template <bool FP64, int MAXNB, bool SMEM>
__global__ void __launch_bounds__(32) qa_sparse_reforder_kernel(
    int8_t* __restrict__ spins, const int32_t* __restrict__ nb_idx, const float* __restrict__ nb_j, int n, int nperm,
    int maxnb, int P, int R, const float* __restrict__ jperp, int nsched, int mcsteps, float temp,
    const int32_t* __restrict__ perms, const int32_t* __restrict__ rands, int64_t rand_stride,
    int64_t* __restrict__ rand_used, int flags, ExpPatch ep, int32_t* status) {
    extern __shared__ __align__(16) int8_t sh_spins[];
    const int r = blockIdx.x;
    if (r >= R) return;
    int8_t* gs = spins + (int64_t)r * n * P;
    int8_t* s = SMEM ? sh_spins : gs;
    if (SMEM) {
        for (int64_t t = threadIdx.x; t < (int64_t)n * P; t += blockDim.x) sh_spins[t] = gs[t];
        __syncwarp();
    }
    if (threadIdx.x == 0) {
        const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * nperm;
        RefRng rng{rands + (int64_t)r * rand_stride, rand_stride, 0, false};
        bool bad = false;
        for (int g = 0; g < nsched; ++g) {
            const float jpf = jperp[g];
            for (int step = 0; step < mcsteps; ++step) {
                const int32_t* perm = pr + (int64_t)(g * mcsteps + step) * nperm;
                for (int k = 0; k < P; ++k) {
                    // Q1 (reference as shipped): tidx is never assigned, so every
                    // slice couples to slices P-1 and 1 (piqmc/qmc.pyx:115-117).
                    int tl = P - 1, tr = 1;
                    if (flags & PQ_FIX_Q1) { tl = k == 0 ? P - 1 : k - 1; tr = k == P - 1 ? 0 : k + 1; }
                    // Q2 (as shipped): ediff is reset once per slice (piqmc/qmc.pyx:134-135).
                    float ediff = 0.0f;
                    for (int t = 0; t < nperm; ++t) {
                        int i = perm[t];
                        if ((unsigned)i >= (unsigned)n) { bad = true; i = 0; }
                        if (flags & PQ_FIX_Q2) ediff = 0.0f;
                        int8_t* si_p = s + (int64_t)i * P;
                        const float s2 = -2.0f * (float)si_p[k];
                        const int32_t* ni = nb_idx + (int64_t)i * maxnb;
                        const float* nj = nb_j + (int64_t)i * maxnb;
                        if constexpr (MAXNB > 0) {
                            int jj[MAXNB];
                            float vv[MAXNB];
                            int8_t sj[MAXNB];
#pragma unroll
                            for (int m = 0; m < MAXNB; ++m) { jj[m] = __ldg(ni + m); vv[m] = __ldg(nj + m); }
#pragma unroll
                            for (int m = 0; m < MAXNB; ++m) {
                                if ((unsigned)jj[m] >= (unsigned)n) { bad = true; jj[m] = i; }
                                sj[m] = s[(int64_t)jj[m] * P + k];
                            }
#pragma unroll
                            for (int m = 0; m < MAXNB; ++m)
                                ediff = acc2<FP64>(ediff, s2, jj[m] == i ? vv[m] : (sj[m] > 0 ? vv[m] : -vv[m]));
                        } else {
                            for (int m = 0; m < maxnb; ++m) {
                                int j = ni[m];
                                const float jv = nj[m];
                                if (j == i) {
                                    ediff = acc2<FP64>(ediff, s2, jv);
                                } else {
                                    if ((unsigned)j >= (unsigned)n) { bad = true; j = i; }
                                    ediff = acc2<FP64>(ediff, s2, s[(int64_t)j * P + k] > 0 ? jv : -jv);
                                }
                            }
                        }
                        ediff = acc2<FP64>(ediff, s2, si_p[tl] > 0 ? jpf : -jpf);
                        ediff = acc2<FP64>(ediff, s2, si_p[tr] > 0 ? jpf : -jpf);
                        if (ref_accept(ediff, temp, false, rng, ep, status)) si_p[k] = (int8_t)-si_p[k];
                        if (rng.dead) goto done;
                    }
                }
            }
        }
    done:
        if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
        rand_used[r] = (rng.dead || bad) ? -1 : rng.used;
    }
    if (SMEM) {
        __syncwarp();
        for (int64_t t = threadIdx.x; t < (int64_t)n * P; t += blockDim.x) gs[t] = sh_spins[t];
    }
}

// The same sweep with the warp sharing the work (replicas whose spins fit in
// shared memory, maxnb 4 or 5).  The permutation is taken in blocks of 32
// positions, lane l owning position l:
//  * each lane loads its spin's neighbour row and couplings (the permutation entry
//    two blocks ahead, the row one block ahead of its use) and folds
//    the current neighbour spins into signed couplings; a neighbour at an earlier
//    position p of the same block is recorded (its term changes sign if p flips);
//  * the accumulator is a sequential chain (FP32, one rounding per term, carried
//    across spins as the reference carries it).  A round takes every open position:
//    they first negate the terms of neighbours whose flips stand, then all lanes walk
//    them in order computing the chain, taking in-block neighbours that are still
//    undecided as not flipping -- the sum of position l and the number of uniforms
//    consumed before it are kept by lane l;
//  * the walked positions then decide in parallel, each lane with its own uniform
//    (from the next values of the stream) and exactly ref_accept's arithmetic.  The
//    decisions stand up to the first position with an in-block neighbour that
//    flipped in this round; from that position the next round walks again, from
//    the chain value and the uniform count before it (flips are rare at annealing
//    temperatures, so most blocks take one round).  Close calls are recorded only
//    for decisions that stand.
// Flips are written back at the end of the block.  Same results, same uniforms
// consumed and the same close calls (recorded by the deciding lane) as
// qa_sparse_reforder_kernel.
template <bool FP64, int MAXNB>
struct RefBlockIn {
    int i;
    int j[MAXNB];
    float v[MAXNB];
};

// The same sweep with two warps per replica: the fold warp prepares block b + 1 --
// neighbour rows, signed couplings and Trotter terms, records, in-block dependencies --
// while the chain warp resolves block b (the walk, speculation and decisions above),
// one 64-thread named barrier per block.  The fold warp reads spins before block b's
// flips are known, so it also notes, per term, the position in block b of a neighbour
// in the same slice, and per spin its own position in block b; after the barrier the
// chain warp negates exactly the terms whose neighbour (or, for a Trotter term, whose
// spin in the slice the term reads) flipped.  The fold warp owns the spins and the
// position tables and applies each block's flips after the barrier; the flip mask of a
// block travels in a control slot chosen by the block's parity.  Same spins, uniforms
// and close calls as the single-thread kernel qa_sparse_reforder_kernel.
struct SparseBlk {
    int g, step, k, blk;
    __device__ __forceinline__ void next(int nblk, int P, int mcsteps) {
        if (++blk == nblk) {
            blk = 0;
            if (++k == P) {
                k = 0;
                if (++step == mcsteps) { step = 0; ++g; }
            }
        }
    }
};

template <int MAXNB>
struct SparsePairLayout {
    size_t pos_of, rec, dep, pp, ppv, self, ctl, total;
    __host__ __device__ SparsePairLayout(int n, int P) {
        auto a16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        pos_of = a16((size_t)n * P);                 // [2][n]
        rec = pos_of + a16((size_t)2 * n);           // float4 [2][33][2]
        dep = rec + (size_t)2 * 33 * 2 * 16;         // uint32 [2][32]
        pp = dep + (size_t)2 * 32 * 4;               // uint8 [2][32][MAXNB]
        ppv = pp + a16((size_t)2 * 32 * MAXNB);      // uint8 [2][32][MAXNB]
        self = ppv + a16((size_t)2 * 32 * MAXNB);    // uint8 [2][32]
        ctl = self + 64;                             // int [2][2] + bad flag
        total = ctl + 32;
    }
};

template <bool FP64, int MAXNB, bool FIXQ2>
__global__ void __launch_bounds__(64) qa_sparse_reforder_pair_kernel(
    int8_t* __restrict__ spins, const int32_t* __restrict__ nb_idx, const float* __restrict__ nb_j, int n, int nperm,
    int maxnb, int P, int R, const float* __restrict__ jperp, int nsched, int mcsteps, float temp,
    const int32_t* __restrict__ perms, const int32_t* __restrict__ rands, int64_t rand_stride,
    int64_t* __restrict__ rand_used, int flags, ExpPatch ep, int32_t* status) {
    static_assert(MAXNB + 3 <= 8, "record holds MAXNB terms, two Trotter terms and s2");
    extern __shared__ __align__(16) int8_t sh[];
    const SparsePairLayout<MAXNB> L(n, P);
    int8_t* s = sh;                                                            // [n][P]
    uint8_t* pos_of = reinterpret_cast<uint8_t*>(sh + L.pos_of);               // [2][n]
    float4* rec = reinterpret_cast<float4*>(sh + L.rec);                       // [2][33][2]
    uint32_t* mdep = reinterpret_cast<uint32_t*>(sh + L.dep);                  // [2][32]
    uint8_t* mpp = reinterpret_cast<uint8_t*>(sh + L.pp);                      // [2][32][MAXNB]
    uint8_t* mppv = reinterpret_cast<uint8_t*>(sh + L.ppv);                    // [2][32][MAXNB]
    uint8_t* mself = reinterpret_cast<uint8_t*>(sh + L.self);                  // [2][32]
    int* ctl = reinterpret_cast<int*>(sh + L.ctl);                             // [2][2], bad
    const int r = blockIdx.x;
    if (r >= R) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int8_t* gs = spins + (int64_t)r * n * P;
    for (int64_t t = threadIdx.x; t < (int64_t)n * P; t += 64) s[t] = gs[t];
    for (int t = threadIdx.x; t < 2 * n; t += 64) pos_of[t] = 0xFF;
    if (threadIdx.x < 5) ctl[threadIdx.x] = 0;
    __syncthreads();
    const int nblk = (nperm + 31) / 32;
    const int64_t total = (int64_t)nsched * mcsteps * P * nblk;   // blocks in the whole run
    const int64_t nsweeps = (int64_t)nsched * mcsteps;
    auto tl_of = [&](int k) { return (flags & PQ_FIX_Q1) ? (k == 0 ? P - 1 : k - 1) : P - 1; };   // Q1 as shipped:
    auto tr_of = [&](int k) { return (flags & PQ_FIX_Q1) ? (k == P - 1 ? 0 : k + 1) : 1; };       // P - 1 and 1
    bool dead = false;
    int64_t used = 0;
    if (total > 0) {
        if (warp == 1) {
            // ---- fold warp ----
            const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * nperm;
            bool bad = false;
            int64_t q_sweep = 0;
            int q_k = 0, q_blk = 0;
            auto perm_next = [&](bool& has) -> int {
                const int t = q_blk * 32 + lane;
                has = q_sweep < nsweeps && t < nperm;
                const int v = __ldg(pr + (has ? q_sweep * nperm + t : 0));
                if (++q_blk == nblk) {
                    q_blk = 0;
                    if (++q_k == P) { q_k = 0; ++q_sweep; }
                }
                return v;
            };
            auto rows_of = [&](bool has, int i, RefBlockIn<FP64, MAXNB>& in) {
                in.i = -1;
                if (!has) return;
                if ((unsigned)i >= (unsigned)n) { bad = true; i = 0; }
                in.i = i;
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) {
                    in.j[m] = __ldg(nb_idx + (int64_t)i * maxnb + m);
                    in.v[m] = __ldg(nb_j + (int64_t)i * maxnb + m);
                }
            };
            // fold block f (rows in `in`) into buffer fb; the block resolved meanwhile has
            // its positions in pos_of[pb] and slice kp (kp < 0: none)
            auto fold = [&](const SparseBlk& f, const RefBlockIn<FP64, MAXNB>& in, int fb, int pb, int kp) {
                const int nb = min(32, nperm - f.blk * 32);
                const int k = f.k, tl = tl_of(k), tr = tr_of(k);
                const float jpf = jperp[f.g];
                const int i = in.i;
                uint8_t* po = pos_of + (size_t)fb * n;
                const uint8_t* pv = pos_of + (size_t)pb * n;
                if (lane < nb) po[i] = (uint8_t)lane;
                __syncwarp();
                float x[8];
                uint8_t pp[MAXNB], ppv[MAXNB];
                uint32_t dep = 0;
#pragma unroll
                for (int m = 0; m < 8; ++m) x[m] = 0.0f;
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) { pp[m] = 0xFF; ppv[m] = 0xFF; }
                uint8_t self = 0xFF;
                if (lane < nb) {
                    const int8_t* si_p = s + (int64_t)i * P;
#pragma unroll
                    for (int m = 0; m < MAXNB; ++m) {
                        int j = in.j[m];
                        if ((unsigned)j >= (unsigned)n) { bad = true; j = i; }
                        float v = in.v[m];
                        if (j != i) {
                            if (s[(int64_t)j * P + k] <= 0) v = -v;
                            const uint8_t q = po[j];
                            if (q < lane) { pp[m] = q; dep |= 1u << q; }
                            if (kp == k) ppv[m] = pv[j];
                        }
                        x[m] = v;
                    }
                    if (kp >= 0) self = pv[i];
                    x[MAXNB] = si_p[tl] > 0 ? jpf : -jpf;
                    x[MAXNB + 1] = si_p[tr] > 0 ? jpf : -jpf;
                    x[MAXNB + 2] = -2.0f * (float)si_p[k];
                    if constexpr (!FP64) {
#pragma unroll
                        for (int m = 0; m < MAXNB + 2; ++m) x[m] = __fmul_rn(x[MAXNB + 2], x[m]);
                    }
                }
                float4* rc = rec + (size_t)fb * 66;
                rc[2 * lane] = make_float4(x[0], x[1], x[2], x[3]);
                rc[2 * lane + 1] = make_float4(x[4], x[5], x[6], x[7]);
                mdep[fb * 32 + lane] = dep;
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) {
                    mpp[(fb * 32 + lane) * MAXNB + m] = pp[m];
                    mppv[(fb * 32 + lane) * MAXNB + m] = ppv[m];
                }
                mself[fb * 32 + lane] = self;
                __syncwarp();
            };
            RefBlockIn<FP64, MAXNB> cur, nxt;
            bool p_has = false;
            int p_next = perm_next(p_has);   // block 0
            rows_of(p_has, p_next, cur);
            p_next = perm_next(p_has);       // block 1
            rows_of(p_has, p_next, nxt);
            p_next = perm_next(p_has);       // block 2
            SparseBlk held{0, 0, 0, 0};      // the block the chain warp resolves
            fold(held, cur, 0, 1, -1);
            int held_i = cur.i;
            pair_barrier();                  // block 0 is folded
            for (int64_t bb = 0; bb < total; ++bb) {
                SparseBlk f = held;
                f.next(nblk, P, mcsteps);
                int fold_i = -1;
                if (bb + 1 < total) {
                    fold(f, nxt, (int)((bb + 1) & 1), (int)(bb & 1), held.k);
                    fold_i = nxt.i;
                    cur = nxt;
                    rows_of(p_has, p_next, nxt);   // block bb + 2
                    p_next = perm_next(p_has);     // block bb + 3
                }
                pair_barrier();                    // the chain warp has resolved block bb
                const int* c = ctl + 2 * (int)(bb & 1);
                const uint32_t fm = (uint32_t)c[0];   // the decisions that stand, also in a block
                const int nb = min(32, nperm - held.blk * 32);   // the stream ran out in
                if (lane < nb) {
                    if ((fm >> lane) & 1u) s[(int64_t)held_i * P + held.k] = (int8_t)-s[(int64_t)held_i * P + held.k];
                    pos_of[(size_t)(bb & 1) * n + held_i] = 0xFF;
                }
                __syncwarp();
                if (c[1]) break;
                held = f;
                held_i = fold_i;
            }
            bad = __any_sync(0xffffffffu, bad);
            if (lane == 0 && bad) ctl[4] = 1;
        } else {
            // ---- chain warp ----
            const int64_t cap = rand_stride;
            UniformRing ring;
            ring.init(rands + (int64_t)r * rand_stride, cap, lane);
            const float rl = quick_scale(temp);
            SparseBlk cb{0, 0, 0, 0};
            uint32_t fm_prev = 0;
            int k_prev = -1;
            float ediff = 0.0f;
            pair_barrier();                  // block 0 is folded
            for (int64_t bb = 0; bb < total; ++bb) {
                const int buf = (int)(bb & 1);
                const int nb = min(32, nperm - cb.blk * 32);
                const int k = cb.k, tl = tl_of(k), tr = tr_of(k);
                if (cb.blk == 0) ediff = 0.0f;   // Q2 as shipped: reset once per slice (piqmc/qmc.pyx:134-135)
                float4* rc = rec + (size_t)buf * 66;
                const float4 r0 = rc[2 * lane], r1 = rc[2 * lane + 1];
                float x[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
                const uint32_t dep = mdep[buf * 32 + lane];
                uint8_t pp[MAXNB];
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) pp[m] = mpp[(buf * 32 + lane) * MAXNB + m];
                // the previous block's flips, folded into this block's terms
                if (lane < nb && fm_prev) {
                    bool ch = false;
#pragma unroll
                    for (int m = 0; m < MAXNB; ++m) {
                        const uint8_t q = mppv[(buf * 32 + lane) * MAXNB + m];
                        if (q != 0xFF && ((fm_prev >> q) & 1u)) { x[m] = -x[m]; ch = true; }
                    }
                    const uint8_t q = mself[buf * 32 + lane];
                    if (q != 0xFF && ((fm_prev >> q) & 1u)) {
                        if (k_prev == tl) { x[MAXNB] = -x[MAXNB]; ch = true; }
                        if (k_prev == tr) { x[MAXNB + 1] = -x[MAXNB + 1]; ch = true; }
                    }
                    if (ch) {
                        rc[2 * lane] = make_float4(x[0], x[1], x[2], x[3]);
                        rc[2 * lane + 1] = make_float4(x[4], x[5], x[6], x[7]);
                    }
                }
                __syncwarp();
                uint32_t flipmask = 0;
                uint32_t applied = 0;
                int cc = 0;
                float my_e = 0.0f;
                int my_c = 0;
                int l = 0;
                int stop = 0;
                while (l < nb) {
                    const int start = l;
                    if (lane >= start && lane < nb) {
                        const uint32_t nf = dep & flipmask & ~applied;
                        if (nf) {
#pragma unroll
                            for (int m = 0; m < MAXNB; ++m)
                                if (pp[m] != 0xFF && ((nf >> pp[m]) & 1u)) x[m] = -x[m];
                            rc[2 * lane] = make_float4(x[0], x[1], x[2], x[3]);
                            rc[2 * lane + 1] = make_float4(x[4], x[5], x[6], x[7]);
                            applied |= nf;
                        }
                    }
                    __syncwarp();
                    float4 ra = rc[2 * l], rb = rc[2 * l + 1];
                    for (; l < nb; ++l) {
                        const float4 ra_n = rc[2 * l + 2], rb_n = rc[2 * l + 3];
                        const float y[8] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z, rb.w};
                        ra = ra_n;
                        rb = rb_n;
                        if (FIXQ2) ediff = 0.0f;
                        if constexpr (FP64) {
                            const float s2 = y[MAXNB + 2];
#pragma unroll
                            for (int m = 0; m < MAXNB + 2; ++m) ediff = acc2<true>(ediff, s2, y[m]);
                        } else {
#pragma unroll
                            for (int m = 0; m < MAXNB + 2; ++m) ediff = __fadd_rn(ediff, y[m]);
                        }
                        if (lane == l) { my_e = ediff; my_c = cc; }
                        cc += ediff > 0.0f ? 0 : 1;
                    }
                    const int32_t rv = ring.get(used + my_c);
                    bool flip = false, out = false, miss = false;
                    float xf = 0.0f;
                    if (lane >= start && lane < nb) {
                        if (my_e > 0.0f) {
                            flip = true;
                        } else if (used + my_c >= cap) {
                            out = true;
                        } else {
                            const int fast = rl != 0.0f ? quick_decide(my_e, rl, rv) : -1;
                            if (fast >= 0) {
                                flip = fast != 0;
                            } else {
                                xf = __fdiv_rn(my_e, temp);
                                const int quick = fp32_decide(xf, rv);
                                if (quick >= 0) {
                                    flip = quick != 0;
                                } else {
                                    const double q = (double)rv / 2147483647.0;   // glibc RAND_MAX
                                    flip = patched_exp(xf, q, ep, &miss) > q;
                                }
                            }
                        }
                    }
                    const uint32_t fl = __ballot_sync(0xffffffffu, flip);
                    const uint32_t wrong = __ballot_sync(0xffffffffu, lane > start && lane < nb && (dep & fl));
                    const int p = wrong ? __ffs(wrong) - 1 : nb;
                    if (__any_sync(0xffffffffu, out && lane < p)) {
                        if (lane == 0) pq_set_status(status, PQ_ERR_RAND_EXHAUSTED);
                        dead = true;
                        stop = 1;
                        break;
                    }
                    if (miss && lane < p) record_close(ep, xf, exp((double)xf));
                    flipmask |= fl & (p >= 32 ? 0xffffffffu : ((1u << p) - 1u));
                    if (p < nb) {
                        ediff = __shfl_sync(0xffffffffu, my_e, p - 1);
                        cc = __shfl_sync(0xffffffffu, my_c, p);
                        l = p;
                    }
                }
                if (!stop) {
                    used += cc;
                    ring.advance(used, lane);
                }
                if (lane == 0) { ctl[2 * buf] = (int)flipmask; ctl[2 * buf + 1] = stop; }
                pair_barrier();                  // the fold warp has folded block bb + 1
                if (stop) break;
                fm_prev = flipmask;
                k_prev = k;
                cb.next(nblk, P, mcsteps);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool bad = ctl[4] != 0;
        if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
        rand_used[r] = (dead || bad) ? -1 : used;
    }
    for (int64_t t = threadIdx.x; t < (int64_t)n * P; t += 64) gs[t] = s[t];
}

__global__ void qa_dense_reforder_kernel(int8_t* __restrict__ spins, const double* __restrict__ J, int n,
                                         int P, int R, const float* __restrict__ jperp, int nsched,
                                         int mcsteps, float temp, const int32_t* __restrict__ perms,
                                         const int32_t* __restrict__ rands, int64_t rand_stride,
                                         int64_t* __restrict__ rand_used, int flags, ExpPatch ep,
                                         int32_t* status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    int8_t* s = spins + (int64_t)r * n * P;
    const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * n;
    RefRng rng{rands + (int64_t)r * rand_stride, rand_stride, 0, false};
    for (int g = 0; g < nsched; ++g) {
        const double jp = (double)jperp[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int32_t* perm = pr + (int64_t)(g * mcsteps + step) * n;
            for (int k = 0; k < P; ++k) {
                int tl = P - 1, tr = 1;
                if (flags & PQ_FIX_Q1) { tl = k == 0 ? P - 1 : k - 1; tr = k == P - 1 ? 0 : k + 1; }
                float ediff = 0.0f;
                for (int t = 0; t < n; ++t) {
                    const int i = perm[t];
                    if ((unsigned)i >= (unsigned)n) { pq_set_status(status, PQ_ERR_BAD_INDEX); rand_used[r] = -1; return; }
                    if (flags & PQ_FIX_Q2) ediff = 0.0f;
                    int8_t* si_p = s + (int64_t)i * P;
                    const double si = (double)si_p[k];
                    // Upper triangle + diagonal only (piqmc/qmc.pyx:206-219); the
                    // coupling stays FP64 here (it is never stored to a float).
                    for (int j = 0; j < n; ++j) {
                        if (j == i) {
                            ediff = acc(ediff, -2.0 * si * J[(int64_t)i * n + i]);
                        } else {
                            const double jv = i < j ? J[(int64_t)i * n + j] : J[(int64_t)j * n + i];
                            ediff = acc(ediff, -2.0 * si * (jv * (double)s[(int64_t)j * P + k]));
                        }
                    }
                    ediff = acc(ediff, -2.0 * si * (jp * (double)si_p[tl]));
                    ediff = acc(ediff, -2.0 * si * (jp * (double)si_p[tr]));
                    if (ref_accept(ediff, temp, false, rng, ep, status)) si_p[k] = (int8_t)-si_p[k];
                    if (rng.dead) { rand_used[r] = -1; return; }
                }
            }
        }
    }
    rand_used[r] = rng.used;
}

template <bool FP64>
__global__ void sa_sparse_reforder_kernel(int8_t* __restrict__ spins, const int32_t* __restrict__ nb_idx,
                                          const float* __restrict__ nb_j, int n, int maxnb, int R,
                                          const float* __restrict__ temps, int nsched, int mcsteps,
                                          const int32_t* __restrict__ perms,
                                          const int32_t* __restrict__ rands, int64_t rand_stride,
                                          int64_t* __restrict__ rand_used, ExpPatch ep, int32_t* status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    int8_t* s = spins + (int64_t)r * n;
    const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * n;
    RefRng rng{rands + (int64_t)r * rand_stride, rand_stride, 0, false};
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int32_t* perm = pr + (int64_t)(g * mcsteps + step) * n;
            for (int t = 0; t < n; ++t) {
                const int i = perm[t];
                if ((unsigned)i >= (unsigned)n) { pq_set_status(status, PQ_ERR_BAD_INDEX); rand_used[r] = -1; return; }
                float ediff = 0.0f;  // reset per spin (piqmc/sa.pyx:119)
                const float s2 = -2.0f * (float)s[i];
                const int32_t* ni = nb_idx + (int64_t)i * maxnb;
                const float* nj = nb_j + (int64_t)i * maxnb;
                for (int m = 0; m < maxnb; ++m) {
                    const int j = ni[m];
                    const float jv = nj[m];
                    if (j == i) {
                        ediff = acc2<FP64>(ediff, s2, jv);
                    } else {
                        if ((unsigned)j >= (unsigned)n) { pq_set_status(status, PQ_ERR_BAD_INDEX); rand_used[r] = -1; return; }
                        ediff = acc2<FP64>(ediff, s2, s[j] > 0 ? jv : -jv);
                    }
                }
                if (ref_accept(ediff, temp, true, rng, ep, status)) s[i] = (int8_t)-s[i];
                if (rng.dead) { rand_used[r] = -1; return; }
            }
        }
    }
    rand_used[r] = rng.used;
}

// sa.Anneal_dense (reference piqmc/sa.pyx:126-187): one thread per replica walks
// the spins in the supplied order; ediff sums every term of the spin's row in the
// FP32 accumulator (upper triangle for off-diagonal pairs, the diagonal as the
// field, :170-179), is reset per spin (:186), and the deterministic branch
// accepts on ediff > 0 (:181).
__global__ void sa_dense_reforder_kernel(int8_t* __restrict__ spins, const double* __restrict__ J, int n, int R,
                                         const float* __restrict__ temps, int nsched, int mcsteps,
                                         const int32_t* __restrict__ perms, const int32_t* __restrict__ rands,
                                         int64_t rand_stride, int64_t* __restrict__ rand_used, ExpPatch ep,
                                         int32_t* status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    int8_t* s = spins + (int64_t)r * n;
    const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * n;
    RefRng rng{rands + (int64_t)r * rand_stride, rand_stride, 0, false};
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int32_t* perm = pr + (int64_t)(g * mcsteps + step) * n;
            for (int t = 0; t < n; ++t) {
                const int i = perm[t];
                if ((unsigned)i >= (unsigned)n) { pq_set_status(status, PQ_ERR_BAD_INDEX); rand_used[r] = -1; return; }
                const double si = (double)s[i];
                float ediff = 0.0f;
                for (int j = 0; j < n; ++j) {
                    if (j == i) {
                        ediff = acc(ediff, -2.0 * si * J[(int64_t)i * n + i]);
                    } else {
                        const double jv = i < j ? J[(int64_t)i * n + j] : J[(int64_t)j * n + i];
                        ediff = acc(ediff, -2.0 * si * (jv * (double)s[j]));
                    }
                }
                if (ref_accept(ediff, temp, false, rng, ep, status)) s[i] = (int8_t)-s[i];
                if (rng.dead) { rand_used[r] = -1; return; }
            }
        }
    }
    rand_used[r] = rng.used;
}

// sa.Anneal_bipartite (reference piqmc/sa.pyx:411-500): left spins in index
// order, then right spins, every step; for left spin i the accumulator takes,
// for every right spin j, ediff - (2 l_i J_ij r_j + lb_i l_i + rb_j r_j) in FP64
// rounded to FP32 (:466-468), and symmetrically for right spins (:478-480).
// spins: int8 [R][nl + nr] (left then right).
__global__ void sa_bipartite_reforder_kernel(int8_t* __restrict__ spins, const double* __restrict__ J, int nl, int nr,
                                             const double* __restrict__ lbias, const double* __restrict__ rbias,
                                             int R, const float* __restrict__ temps, int nsched, int mcsteps,
                                             const int32_t* __restrict__ rands, int64_t rand_stride,
                                             int64_t* __restrict__ rand_used, ExpPatch ep, int32_t* status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    int8_t* lv = spins + (int64_t)r * (nl + nr);
    int8_t* rv = lv + nl;
    RefRng rng{rands + (int64_t)r * rand_stride, rand_stride, 0, false};
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            for (int i = 0; i < nl; ++i) {
                const double li = (double)lv[i];
                float ediff = 0.0f;
                for (int j = 0; j < nr; ++j) {
                    const double rj = (double)rv[j];
                    const double t = 2.0 * li * J[(int64_t)i * nr + j] * rj + lbias[i] * li + rbias[j] * rj;
                    ediff = __double2float_rn(__dsub_rn((double)ediff, t));
                }
                if (ref_accept(ediff, temp, false, rng, ep, status)) lv[i] = (int8_t)-lv[i];
                if (rng.dead) { rand_used[r] = -1; return; }
            }
            for (int i = 0; i < nr; ++i) {
                const double ri = (double)rv[i];
                float ediff = 0.0f;
                for (int j = 0; j < nl; ++j) {
                    const double lj = (double)lv[j];
                    const double t = 2.0 * ri * J[(int64_t)j * nr + i] * lj + lbias[j] * lj + rbias[i] * ri;
                    ediff = __double2float_rn(__dsub_rn((double)ediff, t));
                }
                if (ref_accept(ediff, temp, false, rng, ep, status)) rv[i] = (int8_t)-rv[i];
                if (rng.dead) { rand_used[r] = -1; return; }
            }
        }
    }
    rand_used[r] = rng.used;
}


// Dense reference-order sweeps (QuantumAnneal_dense, piqmc/qmc.pyx:181-242, and
// sa.Anneal_dense, piqmc/sa.pyx:126-187) by warps: for each position of the
// permutation the lanes form the n terms of the reference's sum (and QA's two Trotter
// terms) in parallel -- every term -2 s_i (J_ij s_j) is exactly +-2 J_ij in FP64 --
// into shared memory, and a warp then walks the accumulator chain through them in the
// reference's order.  For rows whose entries are all zero or normal FP32 values with
// 2J finite the terms are formed in FP32 and the chain is FP32 adds:
// (float)((double)e + t) equals the FP32 sum e + t for FP32 e and t (double rounding
// through 53 >= 2*24 + 2 bits is innocuous); otherwise the chain is the reference's
// FP64 add and rounding, term by term.  The J row a position needs -- J[i][j] for
// j >= i and J[j][i] below the diagonal, the upper triangle the reference reads
// (piqmc/qmc.pyx:206-219) -- is copied into shared memory by cp.async ahead of use,
// and the uniforms come from the register ring.
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__host__ __device__ inline size_t dense_warp_align16(size_t x) { return (x + 15) & ~(size_t)15; }

// The FP32 value of an FP64 value that is zero or a normal FP32 number, by its bits.
__device__ __forceinline__ float f32_of_exact(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const uint32_t hi = (uint32_t)(b >> 32);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    const uint32_t sign = hi & 0x80000000u;
    const uint32_t man = (uint32_t)(b >> 29) & 0x7FFFFFu;
    return __uint_as_float(e == 0 ? sign : (sign | ((e - 896u) << 23) | man));
}

// v is zero or a normal FP32 number whose double 2v is finite in FP32: then every
// term +-2v is an FP32 value and f32_of_exact(v) gives v.
__device__ __forceinline__ bool fp32_term_exact(double v) {
    const double a = fabs(v);
    return v == 0.0 || (a >= 1.1754943508222875e-38 && a <= 1.7014117331926443e38 && (double)__double2float_rn(v) == v);
}

// The same sweeps with two warps per replica on two SM sub-partitions: the term warp
// forms the terms of position p + 1 (and copies in J rows) while the chain warp walks
// and decides position p; one 64-thread named barrier per position.  The term warp
// forms position p + 1 before p's flip is known, so after the barrier the chain warp
// corrects them exactly: a flip of spin (i_p, k_p) negates position p + 1's column
// i_p when the slice is the same, all its terms when it is the same spin in the same
// slice (a new sweep of sa.Anneal_dense can start with the spin the last one ended
// on), and a Trotter term of the same spin that reads slice k_p.  The term warp owns
// the spins and applies each flip after the barrier.  Same spins, uniforms and close
// calls as the single-warp kernel.
// One position of the sweep order: field step g, MC step, slice k, index t in the
// permutation; next() steps through g -> step -> k -> t without divisions.
struct DensePos {
    int g, step, k, t;
    __device__ __forceinline__ void next(int n, int Pq, int mcsteps) {
        if (++t == n) {
            t = 0;
            if (++k == Pq) {
                k = 0;
                if (++step == mcsteps) { step = 0; ++g; }
            }
        }
    }
};

// Shared memory of the dense pair kernel: spins [n][P], two J rows, two sets of FP64 and
// FP32 terms (FP32 padded for the chain's read-ahead), one flag per row, control words.
__host__ __device__ inline size_t dense_pair_smem(int n, int P) {
    return dense_warp_align16((size_t)n * P) + (size_t)16 * n + dense_warp_align16((size_t)16 * (n + 2)) +
           6 * dense_warp_align16((size_t)4 * (n + 12)) + dense_warp_align16((size_t)n) + 32;
}

// One step of the FP64 chain, (float)((double)e + t), from FP32 pieces t = t1 + t2 + t3
// (exact): c = fl32(s + fl32(fl32(a + t2) + t3)) with s + a = e + t1 exactly (TwoSum),
// and ok when a bound on |fl64(e + t) - c| is strictly below the half-gap of c's
// rounding interval, so that c is the reference's value.  The bound adds up the
// rounding errors of the tail's sum (<= 2^-23 (|a| + |t2| + |t3|)), of d = fl32((s - c)
// + tail) (s - c exact by Sterbenz's lemma when |tail| <= |s| / 4, checked), and of the
// FP64 rounding of the exact sum (<= 2^-52 |c|), each with a margin of 2 to 4 that also
// covers the rounding of the bound itself.  When ok is false the caller takes the
// reference's FP64 step instead.
__device__ __forceinline__ float chain_step32(float e, float t1, float t2, float t3, bool& ok) {
    const float s = __fadd_rn(e, t1);
    const float bb = __fsub_rn(s, e);
    const float a = __fadd_rn(__fsub_rn(e, __fsub_rn(s, bb)), __fsub_rn(t1, bb));
    const float wf = __fadd_rn(__fadd_rn(a, t2), t3);
    const float c = __fadd_rn(s, wf);
    const float d = __fadd_rn(__fsub_rn(s, c), wf);
    const float sum_abs = __fadd_rn(__fadd_rn(fabsf(a), fabsf(t2)), fabsf(t3));
    const float bound = __fadd_rn(__fadd_rn(__fmul_rn(fabsf(d), 1.0000005f), __fmul_rn(sum_abs, 4.76837158203125e-7f)),
                                  __fadd_rn(__fmul_rn(fabsf(c), 4.44089209850062616e-16f), 1.17549435e-38f));
    const uint32_t cb = __float_as_uint(c) & 0x7FFFFFFFu;
    const uint32_t E = cb >> 23;
    const uint32_t hb = ((cb & 0x7FFFFFu) == 0 ? (E - 25u) : (E - 24u)) << 23;   // half-gap (a power of two:
    ok = E >= 26u && E <= 253u && fabsf(wf) <= __fmul_rn(0.25f, fabsf(s)) &&     // the gap below is half)
         bound < __uint_as_float(hb);
    return c;
}

template <bool QA>
__global__ void __launch_bounds__(64) dense_reforder_pair_kernel(
    int8_t* __restrict__ spins, const double* __restrict__ J, int n, int P, int R,
    const float* __restrict__ per_step,   // QA: J-perp of each field step; SA: its temperature
    int nsched, int mcsteps, float temp_qa, const int32_t* __restrict__ perms, const int32_t* __restrict__ rands,
    int64_t rand_stride, int64_t* __restrict__ rand_used, int flags, ExpPatch ep, int32_t* status) {
    extern __shared__ __align__(16) int8_t sh[];
    const int r = blockIdx.x;
    if (r >= R) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Pq = QA ? P : 1;
    const int nt = QA ? n + 2 : n;
    int8_t* s = sh;                                                                                   // [n][P]
    double* row = reinterpret_cast<double*>(sh + dense_warp_align16((size_t)n * Pq));                 // [2][n]
    double* t64 = row + (size_t)2 * n;                                                               // [2][n + 2]
    float* t32 = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(t64) +
                                          dense_warp_align16((size_t)16 * (n + 2)));                 // [2][t32s]
    const size_t t32s = dense_warp_align16((size_t)4 * (n + 12)) / 4;
    float* q2 = t32 + 2 * t32s;                                                                       // [2][t32s]
    float* q3 = q2 + 2 * t32s;                                                                        // [2][t32s]
    uint8_t* row_f32 = reinterpret_cast<uint8_t*>(q3 + 2 * t32s);                                    // [n]
    int* ctl = reinterpret_cast<int*>(row_f32 + dense_warp_align16((size_t)n));   // flip, stop; split ok
    if (threadIdx.x < 8) ctl[threadIdx.x] = 0;
    int8_t* gs = spins + (int64_t)r * n * Pq;
    for (int64_t t = threadIdx.x; t < (int64_t)n * Pq; t += 64) s[t] = gs[t];
    for (int i = warp; i < n; i += 2) {
        bool ok = true;
        for (int j = lane; j < n; j += 32) ok = ok && fp32_term_exact(j >= i ? J[(int64_t)i * n + j] : J[(int64_t)j * n + i]);
        ok = __all_sync(0xffffffffu, ok);
        if (lane == 0) row_f32[i] = ok ? 1 : 0;
    }
    __syncthreads();
    const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * n;
    const int64_t nsweeps = (int64_t)nsched * mcsteps;
    const int64_t total = nsweeps * Pq * n;
    // each warp walks the permutation entries itself (counters stepped, no division)
    int64_t q_sweep = 0;
    int q_k = 0, q_t = 0;
    auto next_entry = [&]() -> int {
        const bool has = q_sweep < nsweeps;
        const int v = __ldg(pr + (has ? q_sweep * n + q_t : 0));
        if (++q_t == n) {
            q_t = 0;
            if (++q_k == Pq) { q_k = 0; ++q_sweep; }
        }
        return v;
    };
    auto safe = [&](int i) { return (unsigned)i < (unsigned)n ? i : 0; };
    auto jp_of = [&](int g) -> double { return QA ? (double)per_step[g] : 0.0; };
    auto f32_of = [&](int i, int g) -> bool {
        return row_f32[safe(i)] && (!QA || fabs(jp_of(g)) <= 1.7014117331926443e38);
    };
    auto tl_of = [&](int k) { return (QA && (flags & PQ_FIX_Q1)) ? (k == 0 ? P - 1 : k - 1) : P - 1; };
    auto tr_of = [&](int k) { return (QA && (flags & PQ_FIX_Q1)) ? (k == P - 1 ? 0 : k + 1) : 1; };
    bool dead = false, bad = false;
    int64_t used = 0;
    if (total > 0) {
        if (warp == 1) {
            // ---- term warp ----
            auto prefetch_row = [&](int i, int b) {
                i = safe(i);
                double* dst = row + (size_t)b * n;
                for (int j = lane; j < n; j += 32)
                    cp_async8(dst + j, j >= i ? J + (int64_t)i * n + j : J + (int64_t)j * n + i);
                cp_async_commit();
            };
            auto form = [&](int i, int k, int g, const double* rw, int b) {
                float* o32 = t32 + (size_t)b * t32s;
                double* o64 = t64 + (size_t)b * (n + 2);
                float* o2 = q2 + (size_t)b * t32s;
                float* o3 = q3 + (size_t)b * t32s;
                const bool f32 = f32_of(i, g);
                i = safe(i);
                const int8_t si8 = s[(int64_t)i * Pq + k];
                if (f32) {
                    const float m2si = si8 > 0 ? -2.0f : 2.0f;
                    for (int j = lane; j < n; j += 32) {
                        const float jf = f32_of_exact(rw[j]);
                        const uint32_t sgn = j == i ? 0u : ((uint32_t)(int32_t)s[(int64_t)j * Pq + k] & 0x80000000u);
                        o32[j] = __fmul_rn(__uint_as_float(__float_as_uint(m2si) ^ sgn), jf);
                    }
                    if (QA && lane == 0) {
                        const float jpf = (float)jp_of(g);
                        o32[n] = __fmul_rn(m2si, s[(int64_t)i * Pq + tl_of(k)] > 0 ? jpf : -jpf);
                        o32[n + 1] = __fmul_rn(m2si, s[(int64_t)i * Pq + tr_of(k)] > 0 ? jpf : -jpf);
                    }
                } else {
                    // FP64 terms, and each split exactly into FP32 pieces t1 + t2 + t3 for the
                    // chain's FP32 steps (t - t1 and the next remainder are exact in FP64)
                    const double m2si = -2.0 * (double)si8;
                    bool ok = true;
                    auto split = [&](int j, double tt) {
                        o64[j] = tt;
                        const float a1 = __double2float_rn(tt);
                        const double r1 = __dsub_rn(tt, (double)a1);
                        const float a2 = __double2float_rn(r1);
                        const double r2 = __dsub_rn(r1, (double)a2);
                        const float a3 = __double2float_rn(r2);
                        ok &= ((double)a3 == r2) & (fabsf(a1) <= 3.0e38f);
                        o32[j] = a1;
                        o2[j] = a2;
                        o3[j] = a3;
                    };
#pragma unroll 4
                    for (int j = lane; j < n; j += 32) {   // unrolled: independent FP64 chains overlap
                        const double jv = rw[j];
                        split(j, j == i ? m2si * jv : m2si * (jv * (double)s[(int64_t)j * Pq + k]));
                    }
                    if (QA && lane == 0) {
                        const double jp = jp_of(g);
                        split(n, m2si * (jp * (double)s[(int64_t)i * Pq + tl_of(k)]));
                        split(n + 1, m2si * (jp * (double)s[(int64_t)i * Pq + tr_of(k)]));
                    }
                    ok = __all_sync(0xffffffffu, ok);
                    if (lane == 0) ctl[4 + b] = ok ? 1 : 0;
                }
            };
            int e0 = next_entry(), e1 = next_entry(), e2 = next_entry(), e3 = next_entry();
            DensePos nx{0, 0, 0, 0};   // the position whose terms are formed next
            prefetch_row(e0, 0);
            if (total > 1) prefetch_row(e1, 1);
            else cp_async_commit();
            cp_async_wait<1>();
            __syncwarp();
            form(e0, 0, 0, row, 0);          // position 0
            __syncwarp();
            pair_barrier();                  // terms of position 0 are ready
            for (int64_t p = 0; p < total; ++p) {
                // terms of position p + 1 (the row of p + 2 is copied in meanwhile)
                nx.next(n, Pq, mcsteps);
                if (p + 2 < total) prefetch_row(e2, (int)(p & 1));
                else cp_async_commit();
                cp_async_wait<1>();
                __syncwarp();
                if (p + 1 < total) form(e1, nx.k, nx.g, row + (size_t)((p + 1) & 1) * n, (int)((p + 1) & 1));
                __syncwarp();
                pair_barrier();              // the chain warp has decided position p
                const int* c = ctl + 2 * (int)(p & 1);   // two slots: the chain warp writes p + 1's
                if (c[1]) break;                         // only after the next barrier
                if (lane == 0 && c[0] >= 0) {   // position p flipped: (i, k) packed
                    const int fi = c[0] >> 8, fk = c[0] & 0xFF;
                    s[(int64_t)fi * Pq + fk] = (int8_t)-s[(int64_t)fi * Pq + fk];
                }
                __syncwarp();
                e1 = e2;
                e2 = e3;
                e3 = next_entry();
            }
            cp_async_wait<0>();
        } else {
            // ---- chain warp ----
            UniformRing ring;
            ring.init(rands + (int64_t)r * rand_stride, rand_stride, lane);
            const int64_t cap = rand_stride;
            int i0 = next_entry(), i1 = next_entry();
            DensePos cur{0, 0, 0, 0};
            float ediff = 0.0f;
            pair_barrier();                  // terms of position 0 are ready
            for (int64_t p = 0; p < total; ++p) {
                DensePos nx = cur;
                nx.next(n, Pq, mcsteps);
                const int tb = (int)(p & 1);
                const bool f32 = f32_of(i0, cur.g);
                int flip_word = -1, stop = 0;
                if ((unsigned)i0 >= (unsigned)n) {
                    bad = dead = true;
                    stop = 1;
                } else {
                    if (!QA || (flags & PQ_FIX_Q2) || cur.t == 0) ediff = 0.0f;   // QA, Q2 as shipped: per slice
                    if (f32) {
                        const float4* tv = reinterpret_cast<const float4*>(t32 + (size_t)tb * t32s);
                        const int nq = nt >> 2;
                        float4 v = tv[0], v1 = tv[1];
                        for (int q = 0; q < nq; ++q) {
                            const float4 v2 = tv[q + 2];
                            ediff = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(ediff, v.x), v.y), v.z), v.w);
                            v = v1;
                            v1 = v2;
                        }
                        const float* c32 = t32 + (size_t)tb * t32s;
                        for (int j = nq * 4; j < nt; ++j) ediff = __fadd_rn(ediff, c32[j]);
                    } else if (ctl[4 + tb]) {
                        // FP32 steps on the split terms, walked ahead; a step whose check fails is
                        // redone as the reference's FP64 step and the walk resumes after it
                        const float* c1 = t32 + (size_t)tb * t32s;
                        const float* c2 = q2 + (size_t)tb * t32s;
                        const float* c3 = q3 + (size_t)tb * t32s;
                        const double* c64 = t64 + (size_t)tb * (n + 2);
                        int j0 = 0;
                        while (j0 < nt) {
                            int bad = -1;
                            float e_bad = 0.0f, ee = ediff;
                            float x1 = c1[j0], x2 = c2[j0], x3 = c3[j0];   // the next step's pieces
#pragma unroll 4
                            for (int j = j0; j < nt; ++j) {                 // are read a step ahead;
                                                                            // unrolled so that a step's
                                                                            // check overlaps the next adds
                                const int jn = j + 1 < nt ? j + 1 : j;
                                const float y1 = c1[jn], y2 = c2[jn], y3 = c3[jn];
                                bool ok;
                                const float c = chain_step32(ee, x1, x2, x3, ok);
                                if (!ok && bad < 0) { bad = j; e_bad = ee; }
                                ee = c;
                                x1 = y1; x2 = y2; x3 = y3;
                            }
                            if (bad < 0) { ediff = ee; break; }
                            ediff = acc(e_bad, c64[bad]);
                            j0 = bad + 1;
                        }
                    } else {
                        const double* c64 = t64 + (size_t)tb * (n + 2);
                        double v = c64[0];
                        for (int j = 0; j < nt; ++j) {
                            const double vn = c64[j + 1 < nt ? j + 1 : j];
                            ediff = acc(ediff, v);
                            v = vn;
                        }
                    }
                    const float temp = QA ? temp_qa : per_step[cur.g];
                    bool flip = false;
                    if (ediff > 0.0f) {
                        flip = true;
                    } else if (used >= cap) {
                        if (lane == 0) pq_set_status(status, PQ_ERR_RAND_EXHAUSTED);
                        dead = true;
                        stop = 1;
                    } else {
                        const int32_t rv = ring.get(used);
                        ++used;
                        ring.advance(used, lane);
                        const float rl = quick_scale(temp);
                        const int fast = rl != 0.0f ? quick_decide(ediff, rl, rv) : -1;
                        if (fast >= 0) {
                            flip = fast != 0;
                        } else {
                            const float xf = __fdiv_rn(ediff, temp);
                            const int quick = fp32_decide(xf, rv);
                            if (quick >= 0) {
                                flip = quick != 0;
                            } else {
                                const double qv = (double)rv / 2147483647.0;   // glibc RAND_MAX
                                bool miss = false;
                                flip = patched_exp(xf, qv, ep, &miss) > qv;
                                if (miss && lane == 0) record_close(ep, xf, exp((double)xf));
                            }
                        }
                    }
                    if (flip) flip_word = (i0 << 8) | cur.k;
                }
                if (lane == 0) { ctl[2 * (int)(p & 1)] = flip_word; ctl[2 * (int)(p & 1) + 1] = stop; }
                pair_barrier();              // the term warp has formed position p + 1
                if (stop) break;
                if (flip_word >= 0 && p + 1 < total && (unsigned)i1 < (unsigned)n) {
                    // correct position p + 1's terms for this flip
                    // (every form of a term is negated: FP32, FP64 and the FP32 pieces)
                    const int nb = (int)((p + 1) & 1);
                    float* n32 = t32 + (size_t)nb * t32s;
                    float* n2 = q2 + (size_t)nb * t32s;
                    float* n3 = q3 + (size_t)nb * t32s;
                    double* n64 = t64 + (size_t)nb * (n + 2);
                    auto negate = [&](int j) {
                        n32[j] = -n32[j];
                        n2[j] = -n2[j];
                        n3[j] = -n3[j];
                        n64[j] = -n64[j];
                    };
                    if (nx.k == cur.k) {
                        if (i1 == i0) {
                            for (int j = lane; j < n; j += 32) negate(j);
                        } else if (lane == 0) {
                            negate(i0);
                        }
                    }
                    if (QA && lane == 0 && i1 == i0) {
                        if (tl_of(nx.k) == cur.k) negate(n);
                        if (tr_of(nx.k) == cur.k) negate(n + 1);
                    }
                    __syncwarp();
                }
                cur = nx;
                i0 = i1;
                i1 = next_entry();
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
        rand_used[r] = dead ? -1 : used;
    }
    for (int64_t t = threadIdx.x; t < (int64_t)n * Pq; t += 64) gs[t] = s[t];
}

// sa.Anneal_bipartite in reference order (piqmc/sa.pyx:411-500) with one warp per
// replica: the left spins in order, then the right spins, each update's terms
// ((2 s_i J s_j) + b_i s_i) + b_j s_j formed in FP64 by the lanes in parallel and the
// chain ediff = (float)((double)ediff - t) walked in order -- as FP32 subtractions
// when every term of the update is an FP32 value (the same value, see the dense
// kernel), else in FP64 term by term.  The J vector of the next spin (a row for a
// left spin, a column for a right one) is copied into shared memory by cp.async while
// the current spin is resolved.
__host__ __device__ inline size_t bipartite_warp_smem(int nl, int nr) {
    const size_t m = (size_t)(nl > nr ? nl : nr);
    return dense_warp_align16((size_t)nl + nr) + 16 * m + dense_warp_align16(8 * (m + 1)) +
           3 * dense_warp_align16(4 * (m + 12));
}

__global__ void __launch_bounds__(32) sa_bipartite_reforder_warp_kernel(
    int8_t* __restrict__ spins, const double* __restrict__ J, int nl, int nr, const double* __restrict__ lbias,
    const double* __restrict__ rbias, int R, const float* __restrict__ temps, int nsched, int mcsteps,
    const int32_t* __restrict__ rands, int64_t rand_stride, int64_t* __restrict__ rand_used, ExpPatch ep,
    int32_t* status) {
    extern __shared__ __align__(16) int8_t sh[];
    const int r = blockIdx.x;
    if (r >= R) return;
    const int lane = threadIdx.x;
    const int m = nl > nr ? nl : nr;
    int8_t* lv = sh;                                                                                 // [nl]
    int8_t* rv = sh + nl;                                                                            // [nr]
    double* vec = reinterpret_cast<double*>(sh + dense_warp_align16((size_t)nl + nr));              // [2][m]
    double* t64 = vec + (size_t)2 * m;                                                               // [m + 1]
    float* t32 = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(t64) +
                                          dense_warp_align16((size_t)8 * (m + 1)));                 // [m + 12]
    float* p2 = t32 + dense_warp_align16((size_t)4 * (m + 12)) / 4;                                // [m + 12]
    float* p3 = p2 + dense_warp_align16((size_t)4 * (m + 12)) / 4;                                 // [m + 12]
    int8_t* gs = spins + (int64_t)r * (nl + nr);
    for (int t = lane; t < nl + nr; t += 32) sh[t] = gs[t];
    __syncwarp();
    const int64_t cap = rand_stride;
    UniformRing ring;
    ring.init(rands + (int64_t)r * rand_stride, cap, lane);
    int64_t used = 0;
    bool dead = false;
    // J vector of spin (side, i): side 0 = left (row i of J, nr entries), 1 = right (column i, nl entries)
    auto prefetch = [&](int side, int i, int b) {
        double* dst = vec + (size_t)b * m;
        if (side == 0) {
            for (int j = lane; j < nr; j += 32) cp_async8(dst + j, J + (int64_t)i * nr + j);
        } else {
            for (int j = lane; j < nl; j += 32) cp_async8(dst + j, J + (int64_t)j * nr + i);
        }
        cp_async_commit();
    };
    const int64_t total = (int64_t)nsched * mcsteps * (nl + nr);
    if (total > 0) {
        // the spin after (side, i) in the sweep order
        auto after = [&](int& side, int& i) {
            if (side == 0) {
                if (++i == nl) { i = 0; side = nr > 0 ? 1 : 0; }
            } else {
                if (++i == nr) { i = 0; side = nl > 0 ? 0 : 1; }
            }
        };
        int side = nl > 0 ? 0 : 1, i = 0;
        prefetch(side, i, 0);
        int buf = 0;
        int64_t pos = 0;
        for (int g = 0; g < nsched && !dead; ++g) {
            const float temp = temps[g];
            const float rl = quick_scale(temp);
            for (int64_t q = 0; q < (int64_t)mcsteps * (nl + nr) && !dead; ++q, ++pos) {
                int nside = side, ni = i;
                after(nside, ni);
                if (pos + 1 < total) prefetch(nside, ni, buf ^ 1);
                else cp_async_commit();
                cp_async_wait<1>();
                __syncwarp();
                // terms of spin (side, i) against the other side, FP64 in the reference's order
                const double* jv = vec + (size_t)buf * m;
                const int8_t* self = side == 0 ? lv : rv;
                const int8_t* other = side == 0 ? rv : lv;
                const int no = side == 0 ? nr : nl;
                const double si = (double)self[i];
                bool exact = true, split_ok = true;
#pragma unroll 4
                for (int j = lane; j < no; j += 32) {   // unrolled: independent FP64 chains overlap
                    const double sj = (double)other[j];
                    const double t = side == 0 ? 2.0 * si * jv[j] * sj + lbias[i] * si + rbias[j] * sj
                                               : 2.0 * si * jv[j] * sj + lbias[j] * sj + rbias[i] * si;
                    // t = tf + a2 + a3 exactly in FP32 pieces (see chain_step32)
                    const float tf = __double2float_rn(t);
                    const double r1 = __dsub_rn(t, (double)tf);
                    const float a2 = __double2float_rn(r1);
                    const double r2 = __dsub_rn(r1, (double)a2);
                    const float a3 = __double2float_rn(r2);
                    exact &= r1 == 0.0;
                    split_ok &= ((double)a3 == r2) & (fabsf(tf) <= 3.0e38f);
                    t64[j] = t;
                    t32[j] = tf;
                    p2[j] = a2;
                    p3[j] = a3;
                }
                const bool f32 = __all_sync(0xffffffffu, exact);
                const bool split = __all_sync(0xffffffffu, split_ok);
                __syncwarp();
                float ediff = 0.0f;
                if (f32) {
                    const float4* tv = reinterpret_cast<const float4*>(t32);
                    const int nq = no >> 2;
                    float4 v = tv[0], v1 = tv[1];
                    for (int qq = 0; qq < nq; ++qq) {
                        const float4 v2 = tv[qq + 2];
                        ediff = __fsub_rn(__fsub_rn(__fsub_rn(__fsub_rn(ediff, v.x), v.y), v.z), v.w);
                        v = v1;
                        v1 = v2;
                    }
                    for (int j = nq * 4; j < no; ++j) ediff = __fsub_rn(ediff, t32[j]);
                } else if (split) {
                    // FP32 steps on the negated pieces, walked ahead; a failing step is redone
                    // as the reference's FP64 step and the walk resumes after it
                    int j0 = 0;
                    while (j0 < no) {
                        int bad = -1;
                        float e_bad = 0.0f, ee = ediff;
                        float x1 = t32[j0], x2 = p2[j0], x3 = p3[j0];
#pragma unroll 4
                        for (int j = j0; j < no; ++j) {
                            const int jn = j + 1 < no ? j + 1 : j;
                            const float y1 = t32[jn], y2 = p2[jn], y3 = p3[jn];
                            bool ok;
                            const float c = chain_step32(ee, -x1, -x2, -x3, ok);
                            if (!ok && bad < 0) { bad = j; e_bad = ee; }
                            ee = c;
                            x1 = y1; x2 = y2; x3 = y3;
                        }
                        if (bad < 0) { ediff = ee; break; }
                        ediff = __double2float_rn(__dsub_rn((double)e_bad, t64[bad]));
                        j0 = bad + 1;
                    }
                } else {
                    for (int j = 0; j < no; ++j) ediff = __double2float_rn(__dsub_rn((double)ediff, t64[j]));
                }
                bool flip = false;
                if (ediff > 0.0f) {
                    flip = true;
                } else if (used >= cap) {
                    if (lane == 0) pq_set_status(status, PQ_ERR_RAND_EXHAUSTED);
                    dead = true;
                    break;
                } else {
                    const int32_t rvv = ring.get(used);
                    ++used;
                    ring.advance(used, lane);
                    const int fast = rl != 0.0f ? quick_decide(ediff, rl, rvv) : -1;
                    if (fast >= 0) {
                        flip = fast != 0;
                    } else {
                        const float xf = __fdiv_rn(ediff, temp);
                        const int quick = fp32_decide(xf, rvv);
                        if (quick >= 0) {
                            flip = quick != 0;
                        } else {
                            const double qv = (double)rvv / 2147483647.0;   // glibc RAND_MAX
                            bool miss = false;
                            flip = patched_exp(xf, qv, ep, &miss) > qv;
                            if (miss && lane == 0) record_close(ep, xf, exp((double)xf));
                        }
                    }
                }
                if (flip && lane == 0) {
                    int8_t* sp = side == 0 ? lv : rv;
                    sp[i] = (int8_t)-sp[i];
                }
                __syncwarp();
                side = nside;
                i = ni;
                buf ^= 1;
            }
        }
    }
    cp_async_wait<0>();
    __syncwarp();
    if (lane == 0) rand_used[r] = dead ? -1 : used;
    for (int t = lane; t < nl + nr; t += 32) gs[t] = sh[t];
}

// sa.Anneal with warps sharing the work (spins in shared memory, maxnb <= 8).
// The energy difference is reset for every spin (piqmc/sa.pyx:119), so the sums
// of a block's 32 positions are independent except through neighbours flipped
// earlier in the same block.  Each pass takes every open position, with in-block
// neighbours still undecided taken as not flipping: their sums are computed in
// parallel (each lane its own FP32 chain in the reference's term order), the
// uniforms they consume are numbered by a ballot prefix count (a position consumes
// one when ediff < 0, :114-117), and they decide in parallel with ref_accept's
// arithmetic.  The decisions stand up to the first position with an in-block
// neighbour that flipped in the pass, where the next pass starts.
// Two warps per replica, as in qa_sparse_reforder_pair_kernel: the fold warp prepares
// block b + 1 (signed couplings, s2, in-block dependencies, and the positions in
// block b of each neighbour and of the spin itself) while the chain warp resolves
// block b; after the block barrier the chain warp negates exactly the couplings whose
// neighbour flipped in block b, and s2 when the spin itself did (a new sweep can
// revisit a spin of the previous block).  Same results, uniforms and close calls as
// sa_sparse_reforder_kernel.
struct SaPairLayout {
    size_t pos_of, xs, s2, dep, pp, ppv, self, ctl, total;
    __host__ __device__ explicit SaPairLayout(int n) {
        auto a16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
        pos_of = a16((size_t)n);                     // int8 spins [n], then uint8 [2][n]
        xs = pos_of + a16((size_t)2 * n);            // float [2][32][8]
        s2 = xs + (size_t)2 * 32 * 8 * 4;            // float [2][32]
        dep = s2 + (size_t)2 * 32 * 4;               // uint32 [2][32]
        pp = dep + (size_t)2 * 32 * 4;               // uint8 [2][32][8]
        ppv = pp + (size_t)2 * 32 * 8;               // uint8 [2][32][8]
        self = ppv + (size_t)2 * 32 * 8;             // uint8 [2][32]
        ctl = self + 64;                             // int [2][2], bad
        total = ctl + 32;
    }
};

template <bool FP64>
__global__ void __launch_bounds__(64) sa_sparse_reforder_pair_kernel(
    int8_t* __restrict__ spins, const int32_t* __restrict__ nb_idx, const float* __restrict__ nb_j, int n, int maxnb,
    int R, const float* __restrict__ temps, int nsched, int mcsteps, const int32_t* __restrict__ perms,
    const int32_t* __restrict__ rands, int64_t rand_stride, int64_t* __restrict__ rand_used, ExpPatch ep,
    int32_t* status) {
    constexpr int MAXNB = 8;
    extern __shared__ __align__(16) int8_t sh[];
    const SaPairLayout L(n);
    int8_t* s = sh;                                                          // [n]
    uint8_t* pos_of = reinterpret_cast<uint8_t*>(sh + L.pos_of);             // [2][n]
    float* mxs = reinterpret_cast<float*>(sh + L.xs);                        // [2][32][8]
    float* ms2 = reinterpret_cast<float*>(sh + L.s2);                        // [2][32]
    uint32_t* mdep = reinterpret_cast<uint32_t*>(sh + L.dep);                // [2][32]
    uint8_t* mpp = reinterpret_cast<uint8_t*>(sh + L.pp);                    // [2][32][8]
    uint8_t* mppv = reinterpret_cast<uint8_t*>(sh + L.ppv);                  // [2][32][8]
    uint8_t* mself = reinterpret_cast<uint8_t*>(sh + L.self);                // [2][32]
    int* ctl = reinterpret_cast<int*>(sh + L.ctl);                           // [2][2], bad
    const int r = blockIdx.x;
    if (r >= R) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int8_t* gs = spins + (int64_t)r * n;
    for (int t = threadIdx.x; t < n; t += 64) s[t] = gs[t];
    for (int t = threadIdx.x; t < 2 * n; t += 64) pos_of[t] = 0xFF;
    if (threadIdx.x < 5) ctl[threadIdx.x] = 0;
    __syncthreads();
    const int nblk = (n + 31) / 32;
    const int64_t total = (int64_t)nsched * mcsteps * nblk;
    const int64_t nsweeps = (int64_t)nsched * mcsteps;
    bool dead = false;
    int64_t used = 0;
    if (total > 0) {
        if (warp == 1) {
            // ---- fold warp ----
            const int32_t* pr = perms + (int64_t)r * nsched * mcsteps * n;
            bool bad = false;
            struct In { int i; int j[MAXNB]; float v[MAXNB]; };
            int64_t q_sweep = 0;
            int q_blk = 0;
            auto perm_next = [&](bool& has) -> int {
                const int t = q_blk * 32 + lane;
                has = q_sweep < nsweeps && t < n;
                const int v = __ldg(pr + (has ? q_sweep * n + t : 0));
                if (++q_blk == nblk) { q_blk = 0; ++q_sweep; }
                return v;
            };
            auto rows_of = [&](bool has, int i, In& in) {
                in.i = -1;
                if (!has) return;
                if ((unsigned)i >= (unsigned)n) { bad = true; i = 0; }
                in.i = i;
                if (maxnb <= 0) {
#pragma unroll
                    for (int m = 0; m < MAXNB; ++m) { in.j[m] = i; in.v[m] = 0.0f; }
                    return;
                }
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) {   // entries m >= maxnb repeat the last one, never read
                    const int mm = m < maxnb ? m : maxnb - 1;
                    in.j[m] = __ldg(nb_idx + (int64_t)i * maxnb + mm);
                    in.v[m] = __ldg(nb_j + (int64_t)i * maxnb + mm);
                }
            };
            auto fold = [&](int blk, const In& in, int fb, int pb, bool has_prev) {
                const int nb = min(32, n - blk * 32);
                const int i = in.i;
                uint8_t* po = pos_of + (size_t)fb * n;
                const uint8_t* pv = pos_of + (size_t)pb * n;
                if (lane < nb) po[i] = (uint8_t)lane;
                __syncwarp();
                float x[MAXNB];
                uint8_t pp[MAXNB], ppv[MAXNB];
                uint32_t dep = 0;
                float s2 = 0.0f;
                uint8_t self = 0xFF;
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) { x[m] = 0.0f; pp[m] = 0xFF; ppv[m] = 0xFF; }
                if (lane < nb) {
                    s2 = -2.0f * (float)s[i];
#pragma unroll
                    for (int m = 0; m < MAXNB; ++m) {
                        int j = in.j[m];
                        float v = in.v[m];
                        if (m < maxnb && j != i) {
                            if ((unsigned)j >= (unsigned)n) { bad = true; j = i; }
                            else {
                                if (s[j] <= 0) v = -v;
                                const uint8_t q = po[j];
                                if (q < lane) { pp[m] = q; dep |= 1u << q; }
                                if (has_prev) ppv[m] = pv[j];
                            }
                        }
                        x[m] = v;
                    }
                    if (has_prev) self = pv[i];
                }
                const int o = fb * 32 + lane;
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) {
                    mxs[o * MAXNB + m] = x[m];
                    mpp[o * MAXNB + m] = pp[m];
                    mppv[o * MAXNB + m] = ppv[m];
                }
                ms2[o] = s2;
                mdep[o] = dep;
                mself[o] = self;
                __syncwarp();
            };
            In cur, nxt;
            bool p_has = false;
            int p_next = perm_next(p_has);   // block 0
            rows_of(p_has, p_next, cur);
            p_next = perm_next(p_has);       // block 1
            rows_of(p_has, p_next, nxt);
            p_next = perm_next(p_has);       // block 2
            int held_blk = 0;
            fold(0, cur, 0, 1, false);
            int held_i = cur.i;
            pair_barrier();                  // block 0 is folded
            for (int64_t bb = 0; bb < total; ++bb) {
                const int fblk = held_blk + 1 == nblk ? 0 : held_blk + 1;
                int fold_i = -1;
                if (bb + 1 < total) {
                    fold(fblk, nxt, (int)((bb + 1) & 1), (int)(bb & 1), true);
                    fold_i = nxt.i;
                    cur = nxt;
                    rows_of(p_has, p_next, nxt);   // block bb + 2
                    p_next = perm_next(p_has);     // block bb + 3
                }
                pair_barrier();                    // the chain warp has resolved block bb
                const int* c = ctl + 2 * (int)(bb & 1);
                const uint32_t fm = (uint32_t)c[0];
                const int nb = min(32, n - held_blk * 32);
                if (lane < nb) {
                    if ((fm >> lane) & 1u) s[held_i] = (int8_t)-s[held_i];
                    pos_of[(size_t)(bb & 1) * n + held_i] = 0xFF;
                }
                __syncwarp();
                if (c[1]) break;
                held_blk = fblk;
                held_i = fold_i;
            }
            bad = __any_sync(0xffffffffu, bad);
            if (lane == 0 && bad) ctl[4] = 1;
        } else {
            // ---- chain warp ----
            const int64_t cap = rand_stride;
            UniformRing ring;
            ring.init(rands + (int64_t)r * rand_stride, cap, lane);
            int blk = 0, g = 0, step = 0;
            uint32_t fm_prev = 0;
            pair_barrier();                  // block 0 is folded
            for (int64_t bb = 0; bb < total; ++bb) {
                const int buf = (int)(bb & 1);
                const int nb = min(32, n - blk * 32);
                const float temp = temps[g];
                const float rl = quick_scale(temp);
                const int o = buf * 32 + lane;
                float x[MAXNB];
                uint8_t pp[MAXNB];
#pragma unroll
                for (int m = 0; m < MAXNB; ++m) { x[m] = mxs[o * MAXNB + m]; pp[m] = mpp[o * MAXNB + m]; }
                float s2 = ms2[o];
                const uint32_t dep = mdep[o];
                if (lane < nb && fm_prev) {   // the previous block's flips
#pragma unroll
                    for (int m = 0; m < MAXNB; ++m) {
                        const uint8_t q = mppv[o * MAXNB + m];
                        if (q != 0xFF && ((fm_prev >> q) & 1u)) x[m] = -x[m];
                    }
                    const uint8_t q = mself[o];
                    if (q != 0xFF && ((fm_prev >> q) & 1u)) s2 = -s2;
                }
                uint32_t flipmask = 0;
                int cc = 0;
                int start = 0;
                int stop = 0;
                while (start < nb) {
                    const bool mine = lane >= start && lane < nb;
                    float ediff = 0.0f;
                    if (mine) {
#pragma unroll
                        for (int m = 0; m < MAXNB; ++m) {
                            if (m < maxnb) {
                                const float v = (pp[m] != 0xFF && ((flipmask >> pp[m]) & 1u)) ? -x[m] : x[m];
                                ediff = acc2<FP64>(ediff, s2, v);
                            }
                        }
                    }
                    const bool consume = mine && !(ediff >= 0.0f);
                    const uint32_t cons = __ballot_sync(0xffffffffu, consume);
                    const int my_c = cc + __popc(cons & ((1u << lane) - 1u));
                    const int32_t rv = ring.get(used + my_c);
                    bool flip = false, out = false, miss = false;
                    float xf = 0.0f;
                    if (mine) {
                        if (!consume) {
                            flip = true;
                        } else if (used + my_c >= cap) {
                            out = true;
                        } else {
                            const int fast = rl != 0.0f ? quick_decide(ediff, rl, rv) : -1;
                            if (fast >= 0) {
                                flip = fast != 0;
                            } else {
                                xf = __fdiv_rn(ediff, temp);
                                const int quick = fp32_decide(xf, rv);
                                if (quick >= 0) {
                                    flip = quick != 0;
                                } else {
                                    const double q = (double)rv / 2147483647.0;   // glibc RAND_MAX
                                    flip = patched_exp(xf, q, ep, &miss) > q;
                                }
                            }
                        }
                    }
                    const uint32_t fl = __ballot_sync(0xffffffffu, flip);
                    const uint32_t wrong = __ballot_sync(0xffffffffu, lane > start && lane < nb && (dep & fl));
                    const int p = wrong ? __ffs(wrong) - 1 : nb;
                    const uint32_t keep = p >= 32 ? 0xffffffffu : ((1u << p) - 1u);
                    if (__any_sync(0xffffffffu, out && lane < p)) {
                        if (lane == 0) pq_set_status(status, PQ_ERR_RAND_EXHAUSTED);
                        dead = true;
                        stop = 1;
                        break;
                    }
                    if (miss && lane < p) record_close(ep, xf, exp((double)xf));
                    flipmask |= fl & keep;
                    cc += __popc(cons & keep);
                    start = p;
                }
                if (!stop) {
                    used += cc;
                    ring.advance(used, lane);
                }
                if (lane == 0) { ctl[2 * buf] = (int)flipmask; ctl[2 * buf + 1] = stop; }
                pair_barrier();              // the fold warp has folded block bb + 1
                if (stop) break;
                fm_prev = flipmask;
                if (++blk == nblk) {
                    blk = 0;
                    if (++step == mcsteps) { step = 0; ++g; }
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool bad = ctl[4] != 0;
        if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
        rand_used[r] = (dead || bad) ? -1 : used;
    }
    for (int t = threadIdx.x; t < n; t += 64) gs[t] = s[t];
}

__global__ void exp_probe_kernel(const float* __restrict__ x, double* __restrict__ y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = exp((double)x[i]);
}

__global__ void exp_range_probe_kernel(uint32_t first_bits, int64_t count, double* __restrict__ y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) y[i] = exp((double)__uint_as_float(first_bits + (uint32_t)i));
}

constexpr size_t kRefSmemMax = 200 * 1024;

ExpPatch make_patch(const uint32_t* ov_x, const double* ov_y, int ov_n, uint32_t* close_x,
                    double* close_y, int close_cap, int* close_cnt) {
    ExpPatch ep;
    ep.ov_x = ov_x; ep.ov_y = ov_y; ep.ov_n = ov_x && ov_y ? ov_n : 0;
    ep.close_x = close_x; ep.close_y = close_y; ep.close_cnt = close_x && close_y ? close_cnt : nullptr;
    ep.close_cap = close_cap;
    return ep;
}

template <bool FP64, int MAXNB, bool SMEM>
int launch_qa_sparse_t(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int nperm, int maxnb, int P,
                       int R, const float* jperp, int nsched, int mcsteps, float temp, const int32_t* perms,
                       const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags, const ExpPatch& ep,
                       int32_t* status, cudaStream_t stream) {
    const size_t smem = SMEM ? (size_t)n * P : 0;
    if (SMEM) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(qa_sparse_reforder_kernel<FP64, MAXNB, SMEM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    qa_sparse_reforder_kernel<FP64, MAXNB, SMEM><<<R, 32, smem, stream>>>(
        spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms, rands, rand_stride, rand_used,
        flags, ep, status);
    return pq_launch_status();
}

template <bool FP64, int MAXNB>
int launch_qa_sparse_s(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int nperm, int maxnb, int P,
                       int R, const float* jperp, int nsched, int mcsteps, float temp, const int32_t* perms,
                       const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags, const ExpPatch& ep,
                       int32_t* status, cudaStream_t stream) {
    if constexpr (MAXNB > 0) {
        const size_t psmem = SparsePairLayout<MAXNB>(n, P).total;
        if (psmem <= kRefSmemMax + 8192) {
            if (flags & PQ_FIX_Q2) {
                PQ_CUDA_TRY(cudaFuncSetAttribute(qa_sparse_reforder_pair_kernel<FP64, MAXNB, true>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
                qa_sparse_reforder_pair_kernel<FP64, MAXNB, true><<<R, 64, psmem, stream>>>(
                    spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms, rands,
                    rand_stride, rand_used, flags, ep, status);
            } else {
                PQ_CUDA_TRY(cudaFuncSetAttribute(qa_sparse_reforder_pair_kernel<FP64, MAXNB, false>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
                qa_sparse_reforder_pair_kernel<FP64, MAXNB, false><<<R, 64, psmem, stream>>>(
                    spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms, rands,
                    rand_stride, rand_used, flags, ep, status);
            }
            return pq_launch_status();
        }
    }
    if ((size_t)n * P <= kRefSmemMax)
        return launch_qa_sparse_t<FP64, MAXNB, true>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps,
                                                      temp, perms, rands, rand_stride, rand_used, flags, ep, status, stream);
    return launch_qa_sparse_t<FP64, MAXNB, false>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps,
                                                   temp, perms, rands, rand_stride, rand_used, flags, ep, status, stream);
}

template <bool FP64>
int launch_qa_sparse_f(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int nperm, int maxnb, int P,
                       int R, const float* jperp, int nsched, int mcsteps, float temp, const int32_t* perms,
                       const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags, const ExpPatch& ep,
                       int32_t* status, cudaStream_t stream) {
    if (maxnb == 4)
        return launch_qa_sparse_s<FP64, 4>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp,
                                           perms, rands, rand_stride, rand_used, flags, ep, status, stream);
    if (maxnb == 5)
        return launch_qa_sparse_s<FP64, 5>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp,
                                           perms, rands, rand_stride, rand_used, flags, ep, status, stream);
    return launch_qa_sparse_s<FP64, 0>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp,
                                       perms, rands, rand_stride, rand_used, flags, ep, status, stream);
}

int launch_qa_sparse(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int nperm, int maxnb, int P, int R,
                     const float* jperp, int nsched, int mcsteps, float temp, const int32_t* perms,
                     const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags, const ExpPatch& ep,
                     int32_t* status, cudaStream_t stream) {
    if (flags & PQ_ACC_FP64)
        return launch_qa_sparse_f<true>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms,
                                        rands, rand_stride, rand_used, flags, ep, status, stream);
    return launch_qa_sparse_f<false>(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms,
                                     rands, rand_stride, rand_used, flags, ep, status, stream);
}

constexpr int kRefThreads = 32;

}  // namespace

static int check_common(int n, int P, int R, int nsched, int mcsteps, float temp) {
    if (n <= 0 || P < 1 || R < 0 || nsched < 0 || mcsteps < 0) return PQ_ERR_INVALID_ARG;
    if ((double)nsched * mcsteps * n > 2147483647.0 * 64) return PQ_ERR_TOO_LARGE;
    (void)temp;
    return PQ_OK;
}

extern "C" {

int pq_qa_sparse_reforder_ex(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n,
                             int nperm, int maxnb, int P, int R, const float* jperp, int nsched, int mcsteps,
                             float temp, const int32_t* perms, const int32_t* rands,
                             int64_t rand_stride, int64_t* rand_used, int flags,
                             const uint32_t* ov_x, const double* ov_y, int ov_n,
                             uint32_t* close_x, double* close_y, int close_cap, int* close_cnt,
                             int32_t* status, void* stream) {
    int st = check_common(n, P, R, nsched, mcsteps, temp);
    if (st) return st;
    if (P < 2 || maxnb < 0 || nperm < 0 || nperm > n || !spins || !rand_used ||
        (maxnb > 0 && (!nb_idx || !nb_j)))
        return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    ExpPatch ep = make_patch(ov_x, ov_y, ov_n, close_x, close_y, close_cap, close_cnt);
    return launch_qa_sparse(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp, perms, rands,
                            rand_stride, rand_used, flags, ep, status, (cudaStream_t)stream);
}

int pq_qa_sparse_reforder(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int nperm,
                          int maxnb, int P, int R, const float* jperp, int nsched, int mcsteps, float temp,
                          const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                          int64_t* rand_used, int flags, int32_t* status, void* stream) {
    return pq_qa_sparse_reforder_ex(spins, nb_idx, nb_j, n, nperm, maxnb, P, R, jperp, nsched, mcsteps, temp,
                                    perms, rands, rand_stride, rand_used, flags, nullptr, nullptr, 0,
                                    nullptr, nullptr, 0, nullptr, status, stream);
}

int pq_qa_dense_reforder_ex(int8_t* spins, const double* J, int n, int P, int R, const float* jperp,
                            int nsched, int mcsteps, float temp, const int32_t* perms,
                            const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags,
                            const uint32_t* ov_x, const double* ov_y, int ov_n, uint32_t* close_x,
                            double* close_y, int close_cap, int* close_cnt, int32_t* status,
                            void* stream) {
    int st = check_common(n, P, R, nsched, mcsteps, temp);
    if (st) return st;
    if (P < 2 || !spins || !J || !rand_used) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    ExpPatch ep = make_patch(ov_x, ov_y, ov_n, close_x, close_y, close_cap, close_cnt);
    const size_t psmem = dense_pair_smem(n, P);
    if (psmem <= kRefSmemMax && P <= 256 && n <= (1 << 22)) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(dense_reforder_pair_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)psmem));
        dense_reforder_pair_kernel<true><<<R, 64, psmem, (cudaStream_t)stream>>>(
            spins, J, n, P, R, jperp, nsched, mcsteps, temp, perms, rands, rand_stride, rand_used, flags, ep, status);
        return pq_launch_status();
    }
    qa_dense_reforder_kernel<<<(R + kRefThreads - 1) / kRefThreads, kRefThreads, 0, (cudaStream_t)stream>>>(
        spins, J, n, P, R, jperp, nsched, mcsteps, temp, perms, rands, rand_stride, rand_used, flags,
        ep, status);
    return pq_launch_status();
}

int pq_qa_dense_reforder(int8_t* spins, const double* J, int n, int P, int R, const float* jperp,
                         int nsched, int mcsteps, float temp, const int32_t* perms,
                         const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags,
                         int32_t* status, void* stream) {
    return pq_qa_dense_reforder_ex(spins, J, n, P, R, jperp, nsched, mcsteps, temp, perms, rands,
                                   rand_stride, rand_used, flags, nullptr, nullptr, 0, nullptr,
                                   nullptr, 0, nullptr, status, stream);
}

int pq_sa_sparse_reforder_ex(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n,
                             int maxnb, int R, const float* temps, int nsched, int mcsteps,
                             const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                             int64_t* rand_used, int flags, const uint32_t* ov_x, const double* ov_y, int ov_n,
                             uint32_t* close_x, double* close_y, int close_cap, int* close_cnt,
                             int32_t* status, void* stream) {
    int st = check_common(n, 1, R, nsched, mcsteps, 1.0f);
    if (st) return st;
    if (maxnb < 0 || !spins || !rand_used || (maxnb > 0 && (!nb_idx || !nb_j))) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    ExpPatch ep = make_patch(ov_x, ov_y, ov_n, close_x, close_y, close_cap, close_cnt);
    const size_t psmem = SaPairLayout(n).total;
    if (maxnb <= 8 && psmem <= kRefSmemMax) {
        cudaStream_t st = (cudaStream_t)stream;
        if (flags & PQ_ACC_FP64) {
            PQ_CUDA_TRY(cudaFuncSetAttribute(sa_sparse_reforder_pair_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
            sa_sparse_reforder_pair_kernel<true><<<R, 64, psmem, st>>>(spins, nb_idx, nb_j, n, maxnb, R, temps, nsched,
                                                                       mcsteps, perms, rands, rand_stride, rand_used,
                                                                       ep, status);
        } else {
            PQ_CUDA_TRY(cudaFuncSetAttribute(sa_sparse_reforder_pair_kernel<false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
            sa_sparse_reforder_pair_kernel<false><<<R, 64, psmem, st>>>(spins, nb_idx, nb_j, n, maxnb, R, temps,
                                                                        nsched, mcsteps, perms, rands, rand_stride,
                                                                        rand_used, ep, status);
        }
        return pq_launch_status();
    }
    const dim3 grid((R + kRefThreads - 1) / kRefThreads), block(kRefThreads);
    if (flags & PQ_ACC_FP64)
        sa_sparse_reforder_kernel<true><<<grid, block, 0, (cudaStream_t)stream>>>(
            spins, nb_idx, nb_j, n, maxnb, R, temps, nsched, mcsteps, perms, rands, rand_stride, rand_used, ep, status);
    else
        sa_sparse_reforder_kernel<false><<<grid, block, 0, (cudaStream_t)stream>>>(
            spins, nb_idx, nb_j, n, maxnb, R, temps, nsched, mcsteps, perms, rands, rand_stride, rand_used, ep, status);
    return pq_launch_status();
}

int pq_sa_sparse_reforder(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n, int maxnb,
                          int R, const float* temps, int nsched, int mcsteps, const int32_t* perms,
                          const int32_t* rands, int64_t rand_stride, int64_t* rand_used,
                          int32_t* status, void* stream) {
    return pq_sa_sparse_reforder_ex(spins, nb_idx, nb_j, n, maxnb, R, temps, nsched, mcsteps, perms,
                                    rands, rand_stride, rand_used, 0, nullptr, nullptr, 0, nullptr,
                                    nullptr, 0, nullptr, status, stream);
}

int pq_sa_dense_reforder_ex(int8_t* spins, const double* J, int n, int R, const float* temps, int nsched,
                            int mcsteps, const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                            int64_t* rand_used, const uint32_t* ov_x, const double* ov_y, int ov_n,
                            uint32_t* close_x, double* close_y, int close_cap, int* close_cnt, int32_t* status,
                            void* stream) {
    int st = check_common(n, 1, R, nsched, mcsteps, 1.0f);
    if (st) return st;
    if (!spins || !J || !temps || !rand_used || (nsched * mcsteps > 0 && !perms)) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    ExpPatch ep = make_patch(ov_x, ov_y, ov_n, close_x, close_y, close_cap, close_cnt);
    const size_t psmem = dense_pair_smem(n, 1);
    if (psmem <= kRefSmemMax && n <= (1 << 22)) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(dense_reforder_pair_kernel<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
        dense_reforder_pair_kernel<false><<<R, 64, psmem, (cudaStream_t)stream>>>(
            spins, J, n, 1, R, temps, nsched, mcsteps, 1.0f, perms, rands, rand_stride, rand_used, 0, ep, status);
        return pq_launch_status();
    }
    sa_dense_reforder_kernel<<<(R + kRefThreads - 1) / kRefThreads, kRefThreads, 0, (cudaStream_t)stream>>>(
        spins, J, n, R, temps, nsched, mcsteps, perms, rands, rand_stride, rand_used, ep, status);
    return pq_launch_status();
}

int pq_sa_dense_reforder(int8_t* spins, const double* J, int n, int R, const float* temps, int nsched, int mcsteps,
                         const int32_t* perms, const int32_t* rands, int64_t rand_stride, int64_t* rand_used,
                         int32_t* status, void* stream) {
    return pq_sa_dense_reforder_ex(spins, J, n, R, temps, nsched, mcsteps, perms, rands, rand_stride, rand_used,
                                   nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, status, stream);
}

int pq_sa_bipartite_reforder_ex(int8_t* spins, const double* J, int nl, int nr, const double* lbias,
                                const double* rbias, int R, const float* temps, int nsched, int mcsteps,
                                const int32_t* rands, int64_t rand_stride, int64_t* rand_used, const uint32_t* ov_x,
                                const double* ov_y, int ov_n, uint32_t* close_x, double* close_y, int close_cap,
                                int* close_cnt, int32_t* status, void* stream) {
    if (nl < 0 || nr < 0 || R < 0 || nsched < 0 || mcsteps < 0 || !spins || !temps || !rand_used ||
        (nl > 0 && nr > 0 && (!J || !lbias || !rbias)))
        return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    ExpPatch ep = make_patch(ov_x, ov_y, ov_n, close_x, close_y, close_cap, close_cnt);
    const size_t wsmem = bipartite_warp_smem(nl, nr);
    if (nl > 0 && nr > 0 && wsmem <= kRefSmemMax) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(sa_bipartite_reforder_warp_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsmem));
        sa_bipartite_reforder_warp_kernel<<<R, 32, wsmem, (cudaStream_t)stream>>>(
            spins, J, nl, nr, lbias, rbias, R, temps, nsched, mcsteps, rands, rand_stride, rand_used, ep, status);
        return pq_launch_status();
    }
    sa_bipartite_reforder_kernel<<<(R + kRefThreads - 1) / kRefThreads, kRefThreads, 0, (cudaStream_t)stream>>>(
        spins, J, nl, nr, lbias, rbias, R, temps, nsched, mcsteps, rands, rand_stride, rand_used, ep, status);
    return pq_launch_status();
}

// Device exp((double)x) exactly as the reference-order kernels evaluate it.
int pq_exp_probe(const float* x, double* y, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!x || !y))) return PQ_ERR_INVALID_ARG;
    if (n == 0) return PQ_OK;
    exp_probe_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, y, n);
    return pq_launch_status();
}

// Same, for the consecutive FP32 bit patterns first_bits .. first_bits+count-1.
int pq_exp_probe_range(uint32_t first_bits, int64_t count, double* y, void* stream) {
    if (count < 0 || (count > 0 && !y) || (uint64_t)first_bits + (uint64_t)count > 0x100000000ull)
        return PQ_ERR_INVALID_ARG;
    if (count == 0) return PQ_OK;
    exp_range_probe_kernel<<<(unsigned)((count + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        first_bits, count, y);
    return pq_launch_status();
}

}  // extern "C"
