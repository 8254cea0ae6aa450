// Packed fast sweeps: world-lines bit-packed per spin in shared memory,
// independent update classes x Trotter-slice classes updated in parallel,
// Philox4x32-10 uniforms, FP32 local fields.
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
//   ediff = -2 (e + t);  flip if ediff > 0 or u < expf_neg(ediff * beta).
// u = (r >> 9) * 2^-23.  Uniforms: Philox4x32-10, key = seed.  Local update: counter = (device slot i,
// sweep, replica, q << 16 | m >> 2), word m & 3 for the m-th slice of class q.
// World-line move: counter = (i, last sweep of the step, replica,
// 1 << 24 | gm << 16 | class), word 0.  Class order of a sweep: counter =
// (0xFFFFFFFF, sweep, replica, 2 << 24 | b); words w[0..] of blocks b = 0,1,..;
// Fisher-Yates for j = M-1..1 swaps order[j] with order[(w[M-1-j] * (j+1)) >> 32];
// w[M-1] bit p = which slice class goes first for the p-th visited class.
#include "common.cuh"

namespace {

constexpr int kMaxClasses = PQ_MAX_CLASSES;
constexpr int kMaxRpc = 16;

struct FastArgs {
    int n, P, R, maxdeg, nclass, stride, order_mode;
    int class_size[kMaxClasses];
    int nsched, mcsteps, global_moves;
    float beta;
    uint32_t key0, key1;
    int64_t sweep_base;
    int replica_base;
    int rpc;  // replicas per CTA
};

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
__device__ void class_order(const FastArgs& a, uint32_t sweep, uint32_t replica, uint8_t* order,
                            uint32_t* parity) {
    const int M = a.nclass;
    for (int c = 0; c < M; ++c) order[c] = (uint8_t)c;
    if (a.order_mode == 0) { *parity = 0; return; }
    uint32_t w[4];
    int have = 0, used = 0, blk = 0;
    auto next = [&]() -> uint32_t {
        if (used == have) {
            const pq_u32x4 r = pq_philox(pq_u32x4{0xFFFFFFFFu, sweep, replica, (2u << 24) | (uint32_t)blk++},
                                         a.key0, a.key1);
            w[0] = r.x; w[1] = r.y; w[2] = r.z; w[3] = r.w;
            have = 4; used = 0;
        }
        return w[used++];
    };
    for (int j = M - 1; j >= 1; --j) {
        const uint32_t k = (uint32_t)(((uint64_t)next() * (uint32_t)(j + 1)) >> 32);
        const uint8_t t = order[j]; order[j] = order[k]; order[k] = t;
    }
    *parity = next();
}

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
// a 1e-4 relative guard band -- its error against expf_neg is below 2e-5 for every
// argument above -87 -- and expf_neg itself settles the rest, so the result is
// exactly the specification's.
__device__ __forceinline__ bool decide(float sum, float u, float m2beta, float m2blog2e) {
    if (sum < 0.0f) return true;
    const float pf = pq_ex2_approx(__fmul_rn(sum, m2blog2e));
    if (u > __fmul_rn(pf, 1.0001f)) return false;
    if (u < __fmul_rn(pf, 0.9999f) && pf > 1e-30f) return true;
    return u < pq_expf_neg(__fmul_rn(sum, m2beta));
}

// One spin's local update over the slices of slice class q, P = 2 * NQ <= 32
// slices fixed at compile time, DEG couplings.  Same arithmetic and uniforms as
// the generic path.
template <int NQ, int DEG>
__device__ __forceinline__ uint32_t update_fixed(uint32_t wi, const uint32_t (&d)[DEG], const float (&J)[DEG], float h,
                                                 float jp, int q, uint32_t i, uint32_t sweep, uint32_t rep, uint32_t key0,
                                                 uint32_t key1, float m2beta, float m2blog2e) {
    constexpr int P = 2 * NQ;
    constexpr uint32_t MASK = P >= 32 ? 0xffffffffu : ((1u << P) - 1u);
    const uint32_t up = ((wi << 1) | (wi >> (P - 1))) & MASK;
    const uint32_t dn = ((wi >> 1) | (wi << (P - 1))) & MASK;
    const uint32_t wq = wi >> q, dl = (wi ^ up) >> q, dr = (wi ^ dn) >> q;
    uint32_t dq[DEG];
#pragma unroll
    for (int m = 0; m < DEG; ++m) dq[m] = d[m] >> q;
    uint32_t flips = 0;
#pragma unroll
    for (int blk = 0; blk < (NQ + 3) / 4; ++blk) {
        const pq_u32x4 rnd = pq_philox(pq_u32x4{i, sweep, rep, (uint32_t)((q << 16) | blk)}, key0, key1);
        const uint32_t rw4[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int mm = blk * 4 + jj;
            if (mm < NQ) {
                const int sh = 31 - 2 * mm;  // bit 2*mm of the q-shifted words -> sign bit
                float e = flip_sign(h, (wq << sh) & 0x80000000u);
#pragma unroll
                for (int m = 0; m < DEG; ++m) e = __fadd_rn(e, flip_sign(J[m], (dq[m] << sh) & 0x80000000u));
                const float t = __fadd_rn(flip_sign(jp, (dl << sh) & 0x80000000u), flip_sign(jp, (dr << sh) & 0x80000000u));
                const float sum = __fadd_rn(e, t);
                if (decide(sum, pq_u01(rw4[jj]), m2beta, m2blog2e)) flips |= 1u << (2 * mm);
            }
        }
    }
    return flips << q;
}

template <typename W, int MAXDEG, int NQC>
__global__ void __launch_bounds__(512) qa_fast_kernel(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                                      const float* __restrict__ cpl,
                                                      const float* __restrict__ field,
                                                      const float* __restrict__ jperp,
                                                      const float* __restrict__ betas, FastArgs a,
                                                      unsigned long long* __restrict__ accepts,
                                                      int32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int csize[kMaxClasses];
    __shared__ uint8_t sorder[kMaxRpc][kMaxClasses];
    __shared__ uint32_t sparity[kMaxRpc];
    W* sw = reinterpret_cast<W*>(smem_raw);
    const int n = a.n, P = a.P, S = a.stride;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < kMaxClasses; ++c) csize[c] = a.class_size[c];
    }
    const int r0 = blockIdx.x * a.rpc;
    const int nrep = min(a.rpc, a.R - r0);
    if (nrep <= 0) return;
    const W mask = full_mask<W>(P);
    const int nclass_q = P == 1 ? 1 : ((P & 1) ? 3 : 2);

    // stage this CTA's replicas
    for (int t = threadIdx.x; t < nrep * n; t += blockDim.x) sw[t] = words[(int64_t)r0 * n + t];
    __syncthreads();

    bool bad = false;
    unsigned long long nacc = 0;
    for (int g = 0; g < a.nsched; ++g) {
        const float jp = P == 1 ? 0.0f : jperp[g];
        const float beta = betas ? betas[g] : a.beta;
        const float m2beta = __fmul_rn(-2.0f, beta);                          // exact
        const float m2blog2e = __fmul_rn(m2beta, 1.44269502162933349609375f);  // guard-band argument scale
        for (int step = 0; step < a.mcsteps; ++step) {
            const uint32_t sweep = (uint32_t)(a.sweep_base + (int64_t)g * a.mcsteps + step);
            if (threadIdx.x < nrep)
                class_order(a, sweep, (uint32_t)(a.replica_base + r0 + threadIdx.x), sorder[threadIdx.x],
                            &sparity[threadIdx.x]);
            __syncthreads();
            for (int p = 0; p < a.nclass; ++p) {
                for (int qq = 0; qq < nclass_q; ++qq) {
                    int rl = 0, s = threadIdx.x;
                    while (s >= S) { s -= S; ++rl; }
                    for (; rl < nrep;) {
                        const int cls = sorder[rl][p];
                        const int q = nclass_q == 2 ? (qq ^ (int)((sparity[rl] >> p) & 1u)) : qq;
                        if (s < csize[cls]) {
                            const int i = cls * S + s;
                            W* rw = sw + rl * n;
                            const W wi = rw[i];
                            W d[MAXDEG];
                            float J[MAXDEG];
                            load_site<W, MAXDEG>(rw, i, n, a.maxdeg, nbr, cpl, wi, d, J, bad);
                            const float h = __ldg(field + i);
                            const uint32_t ctr2 = (uint32_t)(a.replica_base + r0 + rl);
                            if constexpr (NQC > 0) {
                                const uint32_t fl = update_fixed<NQC, MAXDEG>(
                                    (uint32_t)wi, reinterpret_cast<const uint32_t(&)[MAXDEG]>(d), J, h, jp, q,
                                    (uint32_t)i, sweep, ctr2, a.key0, a.key1, m2beta, m2blog2e);
                                rw[i] = wi ^ (W)fl;
                                nacc += __popc(fl);
                            } else {
                            W dl, dr;
                            trotter_diffs<W>(wi, P, mask, dl, dr);
                            W flips = 0;
                            const int nq = slice_count(P, q);
                            for (int mb = 0; mb * 4 < nq; ++mb) {
                                const pq_u32x4 rnd = pq_philox(
                                    pq_u32x4{(uint32_t)i, sweep, ctr2, (uint32_t)((q << 16) | mb)}, a.key0, a.key1);
                                const uint32_t rw4[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
#pragma unroll
                                for (int jj = 0; jj < 4; ++jj) {
                                    const int mm = mb * 4 + jj;
                                    if (mm < nq) {
                                        const int k = slice_of(P, q, mm);
                                        float e = flip_sign(h, bit_to_sign<W>(wi, k));
#pragma unroll
                                        for (int m = 0; m < MAXDEG; ++m)
                                            if (m < a.maxdeg) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], k)));
                                        const float t = __fadd_rn(flip_sign(jp, bit_to_sign<W>(dl, k)),
                                                                  flip_sign(jp, bit_to_sign<W>(dr, k)));
                                        const bool acc = decide(__fadd_rn(e, t), pq_u01(rw4[jj]), m2beta, m2blog2e);
                                        flips |= (W)acc << k;
                                        nacc += acc;
                                    }
                                }
                            }
                            rw[i] = wi ^ flips;
                            }
                        }
                        s += blockDim.x;
                        while (s >= S) { s -= S; ++rl; }
                    }
                    __syncthreads();
                }
            }
        }
        // world-line moves: flip spin i in every slice at once, classes in order
        for (int gm = 0; gm < a.global_moves; ++gm) {
            const uint32_t sweep = (uint32_t)(a.sweep_base + (int64_t)g * a.mcsteps + a.mcsteps - 1);
            for (int cls = 0; cls < a.nclass; ++cls) {
                int rl = 0, s = threadIdx.x;
                while (s >= S) { s -= S; ++rl; }
                for (; rl < nrep;) {
                    if (s < csize[cls]) {
                        const int i = cls * S + s;
                        W* rw = sw + rl * n;
                        const W wi = rw[i];
                        W d[MAXDEG];
                        float J[MAXDEG];
                        load_site<W, MAXDEG>(rw, i, n, a.maxdeg, nbr, cpl, wi, d, J, bad);
                        const float h = __ldg(field + i);
                        float E = 0.0f;
                        for (int k = 0; k < P; ++k) {
                            float e = flip_sign(h, bit_to_sign<W>(wi, k));
#pragma unroll
                            for (int m = 0; m < MAXDEG; ++m)
                                if (m < a.maxdeg) e = __fadd_rn(e, flip_sign(J[m], bit_to_sign<W>(d[m], k)));
                            E = __fadd_rn(E, e);
                        }
                        const uint32_t ctr2 = (uint32_t)(a.replica_base + r0 + rl);
                        const pq_u32x4 rnd = pq_philox(
                            pq_u32x4{(uint32_t)i, sweep, ctr2, (uint32_t)((1u << 24) | ((uint32_t)gm << 16) | (uint32_t)cls)},
                            a.key0, a.key1);
                        if (decide(E, pq_u01(rnd.x), m2beta, m2blog2e)) rw[i] = wi ^ mask;
                    }
                    s += blockDim.x;
                    while (s >= S) { s -= S; ++rl; }
                }
                __syncthreads();
            }
        }
    }

    for (int t = threadIdx.x; t < nrep * n; t += blockDim.x) words[(int64_t)r0 * n + t] = sw[t];
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
    if (accepts) {
        for (int off = 16; off > 0; off >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, off);
        if ((threadIdx.x & 31) == 0 && nacc) atomicAdd(accepts, nacc);
    }
}

// FP64 energy of one (replica, slice) per warp from the CSR of the coupling matrix.
template <typename W>
__global__ void energy_packed_kernel(const W* __restrict__ words, int n, int P, int R,
                                     const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                     const double* __restrict__ val, double* __restrict__ out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= R * P) return;
    const int r = warp / P, k = warp % P;
    const W* w = words + (int64_t)r * n;
    double acc = 0.0;
    for (int i = lane; i < n; i += 32) {
        const double si = ((w[i] >> k) & 1) ? -1.0 : 1.0;
        double rowsum = 0.0;
        for (int64_t e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
            const int j = col[e];
            const double sj = (j == i) ? 1.0 : ((((unsigned)j < (unsigned)n) && ((w[j] >> k) & 1)) ? -1.0 : 1.0);
            rowsum += val[e] * sj;
        }
        acc += si * rowsum;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) out[warp] = -acc;
}

template <typename W>
__global__ void pack_kernel(const int8_t* __restrict__ spins, int n, int P, int R, const int32_t* __restrict__ perm,
                            W* __restrict__ words, int stride) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)R * n) return;
    const int r = (int)(t / n), i = (int)(t % n);
    const int8_t* s = spins + t * P;
    W w = 0;
    for (int k = 0; k < P; ++k) w |= (W)(s[k] < 0) << k;
    const int di = perm ? perm[i] : i;
    if ((unsigned)di < (unsigned)stride) words[(int64_t)r * stride + di] = w;
}

template <typename W>
__global__ void unpack_kernel(const W* __restrict__ words, int n, int P, int R, const int32_t* __restrict__ perm,
                              int stride, int8_t* __restrict__ spins) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)R * n) return;
    const int r = (int)(t / n), i = (int)(t % n);
    const int di = perm ? perm[i] : i;
    const W w = (unsigned)di < (unsigned)stride ? words[(int64_t)r * stride + di] : (W)0;
    int8_t* s = spins + t * P;
    for (int k = 0; k < P; ++k) s[k] = ((w >> k) & 1) ? -1 : 1;
}

template <typename W, int MAXDEG, int NQC>
int launch_fast(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                const float* betas, const FastArgs& a, int threads, unsigned long long* accepts,
                int32_t* status, cudaStream_t stream) {
    const size_t smem = (size_t)a.rpc * a.n * sizeof(W);
    static bool attr_set = false;
    if (!attr_set) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(qa_fast_kernel<W, MAXDEG, NQC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         220 * 1024));
        attr_set = true;
    }
    const int grid = (a.R + a.rpc - 1) / a.rpc;
    qa_fast_kernel<W, MAXDEG, NQC><<<grid, threads, smem, stream>>>((W*)words, nbr, cpl, field, jperp, betas, a,
                                                                    accepts, status);
    return pq_launch_status();
}

template <typename W>
int dispatch_deg(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                 const float* betas, const FastArgs& a, int threads, unsigned long long* accepts,
                 int32_t* status, cudaStream_t stream) {
    if constexpr (sizeof(W) == 4) {
        // compile-time slice counts for the common even P with exactly four couplings
        if (a.maxdeg == 4) {
            if (a.P == 20) return launch_fast<W, 4, 10>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
            if (a.P == 16) return launch_fast<W, 4, 8>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
            if (a.P == 32) return launch_fast<W, 4, 16>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
        }
    }
    if (a.maxdeg <= 4)
        return launch_fast<W, 4, 0>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
    if (a.maxdeg <= 8)
        return launch_fast<W, 8, 0>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
    if (a.maxdeg <= 16)
        return launch_fast<W, 16, 0>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, stream);
    return PQ_ERR_UNSUPPORTED;
}

// FP32 FMA throughput probe: 8 independent chains per thread.
__global__ void fma_probe_kernel(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fmaf_rn(x0, a, b); x1 = __fmaf_rn(x1, a, b); x2 = __fmaf_rn(x2, a, b); x3 = __fmaf_rn(x3, a, b);
        x4 = __fmaf_rn(x4, a, b); x5 = __fmaf_rn(x5, a, b); x6 = __fmaf_rn(x6, a, b); x7 = __fmaf_rn(x7, a, b);
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1234.5f) out[blockIdx.x] = s;  // keeps the chains live
}

// Largest |ex2.approx(fl(x log2 e)) / expf_neg(x) - 1| over FP32 x with the given
// bit patterns (x >= -87, expf_neg(x) > 1e-30); atomic max on the bit pattern of a
// non-negative double.
__global__ void guard_probe_kernel(uint32_t first_bits, int64_t count, unsigned long long* out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double worst = 0.0;
    if (t < count) {
        const float x = __uint_as_float(first_bits + (uint32_t)t);
        if (x >= -87.0f && x <= 0.0f) {
            const float ps = pq_expf_neg(x);
            const float pf = pq_ex2_approx(__fmul_rn(x, 1.44269502162933349609375f));
            if (ps > 1e-30f) worst = fabs((double)pf / (double)ps - 1.0);
        }
    }
    for (int off = 16; off > 0; off >>= 1) worst = fmax(worst, __shfl_down_sync(0xffffffffu, worst, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(worst));
}

}  // namespace

extern "C" {

// Diagnostic: checks the accuracy the packed sweep's guard band relies on.
int pq_guard_band_probe(uint32_t first_bits, int64_t count, unsigned long long* out, void* stream) {
    if (!out || count < 0 || (uint64_t)first_bits + (uint64_t)count > 0x100000000ull) return PQ_ERR_INVALID_ARG;
    if (count == 0) return PQ_OK;
    guard_probe_kernel<<<(unsigned)((count + 255) / 256), 256, 0, (cudaStream_t)stream>>>(first_bits, count, out);
    return pq_launch_status();
}

// FP32 FMA peak probe: blocks x threads threads, each 8 x iters FMAs (2 flop each).
int pq_fp32_fma_probe(float* out, int iters, int blocks, int threads, void* stream) {
    if (!out || iters < 0 || blocks <= 0 || threads <= 0 || threads > 1024) return PQ_ERR_INVALID_ARG;
    fma_probe_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-6f);
    return pq_launch_status();
}


// Shared-memory budget of one CTA of the packed sweep.
static const size_t kSmemBudget = 200 * 1024;

int pq_qa_fast_ex(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                  const float* betas, const pq_fast_params* prm, unsigned long long* accepts, int32_t* status,
                  void* stream) {
    if (!prm || !words || !field || !jperp) return PQ_ERR_INVALID_ARG;
    const pq_fast_params& p = *prm;
    if (p.n <= 0 || p.R < 0 || p.P < 1 || p.nsched < 0 || p.mcsteps < 0 || p.global_moves < 0 || p.maxdeg < 0)
        return PQ_ERR_INVALID_ARG;
    if (p.P > 64 || p.maxdeg > 16) return PQ_ERR_UNSUPPORTED;
    if (p.maxdeg > 0 && (!nbr || !cpl)) return PQ_ERR_INVALID_ARG;
    if (p.nclass < 1 || p.nclass > kMaxClasses || p.class_stride < 1 || (int64_t)p.nclass * p.class_stride != p.n)
        return PQ_ERR_INVALID_ARG;
    for (int c = 0; c < p.nclass; ++c)
        if (p.class_size[c] < 0 || p.class_size[c] > p.class_stride) return PQ_ERR_INVALID_ARG;
    if (p.order_mode != 0 && p.order_mode != 1) return PQ_ERR_INVALID_ARG;
    if (p.R == 0 || p.nsched == 0) return PQ_OK;
    const size_t wbytes = p.P <= 32 ? 4 : 8;
    FastArgs a;
    a.n = p.n; a.P = p.P; a.R = p.R; a.maxdeg = p.maxdeg; a.nclass = p.nclass; a.stride = p.class_stride;
    a.order_mode = p.order_mode;
    for (int c = 0; c < kMaxClasses; ++c) a.class_size[c] = c < p.nclass ? p.class_size[c] : 0;
    a.nsched = p.nsched; a.mcsteps = p.mcsteps; a.global_moves = p.global_moves;
    a.beta = p.beta;
    a.key0 = (uint32_t)(p.seed & 0xffffffffu);
    a.key1 = (uint32_t)(p.seed >> 32);
    a.sweep_base = p.sweep_base;
    a.replica_base = p.replica_base;
    int threads = p.threads > 0 ? p.threads : 0;
    int rpc = p.replicas_per_cta;
    if (rpc <= 0) {
        // enough replicas per CTA to give every thread work, within the smem budget
        const int tgt = threads > 0 ? threads : 128;
        rpc = (tgt + p.class_stride - 1) / p.class_stride;
        if (rpc < 1) rpc = 1;
        const size_t cap = kSmemBudget / 2 / ((size_t)p.n * wbytes);
        if ((size_t)rpc > cap) rpc = cap < 1 ? 1 : (int)cap;
    }
    if (rpc > kMaxRpc) rpc = kMaxRpc;
    if (threads <= 0) {
        const int items = rpc * p.class_stride;
        threads = items >= 256 ? 256 : ((items + 31) / 32) * 32;
    }
    if (threads % 32 || threads > 512 || threads < rpc) return PQ_ERR_INVALID_ARG;
    if ((size_t)rpc * p.n * wbytes > kSmemBudget) return PQ_ERR_TOO_LARGE;
    a.rpc = rpc;
    cudaStream_t st = (cudaStream_t)stream;
    if (wbytes == 4) return dispatch_deg<uint32_t>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, st);
    return dispatch_deg<uint64_t>(words, nbr, cpl, field, jperp, betas, a, threads, accepts, status, st);
}

int pq_qa_fast(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
               const pq_fast_params* prm, unsigned long long* accepts, int32_t* status, void* stream) {
    return pq_qa_fast_ex(words, nbr, cpl, field, jperp, nullptr, prm, accepts, status, stream);
}

int pq_energy_packed(const void* words, int word_bits, int n, int P, int R, const int64_t* row_ptr,
                     const int32_t* col, const double* val, double* out, void* stream) {
    if (!words || !row_ptr || !out || n <= 0 || P < 1 || R < 0) return PQ_ERR_INVALID_ARG;
    if (!((word_bits == 32 && P <= 32) || (word_bits == 64 && P <= 64))) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    const int64_t warps = (int64_t)R * P;
    const unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (word_bits == 32)
        energy_packed_kernel<uint32_t><<<blocks, 256, 0, st>>>((const uint32_t*)words, n, P, R, row_ptr, col, val, out);
    else
        energy_packed_kernel<uint64_t><<<blocks, 256, 0, st>>>((const uint64_t*)words, n, P, R, row_ptr, col, val, out);
    return pq_launch_status();
}

int pq_pack_spins(const int8_t* spins, int n, int P, int R, const int32_t* perm, void* words, int word_bits,
                  int word_stride, void* stream) {
    if (!spins || !words || n <= 0 || P < 1 || R < 0 || word_stride < (perm ? 1 : n)) return PQ_ERR_INVALID_ARG;
    if (!((word_bits == 32 && P <= 32) || (word_bits == 64 && P <= 64))) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    const int64_t tot = (int64_t)R * n;
    const unsigned blocks = (unsigned)((tot + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (word_bits == 32) pack_kernel<uint32_t><<<blocks, 256, 0, st>>>(spins, n, P, R, perm, (uint32_t*)words, word_stride);
    else pack_kernel<uint64_t><<<blocks, 256, 0, st>>>(spins, n, P, R, perm, (uint64_t*)words, word_stride);
    return pq_launch_status();
}

int pq_unpack_spins(const void* words, int word_bits, int n, int P, int R, const int32_t* perm, int word_stride,
                    int8_t* spins, void* stream) {
    if (!spins || !words || n <= 0 || P < 1 || R < 0 || word_stride < (perm ? 1 : n)) return PQ_ERR_INVALID_ARG;
    if (!((word_bits == 32 && P <= 32) || (word_bits == 64 && P <= 64))) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    const int64_t tot = (int64_t)R * n;
    const unsigned blocks = (unsigned)((tot + 255) / 256);
    cudaStream_t st = (cudaStream_t)stream;
    if (word_bits == 32) unpack_kernel<uint32_t><<<blocks, 256, 0, st>>>((const uint32_t*)words, n, P, R, perm, word_stride, spins);
    else unpack_kernel<uint64_t><<<blocks, 256, 0, st>>>((const uint64_t*)words, n, P, R, perm, word_stride, spins);
    return pq_launch_status();
}

}  // extern "C"
