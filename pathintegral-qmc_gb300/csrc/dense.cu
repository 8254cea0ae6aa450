// Dense-J packed sweep (qmc.QuantumAnneal_dense physics, reference
// piqmc/qmc.pyx:141-242, with both quirks corrected): local fields kept in
// shared memory and updated by rank-1 corrections on every accepted flip;
// periodically recomputed from scratch on the tensor cores (split-BF16 GEMM,
// see piqmc/dense.py).
//
// Every spin couples to every other, so within a Trotter slice the updates are
// sequential; the parallelism is across the slices of one slice class (one
// warp per slice) and across replicas (one CTA per replica).  Within a slice the
// warp still decides 32 positions at once: a decision reads only its own spin's
// field, so all open positions decide from the current fields, the first accepted
// one is final, its rank-1 update is applied, and the positions after it decide
// again; rejected positions cost one lane each instead of a warp each.
//
// Specification of one sweep of replica r (sweep counter `sweep`):
//  * slice classes as in the sparse sweep; warp w handles slice k = 2w + q of
//    class q (slice P-1 alone for the third class of odd P);
//  * spin order of slice k: i_t = (a t + b) mod N, t = 0..N-1, with
//    (w0, w1) = Philox(ctr = {0xFFFFFFFE, sweep, replica, 3 << 24 | kk}) words 0, 1,
//    a = units[w0 % nunits] (a unit mod N), b = w1 % N; kk = 0 (one order shared by
//    every slice of the sweep, as the reference shares its permutation) unless
//    per-slice orders are requested (kk = k: anneals faster, dynamics differ);
//  * update of spin i in slice k (FP32, one rounding per op, in order):
//    e = s_i f_i (f = h + sum_j K_ij s_j, the stored field), t = J-perp s_i s_{k-1}
//    + J-perp s_i s_{k+1}, sum = e + t; flip when sum < 0, else when
//    u < expf_neg(fl(sum * (-2 beta))), u = ((r >> 9) + 1/2) 2^-23 with r = word t & 3 of
//    Philox(ctr = {k, sweep, replica, 4 << 24 | t >> 2});
//  * on a flip, f_j <- fma(2 s_i_new, K_ij, f_j) for every j (K_ii = 0).
#include <cuda_bf16.h>

#include "common.cuh"
#include "sweep_core.cuh"

namespace {

using namespace pq;

struct DenseArgs {
    int N, P, R, nunits, ldf, per_slice_order;
    int nsched, mcsteps;
    float beta;
    uint32_t key0, key1;
    int64_t sweep_base;
    int replica_base;
    long long poll_limit;   // polls of a neighbour's progress before a wait gives up
    int wait_skew;          // added to every awaited progress count (0; > 0 only to test the timeout)
};

// One sweep of slice k of the replica whose fields sf and world-lines sw are in
// shared memory (the specification above), run by one warp; returns the accepted
// flips.
__device__ __forceinline__ unsigned long long sweep_slice(int k, uint32_t sweep, float jp, float m2beta,
                                                          float m2blog2e, float* __restrict__ sf,
                                                          uint32_t* __restrict__ sw, const float* __restrict__ K,
                                                          const int32_t* __restrict__ units, const DenseArgs& a,
                                                          uint32_t rep, int lane) {
    const int N = a.N, P = a.P;
    unsigned long long nacc = 0;
    const uint32_t kk = a.per_slice_order ? (uint32_t)k : 0u;
    const pq_u32x4 ord = pq_philox(pq_u32x4{0xFFFFFFFEu, sweep, rep, (3u << 24) | kk}, a.key0, a.key1);
    const uint32_t am = (uint32_t)__ldg(units + ord.x % (uint32_t)a.nunits);
    const uint32_t bm = ord.y % (uint32_t)N;
    float* fk = sf + (size_t)k * N;
    const int kl = k == 0 ? P - 1 : k - 1, kr = k == P - 1 ? 0 : k + 1;
    // positions are taken 32 at a time, lane l holding position t0 + l: all open
    // positions decide at once from the current fields; the first accepted one is
    // final, its rank-1 update is applied, and the positions after it decide
    // again -- the same decisions, in the same order of updates, as one spin at a time
    const uint32_t off_l = ((uint32_t)lane * am) % (uint32_t)N;     // (l a) mod N
    const uint32_t a32 = (32u * am) % (uint32_t)N;
    uint32_t i0 = bm;                                                // i_{t0}
    pq_u32x4 mine{0, 0, 0, 0};
    for (int t0 = 0; t0 < N; t0 += 32) {
        if ((t0 & 127) == 0)
            mine = pq_philox(pq_u32x4{(uint32_t)k, sweep, rep, (4u << 24) | (uint32_t)((t0 >> 2) + lane)},
                             a.key0, a.key1);
        // position t = t0 + lane uses word t & 3 of Philox block t >> 2
        const int src = ((t0 & 127) >> 2) + (lane >> 2);
        const uint32_t wx = __shfl_sync(0xffffffffu, mine.x, src);
        const uint32_t wy = __shfl_sync(0xffffffffu, mine.y, src);
        const uint32_t wz = __shfl_sync(0xffffffffu, mine.z, src);
        const uint32_t ww = __shfl_sync(0xffffffffu, mine.w, src);
        const uint32_t comp = (lane & 3) == 0 ? wx : (lane & 3) == 1 ? wy : (lane & 3) == 2 ? wz : ww;
        const float u = pq_u01(comp);
        const int nb = min(32, N - t0);
        uint32_t i = i0 + off_l;
        if (i >= (uint32_t)N) i -= (uint32_t)N;
        float tt = 0.0f;
        uint32_t sbit = 0;
        if (lane < nb) {
            const uint32_t wi = sw[i];
            sbit = (wi >> k) & 1u;
            tt = __fadd_rn(flip_sign(jp, (((wi >> k) ^ (wi >> kl)) & 1u) << 31),
                           flip_sign(jp, (((wi >> k) ^ (wi >> kr)) & 1u) << 31));
        }
        int start = 0;
        while (start < nb) {
            bool acc = false;
            if (lane >= start && lane < nb)
                acc = decide(__fadd_rn(flip_sign(fk[i], sbit << 31), tt), u, m2beta, m2blog2e);
            const uint32_t hit = __ballot_sync(0xffffffffu, acc);
            if (!hit) break;
            const int p = __ffs(hit) - 1;
            const uint32_t ip = __shfl_sync(0xffffffffu, i, p);
            const uint32_t sp = __shfl_sync(0xffffffffu, sbit, p);
            // new spin = -old: s_new = +1 when the old bit was set (old spin -1)
            const float c = sp ? 2.0f : -2.0f;
            const float* Ki = K + (size_t)ip * N;
            if (N <= 512) {
                // all row loads in flight at once, then the updates
                float kv[16];
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                    const int j = lane + 32 * m;
                    kv[m] = j < N ? __ldg(Ki + j) : 0.0f;
                }
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                    const int j = lane + 32 * m;
                    if (j < N) fk[j] = __fmaf_rn(c, kv[m], fk[j]);
                }
            } else {
                for (int j = lane; j < N; j += 32) fk[j] = __fmaf_rn(c, __ldg(Ki + j), fk[j]);
            }
            if (lane == 0) atomicXor(sw + ip, 1u << k);
            ++nacc;
            __syncwarp();
            start = p + 1;
        }
        i0 += a32;
        if (i0 >= (uint32_t)N) i0 -= (uint32_t)N;
    }
    return nacc;
}

constexpr long long kWaveWait = 1ll << 24;   // default polls of a neighbour's progress before giving up

// Wait until *flag >= need for every lane (each lane reads the flag itself, then
// fences, so the producer's shared-memory writes before its release are visible).
// Gives up (false) after `limit` unsuccessful polls.
__device__ __forceinline__ bool wait_progress(const volatile int* flag, int need, long long limit) {
    for (long long it = 0;; ++it) {
        if (__all_sync(0xffffffffu, *flag >= need)) {
            __threadfence_block();
            return true;
        }
        if (it >= limit) return false;
        __nanosleep(64);
    }
}

__global__ void __launch_bounds__(512, 2) dense_sweep_kernel(uint32_t* __restrict__ words, float* __restrict__ F,
                                                           const float* __restrict__ K, const int32_t* __restrict__ units,
                                                           const float* __restrict__ jperp, DenseArgs a,
                                                           unsigned long long* __restrict__ accepts,
                                                           int32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int prog[2][32];   // slice phases completed: [class][warp]
    const int N = a.N, P = a.P;
    float* sf = reinterpret_cast<float*>(smem);                       // [P][N] fields
    uint32_t* sw = reinterpret_cast<uint32_t*>(sf + (size_t)P * N);    // [N] world-lines
    const int r = blockIdx.x;
    const uint32_t rep = (uint32_t)(a.replica_base + r);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = threadIdx.x; t < P * N; t += blockDim.x) {
        const int k = t / N, i = t - k * N;
        sf[t] = F[(size_t)(r * P + k) * a.ldf + i];
    }
    for (int t = threadIdx.x; t < N; t += blockDim.x) sw[t] = words[(size_t)r * N + t];
    if (threadIdx.x < 64) prog[threadIdx.x >> 5][threadIdx.x & 31] = 0;
    __syncthreads();
    unsigned long long nacc = 0;
    const float m2beta = __fmul_rn(-2.0f, a.beta);
    const float m2blog2e = __fmul_rn(m2beta, 1.44269502162933349609375f);
    if (P >= 2 && (P & 1) == 0) {
        // Even P: warp w owns slices 2w (even class) and 2w + 1 (odd class) and runs them in
        // turn; a slice only waits for its two Trotter neighbours' previous phases (slice 2w
        // for warp w - 1's odd slice, slice 2w + 1 for warp w + 1's even slice), so the warps
        // run as a wavefront instead of meeting at a CTA barrier after every slice class.
        // The sweeps, and so the results, are the slice-class-by-slice-class ones.
        const int W = P / 2, w = warp;
        const int wl = (w + W - 1) % W, wr = (w + 1) % W;
        volatile int* vprog = &prog[0][0];
        bool ok = true;
        int n = 0;
        for (int g = 0; g < a.nsched && ok; ++g) {
            const float jp = jperp[g];
            for (int step = 0; step < a.mcsteps && ok; ++step, ++n) {
                const uint32_t sweep = (uint32_t)(a.sweep_base + (int64_t)g * a.mcsteps + step);
                if (!(ok = wait_progress(vprog + 32 + wl, n + a.wait_skew, a.poll_limit))) break;
                nacc += sweep_slice(2 * w, sweep, jp, m2beta, m2blog2e, sf, sw, K, units, a, rep, lane);
                __syncwarp();
                __threadfence_block();
                if (lane == 0) vprog[w] = n + 1;
                if (!(ok = wait_progress(vprog + wr, n + 1 + a.wait_skew, a.poll_limit))) break;
                nacc += sweep_slice(2 * w + 1, sweep, jp, m2beta, m2blog2e, sf, sw, K, units, a, rep, lane);
                __syncwarp();
                __threadfence_block();
                if (lane == 0) vprog[32 + w] = n + 1;
            }
        }
        if (!ok) {
            pq_set_status(status, PQ_ERR_TIMEOUT);
            // release the neighbours that wait on this warp
            if (lane == 0) { vprog[w] = 1 << 30; vprog[32 + w] = 1 << 30; }
        }
    } else {
        const int nclass_q = P == 1 ? 1 : 3;
        for (int g = 0; g < a.nsched; ++g) {
            const float jp = P == 1 ? 0.0f : jperp[g];
            for (int step = 0; step < a.mcsteps; ++step) {
                const uint32_t sweep = (uint32_t)(a.sweep_base + (int64_t)g * a.mcsteps + step);
                for (int q = 0; q < nclass_q; ++q) {
                    if (warp < slice_count(P, q))
                        nacc += sweep_slice(slice_of(P, q, warp), sweep, jp, m2beta, m2blog2e, sf, sw, K, units, a,
                                            rep, lane);
                    __syncthreads();
                }
            }
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < N; t += blockDim.x) words[(size_t)r * N + t] = sw[t];
    for (int t = threadIdx.x; t < P * N; t += blockDim.x) {
        const int k = t / N, i = t - k * N;
        F[(size_t)(r * P + k) * a.ldf + i] = sf[t];
    }
    if (accepts && lane == 0 && nacc) atomicAdd(accepts, nacc);   // nacc is warp-uniform
}

// words [R][N] (bits = slices) -> BF16 +-1 rows [R*P (padded to Mpad)][2 Npad]: row c = r*P + k holds
// s_k over spins j twice (columns j and Npad + j), zeros for padding.
__global__ void dense_unpack_kernel(const uint32_t* __restrict__ words, int N, int P, int R, int Npad, int Mpad,
                                    __nv_bfloat16* __restrict__ A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)Mpad * Npad;
    if (t >= total) return;
    const int c = (int)(t / Npad), j = (int)(t % Npad);
    float v = 0.0f;
    if (c < R * P && j < N) {
        const int r = c / P, k = c % P;
        v = ((words[(size_t)r * N + j] >> k) & 1u) ? -1.0f : 1.0f;
    }
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    A[(size_t)c * 2 * Npad + j] = b;
    A[(size_t)c * 2 * Npad + Npad + j] = b;
}

}  // namespace

extern "C" {

int pq_dense_unpack_bf16(const uint32_t* words, int N, int P, int R, int Npad, int Mpad, void* A, void* stream) {
    if (!words || !A || N <= 0 || P < 1 || P > 32 || R <= 0 || Npad < N || Mpad < R * P) return PQ_ERR_INVALID_ARG;
    const int64_t total = (int64_t)Mpad * Npad;
    dense_unpack_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(words, N, P, R, Npad, Mpad,
                                                                                            (__nv_bfloat16*)A);
    return pq_launch_status();
}

int pq_dense_sweep_ex(uint32_t* words, float* F, int ldf, const float* K, const int32_t* units, int nunits,
                      const float* jperp, int N, int P, int R, int nsched, int mcsteps, float beta, uint64_t seed,
                      int64_t sweep_base, int replica_base, int per_slice_order, int64_t poll_limit, int wait_skew,
                      unsigned long long* accepts, int32_t* status, void* stream) {
    if (!words || !F || !K || !units || !jperp || N <= 0 || P < 1 || P > 32 || R < 0 || nsched < 0 || mcsteps < 0 ||
        nunits <= 0 || ldf < N || wait_skew < 0 || wait_skew > (1 << 24))
        return PQ_ERR_INVALID_ARG;
    if (R == 0 || nsched == 0) return PQ_OK;
    const size_t smem = (size_t)P * N * 4 + (size_t)N * 4;
    if (smem > 220 * 1024) return PQ_ERR_TOO_LARGE;
    static PqSmemAttr attr;
    const int rc = pq_set_smem_limit(attr, (const void*)dense_sweep_kernel, 220 * 1024);
    if (rc != PQ_OK) return rc;
    DenseArgs a;
    a.N = N; a.P = P; a.R = R; a.nunits = nunits; a.ldf = ldf; a.per_slice_order = per_slice_order ? 1 : 0; a.nsched = nsched; a.mcsteps = mcsteps; a.beta = beta;
    a.key0 = (uint32_t)seed; a.key1 = (uint32_t)(seed >> 32); a.sweep_base = sweep_base; a.replica_base = replica_base;
    a.poll_limit = poll_limit < 0 ? kWaveWait : poll_limit;
    a.wait_skew = wait_skew;
    const int maxq = P == 1 ? 1 : (P + 1) / 2;
    const int threads = 32 * maxq;
    dense_sweep_kernel<<<R, threads, smem, (cudaStream_t)stream>>>(words, F, K, units, jperp, a, accepts, status);
    return pq_launch_status();
}

int pq_dense_sweep(uint32_t* words, float* F, int ldf, const float* K, const int32_t* units, int nunits,
                   const float* jperp, int N, int P, int R, int nsched, int mcsteps, float beta, uint64_t seed,
                   int64_t sweep_base, int replica_base, int per_slice_order, unsigned long long* accepts,
                   int32_t* status, void* stream) {
    return pq_dense_sweep_ex(words, F, ldf, K, units, nunits, jperp, N, P, R, nsched, mcsteps, beta, seed, sweep_base,
                             replica_base, per_slice_order, -1, 0, accepts, status, stream);
}

}  // extern "C"
