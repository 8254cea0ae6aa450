// Shared device helpers: status words, Philox4x32-10, the sweep's own exp.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "piqmc_gb300.h"

#define PQ_CUDA_TRY(expr)                                 \
    do {                                                  \
        cudaError_t e_ = (expr);                          \
        if (e_ != cudaSuccess) return -(int)e_;           \
    } while (0)

static inline int pq_launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PQ_OK : -(int)e;
}

// ----------------------------------------------------------------------------
// Per-device state.  Kernel attributes, symbol addresses and occupancy belong to
// one device context, so caches of them are keyed by the device ordinal and
// checked against the identity of the context they were made in: a process that
// drives a second GPU, or that resets a device (a new primary context), redoes
// the set-up instead of using a stale value.
// ----------------------------------------------------------------------------
constexpr int kPqMaxDevices = 64;

// Identity of the calling thread's current context, unique for the process's
// lifetime (the driver's cuCtxGetId, looked up through the runtime so the
// library needs no link-time driver dependency); 0 when there is none yet.
inline unsigned long long pq_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(p);
    });
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id + 1;   // 0 stays "unknown"
}

// A kernel's dynamic shared-memory limit, set once per device context.
struct PqSmemAttr {
    std::atomic<unsigned long long> ctx[kPqMaxDevices] = {};
};

inline int pq_set_smem_limit(PqSmemAttr& cache, const void* kernel, int bytes) {
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    const bool slot = dev >= 0 && dev < kPqMaxDevices;
    const unsigned long long id = pq_context_id();
    if (slot && id && cache.ctx[dev].load(std::memory_order_acquire) == id) return PQ_OK;
    PQ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    const unsigned long long now = pq_context_id();   // the call above made the context current
    if (slot && now) cache.ctx[dev].store(now, std::memory_order_release);
    return PQ_OK;
}

// First error wins; later ones are dropped.
__device__ __forceinline__ void pq_set_status(int32_t* status, int code) {
    if (status) atomicCAS(status, 0, code);
}

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of the 4x32 Philox S-box with the published
// multipliers and Weyl key increments.
// ----------------------------------------------------------------------------
struct pq_u32x4 { uint32_t x, y, z, w; };

__device__ __forceinline__ pq_u32x4 pq_philox(pq_u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = pq_u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Round keys of Philox4x32-10: round r uses (k0 + r * 0x9E3779B9, k1 + r * 0xBB67AE85).
// PhiloxKeysReg derives them from the key pair in registers; PhiloxKeysTab reads a
// precomputed table (placed in kernel-parameter space it folds into the XORs as
// constant operands).  Both give pq_philox's values.
struct PhiloxKeyTable {
    uint32_t a[10], b[10];
};
struct PhiloxKeysReg {
    uint32_t k0, k1;
    __device__ __forceinline__ uint32_t ka(int r) const { return k0 + (uint32_t)r * 0x9E3779B9u; }
    __device__ __forceinline__ uint32_t kb(int r) const { return k1 + (uint32_t)r * 0xBB67AE85u; }
};
struct PhiloxKeysTab {
    const PhiloxKeyTable& t;
    __device__ __forceinline__ uint32_t ka(int r) const { return t.a[r]; }
    __device__ __forceinline__ uint32_t kb(int r) const { return t.b[r]; }
};
inline PhiloxKeyTable pq_philox_key_table(uint32_t k0, uint32_t k1) {
    PhiloxKeyTable t;
    for (int r = 0; r < 10; ++r) {
        t.a[r] = k0 + (uint32_t)r * 0x9E3779B9u;
        t.b[r] = k1 + (uint32_t)r * 0xBB67AE85u;
    }
    return t;
}

template <typename KS>
__device__ __forceinline__ pq_u32x4 pq_philox_ks(pq_u32x4 c, const KS& ks) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = pq_u32x4{hi1 ^ c.y ^ ks.ka(r), lo1, hi0 ^ c.w ^ ks.kb(r), lo0};
    }
    return c;
}

// Uniform on the midpoints of 2^23 equal cells of (0, 1): u = ((r >> 9) + 1/2) * 2^-23 =
// (2 (r >> 9) + 1) * 2^-24, computed exactly as (1 + (r >> 9) * 2^-23) - (1 - 2^-24).
// Its smallest value is 2^-24, so a Metropolis test u < p with p <= 2^-24 rejects
// whatever r is: such decisions need no random number.
__device__ __forceinline__ float pq_u01(uint32_t r) {
    return __fsub_rn(__uint_as_float((r >> 9) | 0x3f800000u), 0.999999940395355224609375f);
}

// Hardware 2^x approximation (MUFU), used only inside a guard band that makes the
// final decision independent of its exact rounding.
__device__ __forceinline__ float pq_ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ----------------------------------------------------------------------------
// exp(x) for x <= 0, written for bit-identical results on the GPU and in the CPU
// restatement of the fast sweep (every step is one IEEE-rounded FP32 op or an
// fma, in a fixed order):
//   n = rint(x * log2(e));  r = x - n*ln2 (two-constant Cody-Waite split,
//   ln2 = LN2_HI + LN2_LO with LN2_HI = 0xB17200 * 2^-24 exact in 16 bits);
//   exp(r) by its Taylor series to degree 7 (|r| <= ln2/2, truncation < 5e-9
//   relative); result = poly * 2^n built from exponent bits.
// Inputs below -87 return 0 (exp(-87) < 1.7e-38: below every nonzero 24-bit
// uniform, so only u == 0 could tell the difference).
// ----------------------------------------------------------------------------
__device__ __forceinline__ float pq_expf_neg(float x) {
    if (!(x >= -87.0f)) return 0.0f;
    const float LOG2E = 1.44269502162933349609375f;   // log2(e) rounded to FP32
    const float LN2_HI = 0.693145751953125f;          // 0xB17200p-24
    const float LN2_LO = 1.428606765330187045e-06f;   // ln2 - LN2_HI rounded to FP32
    const float t = __fmul_rn(x, LOG2E);
    const float nf = rintf(t);
    float r = __fmaf_rn(-nf, LN2_HI, x);
    r = __fmaf_rn(-nf, LN2_LO, r);
    // 1/k! for k = 7..2, rounded to FP32
    float p = 1.98412701138295233249664306640625e-04f;       // 1/5040
    p = __fmaf_rn(p, r, 1.388888922519981861114501953125e-03f);  // 1/720
    p = __fmaf_rn(p, r, 8.333333767950534820556640625e-03f);     // 1/120
    p = __fmaf_rn(p, r, 4.16666679084300994873046875e-02f);      // 1/24
    p = __fmaf_rn(p, r, 1.666666716337203979492187500e-01f);     // 1/6
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    const int n = (int)nf;                               // in [-126, 0]
    return __fmul_rn(p, __int_as_float((n + 127) << 23));
}
