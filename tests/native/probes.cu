// Measurement instruments of the tests and the bench -- not part of the product
// library (built separately into tests/native/_build/libpiqmc_probes.so).
//
//  * pqt_fp32_fma_probe: FP32 FMA throughput of this GPU, the denominator of the
//    packed sweep's FP32 roofline (no measured FP32 peak exists otherwise).
//  * pqt_guard_band_probe: the largest relative deviation of the hardware 2^x from
//    the sweep's own expf_neg over a range of FP32 arguments, the bound the
//    packed sweep's exact guard band relies on.
//  * pqt_settle_threshold: the per-step threshold of the quiet-site rule of the
//    packed sweep (pq::settle_threshold), for checking against FP32 arithmetic.
#include "sweep_core.cuh"

namespace {

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

__global__ void settle_threshold_kernel(const float* betas, int count, float* out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) out[t] = pq::settle_threshold(__fmul_rn(-2.0f, betas[t]));
}

}  // namespace

extern "C" {

// The quiet-site threshold of each beta: the smallest s >= 0 with fl(s * -2 beta) <= -16.63553237915039.
int pqt_settle_threshold(const float* betas, int count, float* out, void* stream) {
    if (!betas || !out || count < 0) return PQ_ERR_INVALID_ARG;
    if (count == 0) return PQ_OK;
    settle_threshold_kernel<<<(count + 127) / 128, 128, 0, (cudaStream_t)stream>>>(betas, count, out);
    return pq_launch_status();
}

// Diagnostic: checks the accuracy the packed sweep's guard band relies on.
int pqt_guard_band_probe(uint32_t first_bits, int64_t count, unsigned long long* out, void* stream) {
    if (!out || count < 0 || (uint64_t)first_bits + (uint64_t)count > 0x100000000ull) return PQ_ERR_INVALID_ARG;
    if (count == 0) return PQ_OK;
    guard_probe_kernel<<<(unsigned)((count + 255) / 256), 256, 0, (cudaStream_t)stream>>>(first_bits, count, out);
    return pq_launch_status();
}

// FP32 FMA peak probe: blocks x threads threads, each 8 x iters FMAs (2 flop each).
int pqt_fp32_fma_probe(float* out, int iters, int blocks, int threads, void* stream) {
    if (!out || iters < 0 || blocks <= 0 || threads <= 0 || threads > 1024) return PQ_ERR_INVALID_ARG;
    fma_probe_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-6f);
    return pq_launch_status();
}

}  // extern "C"
