// D[M][N] = A[M][K] * B[N][K]^T with BF16 operands and FP32 accumulation on the
// 5th-generation tensor cores (tcgen05.mma, accumulator in TMEM).
//
// One CTA (4 warps) computes a 128 x BN tile.  For every K chunk of 64 the
// warps copy the A and B tiles into shared memory in the K-major no-swizzle
// layout of tc_gemm.cuh, one thread issues four K = 16 MMAs and commits them to
// an mbarrier, and all threads wait (bounded) before the buffers are reused.
// The epilogue reads the accumulator with tcgen05.ld (warp w owns rows
// 32w..32w+31) and applies D = alpha * acc + (bias[col] if bias).
#include "common.cuh"
#include "tc_gemm.cuh"

namespace {

constexpr int BM = 128;
constexpr int KC = 64;
constexpr long long kWaitIters = 1ll << 24;

template <int BN>
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __nv_bfloat16* __restrict__ A, int lda,
                                                      const __nv_bfloat16* __restrict__ B, int ldb,
                                                      float* __restrict__ D, int ldd, int K, float alpha,
                                                      const float* __restrict__ bias, int32_t* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;
    unsigned char* sB = smem + BM * KC * 2;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sB + BN * KC * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_addr(mbar), 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_addr(tslot), BN);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    constexpr uint32_t idesc = tc::idesc_bf16(BM, BN);

    uint32_t phase = 0;
    bool ok = true;
    for (int k0 = 0; k0 < K && ok; k0 += KC) {
        for (int c = threadIdx.x; c < BM * (KC / 8); c += blockDim.x) {
            const int r = c / (KC / 8), kk = (c % (KC / 8)) * 8;
            const uint4 v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + k0 + kk);
            *reinterpret_cast<uint4*>(sA + tc::tile_off(r, kk, KC)) = v;
        }
        for (int c = threadIdx.x; c < BN * (KC / 8); c += blockDim.x) {
            const int r = c / (KC / 8), kk = (c % (KC / 8)) * 8;
            const uint4 v = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * ldb + k0 + kk);
            *reinterpret_cast<uint4*>(sB + tc::tile_off(r, kk, KC)) = v;
        }
        tc::fence_async_shared();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int s = 0; s < KC / 16; ++s) {
                const uint64_t ad = tc::smem_desc(tc::smem_addr(sA) + s * 256, 128, KC * 16);
                const uint64_t bd = tc::smem_desc(tc::smem_addr(sB) + s * 256, 128, KC * 16);
                tc::mma_bf16(tmem, ad, bd, idesc, (k0 > 0 || s > 0) ? 1u : 0u);
            }
            tc::mma_commit(tc::smem_addr(mbar));
        }
        if (!tc::mbar_wait(tc::smem_addr(mbar), phase, kWaitIters)) ok = false;
        phase ^= 1u;
        tc::fence_after_sync();
    }
    if (ok) {
        const int row = m0 + 32 * warp + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            float* dst = D + (size_t)row * ldd + n0 + c0;
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                float4 o;
                o.x = alpha * v[j] + (bias ? bias[n0 + c0 + j] : 0.0f);
                o.y = alpha * v[j + 1] + (bias ? bias[n0 + c0 + j + 1] : 0.0f);
                o.z = alpha * v[j + 2] + (bias ? bias[n0 + c0 + j + 2] : 0.0f);
                o.w = alpha * v[j + 3] + (bias ? bias[n0 + c0 + j + 3] : 0.0f);
                *reinterpret_cast<float4*>(dst + j) = o;
            }
        }
    } else {
        pq_set_status(status, PQ_ERR_TIMEOUT);
        // give the MMAs in flight one more bounded chance to land before freeing TMEM
        tc::mbar_wait(tc::smem_addr(mbar), phase ^ 1u, kWaitIters);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, BN);
}

template <int BN>
int launch_gemm(const void* A, int lda, const void* B, int ldb, float* D, int ldd, int M, int N, int K, float alpha,
                const float* bias, int32_t* status, cudaStream_t stream) {
    // shared memory sized so that at most 512 / BN CTAs share an SM's TMEM
    size_t smem = (size_t)(BM + BN) * KC * 2 + 16;
    const size_t floor_bytes = BN == 256 ? 80 * 1024 : (BN == 128 ? 60 * 1024 : 29 * 1024);
    if (smem < floor_bytes) smem = floor_bytes;
    static bool attr = false;
    if (!attr) {
        PQ_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr = true;
    }
    dim3 grid(M / BM, N / BN);
    tc_gemm_kernel<BN><<<grid, 128, smem, stream>>>((const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)B, ldb, D,
                                                    ldd, K, alpha, bias, status);
    return pq_launch_status();
}

}  // namespace

extern "C" {

int pq_tc_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* D, int ldd, int M, int N, int K,
                    float alpha, const float* bias, int32_t* status, void* stream) {
    if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0) return PQ_ERR_INVALID_ARG;
    if (M % BM || N % 64 || K % KC || lda % 8 || ldb % 8 || ldd % 4 || lda < K || ldb < K || ldd < N)
        return PQ_ERR_INVALID_ARG;
    if (((uintptr_t)A | (uintptr_t)B) & 15 || ((uintptr_t)D & 15)) return PQ_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (N % 256 == 0) return launch_gemm<256>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
    if (N % 128 == 0) return launch_gemm<128>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
    return launch_gemm<64>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
}

}  // extern "C"
