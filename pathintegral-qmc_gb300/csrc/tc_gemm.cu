// D[M][N] = alpha * A[M][K] * B[N][K]^T (+ bias[N]) with BF16 operands and FP32
// accumulation on the 5th-generation tensor cores.
//
// One CTA (4 warps) computes a 128 x BN tile through a ring of `kStages` shared-
// memory stages:
//  * warp 0 is the TMA producer: per K chunk of 64 it waits for the stage to be
//    free, arms the stage's "full" mbarrier with the chunk's byte count and issues
//    one two-dimensional TMA load (cp.async.bulk.tensor) of A (box 64 x 128) and
//    one of B (box 64 x BN), both with the 128-byte swizzle;
//  * warp 1 is the MMA issuer: it waits for "full", issues four tcgen05.mma
//    (K = 16 each, descriptors advanced by 32 B inside the swizzle atom) into the
//    TMEM accumulator and commits them to the stage's "empty" mbarrier, which hands
//    the stage back to the producer; a final commit signals "done";
//  * all four warps then read the accumulator with tcgen05.ld (warp w owns rows
//    32w..32w+31), apply D = alpha * acc + bias and write it into the (now free)
//    ring in 128-byte-swizzled 128 x 32 panels, which one thread stores with TMA
//    (cp.async.bulk.tensor, coalesced whatever the row stride of D).
// Stage layout: A then B, each [rows][64] BF16 as the TMA swizzle writes it (rows
// of 128 B, 8-row atoms of 1024 B), every stage 1024-byte aligned.
//
// Every wait is bounded: a wait that gives up sets PQ_ERR_TIMEOUT in `status`,
// stops the producer and the MMA issuer, waits (bounded) for the copies and MMAs
// already issued and frees TMEM before returning.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace {

constexpr int BM = 128;
constexpr int KC = 64;
constexpr long long kWaitIters = 1ll << 24;

template <int BN>
struct Cfg {
    static constexpr int kStages = BN == 256 ? 4 : 6;
    static constexpr int kStageA = BM * KC * 2;
    static constexpr int kStageB = BN * KC * 2;
    static constexpr int kStage = kStageA + kStageB;
    static constexpr int kBarOff = kStages * kStage;
    // + 1 KB so the ring can start on a 1024-byte boundary whatever the base alignment
    static constexpr int kSmem = kBarOff + (2 * kStages + 1) * 8 + 16 + 1024;
};

template <int BN>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB,
                                                         const __grid_constant__ CUtensorMap tmD, int K, float alpha,
                                                         const float* __restrict__ bias, int32_t* status) {
    using C = Cfg<BN>;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (tc::smem_addr(smem_raw) & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::kBarOff);
    uint64_t* empty = full + C::kStages;
    uint64_t* done = empty + C::kStages;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int nk = K / KC;
    const uint32_t base = tc::smem_addr(smem);

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::kStages; ++s) {
            tc::mbar_init(tc::smem_addr(full + s), 1);
            tc::mbar_init(tc::smem_addr(empty + s), 1);
        }
        tc::mbar_init(tc::smem_addr(done), 1);
        *abort_flag = 0;
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

    if (warp == 0) {
        // TMA producer
        int issued = 0;
        for (int c = 0; c < nk; ++c) {
            const int s = c % C::kStages;
            const uint32_t round = (uint32_t)(c / C::kStages);
            if (c >= C::kStages && !tc::mbar_wait(tc::smem_addr(empty + s), (round - 1) & 1u, kWaitIters)) {
                if (lane == 0) { *abort_flag = 1; pq_set_status(status, PQ_ERR_TIMEOUT); }
                break;
            }
            if (*abort_flag) break;
            if (lane == 0) {
                const uint32_t sa = base + s * C::kStage, sb = sa + C::kStageA, fb = tc::smem_addr(full + s);
                tc::mbar_arrive_expect_tx(fb, C::kStage);
                tc::tma_load_2d(sa, &tmA, c * KC, m0, fb);
                tc::tma_load_2d(sb, &tmB, c * KC, n0, fb);
            }
            issued = c + 1;
            __syncwarp();
        }
        if (*abort_flag && lane == 0) {
            // copies already issued land before the CTA lets go of its shared memory
            for (int c = issued - C::kStages < 0 ? 0 : issued - C::kStages; c < issued; ++c)
                tc::mbar_wait(tc::smem_addr(full + c % C::kStages), (uint32_t)(c / C::kStages) & 1u, kWaitIters);
        }
        __syncwarp();
    } else if (warp == 1) {
        // MMA issuer
        constexpr uint32_t idesc = tc::idesc_bf16(BM, BN);
        for (int c = 0; c < nk; ++c) {
            const int s = c % C::kStages;
            const uint32_t round = (uint32_t)(c / C::kStages);
            if (!tc::mbar_wait(tc::smem_addr(full + s), round & 1u, kWaitIters)) {
                if (lane == 0) { *abort_flag = 1; pq_set_status(status, PQ_ERR_TIMEOUT); }
                break;
            }
            if (*abort_flag) break;
            tc::fence_after_sync();
            if (lane == 0) {
                const uint32_t sa = base + s * C::kStage, sb = sa + C::kStageA;
#pragma unroll
                for (int kk = 0; kk < KC / 16; ++kk) {
                    const uint64_t ad = tc::smem_desc_sw128(sa + 32 * kk);
                    const uint64_t bd = tc::smem_desc_sw128(sb + 32 * kk);
                    tc::mma_bf16(tmem, ad, bd, idesc, (c > 0 || kk > 0) ? 1u : 0u);
                }
                tc::mma_commit(tc::smem_addr(empty + s));
            }
            __syncwarp();
        }
        // every MMA issued above completes before "done" (also on the abort path)
        if (lane == 0) tc::mma_commit(tc::smem_addr(done));
        __syncwarp();
    }

    const bool waited = tc::mbar_wait(tc::smem_addr(done), 0u, kWaitIters);
    tc::fence_after_sync();
    __syncthreads();
    if (!waited && threadIdx.x == 0) pq_set_status(status, PQ_ERR_TIMEOUT);
    const bool good = waited && !*abort_flag && nk > 0;
    if (good) {
        const int rl = 32 * warp + lane;   // row within the tile = TMEM lane
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
            // panel c0 / 32: [128 rows][32 floats], 16-byte unit u of row r at unit u ^ (r % 8)
            unsigned char* panel = smem + (c0 / 32) * (BM * 128);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int j = 4 * u;
                float4 o;
                o.x = alpha * v[j] + (bias ? bias[n0 + c0 + j] : 0.0f);
                o.y = alpha * v[j + 1] + (bias ? bias[n0 + c0 + j + 1] : 0.0f);
                o.z = alpha * v[j + 2] + (bias ? bias[n0 + c0 + j + 2] : 0.0f);
                o.w = alpha * v[j + 3] + (bias ? bias[n0 + c0 + j + 3] : 0.0f);
                *reinterpret_cast<float4*>(panel + rl * 128 + ((u ^ (rl & 7)) * 16)) = o;
            }
        }
        tc::fence_async_shared();
    }
    __syncthreads();
    if (good && threadIdx.x == 0) {
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 32) tc::tma_store_2d(&tmD, n0 + c0, m0, base + (c0 / 32) * (BM * 128));
        tc::tma_store_commit();
        tc::tma_store_wait_read();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, BN);
}

// Row-major [rows][ld] matrix of `esize`-byte elements (BF16 operands, FP32 result) of
// which the first `cols` columns are used, as a 2-D tensor map with a 128-byte-wide
// x box_rows box and the 128-byte swizzle.
int encode_map(CUtensorMap* map, const void* ptr, int rows, int cols, int ld, int box_rows, int esize = 2) {
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * esize};
    const cuuint32_t box[2] = {(cuuint32_t)(128 / esize), (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1u, 1u};
    // the driver's encoder, looked up through the runtime so the library does not link libcuda
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        PQ_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) return PQ_ERR_NO_DEVICE;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const CUresult r = encode(map, esize == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                              const_cast<void*>(ptr), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? PQ_OK : PQ_ERR_INVALID_ARG;
}

template <int BN>
int launch_gemm(const void* A, int lda, const void* B, int ldb, float* D, int ldd, int M, int N, int K, float alpha,
                const float* bias, int32_t* status, cudaStream_t stream) {
    using C = Cfg<BN>;
    static_assert(BN / 32 * BM * 128 <= C::kBarOff, "the result panels fit in the ring");
    CUtensorMap ta, tb;
    int rc = encode_map(&ta, A, M, K, lda, BM);
    if (rc != PQ_OK) return rc;
    rc = encode_map(&tb, B, N, K, ldb, BN);
    if (rc != PQ_OK) return rc;
    CUtensorMap td;
    rc = encode_map(&td, D, M, N, ldd, BM, 4);
    if (rc != PQ_OK) return rc;
    static PqSmemAttr attr;
    rc = pq_set_smem_limit(attr, (const void*)tc_gemm_kernel<BN>, C::kSmem);
    if (rc != PQ_OK) return rc;
    dim3 grid(M / BM, N / BN);
    tc_gemm_kernel<BN><<<grid, 128, C::kSmem, stream>>>(ta, tb, td, K, alpha, bias, status);
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
    // the widest tile that divides N and still gives the SMs something to do
    const int tiles256 = (N % 256 == 0) ? (M / BM) * (N / 256) : 0;
    if (tiles256 >= 128) return launch_gemm<256>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
    const int tiles128 = (N % 128 == 0) ? (M / BM) * (N / 128) : 0;
    if (tiles128 >= 128) return launch_gemm<128>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
    return launch_gemm<64>(A, lda, B, ldb, D, ldd, M, N, K, alpha, bias, status, st);
}

}  // extern "C"
