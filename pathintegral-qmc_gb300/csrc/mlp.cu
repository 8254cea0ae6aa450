// Learned world-line proposals: per-spin features, the MLP's element-wise
// parts (the 64 x 64 layers run on the tensor cores through pq_tc_gemm_bf16),
// the Metropolis-Hastings world-line move, and the training kernels.
//
// Features of spin i of a replica (P slices, local fields f^k = h_i + sum_j J_ij
// s_j^k from its neighbours, which belong to other update classes):
//   x0 = mean_k f^k / (1 + sum_m |J_im| + |h_i|)   (normalised local field)
//   x1 = std_k f^k / (same scale)
//   x2 = mean_k s^k                                (world-line magnetisation)
//   x3 = #{k : s^k != s^{k+1}} / P                 (slice disagreements, periodic)
//   x4 = mean_k s^k f^k / (same scale)             (alignment; the flip costs 2 P x4 scale)
//   x5 = beta * (classical flip cost) / P, clipped to [-8, 8]
//   x6 = J-perp * beta / P, clipped to [0, 8]      (how stiff the world-lines are)
//   x7 = 1                                         (bias input)
// The flipped world-line (s -> -s in every slice) has x2, x4, x5 negated and the
// rest unchanged; both versions are scored in one pass (rows i and M + i).
#include <cuda_bf16.h>

#include "common.cuh"
#include "sweep_core.cuh"

namespace {

using namespace pq;

constexpr int kFeat = 8;
constexpr int kLd = 64;  // padded feature / hidden width of the GEMM operands

template <typename W>
__device__ void spin_features(const W* __restrict__ words_r, int i, int n, int P, int maxdeg,
                              const int32_t* __restrict__ nbr, const float* __restrict__ cpl, float h, float beta,
                              float jp, float (&x)[kFeat], float& dE) {
    const W wi = words_r[i];
    float scale = 1.0f + fabsf(h);
    float fsum = 0.0f, fsq = 0.0f, align = 0.0f;
    W nbw[16];
    float J[16];
    for (int m = 0; m < maxdeg && m < 16; ++m) {
        const int j = __ldg(nbr + (int64_t)m * n + i);
        J[m] = __ldg(cpl + (int64_t)m * n + i);
        nbw[m] = words_r[(unsigned)j < (unsigned)n ? j : i];
        scale += fabsf(J[m]);
    }
    for (int k = 0; k < P; ++k) {
        float f = h;
        for (int m = 0; m < maxdeg && m < 16; ++m) f += ((nbw[m] >> k) & 1) ? -J[m] : J[m];
        const float s = ((wi >> k) & 1) ? -1.0f : 1.0f;
        fsum += f;
        fsq += f * f;
        align += s * f;
    }
    const float inv = 1.0f / (float)P;
    const float mean = fsum * inv;
    const float var = fmaxf(fsq * inv - mean * mean, 0.0f);
    int mag = 0, dis = 0;
    for (int k = 0; k < P; ++k) {
        mag += ((wi >> k) & 1) ? -1 : 1;
        const int kn = k + 1 == P ? 0 : k + 1;
        dis += (int)(((wi >> k) ^ (wi >> kn)) & 1);
    }
    dE = 2.0f * align;  // classical energy change of flipping the whole world-line
    x[0] = mean / scale;
    x[1] = sqrtf(var) / scale;
    x[2] = (float)mag * inv;
    x[3] = (float)dis * inv;
    x[4] = align * inv / scale;
    x[5] = fminf(fmaxf(beta * dE * inv, -8.0f), 8.0f);
    x[6] = fminf(fmaxf(jp * beta * inv, 0.0f), 8.0f);
    x[7] = 1.0f;
}

// Rows [0, M): features of the current world-lines of class `cls` (all replicas,
// row = r * csize + s); rows [M, 2M): the flipped versions.  dE[row] = classical
// flip cost of the current world-line.
template <typename W>
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
    spin_features<W>(words + (int64_t)r * n, i, n, P, maxdeg, nbr, cpl, __ldg(field + i), beta, jp, x, de);
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

inline unsigned blocks_for(int64_t n, int b = 256) { return (unsigned)((n + b - 1) / b); }

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
    if (word_bits == 32)
        features_kernel<uint32_t><<<blocks_for(M), 256, 0, st>>>((const uint32_t*)words, n, P, R, maxdeg, nbr, cpl,
                                                                 field, cls, stride, csize, beta, jp,
                                                                 (__nv_bfloat16*)X, dE, Mpad);
    else if (word_bits == 64)
        features_kernel<uint64_t><<<blocks_for(M), 256, 0, st>>>((const uint64_t*)words, n, P, R, maxdeg, nbr, cpl,
                                                                 field, cls, stride, csize, beta, jp,
                                                                 (__nv_bfloat16*)X, dE, Mpad);
    else
        return PQ_ERR_INVALID_ARG;
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
