// Packed fast sweeps of one instance: one CTA anneals `rpc` replicas held in
// shared memory for the whole schedule.  The sweep itself (order, arithmetic,
// uniforms) is specified and implemented in sweep_core.cuh.
#include "sweep_core.cuh"

namespace {

using namespace pq;

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
    int qcap; // site-queue entries per CTA (fast_queue_cap)
    PhiloxKeyTable keys;  // round keys of (key0, key1), read as constant operands
};

// Shared-memory budget of one CTA of the packed sweep.
constexpr size_t kSmemBudget = 200 * 1024;

// Site-queue entries of a CTA: a whole phase when the budget allows (the word scan
// then runs each phase in one chunk), else kQueuePerThread per thread.
inline int fast_queue_cap(int rpc, int n, int P, int stride, int threads) {
    const int whole = whole_phase_queue(threads, rpc, stride);
    if (item_smem_bytes(rpc, n, P) + (size_t)whole * 4 + 16 <= kSmemBudget) return whole;
    return kQueuePerThread * threads;
}

// Dynamic shared memory of one CTA: the item, the site queue, its two counters.
inline size_t fast_smem_bytes(int rpc, int n, int P, int stride, int threads) {
    return item_smem_bytes(rpc, n, P) + (size_t)fast_queue_cap(rpc, n, P, stride, threads) * 4 + 16;
}

// One CTA's replicas through the schedule (the body of both kernels below).
template <typename W, int MAXDEG, int NQC, bool STAGED>
__device__ __forceinline__ void fast_cta(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                         const float* __restrict__ cpl, const float* __restrict__ field,
                                         const float* __restrict__ jperp, const float* __restrict__ betas,
                                         const FastArgs& a, unsigned long long* __restrict__ accepts,
                                         int32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int csize[kMaxClasses];
    // the sites a phase visits (fast_queue_cap entries) and two counters, after the item
    const int qcap = a.qcap;
    uint32_t* queue_slots = reinterpret_cast<uint32_t*>(smem_raw + item_smem_bytes(a.rpc, a.n, a.P));
    int* queue_count = reinterpret_cast<int*>(queue_slots + qcap);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < kMaxClasses; ++c) csize[c] = a.class_size[c];
    }
    const int r0 = blockIdx.x * a.rpc;
    const int nrep = min(a.rpc, a.R - r0);
    if (nrep <= 0) return;
    Item it;
    it.nbr = nbr; it.cpl = cpl; it.field = field; it.csize = csize; it.jperp = jperp; it.betas = betas;
    it.words = words + (int64_t)r0 * a.n;
    it.n = a.n; it.P = a.P; it.maxdeg = a.maxdeg; it.nclass = a.nclass; it.stride = a.stride;
    it.order_mode = a.order_mode; it.nrep = nrep; it.replica0 = (uint32_t)(a.replica_base + r0);
    it.key0 = a.key0; it.key1 = a.key1; it.sweep_base = a.sweep_base; it.nsched = a.nsched;
    it.mcsteps = a.mcsteps; it.global_moves = a.global_moves; it.beta = a.beta;
    const Group g{(int)threadIdx.x, (int)blockDim.x, 0};
    W* sw = reinterpret_cast<W*>(smem_raw);
    const size_t words_bytes = ((size_t)nrep * a.n * sizeof(W) + 15) & ~(size_t)15;
    uint8_t* order = smem_raw + words_bytes;
    uint32_t* parity = reinterpret_cast<uint32_t*>(order + (((size_t)nrep * kMaxClasses + 15) & ~(size_t)15));
    bool bad = false;
    unsigned long long nacc = 0;
    stage_in<W>(it, sw, g);   // also publishes csize
    run_item<W, MAXDEG, NQC, STAGED>(it, a.keys, sw, order, parity, SiteQueue{queue_slots, queue_count, qcap}, g, bad,
                                     nacc);
    stage_out<W>(it, sw, g);
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
    if (accepts) {
        for (int off = 16; off > 0; off >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, off);
        if ((threadIdx.x & 31) == 0 && nacc) atomicAdd(accepts, nacc);
    }
}

template <typename W, int MAXDEG, int NQC, bool STAGED>
__global__ void __launch_bounds__(512) qa_fast_kernel(W* __restrict__ words, const int32_t* __restrict__ nbr,
                                                      const float* __restrict__ cpl,
                                                      const float* __restrict__ field,
                                                      const float* __restrict__ jperp,
                                                      const float* __restrict__ betas,
                                                      const __grid_constant__ FastArgs a,
                                                      unsigned long long* __restrict__ accepts,
                                                      int32_t* __restrict__ status) {
    fast_cta<W, MAXDEG, NQC, STAGED>(words, nbr, cpl, field, jperp, betas, a, accepts, status);
}

// The staged 32-bit variants with a cap of 72 registers: seven 128-thread CTAs fit
// an SM (the shared memory of an 80x80 replica allows seven); uncapped they take
// over 90.
template <int MAXDEG, int NQC>
__global__ void __maxnreg__(72) qa_fast_kernel_staged32(uint32_t* __restrict__ words,
                                                        const int32_t* __restrict__ nbr,
                                                        const float* __restrict__ cpl,
                                                        const float* __restrict__ field,
                                                        const float* __restrict__ jperp,
                                                        const float* __restrict__ betas,
                                                        const __grid_constant__ FastArgs a,
                                                        unsigned long long* __restrict__ accepts,
                                                        int32_t* __restrict__ status) {
    fast_cta<uint32_t, MAXDEG, NQC, true>(words, nbr, cpl, field, jperp, betas, a, accepts, status);
}

// The kernel of one variant.
template <typename W, int MAXDEG, int NQC, bool STAGED>
auto fast_kernel() {
    if constexpr (STAGED && sizeof(W) == 4) return qa_fast_kernel_staged32<MAXDEG, NQC>;
    else return qa_fast_kernel<W, MAXDEG, NQC, STAGED>;
}

// FP64 energy of (replica, slice) from the CSR of the coupling matrix.  A warp takes
// kEnergySlices slices of one replica, so each CSR entry it loads serves all of them;
// every slice's operations and their order are those of one warp per slice (per row
// rowsum += val * s_j in CSR order, acc += s_i * rowsum over the lane's rows, then the
// warp's shuffle reduction).  A product with s = +-1 is exactly the value with its sign
// bit flipped, so it is formed on the bits: one FP64 add per entry and slice.
constexpr int kEnergySlices = 8;

__device__ __forceinline__ double signed_by_bit(double v, uint64_t bit) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)(bit << 63));
}

template <typename W>
__global__ void energy_packed_kernel(const W* __restrict__ words, int n, int P, int R,
                                     const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                     const double* __restrict__ val, double* __restrict__ out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int chunks = (P + kEnergySlices - 1) / kEnergySlices;
    if (warp >= R * chunks) return;
    const int r = warp / chunks, k0 = (warp % chunks) * kEnergySlices;
    const W* w = words + (int64_t)r * n;
    double acc[kEnergySlices];
#pragma unroll
    for (int c = 0; c < kEnergySlices; ++c) acc[c] = 0.0;
    for (int i = lane; i < n; i += 32) {
        const W wi = w[i] >> k0;
        double rowsum[kEnergySlices];
#pragma unroll
        for (int c = 0; c < kEnergySlices; ++c) rowsum[c] = 0.0;
        for (int64_t e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
            const int j = col[e];
            const double v = val[e];
            const W wj = j == i ? (W)0 : (((unsigned)j < (unsigned)n) ? (W)(w[j] >> k0) : (W)0);
#pragma unroll
            for (int c = 0; c < kEnergySlices; ++c) rowsum[c] += signed_by_bit(v, (uint64_t)((wj >> c) & 1));
        }
#pragma unroll
        for (int c = 0; c < kEnergySlices; ++c) acc[c] += signed_by_bit(rowsum[c], (uint64_t)((wi >> c) & 1));
    }
#pragma unroll
    for (int c = 0; c < kEnergySlices; ++c)
        for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_down_sync(0xffffffffu, acc[c], off);
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < kEnergySlices; ++c)
            if (k0 + c < P) out[(int64_t)r * P + k0 + c] = -acc[c];
    }
}

// Configuration streaming between the int8 layout [R][n][P] and packed words.
// A block of kStreamThreads threads owns kStreamThreads consecutive (replica, spin)
// items t = r n + i, whose spins are one contiguous run of kStreamThreads * P bytes.
// Unpacking writes each thread's P bytes into shared memory and stores the run as
// 16-byte vectors when its start is 16-byte aligned (byte by byte otherwise).
constexpr int kStreamThreads = 256;

__device__ __forceinline__ bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// Packing reads each item's P spins directly: a warp's loads of one slice index
// touch neighbouring sectors that the next indices reuse from L1 (measured faster
// than staging the run for this direction).
template <typename W>
__global__ void __launch_bounds__(kStreamThreads) pack_kernel(const int8_t* __restrict__ spins, int n, int P, int R,
                                                            const int32_t* __restrict__ perm, W* __restrict__ words,
                                                            int stride) {
    const int64_t t = (int64_t)blockIdx.x * kStreamThreads + threadIdx.x;
    if (t >= (int64_t)R * n) return;
    const int r = (int)(t / n), i = (int)(t % n);
    const int8_t* s = spins + t * P;
    W w = 0;
    for (int k = 0; k < P; ++k) w |= (W)(s[k] < 0) << k;
    const int di = perm ? perm[i] : i;
    if ((unsigned)di < (unsigned)stride) words[(int64_t)r * stride + di] = w;
}

template <typename W>
__global__ void __launch_bounds__(kStreamThreads) unpack_kernel(const W* __restrict__ words, int n, int P, int R,
                                                              const int32_t* __restrict__ perm, int stride,
                                                              int8_t* __restrict__ spins) {
    extern __shared__ __align__(16) int8_t run[];
    const int64_t total = (int64_t)R * n;
    const int64_t t0 = (int64_t)blockIdx.x * kStreamThreads;
    const int items = (int)min((int64_t)kStreamThreads, total - t0);
    if ((int)threadIdx.x < items) {
        const int64_t t = t0 + threadIdx.x;
        const int r = (int)(t / n), i = (int)(t % n);
        const int di = perm ? perm[i] : i;
        const W w = (unsigned)di < (unsigned)stride ? words[(int64_t)r * stride + di] : (W)0;
        int8_t* s = run + threadIdx.x * P;
        for (int k = 0; k < P; ++k) s[k] = ((w >> k) & 1) ? -1 : 1;
    }
    __syncthreads();
    const int nbytes = items * P;
    int8_t* dst = spins + t0 * P;
    if (aligned16(dst)) {
        const int nvec = nbytes >> 4;
        for (int v = threadIdx.x; v < nvec; v += kStreamThreads)
            reinterpret_cast<int4*>(dst)[v] = reinterpret_cast<const int4*>(run)[v];
        for (int b = (nvec << 4) + threadIdx.x; b < nbytes; b += kStreamThreads) dst[b] = run[b];
    } else {
        for (int b = threadIdx.x; b < nbytes; b += kStreamThreads) dst[b] = run[b];
    }
}

template <typename W, int MAXDEG, int NQC, bool STAGED>
int launch_fast_t(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                  const float* betas, const FastArgs& a, int threads, unsigned long long* accepts, int32_t* status,
                  cudaStream_t stream) {
    const size_t smem = fast_smem_bytes(a.rpc, a.n, a.P, a.stride, threads);
    static PqSmemAttr attr;
    const auto kernel = fast_kernel<W, MAXDEG, NQC, STAGED>();
    const int rc = pq_set_smem_limit(attr, (const void*)kernel, 220 * 1024);
    if (rc != PQ_OK) return rc;
    const int grid = (a.R + a.rpc - 1) / a.rpc;
    FastArgs la = a;
    la.qcap = fast_queue_cap(a.rpc, a.n, a.P, a.stride, threads);
    kernel<<<grid, threads, smem, stream>>>((W*)words, nbr, cpl, field, jperp, betas, la, accepts, status);
    return pq_launch_status();
}

template <typename W, int MAXDEG, int NQC>
const void* fast_kernel_for() {
    return (const void*)fast_kernel<W, MAXDEG, NQC, staged_phase(NQC)>();
}

// Waves of CTAs a launch of `threads`-thread CTAs takes on this device (resident
// CTAs per SM from the runtime's occupancy of the variant that would run).
template <typename W, int MAXDEG, int NQC>
int fast_waves(const FastArgs& a, int threads, int64_t* waves) {
    const void* k = fast_kernel_for<W, MAXDEG, NQC>();
    PQ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    int dev = 0, nsm = 0, per_sm = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    PQ_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = fast_smem_bytes(a.rpc, a.n, a.P, a.stride, threads);
    PQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
    const int64_t slots = (int64_t)nsm * (per_sm > 0 ? per_sm : 1);
    const int64_t grid = (a.R + a.rpc - 1) / a.rpc;
    *waves = (grid + slots - 1) / slots;
    return PQ_OK;
}

// Compile-time P: staged phases (staged_phase).  With the thread count chosen
// automatically, CTAs of half the size are taken when that runs the replicas in
// fewer waves (more CTAs resident per SM): the last wave of a launch leaves SMs idle.
template <typename W, int MAXDEG, int NQC>
int launch_fast(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                const float* betas, const FastArgs& a, int threads, bool auto_threads, unsigned long long* accepts,
                int32_t* status, cudaStream_t stream) {
    const int half = threads / 2;
    if (auto_threads && half >= 64 && half % 32 == 0 && half >= a.rpc &&
        ((int64_t)a.rpc * a.stride) % half == 0) {
        int64_t w_full = 0, w_half = 0;
        int rc = fast_waves<W, MAXDEG, NQC>(a, threads, &w_full);
        if (rc != PQ_OK) return rc;
        rc = fast_waves<W, MAXDEG, NQC>(a, half, &w_half);
        if (rc != PQ_OK) return rc;
        if (w_half < w_full) threads = half;
    }
    return launch_fast_t<W, MAXDEG, NQC, staged_phase(NQC)>(words, nbr, cpl, field, jperp, betas, a, threads,
                                                            accepts, status, stream);
}

template <typename W>
int dispatch_deg(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                 const float* betas, const FastArgs& a, int threads, bool auto_threads, unsigned long long* accepts,
                 int32_t* status, cudaStream_t stream) {
    // compile-time slice counts (staged phases, quiet sites) for the common even P and up
    // to eight couplings; a degree below the variant's adds +0 terms, which can change
    // only the sign of a zero sum and no decision
    if (a.maxdeg <= 8) {
        const bool four = a.maxdeg <= 4;
        if constexpr (sizeof(W) == 4) {
            if (a.P == 20)
                return four ? launch_fast<W, 4, 10>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream)
                            : launch_fast<W, 8, 10>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
            if (a.P == 16)
                return four ? launch_fast<W, 4, 8>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream)
                            : launch_fast<W, 8, 8>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
            if (a.P == 32)
                return four ? launch_fast<W, 4, 16>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream)
                            : launch_fast<W, 8, 16>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
        } else {
            if (a.P == 64)
                return four ? launch_fast<W, 4, 32>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream)
                            : launch_fast<W, 8, 32>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
        }
    }
    if (a.maxdeg <= 4)
        return launch_fast<W, 4, 0>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
    if (a.maxdeg <= 8)
        return launch_fast<W, 8, 0>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
    if (a.maxdeg <= 16)
        return launch_fast<W, 16, 0>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, stream);
    return PQ_ERR_UNSUPPORTED;
}

}  // namespace

extern "C" {

int pq_qa_fast_ex(void* words, const int32_t* nbr, const float* cpl, const float* field, const float* jperp,
                  const float* betas, const pq_fast_params* prm, unsigned long long* accepts, int32_t* status,
                  void* stream) {
    if (!prm || !words || !jperp) return PQ_ERR_INVALID_ARG;   // field may be NULL: no fields
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
    a.keys = pq_philox_key_table(a.key0, a.key1);
    a.sweep_base = p.sweep_base;
    a.replica_base = p.replica_base;
    int threads = p.threads > 0 ? p.threads : 0;
    const bool auto_threads = threads == 0;
    int rpc = p.replicas_per_cta;
    if (rpc <= 0) {
        // enough replicas per CTA for 128 items per phase, within the smem budget
        rpc = (128 + p.class_stride - 1) / p.class_stride;
        if (rpc < 1) rpc = 1;
        const size_t cap = kSmemBudget / 2 / item_smem_bytes(1, p.n, p.P);
        if ((size_t)rpc > cap) rpc = cap < 1 ? 1 : (int)cap;
    }
    if (rpc > kMaxRpc) rpc = kMaxRpc;
    if (threads <= 0) {
        // the largest multiple of 32 up to 256 that divides the items of a phase (every
        // thread equally busy in every phase); else round up (measured best on GB300)
        const int items = rpc * p.class_stride;
        threads = 0;
        for (int t = 256; t >= 32 && !threads; t -= 32)
            if (items >= t && items % t == 0) threads = t;
        if (!threads) threads = items >= 256 ? 256 : ((items + 31) / 32) * 32;
    }
    if (threads % 32 || threads > 512 || threads < rpc) return PQ_ERR_INVALID_ARG;
    if (fast_smem_bytes(rpc, p.n, p.P, p.class_stride, threads) > kSmemBudget)
        return PQ_ERR_TOO_LARGE;
    a.rpc = rpc;
    cudaStream_t st = (cudaStream_t)stream;
    if (wbytes == 4)
        return dispatch_deg<uint32_t>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status,
                                      st);
    return dispatch_deg<uint64_t>(words, nbr, cpl, field, jperp, betas, a, threads, auto_threads, accepts, status, st);
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
    const int64_t warps = (int64_t)R * ((P + kEnergySlices - 1) / kEnergySlices);
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
    const unsigned blocks = (unsigned)((tot + kStreamThreads - 1) / kStreamThreads);
    cudaStream_t st = (cudaStream_t)stream;
    if (word_bits == 32)
        pack_kernel<uint32_t><<<blocks, kStreamThreads, 0, st>>>(spins, n, P, R, perm, (uint32_t*)words, word_stride);
    else
        pack_kernel<uint64_t><<<blocks, kStreamThreads, 0, st>>>(spins, n, P, R, perm, (uint64_t*)words, word_stride);
    return pq_launch_status();
}

int pq_unpack_spins(const void* words, int word_bits, int n, int P, int R, const int32_t* perm, int word_stride,
                    int8_t* spins, void* stream) {
    if (!spins || !words || n <= 0 || P < 1 || R < 0 || word_stride < (perm ? 1 : n)) return PQ_ERR_INVALID_ARG;
    if (!((word_bits == 32 && P <= 32) || (word_bits == 64 && P <= 64))) return PQ_ERR_INVALID_ARG;
    if (R == 0) return PQ_OK;
    const int64_t tot = (int64_t)R * n;
    const unsigned blocks = (unsigned)((tot + kStreamThreads - 1) / kStreamThreads);
    const size_t smem = (size_t)kStreamThreads * P;   // at most 16 KB (P <= 64)
    cudaStream_t st = (cudaStream_t)stream;
    if (word_bits == 32)
        unpack_kernel<uint32_t><<<blocks, kStreamThreads, smem, st>>>((const uint32_t*)words, n, P, R, perm,
                                                                      word_stride, spins);
    else
        unpack_kernel<uint64_t><<<blocks, kStreamThreads, smem, st>>>((const uint64_t*)words, n, P, R, perm,
                                                                      word_stride, spins);
    return pq_launch_status();
}

}  // extern "C"
