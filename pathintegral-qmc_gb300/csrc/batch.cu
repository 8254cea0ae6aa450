// Persistent batched packed sweep: many instances of uneven size, slice count
// and replica count annealed in one launch.
//
// Work is cut into items (a few replicas of one instance) and items into tasks
// (up to 8 items that each take `gwarps` warps of a CTA, with a named barrier
// per item; `lanes_per_site` = 2 gives the task's 64-slice items a lane pair per
// site).  Persistent CTAs take tasks from a queue head in global memory
// (one atomicAdd per task) until the queue is empty; the host orders tasks
// longest first.  Each item runs exactly the sweep of sweep_core.cuh, so a
// batched anneal equals the single-instance anneals of its instances bit for
// bit (same keys, replica ids and sweep counters).
#include "sweep_core.cuh"

namespace {

using namespace pq;

__device__ __forceinline__ void run_task_item(const pq_batch_item& bi, const pq_batch_inst& in,
                                              const pq_batch_run& run, const int32_t* nbr_pool,
                                              const float* cpl_pool, const float* field_pool,
                                              const int32_t* csize_pool, const float* jperp_pool,
                                              unsigned char* words_pool, unsigned char* smem, const SiteQueue& q,
                                              const Group& g,
                                              int lanes_per_site, bool& bad, unsigned long long& nacc) {
    Item it;
    it.nbr = nbr_pool + in.tab_off;
    it.cpl = cpl_pool + in.tab_off;
    it.field = field_pool + in.field_off;
    it.csize = csize_pool + in.csize_off;
    it.jperp = jperp_pool + in.jperp_off + run.sched_base;
    it.betas = nullptr;
    it.words = words_pool + bi.word_off;
    it.n = in.n; it.P = in.P; it.maxdeg = in.maxdeg; it.nclass = in.nclass; it.stride = in.stride;
    it.order_mode = run.order_mode;
    it.nrep = bi.nrep;
    it.replica0 = (uint32_t)bi.replica0;
    it.key0 = in.key0; it.key1 = in.key1;
    it.sweep_base = run.sweep_base;
    it.nsched = run.nsched; it.mcsteps = run.mcsteps; it.global_moves = run.global_moves;
    it.beta = run.beta;
    run_item_any(it, smem + bi.smem_off, q, g, bad, nacc, lanes_per_site);
}

__global__ void __launch_bounds__(256, 2) batch_kernel(const pq_batch_task* __restrict__ tasks, int ntasks,
                                                    const pq_batch_item* __restrict__ items,
                                                    const pq_batch_inst* __restrict__ insts, const int32_t* nbr_pool,
                                                    const float* cpl_pool, const float* field_pool,
                                                    const int32_t* csize_pool, const float* jperp_pool,
                                                    unsigned char* words_pool, int* queue_head, pq_batch_run run,
                                                    unsigned long long* accepts, int32_t* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_task;
    __shared__ uint32_t queue_slots[kQueuePerThread * 256];   // unsettled sites of a phase, per group
    __shared__ int queue_count[2 * 8];
    bool bad = false;
    unsigned long long nacc = 0;
    for (;;) {
        if (threadIdx.x == 0) s_task = atomicAdd(queue_head, 1);
        __syncthreads();
        const int t = s_task;
        if (t >= ntasks) break;
        const pq_batch_task task = tasks[t];
        const int gi = (threadIdx.x >> 5) / task.gwarps;
        if (gi < task.nitems) {
            const pq_batch_item bi = items[task.item0 + gi];
            const pq_batch_inst in = insts[bi.inst];
            const int gthr = task.gwarps * 32;
            const Group g{(int)threadIdx.x - gi * gthr, gthr,
                          (task.nitems == 1 && gthr == (int)blockDim.x) ? 0 : 1 + gi};
            run_task_item(bi, in, run, nbr_pool, cpl_pool, field_pool, csize_pool, jperp_pool, words_pool, smem,
                          SiteQueue{queue_slots + kQueuePerThread * gi * gthr, queue_count + 2 * gi,
                                    kQueuePerThread * gthr},
                          g,
                          task.lanes_per_site, bad, nacc);
        }
        __syncthreads();
    }
    if (bad) pq_set_status(status, PQ_ERR_BAD_INDEX);
    if (accepts) {
        for (int off = 16; off > 0; off >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, off);
        if ((threadIdx.x & 31) == 0 && nacc) atomicAdd(accepts, nacc);
    }
}

// Scratch of pq_batch_anneal_noalloc: the persistent CTAs' task counter lives
// here instead of in caller memory.  One 32-bit counter in a 256-byte array
// (the whole array is reserved on every device that loads the library, until
// the process exits).  Every call shares it.
constexpr int kNoAllocScratchInts = 64;
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocScratchInts];

// Device address of the scratch, looked up once per device context (host code
// cannot use the symbol itself: on the host it names a stand-in, not device
// memory).  The lookup is redone after the device's context changes (a reset).
int noalloc_scratch(int** out) {
    static std::mutex mu;
    static unsigned long long ctx[kPqMaxDevices];
    static int* addr[kPqMaxDevices];
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kPqMaxDevices) return PQ_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(mu);
    const unsigned long long id = pq_context_id();
    if (!id || ctx[dev] != id || !addr[dev]) {
        void* p = nullptr;
        PQ_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        addr[dev] = static_cast<int*>(p);
        ctx[dev] = pq_context_id();
    }
    *out = addr[dev];
    return PQ_OK;
}

}  // namespace

extern "C" {

// pq_batch_anneal without the caller's queue_head: for callers that cannot
// allocate device memory.  Rejects ntasks + grid beyond the 32-bit counter.
int pq_batch_anneal_noalloc(const pq_batch_task* tasks, int ntasks, const pq_batch_item* items,
                            const pq_batch_inst* insts, const int32_t* nbr_pool, const float* cpl_pool,
                            const float* field_pool, const int32_t* csize_pool, const float* jperp_pool,
                            void* words_pool, const pq_batch_run* run, int grid, int threads, int smem_bytes,
                            unsigned long long* accepts, int32_t* status, void* stream) {
    if (ntasks < 0 || grid <= 0) return PQ_ERR_INVALID_ARG;
    if ((int64_t)ntasks + grid > (int64_t)INT32_MAX) return PQ_ERR_TOO_LARGE;
    int* head = nullptr;
    const int st = noalloc_scratch(&head);  // first call on a device: symbol lookup
    if (st != PQ_OK) return st;
    return pq_batch_anneal(tasks, ntasks, items, insts, nbr_pool, cpl_pool, field_pool, csize_pool, jperp_pool,
                           words_pool, head, run, grid, threads, smem_bytes, accepts, status, stream);
}


int pq_batch_smem_bytes(int nrep, int n, int P) { return (int)item_smem_bytes(nrep, n, P); }

int pq_batch_occupancy(int threads, int smem_bytes, int* blocks_per_sm, int* sm_count) {
    if (!blocks_per_sm || !sm_count || threads <= 0 || threads > 256 || threads % 32 || smem_bytes < 0)
        return PQ_ERR_INVALID_ARG;
    PQ_CUDA_TRY(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    PQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_kernel, threads, smem_bytes));
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    PQ_CUDA_TRY(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
    return PQ_OK;
}

int pq_batch_anneal(const pq_batch_task* tasks, int ntasks, const pq_batch_item* items, const pq_batch_inst* insts,
                    const int32_t* nbr_pool, const float* cpl_pool, const float* field_pool,
                    const int32_t* csize_pool, const float* jperp_pool, void* words_pool, int* queue_head,
                    const pq_batch_run* run, int grid, int threads, int smem_bytes, unsigned long long* accepts,
                    int32_t* status, void* stream) {
    if (!run || ntasks < 0 || grid <= 0 || threads <= 0 || threads > 256 || threads % 32 || smem_bytes < 0 ||
        smem_bytes > 220 * 1024)
        return PQ_ERR_INVALID_ARG;
    // the task counter is 32-bit: every CTA adds one past the last task before it stops
    if ((int64_t)ntasks + grid > (int64_t)INT32_MAX) return PQ_ERR_TOO_LARGE;
    if (ntasks == 0 || run->nsched == 0) return PQ_OK;
    if (!tasks || !items || !insts || !field_pool || !csize_pool || !jperp_pool || !words_pool || !queue_head)
        return PQ_ERR_INVALID_ARG;
    // instances are checked on the host (maxdeg <= 8: the batched kernel carries no wider variant)
    if (run->order_mode != 0 && run->order_mode != 1) return PQ_ERR_INVALID_ARG;
    static PqSmemAttr attr;
    const int rc = pq_set_smem_limit(attr, (const void*)batch_kernel, 220 * 1024);
    if (rc != PQ_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    PQ_CUDA_TRY(cudaMemsetAsync(queue_head, 0, sizeof(int), st));
    batch_kernel<<<grid, threads, smem_bytes, st>>>(tasks, ntasks, items, insts, nbr_pool, cpl_pool, field_pool,
                                                    csize_pool, jperp_pool, (unsigned char*)words_pool, queue_head,
                                                    *run, accepts, status);
    return pq_launch_status();
}

}  // extern "C"
