/*
 * piqmc_gb300 -- C ABI of the GB300-native path-integral quantum-annealing library.
 *
 * Plain C types only: device pointers are passed as typed pointers, streams as
 * `void*` (a cudaStream_t; NULL = the legacy default stream).  Every entry
 * point returns an int status: 0 = PQ_OK, > 0 = a validation error detected on
 * the host or by a kernel, < 0 = minus a cudaError_t.  Kernels that can fail
 * on data they read (an out-of-range neighbour index, an exhausted random
 * stream, a wait that timed out) record the first such error in a device
 * status word that the caller passes; the entry point does NOT synchronise, so
 * read that word after the stream has been synchronised (the Python layer
 * does this and raises).
 *
 * Spin layouts
 *   int8 layout  : spins[(r*n + i)*P + k] = +1/-1, replica r, spin i, slice k.
 *   packed layout: words[r*n + i] holds the world-line of spin i of replica r,
 *                  bit k = 1 means spin -1 in slice k (tools.spins2bits
 *                  convention, reference piqmc/tools.pyx:24-26); 32-bit words
 *                  for P <= 32, 64-bit words for P <= 64.
 */
#ifndef PIQMC_GB300_H
#define PIQMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PQ_OK 0
#define PQ_ERR_INVALID_ARG 1      /* bad size, null pointer, unsupported combination */
#define PQ_ERR_BAD_INDEX 2        /* a neighbour / permutation index outside [0, n) */
#define PQ_ERR_RAND_EXHAUSTED 3   /* the supplied uniform stream was too short */
#define PQ_ERR_UNSUPPORTED 4      /* e.g. P > 64 for the packed kernels */
#define PQ_ERR_TOO_LARGE 5        /* does not fit the kernel's on-chip tiles */
#define PQ_ERR_TIMEOUT 6          /* a bounded device-side wait gave up */
#define PQ_ERR_LIBC_STATE 7       /* libc rand() state has an unsupported layout */
#define PQ_ERR_NO_DEVICE 8

/* Semantics flags of the reference-order sweeps. 0 = the reference as shipped. */
#define PQ_FIX_Q2 1 /* reset the energy difference per spin (reference resets it per slice) */
#define PQ_FIX_Q1 2 /* couple slice k to k-1, k+1 (reference couples every slice to P-1 and 1) */
#define PQ_ACC_FP64 4 /* accumulate in FP64 exactly as the generated C writes it; needed only when
                         |2 J| or |2 J-perp| can overflow FP32 (the FP32 accumulator is otherwise
                         identical, bit for bit) */

/* Library identification. */
int pq_version(void);
const char* pq_strerror(int status);

/* ---------------------------------------------------------------------------
 * Reference-order sweeps: the reference's exact update order and arithmetic.
 * Each replica runs on a pair of warps (one forms the next spin's energy terms,
 * the other walks the accumulation chain and decides), or on one thread when the
 * problem is larger than the pair kernel's shared memory; R replicas run
 * concurrently, each with its own spin orders (perms) and uniform stream (rands).
 *   perms     int32 [R][nsweeps][n], nsweeps = nsched*mcsteps: the spin order of
 *             each sweep (the successive rng.permutation results).
 *   rands     int32 [R][rand_stride]: successive libc rand() values.
 *   rand_used int64 [R] out: values consumed (the kernel starts at 0).
 *   jperp     float [nsched]: J-perp per schedule step (pq_jperp_schedule).
 *   status    int32 [1] device error word (0 = ok), first error wins.
 * ------------------------------------------------------------------------- */

/* Replaces qmc.QuantumAnneal (reference piqmc/qmc.pyx:30-136).  n = rows of the
 * spin array and of the neighbour table (int32 [n][maxnb] index, float
 * coupling); each sweep updates the nperm <= n spins its permutation lists
 * (nperm = the reference's nspins), so perms is int32 [R][nsweeps][nperm]. */
int pq_qa_sparse_reforder(int8_t* spins, const int32_t* nb_idx, const float* nb_j,
                          int n, int nperm, int maxnb, int P, int R,
                          const float* jperp, int nsched, int mcsteps, float temp,
                          const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                          int64_t* rand_used, int flags, int32_t* status, void* stream);

/* Replaces qmc.QuantumAnneal_dense (reference piqmc/qmc.pyx:141-242).  J is dense
 * float64 row-major n*n; the upper triangle and the diagonal are read. */
int pq_qa_dense_reforder(int8_t* spins, const double* J, int n, int P, int R,
                         const float* jperp, int nsched, int mcsteps, float temp,
                         const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                         int64_t* rand_used, int flags, int32_t* status, void* stream);

/* Replaces sa.Anneal (reference piqmc/sa.pyx:50-120).  temps[g] = (float)sched[g];
 * spins are int8 [R][n]. */
int pq_sa_sparse_reforder(int8_t* spins, const int32_t* nb_idx, const float* nb_j,
                          int n, int maxnb, int R, const float* temps, int nsched, int mcsteps,
                          const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                          int64_t* rand_used, int32_t* status, void* stream);

/* Replaces sa.Anneal_dense (reference piqmc/sa.pyx:126-187): dense float64 J
 * [n][n] (upper triangle + diagonal read), temps[g] = (float)sched[g], spins int8
 * [R][n], perms int32 [R][nsched*mcsteps][n]. */
int pq_sa_dense_reforder(int8_t* spins, const double* J, int n, int R, const float* temps, int nsched, int mcsteps,
                         const int32_t* perms, const int32_t* rands, int64_t rand_stride, int64_t* rand_used,
                         int32_t* status, void* stream);

/* The same three sweeps with the exp-parity hooks.  ov_x/ov_y (device, may be
 * NULL): sorted FP32 bit patterns x and the host libm's exp((double)x), used in
 * place of the device exp for "close calls" (exp(x) within ~4.5 ulp of the
 * uniform, where a last-bit difference between exp implementations could change
 * the decision).  close_x/close_y/close_cnt (device, may be NULL): close calls
 * that found no override, with the device exp value used; the host compares them
 * with its own exp and reruns with overrides when one differs. */
int pq_qa_sparse_reforder_ex(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n,
                             int nperm, int maxnb, int P, int R, const float* jperp, int nsched, int mcsteps,
                             float temp, const int32_t* perms, const int32_t* rands,
                             int64_t rand_stride, int64_t* rand_used, int flags,
                             const uint32_t* ov_x, const double* ov_y, int ov_n,
                             uint32_t* close_x, double* close_y, int close_cap, int* close_cnt,
                             int32_t* status, void* stream);
int pq_qa_dense_reforder_ex(int8_t* spins, const double* J, int n, int P, int R, const float* jperp,
                            int nsched, int mcsteps, float temp, const int32_t* perms,
                            const int32_t* rands, int64_t rand_stride, int64_t* rand_used, int flags,
                            const uint32_t* ov_x, const double* ov_y, int ov_n, uint32_t* close_x,
                            double* close_y, int close_cap, int* close_cnt, int32_t* status,
                            void* stream);
int pq_sa_sparse_reforder_ex(int8_t* spins, const int32_t* nb_idx, const float* nb_j, int n,
                             int maxnb, int R, const float* temps, int nsched, int mcsteps,
                             const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                             int64_t* rand_used, int flags, const uint32_t* ov_x, const double* ov_y, int ov_n,
                             uint32_t* close_x, double* close_y, int close_cap, int* close_cnt,
                             int32_t* status, void* stream);

int pq_sa_dense_reforder_ex(int8_t* spins, const double* J, int n, int R, const float* temps, int nsched,
                            int mcsteps, const int32_t* perms, const int32_t* rands, int64_t rand_stride,
                            int64_t* rand_used, const uint32_t* ov_x, const double* ov_y, int ov_n,
                            uint32_t* close_x, double* close_y, int close_cap, int* close_cnt, int32_t* status,
                            void* stream);
/* Replaces sa.Anneal_bipartite (reference piqmc/sa.pyx:411-500): spins int8
 * [R][nl + nr] (left then right), J float64 [nl][nr], biases float64; spins are
 * visited in index order (the reference draws no permutation). */
int pq_sa_bipartite_reforder_ex(int8_t* spins, const double* J, int nl, int nr, const double* lbias,
                                const double* rbias, int R, const float* temps, int nsched, int mcsteps,
                                const int32_t* rands, int64_t rand_stride, int64_t* rand_used, const uint32_t* ov_x,
                                const double* ov_y, int ov_n, uint32_t* close_x, double* close_y, int close_cap,
                                int* close_cnt, int32_t* status, void* stream);

/* Device exp((double)x) exactly as the reference-order kernels evaluate it
 * (diagnostic for the libm parity scan): y[i] = exp(x[i]), and the range form
 * y[i] = exp(float with bits first_bits + i). */
int pq_exp_probe(const float* x, double* y, int64_t n, void* stream);
int pq_exp_probe_range(uint32_t first_bits, int64_t count, double* y, void* stream);

/* ---------------------------------------------------------------------------
 * Host helpers (host memory, no GPU work).
 * ------------------------------------------------------------------------- */

/* J-perp of reference piqmc/qmc.pyx:95 in its C types (FP32 slices*temp, double
 * log/tanh, FP32 result; generated piqmc/qmc.c:2063-2075).  Returns
 * PQ_ERR_INVALID_ARG when slices*temp == 0 (the reference raises ZeroDivisionError). */
int pq_jperp_schedule(const double* sched, int nsched, int P, float temp, float* out);

/* The next n values of this process's libc rand() WITHOUT advancing it (the
 * state is saved first and put back after; glibc only). */
int pq_libc_rand_peek(int32_t* out, int64_t n);
/* Advance this process's libc rand() by n draws. */
int pq_libc_rand_skip(int64_t n);

/* Host libm exp((double)x[i]) (host memory). */
int pq_host_exp(const float* x, double* y, int64_t n);
/* Number of FP32 inputs with bits in [first_bits, first_bits+count) whose host
 * libm exp differs from dev[i]; the first cap of them go to bad_x/bad_y. */
int64_t pq_host_exp_compare(uint32_t first_bits, int64_t count, const double* dev, uint32_t* bad_x,
                            double* bad_y, int64_t cap);

/* Neighbour table of tools.GenerateNeighbors (reference piqmc/tools.pyx:28-96) in
 * one O(nnz) pass.  keys are the matrix's DOK keys in iteration order; out is
 * float64 [nspins][maxnb][2], zero-filled first.  Returns PQ_ERR_TOO_LARGE when a
 * row needs more than maxnb slots (the reference raises IndexError), and
 * PQ_ERR_BAD_INDEX for keys outside [0, nspins). */
int pq_generate_neighbors(int nspins, int64_t nkeys, const int64_t* rows, const int64_t* cols,
                          const double* vals, int maxnb, double* out);

/* Colouring of the neighbour graph; color[i] in [0, ncolors).  Greedy in spin
 * order; when that needs more than two colours, DSatur too, and the one with
 * fewer colours is kept.  nb_idx is host int32 [n][maxnb] (self entries and
 * padding are ignored when nb_j == 0 or index == i; duplicate edges count once).
 * Returns the number of colours (> 0), or minus a status. */
int pq_color_graph(int n, int maxnb, const int32_t* nb_idx, const float* nb_j, int32_t* color);

/* ---------------------------------------------------------------------------
 * Fast packed sweeps (new; no reference counterpart beyond the physics of
 * qmc.QuantumAnneal with both reference quirks corrected).
 *
 * The graph is in "device order": spins are split into M update classes
 * (independent sets: each colour of pq_color_graph cut into sub-classes),
 * class c occupying device slots [c*S, c*S + class_size[c]) of a padded index
 * space of n = M*S slots (unused slots are never read or written).  Couplings
 * in SoA: nbr[m*n + i] (int32 device slot) and cpl[m*n + i] (float), m <
 * maxdeg, padding = (i, 0.0f); field[i] = diagonal term.  One call anneals R
 * replicas through nsched schedule steps; each step does mcsteps local sweeps
 * then `global_moves` world-line flip passes.  A sweep visits the M classes in
 * order (order_mode 0) or in a fresh random order per replica and sweep
 * (order_mode 1, which brings the annealing dynamics close to the reference's
 * random sequential order).  Counter-based Philox4x32-10 keyed by seed;
 * `sweep_base` offsets the sweep counter so an anneal split over several calls
 * draws the same numbers as one call.
 * ------------------------------------------------------------------------- */
#define PQ_MAX_CLASSES 32
typedef struct pq_fast_params {
    int n;              /* padded device slots = nclass * class_stride */
    int P;              /* Trotter slices, 1..64 */
    int R;              /* replicas */
    int maxdeg;         /* couplings per spin (padded) */
    int nclass;         /* update classes M, 1..PQ_MAX_CLASSES */
    int class_stride;   /* S */
    int class_size[PQ_MAX_CLASSES];
    int order_mode;     /* 0 = fixed class order, 1 = random per (replica, sweep) */
    int nsched;         /* schedule steps in this call */
    int mcsteps;        /* local sweeps per schedule step */
    int global_moves;   /* world-line flip passes per schedule step */
    float temp;         /* temperature T */
    float beta;         /* 1/T as the caller rounded it (FP32) */
    uint64_t seed;      /* Philox key */
    int64_t sweep_base; /* sweep counter of this call's first sweep */
    int replica_base;   /* replica id of this call's first replica (RNG stream) */
    int threads;        /* threads per CTA (0 = auto) */
    int replicas_per_cta; /* (0 = auto) */
} pq_fast_params;

/* words: packed layout in device order, 32-bit words when P <= 32 else 64-bit;
 * in/out.  field may be NULL when every field is zero (the same result as a table
 * of zeros, one load per site less).  jperp: device float [nsched] (ignored for
 * P = 1).  accepts (optional,
 * may be NULL): one device uint64 counter incremented by the accepted local flips. */
int pq_qa_fast(void* words, const int32_t* nbr, const float* cpl, const float* field,
               const float* jperp, const pq_fast_params* prm, unsigned long long* accepts,
               int32_t* status, void* stream);

/* pq_qa_fast with an optional per-step inverse temperature: betas (device float
 * [nsched], may be NULL = prm->beta for every step).  With P = 1 this is a
 * packed classical annealer (sa.Anneal physics, reference piqmc/sa.pyx:50-120,
 * on the colour order). */
int pq_qa_fast_ex(void* words, const int32_t* nbr, const float* cpl, const float* field,
                  const float* jperp, const float* betas, const pq_fast_params* prm,
                  unsigned long long* accepts, int32_t* status, void* stream);

/* ---------------------------------------------------------------------------
 * Batched persistent packed sweep (new): many instances of uneven size, slice
 * count and replica count in one launch.  Per-instance tables live in pools
 * (tab_off indexes nbr_pool/cpl_pool, laid out [maxdeg][n] per instance; the
 * other offsets index their pools); each item is nrep consecutive replicas of one
 * instance whose words start at byte word_off of words_pool, and runs on a group
 * of `gwarps` warps of a CTA using shared memory from byte smem_off of the CTA's
 * dynamic shared memory (pq_batch_smem_bytes each).  A task = items
 * [item0, item0 + nitems), all with the task's gwarps and lanes_per_site,
 * nitems * gwarps <= warps of the CTA.  Persistent CTAs pop tasks from *queue_head (scratch, reset by the
 * call).  Results equal pq_qa_fast on each instance with key0/key1 as its seed
 * and replica0 as its replica_base.
 * ------------------------------------------------------------------------- */
typedef struct pq_batch_inst {
    int64_t tab_off;    /* into nbr_pool / cpl_pool */
    int64_t field_off;  /* into field_pool */
    int csize_off;      /* into csize_pool (nclass entries) */
    int jperp_off;      /* into jperp_pool (the instance's whole schedule) */
    int n, P, maxdeg, nclass, stride;
    uint32_t key0, key1;
    int pad_;
} pq_batch_inst;

typedef struct pq_batch_item {
    int inst, nrep, replica0, smem_off;
    int64_t word_off;   /* bytes into words_pool */
} pq_batch_item;

typedef struct pq_batch_task {
    int item0, nitems, gwarps;
    int lanes_per_site; /* 2: items with P = 64 and 4 couplings per spin give each site a lane
                           pair (one 32-bit half of the world-line each); otherwise 1 */
} pq_batch_task;

typedef struct pq_batch_run {
    int nsched;         /* schedule steps of this call */
    int sched_base;     /* index of its first step in each instance's J-perp schedule */
    int mcsteps, global_moves, order_mode;
    float beta;         /* 1/T (FP32) */
    int64_t sweep_base; /* sweep counter of the first sweep = sched_base * mcsteps for a split anneal */
} pq_batch_run;

int pq_batch_anneal(const pq_batch_task* tasks, int ntasks, const pq_batch_item* items,
                    const pq_batch_inst* insts, const int32_t* nbr_pool, const float* cpl_pool,
                    const float* field_pool, const int32_t* csize_pool, const float* jperp_pool,
                    void* words_pool, int* queue_head, const pq_batch_run* run, int grid, int threads,
                    int smem_bytes, unsigned long long* accepts, int32_t* status, void* stream);
/* (pq_batch_anneal rejects ntasks + grid > 2^31 - 1 with PQ_ERR_TOO_LARGE: its
 * 32-bit task counter would wrap.) */
/* No counterpart in the reference.  The same batched anneal for callers that
 * cannot allocate device memory -- for instance a host application that hands
 * this library only its own input and output buffers, or code running where
 * cudaMalloc is not allowed -- so it has no queue_head argument: the task counter
 * lives in a 256-byte static device array of this library (held on every GPU
 * that loads it until the process exits).  The first call on each device looks
 * that array's address up (cudaGetSymbolAddress), and so does the first call
 * after the device's context was reset, so make those calls before any stream
 * capture.  ntasks < 0 or grid <= 0 is PQ_ERR_INVALID_ARG, as for
 * pq_batch_anneal.  Each call resets the counter; all calls
 * share it, so calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller.  Limit: ntasks + grid <= 2^31 - 1 (the
 * counter is 32-bit), else PQ_ERR_TOO_LARGE.  Allocates nothing. */
int pq_batch_anneal_noalloc(const pq_batch_task* tasks, int ntasks, const pq_batch_item* items,
                            const pq_batch_inst* insts, const int32_t* nbr_pool, const float* cpl_pool,
                            const float* field_pool, const int32_t* csize_pool, const float* jperp_pool,
                            void* words_pool, const pq_batch_run* run, int grid, int threads, int smem_bytes,
                            unsigned long long* accepts, int32_t* status, void* stream);
/* Shared memory one item of nrep replicas of an n-slot, P-slice instance needs. */
int pq_batch_smem_bytes(int nrep, int n, int P);
/* Resident CTAs per SM of the batched kernel for a launch shape, and the SM count. */
int pq_batch_occupancy(int threads, int smem_bytes, int* blocks_per_sm, int* sm_count);

/* ---------------------------------------------------------------------------
 * Instance generators on the GPU (the bond sets of Generate2DIsingInstance,
 * Generate2DLattice and GenerateKblockLattice, reference
 * piqmc/tools.pyx:98-131, :133-175, :177-273).  Writes the neighbour table of
 * tools.GenerateNeighbors (float64 [n][maxnb][2], rows in the reference's key
 * order, zero padding) to device memory and row_len[n] (device int32) the
 * entries of each row.  kind 0: nrows x nrows torus (ncols = nrows); kind 1:
 * nrows x ncols lattice, periodic or not; kind 2: K-block lattice, 1 <= k <= 3.
 * Coupling (a, b) = lo + (hi - lo) u with u the 53-bit uniform of
 * Philox4x32-10(ctr = {a, b, 0, 6 << 24}, key = seed) -- not the caller's
 * MT19937 stream, so the values differ from the host drop-ins' while the table's
 * structure is the same.  A row longer than maxnb sets *status to
 * PQ_ERR_TOO_LARGE (the reference's IndexError).
 * ------------------------------------------------------------------------- */
int pq_generate_lattice_table(int kind, int nrows, int ncols, int periodic, int k, double lo, double hi,
                              uint64_t seed, int maxnb, double* nbs, int32_t* row_len, int32_t* status,
                              void* stream);

/* ---------------------------------------------------------------------------
 * Tensor-core GEMM (new): D[M][N] = alpha * A[M][K] B[N][K]^T (+ bias[n]),
 * BF16 row-major operands (K contiguous, leading dimensions lda/ldb elements,
 * multiples of 8, 16-byte aligned), FP32 D (ldd floats), FP32 accumulation in
 * TMEM via tcgen05.mma.  M % 128 == 0, N % 64 == 0, K % 64 == 0.  bias may be
 * NULL.  A timed-out completion wait sets *status = PQ_ERR_TIMEOUT.
 * ------------------------------------------------------------------------- */
int pq_tc_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* D, int ldd, int M, int N, int K,
                    float alpha, const float* bias, int32_t* status, void* stream);

/* ---------------------------------------------------------------------------
 * Dense packed sweep (new; the physics of qmc.QuantumAnneal_dense, reference
 * piqmc/qmc.pyx:141-242, with both quirks corrected).  words: uint32 [R][N]
 * world-lines (P <= 32).  F: FP32 local fields f = h + K s of every
 * configuration c = r*P + k, row c at F + c*ldf (the split-BF16 tensor-core GEMM
 * of pq_tc_gemm_bf16 produces them); they are copied to shared memory,
 * updated incrementally (rank-1) on every accepted flip and written back at the
 * end, so F holds the fields of the final configurations.  K: FP32 symmetric
 * couplings [N][N] with zero diagonal.  units: the nunits integers coprime to N
 * (spin orders are random affine maps i = a t + b mod N, one per sweep shared by
 * every slice like the reference's permutation, or one per slice when
 * per_slice_order != 0).  For even P the slices of a replica advance as a
 * wavefront (each waits, bounded, only for its Trotter neighbours); a wait that
 * gives up records PQ_ERR_TIMEOUT in status (nullable).
 * ------------------------------------------------------------------------- */
int pq_dense_sweep(uint32_t* words, float* F, int ldf, const float* K, const int32_t* units, int nunits,
                   const float* jperp, int N, int P, int R, int nsched, int mcsteps, float beta, uint64_t seed,
                   int64_t sweep_base, int replica_base, int per_slice_order, unsigned long long* accepts,
                   int32_t* status, void* stream);
/* pq_dense_sweep with its wavefront waits under the caller's control: a warp
 * polls a neighbour's progress at most poll_limit times (< 0: the default,
 * 2^24 polls of ~64 ns) before it gives up, records PQ_ERR_TIMEOUT, releases
 * the warps that wait on it and returns.  wait_skew (0 in use, at most 2^24) is
 * added to every awaited progress count: a positive value is progress that no
 * warp ever reports, so every wait runs to its limit -- how the timeout path is
 * tested without faulting or hanging a GPU. */
int pq_dense_sweep_ex(uint32_t* words, float* F, int ldf, const float* K, const int32_t* units, int nunits,
                      const float* jperp, int N, int P, int R, int nsched, int mcsteps, float beta, uint64_t seed,
                      int64_t sweep_base, int replica_base, int per_slice_order, int64_t poll_limit, int wait_skew,
                      unsigned long long* accepts, int32_t* status, void* stream);
/* words [R][N] -> the GEMM operand: BF16 +-1 rows c = r*P + k (Mpad rows, zero
 * padding), each row = [s over j < Npad, the same again] (2*Npad columns, so one
 * GEMM against [K_hi | K_lo] sums both halves of the split couplings). */
int pq_dense_unpack_bf16(const uint32_t* words, int N, int P, int R, int Npad, int Mpad, void* A, void* stream);

/* ---------------------------------------------------------------------------
 * Learned world-line proposals (new).  An MLP 8 -> 64 -> 64 -> 1 (ReLU) scores
 * every spin of one update class from its world-line features; the two hidden
 * layers run on the tensor cores (pq_tc_gemm_bf16, BF16 weights, FP32
 * accumulation), the rest in these kernels.  Features: see csrc/mlp.cu.
 * ------------------------------------------------------------------------- */
/* Rows r*csize + s of X (BF16, 64 columns, only the first 8 written) get the
 * features of spin slot cls*stride + s of replica r; rows Mpad + r*csize + s the
 * features of the same world-line flipped; dE the classical cost of the flip. */
int pq_mlp_features(const void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                    const float* cpl, const float* field, int cls, int stride, int csize, float beta, float jp,
                    void* X, float* dE, int64_t Mpad, void* stream);
/* out = BF16(relu(H)) element-wise (n elements). */
int pq_mlp_relu_bf16(const float* H, void* out, int64_t n, void* stream);
/* logit[r] = relu(H2[r][0..63]) . w3 + b3. */
int pq_mlp_head(const float* H2, const float* w3, float b3, float* logit, int64_t rows, void* stream);
/* Metropolis-Hastings world-line move of every spin of class cls: proposed with
 * q = clamp(sigmoid(logit[row]), qmin, 1), accepted with
 * min(1, exp(-beta dE) q'/q), q' from logit[Mpad + row] (the flipped features).
 * counters (optional): [proposed, accepted]. */
int pq_mlp_propose(void* words, int word_bits, int n, int P, int R, int cls, int stride, int csize,
                   const float* logit, const float* dE, int64_t Mpad, float qmin, float beta, uint32_t move,
                   uint64_t seed, int replica_base, unsigned long long* counters, void* stream);
/* The whole learned move of class cls in one persistent kernel: features, both
 * MLP layers as tcgen05 MMAs with TMEM accumulators, head, MH decision; the same
 * moves as pq_mlp_features + two pq_tc_gemm_bf16 + pq_mlp_head + pq_mlp_propose.
 * W1, W2: BF16 [64][64] row-major, 16-byte aligned (W1 columns >= 8 zero).
 * logit_out (nullable, FP32 [2][R*csize]): logits of the current and flipped
 * world-lines.  counters (nullable): [proposed, accepted] added to. */
int pq_mlp_learned_move(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                        const float* cpl, const float* field, int cls, int stride, int csize, float beta, float jp,
                        const void* W1, const void* W2, const float* b1, const float* b2, const float* w3, float b3,
                        float qmin, uint32_t move, uint64_t seed, int replica_base, float* logit_out,
                        unsigned long long* counters, int32_t* status, void* stream);
/* Uniform world-line move of every spin of class cls (the plain global move):
 * flip spin i in every slice with probability min(1, exp(-beta dE)); the same
 * uniforms and decision as the learned move with q = q' = 1. */
int pq_worldline_move(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                      const float* cpl, const float* field, int cls, int stride, int csize, float beta, uint32_t move,
                      uint64_t seed, int replica_base, unsigned long long* counters, void* stream);
/* A whole pass: the two moves above for classes 0..nclass-1 in order, one
 * launch per class on `stream` (class_size: host array of nclass sizes). */
int pq_mlp_learned_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                        const float* cpl, const float* field, int nclass, int stride, const int32_t* class_size,
                        float beta, float jp, const void* W1, const void* W2, const float* b1, const float* b2,
                        const float* w3, float b3, float qmin, uint32_t move, uint64_t seed, int replica_base,
                        unsigned long long* counters, int32_t* status, void* stream);
int pq_worldline_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                      const float* cpl, const float* field, int nclass, int stride, const int32_t* class_size,
                      float beta, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                      void* stream);
/* Pair world-line moves (new; no reference counterpart): the world-lines of the
 * two spins of a bond flip together in every slice.  Bonds (device slots
 * bond_i[b] < bond_j[b], total coupling bond_J[b], FP32) are grouped in classes
 * [class_start[c], class_start[c + 1]) whose bonds are at graph distance >= 2
 * (piqmc.pairs builds them), so a class's moves commute.  Cost, decision rule,
 * uniforms and features are specified in csrc/mlp.cu.  pq_pair_pass: the
 * uniform move (every bond tried, Metropolis), all classes in order.
 * pq_pair_features: rows [0, M) the 8 features of the current pairs of bonds
 * [first, first + count) of every replica (row r * count + b; BF16, ld 64), rows
 * [Mpad, Mpad + M) of the flipped pairs, dE the move's classical cost.
 * pq_pair_propose: the learned move of those bonds from the network's logits of
 * both row sets: proposed with q = clamp(sigmoid(logit), qmin, 1), accepted with
 * min(1, exp(-beta dE) q'/q).  counters (nullable): [tried/proposed, accepted].
 * A slot outside [0, n) sets *status (nullable) to PQ_ERR_BAD_INDEX.
 * pq_pair_learned_pass: the learned move of every class in order, fused (one
 * persistent launch per class: features, both layers as tcgen05 MMAs with TMEM
 * accumulators, head and decision on chip); the same moves as features + the
 * network's GEMMs + pq_pair_propose.  Weights as for pq_mlp_learned_pass; a
 * timed-out tensor-core wait sets *status to PQ_ERR_TIMEOUT. */
int pq_pair_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr, const float* cpl,
                 const float* field, const int32_t* bond_i, const int32_t* bond_j, const float* bond_J,
                 const int32_t* class_start, int nclass, float beta, uint32_t move, uint64_t seed, int replica_base,
                 unsigned long long* counters, int32_t* status, void* stream);
int pq_pair_features(const void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                     const float* cpl, const float* field, const int32_t* bond_i, const int32_t* bond_j,
                     const float* bond_J, int first, int count, float beta, float jp, void* X, float* dE,
                     int64_t Mpad, int32_t* status, void* stream);
int pq_pair_propose(void* words, int word_bits, int n, int P, int R, const int32_t* bond_i, const int32_t* bond_j,
                    int first, int count, int cls, const float* logit, const float* dE, int64_t Mpad, float qmin,
                    float beta, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                    int32_t* status, void* stream);
int pq_pair_learned_pass(void* words, int word_bits, int n, int P, int R, int maxdeg, const int32_t* nbr,
                         const float* cpl, const float* field, const int32_t* bond_i, const int32_t* bond_j,
                         const float* bond_J, const int32_t* class_start, int nclass, float beta, float jp,
                         const void* W1, const void* W2, const float* b1, const float* b2, const float* w3, float b3,
                         float qmin, uint32_t move, uint64_t seed, int replica_base, unsigned long long* counters,
                         int32_t* status, void* stream);
/* Training (BCE with soft targets y, mean over the batch B): head backward
 * (dH2 row-major and transposed, grads of w3, b3, loss), hidden backward
 * (mask by relu'(H1), transposed BF16 dH1, grad of b1), column sums, BF16
 * transpose of a [B][64] matrix, Adam update. */
int pq_mlp_head_backward(const float* H2, const float* logit, const float* y, const float* w3, int B, void* dH2,
                         void* dH2T, float* gw3, float* gb3, float* loss, void* stream);
int pq_mlp_hidden_backward(const float* G, const float* H1, int B, void* dH1T, float* gb1, void* stream);
int pq_mlp_colsum_bf16(const void* T, int cols, int B, float* out, void* stream);
int pq_mlp_transpose_bf16(const void* A, int B, void* AT, void* stream);
int pq_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps, int step,
            void* stream);

/* FP64 classical energy of every (replica, slice) from a CSR of the coupling
 * matrix (row_ptr int64 [n+1], col int32, val double; diagonal = field),
 * reference piqmc/sa.pyx:25-44: E = -sum_{(i,j) off-diag} J_ij s_i s_j - sum_i J_ii s_i,
 * every stored entry once.  words (packed) and the CSR use the same spin order;
 * out double [R][P]. */
int pq_energy_packed(const void* words, int word_bits, int n, int P, int R,
                     const int64_t* row_ptr, const int32_t* col, const double* val,
                     double* out, void* stream);

/* int8 layout [R][n][P] -> packed words [R][word_stride] and back.  perm[i] is
 * the word slot of spin i (NULL = identity, then word_stride >= n); slots that no
 * spin maps to are left untouched by packing. */
int pq_pack_spins(const int8_t* spins, int n, int P, int R, const int32_t* perm,
                  void* words, int word_bits, int word_stride, void* stream);
int pq_unpack_spins(const void* words, int word_bits, int n, int P, int R, const int32_t* perm,
                    int word_stride, int8_t* spins, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PIQMC_GB300_H */
