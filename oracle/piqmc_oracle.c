/*
 * piqmc CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's annealing sweeps, used to check
 * the CUDA kernels.  Nothing in the product links, loads or calls this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs do.
 *
 * Pinned against the compiled reference (tests/golden/, generated by
 * tests/golden/make_golden.py from the reference's own Cython modules).
 *
 * Conventions shared by every routine:
 *   spins   int8 +-1, spin-major: s[i*P + k] is spin i in Trotter slice k.
 *   nb_idx  int32 [n*maxnb]: C (int) truncation of nbs[i, m, 0]
 *           (reference piqmc/qmc.pyx:104, generated piqmc/qmc.c:2168).
 *   nb_j    float [n*maxnb]: nbs[i, m, 1] rounded to FP32, because the
 *           reference stores it into `cdef float jval` (piqmc/qmc.pyx:86,106).
 *   perms   int64 [(nsched*mcsteps) * n]: the spin order of each MC sweep,
 *           i.e. the successive results of rng.permutation
 *           (piqmc/qmc.pyx:90-91, :136).
 *   rands   int32 [nrand]: successive libc rand() values; one is consumed
 *           only when the Metropolis test reaches its random branch
 *           (piqmc/qmc.pyx:132, generated piqmc/qmc.c:2417-2428).
 * Return value: number of rand() values consumed, or -1 if `rands` ran out.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_FIX_Q2 1 /* reset ediff per spin instead of per slice */
#define ORC_FIX_Q1 2 /* couple slice k to k-1 and k+1 (periodic) instead of P-1 and 1 */

/* ediff = (float)((double)ediff + t) where t is a double; generated C at
 * piqmc/qmc.c:2201/2233/2346/2375 accumulates into a float this way. */
static inline float acc(float ediff, double t) { return (float)((double)ediff + t); }

/* Accept test of piqmc/qmc.pyx:130-133 (strict ">") and piqmc/sa.pyx:114-117
 * (">=" when ge != 0).  ediff/temp is an FP32 divide; exp is libm's double
 * exp; the uniform is rand()/(double)RAND_MAX. */
static inline int metropolis(float ediff, float temp, int ge, const int32_t* rands, int64_t nrand,
                             int64_t* used, int* exhausted) {
    if (ge ? (ediff >= 0.0f) : (ediff > 0.0f)) return 1;
    if (*used >= nrand) { *exhausted = 1; return 0; }
    int32_t r = rands[(*used)++];
    return exp((double)(ediff / temp)) > (double)r / (double)RAND_MAX;
}

/* qmc.QuantumAnneal, reference piqmc/qmc.pyx:30-136. flags = 0 reproduces the
 * shipped code (Q1: tidx never assigned, so tleft = P-1 and tright = 1 for
 * every slice, :115-117; Q2: ediff reset once per slice, :134-135).  n rows of
 * spins and neighbours; each sweep updates the nperm <= n spins its order lists
 * (the reference's nspins argument, :91), so rows past them are read-only
 * boundary spins; perms is [nsched*mcsteps][nperm]. */
int64_t orc_qa_sparse(int n, int nperm, int P, int maxnb, const int32_t* nb_idx, const float* nb_j,
                      const float* jperp, int nsched, int mcsteps, float temp,
                      const int64_t* perms, const int32_t* rands, int64_t nrand,
                      int8_t* s, int flags) {
    int64_t used = 0;
    int exhausted = 0;
    for (int g = 0; g < nsched; ++g) {
        const float jp = jperp[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int64_t* perm = perms + (int64_t)(g * mcsteps + step) * nperm;
            for (int k = 0; k < P; ++k) {
                float ediff = 0.0f;
                int tl = P - 1, tr = 1;
                if (flags & ORC_FIX_Q1) { tl = (k + P - 1) % P; tr = (k + 1) % P; }
                for (int t = 0; t < nperm; ++t) {
                    const int i = (int)perm[t];
                    if (flags & ORC_FIX_Q2) ediff = 0.0f;
                    const double si = (double)s[(int64_t)i * P + k];
                    for (int m = 0; m < maxnb; ++m) {
                        const int j = nb_idx[(int64_t)i * maxnb + m];
                        const float jv = nb_j[(int64_t)i * maxnb + m];
                        if (j == i) ediff = acc(ediff, -2.0 * si * (double)jv);
                        else ediff = acc(ediff, -2.0 * si * ((double)jv * (double)s[(int64_t)j * P + k]));
                    }
                    ediff = acc(ediff, -2.0 * si * ((double)jp * (double)s[(int64_t)i * P + tl]));
                    ediff = acc(ediff, -2.0 * si * ((double)jp * (double)s[(int64_t)i * P + tr]));
                    if (metropolis(ediff, temp, 0, rands, nrand, &used, &exhausted))
                        s[(int64_t)i * P + k] = (int8_t)-s[(int64_t)i * P + k];
                    if (exhausted) return -1;
                }
            }
        }
    }
    return used;
}

/* qmc.QuantumAnneal_dense, reference piqmc/qmc.pyx:141-242.  J is dense
 * float64 row-major n*n; only the upper triangle and the diagonal are read
 * (:208-219).  The coupling is not rounded to FP32 here (it is read straight
 * from the double matrix), so each term is a full double. */
int64_t orc_qa_dense(int n, int P, const double* J, const float* jperp, int nsched, int mcsteps,
                     float temp, const int64_t* perms, const int32_t* rands, int64_t nrand,
                     int8_t* s, int flags) {
    int64_t used = 0;
    int exhausted = 0;
    for (int g = 0; g < nsched; ++g) {
        const float jp = jperp[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int64_t* perm = perms + (int64_t)(g * mcsteps + step) * n;
            for (int k = 0; k < P; ++k) {
                float ediff = 0.0f;
                int tl = P - 1, tr = 1;
                if (flags & ORC_FIX_Q1) { tl = (k + P - 1) % P; tr = (k + 1) % P; }
                for (int t = 0; t < n; ++t) {
                    const int i = (int)perm[t];
                    if (flags & ORC_FIX_Q2) ediff = 0.0f;
                    const double si = (double)s[(int64_t)i * P + k];
                    for (int j = 0; j < n; ++j) {
                        if (j == i) {
                            ediff = acc(ediff, -2.0 * si * J[(int64_t)i * n + i]);
                        } else {
                            const double jv = i < j ? J[(int64_t)i * n + j] : J[(int64_t)j * n + i];
                            ediff = acc(ediff, -2.0 * si * (jv * (double)s[(int64_t)j * P + k]));
                        }
                    }
                    ediff = acc(ediff, -2.0 * si * ((double)jp * (double)s[(int64_t)i * P + tl]));
                    ediff = acc(ediff, -2.0 * si * ((double)jp * (double)s[(int64_t)i * P + tr]));
                    if (metropolis(ediff, temp, 0, rands, nrand, &used, &exhausted))
                        s[(int64_t)i * P + k] = (int8_t)-s[(int64_t)i * P + k];
                    if (exhausted) return -1;
                }
            }
        }
    }
    return used;
}

/* sa.Anneal, reference piqmc/sa.pyx:50-120.  temps[g] is sched[g] rounded to
 * FP32 (`cdef float temp`, :84, :96); ediff is reset per spin (:119); the
 * deterministic branch accepts on ediff >= 0 (:114). */
int64_t orc_sa_sparse(int n, int maxnb, const int32_t* nb_idx, const float* nb_j,
                      const float* temps, int nsched, int mcsteps,
                      const int64_t* perms, const int32_t* rands, int64_t nrand, int8_t* s) {
    int64_t used = 0;
    int exhausted = 0;
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int64_t* perm = perms + (int64_t)(g * mcsteps + step) * n;
            for (int t = 0; t < n; ++t) {
                const int i = (int)perm[t];
                float ediff = 0.0f;
                const double si = (double)s[i];
                for (int m = 0; m < maxnb; ++m) {
                    const int j = nb_idx[(int64_t)i * maxnb + m];
                    const float jv = nb_j[(int64_t)i * maxnb + m];
                    if (j == i) ediff = acc(ediff, -2.0 * si * (double)jv);
                    else ediff = acc(ediff, -2.0 * si * ((double)jv * (double)s[j]));
                }
                if (metropolis(ediff, temp, 1, rands, nrand, &used, &exhausted)) s[i] = (int8_t)-s[i];
                if (exhausted) return -1;
            }
        }
    }
    return used;
}

/* J-perp schedule of reference piqmc/qmc.pyx:95 in the generated C's types
 * (piqmc/qmc.c:2063-2075): slices*temp is an FP32 product, the quotient and
 * log/tanh are double, the result is stored to FP32. */
/* sa.Anneal_dense, reference piqmc/sa.pyx:126-187: dense float64 J, upper
 * triangle for pairs and the diagonal as field (:170-179), ediff reset per spin
 * (:186), deterministic accept on ediff > 0 (:181). */
int64_t orc_sa_dense(int n, const double* J, const float* temps, int nsched, int mcsteps, const int64_t* perms,
                     const int32_t* rands, int64_t nrand, int8_t* s) {
    int64_t used = 0;
    int exhausted = 0;
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            const int64_t* perm = perms + (int64_t)(g * mcsteps + step) * n;
            for (int t = 0; t < n; ++t) {
                const int i = (int)perm[t];
                const double si = (double)s[i];
                float ediff = 0.0f;
                for (int j = 0; j < n; ++j) {
                    if (j == i) {
                        ediff = acc(ediff, -2.0 * si * J[(int64_t)i * n + i]);
                    } else {
                        const double jv = i < j ? J[(int64_t)i * n + j] : J[(int64_t)j * n + i];
                        ediff = acc(ediff, -2.0 * si * (jv * (double)s[j]));
                    }
                }
                if (metropolis(ediff, temp, 0, rands, nrand, &used, &exhausted)) s[i] = (int8_t)-s[i];
                if (exhausted) return -1;
            }
        }
    }
    return used;
}

/* sa.Anneal_bipartite, reference piqmc/sa.pyx:411-500: left spins in index
 * order then right spins; ediff -= 2 l_i J_ij r_j + lb_i l_i + rb_j r_j over the
 * other side (:466-468, :478-480), FP64 terms into the FP32 accumulator. */
int64_t orc_sa_bipartite(int nl, int nr, const double* J, const double* lbias, const double* rbias,
                         const float* temps, int nsched, int mcsteps, const int32_t* rands, int64_t nrand,
                         int8_t* lv, int8_t* rv) {
    int64_t used = 0;
    int exhausted = 0;
    for (int g = 0; g < nsched; ++g) {
        const float temp = temps[g];
        for (int step = 0; step < mcsteps; ++step) {
            for (int i = 0; i < nl; ++i) {
                const double li = (double)lv[i];
                float ediff = 0.0f;
                for (int j = 0; j < nr; ++j) {
                    const double rj = (double)rv[j];
                    ediff = (float)((double)ediff - (2.0 * li * J[(int64_t)i * nr + j] * rj + lbias[i] * li +
                                                     rbias[j] * rj));
                }
                if (metropolis(ediff, temp, 0, rands, nrand, &used, &exhausted)) lv[i] = (int8_t)-lv[i];
                if (exhausted) return -1;
            }
            for (int i = 0; i < nr; ++i) {
                const double ri = (double)rv[i];
                float ediff = 0.0f;
                for (int j = 0; j < nl; ++j) {
                    const double lj = (double)lv[j];
                    ediff = (float)((double)ediff - (2.0 * ri * J[(int64_t)j * nr + i] * lj + lbias[j] * lj +
                                                     rbias[i] * ri));
                }
                if (metropolis(ediff, temp, 0, rands, nrand, &used, &exhausted)) rv[i] = (int8_t)-rv[i];
                if (exhausted) return -1;
            }
        }
    }
    return used;
}

void orc_jperp(const double* sched, int nsched, int P, float temp, float* out) {
    for (int g = 0; g < nsched; ++g) {
        const float pt = (float)P * temp;
        out[g] = (float)(((-0.5 * P) * (double)temp) * log(tanh(sched[g] / (double)pt)));
    }
}

/* Successive values of this process's libc rand() (the stream the reference
 * draws from). */
void orc_libc_rand(int32_t* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = rand();
}
void orc_libc_srand(unsigned seed) { srand(seed); }
