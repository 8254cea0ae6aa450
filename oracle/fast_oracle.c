/*
 * CPU restatement of the packed fast sweep -- TEST INFRASTRUCTURE ONLY.
 *
 * The packed kernel has no reference counterpart (the reference has no
 * parallel-correct sweep, no Philox and no world-line moves); this file
 * restates, from its specification, the algorithm that kernel runs, so the
 * GPU result can be checked bit for bit.  The algorithm itself is judged
 * against the reference statistically: its physics is qmc.QuantumAnneal
 * (reference piqmc/qmc.pyx:30-136) with the per-spin energy reset and the
 * k-1/k+1 Trotter coupling, which orc_qa_sparse(flags = FIX_Q1|FIX_Q2) runs in
 * the reference's own sequential order.
 *
 * Specification (mirrors the kernel's header comment):
 *  - M update classes (independent sets); class c = device slots [c*S, c*S + size[c]).
 *  - a sweep visits the classes in order ord[0..M-1]: identity when order_mode = 0, else
 *    Fisher-Yates with words w[] of Philox(ctr = {0xFFFFFFFF, sweep, replica, 2 << 24 | b}),
 *    b = 0, 1, ...: for j = M-1..1 swap ord[j], ord[(w[M-1-j] * (j+1)) >> 32]; parity
 *    word = w[M-1] (0 when order_mode = 0).
 *  - for the p-th visited class, slice classes in order qq = 0..nq-1, q = qq ^ bit p of
 *    the parity word when P is even (two slice classes), q = qq otherwise; slice
 *    classes: P even {even k},{odd k}; P odd {even k < P-1},{odd k},{P-1}; P = 1 {0}.
 *  - update of spin i, slice k (FP32, one rounding per op, in order):
 *      e = s_i h_i; e += J_m s_i s_jm (m = 0..maxdeg-1); t = jp s_i s_{k-1} + jp s_i s_{k+1};
 *      ediff = -2 (e + t); flip if ediff > 0 or u < expf_neg(ediff * beta).
 *  - u = ((r >> 9) + 1/2) * 2^-23, r = word (m & 3) of Philox4x32-10(ctr = {i, sweep, replica,
 *    q << 16 | m >> 2}, key = {seed lo, seed hi}) for the m-th slice of class q.
 *  - world-line move after the local sweeps of each schedule step: classes in order
 *    0..M-1, per spin E = sum_k e_k (FP32, k ascending), ediff = -2E, u from word 0 of
 *    Philox(ctr = {i, last sweep of the step, replica, 1 << 24 | gm << 16 | class}).
 *  - expf_neg: Cody-Waite reduction with ln2 = 0xB17200p-24 + lo, Taylor degree 7,
 *    0 below x = -87.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline float fbits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t bitsf(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

float orc_expf(float x) {
    if (!(x >= -87.0f)) return 0.0f;
    const float t = x * 1.44269502162933349609375f;
    const float nf = rintf(t);
    float r = fmaf(-nf, 0.693145751953125f, x);
    r = fmaf(-nf, 1.428606765330187045e-06f, r);
    float p = 1.98412701138295233249664306640625e-04f;
    p = fmaf(p, r, 1.388888922519981861114501953125e-03f);
    p = fmaf(p, r, 8.333333767950534820556640625e-03f);
    p = fmaf(p, r, 4.16666679084300994873046875e-02f);
    p = fmaf(p, r, 1.666666716337203979492187500e-01f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int n = (int)nf;
    return p * fbits((uint32_t)(n + 127) << 23);
}

/* u = (2 (r >> 9) + 1) * 2^-24: (1 + (r >> 9) * 2^-23) - (1 - 2^-24), exact in FP32 */
static inline float u01(uint32_t r) { return fbits((r >> 9) | 0x3f800000u) - 0.999999940395355224609375f; }

float orc_u01(uint32_t r) { return u01(r); }

/* Largest orc_expf(x) over the FP32 inputs with bit patterns in [lo_bits, hi_bits]
 * (negative floats: a larger pattern is more negative). */
float orc_expf_max(uint32_t lo_bits, uint32_t hi_bits) {
    float worst = 0.0f;
    for (uint64_t b = lo_bits; b <= hi_bits; ++b) {
        const float v = orc_expf(fbits((uint32_t)b));
        if (v > worst) worst = v;
    }
    return worst;
}

static inline float signed_by(float v, uint64_t w, int k) {
    return ((w >> k) & 1) ? fbits(bitsf(v) ^ 0x80000000u) : v;
}

/* local field part of one update: e = s_i h_i + sum_m J_m s_i s_jm  (FP32, in order) */
static inline float local_e(const uint64_t* w, int i, int n, int maxdeg, const int32_t* nbr,
                            const float* cpl, float h, int k) {
    const uint64_t wi = w[i];
    float e = signed_by(h, wi, k);
    for (int m = 0; m < maxdeg; ++m) {
        const int j = nbr[(int64_t)m * n + i];
        e = e + signed_by(cpl[(int64_t)m * n + i], wi ^ w[j], k);
    }
    return e;
}

static int slice_count(int P, int q) {
    if (P == 1) return 1;
    if ((P & 1) == 0) return P >> 1;
    return q == 2 ? 1 : (P - 1) >> 1;
}

static void class_order(int M, int order_mode, const uint32_t* key, uint32_t sweep, uint32_t replica,
                        int* ord, uint32_t* parity) {
    for (int c = 0; c < M; ++c) ord[c] = c;
    *parity = 0;
    if (order_mode == 0) return;
    uint32_t w[4 * 9];
    const int nb = (M + 3) / 4;
    for (int b = 0; b < nb; ++b) {
        const uint32_t ctr[4] = {0xFFFFFFFFu, sweep, replica, (2u << 24) | (uint32_t)b};
        orc_philox4x32_10(ctr, key, w + 4 * b);
    }
    for (int j = M - 1; j >= 1; --j) {
        const uint32_t k = (uint32_t)(((uint64_t)w[M - 1 - j] * (uint32_t)(j + 1)) >> 32);
        const int t = ord[j]; ord[j] = ord[k]; ord[k] = t;
    }
    *parity = w[M - 1];
}

/* One replica through nsched schedule steps; w[i] holds device slot i's world-line
 * (bit k set = -1).  betas may be NULL (then beta for every step).  Returns the
 * number of accepted local flips. */
int64_t orc_fast_anneal(int n, int P, int maxdeg, const int32_t* nbr, const float* cpl, const float* field,
                        int M, int S, const int32_t* csize, int order_mode, const float* jperp, int nsched,
                        int mcsteps, float beta, uint64_t seed, int64_t sweep_base, int replica,
                        int global_moves, uint64_t* w, const float* betas) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const int nclass_q = P == 1 ? 1 : ((P & 1) ? 3 : 2);
    int64_t nacc = 0;
    int ord[32];
    for (int g = 0; g < nsched; ++g) {
        const float jp = P == 1 ? 0.0f : jperp[g];
        const float bt = betas ? betas[g] : beta;
        for (int step = 0; step < mcsteps; ++step) {
            const uint32_t sweep = (uint32_t)(sweep_base + (int64_t)g * mcsteps + step);
            uint32_t parity;
            class_order(M, order_mode, key, sweep, (uint32_t)replica, ord, &parity);
            for (int p = 0; p < M; ++p) {
                const int cls = ord[p];
                for (int qq = 0; qq < nclass_q; ++qq) {
                    const int q = nclass_q == 2 ? (qq ^ (int)((parity >> p) & 1u)) : qq;
                    const int nq = slice_count(P, q);
                    for (int i = cls * S; i < cls * S + csize[cls]; ++i) {
                        const uint64_t wi = w[i];
                        uint64_t flips = 0;
                        for (int m = 0; m < nq; ++m) {
                            const int k = q == 2 ? P - 1 : 2 * m + q;
                            uint32_t rnd[4];
                            const uint32_t ctr[4] = {(uint32_t)i, sweep, (uint32_t)replica,
                                                     (uint32_t)((q << 16) | (m >> 2))};
                            orc_philox4x32_10(ctr, key, rnd);
                            const float e = local_e(w, i, n, maxdeg, nbr, cpl, field[i], k);
                            const int kl = k == 0 ? P - 1 : k - 1, kr = k == P - 1 ? 0 : k + 1;
                            const int bl = (int)(((wi >> k) ^ (wi >> kl)) & 1);
                            const int br = (int)(((wi >> k) ^ (wi >> kr)) & 1);
                            const float t = (bl ? -jp : jp) + (br ? -jp : jp);
                            const float ediff = -2.0f * (e + t);
                            int acc = ediff > 0.0f;
                            if (!acc) acc = u01(rnd[m & 3]) < orc_expf(ediff * bt);
                            if (acc) { flips |= (uint64_t)1 << k; ++nacc; }
                        }
                        w[i] = wi ^ flips;
                    }
                }
            }
        }
        for (int gm = 0; gm < global_moves; ++gm) {
            const uint32_t sweep = (uint32_t)(sweep_base + (int64_t)g * mcsteps + mcsteps - 1);
            const uint64_t mask = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
            for (int cls = 0; cls < M; ++cls) {
                for (int i = cls * S; i < cls * S + csize[cls]; ++i) {
                    float E = 0.0f;
                    for (int k = 0; k < P; ++k) E = E + local_e(w, i, n, maxdeg, nbr, cpl, field[i], k);
                    const float ediff = -2.0f * E;
                    uint32_t rnd[4];
                    const uint32_t ctr[4] = {(uint32_t)i, sweep, (uint32_t)replica,
                                             (uint32_t)((1u << 24) | ((uint32_t)gm << 16) | (uint32_t)cls)};
                    orc_philox4x32_10(ctr, key, rnd);
                    int acc = ediff > 0.0f;
                    if (!acc) acc = u01(rnd[0]) < orc_expf(ediff * bt);
                    if (acc) w[i] ^= mask;
                }
            }
        }
    }
    return nacc;
}

/* Largest |orc_expf(x) / exp(x) - 1| over the FP32 inputs with bit patterns in
 * [lo_bits, hi_bits] stepping by `step` (negative floats: larger pattern = more
 * negative).  Used to bound the approximation the fast paths rely on. */
double orc_expf_max_relerr(uint32_t lo_bits, uint32_t hi_bits, uint32_t step) {
    double worst = 0.0;
    for (uint64_t b = lo_bits; b <= hi_bits; b += step) {
        const float x = fbits((uint32_t)b);
        if (!(x >= -87.0f)) continue;
        const double e = exp((double)x);
        const double r = fabs((double)orc_expf(x) / e - 1.0);
        if (r > worst) worst = r;
    }
    return worst;
}

/* Restatement of the dense packed sweep of one replica (spec in the header of
 * csrc/dense.cu), starting from given FP32 fields F (P rows of N) and updating
 * them in place with the kernel's rank-1 corrections.  K: FP32 [N][N] symmetric,
 * zero diagonal; units: the integers coprime to N.  Returns accepted flips. */
int64_t orc_dense_sweep(int N, int P, float* F, const float* K, const int32_t* units, int nunits,
                        const float* jperp, int nsched, int mcsteps, float beta, uint64_t seed, int64_t sweep_base,
                        int replica, uint32_t* w, int per_slice_order) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const int nclass_q = P == 1 ? 1 : ((P & 1) ? 3 : 2);
    int64_t nacc = 0;
    for (int g = 0; g < nsched; ++g) {
        const float jp = P == 1 ? 0.0f : jperp[g];
        for (int step = 0; step < mcsteps; ++step) {
            const uint32_t sweep = (uint32_t)(sweep_base + (int64_t)g * mcsteps + step);
            for (int q = 0; q < nclass_q; ++q) {
                const int nq = slice_count(P, q);
                /* slices of one class are independent: run them one after another */
                for (int m = 0; m < nq; ++m) {
                    const int k = q == 2 ? P - 1 : 2 * m + q;
                    uint32_t ord[4];
                    const uint32_t octr[4] = {0xFFFFFFFEu, sweep, (uint32_t)replica,
                                              (3u << 24) | (uint32_t)(per_slice_order ? k : 0)};
                    orc_philox4x32_10(octr, key, ord);
                    const uint32_t a = (uint32_t)units[ord[0] % (uint32_t)nunits], b = ord[1] % (uint32_t)N;
                    float* fk = F + (size_t)k * N;
                    const int kl = k == 0 ? P - 1 : k - 1, kr = k == P - 1 ? 0 : k + 1;
                    for (int t = 0; t < N; ++t) {
                        uint32_t rnd[4];
                        const uint32_t ctr[4] = {(uint32_t)k, sweep, (uint32_t)replica, (4u << 24) | (uint32_t)(t >> 2)};
                        orc_philox4x32_10(ctr, key, rnd);
                        const int i = (int)(((uint64_t)a * (uint32_t)t + b) % (uint32_t)N);
                        const uint32_t wi = w[i];
                        const int sbit = (int)((wi >> k) & 1u);
                        const float e = sbit ? -fk[i] : fk[i];
                        const int bl = (int)(((wi >> k) ^ (wi >> kl)) & 1u), br = (int)(((wi >> k) ^ (wi >> kr)) & 1u);
                        const float tt = (bl ? -jp : jp) + (br ? -jp : jp);
                        const float ediff = -2.0f * (e + tt);
                        int acc = ediff > 0.0f;
                        if (!acc) acc = u01(rnd[t & 3]) < orc_expf(ediff * beta);
                        if (acc) {
                            const float c = sbit ? 2.0f : -2.0f;
                            const float* Ki = K + (size_t)i * N;
                            for (int j = 0; j < N; ++j) fk[j] = fmaf(c, Ki[j], fk[j]);
                            w[i] ^= 1u << k;
                            ++nacc;
                        }
                    }
                }
            }
        }
    }
    return nacc;
}

/* ---------------------------------------------------------------------------
 * Pair world-line moves (this library's own move; no reference counterpart),
 * restated from the specification in csrc/mlp.cu: the world-lines of the two
 * spins of a bond flip together.  One replica; w holds device slot i's
 * world-line (bit k set = -1).  FP32, one rounding per operation, in order.
 * ------------------------------------------------------------------------- */
static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

/* sum_k s^k f^k of slot s: h (P - 2 popc(w_s)), then + J_m (P - 2 popc(w_s ^ w_m)), m in table order */
static float wl_align(const uint64_t* w, int s, uint64_t ws, int n, int P, int maxdeg, const int32_t* nbr,
                      const float* cpl, const float* field, int si, int sj, uint64_t fi, uint64_t fj, int flipped) {
    const uint64_t mask = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
    float sa = field[s] * (float)(P - 2 * popc64(ws & mask));
    for (int m = 0; m < maxdeg; ++m) {
        const int j = nbr[(int64_t)m * n + s];
        uint64_t wm = w[j];
        if (flipped) wm = j == sj ? fj : (j == si ? fi : wm);
        sa = sa + cpl[(int64_t)m * n + s] * (float)(P - 2 * popc64((ws ^ wm) & mask));
    }
    return sa;
}

static float clip8f(float v) { return v < -8.0f ? -8.0f : (v > 8.0f ? 8.0f : v); }

/* Features x[8] and cost of the pair (si, sj) in the current state (flipped = 0) or
 * with both world-lines flipped (flipped = 1).  Returns the cost dE. */
float orc_pair_features(const uint64_t* w, int n, int P, int maxdeg, const int32_t* nbr, const float* cpl,
                        const float* field, int si, int sj, float Jb, float beta, float jp, int flipped, float* x) {
    const uint64_t mask = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
    const uint64_t fi = w[si] ^ mask, fj = w[sj] ^ mask;
    const uint64_t wi = flipped ? fi : w[si], wj = flipped ? fj : w[sj];
    const float dEi = 2.0f * wl_align(w, si, wi, n, P, maxdeg, nbr, cpl, field, si, sj, fi, fj, flipped);
    const float dEj = 2.0f * wl_align(w, sj, wj, n, P, maxdeg, nbr, cpl, field, si, sj, fi, fj, flipped);
    const int c = P - 2 * popc64((wi ^ wj) & mask);
    const float dE = (dEi + dEj) - 4.0f * (Jb * (float)c);
    if (x) {
        const float inv = 1.0f / (float)P;
        const uint64_t mi = wi & mask, mj = wj & mask;
        const uint64_t roti = ((mi >> 1) | (mi << (P - 1))) & mask, rotj = ((mj >> 1) | (mj << (P - 1))) & mask;
        x[0] = clip8f((beta * dE) * inv);
        x[1] = clip8f((beta * dEi) * inv);
        x[2] = clip8f((beta * dEj) * inv);
        x[3] = ((Jb * (float)c) * inv) / (1.0f + fabsf(Jb));
        x[4] = (float)(popc64(mi ^ roti) + popc64(mj ^ rotj)) / (float)(2 * P);
        x[5] = ((float)(P - 2 * popc64(mi)) * inv) * ((float)(P - 2 * popc64(mj)) * inv);
        {
            float v = (jp * beta) * inv;
            x[6] = v < 0.0f ? 0.0f : (v > 8.0f ? 8.0f : v);
        }
        x[7] = 1.0f;
    }
    return dE;
}

float orc_pair_sigmoid(float z) {
    if (z >= 0.0f) return 1.0f / (1.0f + orc_expf(-z));
    const float e = orc_expf(z);
    return e / (1.0f + e);
}

int orc_pair_accept(float dE, float beta, float q, float qf, float u) {
    const float x = -(beta * dE);
    const float uq = u * q;
    if (x <= 0.0f) return uq < qf * orc_expf(x);
    return (uq * orc_expf(-x)) < qf;
}

/* The pair moves of bonds [first, first + count) of class cls for one replica.
 * logit == NULL: the uniform move (q = q' = 1); else logit[b - first] scores the
 * current pair and logit_f[b - first] the flipped one.  Returns accepted moves. */
int64_t orc_pair_class(uint64_t* w, int n, int P, int maxdeg, const int32_t* nbr, const float* cpl,
                       const float* field, const int32_t* bi, const int32_t* bj, const float* bJ, int first,
                       int count, int cls, float beta, float qmin, const float* logit, const float* logit_f,
                       uint32_t move, uint64_t seed, uint32_t replica) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint64_t mask = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
    int64_t nacc = 0;
    /* the moves of a class commute: decide all from the state at the start of the class */
    uint8_t* flip = (uint8_t*)__builtin_alloca(count > 0 ? count : 1);
    for (int t = 0; t < count; ++t) {
        const int b = first + t;
        uint32_t u[4];
        const uint32_t ctr[4] = {(uint32_t)b, move, replica, (5u << 24) | (uint32_t)cls};
        orc_philox4x32_10(ctr, key, u);
        const float dE = orc_pair_features(w, n, P, maxdeg, nbr, cpl, field, bi[b], bj[b], bJ[b], beta, 0.0f, 0, NULL);
        float q = 1.0f, qf = 1.0f;
        if (logit) {
            q = orc_pair_sigmoid(logit[t]);
            q = q < qmin ? qmin : (q > 1.0f ? 1.0f : q);
            qf = orc_pair_sigmoid(logit_f[t]);
            qf = qf < qmin ? qmin : (qf > 1.0f ? 1.0f : qf);
        }
        const int proposed = u01(u[0]) < q;
        flip[t] = (uint8_t)(proposed && orc_pair_accept(dE, beta, q, qf, u01(u[1])));
    }
    for (int t = 0; t < count; ++t)
        if (flip[t]) {
            w[bi[first + t]] ^= mask;
            w[bj[first + t]] ^= mask;
            ++nacc;
        }
    return nacc;
}
