/*
 * The packed sweep with quiet sites skipped, on the CPU -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the staged phase of csrc/sweep_core.cuh for even P: a phase visits only
 * the sites whose quiet bit is clear (site_visit: class sums settle whole slice
 * classes, the rest is decided slice by slice), and a visit sets the site's bit when
 * every slice of both classes is a rejection whatever its uniform and no slice's sum
 * can fall as J-perp grows.  Any change of a word clears the bits of the site and its
 * neighbours; the first sweep of a call, and of a step whose J-perp or beta is below
 * the previous step's, visits every site and rewrites its bit.
 *
 * tests/test_quiet_sites.py runs this beside orc_fast_anneal (oracle/fast_oracle.c,
 * the per-slice specification, which visits every site) and requires the same final
 * words and accept count: skipping quiet sites must change nothing.  `breaks` removes
 * one part of the rule (1: neighbours' bits are not cleared on a change; 2: slices
 * with both Trotter partners opposite count as calm; 4: no step ever rewrites the
 * bits), for the test's negative controls.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
float orc_expf(float x);

static inline float fbits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t bitsf(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
static inline float u01(uint32_t r) { return fbits((r >> 9) | 0x3f800000u) - 0.999999940395355224609375f; }
static inline float sgn(float v, uint64_t w, int k) { return ((w >> k) & 1) ? fbits(bitsf(v) ^ 0x80000000u) : v; }
static inline float settled_x(void) { return fbits(0xc1851592u); }

/* smallest s >= 0 with fl(s * m2beta) <= settled_x(), by bisection; +inf when m2beta >= 0 */
static float settle_threshold(float m2beta) {
    if (!(m2beta < 0.0f)) return fbits(0x7f800000u);
    uint32_t lo = 0u, hi = 0x7f800000u;
    while (hi - lo > 1u) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        const float prod = fbits(mid) * m2beta;
        if (prod <= settled_x()) hi = mid;
        else lo = mid;
    }
    return fbits(hi);
}

static void class_order(int M, int order_mode, const uint32_t* key, uint32_t sweep, uint32_t replica, int* ord,
                        uint32_t* parity) {
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

enum { KEPT = 0, QUIET = 1, CHANGED = 2 };

typedef struct {
    int n, P, maxdeg;
    const int32_t* nbr;
    const float* cpl;
    const float* field;
    const uint32_t* key;
    int breaks;
} Sim;

static int visit(const Sim* s, uint64_t* w, int i, uint32_t first, float jp, uint32_t sweep, uint32_t rep,
                 float m2beta, float smin, int64_t* nacc) {
    const int P = s->P, NQ = P / 2, n = s->n;
    uint64_t CM0 = 0;
    for (int k = 0; k < NQ; ++k) CM0 |= (uint64_t)1 << (2 * k);
    const uint64_t IN0 = CM0 & ~((uint64_t)1 << (P - 2));
    const uint64_t MASK = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
    const uint64_t w0 = w[i];
    uint64_t wi = w0, d[64];
    float J[64];
    for (int m = 0; m < s->maxdeg; ++m) {
        d[m] = wi ^ w[s->nbr[(int64_t)m * n + i]];
        J[m] = s->cpl[(int64_t)m * n + i];
    }
    const float h = s->field[i];
    const float X = settled_x();
    int qq = 0;
    if (((wi ^ (wi >> 2)) & (IN0 | (IN0 << 1))) == 0) {
        uint64_t full = wi ^ (wi >> 1);
        for (int m = 0; m < s->maxdeg; ++m) full |= d[m] ^ (d[m] >> 1);
        if ((full & (MASK >> 1)) == 0) {
            float e = sgn(h, wi, 0);
            for (int m = 0; m < s->maxdeg; ++m) e = e + sgn(J[m], d[m], 0);
            const float sum = e + (jp + jp);
            if (sum >= 0.0f) {
                if (sum * m2beta <= X) return QUIET;
            } else {
                const uint64_t fl = CM0 << first;
                const float mjp = -jp;
                const float sum2 = e + (mjp + mjp);
                uint64_t fl2 = 0;
                qq = 2;
                if (sum2 < 0.0f) fl2 = CM0 << (first ^ 1u);
                else if (!(sum2 * m2beta <= X)) qq = 1;
                wi ^= fl | fl2;
                for (int m = 0; m < s->maxdeg; ++m) d[m] ^= fl | fl2;
                *nacc += __builtin_popcountll(fl | fl2);
            }
        } else {
            uint64_t nbx = 0;
            for (int m = 0; m < s->maxdeg; ++m) nbx |= d[m] ^ (d[m] >> 2);
            for (; qq < 2; ++qq) {
                const int q = qq ^ (int)first;
                if (nbx & (IN0 << q)) break;
                const uint64_t up = ((wi << 1) | (wi >> (P - 1))) & MASK;
                const uint64_t dn = ((wi >> 1) | (wi << (P - 1))) & MASK;
                float e = sgn(h, wi, q);
                for (int m = 0; m < s->maxdeg; ++m) e = e + sgn(J[m], d[m], q);
                const float t = sgn(jp, wi ^ up, q) + sgn(jp, wi ^ dn, q);
                const float sum = e + t;
                uint64_t fl;
                if (sum < 0.0f) fl = CM0 << q;
                else if (sum * m2beta <= X) fl = 0;
                else break;
                wi ^= fl;
                for (int m = 0; m < s->maxdeg; ++m) d[m] ^= fl;
                *nacc += __builtin_popcountll(fl);
            }
        }
    }
    int calm = qq == 0;
    for (; qq < 2; ++qq) {
        const int q = qq ^ (int)first;
        const uint64_t up = ((wi << 1) | (wi >> (P - 1))) & MASK;
        const uint64_t dn = ((wi >> 1) | (wi << (P - 1))) & MASK;
        const uint64_t dlw = wi ^ up, drw = wi ^ dn;
        if (!(s->breaks & 2) && (dlw & drw & (CM0 << q))) calm = 0;
        uint64_t flips = 0;
        uint32_t rnd[4];
        for (int m = 0; m < NQ; ++m) {
            const int k = 2 * m + q;
            if ((m & 3) == 0) {
                const uint32_t ctr[4] = {(uint32_t)i, sweep, rep, (uint32_t)((q << 16) | (m >> 2))};
                orc_philox4x32_10(ctr, s->key, rnd);
            }
            float e = sgn(h, wi, k);
            for (int mm = 0; mm < s->maxdeg; ++mm) e = e + sgn(J[mm], d[mm], k);
            const float t = sgn(jp, dlw, k) + sgn(jp, drw, k);
            const float sum = e + t;
            if (!(sum >= smin)) calm = 0;
            const int acc = sum < 0.0f || u01(rnd[m & 3]) < orc_expf(sum * m2beta);
            if (acc) flips |= (uint64_t)1 << k;
        }
        wi ^= flips;
        for (int mm = 0; mm < s->maxdeg; ++mm) d[mm] ^= flips;
        *nacc += __builtin_popcountll(flips);
    }
    if (wi == w0) return calm ? QUIET : KEPT;
    w[i] = wi;
    return CHANGED;
}

static void clear_around(const Sim* s, unsigned char* quiet, int i) {
    quiet[i] = 0;
    if (s->breaks & 1) return;
    for (int m = 0; m < s->maxdeg; ++m) quiet[s->nbr[(int64_t)m * s->n + i]] = 0;
}

/* One replica through nsched steps, as orc_fast_anneal (same arguments and result);
 * visits: site visits made (sites skipped as quiet are not counted). */
int64_t qsim_anneal(int n, int P, int maxdeg, const int32_t* nbr, const float* cpl, const float* field, int M,
                    int S, const int32_t* csize, int order_mode, const float* jperp, int nsched, int mcsteps,
                    float beta, uint64_t seed, int64_t sweep_base, int replica, int global_moves, uint64_t* w,
                    const float* betas, int breaks, int64_t* visits) {
    if (P < 2 || (P & 1) || P > 64) return -1;
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    Sim s = {n, P, maxdeg, nbr, cpl, field, key, breaks};
    unsigned char* quiet = (unsigned char*)calloc((size_t)n, 1);
    int64_t nacc = 0;
    *visits = 0;
    int ord[32];
    for (int g = 0; g < nsched; ++g) {
        const float jp = jperp[g];
        const float bt = betas ? betas[g] : beta;
        const float m2beta = -2.0f * bt;
        const float smin = settle_threshold(m2beta);
        int renew = 1;
        if (g > 0) {
            const float jp_prev = jperp[g - 1], bt_prev = betas ? betas[g - 1] : beta;
            renew = !(jp >= jp_prev && bt >= bt_prev && bt_prev > 0.0f);
        }
        if (g > 0 && (breaks & 4)) renew = 0;
        for (int step = 0; step < mcsteps; ++step) {
            const int fresh = renew && step == 0;
            const uint32_t sweep = (uint32_t)(sweep_base + (int64_t)g * mcsteps + step);
            uint32_t parity;
            class_order(M, order_mode, key, sweep, (uint32_t)replica, ord, &parity);
            for (int p = 0; p < M; ++p) {
                const int cls = ord[p];
                const uint32_t first = (parity >> p) & 1u;
                for (int i = cls * S; i < cls * S + csize[cls]; ++i) {
                    if (!fresh && quiet[i]) continue;
                    ++*visits;
                    const int v = visit(&s, w, i, first, jp, sweep, (uint32_t)replica, m2beta, smin, &nacc);
                    if (v == QUIET) {
                        quiet[i] = 1;
                    } else {
                        if (fresh) quiet[i] = 0;
                        if (v == CHANGED) clear_around(&s, quiet, i);
                    }
                }
            }
        }
        for (int gm = 0; gm < global_moves; ++gm) {
            const uint32_t sweep = (uint32_t)(sweep_base + (int64_t)g * mcsteps + mcsteps - 1);
            const uint64_t mask = P >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << P) - 1);
            for (int cls = 0; cls < M; ++cls) {
                for (int i = cls * S; i < cls * S + csize[cls]; ++i) {
                    const uint64_t wi = w[i];
                    float E = 0.0f;
                    for (int k = 0; k < P; ++k) {
                        float e = sgn(field[i], wi, k);
                        for (int m = 0; m < maxdeg; ++m)
                            e = e + sgn(cpl[(int64_t)m * n + i], wi ^ w[nbr[(int64_t)m * n + i]], k);
                        E = E + e;
                    }
                    uint32_t rnd[4];
                    const uint32_t ctr[4] = {(uint32_t)i, sweep, (uint32_t)replica,
                                             (uint32_t)((1u << 24) | ((uint32_t)gm << 16) | (uint32_t)cls)};
                    orc_philox4x32_10(ctr, key, rnd);
                    const float ediff = -2.0f * E;
                    int acc = ediff > 0.0f;
                    if (!acc) acc = u01(rnd[0]) < orc_expf(ediff * bt);
                    if (acc) {
                        w[i] ^= mask;
                        clear_around(&s, quiet, i);
                    }
                }
            }
        }
    }
    free(quiet);
    return nacc;
}
