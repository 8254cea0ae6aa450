// Host-side parts of the C ABI: schedule arithmetic, the libc rand() stream,
// the neighbour table builder and the colouring used by the packed sweeps.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <tuple>
#include <vector>

#include "piqmc_gb300.h"

static_assert(RAND_MAX == 2147483647, "the reference-order kernels assume glibc's RAND_MAX");

extern "C" {

int pq_version(void) { return 1; }

const char* pq_strerror(int status) {
    switch (status) {
        case PQ_OK: return "ok";
        case PQ_ERR_INVALID_ARG: return "invalid argument";
        case PQ_ERR_BAD_INDEX: return "index outside [0, nspins)";
        case PQ_ERR_RAND_EXHAUSTED: return "uniform stream exhausted";
        case PQ_ERR_UNSUPPORTED: return "unsupported configuration";
        case PQ_ERR_TOO_LARGE: return "problem too large for this kernel";
        case PQ_ERR_TIMEOUT: return "bounded device wait timed out";
        case PQ_ERR_LIBC_STATE: return "libc rand() state layout not supported";
        case PQ_ERR_NO_DEVICE: return "no CUDA device";
        default: return status < 0 ? "CUDA error" : "unknown status";
    }
}

// J-perp = -0.5*P*T*log(tanh(G/(P*T))) in the generated C's types
// (reference piqmc/qmc.pyx:95, piqmc/qmc.c:2063-2075).
int pq_jperp_schedule(const double* sched, int nsched, int P, float temp, float* out) {
    if (nsched < 0 || (nsched > 0 && (!sched || !out))) return PQ_ERR_INVALID_ARG;
    const float pt = (float)P * temp;
    if (nsched > 0 && pt == 0.0f) return PQ_ERR_INVALID_ARG;
    for (int g = 0; g < nsched; ++g)
        out[g] = (float)(((-0.5 * P) * (double)temp) * log(tanh(sched[g] / (double)pt)));
    return PQ_OK;
}

// ---------------------------------------------------------------------------
// libc rand() stream.  glibc keeps the generator state in an int32 array whose
// word [-1] holds (rear pointer offset * 5 + type) while the array is not the
// live one (written by initstate/setstate when switching away).  Switching to a
// scratch array therefore exposes the live array with its position, which is
// copied, and switching back restores it.
// ---------------------------------------------------------------------------
static int32_t g_scratch[64];

static int live_state(char** live, size_t* bytes) {
    static const int kDeg[5] = {0, 7, 15, 31, 63};
    char* p = initstate(1u, (char*)g_scratch, sizeof g_scratch);
    if (!p) return PQ_ERR_LIBC_STATE;
    int32_t info;
    memcpy(&info, p, sizeof info);
    const int type = info % 5;
    if (info < 0 || type < 0 || type > 4) { setstate(p); return PQ_ERR_LIBC_STATE; }
    *live = p;
    *bytes = sizeof(int32_t) * (size_t)(1 + kDeg[type]);
    return PQ_OK;
}

int pq_libc_rand_peek(int32_t* out, int64_t n) {
    if (n < 0 || (n > 0 && !out)) return PQ_ERR_INVALID_ARG;
    char* live = nullptr;
    size_t bytes = 0;
    int st = live_state(&live, &bytes);
    if (st) return st;
    std::vector<char> saved(live, live + bytes);
    setstate(live);
    for (int64_t i = 0; i < n; ++i) out[i] = rand();
    // put the saved words and position back
    char* again = initstate(1u, (char*)g_scratch, sizeof g_scratch);
    if (again != live) { setstate(again); return PQ_ERR_LIBC_STATE; }
    memcpy(live, saved.data(), bytes);
    setstate(live);
    return PQ_OK;
}

int pq_libc_rand_skip(int64_t n) {
    if (n < 0) return PQ_ERR_INVALID_ARG;
    for (int64_t i = 0; i < n; ++i) (void)rand();
    return PQ_OK;
}

// libm exp of FP32 inputs, the host side of the reference-order kernels' exp check.
int pq_host_exp(const float* x, double* y, int64_t n) {
    if (n < 0 || (n > 0 && (!x || !y))) return PQ_ERR_INVALID_ARG;
    for (int64_t i = 0; i < n; ++i) y[i] = exp((double)x[i]);
    return PQ_OK;
}

// Count inputs in [first_bits, first_bits+count) whose libm exp differs from dev[i]
// and write up to cap of them (bits and libm value).
int64_t pq_host_exp_compare(uint32_t first_bits, int64_t count, const double* dev, uint32_t* bad_x,
                            double* bad_y, int64_t cap) {
    int64_t nbad = 0;
    for (int64_t i = 0; i < count; ++i) {
        const uint32_t b = first_bits + (uint32_t)i;
        float xf;
        memcpy(&xf, &b, sizeof xf);
        const double h = exp((double)xf);
        if (memcmp(&h, &dev[i], sizeof h) != 0 && !(h != h && dev[i] != dev[i])) {
            if (nbad < cap) { bad_x[nbad] = b; bad_y[nbad] = h; }
            ++nbad;
        }
    }
    return nbad;
}

// tools.GenerateNeighbors in one pass over the DOK keys (reference
// piqmc/tools.pyx:77-92 scans all keys once per spin): key (a, b) appends
// [b, J] to row a and, when b != a, [a, J] to row b, so each row keeps key order.
int pq_generate_neighbors(int nspins, int64_t nkeys, const int64_t* rows, const int64_t* cols,
                          const double* vals, int maxnb, double* out) {
    if (nspins < 0 || nkeys < 0 || maxnb < 0 || (nkeys > 0 && (!rows || !cols || !vals)) ||
        (nspins > 0 && maxnb > 0 && !out))
        return PQ_ERR_INVALID_ARG;
    memset(out, 0, sizeof(double) * 2 * (size_t)nspins * (size_t)maxnb);
    std::vector<int> fill((size_t)nspins, 0);
    for (int64_t t = 0; t < nkeys; ++t) {
        const int64_t a = rows[t], b = cols[t];
        const double v = vals[t];
        if (a >= 0 && a < nspins) {
            if (fill[a] >= maxnb) return PQ_ERR_TOO_LARGE;
            double* e = out + ((size_t)a * maxnb + fill[a]++) * 2;
            e[0] = (double)b;
            e[1] = v;
        }
        if (b != a && b >= 0 && b < nspins) {
            if (fill[b] >= maxnb) return PQ_ERR_TOO_LARGE;
            double* e = out + ((size_t)b * maxnb + fill[b]++) * 2;
            e[0] = (double)a;
            e[1] = v;
        }
    }
    return PQ_OK;
}

// Greedy colouring in spin order over the undirected coupling graph (an entry
// (i, j, J) with j != i and J != 0 couples i and j in both directions).  When
// that needs more than two colours, DSatur (Brelaz, "New methods to color the
// vertices of a graph", CACM 1979: colour next the uncoloured vertex with the
// most distinct colours among its neighbours, ties by degree, then by index)
// is run as well and the colouring with fewer colours is kept, greedy on a tie.
// A periodic lattice of odd side gets 3 colours this way instead of greedy's 4;
// two-colourable graphs keep greedy's colouring.
static int greedy_colors(int n, const std::vector<std::vector<int>>& adj, int32_t* color) {
    int ncol = 0;
    std::vector<int> mark;
    for (int i = 0; i < n; ++i) color[i] = -1;
    for (int i = 0; i < n; ++i) {
        mark.assign((size_t)ncol + 1, 0);
        for (int j : adj[i])
            if (color[j] >= 0) mark[color[j]] = 1;
        int c = 0;
        while (mark[c]) ++c;
        color[i] = c;
        ncol = std::max(ncol, c + 1);
    }
    return ncol;
}

static int dsatur_colors(int n, const std::vector<std::vector<int>>& adj, int32_t* color) {
    // seen[i]: colours among i's coloured neighbours (sorted, distinct); the heap holds
    // (saturation, degree, -index) entries, stale ones skipped when popped
    std::vector<std::vector<int>> seen((size_t)n);
    std::vector<std::tuple<int, int, int>> heap;
    heap.reserve((size_t)n * 2);
    for (int i = 0; i < n; ++i) {
        color[i] = -1;
        heap.emplace_back(0, (int)adj[i].size(), -i);
    }
    std::make_heap(heap.begin(), heap.end());
    int ncol = 0;
    while (!heap.empty()) {
        std::pop_heap(heap.begin(), heap.end());
        const auto [sat, deg, negi] = heap.back();
        heap.pop_back();
        const int i = -negi;
        if (color[i] >= 0 || sat != (int)seen[i].size()) continue;
        int c = 0;
        for (int u : seen[i]) {
            if (u != c) break;
            ++c;
        }
        color[i] = c;
        ncol = std::max(ncol, c + 1);
        for (int j : adj[i]) {
            if (color[j] >= 0) continue;
            auto& sj = seen[j];
            auto it = std::lower_bound(sj.begin(), sj.end(), c);
            if (it != sj.end() && *it == c) continue;
            sj.insert(it, c);
            heap.emplace_back((int)sj.size(), (int)adj[j].size(), -j);
            std::push_heap(heap.begin(), heap.end());
        }
    }
    return ncol;
}

int pq_color_graph(int n, int maxnb, const int32_t* nb_idx, const float* nb_j, int32_t* color) {
    if (n <= 0 || maxnb < 0 || !color || (maxnb > 0 && (!nb_idx || !nb_j))) return -PQ_ERR_INVALID_ARG;
    std::vector<std::vector<int>> adj((size_t)n);
    for (int i = 0; i < n; ++i)
        for (int m = 0; m < maxnb; ++m) {
            const int j = nb_idx[(size_t)i * maxnb + m];
            if (nb_j[(size_t)i * maxnb + m] == 0.0f || j == i) continue;
            if (j < 0 || j >= n) return -PQ_ERR_BAD_INDEX;
            adj[i].push_back(j);
            adj[j].push_back(i);
        }
    for (auto& a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    const int ng = greedy_colors(n, adj, color);
    if (ng <= 2) return ng;
    std::vector<int32_t> alt((size_t)n);
    const int nd = dsatur_colors(n, adj, alt.data());
    if (nd < ng) {
        std::copy(alt.begin(), alt.end(), color);
        return nd;
    }
    return ng;
}

}  // extern "C"
