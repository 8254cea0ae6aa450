// Instance generators on the GPU: the neighbour table (the layout of
// tools.GenerateNeighbors, reference piqmc/tools.pyx:28-96) of the reference's
// lattice instances, written directly in device memory.
//
// The bond set of an instance and the order of its keys are the reference's:
//  * kind 0, Generate2DIsingInstance (piqmc/tools.pyx:98-131): per spin `row` of an
//    nrows x nrows torus, in this order: the vertical wrap (row, row + nrows (nrows - 1))
//    for the first lattice row, the horizontal wrap (row, row + nrows - 1) for the first
//    column, the right bond unless the last column, the down bond unless the last row;
//  * kind 1, Generate2DLattice (piqmc/tools.pyx:133-175): the same four on an
//    nrows x ncols lattice, the two wraps only when periodic;
//  * kind 2, GenerateKblockLattice (piqmc/tools.pyx:177-273): for radius q = 1..k the
//    ring of radius q around the spin, clipped to the lattice, top side, bottom side,
//    left side, right side, keeping the entries above the diagonal.
// A key assigned twice keeps its first position (a dictionary of keys).  The table
// row of spin j lists, in the order of the keys, the other end of every key that
// involves j -- what GenerateNeighbors builds from the reference's DOK matrix.  Keys
// (a, b) always have a <= b here, and the keys that reach spin j come from spins a
// in a small window around j (the bonds are local, the wraps reach a fixed offset),
// so each thread rebuilds the key blocks of those spins and sorts what it finds.
//
// Values: the reference draws them from the caller's MT19937 stream in key order;
// here coupling (a, b) = lo + (hi - lo) u, u = the 53-bit uniform
// ((w0 >> 5) 2^26 + (w1 >> 6)) 2^-53 of Philox4x32-10(ctr = {a, b, 0, 6 << 24}, key =
// seed) words 0 and 1 -- a counter-based stream, so the value of a bond is the same
// from either end and independent of the order of computation.
#include "common.cuh"

namespace {

constexpr int kMaxBlock = 64;   // keys of one spin's block (kind 2 with k <= 3 needs at most 24)

struct GenArgs {
    int kind, nrows, ncols, periodic, k, n, maxnb;
    double lo, hi;
    uint32_t key0, key1;
};

// Spin a's key block (the other ends b, in insertion order, duplicates removed).
__device__ int own_keys(const GenArgs& g, int a, int* out) {
    int cnt = 0;
    auto add = [&](int b) {
        for (int t = 0; t < cnt; ++t)
            if (out[t] == b) return;
        if (cnt < kMaxBlock) out[cnt++] = b;
    };
    const int nr = g.nrows, nc = g.ncols, n = g.n;
    if (g.kind == 0 || g.kind == 1) {
        const bool wraps = g.kind == 0 || g.periodic;
        if (wraps && a < nc) add(a + nc * (nr - 1));
        if (wraps && a % nc == 0) add(a + nc - 1);
        if (a % nc != nc - 1 && a + 1 < n) add(a + 1);
        if (a + nc < n) add(a + nc);
    } else {
        const int c = a % nc;
        const int to_right = (a + 1) % nc ? nc - (a + 1) % nc : 0;
        for (int q = 1; q <= g.k; ++q) {
            const int left = c < q ? c : q;
            const int right = to_right < q ? to_right : q;
            int up = q;
            while (a - up * nc < 0) --up;
            int down = q;
            while (a + down * nc >= n) --down;
            int tlc = a - up * nc - left;
            if (tlc < 0) tlc = 0;
            const int w = left + right + 1, h = up + down;
            for (int r = 0; r < w; ++r) if (tlc + r > a) add(tlc + r);
            for (int r = 0; r < w; ++r) if (tlc + h * nc + r > a) add(tlc + h * nc + r);
            for (int r = 1; r <= h; ++r) if (tlc + r * nc > a) add(tlc + r * nc);
            for (int r = 1; r <= h; ++r) if (tlc + w - 1 + r * nc > a) add(tlc + w - 1 + r * nc);
        }
    }
    return cnt;
}

__device__ double coupling(const GenArgs& g, int a, int b) {
    const pq_u32x4 w = pq_philox(pq_u32x4{(uint32_t)a, (uint32_t)b, 0u, 6u << 24}, g.key0, g.key1);
    const double u = ((double)(w.x >> 5) * 67108864.0 + (double)(w.y >> 6)) * (1.0 / 9007199254740992.0);
    return g.lo + (g.hi - g.lo) * u;
}

// The spins whose key blocks can hold a key (a, j), a <= j.
__device__ int sources(const GenArgs& g, int j, int* src) {
    int cnt = 0;
    auto add = [&](int a) {
        if (a < 0 || a > j) return;
        for (int t = 0; t < cnt; ++t)
            if (src[t] == a) return;
        src[cnt++] = a;
    };
    const int nr = g.nrows, nc = g.ncols;
    if (g.kind == 0 || g.kind == 1) {
        add(j);
        add(j - 1);
        add(j - nc);
        add(j - nc + 1);
        add(j - nc * (nr - 1));
    } else {
        const int rj = j / nc, cj = j % nc;
        for (int dr = -g.k; dr <= 0; ++dr)
            for (int dc = -g.k; dc <= g.k; ++dc) {
                const int r = rj + dr, c = cj + dc;
                if (r >= 0 && c >= 0 && c < nc) add(r * nc + c);
            }
    }
    return cnt;
}

__global__ void neighbor_table_kernel(GenArgs g, double* __restrict__ nbs, int32_t* __restrict__ row_len,
                                      int32_t* __restrict__ status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.n) return;
    int src[64];
    const int ns = sources(g, j, src);
    // (source, position) keys of the entries of row j, and their other ends
    long long order[2 * kMaxBlock];
    int other[2 * kMaxBlock];
    int m = 0;
    int blk[kMaxBlock];
    for (int s = 0; s < ns; ++s) {
        const int a = src[s];
        const int cnt = own_keys(g, a, blk);
        for (int t = 0; t < cnt; ++t) {
            const int b = blk[t];
            if (a == j || b == j) {
                if (m >= 2 * kMaxBlock) { pq_set_status(status, PQ_ERR_TOO_LARGE); return; }
                order[m] = (long long)a * kMaxBlock + t;
                other[m] = a == j ? b : a;
                ++m;
            }
        }
    }
    // insertion order of the keys
    for (int x = 1; x < m; ++x) {
        const long long ko = order[x];
        const int oo = other[x];
        int y = x - 1;
        while (y >= 0 && order[y] > ko) {
            order[y + 1] = order[y];
            other[y + 1] = other[y];
            --y;
        }
        order[y + 1] = ko;
        other[y + 1] = oo;
    }
    row_len[j] = m;
    if (m > g.maxnb) { pq_set_status(status, PQ_ERR_TOO_LARGE); return; }
    double* row = nbs + (int64_t)j * g.maxnb * 2;
    for (int t = 0; t < g.maxnb; ++t) {
        if (t < m) {
            const int o = other[t];
            const int a = o < j ? o : j, b = o < j ? j : o;
            row[2 * t] = (double)o;
            row[2 * t + 1] = coupling(g, a, b);
        } else {
            row[2 * t] = 0.0;
            row[2 * t + 1] = 0.0;
        }
    }
}

}  // namespace

extern "C" {

int pq_generate_lattice_table(int kind, int nrows, int ncols, int periodic, int k, double lo, double hi,
                              uint64_t seed, int maxnb, double* nbs, int32_t* row_len, int32_t* status,
                              void* stream) {
    if (!nbs || !row_len || kind < 0 || kind > 2 || nrows < 1 || ncols < 1 || maxnb < 0 ||
        (kind == 0 && nrows != ncols) || (kind == 2 && (k < 1 || k > 3)))
        return PQ_ERR_INVALID_ARG;
    if ((int64_t)nrows * ncols > (1 << 26)) return PQ_ERR_TOO_LARGE;
    GenArgs g;
    g.kind = kind; g.nrows = nrows; g.ncols = ncols; g.periodic = periodic ? 1 : 0; g.k = kind == 2 ? k : 1;
    g.n = nrows * ncols; g.maxnb = maxnb; g.lo = lo; g.hi = hi;
    g.key0 = (uint32_t)seed; g.key1 = (uint32_t)(seed >> 32);
    neighbor_table_kernel<<<(g.n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g, nbs, row_len, status);
    return pq_launch_status();
}

}  // extern "C"
