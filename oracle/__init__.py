"""piqmc CPU oracle -- TEST INFRASTRUCTURE ONLY.

A plain-C restatement (``piqmc_oracle.c``) of the reference's sweeps, wrapped
with ctypes, plus helpers that rebuild the exact random streams the reference
consumes.  The product never imports this package: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` do, to
check or time beside the CUDA path.

Reference semantics restated here (file:line within hadsed/pathintegral-qmc):

* ``qa_sparse``  -- ``qmc.QuantumAnneal``        piqmc/qmc.pyx:30-136
* ``qa_dense``   -- ``qmc.QuantumAnneal_dense``  piqmc/qmc.pyx:141-242
* ``sa_sparse``  -- ``sa.Anneal``                piqmc/sa.pyx:50-120
* ``sa_dense``   -- ``sa.Anneal_dense``          piqmc/sa.pyx:126-187
* ``sa_bipartite`` -- ``sa.Anneal_bipartite``    piqmc/sa.pyx:411-500
* ``jperp``      -- J-perp formula               piqmc/qmc.pyx:95, piqmc/qmc.c:2063-2075
* ``classical_energy`` -- ``sa.ClassicalIsingEnergy`` piqmc/sa.pyx:25-44
* ``generate_neighbors`` -- ``tools.GenerateNeighbors`` piqmc/tools.pyx:28-96
* ``reference_perms`` -- the ``rng.permutation`` calls of piqmc/qmc.pyx:90-91,136

Pinned to the reference itself: the golden vectors in tests/golden/ were recorded from
its compiled Cython code, and where that code is built here (oracle/build_ref.py)
tests/test_oracle_vs_reference.py compares the two on random cases.

``fast_oracle.c`` (``fast_anneal``, ``dense_sweep``, ``pair_class``, ``pair_features``,
``philox4x32_10``, ``expf_neg``)
restates this library's own packed algorithms, which have no reference counterpart:
it is the bit-exact check of those kernels, pinned by Philox's published known-answer
vectors and, statistically, by the reference (tests/test_statistics.py).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpiqmc_oracle.so")
SOURCES = ("piqmc_oracle.c", "fast_oracle.c")

FIX_Q2 = 1
FIX_Q1 = 2


def build(force=False):
    """Compile the oracle's C with strict IEEE semantics (no contraction)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
                           "-fPIC", "-shared"] + srcs + ["-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i32, i64, f32 = ctypes.c_int, ctypes.c_int64, ctypes.c_float
        L.orc_qa_sparse.argtypes = [i32, i32, i32, i32, P, P, P, i32, i32, f32, P, P, i64, P, i32]
        L.orc_qa_sparse.restype = i64
        L.orc_qa_dense.argtypes = [i32, i32, P, P, i32, i32, f32, P, P, i64, P, i32]
        L.orc_qa_dense.restype = i64
        L.orc_sa_sparse.argtypes = [i32, i32, P, P, P, i32, i32, P, P, i64, P]
        L.orc_sa_sparse.restype = i64
        L.orc_sa_dense.argtypes = [i32, P, P, i32, i32, P, P, i64, P]
        L.orc_sa_dense.restype = i64
        L.orc_sa_bipartite.argtypes = [i32, i32, P, P, P, P, i32, i32, P, i64, P, P]
        L.orc_sa_bipartite.restype = i64
        L.orc_jperp.argtypes = [P, i32, i32, f32, P]
        L.orc_jperp.restype = None
        L.orc_libc_rand.argtypes = [P, i64]
        L.orc_libc_rand.restype = None
        L.orc_libc_srand.argtypes = [ctypes.c_uint]
        L.orc_libc_srand.restype = None
        _setup_fast(L)
        _lib = L
    return _lib


def _setup_fast(L):
    if not hasattr(L, "orc_fast_anneal"):
        return
    P = ctypes.c_void_p
    i32, i64, f32, u64 = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_uint64
    L.orc_philox4x32_10.argtypes = [P, P, P]
    L.orc_philox4x32_10.restype = None
    L.orc_expf.argtypes = [f32]
    L.orc_expf.restype = f32
    L.orc_u01.argtypes = [ctypes.c_uint32]
    L.orc_u01.restype = f32
    L.orc_expf_max.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    L.orc_expf_max.restype = f32
    L.orc_fast_anneal.argtypes = [i32, i32, i32, P, P, P, i32, i32, P, i32, P, i32, i32, f32, u64,
                                  i64, i32, i32, P, P]
    L.orc_fast_anneal.restype = i64
    if hasattr(L, "orc_pair_class"):
        L.orc_pair_features.argtypes = [P, i32, i32, i32, P, P, P, i32, i32, f32, f32, f32, i32, P]
        L.orc_pair_features.restype = f32
        L.orc_pair_class.argtypes = [P, i32, i32, i32, P, P, P, P, P, P, i32, i32, i32, f32, f32, P, P,
                                     ctypes.c_uint32, u64, ctypes.c_uint32]
        L.orc_pair_class.restype = i64
        L.orc_pair_sigmoid.argtypes = [f32]
        L.orc_pair_sigmoid.restype = f32
    if hasattr(L, "orc_dense_sweep"):
        L.orc_dense_sweep.argtypes = [i32, i32, P, P, P, i32, P, i32, i32, f32, u64, i64, i32, P, i32]
        L.orc_dense_sweep.restype = i64


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


# ----------------------------------------------------------------------------------------
# streams the reference consumes
# ----------------------------------------------------------------------------------------

def libc_srand(seed):
    lib().orc_libc_srand(int(seed) & 0xFFFFFFFF)


def libc_rand(count):
    """The next ``count`` values of this process's libc ``rand()``."""
    out = np.empty(int(count), dtype=np.int32)
    if count:
        lib().orc_libc_rand(_p(out), int(count))
    return out


def libc_stream(seed, count):
    libc_srand(seed)
    return libc_rand(count)


def reference_perms(rng, n, nsweeps):
    """Spin orders of ``nsweeps`` sweeps, drawn exactly as the reference draws them.

    The reference draws ``rng.permutation(range(n))`` once (piqmc/qmc.pyx:90-91) and
    then ``rng.permutation(previous)`` after every sweep (piqmc/qmc.pyx:136), so
    ``nsweeps + 1`` calls in total; the last result is never used for a sweep.
    """
    out = np.empty((nsweeps, n), dtype=np.int64)
    cur = rng.permutation(range(n))
    for t in range(nsweeps):
        out[t] = cur
        cur = rng.permutation(cur)
    return out


# ----------------------------------------------------------------------------------------
# reference sweeps
# ----------------------------------------------------------------------------------------

def split_neighbors(nbs):
    """(n, maxnb, 2) float64 -> (int32 index, float32 coupling), as the reference reads them."""
    nbs = np.asarray(nbs, dtype=np.float64)
    idx = np.ascontiguousarray(np.trunc(nbs[:, :, 0]).astype(np.int32))
    jv = np.ascontiguousarray(nbs[:, :, 1].astype(np.float32))
    return idx, jv


def jperp(sched, P, temp):
    sched = np.ascontiguousarray(sched, dtype=np.float64)
    out = np.empty(len(sched), dtype=np.float32)
    lib().orc_jperp(_p(sched), len(sched), int(P), float(np.float32(temp)), _p(out))
    return out


def qa_sparse(spins, nbs, sched, mcsteps, temp, perms, rands, flags=0):
    """Run the QuantumAnneal restatement on int8 spins (n, P), in place.

    ``perms`` is (sweeps, nperm): each sweep updates the nperm <= n spins it lists (the
    reference's ``nspins``); rows past them stay fixed.  Returns the number of ``rands``
    consumed (-1 when the stream ran out).
    """
    n, P = spins.shape
    assert spins.dtype == np.int8 and spins.flags.c_contiguous
    idx, jv = split_neighbors(nbs)
    jp = jperp(sched, P, temp)
    perms = np.ascontiguousarray(perms, dtype=np.int64)
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    assert perms.ndim == 2 and perms.shape[0] == len(sched) * mcsteps and perms.shape[1] <= n
    return lib().orc_qa_sparse(n, perms.shape[1], P, idx.shape[1], _p(idx), _p(jv), _p(jp), len(sched), mcsteps,
                               float(np.float32(temp)), _p(perms), _p(rands), len(rands),
                               _p(spins), flags)


def qa_dense(spins, J, sched, mcsteps, temp, perms, rands, flags=0):
    n, P = spins.shape
    assert spins.dtype == np.int8 and spins.flags.c_contiguous
    J = np.ascontiguousarray(J, dtype=np.float64)
    jp = jperp(sched, P, temp)
    perms = np.ascontiguousarray(perms, dtype=np.int64)
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    return lib().orc_qa_dense(n, P, _p(J), _p(jp), len(sched), mcsteps, float(np.float32(temp)),
                              _p(perms), _p(rands), len(rands), _p(spins), flags)


def sa_sparse(spins, nbs, sched, mcsteps, perms, rands):
    n = spins.shape[0]
    assert spins.dtype == np.int8 and spins.flags.c_contiguous
    idx, jv = split_neighbors(nbs)
    temps = np.ascontiguousarray(np.asarray(sched, dtype=np.float64).astype(np.float32))
    perms = np.ascontiguousarray(perms, dtype=np.int64)
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    return lib().orc_sa_sparse(n, idx.shape[1], _p(idx), _p(jv), _p(temps), len(temps), mcsteps,
                               _p(perms), _p(rands), len(rands), _p(spins))


def sa_dense(spins, J, sched, mcsteps, perms, rands):
    """sa.Anneal_dense of one int8 spin vector in place; returns the rand() count consumed."""
    n = spins.shape[0]
    assert spins.dtype == np.int8 and spins.flags.c_contiguous
    J = np.ascontiguousarray(J, dtype=np.float64)
    temps = np.ascontiguousarray(np.asarray(sched, dtype=np.float64).astype(np.float32))
    perms = np.ascontiguousarray(perms, dtype=np.int64)
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    return lib().orc_sa_dense(n, _p(J), _p(temps), len(temps), mcsteps, _p(perms), _p(rands), len(rands), _p(spins))


def sa_bipartite(lv, rv, J, lbias, rbias, sched, mcsteps, rands):
    """sa.Anneal_bipartite of int8 left / right spin vectors in place; returns the rand() count consumed."""
    assert lv.dtype == np.int8 and rv.dtype == np.int8
    J = np.ascontiguousarray(J, dtype=np.float64)
    lb = np.ascontiguousarray(lbias, dtype=np.float64)
    rb = np.ascontiguousarray(rbias, dtype=np.float64)
    temps = np.ascontiguousarray(np.asarray(sched, dtype=np.float64).astype(np.float32))
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    return lib().orc_sa_bipartite(lv.shape[0], rv.shape[0], _p(J), _p(lb), _p(rb), _p(temps), len(temps), mcsteps,
                                  _p(rands), len(rands), _p(lv), _p(rv))


# ----------------------------------------------------------------------------------------
# packed fast sweep (restated from its specification; see fast_oracle.c)
# ----------------------------------------------------------------------------------------

def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def expf_neg(x):
    return np.float32(lib().orc_expf(float(np.float32(x))))


def u01(r):
    """The packed sweeps' uniform of a 32-bit Philox word: ((r >> 9) + 1/2) * 2^-23."""
    return np.float32(lib().orc_u01(int(r) & 0xFFFFFFFF))


def expf_neg_max(x_hi, x_lo):
    """Largest expf_neg(x) over every FP32 x in [x_lo, x_hi] (both negative)."""
    hi = int(np.float32(x_hi).view(np.uint32))
    lo = int(np.float32(x_lo).view(np.uint32))
    return np.float32(lib().orc_expf_max(hi, lo))


def fast_anneal(nbr, cpl, field, class_size, class_stride, words, P, jperp, mcsteps, beta, seed,
                sweep_base=0, replica=0, global_moves=0, betas=None, order_mode=1):
    """Run one replica (uint64 world-lines ``words``, device order) in place; returns accepted flips.

    nbr/cpl: (maxdeg, n) SoA tables, field (n,), class_size (M,), all in device order.
    """
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    cpl = np.ascontiguousarray(cpl, dtype=np.float32)
    field = np.ascontiguousarray(field, dtype=np.float32)
    csz = np.ascontiguousarray(class_size, dtype=np.int32)
    jp = np.ascontiguousarray(jperp, dtype=np.float32)
    assert words.dtype == np.uint64 and words.flags.c_contiguous
    maxdeg, n = nbr.shape
    bt = None if betas is None else np.ascontiguousarray(betas, dtype=np.float32)
    return lib().orc_fast_anneal(n, int(P), maxdeg, _p(nbr), _p(cpl), _p(field), len(csz), int(class_stride),
                                 _p(csz), int(order_mode), _p(jp), len(jp), int(mcsteps), float(np.float32(beta)),
                                 int(seed) & (2**64 - 1), int(sweep_base), int(replica), int(global_moves),
                                 _p(words), None if bt is None else _p(bt))


def dense_sweep(F, K, units, words, P, jperp, mcsteps, beta, seed, sweep_base=0, replica=0, per_slice_order=False):
    """Run the dense packed sweep of one replica in place on FP32 fields F (P, N) and uint32 words (N,)."""
    F = np.ascontiguousarray(F, dtype=np.float32)
    K = np.ascontiguousarray(K, dtype=np.float32)
    units = np.ascontiguousarray(units, dtype=np.int32)
    jp = np.ascontiguousarray(jperp, dtype=np.float32)
    assert words.dtype == np.uint32 and words.flags.c_contiguous
    N = K.shape[0]
    n = lib().orc_dense_sweep(N, int(P), _p(F), _p(K), _p(units), len(units), _p(jp), len(jp), int(mcsteps),
                              float(np.float32(beta)), int(seed) & (2**64 - 1), int(sweep_base), int(replica),
                              _p(words), int(bool(per_slice_order)))
    return n, F


# ----------------------------------------------------------------------------------------
# energy and neighbour table
# ----------------------------------------------------------------------------------------

def classical_energy(spins, J):
    """E = -s^T J_off s - sum(diag(J) s) in FP64 (reference piqmc/sa.pyx:41-44)."""
    Jd = np.asarray(J.todense() if hasattr(J, "todense") else J, dtype=np.float64).copy()
    d = np.diag(Jd).copy()
    np.fill_diagonal(Jd, 0.0)
    s = np.asarray(spins, dtype=np.float64)
    return -s @ (Jd @ s) - np.sum(d * s)


def generate_neighbors(nspins, J, maxnb):
    """Neighbour table in DOK key order (reference piqmc/tools.pyx:77-92), O(n*nnz) as there."""
    J = J.todok()
    nbs = np.zeros((nspins, maxnb, 2))
    for ispin in range(nspins):
        ipair = 0
        for pair in J.keys():
            if pair[0] == ispin:
                nbs[ispin, ipair] = (pair[1], J[pair])
                ipair += 1
            elif pair[1] == ispin:
                nbs[ispin, ipair] = (pair[0], J[pair])
                ipair += 1
    return nbs


# ----------------------------------------------------------------------------------------
# pair world-line moves (this library's own move; restated in fast_oracle.c)
# ----------------------------------------------------------------------------------------

def _tables(nbr, cpl, field):
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    cpl = np.ascontiguousarray(cpl, dtype=np.float32)
    field = np.ascontiguousarray(field, dtype=np.float32)
    maxdeg = nbr.shape[0] if nbr.ndim == 2 else 0
    return nbr, cpl, field, maxdeg


def pair_features(words, nbr, cpl, field, P, si, sj, Jb, beta, jp, flipped=False):
    """(features[8] FP32, cost dE) of the pair (si, sj) of one replica (words uint64 per slot)."""
    nbr, cpl, field, maxdeg = _tables(nbr, cpl, field)
    w = np.ascontiguousarray(words, dtype=np.uint64)
    x = np.zeros(8, np.float32)
    dE = lib().orc_pair_features(_p(w), len(w), int(P), maxdeg, _p(nbr), _p(cpl), _p(field), int(si), int(sj),
                                 float(np.float32(Jb)), float(np.float32(beta)), float(np.float32(jp)),
                                 int(bool(flipped)), _p(x))
    return x, np.float32(dE)


def pair_class(words, nbr, cpl, field, P, bond_i, bond_j, bond_J, first, count, cls, beta, seed, move, replica,
               qmin=0.05, logit=None, logit_f=None):
    """The pair moves of bonds [first, first + count) of one replica, in place on ``words`` (uint64 per slot).

    Uniform (every bond tried) when ``logit`` is None, else the learned move with the
    network's logits of the current (``logit``) and flipped (``logit_f``) pairs."""
    nbr, cpl, field, maxdeg = _tables(nbr, cpl, field)
    bi = np.ascontiguousarray(bond_i, dtype=np.int32)
    bj = np.ascontiguousarray(bond_j, dtype=np.int32)
    bJ = np.ascontiguousarray(bond_J, dtype=np.float32)
    lg = None if logit is None else np.ascontiguousarray(logit, dtype=np.float32)
    lf = None if logit_f is None else np.ascontiguousarray(logit_f, dtype=np.float32)
    return int(lib().orc_pair_class(_p(words), len(words), int(P), maxdeg, _p(nbr), _p(cpl), _p(field), _p(bi),
                                    _p(bj), _p(bJ), int(first), int(count), int(cls), float(np.float32(beta)),
                                    float(np.float32(qmin)), None if lg is None else _p(lg),
                                    None if lf is None else _p(lf), int(move) & 0xFFFFFFFF,
                                    int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica) & 0xFFFFFFFF))


def pair_sigmoid(z):
    return np.float32(lib().orc_pair_sigmoid(float(np.float32(z))))
