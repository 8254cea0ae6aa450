"""Drop-in for ``piqmc.sa`` (reference piqmc/sa.pyx): classical annealing and the Ising energy.

``Anneal`` keeps the reference's signature and in-place contract;
``mode="reference"`` (default) reproduces the Cython sweep exactly (spin orders
from ``rng``, uniforms from this process's libc ``rand()``), ``mode="fast"``
runs the packed kernel with one slice.  ``Anneal_dense`` and
``Anneal_bipartite`` reproduce their Cython sweeps the same way.
``Anneal_parallel`` and ``Anneal_multispin`` (the reference's OpenMP and
64-configuration bit-packed variants) run the packed kernel.
``ClassicalIsingEnergy`` evaluates the energy on the GPU in FP64.
"""
import numpy as np
import scipy.sparse as sps
import torch

from . import _buffers, _device, _native, fast, reforder

CHUNK_UPDATES = 1 << 24


def _csr(J, n):
    if sps.issparse(J):
        C = sps.csr_matrix(J, dtype=np.float64)
    else:
        C = sps.csr_matrix(np.asarray(J, dtype=np.float64))
    if C.shape[0] != n or C.shape[1] != n:
        raise ValueError("J must be %d x %d, got %r" % (n, n, C.shape))
    C.sum_duplicates()
    return C


def ClassicalIsingEnergy(spins, J):
    """E = -s^T J_off s - sum_i J_ii s_i in FP64 (reference piqmc/sa.pyx:25-44).

    ``spins`` is a +-1 vector of length n, or an (n, m) array whose columns are
    configurations (then an array of m energies is returned).  ``J`` is a scipy
    sparse matrix or a dense array; every stored entry counts once, as in the
    reference's dense ``todense()`` product.  Evaluated by the GPU energy kernel;
    the summation order differs from NumPy's, so results can differ from the
    reference by FP64 rounding (relative ~1e-16 per term).
    """
    s = np.asarray(spins, dtype=np.float64)
    one = s.ndim == 1
    cols = s[:, None] if one else s
    if cols.ndim != 2:
        raise ValueError("spins must be a vector or an (n, m) array")
    n, m = cols.shape
    _buffers.check_pm1(cols, "spins")
    C = _csr(J, n)
    dev = _device.device()
    sp = torch.from_numpy(np.ascontiguousarray(cols.T).astype(np.int8)[:, :, None]).to(dev)   # (m, n, 1)
    words = torch.empty((m, n), dtype=torch.int32, device=dev)
    L = _native.lib()
    _native.check(L.pq_pack_spins(_device.ptr(sp), n, 1, m, None, _device.ptr(words), 32, n, _device.stream_handle()),
                  "pq_pack_spins")
    rp = torch.from_numpy(C.indptr.astype(np.int64)).to(dev)
    ci = torch.from_numpy(C.indices.astype(np.int32)).to(dev)
    cv = torch.from_numpy(C.data.astype(np.float64)).to(dev)
    out = torch.empty((m, 1), dtype=torch.float64, device=dev)
    _native.check(L.pq_energy_packed(_device.ptr(words), 32, n, 1, m, _device.ptr(rp), _device.ptr(ci),
                                     _device.ptr(cv), _device.ptr(out), _device.stream_handle()),
                  "pq_energy_packed")
    e = out[:, 0].cpu().numpy()
    return np.float64(e[0]) if one else e


def Anneal(sched, mcsteps, svec, nbs, rng, *, mode="reference", seed=None):
    """Classical simulated annealing of ``svec`` (+-1) in place through the temperatures ``sched``.

    Reference: piqmc/sa.pyx:50-120.
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    svec = _buffers.float64_buffer(svec, 1, "svec", writable=True)
    nbs = _buffers.float64_buffer(nbs, 3, "nbs")
    nspins = svec.size
    _buffers.check_pm1(svec, "svec")
    if nspins and nbs.shape[0] < nspins:
        raise ValueError("nbs has %d rows, fewer than svec.size=%d" % (nbs.shape[0], nspins))
    if mode == "fast":
        return _anneal_fast(sched, mcsteps, svec, nbs, rng, seed)
    if mode != "reference":
        raise ValueError("mode must be 'reference' or 'fast'")
    idx, jv = reforder.split_neighbors(nbs, nspins)
    bad = ((idx < 0) | (idx >= nspins)) & (idx != np.arange(nspins)[:, None])
    if np.any(bad):
        raise ValueError("neighbour index outside [0, %d)" % nspins)
    cur = _buffers.first_spin_order(rng, nspins)
    nsched = sched.size
    if nsched == 0 or mcsteps <= 0:  # the reference's sweep loop runs no sweep and draws no order
        return None
    spins = torch.from_numpy(svec.astype(np.int8)[None]).to(_device.device())
    gchunk = max(1, CHUNK_UPDATES // max(1, nspins * mcsteps))
    for g0 in range(0, nsched, gchunk):
        g1 = min(nsched, g0 + gchunk)
        count = (g1 - g0) * mcsteps
        perms = np.empty((1, count, nspins), dtype=np.int32)
        for t in range(count):
            perms[0, t] = cur
            cur = rng.permutation(cur)
        rands = reforder.libc_peek(count * nspins)[None]
        spins, used = reforder.anneal(spins, idx, jv, sched[g0:g1], mcsteps, perms, rands)
        reforder.libc_skip(int(used[0]))
    svec[:] = spins[0].cpu().numpy()
    return None


def _anneal_fast(sched, mcsteps, svec, nbs, rng, seed):
    nspins = svec.size
    if mcsteps < 0:
        raise ValueError("mode='fast' needs mcsteps >= 0")
    if nspins == 0:
        return None
    temps = np.asarray(sched, dtype=np.float64).astype(np.float32)
    if np.any(temps <= 0):
        raise ValueError("mode='fast' needs positive temperatures")
    if seed is None:
        seed = _buffers.seed_from_rng(rng)
    prob = fast.Problem(nbs, nrows=nspins)
    words = prob.pack(torch.from_numpy(svec.astype(np.int8)[None, :, None]))
    betas = torch.from_numpy((np.float32(1.0) / temps).astype(np.float32)).to(words.device)
    fast.anneal(prob, words, np.zeros(len(temps)), 1, float(temps[0]) if len(temps) else 1.0, mcsteps=mcsteps,
                seed=seed, jperp=torch.zeros(len(temps), dtype=torch.float32, device=words.device), betas=betas)
    svec[:] = prob.unpack(words, 1)[0, :, 0].cpu().numpy()
    return None


def Anneal_dense(sched, mcsteps, svec, J, rng):
    """Simulated annealing of ``svec`` in place with a dense coupling matrix.

    Reference: piqmc/sa.pyx:126-187 -- pairs are read from the upper triangle of
    ``J`` (either index order), fields from its diagonal; spin orders from
    ``rng.permutation``, uniforms from this process's libc ``rand()``; bit-exact.
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    svec = _buffers.float64_buffer(svec, 1, "svec", writable=True)
    J = _buffers.float64_buffer(J, 2, "J")
    nspins = svec.size
    _buffers.check_pm1(svec, "svec")
    if nspins and (J.shape[0] < nspins or J.shape[1] < nspins):
        raise ValueError("J is %r, smaller than svec.size=%d" % (J.shape, nspins))
    cur = _buffers.first_spin_order(rng, nspins)
    nsched = sched.size
    if nsched == 0 or mcsteps <= 0:  # the reference's sweep loop runs no sweep and draws no order
        return None
    Jc = np.ascontiguousarray(J[:nspins, :nspins])
    spins = torch.from_numpy(svec.astype(np.int8)[None]).to(_device.device())
    gchunk = max(1, CHUNK_UPDATES // max(1, nspins * nspins * mcsteps))
    for g0 in range(0, nsched, gchunk):
        g1 = min(nsched, g0 + gchunk)
        count = (g1 - g0) * mcsteps
        perms = np.empty((1, count, nspins), dtype=np.int32)
        for t in range(count):
            perms[0, t] = cur
            cur = rng.permutation(cur)
        rands = reforder.libc_peek(count * nspins)[None]
        spins, used = reforder.anneal_dense(spins, Jc, sched[g0:g1], mcsteps, perms, rands)
        reforder.libc_skip(int(used[0]))
    svec[:] = spins[0].cpu().numpy()
    return None


def Anneal_bipartite(sched, mcsteps, lvec, rvec, J, lbias, rbias, rng):
    """Simulated annealing of a bipartite graph: ``lvec`` and ``rvec`` in place.

    Reference: piqmc/sa.pyx:411-500 -- left spins in index order, then right
    spins, each step; ``J`` has shape (lvec.size, rvec.size); every term of a
    spin's energy difference carries both biases exactly as the reference sums
    them.  ``rng`` is accepted and unused, as in the reference; uniforms come
    from this process's libc ``rand()``; bit-exact.
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    lvec = _buffers.float64_buffer(lvec, 1, "lvec", writable=True)
    rvec = _buffers.float64_buffer(rvec, 1, "rvec", writable=True)
    J = _buffers.float64_buffer(J, 2, "J")
    lbias = _buffers.float64_buffer(lbias, 1, "lbias")
    rbias = _buffers.float64_buffer(rbias, 1, "rbias")
    nl, nr = lvec.size, rvec.size
    _buffers.check_pm1(lvec, "lvec")
    _buffers.check_pm1(rvec, "rvec")
    if nl and nr and (J.shape[0] < nl or J.shape[1] < nr or lbias.size < nl or rbias.size < nr):
        raise ValueError("J must be at least (%d, %d) and the biases as long as the spin vectors" % (nl, nr))
    nsched = sched.size
    if nsched == 0 or mcsteps <= 0 or nl + nr == 0:
        return None
    spins = torch.from_numpy(np.concatenate([lvec, rvec]).astype(np.int8)[None]).to(_device.device())
    Jc = np.ascontiguousarray(J[:nl, :nr]) if nl and nr else np.zeros((max(nl, 1), max(nr, 1)))
    lb = np.ascontiguousarray(lbias[:nl]) if nl else np.zeros(1)
    rb = np.ascontiguousarray(rbias[:nr]) if nr else np.zeros(1)
    gchunk = max(1, CHUNK_UPDATES // max(1, (nl + nr) * max(nl, nr, 1) * mcsteps))
    for g0 in range(0, nsched, gchunk):
        g1 = min(nsched, g0 + gchunk)
        rands = reforder.libc_peek((g1 - g0) * mcsteps * (nl + nr))[None]
        spins, used = reforder.anneal_bipartite(spins, nl, Jc, lb, rb, sched[g0:g1], mcsteps, rands)
        reforder.libc_skip(int(used[0]))
    out = spins[0].cpu().numpy()
    lvec[:] = out[:nl]
    rvec[:] = out[nl:]
    return None


def Anneal_parallel(sched, mcsteps, svec, nbs, nthreads, *, seed=0):
    """The reference's OpenMP variant (piqmc/sa.pyx:193-266) on the GPU: the packed kernel with one slice.

    The reference threads race on shared spins, so its results are not
    reproducible; this runs ``Anneal(..., mode="fast")`` with Philox key ``seed``.
    ``nthreads`` is accepted for compatibility and unused.
    """
    _buffers.as_c_int(nthreads, "nthreads")
    return Anneal(sched, mcsteps, svec, nbs, None, mode="fast", seed=seed)


def Anneal_multispin(sched, mcsteps, svec_mat, nbs, rng, *, seed=None):
    """Anneal every row of ``svec_mat`` (configurations x spins) in place (reference piqmc/sa.pyx:282-400).

    The reference packs 64 rows into bits and shares one set of 64 uniforms for
    the whole run; here every row is an independent replica of the packed
    kernel with one slice (any number of rows), Philox key from ``rng`` unless
    ``seed`` is given.
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    mat = _buffers.float64_buffer(svec_mat, 2, "svec_mat", writable=True)
    nbs = _buffers.float64_buffer(nbs, 3, "nbs")
    R, nspins = mat.shape
    if mcsteps < 0:
        raise ValueError("mcsteps must be non-negative")
    _buffers.check_pm1(mat, "svec_mat")
    if R == 0 or nspins == 0:
        return None
    temps = np.asarray(sched, dtype=np.float64).astype(np.float32)
    if np.any(temps <= 0):
        raise ValueError("temperatures must be positive")
    if seed is None:
        seed = _buffers.seed_from_rng(rng)
    prob = fast.Problem(nbs, nrows=nspins)
    words = prob.pack(torch.from_numpy(mat.astype(np.int8)[:, :, None]))
    betas = torch.from_numpy((np.float32(1.0) / temps).astype(np.float32)).to(words.device)
    if len(temps):
        fast.anneal(prob, words, np.zeros(len(temps)), 1, float(temps[0]), mcsteps=mcsteps, seed=seed,
                    jperp=torch.zeros(len(temps), dtype=torch.float32, device=words.device), betas=betas)
    mat[:] = prob.unpack(words, 1)[:, :, 0].cpu().numpy()
    return None
