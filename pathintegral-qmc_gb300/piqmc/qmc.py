"""Drop-in for ``piqmc.qmc`` (reference piqmc/qmc.pyx): path-integral quantum annealing.

``QuantumAnneal`` and ``QuantumAnneal_dense`` keep the reference's signatures
and in-place contract.  ``mode="reference"`` (default) runs the
reference-order CUDA kernel: the same spin orders drawn from ``rng`` in the same
order, the same libc ``rand()`` uniforms taken from this process (libc left
advanced by exactly the number consumed), the same FP32/FP64 arithmetic -- so
``confs``, ``rng`` and libc end in the states the Cython code leaves.
``mode="fast"`` runs the packed kernel (both reference quirks corrected; see
``piqmc.fast``), seeded from ``rng``.
"""
import numpy as np
import torch

from . import _buffers, _device, fast, reforder

# uniforms drawn ahead per reference-order chunk (upper bound: one per update)
CHUNK_UPDATES = 1 << 24


def _reference_perms(rng, cur, count, nspins):
    out = np.empty((1, count, nspins), dtype=np.int32)
    for t in range(count):
        out[0, t] = cur
        cur = rng.permutation(cur)
    return out, cur


def QuantumAnneal(sched, mcsteps, slices, temp, nspins, confs, nbs, rng, *, mode="reference", seed=None,
                  global_moves=0):
    """Path-integral quantum annealing of ``confs`` (nspins x slices, +-1) in place.

    Reference: piqmc/qmc.pyx:30-136.  ``sched`` holds the transverse-field
    values, ``mcsteps`` the sweeps per value, ``temp`` the temperature, ``nbs`` the
    neighbour table of ``tools.GenerateNeighbors``, ``rng`` a numpy RandomState.
    Returns None.
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    slices = _buffers.as_c_int(slices, "slices")
    temp = _buffers.as_c_float(temp, "temp")
    nspins = _buffers.as_c_int(nspins, "nspins")
    confs = _buffers.float64_buffer(confs, 2, "confs", writable=True)
    nbs = _buffers.float64_buffer(nbs, 3, "nbs")
    if mode == "reference":
        return _qa_reference(sched, mcsteps, slices, temp, nspins, confs, nbs, rng)
    if mode == "fast":
        return _qa_fast(sched, mcsteps, slices, temp, nspins, confs, nbs, rng, seed, global_moves)
    raise ValueError("mode must be 'reference' or 'fast'")


def _validate(sched, mcsteps, slices, nspins, confs):
    n_rows, ncols = confs.shape
    if nspins < 0:
        raise ValueError("nspins must be non-negative")
    if slices < 2:
        raise ValueError("slices must be >= 2 (the reference reads slices P-1 and 1)")
    if nspins > n_rows or slices > ncols:
        raise ValueError("confs must be at least (nspins, slices) = (%d, %d), got %r"
                         % (nspins, slices, confs.shape))
    _buffers.check_pm1(confs[:, :slices], "confs")


def _qa_reference(sched, mcsteps, slices, temp, nspins, confs, nbs, rng):
    _validate(sched, mcsteps, slices, nspins, confs)
    n_rows = confs.shape[0]
    if nspins and nbs.shape[0] < nspins:
        raise ValueError("nbs has %d rows, fewer than nspins=%d" % (nbs.shape[0], nspins))
    idx, jv = reforder.split_neighbors(nbs, n_rows)
    live = idx[:nspins]
    bad = ((live < 0) | (live >= n_rows)) & (live != np.arange(nspins)[:, None])
    if np.any(bad):
        raise ValueError("neighbour index outside [0, %d)" % n_rows)
    cur = _buffers.first_spin_order(rng, nspins)
    nsched = sched.size
    if nsched == 0:
        return None
    if np.float32(slices) * temp == 0:
        raise ZeroDivisionError("float division")
    if mcsteps <= 0:  # the reference's sweep loop runs no sweep and draws no order
        return None
    jp = reforder.jperp_schedule(sched, slices, temp)
    spins = torch.from_numpy(np.ascontiguousarray(confs[:, :slices]).astype(np.int8)[None]).to(_device.device())
    upd_per_g = max(1, nspins * slices * mcsteps)
    gchunk = max(1, CHUNK_UPDATES // upd_per_g)
    for g0 in range(0, nsched, gchunk):
        g1 = min(nsched, g0 + gchunk)
        perms, cur = _reference_perms(rng, cur, (g1 - g0) * mcsteps, nspins)
        rands = reforder.libc_peek((g1 - g0) * nspins * slices * mcsteps)[None]
        spins, used = reforder.quantum_anneal(spins, idx, jv, sched[g0:g1], mcsteps, temp, perms, rands,
                                              nperm=nspins, jperp=jp[g0:g1])
        reforder.libc_skip(int(used[0]))
    confs[:, :slices] = spins[0].cpu().numpy()
    return None


def _qa_fast(sched, mcsteps, slices, temp, nspins, confs, nbs, rng, seed, global_moves):
    n_rows, ncols = confs.shape
    if nspins != n_rows:
        raise ValueError("mode='fast' updates every row: nspins must equal confs.shape[0]")
    if slices < 1 or slices > ncols or slices > 64:
        raise ValueError("mode='fast' needs 1 <= slices <= min(64, confs.shape[1])")
    if mcsteps < 0 or temp <= 0:
        raise ValueError("mode='fast' needs mcsteps >= 0 and temp > 0")
    _buffers.check_pm1(confs[:, :slices], "confs")
    if seed is None:
        seed = _buffers.seed_from_rng(rng)
    prob = fast.Problem(nbs, nrows=n_rows)
    words = prob.pack(torch.from_numpy(np.ascontiguousarray(confs[:, :slices]).astype(np.int8)[None]))
    fast.anneal(prob, words, sched, slices, temp, mcsteps=mcsteps, seed=seed, global_moves=global_moves)
    confs[:, :slices] = prob.unpack(words, slices)[0].cpu().numpy()
    return None


def QuantumAnneal_dense(sched, mcsteps, slices, temp, nspins, confs, J, rng, *, mode="reference", seed=None,
                        recompute_every=50):
    """Dense-J path-integral quantum annealing of ``confs`` in place.

    Reference: piqmc/qmc.pyx:141-242.  ``J`` is a dense float64 matrix whose upper
    triangle holds the couplings and whose diagonal holds the fields.
    ``mode="fast"`` runs the dense fast path (``piqmc.dense``: local fields kept
    in shared memory with rank-1 updates, recomputed every ``recompute_every``
    field steps by the split-BF16 tensor-core GEMM; both reference quirks
    corrected; slices <= 32; Philox key ``seed`` or drawn from ``rng``).
    """
    sched = _buffers.float64_buffer(sched, 1, "sched")
    mcsteps = _buffers.as_c_int(mcsteps, "mcsteps")
    slices = _buffers.as_c_int(slices, "slices")
    temp = _buffers.as_c_float(temp, "temp")
    nspins = _buffers.as_c_int(nspins, "nspins")
    confs = _buffers.float64_buffer(confs, 2, "confs", writable=True)
    J = _buffers.float64_buffer(J, 2, "J")
    if mode not in ("reference", "fast"):
        raise ValueError("mode must be 'reference' or 'fast'")
    _validate(sched, mcsteps, slices, nspins, confs)
    if J.shape[0] < nspins or J.shape[1] < nspins:
        raise ValueError("J must be at least nspins x nspins")
    if mode == "fast":
        return _qa_dense_fast(sched, mcsteps, slices, temp, nspins, confs, J, rng, seed, recompute_every)
    cur = _buffers.first_spin_order(rng, nspins)
    nsched = sched.size
    if nsched == 0:
        return None
    if np.float32(slices) * temp == 0:
        raise ZeroDivisionError("float division")
    if mcsteps <= 0:  # the reference's sweep loop runs no sweep and draws no order
        return None
    jp = reforder.jperp_schedule(sched, slices, temp)
    Jn = np.ascontiguousarray(J[:nspins, :nspins])
    spins = torch.from_numpy(np.ascontiguousarray(confs[:nspins, :slices]).astype(np.int8)[None]).to(
        _device.device())
    upd_per_g = max(1, nspins * slices * mcsteps)
    gchunk = max(1, CHUNK_UPDATES // upd_per_g)
    for g0 in range(0, nsched, gchunk):
        g1 = min(nsched, g0 + gchunk)
        perms, cur = _reference_perms(rng, cur, (g1 - g0) * mcsteps, nspins)
        rands = reforder.libc_peek((g1 - g0) * nspins * slices * mcsteps)[None]
        spins, used = reforder.quantum_anneal_dense(spins, Jn, sched[g0:g1], mcsteps, temp, perms, rands,
                                                    jperp=jp[g0:g1])
        reforder.libc_skip(int(used[0]))
    confs[:nspins, :slices] = spins[0].cpu().numpy()
    return None


def _qa_dense_fast(sched, mcsteps, slices, temp, nspins, confs, J, rng, seed, recompute_every):
    from . import dense
    if nspins != confs.shape[0]:
        raise ValueError("mode='fast' updates every row: nspins must equal confs.shape[0]")
    if slices < 1 or slices > 32:
        raise ValueError("mode='fast' needs 1 <= slices <= 32")
    if temp <= 0:
        raise ValueError("mode='fast' needs temp > 0")
    if mcsteps < 0:
        raise ValueError("mode='fast' needs mcsteps >= 0")
    if nspins == 0 or sched.size == 0 or mcsteps == 0:
        return None
    _buffers.check_pm1(confs[:, :slices], "confs")
    if seed is None:
        seed = _buffers.seed_from_rng(rng)
    prob = dense.DenseProblem(np.ascontiguousarray(J[:nspins, :nspins]))
    words = prob.pack(torch.from_numpy(np.ascontiguousarray(confs[:, :slices]).astype(np.int8)[None]))
    prob.anneal(words, sched, slices, float(temp), seed=seed, mcsteps=mcsteps, recompute_every=recompute_every)
    confs[:, :slices] = prob.unpack(words, slices)[0].cpu().numpy()
    return None


def QuantumAnneal_parallel(sched, mcsteps, slices, temp, nspins, confs, nbs, nthreads, *, seed=0, global_moves=0):
    """The reference's OpenMP variant (piqmc/qmc.pyx:247-340) on the GPU: the packed kernel.

    The reference threads race on shared spins (its results are not
    reproducible) and it takes no ``rng``; this runs ``QuantumAnneal(...,
    mode="fast")`` with Philox key ``seed``.  ``nthreads`` is accepted for
    compatibility and unused.
    """
    _buffers.as_c_int(nthreads, "nthreads")
    return QuantumAnneal(sched, mcsteps, slices, temp, nspins, confs, nbs, None, mode="fast", seed=seed,
                         global_moves=global_moves)
