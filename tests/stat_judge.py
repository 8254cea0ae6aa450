"""Statistical judge of the packed kernels on the GPU -- TEST INFRASTRUCTURE ONLY.

The packed sweeps (the sparse one of csrc/sweep_core.cuh and the dense one of
csrc/dense.cu) do not follow the reference's spin order, so they are judged by
the distributions they produce.  The judge is the reference's own sweep --
QuantumAnneal (reference piqmc/qmc.pyx:93-136) and QuantumAnneal_dense
(piqmc/qmc.pyx:197-242) with both quirks corrected (flags FIX_Q1 | FIX_Q2: the
energy difference reset per spin, slice k coupled to k - 1 and k + 1) -- run by
the reference-order kernels, which are bit-exact with oracle.qa_sparse(flags=3)
and oracle.qa_dense(flags=3).  Each judge replica draws a fresh random spin
permutation per sweep (shared by its slices, as the reference shares one) and a
fresh stream of 31-bit uniforms, both generated on the GPU, one chunk of field
steps at a time (the streams of a full 80x80, 2000-step anneal would be about a
gigabyte per replica).

Both sides start from the same distribution (independent random +-1 spins per
replica, copied to every slice) and anneal the same instance with the same
schedule; the judge compares the final energy per replica (best slice, and
mean over slices; FP64, ClassicalIsingEnergy's definition) by a 99 % Welch
interval on the difference of the means and a two-sample Kolmogorov-Smirnov
test.
"""
import math

import numpy as np
import scipy.sparse as sps
import scipy.stats as st
import torch

FIX_BOTH = 3   # PQ_FIX_Q2 | PQ_FIX_Q1


def lattice_instance(L, dist, seed):
    """L x L periodic lattice (right and down bonds, FP32-valued couplings) and its neighbour table."""
    from piqmc import tools
    g = np.random.default_rng(seed)
    n = L * L
    J = sps.dok_matrix((n, n))
    for y in range(L):
        for x in range(L):
            i = y * L + x
            J[i, y * L + (x + 1) % L] = float(np.float32(dist(g)))
            J[i, ((y + 1) % L) * L + x] = float(np.float32(dist(g)))
    return J, tools.GenerateNeighbors(n, J, 4)


def dense_instance(N, seed):
    """Dense instance: J_ij ~ N(0, 1/N) on the upper triangle, fields ~ N(0, 0.1) on the diagonal (FP32 values)."""
    g = np.random.default_rng(seed)
    J = np.triu(g.normal(0.0, 1.0 / math.sqrt(N), (N, N)).astype(np.float32).astype(np.float64), 1)
    J += np.diag(g.normal(0.0, math.sqrt(0.1), N).astype(np.float32).astype(np.float64))
    return J


def start_spins(R, n, P, seed):
    """Independent random +-1 spins per replica, the same in every slice: int8 (R, n, P) on the device."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    s = torch.where(torch.rand((R, n), generator=g, device="cuda") < 0.5, -1, 1).to(torch.int8)
    return s[:, :, None].expand(R, n, P).contiguous()


def _streams(R, steps, n, P, gen):
    perms = torch.argsort(torch.rand((R, steps, n), generator=gen, device="cuda"), dim=2).to(torch.int32)
    cap = n * P * steps
    rands = torch.randint(0, 2 ** 31 - 1, (R, cap), generator=gen, device="cuda", dtype=torch.int32)
    return perms, rands, cap


def judge_sparse(nbs, spins, sched, P, temp, seed, chunk=100):
    """Corrected reference order on the GPU: final int8 spins (R, n, P)."""
    from piqmc import _device, _native, reforder
    idx, jv = reforder.split_neighbors(nbs)
    sp = spins.clone()
    R, n, _ = sp.shape
    jp = torch.from_numpy(reforder.jperp_schedule(sched, P, temp)).cuda()
    d_idx, d_j = torch.from_numpy(idx).cuda(), torch.from_numpy(jv).cuda()
    used = torch.zeros(R, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(seed)
    lib = _native.lib()
    for g0 in range(0, len(sched), chunk):
        g1 = min(len(sched), g0 + chunk)
        perms, rands, cap = _streams(R, g1 - g0, n, P, gen)
        used.zero_()
        _native.check(lib.pq_qa_sparse_reforder(
            _device.ptr(sp), _device.ptr(d_idx), _device.ptr(d_j), n, n, idx.shape[1], P, R, _device.ptr(jp[g0:g1]),
            g1 - g0, 1, float(np.float32(temp)), _device.ptr(perms), _device.ptr(rands), cap, _device.ptr(used),
            FIX_BOTH, _device.ptr(status), _device.stream_handle()), "pq_qa_sparse_reforder")
        del perms, rands
    torch.cuda.synchronize()
    if int(status.item()):
        raise _native.PiqmcError(int(status.item()), "judge")
    return sp


def judge_dense(J, spins, sched, P, temp, seed, chunk=100):
    """Corrected reference order of QuantumAnneal_dense on the GPU: final int8 spins (R, N, P)."""
    from piqmc import _device, _native, reforder
    sp = spins.clone()
    R, n, _ = sp.shape
    jp = torch.from_numpy(reforder.jperp_schedule(sched, P, temp)).cuda()
    d_J = torch.from_numpy(np.ascontiguousarray(J, dtype=np.float64)).cuda()
    used = torch.zeros(R, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(seed)
    lib = _native.lib()
    for g0 in range(0, len(sched), chunk):
        g1 = min(len(sched), g0 + chunk)
        perms, rands, cap = _streams(R, g1 - g0, n, P, gen)
        used.zero_()
        _native.check(lib.pq_qa_dense_reforder(
            _device.ptr(sp), _device.ptr(d_J), n, P, R, _device.ptr(jp[g0:g1]), g1 - g0, 1, float(np.float32(temp)),
            _device.ptr(perms), _device.ptr(rands), cap, _device.ptr(used), FIX_BOTH, _device.ptr(status),
            _device.stream_handle()), "pq_qa_dense_reforder")
        del perms, rands
    torch.cuda.synchronize()
    if int(status.item()):
        raise _native.PiqmcError(int(status.item()), "judge")
    return sp


def fast_sparse(prob, spins, sched, P, temp, seed):
    """The packed sweep (random class order): final packed words."""
    from piqmc import fast
    words = prob.pack(spins)
    fast.anneal(prob, words, sched, P, temp, seed=seed)
    return words


def summary(E):
    """(best-slice, slice-mean) final energy per replica from FP64 energies (R, P)."""
    E = np.asarray(E, dtype=np.float64)
    return E.min(axis=1), E.mean(axis=1)


def compare(a, b, level=0.99):
    """Difference of means a - b with its Welch interval at `level`, and the two-sample KS p-value."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    va, vb = a.var(ddof=1) / len(a), b.var(ddof=1) / len(b)
    se = math.sqrt(va + vb)
    df = (va + vb) ** 2 / (va ** 2 / (len(a) - 1) + vb ** 2 / (len(b) - 1)) if se > 0 else 1.0
    half = st.t.ppf(0.5 + level / 2, df) * se
    d = float(a.mean() - b.mean())
    return {"diff": d, "lo": d - half, "hi": d + half, "se": se, "ks_p": float(st.ks_2samp(a, b).pvalue),
            "mean_a": float(a.mean()), "mean_b": float(b.mean()), "sd_a": float(a.std(ddof=1)),
            "sd_b": float(b.std(ddof=1)), "n_a": len(a), "n_b": len(b)}
