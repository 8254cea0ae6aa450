"""The packed algorithm samples the path-integral distribution exactly (CPU, through its
bit-exact oracle): on a frustrated 3-spin triangle with fields, long runs at fixed transverse
field must reproduce the exact expectations of exp(-H/T),

    H = sum_k E_cl(s_k) - J_perp sum_k s_k s_(k+1 mod P),

obtained by enumerating all 2^(3P) states.  Each replica's time average is one independent
sample, so the standard error is the spread over replicas / sqrt(R).  P = 2, 3 (three slice
classes) and 4, local sweeps alone and with world-line moves."""
import itertools

import numpy as np
import pytest
import scipy.sparse as sps

import oracle

N = 3
COUPLINGS = [(0, 1, 0.75), (1, 2, -0.5), (0, 2, 0.625), (0, 0, 0.25), (1, 1, -0.125), (2, 2, 0.375)]


def _problem():
    from piqmc import fast, tools
    J = sps.dok_matrix((N, N))
    for a, b, v in COUPLINGS:
        J[a, b] = v
    return J, fast.Problem(tools.GenerateNeighbors(N, J, 3), on_device=False)


def _observables(s, Jd, jp):
    """s: (..., N, P) spins -> classical energy per slice, Trotter correlation, magnetisations."""
    up = np.triu(Jd, 1)
    h = np.diag(Jd)
    ecl = -np.einsum("...ik,ij,...jk->...k", s, up, s) - np.einsum("i,...ik->...k", h, s)
    trot = (s * np.roll(s, -1, axis=-1)).sum(-2)
    return np.concatenate([ecl.mean(-1)[..., None], trot.mean(-1)[..., None], s.mean(-1)], axis=-1)


def _exact(Jd, jp, P, T):
    states = np.array(list(itertools.product([1.0, -1.0], repeat=N * P))).reshape(-1, N, P)
    obs = _observables(states, Jd, jp)
    H = P * obs[:, 0] - jp * P * obs[:, 1]
    w = np.exp(-(H - H.min()) / T)
    w /= w.sum()
    return (w[:, None] * obs).sum(0)


@pytest.mark.parametrize("P,global_moves", [(2, 0), (3, 0), (4, 0), (4, 1), (3, 1)])
def test_packed_sweep_samples_the_exact_distribution(P, global_moves):
    J, prob = _problem()
    Jd = np.asarray(J.todense())
    T, G = 1.0, 2.5           # J_perp 0.1 .. 1.2: every world-line still mixes by local moves
    jp32 = oracle.jperp(np.array([G]), P, T).astype(np.float32)
    jp = float(jp32[0])
    exact = _exact(Jd, jp, P, T)
    R, burn, sweeps = 96, 100, 400
    g = np.random.default_rng(P * 10 + global_moves)
    means = []
    for r in range(R):
        s0 = np.where(g.random((N, P)) < 0.5, -1, 1)
        w = np.zeros(prob.nslots, np.uint64)
        w[prob.perm] = ((s0 < 0).astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(1).astype(np.uint64)
        acc = []
        for it in range(burn + sweeps):
            oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride,
                               w, P, jp32, 1, np.float32(1) / np.float32(T), 77, sweep_base=it, replica=r,
                               global_moves=global_moves)
            if it >= burn:
                acc.append(np.where((w[prob.perm][:, None] >> np.arange(P, dtype=np.uint64)) & 1, -1.0, 1.0))
        means.append(_observables(np.array(acc), Jd, jp).mean(0))
    means = np.array(means)
    est, se = means.mean(0), means.std(0, ddof=1) / np.sqrt(R)
    assert np.all(np.abs(est - exact) < 4.5 * se + 1e-3), (est, exact, se)


@pytest.mark.parametrize("P,per_slice", [(2, False), (3, False), (4, False), (4, True), (3, True)])
def test_dense_sweep_samples_the_exact_distribution(P, per_slice):
    """The dense packed sweep (affine spin orders shared by the slices or one per slice,
    incremental FP32 fields) on the same triangle as a dense matrix: the same exact
    expectations."""
    import math
    J, _ = _problem()
    Jd = np.asarray(J.todense())
    up = np.triu(Jd, 1)
    K = (up + up.T).astype(np.float32)
    h = np.diag(Jd)
    T, G = 1.0, 2.5
    jp32 = oracle.jperp(np.array([G]), P, T).astype(np.float32)
    exact = _exact(Jd, float(jp32[0]), P, T)
    units = np.array([a for a in range(1, N) if math.gcd(a, N) == 1], np.int32)
    R, burn, sweeps = 96, 100, 400
    g = np.random.default_rng(500 + P)
    means = []
    for r in range(R):
        s0 = np.where(g.random((N, P)) < 0.5, -1, 1)
        w = ((s0 < 0).astype(np.uint32) << np.arange(P, dtype=np.uint32)).sum(1).astype(np.uint32)
        F = (s0.T.astype(np.float64) @ K.T.astype(np.float64) + h[None, :]).astype(np.float32)
        acc = []
        for it in range(burn + sweeps):
            _, F = oracle.dense_sweep(F, K, units, w, P, jp32, 1, np.float32(1) / np.float32(T), 91,
                                      sweep_base=it, replica=r, per_slice_order=per_slice)
            if it >= burn:
                acc.append(np.where((w[:, None] >> np.arange(P, dtype=np.uint32)) & 1, -1.0, 1.0))
        means.append(_observables(np.array(acc), Jd, float(jp32[0])).mean(0))
    means = np.array(means)
    est, se = means.mean(0), means.std(0, ddof=1) / np.sqrt(R)
    assert np.all(np.abs(est - exact) < 4.5 * se + 1e-3), (est, exact, se)
