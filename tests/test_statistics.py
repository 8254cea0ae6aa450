"""Statistical parity of the packed algorithm with the reference (CPU, through the oracles).

The packed kernel is bit-exact with its CPU restatement (GPU tests), so its
statistics can be judged on the CPU: final energies after a full anneal, over
independent seeds, against the reference's QuantumAnneal with both quirks
corrected (per-spin energy reset, k-1/k+1 Trotter coupling) run in the
reference's own random sequential order.  The 99% confidence interval of the
difference of the means must contain 0.  The as-shipped reference (both quirks)
is also run, to show the gap those quirks cause.
"""
import numpy as np
import pytest

import oracle
from pq_testutil import lattice

SEEDS = 400


def _instance():
    from piqmc import fast, tools
    g = np.random.default_rng(0)
    J = lattice(8, True, g)
    nbs = tools.GenerateNeighbors(64, J, 4)
    return J, nbs, fast.Problem(nbs, on_device=False)


def _energies(J, P, spins_cols):
    return np.array([oracle.classical_energy(spins_cols[:, k].astype(np.float64), J) for k in range(P)])


def _run(kind, J, nbs, prob, seed, P=20, T=0.05, ns=100):
    n = 64
    sched = np.linspace(3.0, 1e-8, ns)
    rs = np.random.default_rng(1000 + seed)
    s0 = np.where(rs.random(n) < 0.5, -1, 1).astype(np.int8)
    if kind == "fast":
        w = np.zeros(prob.nslots, np.uint64)
        bits = (np.tile(s0, (P, 1)).T < 0).astype(np.uint64)
        w[prob.perm] = (bits << np.arange(P, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
        oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w,
                           P, oracle.jperp(sched, P, T), 1, np.float32(1) / np.float32(T), seed, replica=seed)
        wo = w[prob.perm]
        sp = np.where((wo[:, None] >> np.arange(P, dtype=np.uint64)) & 1, -1, 1)
    else:
        sp = np.ascontiguousarray(np.tile(s0, (P, 1)).T)
        perms = oracle.reference_perms(np.random.RandomState(seed), n, ns)
        rands = rs.integers(0, 2 ** 31 - 1, size=n * P * ns, dtype=np.int64).astype(np.int32)
        oracle.qa_sparse(sp, nbs, sched, 1, T, perms, rands, flags=3 if kind == "corrected" else 0)
    return _energies(J, P, sp)


@pytest.fixture(scope="module")
def samples():
    J, nbs, prob = _instance()
    out = {}
    for kind in ("fast", "corrected", "shipped"):
        out[kind] = np.array([_run(kind, J, nbs, prob, s) for s in range(SEEDS)])
    return out


@pytest.mark.parametrize("stat", ["best_slice", "slice_mean"])
def test_fast_matches_corrected_reference(samples, stat):
    f = samples["fast"].min(1) if stat == "best_slice" else samples["fast"].mean(1)
    r = samples["corrected"].min(1) if stat == "best_slice" else samples["corrected"].mean(1)
    diff = f.mean() - r.mean()
    se = np.sqrt(f.var(ddof=1) / len(f) + r.var(ddof=1) / len(r))
    assert abs(diff) < 2.576 * se, (diff, se)   # 99% two-sided


def test_distributions_agree(samples):
    """Two-sample Kolmogorov-Smirnov on the best-slice energy at the 1% level."""
    from scipy.stats import ks_2samp
    assert ks_2samp(samples["fast"].min(1), samples["corrected"].min(1)).pvalue > 0.01


def test_shipped_quirks_change_the_physics(samples):
    """The as-shipped reference (energy carried across spins) anneals far worse: the gap the
    packed kernel does not reproduce by design."""
    s = samples["shipped"].min(1)
    r = samples["corrected"].min(1)
    se = np.sqrt(s.var(ddof=1) / len(s) + r.var(ddof=1) / len(r))
    assert s.mean() - r.mean() > 5 * se


def _dense_run(kind, J, seed, P=8, T=0.05, ns=60):
    import math
    N = J.shape[0]
    sched = np.linspace(3.0, 1e-8, ns)
    rs = np.random.default_rng(5000 + seed)
    s0 = np.where(rs.random(N) < 0.5, -1, 1).astype(np.int8)
    if kind == "fast":
        up = np.triu(J, 1)
        K = up + up.T
        sp = np.tile(s0, (P, 1)).astype(np.float64)              # (P, N)
        F = (sp @ K.T + np.diag(J)[None, :]).astype(np.float32)
        w = (((np.tile(s0, (P, 1)).T < 0).astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(1)).astype(np.uint32)
        units = np.array([a for a in range(1, N) if math.gcd(a, N) == 1], np.int32)
        oracle.dense_sweep(F, K.astype(np.float32), units, w, P, oracle.jperp(sched, P, T), 1,
                           np.float32(1) / np.float32(T), seed, replica=seed)
        spins = np.where((w[:, None] >> np.arange(P, dtype=np.uint32)) & 1, -1, 1)
    else:
        spins = np.ascontiguousarray(np.tile(s0, (P, 1)).T)
        perms = oracle.reference_perms(np.random.RandomState(seed), N, ns)
        rands = rs.integers(0, 2 ** 31 - 1, size=N * P * ns, dtype=np.int64).astype(np.int32)
        oracle.qa_dense(spins, J, sched, 1, T, perms, rands, flags=3)
    return np.array([oracle.classical_energy(spins[:, k].astype(np.float64), J) for k in range(P)])


def test_dense_fast_matches_corrected_reference():
    """Dense packed algorithm vs the corrected dense reference (QuantumAnneal_dense), 300 seeds, 99% CI."""
    g = np.random.default_rng(3)
    N = 32
    J = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1) + np.diag(g.normal(0.0, np.sqrt(0.1), N))
    f = np.array([_dense_run("fast", J, s).min() for s in range(300)])
    r = np.array([_dense_run("corrected", J, s).min() for s in range(300)])
    diff = f.mean() - r.mean()
    se = np.sqrt(f.var(ddof=1) / len(f) + r.var(ddof=1) / len(r))
    assert abs(diff) < 2.576 * se, (f.mean(), r.mean(), se)


def _ci_agrees(f, r):
    diff = f.mean() - r.mean()
    se = np.sqrt(f.var(ddof=1) / len(f) + r.var(ddof=1) / len(r))
    return abs(diff) < 2.576 * se, (f.mean(), r.mean(), se)


def test_odd_slices_with_fields_match_corrected_reference():
    """P = 7 (three slice classes: even k < 6, odd k, k = 6), fields, T = 0.3: the packed
    algorithm against the corrected reference, 400 seeds, best-slice and slice-mean energies."""
    from piqmc import fast, tools
    g = np.random.default_rng(11)
    J = lattice(6, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0.0, 0.5))
    nbs = tools.GenerateNeighbors(36, J, 5)
    prob = fast.Problem(nbs, on_device=False)
    P, T, ns, n = 7, 0.3, 60, 36
    sched = np.linspace(2.0, 1e-8, ns)
    res = {"fast": [], "corrected": []}
    for seed in range(400):
        rs = np.random.default_rng(7000 + seed)
        s0 = np.where(rs.random((n, P)) < 0.5, -1, 1).astype(np.int8)
        w = np.zeros(prob.nslots, np.uint64)
        w[prob.perm] = ((s0 < 0).astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
        oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w,
                           P, oracle.jperp(sched, P, T), 1, np.float32(1) / np.float32(T), seed, replica=seed)
        sp = np.where((w[prob.perm][:, None] >> np.arange(P, dtype=np.uint64)) & 1, -1, 1)
        res["fast"].append(_energies(J, P, sp))
        sp = s0.copy()
        perms = oracle.reference_perms(np.random.RandomState(seed), n, ns)
        rands = rs.integers(0, 2 ** 31 - 1, size=n * P * ns, dtype=np.int64).astype(np.int32)
        oracle.qa_sparse(sp, nbs, sched, 1, T, perms, rands, flags=3)
        res["corrected"].append(_energies(J, P, sp))
    f, r = np.array(res["fast"]), np.array(res["corrected"])
    for stat in (lambda a: a.min(1), lambda a: a.mean(1)):
        ok, info = _ci_agrees(stat(f), stat(r))
        assert ok, info


def test_packed_classical_annealer_matches_sa_anneal():
    """P = 1 with a per-step inverse temperature (the packed form of sa.Anneal) against the
    reference's sa.Anneal (no quirks to correct), 400 seeds; energies after a short and a full
    schedule."""
    from piqmc import fast, tools
    g = np.random.default_rng(12)
    J = lattice(8, True, g, fields=lambda r: r.uniform(-1.0, 1.0))
    nbs = tools.GenerateNeighbors(64, J, 5)
    prob = fast.Problem(nbs, on_device=False)
    n = 64
    for tsched in (np.linspace(5.0, 0.5, 8), np.linspace(5.0, 0.05, 60)):
        betas = np.float32(1) / tsched.astype(np.float32)
        res = {"fast": [], "sa": []}
        for seed in range(400):
            rs = np.random.default_rng(9000 + seed)
            s0 = np.where(rs.random(n) < 0.5, -1, 1).astype(np.int8)
            w = np.zeros(prob.nslots, np.uint64)
            w[prob.perm] = (s0 < 0).astype(np.uint64)
            oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w,
                               1, np.zeros(len(tsched), np.float32), 1, betas[0], seed, replica=seed, betas=betas)
            sf = np.where(w[prob.perm] & 1, -1, 1)
            res["fast"].append(oracle.classical_energy(sf.astype(np.float64), J))
            s = s0.copy()
            perms = oracle.reference_perms(np.random.RandomState(seed), n, len(tsched))
            rands = rs.integers(0, 2 ** 31 - 1, size=n * len(tsched), dtype=np.int64).astype(np.int32)
            oracle.sa_sparse(s, nbs, tsched, 1, perms, rands)
            res["sa"].append(oracle.classical_energy(s.astype(np.float64), J))
        ok, info = _ci_agrees(np.array(res["fast"]), np.array(res["sa"]))
        assert ok, (tsched[-1], info)
