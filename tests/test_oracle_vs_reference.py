"""The CPU oracle against the compiled reference itself on random cases (where the recipe in
oracle/build_ref.py has built it into oracle/_ref; skipped elsewhere).

Each case runs the reference's Cython QuantumAnneal, QuantumAnneal_dense, Anneal,
Anneal_dense or Anneal_bipartite with a seeded libc rand() and numpy RandomState, and the
oracle with the same streams rebuilt; final spins, the number of libc values consumed (the
reference's next rand() value sits at the oracle's count) and the caller's rng state must
agree.  Cases: random sparse graphs of irregular degree with general FP64 couplings (the
reference rounds each to FP32) and fields, odd and even slice counts, cold and hot
temperatures, several sweeps per schedule step.
"""
import ctypes
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sps

import oracle
from pq_testutil import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
ref = pytest.importorskip("piqmc_ref.qmc", reason="compiled reference not built here")
from piqmc_ref import qmc, sa, tools  # noqa: E402

libc = ctypes.CDLL(None)
CASES = 24


def _random_graph(g, n, fields):
    J = sps.dok_matrix((n, n), dtype=np.float64)
    m = int(g.integers(n, 3 * n + 1))
    for _ in range(m):
        i, j = sorted(int(v) for v in g.choice(n, 2, replace=False))
        J[i, j] = g.normal(0.0, 1.0) * (10.0 ** g.uniform(-1, 1))
    if fields:
        for i in range(n):
            if g.random() < 0.7:
                J[i, i] = g.normal(0.0, 0.5)
    return J


def _temp_sched(g, lo, hi):
    return np.sort(g.uniform(lo, hi, int(g.integers(2, 10))))[::-1].copy()


@pytest.mark.parametrize("case", range(CASES))
def test_quantum_anneal_random(case):
    g = np.random.default_rng(1000 + case)
    n, P = int(g.integers(3, 40)), int(g.integers(2, 8))
    T = float(g.choice([0.01, 0.3, 2.0]))
    mcsteps = int(g.integers(1, 4))
    J = _random_graph(g, n, fields=case % 2 == 0)
    maxnb = int(max(np.count_nonzero(J.toarray()[i]) + np.count_nonzero(J.toarray()[:, i]) for i in range(n))) + 1
    nbs = np.asarray(tools.GenerateNeighbors(n, J, maxnb))
    np.testing.assert_array_equal(oracle.generate_neighbors(n, J, maxnb), nbs)
    sched = _temp_sched(g, 1e-6, 3.0)
    conf0 = np.where(g.random((n, P)) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(conf0.copy())
    cseed, rseed = 7 + case, 70 + case
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    qmc.QuantumAnneal(sched, mcsteps, P, T, n, confs, nbs, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(rseed)
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(cseed, n * P * len(sched) * mcsteps + 1)
    sp = np.ascontiguousarray(conf0.astype(np.int8))
    used = oracle.qa_sparse(sp, nbs, sched, mcsteps, T, perms, rands)
    np.testing.assert_array_equal(sp, confs.astype(np.int8))
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng


@pytest.mark.parametrize("case", range(CASES))
def test_quantum_anneal_dense_random(case):
    g = np.random.default_rng(2000 + case)
    n, P = int(g.integers(2, 30)), int(g.integers(2, 7))
    T = float(g.choice([0.01, 0.3, 2.0]))
    mcsteps = int(g.integers(1, 3))
    Jd = np.triu(g.normal(0.0, 1.0, (n, n)) * (10.0 ** g.uniform(-1, 1)), 1)
    if case % 2 == 0:
        Jd += np.diag(g.normal(0.0, 0.5, n))
    sched = _temp_sched(g, 1e-6, 3.0)
    conf0 = np.where(g.random((n, P)) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(conf0.copy())
    cseed, rseed = 17 + case, 170 + case
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    qmc.QuantumAnneal_dense(sched, mcsteps, P, T, n, confs, Jd, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(rseed)
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(cseed, n * P * len(sched) * mcsteps + 1)
    sp = np.ascontiguousarray(conf0.astype(np.int8))
    used = oracle.qa_dense(sp, Jd, sched, mcsteps, T, perms, rands)
    np.testing.assert_array_equal(sp, confs.astype(np.int8))
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng


@pytest.mark.parametrize("case", range(CASES))
def test_anneal_random(case):
    g = np.random.default_rng(3000 + case)
    n = int(g.integers(3, 50))
    mcsteps = int(g.integers(1, 4))
    J = _random_graph(g, n, fields=case % 2 == 0)
    maxnb = int(max(np.count_nonzero(J.toarray()[i]) + np.count_nonzero(J.toarray()[:, i]) for i in range(n))) + 1
    nbs = np.asarray(tools.GenerateNeighbors(n, J, maxnb))
    tsched = _temp_sched(g, 0.01, 5.0)
    sv0 = np.where(g.random(n) < 0.5, -1.0, 1.0)
    sv = sv0.copy()
    cseed, rseed = 27 + case, 270 + case
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    sa.Anneal(tsched, mcsteps, sv, nbs, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(rseed)
    perms = oracle.reference_perms(rng, n, len(tsched) * mcsteps)
    rands = oracle.libc_stream(cseed, n * len(tsched) * mcsteps + 1)
    s = sv0.astype(np.int8)
    used = oracle.sa_sparse(s, nbs, tsched, mcsteps, perms, rands)
    np.testing.assert_array_equal(s, sv.astype(np.int8))
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng


@pytest.mark.parametrize("case", range(CASES))
def test_anneal_dense_random(case):
    g = np.random.default_rng(4000 + case)
    n = int(g.integers(2, 40))
    mcsteps = int(g.integers(1, 3))
    Jd = np.triu(g.normal(0.0, 1.0, (n, n)) * (10.0 ** g.uniform(-1, 1)), 1)
    if case % 2 == 0:
        Jd += np.diag(g.normal(0.0, 0.5, n))
    tsched = _temp_sched(g, 0.01, 5.0)
    sv0 = np.where(g.random(n) < 0.5, -1.0, 1.0)
    sv = sv0.copy()
    cseed, rseed = 37 + case, 370 + case
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    sa.Anneal_dense(tsched, mcsteps, sv, Jd, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(rseed)
    perms = oracle.reference_perms(rng, n, len(tsched) * mcsteps)
    rands = oracle.libc_stream(cseed, n * len(tsched) * mcsteps + 1)
    s = sv0.astype(np.int8)
    used = oracle.sa_dense(s, Jd, tsched, mcsteps, perms, rands)
    np.testing.assert_array_equal(s, sv.astype(np.int8))
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng


@pytest.mark.parametrize("case", range(CASES))
def test_anneal_bipartite_random(case):
    g = np.random.default_rng(5000 + case)
    nl, nr = int(g.integers(1, 25)), int(g.integers(1, 25))
    mcsteps = int(g.integers(1, 3))
    Jb = g.normal(0.0, 1.0, (nl, nr)) * (10.0 ** g.uniform(-1, 1))
    lb, rb = g.normal(0.0, 0.3, nl), g.normal(0.0, 0.3, nr)
    tsched = _temp_sched(g, 0.01, 5.0)
    l0, r0 = np.where(g.random(nl) < 0.5, -1.0, 1.0), np.where(g.random(nr) < 0.5, -1.0, 1.0)
    lv, rv = l0.copy(), r0.copy()
    cseed = 47 + case
    libc.srand(cseed)
    rng = np.random.RandomState(470 + case)
    sa.Anneal_bipartite(tsched, mcsteps, lv, rv, Jb, lb, rb, rng)
    next_rand = libc.rand()

    rands = oracle.libc_stream(cseed, (nl + nr) * len(tsched) * mcsteps + 1)
    ls, rs = l0.astype(np.int8), r0.astype(np.int8)
    used = oracle.sa_bipartite(ls, rs, Jb, lb, rb, tsched, mcsteps, rands)
    np.testing.assert_array_equal(ls, lv.astype(np.int8))
    np.testing.assert_array_equal(rs, rv.astype(np.int8))
    assert rands[used] == next_rand


@pytest.mark.parametrize("case", range(12))
def test_quantum_anneal_fewer_spins_than_rows(case):
    """nspins < rows: the sweep visits the first nspins spins only; the rows past them are
    boundary spins that neighbours read and nothing writes (reference piqmc/qmc.pyx:91)."""
    g = np.random.default_rng(6000 + case)
    n, P = int(g.integers(4, 30)), int(g.integers(2, 7))
    nspins = int(g.integers(1, n))
    T = float(g.choice([0.05, 0.5, 2.0]))
    J = _random_graph(g, n, fields=case % 2 == 1)
    maxnb = int(max(np.count_nonzero(J.toarray()[i]) + np.count_nonzero(J.toarray()[:, i]) for i in range(n))) + 1
    nbs = np.asarray(tools.GenerateNeighbors(n, J, maxnb))
    sched = _temp_sched(g, 1e-6, 3.0)
    conf0 = np.where(g.random((n, P)) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(conf0.copy())
    cseed, rseed = 57 + case, 570 + case
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    qmc.QuantumAnneal(sched, 2, P, T, nspins, confs, nbs, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(rseed)
    perms = oracle.reference_perms(rng, nspins, len(sched) * 2)
    rands = oracle.libc_stream(cseed, nspins * P * len(sched) * 2 + 1)
    sp = np.ascontiguousarray(conf0.astype(np.int8))
    used = oracle.qa_sparse(sp, nbs, sched, 2, T, perms, rands)
    np.testing.assert_array_equal(sp, confs.astype(np.int8))
    np.testing.assert_array_equal(sp[nspins:], conf0[nspins:].astype(np.int8))
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng


@pytest.mark.parametrize("nl,nr", [(0, 7), (5, 0), (1, 1), (1, 30)])
def test_anneal_bipartite_empty_and_tiny_sides(nl, nr):
    g = np.random.default_rng(nl * 100 + nr)
    Jb = g.normal(0.0, 1.0, (nl, nr))
    lb, rb = g.normal(0.0, 0.3, nl), g.normal(0.0, 0.3, nr)
    tsched = _temp_sched(g, 0.01, 5.0)
    l0, r0 = np.where(g.random(nl) < 0.5, -1.0, 1.0), np.where(g.random(nr) < 0.5, -1.0, 1.0)
    lv, rv = l0.copy(), r0.copy()
    libc.srand(81)
    sa.Anneal_bipartite(tsched, 2, lv, rv, Jb, lb, rb, np.random.RandomState(0))
    next_rand = libc.rand()
    rands = oracle.libc_stream(81, (nl + nr) * len(tsched) * 2 + 1)
    ls, rs = l0.astype(np.int8), r0.astype(np.int8)
    used = oracle.sa_bipartite(ls, rs, Jb, lb, rb, tsched, 2, rands)
    np.testing.assert_array_equal(ls, lv.astype(np.int8))
    np.testing.assert_array_equal(rs, rv.astype(np.int8))
    assert rands[used] == next_rand


@pytest.mark.parametrize("case", range(6))
def test_quantum_anneal_dense_fewer_spins_than_rows(case):
    """QuantumAnneal_dense with nspins < rows reads only the leading nspins x nspins block of J
    and the first nspins rows of confs (reference piqmc/qmc.pyx:206), the cut the drop-in makes."""
    g = np.random.default_rng(6500 + case)
    n, P = int(g.integers(4, 25)), int(g.integers(2, 6))
    nspins = int(g.integers(1, n))
    Jd = np.triu(g.normal(0.0, 1.0, (n, n)), 1) + np.diag(g.normal(0.0, 0.5, n))
    sched = _temp_sched(g, 1e-6, 3.0)
    conf0 = np.where(g.random((n, P)) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(conf0.copy())
    libc.srand(91 + case)
    rng = np.random.RandomState(910 + case)
    qmc.QuantumAnneal_dense(sched, 1, P, 0.3, nspins, confs, Jd, rng)
    next_rand, next_rng = libc.rand(), rng.randint(2 ** 31)

    rng = np.random.RandomState(910 + case)
    perms = oracle.reference_perms(rng, nspins, len(sched))
    rands = oracle.libc_stream(91 + case, nspins * P * len(sched) + 1)
    sp = np.ascontiguousarray(conf0[:nspins].astype(np.int8))
    used = oracle.qa_dense(sp, np.ascontiguousarray(Jd[:nspins, :nspins]), sched, 1, 0.3, perms, rands)
    np.testing.assert_array_equal(sp, confs[:nspins].astype(np.int8))
    np.testing.assert_array_equal(confs[nspins:], conf0[nspins:])
    assert rands[used] == next_rand
    assert rng.randint(2 ** 31) == next_rng
