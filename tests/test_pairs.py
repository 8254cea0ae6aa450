"""Pair world-line moves on the CPU: the bond classes, and the exactness of the learned move.

The learned pair move proposes a bond's pair flip with q(s) and accepts it with
min(1, exp(-beta dE) q(s') / q(s)); it keeps exp(-beta H) stationary when (a) the
reverse features the kernel scores from s are exactly the features of the flipped
state s', and (b) no other move of the same class changes a bond's cost or
features.  Both are checked on the oracle's restatement (which the GPU kernels
match bit for bit, tests/test_gpu_pairs.py), then stationarity itself by exact
enumeration of a small path-integral system.
"""
import itertools

import numpy as np
import pytest
import scipy.sparse as sps

import oracle
from pq_testutil import lattice


def _problem(J, maxnb):
    from piqmc import fast, tools
    n = J.shape[0]
    return fast.Problem(tools.GenerateNeighbors(n, J, maxnb), on_device=False)


def _random_graph(n, m, g):
    J = sps.dok_matrix((n, n))
    while J.nnz < m:
        a, b = sorted(g.choice(n, 2, replace=False))
        J[int(a), int(b)] = g.normal()
    return J


def _cases():
    g = np.random.default_rng(4)
    yield _problem(lattice(8, True, g, dist=lambda r: r.normal()), 4)
    yield _problem(lattice(7, True, g, dist=lambda r: r.uniform(-2, 2), fields=lambda r: r.normal(0, 0.3)), 5)
    yield _problem(_random_graph(40, 70, g), 12)


@pytest.mark.parametrize("k", range(3))
def test_bond_classes_are_independent_and_cover_every_coupling(k):
    from piqmc import pairs
    prob = list(_cases())[k]
    bc = pairs.BondClasses(prob)
    adj = bc.adjacency
    seen = set()
    for c in range(bc.nclass):
        lo, hi = bc.class_start[c], bc.class_start[c + 1]
        near = []
        for b in range(lo, hi):
            i, j = int(bc.bond_i[b]), int(bc.bond_j[b])
            assert i < j
            seen.add((i, j))
            near.append(({i, j}, {i, j} | adj[i] | adj[j]))
        for x in range(len(near)):
            for y in range(len(near)):
                if x != y:
                    assert not (near[x][0] & near[y][1]), "bonds of class %d interact" % c
    want = set()
    for m in range(prob.nbr_host.shape[0]):
        for i in range(prob.nslots):
            j = int(prob.nbr_host[m, i])
            if j != i and prob.cpl_host[m, i] != 0:
                want.add((min(i, j), max(i, j)))
    assert seen == want


def _words(prob, P, g):
    w = np.zeros(prob.nslots, np.uint64)
    bits = g.random((prob.n, P)) < 0.5
    w[prob.perm] = (bits.astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
    return w


@pytest.mark.parametrize("P", [1, 3, 20, 64])
def test_reverse_features_are_the_features_of_the_flipped_state(P):
    from piqmc import pairs
    g = np.random.default_rng(P)
    mask = np.uint64((1 << P) - 1) if P < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    for prob in _cases():
        bc = pairs.BondClasses(prob)
        w = _words(prob, P, g)
        for b in g.choice(bc.nbonds, 12, replace=False):
            si, sj, Jb = int(bc.bond_i[b]), int(bc.bond_j[b]), bc.bond_J[b]
            xr, dr = oracle.pair_features(w, prob.nbr_host, prob.cpl_host, prob.field_host, P, si, sj, Jb, 20.0, 0.7,
                                          flipped=True)
            xf, df = oracle.pair_features(w, prob.nbr_host, prob.cpl_host, prob.field_host, P, si, sj, Jb, 20.0, 0.7)
            w2 = w.copy()
            w2[si] ^= mask
            w2[sj] ^= mask
            x2, d2 = oracle.pair_features(w2, prob.nbr_host, prob.cpl_host, prob.field_host, P, si, sj, Jb, 20.0, 0.7)
            np.testing.assert_array_equal(xr.view(np.uint32), x2.view(np.uint32))
            assert dr.view(np.uint32) == d2.view(np.uint32)
            assert abs(float(df) + float(d2)) <= 1e-5 * max(1.0, abs(float(df)))   # the move and its reverse


def test_a_pair_flip_leaves_the_other_bonds_of_its_class_unchanged():
    from piqmc import pairs
    g = np.random.default_rng(9)
    P = 12
    mask = np.uint64((1 << P) - 1)
    for prob in _cases():
        bc = pairs.BondClasses(prob)
        w = _words(prob, P, g)
        for c in range(bc.nclass):
            lo, hi = int(bc.class_start[c]), int(bc.class_start[c + 1])
            if hi - lo < 2:
                continue
            feats = lambda ww: [oracle.pair_features(ww, prob.nbr_host, prob.cpl_host, prob.field_host, P,
                                                     bc.bond_i[b], bc.bond_j[b], bc.bond_J[b], 5.0, 0.3)
                                for b in range(lo, hi)]
            before = feats(w)
            w2 = w.copy()
            w2[bc.bond_i[lo]] ^= mask
            w2[bc.bond_j[lo]] ^= mask
            after = feats(w2)
            for (xa, da), (xb, db) in zip(before[1:], after[1:]):
                np.testing.assert_array_equal(xa, xb)
                assert da == db


def _logistic(x):
    a = np.array([-0.9, 0.4, -0.3, 0.8, 1.1, -0.5, 0.2, 0.3], np.float32)
    return np.float32(np.dot(a, x))


def _stationarity_error(wrong_reverse=False):
    """Max |(pi T_c - pi) / pi| over the classes of a 6-spin, 2-slice system (4096 states)."""
    from piqmc import pairs
    g = np.random.default_rng(2)
    J = lattice(3, False, g, dist=lambda r: r.normal())          # 3 x 3 open lattice would be 2^18 states:
    J = J.tocsr()[:6, :6].todok()                                  # keep its first two rows (6 spins, 7 bonds)
    for i in range(6):
        J[i, i] = g.normal(0, 0.3)
    prob = _problem(J, 5)
    bc = pairs.BondClasses(prob)
    P, beta, qmin = 2, np.float32(1.3), np.float32(0.05)
    n = prob.nslots
    mask = np.uint64(3)
    slots = list(prob.perm)
    states = list(itertools.product(range(4), repeat=6))

    def words_of(st):
        w = np.zeros(n, np.uint64)
        for spin, v in enumerate(st):
            w[slots[spin]] = np.uint64(v)
        return w

    def energy(st):   # classical energy summed over the slices (the Trotter terms are invariant)
        e = 0.0
        for k in range(P):
            s = np.array([1.0 - 2.0 * ((v >> k) & 1) for v in st])
            e += oracle.classical_energy(s, J)
        return e

    E = np.array([energy(st) for st in states])
    pi = np.exp(-beta * (E - E.min()))
    index = {st: a for a, st in enumerate(states)}
    worst = 0.0
    for c in range(bc.nclass):
        lo, hi = int(bc.class_start[c]), int(bc.class_start[c + 1])
        new = np.zeros(len(states))
        for a, st in enumerate(states):
            w = words_of(st)
            probs = []
            for b in range(lo, hi):
                si, sj, Jb = int(bc.bond_i[b]), int(bc.bond_j[b]), bc.bond_J[b]
                x, dE = oracle.pair_features(w, prob.nbr_host, prob.cpl_host, prob.field_host, P, si, sj, Jb, beta, 0.5)
                xr, _ = oracle.pair_features(w, prob.nbr_host, prob.cpl_host, prob.field_host, P, si, sj, Jb, beta, 0.5,
                                             flipped=True)
                q = min(max(float(oracle.pair_sigmoid(_logistic(x))), qmin), 1.0)
                qr = q if wrong_reverse else min(max(float(oracle.pair_sigmoid(_logistic(xr))), qmin), 1.0)
                probs.append(min(q, np.exp(-beta * float(dE)) * qr))
            # the bonds of a class move independently: every subset of them flips
            for flips in itertools.product((0, 1), repeat=hi - lo):
                p = 1.0
                st2 = list(st)
                for t, f in enumerate(flips):
                    p *= probs[t] if f else 1.0 - probs[t]
                    if f:
                        b = lo + t
                        for s_ in (bc.bond_i[b], bc.bond_j[b]):
                            spin = slots.index(s_)
                            st2[spin] ^= int(mask)
                new[index[tuple(st2)]] += pi[a] * p
        worst = max(worst, float(np.max(np.abs(new - pi) / pi)))
    return worst


def test_learned_pair_pass_keeps_the_path_integral_distribution():
    assert _stationarity_error() < 2e-5


def test_stationarity_check_fails_without_the_reverse_probability():
    assert _stationarity_error(wrong_reverse=True) > 1e-3
