"""Batched persistent launch: equals the single-instance packed kernel bit for bit."""
import numpy as np
import pytest
import torch

from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def _instances(seed=0):
    from piqmc import tools
    g = np.random.default_rng(seed)
    shapes = [(4, True, 1, 3), (5, True, 7, 2), (8, True, 20, 8), (6, False, 16, 1), (9, True, 33, 3),
              (12, True, 64, 2), (7, True, 20, 5), (10, True, 32, 4), (3, True, 2, 8), (9, True, 64, 5)]
    nbs, R, P = [], [], []
    for L, per, p, r in shapes:
        J = lattice(L, per, g, dist=lambda x: x.normal(), fields=(lambda x: x.normal(0, 0.2)) if L % 2 else None)
        nbs.append(tools.GenerateNeighbors(L * L, J, 5 if L % 2 else 4))
        R.append(r)
        P.append(p)
    import scipy.sparse as sps
    for n, p, r in ((60, 20, 3), (40, 64, 2)):      # rings: two couplings per spin
        J = sps.dok_matrix((n, n))
        for i in range(n):
            J[i, (i + 1) % n] = g.normal()
        nbs.append(tools.GenerateNeighbors(n, J, 2))
        R.append(r)
        P.append(p)
    return nbs, R, P, g


def _single(nbs, R, P, g_spins, sched, T, seed, mcsteps=1, global_moves=0):
    from piqmc import fast
    out = []
    for i, (nb, r, p) in enumerate(zip(nbs, R, P)):
        prob = fast.Problem(nb)
        w = prob.pack(torch.from_numpy(g_spins[i]))
        jp = None if p > 1 else torch.zeros(len(sched), device="cuda")
        fast.anneal(prob, w, sched, p, T, seed=seed + i, mcsteps=mcsteps, global_moves=global_moves, jperp=jp)
        out.append(prob.unpack(w, p).cpu().numpy())
    return out


@pytest.mark.parametrize("tiles", ["heuristic", "mixed", "lane_pairs"])
def test_batch_equals_single(tiles):
    from piqmc import batch
    nbs, R, P, g = _instances()
    spins = [np.where(g.random((r, nb.shape[0], p)) < 0.5, -1, 1).astype(np.int8) for nb, r, p in zip(nbs, R, P)]
    t = None
    if tiles == "mixed":
        t = [(1, 1), (2, 2), (1, 8), (4, 1), (1, 3), (2, 1), (8, 1), (1, 2), (1, 4), (2, 2), (1, 3), (2, 2)]
    elif tiles == "lane_pairs":
        # the 64-slice instances take lane pairs (the others fall back to one lane per site)
        t = [(1, 1, 2), (2, 2, 2), (1, 8, 2), (4, 1, 2), (1, 3, 2), (1, 1, 2), (8, 1, 2), (1, 2, 2), (1, 4, 2),
             (2, 2, 2), (1, 3, 2), (1, 2, 2)]
    B = batch.Batch(nbs, R, P, tiles=t)
    if tiles == "lane_pairs":
        assert [tl[2] for tl in B.tiles] == [2 if p == 64 else 1 for p in P]
    B.set_spins(spins)
    sched = np.linspace(3.0, 1e-8, 9)
    B.anneal(sched, 0.05, seed=11, mcsteps=2, global_moves=1)
    got = [s.cpu().numpy() for s in B.spins()]
    want = _single(nbs, R, P, spins, sched, 0.05, 11, mcsteps=2, global_moves=1)
    for i in range(len(nbs)):
        np.testing.assert_array_equal(got[i], want[i], err_msg="instance %d" % i)


def test_batch_chunks_and_graph_replay():
    from piqmc import batch
    nbs, R, P, g = _instances(1)
    spins = [np.where(g.random((r, nb.shape[0], p)) < 0.5, -1, 1).astype(np.int8) for nb, r, p in zip(nbs, R, P)]
    sched = np.linspace(3.0, 1e-8, 12)
    A = batch.Batch(nbs, R, P)
    A.set_spins(spins)
    A.anneal(sched, 0.05, seed=3)
    A.anneal(sched, 0.05, seed=3)          # two anneals, eager, one launch each
    B = batch.Batch(nbs, R, P)
    B.set_spins(spins)
    B.anneal(sched, 0.05, seed=3, chunk=5, graph=True)   # eager + capture
    B.anneal(sched, 0.05, seed=3, chunk=5, graph=True)   # replay
    for a, b in zip(A.spins(), B.spins()):
        assert torch.equal(a, b)
    EA, EB = A.energies(), B.energies()
    for a, b in zip(EA, EB):
        assert torch.equal(a, b)


def test_batch_equals_the_oracle_directly():
    """Every instance of a batch against the packed sweep's CPU restatement, bit for bit
    (not only through the single-instance kernel): staged items (compile-time P) and per-site
    items (run-time P), P = 1..64."""
    import oracle
    from piqmc import batch, fast
    nbs, R, P, g = _instances(2)
    spins = [np.where(g.random((r, nb.shape[0], p)) < 0.5, -1, 1).astype(np.int8) for nb, r, p in zip(nbs, R, P)]
    B = batch.Batch(nbs, R, P)
    B.set_spins(spins)
    sched = np.linspace(3.0, 1e-8, 7)
    T, seed = 0.05, 21
    B.anneal(sched, T, seed=seed, global_moves=1)
    got = [s.cpu().numpy() for s in B.spins()]
    for i, (nb, r, p) in enumerate(zip(nbs, R, P)):
        prob = fast.Problem(nb, on_device=False)
        jp = oracle.jperp(sched, p, T) if p > 1 else np.zeros(len(sched), np.float32)
        for rr in range(r):
            w = np.zeros(prob.nslots, np.uint64)
            bits = (spins[i][rr] < 0).astype(np.uint64)
            w[prob.perm] = (bits << np.arange(p, dtype=np.uint64)).sum(axis=1, dtype=np.uint64)
            oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w,
                               p, jp, 1, np.float32(1) / np.float32(T), seed + i, replica=rr, global_moves=1)
            want = np.where((w[prob.perm][:, None] >> np.arange(p, dtype=np.uint64)) & np.uint64(1), -1, 1)
            np.testing.assert_array_equal(got[i][rr], want.astype(np.int8), err_msg="instance %d replica %d" % (i, rr))
