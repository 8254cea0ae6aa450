"""Instance generators on the GPU against the host drop-ins' structure.

tools.lattice_table writes the neighbour table of Generate2DIsingInstance,
Generate2DLattice or GenerateKblockLattice (reference piqmc/tools.pyx:98-273) in
device memory.  Its values come from a seeded counter-based stream, not the
caller's MT19937, so the check is structural: every row lists exactly the
neighbours, in exactly the order, that GenerateNeighbors builds from the host
generator's keys (which are bit-exact with the reference's, tests/test_host.py);
each coupling is the same from both ends and inside its range.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = ([("ising2d", r, r, 0, 1) for r in (1, 2, 3, 5, 8, 13)]
         + [("lattice2d", r, c, p, 1) for (r, c) in [(1, 1), (1, 5), (5, 1), (2, 2), (3, 7), (6, 4)] for p in (0, 1)]
         + [("kblock", r, c, 0, k) for (r, c, k) in [(5, 5, 1), (6, 4, 2), (7, 9, 3), (3, 3, 2), (1, 6, 2), (8, 8, 1),
                                                      (2, 7, 3)]])


def _host(kind, r, c, p, k):
    from piqmc import tools
    rng = np.random.RandomState(0)
    if kind == "ising2d":
        return tools.Generate2DIsingInstance(r, rng), (-2.0, 2.0)
    if kind == "lattice2d":
        return tools.Generate2DLattice(r, c, rng, periodic=p), (-1e-8, 1e-8)
    return tools.GenerateKblockLattice(r, c, rng, k=k), (-1e-8, 1e-8)


@pytest.mark.parametrize("kind,r,c,p,k", CASES)
def test_gpu_table_has_the_host_structure(kind, r, c, p, k):
    from piqmc import tools
    J, (lo, hi) = _host(kind, r, c, p, k)
    n = r * c
    rows = [[] for _ in range(n)]
    for (a, b) in J.keys():
        rows[a].append(b)
        if b != a:
            rows[b].append(a)
    maxnb = max(1, max(len(x) for x in rows))
    nbs = tools.lattice_table(kind, r, c, seed=5, periodic=p, k=k, maxnb=maxnb).cpu().numpy()
    val = {}
    for j in range(n):
        m = len(rows[j])
        np.testing.assert_array_equal(nbs[j, :m, 0], rows[j], err_msg="row %d" % j)
        assert (nbs[j, m:] == 0).all()
        for o, v in zip(nbs[j, :m, 0].astype(int), nbs[j, :m, 1]):
            assert lo <= v < hi
            key = (min(j, o), max(j, o))
            assert val.setdefault(key, v) == v          # the same value from both ends
    assert len(val) == len(J.keys())


def test_gpu_table_rejects_a_short_row():
    from piqmc import tools
    with pytest.raises(IndexError):
        tools.lattice_table("kblock", 6, 6, k=2, maxnb=10)


def test_generated_table_anneals():
    """An 80x80 torus generated on the GPU goes straight into the packed sweep."""
    import torch
    from piqmc import fast, tools
    nbs = tools.Generate2DIsingInstanceTable(80, seed=3).cpu().numpy()
    prob = fast.Problem(nbs)
    spins = np.repeat(np.where(np.random.default_rng(0).random((8, 6400)) < 0.5, -1, 1).astype(np.int8)[:, :, None],
                      20, axis=2)
    w = prob.pack(torch.from_numpy(spins))
    E0 = prob.energies(w, 20).cpu().numpy().mean()
    fast.anneal(prob, w, np.linspace(3.0, 1e-8, 50), 20, 0.05, seed=1)
    E1 = prob.energies(w, 20).cpu().numpy().mean()
    assert E1 < E0 - 0.5 * 6400
