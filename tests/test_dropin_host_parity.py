"""The host-side drop-ins against the compiled reference on random inputs (CPU; skipped
where oracle/_ref is not built): ``GenerateNeighbors`` (the C library's one-pass table),
the three instance generators, ``bits2spins`` / ``spins2bits``."""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sps

from pq_testutil import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
pytest.importorskip("piqmc_ref.tools", reason="compiled reference not built here")
from piqmc_ref import tools as rtools  # noqa: E402

from piqmc import tools  # noqa: E402


def _random_dok(g, n):
    """Keys inserted in random order, upper and lower triangle, diagonal, some overwritten."""
    J = sps.dok_matrix((n, n), dtype=np.float64)
    for _ in range(int(g.integers(0, 4 * n + 1))):
        i, j = (int(v) for v in g.integers(0, n, 2))
        J[i, j] = g.normal() if g.random() < 0.9 else float(g.integers(-3, 4))
    return J


def _outcome(mod, n, J, maxnb):
    try:
        return np.asarray(mod.GenerateNeighbors(n, J, maxnb)), None
    except Exception as exc:
        return None, type(exc)


@pytest.mark.parametrize("seed", range(40))
def test_generate_neighbors_random(seed):
    g = np.random.default_rng(seed)
    n = int(g.integers(1, 30))
    J = _random_dok(g, n)
    need = 1
    for i in range(n):
        keys = [k for k in J.keys() if i in k]
        need = max(need, len(keys))
    for maxnb in (need, need + 2, max(1, need - 1)):
        want, werr = _outcome(rtools, n, J, maxnb)
        got, gerr = _outcome(tools, n, J, maxnb)
        assert werr == gerr, (maxnb, werr, gerr)
        if want is not None:
            np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("seed", range(12))
def test_instance_generators_random(seed):
    g = np.random.default_rng(100 + seed)
    rows, cols = int(g.integers(2, 9)), int(g.integers(2, 9))
    calls = [("Generate2DIsingInstance", (int(g.integers(2, 8)),)),
             ("Generate2DLattice", (rows, cols, "rng", int(seed % 2))),
             ("GenerateKblockLattice", (rows, cols, "rng", int(g.integers(1, 4))))]
    for name, args in calls:
        res = []
        for mod in (rtools, tools):
            rs = np.random.RandomState(1000 + seed)
            a = [rs if x == "rng" else x for x in args]
            if name == "Generate2DIsingInstance":
                a = [a[0], rs]
            J = getattr(mod, name)(*a)
            items = list(J.todok().items())
            res.append((items, J.shape, rs.randint(2 ** 31)))
        assert res[0][1] == res[1][1], name
        assert [k for k, _ in res[0][0]] == [k for k, _ in res[1][0]], name + ": key order"
        assert [v for _, v in res[0][0]] == [v for _, v in res[1][0]], name + ": values"
        assert res[0][2] == res[1][2], name + ": rng state"


def test_bits_and_spins_random():
    g = np.random.default_rng(7)
    for _ in range(20):
        bits = list(g.integers(0, 2, int(g.integers(0, 70))))
        assert tools.bits2spins(bits) == list(rtools.bits2spins(bits))
        spins = [int(v) for v in np.where(g.random(len(bits)) < 0.5, -1, 1)]
        assert tools.spins2bits(spins) == list(rtools.spins2bits(spins))
