"""The drop-in functions in mode='fast' (packed kernel behind the reference's signatures)."""
import numpy as np
import pytest

import oracle
from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def test_quantum_anneal_fast_mode():
    import piqmc.qmc as qmc
    import piqmc.tools as tools
    g = np.random.default_rng(0)
    J = lattice(16, True, g)
    nbs = tools.GenerateNeighbors(256, J, 4)
    P = 20
    confs0 = np.asfortranarray(np.tile(np.where(g.random(256) < 0.5, -1.0, 1.0), (P, 1)).T)
    e0 = np.mean([oracle.classical_energy(confs0[:, k], J) for k in range(P)])
    c1 = confs0.copy(order="F")
    c2 = confs0.copy(order="F")
    sched = np.linspace(3.0, 1e-8, 100)
    qmc.QuantumAnneal(sched, 1, P, 0.05, 256, c1, nbs, np.random.RandomState(4), mode="fast")
    qmc.QuantumAnneal(sched, 1, P, 0.05, 256, c2, nbs, np.random.RandomState(4), mode="fast")
    np.testing.assert_array_equal(c1, c2)                 # seeded from rng: reproducible
    assert set(np.unique(c1)) <= {-1.0, 1.0}
    e1 = np.mean([oracle.classical_energy(c1[:, k], J) for k in range(P)])
    assert e1 < e0 - 100


def test_sa_anneal_fast_mode():
    import piqmc.sa as sa
    import piqmc.tools as tools
    g = np.random.default_rng(1)
    J = lattice(16, True, g, fields=lambda r: r.uniform(-0.5, 0.5))
    nbs = tools.GenerateNeighbors(256, J, 5)
    s = np.where(g.random(256) < 0.5, -1.0, 1.0)
    e0 = oracle.classical_energy(s, J)
    sa.Anneal(np.linspace(5.0, 0.05, 200), 2, s, nbs, np.random.RandomState(2), mode="fast")
    assert set(np.unique(s)) <= {-1.0, 1.0}
    assert oracle.classical_energy(s, J) < e0 - 100
    assert abs(sa.ClassicalIsingEnergy(s, J) - oracle.classical_energy(s, J)) < 1e-9
