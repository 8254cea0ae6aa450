"""The drop-in modules' argument and error behaviour against the compiled reference's (CPU).

Each case makes the same call on the reference's Cython module (oracle/_ref, built by
oracle/build_ref.py; skipped where it is absent) and on ``piqmc``: the exception type (or
the return value), the caller's ``rng`` state afterwards and the in-place arrays must agree.
Only calls that the reference rejects, or finishes without a sweep, are used, so nothing
reaches a GPU.
"""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sps

from pq_testutil import ROOT

sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
pytest.importorskip("piqmc_ref.qmc", reason="compiled reference not built here")
from piqmc_ref import qmc as rqmc, sa as rsa, tools as rtools  # noqa: E402

from piqmc import qmc, sa, tools  # noqa: E402

N, P = 16, 4


def _instance():
    g = np.random.default_rng(9)
    J = sps.dok_matrix((N, N), dtype=np.float64)
    for i in range(N):
        J[i, (i + 1) % N] = g.normal()
        J[i, i] = g.normal(0, 0.2)
    nbs = np.asarray(rtools.GenerateNeighbors(N, J, 4))
    Jd = np.triu(g.normal(0, 1, (N, N)))
    confs = np.asfortranarray(np.where(g.random((N, P)) < 0.5, -1.0, 1.0))
    svec = np.where(g.random(N) < 0.5, -1.0, 1.0)
    return J, nbs, Jd, confs, svec


def _outcome(fn, args):
    rng = np.random.RandomState(5)
    args = [a.copy() if isinstance(a, np.ndarray) else a for a in args]
    args = [rng if a is RNG else a for a in args]
    try:
        r = fn(*args)
        kind = ("returned", r)
    except Exception as exc:  # the type is what is compared
        kind = ("raised", type(exc))
    arrays = [a for a in args if isinstance(a, np.ndarray)]
    return kind, rng.randint(2 ** 31), arrays


RNG = object()  # placeholder for a fresh RandomState(5)


def _cases():
    J, nbs, Jd, confs, svec = _instance()
    sched = np.linspace(3.0, 0.1, 5)
    f32 = lambda a: a.astype(np.float32)  # noqa: E731
    return {
        # QuantumAnneal (reference piqmc/qmc.pyx:30)
        "qa_confs_float32": ("QuantumAnneal", [sched, 1, P, 0.05, N, f32(confs), nbs, RNG]),
        "qa_confs_1d": ("QuantumAnneal", [sched, 1, P, 0.05, N, confs[:, 0].copy(), nbs, RNG]),
        "qa_nbs_2d": ("QuantumAnneal", [sched, 1, P, 0.05, N, confs, nbs[:, :, 0].copy(), RNG]),
        "qa_sched_int": ("QuantumAnneal", [np.arange(5), 1, P, 0.05, N, confs, nbs, RNG]),
        "qa_zero_temp": ("QuantumAnneal", [sched, 1, P, 0.0, N, confs, nbs, RNG]),
        "qa_empty_sched": ("QuantumAnneal", [np.zeros(0), 1, P, 0.05, N, confs, nbs, RNG]),
        "qa_no_spins": ("QuantumAnneal", [sched, 2, P, 0.05, 0, confs, nbs, RNG]),
        "qa_no_spins_empty_sched": ("QuantumAnneal", [np.zeros(0), 2, P, 0.0, 0, confs, nbs, RNG]),
        "qa_mcsteps_str": ("QuantumAnneal", [sched, "1", P, 0.05, N, confs, nbs, RNG]),
        "qa_mcsteps_0": ("QuantumAnneal", [sched, 0, P, 0.05, N, confs, nbs, RNG]),
        "qa_mcsteps_neg": ("QuantumAnneal", [sched, -2, P, 0.05, N, confs, nbs, RNG]),
        "qa_mcsteps_0_zero_temp": ("QuantumAnneal", [sched, 0, P, 0.0, N, confs, nbs, RNG]),
        "qad_mcsteps_neg": ("QuantumAnneal_dense", [sched, -1, P, 0.05, N, confs, Jd, RNG]),
        "sa_mcsteps_neg": ("Anneal", [sched, -3, svec, nbs, RNG]),
        "sad_mcsteps_0": ("Anneal_dense", [sched, 0, svec, Jd, RNG]),
        "sab_mcsteps_neg": ("Anneal_bipartite", [sched, -1, svec[:6].copy(), svec[6:].copy(), Jd[:6, 6:].copy(),
                                                 Jd[0, :6].copy(), Jd[1, 6:].copy(), RNG]),
        "qa_temp_str": ("QuantumAnneal", [sched, 1, P, "hot", N, confs, nbs, RNG]),
        # QuantumAnneal_dense (reference piqmc/qmc.pyx:141)
        "qad_J_float32": ("QuantumAnneal_dense", [sched, 1, P, 0.05, N, confs, f32(Jd), RNG]),
        "qad_J_1d": ("QuantumAnneal_dense", [sched, 1, P, 0.05, N, confs, Jd[0].copy(), RNG]),
        "qad_zero_temp": ("QuantumAnneal_dense", [sched, 1, P, 0.0, N, confs, Jd, RNG]),
        "qad_empty_sched": ("QuantumAnneal_dense", [np.zeros(0), 1, P, 0.05, N, confs, Jd, RNG]),
        "qad_no_spins": ("QuantumAnneal_dense", [sched, 1, P, 0.05, 0, confs, Jd, RNG]),
        # sa.Anneal (reference piqmc/sa.pyx:50) and sa.Anneal_dense (piqmc/sa.pyx:126)
        "sa_svec_float32": ("Anneal", [sched, 1, f32(svec), nbs, RNG]),
        "sa_svec_2d": ("Anneal", [sched, 1, svec[None].copy(), nbs, RNG]),
        "sa_nbs_2d": ("Anneal", [sched, 1, svec, nbs[:, :, 0].copy(), RNG]),
        "sa_empty_sched": ("Anneal", [np.zeros(0), 1, svec, nbs, RNG]),
        "sad_J_float32": ("Anneal_dense", [sched, 1, svec, f32(Jd), RNG]),
        "sad_empty_sched": ("Anneal_dense", [np.zeros(0), 1, svec, Jd, RNG]),
        "sa_no_spins": ("Anneal", [sched, 1, np.zeros(0), nbs, RNG]),
        "sad_no_spins": ("Anneal_dense", [sched, 1, np.zeros(0), Jd, RNG]),
    }


def _module(name, reference):
    if name.startswith("Quantum"):
        return rqmc if reference else qmc
    return rsa if reference else sa


@pytest.mark.parametrize("case", sorted(_cases()))
def test_same_outcome_as_reference(case):
    name, args = _cases()[case]
    want = _outcome(getattr(_module(name, True), name), args)
    got = _outcome(getattr(_module(name, False), name), args)
    assert got[0] == want[0], (case, got[0], want[0])
    assert got[1] == want[1], "rng left in a different state"
    for a, b in zip(got[2], want[2]):
        np.testing.assert_array_equal(a, b)


def test_generate_neighbors_overflow_and_savepath(tmp_path):
    J, _, _, _, _ = _instance()
    for maxnb in (1, 2):
        errs = []
        for mod in (rtools, tools):
            try:
                mod.GenerateNeighbors(N, J, maxnb)
                errs.append(None)
            except Exception as exc:
                errs.append(type(exc))
        assert errs[0] == errs[1] and errs[0] is not None
    want = np.asarray(rtools.GenerateNeighbors(N, J, 4))
    got = np.asarray(tools.GenerateNeighbors(N, J, 4, str(tmp_path / "nbs")))
    np.testing.assert_array_equal(got, want)
