"""Generate the golden vectors in this directory from the reference's own compiled code.

Runs the reference's Cython modules as compiled by ``oracle/build_ref.py`` (in
``oracle/_ref``; only where the reference tree is mounted), seeds this process's
libc ``rand()`` with ``srand`` and the reference's ``rng`` with
``np.random.RandomState``, and records inputs, outputs, the next libc value and
the next ``rng`` value after each call (which pins how many of each the call
consumed).  The instances are seeded synthetic ones with the shapes of the
workloads the library is measured on; nothing is read from the reference's
data files.

    python tests/golden/make_golden.py            # every vector
    python tests/golden/make_golden.py boundary   # only qa_boundary_rows.npz
"""
import ctypes
import os
import sys

import numpy as np
import scipy.sparse as sps

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

from piqmc_ref import qmc, sa, tools  # noqa: E402  (the compiled reference)

libc = ctypes.CDLL(None)


def lattice(L, periodic, dist, rng, fields=None):
    n = L * L
    J = sps.dok_matrix((n, n), dtype=np.float64)
    for y in range(L):
        for x in range(L):
            i = y * L + x
            if periodic or x + 1 < L:
                J[i, y * L + (x + 1) % L] = dist(rng)
            if periodic or y + 1 < L:
                J[i, ((y + 1) % L) * L + x] = dist(rng)
    if fields is not None:
        for i in range(n):
            J[i, i] = fields(rng)
    return J


def dok_arrays(J):
    items = list(J.todok().items())
    return (np.array([k[0] for k, _ in items], np.int64), np.array([k[1] for k, _ in items], np.int64),
            np.array([v for _, v in items], np.float64))


def run_qa(J, maxnb, P, T, sched, mcsteps, conf0, cseed, rseed):
    n = J.shape[0]
    nbs = np.asarray(tools.GenerateNeighbors(n, J, maxnb))
    confs = np.asfortranarray(np.tile(conf0, (P, 1)).T.astype(np.float64))
    libc.srand(cseed)
    rng = np.random.RandomState(rseed)
    qmc.QuantumAnneal(sched, mcsteps, P, T, n, confs, nbs, rng)
    return nbs, confs.astype(np.int8), libc.rand(), rng.randint(2 ** 31)


def main():
    out = {}
    g = np.random.default_rng(20150116)
    unif2 = lambda r: r.uniform(-2.0, 2.0)  # noqa: E731
    # 1. 8x8 open lattice, P=20, T=0.05, G 3 -> 1e-8 over 100 steps (the CPU-runnable workload)
    J = lattice(8, False, unif2, g)
    conf0 = np.where(g.random(64) < 0.5, -1.0, 1.0)
    sched = np.linspace(3.0, 1e-8, 100)
    nbs, fin, nr, nn = run_qa(J, 4, 20, 0.05, sched, 1, conf0, 11, 0)
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "qa_8x8_open.npz"), rows=r, cols=c, vals=v, n=64, maxnb=4, P=20,
                        T=0.05, sched=sched, mcsteps=1, conf0=conf0, final=fin, cseed=11, rseed=0,
                        next_rand=nr, next_rng=nn, nbs=nbs)
    # 2. 32x32 periodic, P=20, 1000 steps, 8 reference-order replicas
    J = lattice(32, True, lambda r: float(np.float32(r.uniform(-2.0, 2.0))), g)
    sched = np.linspace(3.0, 1e-8, 1000)
    conf0s, fins, nrs, nns = [], [], [], []
    for rep in range(8):
        conf0 = np.where(g.random(1024) < 0.5, -1.0, 1.0)
        nbs, fin, nr, nn = run_qa(J, 4, 20, 0.05, sched, 1, conf0, 100 + rep, 200 + rep)
        conf0s.append(conf0)
        fins.append(np.packbits(fin < 0, axis=None))
        nrs.append(nr)
        nns.append(nn)
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "qa_32x32_periodic.npz"), rows=r, cols=c, vals=v, n=1024, maxnb=4,
                        P=20, T=0.05, sched=sched, mcsteps=1, conf0=np.array(conf0s), final_bits=np.array(fins),
                        cseed=np.arange(100, 108), rseed=np.arange(200, 208), next_rand=np.array(nrs),
                        next_rng=np.array(nns))
    # 3. sa.Anneal on an 8x8 periodic lattice with fields, 2 sweeps per temperature
    J = lattice(8, True, unif2, g, fields=lambda r: r.uniform(-1.0, 1.0))
    nbs = np.asarray(tools.GenerateNeighbors(64, J, 5))
    sv0 = np.where(g.random(64) < 0.5, -1.0, 1.0)
    sv = sv0.copy()
    tsched = np.linspace(5.0, 0.05, 50)
    libc.srand(21)
    rng = np.random.RandomState(22)
    sa.Anneal(tsched, 2, sv, nbs, rng)
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "sa_8x8_fields.npz"), rows=r, cols=c, vals=v, n=64, maxnb=5,
                        sched=tsched, mcsteps=2, sv0=sv0, final=sv.astype(np.int8), cseed=21, rseed=22,
                        next_rand=libc.rand(), next_rng=rng.randint(2 ** 31), nbs=nbs)
    # 4. QuantumAnneal_dense, N=48, P=8, 20 steps x 2 sweeps
    N = 48
    Jd = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1) + np.diag(g.normal(0.0, np.sqrt(0.1), N))
    conf0 = np.where(g.random(N) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(np.tile(conf0, (8, 1)).T)
    sched = np.linspace(3.0, 1e-8, 20)
    libc.srand(31)
    rng = np.random.RandomState(32)
    qmc.QuantumAnneal_dense(sched, 2, 8, 0.05, N, confs, Jd, rng)
    np.savez_compressed(os.path.join(HERE, "qa_dense_48.npz"), J=Jd, P=8, T=0.05, sched=sched, mcsteps=2,
                        conf0=conf0, final=confs.astype(np.int8), cseed=31, rseed=32, next_rand=libc.rand(),
                        next_rng=rng.randint(2 ** 31))
    # 5. the reference test's 8-spin diamond graph: energies, SA and QA runs
    kvp = [[1, 2, 1.0], [1, 4, 1.0], [1, 5, 1.0], [2, 3, 1.0], [2, 6, 1.0], [3, 4, 1.0], [3, 7, 1.0], [4, 8, 1.0],
           [1, 1, 1.0], [2, 2, 1.0], [3, 3, 1.0], [4, 4, 1.0], [5, 5, -1.0], [6, 6, -1.0], [7, 7, -1.0],
           [8, 8, -1.0]]
    J = sps.dok_matrix((8, 8))
    for i, j, val in kvp:
        J[i - 1, j - 1] = val
    nbs = np.asarray(tools.GenerateNeighbors(8, J, 4, None))
    svecs = np.array([[-1, 1, -1, 1, 1, -1, -1, 1], [1, 1, 1, 1, 1, -1, 1, -1], [1, -1, 1, 1, -1, -1, -1, -1],
                      [1, -1, -1, 1, 1, -1, 1, 1]], dtype=np.float64)
    energies = np.array([sa.ClassicalIsingEnergy(vv, J) for vv in svecs])
    libc.srand(1)
    rng = np.random.RandomState(123)
    conf0 = np.array([2 * rng.randint(2) - 1 for _ in range(8)], dtype=np.float64)
    confs = np.tile(conf0, (5, 1)).T
    qmc.QuantumAnneal(np.linspace(0.5, 1e-8, 10), 3, 5, 0.01, 8, confs, nbs, rng)
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "boixo8.npz"), rows=r, cols=c, vals=v, nbs=nbs, svecs=svecs,
                        energies=energies, conf0=conf0, final=confs.astype(np.int8), next_rand=libc.rand(),
                        next_rng=rng.randint(2 ** 31))
    # 6. the reference test's 5-node neighbour table, in Python 3 DOK order
    J = sps.dok_matrix((5, 5), dtype=np.float64)
    for (i, j) in [(0, 1), (1, 2), (2, 3), (3, 4), (0, 3), (1, 4), (0, 4), (0, 0), (1, 1), (2, 2), (3, 3), (4, 4)]:
        J[i, j] = 1
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "neighbors_5node.npz"), rows=r, cols=c, vals=v,
                        nbs=np.asarray(tools.GenerateNeighbors(5, J, 4)))
    # 7. ClassicalIsingEnergy on a 16x16 periodic N(0,1) lattice with fields, 32 random configurations
    J = lattice(16, True, lambda r: r.normal(), g, fields=lambda r: r.normal(0.0, 0.3))
    S = np.where(g.random((32, 256)) < 0.5, -1.0, 1.0)
    E = np.array([sa.ClassicalIsingEnergy(s, J) for s in S])
    r, c, v = dok_arrays(J)
    np.savez_compressed(os.path.join(HERE, "energy_16x16.npz"), rows=r, cols=c, vals=v, spins=S, energies=E)
    # 8. sa.Anneal_dense, N=48 (upper triangle + fields), 30 temperatures x 2 sweeps
    N = 48
    Jd = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1) + np.diag(g.normal(0.0, np.sqrt(0.1), N))
    sv0 = np.where(g.random(N) < 0.5, -1.0, 1.0)
    sv = sv0.copy()
    tsched = np.linspace(3.0, 0.05, 30)
    libc.srand(41)
    rng = np.random.RandomState(42)
    sa.Anneal_dense(tsched, 2, sv, Jd, rng)
    np.savez_compressed(os.path.join(HERE, "sa_dense_48.npz"), J=Jd, sched=tsched, mcsteps=2, sv0=sv0,
                        final=sv.astype(np.int8), cseed=41, rseed=42, next_rand=libc.rand(),
                        next_rng=rng.randint(2 ** 31))
    # 9. sa.Anneal_bipartite, 12 left x 20 right spins with biases, 25 temperatures x 2 sweeps
    Jb = g.normal(0.0, 0.5, (12, 20))
    lb, rb = g.normal(0.0, 0.2, 12), g.normal(0.0, 0.2, 20)
    l0, r0 = np.where(g.random(12) < 0.5, -1.0, 1.0), np.where(g.random(20) < 0.5, -1.0, 1.0)
    lv, rv = l0.copy(), r0.copy()
    tsched = np.linspace(4.0, 0.1, 25)
    libc.srand(51)
    rng = np.random.RandomState(52)
    sa.Anneal_bipartite(tsched, 2, lv, rv, Jb, lb, rb, rng)
    np.savez_compressed(os.path.join(HERE, "sa_bipartite.npz"), J=Jb, lbias=lb, rbias=rb, sched=tsched, mcsteps=2,
                        l0=l0, r0=r0, lfinal=lv.astype(np.int8), rfinal=rv.astype(np.int8), cseed=51,
                        next_rand=libc.rand(), next_rng=rng.randint(2 ** 31))
    # 10. instance generators: DOK key order, values and the rng state they leave
    gen = {}
    for name, call, seed in [("ising2d_5", lambda rs: tools.Generate2DIsingInstance(5, rs), 61),
                             ("ising2d_2", lambda rs: tools.Generate2DIsingInstance(2, rs), 62),
                             ("lattice_4x5_periodic", lambda rs: tools.Generate2DLattice(4, 5, rs, 1), 63),
                             ("lattice_4x5_open", lambda rs: tools.Generate2DLattice(4, 5, rs, 0), 64),
                             ("kblock_5x6_k2", lambda rs: tools.GenerateKblockLattice(5, 6, rs, 2), 65),
                             ("kblock_4x4_k1", lambda rs: tools.GenerateKblockLattice(4, 4, rs, 1), 66)]:
        rs = np.random.RandomState(seed)
        r, c, v = dok_arrays(call(rs))
        gen[name + "_rows"], gen[name + "_cols"], gen[name + "_vals"] = r, c, v
        gen[name + "_seed"] = seed
        gen[name + "_next_rng"] = rs.randint(2 ** 31)
    np.savez_compressed(os.path.join(HERE, "generators.npz"), **gen)
    print("golden vectors written to", HERE)


def boundary():
    """QuantumAnneal with nspins below the row count: 6x6 periodic lattice, the first 24 spins
    swept, the last 12 rows fixed boundary spins (reference piqmc/qmc.pyx:91)."""
    g = np.random.default_rng(20150117)
    J = lattice(6, True, lambda r: r.normal(), g, fields=lambda r: r.normal(0.0, 0.3))
    nbs = np.asarray(tools.GenerateNeighbors(36, J, 5))
    conf0 = np.where(g.random((36, 5)) < 0.5, -1.0, 1.0)
    confs = np.asfortranarray(conf0.copy())
    sched = np.linspace(2.0, 1e-6, 30)
    libc.srand(71)
    rng = np.random.RandomState(72)
    qmc.QuantumAnneal(sched, 2, 5, 0.2, 24, confs, nbs, rng)
    np.savez_compressed(os.path.join(HERE, "qa_boundary_rows.npz"), nbs=nbs, nspins=24, P=5, T=0.2, sched=sched,
                        mcsteps=2, conf0=conf0, final=confs.astype(np.int8), cseed=71, rseed=72,
                        next_rand=libc.rand(), next_rng=rng.randint(2 ** 31))
    print("boundary-row vector written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:] == ["boundary"]:
        boundary()
    else:
        main()
        boundary()
