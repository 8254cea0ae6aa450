"""Reference-order CUDA kernels: bit-exact against the compiled reference's golden vectors and the oracle.

The drop-in functions take their spin orders from the caller's RandomState and
their uniforms from this process's libc rand(), exactly like the Cython code,
so after each call the spins, the next libc value and the next rng value must
all equal the reference's.
"""
import numpy as np
import pytest

import oracle
from pq_testutil import dok_from, golden, lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def piqmc():
    import piqmc.qmc  # noqa: F401
    import piqmc.sa  # noqa: F401
    import piqmc
    return piqmc


def test_dropin_qa_8x8_open(piqmc):
    g = golden("qa_8x8_open")
    P = int(g["P"])
    confs = np.asfortranarray(np.tile(g["conf0"], (P, 1)).T)
    oracle.libc_srand(int(g["cseed"]))
    rng = np.random.RandomState(int(g["rseed"]))
    piqmc.qmc.QuantumAnneal(g["sched"], int(g["mcsteps"]), P, float(g["T"]), int(g["n"]), confs, g["nbs"], rng)
    np.testing.assert_array_equal(confs.astype(np.int8), g["final"])
    assert oracle.libc_rand(1)[0] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_dropin_sa_8x8_fields(piqmc):
    g = golden("sa_8x8_fields")
    sv = g["sv0"].copy()
    oracle.libc_srand(int(g["cseed"]))
    rng = np.random.RandomState(int(g["rseed"]))
    piqmc.sa.Anneal(g["sched"], int(g["mcsteps"]), sv, g["nbs"], rng)
    np.testing.assert_array_equal(sv.astype(np.int8), g["final"])
    assert oracle.libc_rand(1)[0] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_dropin_qa_dense_48(piqmc):
    g = golden("qa_dense_48")
    P = int(g["P"])
    confs = np.asfortranarray(np.tile(g["conf0"], (P, 1)).T)
    oracle.libc_srand(int(g["cseed"]))
    rng = np.random.RandomState(int(g["rseed"]))
    piqmc.qmc.QuantumAnneal_dense(g["sched"], int(g["mcsteps"]), P, float(g["T"]), g["J"].shape[0], confs, g["J"], rng)
    np.testing.assert_array_equal(confs.astype(np.int8), g["final"])
    assert oracle.libc_rand(1)[0] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_dropin_sa_dense_48(piqmc):
    g = golden("sa_dense_48")
    sv = g["sv0"].copy()
    oracle.libc_srand(int(g["cseed"]))
    rng = np.random.RandomState(int(g["rseed"]))
    piqmc.sa.Anneal_dense(g["sched"], int(g["mcsteps"]), sv, g["J"], rng)
    np.testing.assert_array_equal(sv.astype(np.int8), g["final"])
    assert oracle.libc_rand(1)[0] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_dropin_sa_bipartite(piqmc):
    g = golden("sa_bipartite")
    lv, rv = g["l0"].copy(), g["r0"].copy()
    oracle.libc_srand(int(g["cseed"]))
    rng = np.random.RandomState(0)
    piqmc.sa.Anneal_bipartite(g["sched"], int(g["mcsteps"]), lv, rv, g["J"], g["lbias"], g["rbias"], rng)
    np.testing.assert_array_equal(lv.astype(np.int8), g["lfinal"])
    np.testing.assert_array_equal(rv.astype(np.int8), g["rfinal"])
    assert oracle.libc_rand(1)[0] == g["next_rand"]


def test_parallel_and_multispin_aliases_run_the_packed_kernel(piqmc):
    """QuantumAnneal_parallel / Anneal_parallel / Anneal_multispin: the packed kernel with a fixed key."""
    from piqmc import tools
    J = tools.Generate2DIsingInstance(8, np.random.RandomState(1))
    nbs = tools.GenerateNeighbors(64, J, 4)
    g = np.random.default_rng(2)
    confs = np.tile(np.where(g.random(64) < 0.5, -1.0, 1.0), (8, 1)).T.copy()
    c2 = confs.copy()
    sched = np.linspace(3.0, 1e-8, 50)
    piqmc.qmc.QuantumAnneal_parallel(sched, 1, 8, 0.05, 64, confs, nbs, 4)
    piqmc.qmc.QuantumAnneal(sched, 1, 8, 0.05, 64, c2, nbs, None, mode="fast", seed=0)
    np.testing.assert_array_equal(confs, c2)
    sv = np.where(g.random(64) < 0.5, -1.0, 1.0)
    sv2 = sv.copy()
    tsched = np.linspace(3.0, 0.05, 40)
    piqmc.sa.Anneal_parallel(tsched, 1, sv, nbs, 8, seed=5)
    piqmc.sa.Anneal(tsched, 1, sv2, nbs, None, mode="fast", seed=5)
    np.testing.assert_array_equal(sv, sv2)
    mat = np.where(g.random((64, 64)) < 0.5, -1.0, 1.0)
    e0 = piqmc.sa.ClassicalIsingEnergy(mat.T, J)
    piqmc.sa.Anneal_multispin(tsched, 2, mat, nbs, np.random.RandomState(4))
    assert set(np.unique(mat)) <= {-1.0, 1.0}
    assert np.all(piqmc.sa.ClassicalIsingEnergy(mat.T, J) <= e0.max()) and np.median(
        piqmc.sa.ClassicalIsingEnergy(mat.T, J)) < np.median(e0)


def test_dense_fast_mode_anneals_like_the_reference_semantics(piqmc):
    """QuantumAnneal_dense(mode='fast') runs the dense fast path in place."""
    g = golden("qa_dense_48")
    J, P = g["J"], int(g["P"])
    confs = np.tile(g["conf0"], (P, 1)).T.copy()
    e0 = piqmc.sa.ClassicalIsingEnergy(confs[:, 0], J)
    piqmc.qmc.QuantumAnneal_dense(np.linspace(3.0, 1e-8, 200), 1, P, 0.05, J.shape[0], confs, J,
                                  np.random.RandomState(1), mode="fast")
    assert set(np.unique(confs)) <= {-1.0, 1.0}
    assert min(piqmc.sa.ClassicalIsingEnergy(confs[:, k], J) for k in range(P)) < e0


def test_dropin_boixo8(piqmc):
    """The reference's own diamond-graph test (testing/test_boixo.py:90-114), bit-exact."""
    g = golden("boixo8")
    rng = np.random.RandomState(123)
    confs = np.tile(np.array([2 * rng.randint(2) - 1 for _ in range(8)], dtype=np.float64), (5, 1)).T
    oracle.libc_srand(1)
    piqmc.qmc.QuantumAnneal(np.linspace(0.5, 1e-8, 10), 3, 5, 0.01, 8, confs, g["nbs"], rng)
    np.testing.assert_array_equal(confs.astype(np.int8), g["final"])
    J = dok_from(g["rows"], g["cols"], g["vals"], 8)
    energies = [piqmc.sa.ClassicalIsingEnergy(confs[:, k], J) for k in range(5)]
    assert np.sum(energies) == -8.0 * 5
    for s, e in zip(g["svecs"], g["energies"]):
        assert piqmc.sa.ClassicalIsingEnergy(s, J) == e


def test_batch_32x32_eight_replicas(piqmc):
    """Eight reference-order replicas in one launch, each with its recorded streams."""
    from piqmc import reforder
    g = golden("qa_32x32_periodic")
    n, P, sched = int(g["n"]), int(g["P"]), g["sched"]
    J = dok_from(g["rows"], g["cols"], g["vals"], n)
    nbs = oracle.generate_neighbors(n, J, 4)
    idx, jv = reforder.split_neighbors(nbs)
    perms, rands, spins, rngs = [], [], [], []
    L = n * P * len(sched) + 1
    for rep in range(8):
        rng = np.random.RandomState(int(g["rseed"][rep]))
        perms.append(oracle.reference_perms(rng, n, len(sched)).astype(np.int32))
        rngs.append(rng)
        rands.append(oracle.libc_stream(int(g["cseed"][rep]), L))
        spins.append(np.tile(g["conf0"][rep], (P, 1)).T.astype(np.int8))
    out, used = reforder.quantum_anneal(np.array(spins), idx, jv, sched, 1, float(g["T"]), np.array(perms),
                                        np.array(rands))
    out = out.cpu().numpy()
    for rep in range(8):
        bits = np.unpackbits(g["final_bits"][rep])[: n * P].reshape(n, P).astype(bool)
        np.testing.assert_array_equal(out[rep] < 0, bits)
        assert rands[rep][used[rep]] == g["next_rand"][rep]
        assert rngs[rep].randint(2 ** 31) == g["next_rng"][rep]


@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_random_cases_vs_oracle(piqmc, flags):
    from piqmc import reforder
    g = np.random.default_rng(flags)
    for L, P, periodic in [(5, 7, True), (6, 4, False), (4, 2, True)]:
        J = lattice(L, periodic, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.5))
        n = L * L
        nbs = oracle.generate_neighbors(n, J, 5)
        idx, jv = reforder.split_neighbors(nbs)
        sched = np.linspace(2.0, 1e-6, 15)
        R = 3
        spins = np.where(g.random((R, n, P)) < 0.5, -1, 1).astype(np.int8)
        perms = np.array([oracle.reference_perms(np.random.RandomState(r), n, 30) for r in range(R)])
        rands = g.integers(0, 2 ** 31 - 1, size=(R, n * P * 30), dtype=np.int64).astype(np.int32)
        out, used = reforder.quantum_anneal(spins, idx, jv, sched, 2, 0.3, perms, rands, flags=flags)
        out = out.cpu().numpy()
        for r in range(R):
            sp = spins[r].copy()
            u = oracle.qa_sparse(sp, nbs, sched, 2, 0.3, perms[r], rands[r], flags=flags)
            np.testing.assert_array_equal(out[r], sp)
            assert used[r] == u


@pytest.mark.parametrize("seed", [0, 1])
def test_random_sa_cases_vs_oracle(piqmc, seed):
    """sa.Anneal's reference-order sweep (several blocks of 32 positions, fields, a hot schedule)."""
    from piqmc import reforder
    g = np.random.default_rng(10 + seed)
    for L, periodic in [(7, True), (5, False), (9, True)]:
        J = lattice(L, periodic, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.5))
        n = L * L
        nbs = oracle.generate_neighbors(n, J, 5)
        idx, jv = reforder.split_neighbors(nbs)
        sched = np.linspace(3.0, 0.2, 12)
        R = 3
        spins = np.where(g.random((R, n)) < 0.5, -1, 1).astype(np.int8)
        perms = np.array([oracle.reference_perms(np.random.RandomState(r), n, 24) for r in range(R)])
        rands = g.integers(0, 2 ** 31 - 1, size=(R, n * 24), dtype=np.int64).astype(np.int32)
        out, used = reforder.anneal(spins, idx, jv, sched, 2, perms, rands)
        out = out.cpu().numpy()
        for r in range(R):
            sp = spins[r].copy()
            u = oracle.sa_sparse(sp, nbs, sched, 2, perms[r], rands[r])
            np.testing.assert_array_equal(out[r], sp)
            assert used[r] == u


def _dense_j(g, n, kind):
    """Upper triangle + diagonal as the reference reads them, junk below (never read)."""
    J = np.triu(g.normal(0, 1, (n, n)), 1) + np.diag(g.normal(0, 0.3, n))
    if kind == "fp32":
        J = J.astype(np.float32).astype(np.float64)
    elif kind == "mixed":   # some rows FP32-valued: updates switch between the FP32 and FP64 chains
        rows = g.random(n) < 0.5
        J[rows] = J[rows].astype(np.float32).astype(np.float64)
    return J + np.tril(g.normal(0, 5, (n, n)), -1)


@pytest.mark.parametrize("kind", ["fp32", "fp64", "mixed"])
@pytest.mark.parametrize("flags", [0, 1, 2, 3])
def test_random_dense_cases_vs_oracle(piqmc, flags, kind):
    """QuantumAnneal_dense in reference order (two warps per replica) against the oracle: every
    Q1/Q2 flag, FP32-valued, general FP64 and mixed J, n across 32-lane chunks, hot and cold."""
    from piqmc import reforder
    g = np.random.default_rng(100 + flags)
    for n, P in [(37, 5), (70, 4), (8, 2)]:
        J = _dense_j(g, n, kind)
        sched = np.linspace(2.0, 1e-6, 6)
        R = 3
        spins = np.where(g.random((R, n, P)) < 0.5, -1, 1).astype(np.int8)
        perms = np.array([oracle.reference_perms(np.random.RandomState(r + 5), n, 12) for r in range(R)])
        rands = g.integers(0, 2 ** 31 - 1, size=(R, n * P * 12), dtype=np.int64).astype(np.int32)
        for T in (0.3, 5.0):
            out, used = reforder.quantum_anneal_dense(spins, J, sched, 2, T, perms, rands, flags=flags)
            out = out.cpu().numpy()
            for r in range(R):
                sp = spins[r].copy()
                u = oracle.qa_dense(sp, J, sched, 2, T, perms[r], rands[r], flags=flags)
                np.testing.assert_array_equal(out[r], sp)
                assert used[r] == u


@pytest.mark.parametrize("kind", ["fp32", "fp64"])
def test_random_sa_dense_cases_vs_oracle(piqmc, kind):
    """sa.Anneal_dense in reference order (two warps per replica) against the oracle."""
    from piqmc import reforder
    g = np.random.default_rng(7)
    for n in (45, 96, 3):
        J = _dense_j(g, n, kind)
        sched = np.linspace(3.0, 0.1, 8)
        R = 3
        spins = np.where(g.random((R, n)) < 0.5, -1, 1).astype(np.int8)
        perms = np.array([oracle.reference_perms(np.random.RandomState(r + 9), n, 16) for r in range(R)])
        rands = g.integers(0, 2 ** 31 - 1, size=(R, n * 16), dtype=np.int64).astype(np.int32)
        out, used = reforder.anneal_dense(spins, J, sched, 2, perms, rands)
        out = out.cpu().numpy()
        for r in range(R):
            sp = spins[r].copy()
            u = oracle.sa_dense(sp, J, sched, 2, perms[r], rands[r])
            np.testing.assert_array_equal(out[r], sp)
            assert used[r] == u


@pytest.mark.parametrize("kind", ["fp32", "fp64"])
def test_random_bipartite_cases_vs_oracle(piqmc, kind):
    """sa.Anneal_bipartite in reference order (one warp per replica) against the oracle:
    FP32-valued weights and biases (FP32 chain) and general FP64 ones, uneven sides."""
    from piqmc import reforder
    g = np.random.default_rng(21)
    for nl, nr in [(37, 70), (70, 5), (1, 33), (40, 40)]:
        J = g.normal(0, 1, (nl, nr))
        lb, rb = g.normal(0, 0.5, nl), g.normal(0, 0.5, nr)
        if kind == "fp32":
            J, lb, rb = (a.astype(np.float32).astype(np.float64) for a in (J, lb, rb))
            lb[:] = np.round(lb * 4) / 4   # terms stay FP32 values: 2J +- b with b on a coarse grid
            rb[:] = np.round(rb * 4) / 4
            J = np.round(J * 64) / 64
        sched = np.linspace(3.0, 0.1, 6)
        R = 3
        spins = np.where(g.random((R, nl + nr)) < 0.5, -1, 1).astype(np.int8)
        rands = g.integers(0, 2 ** 31 - 1, size=(R, (nl + nr) * 12), dtype=np.int64).astype(np.int32)
        out, used = reforder.anneal_bipartite(spins, nl, J, lb, rb, sched, 2, rands)
        out = out.cpu().numpy()
        for r in range(R):
            lv, rv = spins[r, :nl].copy(), spins[r, nl:].copy()
            u = oracle.sa_bipartite(lv, rv, J, lb, rb, sched, 2, rands[r])
            np.testing.assert_array_equal(out[r, :nl], lv)
            np.testing.assert_array_equal(out[r, nl:], rv)
            assert used[r] == u


def test_fp64_accumulator_with_huge_couplings(piqmc):
    """Couplings near FP32's range switch the sweeps to the FP64 accumulator (2J would overflow)."""
    from piqmc import reforder
    g = np.random.default_rng(5)
    J = lattice(6, True, g, dist=lambda r: float(np.float32(r.choice([-1, 1]) * r.uniform(1.0, 1.6) * 2.0 ** 126)))
    n = 36
    nbs = oracle.generate_neighbors(n, J, 4)
    idx, jv = reforder.split_neighbors(nbs)
    assert reforder._acc_flag(jv)
    R, P = 2, 4
    spins = np.where(g.random((R, n, P)) < 0.5, -1, 1).astype(np.int8)
    sched = np.linspace(2.0, 0.5, 6)
    perms = np.array([oracle.reference_perms(np.random.RandomState(r), n, 6) for r in range(R)])
    rands = g.integers(0, 2 ** 31 - 1, size=(R, n * P * 6), dtype=np.int64).astype(np.int32)
    out, used = reforder.quantum_anneal(spins, idx, jv, sched, 1, 1e30, perms, rands, flags=3)
    out = out.cpu().numpy()
    for r in range(R):
        sp = spins[r].copy()
        u = oracle.qa_sparse(sp, nbs, sched, 1, 1e30, perms[r], rands[r], flags=3)
        np.testing.assert_array_equal(out[r], sp)
        assert used[r] == u
    s1 = np.where(g.random((R, n)) < 0.5, -1, 1).astype(np.int8)
    out, used = reforder.anneal(s1, idx, jv, np.linspace(1e30, 1e29, 6), 1, perms, rands[:, : n * 6])
    out = out.cpu().numpy()
    for r in range(R):
        sp = s1[r].copy()
        u = oracle.sa_sparse(sp, nbs, np.linspace(1e30, 1e29, 6), 1, perms[r], rands[r, : n * 6])
        np.testing.assert_array_equal(out[r], sp)
        assert used[r] == u


def test_edge_cases(piqmc):
    g = np.random.default_rng(7)
    J = lattice(4, True, g)
    nbs = oracle.generate_neighbors(16, J, 4)
    confs = np.ones((16, 4))
    rng = np.random.RandomState(0)
    before = rng.get_state()[1].copy()
    # empty schedule: one permutation drawn, nothing else
    piqmc.qmc.QuantumAnneal(np.zeros(0), 1, 4, 0.1, 16, confs, nbs, rng)
    assert np.all(confs == 1)
    # zero temperature: ZeroDivisionError like the reference (slices*temp == 0)
    with pytest.raises(ZeroDivisionError):
        piqmc.qmc.QuantumAnneal(np.ones(3), 1, 4, 0.0, 16, confs, nbs, rng)
    with pytest.raises(ValueError):
        piqmc.qmc.QuantumAnneal(np.ones(3, dtype=np.float32), 1, 4, 0.1, 16, confs, nbs, rng)
    with pytest.raises(ValueError):
        piqmc.qmc.QuantumAnneal(np.ones(3), 1, 4, 0.1, 16, confs[:, 0], nbs, rng)
    bad = nbs.copy()
    bad[3, 1, 0] = 99
    with pytest.raises(ValueError):
        piqmc.qmc.QuantumAnneal(np.ones(3), 1, 4, 0.1, 16, confs, bad, rng)
    with pytest.raises(ValueError):
        piqmc.qmc.QuantumAnneal(np.ones(3), 1, 4, 0.1, 16, confs * 0.5, nbs, rng)
    del before
    # nspins smaller than the rows: the rows beyond nspins are fixed boundary spins
    confs = np.where(g.random((16, 6)) < 0.5, -1.0, 1.0)
    c2 = confs.copy()
    oracle.libc_srand(5)
    piqmc.qmc.QuantumAnneal(np.linspace(1, 0.1, 4), 2, 6, 0.2, 10, confs, nbs, np.random.RandomState(3))
    np.testing.assert_array_equal(confs[10:], c2[10:])
    rands = oracle.libc_stream(5, 10 * 6 * 8 + 1)
    perms = oracle.reference_perms(np.random.RandomState(3), 10, 8)
    # oracle on the full rows with a permutation over the first 10 spins only
    sp = c2.astype(np.int8)
    import piqmc.reforder as rf
    idx, jv = rf.split_neighbors(nbs)
    out, used = rf.quantum_anneal(sp[None], idx, jv, np.linspace(1, 0.1, 4), 2, 0.2, perms[None], rands[None],
                                  nperm=10)
    np.testing.assert_array_equal(out.cpu().numpy()[0], confs.astype(np.int8))
    # and the oracle (checked against the compiled reference for nspins < rows on the CPU)
    so = np.ascontiguousarray(c2.astype(np.int8))
    assert oracle.qa_sparse(so, nbs, np.linspace(1, 0.1, 4), 2, 0.2, perms, rands) == int(used[0])
    np.testing.assert_array_equal(so, confs.astype(np.int8))


def test_single_thread_kernels_beyond_shared_memory(piqmc):
    """Problems too large for the warp kernels' shared memory run the single-thread kernels,
    with the same results as the oracle (sizes just past each warp kernel's limit)."""
    from piqmc import reforder, tools
    g = np.random.default_rng(77)
    # QuantumAnneal_dense, n = 3500, P = 2 (the pair kernel holds n <= ~3470 at P = 2)
    n, P = 3500, 2
    J = np.triu(g.normal(0, 1 / np.sqrt(n), (n, n)), 1) + np.diag(g.normal(0, 0.1, n))
    sched = np.array([1.5])
    spins = np.where(g.random((1, n, P)) < 0.5, -1, 1).astype(np.int8)
    perms = oracle.reference_perms(np.random.RandomState(1), n, 1)[None]
    rands = g.integers(0, 2 ** 31 - 1, size=(1, n * P + 1), dtype=np.int64).astype(np.int32)
    out, used = reforder.quantum_anneal_dense(spins, J, sched, 1, 0.5, perms, rands)
    sp = spins[0].copy()
    assert used[0] == oracle.qa_dense(sp, J, sched, 1, 0.5, perms[0], rands[0])
    np.testing.assert_array_equal(out.cpu().numpy()[0], sp)
    # sa.Anneal_dense, n = 3550
    n = 3550
    J = np.triu(g.normal(0, 1 / np.sqrt(n), (n, n)), 1) + np.diag(g.normal(0, 0.1, n))
    spins = np.where(g.random((1, n)) < 0.5, -1, 1).astype(np.int8)
    perms = oracle.reference_perms(np.random.RandomState(2), n, 1)[None]
    rands = g.integers(0, 2 ** 31 - 1, size=(1, n + 1), dtype=np.int64).astype(np.int32)
    out, used = reforder.anneal_dense(spins, J, np.array([0.7]), 1, perms, rands)
    sp = spins[0].copy()
    assert used[0] == oracle.sa_dense(sp, J, np.array([0.7]), 1, perms[0], rands[0])
    np.testing.assert_array_equal(out.cpu().numpy()[0], sp)
    # QuantumAnneal (sparse), 100 x 100 periodic with fields, P = 21
    L, P = 100, 21
    Js = lattice(L, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.5))
    n = L * L
    nbs = tools.GenerateNeighbors(n, Js, 5)   # (tested against the oracle elsewhere; fast)
    idx, jv = reforder.split_neighbors(nbs)
    sched = np.linspace(2.0, 1.0, 2)
    spins = np.where(g.random((1, n, P)) < 0.5, -1, 1).astype(np.int8)
    perms = oracle.reference_perms(np.random.RandomState(3), n, 2)[None]
    rands = g.integers(0, 2 ** 31 - 1, size=(1, n * P * 2 + 1), dtype=np.int64).astype(np.int32)
    out, used = reforder.quantum_anneal(spins, idx, jv, sched, 1, 0.3, perms, rands)
    sp = spins[0].copy()
    assert used[0] == oracle.qa_sparse(sp, nbs, sched, 1, 0.3, perms[0], rands[0])
    np.testing.assert_array_equal(out.cpu().numpy()[0], sp)
    # sa.Anneal (sparse), 260 x 260 periodic
    L = 260
    Js = lattice(L, True, g, dist=lambda r: r.normal())
    n = L * L
    nbs = tools.GenerateNeighbors(n, Js, 4)
    idx, jv = reforder.split_neighbors(nbs)
    spins = np.where(g.random((1, n)) < 0.5, -1, 1).astype(np.int8)
    perms = oracle.reference_perms(np.random.RandomState(4), n, 1)[None]
    rands = g.integers(0, 2 ** 31 - 1, size=(1, n + 1), dtype=np.int64).astype(np.int32)
    out, used = reforder.anneal(spins, idx, jv, np.array([0.8]), 1, perms, rands)
    sp = spins[0].copy()
    assert used[0] == oracle.sa_sparse(sp, nbs, np.array([0.8]), 1, perms[0], rands[0])
    np.testing.assert_array_equal(out.cpu().numpy()[0], sp)
    # sa.Anneal_bipartite, 5400 + 2 spins
    nl, nr = 5400, 2
    Jb, lb, rb = g.normal(0, 1, (nl, nr)), g.normal(0, 0.5, nl), g.normal(0, 0.5, nr)
    spins = np.where(g.random((1, nl + nr)) < 0.5, -1, 1).astype(np.int8)
    rands = g.integers(0, 2 ** 31 - 1, size=(1, 2 * (nl + nr) + 1), dtype=np.int64).astype(np.int32)
    out, used = reforder.anneal_bipartite(spins, nl, Jb, lb, rb, np.array([2.0, 0.5]), 1, rands)
    lv, rv = spins[0, :nl].copy(), spins[0, nl:].copy()
    assert used[0] == oracle.sa_bipartite(lv, rv, Jb, lb, rb, np.array([2.0, 0.5]), 1, rands[0])
    np.testing.assert_array_equal(out.cpu().numpy()[0, :nl], lv)
    np.testing.assert_array_equal(out.cpu().numpy()[0, nl:], rv)
