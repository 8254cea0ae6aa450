"""The CPU oracle against the golden vectors recorded from the compiled reference.

Each golden case was produced by the reference's own Cython code with a seeded
libc rand() and numpy RandomState (tests/golden/make_golden.py).  The oracle
gets the same streams, rebuilt here: it must give the same final spins and
consume exactly as many libc values (the recorded next rand() value sits at the
consumed count) and permutations (the recorded next rng value follows).
"""
import numpy as np
import pytest

import oracle
from pq_testutil import dok_from, golden


def _qa_case(g, conf0, cseed, rseed, final):
    nbs = g["nbs"] if "nbs" in g else oracle.generate_neighbors(int(g["n"]), dok_from(g["rows"], g["cols"], g["vals"], g["n"]), int(g["maxnb"]))
    n, P = int(g["n"]), int(g["P"])
    sched, mcsteps, T = g["sched"], int(g["mcsteps"]), float(g["T"])
    rng = np.random.RandomState(int(rseed))
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(int(cseed), n * P * len(sched) * mcsteps + 1)
    sp = np.ascontiguousarray(np.tile(conf0, (P, 1)).T.astype(np.int8))
    used = oracle.qa_sparse(sp, nbs, sched, mcsteps, T, perms, rands)
    return sp, used, rands, rng


def test_qa_8x8_open():
    g = golden("qa_8x8_open")
    sp, used, rands, rng = _qa_case(g, g["conf0"], g["cseed"], g["rseed"], g["final"])
    np.testing.assert_array_equal(sp, g["final"])
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


@pytest.mark.parametrize("rep", range(8))
def test_qa_32x32_periodic(rep):
    g = golden("qa_32x32_periodic")
    sp, used, rands, rng = _qa_case(g, g["conf0"][rep], g["cseed"][rep], g["rseed"][rep], None)
    bits = np.unpackbits(g["final_bits"][rep])[: sp.size].reshape(sp.shape)
    np.testing.assert_array_equal(sp < 0, bits.astype(bool))
    assert rands[used] == g["next_rand"][rep]
    assert rng.randint(2 ** 31) == g["next_rng"][rep]


def test_sa_8x8_fields():
    g = golden("sa_8x8_fields")
    n, mcsteps, sched = int(g["n"]), int(g["mcsteps"]), g["sched"]
    rng = np.random.RandomState(int(g["rseed"]))
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(int(g["cseed"]), n * len(sched) * mcsteps + 1)
    s = g["sv0"].astype(np.int8).copy()
    used = oracle.sa_sparse(s, g["nbs"], sched, mcsteps, perms, rands)
    np.testing.assert_array_equal(s, g["final"])
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_qa_dense_48():
    g = golden("qa_dense_48")
    J, P, sched, mcsteps, T = g["J"], int(g["P"]), g["sched"], int(g["mcsteps"]), float(g["T"])
    n = J.shape[0]
    rng = np.random.RandomState(int(g["rseed"]))
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(int(g["cseed"]), n * P * len(sched) * mcsteps + 1)
    sp = np.ascontiguousarray(np.tile(g["conf0"], (P, 1)).T.astype(np.int8))
    used = oracle.qa_dense(sp, J, sched, mcsteps, T, perms, rands)
    np.testing.assert_array_equal(sp, g["final"])
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_sa_dense_48():
    g = golden("sa_dense_48")
    J, sched, mcsteps = g["J"], g["sched"], int(g["mcsteps"])
    n = J.shape[0]
    rng = np.random.RandomState(int(g["rseed"]))
    perms = oracle.reference_perms(rng, n, len(sched) * mcsteps)
    rands = oracle.libc_stream(int(g["cseed"]), n * len(sched) * mcsteps + 1)
    s = g["sv0"].astype(np.int8).copy()
    used = oracle.sa_dense(s, J, sched, mcsteps, perms, rands)
    np.testing.assert_array_equal(s, g["final"])
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_sa_bipartite():
    g = golden("sa_bipartite")
    sched, mcsteps = g["sched"], int(g["mcsteps"])
    lv, rv = g["l0"].astype(np.int8).copy(), g["r0"].astype(np.int8).copy()
    rands = oracle.libc_stream(int(g["cseed"]), (lv.size + rv.size) * len(sched) * mcsteps + 1)
    used = oracle.sa_bipartite(lv, rv, g["J"], g["lbias"], g["rbias"], sched, mcsteps, rands)
    np.testing.assert_array_equal(lv, g["lfinal"])
    np.testing.assert_array_equal(rv, g["rfinal"])
    assert rands[used] == g["next_rand"]


def test_boixo8_qa_and_energies():
    g = golden("boixo8")
    J = dok_from(g["rows"], g["cols"], g["vals"], 8)
    for s, e in zip(g["svecs"], g["energies"]):
        assert oracle.classical_energy(s, J) == e
    np.testing.assert_array_equal(g["energies"], [4.0, -8.0, -4.0, 0.0])
    rng = np.random.RandomState(123)
    conf0 = np.array([2 * rng.randint(2) - 1 for _ in range(8)], dtype=np.float64)
    np.testing.assert_array_equal(conf0, g["conf0"])
    sched = np.linspace(0.5, 1e-8, 10)
    perms = oracle.reference_perms(rng, 8, 30)
    rands = oracle.libc_stream(1, 8 * 5 * 30 + 1)
    sp = np.ascontiguousarray(np.tile(conf0, (5, 1)).T.astype(np.int8))
    used = oracle.qa_sparse(sp, g["nbs"], sched, 3, 0.01, perms, rands)
    np.testing.assert_array_equal(sp, g["final"])
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]


def test_neighbors_5node():
    g = golden("neighbors_5node")
    J = dok_from(g["rows"], g["cols"], g["vals"], 5)
    np.testing.assert_array_equal(oracle.generate_neighbors(5, J, 4), g["nbs"])


def test_energy_16x16():
    g = golden("energy_16x16")
    J = dok_from(g["rows"], g["cols"], g["vals"], 256)
    for s, e in zip(g["spins"], g["energies"]):
        assert abs(oracle.classical_energy(s, J) - e) <= 1e-12 * max(1.0, abs(e))


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of its authors' reference distribution (Random123)."""
    kat = [([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
           ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
           ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
            [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1])]
    for ctr, key, want in kat:
        np.testing.assert_array_equal(oracle.philox4x32_10(ctr, key), np.array(want, dtype=np.uint32))


def test_expf_accuracy():
    xs = np.concatenate([np.linspace(-87.0, 0.0, 20001), -np.logspace(-8, 1.9, 2001)]).astype(np.float32)
    got = np.array([oracle.expf_neg(x) for x in xs], dtype=np.float64)
    rel = np.abs(got / np.exp(xs.astype(np.float64)) - 1.0)
    assert rel.max() < 2.5e-7   # within ~2 FP32 ulps
    assert oracle.expf_neg(-87.5) == 0.0 and oracle.expf_neg(0.0) == 1.0


def test_expf_error_bound_sampled():
    """The bound the reference-order FP32 fast path relies on (max relative error < 1e-7;
    the full exhaustive scan over all 1.1e9 inputs gives 7.9e-8)."""
    import ctypes
    L = oracle.lib()
    L.orc_expf_max_relerr.argtypes = [ctypes.c_uint32] * 3
    L.orc_expf_max_relerr.restype = ctypes.c_double
    hi = int(np.array([-87.0], np.float32).view(np.uint32)[0])
    assert L.orc_expf_max_relerr(0x80000000, hi, 101) < 1e-7


def test_qa_boundary_rows():
    """nspins below the row count: the oracle sweeps the listed spins only and leaves the
    boundary rows as they were, like the reference."""
    g = golden("qa_boundary_rows")
    nspins, P, sched, mcsteps, T = int(g["nspins"]), int(g["P"]), g["sched"], int(g["mcsteps"]), float(g["T"])
    rng = np.random.RandomState(int(g["rseed"]))
    perms = oracle.reference_perms(rng, nspins, len(sched) * mcsteps)
    rands = oracle.libc_stream(int(g["cseed"]), nspins * P * len(sched) * mcsteps + 1)
    sp = np.ascontiguousarray(g["conf0"].astype(np.int8))
    used = oracle.qa_sparse(sp, g["nbs"], sched, mcsteps, T, perms, rands)
    np.testing.assert_array_equal(sp, g["final"])
    np.testing.assert_array_equal(sp[nspins:], g["conf0"][nspins:].astype(np.int8))
    assert (sp[:nspins] != g["conf0"][:nspins]).any()
    assert rands[used] == g["next_rand"]
    assert rng.randint(2 ** 31) == g["next_rng"]
