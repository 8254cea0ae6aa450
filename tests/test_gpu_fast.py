"""Packed fast kernel: bit-exact against its CPU restatement, and the FP64 energy pass against FP64 NumPy."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def _words_u64(words):
    w = words.cpu().numpy()
    return (w.view(np.uint32).astype(np.uint64) if w.dtype == np.int32 else w.view(np.uint64)).copy()


def _run_both(prob, P, R, sched, T, mcsteps, seed, global_moves=0, order_mode=1, betas=None, sweep_base=0,
              replica_base=0, threads=0, rpc=0, rng=None):
    from piqmc import fast
    rng = rng or np.random.default_rng(seed)
    spins = np.where(rng.random((R, prob.n, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    w0 = _words_u64(words)
    if P > 1:
        jp = oracle.jperp(sched, P, T)
    else:
        jp = np.zeros(len(sched), np.float32)
    bt = None if betas is None else torch.from_numpy(betas).cuda()
    acc = torch.zeros(1, dtype=torch.int64, device="cuda")
    fast.anneal(prob, words, sched, P, T, mcsteps=mcsteps, seed=seed, global_moves=global_moves,
                order_mode=order_mode, betas=bt, sweep_base=sweep_base, replica_base=replica_base,
                threads=threads, replicas_per_cta=rpc, accepts=acc,
                jperp=torch.from_numpy(jp).cuda())
    got = _words_u64(words)
    tot = 0
    for r in range(R):
        w = w0[r].copy()
        tot += oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size,
                                  prob.class_stride, w, P, jp, mcsteps, np.float32(1.0) / np.float32(T), seed,
                                  sweep_base=sweep_base, replica=replica_base + r, global_moves=global_moves,
                                  betas=betas, order_mode=order_mode)
        np.testing.assert_array_equal(got[r], w, err_msg="replica %d" % r)
    assert int(acc.item()) == tot
    return prob, words


@pytest.mark.parametrize("P", [1, 2, 3, 7, 20, 32, 33, 64])
def test_fast_bit_exact_P(P):
    from piqmc import fast, tools
    g = np.random.default_rng(P)
    J = lattice(6, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.3))
    prob = fast.Problem(tools.GenerateNeighbors(36, J, 5))
    _run_both(prob, P, 3, np.linspace(3.0, 1e-8, 12), 0.05 if P > 1 else 0.5, 1, seed=1000 + P)


@pytest.mark.parametrize("order_mode,global_moves,mcsteps", [(0, 0, 1), (1, 1, 1), (1, 2, 3), (0, 1, 2)])
def test_fast_bit_exact_modes(order_mode, global_moves, mcsteps):
    from piqmc import fast, tools
    g = np.random.default_rng(11)
    J = lattice(7, True, g, dist=lambda r: r.uniform(-2, 2))   # odd periodic: not bipartite
    prob = fast.Problem(tools.GenerateNeighbors(49, J, 4))
    assert prob.ncolors >= 3
    _run_both(prob, 20, 5, np.linspace(3.0, 1e-8, 10), 0.05, mcsteps, seed=77, global_moves=global_moves,
              order_mode=order_mode, sweep_base=123, replica_base=9)


@pytest.mark.parametrize("threads,rpc", [(32, 1), (64, 2), (128, 4), (256, 0), (96, 3)])
def test_fast_launch_shapes_do_not_change_results(threads, rpc):
    from piqmc import fast, tools
    g = np.random.default_rng(5)
    J = lattice(8, True, g)
    prob = fast.Problem(tools.GenerateNeighbors(64, J, 4))
    _run_both(prob, 16, 7, np.linspace(3.0, 1e-8, 8), 0.05, 1, seed=3, threads=threads, rpc=rpc)


_UP_DOWN = np.concatenate([np.linspace(3.0, 0.2, 14), np.linspace(0.3, 1.5, 6), np.linspace(1.5, 1e-8, 20)])


@pytest.mark.parametrize("P,sched,mcsteps,global_moves,threads,rpc", [
    (20, np.linspace(3.0, 1e-8, 40), 1, 0, 32, 1),
    (20, np.linspace(3.0, 1e-8, 40), 1, 0, 64, 2),
    (16, np.linspace(3.0, 1e-8, 40), 2, 1, 32, 1),
    (32, _UP_DOWN, 1, 0, 32, 1),
    (20, _UP_DOWN, 2, 1, 64, 2),
    (64, np.linspace(3.0, 1e-8, 30), 1, 1, 64, 2),
])
def test_fast_staged_phases_bit_exact(P, sched, mcsteps, global_moves, threads, rpc):
    """Staged phases (scan, then visits of the queued sites) on a lattice large enough
    for them, long enough that most sites are quiet (skipped: both slice classes
    certain to reject) in the later sweeps.  A schedule whose J-perp goes down and up
    again makes the kernel rewrite every quiet bit; world-line moves clear the bits
    around a flipped world-line."""
    from piqmc import fast, tools
    g = np.random.default_rng(P + len(sched))
    J = lattice(32, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.2))
    prob = fast.Problem(tools.GenerateNeighbors(1024, J, 5))
    assert prob.maxdeg == 4     # four couplings, P in {16, 20, 32, 64}: the compile-time (staged) variants
    _run_both(prob, P, 4, sched, 0.05, mcsteps, seed=31 + P, global_moves=global_moves, threads=threads, rpc=rpc)


def _graph(kind, g):
    """Coupling graphs of other degrees: a ring, random graphs, a periodic King's graph (8)."""
    import scipy.sparse as sps
    if kind == "ring":
        n = 300
        J = sps.dok_matrix((n, n))
        for i in range(n):
            J[i, (i + 1) % n] = g.normal()
    elif kind.startswith("random"):
        dmax = int(kind[6:])
        n = 400
        J = sps.dok_matrix((n, n))
        deg = np.zeros(n, int)
        for _ in range(n * dmax // 2):
            a, b = sorted(g.choice(n - 1, 2, replace=False))     # spin n - 1 stays isolated
            if deg[a] < dmax and deg[b] < dmax and (a, b) not in J:
                J[int(a), int(b)] = g.normal()
                deg[a] += 1
                deg[b] += 1
    else:   # King's graph, 20 x 20 torus
        L = 20
        n = L * L
        J = sps.dok_matrix((n, n))
        for y in range(L):
            for x in range(L):
                i = y * L + x
                for dx, dy in ((1, 0), (0, 1), (1, 1), (1, -1)):
                    j = ((y + dy) % L) * L + (x + dx) % L
                    a, b = min(i, j), max(i, j)
                    J[a, b] = g.normal()
    for i in range(n):                                  # fields, a third of them zero
        if g.random() < 2 / 3:
            J[i, i] = g.normal(0, 0.3)
    return J


@pytest.mark.parametrize("kind,P", [("ring", 20), ("random3", 16), ("random6", 20), ("random6", 64),
                                    ("random8", 32), ("kings", 20), ("kings", 64)])
def test_fast_staged_phases_other_degrees(kind, P):
    """Degrees up to four take the four-coupling variants, five to eight the eight-coupling
    ones: the padded terms add +0, which changes no decision (an isolated spin with no field
    has a zero energy sum)."""
    from piqmc import fast, tools
    g = np.random.default_rng(len(kind) * 100 + P)
    J = _graph(kind, g)
    n = J.shape[0]
    prob = fast.Problem(tools.GenerateNeighbors(n, J, 9))
    assert prob.maxdeg <= 8
    _run_both(prob, P, 3, np.linspace(3.0, 1e-8, 30), 0.05, 1, seed=P + n, global_moves=1, threads=64, rpc=1)


def test_benchmark_workload_bit_exact_at_full_length():
    """The benchmark's own workload -- its seeded 80 x 80 instance, straight starts, key and
    the whole 2000-step schedule, P = 20, 1024 replicas in one launch -- equals the
    oracle bit for bit on the first and the last replica (about 15 s of oracle each)."""
    import bench
    from piqmc import fast, tools
    import scipy.sparse as sps
    n, P, R = bench.L_SIDE * bench.L_SIDE, bench.P_SLICES, bench.REPLICAS
    rows, cols, vals = bench.instance_arrays()
    J = sps.dok_matrix((n, n))
    for a, b, v in zip(rows, cols, vals):
        J[int(a), int(b)] = v
    prob = fast.Problem(tools.GenerateNeighbors(n, J, 4))
    sched = bench.schedule(bench.NSCHED)
    jp = fast.jperp_schedule(sched, P, bench.TEMP)
    spins = np.ascontiguousarray(np.repeat(bench.initial_spins(0, R, n)[:, :, None], P, axis=2))
    words = prob.pack(torch.from_numpy(spins))
    w0 = _words_u64(words)
    seed = bench.BENCH_SEED
    fast.anneal(prob, words, sched, P, bench.TEMP, seed=seed, jperp=torch.from_numpy(jp).cuda())
    got = _words_u64(words)
    for r in (0, R - 1):
        w = w0[r].copy()
        oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w, P,
                           jp, 1, np.float32(1.0) / np.float32(bench.TEMP), seed, replica=r)
        np.testing.assert_array_equal(got[r], w, err_msg="replica %d" % r)


def test_fast_staged_phases_in_chunks():
    """A 220 x 220 lattice with 128-thread CTAs: a queue that holds a whole phase would pass
    the shared-memory budget, so the scan goes through each phase in chunks of words the
    smaller queue holds (about twelve per phase), each scanned and then visited."""
    from piqmc import fast, tools
    g = np.random.default_rng(220)
    L = 220
    J = lattice(L, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.2))
    prob = fast.Problem(tools.GenerateNeighbors(L * L, J, 5))
    assert prob.maxdeg == 4
    words_kb = prob.nslots * 4 / 1024
    assert words_kb + ((prob.class_stride + 31) // 32 + 1) * 32 * 4 / 1024 > 200 > words_kb + 2   # chunked
    _run_both(prob, 16, 2, np.linspace(3.0, 1e-8, 6), 0.05, 1, seed=220, threads=128, rpc=1)


def test_fast_staged_phases_with_rising_temperature():
    """Per-step betas that fall mid-schedule: quiet bits are rewritten at that step."""
    from piqmc import fast, tools
    g = np.random.default_rng(12)
    J = lattice(32, True, g, dist=lambda r: r.normal())
    prob = fast.Problem(tools.GenerateNeighbors(1024, J, 4))
    temps = np.concatenate([np.linspace(0.5, 0.02, 15), np.full(5, 0.3), np.linspace(0.3, 0.02, 15)])
    betas = (np.float32(1.0) / temps.astype(np.float32)).astype(np.float32)
    _run_both(prob, 20, 3, np.linspace(2.0, 1e-8, len(temps)), 0.05, 1, seed=6, betas=betas, threads=32, rpc=1)


def test_fast_classical_p1_temperature_down_up_down():
    """P = 1 (the packed classical annealer; per-site phases: staged ones with quiet sites
    measured slower for its single cheap decision per site, 763 against 582 ms on 80 x 80
    with 4096 replicas): a 32 x 32 lattice, temperature down, up and down again,
    world-line moves."""
    from piqmc import fast, tools
    g = np.random.default_rng(41)
    J = lattice(32, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.2))
    prob = fast.Problem(tools.GenerateNeighbors(1024, J, 5))
    temps = np.concatenate([np.linspace(3.0, 0.1, 40), np.full(5, 1.0), np.linspace(1.0, 0.05, 35)])
    betas = (np.float32(1.0) / temps.astype(np.float32)).astype(np.float32)
    _run_both(prob, 1, 4, np.zeros(len(temps)), 1.0, 1, seed=41, betas=betas, global_moves=1, threads=64, rpc=1)


def test_fast_sa_betas():
    """P = 1 with a per-step inverse temperature: the packed classical annealer."""
    from piqmc import fast, tools
    g = np.random.default_rng(8)
    J = lattice(8, True, g, fields=lambda r: r.uniform(-1, 1))
    prob = fast.Problem(tools.GenerateNeighbors(64, J, 5))
    temps = np.linspace(5.0, 0.05, 20).astype(np.float32)
    _run_both(prob, 1, 4, np.zeros(20), 1.0, 2, seed=5, betas=(np.float32(1.0) / temps).astype(np.float32))


def test_split_calls_equal_one_call():
    """sweep_base makes an anneal split over calls draw the same numbers as one call."""
    from piqmc import fast, tools
    g = np.random.default_rng(9)
    J = lattice(8, True, g)
    prob = fast.Problem(tools.GenerateNeighbors(64, J, 4))
    sched = np.linspace(3.0, 1e-8, 20)
    spins = torch.from_numpy(np.where(g.random((4, 64, 20)) < 0.5, -1, 1).astype(np.int8))
    a = prob.pack(spins)
    b = a.clone()
    fast.anneal(prob, a, sched, 20, 0.05, seed=4)
    jp = torch.from_numpy(oracle.jperp(sched, 20, 0.05)).cuda()
    fast.anneal(prob, b, sched[:7], 20, 0.05, seed=4, jperp=jp[:7])
    fast.anneal(prob, b, sched[7:], 20, 0.05, seed=4, jperp=jp[7:], sweep_base=7)
    assert torch.equal(a, b)


def test_energy_pass_vs_fp64_numpy():
    from piqmc import fast, tools
    g = np.random.default_rng(10)
    J = lattice(12, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.3))
    prob = fast.Problem(tools.GenerateNeighbors(144, J, 5))
    P, R = 20, 6
    spins = np.where(g.random((R, 144, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    E = prob.energies(words, P).cpu().numpy()
    back = prob.unpack(words, P).cpu().numpy()
    np.testing.assert_array_equal(back, spins)
    for r in range(R):
        for k in range(P):
            ref = oracle.classical_energy(spins[r, :, k].astype(np.float64), J)
            assert abs(E[r, k] - ref) <= 1e-12 * max(1.0, abs(ref))


def test_classical_ising_energy_dropin():
    import piqmc.sa as sa
    from pq_testutil import dok_from, golden
    g = golden("energy_16x16")
    J = dok_from(g["rows"], g["cols"], g["vals"], 256)
    got = sa.ClassicalIsingEnergy(g["spins"].T, J)
    np.testing.assert_allclose(got, g["energies"], rtol=1e-13, atol=1e-12)
    assert sa.ClassicalIsingEnergy(g["spins"][0], J) == pytest.approx(g["energies"][0], rel=1e-13)


@pytest.mark.parametrize("P", [1, 7, 20, 33, 64])
@pytest.mark.parametrize("offset", [0, 1, 16])
def test_pack_unpack_round_trip_any_alignment(P, offset):
    """pq_pack_spins / pq_unpack_spins on buffers at any byte offset, with a partial last block."""
    from piqmc import _device, _native
    g = np.random.default_rng(P * 10 + offset)
    R, n = 3, 301                                    # 903 items: not a multiple of the block size
    spins = np.where(g.random((R, n, P)) < 0.5, -1, 1).astype(np.int8)
    buf = torch.zeros(R * n * P + 32, dtype=torch.int8, device="cuda")
    buf[offset:offset + R * n * P] = torch.from_numpy(spins.ravel()).cuda()
    perm = torch.from_numpy(g.permutation(n).astype(np.int32)).cuda()
    bits = 32 if P <= 32 else 64
    words = torch.zeros((R, n), dtype=torch.int32 if bits == 32 else torch.int64, device="cuda")
    lib = _native.lib()
    base = buf.data_ptr()
    _native.check(lib.pq_pack_spins(ctypes.c_void_p(base + offset), n, P, R, _device.ptr(perm), _device.ptr(words), bits,
                                    n, _device.stream_handle()), "pack")
    w = words.cpu().numpy().astype(np.uint64) & ((1 << bits) - 1) if bits == 32 else words.cpu().numpy().view(np.uint64)
    expect = ((spins < 0).astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(axis=2, dtype=np.uint64)
    np.testing.assert_array_equal(w[:, perm.cpu().numpy()], expect)
    out = torch.full((R * n * P + 32,), 7, dtype=torch.int8, device="cuda")
    _native.check(lib.pq_unpack_spins(_device.ptr(words), bits, n, P, R, _device.ptr(perm), n,
                                      ctypes.c_void_p(out.data_ptr() + offset), _device.stream_handle()), "unpack")
    o = out.cpu().numpy()
    np.testing.assert_array_equal(o[offset:offset + R * n * P], spins.ravel())
    assert (o[:offset] == 7).all() and (o[offset + R * n * P:] == 7).all()   # nothing written outside
