"""The N-rank path on CPU: two gloo ranks shard replicas with no data-path collective.

Each rank anneals its replicas of a small lattice through the packed sweep's CPU
oracle with the job's key and its own global replica ids (``piqmc.shard.rank_plan``);
the gathered results must equal one process annealing all replicas, and the
timing reduction must return the slowest rank's time.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

import oracle
from pq_testutil import ROOT, lattice


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


SEED = 7


def _setup():
    from piqmc import fast, shard, tools
    J = lattice(6, True, np.random.default_rng(3), dist=lambda r: r.normal())
    nbs = tools.GenerateNeighbors(36, J, 4)
    return shard, fast.Problem(nbs, on_device=False)


def _anneal(prob, spins, replica_base, P, seed):
    sched = np.linspace(3.0, 1e-8, 12)
    jp = oracle.jperp(sched, P, 0.05)
    out = []
    for j, s0 in enumerate(spins):
        w = np.zeros(prob.nslots, np.uint64)
        bits = (np.tile(s0, (P, 1)).T < 0).astype(np.uint64)
        w[prob.perm] = (bits << np.arange(P, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
        oracle.fast_anneal(prob.nbr_host, prob.cpl_host, prob.field_host, prob.class_size, prob.class_stride, w, P,
                           jp, 1, np.float32(20.0), seed, replica=replica_base + j, global_moves=1)
        out.append(w[prob.perm])
    return np.array(out)


def _rank(rank, world, port, R, P, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        shard, prob = _setup()
        plan = shard.rank_plan(rank, world, R, SEED)
        spins = shard.initial_spins(plan.replica_base, R, prob.n)
        w = torch.from_numpy(_anneal(prob, spins, plan.replica_base, P, plan.seed).view(np.int64))
        parts = [torch.empty_like(w) for _ in range(world)]
        dist.all_gather(parts, w)                # gathered here only to check; the bench never gathers
        slow = shard.max_over_ranks(0.5 + rank, dist, "cpu")
        if rank == 0:
            q.put((np.concatenate([p.numpy() for p in parts]).view(np.uint64), slow))
    finally:
        dist.destroy_process_group()


def test_rank_plan_is_a_partition():
    from piqmc import shard
    plans = [shard.rank_plan(r, 4, 8, SEED) for r in range(4)]
    ids = np.concatenate([np.arange(p.replica_base, p.replica_base + p.replicas) for p in plans])
    np.testing.assert_array_equal(ids, np.arange(32))
    assert len({p.seed for p in plans}) == 1 and plans[0].total_replicas == 32
    np.testing.assert_array_equal(shard.initial_spins(8, 8, 36), shard.initial_spins(0, 16, 36)[8:])
    assert shard.whole_job_rate(100.0, 3, 4, 2.0) == 600.0
    with pytest.raises(ValueError):
        shard.rank_plan(4, 4, 8)


def test_plan_from_env(monkeypatch):
    from piqmc import shard
    monkeypatch.setenv("RANK", "3")
    monkeypatch.setenv("WORLD_SIZE", "4")
    p = shard.plan_from_env(16, seed=5)
    assert (p.rank, p.world, p.replica_base, p.replicas, p.seed) == (3, 4, 48, 16, 5)


def test_bench_uses_the_package_plan():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    from piqmc import shard
    assert bench.rank_plan(1, 2, 8) == shard.rank_plan(1, 2, 8, bench.BENCH_SEED)
    assert bench.initial_spins is shard.initial_spins


def test_two_gloo_ranks_equal_one_process():
    R, P, world = 3, 8, 2
    ctx = tmp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, R, P, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    gathered, slow = q.get()
    shard, prob = _setup()
    single = _anneal(prob, shard.initial_spins(0, world * R, prob.n), 0, P, SEED)
    np.testing.assert_array_equal(gathered, single)
    assert slow == 1.5
