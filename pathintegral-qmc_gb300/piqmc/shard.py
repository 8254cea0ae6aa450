"""Replica sharding over ranks: one process per GPU, replicas only, no data-path collective.

The reference runs independent anneals in separate MPI processes
(examples/spinglass32_mpi.py:20-26): every rank anneals its own copies of the
instance and the results are gathered at the end.  Here the unit of work is a
replica of the packed sweep.  A replica's random stream depends only on (the
job's Philox key, its global replica id, the sweep counter) and its start state
only on its global id, so splitting the job's replicas into contiguous ranges
per rank gives exactly the results of one process annealing all of them.  The
only collective a job needs is the max-over-ranks reduction of its timing.

    plan = shard.rank_plan(rank, world, replicas_per_rank, seed)
    spins = shard.initial_spins(plan.replica_base, plan.replicas, n)
    fast.anneal(problem, words, sched, P, T, seed=plan.seed, replica_base=plan.replica_base)
"""
import os
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class RankPlan:
    """The global replicas [replica_base, replica_base + replicas) of one rank, and the job's key."""
    rank: int
    world: int
    replica_base: int
    replicas: int
    seed: int

    @property
    def total_replicas(self):
        return self.world * self.replicas

    def __getitem__(self, key):   # dict-style access for callers that log the plan
        return getattr(self, key)


def rank_plan(rank, world, replicas_per_rank, seed=0):
    """Rank `rank` of `world` anneals the global replicas [rank R, (rank + 1) R) with the job's Philox key."""
    if not 0 <= rank < world or replicas_per_rank <= 0:
        raise ValueError("bad rank plan: rank %d of %d, %d replicas" % (rank, world, replicas_per_rank))
    return RankPlan(rank=int(rank), world=int(world), replica_base=int(rank) * int(replicas_per_rank),
                    replicas=int(replicas_per_rank), seed=int(seed))


def plan_from_env(replicas_per_rank, seed=0):
    """The plan of this process under torchrun (RANK / WORLD_SIZE; a single process otherwise)."""
    return rank_plan(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), replicas_per_rank,
                     seed)


def initial_spins(replica_base, R, n, seed=1234):
    """+-1 start vectors (int8 [R][n]) of global replicas replica_base .. replica_base + R - 1.

    Each replica's vector comes from its own generator seeded by (seed, global id),
    so it is the same on any rank layout."""
    out = np.empty((R, n), dtype=np.int8)
    for j in range(R):
        g = np.random.default_rng([seed, replica_base + j])
        out[j] = np.where(g.random(n) < 0.5, -1, 1)
    return out


def max_over_ranks(x, dist, device):
    """The largest of the ranks' values of x (a job's time is its slowest rank's)."""
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step, steps, world, total_s):
    """Units all ranks processed / the slowest rank's time."""
    return units_per_rank_step * steps * world / total_s
