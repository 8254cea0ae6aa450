"""Autotuner of the batched kernel's tiles.

For each instance shape (padded slot count rounded up to a power of two, P,
couplings per spin, replicas) it times every candidate tile -- ``gwarps`` warps
per work item and ``rpc`` replicas per item -- on a probe batch made of copies
of the instance large enough to fill the GPU, for a few field steps, and keeps
the fastest.  Results are cached per GPU name in memory and, when
``PIQMC_TUNE_CACHE`` names a file, on disk (JSON).

Use: ``Batch(nbs_list, replicas, slices, tuner=autotune.tune)``.
"""
import json
import os

import numpy as np
import torch

CANDIDATES = ((1, 1), (1, 2), (1, 4), (1, 8), (2, 1), (2, 2), (2, 4), (4, 1), (4, 2), (8, 1), (8, 2))
_cache = {}
_loaded = False


def _cache_file():
    return os.environ.get("PIQMC_TUNE_CACHE")


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    path = _cache_file()
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                for k, v in json.load(f).items():
                    _cache[k] = (tuple(v[0]), float(v[1]))
        except (OSError, ValueError):
            pass


def _save():
    path = _cache_file()
    if path:
        try:
            with open(path, "w") as f:
                json.dump({k: [list(v[0]), v[1]] for k, v in _cache.items()}, f, indent=1, sort_keys=True)
        except OSError:
            pass


def shape_key(problem, P, R):
    b = 1
    while b < problem.nslots:
        b *= 2
    return "%s|%d|%d|%d|%d" % (torch.cuda.get_device_name(), b, P, problem.maxdeg, min(R, 8))


def measure(problem, P, R, steps=8, candidates=CANDIDATES, repeats=2):
    """Time each candidate tile on a probe batch; returns ((gwarps, rpc), updates/s) of the best.

    Each candidate is timed ``repeats`` times over ``steps`` field steps and keeps its best time."""
    from . import _native
    from .batch import SMEM_TASK_BUDGET, Batch
    lib = _native.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    copies = max(1, (sms * 8) // R)
    g = np.random.default_rng(0)
    spins = np.where(g.random((R, problem.n, P)) < 0.5, -1, 1).astype(np.int8)
    sched = np.linspace(3.0, 1e-8, steps + 1)
    best = None
    for gw, rpc in candidates:
        if rpc > R or lib.pq_batch_smem_bytes(rpc, problem.nslots, P) > SMEM_TASK_BUDGET:
            continue
        B = Batch([problem] * copies, [R] * copies, [P] * copies, tiles=[(gw, rpc)] * copies)
        B.set_spins([spins] * copies)
        B.anneal(sched[:1], 0.05, seed=1)
        torch.cuda.synchronize()
        best_ms = None
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            B.anneal(sched[1:], 0.05, seed=2)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best_ms = ms if best_ms is None else min(best_ms, ms)
        rate = copies * R * problem.n * P * steps / (best_ms * 1e-3)
        if best is None or rate > best[1]:
            best = ((gw, rpc), rate)
    return best


def tune(batch):
    """Tiles for every instance of ``batch`` (a Batch under construction)."""
    _load()
    tiles = []
    changed = False
    for pb, P, R in zip(batch.problems, batch.P, batch.R):
        key = shape_key(pb, P, R)
        if key not in _cache:
            _cache[key] = measure(pb, P, R)
            changed = True
        tiles.append(_cache[key][0])
    if changed:
        _save()
    return tiles


def table():
    """The cached measurements: {shape key: ((gwarps, rpc), updates/s)}."""
    _load()
    return dict(_cache)
