"""Autotuner of the batched kernel's tiles.

Two levels.  Per instance shape (padded slot count rounded up to a power of
two, P, couplings per spin, replicas) ``measure`` times every candidate tile --
``gwarps`` warps per work item, ``rpc`` replicas per item, and for 64-slice
instances one lane or a lane pair per site -- on a probe batch
made of enough copies of the instance that the tile's tasks fill two CTAs per
SM, for a few field steps: its rate is the GPU's throughput on that shape with
every warp slot busy.  Per batch, ``plan`` then picks one tile per instance to
minimise the predicted time of one field step,

    max( sum_i warp-seconds_i / warp slots ,  longest item ),

where an item of instance i with tile (gw, rpc) takes ``n_i P_i rpc / (gw w)``
seconds per field step and ``w`` is the measured per-warp-slot rate of that
tile.  The most efficient tile of a small instance is often one warp on eight replicas; the
largest instances of a batch need more warps per item, or their items outlast
the rest of the batch.  Rate tables are cached per GPU name in
memory and, when ``PIQMC_TUNE_CACHE`` names a file, on disk (JSON).

Use: ``Batch(nbs_list, replicas, slices, tuner=autotune.tune)``.
"""
import json
import os

import numpy as np
import torch

_BASE = ((1, 1), (1, 2), (1, 4), (1, 8), (2, 1), (2, 2), (2, 4), (4, 1), (4, 2), (8, 1), (8, 2))
# (gwarps, rpc, lanes_per_site); lane pairs only for instances that support them
CANDIDATES = tuple((gw, rpc, 1) for gw, rpc in _BASE) + tuple((gw, rpc, 2) for gw, rpc in _BASE)
CTAS_PER_SM = 2
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
                    if isinstance(v, dict):
                        _cache[k] = {(tuple(int(x) for x in t.split(",")) + (1,))[:3]: float(r)
                                     for t, r in v.items()}
        except (OSError, ValueError):
            pass


def _save():
    path = _cache_file()
    if path:
        try:
            with open(path, "w") as f:
                json.dump({k: {"%d,%d,%d" % t: r for t, r in v.items()} for k, v in _cache.items()}, f, indent=1,
                          sort_keys=True)
        except OSError:
            pass


def shape_key(problem, P, R):
    b = 1
    while b < problem.nslots:
        b *= 2
    return "%s|%d|%d|%d|%d" % (torch.cuda.get_device_name(), b, P, problem.maxdeg, min(R, 8))


def warp_slots(sms):
    from .batch import WARPS
    return CTAS_PER_SM * WARPS * sms


def measure(problem, P, R, steps=8, candidates=CANDIDATES, repeats=2):
    """Time each candidate tile on a probe batch that fills the GPU; returns {(gwarps, rpc, lanes): updates/s}.

    Each candidate is timed ``repeats`` times over ``steps`` field steps and keeps its best time."""
    from . import _native
    from .batch import SMEM_TASK_BUDGET, WARPS, Batch, lane_pairs_supported
    lib = _native.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    g = np.random.default_rng(0)
    spins = np.where(g.random((R, problem.n, P)) < 0.5, -1, 1).astype(np.int8)
    sched = np.linspace(3.0, 1e-8, steps + 1)
    rates = {}
    for gw, rpc, lps in candidates:
        if rpc > R or lib.pq_batch_smem_bytes(rpc, problem.nslots, P) > SMEM_TASK_BUDGET:
            continue
        if lps == 2 and not lane_pairs_supported(problem, P):
            continue
        items = -(-R // rpc)
        copies = max(1, -(-CTAS_PER_SM * sms * (WARPS // gw) // items))
        B = Batch([problem] * copies, [R] * copies, [P] * copies, tiles=[(gw, rpc, lps)] * copies)
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
        rates[(gw, rpc, lps)] = copies * R * problem.n * P * steps / (best_ms * 1e-3)
    return rates


def plan(shapes, tables, slots, candidates=CANDIDATES):
    """Tiles minimising the predicted field-step time of a batch.

    ``shapes``: (slots n_i, P_i, R_i) per instance; ``tables``: {(gwarps, rpc, lanes): updates/s at fill}
    per instance; ``slots``: warp slots of the GPU.  For a cap T on the item duration every
    instance takes its cheapest tile (fewest warp-seconds) whose items last at most T; the
    prediction of a choice is max(warp-seconds / slots, longest item), minimised over the caps.
    Returns (tiles, predicted seconds per field step)."""
    n_inst, C = len(shapes), len(candidates)
    if n_inst == 0:
        return [], 0.0
    dur = np.full((n_inst, C), np.inf)
    cost = np.full((n_inst, C), np.inf)
    for i, ((n, P, R), tab) in enumerate(zip(shapes, tables)):
        for c, (gw, rpc, _) in enumerate(candidates):
            rate = tab.get(candidates[c])
            if not rate or rpc > R:
                continue
            w = rate / slots                        # updates/s of one busy warp slot
            dur[i, c] = n * P * rpc / (gw * w)
            cost[i, c] = n * P * R / w              # warp-seconds per field step
    if np.isinf(dur).all(axis=1).any():
        raise ValueError("an instance has no measured tile")
    rows = np.arange(n_inst)
    best = None
    for T in np.unique(dur[np.isfinite(dur)]):
        m = np.where(dur <= T, cost, np.inf)
        ch = m.argmin(axis=1)
        if np.isinf(m[rows, ch]).any():
            continue
        pred = max(m[rows, ch].sum() / slots, dur[rows, ch].max())
        if best is None or pred < best[1]:
            best = (ch, pred)
    ch, pred = best
    return [candidates[c] for c in ch], float(pred)


def tune(batch):
    """Tiles for every instance of ``batch`` (a Batch under construction)."""
    _load()
    tables = []
    changed = False
    for pb, P, R in zip(batch.problems, batch.P, batch.R):
        key = shape_key(pb, P, R)
        if key not in _cache:
            _cache[key] = measure(pb, P, R)
            changed = True
        tables.append(_cache[key])
    if changed:
        _save()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    shapes = [(pb.nslots, P, R) for pb, P, R in zip(batch.problems, batch.P, batch.R)]
    tiles, batch.predicted_step_s = plan(shapes, tables, warp_slots(sms))
    return tiles


def table():
    """The cached measurements: {shape key: {(gwarps, rpc, lanes): updates/s at fill}}."""
    _load()
    return dict(_cache)
