"""Batched persistent packed sweeps: many uneven instances in one launch.

A ``Batch`` holds instances of different size, slice count and replica count.
Their tables are concatenated into pools, their world-lines into one byte pool,
and the work is cut into *items* (``rpc`` replicas of one instance, run by a
group of ``gwarps`` warps) packed into *tasks* (items sharing a CTA, each with
its own named barrier).  A tile may add ``lanes_per_site`` = 2: a 64-slice
instance then gives each site a lane pair, one 32-bit half of the world-line
each, which halves the serial work of a sweep (same result).  One persistent launch (``pq_batch_anneal``) drains the
task queue; tasks are ordered longest first.  The tile of each instance --
``(gwarps, rpc[, lanes_per_site])`` -- comes from ``piqmc.autotune`` (measured)
or a size heuristic.

``anneal`` splits the schedule into chunks of ``chunk`` field steps, one launch
each, and can capture the chunk sequence as a CUDA graph that is replayed for
every later anneal of the same shape (``graph=True``): the field-schedule loop
then costs one graph launch.

Instance i anneals with Philox key ``seed + i`` and replica ids 0..R_i-1, so a
batched anneal equals ``fast.anneal`` of each instance with ``seed=seed + i``
bit for bit.
"""
import ctypes

import numpy as np
import torch

from . import _device, _native
from .fast import Problem, jperp_schedule, word_dtype

INST_DTYPE = np.dtype([("tab_off", "<i8"), ("field_off", "<i8"), ("csize_off", "<i4"), ("jperp_off", "<i4"),
                       ("n", "<i4"), ("P", "<i4"), ("maxdeg", "<i4"), ("nclass", "<i4"), ("stride", "<i4"),
                       ("key0", "<u4"), ("key1", "<u4"), ("pad", "<i4")])
ITEM_DTYPE = np.dtype([("inst", "<i4"), ("nrep", "<i4"), ("replica0", "<i4"), ("smem_off", "<i4"),
                       ("word_off", "<i8")])
TASK_DTYPE = np.dtype([("item0", "<i4"), ("nitems", "<i4"), ("gwarps", "<i4"), ("lanes_per_site", "<i4")])
assert INST_DTYPE.itemsize == 56 and ITEM_DTYPE.itemsize == 24 and TASK_DTYPE.itemsize == 16

THREADS = 256
WARPS = THREADS // 32
SMEM_TASK_BUDGET = 110 * 1024


def _align(x, a=16):
    return (x + a - 1) // a * a


def heuristic_tile(nslots, P, R):
    """(gwarps, rpc) without measurements: about one spin-slot of work per thread per phase."""
    S = max(1, nslots // 16)
    for gw in (8, 4, 2, 1):
        if S >= 32 * gw * 2:
            return gw, 1
    rpc = 1
    while rpc < R and rpc * S < 32 and _native.lib().pq_batch_smem_bytes(rpc * 2, nslots, P) < SMEM_TASK_BUDGET // 2:
        rpc *= 2
    return 1, min(rpc, R)


def lane_pairs_supported(problem, P):
    """Items of this instance can give each site a lane pair (64-slice world-lines, up to 4 couplings)."""
    return P == 64 and problem.maxdeg <= 4


def normalise_tile(tile, problem, P):
    """(gwarps, rpc[, lanes_per_site]) -> (gwarps, rpc, lanes_per_site); lane pairs only where supported."""
    gw, rpc = int(tile[0]), int(tile[1])
    lps = int(tile[2]) if len(tile) > 2 else 1
    if gw not in (1, 2, 4, 8) or rpc < 1 or lps not in (1, 2):
        raise ValueError("tile %r: gwarps in {1, 2, 4, 8}, rpc >= 1, lanes_per_site in {1, 2}" % (tuple(tile),))
    if lps == 2 and not lane_pairs_supported(problem, P):
        lps = 1
    return gw, rpc, lps


def sweep_variant(P):
    """Which compiled sweep an item of P slices runs (the kernel has one per fixed P it
    specialises, and one generic per word size)."""
    return P if P in (16, 20, 32, 64) else (0 if P <= 32 else 1)


def pack_tasks(items):
    """Items ``(cost, (gwarps, lanes, variant), smem bytes, ...)`` -> tasks ``[(kind, [items])]``.

    Items of one kind, in decreasing cost, fill a task up to ``WARPS // gwarps`` items
    within the shared-memory budget, so the warps of a CTA run one compiled sweep; tasks
    are ordered by their longest item, longest first (the persistent CTAs take them in
    that order)."""
    items = sorted(items, key=lambda t: -t[0])
    by_kind = {}
    for it in items:
        by_kind.setdefault(it[1], []).append(it)
    tasks = []
    for kind, lst in by_kind.items():
        gw = kind[0]
        per = WARPS // gw
        cur = []
        used = 0
        for it in lst:
            if cur and (len(cur) == per or used + _align(it[2]) > SMEM_TASK_BUDGET):
                tasks.append((kind, cur))
                cur, used = [], 0
            cur.append(it)
            used += _align(it[2])
        if cur:
            tasks.append((kind, cur))
    tasks.sort(key=lambda t: -max(it[0] for it in t[1]))
    return tasks


class Batch:
    """Many sparse instances with their replicas, resident on the device."""

    def __init__(self, nbs_list, replicas, slices, subclasses=8, tiles=None, tuner=None):
        n_inst = len(nbs_list)
        if not (len(replicas) == len(slices) == n_inst):
            raise ValueError("nbs_list, replicas and slices must have the same length")
        self.P = [int(p) for p in slices]
        self.R = [int(r) for r in replicas]
        if any(p < 1 or p > 64 for p in self.P) or any(r < 1 for r in self.R):
            raise ValueError("slices must be in 1..64 and replicas >= 1")
        self.problems = [nbs if isinstance(nbs, Problem) else Problem(nbs, on_device=False, subclasses=subclasses)
                         for nbs in nbs_list]
        if any(pb.maxdeg > 8 for pb in self.problems):
            raise _native.PiqmcError(_native.PQ_ERR_UNSUPPORTED, "batched sweeps support at most 8 couplings per spin")
        lib = _native.lib()
        # pools
        inst = np.zeros(n_inst, dtype=INST_DTYPE)
        nbr, cpl, field, csize = [], [], [], []
        tab = fld = cs = 0
        word_off = 0
        self.word_offsets = []
        for i, (pb, P) in enumerate(zip(self.problems, self.P)):
            D = pb.nbr_host.shape[0]
            inst[i]["tab_off"], inst[i]["field_off"], inst[i]["csize_off"] = tab, fld, cs
            inst[i]["n"], inst[i]["P"], inst[i]["maxdeg"] = pb.nslots, P, pb.maxdeg
            inst[i]["nclass"], inst[i]["stride"] = pb.nclass, pb.class_stride
            nbr.append(pb.nbr_host.ravel())
            cpl.append(pb.cpl_host.ravel())
            field.append(pb.field_host)
            csize.append(pb.class_size.astype(np.int32))
            tab += D * pb.nslots
            fld += pb.nslots
            cs += pb.nclass
            self.word_offsets.append(word_off)
            word_off = _align(word_off + self.R[i] * pb.nslots * (4 if P <= 32 else 8))
        self.inst = inst
        self.words_bytes = max(word_off, 16)
        dev = _device.device()
        self.d_nbr = torch.from_numpy(np.concatenate(nbr).astype(np.int32)).to(dev)
        self.d_cpl = torch.from_numpy(np.concatenate(cpl).astype(np.float32)).to(dev)
        self.d_field = torch.from_numpy(np.concatenate(field).astype(np.float32)).to(dev)
        self.d_csize = torch.from_numpy(np.concatenate(csize)).to(dev)
        self.words = torch.zeros(self.words_bytes, dtype=torch.uint8, device=dev)
        self.queue_head = torch.zeros(1, dtype=torch.int32, device=dev)
        self.status = _device.Status()
        self.d_perm = [torch.from_numpy(pb.perm).to(dev) for pb in self.problems]
        # tiles, items, tasks
        if tiles is None and tuner is not None:
            tiles = tuner(self)
        tiles = tiles or [heuristic_tile(pb.nslots, P, R) for pb, P, R in zip(self.problems, self.P, self.R)]
        self.tiles = [normalise_tile(t, pb, P) for t, pb, P in zip(tiles, self.problems, self.P)]
        self._build_tasks(lib)
        self._jperp_key = None
        self._graphs = {}
        self._seed = None

    # ------------------------------------------------------------------------------------------
    def _build_tasks(self, lib):
        items = []
        for i, (pb, P, R) in enumerate(zip(self.problems, self.P, self.R)):
            gw, rpc, lps = self.tiles[i]
            wbytes = 4 if P <= 32 else 8
            for r0 in range(0, R, rpc):
                nrep = min(rpc, R - r0)
                smem = lib.pq_batch_smem_bytes(nrep, pb.nslots, P)
                cost = pb.nslots * P * nrep / (32.0 * gw)
                items.append((cost, (gw, lps, sweep_variant(P)), smem, i, nrep, r0,
                              self.word_offsets[i] + r0 * pb.nslots * wbytes))
        if any(it[2] > SMEM_TASK_BUDGET for it in items):
            raise _native.PiqmcError(_native.PQ_ERR_TOO_LARGE, "an item needs more than %d B of shared memory"
                                     % SMEM_TASK_BUDGET)
        tasks = pack_tasks(items)
        item_arr = np.zeros(len(items), dtype=ITEM_DTYPE)
        task_arr = np.zeros(len(tasks), dtype=TASK_DTYPE)
        k = 0
        max_smem = 16
        for t, (kind, lst) in enumerate(tasks):
            task_arr[t] = (k, len(lst), kind[0], kind[1])
            off = 0
            for it in lst:
                item_arr[k] = (it[3], it[4], it[5], off, it[6])
                off += _align(it[2])
                k += 1
            max_smem = max(max_smem, off)
        self.items, self.tasks = item_arr, task_arr
        self.smem_bytes = int(max_smem)
        dev = self.words.device
        self.d_items = torch.from_numpy(item_arr.view(np.uint8).copy()).to(dev)
        self.d_tasks = torch.from_numpy(task_arr.view(np.uint8).copy()).to(dev)
        bps, sms = ctypes.c_int(0), ctypes.c_int(0)
        _native.check(lib.pq_batch_occupancy(THREADS, self.smem_bytes, ctypes.byref(bps), ctypes.byref(sms)),
                      "pq_batch_occupancy")
        self.grid = max(1, min(len(tasks), bps.value * sms.value))

    # ------------------------------------------------------------------------------------------
    def _words_view(self, i):
        pb, P, R = self.problems[i], self.P[i], self.R[i]
        dt, _ = word_dtype(P)
        wb = 4 if P <= 32 else 8
        off = self.word_offsets[i]
        return self.words[off:off + R * pb.nslots * wb].view(dt).view(R, pb.nslots)

    def set_spins(self, spins_list):
        """Load int8 (R_i, n_i, P_i) +-1 configurations (host or device) for every instance."""
        lib = _native.lib()
        self.words.zero_()
        for i, sp in enumerate(spins_list):
            pb, P, R = self.problems[i], self.P[i], self.R[i]
            s = torch.as_tensor(sp).to(self.words.device, torch.int8).contiguous()
            if tuple(s.shape) != (R, pb.n, P):
                raise ValueError("instance %d: spins must have shape %r" % (i, (R, pb.n, P)))
            w = self._words_view(i)
            _native.check(lib.pq_pack_spins(_device.ptr(s), pb.n, P, R, _device.ptr(self.d_perm[i]), _device.ptr(w),
                                            32 if P <= 32 else 64, pb.nslots, _device.stream_handle()),
                          "pq_pack_spins")

    def spins(self):
        """Current configurations: list of int8 (R_i, n_i, P_i) device tensors."""
        lib = _native.lib()
        out = []
        for i, pb in enumerate(self.problems):
            P, R = self.P[i], self.R[i]
            o = torch.empty((R, pb.n, P), dtype=torch.int8, device=self.words.device)
            _native.check(lib.pq_unpack_spins(_device.ptr(self._words_view(i)), 32 if P <= 32 else 64, pb.n, P, R,
                                              _device.ptr(self.d_perm[i]), pb.nslots, _device.ptr(o),
                                              _device.stream_handle()), "pq_unpack_spins")
            out.append(o)
        return out

    def energies(self):
        """FP64 energies: list of (R_i, P_i) device tensors."""
        out = []
        for i, pb in enumerate(self.problems):
            if not hasattr(pb, "d_csr_ptr"):
                pb.to_device()
            out.append(pb.energies(self._words_view(i), self.P[i]))
        return out

    def _prepare(self, sched, temp, seed):
        sched = np.ascontiguousarray(sched, dtype=np.float64)
        if self._jperp_key != (sched.tobytes(), float(np.float32(temp))):
            per_p = {}
            parts, off = [], 0
            for i, P in enumerate(self.P):
                if P not in per_p:
                    per_p[P] = (jperp_schedule(sched, P, temp) if P > 1 else np.zeros(len(sched), np.float32))
                self.inst[i]["jperp_off"] = off
                parts.append(per_p[P])
                off += len(sched)
            self.d_jperp = torch.from_numpy(np.concatenate(parts).astype(np.float32)).to(self.words.device)
            self._jperp_key = (sched.tobytes(), float(np.float32(temp)))
            self._seed = None
            self._graphs.clear()
        if self._seed != seed:
            for i in range(len(self.P)):
                k = (int(seed) + i) & 0xFFFFFFFFFFFFFFFF
                self.inst[i]["key0"], self.inst[i]["key1"] = k & 0xFFFFFFFF, k >> 32
            self.d_inst = torch.from_numpy(self.inst.view(np.uint8).copy()).to(self.words.device)
            self._seed = seed

    def _launch(self, run, accepts=None):
        lib = _native.lib()
        return lib.pq_batch_anneal(
            _device.ptr(self.d_tasks), len(self.tasks), _device.ptr(self.d_items), _device.ptr(self.d_inst),
            _device.ptr(self.d_nbr), _device.ptr(self.d_cpl), _device.ptr(self.d_field), _device.ptr(self.d_csize),
            _device.ptr(self.d_jperp), _device.ptr(self.words), _device.ptr(self.queue_head), ctypes.byref(run),
            self.grid, THREADS, self.smem_bytes, _device.ptr(accepts), self.status.ptr, _device.stream_handle())

    def _runs(self, nsched, temp, mcsteps, global_moves, order_mode, chunk):
        chunk = nsched if not chunk else int(chunk)
        runs = []
        for g0 in range(0, nsched, chunk):
            r = _native.BatchRun()
            r.nsched = min(chunk, nsched - g0)
            r.sched_base = g0
            r.mcsteps, r.global_moves, r.order_mode = int(mcsteps), int(global_moves), int(order_mode)
            r.beta = float(np.float32(1.0) / np.float32(temp))
            r.sweep_base = g0 * int(mcsteps)
            runs.append(r)
        return runs

    def anneal(self, sched, temp, seed=0, mcsteps=1, global_moves=0, order_mode=1, chunk=None, graph=False,
               accepts=None, check=True):
        """Anneal every replica of every instance through ``sched`` (transverse-field values).

        With ``graph=True`` the first call of a given shape runs eagerly and captures the
        chunk launches as a CUDA graph; later calls replay it.
        """
        self._prepare(sched, temp, seed)
        runs = self._runs(len(sched), temp, mcsteps, global_moves, order_mode, chunk)
        gkey = (len(sched), float(np.float32(temp)), mcsteps, global_moves, order_mode, chunk,
                None if accepts is None else accepts.data_ptr())
        g = self._graphs.get(gkey) if graph else None
        if g is not None:
            g.replay()
        else:
            for r in runs:
                _native.check(self._launch(r, accepts), "pq_batch_anneal")
            if graph:
                torch.cuda.synchronize()
                self._graphs[gkey] = self._capture(runs, accepts)
        if check:
            self.status.raise_if_set("pq_batch_anneal")

    def _capture(self, runs, accepts=None):
        g = torch.cuda.CUDAGraph()
        self._graph_runs = runs   # the ctypes structs outlive the capture
        with torch.cuda.graph(g):
            for r in runs:
                _native.check(self._launch(r, accepts), "pq_batch_anneal")
        return g

    def graph_for(self, sched, temp, seed=0, mcsteps=1, global_moves=0, order_mode=1, chunk=None):
        """The CUDA graph of one anneal (``replay()`` re-runs it on the current state)."""
        self._prepare(sched, temp, seed)
        gkey = (len(sched), float(np.float32(temp)), mcsteps, global_moves, order_mode, chunk, None)
        if gkey not in self._graphs:
            runs = self._runs(len(sched), temp, mcsteps, global_moves, order_mode, chunk)
            self._graphs[gkey] = self._capture(runs)
        return self._graphs[gkey]
