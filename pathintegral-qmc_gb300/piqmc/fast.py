"""Packed fast sweeps: a sparse Ising instance on the device, and the kernels that anneal it.

``Problem`` turns a neighbour table (``tools.GenerateNeighbors`` layout) into the
device form the packed kernel reads:

* self entries become the field h_i; zero couplings (the table's padding) are
  dropped -- adding +-0 never changes a decision;
* spins are coloured (greedy in spin order, or DSatur when that needs fewer
  colours); each colour is cut, in the order of a fixed hash of the spin index,
  into update classes of T = ceil(n / (2 * subclasses)) spins (T rounded up to a
  multiple of ``quantum`` once the classes are that large) plus one class with
  the remainder, giving M independent sets (M <= 32; T grows if needed).  A
  two-colourable graph with colours of n/2 spins gets ``subclasses`` classes per
  colour; a small third colour gets one class instead of ``subclasses``
  near-empty ones.  Visiting many small classes in a random order per sweep
  makes the sweep behave like the reference's random sequential order; plain
  colour order anneals measurably worse;
* spins are relabelled into "device order": class c occupies slots
  [c*S, c*S + size_c) of a padded space of M*S slots; ``perm[i]`` is the slot of
  original spin i;
* couplings go to structure-of-arrays tables ``nbr[m, slot]`` / ``cpl[m, slot]``
  padded with (slot, 0.0);
* a CSR of the couplings in device order, FP64, serves the energy pass
  (off-diagonal table entries at half weight, since the table lists each
  coupling from both ends).

World-lines are packed one word per slot: int32 words for P <= 32, int64 for
P <= 64; bit k set = spin -1 in slice k.
"""
import ctypes

import numpy as np
import torch

from . import _device, _native
from .reforder import jperp_schedule, split_neighbors

MAX_CLASSES = 32
MAX_DEG = 16


def _mix32(x):
    """A fixed 32-bit integer hash (splitmix64 finaliser, low half) of the spin index."""
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return (x ^ (x >> np.uint64(31))) & np.uint64(0xFFFFFFFF)


def word_dtype(P):
    if P <= 32:
        return torch.int32, 32
    if P <= 64:
        return torch.int64, 64
    raise _native.PiqmcError(_native.PQ_ERR_UNSUPPORTED, "packed sweeps hold at most 64 slices")


class Problem:
    """A sparse Ising instance in device order (see module docstring)."""

    def __init__(self, nbs, nrows=None, on_device=True, subclasses=8, quantum=None):
        idx, jv = split_neighbors(nbs, nrows)
        nbs = np.asarray(nbs, dtype=np.float64)
        n, maxnb = idx.shape
        jv64 = np.zeros((n, maxnb))
        m0 = min(n, nbs.shape[0])
        jv64[:m0] = nbs[:m0, :, 1]
        self.n = n
        rows = np.repeat(np.arange(n), maxnb).reshape(n, maxnb)
        self_mask = idx == rows
        off_mask = (~self_mask) & (jv64 != 0.0)
        if np.any((idx[off_mask] < 0) | (idx[off_mask] >= n)):
            raise ValueError("neighbour index outside [0, %d)" % n)
        # field: sum of the self entries (one per spin in GenerateNeighbors tables)
        h64 = np.where(self_mask, jv64, 0.0).sum(axis=1)
        deg = off_mask.sum(axis=1)
        self.maxdeg = int(deg.max()) if n else 0
        if self.maxdeg > MAX_DEG:
            raise _native.PiqmcError(_native.PQ_ERR_UNSUPPORTED,
                                     "packed sparse sweep supports at most %d couplings per spin" % MAX_DEG)
        # colouring on the compacted graph
        cidx = np.where(off_mask, idx, rows).astype(np.int32)
        cj = np.where(off_mask, jv, 0.0).astype(np.float32)
        color = np.empty(n, dtype=np.int32)
        nc = _native.lib().pq_color_graph(n, maxnb, _device.ptr(np.ascontiguousarray(cidx)),
                                          _device.ptr(np.ascontiguousarray(cj)), _device.ptr(color))
        if nc < 0:
            _native.check(-nc, "pq_color_graph")
        if nc > MAX_CLASSES:
            raise _native.PiqmcError(_native.PQ_ERR_UNSUPPORTED, "graph needs %d colours (> %d)" % (nc, MAX_CLASSES))
        self.ncolors = int(nc)
        K = max(1, int(subclasses))
        self.subclasses = K
        # class size T: n / (2K) spins, a multiple of `quantum` (the thread count a
        # replica's CTA uses) once classes are that large, so that every thread has
        # the same work in the phases of full classes
        if quantum is None:
            quantum = 128 if n >= 4096 else 32
        self.quantum = int(quantum)
        counts = np.bincount(color, minlength=self.ncolors)
        T = max(1, -(-n // (2 * K)))
        if n >= 2 * K * self.quantum:
            T = -(-T // self.quantum) * self.quantum
        while int(np.sum(-(-np.maximum(counts, 1) // T))) > MAX_CLASSES:
            T += 1
        h = _mix32(np.arange(n, dtype=np.uint64))
        cls = np.empty(n, dtype=np.int64)
        base = 0
        for c in range(self.ncolors):
            members = np.nonzero(color == c)[0]
            ranked = members[np.argsort(h[members], kind="stable")]
            m = len(members)
            cls[ranked] = base + np.arange(m) // T
            base += -(-m // T) if m else 0
        M = int(base)
        sizes = np.bincount(cls, minlength=M)
        S = int(sizes.max()) if n else 1
        self.nclass, self.class_stride, self.class_size = M, S, sizes.astype(np.int32)
        self.nslots = M * S
        # slot = class * S + rank of the spin (by original index) within its class
        order = np.lexsort((np.arange(n), cls))
        rank = np.empty(n, dtype=np.int64)
        starts = np.concatenate([[0], np.cumsum(sizes)])
        rank[order] = np.arange(n) - starts[cls[order]]
        self.perm = (cls * S + rank).astype(np.int32)     # original spin -> device slot
        self.inv = np.full(self.nslots, -1, dtype=np.int32)
        self.inv[self.perm] = np.arange(n, dtype=np.int32)
        # SoA tables in device order, compacted per spin in table order
        D = max(self.maxdeg, 1)
        NS = self.nslots
        nbr = np.empty((D, NS), dtype=np.int32)
        cpl = np.zeros((D, NS), dtype=np.float32)
        field = np.zeros(NS, dtype=np.float32)
        nbr[:] = np.arange(NS, dtype=np.int32)[None, :]
        # vectorised compaction: rank of each kept entry within its row
        rank = np.cumsum(off_mask, axis=1) - 1
        r_i, r_m = np.nonzero(off_mask)
        dev_rows = self.perm[r_i]
        slots = rank[r_i, r_m]
        nbr[slots, dev_rows] = self.perm[idx[r_i, r_m]]
        cpl[slots, dev_rows] = jv[r_i, r_m]
        field[self.perm] = h64.astype(np.float32)
        self.nbr_host, self.cpl_host, self.field_host = nbr, cpl, field
        self.no_field = not np.any(field)
        # FP64 CSR for energies, device order
        e_r, e_m = np.nonzero(self_mask | off_mask)
        vals = np.where(self_mask, jv64, 0.5 * jv64)
        dr = self.perm[e_r]
        dc = np.where(self_mask[e_r, e_m], dr, self.perm[np.clip(idx[e_r, e_m], 0, n - 1)])
        o = np.lexsort((np.arange(len(dr)), dr))
        self.csr_ptr = np.concatenate([[0], np.cumsum(np.bincount(dr, minlength=NS))]).astype(np.int64)
        self.csr_col = dc[o].astype(np.int32)
        self.csr_val = vals[e_r, e_m][o].astype(np.float64)
        if on_device:
            self.to_device()

    def to_device(self):
        dev = _device.device()
        self.nbr = torch.from_numpy(self.nbr_host).to(dev)
        self.cpl = torch.from_numpy(self.cpl_host).to(dev)
        self.field = torch.from_numpy(self.field_host).to(dev)
        self.d_perm = torch.from_numpy(self.perm).to(dev)
        self.d_csr_ptr = torch.from_numpy(self.csr_ptr).to(dev)
        self.d_csr_col = torch.from_numpy(self.csr_col).to(dev)
        self.d_csr_val = torch.from_numpy(self.csr_val).to(dev)
        return self

    @classmethod
    def from_sparse(cls, J, maxnb=None):
        from .tools import GenerateNeighbors
        J = J.todok() if hasattr(J, "todok") else J
        n = J.shape[0]
        if maxnb is None:
            counts = np.zeros(n, dtype=np.int64)
            for (a, b) in J.keys():
                counts[a] += 1
                if b != a:
                    counts[b] += 1
            maxnb = int(counts.max()) if n else 0
        return cls(GenerateNeighbors(n, J, maxnb))

    # --------------------------------------------------------------------------------------
    def pack(self, spins):
        """int8 (R, n, P) +-1 in original order (host or device) -> packed words in device order."""
        sp = torch.as_tensor(spins).to(_device.device(), torch.int8).contiguous()
        R, n, P = sp.shape
        if n != self.n:
            raise ValueError("spins have %d rows, problem has %d spins" % (n, self.n))
        dt, bits = word_dtype(P)
        words = torch.zeros((R, self.nslots), dtype=dt, device=sp.device)
        _native.check(_native.lib().pq_pack_spins(_device.ptr(sp), n, P, R, _device.ptr(self.d_perm),
                                                   _device.ptr(words), bits, self.nslots, _device.stream_handle()),
                      "pq_pack_spins")
        return words

    def unpack(self, words, P):
        R = words.shape[0]
        _, bits = word_dtype(P)
        out = torch.empty((R, self.n, P), dtype=torch.int8, device=words.device)
        _native.check(_native.lib().pq_unpack_spins(_device.ptr(words), bits, self.n, P, R, _device.ptr(self.d_perm),
                                                     self.nslots, _device.ptr(out), _device.stream_handle()),
                      "pq_unpack_spins")
        return out

    def energies(self, words, P, out=None):
        """FP64 classical energy of every (replica, slice): double tensor (R, P)."""
        R, n = words.shape
        _, bits = word_dtype(P)
        if out is None:
            out = torch.empty((R, P), dtype=torch.float64, device=words.device)
        _native.check(_native.lib().pq_energy_packed(
            _device.ptr(words), bits, n, P, R, _device.ptr(self.d_csr_ptr), _device.ptr(self.d_csr_col),
            _device.ptr(self.d_csr_val), _device.ptr(out), _device.stream_handle()), "pq_energy_packed")
        return out

    def params(self, P, R, nsched, mcsteps, temp, seed, global_moves=0, sweep_base=0, replica_base=0,
               threads=0, replicas_per_cta=0, order_mode=1):
        p = _native.FastParams()
        p.n, p.P, p.R, p.maxdeg = self.nslots, int(P), int(R), self.maxdeg
        p.nclass, p.class_stride = self.nclass, self.class_stride
        for c in range(self.nclass):
            p.class_size[c] = int(self.class_size[c])
        p.order_mode = int(order_mode)
        p.nsched, p.mcsteps, p.global_moves = int(nsched), int(mcsteps), int(global_moves)
        p.temp = float(np.float32(temp))
        p.beta = float(np.float32(1.0) / np.float32(temp))
        p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        p.sweep_base, p.replica_base = int(sweep_base), int(replica_base)
        p.threads, p.replicas_per_cta = int(threads), int(replicas_per_cta)
        return p


def anneal(problem, words, sched, P, temp, mcsteps=1, seed=0, global_moves=0, sweep_base=0, replica_base=0,
           threads=0, replicas_per_cta=0, jperp=None, betas=None, accepts=None, status=None, stream=None,
           check=True, order_mode=1):
    """Anneal packed replicas in place through ``sched`` (transverse-field values).

    words: (R, n) int32/int64 device tensor in device order (``Problem.pack``).
    Returns the device status word (already checked when ``check``).
    """
    R, n = words.shape
    if n != problem.nslots:
        raise ValueError("words have %d slots, problem has %d" % (n, problem.nslots))
    nsched = len(sched) if jperp is None else len(jperp)
    if jperp is None:
        jp = jperp_schedule(sched, P, temp) if P > 1 else np.zeros(nsched, np.float32)
        jperp = torch.from_numpy(jp).to(words.device)
    st = status if status is not None else _device.Status()
    prm = problem.params(P, R, nsched, mcsteps, temp, seed, global_moves, sweep_base, replica_base, threads,
                         replicas_per_cta, order_mode)
    field = None if problem.no_field else problem.field     # no table when every field is zero
    code = _native.lib().pq_qa_fast_ex(
        _device.ptr(words), _device.ptr(problem.nbr), _device.ptr(problem.cpl), _device.ptr(field),
        _device.ptr(jperp), _device.ptr(betas), ctypes.byref(prm), _device.ptr(accepts), st.ptr,
        _device.stream_handle(stream))
    _native.check(code, "pq_qa_fast")
    if check:
        st.raise_if_set("pq_qa_fast", stream)
    return st


def anneal_replicas(problem, confs, sched, P, temp, mcsteps=1, seed=0, global_moves=0, order_mode=1,
                    out=None, energies_out=None, stream=None, replica_base=0):
    """Host-buffer entry point: anneal R replicas given as int8 (R, n, P) +-1 host arrays.

    Copies the configurations to the device, packs them, anneals, computes the
    FP64 energy of every (replica, slice), unpacks and copies spins and energies
    back.  ``confs`` may be a numpy array or a (pinned) CPU tensor; ``out`` and
    ``energies_out`` optional (pinned) CPU tensors receive the results.  Returns
    (final spins, energies) as CPU tensors.
    """
    src = confs if isinstance(confs, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(confs))
    R = src.shape[0]
    dev = _device.device()
    d_spins = src.to(dev, non_blocking=True)
    words = problem.pack(d_spins)
    anneal(problem, words, sched, P, temp, mcsteps=mcsteps, seed=seed, global_moves=global_moves,
           order_mode=order_mode, stream=stream, replica_base=replica_base)
    E = problem.energies(words, P)
    fin = problem.unpack(words, P)
    if out is None:
        out = torch.empty((R, problem.n, P), dtype=torch.int8, pin_memory=True)
    if energies_out is None:
        energies_out = torch.empty((R, P), dtype=torch.float64, pin_memory=True)
    out.copy_(fin, non_blocking=True)
    energies_out.copy_(E, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return out, energies_out
