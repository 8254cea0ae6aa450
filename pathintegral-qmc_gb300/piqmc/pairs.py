"""Pair world-line moves: the world-lines of two coupled spins flip together, in every slice.

A local sweep and the single world-line move leave an anneal, once the Trotter
coupling has stiffened the world-lines, in states that no single flip improves
but where flipping two coupled spins together still lowers the energy.  The pair
move reaches them.  It has no counterpart in the reference (whose sweeps flip
one spin in one slice at a time, piqmc/qmc.pyx:93-133); like the single
world-line move its cost is classical only (the Trotter terms of a flipped
world-line are unchanged).

``bond_classes`` lists every coupled pair of a ``fast.Problem`` once (device
slots i < j, the total coupling between them) and colours the bonds greedily so
that no endpoint of a bond of a class is an endpoint of, or a neighbour of an
endpoint of, another bond of the class: a pair flip then changes neither the
cost nor the features of any other bond of its class, so the moves of a class
commute and the reverse proposal probability of a learned move is exactly what
the network gives in the new state (detailed balance; the argument of the single
world-line move in ``piqmc.learned``).

``pair_pass`` tries every bond (Metropolis, q = 1).  ``learned_pair_pass`` lets a
``learned.ProposalMLP`` choose which bonds to try, from 8 features of the pair
(its cost, both single flip costs, the bond's alignment, kinks, magnetisations,
the Trotter stiffness), with the exact Metropolis-Hastings correction.
``record_pair_moves`` scores every pair move for training.  Arithmetic, uniforms
and features are specified in csrc/mlp.cu.
"""
import numpy as np
import torch

from . import _device, _native

QMIN = 0.05


def _pad(x, m):
    return (x + m - 1) // m * m


class BondClasses:
    """The bonds of a problem in device slots, grouped in independent classes."""

    def __init__(self, problem):
        nbr, cpl = problem.nbr_host, problem.cpl_host
        NS = problem.nslots
        D = nbr.shape[0] if problem.maxdeg > 0 else 0
        acc = {}
        adj = [set() for _ in range(NS)]
        for m in range(D):
            for i in range(NS):
                j = int(nbr[m, i])
                v = float(cpl[m, i])
                if j == i or v == 0.0:
                    continue
                adj[i].add(j)
                if i < j:                       # each coupling is listed from both ends: keep one
                    acc[(i, j)] = acc.get((i, j), np.float32(0.0)) + np.float32(v)
        bonds = sorted(k for k, v in acc.items() if v != 0.0)
        incident = [[] for _ in range(NS)]
        for b, (i, j) in enumerate(bonds):
            incident[i].append(b)
            incident[j].append(b)
        color = np.full(len(bonds), -1, dtype=np.int64)
        for b, (i, j) in enumerate(bonds):
            used = set()
            for v in {i, j} | adj[i] | adj[j]:
                for o in incident[v]:
                    if color[o] >= 0:
                        used.add(int(color[o]))
            c = 0
            while c in used:
                c += 1
            color[b] = c
        order = np.lexsort((np.arange(len(bonds)), color))
        self.nclass = int(color.max()) + 1 if len(bonds) else 0
        self.bond_i = np.array([bonds[b][0] for b in order], dtype=np.int32)
        self.bond_j = np.array([bonds[b][1] for b in order], dtype=np.int32)
        self.bond_J = np.array([acc[bonds[b]] for b in order], dtype=np.float32)
        self.class_start = np.concatenate([[0], np.cumsum(np.bincount(color, minlength=self.nclass))]).astype(np.int32)
        self.nbonds = len(bonds)
        self.adjacency = adj
        self._dev = None

    def _device_arrays(self):
        if self._dev is None:
            dev = _device.device()
            self._dev = tuple(torch.from_numpy(a).to(dev) for a in (self.bond_i, self.bond_j, self.bond_J))
        return self._dev

    @property
    def d_i(self):
        return self._device_arrays()[0]

    @property
    def d_j(self):
        return self._device_arrays()[1]

    @property
    def d_J(self):
        return self._device_arrays()[2]


def bond_classes(problem):
    """The problem's bond classes (built once and kept on the problem)."""
    bc = getattr(problem, "_bond_classes", None)
    if bc is None:
        bc = problem._bond_classes = BondClasses(problem)
    return bc


def _status(status, dev):
    return status if status is not None else torch.zeros(1, dtype=torch.int32, device=dev)


def _raise(status, where):
    code = int(status.item())
    if code:
        raise _native.PiqmcError(code, where)


def pair_pass(problem, words, P, beta, seed, move, counters=None, replica_base=0, status=None, check=True):
    """Every bond tried once, class by class (Metropolis); in place on ``words``."""
    bc = bond_classes(problem)
    R = words.shape[0]
    bits = 32 if P <= 32 else 64
    st = _status(status, words.device)
    _native.check(_native.lib().pq_pair_pass(
        _device.ptr(words), bits, problem.nslots, int(P), R, problem.maxdeg, _device.ptr(problem.nbr),
        _device.ptr(problem.cpl), _device.ptr(problem.field), _device.ptr(bc.d_i), _device.ptr(bc.d_j),
        _device.ptr(bc.d_J), _device.ptr(bc.class_start), bc.nclass, float(beta), int(move) & 0xFFFFFFFF,
        int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica_base), _device.ptr(counters), _device.ptr(st),
        _device.stream_handle()), "pq_pair_pass")
    if check:
        _raise(st, "pq_pair_pass")


class _Rows:
    def __init__(self):
        self.X = None
        self.dE = None

    def get(self, Mpad, dev):
        if self.X is None or self.X.shape[0] < 2 * Mpad or self.X.device != dev:
            self.X = torch.zeros((2 * Mpad, 64), dtype=torch.bfloat16, device=dev)
            self.dE = torch.empty(Mpad, dtype=torch.float32, device=dev)
        return self.X[:2 * Mpad], self.dE[:Mpad]


_rows = _Rows()


def pair_features(problem, words, P, beta, jp, cls, status=None):
    """(X, dE, M, Mpad) of the pair moves of bond class ``cls``: rows [0, M) current, [Mpad, Mpad + M) flipped."""
    bc = bond_classes(problem)
    R = words.shape[0]
    first = int(bc.class_start[cls])
    count = int(bc.class_start[cls + 1]) - first
    M = R * count
    Mpad = _pad(max(M, 1), 128)
    X, dE = _rows.get(Mpad, words.device)
    _native.check(_native.lib().pq_pair_features(
        _device.ptr(words), 32 if P <= 32 else 64, problem.nslots, int(P), R, problem.maxdeg, _device.ptr(problem.nbr),
        _device.ptr(problem.cpl), _device.ptr(problem.field), _device.ptr(bc.d_i), _device.ptr(bc.d_j),
        _device.ptr(bc.d_J), first, count, float(beta), float(jp), _device.ptr(X), _device.ptr(dE), Mpad,
        _device.ptr(status), _device.stream_handle()), "pq_pair_features")
    return X, dE, M, Mpad


def learned_pair_pass(problem, words, P, mlp, beta, jp, seed, move, qmin=QMIN, counters=None, replica_base=0,
                      status=None, check=True, fused=True):
    """One learned pair move per bond, class by class: the network chooses which bonds to try.

    ``fused`` runs each class in one launch (features, network on the tensor cores,
    decision); otherwise the feature kernel, the network's GEMMs and the propose
    kernel run one after another -- the same moves."""
    bc = bond_classes(problem)
    R = words.shape[0]
    bits = 32 if P <= 32 else 64
    st = _status(status, words.device)
    lib = _native.lib()
    if fused:
        _native.check(lib.pq_pair_learned_pass(
            _device.ptr(words), bits, problem.nslots, int(P), R, problem.maxdeg, _device.ptr(problem.nbr),
            _device.ptr(problem.cpl), _device.ptr(problem.field), _device.ptr(bc.d_i), _device.ptr(bc.d_j),
            _device.ptr(bc.d_J), _device.ptr(bc.class_start), bc.nclass, float(beta), float(jp), _device.ptr(mlp.W1b),
            _device.ptr(mlp.W2b), _device.ptr(mlp.params["b1"]), _device.ptr(mlp.params["b2"]),
            _device.ptr(mlp.params["w3"]), mlp.b3_host, float(qmin), int(move) & 0xFFFFFFFF,
            int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica_base), _device.ptr(counters), _device.ptr(st),
            _device.stream_handle()), "pq_pair_learned_pass")
        if check:
            _raise(st, "learned pair pass")
        return
    for cls in range(bc.nclass):
        X, dE, M, Mpad = pair_features(problem, words, P, beta, jp, cls, status=st)
        if M == 0:
            continue
        logit = mlp.forward(X)
        first = int(bc.class_start[cls])
        _native.check(lib.pq_pair_propose(
            _device.ptr(words), bits, problem.nslots, int(P), R, _device.ptr(bc.d_i), _device.ptr(bc.d_j), first,
            int(bc.class_start[cls + 1]) - first, cls, _device.ptr(logit), _device.ptr(dE), Mpad, float(qmin),
            float(beta), int(move) & 0xFFFFFFFF, int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica_base),
            _device.ptr(counters), _device.ptr(st), _device.stream_handle()), "pq_pair_propose")
    if check:
        _raise(st, "learned pair pass")


def record_pair_moves(problem, words, P, beta, jp, max_rows=None):
    """Features of every pair move the uniform pass tries now, with its Metropolis acceptance probability."""
    bc = bond_classes(problem)
    Xs, ys = [], []
    for cls in range(bc.nclass):
        X, dE, M, _ = pair_features(problem, words, P, beta, jp, cls)
        if M == 0:
            continue
        Xs.append(X[:M].clone())
        ys.append(torch.clamp(torch.exp(-float(beta) * dE[:M]), max=1.0))
    X, y = torch.cat(Xs), torch.cat(ys)
    if max_rows is not None and X.shape[0] > max_rows:
        idx = torch.randperm(X.shape[0], device=X.device)[:max_rows]
        X, y = X[idx], y[idx]
    return X, y
