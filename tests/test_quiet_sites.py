"""Skipping quiet sites changes nothing, on the CPU.

The packed sweep's staged phases visit only the sites whose quiet bit is clear
(csrc/sweep_core.cuh, site_visit and the scan).  tests/native/quiet_sim.c restates that
rule -- class sums, the per-slice update, when a visit sets a bit, which changes clear
bits, when a step rewrites them -- and this test runs it beside the oracle's per-slice
specification (oracle/fast_oracle.c, every site every sweep): the final world-lines and
accept counts must be equal, bit for bit, while the restatement skips most visits.
Negative controls: each part of the rule removed in turn makes some case differ.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle
from pq_testutil import lattice

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "quiet_sim.c")
ORC = os.path.join(os.path.dirname(HERE), "oracle", "fast_oracle.c")
LIB = os.path.join(HERE, "native", "_build", "libquiet_sim.so")

_lib = None


def _sim():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(SRC), os.path.getmtime(ORC)):
            os.makedirs(os.path.dirname(LIB), exist_ok=True)
            tmp = LIB + ".tmp%d" % os.getpid()
            subprocess.check_call(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                                   SRC, ORC, "-o", tmp, "-lm"])
            os.replace(tmp, LIB)
        L = ctypes.CDLL(LIB)
        V, I32, I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        L.qsim_anneal.argtypes = [I32, I32, I32, V, V, V, I32, I32, V, I32, V, I32, I32, ctypes.c_float,
                                  ctypes.c_uint64, I64, I32, I32, V, V, I32, ctypes.POINTER(I64)]
        L.qsim_anneal.restype = I64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _kings(L, g):
    """A periodic King's graph (eight couplings per spin), fields on every spin."""
    import scipy.sparse as sps
    n = L * L
    J = sps.dok_matrix((n, n))
    for y in range(L):
        for x in range(L):
            i = y * L + x
            for dx, dy in ((1, 0), (0, 1), (1, 1), (1, -1)):
                j = ((y + dy) % L) * L + (x + dx) % L
                J[min(i, j), max(i, j)] = g.normal()
            J[i, i] = g.normal(0, 0.3)
    return J


def _problem(L, periodic, seed, fields):
    from piqmc import fast, tools
    g = np.random.default_rng(seed)
    if fields == "kings":
        return fast.Problem(tools.GenerateNeighbors(L * L, _kings(L, g), 9), on_device=False)
    J = lattice(L, periodic, g, dist=lambda r: r.normal(),
                fields=(lambda r: r.normal(0, 0.3)) if fields else None)
    return fast.Problem(tools.GenerateNeighbors(L * L, J, 5), on_device=False)


def _run(prob, P, sched, T, mcsteps=1, global_moves=0, betas=None, seed=5, breaks=0, replicas=3, straight=True):
    jp = oracle.jperp(sched, P, T)
    beta = np.float32(1.0) / np.float32(T)
    nbr = np.ascontiguousarray(prob.nbr_host, np.int32)
    cpl = np.ascontiguousarray(prob.cpl_host, np.float32)
    fld = np.ascontiguousarray(prob.field_host, np.float32)
    csz = np.ascontiguousarray(prob.class_size, np.int32)
    bt = None if betas is None else np.ascontiguousarray(betas, np.float32)
    g = np.random.default_rng(seed)
    same, visits, total = True, 0, 0
    for r in range(replicas):
        # straight world-lines to start (the bench's start), or every slice drawn on its own
        bits = np.repeat(g.random((prob.n, 1)) < 0.5, P, axis=1) if straight else g.random((prob.n, P)) < 0.5
        w0 = np.zeros(prob.nslots, np.uint64)
        w0[prob.perm] = (bits.astype(np.uint64) << np.arange(P, dtype=np.uint64)).sum(axis=1).astype(np.uint64)
        a = w0.copy()
        na = oracle.fast_anneal(nbr, cpl, fld, csz, prob.class_stride, a, P, jp, mcsteps, beta, seed,
                                replica=r, global_moves=global_moves, betas=bt)
        b = w0.copy()
        v = ctypes.c_int64(0)
        nb = _sim().qsim_anneal(prob.nslots, P, nbr.shape[0], _p(nbr), _p(cpl), _p(fld), len(csz),
                                prob.class_stride, _p(csz), 1, _p(jp), len(jp), mcsteps, float(beta), seed, 0, r,
                                global_moves, _p(b), None if bt is None else _p(bt), breaks, ctypes.byref(v))
        same = same and np.array_equal(a, b) and na == nb
        visits += v.value
        total += prob.n * len(sched) * mcsteps
    return same, visits / total


_UP_DOWN = np.concatenate([np.linspace(3.0, 0.2, 30), np.linspace(0.3, 1.5, 10), np.linspace(1.5, 1e-8, 40)])

CASES = [
    # (lattice side, periodic, fields (or "kings" for a King's graph), P, schedule, T, mcsteps,
    #  global moves, betas, straight start)
    (12, True, True, 20, np.linspace(3.0, 1e-8, 120), 0.05, 1, 0, None, True),
    (12, True, False, 16, np.linspace(3.0, 1e-8, 120), 0.05, 2, 1, None, True),
    (11, True, True, 8, _UP_DOWN, 0.05, 1, 0, None, True),            # odd torus: three colours
    (10, False, True, 32, np.linspace(2.0, 1e-8, 80), 0.1, 1, 2, None, True),
    (12, True, True, 4, np.linspace(3.0, 1e-8, 60), 1.0, 1, 0,
     (1.0 / np.concatenate([np.linspace(1.0, 0.05, 30), np.full(6, 0.4), np.linspace(0.4, 0.05, 24)])), True),
    (9, True, False, 64, np.linspace(3.0, 1e-8, 60), 0.05, 1, 1, None, True),
    (12, True, True, 20, np.linspace(3.0, 1e-8, 300), 0.05, 1, 0, None, False),   # kinked start
    (12, True, "kings", 20, np.linspace(3.0, 1e-8, 120), 0.05, 1, 1, None, True),  # eight couplings
]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_skipping_quiet_sites_is_exact(k):
    L, periodic, fields, P, sched, T, mc, gm, betas, straight = CASES[k]
    prob = _problem(L, periodic, 100 + k, fields)
    same, frac = _run(prob, P, sched, T, mcsteps=mc, global_moves=gm, betas=betas, straight=straight)
    assert same
    print("case %d: %.2f of the site visits made" % (k, frac))
    # straight starts settle into quiet sites; a kinked start at T = 0.05 keeps most kinks
    assert frac < (0.8 if straight else 1.0), "the rule should skip visits here (visited %.2f)" % frac


@pytest.mark.parametrize("breaks", [1, 2, 4])
def test_each_part_of_the_rule_is_needed(breaks):
    """Without clearing neighbours' bits, with t = -2 J-perp counted as calm, or with no step
    rewriting the bits after J-perp or beta fell, some case ends in a different state."""
    differs = False
    for k in range(len(CASES)):
        L, periodic, fields, P, sched, T, mc, gm, betas, straight = CASES[k]
        prob = _problem(L, periodic, 100 + k, fields)
        same, _ = _run(prob, P, sched, T, mcsteps=mc, global_moves=gm, betas=betas, breaks=breaks,
                       straight=straight)
        if not same:
            differs = True
            break
    assert differs
