"""Shared helpers of the test-suite (fixtures loading, seeded instances)."""
import os

import numpy as np
import scipy.sparse as sps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def dok_from(rows, cols, vals, n):
    J = sps.dok_matrix((int(n), int(n)), dtype=np.float64)
    for a, b, v in zip(rows, cols, vals):
        J[int(a), int(b)] = float(v)
    return J


def lattice(L, periodic, rng, dist=None, fields=None):
    """Seeded L x L lattice as a DOK matrix (right and down bonds)."""
    dist = dist or (lambda r: r.uniform(-2.0, 2.0))
    n = L * L
    J = sps.dok_matrix((n, n), dtype=np.float64)
    for y in range(L):
        for x in range(L):
            i = y * L + x
            if periodic or x + 1 < L:
                J[i, y * L + (x + 1) % L] = dist(rng)
            if periodic or y + 1 < L:
                J[i, ((y + 1) % L) * L + x] = dist(rng)
    if fields is not None:
        for i in range(n):
            J[i, i] = fields(rng)
    return J
