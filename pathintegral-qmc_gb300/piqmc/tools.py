"""Drop-in for ``piqmc.tools`` (reference piqmc/tools.pyx): spin/bit conversion and the neighbour table."""
import ctypes

import numpy as np

from . import _native


def bits2spins(vec):
    """Convert a bitvector to a spin vector: 1 -> -1, else +1 (reference piqmc/tools.pyx:20-22)."""
    return [-1 if k == 1 else 1 for k in vec]


def spins2bits(vec):
    """Convert a spin vector to a bitvector: +1 -> 0, else 1 (reference piqmc/tools.pyx:24-26)."""
    return [0 if k == 1 else 1 for k in vec]


def GenerateNeighbors(nspins, J, maxnb, savepath=None):
    """Neighbour table ``nbs[i, m] = [neighbour index, coupling]``, float64 (nspins, maxnb, 2).

    Reference: piqmc/tools.pyx:28-96.  Rows list, in the matrix's DOK key order,
    ``[j, J]`` for every key (i, j) and ``[i, J]`` for every key (j, i); a diagonal
    key (i, i) appears once.  Unused slots stay [0, 0].  Built by the native
    library in one pass over the keys (the reference rescans all keys for every
    spin).  Raises IndexError when a spin needs more than ``maxnb`` slots, as the
    bounds-checked reference does.  Returns an ndarray (the reference returns a
    memoryview over the same data layout).
    """
    nspins = int(nspins)
    maxnb = int(maxnb)
    if nspins < 0 or maxnb < 0:
        raise ValueError("nspins and maxnb must be non-negative")
    D = J.todok()
    items = list(D.items())
    nk = len(items)
    rows = np.fromiter((k[0] for k, _ in items), dtype=np.int64, count=nk)
    cols = np.fromiter((k[1] for k, _ in items), dtype=np.int64, count=nk)
    vals = np.fromiter((v for _, v in items), dtype=np.float64, count=nk)
    out = np.zeros((nspins, maxnb, 2), dtype=np.float64)
    if nspins and maxnb:
        st = _native.lib().pq_generate_neighbors(
            nspins, nk, ctypes.c_void_p(rows.ctypes.data), ctypes.c_void_p(cols.ctypes.data),
            ctypes.c_void_p(vals.ctypes.data), maxnb, ctypes.c_void_p(out.ctypes.data))
        if st == _native.PQ_ERR_TOO_LARGE:
            raise IndexError("Out of bounds on buffer access (axis 1)")
        _native.check(st, "pq_generate_neighbors")
    elif nk and maxnb == 0:
        # any matching key would overflow a zero-width row
        if np.any((rows >= 0) & (rows < nspins)) or np.any((cols >= 0) & (cols < nspins)):
            raise IndexError("Out of bounds on buffer access (axis 1)")
    if savepath is not None:
        np.save(savepath, out)
    return out
