"""Drop-in for ``piqmc.tools`` (reference piqmc/tools.pyx): spin/bit conversion, the neighbour
table, the instance generators, and instance / neighbour-table file I/O."""
import ctypes

import numpy as np
import scipy.sparse as sps

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


# ------------------------------------------------------------------------------------------
# instance generators (reference piqmc/tools.pyx:98-273)
#
# Each generator first lists the (row, column) assignments the reference makes, in
# the order it makes them, then draws all their values with one vectorised
# ``rng.uniform`` call (the same MT19937 doubles, in the same order, as one scalar
# draw per assignment), then replays the assignments into a DOK matrix with the
# DOK's own semantics (a later assignment overwrites the value and keeps the key's
# position; an exact zero removes the key).  So the matrix, its key order (which
# ``GenerateNeighbors`` follows) and the state ``rng`` is left in match the
# reference's, in O(assignments) instead of the reference's O(nspins^2) scan.
# ------------------------------------------------------------------------------------------

def _replay(n, rows, cols, vals):
    d = {}
    for i, j, v in zip(rows, cols, vals.tolist()):
        if v == 0.0:
            d.pop((i, j), None)
        else:
            d[(i, j)] = v
    J = sps.dok_matrix((n, n), dtype=np.float64)
    for (i, j), v in d.items():
        J[i, j] = v
    return J


def Generate2DIsingInstance(nRows, rng):
    """Periodic nRows x nRows lattice, couplings U[-2, 2] (reference piqmc/tools.pyx:98-131).

    Assignment order of the reference, per spin ``row`` (n = nRows^2): the
    vertical wrap bond (row, row + nRows (nRows - 1)) for the first lattice row;
    then, for every column index ``col`` from ``row`` to n - 1: the horizontal
    wrap bond (row, row + nRows - 1) when ``row`` starts a lattice row (so that
    bond is drawn n - row times, the last draw kept), the right bond at
    col = row + 1 unless ``row`` ends a lattice row, and the down bond at
    col = row + nRows.
    """
    nRows = int(nRows)
    n = nRows * nRows
    rows, cols = [], []
    for row in range(n):
        if row < nRows:
            rows.append(row)
            cols.append(row + nRows * (nRows - 1))
        right = row % nRows != nRows - 1 and row + 1 < n
        down = row + nRows < n
        if row % nRows == 0:
            wrap = row + nRows - 1
            for col in range(row, n):
                rows.append(row)
                cols.append(wrap)
                if right and col == row + 1:
                    rows.append(row)
                    cols.append(col)
                if down and col == row + nRows:
                    rows.append(row)
                    cols.append(col)
        else:
            if right:
                rows.append(row)
                cols.append(row + 1)
            if down:
                rows.append(row)
                cols.append(row + nRows)
    vals = rng.uniform(low=-2, high=2, size=len(rows)) if rows else np.zeros(0)
    return _replay(n, rows, cols, vals)


def Generate2DLattice(nrows, ncols, rng, periodic=0):
    """nrows x ncols lattice, couplings U[-1e-8, 1e-8] (reference piqmc/tools.pyx:133-175).

    Per spin: the vertical wrap bond (first lattice row, periodic only), the
    horizontal wrap bond (first lattice column, periodic only), the right bond
    (unless last lattice column), the down bond (unless last lattice row).
    """
    nrows, ncols, periodic = int(nrows), int(ncols), int(periodic)
    n = nrows * ncols
    rows, cols = [], []
    for j in range(n):
        if periodic and j < ncols:
            rows.append(j)
            cols.append(j + ncols * (nrows - 1))
        if periodic and j % ncols == 0:
            rows.append(j)
            cols.append(j + ncols - 1)
        if j + 1 < n and j % ncols != ncols - 1:
            rows.append(j)
            cols.append(j + 1)
        if j + ncols < n:
            rows.append(j)
            cols.append(j + ncols)
    vals = rng.uniform(low=-1e-8, high=1e-8, size=len(rows)) if rows else np.zeros(0)
    return _replay(n, rows, cols, vals)


def GenerateKblockLattice(nrows, ncols, rng, k=1):
    """Every spin coupled to the spins on the rings of radius 1..k around it (reference piqmc/tools.pyx:177-273).

    For spin i and radius q, the ring is clipped to the lattice (q' = min(q,
    distance to each edge)); its top-left corner is tlc = i - up' ncols - left'.
    The reference assigns, in this order, the top side (tlc + r, r = 0..w - 1),
    the bottom side (same, plus up' + down' rows), the left side (tlc + r ncols)
    and the right side (tlc + w - 1 + r ncols), r = 1..up' + down' for the sides,
    w = left' + right' + 1 -- keeping only entries above the diagonal (i < idx).
    Couplings U[-1e-8, 1e-8].
    """
    nrows, ncols, k = int(nrows), int(ncols), int(k)
    n = nrows * ncols
    rows, cols = [], []
    for i in range(n):
        c = i % ncols
        to_right = (ncols - (i + 1) % ncols) if (i + 1) % ncols else 0
        for q in range(1, k + 1):
            left = min(c, q)
            right = min(to_right, q)
            up = q
            while i - up * ncols < 0:
                up -= 1
            down = q
            while i + down * ncols >= n:
                down -= 1
            tlc = max(i - up * ncols - left, 0)
            w = left + right + 1
            h = up + down
            ring = np.concatenate([tlc + np.arange(w), tlc + h * ncols + np.arange(w),
                                   tlc + ncols * np.arange(1, h + 1), tlc + w - 1 + ncols * np.arange(1, h + 1)])
            ring = ring[ring > i].tolist()
            rows.extend([i] * len(ring))
            cols.extend(ring)
    vals = rng.uniform(low=-1e-8, high=1e-8, size=len(rows)) if rows else np.zeros(0)
    return _replay(n, rows, cols, vals)


# ------------------------------------------------------------------------------------------
# the same instances generated on the GPU (neighbour table in device memory)
# ------------------------------------------------------------------------------------------

def lattice_table(kind, nrows, ncols=None, seed=0, periodic=0, k=1, maxnb=None, lo=None, hi=None, check=True):
    """Neighbour table (GenerateNeighbors layout, float64 (n, maxnb, 2)) of a generated instance, on the GPU.

    kind "ising2d" (Generate2DIsingInstance, nrows x nrows torus, U[-2, 2]), "lattice2d"
    (Generate2DLattice, U[-1e-8, 1e-8]) or "kblock" (GenerateKblockLattice, U[-1e-8, 1e-8]).
    The bonds and the order of every row are those GenerateNeighbors builds from the
    host generators; the values come from a seeded counter-based stream (not the
    caller's ``rng``), so use the host functions when the reference's values matter.
    Returns the device tensor.
    """
    import torch
    from . import _device
    kinds = {"ising2d": 0, "lattice2d": 1, "kblock": 2}
    if kind not in kinds:
        raise ValueError("kind must be one of %s" % sorted(kinds))
    kd = kinds[kind]
    nrows = int(nrows)
    ncols = nrows if ncols is None else int(ncols)
    if kd == 0 and ncols != nrows:
        raise ValueError("ising2d is square: ncols must equal nrows")
    if maxnb is None:
        maxnb = (2 * int(k) + 1) ** 2 - 1 if kd == 2 else 4
    default = (-2.0, 2.0) if kd == 0 else (-1e-8, 1e-8)
    lo = default[0] if lo is None else float(lo)
    hi = default[1] if hi is None else float(hi)
    n = nrows * ncols
    dev = _device.device()
    nbs = torch.empty((n, int(maxnb), 2), dtype=torch.float64, device=dev)
    row_len = torch.empty(n, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    _native.check(_native.lib().pq_generate_lattice_table(
        kd, nrows, ncols, int(bool(periodic)), int(k), lo, hi, int(seed) & 0xFFFFFFFFFFFFFFFF, int(maxnb),
        _device.ptr(nbs), _device.ptr(row_len), _device.ptr(status), _device.stream_handle()),
        "pq_generate_lattice_table")
    if check:
        code = int(status.item())
        if code == _native.PQ_ERR_TOO_LARGE:
            raise IndexError("a spin has more than maxnb=%d neighbours" % int(maxnb))
        if code:
            raise _native.PiqmcError(code, "pq_generate_lattice_table")
    return nbs


def Generate2DIsingInstanceTable(nRows, seed=0, maxnb=4):
    """Generate2DIsingInstance's neighbour table, generated on the GPU (values from ``seed``)."""
    return lattice_table("ising2d", nRows, seed=seed, maxnb=maxnb)


def Generate2DLatticeTable(nrows, ncols, seed=0, periodic=0, maxnb=4):
    """Generate2DLattice's neighbour table, generated on the GPU (values from ``seed``)."""
    return lattice_table("lattice2d", nrows, ncols, seed=seed, periodic=periodic, maxnb=maxnb)


def GenerateKblockLatticeTable(nrows, ncols, seed=0, k=1, maxnb=None):
    """GenerateKblockLattice's neighbour table, generated on the GPU (values from ``seed``)."""
    return lattice_table("kblock", nrows, ncols, seed=seed, k=k, maxnb=maxnb)


# ------------------------------------------------------------------------------------------
# instance and neighbour-table files
# ------------------------------------------------------------------------------------------

def LoadIsingInstance(fname, nspins=None):
    """An instance text file of ``i j J`` lines with 1-based spin indices, as a DOK matrix.

    The format of the reference's instance files, read as its examples do
    (examples/santoro80.py:265-268): entry (i - 1, j - 1) = J, file order is DOK
    key order (a repeated pair keeps its first position and its last value).
    ``nspins`` defaults to the largest index in the file.
    """
    data = np.loadtxt(fname, ndmin=2)
    if data.size == 0:
        return sps.dok_matrix((int(nspins or 0), int(nspins or 0)), dtype=np.float64)
    if data.shape[1] != 3:
        raise ValueError("%s: expected 3 columns (i j J), got %d" % (fname, data.shape[1]))
    ij = data[:, :2]
    if np.any(ij != np.round(ij)) or np.any(ij < 1):
        raise ValueError("%s: spin indices must be integers >= 1" % fname)
    ii = ij.astype(np.int64) - 1
    n = int(nspins) if nspins is not None else int(ii.max()) + 1
    if ii.max() >= n:
        raise ValueError("%s: spin index %d > nspins=%d" % (fname, int(ii.max()) + 1, n))
    return _replay(n, ii[:, 0].tolist(), ii[:, 1].tolist(), data[:, 2].copy())


def LoadNeighbors(path):
    """A neighbour table saved by ``GenerateNeighbors(..., savepath)`` (``np.save`` of the
    float64 (nspins, maxnb, 2) table, reference piqmc/tools.pyx:94-95)."""
    nbs = np.load(path)
    if nbs.dtype != np.float64 or nbs.ndim != 3 or nbs.shape[2] != 2:
        raise ValueError("%s: not a neighbour table (float64, shape (nspins, maxnb, 2))" % path)
    return nbs
