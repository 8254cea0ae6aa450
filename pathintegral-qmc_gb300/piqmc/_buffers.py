"""Argument unpacking with the reference's typed-memoryview rules.

The reference's ``cpdef`` functions take ``np.float_t[:]``-style memoryviews:
any object exposing a float64 buffer of the right rank is accepted without a
copy (C or Fortran order, any strides), and anything else raises ``ValueError``
before the body runs (generated piqmc/qmc.c argument unpacking).
"""
import numpy as np


def float64_buffer(obj, ndim, name, writable=False):
    try:
        arr = np.asarray(obj)
    except Exception as exc:  # pragma: no cover - mirrors Cython's buffer error
        raise ValueError("%s: object does not expose a buffer (%s)" % (name, exc))
    if arr.dtype != np.float64:
        raise ValueError("Buffer dtype mismatch, expected 'float_t' but got '%s' (argument %s)"
                         % (arr.dtype, name))
    if arr.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d) (argument %s)"
                         % (ndim, arr.ndim, name))
    if writable and not arr.flags.writeable:
        raise ValueError("buffer source array is read-only (argument %s)" % name)
    return arr


def as_c_int(v, name):
    try:
        iv = int(v)
    except (TypeError, ValueError):
        raise TypeError("an integer is required (argument %s)" % name)
    if iv != v and not isinstance(v, (int, np.integer)):
        raise TypeError("an integer is required (argument %s)" % name)
    if not -2 ** 31 <= iv < 2 ** 31:
        raise OverflowError("value too large to convert to int (argument %s)" % name)
    return iv


def as_c_float(v, name):
    try:
        return np.float32(float(v))
    except (TypeError, ValueError):
        raise TypeError("must be real number, not %s (argument %s)" % (type(v).__name__, name))


def first_spin_order(rng, nspins):
    """``rng.permutation(range(nspins))`` taken into an int64 buffer as the reference does
    (piqmc/qmc.pyx:90-91, :194-195; piqmc/sa.pyx:91-92, :158-159).  For nspins == 0 numpy
    returns an empty float64 array (drawing nothing), and the reference's buffer assignment
    raises ValueError there, before the schedule is read."""
    cur = rng.permutation(range(nspins))
    if cur.dtype.kind not in "iu":
        raise ValueError("Buffer dtype mismatch, expected 'int_t' but got '%s' (first spin order)" % cur.dtype)
    return cur


def check_pm1(a, name):
    """The GPU kernels keep spins as int8 +-1; other values are rejected."""
    if a.size and not np.all((a == 1.0) | (a == -1.0)):
        raise ValueError("%s must hold only +1/-1 spin values" % name)


def seed_from_rng(rng):
    """A 64-bit Philox key drawn from a numpy RandomState or Generator."""
    if hasattr(rng, "integers"):
        hi, lo = rng.integers(0, 2 ** 32, size=2, dtype=np.uint64)
    else:
        hi, lo = rng.randint(0, 2 ** 32, size=2, dtype=np.uint64)
    return (int(hi) << 32) | int(lo)
