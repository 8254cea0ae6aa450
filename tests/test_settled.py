"""The settled-decision rule of the packed sweeps (csrc/sweep_core.cuh, site_visit and the quiet sites).

The packed sweep settles an update without its uniform when sum < 0 (flip) or when
fl(sum * -2 beta) <= -16.63553237915039 (reject).  The second rule is exact only
because (i) the smallest uniform is 2^-24 and (ii) expf_neg is at most 2^-24 on
every FP32 argument at or below that threshold.  Both facts are checked here on the
oracle's exp, which the GPU's expf_neg matches bit for bit."""
import numpy as np

import oracle

SETTLED_X = np.uint32(0xC1851592).view(np.float32)
TWO_M24 = np.float32(2.0 ** -24)


def test_threshold_value():
    assert float(SETTLED_X) == -16.63553237915039


def test_uniform_range_and_grid():
    assert oracle.u01(0) == TWO_M24
    assert oracle.u01(0x1FF) == TWO_M24                     # the low 9 bits are dropped
    assert oracle.u01(0xFFFFFFFF) == np.float32(1.0) - TWO_M24
    g = np.random.default_rng(0)
    for r in g.integers(0, 2 ** 32, size=2000, dtype=np.uint64):
        m = int(r) >> 9
        assert oracle.u01(int(r)) == np.float32((2 * m + 1) * 2.0 ** -24)


def test_exp_at_or_below_threshold_never_beats_smallest_uniform():
    # every FP32 argument in [-87, SETTLED_X]; below -87 expf_neg returns 0
    assert oracle.expf_neg_max(SETTLED_X, -87.0) <= TWO_M24
    assert oracle.expf_neg(np.float32(-87.5)) == 0.0
    assert oracle.expf_neg(np.float32(-1e30)) == 0.0


def test_threshold_is_tight():
    # the next FP32 value towards zero is no longer settled
    nxt = (SETTLED_X.view(np.uint32) - np.uint32(1)).view(np.float32)
    assert oracle.expf_neg(nxt) > TWO_M24
