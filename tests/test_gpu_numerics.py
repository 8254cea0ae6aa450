"""Exhaustive numerical checks of the kernels' exact fast paths (all on the GPU)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_guard_band_covers_hardware_exp2():
    """Every FP32 argument in [-87, 0]: the hardware 2^x stays far inside the 1e-4 guard band."""
    from piqmc import _device, _native
    from native import probes
    L = probes.lib()
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    lo = 0x80000000  # -0.0; more negative floats have larger patterns
    hi = int(np.array([-87.0], np.float32).view(np.uint32)[0])
    step = 1 << 28
    b = lo
    while b <= hi:
        cnt = min(step, hi - b + 1)
        _native.check(L.pqt_guard_band_probe(b, cnt, _device.ptr(out), _device.stream_handle()), "probe")
        b += cnt
    torch.cuda.synchronize()
    worst = float(np.array([out.item()], dtype=np.int64).view(np.float64)[0])
    # argument rounding adds < 1.7e-5 on top of this; the band is 1e-4
    print("max relative deviation of the hardware 2^x from expf_neg: %.3g" % worst)
    assert worst < 5e-5, worst
