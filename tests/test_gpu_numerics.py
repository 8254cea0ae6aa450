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


def test_settle_threshold_is_exact():
    """The quiet-site threshold smin of a step: s >= smin exactly when fl(s * -2 beta) <= the settled
    bound, for s >= 0 (checked at smin and the float below it, in FP32 arithmetic)."""
    from piqmc import _device, _native
    from native import probes
    g = np.random.default_rng(3)
    betas = np.concatenate([[20.0, 1.0 / 0.05, 0.5, 1.0, 7.3, 1e-3, 1e3, 3e38, 1e-30, 0.0, -1.0],
                            np.exp(g.uniform(-12, 12, 2000))]).astype(np.float32)
    out = torch.empty(len(betas), dtype=torch.float32, device="cuda")
    _native.check(probes.lib().pqt_settle_threshold(_device.ptr(torch.from_numpy(betas).cuda()), len(betas),
                                                    _device.ptr(out), _device.stream_handle()), "probe")
    smin = out.cpu().numpy()
    X = np.array([0xc1851592], np.uint32).view(np.float32)[0]
    with np.errstate(over="ignore", invalid="ignore"):   # -2 beta overflows for beta = 3e38; 0 * -inf
        m2b = (np.float32(-2.0) * betas).astype(np.float32)
        for b, m, s in zip(betas, m2b, smin):
            if not m < 0:
                assert np.isinf(s) and s > 0, (b, s)
                continue
            assert s > 0 and np.float32(s * m) <= X, (b, s)
            below = np.nextafter(np.float32(s), np.float32(0))
            assert not np.float32(below * m) <= X, (b, s)
