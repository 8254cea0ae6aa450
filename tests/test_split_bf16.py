"""The split-BF16 coupling operand of the dense fast path (piqmc/dense.py), modelled on the CPU
with torch's round-to-nearest BF16 conversion: K_hi = bf16(K), K_lo = bf16(K - K_hi).

* every FP32 coupling is carried to within 2^-17 of itself (relative), the bound the module
  states: |K - K_hi| <= 2^(e-8) for a leading bit 2^e, so the remainder's leading bit is at
  most 2^(e-9) unless it is a power of two (then K_lo holds it exactly);
* the field recompute f = h + (K_hi + K_lo) s with +-1 spins and FP32 accumulation stays
  far inside the tolerance the GPU test applies (1e-4 of max(1, |f|)) on N(0, 1/N)
  couplings, where a single BF16 operand would not."""
import numpy as np
import torch


def _split(K32):
    hi = K32.to(torch.bfloat16)
    lo = (K32 - hi.float()).to(torch.bfloat16)
    return hi, lo


def test_split_carries_16_bits():
    g = np.random.default_rng(0)
    x = (g.normal(0, 1, 2_000_000) * np.exp(g.uniform(-30, 30, 2_000_000))).astype(np.float32)
    x = np.concatenate([x, np.float32(2.0) ** np.arange(-60, 60, dtype=np.float32),
                        np.nextafter(np.float32(1.0), np.float32(2.0)) * np.float32(2.0) ** np.arange(-20, 20)])
    K = torch.from_numpy(x)
    hi, lo = _split(K)
    err = (K.double() - hi.double() - lo.double()).abs()
    assert bool((err <= K.double().abs() * 2.0 ** -17).all())
    # a single BF16 operand keeps only about 8 bits
    assert float(((K.double() - hi.double()).abs() / K.double().abs()).max()) > 2.0 ** -10


def test_field_recompute_error_model():
    g = np.random.default_rng(1)
    N, C = 512, 256
    up = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1).astype(np.float32)
    K = torch.from_numpy(up + up.T)
    h = torch.from_numpy(g.normal(0.0, 0.3, N).astype(np.float32))
    S = torch.from_numpy(np.where(g.random((C, N)) < 0.5, -1.0, 1.0).astype(np.float32))
    exact = S.double() @ K.double().T + h.double()
    hi, lo = _split(K)
    split = (S @ hi.float().T + S @ lo.float().T) + h           # FP32 products of exact values
    single = S @ hi.float().T + h
    scale = max(1.0, float(exact.abs().max()))
    err_split = float((split.double() - exact).abs().max())
    err_single = float((single.double() - exact).abs().max())
    assert err_split <= 1e-4 * scale / 4, (err_split, scale)
    assert err_single > 1e-4 * scale, (err_single, scale)
