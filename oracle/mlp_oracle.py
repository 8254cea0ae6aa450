"""CPU restatement of the proposal MLP's forward and backward -- TEST INFRASTRUCTURE ONLY.

FP64 arithmetic with BF16 rounding (round to nearest even) applied at the same
points as the GPU path: the GEMM operands (features, the first hidden layer after
ReLU, the upstream gradients dH2 and dH1, and the weights) are BF16; every
accumulation is exact here and FP32 on the GPU, so gradients agree to FP32/BF16
rounding, not bit for bit.
"""
import numpy as np


def bf16(x):
    """Round to BF16 (nearest even) and return as float64."""
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    b = x32.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, X):
    """p: FP32 parameters (dict of arrays); X: (B, 8) features.  Returns logits and intermediates."""
    Xb = bf16(X)
    W1 = bf16(p["W1"])
    W2 = bf16(p["W2"])
    H1 = Xb @ W1.T + p["b1"]
    H1b = bf16(np.maximum(H1, 0.0))
    H2 = H1b @ W2.T + p["b2"]
    logit = np.maximum(H2, 0.0) @ p["w3"].astype(np.float64) + float(p["b3"][0])
    return logit, (Xb, H1, H1b, H2)


def gradients(p, X, y):
    """Mean BCE of sigmoid(logit) against soft targets y, and its gradients."""
    B = X.shape[0]
    logit, (Xb, H1, H1b, H2) = forward(p, X)
    z = logit
    prob = 1.0 / (1.0 + np.exp(-z))
    loss = np.mean(np.maximum(z, 0.0) - z * y + np.log1p(np.exp(-np.abs(z))))
    dl = (prob - y) / B
    g = {}
    g["w3"] = np.maximum(H2, 0.0).T @ dl
    g["b3"] = np.array([dl.sum()])
    dH2 = bf16(np.where(H2 > 0.0, dl[:, None] * p["w3"][None, :].astype(np.float64), 0.0))
    g["W2"] = dH2.T @ H1b
    g["b2"] = dH2.sum(0)
    G = dH2 @ bf16(p["W2"])
    gh1 = np.where(H1 > 0.0, G, 0.0)
    g["b1"] = gh1.sum(0)
    g["W1"] = bf16(gh1).T @ Xb
    return loss, g
