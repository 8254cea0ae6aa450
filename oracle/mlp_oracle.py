"""CPU restatement of the proposal MLP's features, forward and backward -- TEST INFRASTRUCTURE ONLY.

The reference has no learned proposals (its moves are piqmc/qmc.pyx:83-123, local
and world-line flips with uniform proposals); this module restates the GPU
path's own definitions so its kernels can be checked.

``features`` is FP32, operation for operation as the device computes them
(every product and sum rounded to FP32 in the same order), so it matches the
feature kernel bit for bit.

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


_POPC8 = np.array([bin(v).count("1") for v in range(256)], dtype=np.int64)


def _popc(x):
    x = np.asarray(x, dtype=np.uint64)
    c = np.zeros(x.shape, dtype=np.int64)
    for b in range(8):
        c += _POPC8[((x >> np.uint64(8 * b)) & np.uint64(0xFF)).astype(np.int64)]
    return c


def features(words, P, nbr, cpl, field, cls, stride, csize, beta, jp):
    """Features (M, 8) FP32 and world-line flip costs dE (M,) of every spin of class ``cls``.

    words: (R, nslots) packed world-lines (bit k = spin -1 in slice k); nbr / cpl:
    (maxdeg, nslots) neighbour slots and couplings (padding: the spin itself with
    coupling 0); field: (nslots,).  Row t = r * csize + s is spin cls * stride + s
    of replica r.  Sums over slices come from popcounts:
    sum_k t^k = P - 2 popc(w), sum_k s^k t^k = P - 2 popc(w_i ^ w_m).
    """
    f32 = np.float32
    W = np.asarray(words)
    W = (W.astype(np.int64) & 0xFFFFFFFF).astype(np.uint64) if W.dtype.itemsize == 4 else W.view(np.uint64)
    R, NS = W.shape
    D = nbr.shape[0]
    mask = np.uint64((1 << P) - 1) if P < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    r = np.repeat(np.arange(R), csize)
    i = cls * stride + np.tile(np.arange(csize), R)
    wi = W[r, i] & mask
    h = np.asarray(field, dtype=f32)[i]
    J = [np.asarray(cpl[m], dtype=f32)[i] for m in range(D)]
    nb = []
    for m in range(D):
        j = np.asarray(nbr[m])[i]
        nb.append(W[r, np.where((j >= 0) & (j < NS), j, i)])
    Pf = f32(P)

    def tsum(x):
        return (P - 2 * _popc(x & mask)).astype(f32)

    scale = f32(1.0) + np.abs(h)
    s1 = Pf * h
    s2 = Pf * (h * h)
    h2 = f32(2.0) * h
    for m in range(D):
        scale = scale + np.abs(J[m])
        tm = tsum(nb[m])
        s1 = s1 + J[m] * tm
        s2 = s2 + (h2 * J[m]) * tm
        s2 = s2 + (J[m] * J[m]) * Pf
        for l in range(m):
            s2 = s2 + (f32(2.0) * (J[m] * J[l])) * tsum(nb[m] ^ nb[l])
    sa = h * tsum(wi)
    for m in range(D):
        sa = sa + J[m] * tsum(wi ^ nb[m])
    inv = f32(1.0) / Pf
    mean = s1 * inv
    var = np.fmax(s2 * inv - mean * mean, f32(0.0))
    rot = ((wi >> np.uint64(1)) | (wi << np.uint64(P - 1))) & mask
    dE = f32(2.0) * sa
    X = np.empty((R * csize, 8), dtype=f32)
    X[:, 0] = mean / scale
    X[:, 1] = np.sqrt(var) / scale
    X[:, 2] = tsum(wi) * inv
    X[:, 3] = _popc(wi ^ rot).astype(f32) * inv
    X[:, 4] = (sa * inv) / scale
    X[:, 5] = np.fmin(np.fmax((f32(beta) * dE) * inv, f32(-8.0)), f32(8.0))
    X[:, 6] = np.fmin(np.fmax((f32(jp) * f32(beta)) * inv, f32(0.0)), f32(8.0))
    X[:, 7] = 1.0
    return X, dE


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
