"""Learned world-line proposals with an exact Metropolis-Hastings correction.

``ProposalMLP`` is an 8 -> 64 -> 64 -> 1 ReLU network.  Its weights are kept in
FP32 (the trained parameters) and used as BF16 copies by the tensor-core GEMMs
(FP32 accumulation); forward and backward both run on the GPU:

* forward: H1 = X W1^T + b1 (tcgen05 GEMM), relu -> BF16, H2 = H1 W2^T + b2
  (tcgen05 GEMM), logit = relu(H2) . w3 + b3;
* backward (binary cross-entropy against soft targets): dW2 = dH2^T H1 and
  dW1 = dH1^T X are tcgen05 GEMMs over the batch, dH1 = dH2 W2 as well;
  Adam updates the FP32 parameters.

``learned_pass`` runs one world-line move per spin with the network choosing
which spins to try; by default every class is one launch of the fused kernel
(features, both layers as tcgen05 MMAs with TMEM accumulators, head and MH
decision without leaving the SM), the unfused path (feature kernel, two GEMMs,
head, propose) giving the same moves.  Update classes are visited in order; for every spin of a
class, the features of its current world-line and of the flipped one are scored,
the flip is proposed with q = clamp(sigmoid(logit), qmin, 1) and accepted with
min(1, exp(-beta dE) q'/q).  Spins of one class share no coupling, so a flip
never changes another class member's features during the phase: the reverse
proposal probability q' is exactly what the network would give in the new
state, and detailed balance holds.  ``uniform_pass`` is the same move with
q = 1 (every spin tried), the plain form the learned one is judged against;
its default kernel computes only the flip cost.

Training data: ``record_moves`` scores the moves the plain method tries at
snapshots of plain anneals -- features and their Metropolis acceptance
probabilities min(1, exp(-beta dE)) -- and ``train`` fits the network to them.
"""
import ctypes

import numpy as np
import torch

from . import _device, _native
from .tensor import gemm_bf16

HID = 64
NFEAT = 8


def _pad(x, m):
    return (x + m - 1) // m * m


class ProposalMLP:
    def __init__(self, seed=0, device=None):
        dev = device or _device.device()
        g = np.random.default_rng(seed)
        lim1, lim2, lim3 = np.sqrt(6.0 / NFEAT), np.sqrt(6.0 / HID), np.sqrt(3.0 / HID)
        p = {
            "W1": g.uniform(-lim1, lim1, (HID, NFEAT)),
            "b1": np.zeros(HID),
            "W2": g.uniform(-lim2, lim2, (HID, HID)),
            "b2": np.zeros(HID),
            "w3": g.uniform(-lim3, lim3, HID),
            "b3": np.zeros(1),
        }
        self.params = {k: torch.tensor(v, dtype=torch.float32, device=dev) for k, v in p.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.t = 0
        self.device = dev
        self.refresh()

    def refresh(self):
        """BF16 operands of the GEMMs from the FP32 parameters."""
        W1p = torch.zeros((HID, HID), dtype=torch.float32, device=self.device)
        W1p[:, :NFEAT] = self.params["W1"]
        self.W1b = W1p.to(torch.bfloat16).contiguous()
        self.W2b = self.params["W2"].to(torch.bfloat16).contiguous()
        self.W2Tb = self.params["W2"].t().contiguous().to(torch.bfloat16)
        self.b3_host = float(self.params["b3"][0].item())

    def state_dict(self):
        return {k: v.detach().cpu().numpy().copy() for k, v in self.params.items()}

    def load_state_dict(self, d):
        for k, v in d.items():
            self.params[k].copy_(torch.as_tensor(v, dtype=torch.float32))
        self.refresh()

    # --------------------------------------------------------------------------------------
    def forward(self, X, keep=False):
        """logits for BF16 rows X (rows x 64, features in the first 8 columns, rows % 128 == 0)."""
        lib = _native.lib()
        rows = X.shape[0]
        H1 = gemm_bf16(X, self.W1b, bias=self.params["b1"])
        H1b = torch.empty((rows, HID), dtype=torch.bfloat16, device=X.device)
        _native.check(lib.pq_mlp_relu_bf16(_device.ptr(H1), _device.ptr(H1b), H1.numel(), _device.stream_handle()),
                      "pq_mlp_relu_bf16")
        H2 = gemm_bf16(H1b, self.W2b, bias=self.params["b2"])
        logit = torch.empty(rows, dtype=torch.float32, device=X.device)
        _native.check(lib.pq_mlp_head(_device.ptr(H2), _device.ptr(self.params["w3"]), float(self.params["b3"].item()),
                                      _device.ptr(logit), rows, _device.stream_handle()), "pq_mlp_head")
        if keep:
            self._cache = (X, H1, H1b, H2, logit)
        return logit

    def gradients(self, X, y):
        """Loss and gradients of the mean BCE of sigmoid(logit(X)) against y (batch % 128 == 0)."""
        lib = _native.lib()
        B = X.shape[0]
        dev = X.device
        logit = self.forward(X, keep=True)
        _, H1, H1b, H2, _ = self._cache
        g = {k: torch.zeros_like(v) for k, v in self.params.items()}
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        dH2 = torch.empty((B, HID), dtype=torch.bfloat16, device=dev)
        dH2T = torch.zeros((128, B), dtype=torch.bfloat16, device=dev)     # rows 64..127 stay zero
        st = _device.stream_handle()
        _native.check(lib.pq_mlp_head_backward(_device.ptr(H2), _device.ptr(logit), _device.ptr(y),
                                               _device.ptr(self.params["w3"]), B, _device.ptr(dH2), _device.ptr(dH2T),
                                               _device.ptr(g["w3"]), _device.ptr(g["b3"]), _device.ptr(loss), st),
                      "pq_mlp_head_backward")
        H1bT = torch.empty((HID, B), dtype=torch.bfloat16, device=dev)
        _native.check(lib.pq_mlp_transpose_bf16(_device.ptr(H1b), B, _device.ptr(H1bT), st), "transpose")
        g["W2"].copy_(gemm_bf16(dH2T, H1bT)[:HID])
        _native.check(lib.pq_mlp_colsum_bf16(_device.ptr(dH2T), HID, B, _device.ptr(g["b2"]), st), "colsum")
        G = gemm_bf16(dH2, self.W2Tb)
        dH1T = torch.zeros((128, B), dtype=torch.bfloat16, device=dev)
        _native.check(lib.pq_mlp_hidden_backward(_device.ptr(G), _device.ptr(H1), B, _device.ptr(dH1T),
                                                 _device.ptr(g["b1"]), st), "hidden_backward")
        XT = torch.empty((HID, B), dtype=torch.bfloat16, device=dev)
        _native.check(lib.pq_mlp_transpose_bf16(_device.ptr(X), B, _device.ptr(XT), st), "transpose")
        g["W1"].copy_(gemm_bf16(dH1T, XT)[:HID, :NFEAT])
        return float(loss.item()), g

    def step(self, g, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        lib = _native.lib()
        self.t += 1
        for k, p in self.params.items():
            _native.check(lib.pq_adam(_device.ptr(p), _device.ptr(g[k]), _device.ptr(self.m[k]), _device.ptr(self.v[k]),
                                      p.numel(), float(lr), float(b1), float(b2), float(eps), self.t,
                                      _device.stream_handle()), "pq_adam")
        self.refresh()

    def train(self, X, y, epochs=3, batch=8192, lr=2e-3, seed=0):
        """Fit to recorded moves X (N x 64 BF16), y (N FP32 soft targets); returns the loss history."""
        N = (X.shape[0] // batch) * batch
        if N == 0:
            raise ValueError("need at least one batch of %d samples" % batch)
        gen = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for _ in range(epochs):
            order = torch.randperm(X.shape[0], generator=gen)[:N].to(X.device)
            for b0 in range(0, N, batch):
                idx = order[b0:b0 + batch]
                loss, g = self.gradients(X[idx].contiguous(), y[idx].contiguous())
                self.step(g, lr=lr)
                hist.append(loss)
        return hist


class _Buffers:
    def __init__(self):
        self.X = None
        self.dE = None

    def get(self, Mpad, dev):
        if self.X is None or self.X.shape[0] < 2 * Mpad:
            self.X = torch.zeros((2 * Mpad, HID), dtype=torch.bfloat16, device=dev)
            self.dE = torch.empty(Mpad, dtype=torch.float32, device=dev)
        return self.X[:2 * Mpad], self.dE[:Mpad]


_bufs = _Buffers()


def _features(problem, words, P, cls, beta, jp, X, dE, Mpad):
    R = words.shape[0]
    bits = 32 if P <= 32 else 64
    _native.check(_native.lib().pq_mlp_features(
        _device.ptr(words), bits, problem.nslots, P, R, problem.maxdeg, _device.ptr(problem.nbr),
        _device.ptr(problem.cpl), _device.ptr(problem.field), cls, problem.class_stride,
        int(problem.class_size[cls]), float(beta), float(jp), _device.ptr(X), _device.ptr(dE), Mpad,
        _device.stream_handle()), "pq_mlp_features")


_status = {}


def _status_buffer(dev):
    buf = _status.get(dev)
    if buf is None:
        buf = _status[dev] = torch.zeros(1, dtype=torch.int32, device=dev)
    return buf


def check_status(device=None):
    """Raise if a fused learned move gave up on a tensor-core wait since the last check."""
    buf = _status_buffer(device or _device.device())
    code = int(buf.item())
    if code:
        buf.zero_()
        raise _native.PiqmcError(code, "pq_mlp_learned_move")


def learned_pass(problem, words, P, mlp, beta, jp, seed, move, qmin=0.05, counters=None, uniform=False, fused=True,
                 check=True):
    """One world-line move per spin, class by class (see module docstring); in place on ``words``.

    ``check=False`` leaves the device status unread (no host sync); ``check_status`` reads it later.
    """
    R = words.shape[0]
    bits = 32 if P <= 32 else 64
    lib = _native.lib()
    st = _device.stream_handle()
    key = int(seed) & 0xFFFFFFFFFFFFFFFF
    mv = int(move) & 0xFFFFFFFF
    if fused:
        sizes = problem.class_size.ctypes.data_as(ctypes.c_void_p)
        args = (_device.ptr(words), bits, problem.nslots, P, R, problem.maxdeg, _device.ptr(problem.nbr),
                _device.ptr(problem.cpl), _device.ptr(problem.field), problem.nclass, problem.class_stride, sizes)
        if uniform:
            _native.check(lib.pq_worldline_pass(*args, float(beta), mv, key, 0, _device.ptr(counters), st),
                          "pq_worldline_pass")
            return
        status = _status_buffer(words.device)
        _native.check(lib.pq_mlp_learned_pass(
            *args, float(beta), float(jp), _device.ptr(mlp.W1b), _device.ptr(mlp.W2b), _device.ptr(mlp.params["b1"]),
            _device.ptr(mlp.params["b2"]), _device.ptr(mlp.params["w3"]), mlp.b3_host, float(qmin), mv, key, 0,
            _device.ptr(counters), _device.ptr(status), st), "pq_mlp_learned_pass")
        if check:
            check_status(words.device)
        return
    for cls in range(problem.nclass):
        csize = int(problem.class_size[cls])
        M = R * csize
        Mpad = _pad(M, 128)
        X, dE = _bufs.get(Mpad, words.device)
        _features(problem, words, P, cls, beta, jp, X, dE, Mpad)
        if uniform:
            logit = torch.full((2 * Mpad,), 40.0, dtype=torch.float32, device=words.device)   # q = q' = 1
        else:
            logit = mlp.forward(X)
        _native.check(lib.pq_mlp_propose(
            _device.ptr(words), bits, problem.nslots, P, R, cls, problem.class_stride, csize, _device.ptr(logit),
            _device.ptr(dE), Mpad, float(qmin), float(beta), mv, key, 0, _device.ptr(counters), st), "pq_mlp_propose")


def uniform_pass(problem, words, P, beta, jp, seed, move, counters=None, fused=True):
    learned_pass(problem, words, P, None, beta, jp, seed, move, counters=counters, uniform=True, fused=fused)


def record_moves(problem, words, P, beta, jp, max_rows=None):
    """Features of every world-line move the plain method tries now, with its Metropolis acceptance probability."""
    R = words.shape[0]
    Xs, ys = [], []
    for cls in range(problem.nclass):
        csize = int(problem.class_size[cls])
        M = R * csize
        Mpad = _pad(M, 128)
        X, dE = _bufs.get(Mpad, words.device)
        _features(problem, words, P, cls, beta, jp, X, dE, Mpad)
        Xs.append(X[:M].clone())
        ys.append(torch.clamp(torch.exp(-float(beta) * dE[:M]), max=1.0))
    X = torch.cat(Xs)
    y = torch.cat(ys)
    if max_rows is not None and X.shape[0] > max_rows:
        idx = torch.randperm(X.shape[0], device=X.device)[:max_rows]
        X, y = X[idx], y[idx]
    return X, y
