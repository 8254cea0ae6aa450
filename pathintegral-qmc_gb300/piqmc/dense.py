"""Dense-J fast path: local fields on the tensor cores, rank-1 updates in the sweep.

``DenseProblem`` holds a dense instance the way ``qmc.QuantumAnneal_dense``
reads it (reference piqmc/qmc.pyx:206-219): the upper triangle of ``J`` holds
the couplings, the diagonal the fields.  On the device it keeps

* K, the symmetric FP32 coupling matrix with a zero diagonal (for the sweep's
  rank-1 field updates);
* the split-BF16 form of K for the tensor cores: K = K_hi + K_lo with
  K_hi = bf16(K), K_lo = bf16(K - K_hi), stored side by side as one (Npad x 2 Npad)
  operand, so a single GEMM with [s | s] rows gives K_hi s + K_lo s;
* h, the fields (the GEMM's bias).

``fields`` recomputes f = h + K s for every (replica, slice) with one tcgen05
GEMM; ``anneal`` alternates that recompute with ``recompute_every`` field steps
of the dense sweep (``csrc/dense.cu``), which keeps f in shared memory and
updates it on every accepted flip.

Accuracy of the recompute against FP64: K_hi + K_lo carries 16 significant
bits of each FP32 coupling (relative error <= 2^-17), and the tensor cores
accumulate the exact BF16 x (+-1) products in FP32; the test suite measures
max |f_gemm - f_fp64| on N(0, 1/N) couplings (see ``field_error``).
"""
import math

import numpy as np
import torch

from . import _device, _native, tensor
from .reforder import jperp_schedule
from .tensor import gemm_bf16


def _pad(x, m):
    return (x + m - 1) // m * m


class DenseProblem:
    def __init__(self, J):
        J = np.asarray(J, dtype=np.float64)
        if J.ndim != 2 or J.shape[0] != J.shape[1]:
            raise ValueError("J must be a square matrix")
        N = J.shape[0]
        self.N = N
        self.Npad = _pad(N, 64)
        up = np.triu(J, 1)
        K = up + up.T
        self.K64 = K
        self.h64 = np.diag(J).copy()
        self.J64 = J
        dev = _device.device()
        K32 = torch.from_numpy(K.astype(np.float32))
        k_hi = K32.to(torch.bfloat16)
        k_lo = (K32 - k_hi.float()).to(torch.bfloat16)
        B = torch.zeros((self.Npad, 2 * self.Npad), dtype=torch.bfloat16)
        B[:N, :N] = k_hi
        B[:N, self.Npad:self.Npad + N] = k_lo
        self.K = K32.to(dev).contiguous()
        self.B = B.to(dev)
        h = torch.zeros(self.Npad, dtype=torch.float32)
        h[:N] = torch.from_numpy(self.h64.astype(np.float32))
        self.h = h.to(dev)
        units = [a for a in range(1, max(N, 2)) if math.gcd(a, N) == 1] if N > 1 else [0]
        self.units = torch.tensor(units, dtype=torch.int32, device=dev)
        # CSR of J as given, for the FP64 energy pass (ClassicalIsingEnergy semantics)
        rows, cols = np.nonzero(J)
        self.csr_ptr = torch.from_numpy(np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=N))]).astype(np.int64)).to(dev)
        self.csr_col = torch.from_numpy(cols.astype(np.int32)).to(dev)
        self.csr_val = torch.from_numpy(J[rows, cols].astype(np.float64)).to(dev)
        self._status = _device.Status()   # timed-out waits of the sweep

    # --------------------------------------------------------------------------------------
    def pack(self, spins):
        """int8 (R, N, P) +-1 -> uint32 words (R, N) as int32, bit k = spin -1 in slice k."""
        sp = torch.as_tensor(spins).to(_device.device(), torch.int8).contiguous()
        R, N, P = sp.shape
        if N != self.N or P > 32:
            raise ValueError("spins must be (R, %d, P<=32)" % self.N)
        words = torch.zeros((R, N), dtype=torch.int32, device=sp.device)
        _native.check(_native.lib().pq_pack_spins(_device.ptr(sp), N, P, R, None, _device.ptr(words), 32, N,
                                                   _device.stream_handle()), "pq_pack_spins")
        return words

    def unpack(self, words, P):
        R = words.shape[0]
        out = torch.empty((R, self.N, P), dtype=torch.int8, device=words.device)
        _native.check(_native.lib().pq_unpack_spins(_device.ptr(words), 32, self.N, P, R, None, self.N,
                                                     _device.ptr(out), _device.stream_handle()), "pq_unpack_spins")
        return out

    def fields(self, words, P, out=None, scratch=None, check=True):
        """f = h + K s for every configuration c = r*P + k: FP32 (Mpad, Npad), rows c < R*P valid."""
        R = words.shape[0]
        Mpad = _pad(R * P, 128)
        if scratch is None or scratch.shape != (Mpad, 2 * self.Npad):
            scratch = torch.empty((Mpad, 2 * self.Npad), dtype=torch.bfloat16, device=words.device)
        _native.check(_native.lib().pq_dense_unpack_bf16(_device.ptr(words), self.N, P, R, self.Npad, Mpad,
                                                           _device.ptr(scratch), _device.stream_handle()),
                      "pq_dense_unpack_bf16")
        return gemm_bf16(scratch, self.B, bias=self.h, out=out, check=check), scratch

    def energies(self, words, P):
        """FP64 energy of every (replica, slice), exactly sa.ClassicalIsingEnergy's definition."""
        R = words.shape[0]
        out = torch.empty((R, P), dtype=torch.float64, device=words.device)
        _native.check(_native.lib().pq_energy_packed(_device.ptr(words), 32, self.N, P, R, _device.ptr(self.csr_ptr),
                                                      _device.ptr(self.csr_col), _device.ptr(self.csr_val),
                                                      _device.ptr(out), _device.stream_handle()), "pq_energy_packed")
        return out

    def sweep(self, words, F, P, jperp, beta, seed, mcsteps=1, sweep_base=0, replica_base=0, accepts=None,
              per_slice_order=False, status=None, poll_limit=-1, wait_skew=0):
        """Dense sweeps of every replica through len(jperp) field steps starting from fields F (updated in place).

        The spin order of a sweep is shared by every slice (as in the reference) unless
        ``per_slice_order`` -- which anneals faster but with different dynamics.
        ``poll_limit`` bounds each wavefront wait (< 0: the kernel's default);
        ``wait_skew`` > 0 makes every wait run to that bound (to test the timeout path).
        """
        R = words.shape[0]
        _native.check(_native.lib().pq_dense_sweep_ex(
            _device.ptr(words), _device.ptr(F), F.stride(0), _device.ptr(self.K), _device.ptr(self.units),
            self.units.numel(), _device.ptr(jperp), self.N, int(P), R, int(jperp.numel()), int(mcsteps),
            float(np.float32(beta)), int(seed) & 0xFFFFFFFFFFFFFFFF, int(sweep_base), int(replica_base),
            int(bool(per_slice_order)), int(poll_limit), int(wait_skew), _device.ptr(accepts),
            (status or self._status).ptr, _device.stream_handle()), "pq_dense_sweep")

    def anneal(self, words, sched, P, temp, seed=0, mcsteps=1, recompute_every=50, accepts=None,
               per_slice_order=False, check=True):
        """Anneal packed replicas in place: GEMM field recompute, then up to ``recompute_every`` steps.

        ``check`` reads the GEMMs' device status once at the end (one host synchronisation)."""
        jp = torch.from_numpy(jperp_schedule(sched, P, temp) if P > 1 else np.zeros(len(sched), np.float32)).to(
            words.device)
        beta = np.float32(1.0) / np.float32(temp)
        F = scratch = None
        for g0 in range(0, len(sched), recompute_every):
            g1 = min(len(sched), g0 + recompute_every)
            F, scratch = self.fields(words, P, out=F, scratch=scratch, check=False)
            self.sweep(words, F, P, jp[g0:g1], beta, seed, mcsteps=mcsteps, sweep_base=g0 * mcsteps,
                       accepts=accepts, per_slice_order=per_slice_order)
        if check:
            tensor.check_status(words.device)
            self.check_status()
        return words

    def check_status(self):
        """Raise if a sweep gave up waiting for a neighbouring slice (and clear the flag)."""
        try:
            self._status.raise_if_set("pq_dense_sweep")
        finally:
            self._status.reset()


def field_error(problem, words, P):
    """max |f_gemm - f_fp64| and max |f_fp64| over every configuration (the recompute's error)."""
    F, _ = problem.fields(words, P)
    sp = problem.unpack(words, P).cpu().numpy().astype(np.float64)      # (R, N, P)
    R = sp.shape[0]
    exact = np.einsum("ij,rjk->rki", problem.K64, sp) + problem.h64[None, None, :]
    got = F[:R * P, :problem.N].double().cpu().numpy().reshape(R, P, problem.N)
    return float(np.abs(got - exact).max()), float(np.abs(exact).max())
