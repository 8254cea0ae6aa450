"""Tensor-core helpers: the tcgen05 BF16 GEMM of the C ABI on torch tensors."""
import torch

from . import _device, _native


_status = {}


def _status_for(dev):
    st = _status.get(dev)
    if st is None:
        st = _status[dev] = _device.Status()
    return st


def check_status(device=None):
    """Raise if a GEMM launched with ``check=False`` gave up on a wait since the last check."""
    st = _status_for(device or _device.device())
    try:
        st.raise_if_set("pq_tc_gemm_bf16")
    finally:
        st.reset()


def gemm_bf16(A, B, alpha=1.0, bias=None, out=None, status=None, check=True):
    """alpha * A @ B.T (+ bias) in FP32 from BF16 A (M x K) and B (N x K), on the tensor cores.

    M must be a multiple of 128, N of 64 and K of 64 (pad with zeros otherwise).
    The kernel records a timed-out wait in ``status`` (a ``_device.Status``) or, by
    default, in a per-device word; ``check=True`` reads it after the call (a host
    synchronisation), ``check=False`` leaves that to a later ``check_status()``.
    """
    if A.dtype != torch.bfloat16 or B.dtype != torch.bfloat16:
        raise TypeError("A and B must be bfloat16")
    M, K = A.shape
    N, K2 = B.shape
    if K != K2:
        raise ValueError("inner dimensions differ")
    if A.stride(1) != 1 or B.stride(1) != 1:
        raise ValueError("A and B must have unit stride along K")
    if out is None:
        out = torch.empty((M, N), dtype=torch.float32, device=A.device)
    st = status if status is not None else _status_for(A.device)
    code = _native.lib().pq_tc_gemm_bf16(_device.ptr(A), A.stride(0), _device.ptr(B), B.stride(0), _device.ptr(out),
                                         out.stride(0), M, N, K, float(alpha), _device.ptr(bias), st.ptr,
                                         _device.stream_handle())
    _native.check(code, "pq_tc_gemm_bf16")
    if check and status is None:
        check_status(A.device)
    return out
