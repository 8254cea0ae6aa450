"""Device plumbing: the CUDA device, the current stream, pointers and status words."""
import ctypes

import numpy as np
import torch

from . import _native


def device():
    """The current CUDA device; there is no CPU path, so no device is an error."""
    if not torch.cuda.is_available():
        raise _native.PiqmcError(_native.PQ_ERR_NO_DEVICE, "piqmc runs on a CUDA device only")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t):
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return ctypes.c_void_p(t.ctypes.data)
    return ctypes.c_void_p(t.data_ptr())


def to_device(a, dtype=None):
    """Host array -> contiguous device tensor (pinned staging for large copies)."""
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(device(), non_blocking=False)


class Status:
    """A device status word: the kernels record their first error in it."""

    def __init__(self):
        self.t = torch.zeros(1, dtype=torch.int32, device=device())

    def reset(self):
        self.t.zero_()

    @property
    def ptr(self):
        return ptr(self.t)

    def raise_if_set(self, where, stream=None):
        (stream or torch.cuda.current_stream()).synchronize()
        code = int(self.t.item())
        if code:
            raise _native.PiqmcError(code, where)
