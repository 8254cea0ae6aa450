"""The allocation-free batched anneal against the regular one, through the C ABI.

pq_batch_anneal_noalloc serves callers that may not allocate GPU memory (a host
program that owns every device buffer and passes this library only its inputs
and outputs, or code where cudaMalloc is forbidden): it keeps its task counter in
a static device array instead of a caller-provided buffer.  Its results must
equal pq_batch_anneal's on the same inputs, bit for bit, on two calls in a row
(the second call also checks that the shared counter is reset between calls).
This file is collected last so that a failure here cannot hide other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def _batch():
    from piqmc import batch, tools
    g = np.random.default_rng(42)
    nbs, R, P = [], [], []
    for L, p, r in [(6, 20, 4), (9, 64, 2), (5, 7, 3), (8, 16, 8)]:
        J = lattice(L, True, g, dist=lambda x: x.normal())
        nbs.append(tools.GenerateNeighbors(L * L, J, 4))
        R.append(r)
        P.append(p)
    B = batch.Batch(nbs, R, P)
    B.set_spins([np.where(g.random((r, nb.shape[0], p)) < 0.5, -1, 1).astype(np.int8)
                 for nb, r, p in zip(nbs, R, P)])
    B._prepare(np.linspace(3.0, 1e-8, 6), 0.05, seed=9)
    return B


def _call(B, words, noalloc, status=None):
    from piqmc import _device, _native
    lib = _native.lib()
    run = B._runs(6, 0.05, 1, 0, 1, None)[0]
    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
    args_head = [_device.ptr(B.d_tasks), len(B.tasks), _device.ptr(B.d_items), _device.ptr(B.d_inst),
                 _device.ptr(B.d_nbr), _device.ptr(B.d_cpl), _device.ptr(B.d_field), _device.ptr(B.d_csize),
                 _device.ptr(B.d_jperp), _device.ptr(words)]
    tail = [ctypes.byref(run), B.grid, 256, B.smem_bytes, None, _device.ptr(status), _device.stream_handle()]
    if noalloc:
        rc = lib.pq_batch_anneal_noalloc(*args_head, *tail)
    else:
        rc = lib.pq_batch_anneal(*args_head, _device.ptr(B.queue_head), *tail)
    torch.cuda.synchronize()
    assert rc == 0, _native.PiqmcError(rc).args
    assert int(status.item()) == 0


def test_noalloc_matches_regular_entry_point_twice():
    B = _batch()
    regular = B.words.clone()
    noalloc = B.words.clone()
    for _ in range(2):
        _call(B, regular, noalloc=False)
        _call(B, noalloc, noalloc=True)
        assert torch.equal(regular, noalloc)
    assert not torch.equal(regular, B.words)   # the anneal did change the state


def test_noalloc_call_allocates_nothing():
    """After a first call (which loads the kernel and looks up the scratch's address),
    a call changes neither torch's allocated bytes nor the device's free memory."""
    B = _batch()
    words = B.words.clone()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _call(B, words, noalloc=True, status=status)
    torch.cuda.synchronize()
    allocated, (free, _) = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()
    _call(B, words, noalloc=True, status=status)
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == allocated
    assert torch.cuda.mem_get_info()[0] == free


def test_noalloc_rejects_bad_arguments_like_the_regular_entry_point():
    from piqmc import _native
    lib = _native.lib()
    B = _batch()
    run = B._runs(6, 0.05, 1, 0, 1, None)[0]
    nulls = [None] * 8   # items .. words_pool
    # the 32-bit task counter: ntasks + grid must fit
    assert lib.pq_batch_anneal_noalloc(None, 2 ** 31 - 10, *nulls, ctypes.byref(run), 64, 256, 0, None, None,
                                       None) == _native.PQ_ERR_TOO_LARGE
    assert lib.pq_batch_anneal(None, 2 ** 31 - 10, *nulls, None, ctypes.byref(run), 64, 256, 0, None, None,
                               None) == _native.PQ_ERR_TOO_LARGE
    # a negative task count or an empty grid is an argument error on both entry points
    for ntasks, grid in [(-1, 64), (4, 0)]:
        assert lib.pq_batch_anneal_noalloc(None, ntasks, *nulls, ctypes.byref(run), grid, 256, 0, None, None,
                                           None) == _native.PQ_ERR_INVALID_ARG
        assert lib.pq_batch_anneal(None, ntasks, *nulls, None, ctypes.byref(run), grid, 256, 0, None, None,
                                   None) == _native.PQ_ERR_INVALID_ARG
