"""Reference-order sweeps on the GPU: the reference's own spin order, arithmetic and uniforms.

``quantum_anneal``/``quantum_anneal_dense``/``anneal`` run R replicas, each with
its own explicit spin orders (``perms``) and uniform stream (``rands``), and
return the final int8 spins and the number of uniforms each replica consumed.
The drop-in functions in ``piqmc.qmc`` and ``piqmc.sa`` build those streams from
the caller's ``rng`` and this process's libc ``rand()`` exactly as the reference
consumes them.

exp parity: see ``csrc/reforder.cu``.  ``_run_with_exp_check`` reruns a launch
with host-libm overrides whenever a "close call" used a device exp value that
differs from the host libm's, so decisions always follow the host libm.
"""
import numpy as np
import torch

from . import _device, _native

CLOSE_CAP = 1024

# FP32 bit pattern -> host libm exp((double)x); grows only on a verified mismatch.
_exp_overrides = {}
_ov_tensors = {}
_exp_stats = {"close_calls": 0, "mismatches": 0, "reruns": 0}


def exp_stats():
    """Counters of the exp-parity machinery in this process (close calls seen, mismatches, reruns)."""
    return dict(_exp_stats, overrides=len(_exp_overrides))


def _override_tensors(dev):
    key = (str(dev), len(_exp_overrides))
    got = _ov_tensors.get(key)
    if got is None:
        xs = np.array(sorted(_exp_overrides), dtype=np.uint32)
        ys = np.array([_exp_overrides[int(x)] for x in xs], dtype=np.float64)
        if len(xs) == 0:
            xs = np.zeros(1, np.uint32)
            ys = np.zeros(1, np.float64)
        got = (torch.from_numpy(xs.view(np.int32)).to(dev), torch.from_numpy(ys).to(dev), len(_exp_overrides))
        _ov_tensors.clear()
        _ov_tensors[key] = got
    return got


def host_exp(xbits):
    """Host libm exp((double)x) for FP32 bit patterns (the reference's own exp)."""
    x = np.ascontiguousarray(np.asarray(xbits, dtype=np.uint32).view(np.float32))
    y = np.empty(len(x), dtype=np.float64)
    _native.check(_native.lib().pq_host_exp(_device.ptr(x), _device.ptr(y), len(x)), "pq_host_exp")
    return y


def _run_with_exp_check(launch, spins, where):
    """Run ``launch`` until every close call it made used the host libm's exp value."""
    dev = spins.device
    saved = spins.clone()
    cap = CLOSE_CAP
    close_x = torch.empty(cap, dtype=torch.int32, device=dev)
    close_y = torch.empty(cap, dtype=torch.float64, device=dev)
    close_cnt = torch.zeros(1, dtype=torch.int32, device=dev)
    status = _device.Status()
    for _ in range(1000):
        ov_x, ov_y, ov_n = _override_tensors(dev)
        close_cnt.zero_()
        status.reset()
        _native.check(launch(ov_x, ov_y, ov_n, close_x, close_y, cap, close_cnt, status), where)
        status.raise_if_set(where)
        cnt = int(close_cnt.item())
        if cnt == 0:
            return
        _exp_stats["close_calls"] += min(cnt, cap)
        m = min(cnt, cap)
        xs = close_x[:m].cpu().numpy().view(np.uint32)
        ys = close_y[:m].cpu().numpy()
        hs = host_exp(xs)
        bad = hs.view(np.uint64) != ys.view(np.uint64)
        new = {int(x): float(h) for x, h in zip(xs[bad], hs[bad]) if int(x) not in _exp_overrides}
        if not new and cnt <= cap:
            return
        _exp_stats["mismatches"] += len(new)
        _exp_stats["reruns"] += 1
        _exp_overrides.update(new)
        if cnt > cap:
            cap = 2 * cnt
            close_x = torch.empty(cap, dtype=torch.int32, device=dev)
            close_y = torch.empty(cap, dtype=torch.float64, device=dev)
        spins.copy_(saved)
    raise _native.PiqmcError(_native.PQ_ERR_TIMEOUT, where + ": exp parity did not converge")


def jperp_schedule(sched, P, temp):
    """J-perp per schedule step in the reference's C types (piqmc/qmc.pyx:95)."""
    sched = np.ascontiguousarray(sched, dtype=np.float64)
    out = np.empty(len(sched), dtype=np.float32)
    st = _native.lib().pq_jperp_schedule(_device.ptr(sched), len(sched), int(P), float(np.float32(temp)),
                                         _device.ptr(out))
    if st == _native.PQ_ERR_INVALID_ARG and len(sched) and np.float32(P) * np.float32(temp) == 0:
        raise ZeroDivisionError("float division")
    _native.check(st, "pq_jperp_schedule")
    return out


def split_neighbors(nbs, nrows=None):
    """(n, maxnb, 2) float64 table -> int32 index (C truncation) and FP32 coupling, padded to nrows."""
    nbs = np.asarray(nbs, dtype=np.float64)
    n0, maxnb = nbs.shape[0], nbs.shape[1]
    nrows = n0 if nrows is None else nrows
    idx = np.zeros((nrows, maxnb), dtype=np.int32)
    jv = np.zeros((nrows, maxnb), dtype=np.float32)
    m = min(n0, nrows)
    raw = nbs[:m, :, 0]
    if not np.all(np.isfinite(raw)) or np.any(np.abs(raw) >= 2 ** 31):
        raise ValueError("neighbour indices must be finite and fit in a C int")
    idx[:m] = np.trunc(raw).astype(np.int32)
    jv[:m] = nbs[:m, :, 1].astype(np.float32)
    return idx, jv


def _acc_flag(*arrays):
    """PQ_ACC_FP64 when some finite coupling is so large that 2*J overflows FP32."""
    for a in arrays:
        a = np.abs(np.asarray(a, dtype=np.float64))
        a = a[np.isfinite(a)]
        if a.size and a.max() >= 2.0 ** 126:
            return _native.PQ_ACC_FP64
    return 0


def _as_perms(perms, R, nsweeps, nperm):
    perms = np.ascontiguousarray(perms, dtype=np.int32)
    if perms.shape != (R, nsweeps, nperm):
        raise ValueError("perms must have shape (R, nsweeps, nperm) = %r, got %r" % ((R, nsweeps, nperm), perms.shape))
    return perms


def _as_rands(rands, R):
    rands = np.ascontiguousarray(rands, dtype=np.int32)
    if rands.ndim != 2 or rands.shape[0] != R:
        raise ValueError("rands must have shape (R, stream length)")
    return rands


def quantum_anneal(spins, nb_idx, nb_j, sched, mcsteps, temp, perms, rands, flags=0, nperm=None,
                   jperp=None):
    """Reference-order QuantumAnneal of R replicas.

    spins int8 (R, n, P) +-1 (host or device), nb_idx/nb_j (n, maxnb), perms int
    (R, nsched*mcsteps, nperm), rands int32 (R, L).  Returns (spins device tensor,
    consumed uniforms per replica as a numpy int64 array).
    """
    dev = _device.device()
    sp = torch.as_tensor(spins).to(dev, torch.int8).contiguous()
    R, n, P = sp.shape
    nperm = n if nperm is None else int(nperm)
    nsched = len(sched)
    perms = _as_perms(perms, R, nsched * mcsteps, nperm)
    rands = _as_rands(rands, R)
    jp = jperp_schedule(sched, P, temp) if jperp is None else np.asarray(jperp, np.float32)
    d_idx = _device.to_device(nb_idx, torch.int32)
    d_j = _device.to_device(nb_j, torch.float32)
    d_jp = _device.to_device(jp)
    d_perm = _device.to_device(perms)
    d_rand = _device.to_device(rands)
    used = torch.zeros(R, dtype=torch.int64, device=dev)
    maxnb = d_idx.shape[1] if d_idx.dim() == 2 else 0
    flags = int(flags) | _acc_flag(nb_j, jp)
    L = _native.lib()

    def launch(ov_x, ov_y, ov_n, cx, cy, cap, ccnt, status):
        return L.pq_qa_sparse_reforder_ex(
            _device.ptr(sp), _device.ptr(d_idx), _device.ptr(d_j), n, nperm, maxnb, P, R, _device.ptr(d_jp),
            nsched, int(mcsteps), float(np.float32(temp)), _device.ptr(d_perm), _device.ptr(d_rand),
            rands.shape[1], _device.ptr(used), int(flags), _device.ptr(ov_x), _device.ptr(ov_y), ov_n,
            _device.ptr(cx), _device.ptr(cy), cap, _device.ptr(ccnt), status.ptr, _device.stream_handle())

    _run_with_exp_check(launch, sp, "pq_qa_sparse_reforder")
    return sp, used.cpu().numpy()


def quantum_anneal_dense(spins, J, sched, mcsteps, temp, perms, rands, flags=0, jperp=None):
    """Reference-order QuantumAnneal_dense of R replicas (J dense float64 (n, n))."""
    dev = _device.device()
    sp = torch.as_tensor(spins).to(dev, torch.int8).contiguous()
    R, n, P = sp.shape
    nsched = len(sched)
    perms = _as_perms(perms, R, nsched * mcsteps, n)
    rands = _as_rands(rands, R)
    jp = jperp_schedule(sched, P, temp) if jperp is None else np.asarray(jperp, np.float32)
    d_J = _device.to_device(np.asarray(J, dtype=np.float64)[:n, :n])
    d_jp = _device.to_device(jp)
    d_perm = _device.to_device(perms)
    d_rand = _device.to_device(rands)
    used = torch.zeros(R, dtype=torch.int64, device=dev)
    L = _native.lib()

    def launch(ov_x, ov_y, ov_n, cx, cy, cap, ccnt, status):
        return L.pq_qa_dense_reforder_ex(
            _device.ptr(sp), _device.ptr(d_J), n, P, R, _device.ptr(d_jp), nsched, int(mcsteps),
            float(np.float32(temp)), _device.ptr(d_perm), _device.ptr(d_rand), rands.shape[1], _device.ptr(used),
            int(flags), _device.ptr(ov_x), _device.ptr(ov_y), ov_n, _device.ptr(cx), _device.ptr(cy), cap,
            _device.ptr(ccnt), status.ptr, _device.stream_handle())

    _run_with_exp_check(launch, sp, "pq_qa_dense_reforder")
    return sp, used.cpu().numpy()


def anneal(spins, nb_idx, nb_j, sched, mcsteps, perms, rands):
    """Reference-order sa.Anneal of R replicas (spins int8 (R, n))."""
    dev = _device.device()
    sp = torch.as_tensor(spins).to(dev, torch.int8).contiguous()
    R, n = sp.shape
    nsched = len(sched)
    perms = _as_perms(perms, R, nsched * mcsteps, n)
    rands = _as_rands(rands, R)
    temps = np.asarray(sched, dtype=np.float64).astype(np.float32)
    d_idx = _device.to_device(nb_idx, torch.int32)
    d_j = _device.to_device(nb_j, torch.float32)
    d_t = _device.to_device(temps)
    d_perm = _device.to_device(perms)
    d_rand = _device.to_device(rands)
    used = torch.zeros(R, dtype=torch.int64, device=dev)
    maxnb = d_idx.shape[1]
    flags = _acc_flag(nb_j)
    L = _native.lib()

    def launch(ov_x, ov_y, ov_n, cx, cy, cap, ccnt, status):
        return L.pq_sa_sparse_reforder_ex(
            _device.ptr(sp), _device.ptr(d_idx), _device.ptr(d_j), n, maxnb, R, _device.ptr(d_t), nsched,
            int(mcsteps), _device.ptr(d_perm), _device.ptr(d_rand), rands.shape[1], _device.ptr(used), flags,
            _device.ptr(ov_x), _device.ptr(ov_y), ov_n, _device.ptr(cx), _device.ptr(cy), cap, _device.ptr(ccnt),
            status.ptr, _device.stream_handle())

    _run_with_exp_check(launch, sp, "pq_sa_sparse_reforder")
    return sp, used.cpu().numpy()


def anneal_dense(spins, J, sched, mcsteps, perms, rands):
    """Reference-order sa.Anneal_dense of R replicas (spins int8 (R, n), J dense float64 (n, n))."""
    dev = _device.device()
    sp = torch.as_tensor(spins).to(dev, torch.int8).contiguous()
    R, n = sp.shape
    nsched = len(sched)
    perms = _as_perms(perms, R, nsched * mcsteps, n)
    rands = _as_rands(rands, R)
    d_J = _device.to_device(np.ascontiguousarray(np.asarray(J, dtype=np.float64)[:n, :n]))
    d_t = _device.to_device(np.asarray(sched, dtype=np.float64).astype(np.float32))
    d_perm = _device.to_device(perms)
    d_rand = _device.to_device(rands)
    used = torch.zeros(R, dtype=torch.int64, device=dev)
    L = _native.lib()

    def launch(ov_x, ov_y, ov_n, cx, cy, cap, ccnt, status):
        return L.pq_sa_dense_reforder_ex(
            _device.ptr(sp), _device.ptr(d_J), n, R, _device.ptr(d_t), nsched, int(mcsteps), _device.ptr(d_perm),
            _device.ptr(d_rand), rands.shape[1], _device.ptr(used), _device.ptr(ov_x), _device.ptr(ov_y), ov_n,
            _device.ptr(cx), _device.ptr(cy), cap, _device.ptr(ccnt), status.ptr, _device.stream_handle())

    _run_with_exp_check(launch, sp, "pq_sa_dense_reforder")
    return sp, used.cpu().numpy()


def anneal_bipartite(spins, nl, J, lbias, rbias, sched, mcsteps, rands):
    """Reference-order sa.Anneal_bipartite of R replicas (spins int8 (R, nl + nr): left then right)."""
    dev = _device.device()
    sp = torch.as_tensor(spins).to(dev, torch.int8).contiguous()
    R, ntot = sp.shape
    nr = ntot - nl
    nsched = len(sched)
    rands = _as_rands(rands, R)
    d_J = _device.to_device(np.ascontiguousarray(np.asarray(J, dtype=np.float64).reshape(nl, nr)))
    d_lb = _device.to_device(np.ascontiguousarray(lbias, dtype=np.float64))
    d_rb = _device.to_device(np.ascontiguousarray(rbias, dtype=np.float64))
    d_t = _device.to_device(np.asarray(sched, dtype=np.float64).astype(np.float32))
    d_rand = _device.to_device(rands)
    used = torch.zeros(R, dtype=torch.int64, device=dev)
    L = _native.lib()

    def launch(ov_x, ov_y, ov_n, cx, cy, cap, ccnt, status):
        return L.pq_sa_bipartite_reforder_ex(
            _device.ptr(sp), _device.ptr(d_J), nl, nr, _device.ptr(d_lb), _device.ptr(d_rb), R, _device.ptr(d_t),
            nsched, int(mcsteps), _device.ptr(d_rand), rands.shape[1], _device.ptr(used), _device.ptr(ov_x),
            _device.ptr(ov_y), ov_n, _device.ptr(cx), _device.ptr(cy), cap, _device.ptr(ccnt), status.ptr,
            _device.stream_handle())

    _run_with_exp_check(launch, sp, "pq_sa_bipartite_reforder")
    return sp, used.cpu().numpy()


# ------------------------------------------------------------------------------------------
# libc rand() stream of this process
# ------------------------------------------------------------------------------------------

def libc_peek(count):
    """The next ``count`` libc rand() values, without advancing libc."""
    out = np.empty(int(count), dtype=np.int32)
    _native.check(_native.lib().pq_libc_rand_peek(_device.ptr(out), int(count)), "pq_libc_rand_peek")
    return out


def libc_skip(count):
    _native.check(_native.lib().pq_libc_rand_skip(int(count)), "pq_libc_rand_skip")
