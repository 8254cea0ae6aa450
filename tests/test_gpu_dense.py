"""Dense fast path: split-BF16 tensor-core field recompute and the rank-1 dense sweep."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _instance(N, seed=0):
    g = np.random.default_rng(seed)
    J = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1) + np.diag(g.normal(0.0, np.sqrt(0.1), N))
    return J, g


@pytest.mark.parametrize("N,P,R", [(512, 32, 8), (100, 20, 7), (64, 8, 16)])
def test_field_recompute_error_vs_fp64(N, P, R):
    from piqmc import dense
    J, g = _instance(N, N)
    prob = dense.DenseProblem(J)
    spins = np.where(g.random((R, N, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    err, scale = dense.field_error(prob, words, P)
    print("N=%d: max |f_gemm - f_fp64| = %.3g (max |f| = %.3g)" % (N, err, scale))
    # 16 significant bits of each coupling: |error| <= sum_j |K_ij| 2^-17 + FP32 accumulation
    bound = np.abs(prob.K64).sum(1).max() * 2.0 ** -16 + 1e-5 * scale
    assert err <= bound, (err, bound)


@pytest.mark.parametrize("N,P,per_slice", [(64, 8, False), (50, 7, True), (96, 16, False), (64, 32, True),
                                           (600, 4, False), (40, 2, False), (33, 1, False)])
def test_dense_sweep_bit_exact_with_oracle(N, P, per_slice):
    from piqmc import dense
    J, g = _instance(N, 100 + N)
    prob = dense.DenseProblem(J)
    R = 3
    spins = np.where(g.random((R, N, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    F, _ = prob.fields(words, P)
    F0 = F.clone()
    w0 = words.clone()
    sched = np.linspace(3.0, 1e-8, 6)
    jp = oracle.jperp(sched, P, 0.05)
    acc = torch.zeros(1, dtype=torch.int64, device="cuda")
    prob.sweep(words, F, P, torch.from_numpy(jp).cuda(), np.float32(1) / np.float32(0.05), 77, mcsteps=2,
               sweep_base=5, accepts=acc, per_slice_order=per_slice)
    prob.check_status()
    got = words.cpu().numpy().view(np.uint32)
    tot = 0
    for r in range(R):
        w = w0[r].cpu().numpy().view(np.uint32).copy()
        f = F0[r * P:(r + 1) * P, :N].cpu().numpy().copy()
        n, f_after = oracle.dense_sweep(f, prob.K.cpu().numpy(), prob.units.cpu().numpy(), w, P, jp, 2,
                                        np.float32(1) / np.float32(0.05), 77, sweep_base=5, replica=r,
                                        per_slice_order=per_slice)
        tot += n
        np.testing.assert_array_equal(got[r], w, err_msg="replica %d" % r)
        np.testing.assert_array_equal(F[r * P:(r + 1) * P, :N].cpu().numpy(), f_after, err_msg="fields %d" % r)
    assert int(acc.item()) == tot


def test_dense_anneal_reaches_low_energy_and_energies_match():
    from piqmc import dense
    N, P, R = 128, 16, 8
    J, g = _instance(N, 5)
    prob = dense.DenseProblem(J)
    spins = np.repeat(np.where(g.random((R, N)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    words = prob.pack(torch.from_numpy(spins))
    E0 = prob.energies(words, P).cpu().numpy()
    prob.anneal(words, np.linspace(3.0, 1e-8, 100), P, 0.05, seed=3, recompute_every=25)
    E = prob.energies(words, P).cpu().numpy()
    fin = prob.unpack(words, P).cpu().numpy()
    for r in range(R):
        for k in (0, P - 1):
            ref = oracle.classical_energy(fin[r, :, k].astype(np.float64), J)
            assert abs(E[r, k] - ref) <= 1e-10 * max(1.0, abs(ref))
    assert E.mean() < E0.mean() - 0.3 * N ** 0.5


def test_wavefront_wait_runs_to_its_limit_and_the_kernel_returns():
    """A wait for progress that no warp reports gives up after its poll limit: the kernel
    records PQ_ERR_TIMEOUT, returns, and the context stays usable (the same sweep then runs
    normally and matches the oracle).  No GPU is hung: every wait is bounded."""
    from piqmc import _device, _native, dense
    N, P, R = 64, 8, 2
    J, g = _instance(N, 11)
    prob = dense.DenseProblem(J)
    spins = np.where(g.random((R, N, P)) < 0.5, -1, 1).astype(np.int8)
    words0 = prob.pack(torch.from_numpy(spins))
    F0, _ = prob.fields(words0, P)
    sched = np.linspace(3.0, 1e-8, 4)
    jp = oracle.jperp(sched, P, 0.05)
    beta = np.float32(1) / np.float32(0.05)
    status = _device.Status()
    words, F = words0.clone(), F0.clone()
    prob.sweep(words, F, P, torch.from_numpy(jp).cuda(), beta, 5, status=status, poll_limit=1000, wait_skew=1 << 20)
    torch.cuda.synchronize()
    assert int(status.t.item()) == _native.PQ_ERR_TIMEOUT
    # the same call with the waits in use completes and is exact
    words, F = words0.clone(), F0.clone()
    status.reset()
    prob.sweep(words, F, P, torch.from_numpy(jp).cuda(), beta, 5, status=status, poll_limit=1000)
    torch.cuda.synchronize()
    assert int(status.t.item()) == 0
    got = words.cpu().numpy().view(np.uint32)
    for r in range(R):
        w = words0[r].cpu().numpy().view(np.uint32).copy()
        f = F0[r * P:(r + 1) * P, :N].cpu().numpy().copy()
        oracle.dense_sweep(f, prob.K.cpu().numpy(), prob.units.cpu().numpy(), w, P, jp, 1, beta, 5, replica=r)
        np.testing.assert_array_equal(got[r], w)


def test_wait_skew_is_bounded():
    from piqmc import _native, dense
    J, g = _instance(16, 12)
    prob = dense.DenseProblem(J)
    words = prob.pack(torch.from_numpy(np.ones((1, 16, 4), np.int8)))
    F, _ = prob.fields(words, 4)
    with pytest.raises(_native.PiqmcError):
        prob.sweep(words, F, 4, torch.zeros(1, device="cuda"), 1.0, 0, wait_skew=-1)
