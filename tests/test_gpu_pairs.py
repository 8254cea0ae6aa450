"""Pair world-line moves on the GPU: bit for bit against the oracle's restatement.

pq_pair_pass (every bond tried), pq_pair_features (both row sets, BF16) and
pq_pair_propose (the learned move, from the network's logits) against
oracle.pair_class / oracle.pair_features (oracle/fast_oracle.c), several passes
over random instances with slice counts 3, 20, 33 and 64 and 32- and 64-bit words.
"""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

import oracle
from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def _problem(kind, g):
    from piqmc import fast, tools
    if kind == "lattice":
        J = lattice(9, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.3))
        return J, fast.Problem(tools.GenerateNeighbors(81, J, 5))
    n = 60
    J = sps.dok_matrix((n, n))
    while J.nnz < 110:
        a, b = sorted(g.choice(n, 2, replace=False))
        J[int(a), int(b)] = g.uniform(-2, 2)
    return J, fast.Problem(tools.GenerateNeighbors(n, J, 14))


def _words_u64(words):
    w = words.cpu().numpy()
    return (w.view(np.uint32).astype(np.uint64) if w.dtype == np.int32 else w.view(np.uint64)).copy()


@pytest.mark.parametrize("P", [3, 20, 33, 64])
@pytest.mark.parametrize("kind", ["lattice", "graph"])
def test_uniform_pair_pass_bit_exact(P, kind):
    from piqmc import pairs
    g = np.random.default_rng(P + len(kind))
    J, prob = _problem(kind, g)
    bc = pairs.bond_classes(prob)
    R = 3
    spins = np.where(g.random((R, prob.n, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    host = [_words_u64(words)[r] for r in range(R)]
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    beta = np.float32(1.0 / 0.4)
    acc = 0
    for move in range(3):
        pairs.pair_pass(prob, words, P, beta, seed=11, move=move, counters=cnt, replica_base=5)
        for r in range(R):
            for c in range(bc.nclass):
                lo, hi = int(bc.class_start[c]), int(bc.class_start[c + 1])
                acc += oracle.pair_class(host[r], prob.nbr_host, prob.cpl_host, prob.field_host, P, bc.bond_i,
                                         bc.bond_j, bc.bond_J, lo, hi - lo, c, beta, 11, move, 5 + r)
    got = _words_u64(words)
    for r in range(R):
        np.testing.assert_array_equal(got[r], host[r], err_msg="replica %d" % r)
    c = cnt.cpu().numpy()
    assert c[0] == 3 * R * bc.nbonds and c[1] == acc and acc > 0


@pytest.mark.parametrize("P", [20, 64])
def test_pair_features_bit_exact(P):
    from piqmc import pairs
    g = np.random.default_rng(P)
    J, prob = _problem("lattice", g)
    bc = pairs.bond_classes(prob)
    R = 2
    spins = np.where(g.random((R, prob.n, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    host = _words_u64(words)
    beta, jp = np.float32(3.0), np.float32(0.8)
    for c in (0, bc.nclass - 1):
        X, dE, M, Mpad = pairs.pair_features(prob, words, P, beta, jp, c)
        Xh = X.float().cpu().numpy()
        dEh = dE.cpu().numpy()
        lo, hi = int(bc.class_start[c]), int(bc.class_start[c + 1])
        for t in range(M):
            r, b = divmod(t, hi - lo)
            b += lo
            for row, flipped in ((t, False), (Mpad + t, True)):
                x, d = oracle.pair_features(host[r], prob.nbr_host, prob.cpl_host, prob.field_host, P, bc.bond_i[b],
                                            bc.bond_j[b], bc.bond_J[b], beta, jp, flipped=flipped)
                want = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
                np.testing.assert_array_equal(Xh[row, :8], want)
                if not flipped:
                    assert dEh[t] == d


@pytest.mark.parametrize("P", [20, 33])
def test_learned_pair_pass_bit_exact(P):
    """The learned move against the oracle given the same logits (the network itself is checked elsewhere)."""
    from piqmc import _device, _native, learned, pairs
    g = np.random.default_rng(7 + P)
    J, prob = _problem("lattice", g)
    bc = pairs.bond_classes(prob)
    R = 4
    spins = np.where(g.random((R, prob.n, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    host = _words_u64(words)
    mlp = learned.ProposalMLP(seed=3)
    beta, jp = np.float32(2.0), np.float32(0.6)
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    bits = 32 if P <= 32 else 64
    acc = 0
    for c in range(bc.nclass):
        X, dE, M, Mpad = pairs.pair_features(prob, words, P, beta, jp, c)
        logit = mlp.forward(X)
        lo, hi = int(bc.class_start[c]), int(bc.class_start[c + 1])
        _native.check(_native.lib().pq_pair_propose(
            _device.ptr(words), bits, prob.nslots, P, R, _device.ptr(bc.d_i), _device.ptr(bc.d_j), lo, hi - lo, c,
            _device.ptr(logit), _device.ptr(dE), Mpad, 0.05, float(beta), 9, 21, 0, _device.ptr(cnt),
            _device.ptr(status), _device.stream_handle()), "propose")
        lg = logit.cpu().numpy()
        for r in range(R):
            cur = lg[r * (hi - lo):(r + 1) * (hi - lo)]
            flp = lg[Mpad + r * (hi - lo):Mpad + (r + 1) * (hi - lo)]
            acc += oracle.pair_class(host[r], prob.nbr_host, prob.cpl_host, prob.field_host, P, bc.bond_i, bc.bond_j,
                                     bc.bond_J, lo, hi - lo, c, beta, 21, 9, r, qmin=0.05, logit=cur, logit_f=flp)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got = _words_u64(words)
    for r in range(R):
        np.testing.assert_array_equal(got[r], host[r], err_msg="replica %d" % r)
    assert int(cnt[1].item()) == acc


def test_pair_passes_lower_the_final_energy():
    """Sanity: a 16x16 anneal with a pair pass every 10 steps ends lower than without it."""
    from piqmc import fast, pairs, tools
    g = np.random.default_rng(1)
    J = lattice(16, True, g, dist=lambda r: r.normal())
    prob = fast.Problem(tools.GenerateNeighbors(256, J, 4))
    P, R, T = 20, 64, 0.05
    sched = np.linspace(3.0, 1e-8, 200)
    jp = torch.from_numpy(oracle.jperp(sched, P, T)).cuda()
    spins = np.repeat(np.where(g.random((R, 256)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    out = []
    for with_pairs in (False, True):
        w = prob.pack(torch.from_numpy(spins))
        for g0 in range(0, 200, 10):
            fast.anneal(prob, w, sched[g0:g0 + 10], P, T, seed=3, sweep_base=g0, jperp=jp[g0:g0 + 10])
            if with_pairs:
                pairs.pair_pass(prob, w, P, 1.0 / T, seed=4, move=g0)
        out.append(prob.energies(w, P).cpu().numpy().min(axis=1).mean() / 256)
    print("mean best-slice energy per spin: plain %.4f, with pair moves %.4f" % tuple(out))
    assert out[1] < out[0] - 0.02


@pytest.mark.parametrize("P", [20, 64])
def test_fused_learned_pair_pass_equals_unfused(P):
    """One launch per class (features, tcgen05 layers in TMEM, head, decision) makes the unfused path's moves."""
    from piqmc import learned, pairs
    g = np.random.default_rng(40 + P)
    J, prob = _problem("lattice", g)
    R = 5
    spins = np.where(g.random((R, prob.n, P)) < 0.5, -1, 1).astype(np.int8)
    words = prob.pack(torch.from_numpy(spins))
    mlp = learned.ProposalMLP(seed=8)
    out = []
    for fused in (True, False):
        w = words.clone()
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        for move in range(3):
            pairs.learned_pair_pass(prob, w, P, mlp, 2.5, 0.4, seed=6, move=move, counters=cnt, fused=fused)
        out.append((w, cnt.cpu().numpy()))
    assert torch.equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][1][1] > 0
