"""Learned world-line proposals: gradients against the CPU oracle, training, exact MH, and the gain."""
import itertools

import numpy as np
import pytest
import torch

import oracle
from oracle import mlp_oracle
from pq_testutil import lattice

pytestmark = pytest.mark.gpu


def test_forward_and_gradients_match_cpu_oracle():
    from piqmc import learned
    mlp = learned.ProposalMLP(seed=3)
    g = np.random.default_rng(1)
    with torch.no_grad():   # make the biases non-trivial
        for k in ("b1", "b2", "b3"):
            mlp.params[k].copy_(torch.tensor(g.normal(0, 0.3, mlp.params[k].shape), dtype=torch.float32))
    mlp.refresh()
    B = 1024
    Xf = g.normal(0, 1, (B, 8)).astype(np.float32)
    Xf[:, 7] = 1.0
    y = g.random(B).astype(np.float32)
    X = torch.zeros((B, 64), dtype=torch.bfloat16, device="cuda")
    X[:, :8] = torch.from_numpy(Xf).to(torch.bfloat16)
    p = mlp.state_dict()
    logit_ref, _ = mlp_oracle.forward(p, Xf)
    logit = mlp.forward(X).cpu().numpy()
    assert np.abs(logit - logit_ref).max() <= 1e-4 * (1 + np.abs(logit_ref).max())
    loss, grads = mlp.gradients(X, torch.from_numpy(y).cuda())
    loss_ref, grads_ref = mlp_oracle.gradients(p, Xf, y.astype(np.float64))
    assert abs(loss - loss_ref) <= 1e-5 * (1 + abs(loss_ref))
    for k, gr in grads_ref.items():
        gg = grads[k].cpu().numpy().reshape(gr.shape)
        rel = np.linalg.norm(gg - gr) / max(np.linalg.norm(gr), 1e-30)
        assert rel < 1e-2, (k, rel)


def _random_mlp(seed):
    from piqmc import learned
    mlp = learned.ProposalMLP(seed=seed)
    g = np.random.default_rng(seed)
    with torch.no_grad():
        for k in ("b1", "b2", "b3"):
            mlp.params[k].copy_(torch.tensor(g.normal(0, 0.3, mlp.params[k].shape), dtype=torch.float32))
    mlp.refresh()
    return mlp


def _feature_problem(kind, seed):
    """A periodic 10x10 lattice with fields (degree 4) or a random graph with degrees up to 9."""
    import scipy.sparse as sps
    from piqmc import fast, tools
    g = np.random.default_rng(seed)
    if kind == "lattice":
        J = lattice(10, True, g, dist=lambda r: r.normal(), fields=lambda r: r.normal(0, 0.3))
        n = 100
    else:
        n = 90
        J = sps.dok_matrix((n, n))
        for a in range(n):
            for b in g.choice(n, size=3, replace=False):
                if a != b:
                    J[min(a, b), max(a, b)] = float(np.float32(g.uniform(-1.5, 1.5)))
            J[a, a] = float(np.float32(g.normal(0, 0.2)))
    return fast.Problem(tools.GenerateNeighbors(n, J, 12))


def _random_words(prob, P, R, seed):
    g = np.random.default_rng(seed)
    if P <= 32:
        w = (g.integers(0, 2 ** 32, size=(R, prob.nslots), dtype=np.uint64) & ((1 << P) - 1)).astype(np.uint32)
        return torch.from_numpy(w.view(np.int32)).cuda()
    return torch.from_numpy(g.integers(0, 2 ** 64, size=(R, prob.nslots), dtype=np.uint64).view(np.int64)).cuda()


@pytest.mark.parametrize("kind", ["lattice", "graph"])
@pytest.mark.parametrize("P", [20, 64])
def test_features_match_oracle_bit_exact(kind, P):
    from piqmc import learned
    prob = _feature_problem(kind, 3)
    R, beta, jp = 6, 20.0, 0.37
    w = _random_words(prob, P, R, 4)
    D = prob.maxdeg
    for cls in range(prob.nclass):
        csize = int(prob.class_size[cls])
        M = R * csize
        Mpad = (M + 127) // 128 * 128
        X = torch.zeros((2 * Mpad, 64), dtype=torch.bfloat16, device="cuda")
        dE = torch.empty(Mpad, dtype=torch.float32, device="cuda")
        learned._features(prob, w, P, cls, beta, jp, X, dE, Mpad)
        Xo, dEo = mlp_oracle.features(w.cpu().numpy(), P, prob.nbr_host[:D], prob.cpl_host[:D], prob.field_host,
                                      cls, prob.class_stride, csize, beta, jp)
        got = X[:M, :8].float().cpu().numpy()
        assert np.array_equal(got, mlp_oracle.bf16(Xo).astype(np.float32)), (cls, np.abs(got - Xo).max())
        flipped = Xo.copy()
        flipped[:, [2, 4, 5]] *= -1
        assert np.array_equal(X[Mpad:Mpad + M, :8].float().cpu().numpy(), mlp_oracle.bf16(flipped).astype(np.float32))
        assert np.array_equal(dE[:M].cpu().numpy(), dEo), cls


@pytest.mark.parametrize("P", [20, 64])
def test_fused_learned_move_matches_unfused_path(P):
    """One kernel per class (features, tcgen05 layers, head, MH) against features + GEMMs + head + propose."""
    from piqmc import _device, _native, learned
    prob = _feature_problem("lattice", 5)
    mlp = _random_mlp(7)
    R, beta, jp = 24, 4.0, 0.2
    w0 = _random_words(prob, P, R, 6)
    # logits of one class against the unfused forward
    cls, csize = 0, int(prob.class_size[0])
    M = R * csize
    Mpad = (M + 127) // 128 * 128
    X = torch.zeros((2 * Mpad, 64), dtype=torch.bfloat16, device="cuda")
    dE = torch.empty(Mpad, dtype=torch.float32, device="cuda")
    learned._features(prob, w0, P, cls, beta, jp, X, dE, Mpad)
    ref = mlp.forward(X)
    logits = torch.full((2, M), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    wt = w0.clone()
    _native.check(_native.lib().pq_mlp_learned_move(
        _device.ptr(wt), 32 if P <= 32 else 64, prob.nslots, P, R, prob.maxdeg, _device.ptr(prob.nbr),
        _device.ptr(prob.cpl), _device.ptr(prob.field), cls, prob.class_stride, csize, beta, jp,
        _device.ptr(mlp.W1b), _device.ptr(mlp.W2b), _device.ptr(mlp.params["b1"]), _device.ptr(mlp.params["b2"]),
        _device.ptr(mlp.params["w3"]), mlp.b3_host, 0.05, 0, 11, 0, _device.ptr(logits), None, _device.ptr(status),
        _device.stream_handle()), "pq_mlp_learned_move")
    assert int(status.item()) == 0
    assert torch.equal(logits[0], ref[:M]) and torch.equal(logits[1], ref[Mpad:Mpad + M])
    # whole passes, every class
    out = {}
    for fused in (True, False):
        w = w0.clone()
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        for move in range(3):
            learned.learned_pass(prob, w, P, mlp, beta, jp, seed=11, move=move, counters=cnt, fused=fused)
        out[fused] = (w, cnt.cpu().numpy())
    assert torch.equal(out[True][0], out[False][0])
    assert np.array_equal(out[True][1], out[False][1]) and out[True][1][1] > 0


@pytest.mark.parametrize("P", [20, 64])
def test_uniform_move_kernel_matches_q1_path(P):
    from piqmc import learned
    prob = _feature_problem("graph", 8)
    R, beta = 16, 1.5
    w0 = _random_words(prob, P, R, 9)
    out = {}
    for fused in (True, False):
        w = w0.clone()
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        for move in range(3):
            learned.uniform_pass(prob, w, P, beta, 0.1, seed=12, move=move, counters=cnt, fused=fused)
        out[fused] = (w, cnt.cpu().numpy())
    assert torch.equal(out[True][0], out[False][0])
    assert np.array_equal(out[True][1], out[False][1]) and out[True][1][1] > 0


def _problem(L, seed):
    from piqmc import fast, tools
    J = lattice(L, True, np.random.default_rng(seed), dist=lambda r: r.normal())
    return J, fast.Problem(tools.GenerateNeighbors(L * L, J, 4))


def _plain_records(prob, P, R, steps=60, T=0.05):
    from piqmc import fast, learned
    g = np.random.default_rng(0)
    spins = np.repeat(np.where(g.random((R, prob.n)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    w = prob.pack(torch.from_numpy(spins))
    sched = np.linspace(3.0, 1e-8, steps)
    jp = fast.jperp_schedule(sched, P, T)
    Xs, ys = [], []
    for g0 in range(0, steps, 10):
        fast.anneal(prob, w, sched[g0:g0 + 10], P, T, seed=1, sweep_base=g0, jperp=torch.from_numpy(jp[g0:g0 + 10]).cuda())
        X, y = learned.record_moves(prob, w, P, 1.0 / T, float(jp[min(g0 + 9, steps - 1)]))
        Xs.append(X)
        ys.append(y)
    return torch.cat(Xs), torch.cat(ys)


def test_training_on_recorded_moves_reduces_the_loss():
    from piqmc import learned
    _, prob = _problem(16, 2)
    X, y = _plain_records(prob, 16, 32)
    mlp = learned.ProposalMLP(seed=0)
    hist = mlp.train(X, y, epochs=4, batch=4096, lr=3e-3)
    assert np.mean(hist[-3:]) < 0.8 * hist[0], hist


def test_learned_pass_keeps_detailed_balance():
    """Exact enumeration: 4-spin ring, P = 4, fixed field; local sweeps + learned world-line moves."""
    from piqmc import fast, learned
    n, P, T, G = 4, 4, 1.0, 2.0
    import scipy.sparse as sps
    from piqmc import tools
    J = sps.dok_matrix((n, n))
    for (a, b, v) in [(0, 1, 0.7), (1, 2, -0.4), (2, 3, 0.5), (0, 3, -0.9), (0, 0, 0.3), (1, 1, -0.2), (2, 2, 0.1)]:
        J[a, b] = v
    prob = fast.Problem(tools.GenerateNeighbors(n, J, 3))
    mlp = learned.ProposalMLP(seed=5)
    R = 512
    jp = float(oracle.jperp(np.array([G]), P, T)[0])
    w = prob.pack(torch.from_numpy(np.ones((R, n, P), np.int8)))
    states = np.array(list(itertools.product([1, -1], repeat=n * P))).reshape(-1, n, P)
    Jd = np.asarray(J.todense())
    up = np.triu(Jd, 1) + np.tril(Jd, -1).T
    H = np.array([sum(-(s[:, k] @ up @ s[:, k]) - np.diag(Jd) @ s[:, k] - jp * np.sum(s[:, k] * s[:, (k + 1) % P])
                      for k in range(P)) for s in states])
    pex = np.exp(-(H - H.min()) / T)
    pex /= pex.sum()
    Eex = (pex * H).sum()
    jpt = torch.tensor([jp], device="cuda")
    energies = []
    for it in range(400):
        fast.anneal(prob, w, [G], P, T, seed=7, sweep_base=it, jperp=jpt)
        learned.learned_pass(prob, w, P, mlp, 1.0 / T, jp, seed=8, move=it, qmin=0.05)
        if it >= 50:
            sp = prob.unpack(w, P).cpu().numpy().astype(np.float64)
            e = [sum(-(sp[r, :, k] @ up @ sp[r, :, k]) - np.diag(Jd) @ sp[r, :, k]
                     - jp * np.sum(sp[r, :, k] * sp[r, :, (k + 1) % P]) for k in range(P)) for r in range(0, R, 8)]
            energies.append(np.mean(e))
    e = np.array(energies)
    se = e.std(ddof=1) / np.sqrt(len(e) / 10.0)   # successive sweeps are correlated
    assert abs(e.mean() - Eex) < 4 * se + 0.02 * abs(Eex), (e.mean(), Eex, se)


def test_trained_proposals_accept_more_per_proposal():
    """What the network gains: fewer tried moves for the accepted ones (uniform moves are the judge)."""
    from piqmc import fast, learned
    _, prob = _problem(16, 4)
    P, R, T = 16, 32, 0.05
    X, y = _plain_records(prob, P, R)
    mlp = learned.ProposalMLP(seed=1)
    mlp.train(X, y, epochs=4, batch=4096, lr=3e-3)
    g = np.random.default_rng(9)
    spins = np.repeat(np.where(g.random((R, prob.n)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    sched = np.linspace(3.0, 1e-8, 60)
    jp = fast.jperp_schedule(sched, P, T)
    res = {}
    for kind in ("uniform", "learned"):
        w = prob.pack(torch.from_numpy(spins))
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        for gs in range(len(sched)):
            fast.anneal(prob, w, sched[gs:gs + 1], P, T, seed=3, sweep_base=gs, jperp=torch.from_numpy(jp[gs:gs + 1]).cuda())
            if kind == "uniform":
                learned.uniform_pass(prob, w, P, 1.0 / T, float(jp[gs]), seed=4, move=gs, counters=cnt)
            else:
                learned.learned_pass(prob, w, P, mlp, 1.0 / T, float(jp[gs]), seed=4, move=gs, counters=cnt)
        c = cnt.cpu().numpy()
        E = prob.energies(w, P).cpu().numpy().min(axis=1)
        res[kind] = (c[0], c[1], float(np.median(E)))
    print("uniform: proposed %d accepted %d median best E %.3f" % res["uniform"])
    print("learned: proposed %d accepted %d median best E %.3f" % res["learned"])
    assert res["learned"][0] < 0.5 * res["uniform"][0]
    assert res["learned"][1] / max(res["learned"][0], 1) > res["uniform"][1] / max(res["uniform"][0], 1)
