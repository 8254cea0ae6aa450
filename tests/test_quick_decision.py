"""The quick Metropolis decision of the reference-order kernels (quick_decide and quick_scale
in csrc/reforder.cu), restated with numpy float32 arithmetic: whenever it decides, it agrees
with the reference's test exp((double)(e / T)) > rand() / RAND_MAX (generated piqmc/qmc.c:
2417-2428, FP32 quotient, FP64 exp), and it never decides a close call of the exact path.

ex2.approx is hardware; here it is modelled as the exact 2^x times (1 + eps) with eps at the
edges of the bound that pq_guard_band_probe checks on the GPU (5e-5), both signs.  The
argument roundings (fl(1/T), fl(.. * log2 e), fl(e * rl)) and the uniform's rounding are
exact IEEE float32 operations here as on the device."""
import numpy as np

f32 = np.float32
f64 = np.float64
RAND_MAX = 2 ** 31 - 1
EX2_BOUND = 5e-5


def quick_scale(T):
    return (f32(1.0) / T) * f32(1.44269502162933349609375)


def quick_decide(e, rl, rv, eps):
    """1 accept, 0 reject, -1 undecided; the hardware 2^x is exact * (1 + eps)."""
    x = e * rl
    with np.errstate(over="ignore", under="ignore"):
        pf = (np.exp2(x.astype(f64)) * (1.0 + eps)).astype(f32)
        qf = rv.astype(f32) * f32(4.656612873077392578125e-10)
        acc = pf > qf * f32(1.0001)
        rej = pf < qf * f32(0.9999)
    out = np.where(acc, 1, np.where(rej, 0, -1))
    return np.where((rv <= 0) | ~(e <= 0), -1, out)


def reference_decision(e, T, rv):
    with np.errstate(under="ignore", over="ignore"):
        ex = np.exp((e / T).astype(f64))
    q = rv.astype(f64) / RAND_MAX
    return ex > q, ex, q


def check(e, T, rv):
    e, T = e.astype(f32), f32(T)
    rl = quick_scale(T)
    ref, ex, q = reference_decision(e, T, rv)
    close = (np.abs(ex - q) <= 1e-15 * np.maximum(ex, q)) | ((q == 0.0) & (ex < 1e-300))
    decided = 0
    for eps in (-EX2_BOUND, 0.0, EX2_BOUND):
        d = quick_decide(e, rl, rv, eps)
        m = d >= 0
        bad = m & ((d == 1) != ref)
        assert not bad.any(), (e[bad][:4], T, rv[bad][:4], d[bad][:4])
        assert not (m & close).any()
        decided = max(decided, m.mean())
    return decided


def test_random_energies_and_temperatures():
    g = np.random.default_rng(0)
    m = 400_000
    for T in (1e-6, 0.05, 0.3, 1.0, 7.5, 1e3, 3.0e30):
        e = -np.abs(g.normal(0, 1, m) * np.exp(g.uniform(-10, 6, m))) * T
        rv = g.integers(0, RAND_MAX + 1, m)
        assert check(e, T, rv) > 0.99


def test_decisions_at_the_uniform():
    """Energies whose exp lands within a few FP32 ulps of the uniform, where the band matters."""
    g = np.random.default_rng(1)
    m = 400_000
    for T in (0.05, 1.0, 13.0):
        rv = g.integers(1, RAND_MAX + 1, m)
        q = rv / RAND_MAX
        e = (np.log(q) * T).astype(f32)
        for k in (-3, -1, 0, 1, 3):
            ek = e.copy()
            for _ in range(abs(k)):
                ek = np.nextafter(ek, f32(0) if k > 0 else f32(-np.inf), dtype=f32)
            check(np.minimum(ek, f32(0)), T, rv)
        # a relative distance just outside the band decides
        e_far = (np.log(q * (1 + 3e-4)) * T).astype(f32)
        assert check(np.minimum(e_far, f32(0)), T, rv) > 0.9


def test_tiny_uniforms_and_deep_exponents():
    """Near the smallest nonzero uniform (2^-31) and for exponents far below it."""
    g = np.random.default_rng(2)
    m = 200_000
    T = 0.05
    rv = g.integers(1, 64, m)
    e = (np.log(rv / RAND_MAX) * T * g.uniform(0.98, 1.02, m)).astype(f32)
    check(e, T, rv)
    e = (-g.uniform(20, 200, m) * T).astype(f32)        # exp(-20 .. -200): below 2^-31 or denormal
    assert check(e, T, g.integers(1, RAND_MAX + 1, m)) > 0.99
    # rv == 0 and e > 0 are left to the exact path
    assert (quick_decide(np.array([-1.0, 0.5], f32), quick_scale(f32(1)), np.array([0, 5]), 0.0) == -1).all()


def _orc_expf(y):
    import oracle
    f = np.frompyfunc(lambda v: float(oracle.lib().orc_expf(float(v))), 1, 1)
    return f(y).astype(f32)


def packed_decide(s, u, m2beta, eps):
    """decide() of the packed sweep (csrc/sweep_core.cuh): flip when s < 0, else the guard
    band around the hardware 2^x (modelled exact * (1 + eps), flushed below FLT_MIN), else
    u < expf_neg(fl(s * m2beta))."""
    m2blog2e = m2beta * f32(1.44269502162933349609375)
    with np.errstate(over="ignore", under="ignore"):
        pf = (np.exp2((s * m2blog2e).astype(f64)) * (1.0 + eps)).astype(f32)
    pf = np.where(pf < f32(1.17549435e-38), f32(0), pf)
    rej = u > pf * f32(1.0001)
    acc = (u < pf * f32(0.9999)) & (pf > f32(1e-30))
    quick = np.where(rej, 0, np.where(acc, 1, -1))
    quick = np.where(s < 0, 1, quick)
    return quick


def test_packed_sweep_decision_band():
    """The packed sweep's quick decision equals the oracle's rule u < expf_neg(fl(-2 sum beta))
    (oracle/fast_oracle.c) wherever it decides."""
    g = np.random.default_rng(3)
    m = 150_000
    for beta in (f32(0.3), f32(1.0), f32(20.0), f32(1.0e3)):
        m2beta = f32(-2.0) * beta
        s = np.abs(g.normal(0, 1, m) * np.exp(g.uniform(-12, 4, m))).astype(f32) / beta
        y = s * m2beta
        ex = _orc_expf(y)
        # uniforms of the kernel (k 2^-23): random, and the grid points next to expf_neg
        k = np.floor(ex.astype(f64) * 2 ** 23)
        us = [g.integers(0, 2 ** 23, m) * 2.0 ** -23]
        us += [np.clip(k + d, 0, 2 ** 23 - 1) * 2.0 ** -23 for d in (-2, -1, 0, 1, 2)]
        for u in us:
            u = u.astype(f32)
            want = u < ex
            for eps in (-EX2_BOUND, 0.0, EX2_BOUND):
                d = packed_decide(s, u, m2beta, eps)
                bad = (d >= 0) & ((d == 1) != want)
                assert not bad.any(), (beta, s[bad][:4], u[bad][:4], ex[bad][:4])
    # negative sums always flip
    assert (packed_decide(np.array([-1e-30, -5.0], f32), np.array([0.9, 0.0], f32), f32(-2), 0.0) == 1).all()


def fp32_decide(x, rv):
    """fp32_decide of the reference-order kernels: expf_neg (the oracle's orc_expf, the same
    function bit for bit) against the FP32 uniform with a 2e-6 band; -1 undecided."""
    ef = _orc_expf(x)
    qf = rv.astype(f32) * f32(4.656612873077392578125e-10)
    out = np.where(ef > qf * f32(1.000002), 1, np.where(ef < qf * f32(0.999998), 0, -1))
    return np.where((rv <= 0) | ~(x <= 0), -1, out)


def test_fp32_decision_band():
    """Wherever fp32_decide decides, it equals exp((double)x) > rv / RAND_MAX and the case is
    not a close call of the FP64 path."""
    g = np.random.default_rng(4)
    m = 200_000
    x = (-np.abs(g.normal(0, 1, m)) * np.exp(g.uniform(-12, 4.5, m))).astype(f32)
    ex = np.exp(x.astype(f64))
    rvs = [g.integers(0, RAND_MAX + 1, m)]
    k = np.floor(ex * RAND_MAX)
    # offsets past the FP32 rounding of rv (up to 64 units near 2^31)
    rvs += [np.clip(k + d, 0, RAND_MAX).astype(np.int64) for d in (-100, -63, -31, -1, 0, 1, 2, 32, 64, 100)]
    for rv in rvs:
        q = rv / RAND_MAX
        close = (np.abs(ex - q) <= 1e-15 * np.maximum(ex, q)) | ((q == 0.0) & (ex < 1e-300))
        d = fp32_decide(x, rv)
        m_ = d >= 0
        assert not (m_ & ((d == 1) != (ex > q))).any()
        assert not (m_ & close).any()
    assert (fp32_decide(np.array([-1.0, 0.5], f32), np.array([0, 5])) == -1).all()
