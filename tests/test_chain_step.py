"""The FP32 step of the reference-order FP64 chains (chain_step32 in csrc/reforder.cu), restated
with numpy float32 arithmetic (IEEE round to nearest, no fused operations): whenever its check
accepts, the candidate is the reference's (float)((double)e + t).  Random and adversarial inputs:
sums within a few FP64 ulps of an FP32 rounding midpoint, cancellation, results at powers of
two, tiny and huge magnitudes."""
import numpy as np

f32 = np.float32
f64 = np.float64


def split(t):
    """t (FP64) = t1 + t2 + t3 in FP32 pieces, and whether the split is exact (the term warp's)."""
    with np.errstate(over="ignore", invalid="ignore"):
        t1 = t.astype(f32)
        r1 = t - t1.astype(f64)
        t2 = r1.astype(f32)
        r2 = r1 - t2.astype(f64)
        t3 = r2.astype(f32)
        ok = (t3.astype(f64) == r2) & (np.abs(t1) <= f32(3.0e38))
    return t1, t2, t3, ok


def chain_step32(e, t1, t2, t3):
    """The device step, operation for operation."""
    with np.errstate(over="ignore", invalid="ignore"):
        s = e + t1
        bb = s - e
        a = (e - (s - bb)) + (t1 - bb)
        wf = (a + t2) + t3
        c = s + wf
        d = (s - c) + wf
        sum_abs = (np.abs(a) + np.abs(t2)) + np.abs(t3)
        bound = ((np.abs(d) * f32(1.0000005)) + (sum_abs * f32(4.76837158203125e-7))) + \
                ((np.abs(c) * f32(4.44089209850062616e-16)) + f32(1.17549435e-38))
        cb = c.view(np.uint32) & np.uint32(0x7FFFFFFF)
        E = cb >> np.uint32(23)
        pow2 = (cb & np.uint32(0x7FFFFF)) == 0
        hb = np.where(pow2, E - np.uint32(25), E - np.uint32(24)).astype(np.uint32) << np.uint32(23)
        h = hb.view(f32)
        ok = (E >= 26) & (E <= 253) & (np.abs(wf) <= f32(0.25) * np.abs(s)) & (bound < h)
    return c, ok


def reference(e, t):
    with np.errstate(over="ignore"):
        return (e.astype(f64) + t).astype(f32)


def check(e, t):
    e = e.astype(f32)
    t1, t2, t3, sok = split(t)
    c, ok = chain_step32(e, t1, t2, t3)
    acc = ok & sok
    ref = reference(e, t)
    bad = acc & (c != ref) & ~(np.isnan(ref))
    assert not bad.any(), (e[bad][:5], t[bad][:5], c[bad][:5], ref[bad][:5])
    return acc.mean()


def test_random_terms_and_sums():
    g = np.random.default_rng(0)
    m = 2_000_000
    e = (g.normal(0, 1, m) * np.exp(g.uniform(-20, 20, m))).astype(f32)
    t = g.normal(0, 1, m) * np.exp(g.uniform(-20, 20, m))
    assert check(e, t) > 0.9
    # the dense chain's regime: a running sum of +-2J terms, J ~ N(0, 1/n)
    t = 2 * g.normal(0, 1 / np.sqrt(512), m)
    e = (g.normal(0, 1, m) * np.sqrt(g.integers(1, 514, m)) * 0.09).astype(f32)
    assert check(e, t) > 0.99


def test_near_ties_and_cancellation():
    g = np.random.default_rng(1)
    m = 1_000_000
    # e + t lands within a few FP64 ulps of a midpoint between two FP32 numbers
    c = (g.normal(0, 1, m) * np.exp(g.uniform(-10, 10, m))).astype(f32)
    up = np.nextafter(c, np.inf, dtype=f32)
    mid = (c.astype(f64) + up.astype(f64)) / 2
    e = (g.normal(0, 1, m) * np.exp(g.uniform(-12, 12, m))).astype(f32)
    jitter = g.integers(-4, 5, m) * np.spacing(mid)
    t = (mid - e.astype(f64)) + jitter
    check(e, t)
    # cancellation: e nearly -t
    t = g.normal(0, 1, m) * np.exp(g.uniform(-5, 5, m))
    e = (-t).astype(f32)
    check(e, t)
    check(np.nextafter(e, np.inf, dtype=f32), t)


def test_powers_of_two_and_extremes():
    g = np.random.default_rng(2)
    m = 500_000
    k = g.integers(-120, 120, m)
    sign = np.where(g.random(m) < 0.5, -1.0, 1.0)
    p2 = np.ldexp(1.0, k) * sign
    ulp = np.ldexp(1.0, k - 23)
    # sums a few FP64 ulps from the rounding midpoints on either side of a power of two: the
    # gap below it (toward zero) is half the gap above
    for off in (-ulp / 4, ulp / 2, 0.0):
        target = p2 + sign * off
        e = (target * g.uniform(0.3, 0.7, m)).astype(f32)
        t = target - e.astype(f64) + g.integers(-3, 4, m) * np.spacing(target)
        check(e, t)
    # tiny (FP32 subnormal range) and huge (near FP32 overflow) values are rejected or exact
    with np.errstate(over="ignore"):
        e = (g.normal(0, 1, m) * 1e-39).astype(f32)
        t = g.normal(0, 1, m) * 1e-39
        check(e, t)
        e = (g.normal(0, 1, m) * 1e38).astype(f32)
        t = g.normal(0, 1, m) * 1e38
        check(e, t)


def f32_of_exact(d):
    """The device's bit conversion of an FP64 value that is zero or a normal FP32 number."""
    b = d.view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    e = (hi >> np.uint32(20)) & np.uint32(0x7FF)
    sign = hi & np.uint32(0x80000000)
    man = ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)).astype(np.uint32)
    with np.errstate(over="ignore"):
        bits = np.where(e == 0, sign, sign | ((e - np.uint32(896)) << np.uint32(23)) | man).astype(np.uint32)
    return bits.view(f32)


def fp32_term_exact(v):
    a = np.abs(v)
    with np.errstate(over="ignore"):
        return (v == 0.0) | ((a >= 1.1754943508222875e-38) & (a <= 1.7014117331926443e38) &
                             (v.astype(f32).astype(f64) == v))


def test_fp32_row_conversion():
    """Rows marked FP32-valued convert bit for bit, and +-2J of them is an FP32 value."""
    g = np.random.default_rng(3)
    m = 1_000_000
    x = (g.normal(0, 1, m) * np.exp(g.uniform(-80, 80, m))).astype(f32)
    x = np.concatenate([x, np.array([0.0, -0.0, 1.17549435e-38, -3.4e38, 1.7e38], dtype=f32)])
    d = x.astype(f64)
    ok = fp32_term_exact(d)
    got = f32_of_exact(d[ok])
    assert np.array_equal(got.view(np.uint32), x[ok].view(np.uint32))
    with np.errstate(over="ignore"):
        assert np.all(np.isfinite(2 * got)) and np.array_equal((2 * got).astype(f64), 2 * d[ok])
    # values that are not FP32 numbers (or FP32 subnormals) are never marked
    y = g.normal(0, 1, m)
    assert not fp32_term_exact(y[y.astype(f32).astype(f64) != y]).any()
    assert not fp32_term_exact(np.array([1e-40, 3.0e38])).any()
