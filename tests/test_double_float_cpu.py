"""Error bounds of the double-float arithmetic of the fast path.

The fast path's pole sums and principal-value sums run in double-float
arithmetic: a value is a pair of floats h + l handled with error-free
transformations (alps_gb300/csrc/device_math.cuh: df_two_sum, df_add,
df_mul, df_mac, df_rcp_approx).  This file restates those algorithms in
numpy float32, with a fused multiply-add emulated exactly (the product of
two floats is exact in float64), and checks the error bounds the design
relies on:

  * df_rcp_approx, the reciprocal from an FP32 estimate within 1 ulp and the
    two-term series r0 (1 + d + d^2): relative error below 2^-44;
  * df_mul: relative error below 2^-44;
  * a sum of 255 products accumulated with df_mac (the node sums): error
    below 2^-40 (about 1e-12) of the sum of the terms' magnitudes.  The low
    part is normalised only when the sum is read, so its own FP32 roundings
    add up: the worst of several hundred random sums is near 2^-42, the
    median near 2^-47 (FP64 accumulation: 2^-53 per term);
  * df_exp_scaled, exp(x) = 2^k m from a Cody-Waite reduction and the
    Taylor polynomial of degree 13: relative error below 2^-46 against FP64;
  * df_cis, cos y + i sin y from a Cody-Waite reduction by pi/2 and Taylor
    polynomials in r^2: absolute error below 2^-45 against FP64 (the
    factorised Landau term of the resonant kernel uses both).

The GPU parity tests hold the device code itself to the oracle; this file
checks the algorithms' bounds on the CPU.
"""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    """float32 fused multiply-add: a*b is exact in float64; the float64 sum
    can round once before the rounding to float32, which moves a result by
    at most one float32 ulp in rare cases and is far inside the bounds
    checked here."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def quick(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def df_add(a, b):
    sh, sl = two_sum(a[0], b[0])
    return quick(sh, f32(sl + f32(a[1] + b[1])))


def df_mul(a, b):
    p = f32(a[0] * b[0])
    e = fma(a[0], b[1], fma(a[1], b[0], fma(a[0], b[0], -p)))
    return quick(p, e)


def df_mac(acc, vh, vl, r):
    p = f32(vh * r[0])
    pl = fma(vh, r[1], fma(vl, r[0], fma(vh, r[0], -p)))
    sh, sl = two_sum(acc[0], p)
    return sh, f32(acc[1] + f32(sl + pl))


def df_rcp_approx(a, r0):
    d = fma(-a[1], r0, fma(-a[0], r0, f32(1.0)))
    return r0, f32(r0 * fma(d, d, d))


def df_of(x):
    h = f32(x)
    return h, f32(x - np.float64(h))


def val(a):
    return np.float64(a[0]) + np.float64(a[1])


def _rcp_estimate(h, rng):
    """an FP32 reciprocal within 1 ulp (rcp.approx's bound): the rounded
    reciprocal moved by up to one ulp either way"""
    r = f32(1.0 / np.float64(h))
    k = rng.integers(-1, 2)
    if k > 0:
        r = np.nextafter(r, f32(np.inf), dtype=np.float32)
    elif k < 0:
        r = np.nextafter(r, f32(-np.inf), dtype=np.float32)
    return r


def test_reciprocal_bound():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(4000):
        x = rng.uniform(0.5, 2.0) * 2.0 ** rng.integers(-30, 30) * rng.choice([-1.0, 1.0])
        a = df_of(x)
        r = df_rcp_approx(a, _rcp_estimate(a[0], rng))
        exact = 1.0 / val(a)
        worst = max(worst, abs(val(r) - exact) / abs(exact))
    assert worst < 2.0 ** -44, worst


def test_product_bound():
    rng = np.random.default_rng(12)
    worst = 0.0
    for _ in range(4000):
        a = df_of(rng.normal() * 2.0 ** rng.integers(-20, 20))
        b = df_of(rng.normal() * 2.0 ** rng.integers(-20, 20))
        p = df_mul(a, b)
        exact = val(a) * val(b)
        if exact != 0.0:
            worst = max(worst, abs(val(p) - exact) / abs(exact))
    assert worst < 2.0 ** -44, worst


def test_node_sum_bound():
    """255 terms V_j R_j with V as float pairs and R a double-float weight,
    accumulated with df_mac from zero, as one node sum of the pole-sum
    kernel does; sums with cancelling signs and with one sign."""
    rng = np.random.default_rng(13)
    for trial in range(40):
        v = rng.normal(size=255) * np.exp(rng.normal(size=255))
        w = 1.0 / rng.uniform(0.05, 3.0, size=255)
        if trial % 2:
            v = np.abs(v)
        else:
            w = w * rng.choice([-1.0, 1.0], size=255)
        acc = (f32(0.0), f32(0.0))
        exact = 0.0
        mag = 0.0
        for vj, wj in zip(v, w):
            vp = df_of(vj)
            rp = df_of(wj)
            acc = df_mac(acc, vp[0], vp[1], rp)
            t = val(vp) * val(rp)
            exact += t
            mag += abs(t)
        assert abs(val(acc) - exact) <= 2.0 ** -40 * mag, (trial, val(acc), exact, mag)


# 1/j! as float pairs, as in device_math.cuh (c_inv_fact)
def _inv_fact_pairs():
    from fractions import Fraction
    out = []
    f = Fraction(1)
    for j in range(19):
        if j:
            f /= j
        h = f32(float(f))
        out.append((h, f32(float(f - Fraction(float(h))))))
    return out


INV_FACT = _inv_fact_pairs()


def df_scale(a, s):
    return f32(a[0] * s), f32(a[1] * s)


def df_exp_scaled(x):
    """exp(x) = 2^k m (device_math.cuh df_exp_scaled): Cody-Waite reduction
    in FP64, Taylor polynomial of degree 13 of exp(r), |r| <= ln(2)/2"""
    kd = np.rint(x * 1.4426950408889634)
    r = np.float64(x) - kd * 0.6931471803691238  # exact product (|k| < 2^21, 32-bit ln2_hi)
    r = r - kd * 1.9082149292705877e-10
    q = df_of(r)
    p = INV_FACT[13]
    for j in range(12, -1, -1):
        p = df_add(df_mul(p, q), INV_FACT[j])
    return int(kd), p


def df_cis(y):
    """cos y + i sin y (device_math.cuh df_cis): Cody-Waite reduction by
    pi/2 in FP64, Taylor polynomials in r^2 of degree 8, quadrant by q mod 4"""
    qd = np.rint(y * 0.6366197723675814)
    r = np.float64(y) - qd * 1.5707963267341256
    r = r - qd * 6.077100506303966e-11
    r = r - qd * 2.0222662487959506e-21
    rd = df_of(r)
    sq = df_mul(rd, rd)
    ms = (f32(-sq[0]), f32(-sq[1]))
    ps, pc = INV_FACT[17], INV_FACT[16]
    for j in range(7, -1, -1):
        ps = df_add(df_mul(ps, ms), INV_FACT[2 * j + 1])
        pc = df_add(df_mul(pc, ms), INV_FACT[2 * j])
    sv = df_mul(ps, rd)
    neg = lambda a: (f32(-a[0]), f32(-a[1]))
    qm = int(qd) & 3
    c = [pc, neg(sv), neg(pc), sv][qm]
    s = [sv, pc, neg(sv), neg(pc)][qm]
    return c, s


def test_exp_scaled_bound():
    """relative error of 2^k m against FP64 exp on |x| <= 700: below 2^-46
    (the argument is taken as exact; FP64 exp rounds its result, 2^-53)"""
    rng = np.random.default_rng(14)
    worst = 0.0
    for x in np.concatenate([rng.uniform(-700, 700, 1500), rng.uniform(-2, 2, 500), [0.0, 1e-300, -0.3465, 0.3466]]):
        k, m = df_exp_scaled(x)
        got = np.ldexp(val(m), k)
        exact = np.exp(np.float64(x))
        worst = max(worst, abs(got - exact) / exact)
        assert 0.69 < val(m) < 1.43
    assert worst < 2.0 ** -46, worst


def test_cis_bound():
    """absolute error of cos and sin against FP64 on |y| <= 1000: below
    2^-45 (FP64's own result and the input's rounding dominate near 1000)"""
    rng = np.random.default_rng(15)
    worst = 0.0
    for y in np.concatenate([rng.uniform(-1000, 1000, 1000), rng.uniform(-4, 4, 1000), [0.0, np.pi / 4, -np.pi / 2]]):
        c, s = df_cis(y)
        worst = max(worst, abs(val(c) - np.cos(y)), abs(val(s) - np.sin(y)))
    assert worst < 2.0 ** -45, worst
