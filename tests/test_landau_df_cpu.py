"""The factorised Landau term of the resonant kernel's item phase
(disp_kernels.cu, one Maxwellian row Gaussian), restated twice on the CPU:
as the FP64 formula it replaces and as the kernel's double-float form
(numpy float32 restatements of device_math.cuh from
test_double_float_cpu.py).  The double-float form keeps the powers of two
of exp(-p2r (p - p3r)^2) and of X = exp(-2 p2r pd (p - p3r)) apart and
applies them at the end, so it holds where |Re| of either exponent is in
the hundreds (X or 1/X beyond the float range); the check is 1e-12 of the
largest entry of the family's result against the FP64 form, for resonance
momenta with small and large real and imaginary parts, and the sign of a
negative charge.
"""
import numpy as np

from test_double_float_cpu import (df_add, df_cis, df_exp_scaled, df_mul, df_of, df_rcp_approx, f32, val)


def _neg(a):
    return f32(-a[0]), f32(-a[1])


def _scale(a, s):
    return f32(a[0] * s), f32(a[1] * s)


def _cmul(a, b):
    return (df_add(df_mul(a[0], b[0]), _neg(df_mul(a[1], b[1]))), df_add(df_mul(a[0], b[1]), df_mul(a[1], b[0])))


def _cadd(a, b):
    return df_add(a[0], b[0]), df_add(a[1], b[1])


def _rmul(a, s):
    return df_mul(a[0], s), df_mul(a[1], s)


def _fp64(p, pd, p2r, p3r, lm, om, kap, ql, pref, fi):
    """the FP64 formula (the plain path's factorised rows)"""
    G = lambda x: np.exp(-p2r * (x - p3r) ** 2)
    lgc = np.exp(-p2r * pd * pd)
    G0 = G(p)
    X = np.exp(-2.0 * p2r * pd * (p - p3r))
    Gp, Gm = lgc * G0 * X, lgc * G0 / X
    poly = lambda c, x: sum(c[m] * x ** m for m in range(5))
    sumF = []
    for F in range(3):
        c = lm[F]
        Spar = (Gp * poly(c[:5], p + pd) - Gm * poly(c[:5], p - pd)) / (2.0 * pd)
        Sperp = G0 * poly(c[5:], p)
        sumF.append(ql * (kap * (Spar - p * Sperp) + om * Sperp))
    res = []
    for e in range(6):
        ce = p * p if e == 2 else (p if e in (4, 5) else 1.0)
        fam = 1 if e == 1 else (2 if e in (3, 5) else 0)
        res.append(pref[e] * ce * sumF[fam] * (1j * fi))
    return np.array(res)


def _df(p, pd, p2r, p3r, lm, om, kap, ql, pref, fi):
    """the kernel's double-float form, exponents kept apart"""
    lgc = np.exp(-p2r * pd * pd)
    dx, dy = p.real - p3r, p.imag
    k0, m0 = df_exp_scaled(-p2r * ((dx - dy) * (dx + dy)))
    c0, s0 = df_cis(-2.0 * p2r * dx * dy)
    lcx = -2.0 * p2r * pd
    kx, mx = df_exp_scaled(lcx * dx)
    cx, sx = df_cis(lcx * dy)
    akx = abs(kx)
    g0 = (df_mul(m0, c0), df_mul(m0, s0))
    xm = (df_mul(mx, cx), df_mul(mx, sx))
    ixm = df_rcp_approx(mx, f32(1.0 / np.float64(mx[0])))
    xi = (df_mul(ixm, cx), _neg(df_mul(ixm, sx)))
    sc = f32(np.ldexp(1.0, -2 * akx)) if 2 * akx <= 126 else f32(0.0)
    fa = xm if kx >= 0 else (_scale(xm[0], sc), _scale(xm[1], sc))
    fb = (_scale(xi[0], sc), _scale(xi[1], sc)) if kx >= 0 else xi
    pz = (df_of(p.real), df_of(p.imag))
    pdd = df_of(pd)
    zp = [[None] * 5 for _ in range(3)]
    zp[0][1] = (df_add(pz[0], pdd), pz[1])
    zp[1][1] = (df_add(pz[0], _neg(pdd)), pz[1])
    zp[2][1] = pz
    for u in range(3):
        zp[u][2] = _cmul(zp[u][1], zp[u][1])
        zp[u][3] = _cmul(zp[u][2], zp[u][1])
        zp[u][4] = _cmul(zp[u][2], zp[u][2])

    def poly(c, u):
        acc = (df_of(c[0]), (f32(0), f32(0)))
        for m in range(1, 5):
            acc = _cadd(acc, _rmul(zp[u][m], df_of(c[m])))
        return acc

    omd, kapd, qld = (df_of(om.real), df_of(om.imag)), df_of(kap), df_of(ql)
    wk = (df_add(omd[0], _neg(df_mul(kapd, pz[0]))), df_add(omd[1], _neg(df_mul(kapd, pz[1]))))
    two_pd = _scale(pdd, f32(2.0))
    lgd = df_mul(df_of(lgc), df_rcp_approx(two_pd, f32(1.0 / np.float64(two_pd[0]))))
    sp = f32(np.ldexp(1.0, -akx)) if akx <= 126 else f32(0.0)
    sumF = []
    for F in range(3):
        c = lm[F]
        Pp, Pm, Qp = poly(c[:5], 0), poly(c[:5], 1), poly(c[5:], 2)
        A, B = _cmul(fa, Pp), _cmul(fb, Pm)
        br = (df_add(A[0], _neg(B[0])), df_add(A[1], _neg(B[1])))
        spar = _rmul(_cmul(g0, br), lgd)
        sperp = _cmul(_cmul(g0, Qp), wk)
        t = (df_add(df_mul(spar[0], kapd), _scale(sperp[0], sp)), df_add(df_mul(spar[1], kapd), _scale(sperp[1], sp)))
        sumF.append(_rmul(t, qld))
    e_all = k0 + akx
    p2 = _cmul(pz, pz)
    res = []
    for e in range(6):
        fam = 1 if e == 1 else (2 if e in (3, 5) else 0)
        v = sumF[fam]
        if e == 2:
            v = _cmul(v, p2)
        elif e in (4, 5):
            v = _cmul(v, pz)
        im = e in (3, 5)
        f = df_of(-pref[e].imag * fi if im else pref[e].real * fi)
        vx, vy = val(df_mul(v[0], f)), val(df_mul(v[1], f))
        z = complex(vx, vy) if im else complex(-vy, vx)
        res.append(np.ldexp(z.real, e_all) + 1j * np.ldexp(z.imag, e_all))
    return np.array(res)


def test_factorised_landau_double_float_form():
    rng = np.random.default_rng(21)
    pd, p2r, p3r = 0.047, 0.9, 0.3
    cases = [1.2 - 0.3j, -2.5 - 1.1j, 4.0 - 0.05j, 0.1 - 2.5j, 6.0 - 4.0j, -30.0 - 2.0j]
    for k, p in enumerate(cases):
        lm = rng.standard_normal((3, 10))
        om = complex(rng.uniform(0.2, 3.0), rng.uniform(-0.5, 0.0))
        kap = rng.uniform(0.05, 2.0)
        ql = -3.3 if k % 2 else 3.3  # the charge's sign stays in q / |k_par|
        pref = np.array([1.7, 0.8, 0.8, 0.6j, 1.1, -0.8j])
        fi = -0.02 * np.pi * 2.0 * np.pi * 2.0
        a = _fp64(p, pd, p2r, p3r, lm, om, kap, ql, pref, fi)
        b = _df(p, pd, p2r, p3r, lm, om, kap, ql, pref, fi)
        assert np.all(np.isfinite(b)), (p, b)
        for fam_entries in ([0, 2, 4], [1], [3, 5]):
            scale = np.abs(a[fam_entries]).max()
            assert np.abs(b[fam_entries] - a[fam_entries]).max() <= 1e-12 * scale, (p, fam_entries)


def test_factorised_landau_exponents_beyond_the_float_range():
    """narrow row Gaussians and wide cells: X = exp(-2 p2r pd (p - p3r))
    near 2^(+-216), far outside FP32, and G(p) near 2^90"""
    rng = np.random.default_rng(5)
    pref = np.array([1.7, 0.8, 0.8, 0.6j, 1.1, -0.8j])
    fi = -0.02 * np.pi * 2.0 * np.pi * 2.0
    for p2r, pd, p3r, p in [(50.0, 0.5, 0.3, 3.3 - 3.2j), (50.0, 0.5, 0.3, -2.7 - 3.1j),
                            (20.0, 1.0, 0.0, 4.0 - 4.1j), (20.0, 1.0, 0.0, -4.0 - 4.05j)]:
        lm = rng.standard_normal((3, 10))
        a = _fp64(p, pd, p2r, p3r, lm, 0.7 - 0.2j, 0.6, -3.3, pref, fi)
        b = _df(p, pd, p2r, p3r, lm, 0.7 - 0.2j, 0.6, -3.3, pref, fi)
        for fam_entries in ([0, 2, 4], [1], [3, 5]):
            scale = np.abs(a[fam_entries]).max()
            assert scale > 0 and np.abs(b[fam_entries] - a[fam_entries]).max() <= 1e-12 * scale, (p, fam_entries)
