"""Error of the fast path's node sums in their base-vector form, restated in
numpy float32 double-float arithmetic (the helpers of
test_double_float_cpu.py, which restate device_math.cuh).

For one signed order the kernel (disp_kernels.cu pole_fused) forms
R_j = (dr - iD) / (dr^2 + D^2), dr = A - k_par p_j, in double-float, sums
the 6 base vectors (three Bessel families against g1 and g2, float pairs)
against R with df_mac, combines each family as omega Q_1 + kappa Q_2 and
derives xz = zeta P_1 - C_1/k_par, zz = zeta xz - C_p1/k_par, yz = zeta P_3 -
C_3/k_par.  The check: each of the six entries within 2^-40 (9e-13) of the
FP64 sum of its 12-vector form, relative to the sum of the magnitudes of
that form's terms (what an FP64 summation's own rounding is measured
against), on poles the kernel sums over nodes: above or below the axis
inside the grid, or near its ends.  (A pole within a spacing or so of a
node and close to the axis is a resonant order: its window goes to the
principal-value sum, not to the node sum; summed over nodes anyway, the
cancellation in A - k_par p_j costs a few more bits in double-float.)
The far-pole path is checked the same way: the Laurent series of the base
vectors with the T/U split (terms k >= 2 in double-float, the tail in
FP32, the k = 0, 1 terms and the d, p_cen products in the combination),
also on grids whose centre is away from zero.
"""
import numpy as np

from test_double_float_cpu import df_add, df_mac, df_mul, df_of, df_rcp_approx, f32, val


def _neg(a):
    return f32(-a[0]), f32(-a[1])


def _cmul(a, b):
    """(a.x + i a.y)(b.x + i b.y) in double-float, as df_cmul2"""
    x = df_add(df_mul(a[0], b[0]), _neg(df_mul(a[1], b[1])))
    y = df_add(df_mul(a[0], b[1]), df_mul(a[1], b[0]))
    return x, y


def _om_comb(om, kap, v1, v2):
    r = _cmul(om, v1)
    return df_add(r[0], df_mul(kap, v2[0])), df_add(r[1], df_mul(kap, v2[1]))


def _om_combr(om, kap, c1, c2):
    return df_add(df_mul(om[0], c1), df_mul(kap, c2)), df_mul(om[1], c1)


def _case(seed, zeta, M=64, kpar=0.3):
    rng = np.random.default_rng(seed)
    pp = np.linspace(-6.0, 6.0, M + 1)
    gauss = np.exp(-0.5 * pp ** 2)
    F = rng.standard_normal((3, 2, M + 1)) * gauss  # family, g, node
    w = np.ones(M + 1)
    w[0] = w[M] = 0.0
    w[1] = w[M - 1] = 0.5
    om = complex(rng.uniform(0.2, 2.0), rng.uniform(-0.3, 0.1))
    kap = rng.uniform(0.1, 1.0)
    A, D = kpar * zeta.real, kpar * zeta.imag
    # FP64 reference: the 12-vector form (p_par factors on the vectors)
    R = 1.0 / (A - kpar * pp + 1j * D)
    fam_pow = [(0, 0), (1, 0), (0, 2), (2, 0), (0, 1), (2, 1)]  # xx yy zz xy xz yz
    ref, mag = [], []
    for fm, pw in fam_pow:
        t1 = w * F[fm, 0] * pp ** pw * R
        t2 = w * F[fm, 1] * pp ** pw * R
        ref.append(om * t1.sum() + kap * t2.sum())
        mag.append(np.sum(np.abs(om * t1)) + np.sum(np.abs(kap * t2)))
    # the kernel's double-float form
    Ad, Dd, kd, ikd = df_of(A), df_of(D), df_of(kpar), df_of(1.0 / kpar)
    D2 = df_mul(Dd, Dd)
    Q = [[(f32(0), f32(0)), (f32(0), f32(0))] for _ in range(6)]
    for j in range(1, M):
        ph = df_of(pp[j])
        dr = df_add(Ad, _neg(df_mul(kd, ph)))
        den = df_add(df_mul(dr, dr), D2)
        r0 = f32(1.0 / np.float64(den[0]))  # an FP32 estimate within 1 ulp
        r = df_rcp_approx(den, r0)
        Rr, Ri = df_mul(dr, r), _neg(df_mul(Dd, r))
        if w[j] != 1.0:
            Rr, Ri = (f32(Rr[0] * 0.5), f32(Rr[1] * 0.5)), (f32(Ri[0] * 0.5), f32(Ri[1] * 0.5))
        for b in range(6):
            vh, vl = df_of(F[b // 2, b % 2, j])
            Q[b][0] = df_mac(Q[b][0], vh, vl, Rr)
            Q[b][1] = df_mac(Q[b][1], vh, vl, Ri)
    omd, kapd = (df_of(om.real), df_of(om.imag)), df_of(kap)
    P = [_om_comb(omd, kapd, Q[2 * fm], Q[2 * fm + 1]) for fm in range(3)]
    zd = (df_mul(Ad, ikd), df_mul(Dd, ikd))
    C = lambda fm, pw, g: float(np.sum(w * F[fm, g] * pp ** pw))

    def sub_c(x, fm, pw):
        c = _om_combr(omd, kapd, df_of(C(fm, pw, 0)), df_of(C(fm, pw, 1)))
        c = (df_mul(c[0], ikd), df_mul(c[1], ikd))
        return df_add(x[0], _neg(c[0])), df_add(x[1], _neg(c[1]))

    xz = sub_c(_cmul(zd, P[0]), 0, 0)
    zz = sub_c(_cmul(zd, xz), 0, 1)
    yz = sub_c(_cmul(zd, P[2]), 2, 0)
    got = [P[0], P[1], zz, P[2], xz, yz]
    return [abs(complex(val(g[0]), val(g[1])) - rf) / mg for g, rf, mg in zip(got, ref, mag)]


def test_base_vector_node_sums_within_bound():
    worst = 0.0
    for seed, zeta in enumerate([1.3 + 0.2j, -2.1 - 0.05j, 4.0 + 1.0j, 0.02 + 0.3j, 5.9 - 0.01j, -7.5 + 0.4j]):
        worst = max(worst, max(_case(seed, zeta)))
    assert worst < 2.0 ** -40, worst


def _series_case(seed, zeta, M=64, kpar=0.3, pshift=0.0):
    """the far-pole path: Laurent series of the base vectors with the T/U
    split, terms k >= 2 in double-float up to rho^K32 <= 2^-33 (1 - rho),
    the rest in FP32, against the FP64 12-vector node sums"""
    rng = np.random.default_rng(100 + seed)
    pp = np.linspace(-6.0, 6.0, M + 1) + pshift
    F = rng.standard_normal((3, 2, M + 1)) * np.exp(-0.5 * (pp - pshift) ** 2)
    w = np.ones(M + 1)
    w[0] = w[M] = 0.0
    w[1] = w[M - 1] = 0.5
    om = complex(rng.uniform(0.2, 2.0), rng.uniform(-0.3, 0.1))
    kap = rng.uniform(0.1, 1.0)
    R = 1.0 / (kpar * (zeta - pp))
    fam_pow = [(0, 0), (1, 0), (0, 2), (2, 0), (0, 1), (2, 1)]
    ref, mag = [], []
    for fm, pw in fam_pow:
        t1 = w * F[fm, 0] * pp ** pw * R
        t2 = w * F[fm, 1] * pp ** pw * R
        ref.append(om * t1.sum() + kap * t2.sum())
        mag.append(np.sum(np.abs(om * t1)) + np.sum(np.abs(kap * t2)))
    pcen, prad = 0.5 * (pp[1] + pp[M - 1]), 0.5 * (pp[M - 1] - pp[1])
    x = (pp - pcen) / prad
    d = zeta - pcen
    rho = prad / abs(d)
    K = int(np.ceil((53 * np.log(2) - np.log1p(-rho)) / -np.log(rho))) + 1
    K32 = int(np.ceil((33 * np.log(2) - np.log1p(-rho)) / -np.log(rho))) + 1
    mom = np.array([[np.sum(w * F[b // 2, b % 2] * x ** k) for b in range(6)] for k in range(K + 1)])
    dd = (df_of(d.real), df_of(d.imag))
    den = df_add(df_mul(dd[0], dd[0]), df_mul(dd[1], dd[1]))
    r = df_rcp_approx(den, f32(1.0 / np.float64(den[0])))
    iv = (df_mul(dd[0], r), _neg(df_mul(dd[1], r)))
    prd, ikd = df_of(prad), df_of(1.0 / kpar)
    t1 = (df_mul(iv[0], prd), df_mul(iv[1], prd))
    f = (df_mul(iv[0], ikd), df_mul(iv[1], ikd))
    tp = _cmul(_cmul(f, t1), t1)  # f t^2
    U = [[(f32(0), f32(0)), (f32(0), f32(0))] for _ in range(6)]
    Uf = np.zeros((6, 2), dtype=np.float32)
    for k in range(2, K):
        if k < K32:
            for b in range(6):
                mh, ml = df_of(mom[k, b])
                U[b][0] = df_mac(U[b][0], mh, ml, tp[0])
                U[b][1] = df_mac(U[b][1], mh, ml, tp[1])
        else:
            fx, fy = f32(tp[0][0] + tp[0][1]), f32(tp[1][0] + tp[1][1])
            for b in range(6):
                m = f32(mom[k, b])
                Uf[b, 0] = f32(Uf[b, 0] + f32(m * fx))
                Uf[b, 1] = f32(Uf[b, 1] + f32(m * fy))
        tp = _cmul(tp, t1)
    Ub = [(df_add(U[b][0], (Uf[b, 0], f32(0))), df_add(U[b][1], (Uf[b, 1], f32(0)))) for b in range(6)]
    omd, kapd = (df_of(om.real), df_of(om.imag)), df_of(kap)
    Uw = [_om_comb(omd, kapd, Ub[2 * fm], Ub[2 * fm + 1]) for fm in range(3)]
    ft = _cmul(f, t1)

    def mterm(k, wgt, out):
        res = []
        for fm in range(3):
            mw = _om_combr(omd, kapd, df_of(mom[k, 2 * fm]), df_of(mom[k, 2 * fm + 1]))
            add = _cmul(wgt, mw)
            res.append((df_add(out[fm][0], add[0]), df_add(out[fm][1], add[1])))
        return res

    T = mterm(1, ft, Uw)
    Q = mterm(0, f, T)
    pcd = df_of(pcen)
    rmul = lambda a, s_: (df_mul(a[0], s_), df_mul(a[1], s_))
    cadd = lambda a, b: (df_add(a[0], b[0]), df_add(a[1], b[1]))
    xz = cadd(rmul(Q[0], pcd), _cmul(dd, T[0]))
    yz = cadd(rmul(Q[2], pcd), _cmul(dd, T[2]))
    zz = cadd(rmul(xz, pcd), _cmul(dd, cadd(rmul(T[0], pcd), _cmul(dd, Uw[0]))))
    got = [Q[0], Q[1], zz, Q[2], xz, yz]
    return [abs(complex(val(g[0]), val(g[1])) - rf) / mg for g, rf, mg in zip(got, ref, mag)]


def test_laurent_series_within_bound():
    worst = 0.0
    for seed, (zeta, shift) in enumerate([(9.0 + 0.3j, 0.0), (-12.0 - 0.2j, 0.0), (40.0 + 1.0j, 0.0),
                                          (150.0 - 0.5j, 0.0), (11.0 + 0.1j, 2.0), (-30.0 + 0.05j, -1.5)]):
        worst = max(worst, max(_series_case(seed, zeta, pshift=shift)))
    assert worst < 2.0 ** -40, worst
