"""The algebra of the fast path's pole sums (disp_kernels.cu pole_fused),
restated in numpy FP64 and checked against the direct sums it replaces.

Per signed order the kernel sums only the three Bessel families F against
R_j = 1/(k_par (zeta - p_j)) and derives the p_par-weighted entries:

  * node sums: sum w F p R = zeta Q - C/k_par, sum w F p^2 R = zeta (sum w F
    p R) - C_p/k_par, with C, C_p the sums of w F and w F p over the summed
    ranges (the full range, or the ranges left of and right of a resonance
    window, from prefix sums);
  * far poles, Laurent series Q = f sum_k m_k t^k (d = zeta - pcen,
    t = prad/d, f = 1/(k_par d), m_k the moments of w F in x = (p -
    pcen)/prad): with T = f sum_{k>=1}, U = f sum_{k>=2}, sum w F p R =
    pcen Q + d T and sum w F p^2 R = pcen^2 Q + 2 pcen d T + d^2 U, each
    slice of js_count summing its own k (k = js mod js_count) and the
    slices owning k = 0 and k = 1 adding those terms.

These are exact identities; the check is at FP64 rounding level on grids
with a centre away from zero (a drifting species) and at poles near and
far from the grid.
"""
import numpy as np


def _grid(M=48, lo=-5.5, hi=6.5, seed=3):
    rng = np.random.default_rng(seed)
    pp = np.linspace(lo, hi, M + 1)
    F = rng.standard_normal(M + 1) * np.exp(-0.1 * pp ** 2)
    return pp, F


def _weights(M, ranges):
    """the kernel's node weights: 1 on every node of the summed ranges
    (clipped to 1..M-1), -1/2 more at each end of a range of two or more
    nodes"""
    w = np.zeros(M + 1)
    for lo, hi in ranges:
        a, b = max(lo, 1), min(hi, M - 1)
        if a > b:
            continue
        w[a:b + 1] += 1.0
        if lo < hi:
            w[a] -= 0.5
            w[b] -= 0.5
    return w


def _direct(pp, F, w, zeta, kpar, power):
    return np.sum(w * F * pp ** power / (kpar * (zeta - pp)))


def test_node_sum_identities():
    pp, F = _grid()
    M = len(pp) - 1
    kpar = 0.37
    pre = np.concatenate([[0.0], np.cumsum(F[1:M])])           # prefix sums of F over j = 1..M-1
    prep = np.concatenate([[0.0], np.cumsum((F * pp)[1:M])])
    cases = [[(1, M - 1)], [(1, 17), (25, M - 1)], [(9, M - 1)], [(1, 30)], [(5, 5)]]
    for ranges in cases:
        w = _weights(M, ranges)
        # the range sums as the kernel forms them: prefix differences minus
        # half of each end of a range of two or more nodes
        C = Cp = 0.0
        for lo, hi in ranges:
            a, b = max(lo, 1), min(hi, M - 1)
            if a > b:
                continue
            c, cp = pre[b] - pre[a - 1], prep[b] - prep[a - 1]
            if lo < hi:
                c -= 0.5 * (F[a] + F[b])
                cp -= 0.5 * (F[a] * pp[a] + F[b] * pp[b])
            C, Cp = C + c, Cp + cp
        assert abs(C - np.sum(w * F)) <= 1e-13 * np.sum(np.abs(F))
        for zeta in [1.3 + 0.2j, -3.1 - 0.05j, 4.0 + 1.0j, 0.02 + 0.3j]:
            Q = _direct(pp, F, w, zeta, kpar, 0)
            xz = zeta * Q - C / kpar
            zz = zeta * xz - Cp / kpar
            mag1 = np.sum(np.abs(w * F * pp / (kpar * (zeta - pp))))
            mag2 = np.sum(np.abs(w * F * pp ** 2 / (kpar * (zeta - pp))))
            assert abs(xz - _direct(pp, F, w, zeta, kpar, 1)) <= 1e-13 * (mag1 + abs(zeta * Q) + abs(C / kpar))
            assert abs(zz - _direct(pp, F, w, zeta, kpar, 2)) <= 1e-13 * (mag2 + abs(zeta * xz) + abs(Cp / kpar))


def test_laurent_split_over_slices():
    pp, F = _grid()
    M = len(pp) - 1
    kpar = 0.37
    w = _weights(M, [(1, M - 1)])
    pcen, prad = 0.5 * (pp[1] + pp[M - 1]), 0.5 * (pp[M - 1] - pp[1])
    x = (pp - pcen) / prad
    K = 220
    mom = np.array([np.sum(w * F * x ** k) for k in range(K)])
    for zeta in [30 + 2j, -25 - 0.3j, 15 + 0.0j, 9.0 + 4.0j]:
        d = zeta - pcen
        t, f = prad / d, 1.0 / (kpar * d)
        exact = [_direct(pp, F, w, zeta, kpar, q) for q in range(3)]
        for jsc in [1, 2, 4, 32]:
            tot = np.zeros(3, dtype=complex)
            for js in range(jsc):
                k0 = js if js >= 2 else js + jsc * ((2 - js + jsc - 1) // jsc)  # the slice's first k >= 2
                U = sum(mom[k] * f * t ** k for k in range(k0, K, jsc))
                T = U + (f * t * mom[1] if js == 1 % jsc else 0.0)
                Q = T + (f * mom[0] if js == 0 else 0.0)
                xz = pcen * Q + d * T
                tot += [Q, xz, pcen * xz + d * (pcen * T + d * U)]
            for q in range(3):
                assert abs(tot[q] - exact[q]) <= 1e-13 * abs(exact[q]), (zeta, jsc, q)
