"""om_double_scan (src/ALPS_fns.f90:2904-3591) restated in Python over the
oracle, for checking the library's scan_option 2 driver (alps_run_input).

Test infrastructure: it drives an oracle.pyoracle.OraclePlasma.
"""
import math

import numpy as np


def scan_k(sc, it, kp0, kz0, th0, k0, kperp, kpar):
    """One step of a k scan (the select case of om_scan / om_double_scan)."""
    t, lg = sc["type_s"], math.log10
    if t == 0:
        if sc["log_scan"]:
            return 10.0 ** (lg(kp0) + sc["diff"] * it), 10.0 ** (lg(kz0) + sc["diff2"] * it)
        return kp0 + sc["diff"] * it, kz0 + sc["diff2"] * it
    if t == 1:
        th = 10.0 ** (lg(th0) + sc["diff"] * it) if sc["log_scan"] else th0 + sc["diff"] * it
        return k0 * math.sin(th), k0 * math.cos(th)
    if t == 2:
        kt = 10.0 ** (lg(k0) + sc["diff"] * it) if sc["log_scan"] else k0 + sc["diff"] * it
        return kt * math.sin(th0), kt * math.cos(th0)
    if t == 3:
        return (10.0 ** (lg(kp0) + sc["diff"] * it) if sc["log_scan"] else kp0 + sc["diff"] * it), kpar
    return kperp, (10.0 ** (lg(kz0) + sc["diff"] * it) if sc["log_scan"] else kz0 + sc["diff"] * it)


def double_scan(P, s1, s2, wroots, kperp, kpar, D_gap, method=2):
    """Rows of the .scan files: out[root] = list of blocks, each block the
    rows (kperp, kpar, Re, Im) of one inner scan."""
    nroots = len(wroots)
    wroots = list(wroots)
    nt, nt2 = s1["n_out"] * s1["n_res"], s2["n_out"] * s2["n_res"]
    kperp_last, kpar_last = kperp, kpar
    theta_0 = math.atan(kperp_last / kpar_last)
    k_0 = math.sqrt(kperp_last ** 2 + kpar_last ** 2)
    omlast = list(wroots)
    jump = [True] * nroots
    out = [[] for _ in range(nroots)]
    for it in range(nt + 1):
        kperp, kpar = scan_k(s1, it, kperp_last, kpar_last, theta_0, k_0, kperp, kpar)
        P.set_k(kperp, kpar)
        if not any(jump):
            raise RuntimeError("roots diverged")
        for r in range(nroots):
            if not jump[r]:
                continue
            om = P.secant(omlast[r], method)[0]
            wroots[r] = omlast[r] = om
            if not math.isfinite(om.real):
                jump[r] = False
            for imm in range(r):
                if abs(wroots[r] - wroots[imm]) < D_gap:
                    wroots[r] = 0j
                    jump[r] = False
        if it % s1["n_res"] == 0:
            blocks = [[] for _ in range(nroots)]
            for it2 in range(nt2 + 1):
                if it2 == 0:
                    kperpi, kpari = kperp, kpar
                    theta_i = math.atan(kperpi / kpari)
                    k_i = math.sqrt(kperpi ** 2 + kpari ** 2)
                    wroots = list(omlast)
                kperp, kpar = scan_k(s2, it2, kperpi, kpari, theta_i, k_i, kperp, kpar)
                P.set_k(kperp, kpar)
                for r in range(nroots):
                    if not jump[r]:
                        continue
                    om = P.secant(wroots[r], method)[0]
                    wroots[r] = om
                    tmp = P.disp(om)[0]
                    if not math.isfinite(om.real) or abs(tmp) > 1e100:
                        jump[r] = False
                    for imm in range(r):
                        if abs(wroots[r] - wroots[imm]) < D_gap:
                            wroots[r] = 0j
                            jump[r] = False
                    if it2 % s2["n_res"] == 0:
                        blocks[r].append((kperp, kpar, wroots[r].real, wroots[r].imag))
            for r in range(nroots):
                out[r].append(np.array(blocks[r]))
        if s2["type_s"] == 2:
            kperp, kpar = scan_k(dict(s2, type_s=0), 0, kperp_last, kpar_last, theta_0, k_0, kperp, kpar)
        else:
            kperp, kpar = scan_k(s2, 0, kperp_last, kpar_last, theta_0, k_0, kperp, kpar)
    return out
