"""Parity of the relativistic CUDA path with the oracle's relativistic branch
(src/ALPS_fns_rel.f90: derivative_f0_rel, integrate_res_rel,
landau_integrate_rel, int_ee_rel; the Lorentz factor in resU).

The reference ships no golden output for a relativistic run, so the oracle's
relativistic branch is unpinned; these tests hold the GPU path to it.

Tolerances.  The thin-plate spline behind f0_rel is a dense saddle-point
solve (LU with the same partial pivoting, no FMA contraction) whose kernel
values r^2 log r come from the device's log and pow; their last-ulp
differences from the host's leave f0_rel within F0_RTOL of the oracle's (the
cone mask, the grid vectors and every index decision are identical; measured
1.3e-14 on the reference input).  With the continuation fits shared, chi
agrees to CHI_RTOL of max(|chi_ij|, 1e-3 mag_ij), mag the sum over orders of
|contribution| (measured <= 2.7e-9, at a damped frequency where the doubled
Landau term of the type-5 continuation dominates).
"""
import os

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

F0_RTOL = 1e-12
CHI_RTOL = 1e-8
FIT_RTOL = 1e-10
ROOT_RTOL = 1e-9


def _oracle():
    from oracle import pyoracle as po
    po.set_threads(os.cpu_count() or 1)
    return po


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    return A


def _reference_input(golden_dir, ngamma=60, npparbar=60):
    """tests/test_relativistic.in with its Juettner tables (two relativistic
    species, fit type 4), on a coarser (Gamma, pparbar) grid."""
    from alps_gb300 import api as A
    from alps_gb300.distribution import read_distribution_input
    po = _oracle()
    ref = os.path.join(golden_dir, "ref", "inputs")
    inp = A.read_input(os.path.join(ref, "tests", "test_relativistic.in"))
    dist = read_distribution_input(os.path.join(ref, "distribution", "test_relativistic_dist.in"))
    s = inp.sys
    s.ngamma, s.npparbar = ngamma, npparbar
    species = [(inp.species[i],) + po.generate_f0(dist["species"][i], s.nperp, s.npar)[:3] for i in range(s.nspec)]
    return inp, s, species


def _limit_case(vA=0.1, N=30, M=60, mixed=False):
    """A Maxwellian at v_A/c = vA through fit type 5 on the Gamma rows; with
    mixed, a non-relativistic Maxwellian electron species beside it."""
    po = _oracle()
    d = workloads._dist(kind=1, ms=1.0, vA=vA, maxP=5.0)
    pp, pl, f0, ideal = po.generate_f0(d, N, M)
    sysd = _abi.system_defaults(nspec=2 if mixed else 1, nperp=N, npar=M, kperp=0.3, kpar=0.2, vA=vA,
                                Bessel_zero=1e-20, positions_principal=3, ngamma=80, npparbar=80)
    pc = 2.0 / (vA * vA)
    spT = _abi.species_defaults(ns=1, qs=1, ms=1, relat=1, fits=[(5, [ideal[0] * np.exp(pc), 1e-12, 0, 0, 0], pc)])
    species = [(spT, pp, pl, f0)]
    if mixed:
        me = 1.0 / 1836.0
        de = workloads._dist(kind=1, ms=me, vA=vA, maxP=5.0)
        pe, qe, fe, ie = po.generate_f0(de, N, M)
        spE = _abi.species_defaults(ns=1, qs=-1, ms=me, fits=[(1, list(ie[:3]) + [0, 0], ie[5])])
        species.append((spE, pe, qe, fe))
    return sysd, species


def _pair(api, sysd, species, share_fit=True):
    po = _oracle()
    O = po.OraclePlasma(sysd, species)
    G = api.Plasma(sysd, species)
    if share_fit:
        for i in range(sysd.nspec):
            G.set_fit(i, O.get_fit(i))
    O.set_k(sysd.kperp, sysd.kpar)
    G.set_k(sysd.kperp, sysd.kpar)
    return O, G


def _check_disp(O, G, om):
    Do, co, clo, wo = O.disp(om)
    Dg, cg, clg, wg = G.disp(om)
    mag = O.disp_mag(om)
    vA, kp = O.sys.vA, O.sys.kperp
    denom = abs(om * om) * vA ** 2 * (1.0 if O.sys.kperp_norm else kp ** 2)
    mag0 = mag.reshape(len(co), 9) / denom
    for s in range(len(co)):
        scale = np.maximum(np.abs(co[s].ravel()), 1e-3 * mag0[s])
        # the ee term enters chi_zz alone; give it its own scale
        scale[8] = max(scale[8], 1e-12 * np.abs(co[s]).max())
        err = np.abs(cg[s].ravel() - co[s].ravel())
        rel = (err / np.maximum(scale, 1e-300)).max()
        assert rel <= CHI_RTOL, ("chi0", s, om, rel)
    # det D through the wave tensor
    wscale = np.abs(wo).max()
    assert abs(Dg - Do) <= CHI_RTOL * 10 * (abs(Do) + wscale ** 3 * 1e-6), (om, Dg, Do)


def test_f0_rel_tables(api, golden_dir):
    inp, s, species = _reference_input(golden_dir)
    po = _oracle()
    O = po.OraclePlasma(s, species)
    G = api.Plasma(s, species)
    for i in range(s.nspec):
        go, po_, fo, ao, bo = O.get_f0_rel(i)
        gg, pg, fg, ag, bg = G.get_f0_rel(i)
        assert np.array_equal(go, gg) and np.array_equal(po_, pg)
        assert np.array_equal(fo == -1.0, fg == -1.0)       # same cone mask
        inside = fo > -1.0
        rel = np.abs(fg[inside] - fo[inside]) / np.abs(fo[inside]).max()
        assert rel.max() <= F0_RTOL, rel.max()
        # difference quotients: an error e in f0_rel moves them by <= 2 e / h
        ferr = F0_RTOL * np.abs(fo[inside]).max()
        for a, b, h in ((ag, ao, go[1] - go[0]), (bg, bo, po_[1] - po_[0])):
            assert np.abs(a - b).max() <= 2.0 * ferr / h, (np.abs(a - b).max(), ferr / h)


def test_rel_fit_gamma_rows(api, golden_dir):
    """determine_param_fit on the Gamma rows (fit type 4) from the device's
    own f0_rel."""
    inp, s, species = _reference_input(golden_dir)
    po = _oracle()
    O = po.OraclePlasma(s, species)
    G = api.Plasma(s, species)
    for i in range(s.nspec):
        a, b = G.get_fit(i), O.get_fit(i)
        assert a.shape == b.shape
        np.testing.assert_allclose(a, b, rtol=FIT_RTOL, atol=1e-300)


def test_rel_disp_reference_input(api, golden_dir):
    inp, s, species = _reference_input(golden_dir)
    O, G = _pair(api, s, species)
    assert G.nmax() == O.nmax()
    oms = [complex(g.re, g.im) for g in inp.guess[:2]] + [0.3 + 0.05j, 0.3 - 0.05j, 1.5 + 0j, 0.8 - 0.2j]
    for om in oms:
        _check_disp(O, G, om)


@pytest.mark.parametrize("mixed", [False, True])
def test_rel_disp_limit_case(api, mixed):
    """Type-5 continuation at v_A/c = 0.1 and k_perp = 0.3 (orders with
    resonant Gamma rows and non-resonant regular-grid orders), alone and beside
    a non-relativistic electron species."""
    sysd, species = _limit_case(mixed=mixed)
    O, G = _pair(api, sysd, species)
    assert G.nmax() == O.nmax()
    for om in [0.5 + 0.1j, 1.2 + 0.05j, 0.9 - 0.05j, 0.7 + 0j, 2.5 - 0.3j]:
        _check_disp(O, G, om)


def test_rel_batch_matches_single(api):
    sysd, species = _limit_case()
    O, G = _pair(api, sysd, species)
    oms = np.array([0.5 + 0.1j, 1.2 + 0.05j, 0.9 - 0.05j, 0.7 + 0j])
    batch = G.disp_batch(oms)
    single = np.array([G.disp(om)[0] for om in oms])
    np.testing.assert_allclose(batch, single, rtol=1e-13)


def test_rel_secant(api, golden_dir):
    """secant_osc polish of the reference input's two guesses."""
    inp, s, species = _reference_input(golden_dir)
    O, G = _pair(api, s, species)
    guesses = np.array([complex(g.re, g.im) for g in inp.guess[:2]])
    rg, ig, _ = G.secant(guesses, method=2)
    ro = np.array([O.secant(g, method=2)[0] for g in guesses])
    np.testing.assert_allclose(rg, ro, rtol=ROOT_RTOL)
