"""Closed-form bi-Maxwellian and cold species (use_bM = T, the NHDS branch
src/ALPS_NHDS.f90) on the GPU against the oracle's restatement.

Both evaluate the same closed form; they differ in the order of the Bessel
sum (a block reduction here, the sequential n loop in the oracle) and in the
last ulp of exp / cos / sin, so chi agrees to CHI_RTOL of max(|chi_ij|,
1e-3 mag_ij), mag the sum over orders of |Y_n(i,j)| / ell^2 (measured up
to 1.05e-11, for the electrons at the strongly damped 2.5 - 0.3i, where w(z)
in the lower half plane adds 2 exp(-z^2)).
"""
import os

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

CHI_RTOL = 1e-10


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


def _check(O, G, om):
    Do, co, clo, wo = O.disp(om)
    Dg, cg, clg, wg = G.disp(om)
    mag = O.disp_mag(om)
    vA, kp = O.sys.vA, O.sys.kperp
    denom = abs(om * om) * vA ** 2 * (1.0 if O.sys.kperp_norm else kp ** 2)
    mag0 = mag.reshape(len(co), 9) / denom
    for s in range(len(co)):
        scale = np.maximum(np.abs(co[s].ravel()), 1e-3 * mag0[s])
        rel = (np.abs(cg[s].ravel() - co[s].ravel()) / np.maximum(scale, 1e-300)).max()
        assert rel <= CHI_RTOL, ("chi0", s, om, rel)
        for l in range(3):
            sl = np.maximum(np.abs(clo[s, l].ravel()), 1e-3 * mag0[s])
            rl = (np.abs(clg[s, l].ravel() - clo[s, l].ravel()) / np.maximum(sl, 1e-300)).max()
            assert rl <= CHI_RTOL, ("chi0_low", s, l - 1, om, rl)
    assert abs(Dg - Do) <= 1e-9 * max(abs(Do), np.abs(wo).max() ** 3 * 1e-12), (om, Dg, Do)


def _pair(api, sysd, species):
    po = _oracle()
    O = po.OraclePlasma(sysd, species)
    G = api.Plasma(sysd, species)
    O.set_k(sysd.kperp, sysd.kpar)
    G.set_k(sysd.kperp, sysd.kpar)
    return O, G


def _bm(**kw):
    base = dict(ns=1, qs=1, ms=1, use_bM=1, bM_nmaxs=500, bM_Bessel_zeros=1e-50, bM_betas=1.0, bM_alphas=1.0)
    base.update(kw)
    return _abi.species_defaults(**base)


@pytest.mark.parametrize("kperp_norm", [1, 0])
def test_bimaxwellian_species(api, kperp_norm):
    """Drifting anisotropic protons and electrons in closed form, both
    kperp normalisations, frequencies above, on and below the real axis."""
    sysd = _abi.system_defaults(nspec=2, nperp=8, npar=24, kperp=0.4, kpar=0.25, vA=1e-4, kperp_norm=kperp_norm)
    sp = [(_bm(bM_betas=0.8, bM_alphas=2.0, bM_pdrifts=0.2), None, None, None),
          (_bm(qs=-1, ms=1 / 1836.0, bM_betas=1.2, bM_alphas=0.7), None, None, None)]
    O, G = _pair(api, sysd, sp)
    assert G.nmax() == O.nmax() == [1, 1]
    for om in [0.5 + 0.1j, 1.2 + 0.05j, 0.9 - 0.05j, 0.3 + 0j, 2.5 - 0.3j]:
        _check(O, G, om)


def test_cold_species(api):
    sysd = _abi.system_defaults(nspec=2, nperp=8, npar=24, kperp=0.3, kpar=0.2, vA=1e-4)
    sp = [(_bm(bM_betas=0.0, bM_pdrifts=0.1), None, None, None),
          (_bm(qs=-1, ms=1 / 1836.0, bM_betas=0.0), None, None, None)]
    O, G = _pair(api, sysd, sp)
    for om in [0.18 - 1e-15j, 0.25 + 0.01j, 1.5 + 0.2j]:
        _check(O, G, om)


def test_closed_form_beside_numerical_species(api):
    """A closed-form proton species beside a numerically integrated
    electron species (the layout of the reference's test_bimax.in)."""
    po = _oracle()
    me = 1.0 / 1836.0
    de = workloads._dist(kind=1, ms=me, vA=1e-4, maxP=6.0)
    pe, qe, fe, ie = po.generate_f0(de, 24, 48)
    sysd = _abi.system_defaults(nspec=2, nperp=24, npar=48, kperp=0.3, kpar=0.2, vA=1e-4, Bessel_zero=1e-20)
    spE = _abi.species_defaults(ns=1, qs=-1, ms=me, fits=[(1, list(ie[:3]) + [0, 0], ie[5])])
    sp = [(_bm(bM_pdrifts=0.1), None, None, None), (spE, pe, qe, fe)]
    po_ = po.OraclePlasma(sysd, sp)
    G = api.Plasma(sysd, sp)
    G.set_fit(1, po_.get_fit(1))
    po_.set_k(0.3, 0.2)
    G.set_k(0.3, 0.2)
    for om in [0.5 + 0.1j, 0.9 - 0.05j, 0.3 + 0j]:
        _check(po_, G, om)
    # eigenfunctions use the closed-form species' drift for its parallel flow
    eg = G.calc_eigen([0.5 + 0.01j])[0]
    eo = po_.calc_eigen(0.5 + 0.01j)
    a = np.array(sum(_abi.eigen_columns(eg, 2), []))
    b = np.array(sum(_abi.eigen_columns(eo, 2), []))
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()


@pytest.mark.parametrize("name", ["test_bimax", "test_cold_plasma"])
def test_run_input_closed_form_inputs(api, golden_dir, tmp_path, name):
    """The reference's inputs with use_bM species run end to end (guesses,
    refine_guess, one scan); their roots match the oracle's secant on the
    same plasma."""
    import shutil
    from alps_gb300.distribution import generate_distribution
    ref = os.path.join(golden_dir, "ref", "inputs")
    dist = os.path.join(ref, "distribution", name + "_dist.in")
    if os.path.exists(dist):
        generate_distribution(dist, str(tmp_path / "distribution"))
    shutil.copyfile(os.path.join(ref, "tests", name + ".in"), str(tmp_path / (name + ".in")))
    api.run_input(str(tmp_path / (name + ".in")), str(tmp_path))
    roots = np.loadtxt(str(tmp_path / "solution" / (name + ".roots")), ndmin=2)
    assert roots.shape[0] >= 1 and np.all(np.isfinite(roots[:, 1:3]))
    scans = [f for f in os.listdir(str(tmp_path / "solution")) if ".scan_" in f]
    assert scans
