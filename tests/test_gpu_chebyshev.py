"""Chebyshev continuation (ACmethod 2: set_polynomial_basis, determine_GLLS,
least_squares_fit and fit_function_poly, src/ALPS_analyt.f90:268-363,
731-889) on the GPU against the oracle.

The basis, the normal matrix and its LU are computed in the same order and
rounding on both sides; the right-hand sides take log10 of f0, whose last
ulp may differ between the device and the host, so the coefficients agree
to FIT_RTOL of the largest coefficient of a row.  With the coefficients
shared, chi follows the main path's tolerance.
"""
import os

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

FIT_RTOL = 1e-11
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


def _plasma(log_max=18.0, order=30, N=40, M=80):
    po = _oracle()
    me = 1.0 / 1836.0
    sp, tabs = [], []
    for ms, qs in ((1.0, 1.0), (me, -1.0)):
        d = workloads._dist(kind=1, ms=ms, vA=1e-4, maxP=6.0)
        pp, pl, f0, _ = po.generate_f0(d, N, M)
        s = _abi.species_defaults(ns=1, qs=qs, ms=ms, ac_method=2, poly_kind=1, poly_order=order,
                                  poly_log_max=log_max)
        sp.append((s, pp, pl, f0))
    sysd = _abi.system_defaults(nspec=2, nperp=N, npar=M, kperp=0.5, kpar=0.3, vA=1e-4, Bessel_zero=1e-20)
    return sysd, sp


@pytest.mark.parametrize("log_max", [18.0, 40.0])
def test_glls_coefficients_and_disp(api, log_max):
    po = _oracle()
    sysd, sp = _plasma(log_max)
    O = po.OraclePlasma(sysd, sp)
    G = api.Plasma(sysd, sp)
    for i in range(2):
        a = G.get_fit(i).reshape(sysd.nperp + 1, -1)
        b = O.get_fit(i).reshape(sysd.nperp + 1, -1)
        scale = np.abs(b).max(axis=1, keepdims=True)
        assert np.all(np.abs(a - b) <= FIT_RTOL * scale)
        G.set_fit(i, O.get_fit(i))
    O.set_k(0.5, 0.3)
    G.set_k(0.5, 0.3)
    for om in [0.9 - 0.01j, 0.9 - 0.05j, 0.5 - 0.2j, 1.5 + 0j, 1.2 + 0.05j]:
        Do, co, _, _ = O.disp(om)
        Dg, cg, _, _ = G.disp(om)
        mag = O.disp_mag(om).reshape(2, 9) / (abs(om * om) * sysd.vA ** 2)
        for s in range(2):
            scale = np.maximum(np.abs(co[s].ravel()), 1e-3 * mag[s])
            rel = (np.abs(cg[s].ravel() - co[s].ravel()) / np.maximum(scale, 1e-300)).max()
            assert rel <= CHI_RTOL, (log_max, om, s, rel)


def test_run_input_chebyshev(api, golden_dir, tmp_path):
    """The reference's test_chebyshev.in (both species ACmethod 2, order 30)
    runs end to end on its bi-Maxwellian tables."""
    import shutil
    from alps_gb300.distribution import generate_distribution
    ref = os.path.join(golden_dir, "ref", "inputs")
    generate_distribution(os.path.join(ref, "distribution", "test_bimax_dist.in"), str(tmp_path / "distribution"))
    shutil.copyfile(os.path.join(ref, "tests", "test_chebyshev.in"), str(tmp_path / "test_chebyshev.in"))
    api.run_input(str(tmp_path / "test_chebyshev.in"), str(tmp_path))
    roots = np.loadtxt(str(tmp_path / "solution" / "test_chebyshev.roots"), ndmin=2)
    assert roots.shape[0] >= 1 and np.all(np.isfinite(roots[:, 1:3]))
