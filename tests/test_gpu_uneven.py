"""Parity on draws of the uneven-batch configuration (1-3 species from
{bi-Maxwellian, drifting proton beam, bi-kappa}, random anisotropy, beta,
k_perp rho_p in [0.01, 10] and angle in [20, 88] degrees), on grids small
enough for the oracle.  Seeded; both precision paths; fits shared so that
only the dispersion path is compared (tolerances of test_gpu_parity).
"""
import os

import numpy as np
import pytest

from alps_gb300 import workloads

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


def _draws(n=8, seed=3):
    rng = np.random.default_rng(seed)
    return [workloads.uneven_plasma(rng, grid=(32, 64) if i % 2 == 0 else (48, 96)) for i in range(n)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_uneven_draws_match_oracle(api, precision):
    po = _oracle()
    for w in _draws():
        s, sp = workloads.build_uneven(w, po.generate_f0)
        O = po.OraclePlasma(s, sp)
        G = api.Plasma(s, sp, precision=precision)
        for i in range(s.nspec):
            G.set_fit(i, O.get_fit(i))
        O.set_k(*w["k"])
        G.set_k(*w["k"])
        assert G.nmax() == O.nmax()
        for om in [0.5 - 0.05j, 1.3 + 0.02j, 0.2 - 0.3j]:
            Do, co, _, _ = O.disp(om)
            Dg, cg, _, _ = G.disp(om)
            mag = O.disp_mag(om).reshape(s.nspec, 9) / (abs(om * om) * s.vA ** 2)
            for k in range(s.nspec):
                scale = np.maximum(np.abs(co[k].ravel()), 1e-3 * mag[k])
                rel = (np.abs(cg[k].ravel() - co[k].ravel()) / np.maximum(scale, 1e-300)).max()
                assert rel <= CHI_RTOL, (w["species_kinds"], w["k"], om, k, rel)


def test_uneven_batches(api):
    """Each draw's batch equals its single evaluations; different plasmas
    evaluated one after another on the device do not disturb each other."""
    po = _oracle()
    plasmas = []
    for w in _draws(4, seed=5):
        s, sp = workloads.build_uneven(w, po.generate_f0)
        G = api.Plasma(s, sp)
        G.set_k(*w["k"])
        plasmas.append(G)
    oms = np.array([0.5 - 0.05j, 1.3 + 0.02j, 0.2 - 0.3j, 0.9 + 0j])
    first = [G.disp_batch(oms) for G in plasmas]
    again = [G.disp_batch(oms) for G in reversed(plasmas)][::-1]
    for a, b, G in zip(first, again, plasmas):
        assert np.array_equal(a, b)
        single = np.array([G.disp(om)[0] for om in oms])
        np.testing.assert_allclose(a, single, rtol=1e-13)
