"""calc_eigen on the GPU path (src/ALPS_fns.f90:2605-2899): fields,
velocity and density fluctuations, heating rates and their split, against
the oracle's restatement (itself pinned to the reference's .eigen/.heat
golden files) and against those files directly.

Tolerances.  E, B, U_s and delta n_s are rational functions of chi at the
root: EIG_RTOL relative to the largest entry of each vector.  The heating
rates use the anti-Hermitian part of chi and the wave energy a forward
difference over 1e-6 * Re(omega), which multiplies the 1e-10 agreement of
chi by up to ~1e6: HEAT_RTOL relative to the largest heating rate.
"""
import os

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

EIG_RTOL = 1e-8
HEAT_RTOL = 1e-4


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


@pytest.fixture(scope="module")
def kpar_fast_pair(api):
    po = _oracle()
    w = workloads.kpar_fast(nproc=4)
    system, species = workloads.build(w, po.generate_f0)
    O = po.OraclePlasma(system, species)
    G = api.Plasma(system, species)
    for i in range(system.nspec):
        G.set_fit(i, O.get_fit(i))
    O.set_k(*w["k"])
    G.set_k(*w["k"])
    return O, G, w


def _close_vec(a, b, rtol, what):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).max()
    assert np.abs(a - b).max() <= rtol * scale, (what, np.abs(a - b).max() / scale)


def _compare(eg, eo, nspec):
    ag, hg, mg = _abi.eigen_columns(eg, nspec)
    ao, ho, mo = _abi.eigen_columns(eo, nspec)
    cx = lambda v: np.array(v[0::2]) + 1j * np.array(v[1::2])
    E = slice(0, 3)
    B = slice(3, 6)
    _close_vec(cx(ag)[E], cx(ao)[E], EIG_RTOL, "electric")
    _close_vec(cx(ag)[B], cx(ao)[B], EIG_RTOL, "magnetic")
    for s in range(nspec):
        U = slice(6 + 3 * s, 9 + 3 * s)
        _close_vec(cx(ag)[U], cx(ao)[U], EIG_RTOL, "vmean")
    _close_vec(cx(ag)[6 + 3 * nspec:], cx(ao)[6 + 3 * nspec:], EIG_RTOL, "ds")
    _close_vec(hg, ho, HEAT_RTOL, "Ps, W_EM")
    _close_vec(mg, mo, HEAT_RTOL, "Ps_split")
    # exact zeros (non-resonant cyclotron terms) stay exact
    assert np.array_equal(np.array(mg) == 0.0, np.array(mo) == 0.0)


def test_calc_eigen_matches_oracle(kpar_fast_pair):
    O, G, w = kpar_fast_pair
    om, _, _ = O.secant(w["extra"]["guess"][0])
    eg = G.calc_eigen([om])[0]
    eo = O.calc_eigen(om)
    _compare(eg, eo, w["system"].nspec)


def test_calc_eigen_batch_equals_single(kpar_fast_pair):
    O, G, w = kpar_fast_pair
    oms = [0.0099881 - 2.3e-7j, 0.012 - 1e-6j, 0.02 + 0.001j]
    batch = G.calc_eigen(oms)
    # a batch of 9 evaluations and one of 3 sum the Bessel orders in chunks
    # of different length (the launch shape follows the batch size), so chi
    # agrees to rounding, about 1e-15; the heating rates difference chi over
    # 1e-6 Re(omega), which takes that to about 1e-9
    for om, eb in zip(oms, batch):
        es = G.calc_eigen([om])[0]
        a = np.array(sum(_abi.eigen_columns(eb, 2), []))
        b = np.array(sum(_abi.eigen_columns(es, 2), []))
        np.testing.assert_allclose(a, b, rtol=1e-8, atol=1e-300)


def test_calc_eigen_flags(kpar_fast_pair):
    O, G, w = kpar_fast_pair
    om = 0.0099881 - 2.3e-7j
    e_only = G.calc_eigen([om], eigen=True, heat=False)[0]
    h_only = G.calc_eigen([om], eigen=False, heat=True)[0]
    assert e_only.ewave == 0.0 and all(e_only.Ps[s] == 0.0 for s in range(2))
    assert h_only.ds[0].re == 0.0 and h_only.vmean[0][0].re == 0.0
    assert h_only.ewave != 0.0 and e_only.ds[0].re != 0.0


def test_scan_eigen_heat_match_golden(kpar_fast_pair, golden_dir):
    """Python om_scan driver with eigen + heating through the library,
    against the reference's .eigen and .heat files (the reference's own
    rtol 1e-2, and every printed digit for the eigenfunctions)."""
    O, G, w = kpar_fast_pair
    om, _, _ = G.secant([w["extra"]["guess"][0]])
    sc = w["extra"]["scan"]
    G.set_k(*w["k"])
    rows, _, eig = G.om_scan(sc["type_s"], sc["swi"], sc["swf"], sc["log_scan"], sc["n_out"], sc["n_res"], om,
                             eigen=True, heat=True)
    rows = rows[:, 0, :]
    nspec = w["system"].nspec
    for which, col in (("eigen", 0), ("heat", 1)):
        tab = np.array([list(r) + _abi.eigen_columns(e[0], nspec)[col] for r, e in zip(rows, eig)])
        gold = np.loadtxt(os.path.join(golden_dir, "ref", "test_kpar_fast.%s_kpara_1.root_1" % which))
        assert tab.shape == gold.shape
        np.testing.assert_allclose(tab, gold, rtol=1e-2)
        if which == "eigen":
            for a, b in zip(tab.ravel(), gold.ravel()):
                assert ("%.4E" % a) == ("%.4E" % b), (a, b)
