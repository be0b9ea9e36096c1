"""A k step that keeps k_perp keeps the k tables.

nmax, the Bessel tables and the p_perp contractions depend on k_perp alone;
k_par enters per frequency.  alps_set_k and alps_set_k_many therefore keep
the tables when k_perp stays bit for bit, as om_scan skips determine_nmax
and determine_bessel_array for a k_par scan (src/ALPS_fns.f90:2465-2471).
det D after such a step must equal, bit for bit, det D of a context built
at that k from scratch, on both precision paths and for grid, closed-form
and relativistic species.
"""
import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

OMS = np.array([0.45 - 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 0.7 + 0.0j, 2.2 - 0.35j])


def _bimax(api):
    w = workloads.proton_electron(24, 48, 1.0, 0.3, 1e-14)
    return workloads.build(w, api.generate_f0)


def _closed_form(api):
    me = 1.0 / 1836.0
    de = workloads._dist(kind=1, ms=me, vA=1e-4, maxP=6.0)
    pe, qe, fe, ie = api.generate_f0(de, 24, 48)
    sysd = _abi.system_defaults(nspec=2, nperp=24, npar=48, kperp=0.3, kpar=0.2, vA=1e-4, Bessel_zero=1e-20)
    spB = _abi.species_defaults(ns=1, qs=1, ms=1, use_bM=1, bM_nmaxs=500, bM_Bessel_zeros=1e-50, bM_betas=1.0,
                                bM_alphas=1.0, bM_pdrifts=0.1)
    spE = _abi.species_defaults(ns=1, qs=-1, ms=me, fits=[(1, list(ie[:3]) + [0, 0], ie[5])])
    return sysd, [(spB, None, None, None), (spE, pe, qe, fe)]


def _relativistic(api):
    vA = 0.1
    d = workloads._dist(kind=1, ms=1.0, vA=vA, maxP=5.0)
    pp, pl, f0, ideal = api.generate_f0(d, 30, 80)
    sysd = _abi.system_defaults(nspec=1, nperp=30, npar=80, kperp=0.3, kpar=0.2, vA=vA, Bessel_zero=1e-20,
                                positions_principal=3, ngamma=40, npparbar=40)
    pc = 2.0 / (vA * vA)
    sp = _abi.species_defaults(ns=1, qs=1, ms=1, relat=1, fits=[(5, [ideal[0] * np.exp(pc), 1e-12, 0, 0, 0], pc)])
    return sysd, [(sp, pp, pl, f0)]


CASES = {"bimaxwellian": _bimax, "closed_form": _closed_form, "relativistic": _relativistic}


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    return A


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", list(CASES))
def test_kpar_step_equals_fresh_tables(api, name, precision):
    system, species = CASES[name](api)
    kperp = 0.3
    G = api.Plasma(system, species, precision=precision)
    G.set_k(kperp, 0.2)
    G.disp_batch(OMS)
    before = G.stats().k_reused
    G.set_k(kperp, 0.35)  # a k_par step
    assert G.stats().k_reused == before + 1
    H = api.Plasma(system, species, precision=precision)
    H.set_k(kperp, 0.35)
    assert G.nmax() == H.nmax()
    assert np.array_equal(G.disp_batch(OMS), H.disp_batch(OMS))
    # a k_perp step rebuilds
    G.set_k(kperp * 1.5, 0.35)
    assert G.stats().k_reused == before + 1
    H.set_k(kperp * 1.5, 0.35)
    assert np.array_equal(G.disp_batch(OMS), H.disp_batch(OMS))


def test_set_k_many_mixes_kept_and_rebuilt_tables(api):
    system, species = _bimax(api)
    P = [api.Plasma(system, species, precision=("fp64", "mixed")[i % 2]) for i in range(4)]
    for G in P:
        G.set_k(1.0, 0.3)
    ks = [(1.0, 0.4), (1.7, 0.4), (1.0, 0.25), (0.6, 0.3)]
    api.set_k_many(P, ks)
    assert [G.stats().k_reused for G in P] == [1, 0, 1, 0]
    for G, k in zip(P, ks):
        H = api.Plasma(system, species, precision=G.precision)
        H.set_k(*k)
        assert G.nmax() == H.nmax()
        assert np.array_equal(G.disp_batch(OMS), H.disp_batch(OMS))
