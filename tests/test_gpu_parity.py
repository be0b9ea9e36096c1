"""Parity of the CUDA path with the CPU oracle (FP64 plain path).

Tolerances (FP64 path):
  chi entries: |chi_gpu - chi_oracle| <= 1e-10 * max(|chi_ij|, 1e-3 * mag_ij)
    where mag_ij = sum over Bessel orders of |contribution to chi_ij| (the
    oracle reports it).  Entries that are small differences of large order
    terms (e.g. electron chi_xx at omega << Omega_e, where the n = +-1 terms
    cancel to 1 part in 1e5) carry rounding of order eps * mag_ij in ANY FP64
    summation order, the reference's included; the floor keeps the 1e-10
    relative gate meaningful for them.
  det D: first-order propagation of the chi bound through the cofactors of
    the wave tensor, |dD| <= 1e-10 * sum_ij |cof_ij| * max(|w_ij|, 1e-3 mag_ij).
  roots: relative 1e-9 in complex omega.
The summation order differs from the reference (the p_perp sum runs first),
so results agree to rounding, not bitwise; index decisions (nmax, resonance
windows) are bitwise identical.
"""
import os

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

CHI_RTOL = 1e-10
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


PRECISIONS = ["fp64", "mixed"]


def _pair(api, w, share_fit=True, precision="fp64"):
    po = _oracle()
    system, species = workloads.build(w, po.generate_f0)
    O = po.OraclePlasma(system, species)
    G = api.Plasma(system, species, precision=precision)
    if share_fit:
        for i in range(system.nspec):
            G.set_fit(i, O.get_fit(i))
    return O, G


def _small(kperp=1.0, kpar=0.3, nperp=24, npar=48, bz=1e-14, me=1.0 / 1836.0):
    return workloads.proton_electron(nperp, npar, kperp, kpar, bz, me=me)


def _chi_close(a, b, mag, what):
    """a, b: [S, 9] chi values (GPU, oracle); mag: [S, 9] order-sum scales
    (in the same units as a and b)."""
    a, b, mag = (np.asarray(x).reshape(len(x), -1) for x in (a, b, mag))
    scale = np.maximum(np.abs(b), 1e-3 * mag)
    err = np.abs(a - b)
    ok = err <= CHI_RTOL * scale + 1e-300
    assert np.all(ok), (what, (err / np.maximum(scale, 1e-300)).max())


def _disp_close(O, G, om, what):
    Do, co, clo, wo = O.disp(om)
    Dg, cg, clg, wg = G.disp(om)
    mag = O.disp_mag(om)                       # units of chi (before / om^2 vA^2)
    denom = abs(om * om) * O.sys.vA ** 2 if O.sys.kperp_norm else abs(om * om) * O.sys.vA ** 2 * O.sys.kperp ** 2
    mag0 = mag / denom                        # units of chi0
    _chi_close(cg, co, mag0, "chi0 " + what)
    _chi_close(clg.reshape(len(clg), 3, 9), clo.reshape(len(clo), 3, 9),
               np.repeat(mag0.reshape(len(mag0), 1, 9), 3, axis=1), "chi0_low " + what)
    # det D: cofactor propagation of the chi bound
    cof = np.array([[np.linalg.det(np.delete(np.delete(wo, i, 0), j, 1)) for j in range(3)] for i in range(3)])
    magw = mag.sum(axis=0)
    bound = CHI_RTOL * np.sum(np.abs(cof) * np.maximum(np.abs(wo), 1e-3 * magw))
    assert abs(Dg - Do) <= max(bound, 1e-12 * abs(Do)), (what, Dg, Do, bound)


OMEGAS = [0.45 - 0.2j, 0.45 + 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 0.7 + 0.0j, 2.2 - 0.35j, 0.05 - 0.01j,
          1.0 + 0.05j]


def test_nmax_and_bessel_table_match(api):
    O, G = _pair(api, _small())
    for k in [(1.0, 0.3), (2.0, 0.3), (0.3, 1.0)]:
        O.set_k(*k)
        G.set_k(*k)
        assert O.nmax() == G.nmax()


def test_fit_matches_oracle(api):
    po = _oracle()
    w = _small()
    system, species = workloads.build(w, po.generate_f0)
    O = po.OraclePlasma(system, species)
    G = api.Plasma(system, species)
    for i in range(system.nspec):
        a, b = G.get_fit(i), O.get_fit(i)
        scale = np.abs(b).max()
        assert np.abs(a - b).max() <= 1e-10 * scale


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", [(1.0, 0.3), (2.0, 0.15), (0.5, 0.05)])
def test_disp_chi_parity_small(api, k, precision):
    O, G = _pair(api, _small(), precision=precision)
    O.set_k(*k)
    G.set_k(*k)
    for om in OMEGAS:
        _disp_close(O, G, om, "%s k=%s" % (om, k))


@pytest.mark.parametrize("precision", PRECISIONS)
def test_principal_value_point_on_piece_boundary(api, precision):
    """At omega = 1 + 0.05i, k = (1, 0.3) the proton order n = 2 resonates at
    p_res = -10/3 and the symmetric sum's point k = 50 lands exactly on
    p_par = -2.875 = pp(12) + dppar/2, the boundary between two pieces of
    funct_g.  Rounding that point through a fused multiply-add moves it to
    the other piece (chi off by ~1e-6); the reference's rounding keeps it."""
    O, G = _pair(api, _small(), precision=precision)
    O.set_k(1.0, 0.3)
    G.set_k(1.0, 0.3)
    for om in (1.0 + 0.05j, 2.0 - 0.1j, 1.0 - 0.05j):
        _disp_close(O, G, om, "%s boundary point" % om)


def test_disp_batch_matches_single(api):
    # the split of the p_par sums over threads depends on the batch size, so a
    # value alone and in a batch agree to rounding; the same batch twice is
    # bitwise identical (fixed summation order, no atomics)
    O, G = _pair(api, _small())
    G.set_k(1.0, 0.3)
    oms = np.array(OMEGAS)
    Db = G.disp_batch(oms)
    assert np.array_equal(Db, G.disp_batch(oms))
    for om, d in zip(oms, Db):
        s = G.disp(om)[0]
        assert abs(s - d) <= 1e-13 * abs(d)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_disp_parity_kpar_fast(api, precision):
    w = workloads.kpar_fast(nproc=4)
    O, G = _pair(api, w, precision=precision)
    O.set_k(*w["k"])
    G.set_k(*w["k"])
    assert G.nmax() == [21, 13]
    for om in [9.9e-3 - 5.5e-6j, 1.2e-2 - 1e-6j, 9.9e-3 + 2e-4j]:
        _disp_close(O, G, om, "kpar_fast %s" % om)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_secant_parity(api, precision):
    O, G = _pair(api, _small(), precision=precision)
    O.set_k(1.0, 0.3)
    G.set_k(1.0, 0.3)
    for method in (2, 0, 1):
        guess = 0.3 - 0.05j
        ro, ito, _ = O.secant(guess, method)
        rg, itg, _ = G.secant([guess], method)
        assert abs(rg[0] - ro) <= ROOT_RTOL * abs(ro), (method, rg[0], ro)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_map_and_minima_parity(api, precision):
    po = _oracle()
    O, G = _pair(api, _small(nperp=16, npar=32, bz=1e-10), precision=precision)
    O.set_k(1.0, 0.3)
    G.set_k(1.0, 0.3)
    mp = _abi.alps_map_params()
    mp.omi, mp.omf, mp.gami, mp.gamf, mp.nr, mp.ni = 0.05, 1.5, -0.3, 0.05, 12, 8
    mp.loggridw = mp.loggridg = 0
    omo, calo, valo = O.map(mp, nthreads=os.cpu_count() or 1)
    omg, calg, valg = G.map_search(mp)
    assert np.array_equal(omo, omg)
    rel = np.abs(calg - calo) / np.maximum(np.abs(calo), 1e-300)
    assert rel.max() < 1e-9
    assert po.find_minima(valo, 12, 8) == api.find_minima(valg, 12, 8)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_disp_parity_map_config_samples(api, precision):
    """The benchmark plasma (128x256 grid, nmax 30/7) at a few lattice
    points covering Im omega < 0, = 0 (none on the lattice) and > 0."""
    w = workloads.config_map(8, 8)
    O, G = _pair(api, w, precision=precision)
    s = w["system"]
    O.set_k(s.kperp, s.kpar)
    G.set_k(s.kperp, s.kpar)
    assert O.nmax() == G.nmax() == [30, 7]
    for om in [1.5 - 0.3j, 0.2 - 0.01j, 2.9 + 0.05j, 0.75 - 0.004j]:
        _disp_close(O, G, om, "map config %s" % om)


@pytest.mark.slow
def test_kpar_fast_scan_on_gpu_matches_golden(api, golden_dir):
    w = workloads.kpar_fast(nproc=4)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species)
    G.set_k(*w["k"])
    om, _, _ = G.secant([w["extra"]["guess"][0]])
    sc = w["extra"]["scan"]
    rows, _ = G.om_scan(sc["type_s"], sc["swi"], sc["swf"], sc["log_scan"], sc["n_out"], sc["n_res"], om)
    gold = np.loadtxt(os.path.join(golden_dir, "ref", "test_kpar_fast.scan_kpara_1.root_1"))
    rows = rows[:, 0, :]
    np.testing.assert_allclose(rows, gold, rtol=1e-2)
    for a, b in zip(rows.ravel(), gold.ravel()):
        assert ("%.4E" % a) == ("%.4E" % b), (a, b)


def test_run_input_kpar_fast_reproduces_golden_files(api, golden_dir, tmp_path):
    """alps_run_input on the reference's CI input writes the .scan and
    .eigen files the reference's CI asserts on byte for byte, and the .heat
    file to its last printed digit."""
    import shutil
    from alps_gb300.distribution import generate_distribution
    ref = os.path.join(golden_dir, "ref")
    generate_distribution(os.path.join(ref, "inputs", "distribution", "test_kpar_fast_dist.in"),
                          str(tmp_path / "distribution"))
    shutil.copyfile(os.path.join(ref, "inputs", "tests", "test_kpar_fast.in"), str(tmp_path / "test_kpar_fast.in"))
    api.run_input(str(tmp_path / "test_kpar_fast.in"), str(tmp_path))
    sol = tmp_path / "solution"
    for name in ("scan", "eigen"):
        got = open(str(sol / ("test_kpar_fast.%s_kpara_1.root_1" % name))).read()
        want = open(os.path.join(ref, "test_kpar_fast.%s_kpara_1.root_1" % name)).read()
        assert got == want, name
    # heating rates: a forward difference over 1e-6 Re(omega) amplifies the
    # chi rounding, so the last printed digit may differ by one
    got = np.loadtxt(str(sol / "test_kpar_fast.heat_kpara_1.root_1"))
    want = np.loadtxt(os.path.join(ref, "test_kpar_fast.heat_kpara_1.root_1"))
    np.testing.assert_allclose(got, want, rtol=1e-2)
    np.testing.assert_allclose(got, want, rtol=2e-4)
    got = np.loadtxt(str(sol / "test_kpar_fast.heat_mech_kpara_1.root_1"))
    want = np.loadtxt(os.path.join(ref, "test_kpar_fast.heat_mech_kpara_1.root_1"))
    np.testing.assert_allclose(got, want, rtol=1e-2)
    assert np.array_equal(got == 0.0, want == 0.0)
    roots = open(str(sol / "test_kpar_fast.roots")).read().split()
    assert roots[0] == "1" and len(roots) == 6
