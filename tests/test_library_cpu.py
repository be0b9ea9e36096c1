"""CPU-side checks of the native library: it builds, loads, exports every
symbol of include/alps_gb300.h, and its host-only entry points agree with the
oracle.  No det D is evaluated here (that needs a GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from alps_gb300 import _abi, _native, api, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from alps_gb300 import build
    build.build()
    return _native.lib()


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "alps_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(alps_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    declared = _header_functions()
    assert declared == sorted(_native.exported_symbols())
    for name in declared:
        assert hasattr(lib, name), name


def test_error_strings(lib):
    assert lib.alps_error_string(0) == b"ok"
    assert b"roots diverged" in lib.alps_error_string(9)


def test_create_without_device_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = _abi.system_defaults(nspec=1, nperp=16, npar=32)
    h = C.c_void_p()
    assert lib.alps_create(C.byref(s), C.byref(h)) == 28  # ALPS_E_NO_DEVICE


@pytest.mark.parametrize("kind", [1, 2, 4])
def test_generator_matches_oracle_bitwise(lib, kind):
    from oracle import pyoracle as po
    d = workloads._dist(kind=kind, ms=0.3, tau=1.7, alph=0.6, p_drift=0.4, kappa=5.0)
    a = api.generate_f0(d, 20, 40)
    b = po.generate_f0(d, 20, 40)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_find_minima_matches_oracle(lib):
    from oracle import pyoracle as po
    rng = np.random.default_rng(1)
    for nr, ni in [(9, 7), (16, 16), (2, 2)]:
        val = rng.normal(size=nr * ni)
        assert api.find_minima(val, nr, ni) == po.find_minima(val, nr, ni)


def _ref_input(golden_dir, name):
    return os.path.join(golden_dir, "ref", "inputs", "tests", name)


def test_read_all_reference_inputs(lib, golden_dir):
    d = os.path.join(golden_dir, "ref", "inputs", "tests")
    names = sorted(f for f in os.listdir(d) if f.endswith(".in"))
    assert len(names) == 12
    for name in names:
        inp = api.read_input(os.path.join(d, name))
        assert inp.sys.nspec >= 1 and inp.sys.nperp > 0 and inp.sys.npar > 0, name
        assert inp.runname.decode() == name[:-3]


def test_read_input_kpar_fast_values(lib, golden_dir):
    inp = api.read_input(_ref_input(golden_dir, "test_kpar_fast.in"))
    s = inp.sys
    assert (s.nspec, s.nperp, s.npar) == (2, 120, 240)
    assert (s.kperp, s.kpar, s.vA, s.Bessel_zero) == (1e-2, 1e-2, 1e-4, 1e-50)
    assert (s.secant_method, s.numiter, s.positions_principal, s.n_resonance_interval) == (2, 50, 3, 100)
    assert (s.D_threshold, s.D_prec, s.D_gap, s.D_tol, s.Tlim) == (1e-15, 1e-5, 1e-5, 1e-7, 0.01)
    assert inp.arrayName.decode() == "test_kpar_fast" and inp.nroots == 1 and not inp.use_map
    assert (inp.guess[0].re, inp.guess[0].im) == (9.9e-3, -5.5e-6)
    sp2 = inp.species[1]
    assert (sp2.ns, sp2.qs, sp2.ms, sp2.ac_method, sp2.n_fits, sp2.log_fit) == (1.0, -1.0, 5.44662e-4, 1, 1, 1)
    assert sp2.fit_type[0] == 1 and list(sp2.fit_init[0])[:3] == [1.4128e4, 1.836e3, 0.0]
    assert sp2.perp_correction[0] == 1.836e3
    sc = inp.scan[0]
    assert (inp.n_scan, sc.type_s, sc.n_out, sc.n_res, sc.log_scan, sc.heating, sc.eigen) == (1, 4, 32, 1, 1, 1, 1)
    import math
    assert sc.diff == (math.log10(1e-1) - math.log10(1e-2)) / 32.0


def test_read_input_map_values(lib, golden_dir):
    inp = api.read_input(_ref_input(golden_dir, "test_map.in"))
    assert inp.use_map == 1
    m = inp.map
    assert (m.omi, m.omf, m.gami, m.gamf, m.nr, m.ni) == (-3e-2, 3e-2, -1e-3, 3e-4, 50, 50)


def test_f0_file_round_trip(lib, tmp_path):
    d = workloads._dist(kind=1, ms=1.0)
    a = api.generate_f0(d, 12, 24)
    p = str(tmp_path / "x.1.array")
    api.write_f0(p, *a[:3])
    b = api.read_f0(p, 12, 24)
    for x, y in zip(a[:3], b):
        assert np.array_equal(x, y)
