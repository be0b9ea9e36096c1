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
