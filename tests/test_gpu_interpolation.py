"""The interpolation tool on the GPU (alps_interpolate,
alps_run_interpolation) against the oracle's restatement of
interpolation/interpolation.f90, on the reference's own input.

Tolerance: the spline system (n + 3 = 703 unknowns, LU with the same
pivoting) and its evaluation run in FP64 on both sides; the device's log,
exp, pow and reduction order differ in the last bits.  f agrees to 1e-10."""
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REF = os.path.join(os.path.dirname(__file__), "golden", "ref", "inputs", "interpolation")
RTOL = 1e-10


@pytest.fixture(scope="module")
def interp():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import interpolation
    return interpolation


def _coarse():
    a = np.loadtxt(os.path.join(REF, "test_interp_coarse.array"))
    return a[:, 0], a[:, 1], a[:, 2]


@pytest.mark.parametrize("smoothing,normalize", [(0.1, True), (0.0, False), (1.0, True)])
def test_interpolate_matches_oracle(interp, smoothing, normalize):
    from oracle import pyoracle as po
    pp, pl, f = _coarse()
    rng = (0.0, pp.max()), (pl.min(), pl.max())
    gp, gl, gf = interp.interpolate(pp, pl, f, 50, 100, smoothing, rng[0], rng[1], normalize)
    of = po.interpolate(pp, pl, f, 50, 100, smoothing, rng[0], rng[1], normalize)
    np.testing.assert_allclose(gf, of, rtol=RTOL)
    assert np.array_equal(gp[:, 0], 0.0 + (pp.max() - 0.0) * np.arange(51) / 50.0)


def test_run_interpolation_on_reference_input(interp, tmp_path):
    """The whole program on test_interp.in (empty values in its namelist keep
    the defaults; pperp_min_set = 0): test_interp.array in the workdir."""
    from oracle import pyoracle as po
    for name in ("test_interp.in", "test_interp_coarse.array"):
        shutil.copyfile(os.path.join(REF, name), tmp_path / name)
    interp.run(str(tmp_path / "test_interp.in"), str(tmp_path))
    out = np.loadtxt(tmp_path / "test_interp.array")
    assert out.shape == (51 * 101, 3)
    pp, pl, f = _coarse()
    of = po.interpolate(pp, pl, f, 50, 100, 0.1, (0.0, pp.max()), (pl.min(), pl.max()), True)
    np.testing.assert_allclose(out[:, 2], of.ravel(), rtol=RTOL)
    np.testing.assert_allclose(out[:, 0].reshape(51, 101)[:, 0], np.linspace(0.0, pp.max(), 51), rtol=1e-14)


def test_interpolate_rejects_bad_input(interp):
    from alps_gb300._abi import AlpsError
    with pytest.raises(AlpsError):
        interp.interpolate([0.1, 0.2], [0.0, 0.1], [1.0, 0.0], 10, 10)  # f <= 0
    with pytest.raises(AlpsError):
        interp.interpolate([0.1], [0.0], [1.0], 1, 10)                   # nperp < 2
