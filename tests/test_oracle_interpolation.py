"""The oracle's restatement of the interpolation tool
(interpolation/interpolation.f90).  The reference ships its input
(test_interp.in, test_interp_coarse.array) but no output, so the
restatement is held to properties of the spline instead: the
normalisation, exact interpolation without smoothing, and the recovery of a
smooth distribution."""
import os

import numpy as np
import pytest

REF = os.path.join(os.path.dirname(__file__), "golden", "ref", "inputs", "interpolation")


def _po():
    from oracle import pyoracle as po
    return po


def _coarse():
    a = np.loadtxt(os.path.join(REF, "test_interp_coarse.array"))
    return a[:, 0], a[:, 1], a[:, 2]


def test_reference_input_is_normalised():
    """test_interp.in: smoothing 0.1, 50 x 100, pperp_min 0, normalised."""
    po = _po()
    pp, pl, f = _coarse()
    out = po.interpolate(pp, pl, f, 50, 100, 0.1, (0.0, pp.max()), (pl.min(), pl.max()), True)
    assert np.all(np.isfinite(out)) and np.all(out > 0)
    gp = np.linspace(0.0, pp.max(), 51)
    gl = np.linspace(pl.min(), pl.max(), 101)
    total = 2 * np.pi * (out * gp[:, None]).sum() * (gp[2] - gp[1]) * (gl[2] - gl[1])
    assert abs(total - 1.0) < 1e-12


def test_exact_at_samples_without_smoothing():
    """With zero smoothing the spline passes through every sample: samples
    placed on fine-grid nodes come back unchanged."""
    po = _po()
    rng = np.random.default_rng(4)
    nperp, npar = 20, 30
    gp, gl = np.linspace(0.0, 4.0, nperp + 1), np.linspace(-3.0, 3.0, npar + 1)
    ii, jj = rng.integers(0, nperp + 1, 60), rng.integers(0, npar + 1, 60)
    keep = np.unique(ii * 1000 + jj, return_index=True)[1]
    ii, jj = ii[keep], jj[keep]
    f = np.exp(-(gp[ii] ** 2 + gl[jj] ** 2) / 2) * (1 + 0.1 * rng.random(len(ii)))
    out = po.interpolate(gp[ii], gl[jj], f, nperp, npar, 0.0, (0.0, 4.0), (-3.0, 3.0), False)
    np.testing.assert_allclose(out[ii, jj], f, rtol=1e-9)


def test_recovers_a_maxwellian():
    """log f of a Maxwellian is a quadratic; sampled on a scattered set it is
    recovered on the interior of the fine grid."""
    po = _po()
    rng = np.random.default_rng(7)
    pp = rng.uniform(0.0, 3.0, 300)
    pl = rng.uniform(-3.0, 3.0, 300)
    f = np.exp(-(pp ** 2 + pl ** 2))
    out = po.interpolate(pp, pl, f, 30, 60, 0.0, (0.0, 3.0), (-3.0, 3.0), False)
    gp, gl = np.linspace(0.0, 3.0, 31), np.linspace(-3.0, 3.0, 61)
    exact = np.exp(-(gp[:, None] ** 2 + gl[None, :] ** 2))
    inner = (slice(5, 26), slice(10, 51))
    rel = np.abs(np.log(out[inner]) - np.log(exact[inner]))
    assert rel.max() < 2e-2, rel.max()
