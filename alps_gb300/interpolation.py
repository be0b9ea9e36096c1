"""The ALPS interpolation tool on the GPU (interpolation/interpolation.f90).

Fills a regular (p_perp, p_par) grid from scattered samples of f0: a
thin-plate spline of log f with smoothing (polyharmonic_spline), optionally
normalised to one over the grid (normalize).  The spline system is solved
and evaluated on the device.

    python -m alps_gb300.interpolation input.in [workdir]

reads the reference's &system namelist and writes <workdir>/<input>.array
(out_to_file) or prints the same lines.
"""
import ctypes as C
import os
import sys

import numpy as np

from . import _abi
from ._native import check, lib


def interpolate(pperp_c, ppar_c, f_c, nperp=50, npar=100, smoothing=1.0, pperp_range=None, ppar_range=None,
                normalize=False, mult_f=1.0):
    """Spline of log f through the samples (coordinates already scaled) on
    the fine grid; returns (pperp, ppar, f), each [nperp+1, npar+1].  The
    ranges default to the samples' extents, as in the reference."""
    pp = np.ascontiguousarray(pperp_c, dtype=np.float64)
    pl = np.ascontiguousarray(ppar_c, dtype=np.float64)
    ff = np.ascontiguousarray(f_c, dtype=np.float64)
    p = _abi.alps_interp_params()
    p.nperp, p.npar, p.smoothing = int(nperp), int(npar), float(smoothing)
    p.pperp_min, p.pperp_max = pperp_range if pperp_range is not None else (pp.min(), pp.max())
    p.ppar_min, p.ppar_max = ppar_range if ppar_range is not None else (pl.min(), pl.max())
    p.do_normalize, p.mult_f = int(bool(normalize)), float(mult_f)
    shape = (nperp + 1, npar + 1)
    op, ol, of = np.empty(shape), np.empty(shape), np.empty(shape)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    check(lib().alps_interpolate(dp(pp), dp(pl), dp(ff), len(ff), C.byref(p), dp(op), dp(ol), dp(of)),
          "alps_interpolate")
    return op, ol, of


def run(input_path, workdir="."):
    """The whole program on an input file (alps_run_interpolation)."""
    check(lib().alps_run_interpolation(os.fsencode(input_path), os.fsencode(workdir)), "alps_run_interpolation")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python -m alps_gb300.interpolation input.in [workdir]")
    run(sys.argv[1], sys.argv[2] if len(sys.argv) > 2 else ".")
