"""Every input the reference ships (tests/*.in, with its distribution
tables generated from distribution/*_dist.in) runs end to end on the GPU
through alps_run_input: maps, guesses, scans, double scans, eigenfunctions,
heating, bi-Maxwellian/cold, Chebyshev and relativistic species.  Only
test_kpar_fast has golden output upstream (checked in test_gpu_parity.py);
here every run must succeed and write finite numbers to the files the
reference writes."""
import glob
import os
import re
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "golden", "ref", "inputs")
INPUTS = sorted(os.path.basename(p)[:-3] for p in glob.glob(os.path.join(REF, "tests", "*.in")))


def _write_names():
    """writeName of every distribution input -> its path."""
    out = {}
    for p in glob.glob(os.path.join(REF, "distribution", "*_dist.in")):
        m = re.search(r"writeName\s*=\s*['\"]([^'\"]+)['\"]", open(p).read())
        if m:
            out[m.group(1)] = p
    return out


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    return A


@pytest.mark.parametrize("name", INPUTS)
def test_reference_input_runs(api, name, tmp_path):
    from alps_gb300._abi import AlpsError
    from alps_gb300.distribution import generate_distribution
    text = open(os.path.join(REF, "tests", name + ".in")).read()
    names = set(re.findall(r"arrayName\s*=\s*['\"]([^'\"]+)['\"]", text))
    wn = _write_names()
    for arr in names:
        if arr in wn:
            generate_distribution(wn[arr], str(tmp_path / "distribution"))
    shutil.copyfile(os.path.join(REF, "tests", name + ".in"), str(tmp_path / (name + ".in")))
    missing = sorted(arr for arr in names if arr not in wn)
    try:
        api.run_input(str(tmp_path / (name + ".in")), str(tmp_path))
    except AlpsError as e:
        if missing and e.status == 27:  # ALPS_E_IO: its f0 tables do not exist
            pytest.skip("the reference ships no distribution input for %s" % missing)
        raise
    written = [p for p in glob.glob(str(tmp_path / "solution" / "*")) if os.path.isfile(p)]
    assert written, "no output files"
    for p in written:
        rows = [ln.split() for ln in open(p) if ln.strip()]
        vals = np.array([float(v.replace("D", "E")) for r in rows for v in r])
        assert vals.size > 0 and np.all(np.isfinite(vals)), p
