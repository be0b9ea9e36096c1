"""scan_option 2 (om_double_scan, src/ALPS_fns.f90:2904-3591) through
alps_run_input, against the same double scan driven over the oracle
(tests/scan_drivers.py) on the reference's kpar_fast plasma at a coarser
grid: scan 1 in k_par, scan 2 in k_perp from every output point of scan 1,
one block of rows per inner scan, blank lines between blocks.
"""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    return A


def _write_inputs(golden_dir, tmp_path, N=32, M=64):
    from alps_gb300.distribution import read_distribution_input
    from alps_gb300 import api as A
    ref = os.path.join(golden_dir, "ref", "inputs")
    txt = open(os.path.join(ref, "tests", "test_kpar_fast.in")).read()
    txt = re.sub(r"(?m)^nperp=\d+", "nperp=%d" % N, txt)
    txt = re.sub(r"(?m)^npar=\d+", "npar=%d" % M, txt)
    txt = re.sub(r"(?m)^scan_option=\d+", "scan_option=2", txt)
    txt = re.sub(r"(?m)^n_scan=\d+", "n_scan=2", txt)
    txt = re.sub(r"(?m)^ns=\d+", "ns=2", txt)
    txt = re.sub(r"(?m)^swf=1.0d-1", "swf=2.0d-2", txt)
    txt = re.sub(r"(?m)^heating=\.true\.", "heating=.false.", txt)
    txt = re.sub(r"(?m)^eigen=\.true\.", "eigen=.false.", txt)
    txt += "\n&scan_input_2\nscan_type=3\nswi=1.0d-2\nswf=2.0d-2\nswlog=.true.\nns=2\nnres=1\n" \
           "heating=.false.\neigen=.false.\n/\n"
    path = tmp_path / "dscan.in"
    path.write_text(txt)
    dist = read_distribution_input(os.path.join(ref, "distribution", "test_kpar_fast_dist.in"))
    os.makedirs(str(tmp_path / "distribution"), exist_ok=True)
    species = []
    inp = A.read_input(str(path))
    for i, d in enumerate(dist["species"], start=1):
        pp, pl, f0, _ = A.generate_f0(d, N, M)
        A.write_f0(str(tmp_path / "distribution" / ("test_kpar_fast.%d.array" % i)), pp, pl, f0)
        species.append((inp.species[i - 1], pp, pl, f0))
    return str(path), inp, species


def _blocks(path):
    blocks, cur = [], []
    for line in open(path).read().split("\n")[:-1]:
        if line.strip():
            cur.append([float(x) for x in line.split()])
        else:
            blocks.append(np.array(cur))
            cur = []
    assert not cur
    return blocks


def test_double_scan_matches_oracle_driver(api, golden_dir, tmp_path):
    from oracle import pyoracle as po
    from scan_drivers import double_scan
    po.set_threads(os.cpu_count() or 1)
    path, inp, species = _write_inputs(golden_dir, tmp_path)
    api.run_input(path, str(tmp_path))
    got = _blocks(str(tmp_path / "solution" / "dscan.scan_kpara_kperp.root_1"))
    s = inp.sys
    O = po.OraclePlasma(s, species)
    O.set_k(s.kperp, s.kpar)
    guess = complex(inp.guess[0].re, inp.guess[0].im)
    w0 = O.secant(guess, s.secant_method)[0]
    sc = [dict(type_s=inp.scan[k].type_s, log_scan=inp.scan[k].log_scan, n_out=inp.scan[k].n_out,
               n_res=inp.scan[k].n_res, diff=inp.scan[k].diff, diff2=inp.scan[k].diff2) for k in range(2)]
    want = double_scan(O, sc[0], sc[1], [w0], s.kperp, s.kpar, s.D_gap, s.secant_method)[0]
    assert len(got) == len(want) == 3
    for g, w in zip(got, want):
        assert g.shape == w.shape == (3, 4)
        np.testing.assert_allclose(g, w, rtol=2e-4)
