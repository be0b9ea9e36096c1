"""alps_autotune: the launch-shape autotuner of the batch kernels.

A tuned shape changes only the pole sums' summation order (j slices, order
chunks) and how resonant items spread over warps, so det D after tuning
stays within rounding of the default shapes' (1e-12 relative here, far below
the parity gates).  Lone and fused batches of a bucket take the same shape,
so a root solved alone and in a batch stays bit for bit the same after
tuning, and alps_tune_clear returns every bucket to the default rule (det D
bit for bit as before tuning).
"""
import numpy as np
import pytest

from alps_gb300 import workloads

pytestmark = pytest.mark.gpu

OMS = np.array([0.45 - 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 0.7 + 0.0j, 2.2 - 0.35j] * 13)[:64]


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    A.tune_clear()
    yield A
    A.tune_clear()


def _plasma(api, precision):
    w = workloads.proton_electron(24, 48, 1.0, 0.3, 1e-14)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species, precision=precision)
    G.set_k(1.0, 0.3)
    return G


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tuned_shape_keeps_det(api, precision):
    G = _plasma(api, precision)
    D0 = G.disp_batch(OMS)
    r = api_tune(G, len(OMS))
    assert r["candidates"] == 54
    assert r["js"] in (1, 2, 4, 8, 16, 32) and r["blocks_per_sm"] in (2, 4, 8) and r["warps_per_sm"] in (6, 12, 24)
    assert 0 < r["ms_best"] <= r["ms_default"]
    D1 = G.disp_batch(OMS)
    assert np.all(np.abs(D1 - D0) <= 1e-12 * np.abs(D0)), np.max(np.abs(D1 - D0) / np.abs(D0))
    api.tune_clear()
    assert np.array_equal(G.disp_batch(OMS), D0)


def api_tune(G, n):
    return G.autotune(n)


def test_alone_equals_fused_after_tuning(api):
    rng = np.random.default_rng(21)
    P = []
    for i in range(4):
        w = workloads.uneven_plasma(rng, grid=(32, 64))
        s, sp = workloads.build_uneven(w, api.generate_f0)
        G = api.Plasma(s, sp, precision="mixed")
        G.set_k(*w["k"])
        P.append(G)
    for G in P:  # the batches of a root solve: two frequencies per root
        G.autotune(2)
    g = rng.uniform(0.2, 1.5, 4) - 1j * rng.uniform(0.0, 0.1, 4)
    roots, iters, _, _ = api.solve_many(P, g)
    for k in (0, 3):
        ra, ia, _, _ = api.solve_many([P[k]], [g[k]])
        assert ra[0] == roots[k] and ia[0] == iters[k]
