"""alps_solve_many: root solves of uneven plasmas advanced together on the
device inside one graph launch (the C3 uneven-batch entry point).

Each root's determinants come from a job with the launch shape of a lone
batch of two frequencies on its own context, and the root machines are the
same code on host and device, so:
  * a root's result alone and in any batch is bit for bit the same;
  * against the host-driven secant (alps_secant_ex, whose batches take other
    launch shapes) converged roots agree to rounding (1e-9, the roots' gate),
    and each is a root of the oracle's det D to the same gate.
"""
import os

import numpy as np
import pytest

from alps_gb300 import workloads

pytestmark = pytest.mark.gpu

ROOT_RTOL = 1e-9


@pytest.fixture(scope="module")
def plasmas():
    import torch
    assert torch.cuda.is_available()
    from alps_gb300 import api
    rng = np.random.default_rng(21)
    out = []
    for i in range(16):
        N = (32, 40, 48)[i % 3]
        w = workloads.uneven_plasma(rng, grid=(N, 2 * N))
        s, sp = workloads.build_uneven(w, api.generate_f0)
        G = api.Plasma(s, sp, precision="mixed" if i % 2 else "fp64")
        G.set_k(*w["k"])
        out.append((w, s, sp, G))
    return out


def _guesses(n):
    rng = np.random.default_rng(4)
    return rng.uniform(0.2, 1.5, n) - 1j * rng.uniform(0.0, 0.1, n)


def test_alone_equals_in_batch(plasmas):
    from alps_gb300 import api
    G = [p[3] for p in plasmas]
    g = _guesses(len(G))
    roots, iters, Df, conv = api.solve_many(G, g)
    for r in (0, 5, 11):
        ra, ia, Da, ca = api.solve_many([G[r]], [g[r]])
        assert ra[0] == roots[r] and ia[0] == iters[r] and Da[0] == Df[r] and ca[0] == conv[r]
    # a batch with a context repeated and in another order
    idx = [3, 3, 7, 1]
    rb, ib, _, _ = api.solve_many([G[k] for k in idx], [g[k] for k in idx])
    assert np.array_equal(rb, roots[idx]) and np.array_equal(ib, iters[idx])


def test_matches_host_secant_and_the_oracle(plasmas):
    from alps_gb300 import api
    from oracle import pyoracle as po
    po.set_threads(os.cpu_count() or 1)
    G = [p[3] for p in plasmas]
    g = _guesses(len(G))
    roots, iters, _, conv = api.solve_many(G, g)
    # random guesses on random plasmas: not every root converges within
    # numiter, and those that do are checked
    assert conv.sum() >= 4
    for r in range(len(G)):
        hr, hi, _, hc = G[r].polish([g[r]], om_rtol=1e-12)
        if not (conv[r] and hc[0]):
            continue
        assert abs(hr[0] - roots[r]) <= ROOT_RTOL * abs(roots[r]), r
    # converged roots are roots of the oracle's det D (shared fits)
    for r in [k for k in range(len(G)) if conv[k]][:4]:
        w, s, sp, Gr = plasmas[r]
        O = po.OraclePlasma(s, sp)
        Gc = api.Plasma(s, sp)
        for i in range(s.nspec):
            Gc.set_fit(i, O.get_fit(i))
        Gc.set_k(*w["k"])
        O.set_k(*w["k"])
        rc, _, _, cc = api.solve_many([Gc], [g[r]])
        if not cc[0]:
            continue
        h = 1e-7 * abs(rc[0])
        D = O.disp_batch(np.array([rc[0], rc[0] + h, rc[0] - h]), nthreads=os.cpu_count() or 1)
        step = abs(D[0] / ((D[1] - D[2]) / (2 * h))) / abs(rc[0])
        assert step <= ROOT_RTOL, (r, step)


def test_map_minima_on_one_context():
    """The same context repeated: the map plasma's polish through the
    device loop agrees with the host-driven secant."""
    from alps_gb300 import api
    w = workloads.config_map(16, 16)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species, precision="mixed")
    G.set_k(system.kperp, system.kpar)
    g = np.array([0.43 - 0.027j, 1.41 - 0.07j, 0.33 - 0.32j])
    rd, _, _, cd = api.solve_many([G] * len(g), g)
    rh, _, _, ch = G.polish(g, om_rtol=1e-12)
    for k in range(len(g)):
        if cd[k] and ch[k]:
            assert abs(rd[k] - rh[k]) <= ROOT_RTOL * abs(rh[k])


def test_batched_setup_equals_one_by_one():
    """alps_prepare_many + alps_set_k_many give the contexts alps_prepare +
    alps_set_k give: the same fits and nmax, and det D bit for bit."""
    import torch
    from alps_gb300 import api
    rng = np.random.default_rng(33)
    draws = [workloads.uneven_plasma(rng, grid=(N, 2 * N)) for N in (32, 48, 40, 64, 32, 48)]
    built = [workloads.build_uneven(w, api.generate_f0) for w in draws]
    for precision in ("fp64", "mixed"):
        many = api.make_many(built, precision=precision, ks=[w["k"] for w in draws])
        oms = np.array([0.5 - 0.05j, 1.2 + 0.01j, 0.8 + 0.0j])
        for (s, sp), w, Gm in zip(built, draws, many):
            G1 = api.Plasma(s, sp, precision=precision)
            G1.set_k(*w["k"])
            assert Gm.nmax() == G1.nmax()
            for i in range(s.nspec):
                assert np.array_equal(Gm.get_fit(i), G1.get_fit(i))
            assert np.array_equal(Gm.disp_batch(oms), G1.disp_batch(oms))
