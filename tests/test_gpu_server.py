"""The request server (alps_server_*): continuous batching of root
polishes, k scans and maps over several plasmas.  Every result must equal
the same request run alone through the single-plasma entry points, bit for
bit, whatever else is in flight; admission by device footprint only delays
requests."""
import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from alps_gb300 import api as A
    return A


def _plasmas(api, n=6, seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        w = workloads.uneven_plasma(rng, grid=(32, 64) if i % 2 else (48, 96))
        s, sp = workloads.build_uneven(w, api.generate_f0)
        G = api.Plasma(s, sp, precision="mixed" if i % 3 == 0 else "fp64")
        G.set_k(*w["k"])
        out.append(G)
    return out


def _map(nr=24, ni=16):
    mp = _abi.alps_map_params()
    mp.omi, mp.omf, mp.gami, mp.gamf = 0.05, 2.0, -0.3, 0.05
    mp.nr, mp.ni = nr, ni
    return mp


GUESSES = [0.3 - 0.02j, 1.1 - 0.05j]


def test_mixed_stream_equals_alone(api):
    P = _plasmas(api)
    # alone
    alone_roots = [P[i].secant(GUESSES)[0] for i in range(4)]
    alone_map = P[4].map_search(_map())
    r0 = P[5].secant([0.5 - 0.01j])[0]
    sc = api.scan_def(4, 0.0, P[5].kpar * 1.5, True, 4, 1, P[5].kperp, P[5].kpar)
    alone_scan = P[5].om_scan(4, 0.0, P[5].kpar * 1.5, True, 4, 1, r0)
    P[5].set_k(P[5].kperp, alone_scan[0][0, 0, 1])  # back to the scan's start
    # in the mix
    srv = api.Server()
    reqs = [srv.polish(P[i], GUESSES) for i in range(4)]
    rmap = srv.map(P[4], _map())
    rscan = srv.scan(P[5], sc, r0)
    got = [r.wait() for r in reqs]
    cal, val = rmap.wait()
    rows, _ = rscan.wait()
    for a, b in zip(got, alone_roots):
        assert np.array_equal(a, b, equal_nan=True)
    assert np.array_equal(cal, alone_map[1], equal_nan=True)
    assert np.array_equal(val, alone_map[2], equal_nan=True)
    assert np.array_equal(rows, alone_scan[0], equal_nan=True)
    st = srv.stats()
    assert st["peak_active"] >= 2
    assert all(r.latency_ms > 0 for r in reqs)
    srv.close()


def test_budget_serialises_but_keeps_results(api):
    P = _plasmas(api, n=3, seed=12)
    alone = [G.secant(GUESSES)[0] for G in P]
    srv = api.Server(hbm_budget=1)  # below any request: one at a time
    reqs = [srv.polish(G, GUESSES) for G in P]
    for r, a in zip(reqs, alone):
        assert np.array_equal(r.wait(), a, equal_nan=True)
    assert srv.stats()["peak_active"] == 1
    srv.close()


def test_requests_arriving_while_others_run(api):
    """Continuous batching: requests submitted after the first ones started
    join later rounds and still match their lone runs."""
    P = _plasmas(api, n=4, seed=13)
    alone = [G.secant(GUESSES)[0] for G in P]
    srv = api.Server()
    first = [srv.polish(P[0], GUESSES), srv.polish(P[1], GUESSES)]
    later = []
    while not first[0].done() and len(later) < 2:
        later.append(srv.polish(P[2 + len(later)], GUESSES))
    later += [srv.polish(P[2 + k], GUESSES) for k in range(len(later), 2)]
    res = [r.wait() for r in first + later]
    for a, b in zip(res, alone):
        assert np.array_equal(a, b, equal_nan=True)
    srv.close()


def test_requests_on_one_plasma_share_batches(api):
    """Polishes (and a map) on the same plasma run in shared batches; a
    shared batch changes how the device splits the node sums, so results
    agree with the lone runs to rounding (roots 1e-12, det D 1e-12)."""
    w = workloads.kpar_fast(nproc=0)
    s, sp = workloads.build(w, api.generate_f0)
    G = api.Plasma(s, sp)
    G.set_k(*w["k"])
    guesses = [[0.0099881 - 2.3e-7j * (1 + 0.1 * k)] for k in range(5)]
    alone = [G.secant(g)[0] for g in guesses]
    mp = _map(16, 8)
    mp.omi, mp.omf, mp.gami, mp.gamf = 0.005, 0.02, -1e-5, 1e-5
    alone_map = G.map_search(mp)
    srv = api.Server()
    reqs = [srv.polish(G, g) for g in guesses]
    rmap = srv.map(G, mp)
    for r, a in zip(reqs, alone):
        np.testing.assert_allclose(r.wait(), a, rtol=1e-12)
    cal, val = rmap.wait()
    np.testing.assert_allclose(cal, alone_map[1], rtol=1e-12)
    assert srv.stats()["peak_active"] >= 2
    srv.close()


def test_fused_rounds_of_many_plasmas_equal_alone(api):
    """Two dozen plasmas of different grids, species counts, nmax and
    precision polish at once: their evaluations share fused launches (one
    job per plasma), each with the launch shape of its lone batch, so every
    root is bit for bit the lone one."""
    rng = np.random.default_rng(21)
    P = []
    for i in range(24):
        w = workloads.uneven_plasma(rng, grid=((32, 64), (48, 96), (64, 128))[i % 3])
        s, sp = workloads.build_uneven(w, api.generate_f0)
        G = api.Plasma(s, sp, precision="mixed" if i % 2 else "fp64")
        G.set_k(*w["k"])
        P.append(G)
    guesses = [[complex(0.2 + 0.05 * i, -0.02)] for i in range(len(P))]
    alone = [G.secant(g)[0] for G, g in zip(P, guesses)]
    srv = api.Server()
    reqs = [srv.polish(G, g) for G, g in zip(P, guesses)]
    for r, a in zip(reqs, alone):
        assert np.array_equal(r.wait(), a, equal_nan=True)
    assert srv.stats()["peak_active"] >= 8
    srv.close()


def test_large_map_in_chunks(api):
    """A lattice larger than the server's map chunk (2048 frequencies) goes
    to the device in chunk-sized batches between the other requests' rounds:
    the same values as alps_map's single batch up to the last bits of the
    sums (whose order follows the batch size), the same sentinels, and the
    same values alone and beside other requests."""
    P = _plasmas(api, n=3, seed=23)
    mp = _map(64, 48)  # 3072 points: a chunk of 2048 and one of 1024
    alone = P[0].map_search(mp)
    srv = api.Server()
    r1 = srv.map(P[0], mp)
    cal1, val1 = r1.wait()
    reqs = [srv.polish(P[i], GUESSES) for i in (1, 2)]
    r2 = srv.map(P[0], mp)
    cal2, val2 = r2.wait()
    for r in reqs:
        r.wait()
    srv.close()
    assert np.array_equal(cal1, cal2, equal_nan=True) and np.array_equal(val1, val2, equal_nan=True)
    fin = np.isfinite(alone[2])
    assert np.array_equal(fin, np.isfinite(val1))
    assert np.array_equal(val1[~fin], alone[2][~fin], equal_nan=True)
    # det D of the same path in another batch shape: within 1e-10 of each
    # value plus 1e-13 of the map's largest (near its zeros the sums cancel)
    a, b = cal1[fin], alone[1][fin]
    assert np.all(np.abs(a - b) <= 1e-10 * np.abs(b) + 1e-13 * np.abs(b).max())
    assert np.all(np.abs(val1[fin] - alone[2][fin]) <= 1e-8)
