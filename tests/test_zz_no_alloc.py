"""alps_disp_batch_noalloc: det D for a device batch without any allocation
by the library.

It serves callers that cannot let the library allocate device memory while
they run (an application whose caching allocator owns the device heap, a
real-time loop that cannot absorb cudaMalloc's device-wide synchronisation, a
plugin host that forbids plugin allocations).  Its scratch comes from one
static device array, so its results must equal those of the allocating entry
point alps_disp_batch_device on the same inputs, call after call (the array
keeps the previous call's contents).  The plasmas cover every carve-out of
the array: the bi-Maxwellian grid species (pole sums and resonant items), a
relativistic species (per-order relativistic results) and a closed-form
species beside a grid species (the NHDS results).  Device errors come back
through alps_batch_status, whose word also sits in the array.  This file is
collected last; it passes alone in a fresh process (where the first call
performs the per-device address lookup) and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from alps_gb300 import _abi, workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-13   # the tolerance used for batch-vs-batch comparisons elsewhere


def _bimax():
    from alps_gb300 import api
    w = workloads.proton_electron(24, 48, 1.0, 0.3, 1e-14)
    return workloads.build(w, api.generate_f0), (1.0, 0.3)


def _relativistic(M_I=3):
    from alps_gb300 import api
    vA = 0.1
    d = workloads._dist(kind=1, ms=1.0, vA=vA, maxP=5.0)
    pp, pl, f0, ideal = api.generate_f0(d, 30, 80)
    sysd = _abi.system_defaults(nspec=1, nperp=30, npar=80, kperp=0.3, kpar=0.2, vA=vA, Bessel_zero=1e-20,
                                positions_principal=M_I, ngamma=40, npparbar=40)
    pc = 2.0 / (vA * vA)
    sp = _abi.species_defaults(ns=1, qs=1, ms=1, relat=1, fits=[(5, [ideal[0] * np.exp(pc), 1e-12, 0, 0, 0], pc)])
    return (sysd, [(sp, pp, pl, f0)]), (0.3, 0.2)


def _closed_form():
    from alps_gb300 import api
    me = 1.0 / 1836.0
    de = workloads._dist(kind=1, ms=me, vA=1e-4, maxP=6.0)
    pe, qe, fe, ie = api.generate_f0(de, 24, 48)
    sysd = _abi.system_defaults(nspec=2, nperp=24, npar=48, kperp=0.3, kpar=0.2, vA=1e-4, Bessel_zero=1e-20)
    spB = _abi.species_defaults(ns=1, qs=1, ms=1, use_bM=1, bM_nmaxs=500, bM_Bessel_zeros=1e-50, bM_betas=1.0,
                                bM_alphas=1.0, bM_pdrifts=0.1)
    spE = _abi.species_defaults(ns=1, qs=-1, ms=me, fits=[(1, list(ie[:3]) + [0, 0], ie[5])])
    return (sysd, [(spB, None, None, None), (spE, pe, qe, fe)]), (0.3, 0.2)


PLASMAS = {"bimaxwellian": _bimax, "relativistic": _relativistic, "closed_form": _closed_form}


def _plasma(name):
    import torch
    assert torch.cuda.is_available(), "needs a CUDA device"
    from alps_gb300 import api
    (system, species), k = PLASMAS[name]()
    G = api.Plasma(system, species)
    G.set_k(*k)
    return G


def _dev(torch, oms):
    return torch.from_numpy(np.stack([oms.real, oms.imag], 1).copy()).cuda()


def _noalloc(G, n, om_d, out_d):
    from alps_gb300._native import lib
    need = C.c_size_t()
    st = lib().alps_disp_batch_noalloc(G.handle, n, C.c_void_p(om_d.data_ptr()), C.c_void_p(out_d.data_ptr()),
                                       None, C.byref(need))
    return st, need.value


@pytest.mark.parametrize("name", list(PLASMAS))
def test_noalloc_matches_allocating_entry_point_twice(name):
    import torch
    from alps_gb300._native import lib
    G = _plasma(name)
    rng = np.random.default_rng(7)
    for oms in (np.array([0.45 - 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 0.7 + 0.0j, 2.2 - 0.35j]),
                rng.uniform(0.05, 2.5, 300) + 1j * rng.uniform(-0.4, 0.1, 300)):
        n = len(oms)
        om_d = _dev(torch, oms)
        ref_d = torch.empty_like(om_d)
        G.disp_batch_device(n, om_d.data_ptr(), ref_d.data_ptr(), 0)
        torch.cuda.synchronize()
        # a few random frequencies put the relativistic species' resonance
        # window over the whole subluminal cone (alps_error(8)); the status
        # must then be the same through both entry points
        ref_status = G.batch_status()
        assert ref_status in (0, 8)
        ref = ref_d[:, 0].cpu().numpy() + 1j * ref_d[:, 1].cpu().numpy()
        for _ in range(2):
            out_d = torch.full_like(om_d, float("nan"))
            st, need = _noalloc(G, n, om_d, out_d)
            assert st == 0, lib().alps_error_string(st)
            assert G.batch_status() == ref_status
            torch.cuda.synchronize()
            out = out_d[:, 0].cpu().numpy() + 1j * out_d[:, 1].cpu().numpy()
            ok = np.isfinite(ref)
            assert np.array_equal(np.isfinite(out), ok)
            assert np.all(np.abs(out[ok] - ref[ok]) <= RTOL * np.abs(ref[ok])), np.abs(out[ok] - ref[ok]).max()
            assert 0 < need <= 16 << 20


def test_noalloc_reports_device_errors():
    """A relativistic case whose resonance windows cover the subluminal cone
    (alps_error(8), confirmed on the oracle in test_gpu_async_status.py): the
    error word in the static scratch reaches the caller, and the next clean
    call clears it."""
    import torch
    from alps_gb300 import api
    (system, species), k = _relativistic(M_I=20)
    G = api.Plasma(system, species)
    G.set_k(*k)
    oms = np.array([0.5 - 0.1j, 1.0 - 0.05j])
    om_d = _dev(torch, oms)
    out_d = torch.empty_like(om_d)
    st, _ = _noalloc(G, len(oms), om_d, out_d)
    assert st == 0
    assert G.batch_status() == 8  # ALPS_E_SUBLUMINAL
    G2 = _plasma("relativistic")
    st, _ = _noalloc(G2, len(oms), om_d, out_d)
    assert st == 0
    assert G2.batch_status() == 0


def test_noalloc_rejects_batches_beyond_the_scratch_limit():
    from alps_gb300._native import lib
    G = _plasma("bimaxwellian")
    need = C.c_size_t()
    # 10^6 frequencies need far more than the 16 MiB of static scratch; the
    # size check runs on the host before any launch, so the buffers are never
    # touched (dummy non-null pointers)
    st = lib().alps_disp_batch_noalloc(G.handle, 1000000, C.c_void_p(16), C.c_void_p(16), None, C.byref(need))
    assert st == 20  # ALPS_E_INVALID
    assert need.value > 16 << 20
