"""alps_disp_batch_noalloc: det D for a device batch without any allocation
by the library.

It serves callers that cannot let the library allocate device memory while
they run (an application whose caching allocator owns the device heap, a
real-time loop that cannot absorb cudaMalloc's device-wide synchronisation, a
plugin host that forbids plugin allocations).  Its scratch comes from one
static device array, so its results must equal those of the allocating entry
point alps_disp_batch_device on the same inputs, call after call (the array
keeps the previous call's contents).  This file is collected last; it passes
alone in a fresh process (where the first call performs the per-device
address lookup) and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from alps_gb300 import workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-13   # the tolerance used for batch-vs-batch comparisons elsewhere


@pytest.fixture(scope="module")
def plasma():
    import torch
    assert torch.cuda.is_available(), "needs a CUDA device"
    from alps_gb300 import api
    w = workloads.proton_electron(24, 48, 1.0, 0.3, 1e-14)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species)
    G.set_k(1.0, 0.3)
    return G


def _dev(torch, oms):
    return torch.from_numpy(np.stack([oms.real, oms.imag], 1).copy()).cuda()


def test_noalloc_matches_allocating_entry_point_twice(plasma):
    import torch
    from alps_gb300._native import lib
    G = plasma
    rng = np.random.default_rng(7)
    for oms in (np.array([0.45 - 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 0.7 + 0.0j, 2.2 - 0.35j]),
                rng.uniform(0.05, 2.5, 300) + 1j * rng.uniform(-0.4, 0.1, 300)):
        n = len(oms)
        om_d = _dev(torch, oms)
        ref_d = torch.empty_like(om_d)
        G.disp_batch_device(n, om_d.data_ptr(), ref_d.data_ptr(), 0)
        torch.cuda.synchronize()
        ref = ref_d[:, 0].cpu().numpy() + 1j * ref_d[:, 1].cpu().numpy()
        for _ in range(2):
            out_d = torch.full_like(om_d, float("nan"))
            need = C.c_size_t()
            st = lib().alps_disp_batch_noalloc(G.handle, n, C.c_void_p(om_d.data_ptr()),
                                               C.c_void_p(out_d.data_ptr()), None, C.byref(need))
            assert st == 0, lib().alps_error_string(st)
            torch.cuda.synchronize()
            out = out_d[:, 0].cpu().numpy() + 1j * out_d[:, 1].cpu().numpy()
            assert np.all(np.abs(out - ref) <= RTOL * np.abs(ref)), np.abs(out - ref).max()
            assert 0 < need.value <= 16 << 20


def test_noalloc_rejects_batches_beyond_the_scratch_limit(plasma):
    from alps_gb300._native import lib
    G = plasma
    need = C.c_size_t()
    # 10^6 frequencies need far more than the 16 MiB of static scratch; the
    # size check runs on the host before any launch, so the buffers are never
    # touched (dummy non-null pointers)
    st = lib().alps_disp_batch_noalloc(G.handle, 1000000, C.c_void_p(16), C.c_void_p(16), None, C.byref(need))
    assert st == 20  # ALPS_E_INVALID
    assert need.value > 16 << 20
