"""Device errors of the asynchronous entry point reach the caller.

alps_disp_batch_device returns as soon as its kernels are queued, so a
device-side error (here alps_error(8): a relativistic resonance window that
covers the whole subluminal cone, src/ALPS_fns_rel.f90:656) cannot be its
return value.  alps_batch_status reads the batch's error word after the
stream drains.  The failing case is first confirmed on the oracle, on the
CPU; on the GPU the kernel only records the condition in its error word.
"""
import numpy as np
import pytest

from alps_gb300 import _abi, workloads

SUBLUMINAL = 8


def relativistic_case(M_I):
    """A relativistic Maxwellian at v_A/c = 0.1 (fit type 5 on the Gamma
    rows) on a 30x80 grid with a 40x40 (Gamma, pparbar) grid: with a
    principal-value window of M_I = 20 nodes every resonant order's window
    covers the narrow cone rows near Gamma = 1; with M_I = 3 none does."""
    from oracle import pyoracle as po
    vA = 0.1
    d = workloads._dist(kind=1, ms=1.0, vA=vA, maxP=5.0)
    pp, pl, f0, ideal = po.generate_f0(d, 30, 80)
    sysd = _abi.system_defaults(nspec=1, nperp=30, npar=80, kperp=0.3, kpar=0.2, vA=vA, Bessel_zero=1e-20,
                                positions_principal=M_I, ngamma=40, npparbar=40)
    pc = 2.0 / (vA * vA)
    sp = _abi.species_defaults(ns=1, qs=1, ms=1, relat=1, fits=[(5, [ideal[0] * np.exp(pc), 1e-12, 0, 0, 0], pc)])
    return sysd, [(sp, pp, pl, f0)]


OMS = np.array([0.5 - 0.1j, 1.0 - 0.05j, 0.2 + 0.01j])


def test_oracle_raises_subluminal_on_the_case():
    from oracle import pyoracle as po
    sysd, species = relativistic_case(20)
    P = po.OraclePlasma(sysd, species)
    P.set_k(0.3, 0.2)
    with pytest.raises(_abi.AlpsError) as e:
        P.disp(OMS[0])
    assert e.value.status == SUBLUMINAL


@pytest.mark.gpu
@pytest.mark.parametrize("M_I,expect", [(20, SUBLUMINAL), (3, 0)])
def test_device_batch_reports_device_error(M_I, expect):
    import torch
    assert torch.cuda.is_available()
    from alps_gb300 import api
    sysd, species = relativistic_case(M_I)
    G = api.Plasma(sysd, species)
    G.set_k(0.3, 0.2)
    # the synchronous entry point returns the code itself
    if expect:
        with pytest.raises(_abi.AlpsError) as e:
            G.disp_batch(OMS)
        assert e.value.status == expect
    else:
        G.disp_batch(OMS)
    # the asynchronous one through alps_batch_status, after the stream drains
    om_d = torch.from_numpy(np.stack([OMS.real, OMS.imag], 1).copy()).cuda()
    D_d = torch.empty_like(om_d)
    G.disp_batch_device(len(OMS), om_d.data_ptr(), D_d.data_ptr(), 0)
    assert G.batch_status() == expect
    # the status belongs to the context: a clean batch elsewhere reports 0
    if expect:
        G2 = api.Plasma(*relativistic_case(3))
        G2.set_k(0.3, 0.2)
        G2.disp_batch_device(len(OMS), om_d.data_ptr(), D_d.data_ptr(), 0)
        assert G2.batch_status() == 0
