"""The tensor-core FP64-accurate product (tc_gemm.cu, alps_tc_product) and
its use in the mixed path's p_perp contraction.

Reference values are computed in numpy's extended precision (longdouble:
80-bit on x86, 128-bit on Arm), far below the errors checked here.
"""
import ctypes as C

import numpy as np
import pytest

from alps_gb300 import workloads

pytestmark = pytest.mark.gpu


def _tc(torch, A, B, checked):
    from alps_gb300._native import lib
    M, K = A.shape
    N = B.shape[1]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    dC = torch.full((M, N), float("nan"), dtype=torch.float64, device="cuda")
    nf = C.c_int(-1)
    st = lib().alps_tc_product(C.c_void_p(dA.data_ptr()), C.c_void_p(dB.data_ptr()), C.c_void_p(dC.data_ptr()),
                               M, N, K, int(checked), C.byref(nf))
    assert st == 0, lib().alps_error_string(st)
    return dC.cpu().numpy(), nf.value


def _exact(A, B):
    return np.dot(A.astype(np.longdouble), B.astype(np.longdouble))


@pytest.mark.parametrize("shape", [(300, 200, 255), (128, 64, 32), (5, 7, 3), (260, 130, 256)])
def test_bare_product_within_its_bound(shape):
    import torch
    assert torch.cuda.is_available()
    M, N, K = shape
    rng = np.random.default_rng(11)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-8, 8, (M, K)))
    B = rng.standard_normal((K, N)) * np.exp(rng.uniform(-8, 8, (K, N)))
    A[0, :] = 0.0  # a zero row
    got, _ = _tc(torch, A, B, checked=False)
    ref = _exact(A, B)
    ea = np.frexp(np.abs(A).max(axis=1))[1]
    eb = np.frexp(np.abs(B).max(axis=0))[1]
    bound = 10.0 * K * 2.0 ** -56 * np.ldexp(1.0, ea[:, None] + eb[None, :])
    err = np.abs(got.astype(np.longdouble) - ref).astype(np.float64)
    assert np.all(err <= bound), (err / bound).max()
    assert np.all(got[0] == 0.0)


def test_checked_product_on_misaligned_rows():
    """Rows whose large elements sit where the columns are tiny (Bessel rows
    of high order against Maxwellian columns): the fixed-point bound is far
    above such entries, the check sends them to FP64, and every entry ends
    within FP64 GEMM's own bound."""
    import torch
    M, N, K = 90, 300, 255
    p = np.linspace(0.0, 6.0, K)
    n = np.arange(M // 3)
    rows = np.exp(-((p[None, :] - 0.2 * n[:, None]) ** 2) * 3.0) * (1.0 + 0.1 * np.sin(p[None, :] * n[:, None]))
    A = np.concatenate([rows, rows * p[None, :], -rows * p[None, :] ** 2])
    q = np.linspace(-6.0, 6.0, N)
    B = np.exp(-p[:, None] ** 2 - q[None, :] ** 2) * (q[None, :] - 0.3 * p[:, None])
    got, nfixed = _tc(torch, A, B, checked=True)
    ref = _exact(A, B)
    mag = np.abs(A) @ np.abs(B)
    err = np.abs(got.astype(np.longdouble) - ref).astype(np.float64)
    assert np.all(err <= 2.0 ** -44 * mag + 1e-300), (err / mag).max()
    assert nfixed > 0


def test_mixed_path_contraction_runs_on_tensor_cores():
    """The mixed path's k tables come from the tensor-core contraction; its
    det D stays within the parity gates' reach of the plain path's."""
    import torch
    from alps_gb300 import api
    w = workloads.proton_electron(64, 128, 2.0, 0.3, 1e-12)
    system, species = workloads.build(w, api.generate_f0)
    G = api.Plasma(system, species, precision="mixed")
    G.set_k(2.0, 0.3)
    st = G.stats()
    assert st.tc_contractions == 2
    assert 0 <= st.tc_fixed_entries < st.tc_entries
    oms = np.array([0.45 - 0.2j, 1.3 - 0.004j, 0.9 + 0.003j, 2.2 - 0.35j])
    Dm = G.disp_batch(oms)
    G.set_precision("fp64")
    assert G.stats().tc_contractions == 0
    Dp = G.disp_batch(oms)
    assert np.all(np.abs(Dm - Dp) <= 1e-9 * np.abs(Dp)), np.abs(Dm - Dp) / np.abs(Dp)
