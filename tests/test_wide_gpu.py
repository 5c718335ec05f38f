"""The mixed solver's internal FP32 factorization with 128-column trailing
updates on the tensor cores (three BF16 slices, six products, FP32
accumulation) against the same factorization with rank-32 trailing updates on
the CUDA cores: R, V and tau agree to FP32 accuracy, and Q R reproduces A.
Shapes cover full and ragged last blocks, ragged last row tiles (m not a
multiple of 128) and a leading dimension larger than m."""
import ctypes as C

import numpy as np
import pytest

from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import rnp2_gb300  # noqa: E402
from rnp2_gb300 import _capi  # noqa: E402
from rnp2_gb300 import qr as gq  # noqa: E402

SZ = C.c_size_t


def mixed_factor(A, rank32):
    """(factor, tau, launches per kernel class) of rnpgpu_sgeqrf_mixed on a copy of A."""
    lib = rnp2_gb300.lib()
    lib.rnpgpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    m, n = A.shape
    F = gq.to_colmajor(A, lda=A.stride(1))
    a, lda = gq.colmajor(F)
    tau = torch.zeros(min(m, n), dtype=torch.float32, device="cuda")
    ts = torch.zeros(((n + 31) // 32) * 1024, dtype=torch.float32, device="cuda")
    lw = SZ(0)
    failed = C.c_int(0)
    flags = 2 if rank32 else 0
    assert lib.rnpgpu_sgeqrf_mixed(m, n, a, lda, tau.data_ptr(), ts.data_ptr(), flags, C.byref(failed), C.byref(lw), None) == 0
    work = torch.empty(lw.value, dtype=torch.float32, device="cuda")
    lib.rnpgpu_timing_enable(1)
    _capi.timing_report()
    try:
        rc = lib.rnpgpu_sgeqrf_mixed(m, n, a, lda, tau.data_ptr(), ts.data_ptr(), flags, C.byref(failed), C.byref(lw), work.data_ptr())
        torch.cuda.synchronize()
        rep = _capi.timing_report()
    finally:
        lib.rnpgpu_timing_enable(0)
    assert rc == 0, (rc, lib.rnpgpu_get_last_error())
    assert failed.value == 0
    assert lib.rnpgpu_device_status(1) == 0
    return F, tau, {k: v[0] for k, v in rep.items()}


@pytest.mark.parametrize("mnl", [(4096, 512, 4096), (3000, 300, 3000), (1032, 257, 1032), (4099, 384, 4100), (65536, 512, 65536)])
def test_wide_update_matches_rank32_updates(mnl):
    m, n, lda = mnl
    g = torch.Generator(device="cuda").manual_seed(m + n)
    A = torch.randn((n, lda), generator=g, dtype=torch.float32, device="cuda").t()[:m]
    Fw, tw, kw = mixed_factor(A, rank32=False)
    Fr, tr, kr = mixed_factor(A, rank32=True)
    full_blocks_with_trailing = max(0, (n - 1) // 128)
    assert kw.get("wide_update", 0) == full_blocks_with_trailing, kw
    assert "wide_update" not in kr
    Rw, Rr = torch.triu(Fw[:n]), torch.triu(Fr[:n])
    assert float(torch.linalg.norm(Rw - Rr) / torch.linalg.norm(Rr)) <= 2e-5
    Vw, Vr = torch.tril(Fw, -1), torch.tril(Fr, -1)
    assert float(torch.linalg.norm(Vw - Vr) / torch.linalg.norm(Vr)) <= 2e-4
    assert float(torch.max(torch.abs(tw - tr))) <= 1e-4
    # Q R = A for the tensor-core result (Q from the drop-in GenerateQ)
    Q = gq.generate_q(gq.to_colmajor(Fw[:, :n]), tw, n)
    res = torch.linalg.norm(Q.double() @ Rw.double() - A.double()) / torch.linalg.norm(A.double())
    assert float(res) <= 2e-6 * np.sqrt(n), float(res)
    orth = torch.linalg.norm(Q.double().t() @ Q.double() - torch.eye(n, dtype=torch.float64, device="cuda"))
    assert float(orth) <= 2e-6 * n, float(orth)


@pytest.mark.parametrize("fill", [0.0, 1e30, float("nan")])
def test_mixed_solve_does_not_depend_on_workspace_contents(fill):
    # every workspace region the wide path reads is written first in the same
    # call (the panel T factors are read as upper triangles only): the result
    # is the same bit for bit whatever the workspace held before
    from rnp2_gb300 import ls as gls

    m, n, nrhs = 4096, 384, 2
    g = torch.Generator(device="cuda").manual_seed(5)
    A = gq.to_colmajor(torch.randn((n, m), generator=g, dtype=torch.float64, device="cuda").t())
    B = gq.to_colmajor(torch.randn((nrhs, m), generator=g, dtype=torch.float64, device="cuda").t())
    lw = gls.refine_workspace(A, nrhs)
    X0, info0 = gls.gels_refine(A, B, work=torch.zeros(lw, dtype=torch.float64, device="cuda"))
    X1, info1 = gls.gels_refine(A, B, work=torch.full((lw,), fill, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    assert info0["converged"] == 1 and info1 == info0
    assert torch.equal(X0, X1)
