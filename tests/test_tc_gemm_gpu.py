"""The FP32 tensor-core contraction (tcgen05, three-term BF16 split) against an
FP64 reference: its error must stay at FP32 level (the accuracy the mixed
least-squares refinement relies on), for every op combination and for sizes
that are not tile multiples."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import rnp2_gb300  # noqa: E402


def colmajor(t):
    return t.t().contiguous().t()


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("mnk", [(128, 32, 32), (300, 70, 100), (1000, 129, 513), (4096, 16, 32)])
@pytest.mark.parametrize("beta", [0.0, 1.0])
def test_sgemm_tc_is_fp32_accurate(ta, tb, mnk, beta):
    m, n, k = mnk
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    A = colmajor(torch.randn((k, m) if ta == "T" else (m, k), generator=g, device="cuda", dtype=torch.float32))
    B = colmajor(torch.randn((n, k) if tb == "T" else (k, n), generator=g, device="cuda", dtype=torch.float32))
    Cm = colmajor(torch.randn((m, n), generator=g, device="cuda", dtype=torch.float32))
    C0 = Cm.clone()
    alpha = -0.75
    lib = rnp2_gb300.lib()
    lib.rnpgpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    rc = lib.rnpgpu_sgemm_tc(ta.encode(), tb.encode(), m, n, k, alpha, A.data_ptr(), A.stride(1), B.data_ptr(), B.stride(1), beta, Cm.data_ptr(), Cm.stride(1))
    assert rc == 0
    torch.cuda.synchronize()
    Ad = A.double().t() if ta == "T" else A.double()
    Bd = B.double().t() if tb == "T" else B.double()
    ref = alpha * (Ad @ Bd) + beta * C0.double()
    scale = (Ad.abs() @ Bd.abs()).abs() * abs(alpha) + beta * C0.double().abs()
    err = ((Cm.double() - ref).abs() / scale.clamp_min(1e-30)).max().item()
    # FP32 dot products of length k carry about k * 2^-24 relative error in the worst case
    assert err <= 4 * k * 2.0 ** -24 + 2.0 ** -22, err
    assert lib.rnpgpu_device_status(1) == 0
