"""rnpgpu_dgeqrf_noalloc: Factor for callers that cannot allocate device memory
(frameworks that own and pre-budget it, fixed-budget real-time loops).  It
must give the same factorization as rnpgpu_dgeqrf with a caller work block,
call after call, and reject matrices too wide for its built-in scratch.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from qr_checks import R_TOL, V_TOL, rel, split_factor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import rnp2_gb300  # noqa: E402
from rnp2_gb300 import qr as gq  # noqa: E402

SZ, P = C.c_size_t, C.c_void_p


def noalloc_fn():
    f = rnp2_gb300.lib().rnpgpu_dgeqrf_noalloc
    f.argtypes = [SZ, SZ, P, SZ, P]
    f.restype = C.c_int
    return f


def factor_with_work(A):
    """rnpgpu_dgeqrf with a caller-owned work block (the regular entry point)."""
    lib = rnp2_gb300.lib()
    m, n = A.shape
    a, lda = gq.colmajor(A)
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    lw = SZ(0)
    assert lib.rnpgpu_dgeqrf(m, n, a, lda, tau.data_ptr(), C.byref(lw), None) == 0
    work = torch.empty(lw.value, dtype=torch.float64, device="cuda")
    assert lib.rnpgpu_dgeqrf(m, n, a, lda, tau.data_ptr(), C.byref(lw), work.data_ptr()) == 0
    return tau


def factor_noalloc(A):
    m, n = A.shape
    a, lda = gq.colmajor(A)
    tau = torch.zeros(min(m, n), dtype=torch.float64, device="cuda")
    lib = rnp2_gb300.lib()
    lib.rnpgpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    rc = noalloc_fn()(m, n, a, lda, tau.data_ptr())
    assert rc == 0, (rc, lib.rnpgpu_get_last_error())
    return tau


def random_colmajor(m, n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn((n, m), generator=g, dtype=torch.float64, device="cuda").t()


def test_noalloc_factor_matches_regular_factor_twice_in_a_row():
    # two calls in a row, different shapes: the second reuses the scratch the
    # first one left behind
    for (m, n, seed) in ((3000, 200, 1), (1500, 333, 2)):
        A = random_colmajor(m, n, seed)
        A1 = gq.to_colmajor(A)
        A2 = gq.to_colmajor(A)
        t1 = factor_with_work(A1)
        t2 = factor_noalloc(A2)
        torch.cuda.synchronize()
        f1 = A1.cpu().numpy()
        f2 = A2.cpu().numpy()
        R1, V1 = split_factor(f1, m, n)
        R2, V2 = split_factor(f2, m, n)
        assert rel(R2, R1) <= R_TOL["d"]
        assert rel(V2, V1) <= V_TOL["d"]
        assert np.max(np.abs(t2.cpu().numpy() - t1.cpu().numpy())) <= 10 * R_TOL["d"]


def test_noalloc_rejects_too_wide_matrices():
    # nothing is enqueued: the size is checked before any launch
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = noalloc_fn()(40000, 40000, buf.data_ptr(), 40000, buf.data_ptr())
    assert rc == -2
    assert b"scratch" in rnp2_gb300.lib().rnpgpu_get_last_error()


def test_noalloc_width_limit():
    # the documented limit: 16,000 columns always fit (W alone needs 512 bytes
    # a column of the 8 MiB scratch), and the result is the regular Factor's;
    # 16,400 columns need more than the whole scratch and are rejected
    m, n = 64, 16000
    A = random_colmajor(m, n, 3)
    A1 = gq.to_colmajor(A)
    A2 = gq.to_colmajor(A)
    t1 = factor_with_work(A1)
    t2 = factor_noalloc(A2)
    torch.cuda.synchronize()
    R1, V1 = split_factor(A1.cpu().numpy(), m, n)
    R2, V2 = split_factor(A2.cpu().numpy(), m, n)
    assert rel(R2, R1) <= R_TOL["d"]
    assert rel(V2, V1) <= V_TOL["d"]
    assert np.max(np.abs(t2.cpu().numpy() - t1.cpu().numpy())) <= 10 * R_TOL["d"]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    assert noalloc_fn()(m, 16400, buf.data_ptr(), m, buf.data_ptr()) == -2
