"""The workspace layout a caller of QR inside the reference's generalized
eigensolver uses (RNP/LA/GeneralizedEigensystems.hpp:376-389, 456-469): one
work array whose first n entries are tau and whose rest is the work block of
Factor, MultQ("L","C") and GenerateQ, on a sub-block of B at an offset
(ilo, ilo).  The workspace query there passes `work` as tau and as the work
block at once.  Checked through the C ABI against the oracle running the same
sequence."""
import ctypes as C

import numpy as np
import pytest

from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import rnp2_gb300  # noqa: E402
from rnp2_gb300 import qr as gq  # noqa: E402

SZ = C.c_size_t


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


@pytest.mark.parametrize("p", ["z", "d"])
def test_tau_and_work_carved_from_one_buffer(oracle, p):
    lib = rnp2_gb300.lib()
    lib.rnpgpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    dt = {"z": torch.complex128, "d": torch.float64}[p]
    esz = {"z": 16, "d": 8}[p]
    n, ilo, ihi = 300, 7, 290
    irows = ihi - ilo
    q = "z" if p == "z" else "d"
    va, _ = oracle.larnv(q, 2, [1, 3, 5, 7], n * n)
    vb, _ = oracle.larnv(q, 2, [2, 4, 6, 8], n * n)
    A = np.asfortranarray(va.reshape(n, n).T)
    B = np.asfortranarray(vb.reshape(n, n).T)

    # workspace query, as the caller makes it: tau and work are the same pointer
    fac, mq, gen = (getattr(lib, "rnpgpu_%s%s" % (p, f)) for f in ("geqrf", "unmqr", "ungqr"))
    dummy = torch.zeros(1, dtype=dt, device="cuda")
    lw = 0
    for call in (lambda s: fac(n, n, None, n, dummy.data_ptr(), C.byref(s), dummy.data_ptr()),
                 lambda s: mq(b"L", b"C", n, n, n, None, n, dummy.data_ptr(), None, n, C.byref(s), dummy.data_ptr()),
                 lambda s: gen(n, n, n, None, n, dummy.data_ptr(), C.byref(s), dummy.data_ptr())):
        s = SZ(0)
        assert call(s) == 0
        lw = max(lw, s.value)
    lwork = lw + n
    work = torch.zeros(lwork, dtype=dt, device="cuda")
    tau = work.data_ptr()
    work2 = tau + n * esz
    lwork2 = lwork - n

    dA, dB = to_dev(A), to_dev(B)
    vl = gq.empty_colmajor(n, n, dt, "cuda")
    vl.zero_()
    vl.diagonal().fill_(1)
    ldb = dB.stride(1)
    lda = dA.stride(1)
    ldv = vl.stride(1)
    off = lambda t, ld: t.data_ptr() + (ilo + ilo * ld) * esz
    s = SZ(lwork2)
    assert fac(irows, irows, off(dB, ldb), ldb, tau, C.byref(s), work2) == 0
    s = SZ(lwork2)
    assert mq(b"L", b"C", irows, irows, irows, off(dB, ldb), ldb, tau, off(dA, lda), lda, C.byref(s), work2) == 0
    # lower part of the factor into vl, then Q in place there
    torch.cuda.synchronize()
    sub = dB[ilo + 1:ihi, ilo:ihi - 1]
    vl[ilo + 1:ihi, ilo:ihi - 1] = torch.tril(sub)
    s = SZ(lwork2)
    assert gen(irows, irows, irows, off(vl, ldv), ldv, tau, C.byref(s), work2) == 0
    torch.cuda.synchronize()

    Bo, Ao = B.copy(order="F"), A.copy(order="F")
    sb = np.asfortranarray(Bo[ilo:ihi, ilo:ihi])
    to = oracle.geqrf(p, irows, irows, sb)
    sa = np.asfortranarray(Ao[ilo:ihi, ilo:ihi])
    oracle.unmqr(p, "L", "C", irows, irows, irows, sb, to, sa)
    sq = np.asfortranarray(np.tril(sb, -1) + np.eye(irows))
    oracle.ungqr(p, irows, irows, irows, sq, to)

    gB = dB.cpu().numpy()
    gA = dA.cpu().numpy()
    assert rel(np.triu(gB[ilo:ihi, ilo:ihi]), np.triu(sb)) <= 1e-12
    assert rel(work[:irows].cpu().numpy(), to) <= 1e-12
    assert rel(gA[ilo:ihi, ilo:ihi], sa) <= 1e-12
    assert rel(vl[ilo:ihi, ilo:ihi].cpu().numpy(), sq) <= 1e-12
    # outside the sub-blocks nothing moved
    assert np.array_equal(gB[:ilo], B[:ilo]) and np.array_equal(gA[:, :ilo], A[:, :ilo])
