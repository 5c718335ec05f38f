"""RNP::LA::QR for torch CUDA tensors (RNP/LA/QR.hpp), on the GB300 library.

Matrices are column-major torch tensors: shape (m, n) with stride (1, lda),
e.g. ``torch.empty((n, lda), dtype=..., device="cuda").t()[:m]``.  Every
routine works in place exactly like its reference counterpart and runs on the
current torch CUDA stream.  Workspace is caller-owned, as in the reference:
pass ``work`` (a 1-D tensor of the same dtype) or let the wrapper allocate
one of the queried length.

  factor(A, tau)                       RNP::LA::QR::Factor            (geqrf)
  factor_unblocked(A, tau)             RNP::LA::QR::Factor_unblocked  (geqr2)
  mult_q(side, trans, A, tau, C, k)    RNP::LA::QR::MultQ             (unmqr)
  mult_q_unblocked(...)                RNP::LA::QR::MultQ_unblocked   (unm2r)
  generate_q(A, tau, k)                RNP::LA::QR::GenerateQ         (ungqr)
  generate_q_unblocked(A, tau, k)      RNP::LA::QR::GenerateQ_unblocked (ung2r)
"""
import ctypes as C

import torch

from ._capi import lib

_PREFIX = {torch.float32: "s", torch.float64: "d", torch.complex64: "c", torch.complex128: "z"}


class RNPGPUError(RuntimeError):
    def __init__(self, routine, code):
        msg = lib().rnpgpu_get_last_error().decode() if code > 0 else "argument %d is invalid" % (-code)
        super().__init__("%s returned %d: %s" % (routine, code, msg))
        self.code = code


def _prefix(t):
    try:
        return _PREFIX[t.dtype]
    except KeyError:
        raise TypeError("unsupported dtype %s" % t.dtype)


def colmajor(t):
    """(pointer, leading dimension) of a column-major CUDA tensor (m, n)."""
    if t.dim() != 2:
        raise ValueError("expected a 2-D tensor")
    m, n = t.shape
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if m > 1 and t.stride(0) != 1:
        raise ValueError("expected a column-major tensor (stride(0) == 1)")
    ld = t.stride(1) if n > 1 else max(m, 1)
    return t.data_ptr(), max(ld, 1)


def empty_colmajor(m, n, dtype, device="cuda", lda=None):
    lda = max(lda or m, 1)
    return torch.empty((max(n, 1), lda), dtype=dtype, device=device).t()[:m, :n]


def to_colmajor(x, lda=None):
    out = empty_colmajor(x.shape[0], x.shape[1], x.dtype, x.device, lda)
    out.copy_(x)
    return out


def _bind_stream():
    lib().rnpgpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))


def _check(routine, rc):
    if rc != 0:
        raise RNPGPUError(routine, rc)


def _work(dtype, device, need, work):
    if work is not None:
        return work.data_ptr(), work.numel()
    buf = torch.empty(max(int(need), 1), dtype=dtype, device=device)
    return buf.data_ptr(), buf.numel(), buf


def _query(fn, args_before, args_after):
    lw = C.c_size_t(0)
    rc = fn(*args_before, C.byref(lw), None, *args_after)
    return rc, lw.value


def factor(A, tau=None, work=None):
    """In-place QR of A (m x n); returns tau (length min(m, n))."""
    p = _prefix(A)
    m, n = A.shape
    k = min(m, n)
    if tau is None:
        tau = torch.zeros(max(k, 1), dtype=A.dtype, device=A.device)
    a, lda = colmajor(A)
    fn = getattr(lib(), "rnpgpu_%sgeqrf" % p)
    _bind_stream()
    keep = None
    if work is None:
        lw = C.c_size_t(0)
        _check("geqrf", fn(m, n, a, lda, tau.data_ptr(), C.byref(lw), None))
        keep = torch.empty(max(lw.value, 1), dtype=A.dtype, device=A.device)
        work = keep
    lw = C.c_size_t(work.numel())
    _check("geqrf", fn(m, n, a, lda, tau.data_ptr(), C.byref(lw), work.data_ptr()))
    return tau[:k]


def factor_unblocked(A, tau=None, work=None):
    p = _prefix(A)
    m, n = A.shape
    k = min(m, n)
    if tau is None:
        tau = torch.zeros(max(k, 1), dtype=A.dtype, device=A.device)
    if work is None:
        work = torch.empty(max(n, 1), dtype=A.dtype, device=A.device)
    a, lda = colmajor(A)
    _bind_stream()
    _check("geqr2", getattr(lib(), "rnpgpu_%sgeqr2" % p)(m, n, a, lda, tau.data_ptr(), work.data_ptr()))
    return tau[:k]


def mult_q(side, trans, A, tau, Cm, k=None, work=None):
    """C <- Q C, Q^H C, C Q or C Q^H (side "L"/"R", trans "N"/"C"), in place."""
    p = _prefix(Cm)
    m, n = Cm.shape
    nq = m if side[0] == "L" else n
    k = min(A.shape[1], nq) if k is None else k
    a, lda = colmajor(A)
    c, ldc = colmajor(Cm)
    fn = getattr(lib(), "rnpgpu_%sunmqr" % p)
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check("unmqr", fn(side.encode(), trans.encode(), m, n, k, a, lda, tau.data_ptr(), c, ldc, C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=Cm.dtype, device=Cm.device)
    lw = C.c_size_t(work.numel())
    _check("unmqr", fn(side.encode(), trans.encode(), m, n, k, a, lda, tau.data_ptr(), c, ldc, C.byref(lw), work.data_ptr()))
    return Cm


def mult_q_unblocked(side, trans, A, tau, Cm, k=None, work=None):
    p = _prefix(Cm)
    m, n = Cm.shape
    nq = m if side[0] == "L" else n
    k = min(A.shape[1], nq) if k is None else k
    if work is None:
        work = torch.empty(max(n if side[0] == "L" else m, 1), dtype=Cm.dtype, device=Cm.device)
    a, lda = colmajor(A)
    c, ldc = colmajor(Cm)
    _bind_stream()
    _check("unm2r", getattr(lib(), "rnpgpu_%sunm2r" % p)(side.encode(), trans.encode(), m, n, k, a, lda, tau.data_ptr(), c, ldc, work.data_ptr()))
    return Cm


def generate_q(A, tau, k=None, work=None):
    """Overwrite A (m x n, m >= n) with the first n columns of Q."""
    p = _prefix(A)
    m, n = A.shape
    k = n if k is None else k
    a, lda = colmajor(A)
    fn = getattr(lib(), "rnpgpu_%sungqr" % p)
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check("ungqr", fn(m, n, k, a, lda, tau.data_ptr(), C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=A.dtype, device=A.device)
    lw = C.c_size_t(work.numel())
    _check("ungqr", fn(m, n, k, a, lda, tau.data_ptr(), C.byref(lw), work.data_ptr()))
    return A


def generate_q_unblocked(A, tau, k=None, work=None):
    p = _prefix(A)
    m, n = A.shape
    k = n if k is None else k
    if work is None:
        work = torch.empty(max(n, 1), dtype=A.dtype, device=A.device)
    a, lda = colmajor(A)
    _bind_stream()
    _check("ung2r", getattr(lib(), "rnpgpu_%sung2r" % p)(m, n, k, a, lda, tau.data_ptr(), work.data_ptr()))
    return A


def workspace_query(routine, dtype, *dims, side="L", trans="N"):
    """Optimal *lwork of a blocked routine ("geqrf", "unmqr", "ungqr")."""
    p = _PREFIX[dtype]
    lw = C.c_size_t(0)
    L = lib()
    if routine == "geqrf":
        m, n = dims
        rc = L.rnpgpu_dgeqrf if p == "d" else getattr(L, "rnpgpu_%sgeqrf" % p)
        rc = rc(m, n, None, max(m, 1), None, C.byref(lw), None)
    elif routine == "unmqr":
        m, n, k = dims
        nq = m if side == "L" else n
        rc = getattr(L, "rnpgpu_%sunmqr" % p)(side.encode(), trans.encode(), m, n, k, None, max(nq, 1), None, None, max(m, 1), C.byref(lw), None)
    elif routine == "ungqr":
        m, n, k = dims
        rc = getattr(L, "rnpgpu_%sungqr" % p)(m, n, k, None, max(m, 1), None, C.byref(lw), None)
    else:
        raise ValueError(routine)
    _check(routine, rc)
    return lw.value
