"""RNP::LA::LQ, QL and RQ for torch CUDA tensors (RNP/LA/LQ.hpp, QL.hpp,
RQ.hpp), on the GB300 library (include/rnp_gpu/lqr_gb300.h).

Matrices are column-major torch tensors as in rnp2_gb300.qr.  ``kind`` is
"lq", "ql" or "rq"; every routine works in place like its reference
counterpart, with a caller-owned workspace (``work``) or one of the queried
length allocated here.

  factor(kind, A, tau)                    Factor       (_gelqf / _geqlf / _gerqf)
  mult_q(kind, side, trans, V, tau, C)    MultQ        (_unmlq / _unmql / _unmrq)
                                          V: the k reflectors (k x nq rows for
                                          lq and rq, nq x k columns for ql)
  generate_q(kind, A, tau, k)             GenerateQ    (_unglq / _ungql / _ungrq)
"""
import ctypes as C

import torch

from ._capi import lib
from .qr import _bind_stream, _check, _prefix, colmajor

_NAMES = {"lq": ("gelqf", "unmlq", "unglq"), "ql": ("geqlf", "unmql", "ungql"), "rq": ("gerqf", "unmrq", "ungrq")}


def _fn(kind, which, t):
    return getattr(lib(), "rnpgpu_%s%s" % (_prefix(t), _NAMES[kind][which]))


def factor(kind, A, tau=None, work=None):
    """A = L Q (lq), Q L (ql) or R Q (rq) in place; returns tau."""
    m, n = A.shape
    if tau is None:
        tau = torch.zeros(max(min(m, n), 1), dtype=A.dtype, device=A.device)
    a, lda = colmajor(A)
    f = _fn(kind, 0, A)
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check(_NAMES[kind][0], f(m, n, a, lda, tau.data_ptr(), C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=A.dtype, device=A.device)
    lw = C.c_size_t(work.numel())
    _check(_NAMES[kind][0], f(m, n, a, lda, tau.data_ptr(), C.byref(lw), work.data_ptr()))
    return tau


def mult_q(kind, side, trans, V, tau, Cm, k=None, work=None):
    """C <- Q C, Q^H C, C Q or C Q^H with the reflectors V (see module doc)."""
    m, n = Cm.shape
    if k is None:
        k = V.shape[1] if kind == "ql" else V.shape[0]
    v, ldv = colmajor(V)
    c, ldc = colmajor(Cm)
    f = _fn(kind, 1, Cm)
    _bind_stream()
    args = (side.encode(), trans.encode(), m, n, k, v, ldv, tau.data_ptr(), c, ldc)
    if work is None:
        lw = C.c_size_t(0)
        _check(_NAMES[kind][1], f(*args, C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=Cm.dtype, device=Cm.device)
    lw = C.c_size_t(work.numel())
    _check(_NAMES[kind][1], f(*args, C.byref(lw), work.data_ptr()))
    return Cm


def generate_q(kind, A, tau, k=None, work=None):
    """Q in place of the factored A (rows of Q for lq and rq: m <= n;
    columns for ql: m >= n)."""
    m, n = A.shape
    if k is None:
        k = min(m, n)
    a, lda = colmajor(A)
    f = _fn(kind, 2, A)
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check(_NAMES[kind][2], f(m, n, k, a, lda, tau.data_ptr(), C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=A.dtype, device=A.device)
    lw = C.c_size_t(work.numel())
    _check(_NAMES[kind][2], f(m, n, k, a, lda, tau.data_ptr(), C.byref(lw), work.data_ptr()))
    return A
