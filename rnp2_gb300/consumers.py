"""The reference's callers of QR and QL for torch CUDA tensors, on the GB300
library (include/rnp_gpu/consumers_gb300.h).

Matrices are column-major torch tensors as in rnp2_gb300.qr; every routine
works in place like its reference counterpart, with a caller-owned workspace
(``work``) or one of the queried length allocated here.

  hessenberg_mult_q(side, trans, ilo, ihi, A, tau, C)
        RNP::LA::Hessenberg::MultQ (RNP/LA/Hessenberg.hpp:477-512), _unmhr
  hessenberg_generate_q(ilo, ihi, A, tau)
        RNP::LA::Hessenberg::GenerateQ (Hessenberg.hpp:539-590), _unghr
  tridiagonal_generate_q(uplo, A, tau)
        RNP::LA::Tridiagonal::GenerateQHerm (RNP/LA/Tridiagonal.hpp:1037-1097), _ungtr
  tridiagonal_mult_q(side, uplo, trans, A, tau, C)
        RNP::LA::Tridiagonal::MultQHerm (Tridiagonal.hpp:1140-1188), _unmtr
  generalized_triangularize_b(ilo, ihi, A, B, VL=None, VR=None)
        the QR step of ComplexGeneralizedEigensystem
        (RNP/LA/GeneralizedEigensystems.hpp:457-472); returns tau
"""
import ctypes as C

import torch

from ._capi import lib
from .qr import _bind_stream, _check, _prefix, colmajor


def _fn(t, name):
    return getattr(lib(), "rnpgpu_%s%s" % (_prefix(t), name))


def _run(name, f, args, like, work):
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check(name, f(*args, C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=like.dtype, device=like.device)
    lw = C.c_size_t(work.numel())
    _check(name, f(*args, C.byref(lw), work.data_ptr()))
    return work


def hessenberg_mult_q(side, trans, ilo, ihi, A, tau, Cm, work=None):
    """C <- Q C, Q^H C, C Q or C Q^H for the Q of a Hessenberg reduction A."""
    m, n = Cm.shape
    a, lda = colmajor(A)
    c, ldc = colmajor(Cm)
    _run("unmhr", _fn(Cm, "unmhr"), (side.encode(), trans.encode(), m, n, ilo, ihi, a, lda, tau.data_ptr(), c, ldc), Cm, work)
    return Cm


def hessenberg_generate_q(ilo, ihi, A, tau, work=None):
    """The n x n Q in place of the Hessenberg reduction A."""
    n = A.shape[0]
    a, lda = colmajor(A)
    _run("unghr", _fn(A, "unghr"), (n, ilo, ihi, a, lda, tau.data_ptr()), A, work)
    return A


def tridiagonal_generate_q(uplo, A, tau, work=None):
    """The n x n Q in place of the Hermitian tridiagonal reduction A."""
    n = A.shape[0]
    a, lda = colmajor(A)
    _run("ungtr", _fn(A, "ungtr"), (uplo.encode(), n, a, lda, tau.data_ptr()), A, work)
    return A


def tridiagonal_mult_q(side, uplo, trans, A, tau, Cm, work=None):
    """C <- op(Q) C or C op(Q) for the Q of a Hermitian tridiagonal reduction."""
    m, n = Cm.shape
    a, lda = colmajor(A)
    c, ldc = colmajor(Cm)
    _run("unmtr", _fn(Cm, "unmtr"), (side.encode(), uplo.encode(), trans.encode(), m, n, a, lda, tau.data_ptr(), c, ldc), Cm, work)
    return Cm


def generalized_triangularize_b(ilo, ihi, A, B, VL=None, VR=None, work=None):
    """B's rows ilo:ihi triangularized, Q^H applied to A, VL / VR started from
    Q / I (complex tensors); returns tau (n), the first n workspace entries."""
    n = A.shape[0]
    a, lda = colmajor(A)
    b, ldb = colmajor(B)
    vl, ldvl = colmajor(VL) if VL is not None else (None, 1)
    vr, ldvr = colmajor(VR) if VR is not None else (None, 1)
    work = _run("gg_triangularize_b", _fn(A, "gg_triangularize_b"), (n, ilo, ihi, a, lda, b, ldb, vl, ldvl, vr, ldvr), A, work)
    return work[:n]
