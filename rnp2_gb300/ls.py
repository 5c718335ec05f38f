"""Least squares on the GB300 QR (include/rnp_gpu/ls_gb300.h), for torch CUDA
tensors in column-major layout (see rnp2_gb300.qr).

  gels(A, B)            plain: Factor, MultQ("L","C"), triangular solve; in place
  gels_refine(A, B)     mixed: FP32 factor + FP64 iterative refinement
  trsm_upper(R, B)      B <- R^{-1} B, R upper triangular (SolveTrM "L","U","N","N")
  residual(A, X, B)     R = B - A X and optionally G = A^T R, FP64-accurate on
                        the tensor cores (FP64 real data)
"""
import ctypes as C

import torch

from ._capi import RefineInfo, lib
from .qr import _PREFIX, _bind_stream, _check, colmajor, empty_colmajor


def trsm_upper(R, B):
    p = _PREFIX[B.dtype]
    n = R.shape[1]
    r, ldr = colmajor(R)
    b, ldb = colmajor(B)
    _bind_stream()
    _check("trsm_lunn", getattr(lib(), "rnpgpu_%strsm_lunn" % p)(n, B.shape[1], r, ldr, b, ldb))
    return B


def gels(A, B, tau=None, work=None):
    """min ||A X - B||: A (m x n, m >= n) and B (m x nrhs) are overwritten;
    returns the solution view B[:n]."""
    p = _PREFIX[A.dtype]
    m, n = A.shape
    nrhs = B.shape[1]
    if tau is None:
        tau = torch.zeros(max(n, 1), dtype=A.dtype, device=A.device)
    a, lda = colmajor(A)
    b, ldb = colmajor(B)
    fn = getattr(lib(), "rnpgpu_%sgels" % p)
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check("gels", fn(m, n, nrhs, a, lda, tau.data_ptr(), b, ldb, C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=A.dtype, device=A.device)
    lw = C.c_size_t(work.numel())
    _check("gels", fn(m, n, nrhs, a, lda, tau.data_ptr(), b, ldb, C.byref(lw), work.data_ptr()))
    return B[:n]


def refine_workspace(A, nrhs):
    p = {torch.float64: "ds", torch.complex128: "zc"}[A.dtype]
    m, n = A.shape
    lw = C.c_size_t(0)
    fn = getattr(lib(), "rnpgpu_%sgels" % p)
    _check("gels_refine", fn(m, n, nrhs, None, max(m, 1), None, max(m, 1), None, max(n, 1), 0, 0, None, C.byref(lw), None))
    return lw.value


def gels_refine(A, B, X=None, max_iter=0, work=None, forward=False, rank32=False):
    """Mixed-precision least squares (FP32 factor, FP64 refinement) of an FP64
    (or complex128) problem; A and B are not modified.  forward=True adds the
    corrected seminormal-equation steps for FP64 forward accuracy;
    rank32=True keeps the real FP32 factor's trailing updates at 32 columns
    on the CUDA cores (instead of 128 columns on the tensor cores).
    max_iter <= 0 selects the default (10 steps, 30 in forward mode).
    Returns (X, info)."""
    p = {torch.float64: "ds", torch.complex128: "zc"}[A.dtype]
    m, n = A.shape
    nrhs = B.shape[1]
    if X is None:
        X = empty_colmajor(n, nrhs, A.dtype, A.device)
    a, lda = colmajor(A)
    b, ldb = colmajor(B)
    x, ldx = colmajor(X)
    fn = getattr(lib(), "rnpgpu_%sgels" % p)
    _bind_stream()
    if work is None:
        work = torch.empty(max(refine_workspace(A, nrhs), 1), dtype=A.dtype, device=A.device)
    info = RefineInfo()
    lw = C.c_size_t(work.numel())
    _check("gels_refine", fn(m, n, nrhs, a, lda, b, ldb, x, ldx, int(max_iter), (1 if forward else 0) | (2 if rank32 else 0), C.byref(info), C.byref(lw), work.data_ptr()))
    return X, info.as_dict()


def _host_colmajor(t):
    """(pointer, leading dimension) of a column-major CPU tensor (m, n)."""
    if t.dim() != 2 or t.is_cuda:
        raise ValueError("expected a 2-D CPU tensor")
    m, n = t.shape
    if m > 1 and t.stride(0) != 1:
        raise ValueError("expected a column-major tensor (stride(0) == 1)")
    return t.data_ptr(), max(t.stride(1) if n > 1 else m, 1)


def host_refine_workspace(m, n, nrhs):
    lw = C.c_size_t(0)
    _check("gels_refine_host", lib().rnpgpu_dsgels_host(m, n, nrhs, None, max(m, 1), None, max(m, 1), None, max(n, 1), 0, 0, None, C.byref(lw), None))
    return lw.value


def gels_refine_host(A, B, X, max_iter=0, work=None, forward=False, rank32=False, device="cuda"):
    """The mixed-precision solve of gels_refine from HOST (CPU, preferably
    pinned) FP64 tensors A (m x n), B (m x nrhs) into the host tensor X
    (n x nrhs), all column-major: A is copied in 128-column ranges that the
    GPU starts on as they land.  X is complete once the current stream is
    synchronized.  Returns info."""
    m, n = A.shape
    nrhs = B.shape[1]
    a, lda = _host_colmajor(A)
    b, ldb = _host_colmajor(B)
    x, ldx = _host_colmajor(X)
    _bind_stream()
    if work is None:
        work = torch.empty(max(host_refine_workspace(m, n, nrhs), 1), dtype=torch.float64, device=device)
    info = RefineInfo()
    lw = C.c_size_t(work.numel())
    _check("gels_refine_host", lib().rnpgpu_dsgels_host(m, n, nrhs, a, lda, b, ldb, x, ldx, int(max_iter), (1 if forward else 0) | (2 if rank32 else 0), C.byref(info), C.byref(lw), work.data_ptr()))
    return info.as_dict()


def residual(A, X, B, R=None, normal=False, work=None):
    """R = B - A X (and G = A^T R when normal=True) for FP64 A (m x n), X
    (n x nrhs), B (m x nrhs), computed from exact fixed-point slices on the
    tensor cores.  Returns R, or (R, G)."""
    m, n = A.shape
    nrhs = B.shape[1]
    if R is None:
        R = empty_colmajor(m, nrhs, torch.float64, A.device)
    G = empty_colmajor(n, nrhs, torch.float64, A.device) if normal else None
    a, lda = colmajor(A)
    x, ldx = colmajor(X)
    b, ldb = colmajor(B)
    r, ldr = colmajor(R)
    g, ldg = colmajor(G) if normal else (None, max(n, 1))
    fn = lib().rnpgpu_dls_residual
    _bind_stream()
    if work is None:
        lw = C.c_size_t(0)
        _check("dls_residual", fn(m, n, nrhs, a, lda, x, ldx, b, ldb, r, ldr, g, ldg, None, C.byref(lw)))
        work = torch.empty(max(lw.value, 1), dtype=torch.uint8, device=A.device)
    lw = C.c_size_t(work.numel())
    _check("dls_residual", fn(m, n, nrhs, a, lda, x, ldx, b, ldb, r, ldr, g, ldg, work.data_ptr(), C.byref(lw)))
    return (R, G) if normal else R
