"""Shared parity checks for the QR path (norms and tolerances).

Tolerances, in the terms the parity contract states them:
  * R equal to the reference's R within 1e-12 relative (Frobenius) for FP64,
  * ||A - QR|| / (||A|| n eps) <= 10 and ||Q^H Q - I|| / (n eps) <= 10,
  * FP32 types: R within 1e-4 relative (single precision, FP64 norms/beta).
"""
import numpy as np

EPS = {"s": np.finfo(np.float32).eps, "c": np.finfo(np.float32).eps, "d": np.finfo(np.float64).eps, "z": np.finfo(np.float64).eps}
R_TOL = {"d": 1e-12, "z": 1e-12, "s": 1e-4, "c": 1e-4}
V_TOL = {"d": 1e-10, "z": 1e-10, "s": 1e-3, "c": 1e-3}
RESID_TOL = 10.0


def fnorm(x):
    """Frobenius norm without overflow/underflow (scaled by the max entry)."""
    x = np.asarray(x)
    if x.size == 0:
        return 0.0
    s = np.max(np.abs(x))
    if s == 0 or not np.isfinite(s):
        return float(s)
    return float(s * np.linalg.norm(x / s))


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    s = max(np.max(np.abs(a), initial=0.0), np.max(np.abs(b), initial=0.0))
    if s == 0:
        return 0.0
    nb = fnorm(b / s)
    d = fnorm(a / s - b / s)
    if nb == 0:
        return d
    return d / nb


def split_factor(fac, m, n):
    """(R, V below the diagonal) of a factored m x n array."""
    k = min(m, n)
    f = fac[:m, :n]
    return np.triu(f)[:k, :], np.tril(f, -1)[:, :k]


def q_explicit(fac, tau, m, n):
    """Q (m x m) from reflectors, in numpy (H_0 H_1 ... H_{k-1})."""
    k = min(m, n)
    Q = np.eye(m, dtype=fac.dtype)
    for i in reversed(range(k)):
        v = np.zeros(m, dtype=fac.dtype)
        v[i] = 1
        v[i + 1:] = fac[i + 1:m, i]
        Q = Q - tau[i] * np.outer(v, v.conj() @ Q)
    return Q


def factor_residuals(a, fac, tau, m, n):
    """(||A - QR||_1 / (||A||_1 n eps), ||Q^H Q - I||_1 / (k eps)) with Q built
    from the reflectors in FP64/complex128; the orthogonality is measured on
    the k = min(m, n) columns GenerateQ would form (the full m x m Q's
    1-norm grows with m: the reference's own factors score 12 on it for a
    33 x 1 matrix)."""
    p = {np.dtype(np.float32): "s", np.dtype(np.float64): "d", np.dtype(np.complex64): "c", np.dtype(np.complex128): "z"}[np.dtype(fac.dtype)]
    hi = np.complex128 if np.iscomplexobj(fac) else np.float64
    A = a[:m, :n].astype(hi)
    F = fac.astype(hi)
    Q = q_explicit(F, tau.astype(hi), m, n)
    R = np.triu(F[:m, :n])
    eps = EPS[p]
    na = max(np.linalg.norm(A, 1), np.finfo(np.float64).tiny)
    r1 = np.linalg.norm(A - Q @ R, 1) / (na * max(n, 1) * eps)
    k = min(m, n)
    Qk = Q[:, :k]
    r2 = np.linalg.norm(Qk.conj().T @ Qk - np.eye(k), 1) / (max(k, 1) * eps)
    return r1, r2
