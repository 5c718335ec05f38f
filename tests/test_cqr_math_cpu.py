"""The algebra of the mixed solver's CholeskyQR2 panel (panel_cqr.cuh), in
float64 numpy on the CPU, in the order the kernel forms it: CholeskyQR2
(R1 from A^T A, Q1 = A R1^-1, R2 from Q1^T Q1), the LU without pivoting of
Q1_top - S R2 = L M with s_j = -sign of the j-th eliminated pivot (M = U R2),
V = L on the top block and Q1 M^-1 below it, T = -M R2^-1 S L1^-T and
R = S R2 R1, with narrow panels padded by zero columns and a unit Gram
diagonal.  The result must be a compact-WY Householder QR of the panel:
V unit lower trapezoidal, T upper triangular, I - V T V^T orthogonal, and its
first columns times R equal to the panel."""
import numpy as np
import pytest

NB = 32


def cqr_householder(A):
    m, n = A.shape
    Ap = np.zeros((m, NB))
    Ap[:, :n] = A
    G1 = Ap.T @ Ap
    G1[np.arange(n, NB), np.arange(n, NB)] = 1.0  # padding columns
    R1 = np.linalg.cholesky(G1).T
    Q1 = np.linalg.solve(R1.T, Ap.T).T
    G2 = Q1.T @ Q1
    G2[np.arange(n, NB), np.arange(n, NB)] = 1.0
    R2 = np.linalg.cholesky(G2).T
    # LU of Q1_top - S R2 by rows, the sign of each pivot chosen on the way
    E = Q1[:NB].copy()
    Mt = np.zeros((NB, NB))
    L = np.eye(NB)
    s = np.zeros(NB)
    for j in range(NB):
        s[j] = -1.0 if E[j, j] >= 0 else 1.0
        Mt[j, j:] = E[j, j:] - s[j] * R2[j, j:]
        for i in range(j + 1, NB):
            L[i, j] = E[i, j] / Mt[j, j]
            E[i, j + 1:] -= L[i, j] * Mt[j, j + 1:]
    V = np.zeros((m, NB))
    V[:NB] = L
    V[NB:] = np.linalg.solve(Mt.T, Q1[NB:].T).T  # x M = q1 below the top block
    P = np.linalg.inv(R2) @ np.diag(s) @ np.linalg.inv(L).T
    T = -Mt @ P
    R = np.diag(s) @ R2 @ R1
    return V[:, :n], T[:n, :n], R[:n, :n]


@pytest.mark.parametrize("mn", [(500, 32), (300, 20), (1000, 1), (64, 32), (200, 7)])
def test_reconstruction_is_a_householder_qr(mn):
    m, n = mn
    rng = np.random.default_rng(m * 31 + n)
    A = rng.standard_normal((m, n)) * np.exp2(rng.integers(-5, 5, size=n))[None, :]
    V, T, R = cqr_householder(A)
    assert np.allclose(np.triu(V[:n], 1), 0) and np.allclose(np.diag(V[:n]), 1)
    assert np.allclose(np.tril(T, -1), 0) and np.allclose(np.tril(R, -1), 0)
    H = np.eye(m) - V @ T @ V.T
    assert np.abs(H.T @ H - np.eye(m)).max() < 1e-12
    assert np.abs(H[:, :n] @ R - A).max() < 1e-12 * np.abs(A).max() * m
    # tau = diag(T): each reflector I - tau v v^T is orthogonal (tau = 2 / v^T v)
    tau = np.diag(T)
    assert np.allclose(tau * np.einsum("ij,ij->j", V, V), 2.0)


def test_sign_choice_keeps_the_pivots_away_from_zero():
    # a top block whose eliminated pivots are near zero: s_j = -sign(pivot)
    # makes |u_jj| >= 1, so the LU needs no pivoting
    m, n = 400, 32
    rng = np.random.default_rng(9)
    Q, _ = np.linalg.qr(rng.standard_normal((m, n)))
    Q[:n] *= 1e-3  # top block nearly zero
    A = Q @ np.triu(rng.standard_normal((n, n)) + 5 * np.eye(n))
    V, T, R = cqr_householder(A)
    H = np.eye(m) - V @ T @ V.T
    assert np.abs(H[:, :n] @ R - A).max() < 1e-10 * np.abs(A).max()
