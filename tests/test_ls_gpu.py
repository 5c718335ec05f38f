"""Least squares on the GPU: the plain form against the reference's golden LS
solution and the oracle; the mixed form (FP32 factor + FP64 refinement)
against the FP64 oracle, with the backward-error bound 10 n eps."""
import numpy as np
import pytest

from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import ls as gls  # noqa: E402

NP = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def from_dev(t):
    return np.asfortranarray(t.t().cpu().numpy().T)


def mat(oracle, p, m, n, seed, dist=2):
    # drawn in double precision and rounded: the reference's single-precision
    # normal generator can return inf when 1 - u rounds to 1 (RNP/Random.hpp:172-180)
    q = {"s": "d", "c": "z"}.get(p, p)
    v, _ = oracle.larnv(q, dist, seed, m * n)
    return np.asfortranarray(v.astype(NP[p]).reshape(n, m).T)


@pytest.mark.parametrize("p", ["d", "z"])
def test_gels_matches_reference_golden(golden, oracle, p):
    c = golden.cases["ls_%s" % p]
    m, n, nrhs = int(c["m"]), int(c["n"]), int(c["nrhs"])
    A = mat(oracle, p, m, n, [3, 1, 4, 1])
    B = mat(oracle, p, m, nrhs, [2, 7, 1, 9])
    dA, dB = to_dev(A), to_dev(B)
    X = gls.gels(dA, dB)
    torch.cuda.synchronize()
    assert rel(X.cpu().numpy(), c["x"]) <= 1e-12


@pytest.mark.parametrize("p", ["s", "d", "c", "z"])
@pytest.mark.parametrize("mnr", [(500, 100, 3), (2000, 257, 16), (64, 64, 1)])
def test_gels_against_oracle(oracle, p, mnr):
    m, n, nrhs = mnr
    A = mat(oracle, p, m, n, [1, 9, 9, 7])
    B = mat(oracle, p, m, nrhs, [7, 9, 9, 1])
    Ao, Bo = A.copy(order="F"), B.copy(order="F")
    oracle.gels(p, m, n, nrhs, Ao, Bo)
    X = gls.gels(to_dev(A), to_dev(B))
    torch.cuda.synchronize()
    tol = 1e-10 if p in "dz" else 2e-3
    assert rel(X.cpu().numpy(), Bo[:n]) <= tol


@pytest.mark.parametrize("p", ["d", "z"])
def test_trsm_upper(oracle, p):
    n, nrhs = 300, 5
    # well conditioned: unit diagonal plus a small strictly upper part
    R = np.asfortranarray(np.eye(n) + np.triu(mat(oracle, p, n, n, [5, 5, 5, 5]), 1) / n)
    B = mat(oracle, p, n, nrhs, [6, 6, 6, 7])
    dB = to_dev(B)
    gls.trsm_upper(to_dev(R), dB)
    torch.cuda.synchronize()
    assert rel(R @ from_dev(dB), B) <= 1e-14


def conditioned(m, n, nrhs, cond, cplx, seed=0):
    rng = np.random.default_rng(seed)

    def gauss(*s):
        g = rng.standard_normal(s)
        return g + 1j * rng.standard_normal(s) if cplx else g

    U, _ = np.linalg.qr(gauss(m, n))
    V, _ = np.linalg.qr(gauss(n, n))
    s = cond ** (-np.arange(n) / (n - 1))
    A = np.asfortranarray((U * s) @ V.conj().T)
    b = np.asfortranarray(A @ gauss(n, nrhs) + 1e-10 * gauss(m, nrhs))
    return A, b


def ls_backward_error(A, b, x):
    """Karlson-Walden estimate of the normwise LS backward error (max over RHS)."""
    r = b - A @ x
    U, s, Vh = np.linalg.svd(A, full_matrices=False)
    out = 0.0
    for j in range(b.shape[1]):
        th = np.linalg.norm(r[:, j]) / np.linalg.norm(x[:, j])
        v = (Vh @ (A.conj().T @ r[:, j])) / np.sqrt(s ** 2 + th ** 2)
        out = max(out, np.linalg.norm(v) / np.linalg.norm(x[:, j]))
    return out


@pytest.mark.parametrize("forward", [False, True])
@pytest.mark.parametrize("cplx", [False, True])
def test_mixed_refinement_reaches_fp64(oracle, cplx, forward):
    m, n, nrhs = 4096, 256, 4
    A, b = conditioned(m, n, nrhs, 1e6, cplx)
    p = "z" if cplx else "d"
    Ao, bo = A.copy(order="F"), b.copy(order="F")
    oracle.gels(p, m, n, nrhs, Ao, bo)
    x_oracle = bo[:n]
    dA, db = to_dev(A), to_dev(b)
    X, info = gls.gels_refine(dA, db, forward=forward)
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    bound = 10 * n * np.finfo(np.float64).eps
    assert info["converged"] == 1, info
    assert info["backward_error"] <= bound and info["normal_residual"] <= bound
    # independent checks in numpy: the Karlson-Walden LS backward error
    # estimate and the normal-equation residual
    assert ls_backward_error(A, b, x) <= bound
    r = b - A @ x
    an = np.linalg.norm(A)
    eta = np.max(np.linalg.norm(A.conj().T @ r, axis=0) / (an * (an * np.linalg.norm(x, axis=0) + np.linalg.norm(b, axis=0))))
    assert eta <= bound
    ferr = rel(x, x_oracle)
    if forward:
        # FP64-level forward accuracy: within the FP64 oracle's own sensitivity
        assert ferr <= 1e6 * 1e-14, ferr
    else:
        # backward-error target only: the FP32 factor's Q leaves a forward
        # error of order cond * u32 * ||r|| / ||A x||
        assert ferr <= 1e-5, ferr
    # A and b untouched
    assert np.array_equal(from_dev(dA), A) and np.array_equal(from_dev(db), b)
