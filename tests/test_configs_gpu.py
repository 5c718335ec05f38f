"""Parity at the full sizes of two benchmark configurations.

  * 4096 x 4096 complex<double> Factor (re, im iid N(0,1)) followed by
    MultQ("L","C") on a 4096 x 64 block: R, tau and Q^H C against the oracle
    within 1e-12 relative;
  * 65536 x 512 real least squares with 16 right-hand sides, A = U diag(s) V^T
    with s geometric from 1 to 1e-6 (condition 1e6), b = A x + 1e-10 N(0,1):
    the plain FP64 solve against the oracle's solution, and the mixed solve
    (FP32 factor, FP64 refinement) to an LS backward error of 10 n eps by an
    independent Karlson-Walden estimate, in both refinement modes.

The oracle runs with its BLAS calls through OpenBLAS (the reference forwards
the same calls to its BLAS); its plain loops would take minutes here.
"""
import numpy as np
import pytest

from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import ls as gls  # noqa: E402
from rnp2_gb300 import qr as gq  # noqa: E402


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def test_complex_4096_factor_and_multq_match_the_oracle(oracle_blas):
    n, nc = 4096, 64
    v, _ = oracle_blas.larnv("z", 2, [4, 0, 9, 6], n * n)
    A = np.asfortranarray(v.reshape(n, n).T)
    v, _ = oracle_blas.larnv("z", 2, [6, 4, 0, 1], n * nc)
    Cm = np.asfortranarray(v.reshape(nc, n).T)
    dA, dC = to_dev(A), to_dev(Cm)
    tau = gq.factor(dA)
    gq.mult_q("L", "C", dA, tau, dC, n)
    torch.cuda.synchronize()
    Ao, Co = A.copy(order="F"), Cm.copy(order="F")
    to = oracle_blas.geqrf("z", n, n, Ao)
    oracle_blas.unmqr("z", "L", "C", n, nc, n, Ao, to, Co)
    fa = dA.t().cpu().numpy().T
    assert rel(np.triu(fa), np.triu(Ao)) <= 1e-12
    assert np.max(np.abs(tau.cpu().numpy() - to)) <= 1e-12
    assert rel(dC.t().cpu().numpy().T, Co) <= 1e-12


M, N, NRHS = 65536, 512, 16
BOUND = 10 * N * np.finfo(np.float64).eps


@pytest.fixture(scope="module")
def c3_problem():
    rng = np.random.default_rng(2024)
    U, _ = np.linalg.qr(rng.standard_normal((M, N)))
    V, _ = np.linalg.qr(rng.standard_normal((N, N)))
    s = 10.0 ** (-6.0 * np.arange(N) / (N - 1))
    A = np.asfortranarray((U * s) @ V.T)
    b = np.asfortranarray(A @ rng.standard_normal((N, NRHS)) + 1e-10 * rng.standard_normal((M, NRHS)))
    return A, b


@pytest.fixture(scope="module")
def c3_oracle(c3_problem):
    import oracle as orc

    o = orc.load()
    blas = orc.find_openblas()
    if not blas or orc.use_blas(o, blas, "scipy_", 0) != 0:
        pytest.skip("no OpenBLAS for the oracle")
    try:
        A, b = c3_problem
        Ao, bo = A.copy(order="F"), b.copy(order="F")
        o.gels("d", M, N, NRHS, Ao, bo)
    finally:
        orc.use_blas(o, None)
    return bo[:N].copy(), np.triu(Ao[:N, :N])


def kw_estimate(A, b, x, R):
    """Karlson-Walden estimate of the LS backward error (max over RHS), with
    A^T A = R^T R from the oracle's FP64 factor."""
    r = b - A @ x
    g = A.T @ r
    _, s, vh = np.linalg.svd(R)
    out = 0.0
    for j in range(b.shape[1]):
        th = np.linalg.norm(r[:, j]) / np.linalg.norm(x[:, j])
        out = max(out, np.linalg.norm((vh @ g[:, j]) / np.sqrt(s * s + th * th)) / np.linalg.norm(x[:, j]))
    return out


def test_plain_fp64_ls_65536x512_matches_the_oracle(c3_problem, c3_oracle):
    A, b = c3_problem
    x_o, R_o = c3_oracle
    dA, db = to_dev(A), to_dev(b)
    X = gls.gels(dA, db)
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    # two backward-stable FP64 solvers agree to about cond * eps = 1.1e-10
    assert rel(x, x_o) <= 1e-9
    assert kw_estimate(A, b, x, R_o) <= BOUND
    R = np.triu(dA[:N, :N].cpu().numpy())
    assert rel(R, R_o) <= 1e-12


@pytest.mark.parametrize("forward", [False, True])
def test_mixed_ls_65536x512_reaches_fp64_backward_error(c3_problem, c3_oracle, forward):
    A, b = c3_problem
    x_o, R_o = c3_oracle
    X, info = gls.gels_refine(to_dev(A), to_dev(b), forward=forward)
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    assert info["converged"] == 1, info
    assert info["backward_error"] <= BOUND and info["normal_residual"] <= BOUND
    assert kw_estimate(A, b, x, R_o) <= BOUND
    if forward:
        # FP64 forward accuracy: as close to the oracle as the plain FP64 solve
        assert rel(x, x_o) <= 1e-9
    else:
        # the backward-error target only; the FP32 factor's Q leaves a forward
        # error of order cond * u32 * (its sensitivity)
        assert rel(x, x_o) <= 1e-5
