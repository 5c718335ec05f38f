"""LQ, QL and RQ on the GPU through the C ABI (include/rnp_gpu/lqr_gb300.h):
against the reference's own outputs (tests/golden/lqr_golden.npz) at the
reference tests' sizes and past the blocking crossover, and against the
oracle with residual checks at larger sizes."""
import numpy as np
import pytest

from lqr_cases import TOL, case_input, genq_ok, load, reflectors, tri
from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import lqr  # noqa: E402

NAMES, CASES = load()


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def from_dev(t):
    return np.asfortranarray(t.t().cpu().numpy().T)


@pytest.mark.parametrize("name", NAMES)
def test_lqr_matches_reference_golden(oracle, name):
    c = CASES[name]
    kind, p, m, n = str(c["kind"]), str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    a = case_input(oracle, c)
    dA = to_dev(a)
    tau = lqr.factor(kind, dA)
    torch.cuda.synchronize()
    f = from_dev(dA)
    tg = tau.cpu().numpy()[:k]
    assert np.max(np.abs(tg - c["tau"])) <= 10 * TOL[p]
    if "fac" in c:
        assert rel(f, c["fac"]) <= TOL[p]
    if "tri" in c:
        assert rel(tri(kind, f, m, n), c["tri"]) <= TOL[p]
    if "c_L" in c:
        V = to_dev(reflectors(kind, f, m, n))
        for side in "LR":
            for trans in "NC":
                dC = to_dev(c["c_%s" % side])
                lqr.mult_q(kind, side, trans, V, tau, dC, k)
                torch.cuda.synchronize()
                assert rel(from_dev(dC), c["mq_%s%s" % (side, trans)]) <= TOL[p], (side, trans)
    if genq_ok(kind, m, n) and ("q" in c or "q_head" in c):
        dQ = to_dev(f)
        lqr.generate_q(kind, dQ, tau, k)
        torch.cuda.synchronize()
        q = from_dev(dQ)
        if "q" in c:
            assert rel(q, c["q"]) <= TOL[p]
        else:
            assert rel(q[:, :8], c["q_head"]) <= TOL[p] and rel(q[:, -8:], c["q_tail"]) <= TOL[p]


@pytest.mark.parametrize("kind", ["lq", "ql", "rq"])
@pytest.mark.parametrize("p", ["d", "z", "s"])
@pytest.mark.parametrize("mn", [(1000, 700), (700, 1000), (64, 2000)])
def test_lqr_against_oracle_and_residuals(oracle, kind, p, mn):
    m, n = mn
    k = min(m, n)
    rng = np.random.default_rng(m + 3 * n)
    dt = {"d": np.float64, "z": np.complex128, "s": np.float32}[p]
    a = rng.standard_normal((m, n)) + (1j * rng.standard_normal((m, n)) if p == "z" else 0)
    a = np.asfortranarray(a.astype(dt))
    fo = a.copy(order="F")
    to = oracle.xgeqrf(kind, p, m, n, fo)
    dA = to_dev(a)
    tau = lqr.factor(kind, dA)
    torch.cuda.synchronize()
    f = from_dev(dA)
    tol = TOL[p] if p != "s" else 2e-4
    assert rel(tri(kind, f, m, n), tri(kind, fo, m, n)) <= tol
    assert np.max(np.abs(tau.cpu().numpy()[:k] - to)) <= 10 * tol
    # the triangular factor, padded to m x n, times Q reproduces A:
    # A = L Q (lq), Q L (ql), R Q (rq)
    Tpad = np.zeros((m, n), dtype=dt)
    if kind == "lq":
        Tpad[:, :k] = np.tril(f[:, :k])
    elif kind == "ql":
        Tpad[m - k:, :] = np.tril(f[m - k:, :], n - k)
    else:
        Tpad[:, n - k:] = np.triu(f[:, n - k:], -(m - k))
    dC = to_dev(Tpad)
    lqr.mult_q(kind, "L" if kind == "ql" else "R", "N", to_dev(reflectors(kind, f, m, n)), tau, dC, k)
    torch.cuda.synchronize()
    res = np.linalg.norm(from_dev(dC) - a) / (np.linalg.norm(a) * max(m, n) * np.finfo(dt).eps)
    assert res <= 10, res
