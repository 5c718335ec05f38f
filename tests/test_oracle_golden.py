"""The CPU oracle (oracle/qr_oracle.cpp) pinned against golden vectors that the
reference itself produced (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import golden_input
from qr_checks import R_TOL, V_TOL, rel, split_factor

DTYPES = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}


@pytest.mark.parametrize("p", ["s", "d", "z"])
@pytest.mark.parametrize("dist", [0, 1, 2])
def test_generator_bit_exact(golden, oracle, p, dist):
    c = golden.cases["rng_%s_%d" % (p, dist)]
    x, seed = oracle.larnv(p, dist, [1, 2, 3, 5], 300)
    assert np.array_equal(x, c["x"])
    assert seed == [int(s) for s in c["seed_out"]]


def _cases(golden):
    return golden.qr_cases()


def pytest_generate_tests(metafunc):
    if "qr_case" in metafunc.fixturenames:
        from conftest import GOLDEN, Golden

        metafunc.parametrize("qr_case", Golden(GOLDEN).qr_cases())


def test_factor_matches_reference(golden, oracle, qr_case):
    c = golden.cases[qr_case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    a = golden_input(c, oracle)
    fac = a.copy(order="F")
    tau = oracle.geqrf(p, m, n, fac)
    k = min(m, n)
    if "fac" in c:
        R, V = split_factor(fac, m, n)
        Rg, Vg = split_factor(c["fac"], m, n)
        assert rel(R, Rg) <= R_TOL[p]
        assert rel(V, Vg) <= V_TOL[p]
        # entries outside the m x n matrix (lda > m) are untouched
        assert np.array_equal(fac[m:, :n], a[m:, :n])
    else:
        Rg = np.zeros((k, n), dtype=fac.dtype)
        Rg[np.triu_indices(k, 0, n)] = c["r_packed"]
        assert rel(np.triu(fac[:k, :n]), Rg) <= R_TOL[p]
    assert np.max(np.abs(tau - c["tau"]), initial=0) <= 10 * R_TOL[p]


def test_factor_unblocked_matches_reference(golden, oracle, qr_case):
    c = golden.cases[qr_case]
    if "fac_unblocked" not in c:
        pytest.skip("no unblocked golden for this case")
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    fac = golden_input(c, oracle)
    tau = oracle.geqr2(p, m, n, fac)
    R, V = split_factor(fac, m, n)
    Rg, Vg = split_factor(c["fac_unblocked"], m, n)
    assert rel(R, Rg) <= R_TOL[p]
    assert rel(V, Vg) <= V_TOL[p]
    assert np.max(np.abs(tau - c["tau_unblocked"]), initial=0) <= 10 * R_TOL[p]


def test_generate_q_matches_reference(golden, oracle, qr_case):
    c = golden.cases[qr_case]
    if "q" not in c and "q_head" not in c:
        pytest.skip("no Q golden for this case")
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    nq = n if m >= n else m
    fac = golden_input(c, oracle)
    tau = oracle.geqrf(p, m, n, fac)
    for blocked, key in ((True, "q"), (False, "q_unblocked")):
        if key not in c and not (blocked and "q_head" in c):
            continue
        q = np.asfortranarray(fac[:, :nq].copy())
        oracle.ungqr(p, m, nq, k, q, tau, blocked=blocked)
        if key in c:
            assert rel(q[:m, :], c[key]) <= R_TOL[p]
        else:
            assert rel(q[:m, :16], c["q_head"]) <= R_TOL[p]
            assert rel(q[:m, -16:], c["q_tail"]) <= R_TOL[p]


def test_mult_q_matches_reference(golden, oracle, qr_case):
    c = golden.cases[qr_case]
    if "c_left" not in c:
        pytest.skip("no MultQ golden for this case")
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    fac = golden_input(c, oracle)
    tau = oracle.geqrf(p, m, n, fac)
    for side, c0 in (("L", c["c_left"]), ("R", c["c_right"])):
        cm, cn = c0.shape
        for trans in ("N", "C"):
            for blocked in (True, False):
                key = "mq_%s%s%s" % (side, trans, "" if blocked else "_unblocked")
                x = np.asfortranarray(c0.copy())
                oracle.unmqr(p, side, trans, cm, cn, k, fac, tau, x, blocked)
                assert rel(x, c[key]) <= R_TOL[p], key


@pytest.mark.parametrize("p", ["d", "z"])
def test_least_squares_matches_reference(golden, oracle, p):
    c = golden.cases["ls_%s" % p]
    m, n, nrhs = int(c["m"]), int(c["n"]), int(c["nrhs"])
    a, _ = oracle.larnv(p, 2, [3, 1, 4, 1], m * n)
    b, _ = oracle.larnv(p, 2, [2, 7, 1, 9], m * nrhs)
    A = np.asfortranarray(a.reshape(n, m).T)
    B = np.asfortranarray(b.reshape(nrhs, m).T)
    assert A.sum() == c["a_sum"] and B.sum() == c["b_sum"]
    oracle.gels(p, m, n, nrhs, A, B)
    assert rel(B[:n, :], c["x"]) <= 1e-12


def test_reference_outputs_meet_residual_contract(golden, oracle, qr_case):
    """The residual metrics the GPU is held to, applied to the reference's own
    factors: they must pass there too, or the metric is unfair."""
    from qr_checks import RESID_TOL, factor_residuals

    c = golden.cases[qr_case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    if "fac" not in c or m * n > 300 * 300:
        pytest.skip("small factored cases only")
    a = golden_input(c, oracle)
    if not np.isfinite(c["fac"]).all():
        pytest.skip("non-finite")
    r1, r2 = factor_residuals(a, c["fac"], c["tau"], m, n)
    assert r1 <= RESID_TOL and r2 <= RESID_TOL


def test_blas_routed_oracle_matches_reference(golden, oracle_blas, qr_case):
    """The restatement with its level-2/3 calls through OpenBLAS (how the
    full-size checks and the CPU baseline run it, and how the reference runs)
    against the same golden vectors: Factor, and MultQ where it has goldens."""
    c = golden.cases[qr_case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    a = golden_input(c, oracle_blas)
    fac = a.copy(order="F")
    tau = oracle_blas.geqrf(p, m, n, fac)
    if "fac" in c:
        R, V = split_factor(fac, m, n)
        Rg, Vg = split_factor(c["fac"], m, n)
        assert rel(R, Rg) <= R_TOL[p]
        assert rel(V, Vg) <= V_TOL[p]
    else:
        Rg = np.zeros((k, n), dtype=fac.dtype)
        Rg[np.triu_indices(k, 0, n)] = c["r_packed"]
        assert rel(np.triu(fac[:k, :n]), Rg) <= R_TOL[p]
    assert np.max(np.abs(tau - c["tau"]), initial=0) <= 10 * R_TOL[p]
    if "c_left" in c:
        for side, c0 in (("L", c["c_left"]), ("R", c["c_right"])):
            cm, cn = c0.shape
            for trans in ("N", "C"):
                x = np.asfortranarray(c0.copy())
                oracle_blas.unmqr(p, side, trans, cm, cn, k, fac, tau, x, True)
                assert rel(x, c["mq_%s%s" % (side, trans)]) <= R_TOL[p]


@pytest.mark.parametrize("p", ["d", "z"])
def test_blas_routed_least_squares_matches_reference(golden, oracle_blas, p):
    c = golden.cases["ls_%s" % p]
    m, n, nrhs = int(c["m"]), int(c["n"]), int(c["nrhs"])
    a, _ = oracle_blas.larnv(p, 2, [3, 1, 4, 1], m * n)
    b, _ = oracle_blas.larnv(p, 2, [2, 7, 1, 9], m * nrhs)
    A = np.asfortranarray(a.reshape(n, m).T)
    B = np.asfortranarray(b.reshape(nrhs, m).T)
    oracle_blas.gels(p, m, n, nrhs, A, B)
    assert rel(B[:n, :], c["x"]) <= 1e-12
