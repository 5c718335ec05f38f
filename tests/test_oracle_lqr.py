"""The oracle's LQ, QL and RQ (restated through the QR of a transformed
matrix, oracle/qr_oracle.cpp) against golden vectors the reference itself
produced (tests/golden/make_lqr_golden.py).  CPU only."""
import numpy as np
import pytest

from lqr_cases import TOL, case_input, genq_ok, load, reflectors, tri
from qr_checks import rel

NAMES, CASES = load()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_lqr_matches_reference(oracle, name):
    c = CASES[name]
    kind, p, m, n = str(c["kind"]), str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    f = case_input(oracle, c)
    tau = oracle.xgeqrf(kind, p, m, n, f)
    assert np.max(np.abs(tau - c["tau"])) <= 10 * TOL[p]
    if "fac" in c:
        assert rel(f, c["fac"]) <= TOL[p]
    if "tri" in c:
        assert rel(tri(kind, f, m, n), c["tri"]) <= TOL[p]
    if "c_L" in c:
        refl = reflectors(kind, f, m, n)
        for side in "LR":
            for trans in "NC":
                x = np.asfortranarray(c["c_%s" % side].copy())
                oracle.xunmqr(kind, p, side, trans, x.shape[0], x.shape[1], k, refl, tau, x)
                assert rel(x, c["mq_%s%s" % (side, trans)]) <= TOL[p], (side, trans)
    if genq_ok(kind, m, n) and ("q" in c or "q_head" in c):
        q = np.asfortranarray(f.copy())
        oracle.xungqr(kind, p, m, n, k, q, tau)
        if "q" in c:
            assert rel(q, c["q"]) <= TOL[p]
        else:
            assert rel(q[:, :8], c["q_head"]) <= TOL[p] and rel(q[:, -8:], c["q_tail"]) <= TOL[p]
