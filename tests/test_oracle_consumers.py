"""The oracle's restatement of the reference's callers of QR / QL
(Hessenberg::MultQ / GenerateQ, Tridiagonal::MultQHerm / GenerateQHerm, the
generalized eigensystem's QR step; oracle/qr_oracle.cpp) against golden
vectors the reference itself produced (tests/golden/make_consumers_golden.py).
CPU only."""
import numpy as np
import pytest

from consumer_cases import TOL, fortran, kind, load
from qr_checks import rel

NAMES, CASES = load()


def check_q(q, c, p):
    if "q" in c:
        assert rel(q, c["q"]) <= TOL[p]
    else:
        assert rel(q[:, :8], c["q_head"]) <= TOL[p] and rel(q[:, -8:], c["q_tail"]) <= TOL[p]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_consumers_match_reference(oracle, name):
    c = CASES[name]
    p, n = str(c["p"]), int(c["n"])
    k = kind(name)
    if k == "hess":
        ilo, ihi = int(c["ilo"]), int(c["ihi"])
        red, tau = fortran(c["red"]), c["tau"]
        for side in "LR":
            for trans in "NC":
                x = fortran(c["c_%s" % side])
                oracle.unmhr(p, side, trans, x.shape[0], x.shape[1], ilo, ihi, red, tau, x)
                assert rel(x, c["mq_%s%s" % (side, trans)]) <= TOL[p], (side, trans)
        q = fortran(red)
        oracle.unghr(p, n, ilo, ihi, q, tau)
        check_q(q, c, p)
    elif k == "trid":
        uplo = str(c["uplo"])
        red, tau = fortran(c["red"]), c["tau"]
        for side in "LR":
            for trans in "NC":
                x = fortran(c["c_%s" % side])
                oracle.unmtr(p, side, uplo, trans, x.shape[0], x.shape[1], red, tau, x)
                assert rel(x, c["mq_%s%s" % (side, trans)]) <= TOL[p], (side, trans)
        q = fortran(red)
        oracle.ungtr(p, uplo, n, q, tau)
        check_q(q, c, p)
    else:
        ilo, ihi = int(c["ilo"]), int(c["ihi"])
        a, b = fortran(c["a_in"]), fortran(c["b_in"])
        vl = np.zeros((n, n), dtype=a.dtype, order="F") if int(c["want_vl"]) else None
        vr = np.zeros((n, n), dtype=a.dtype, order="F") if int(c["want_vr"]) else None
        tau = oracle.gg_triangularize_b(p, n, ilo, ihi, a, b, vl, vr)
        k = ihi - ilo  # tau entries past irows are workspace
        assert rel(a, c["a"]) <= TOL[p] and rel(b, c["b"]) <= TOL[p] and rel(tau[:k], c["tau"][:k]) <= TOL[p]
        if vl is not None:
            assert rel(vl, c["vl"]) <= TOL[p]
        if vr is not None:
            assert np.array_equal(vr, c["vr"])


def test_consumer_goldens_are_valid_reductions(oracle):
    """The fixtures mean what they say: each Q is unitary, and for the
    tridiagonal cases Q^H A Q = T(d, e) with A = X + X^H rebuilt from the
    reference's generator (restated bit-exactly by the oracle)."""
    for name in NAMES:
        c = CASES[name]
        if kind(name) not in ("hess", "trid") or "q" not in c:
            continue
        p = str(c["p"])
        q = c["q"].astype(np.complex128)
        n = q.shape[0]
        assert np.abs(q.conj().T @ q - np.eye(n)).max() <= 100 * TOL[p], name
        if kind(name) == "trid":
            gp = "z" if p == "c" else ("d" if p == "s" else p)
            vals, _ = oracle.larnv(gp, 2, [2, 7, 1, 8], n * n)
            x = vals.astype(c["q"].dtype).reshape(n, n).T.astype(np.complex128)
            a = x + x.conj().T
            t = np.diag(c["d"]) + np.diag(c["e"], 1) + np.diag(c["e"], -1)
            assert np.abs(q.conj().T @ a @ q - t).max() <= 1000 * TOL[p] * np.abs(a).max(), name
