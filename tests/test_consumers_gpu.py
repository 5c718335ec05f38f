"""The reference's callers of QR / QL on the GPU through the C ABI
(include/rnp_gpu/consumers_gb300.h): Hessenberg::MultQ / GenerateQ,
Tridiagonal::MultQHerm / GenerateQHerm and the generalized eigensystem's QR
step, against the reference's own outputs (tests/golden/consumers_golden.npz)
and, at larger sizes, against the oracle on reflector sets made by the
oracle's QR / QL (the storage these routines read is the QR / QL storage of a
sub-block)."""
import numpy as np
import pytest

from consumer_cases import DT, TOL, fortran, kind, load
from qr_checks import rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import consumers  # noqa: E402

NAMES, CASES = load()


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda().t()


def from_dev(t):
    return np.asfortranarray(t.t().cpu().numpy().T)


def tau_dev(t):
    return torch.from_numpy(np.ascontiguousarray(t)).cuda()


def check_q(q, c, p):
    if "q" in c:
        assert rel(q, c["q"]) <= TOL[p]
    else:
        assert rel(q[:, :8], c["q_head"]) <= TOL[p] and rel(q[:, -8:], c["q_tail"]) <= TOL[p]


@pytest.mark.parametrize("name", NAMES)
def test_consumers_match_reference_golden(name):
    c = CASES[name]
    p, n = str(c["p"]), int(c["n"])
    k = kind(name)
    if k in ("hess", "trid"):
        dA = to_dev(c["red"])
        t = tau_dev(c["tau"]) if c["tau"].size else tau_dev(np.zeros(1, dtype=DT[p]))
        for side in "LR":
            for trans in "NC":
                dC = to_dev(c["c_%s" % side])
                if k == "hess":
                    consumers.hessenberg_mult_q(side, trans, int(c["ilo"]), int(c["ihi"]), dA, t, dC)
                else:
                    consumers.tridiagonal_mult_q(side, str(c["uplo"]), trans, dA, t, dC)
                torch.cuda.synchronize()
                assert rel(from_dev(dC), c["mq_%s%s" % (side, trans)]) <= TOL[p], (side, trans)
        if k == "hess":
            consumers.hessenberg_generate_q(int(c["ilo"]), int(c["ihi"]), dA, t)
        else:
            consumers.tridiagonal_generate_q(str(c["uplo"]), dA, t)
        torch.cuda.synchronize()
        check_q(from_dev(dA), c, p)
    else:
        dA, dB = to_dev(c["a_in"]), to_dev(c["b_in"])
        dVL = to_dev(np.full((n, n), 3.0, dtype=DT[p])) if int(c["want_vl"]) else None
        dVR = to_dev(np.full((n, n), 3.0, dtype=DT[p])) if int(c["want_vr"]) else None
        tau = consumers.generalized_triangularize_b(int(c["ilo"]), int(c["ihi"]), dA, dB, dVL, dVR)
        torch.cuda.synchronize()
        assert rel(from_dev(dA), c["a"]) <= TOL[p]
        assert rel(from_dev(dB), c["b"]) <= TOL[p]
        k = int(c["ihi"]) - int(c["ilo"])  # entries past irows are workspace, set by neither
        assert rel(tau.cpu().numpy()[:k], c["tau"][:k]) <= TOL[p]
        if dVL is not None:
            assert rel(from_dev(dVL), c["vl"]) <= TOL[p]
        if dVR is not None:
            assert np.array_equal(from_dev(dVR), c["vr"])


def rand(rng, shape, p):
    x = rng.standard_normal(shape)
    if p in "cz":
        x = x + 1j * rng.standard_normal(shape)
    return np.asfortranarray(x.astype(DT[p]))


def hess_input(oracle, rng, p, n, ilo, ihi):
    """A Hessenberg reduction's storage: the QR reflectors of a random
    nh x nh block below the subdiagonal of columns ilo .. ihi-2."""
    red = rand(rng, (n, n), p)
    nh = ihi - ilo - 1
    tau = np.zeros(max(n - 1, 1), dtype=DT[p])
    if nh > 0:
        blk = rand(rng, (nh, nh), p)
        tau[ilo:ihi - 1] = oracle.geqrf(p, nh, nh, blk)
        red[ilo + 1:ihi, ilo:ihi - 1] = blk
    return red, tau


def trid_input(oracle, rng, p, n, uplo):
    """A tridiagonal reduction's storage: QL reflectors of a random
    (n-1) x (n-1) block in columns 1.. ("U"), or QR reflectors in rows 1..
    ("L")."""
    red = rand(rng, (n, n), p)
    blk = rand(rng, (n - 1, n - 1), p)
    if uplo == "U":
        tau = oracle.xgeqrf("ql", p, n - 1, n - 1, blk)
        red[: n - 1, 1:] = blk
    else:
        tau = oracle.geqrf(p, n - 1, n - 1, blk)
        red[1:, : n - 1] = blk
    return red, np.ascontiguousarray(tau)


@pytest.mark.parametrize("p,n,ilo,ihi", [("d", 600, 10, 580), ("z", 400, 0, 400), ("s", 300, 5, 290), ("c", 257, 1, 256), ("d", 130, 0, 130), ("d", 50, 20, 21)])
def test_hessenberg_against_oracle(oracle, p, n, ilo, ihi):
    rng = np.random.default_rng(n + ilo)
    red, tau = hess_input(oracle, rng, p, n, ilo, ihi)
    dA, t = to_dev(red), tau_dev(tau)
    for side, shape in (("L", (n, 24)), ("R", (70, n))):
        for trans in "NC":
            c0 = rand(rng, shape, p)
            x = c0.copy(order="F")
            oracle.unmhr(p, side, trans, shape[0], shape[1], ilo, ihi, red, tau, x)
            dC = to_dev(c0)
            consumers.hessenberg_mult_q(side, trans, ilo, ihi, dA, t, dC)
            torch.cuda.synchronize()
            assert rel(from_dev(dC), x) <= TOL[p], (side, trans)
    q = red.copy(order="F")
    oracle.unghr(p, n, ilo, ihi, q, tau)
    consumers.hessenberg_generate_q(ilo, ihi, dA, t)
    torch.cuda.synchronize()
    qg = from_dev(dA)
    assert rel(qg, q) <= TOL[p]
    assert np.abs(qg.conj().T @ qg - np.eye(n)).max() <= 50 * n * np.finfo(DT[p]).eps


@pytest.mark.parametrize("p,n,uplo", [("d", 500, "U"), ("d", 500, "L"), ("z", 300, "U"), ("z", 300, "L"), ("s", 200, "L"), ("c", 160, "U"), ("d", 2, "U"), ("d", 1, "L")])
def test_tridiagonal_against_oracle(oracle, p, n, uplo):
    rng = np.random.default_rng(n + (uplo == "U"))
    if n > 1:
        red, tau = trid_input(oracle, rng, p, n, uplo)
    else:
        red, tau = rand(rng, (1, 1), p), np.zeros(1, dtype=DT[p])
    dA, t = to_dev(red), tau_dev(tau)
    for side, shape in (("L", (n, 17)), ("R", (33, n))):
        for trans in "NC":
            c0 = rand(rng, shape, p)
            x = c0.copy(order="F")
            oracle.unmtr(p, side, uplo, trans, shape[0], shape[1], red, tau, x)
            dC = to_dev(c0)
            consumers.tridiagonal_mult_q(side, uplo, trans, dA, t, dC)
            torch.cuda.synchronize()
            assert rel(from_dev(dC), x) <= TOL[p], (side, trans)
    q = red.copy(order="F")
    oracle.ungtr(p, uplo, n, q, tau)
    consumers.tridiagonal_generate_q(uplo, dA, t)
    torch.cuda.synchronize()
    assert rel(from_dev(dA), q) <= TOL[p]


@pytest.mark.parametrize("p,n,ilo,ihi,vl,vr", [("z", 300, 7, 290, 1, 1), ("c", 200, 0, 200, 1, 0), ("z", 129, 3, 100, 0, 0), ("z", 64, 0, 1, 1, 1)])
def test_generalized_step_against_oracle(oracle, p, n, ilo, ihi, vl, vr):
    rng = np.random.default_rng(n)
    a, b = rand(rng, (n, n), p), rand(rng, (n, n), p)
    ao, bo = a.copy(order="F"), b.copy(order="F")
    vlo = np.zeros((n, n), dtype=DT[p], order="F") if vl else None
    vro = np.zeros((n, n), dtype=DT[p], order="F") if vr else None
    tau_o = oracle.gg_triangularize_b(p, n, ilo, ihi, ao, bo, vlo, vro)
    dA, dB = to_dev(a), to_dev(b)
    dVL = to_dev(np.full((n, n), 5.0, dtype=DT[p])) if vl else None
    dVR = to_dev(np.full((n, n), 5.0, dtype=DT[p])) if vr else None
    tau = consumers.generalized_triangularize_b(ilo, ihi, dA, dB, dVL, dVR)
    torch.cuda.synchronize()
    assert rel(tau.cpu().numpy()[: ihi - ilo], tau_o[: ihi - ilo]) <= TOL[p]
    assert rel(from_dev(dA), ao) <= TOL[p] and rel(from_dev(dB), bo) <= TOL[p]
    if vl:
        assert rel(from_dev(dVL), vlo) <= TOL[p]
    if vr:
        assert np.array_equal(from_dev(dVR), vro)


def test_tau_and_work_share_one_buffer():
    """The generalized step returns tau in the first n workspace entries, as
    the reference's [tau | work] layout (GeneralizedEigensystems.hpp:377-381)."""
    rng = np.random.default_rng(5)
    n = 96
    a, b = rand(rng, (n, n), "z"), rand(rng, (n, n), "z")
    dA, dB = to_dev(a), to_dev(b)
    import ctypes as C

    from rnp2_gb300._capi import lib

    f = lib().rnpgpu_zgg_triangularize_b
    lw = C.c_size_t(0)
    assert f(n, 0, n, dA.data_ptr(), n, dB.data_ptr(), n, None, 1, None, 1, C.byref(lw), None) == 0
    work = torch.full((lw.value,), float("nan"), dtype=torch.complex128, device="cuda")
    lw2 = C.c_size_t(work.numel())
    assert f(n, 0, n, dA.data_ptr(), n, dB.data_ptr(), n, None, 1, None, 1, C.byref(lw2), work.data_ptr()) == 0
    torch.cuda.synchronize()
    tau = work[:n].cpu().numpy()
    assert np.all(np.isfinite(tau))
    r = np.triu(from_dev(dB))
    assert np.allclose(np.abs(np.diag(r)), np.abs(np.diag(np.linalg.qr(b)[1])), rtol=1e-10)
