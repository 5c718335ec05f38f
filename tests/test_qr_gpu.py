"""Parity of the GB300 QR path with the reference, on the GPU.

Each golden case (produced by the reference itself) is run through the C ABI
(via rnp2_gb300.qr) and compared with the reference's R, V, tau, Q and MultQ
results; the factorization residuals are checked against the contract's
thresholds; sizes without golden vectors are compared with the oracle.
"""
import numpy as np
import pytest

from conftest import GOLDEN, Golden, golden_input
from qr_checks import EPS, R_TOL, RESID_TOL, V_TOL, factor_residuals, rel, split_factor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import qr as gq  # noqa: E402

TORCH = {"s": torch.float32, "d": torch.float64, "c": torch.complex64, "z": torch.complex128}
NP = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}
_G = Golden(GOLDEN)


def to_dev(a):
    """Fortran numpy (ld, cols) -> column-major CUDA tensor (ld, cols)."""
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


def from_dev(t):
    return np.asfortranarray(t.t().cpu().numpy().T)


def run_factor(a, p, m, n, unblocked=False):
    d = to_dev(a)
    A = d[:m, :n]
    tau = gq.factor_unblocked(A) if unblocked else gq.factor(A)
    torch.cuda.synchronize()
    return from_dev(d), tau.cpu().numpy()


@pytest.mark.parametrize("case", _G.qr_cases())
def test_factor_parity(golden, oracle, case):
    c = golden.cases[case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    a = golden_input(c, oracle)
    fac, tau = run_factor(a, p, m, n)
    k = min(m, n)
    if "fac" in c:
        R, V = split_factor(fac, m, n)
        Rg, Vg = split_factor(c["fac"], m, n)
        assert rel(R, Rg) <= R_TOL[p]
        assert rel(V, Vg) <= V_TOL[p]
        assert np.array_equal(fac[m:, :n], a[m:, :n])
    else:
        Rg = np.zeros((k, n), dtype=fac.dtype)
        Rg[np.triu_indices(k, 0, n)] = c["r_packed"]
        assert rel(np.triu(fac[:k, :n]), Rg) <= R_TOL[p]
    assert np.max(np.abs(tau - c["tau"]), initial=0) <= 10 * R_TOL[p]
    if m * n <= 300 * 300 and np.isfinite(fac).all():
        r1, r2 = factor_residuals(a, fac, tau, m, n)
        assert r1 <= RESID_TOL and r2 <= RESID_TOL


@pytest.mark.parametrize("case", [n for n in _G.qr_cases() if "fac_unblocked" in _G.cases[n]])
def test_factor_unblocked_parity(golden, oracle, case):
    c = golden.cases[case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    fac, tau = run_factor(golden_input(c, oracle), p, m, n, unblocked=True)
    R, V = split_factor(fac, m, n)
    Rg, Vg = split_factor(c["fac_unblocked"], m, n)
    assert rel(R, Rg) <= R_TOL[p]
    assert rel(V, Vg) <= V_TOL[p]
    assert np.max(np.abs(tau - c["tau_unblocked"]), initial=0) <= 10 * R_TOL[p]


@pytest.mark.parametrize("case", [n for n in _G.qr_cases() if "q" in _G.cases[n] or "q_head" in _G.cases[n]])
@pytest.mark.parametrize("blocked", [True, False])
def test_generate_q_parity(golden, oracle, case, blocked):
    c = golden.cases[case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    if not blocked and "q_unblocked" not in c:
        pytest.skip("no unblocked golden")
    k = min(m, n)
    nq = n if m >= n else m
    fac, tau = run_factor(golden_input(c, oracle), p, m, n)
    d = to_dev(np.asfortranarray(fac[:, :nq]))
    Q = d[:m, :nq]
    t = torch.from_numpy(np.ascontiguousarray(tau)).cuda()
    if blocked:
        gq.generate_q(Q, t, k)
    else:
        gq.generate_q_unblocked(Q, t, k)
    torch.cuda.synchronize()
    q = from_dev(d)[:m, :]
    key = "q" if blocked else "q_unblocked"
    if key in c:
        assert rel(q, c[key]) <= R_TOL[p]
    else:
        assert rel(q[:, :16], c["q_head"]) <= R_TOL[p]
        assert rel(q[:, -16:], c["q_tail"]) <= R_TOL[p]
    # orthonormal columns: ||Q^H Q - I|| / (n eps) <= 10
    qq = q.astype(np.complex128 if np.iscomplexobj(q) else np.float64)
    err = np.linalg.norm(qq.conj().T @ qq - np.eye(nq), 1) / (max(nq, 1) * EPS[p])
    assert err <= RESID_TOL


@pytest.mark.parametrize("case", [n for n in _G.qr_cases() if "c_left" in _G.cases[n]])
def test_mult_q_parity(golden, oracle, case):
    c = golden.cases[case]
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    k = min(m, n)
    fac, tau = run_factor(golden_input(c, oracle), p, m, n)
    dA = to_dev(fac)
    A = dA[:m, :]
    t = torch.from_numpy(np.ascontiguousarray(tau)).cuda()
    for side, c0 in (("L", c["c_left"]), ("R", c["c_right"])):
        for trans in ("N", "C"):
            for blocked in (True, False):
                key = "mq_%s%s%s" % (side, trans, "" if blocked else "_unblocked")
                dc = to_dev(np.asfortranarray(c0))
                if blocked:
                    gq.mult_q(side, trans, A, t, dc, k)
                else:
                    gq.mult_q_unblocked(side, trans, A, t, dc, k)
                torch.cuda.synchronize()
                assert rel(from_dev(dc), c[key]) <= R_TOL[p], key


SIZES = [(1000, 300), (300, 1000), (2048, 64), (64, 33), (4096, 100), (97, 97), (513, 77)]


@pytest.mark.parametrize("p", ["d", "z", "s", "c"])
@pytest.mark.parametrize("mn", SIZES)
def test_factor_against_oracle(oracle, p, mn):
    m, n = mn
    q = "z" if p == "c" else p
    vals, _ = oracle.larnv(q, 2, [4, 3, 2, 1], m * n)
    a = np.asfortranarray(vals.astype(NP[p]).reshape(n, m).T)
    fo = a.copy(order="F")
    to = oracle.geqrf(p, m, n, fo)
    fg, tg = run_factor(a, p, m, n)
    R, V = split_factor(fg, m, n)
    Ro, Vo = split_factor(fo, m, n)
    assert rel(R, Ro) <= R_TOL[p]
    assert rel(V, Vo) <= V_TOL[p]
    assert np.max(np.abs(tg - to)) <= 100 * R_TOL[p]


@pytest.mark.parametrize("ld", [1029, 1032])
def test_fp32_factor_ragged_rows(oracle, ld):
    # 1029 rows: the FP32 trailing passes (W from 1024 rows up) with a ragged
    # last row tile, through scalar loads (ld 1029) and through 16-byte
    # copies with a padded leading dimension (ld 1032)
    p, m, n = "s", 1029, 70
    vals, _ = oracle.larnv("d", 2, [7, 3, 5, 1], m * n)
    a = np.asfortranarray(vals.astype(np.float32).reshape(n, m).T)
    fo = a.copy(order="F")
    to = oracle.geqrf(p, m, n, fo)
    apad = np.zeros((ld, n), dtype=np.float32, order="F")
    apad[:m] = a
    fg, tg = run_factor(apad, p, m, n)
    R, V = split_factor(fg[:m], m, n)
    Ro, Vo = split_factor(fo, m, n)
    assert rel(R, Ro) <= R_TOL[p]
    assert rel(V, Vo) <= V_TOL[p]
    assert np.max(np.abs(tg - to)) <= 100 * R_TOL[p]
    assert np.all(fg[m:] == 0)  # rows past m untouched


@pytest.mark.parametrize("p", ["d", "z"])
def test_apply_and_generate_against_oracle(oracle, p):
    m, n, nrhs = 1500, 200, 9
    vals, _ = oracle.larnv(p, 2, [1, 1, 1, 1], m * n)
    a = np.asfortranarray(vals.reshape(n, m).T)
    fac, tau = run_factor(a, p, m, n)
    cv, _ = oracle.larnv(p, 2, [2, 2, 2, 3], m * nrhs)
    c0 = np.asfortranarray(cv.reshape(nrhs, m).T)
    t = torch.from_numpy(np.ascontiguousarray(tau)).cuda()
    A = to_dev(fac)
    for trans in ("N", "C"):
        co = c0.copy(order="F")
        oracle.unmqr(p, "L", trans, m, nrhs, n, fac, tau, co)
        dc = to_dev(c0)
        gq.mult_q("L", trans, A, t, dc, n)
        torch.cuda.synchronize()
        assert rel(from_dev(dc), co) <= 1e-12
    # right side on an nrhs x m block
    cr = np.asfortranarray(c0.T.copy())
    for trans in ("N", "C"):
        co = cr.copy(order="F")
        oracle.unmqr(p, "R", trans, nrhs, m, n, fac, tau, co)
        dc = to_dev(cr)
        gq.mult_q("R", trans, A, t, dc, n)
        torch.cuda.synchronize()
        assert rel(from_dev(dc), co) <= 1e-12
    qo = np.asfortranarray(fac.copy())
    oracle.ungqr(p, m, n, n, qo, tau)
    dq = to_dev(fac)
    gq.generate_q(dq, t, n)
    torch.cuda.synchronize()
    assert rel(from_dev(dq), qo) <= 1e-12


def test_empty_inputs_are_quick_returns():
    a = torch.zeros((4, 0), dtype=torch.float64, device="cuda")
    tau = gq.factor(gq.empty_colmajor(0, 3, torch.float64))
    assert tau.numel() == 0
    c = gq.empty_colmajor(5, 0, torch.float64)
    gq.mult_q("L", "N", gq.empty_colmajor(5, 2, torch.float64), torch.zeros(2, dtype=torch.float64, device="cuda"), c, 2)
    del a


# MultQ on the left with a thin C goes through the one-launch kernel; C's
# rows are held in shared memory or, when they do not fit, in place.
# (k >= m / 4 takes the variant that re-splits the active rows per reflector
# block: the last three and the 129-row case)
# FP32 with a multiple of 4 columns, blocks of a multiple of 4 rows and a
# 16-byte aligned A takes the 4-row-quad path (6000: 40 rows per block); 6001
# (ld 6001) must leave it; LD_PAD below runs 6001 rows with ld 6004 through it,
# a ragged last block whose quad past the end must read zeros
THIN = [("d", 3000, 1, 70), ("d", 2000, 16, 256), ("s", 5000, 33, 100), ("z", 40000, 64, 64), ("c", 700, 64, 45), ("z", 129, 7, 129),
        ("z", 600, 48, 600), ("d", 1000, 64, 999), ("s", 2000, 5, 1500), ("s", 6000, 16, 256), ("s", 6001, 8, 96), ("s", 20000, 64, 130)]


@pytest.mark.parametrize("p,m,nrhs,k", THIN)
def test_mult_q_thin_against_oracle(oracle, p, m, nrhs, k):
    q = "z" if p == "c" else p
    vals, _ = oracle.larnv(q, 2, [3, 1, 4, 1], m * k)
    a = np.asfortranarray(vals.astype(NP[p]).reshape(k, m).T)
    fac, tau = run_factor(a, p, m, k)
    cv, _ = oracle.larnv(q, 2, [5, 9, 2, 7], m * nrhs)
    c0 = np.asfortranarray(cv.astype(NP[p]).reshape(nrhs, m).T)
    t = torch.from_numpy(np.ascontiguousarray(tau)).cuda()
    A = to_dev(fac)
    tol = 1e-12 if p in "dz" else 1e-5
    for trans in ("N", "C"):
        co = c0.copy(order="F")
        oracle.unmqr(p, "L", trans, m, nrhs, k, fac, tau, co)
        dc = to_dev(c0)
        gq.mult_q("L", trans, A, t, dc, k)
        torch.cuda.synchronize()
        assert rel(from_dev(dc), co) <= tol, trans


def test_mult_q_thin_quads_ragged_block(oracle):
    # 6001 rows stored with leading dimension 6004 (16-byte aligned columns):
    # the FP32 quad path with a ragged last block
    p, m, nrhs, k, ld = "s", 6001, 8, 96, 6004
    vals, _ = oracle.larnv("s", 2, [3, 1, 4, 1], m * k)
    a = np.asfortranarray(vals.astype(np.float32).reshape(k, m).T)
    fac, tau = run_factor(a, p, m, k)
    cv, _ = oracle.larnv("s", 2, [5, 9, 2, 7], m * nrhs)
    c0 = np.asfortranarray(cv.astype(np.float32).reshape(nrhs, m).T)
    t = torch.from_numpy(np.ascontiguousarray(tau)).cuda()
    Apad = torch.zeros((k, ld), dtype=torch.float32, device="cuda").t()
    Apad[:m] = to_dev(fac)
    A = Apad[:m]
    assert A.stride(1) == ld
    for trans in ("N", "C"):
        co = c0.copy(order="F")
        oracle.unmqr(p, "L", trans, m, nrhs, k, fac, tau, co)
        dc = to_dev(c0)
        gq.mult_q("L", trans, A, t, dc, k)
        torch.cuda.synchronize()
        assert rel(from_dev(dc), co) <= 1e-5, trans


# FP32 panels sum squares error-free in FP32; columns whose magnitudes leave
# the safe squaring range take the exact FP64 norm, and the reflector scale
# factor carries a power-of-two shift at the ends of the FP32 range.
@pytest.mark.parametrize("p", ["s", "c"])
@pytest.mark.parametrize("scale", [2.0 ** -120, 2.0 ** -70, 2.0 ** 55, 2.0 ** 100, "mixed"])
def test_fp32_factor_extreme_magnitudes(oracle, p, scale):
    m, n = 700, 40
    q = "z" if p == "c" else p
    vals, _ = oracle.larnv(q, 2, [7, 7, 7, 7], m * n)
    hi = np.complex128 if p == "c" else np.float64
    a64 = np.asfortranarray(vals.astype(hi).reshape(n, m).T)
    if scale == "mixed":
        s = 2.0 ** np.linspace(-110, 110, n)
    else:
        s = np.full(n, scale)
    a = np.asfortranarray((a64 * s[None, :]).astype(NP[p]))
    fac, tau = run_factor(a, p, m, n)
    assert np.all(np.isfinite(fac)) and np.all(np.isfinite(tau))
    fo = np.asfortranarray(a.astype(hi))
    oracle.geqrf("z" if p == "c" else "d", m, n, fo)
    R, _ = split_factor(fac, m, n)
    Ro, _ = split_factor(fo, m, n)
    # compare column by column (columns differ by up to 2^220 in the mixed case)
    for j in range(n):
        assert rel(R[:, j], Ro[:, j]) <= 1e-4, j
