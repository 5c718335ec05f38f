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


@pytest.mark.parametrize("p", ["s", "d", "c", "z"])
@pytest.mark.parametrize("n", [300, 17, 512, 600])
def test_trsm_upper(oracle, p, n):
    # n <= 512 with 4- and 8-byte elements: the latency-hiding kernel (ragged
    # last block at 300 and 17); 600 and complex FP64: the general one
    nrhs = 5
    # well conditioned: unit diagonal plus a small strictly upper part
    R = np.asfortranarray((np.eye(n) + np.triu(mat(oracle, p, n, n, [5, 5, 5, 5]), 1) / n).astype(NP[p]))
    B = mat(oracle, p, n, nrhs, [6, 6, 6, 7])
    dB = to_dev(B)
    gls.trsm_upper(to_dev(R), dB)
    torch.cuda.synchronize()
    tol = 1e-14 if p in "dz" else 2e-6
    assert rel(R.astype(np.complex128) @ from_dev(dB), B) <= tol


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


def panel_kinds(fn):
    """Run fn with kernel-class timing on; {class: launches} of its panels."""
    from rnp2_gb300 import _capi

    lib = _capi.lib()
    lib.rnpgpu_timing_enable(1)
    _capi.timing_report()
    try:
        out = fn()
        torch.cuda.synchronize()
        rep = _capi.timing_report()
    finally:
        lib.rnpgpu_timing_enable(0)
    return out, {k: v[0] for k, v in rep.items() if k.startswith("panel")}


def check_refined(A, b, X, info):
    n = A.shape[1]
    bound = 10 * n * np.finfo(np.float64).eps
    assert info["converged"] == 1, info
    assert info["backward_error"] <= bound and info["normal_residual"] <= bound
    assert ls_backward_error(A, b, X.cpu().numpy()) <= bound


@pytest.mark.parametrize("mn", [(4096, 100), (3000, 64), (1000, 33)])
@pytest.mark.parametrize("forward", [False, True])
def test_mixed_fp32_factor_uses_cholesky_qr2_panels(mn, forward):
    # the mixed solver's FP32 factor takes CholeskyQR2 panels on real data;
    # widths that are not a multiple of 32 pad the last panel (forward mode
    # also runs the R^-T solves of the seminormal steps on ragged blocks)
    m, n = mn
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n))
    b = A @ rng.standard_normal((n, 3)) + 1e-8 * rng.standard_normal((m, 3))
    (X, info), kinds = panel_kinds(lambda: gls.gels_refine(to_dev(A), to_dev(b), forward=forward))
    assert kinds == {"panel_cqr": (n + 31) // 32}, kinds
    check_refined(A, b, X, info)


def test_mixed_fp32_factor_redoes_ill_conditioned_panels_in_double_float():
    # two columns 1e-4 apart in angle: the FP32 first pass of their panel keeps
    # a pivot of 1e-8 of the column's squared norm (below its 2^-20 limit), so
    # the panel is redone with the double-float first pass (limit 2^-38) and
    # stays a CholeskyQR2 panel; condition ~1e4, which the refinement handles
    m, n = 4096, 96
    rng = np.random.default_rng(22)
    A = rng.standard_normal((m, n))
    u = rng.standard_normal(m)
    u -= A[:, 40] * (u @ A[:, 40]) / (A[:, 40] @ A[:, 40])
    A[:, 41] = A[:, 40] + 1e-4 * np.linalg.norm(A[:, 40]) * u / np.linalg.norm(u)
    b = A @ rng.standard_normal((n, 2)) + 1e-8 * rng.standard_normal((m, 2))
    (X, info), kinds = panel_kinds(lambda: gls.gels_refine(to_dev(A), to_dev(b)))
    assert kinds == {"panel_cqr": 3}, kinds
    check_refined(A, b, X, info)


def test_mixed_fp32_factor_falls_back_to_householder_panels():
    # two columns 1e-6 apart in angle: the first Cholesky pivot of their panel
    # keeps 1e-12 of the column's squared norm, below the CholeskyQR2 limit, so
    # the factor is redone with Householder panels.  Any panel that fails has a
    # condition number near 10^6 or more, where the refinement contracts slowly:
    # the check is that it refines far below FP32 accuracy from the redone
    # factor (a stale or damaged factor would not), and that the error it
    # reports is the true one
    m, n = 4096, 96
    rng = np.random.default_rng(21)
    A = rng.standard_normal((m, n))
    u = rng.standard_normal(m)
    u -= A[:, 40] * (u @ A[:, 40]) / (A[:, 40] @ A[:, 40])
    A[:, 41] = A[:, 40] + 1e-6 * np.linalg.norm(A[:, 40]) * u / np.linalg.norm(u)
    b = A @ rng.standard_normal((n, 2)) + 1e-8 * rng.standard_normal((m, 2))
    (X, info), kinds = panel_kinds(lambda: gls.gels_refine(to_dev(A), to_dev(b)))
    assert kinds.get("panel") == 3 and kinds.get("panel_cqr", 0) >= 2, kinds
    be = ls_backward_error(A, b, X.cpu().numpy())
    # far below FP32 accuracy (a stale or damaged factor leaves ~1e-3); at
    # this condition number ten steps end between 1e-12 and 1e-9 depending on
    # the rounding of the FP32 factor
    assert info["backward_error"] <= 1e-9 and be <= 1e-9, (info, be)
    if info["converged"] == 1:
        assert be <= 10 * n * np.finfo(np.float64).eps


@pytest.mark.parametrize("m,n,nrhs", [(4096, 300, 3), (2000, 130, 1), (1000, 100, 2), (8192, 512, 16), (4096, 384, 20)])
def test_gels_refine_host_matches_device_solve(m, n, nrhs):
    """rnpgpu_dsgels_host (host buffers, A staged in 128-column ranges while
    the GPU factors the ranges already landed, left-looking by 128-column
    blocks) converges like the device solve, to the same solution within the
    refinement's accuracy."""
    from rnp2_gb300 import ls as gls
    from rnp2_gb300.qr import to_colmajor

    g = torch.Generator(device="cuda").manual_seed(m + n)
    A = to_colmajor(torch.randn((m, n), generator=g, dtype=torch.float64, device="cuda"))
    B = to_colmajor(torch.randn((m, nrhs), generator=g, dtype=torch.float64, device="cuda"))
    X, info = gls.gels_refine(A, B)
    A_h = torch.empty((n, m), dtype=torch.float64).pin_memory().t()
    A_h.copy_(A)
    B_h = torch.empty((nrhs, m), dtype=torch.float64).pin_memory().t()
    B_h.copy_(B)
    X_h = torch.full((nrhs, n), float("nan"), dtype=torch.float64).pin_memory().t()
    info_h = gls.gels_refine_host(A_h, B_h, X_h)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(X).all()) and info["converged"] == 1, info
    assert info_h["converged"] == 1, info_h
    bound = 10 * n * np.finfo(np.float64).eps
    assert info_h["backward_error"] <= bound and info_h["normal_residual"] <= bound, info_h
    Xd = X.cpu()
    assert float((X_h - Xd).abs().max() / Xd.abs().max()) <= 1e-11
    # the same staged call twice: the same bits
    X_h2 = torch.full((nrhs, n), float("nan"), dtype=torch.float64).pin_memory().t()
    gls.gels_refine_host(A_h, B_h, X_h2)
    torch.cuda.synchronize()
    assert torch.equal(X_h, X_h2)


@pytest.mark.parametrize("m,n", [(2000, 130), (3000, 130), (1500, 70), (4096, 97)])
def test_refinement_with_partial_last_block(m, n):
    """n not a multiple of 32: the corrected seminormal steps solve with R over
    a partial last 32-row block (entries past n must not enter the update;
    stale shared memory once turned them into NaN)."""
    rng = np.random.default_rng(m + n)
    A, b = rng.standard_normal((m, n)), rng.standard_normal((m, 2))
    for forward in (False, True):
        X, info = gls.gels_refine(to_dev(A), to_dev(b), forward=forward)
        torch.cuda.synchronize()
        assert bool(torch.isfinite(X).all()), (forward, info)
        assert info["converged"] == 1, (forward, info)
        assert ls_backward_error(A, b, X.cpu().numpy()) <= 10 * n * np.finfo(np.float64).eps


def test_refinement_reports_nonfinite_data():
    """A NaN in A never passes the stopping test: converged 0 and a NaN
    backward error (the solve does not fault or loop)."""
    m, n = 1000, 64
    rng = np.random.default_rng(8)
    A = rng.standard_normal((m, n))
    A[17, 5] = np.nan
    b = rng.standard_normal((m, 1))
    X, info = gls.gels_refine(to_dev(A), to_dev(b))
    torch.cuda.synchronize()
    assert info["converged"] == 0, info
    assert not np.isfinite(info["backward_error"]), info


def test_gels_refine_host_from_pageable_buffers():
    """Host buffers that are not pinned: the copies are synchronous, the result
    the same as from pinned buffers (same staged order, same bits)."""
    m, n, nrhs = 3000, 260, 2
    g = torch.Generator(device="cuda").manual_seed(11)
    A = torch.randn((m, n), generator=g, dtype=torch.float64, device="cuda")
    B = torch.randn((m, nrhs), generator=g, dtype=torch.float64, device="cuda")
    A_p = torch.empty((n, m), dtype=torch.float64).pin_memory().t()
    A_p.copy_(A)
    B_p = torch.empty((nrhs, m), dtype=torch.float64).pin_memory().t()
    B_p.copy_(B)
    X_p = torch.empty((nrhs, n), dtype=torch.float64).pin_memory().t()
    info_p = gls.gels_refine_host(A_p, B_p, X_p)
    torch.cuda.synchronize()
    A_u = torch.empty((n, m), dtype=torch.float64).t()
    A_u.copy_(A)
    B_u = torch.empty((nrhs, m), dtype=torch.float64).t()
    B_u.copy_(B)
    X_u = torch.empty((nrhs, n), dtype=torch.float64).t()
    info_u = gls.gels_refine_host(A_u, B_u, X_u)
    torch.cuda.synchronize()
    assert info_p["converged"] == 1 and info_u == info_p, (info_p, info_u)
    assert torch.equal(X_u, X_p)


@pytest.mark.parametrize("rank32,forward", [(True, False), (False, True)])
def test_gels_refine_host_modes(rank32, forward):
    """The host-buffer solve with the rank-32 FP32 updates (its staged input
    then waits for every range before the factor) and in forward mode meets
    the same stopping tests as the device solve in the same mode."""
    m, n, nrhs = 4096, 300, 2
    g = torch.Generator(device="cuda").manual_seed(13 + rank32 + 2 * forward)
    A = torch.randn((m, n), generator=g, dtype=torch.float64, device="cuda")
    B = torch.randn((m, nrhs), generator=g, dtype=torch.float64, device="cuda")
    from rnp2_gb300.qr import to_colmajor

    X, info = gls.gels_refine(to_colmajor(A), to_colmajor(B), forward=forward, rank32=rank32)
    A_h = torch.empty((n, m), dtype=torch.float64).pin_memory().t()
    A_h.copy_(A)
    B_h = torch.empty((nrhs, m), dtype=torch.float64).pin_memory().t()
    B_h.copy_(B)
    X_h = torch.empty((nrhs, n), dtype=torch.float64).pin_memory().t()
    info_h = gls.gels_refine_host(A_h, B_h, X_h, forward=forward, rank32=rank32)
    torch.cuda.synchronize()
    assert info["converged"] == 1 and info_h["converged"] == 1, (info, info_h)
    Xd = X.cpu()
    assert float((X_h - Xd).abs().max() / Xd.abs().max()) <= 1e-11
    if rank32:
        # no left-looking order without the wide blocks: the same operations, the same bits
        assert torch.equal(X_h, Xd)
