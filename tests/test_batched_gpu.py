"""Batched QR: every matrix of an uneven batch must match the oracle's
Factor (R, V and tau), across size classes, block shapes chosen by the
autotuner, and when the run is captured into a CUDA graph and replayed.
Batched least squares: the plain solve matches the oracle's QR least squares
per problem; the mixed solve (FP32 factorization, FP64 refinement) reaches
FP64-level backward error on every problem."""
import numpy as np
import pytest

from qr_checks import R_TOL, V_TOL, rel, split_factor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300.batched import BatchedLS, BatchedQR  # noqa: E402

NP = {torch.float32: np.float32, torch.float64: np.float64, torch.complex64: np.complex64, torch.complex128: np.complex128}
PFX = {torch.float32: "s", torch.float64: "d", torch.complex64: "c", torch.complex128: "z"}


def make_batch(count, dtype, seed=0, mmax=512):
    rng = np.random.default_rng(seed)
    ms = rng.integers(16, mmax + 1, count)
    ns = np.array([rng.integers(8, min(m, 300) + 1) for m in ms])
    ms[:5] = [1, 256, 40, 512, 65]
    ns[:5] = [1, 256, 200, 300, 64]
    b = BatchedQR(ms, ns, dtype)
    vals = []
    for i in range(count):
        x = rng.standard_normal((ms[i], ns[i]))
        if dtype.is_complex:
            x = x + 1j * rng.standard_normal((ms[i], ns[i]))
        vals.append(np.asfortranarray(x.astype(NP[dtype])))
        b.matrix(i).copy_(torch.from_numpy(vals[-1]))
    return b, vals


def check(b, vals, oracle, dtype):
    p = PFX[dtype]
    for i, a in enumerate(vals):
        m, n = a.shape
        fo = a.copy(order="F")
        to = oracle.geqrf(p, m, n, fo)
        fg = b.matrix(i).cpu().numpy()
        R, V = split_factor(fg, m, n)
        Ro, Vo = split_factor(fo, m, n)
        assert rel(R, Ro) <= R_TOL[p], (i, m, n)
        assert rel(V, Vo) <= V_TOL[p], (i, m, n)
        assert np.max(np.abs(b.tau_of(i).cpu().numpy() - to), initial=0) <= 100 * R_TOL[p], (i, m, n)


@pytest.mark.parametrize("dtype", [torch.float64, torch.complex128, torch.float32, torch.complex64])
def test_batched_matches_oracle(oracle, dtype):
    b, vals = make_batch(120, dtype, seed=1)
    b.factor()
    torch.cuda.synchronize()
    check(b, vals, oracle, dtype)


@pytest.mark.parametrize("dtype", [torch.float64, torch.complex64])
@pytest.mark.parametrize("warp", [True, False])
def test_batched_small_class_warp_and_block(oracle, dtype, warp):
    """Matrices with m, n <= 32 (tall, square and fat) go to the smallest
    class, factored by one warp per matrix or by a small block; both must
    match the oracle."""
    rng = np.random.default_rng(7)
    count = 300
    ms = rng.integers(1, 33, count)
    ns = rng.integers(1, 33, count)
    b = BatchedQR(ms, ns, dtype)
    vals = []
    for i in range(count):
        x = rng.standard_normal((ms[i], ns[i]))
        if dtype.is_complex:
            x = x + 1j * rng.standard_normal((ms[i], ns[i]))
        vals.append(np.asfortranarray(x.astype(NP[dtype])))
        b.matrix(i).copy_(torch.from_numpy(vals[-1]))
    assert b.config(0)["count"] == count
    if not warp:
        b.force_config(0, 64, 8)
    b.factor()
    torch.cuda.synchronize()
    assert b.config(0)["threads"] == (32 if warp else 64)
    check(b, vals, oracle, dtype)


def test_batched_autotuned_and_graph_replayed(oracle):
    dtype = torch.float64
    b, vals = make_batch(200, dtype, seed=2)
    a0 = b.a.clone()
    b.tune()
    cfg = [b.config(c) for c in range(4)]
    assert sum(c["count"] for c in cfg) == 200 and all(c["count"] > 0 for c in cfg)
    # capture one run into a CUDA graph, replay it twice on fresh inputs
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        b.a.copy_(a0)
        b.factor()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        b.factor()
    for _ in range(2):
        b.a.copy_(a0)
        g.replay()
    torch.cuda.synchronize()
    check(b, vals, oracle, dtype)


def ls_problems(count, dtype, seed, cond=1e4, mmax=512, noise=1e-10):
    """A = U diag(s) V^H (U, V Householder reflectors of Gaussian vectors, s
    log-uniform on [1/cond, 1]), b = A x + noise N(0,1)."""
    rng = np.random.default_rng(seed)
    ms = rng.integers(32, mmax + 1, count)
    ns = np.array([rng.integers(8, m // 2 + 1) for m in ms])
    ms[:3] = [32, 512, 33]
    ns[:3] = [8, 256, 33]
    cplx = dtype.is_complex

    def gauss(*shape):
        x = rng.standard_normal(shape)
        return x + 1j * rng.standard_normal(shape) if cplx else x

    probs = []
    for m, n in zip(ms, ns):
        s = 10.0 ** (-np.log10(cond) * rng.random(n))
        u = gauss(m)
        w = gauss(n)
        V = np.eye(n) - 2.0 * np.outer(w, w.conj()) / np.vdot(w, w).real
        D = np.zeros((m, n), dtype=complex if cplx else float)
        D[:n] = s[:, None] * V.conj().T
        A = D - 2.0 * np.outer(u, u.conj() @ D) / np.vdot(u, u).real
        x = gauss(n)
        b = A @ x + noise * gauss(m)
        probs.append((np.asfortranarray(A.astype(NP[dtype])), b.astype(NP[dtype])))
    return ms, ns, probs


def fill(ls, probs):
    for i, (A, b) in enumerate(probs):
        ls.matrix(i).copy_(torch.from_numpy(A))
        ls.rhs(i).copy_(torch.from_numpy(b))


@pytest.mark.parametrize("dtype", [torch.float64, torch.complex128, torch.float32, torch.complex64])
def test_batched_ls_plain_matches_oracle(oracle, dtype):
    ms, ns, probs = ls_problems(48, dtype, seed=3, cond=1e2)
    ls = BatchedLS(ms, ns, dtype)
    fill(ls, probs)
    ls.solve_plain()
    torch.cuda.synchronize()
    p = PFX[dtype]
    tol = 1e-11 if p in "dz" else 1e-3
    for i, (A, b) in enumerate(probs):
        m, n = A.shape
        ao = A.copy(order="F")
        bo = np.asfortranarray(b.reshape(m, 1).copy())
        oracle.gels(p, m, n, 1, ao, bo)
        assert rel(ls.solution(i).cpu().numpy(), bo[:n, 0]) <= tol, (i, m, n)


@pytest.mark.parametrize("dtype", [torch.complex128, torch.float64])
def test_batched_ls_mixed_reaches_fp64_backward_error(oracle, dtype):
    ms, ns, probs = ls_problems(64, dtype, seed=4, cond=1e4)
    ls = BatchedLS(ms, ns, dtype)
    fill(ls, probs)
    ls.tune_mixed()
    ls.solve_mixed()
    torch.cuda.synchronize()
    eps = np.finfo(np.float64).eps
    berr = ls.berr.cpu().numpy()
    eta = ls.eta.cpu().numpy()
    iters = ls.iters.cpu().numpy()
    p = PFX[dtype]
    for i, (A, b) in enumerate(probs):
        m, n = A.shape
        assert berr[i] <= 10 * n * eps and eta[i] <= 10 * n * eps, (i, m, n, berr[i], eta[i])
        assert 1 <= iters[i] <= 10
        # forward error against the FP64 oracle solution: cond 1e4
        ao = A.copy(order="F")
        bo = np.asfortranarray(b.reshape(m, 1).copy())
        oracle.gels(p, m, n, 1, ao, bo)
        assert rel(ls.solution(i).cpu().numpy(), bo[:n, 0]) <= 1e-10, (i, m, n)
        # the FP64 backward error measured independently in numpy
        x = ls.solution(i).cpu().numpy()
        r = b - A @ x
        an = np.linalg.norm(A)
        assert np.linalg.norm(A.conj().T @ r) / (an * (an * np.linalg.norm(x) + np.linalg.norm(b))) <= 10 * n * eps


def test_batched_ls_mixed_graph_replay():
    dtype = torch.complex128
    ms, ns, probs = ls_problems(40, dtype, seed=5)
    ls = BatchedLS(ms, ns, dtype)
    fill(ls, probs)
    ls.solve_mixed()
    torch.cuda.synchronize()
    x0 = ls.x.clone()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        ls.solve_mixed()
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        ls.solve_mixed()
    ls.x.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(ls.x, x0)
