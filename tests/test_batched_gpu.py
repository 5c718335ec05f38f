"""Batched QR: every matrix of an uneven batch must match the oracle's
Factor (R, V and tau), across size classes, block shapes chosen by the
autotuner, and when the run is captured into a CUDA graph and replayed."""
import numpy as np
import pytest

from qr_checks import R_TOL, V_TOL, rel, split_factor

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300.batched import BatchedQR  # noqa: E402

NP = {torch.float32: np.float32, torch.float64: np.float64, torch.complex64: np.complex64, torch.complex128: np.complex128}
PFX = {torch.float32: "s", torch.float64: "d", torch.complex64: "c", torch.complex128: "z"}


def make_batch(count, dtype, seed=0, mmax=256):
    rng = np.random.default_rng(seed)
    ms = rng.integers(16, mmax + 1, count)
    ns = np.array([rng.integers(8, m + 1) for m in ms])
    ms[:3] = [1, 256, 40]
    ns[:3] = [1, 256, 200]
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


def test_batched_autotuned_and_graph_replayed(oracle):
    dtype = torch.float64
    b, vals = make_batch(200, dtype, seed=2)
    a0 = b.a.clone()
    b.tune()
    cfg = [b.config(0), b.config(1)]
    assert cfg[0]["count"] + cfg[1]["count"] == 200
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
