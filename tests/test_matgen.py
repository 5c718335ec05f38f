"""RNP::MatrixGen::RandomMatrix: the oracle's restatement (CPU) and the GPU
entry point against outputs of the reference itself
(tests/golden/matgen_golden.npz): the matrix, the diagonal and the seed the
call leaves behind; on the GPU also the generator's uniforms bit for bit, and
the singular values at a larger size."""
import os

import numpy as np
import pytest

from qr_checks import rel

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "matgen_golden.npz"))
CASES = {}
for key in Z.files:
    if key != "__cases__":
        name, field = key.split("__", 1)
        CASES.setdefault(name, {})[field] = Z[key]
NAMES = [str(n) for n in Z["__cases__"]]
TOL = {"d": 1e-12, "s": 1e-4}


def args(c):
    return (int(c["sym"]), int(c["dist"]), int(c["mode"]), int(c["reverse"]), float(c["cond"]), float(c["dmax"]), int(c["m"]), int(c["n"]))


def check(c, a, d, seed_out):
    p = str(c["p"])
    assert seed_out == [int(x) for x in c["seed_out"]]
    assert rel(d, c["d"]) <= TOL[p]
    if "a" in c:
        assert rel(a, c["a"]) <= TOL[p]
    else:
        assert rel(a[:, :8], c["a_head"]) <= TOL[p] and rel(a[:, -8:], c["a_tail"]) <= TOL[p]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_random_matrix_matches_reference(oracle, name):
    c = CASES[name]
    sym, dist, mode, rev, cond, dmax, m, n = args(c)
    a, d, s = oracle.random_matrix(str(c["p"]), sym, dist, mode, rev, cond, dmax, m, n, [int(x) for x in c["seed"]])
    check(c, a, d, s)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_random_matrix_matches_reference(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rnp2_gb300 import matgen

    c = CASES[name]
    sym, dist, mode, rev, cond, dmax, m, n = args(c)
    dt = torch.float64 if str(c["p"]) == "d" else torch.float32
    A, d, s = matgen.random_matrix(m, n, sym=sym, dist=dist, mode=mode, cond=cond, dmax=dmax, reverse=bool(rev), seed=[int(x) for x in c["seed"]], dtype=dt)
    torch.cuda.synchronize()
    check(c, A.cpu().numpy(), d.cpu().numpy(), s)


@pytest.mark.gpu
@pytest.mark.parametrize("p", ["s", "d"])
def test_gpu_generator_is_bit_exact(oracle, p):
    # mode RandomDist with Uniform01: the diagonal is the generator's raw
    # uniforms, bit for bit the reference's (restated generator, pinned by the
    # golden tests of the oracle); Normal01 within an ulp or two (libm)
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rnp2_gb300 import matgen

    dt = torch.float64 if p == "d" else torch.float32
    k = 3000
    seed = [11, 22, 33, 45]
    _, d, s = matgen.random_matrix(k, k, sym=0, dist=0, mode=6, seed=seed, dtype=dt)
    u, s_ref = oracle.larnv(p, 0, seed, k)
    assert np.array_equal(d.cpu().numpy(), u)
    _, d, s = matgen.random_matrix(k, k, sym=0, dist=2, mode=6, seed=seed, dtype=dt)
    g, _ = oracle.larnv(p, 2, seed, k)
    eps = np.finfo(np.float64 if p == "d" else np.float32).eps
    assert np.max(np.abs(d.cpu().numpy() - g) / np.maximum(np.abs(g), 1e-30)) <= 4 * eps


@pytest.mark.gpu
def test_gpu_random_matrix_singular_values():
    # nonsymmetric, graded exponentially: the singular values are d
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rnp2_gb300 import matgen

    m, n, cond = 4096, 512, 1e6
    A, d, _ = matgen.random_matrix(m, n, sym=0, dist=2, mode=3, cond=cond, dmax=1.0, seed=[1, 2, 3, 5])
    sv = torch.linalg.svdvals(A)
    dd = torch.sort(torch.abs(d), descending=True).values
    assert float(torch.max(torch.abs(sv - dd) / dd)) <= 1e-8
    assert abs(float(sv[0] / sv[-1]) / cond - 1) <= 1e-8
