import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "qr_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


class Golden:
    """Cases of tests/golden/qr_golden.npz: name -> {field: array}."""

    def __init__(self, path):
        z = np.load(path)
        self.cases = {}
        for key in z.files:
            if key == "__cases__":
                continue
            name, field = key.split("__", 1)
            self.cases.setdefault(name, {})[field] = z[key]
        self.names = [str(n) for n in z["__cases__"]]

    def qr_cases(self, prefix=None, p=None):
        out = []
        for n in self.names:
            c = self.cases[n]
            if "tau" not in c:
                continue
            if prefix and not n.startswith(prefix):
                continue
            if p and str(c["p"]) != p:
                continue
            out.append(n)
        return out


@pytest.fixture(scope="session")
def golden():
    return Golden(GOLDEN)


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    return orc.load()


def golden_input(golden_case, orc_lib):
    """The case's input matrix (ld x n, Fortran order): stored, or regenerated
    from its seed by the oracle's restated generator (bit-exact with the
    reference's) and checked against the stored checksum."""
    c = golden_case
    p = str(c["p"])
    m, n, ld = int(c["m"]), int(c["n"]), int(c["lda"])
    if "a" in c:
        return np.asfortranarray(c["a"].copy())
    q = "z" if p == "c" else p
    vals, _ = orc_lib.larnv(q, int(c["dist"]), [int(s) for s in c["seed"]], m * n)
    vals = vals.astype({"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}[p])
    a = np.zeros((ld, max(n, 1)), dtype=vals.dtype, order="F")
    a[:m, :n] = vals.reshape(n, m).T
    assert np.array_equal(a[:m, 0], c["a_col0"])
    assert a[:m, :n].sum() == c["a_sum"]
    return a


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture
def oracle_blas(oracle):
    """The oracle with every level-2/3 call routed through OpenBLAS on all
    host cores, as the reference forwards them to its BLAS: for checks at the
    full workload sizes, where the restatement's plain loops take minutes.
    Skips where no OpenBLAS is available; switched back to the plain loops
    afterwards."""
    import oracle as orc

    blas = orc.find_openblas()
    if not blas or orc.use_blas(oracle, blas, "scipy_", os.cpu_count() or 1) != 0:
        pytest.skip("no OpenBLAS for the oracle")
    try:
        yield oracle
    finally:
        orc.use_blas(oracle, None)
