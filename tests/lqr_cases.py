"""Shared helpers of the LQ / QL / RQ parity tests: the golden cases of
tests/golden/lqr_golden.npz (outputs of the reference itself) and their
inputs, regenerated bit-exactly with the oracle's restated generator."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "lqr_golden.npz")
DT = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}
TOL = {"s": 1e-4, "c": 1e-4, "d": 1e-12, "z": 1e-12}


def load():
    z = np.load(PATH)
    cases = {}
    for key in z.files:
        if key == "__cases__":
            continue
        name, field = key.split("__", 1)
        cases.setdefault(name, {})[field] = z[key]
    return [str(n) for n in z["__cases__"]], cases


def gen(orc_lib, p, m, n, seed):
    q = "z" if p == "c" else ("d" if p == "s" else p)
    vals, _ = orc_lib.larnv(q, 2, seed, m * n)
    return np.asfortranarray(vals.astype(DT[p]).reshape(n, m).T)


def case_input(orc_lib, c):
    p, m, n = str(c["p"]), int(c["m"]), int(c["n"])
    a = gen(orc_lib, p, m, n, [int(s) for s in c["seed"]])
    assert np.array_equal(a[:, 0], c["a_col0"]) and a.sum() == c["a_sum"]
    return a


def tri(kind, f, m, n):
    k = min(m, n)
    if kind == "lq":
        blk, lower = f[:k, :k], True
    elif kind == "ql":
        blk, lower = f[m - k:, n - k:], True
    else:
        blk, lower = f[m - k:, n - k:], False
    return blk[np.tril_indices(k) if lower else np.triu_indices(k)]


def reflectors(kind, f, m, n):
    k = min(m, n)
    if kind == "lq":
        return np.asfortranarray(f[:k, :])
    if kind == "ql":
        return np.asfortranarray(f[:, n - k:])
    return np.asfortranarray(f[m - k:, :])


def genq_ok(kind, m, n):
    return (kind == "ql" and m >= n) or (kind != "ql" and m <= n)
