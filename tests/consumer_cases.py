"""Shared helpers of the parity tests of the reference's callers of QR / QL
(Hessenberg and tridiagonal Q, the generalized eigensystem's QR step): the
golden cases of tests/golden/consumers_golden.npz, outputs of the reference
itself with the reductions' outputs as their inputs."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "golden", "consumers_golden.npz")
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


def kind(name):
    return name.split("_", 1)[0]


def fortran(x):
    return np.asfortranarray(np.array(x))
