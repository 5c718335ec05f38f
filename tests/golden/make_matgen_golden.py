"""Golden vectors for RNP::MatrixGen::RandomMatrix from the REFERENCE ITSELF.

Runs RNP2's own RandomMatrix (RNP/MatrixGen.hpp:120-272), compiled from the
reference tree by ``make -C oracle ref`` into ``oracle/_ref/libref_qr.so``,
and stores its outputs (the matrix, the diagonal and the advanced seed) in
``tests/golden/matgen_golden.npz``.  The reference's RandomMatrix compiles for
real types only.  Cases: every symmetry kind and diagonal mode, every
distribution of the RandomDist mode, tall, wide and square shapes, float and
double; 260 x 300 stores the first and last 8 columns only.

Usage:  python tests/golden/make_matgen_golden.py   (after ``make -C oracle ref``)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as orc  # noqa: E402

CASES = [
    # (p, sym, dist, mode, reverse, cond, dmax, m, n)
    ("d", 0, 2, 3, 0, 1e3, 1.0, 40, 30),
    ("d", 0, 2, 5, 1, 1e4, 2.0, 30, 40),
    ("d", 0, 0, 6, 0, 1.0, 1.0, 35, 35),
    ("d", 0, 1, 6, 0, 1.0, 1.0, 33, 20),
    ("d", 0, 2, 6, 0, 1.0, 1.0, 20, 33),
    ("d", 0, 3, 6, 0, 1.0, 1.0, 70, 70),
    ("d", 0, 4, 6, 0, 1.0, 1.0, 70, 66),
    ("d", 0, 2, 1, 0, 1e2, 3.0, 64, 64),
    ("d", 0, 2, 2, 0, 1e2, 1.0, 50, 64),
    ("d", 0, 2, 4, 1, 1e2, 1.0, 64, 50),
    ("d", 1, 2, 3, 0, 1e3, 1.0, 35, 35),
    ("d", 1, 2, 5, 0, 1e3, 1.0, 48, 48),
    ("d", 2, 2, 5, 0, 1e4, 1.0, 35, 35),
    ("d", 3, 2, 4, 0, 1e2, 1.0, 35, 35),
    ("d", 0, 2, 3, 0, 1e6, 1.0, 260, 300),
    ("s", 0, 2, 3, 0, 1e3, 1.0, 40, 30),
    ("s", 1, 2, 5, 0, 1e2, 1.0, 35, 35),
    ("s", 0, 2, 6, 0, 1.0, 1.0, 30, 40),
]


def main():
    ref = orc.load_reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_qr.so is missing: run make -C oracle ref")
    out = {}
    names = []
    for (p, sym, dist, mode, rev, cond, dmax, m, n) in CASES:
        name = "mg_%s_s%d_d%d_m%d_%dx%d" % (p, sym, dist, mode, m, n)
        seed = [3, 5, 7, 9]
        a, d, s_out = ref.random_matrix(p, sym, dist, mode, rev, cond, dmax, m, n, seed)
        e = {"p": p, "sym": sym, "dist": dist, "mode": mode, "reverse": rev, "cond": cond, "dmax": dmax, "m": m, "n": n,
             "seed": np.array(seed), "seed_out": np.array(s_out), "d": d}
        if m * n > 20000:
            e["a_head"] = np.asfortranarray(a[:, :8])
            e["a_tail"] = np.asfortranarray(a[:, -8:])
        else:
            e["a"] = np.asfortranarray(a)
        for key, v in e.items():
            out["%s__%s" % (name, key)] = np.asarray(v)
        names.append(name)
    out["__cases__"] = np.array(names)
    path = os.path.join(HERE, "matgen_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(names), "cases")


if __name__ == "__main__":
    main()
