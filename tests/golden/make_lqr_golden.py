"""Golden vectors for the LQ, QL and RQ factorizations from the REFERENCE ITSELF.

Runs RNP2's own RNP::LA::LQ, QL and RQ (Factor, MultQ, GenerateQ), compiled
from the reference tree by ``make -C oracle ref`` into
``oracle/_ref/libref_qr.so``, on inputs drawn with the reference's generator,
and stores inputs' checksums and outputs in ``tests/golden/lqr_golden.npz``.
The fixtures are committed; this script only runs where the reference tree
exists.

Cases, for each of lq, ql, rq:
  * the sizes of the reference's own tests (tests/test_lq_tall.cpp 170x150,
    test_lq_fat.cpp 166x170, test_ql_tall.cpp 170x150, test_ql_fat.cpp
    140x150, test_rq_tall.cpp 170x150, test_rq_fat.cpp 150x170), double and
    complex<double>: tau and the triangular factor;
  * 40x30 and 30x40 for all four types: the whole factor, tau, MultQ in all
    four side/trans combinations and GenerateQ where the shape allows it
    (LQ MultQ on the left with fewer than 32 reflectors: the product with the
    reference's own GenerateQ, see below);
  * 300x260 and 260x300 in double (past the nb = 32 block and the nx = 128
    crossover): tau, MultQ and the first and last 8 columns of GenerateQ.

The reference's LQ::MultQ with side "L" and fewer than 32 reflectors runs
LQ::MultQ_unblocked, whose Reflector::Apply(side "L", vone, vconj) updates
only the first column of C (RNP/LA/Reflector.hpp:260-265 index c[i+0*ldc]
where c[i+j*ldc] is meant): its output agrees neither with Q C nor with
Q^H C for the Q its GenerateQ forms.  Those cases record Q C and Q^H C with
that Q (the blocked route, k >= 32, agrees with it to rounding).

Usage:  python tests/golden/make_lqr_golden.py   (after ``make -C oracle ref``)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as orc  # noqa: E402

REF_SIZES = {"lq": [(170, 150), (166, 170)], "ql": [(170, 150), (140, 150)], "rq": [(170, 150), (150, 170)]}


def gen(ref, p, m, n, seed):
    """m x n Fortran matrix from the reference's generator (normal entries;
    complex<float> drawn as complex<double> and rounded)."""
    q = "z" if p == "c" else ("d" if p == "s" else p)
    vals, _ = ref.larnv(q, 2, seed, m * n)
    return np.asfortranarray(vals.astype(orc.DT[p]).reshape(n, m).T)


def tri(kind, f, m, n):
    """The triangular factor of a kind's storage, packed (k (k + 1) / 2
    values: its k x k block's lower triangle for lq and ql, upper for rq,
    column by column)."""
    k = min(m, n)
    if kind == "lq":
        blk, lower = f[:k, :k], True
    elif kind == "ql":
        blk, lower = f[m - k:, n - k:], True
    else:
        blk, lower = f[m - k:, n - k:], False
    idx = np.tril_indices(k) if lower else np.triu_indices(k)
    return blk[idx]


def reflectors(kind, f, m, n):
    k = min(m, n)
    if kind == "lq":
        return np.asfortranarray(f[:k, :])
    if kind == "ql":
        return np.asfortranarray(f[:, n - k:])
    return np.asfortranarray(f[m - k:, :])


def main():
    ref = orc.load_reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_qr.so is missing: run make -C oracle ref")
    out = {}
    names = []

    def add(kind, p, m, n, seed, full, medium=False):
        name = "%s_%s_%dx%d" % (kind, p, m, n)
        a = gen(ref, p, m, n, seed)
        e = {"p": p, "kind": kind, "m": m, "n": n, "seed": np.array(seed), "a_sum": a.sum(), "a_col0": a[:, 0].copy()}
        f = a.copy(order="F")
        tau = ref.xgeqrf(kind, p, m, n, f)
        e["tau"] = tau
        k = min(m, n)
        if not full:
            e["tri"] = tri(kind, f, m, n)
        else:
            if not medium:
                e["fac"] = f
            refl = reflectors(kind, f, m, n)
            nq_l = n if kind in ("lq", "rq") else m
            for side in "LR":
                shape = (nq_l, 5) if side == "L" else (5, nq_l)
                cseed = [7, 5, 3, 1] if side == "L" else [1, 3, 5, 7]
                c0 = gen(ref, p, shape[0], shape[1], cseed)
                e["c_%s" % side] = c0
                for trans in "NC":
                    c = c0.copy(order="F")
                    if kind == "lq" and side == "L" and k < 32:
                        # the reference's LQ::MultQ takes its unblocked route
                        # for k < 32, whose side-"L" reflector application
                        # (Reflector::Apply with vone and vconj,
                        # RNP/LA/Reflector.hpp:260-265) updates only the first
                        # column of C; record the product with the reference's
                        # own Q from its GenerateQ instead
                        Q = np.zeros((nq_l, nq_l), dtype=orc.DT[p], order="F")
                        Q[:k, :] = refl
                        tq = np.zeros(nq_l, dtype=orc.DT[p])
                        tq[:k] = tau
                        ref.xungqr(kind, p, nq_l, nq_l, k, Q, tq)
                        c = (Q if trans == "N" else Q.conj().T) @ c0
                        e["mq_L_from_genq"] = 1
                    else:
                        ref.xunmqr(kind, p, side, trans, shape[0], shape[1], k, refl, tau, c)
                    e["mq_%s%s" % (side, trans)] = np.asfortranarray(c)
            if (kind == "ql" and m >= n) or (kind != "ql" and m <= n):
                q = f.copy(order="F")
                ref.xungqr(kind, p, m, n, k, q, tau)
                if medium:
                    e["q_head"] = q[:, :8].copy()
                    e["q_tail"] = q[:, -8:].copy()
                else:
                    e["q"] = q
        for key, v in e.items():
            out["%s__%s" % (name, key)] = np.asarray(v)
        names.append(name)

    for kind in ("lq", "ql", "rq"):
        for p in "dz":
            for (m, n) in REF_SIZES[kind]:
                add(kind, p, m, n, [1, 2, 3, 5], full=False)
        for p in "sdcz":
            for (m, n) in ((40, 30), (30, 40)):
                add(kind, p, m, n, [3, 1, 4, 1], full=True)
        for (m, n) in ((300, 260), (260, 300)):
            add(kind, "d", m, n, [2, 7, 1, 8], full=True, medium=True)
    out["__cases__"] = np.array(names)
    path = os.path.join(HERE, "lqr_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(names), "cases")


if __name__ == "__main__":
    main()
