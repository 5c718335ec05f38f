"""Golden vectors for the reference's callers of QR / QL, from the REFERENCE ITSELF.

Runs RNP2's own RNP::LA::Hessenberg::{Reduce, MultQ, GenerateQ},
RNP::LA::Tridiagonal::{ReduceHerm, MultQHerm, GenerateQHerm} and the QR step
of ComplexGeneralizedEigensystem (the reference's calls of
RNP/LA/GeneralizedEigensystems.hpp:457-472 in their order), compiled from the
reference tree by ``make -C oracle ref`` into ``oracle/_ref/libref_qr.so``, on
inputs drawn with the reference's generator, and stores the inputs of the
QR-calling routines (the reductions' outputs) and their outputs in
``tests/golden/consumers_golden.npz``.  The fixtures are committed; this
script only runs where the reference tree exists.

Cases:
  * Hessenberg, all four types, n = 40 with (ilo, ihi) = (0, 40) and (3, 35):
    the reduction, tau, MultQ in all four side/trans combinations and
    GenerateQ; double and complex<double>, n = 200, (0, 200) (past the
    nb = 32 block and nx = 128 crossover): MultQ and the first and last 8
    columns of GenerateQ;
  * Tridiagonal (Hermitian input A + A^H), all four types, n = 40, uplo "U"
    and "L": the reduction, tau, MultQHerm in all four combinations and
    GenerateQHerm; double and complex<double>, n = 200: the same with Q's
    first and last 8 columns;
  * the generalized eigensystem's QR step, complex types: n = 40 with
    (ilo, ihi) = (2, 37) and both vector matrices, n = 40 with (0, 40) and
    none; complex<double>, n = 150, (5, 140), left vectors only.

Usage:  python tests/golden/make_consumers_golden.py   (after ``make -C oracle ref``)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as orc  # noqa: E402


def gen(ref, p, m, n, seed):
    """m x n Fortran matrix from the reference's generator (normal entries;
    complex<float> drawn as complex<double> and rounded)."""
    q = "z" if p == "c" else ("d" if p == "s" else p)
    vals, _ = ref.larnv(q, 2, seed, m * n)
    return np.asfortranarray(vals.astype(orc.DT[p]).reshape(n, m).T)


def main():
    ref = orc.load_reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_qr.so is missing: run make -C oracle ref")
    out = {}
    names = []

    def put(name, e):
        for key, v in e.items():
            out["%s__%s" % (name, key)] = np.asarray(v)
        names.append(name)

    def multq_cases(e, p, n, call):
        for side in "LR":
            shape = (n, 5) if side == "L" else (5, n)
            c0 = gen(ref, p, shape[0], shape[1], [7, 5, 3, 1] if side == "L" else [1, 3, 5, 7])
            e["c_%s" % side] = c0
            for trans in "NC":
                c = c0.copy(order="F")
                call(side, trans, shape[0], shape[1], c)
                e["mq_%s%s" % (side, trans)] = c

    def q_out(e, q, medium):
        if medium:
            e["q_head"] = q[:, :8].copy()
            e["q_tail"] = q[:, -8:].copy()
        else:
            e["q"] = q

    # Hessenberg::Reduce -> MultQ / GenerateQ
    def hess(p, n, ilo, ihi, medium=False):
        name = "hess_%s_%d_%d_%d" % (p, n, ilo, ihi)
        a = gen(ref, p, n, n, [3, 1, 4, 1])
        tau = ref.gehrd(p, n, ilo, ihi, a)
        e = {"p": p, "n": n, "ilo": ilo, "ihi": ihi, "red": a.copy(), "tau": tau}
        multq_cases(e, p, n, lambda side, trans, m_, n_, c: ref.unmhr(p, side, trans, m_, n_, ilo, ihi, a, tau, c))
        q = a.copy(order="F")
        ref.unghr(p, n, ilo, ihi, q, tau)
        q_out(e, q, medium)
        put(name, e)

    # Tridiagonal::ReduceHerm -> MultQHerm / GenerateQHerm
    def trid(p, n, uplo, medium=False):
        name = "trid_%s_%d_%s" % (p, n, uplo)
        x = gen(ref, p, n, n, [2, 7, 1, 8])
        a = np.asfortranarray(x + x.conj().T)
        tau, d, off = ref.hetrd(p, uplo, n, a)
        e = {"p": p, "n": n, "uplo": uplo, "red": a.copy(), "tau": tau, "d": d, "e": off}
        multq_cases(e, p, n, lambda side, trans, m_, n_, c: ref.unmtr(p, side, uplo, trans, m_, n_, a, tau, c))
        q = a.copy(order="F")
        ref.ungtr(p, uplo, n, q, tau)
        q_out(e, q, medium)
        put(name, e)

    # the generalized eigensystem's QR step
    def gg(p, n, ilo, ihi, want_vl, want_vr):
        name = "gg_%s_%d_%d_%d_%d%d" % (p, n, ilo, ihi, want_vl, want_vr)
        a = gen(ref, p, n, n, [1, 1, 2, 3])
        b = gen(ref, p, n, n, [5, 8, 13, 21])
        e = {"p": p, "n": n, "ilo": ilo, "ihi": ihi, "want_vl": want_vl, "want_vr": want_vr, "a_in": a.copy(), "b_in": b.copy()}
        vl = np.full((n, n), 7.0, dtype=orc.DT[p], order="F") if want_vl else None
        vr = np.full((n, n), 7.0, dtype=orc.DT[p], order="F") if want_vr else None
        tau = ref.gg_triangularize_b(p, n, ilo, ihi, a, b, vl, vr)
        e.update({"a": a, "b": b, "tau": tau})
        if want_vl:
            e["vl"] = vl
        if want_vr:
            e["vr"] = vr
        put(name, e)

    for p in "sdcz":
        hess(p, 40, 0, 40)
        hess(p, 40, 3, 35)
        for uplo in "UL":
            trid(p, 40, uplo)
    for p in "dz":
        hess(p, 200, 0, 200, medium=True)
        for uplo in "UL":
            trid(p, 200, uplo, medium=True)
    for p in "cz":
        gg(p, 40, 2, 37, 1, 1)
        gg(p, 40, 0, 40, 0, 0)
    gg("z", 150, 5, 140, 1, 0)
    out["__cases__"] = np.array(names)
    path = os.path.join(HERE, "consumers_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(names), "cases")


if __name__ == "__main__":
    main()
