"""Generate golden vectors for the QR path from the REFERENCE ITSELF.

Runs RNP2's own RNP::LA::QR (Factor, Factor_unblocked, MultQ,
MultQ_unblocked, GenerateQ, GenerateQ_unblocked) and RNP::Random::
GenerateVector, compiled from the reference tree by ``make -C oracle ref``
into ``oracle/_ref/libref_qr.so``, and stores inputs and outputs in
``tests/golden/qr_golden.npz``.  The fixtures are committed; this script only
runs where the reference tree exists.

Cases:
  * the reference's own test sizes: tests/test_qr_tall.cpp (170x160) and
    tests/test_qr_fat.cpp (166x170), double and complex<double>, plus float
    and complex<float> for the FP32 form;
  * the 1024x256 double Factor + GenerateQ workload (seed {1,2,3,5});
  * edge cases: 1x1, 1xn, mx1, zero matrices, a zero column, tiny (subnormal)
    and huge columns, lda > m, sizes around the nb=32 block and the
    nx=128 crossover (RNP/LA/QR.hpp:41-51);
  * MultQ in all four side/trans combinations, blocked and unblocked;
  * a least-squares solve composed as Factor + MultQ("L","C") + SolveTrM.

Usage:  python tests/golden/make_golden.py   (after ``make -C oracle ref``)
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_qr.so")

SZ = C.c_size_t
DT = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Ref:
    def __init__(self, path=LIB):
        self.lib = C.CDLL(path)

    def larnv(self, p, dist, seed, n):
        """RNP::Random::GenerateVector; complex<float> is drawn as complex<double>
        and rounded (the reference's complex<float> generator does not compile)."""
        q = "z" if p == "c" else p
        x = np.zeros(n, dtype=DT[q])
        s = (C.c_int * 4)(*seed)
        getattr(self.lib, "ref_%slarnv" % q)(C.c_int(dist), s, SZ(n), ptr(x))
        return x.astype(DT[p]), list(s)

    # All matrices are Fortran-ordered buffers of shape (ld, cols); the logical
    # sizes are passed explicitly and ld = buffer rows.
    def geqrf(self, p, m, n, a):
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        lw = SZ(0)
        f = getattr(self.lib, "ref_%sgeqrf" % p)
        f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
        w = np.zeros(max(lw.value, 1), dtype=DT[p])
        f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        return tau[: min(m, n)]

    def geqr2(self, p, m, n, a):
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        w = np.zeros(max(n, 1), dtype=DT[p])
        getattr(self.lib, "ref_%sgeqr2" % p)(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(w))
        return tau[: min(m, n)]

    def unmqr(self, p, side, trans, m, n, k, a, tau, c, blocked=True):
        tau = np.ascontiguousarray(tau)
        args = (side.encode(), trans.encode(), SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(c), SZ(c.shape[0]))
        if blocked:
            lw = SZ(0)
            f = getattr(self.lib, "ref_%sunmqr" % p)
            f(*args, C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(*args, C.byref(lw), ptr(w))
        else:
            w = np.zeros(max(m, n, 1), dtype=DT[p])
            getattr(self.lib, "ref_%sunm2r" % p)(*args, ptr(w))

    def ungqr(self, p, m, n, k, a, tau, blocked=True):
        tau = np.ascontiguousarray(tau)
        if blocked:
            lw = SZ(0)
            f = getattr(self.lib, "ref_%sungqr" % p)
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        else:
            w = np.zeros(max(n, 1), dtype=DT[p])
            getattr(self.lib, "ref_%sung2r" % p)(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(w))

    def trsm(self, p, n, nrhs, a, b):
        getattr(self.lib, "ref_%strsm_lunn" % p)(SZ(n), SZ(nrhs), ptr(a), SZ(a.shape[0]), ptr(b), SZ(b.shape[0]))


def fmat(ref, p, m, n, seed, dist=1, lda=None):
    """Column-major m-by-n matrix (leading dimension lda) filled column by column
    with GenerateVector, like tests/test_qr_tall.cpp:13-15."""
    lda = lda or m
    buf = np.zeros((max(lda, 1), max(n, 1)), dtype=DT[p], order="F")
    vals, seed_out = ref.larnv(p, dist, seed, m * n)
    buf[:m, :n] = vals.reshape(n, m).T
    return buf, seed_out


def main():
    if not os.path.exists(LIB):
        sys.exit("build the reference first: make -C oracle ref")
    ref = Ref()
    out = {}
    cases = []

    def add_qr_case(name, p, m, n, seed, dist=1, lda=None, mutate=None, genq=True, multq=True, unblocked=True, store_full=True, drop=()):
        buf, _ = fmat(ref, p, m, n, seed, dist, lda)
        if mutate is not None:
            mutate(buf, m, n)
        a0 = buf.copy(order="F")
        fac = buf.copy(order="F")
        tau = ref.geqrf(p, m, n, fac)
        k = min(m, n)
        entry = {"p": p, "m": m, "n": n, "lda": buf.shape[0], "seed": np.array(seed), "dist": dist}
        entry["a"] = a0
        entry["fac"] = fac
        entry["tau"] = tau
        if unblocked:
            fac2 = a0.copy(order="F")
            entry["tau_unblocked"] = ref.geqr2(p, m, n, fac2)
            entry["fac_unblocked"] = fac2
        if genq and k > 0:
            # tall: Q is m-by-n with k = n; fat: Q is m-by-m with k = m,
            # as tests/test_qr_tall.cpp:143-146 and tests/test_qr_fat.cpp:143-146 do
            nq = n if m >= n else m
            q = np.asfortranarray(fac[:, :nq].copy())
            ref.ungqr(p, m, nq, k, q, tau)
            entry["q"] = q[:m, :]
            if unblocked:
                q2 = np.asfortranarray(fac[:, :nq].copy())
                ref.ungqr(p, m, nq, k, q2, tau, blocked=False)
                entry["q_unblocked"] = q2[:m, :]
        if multq and k > 0:
            nc = 7
            cl, _ = fmat(ref, p, m, nc, [7, 7, 7, 9])
            cr, _ = fmat(ref, p, nc, m, [9, 9, 9, 11])
            entry["c_left"] = cl
            entry["c_right"] = cr
            for side, c0 in (("L", cl), ("R", cr)):
                cm, cn = c0.shape
                for trans in ("N", "C"):
                    for blocked in (True, False):
                        c = c0.copy(order="F")
                        ref.unmqr(p, side, trans, cm, cn, k, fac, tau, c, blocked)
                        entry["mq_%s%s%s" % (side, trans, "" if blocked else "_unblocked")] = c
        if not store_full:
            # keep only what the tests compare at this size
            a = entry.pop("a")
            entry["a_sum"] = np.array(a[:m, :n].sum())
            entry["a_col0"] = a[:m, 0]
            entry.pop("fac_unblocked", None)
            entry.pop("q_unblocked", None)
            r = entry.pop("fac")[:k, :]
            entry["r_packed"] = r[np.triu_indices(k, 0, r.shape[1])]
            q = entry.pop("q")
            entry["q_head"] = q[:, :16]
            entry["q_tail"] = q[:, -16:]
        if mutate is None and m * n > 4096 and "a" in entry:
            # the input is regenerated exactly from the seed by the oracle's
            # restated generator; keep a checksum to prove it
            a = entry.pop("a")
            entry["a_sum"] = np.array(a[:m, :n].sum())
            entry["a_col0"] = a[:m, 0]
        for key in drop:
            entry.pop(key, None)
        for key, val in entry.items():
            out["%s__%s" % (name, key)] = np.asarray(val)
        cases.append(name)

    S = [1, 2, 3, 5]
    for p in ("d", "z", "s", "c"):
        add_qr_case("tall_%s" % p, p, 170, 160, S, unblocked=False, multq=p in "dz")
        add_qr_case("fat_%s" % p, p, 166, 170, S, unblocked=False, multq=p in "dz")
    add_qr_case("blocked_d", "d", 300, 260, S, unblocked=False, genq=False, multq=False)
    add_qr_case("blocked_z", "z", 200, 170, S, unblocked=False, genq=False, multq=False)
    for p in ("d", "z"):
        add_qr_case("normal_%s" % p, p, 96, 40, S, dist=2)
        add_qr_case("lda_%s" % p, p, 40, 30, S, lda=48)
        for (m, n) in ((1, 1), (1, 5), (5, 1), (2, 2), (3, 7), (33, 1), (65, 33), (33, 65), (64, 32), (31, 33)):
            add_qr_case("shape_%dx%d_%s" % (m, n, p), p, m, n, S)
        if p == "d":
            add_qr_case("shape_200x129_%s" % p, p, 200, 129, S, unblocked=False, drop=("q",))
            add_qr_case("shape_129x200_%s" % p, p, 129, 200, S, unblocked=False, drop=("q",))

        def zero_all(b, m, n):
            b[:m, :n] = 0

        def zero_col(b, m, n):
            b[:m, 3] = 0

        def tiny_col(b, m, n):
            b[:m, 0] *= 1e-310
            b[:m, 2] *= 1e-300

        def huge_col(b, m, n):
            b[:m, 1] *= 1e300

        add_qr_case("zeros_%s" % p, p, 10, 5, S, mutate=zero_all)
        add_qr_case("zerocol_%s" % p, p, 20, 8, S, mutate=zero_col)
        add_qr_case("tiny_%s" % p, p, 20, 8, S, mutate=tiny_col)
        add_qr_case("huge_%s" % p, p, 20, 8, S, mutate=huge_col)
    # the 1024x256 double Factor + GenerateQ workload
    add_qr_case("c1_d", "d", 1024, 256, S, multq=False, unblocked=False, store_full=False)

    # least squares: Factor, MultQ("L","C") on B, SolveTrM("L","U","N","N")
    for p in ("d", "z"):
        m, n, nrhs = 300, 40, 3
        a, _ = fmat(ref, p, m, n, [3, 1, 4, 1], dist=2)
        b, _ = fmat(ref, p, m, nrhs, [2, 7, 1, 9], dist=2)
        fac = a.copy(order="F")
        tau = ref.geqrf(p, m, n, fac)
        qb = b.copy(order="F")
        ref.unmqr(p, "L", "C", m, nrhs, n, fac, tau, qb)
        x = np.asfortranarray(qb[:n, :].copy())
        ref.trsm(p, n, nrhs, fac, x)
        name = "ls_%s" % p
        for key, val in {"p": p, "m": m, "n": n, "nrhs": nrhs, "a_sum": a[:m, :n].sum(), "b_sum": b.sum(), "x": x}.items():
            out["%s__%s" % (name, key)] = np.asarray(val)
        cases.append(name)

    # generator vectors (RNP/Random.hpp): first 300 draws per distribution
    for p in ("s", "d", "z"):
        for dist in (0, 1, 2):
            v, s_out = ref.larnv(p, dist, S, 300)
            out["rng_%s_%d__x" % (p, dist)] = v
            out["rng_%s_%d__seed_out" % (p, dist)] = np.array(s_out)
    out["__cases__"] = np.array(cases)
    path = os.path.join(HERE, "qr_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%d cases, %.1f MB)" % (path, len(cases), os.path.getsize(path) / 1e6))


if __name__ == "__main__":
    main()
