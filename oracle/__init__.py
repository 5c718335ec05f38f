"""ctypes binding of the CPU oracle (oracle/qr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg.  The product library never
uses it.  The restatement is pinned against golden vectors produced by the
reference itself (tests/golden/qr_golden.npz).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "liboracle_qr.so")
REFPATH = os.path.join(HERE, "_ref", "libref_qr.so")

SZ = C.c_size_t
DT = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}
PREFIX = {np.dtype(v): k for k, v in DT.items()}


def build():
    """Compile the restatement (make -C oracle); cheap when up to date."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIBPATH


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class QRLib:
    """Column-major QR routines of a CPU library with the oracle's (or the
    reference build's) extern "C" surface; matrices are Fortran-ordered numpy
    arrays of shape (ld, cols), logical sizes passed explicitly."""

    def __init__(self, path, prefix):
        self.lib = C.CDLL(path)
        self.pre = prefix

    def fn(self, p, name):
        return getattr(self.lib, "%s%s%s" % (self.pre, p, name))

    def larnv(self, p, dist, seed, n):
        x = np.zeros(n, dtype=DT[p])
        s = (C.c_int * 4)(*seed)
        self.fn(p, "larnv")(C.c_int(dist), s, SZ(n), ptr(x))
        return x, list(s)

    def geqrf(self, p, m, n, a):
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        lw = SZ(0)
        f = self.fn(p, "geqrf")
        f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
        w = np.zeros(max(lw.value, 1), dtype=DT[p])
        f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        return tau[: min(m, n)]

    def geqr2(self, p, m, n, a):
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        w = np.zeros(max(n, 1), dtype=DT[p])
        self.fn(p, "geqr2")(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(w))
        return tau[: min(m, n)]

    def unmqr(self, p, side, trans, m, n, k, a, tau, c, blocked=True):
        tau = np.ascontiguousarray(tau)
        args = (side.encode(), trans.encode(), SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(c), SZ(c.shape[0]))
        if blocked:
            lw = SZ(0)
            f = self.fn(p, "unmqr")
            f(*args, C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(*args, C.byref(lw), ptr(w))
        else:
            w = np.zeros(max(m, n, 1), dtype=DT[p])
            self.fn(p, "unm2r")(*args, ptr(w))

    def ungqr(self, p, m, n, k, a, tau, blocked=True):
        tau = np.ascontiguousarray(tau)
        if blocked:
            lw = SZ(0)
            f = self.fn(p, "ungqr")
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        else:
            w = np.zeros(max(n, 1), dtype=DT[p])
            self.fn(p, "ung2r")(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(w))

    # LQ / QL / RQ: kind in ("lq", "ql", "rq"); LAPACK-style names
    XNAMES = {"lq": ("gelqf", "unmlq", "unglq"), "ql": ("geqlf", "unmql", "ungql"), "rq": ("gerqf", "unmrq", "ungrq")}

    def xgeqrf(self, kind, p, m, n, a):
        """Factor of kind on a (Fortran-ordered, ld = a.shape[0]); returns tau."""
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        f = self.fn(p, self.XNAMES[kind][0])
        if self.pre == "ref_":
            lw = SZ(0)
            f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        else:
            f(SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau))
        return tau[: min(m, n)]

    def xunmqr(self, kind, p, side, trans, m, n, k, a, tau, c):
        """MultQ of kind: a holds the k reflectors (k x nq for lq/rq, nq x k for ql)."""
        tau = np.ascontiguousarray(tau)
        f = self.fn(p, self.XNAMES[kind][1])
        args = (side.encode(), trans.encode(), SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(c), SZ(c.shape[0]))
        if self.pre == "ref_":
            lw = SZ(0)
            f(*args, C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(*args, C.byref(lw), ptr(w))
        else:
            f(*args)

    def xungqr(self, kind, p, m, n, k, a, tau):
        tau = np.ascontiguousarray(tau)
        f = self.fn(p, self.XNAMES[kind][2])
        if self.pre == "ref_":
            lw = SZ(0)
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), None)
            w = np.zeros(max(lw.value, 1), dtype=DT[p])
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau), C.byref(lw), ptr(w))
        else:
            f(SZ(m), SZ(n), SZ(k), ptr(a), SZ(a.shape[0]), ptr(tau))

    def random_matrix(self, p, sym, dist, mode, reverse, cond, dmax, m, n, seed, d=None):
        """RNP::MatrixGen::RandomMatrix (real p only): returns (a, d, seed_out)."""
        R = C.c_double if p == "d" else C.c_float
        a = np.zeros((max(m, 1), max(n, 1)), dtype=DT[p], order="F")
        k = min(m, n)
        dd = np.zeros(max(k, 1), dtype=DT[p]) if d is None else np.array(d, dtype=DT[p])
        s = (C.c_int * 4)(*seed)
        self.fn(p, "random_matrix")(C.c_int(sym), C.c_int(dist), C.c_int(mode), C.c_int(reverse), R(cond), R(dmax), ptr(dd), SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), s)
        return a[:m, :n], dd[:k], list(s)

    # callers of QR / QL (Hessenberg and tridiagonal Q, generalized
    # eigensystem QR step); the reference build takes a workspace query first
    def _call_lw(self, f, args):
        if self.pre == "ref_":
            lw = SZ(0)
            f(*args, C.byref(lw), None)
            # generous: some of the reference's queries return less than the
            # blocked path then takes (Tridiagonal::MultQHerm asks nw*nb, its
            # QL::MultQ uses nw*nb + nb*nb and mis-sizes nb below that)
            w = np.zeros(max(lw.value, 1) + 65536, dtype=self._dt)
            lw = SZ(w.size)
            f(*args, C.byref(lw), ptr(w))
        else:
            f(*args)

    def gehrd(self, p, n, ilo, ihi, a):
        """Hessenberg::Reduce (reference build only); returns tau (n - 1)."""
        tau = np.zeros(max(n - 1, 1), dtype=DT[p])
        self._dt = DT[p]
        self._call_lw(self.fn(p, "gehrd"), (SZ(n), SZ(ilo), SZ(ihi), ptr(a), SZ(a.shape[0]), ptr(tau)))
        return tau[: max(n - 1, 0)]

    def unmhr(self, p, side, trans, m, n, ilo, ihi, a, tau, c):
        tau = np.ascontiguousarray(tau)
        self._dt = DT[p]
        self._call_lw(self.fn(p, "unmhr"), (side.encode(), trans.encode(), SZ(m), SZ(n), SZ(ilo), SZ(ihi), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(c), SZ(c.shape[0])))

    def unghr(self, p, n, ilo, ihi, a, tau):
        tau = np.ascontiguousarray(tau)
        self._dt = DT[p]
        self._call_lw(self.fn(p, "unghr"), (SZ(n), SZ(ilo), SZ(ihi), ptr(a), SZ(a.shape[0]), ptr(tau)))

    def hetrd(self, p, uplo, n, a):
        """Tridiagonal::ReduceHerm (reference build only); returns tau, diag, offdiag."""
        R = np.float32 if p in "sc" else np.float64
        tau = np.zeros(max(n - 1, 1), dtype=DT[p])
        d = np.zeros(max(n, 1), dtype=R)
        e = np.zeros(max(n - 1, 1), dtype=R)
        # one call with a workspace: ReduceHerm answers a query only when work
        # is given (RNP/LA/Tridiagonal.hpp:939-947) and reduces in place when
        # it is NULL
        w = np.zeros(64 * max(n, 1) + 65536, dtype=DT[p])
        lw = SZ(w.size)
        self.fn(p, "hetrd")(uplo.encode(), SZ(n), ptr(a), SZ(a.shape[0]), ptr(d), ptr(e), ptr(tau), C.byref(lw), ptr(w))
        return tau[: max(n - 1, 0)], d[:n], e[: max(n - 1, 0)]

    def unmtr(self, p, side, uplo, trans, m, n, a, tau, c):
        tau = np.ascontiguousarray(tau)
        self._dt = DT[p]
        self._call_lw(self.fn(p, "unmtr"), (side.encode(), uplo.encode(), trans.encode(), SZ(m), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(c), SZ(c.shape[0])))

    def ungtr(self, p, uplo, n, a, tau):
        tau = np.ascontiguousarray(tau)
        self._dt = DT[p]
        self._call_lw(self.fn(p, "ungtr"), (uplo.encode(), SZ(n), ptr(a), SZ(a.shape[0]), ptr(tau)))

    def gg_triangularize_b(self, p, n, ilo, ihi, a, b, vl=None, vr=None):
        """The complex generalized eigensystem's QR step (p in "cz"); returns tau (n)."""
        f = self.fn(p, "gg_triangularize_b")
        pv = lambda x: ptr(x) if x is not None else None
        ld = lambda x: SZ(x.shape[0] if x is not None else 1)
        head = (SZ(n), SZ(ilo), SZ(ihi), ptr(a), SZ(a.shape[0]), ptr(b), SZ(b.shape[0]), pv(vl), ld(vl), pv(vr), ld(vr))
        if self.pre == "ref_":
            w = np.zeros(n + 64 * max(n, 1) + 4096, dtype=DT[p])
            f(*head, SZ(w.size), ptr(w))
            return w[:n].copy()
        tau = np.zeros(max(n, 1), dtype=DT[p])
        f(*head, ptr(tau))
        return tau[:n]

    def gels(self, p, m, n, nrhs, a, b):
        """Least squares by Factor + MultQ("L","C") + triangular solve; a, b overwritten."""
        tau = np.zeros(max(min(m, n), 1), dtype=DT[p])
        self.fn(p, "gels")(SZ(m), SZ(n), SZ(nrhs), ptr(a), SZ(a.shape[0]), ptr(tau), ptr(b), SZ(b.shape[0]))
        return tau


def load():
    """The oracle restatement (built on demand)."""
    if not os.path.exists(LIBPATH) or os.path.getmtime(LIBPATH) < os.path.getmtime(os.path.join(HERE, "qr_oracle.cpp")):
        build()
    lib = QRLib(LIBPATH, "oracle_")
    lib.lib.oracle_use_blas.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
    lib.lib.oracle_use_blas.restype = C.c_int
    return lib


def use_blas(lib, path, prefix="scipy_", nthreads=0):
    """CPU baseline only: route the oracle's level-3 calls through an external
    Fortran BLAS (e.g. scipy's bundled OpenBLAS)."""
    return lib.lib.oracle_use_blas(path.encode() if path else None, prefix.encode(), nthreads)


def find_openblas():
    """Path of scipy's bundled OpenBLAS (LP64, "scipy_" symbols), or None."""
    try:
        import glob

        import scipy

        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        g = sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so")) + glob.glob(os.path.join(d, "libscipy_openblas.so")))
        return os.path.realpath(g[0]) if g else None
    except Exception:
        return None


def load_reference():
    """The reference itself (oracle/_ref/libref_qr.so), or None where the
    reference tree was not available to build it."""
    if not os.path.exists(REFPATH):
        return None
    return QRLib(REFPATH, "ref_")
