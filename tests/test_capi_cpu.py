"""C ABI checks that need no GPU: the library builds for sm_103a, loads, exports
every entry point its header declares, answers workspace queries and rejects
invalid arguments before enqueuing any work."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "include", "rnp_gpu")


@pytest.fixture(scope="module")
def lib():
    from rnp2_gb300 import _build

    _build.build()
    from rnp2_gb300._capi import lib as load

    return load()


def declared_symbols():
    names = set()
    for f in os.listdir(HEADER_DIR):
        if f.endswith(".h"):
            txt = open(os.path.join(HEADER_DIR, f)).read()
            names.update(re.findall(r"\b(rnpgpu_\w+)\s*\(", txt))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 28
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version(lib):
    assert b"sm_103a" in lib.rnpgpu_version()


@pytest.mark.parametrize("p", "sdcz")
def test_workspace_queries(lib, p):
    lw = C.c_size_t(0)
    rc = getattr(lib, "rnpgpu_%sgeqrf" % p)(1024, 256, None, 1024, None, C.byref(lw), None)
    assert rc == 0 and lw.value >= 32 * 256
    lw = C.c_size_t(0)
    rc = getattr(lib, "rnpgpu_%sunmqr" % p)(b"L", b"C", 4096, 64, 4096, None, 4096, None, None, 4096, C.byref(lw), None)
    assert rc == 0 and lw.value >= 32 * 64
    lw = C.c_size_t(0)
    rc = getattr(lib, "rnpgpu_%sungqr" % p)(1024, 256, 256, None, 1024, None, C.byref(lw), None)
    assert rc == 0 and lw.value >= 32 * 256


def test_quick_returns_touch_nothing(lib):
    # k = min(m, n) = 0: the reference returns before the query (RNP/LA/QR.hpp:136-139)
    lw = C.c_size_t(7)
    assert lib.rnpgpu_dgeqrf(0, 5, None, 1, None, C.byref(lw), None) == 0
    assert lw.value == 7
    assert lib.rnpgpu_dunmqr(b"L", b"N", 0, 3, 0, None, 1, None, None, 1, C.byref(lw), None) == 0
    assert lib.rnpgpu_dungqr(4, 0, 0, None, 4, None, C.byref(lw), None) == 0


def test_invalid_arguments_are_rejected(lib):
    lw = C.c_size_t(0)
    # lda < m
    assert lib.rnpgpu_dgeqrf(10, 5, None, 9, None, C.byref(lw), None) == -4
    # NULL lwork
    assert lib.rnpgpu_dgeqrf(10, 5, None, 10, None, None, None) == -6
    # workspace given but no matrix
    lw = C.c_size_t(1 << 20)
    assert lib.rnpgpu_dgeqrf(10, 5, None, 10, None, C.byref(lw), C.c_void_p(256)) == -3
    # k > nq for MultQ, lda < nq, ldc < m
    lw = C.c_size_t(0)
    assert lib.rnpgpu_zunmqr(b"L", b"C", 10, 4, 11, None, 10, None, None, 10, C.byref(lw), None) == -5
    assert lib.rnpgpu_zunmqr(b"R", b"C", 10, 4, 2, None, 3, None, None, 10, C.byref(lw), None) == -7
    assert lib.rnpgpu_zunmqr(b"L", b"C", 10, 4, 2, None, 10, None, None, 9, C.byref(lw), None) == -10
    # GenerateQ needs m >= n >= k
    assert lib.rnpgpu_sungqr(4, 5, 2, None, 4, None, C.byref(lw), None) == -2
    assert lib.rnpgpu_sungqr(8, 5, 6, None, 8, None, C.byref(lw), None) == -3
    # unblocked forms validate their pointers before launching
    assert lib.rnpgpu_dgeqr2(10, 5, None, 10, None, None) == -3
    assert lib.rnpgpu_cung2r(8, 5, 5, None, 8, None, None) == -4


def test_workspace_shrinks_then_rejects(lib):
    # a workspace below the blocked requirement but >= n takes the level-2 path;
    # below n it is an lwork error (argument 6), never an out-of-bounds write
    lw = C.c_size_t(3)
    assert lib.rnpgpu_dgeqrf(10, 5, C.c_void_p(256), 10, C.c_void_p(512), C.byref(lw), C.c_void_p(1024)) == -6


def test_consumer_arguments_are_rejected(lib):
    """Hessenberg / tridiagonal Q and the generalized QR step validate their
    arguments before any device work (argument positions as the reference's
    signatures)."""
    lw = C.c_size_t(0)
    # Hessenberg::MultQ: ilo > nq, ihi <= ilo, lda < nq, ldc < m
    assert lib.rnpgpu_dunmhr(b"L", b"N", 10, 4, 11, 12, None, 10, None, None, 10, C.byref(lw), None) == -5
    assert lib.rnpgpu_dunmhr(b"L", b"N", 10, 4, 3, 3, None, 10, None, None, 10, C.byref(lw), None) == -6
    assert lib.rnpgpu_zunmhr(b"R", b"C", 4, 10, 0, 10, None, 9, None, None, 4, C.byref(lw), None) == -8
    assert lib.rnpgpu_sunmhr(b"L", b"N", 10, 4, 0, 10, None, 10, None, None, 9, C.byref(lw), None) == -11
    assert lib.rnpgpu_cunmhr(b"X", b"N", 10, 4, 0, 10, None, 10, None, None, 10, C.byref(lw), None) == -1
    assert lib.rnpgpu_dunmhr(b"L", b"N", 10, 4, 0, 10, None, 10, None, None, 10, None, None) == -12
    # Hessenberg::GenerateQ: ihi > n, lda < n; the query answers
    assert lib.rnpgpu_dunghr(10, 2, 11, None, 10, None, C.byref(lw), None) == -3
    assert lib.rnpgpu_zunghr(10, 0, 10, None, 9, None, C.byref(lw), None) == -5
    lw = C.c_size_t(0)
    assert lib.rnpgpu_dunghr(300, 0, 300, None, 300, None, C.byref(lw), None) == 0 and lw.value >= 299
    # Tridiagonal::GenerateQHerm / MultQHerm
    assert lib.rnpgpu_dungtr(b"X", 10, None, 10, None, C.byref(lw), None) == -1
    assert lib.rnpgpu_cungtr(b"U", 10, None, 9, None, C.byref(lw), None) == -4
    assert lib.rnpgpu_dunmtr(b"L", b"U", b"N", 10, 4, None, 9, None, None, 10, C.byref(lw), None) == -7
    assert lib.rnpgpu_zunmtr(b"L", b"L", b"Q", 10, 4, None, 10, None, None, 10, C.byref(lw), None) == -3
    lw = C.c_size_t(0)
    assert lib.rnpgpu_zungtr(b"U", 200, None, 200, None, C.byref(lw), None) == 0 and lw.value >= 199
    # the generalized step: ihi > n, ldb < n, a missing workspace length
    assert lib.rnpgpu_zgg_triangularize_b(10, 0, 11, None, 10, None, 10, None, 1, None, 1, C.byref(lw), None) == -3
    assert lib.rnpgpu_zgg_triangularize_b(10, 0, 10, None, 10, None, 9, None, 1, None, 1, C.byref(lw), None) == -7
    assert lib.rnpgpu_cgg_triangularize_b(10, 0, 10, None, 10, None, 10, None, 1, None, 1, None, None) == -12
    lw = C.c_size_t(0)
    assert lib.rnpgpu_zgg_triangularize_b(100, 0, 100, None, 100, None, 100, None, 1, None, 1, C.byref(lw), None) == 0 and lw.value > 100


def test_host_buffer_solve_arguments_are_rejected(lib):
    """rnpgpu_dsgels_host checks its shapes and leading dimensions before any
    device call (argument positions as in ls_gb300.h)."""
    lw = C.c_size_t(0)
    # m < n, lda < m, ldb < m, ldx < n, no workspace length
    assert lib.rnpgpu_dsgels_host(10, 11, 1, None, 10, None, 10, None, 11, 0, 0, None, C.byref(lw), None) == -2
    assert lib.rnpgpu_dsgels_host(10, 4, 1, None, 9, None, 10, None, 4, 0, 0, None, C.byref(lw), None) == -5
    assert lib.rnpgpu_dsgels_host(10, 4, 1, None, 10, None, 9, None, 4, 0, 0, None, C.byref(lw), None) == -7
    assert lib.rnpgpu_dsgels_host(10, 4, 1, None, 10, None, 10, None, 3, 0, 0, None, C.byref(lw), None) == -9
    assert lib.rnpgpu_dsgels_host(10, 4, 1, None, 10, None, 10, None, 4, 0, 0, None, None, None) == -13
    # an empty problem returns at once and leaves the length alone
    lw = C.c_size_t(5)
    assert lib.rnpgpu_dsgels_host(0, 0, 1, None, 1, None, 1, None, 1, 0, 0, None, C.byref(lw), None) == 0
    assert lw.value == 5
