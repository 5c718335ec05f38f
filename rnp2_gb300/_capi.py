"""ctypes binding of the C ABI declared in include/rnp_gpu/qr_gb300.h.

The library must have been built (``python -m rnp2_gb300._build`` or
``__graft_entry__.build()``); there is no fallback implementation, so a
missing library raises immediately.
"""
import ctypes as C
import os

from ._build import LIBPATH

SZ = C.c_size_t
P = C.c_void_p
CH = C.c_char_p
PSZ = C.POINTER(C.c_size_t)

_lib = None


class RefineInfo(C.Structure):
    """rnpgpu_refine_info (include/rnp_gpu/ls_gb300.h)"""

    _fields_ = [
        ("iterations", C.c_int),
        ("converged", C.c_int),
        ("backward_error", C.c_double),
        ("normal_residual", C.c_double),
        ("correction", C.c_double),
        ("anorm", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LibraryNotBuilt(RuntimeError):
    pass


def _signatures():
    sig = {}
    for p in "sdcz":
        sig["rnpgpu_%sgeqrf" % p] = [SZ, SZ, P, SZ, P, PSZ, P]
        sig["rnpgpu_%sgeqr2" % p] = [SZ, SZ, P, SZ, P, P]
        sig["rnpgpu_%sunmqr" % p] = [CH, CH, SZ, SZ, SZ, P, SZ, P, P, SZ, PSZ, P]
        sig["rnpgpu_%sunm2r" % p] = [CH, CH, SZ, SZ, SZ, P, SZ, P, P, SZ, P]
        sig["rnpgpu_%sungqr" % p] = [SZ, SZ, SZ, P, SZ, P, PSZ, P]
        sig["rnpgpu_%sung2r" % p] = [SZ, SZ, SZ, P, SZ, P, P]
        sig["rnpgpu_%strsm_lunn" % p] = [SZ, SZ, P, SZ, P, SZ]
        sig["rnpgpu_%sgels" % p] = [SZ, SZ, SZ, P, SZ, P, P, SZ, PSZ, P]
        for f, mq, g in (("gelqf", "unmlq", "unglq"), ("geqlf", "unmql", "ungql"), ("gerqf", "unmrq", "ungrq")):
            sig["rnpgpu_%s%s" % (p, f)] = [SZ, SZ, P, SZ, P, PSZ, P]
            sig["rnpgpu_%s%s" % (p, mq)] = [CH, CH, SZ, SZ, SZ, P, SZ, P, P, SZ, PSZ, P]
            sig["rnpgpu_%s%s" % (p, g)] = [SZ, SZ, SZ, P, SZ, P, PSZ, P]
        sig["rnpgpu_%sunmhr" % p] = [CH, CH, SZ, SZ, SZ, SZ, P, SZ, P, P, SZ, PSZ, P]
        sig["rnpgpu_%sunghr" % p] = [SZ, SZ, SZ, P, SZ, P, PSZ, P]
        sig["rnpgpu_%sungtr" % p] = [CH, SZ, P, SZ, P, PSZ, P]
        sig["rnpgpu_%sunmtr" % p] = [CH, CH, CH, SZ, SZ, P, SZ, P, P, SZ, PSZ, P]
    for p in "cz":
        sig["rnpgpu_%sgg_triangularize_b" % p] = [SZ, SZ, SZ, P, SZ, P, SZ, P, SZ, P, SZ, PSZ, P]
    for name in ("rnpgpu_dsgels", "rnpgpu_zcgels", "rnpgpu_dsgels_host"):
        sig[name] = [SZ, SZ, SZ, P, SZ, P, SZ, P, SZ, C.c_int, C.c_int, C.POINTER(RefineInfo), PSZ, P]
    sig["rnpgpu_srandom_matrix"] = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, P, SZ, SZ, P, SZ, C.POINTER(C.c_int), PSZ, P]
    sig["rnpgpu_drandom_matrix"] = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, P, SZ, SZ, P, SZ, C.POINTER(C.c_int), PSZ, P]
    sig["rnpgpu_dls_residual"] = [SZ, SZ, SZ, P, SZ, P, SZ, P, SZ, P, SZ, P, SZ, P, PSZ]
    sig["rnpgpu_set_stream"] = [P]
    sig["rnpgpu_get_stream"] = []
    sig["rnpgpu_get_last_error"] = []
    sig["rnpgpu_version"] = []
    sig["rnpgpu_launch_count"] = []
    sig["rnpgpu_device_status"] = [C.c_int]
    sig["rnpgpu_sgemm_tc"] = [CH, CH, SZ, SZ, SZ, C.c_float, P, SZ, P, SZ, C.c_float, P, SZ]
    sig["rnpgpu_sgeqrf_mixed"] = [SZ, SZ, P, SZ, P, P, C.c_int, C.POINTER(C.c_int), PSZ, P]
    sig["rnpgpu_timing_enable"] = [C.c_int]
    sig["rnpgpu_timing_report"] = [C.c_char_p, SZ]
    sig["rnpgpu_probe_peak"] = [C.c_int, P, SZ, C.POINTER(C.c_double)]
    return sig


RESTYPES = {"rnpgpu_get_stream": P, "rnpgpu_get_last_error": CH, "rnpgpu_version": CH, "rnpgpu_launch_count": C.c_ulonglong}


def timing_report():
    """{kernel class: (launches, total ms)} since the last report."""
    buf = C.create_string_buffer(1 << 16)
    lib().rnpgpu_timing_report(buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


def lib():
    """The loaded library; raises LibraryNotBuilt if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise LibraryNotBuilt("%s is missing: build it with __graft_entry__.build()" % LIBPATH)
        l = C.CDLL(LIBPATH)
        for name, args in _signatures().items():
            f = getattr(l, name)
            f.argtypes = args
            f.restype = RESTYPES.get(name, C.c_int)
        _lib = l
    return _lib


def exported_names():
    return sorted(_signatures().keys())
