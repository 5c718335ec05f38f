"""Batched Householder QR and least squares (include/rnp_gpu/batched_gb300.h)
for torch CUDA tensors: many uneven matrices packed in one buffer, factored
(and solved) by one plan."""
import ctypes as C

import torch

from ._capi import lib
from .qr import RNPGPUError, _bind_stream

_TYPE = {torch.float32: (0, "s"), torch.float64: (1, "d"), torch.complex64: (2, "c"), torch.complex128: (3, "z")}


def _setup(L):
    P = C.c_void_p
    if getattr(L, "_batched_ready", False):
        return
    L.rnpgpu_geqrf_batched_plan.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, C.POINTER(C.c_size_t), C.POINTER(P)]
    L.rnpgpu_geqrf_batched_plan.restype = C.c_int
    L.rnpgpu_gels_batched_plan.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, C.POINTER(C.c_size_t), C.POINTER(P)]
    L.rnpgpu_gels_batched_plan.restype = C.c_int
    L.rnpgpu_batch_plan_destroy.argtypes = [P]
    L.rnpgpu_batch_plan_config.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.rnpgpu_batch_plan_set_config.argtypes = [P, C.c_int, C.c_int, C.c_int]
    L.rnpgpu_batch_plan_set_config.restype = C.c_int
    for p in "sdcz":
        f = getattr(L, "rnpgpu_%sgeqrf_batched" % p)
        f.argtypes = [P, P, P]
        f.restype = C.c_int
        f = getattr(L, "rnpgpu_%sgeqrf_batched_tune" % p)
        f.argtypes = [P, P, P, C.POINTER(C.c_double)]
        f.restype = C.c_int
        f = getattr(L, "rnpgpu_%sgels_batched" % p)
        f.argtypes = [P, P, P, P, P]
        f.restype = C.c_int
    for name in ("rnpgpu_dsgels_batched", "rnpgpu_zcgels_batched"):
        f = getattr(L, name)
        f.argtypes = [P, P, P, P, C.c_int, P, P, P, P, C.POINTER(C.c_size_t)]
        f.restype = C.c_int
        f = getattr(L, name + "_tune")
        f.argtypes = [P, P, P, C.POINTER(C.c_size_t), C.POINTER(C.c_double)]
        f.restype = C.c_int
    L._batched_ready = True


class BatchedQR:
    """Packed batch of column-major matrices m[i] x n[i] (lda = m[i]).

    ``a`` (1-D tensor) holds the matrices back to back, ``tau`` their tau
    vectors; ``matrix(i)`` / ``tau_of(i)`` are views.  ``factor()`` runs the
    persistent batched kernels; ``tune()`` picks the block shapes."""

    def __init__(self, ms, ns, dtype=torch.float64, device="cuda"):
        import numpy as np

        self.ms = [int(x) for x in ms]
        self.ns = [int(x) for x in ns]
        self.dtype = dtype
        self.type, self.p = _TYPE[dtype]
        sizes = np.array([m * n for m, n in zip(self.ms, self.ns)], dtype=np.int64)
        ks = np.array([min(m, n) for m, n in zip(self.ms, self.ns)], dtype=np.int64)
        self.a_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        self.t_off = np.concatenate([[0], np.cumsum(ks)[:-1]]).astype(np.int64)
        self.a = torch.zeros(int(sizes.sum()) or 1, dtype=dtype, device=device)
        self.tau = torch.zeros(int(ks.sum()) or 1, dtype=dtype, device=device)
        L = lib()
        _setup(L)
        self._L = L
        m32 = np.array(self.ms, dtype=np.int32)
        n32 = np.array(self.ns, dtype=np.int32)
        self._keep = (m32, n32, self.a_off, self.t_off)
        lw = C.c_size_t(0)
        plan = C.c_void_p()
        _bind_stream()
        args = (self.type, len(self.ms), m32.ctypes.data, n32.ctypes.data, m32.ctypes.data, self.a_off.ctypes.data, self.t_off.ctypes.data)
        rc = L.rnpgpu_geqrf_batched_plan(*args, None, C.byref(lw), C.byref(plan))
        if rc:
            raise RNPGPUError("geqrf_batched_plan", rc)
        self.work = torch.empty(max(lw.value, 1), dtype=torch.uint8, device=device)
        rc = L.rnpgpu_geqrf_batched_plan(*args, self.work.data_ptr(), C.byref(lw), C.byref(plan))
        if rc:
            raise RNPGPUError("geqrf_batched_plan", rc)
        self.plan = plan

    def matrix(self, i):
        m, n, o = self.ms[i], self.ns[i], int(self.a_off[i])
        return self.a[o:o + m * n].view(n, m).t()

    def tau_of(self, i):
        o = int(self.t_off[i])
        return self.tau[o:o + min(self.ms[i], self.ns[i])]

    def factor(self):
        _bind_stream()
        rc = getattr(self._L, "rnpgpu_%sgeqrf_batched" % self.p)(self.plan, self.a.data_ptr(), self.tau.data_ptr())
        if rc:
            raise RNPGPUError("geqrf_batched", rc)

    def tune(self, scratch_a=None, scratch_tau=None):
        """Autotune the block shapes on a scratch copy; returns the best time (ms)."""
        sa = self.a.clone() if scratch_a is None else scratch_a
        st = self.tau.clone() if scratch_tau is None else scratch_tau
        ms = C.c_double(0)
        _bind_stream()
        rc = getattr(self._L, "rnpgpu_%sgeqrf_batched_tune" % self.p)(self.plan, sa.data_ptr(), st.data_ptr(), C.byref(ms))
        if rc:
            raise RNPGPUError("geqrf_batched_tune", rc)
        return ms.value

    def config(self, cls):
        t, nb, cnt = C.c_int(), C.c_int(), C.c_int()
        self._L.rnpgpu_batch_plan_config(self.plan, cls, C.byref(t), C.byref(nb), C.byref(cnt))
        return {"threads": t.value, "nb": nb.value, "count": cnt.value}

    def force_config(self, cls, threads, nb):
        """Pin the block shape of a size class (one of the autotuner's candidates)."""
        rc = self._L.rnpgpu_batch_plan_set_config(self.plan, cls, threads, nb)
        if rc:
            raise RNPGPUError("batch_plan_set_config", rc)

    def __del__(self):
        try:
            if getattr(self, "plan", None):
                self._L.rnpgpu_batch_plan_destroy(self.plan)
                self.plan = None
        except Exception:
            pass


_MIXED = {torch.float64: "rnpgpu_dsgels_batched", torch.complex128: "rnpgpu_zcgels_batched"}


class BatchedLS:
    """Packed batch of least-squares problems min ||A_i x_i - b_i||, one
    right-hand side each (m[i] >= n[i], lda = m[i]).

    ``a``, ``b`` and ``x`` (1-D tensors) hold the matrices, right-hand sides
    and solutions back to back; ``matrix(i)``, ``rhs(i)`` and ``solution(i)``
    are views.  ``solve_mixed()`` runs the FP32 factorization plus FP64
    refinement (FP64 and complex128 batches); ``solve_plain(a, tau)``
    factors ``a`` (a copy of the batch, overwritten) in the batch's precision
    and writes x."""

    def __init__(self, ms, ns, dtype=torch.complex128, device="cuda"):
        import numpy as np

        self.ms = [int(x) for x in ms]
        self.ns = [int(x) for x in ns]
        if any(m < n for m, n in zip(self.ms, self.ns)):
            raise ValueError("least squares needs m >= n for every problem")
        self.dtype = dtype
        self.type, self.p = _TYPE[dtype]
        mm = np.array(self.ms, dtype=np.int64)
        nn = np.array(self.ns, dtype=np.int64)

        def offs(sz):
            return np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)

        self.a_off, self.t_off, self.b_off, self.x_off = offs(mm * nn), offs(nn), offs(mm), offs(nn)
        self.a = torch.zeros(int((mm * nn).sum()) or 1, dtype=dtype, device=device)
        self.b = torch.zeros(int(mm.sum()) or 1, dtype=dtype, device=device)
        self.x = torch.zeros(int(nn.sum()) or 1, dtype=dtype, device=device)
        self.ntau = int(nn.sum()) or 1
        L = lib()
        _setup(L)
        self._L = L
        m32 = mm.astype(np.int32)
        n32 = nn.astype(np.int32)
        self._keep = (m32, n32)
        lw = C.c_size_t(0)
        plan = C.c_void_p()
        _bind_stream()
        args = (self.type, len(self.ms), m32.ctypes.data, n32.ctypes.data, m32.ctypes.data, self.a_off.ctypes.data, self.t_off.ctypes.data,
                self.b_off.ctypes.data, self.x_off.ctypes.data)
        rc = L.rnpgpu_gels_batched_plan(*args, None, C.byref(lw), C.byref(plan))
        if rc:
            raise RNPGPUError("gels_batched_plan", rc)
        self.work = torch.empty(max(lw.value, 1), dtype=torch.uint8, device=device)
        rc = L.rnpgpu_gels_batched_plan(*args, self.work.data_ptr(), C.byref(lw), C.byref(plan))
        if rc:
            raise RNPGPUError("gels_batched_plan", rc)
        self.plan = plan
        self.iters = torch.zeros(max(len(self.ms), 1), dtype=torch.int32, device=device)
        self.berr = torch.zeros(max(len(self.ms), 1), dtype=torch.float64, device=device)
        self.eta = torch.zeros(max(len(self.ms), 1), dtype=torch.float64, device=device)
        self.mixed_work = None

    def matrix(self, i):
        m, n, o = self.ms[i], self.ns[i], int(self.a_off[i])
        return self.a[o:o + m * n].view(n, m).t()

    def rhs(self, i):
        o = int(self.b_off[i])
        return self.b[o:o + self.ms[i]]

    def solution(self, i):
        o = int(self.x_off[i])
        return self.x[o:o + self.ns[i]]

    def _mixed_ws(self):
        if self.mixed_work is None:
            f = getattr(self._L, _MIXED[self.dtype])
            lw = C.c_size_t(0)
            rc = f(self.plan, self.a.data_ptr(), None, None, 0, None, None, None, None, C.byref(lw))
            if rc:
                raise RNPGPUError("mixed workspace query", rc)
            self.mixed_work = torch.empty(max(lw.value, 1), dtype=torch.uint8, device=self.a.device)
        return self.mixed_work

    def solve_mixed(self, max_iter=0):
        """x by FP32 factorization + FP64 refinement; fills iters, berr, eta."""
        if self.dtype not in _MIXED:
            raise ValueError("mixed form needs a float64 or complex128 batch")
        ws = self._mixed_ws()
        lw = C.c_size_t(ws.numel())
        _bind_stream()
        rc = getattr(self._L, _MIXED[self.dtype])(self.plan, self.a.data_ptr(), self.b.data_ptr(), self.x.data_ptr(), int(max_iter), self.iters.data_ptr(),
                                                   self.berr.data_ptr(), self.eta.data_ptr(), ws.data_ptr(), C.byref(lw))
        if rc:
            raise RNPGPUError("gels_batched mixed", rc)

    def tune_mixed(self):
        """Autotune the FP32 factorization's block shapes; returns the best time (ms)."""
        ws = self._mixed_ws()
        lw = C.c_size_t(ws.numel())
        ms = C.c_double(0)
        _bind_stream()
        rc = getattr(self._L, _MIXED[self.dtype] + "_tune")(self.plan, self.a.data_ptr(), ws.data_ptr(), C.byref(lw), C.byref(ms))
        if rc:
            raise RNPGPUError("gels_batched mixed tune", rc)
        return ms.value

    def solve_plain(self, a=None, tau=None):
        """x in the batch's precision; ``a`` (default: a copy of self.a) is overwritten by the factors."""
        fa = self.a.clone() if a is None else a
        ft = torch.empty(self.ntau, dtype=self.dtype, device=self.a.device) if tau is None else tau
        _bind_stream()
        rc = getattr(self._L, "rnpgpu_%sgels_batched" % self.p)(self.plan, fa.data_ptr(), ft.data_ptr(), self.b.data_ptr(), self.x.data_ptr())
        if rc:
            raise RNPGPUError("gels_batched", rc)
        return fa, ft

    def config(self, cls):
        t, nb, cnt = C.c_int(), C.c_int(), C.c_int()
        self._L.rnpgpu_batch_plan_config(self.plan, cls, C.byref(t), C.byref(nb), C.byref(cnt))
        return {"threads": t.value, "nb": nb.value, "count": cnt.value}

    def force_config(self, cls, threads, nb):
        """Pin the block shape of a size class (one of the autotuner's candidates)."""
        rc = self._L.rnpgpu_batch_plan_set_config(self.plan, cls, threads, nb)
        if rc:
            raise RNPGPUError("batch_plan_set_config", rc)

    def __del__(self):
        try:
            if getattr(self, "plan", None):
                self._L.rnpgpu_batch_plan_destroy(self.plan)
                self.plan = None
        except Exception:
            pass
