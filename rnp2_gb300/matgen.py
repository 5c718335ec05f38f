"""RNP::MatrixGen::RandomMatrix on the GPU (include/rnp_gpu/matgen_gb300.h),
for torch CUDA tensors (float32 / float64, column-major as rnp2_gb300.qr).

  random_matrix(m, n, sym=..., dist=..., mode=..., cond=..., dmax=..., seed=[...])
      -> (A, d, seed_out)

The arguments mean what RNP::MatrixGen::RandomMatrix's do (RNP/MatrixGen.hpp:
Symmetry, Random::Distribution, DiagonalMode); seed is the reference's 4-int
seed and seed_out the seed after every number drawn, as the reference leaves
it.
"""
import ctypes as C

import torch

from ._capi import lib
from .qr import _bind_stream, _check, empty_colmajor

SYM = {"nonsymmetric": 0, "hermitian": 1, "hpd": 2, "symmetric": 3}
MODE = {"given": 0, "first1": 1, "lastcond": 2, "graded_exp": 3, "graded_lin": 4, "random_exp": 5, "random_dist": 6}
DIST = {"uniform01": 0, "uniform_11": 1, "normal01": 2, "unit_disc": 3, "unit_circle": 4}


def random_matrix(m, n, sym=0, dist=2, mode=3, cond=1.0, dmax=1.0, seed=(1, 2, 3, 5), d=None, reverse=False, dtype=torch.float64, device="cuda", work=None):
    sym = SYM.get(sym, sym)
    mode = MODE.get(mode, mode)
    dist = DIST.get(dist, dist)
    p = {torch.float32: "s", torch.float64: "d"}[dtype]
    fn = getattr(lib(), "rnpgpu_%srandom_matrix" % p)
    R = C.c_float if p == "s" else C.c_double
    A = empty_colmajor(m, n, dtype, device)
    k = min(m, n)
    if d is None:
        d = torch.zeros(max(k, 1), dtype=dtype, device=device)
    s = (C.c_int * 4)(*seed)
    _bind_stream()
    args = (sym, dist, mode, 1 if reverse else 0, R(cond), R(dmax), d.data_ptr(), m, n, A.data_ptr(), max(A.stride(1), 1), s)
    if work is None:
        lw = C.c_size_t(0)
        _check("random_matrix", fn(*args, C.byref(lw), None))
        work = torch.empty(max(lw.value, 1), dtype=dtype, device=device)
    lw = C.c_size_t(work.numel())
    _check("random_matrix", fn(*args, C.byref(lw), work.data_ptr()))
    return A, d[:k], list(s)
