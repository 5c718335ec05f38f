"""rnp2_gb300 — GB300-native blocked Householder QR, a drop-in for the QR path
of RNP2 (RNP::LA::QR: Factor, MultQ, GenerateQ and their unblocked forms).

The compute path is the CUDA library built from ``rnp2_gb300/csrc`` for
sm_103a and called through its C ABI (``include/rnp_gpu/qr_gb300.h``);
``rnp2_gb300.qr`` mirrors the reference's routines for torch CUDA tensors.
"""
from ._capi import LibraryNotBuilt, lib  # noqa: F401
from . import qr  # noqa: F401

__all__ = ["lib", "qr", "LibraryNotBuilt"]
