"""qvnt_gb300: a GB300 (sm_103a) state-vector engine behind qvnt's register and operator API.

    from qvnt_gb300 import QReg, op
    q = QReg.with_state(10, 0b0011100000)
    q.apply(op.qft(0b0000011111))
    measured = q.measure_mask(0b0000000111)

The state vector lives only in GPU memory; every gate, reduction and measurement runs in the
library's CUDA kernels (qvnt_gb300/csrc/).  This package is the Python side of the C ABI in
include/qvnt_gb300.h.
"""
import os as _os

# Independent registers run on independent CUDA streams; 32 hardware work queues (instead of the
# default 8) keep their kernels from serialising behind each other.  Read when the process creates
# its CUDA context, so it must be set before any CUDA use (e.g. by torch).
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import operator as op  # noqa: E402
from ._abi import ENGINE_FUSED, ENGINE_PLAIN, ENGINE_PRECISION, ENGINE_TENSOR64, KIND, KINDS, MaskError, QvntError, QvntGate
from .operator import MultiOp, SingleOp
from .register import Context, CReg, QReg, VReg, bits_iter, default_context

__all__ = ["op", "QReg", "CReg", "VReg", "MultiOp", "SingleOp", "Context", "default_context", "bits_iter",
           "QvntGate", "QvntError", "MaskError", "KIND", "KINDS", "ENGINE_FUSED", "ENGINE_PLAIN",
           "ENGINE_PRECISION", "ENGINE_TENSOR64"]
