"""ctypes wrapper of libfullmag_fdm_plain.so, the cuFFT + unfused measurement baseline.

The plain path restates the reference backend's per-step kernel structure
(native/backends/fdm/src/llg_rk4_fp32.cu:37-232, demag_fp32.cu:406-502,
exchange_fp32.cu:21-156, reductions_fp64.cu:123-393) with one kernel per operation
and cuFFT C2C transforms of the full padded grid.  It exists only to be timed next to
the fused engine; it is not part of libfullmag_fdm.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .backend import FdmError, make_plan
from .build import PLAIN_LIB, build

_PLAIN = None


def _lib():
    global _PLAIN
    if _PLAIN is None:
        if not PLAIN_LIB.exists():
            build()
        L = C.CDLL(str(PLAIN_LIB))
        L.fullmag_fdm_plain_create.restype = C.c_void_p
        L.fullmag_fdm_plain_create.argtypes = [C.POINTER(_abi.PlanDesc)]
        L.fullmag_fdm_plain_create_error.restype = C.c_char_p
        L.fullmag_fdm_plain_step.restype = C.c_int
        L.fullmag_fdm_plain_step.argtypes = [C.c_void_p, C.c_double, C.POINTER(_abi.StepStats)]
        L.fullmag_fdm_plain_copy_m.restype = C.c_int
        L.fullmag_fdm_plain_copy_m.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_uint64]
        L.fullmag_fdm_plain_destroy.argtypes = [C.c_void_p]
        _PLAIN = L
    return _PLAIN


class PlainBaseline:
    """Same plan keywords as FdmBackend (Heun or RK4, no mask)."""

    def __init__(self, **plan_kwargs):
        self.lib = _lib()
        p, keep = make_plan(**plan_kwargs)
        self.n = p.grid.nx * p.grid.ny * p.grid.nz
        self.handle = self.lib.fullmag_fdm_plain_create(C.byref(p))
        del keep
        if not self.handle:
            raise FdmError(_abi.ERR_INVALID, self.lib.fullmag_fdm_plain_create_error().decode())

    def step(self, dt: float) -> dict:
        st = _abi.StepStats()
        rc = self.lib.fullmag_fdm_plain_step(self.handle, dt, C.byref(st))
        if rc != _abi.OK:
            raise FdmError(rc, "plain step failed")
        return st.as_dict()

    def magnetization(self) -> np.ndarray:
        out = np.empty(3 * self.n)
        rc = self.lib.fullmag_fdm_plain_copy_m(self.handle, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
        if rc != _abi.OK:
            raise FdmError(rc, "plain copy failed")
        return out.reshape(self.n, 3)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fullmag_fdm_plain_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
