"""GB300-native finite-difference LLG engine.

The product is ``libfullmag_fdm.so`` (C ABI in ``include/fullmag_fdm.h``, a drop-in for
the FDM backend interface of mzrptu/fullmag).  This package builds it in-tree and
offers a Python mirror of the reference's safe wrapper
(crates/fullmag-runner/src/native_fdm.rs) for Python callers and tests.
"""
from .backend import FdmBackend, FdmBatch, FdmError, FdmInterrupted, library, load_library, make_plan  # noqa: F401

__all__ = ["FdmBackend", "FdmBatch", "FdmError", "FdmInterrupted", "library", "load_library", "make_plan"]
