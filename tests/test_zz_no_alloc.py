"""Allocation-free upload (fullmag_fdm_backend_upload_magnetization_f64_noalloc) vs the
regular upload, through the C ABI.  Collected last on purpose: it must hold both alone
and after every other GPU test has used the device."""
import ctypes as C

import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmError, _abi
from helpers import problem, random_unit

pytestmark = pytest.mark.gpu


def _noalloc(lib, handle, m):
    f = lib.fullmag_fdm_backend_upload_magnetization_f64_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_uint64]
    a = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
    return f(handle, a.ctypes.data_as(C.POINTER(C.c_double)), a.size)


def _state(be):
    be.refresh()
    return be.copy_field(_abi.OBSERVABLE_M), be.copy_field(_abi.OBSERVABLE_H_EFF), be.stats()


def test_noalloc_upload_matches_regular_upload(gpu_lib):
    kw = problem(24, 16, 2, seed=21)
    n = 24 * 16 * 2
    mask = np.ones(n, dtype=np.uint8)
    mask[::7] = 0
    regular = FdmBackend(**kw, active_mask=mask)
    noalloc = FdmBackend(**kw, active_mask=mask)
    for seed in (31, 32):  # two consecutive calls with different states
        m = random_unit(n, seed)
        regular.upload(m)
        assert _noalloc(gpu_lib, noalloc.handle, m) == _abi.OK
        m_r, h_r, st_r = _state(regular)
        m_n, h_n, st_n = _state(noalloc)
        assert np.array_equal(m_r, m_n)
        assert np.array_equal(h_r, h_n)
        assert st_r["total_energy_joules"] == st_n["total_energy_joules"]
        assert np.all(m_n[mask == 0] == 0.0)
        regular.step(1e-14)
        noalloc.step(1e-14)
        assert np.array_equal(regular.magnetization(), noalloc.magnetization())


def test_noalloc_upload_allocates_nothing(gpu_lib):
    """A fresh handle that only ever receives allocation-free uploads and steps: the
    device's free memory is the same before and after the uploads (the regular upload's
    staging buffer would take 3 n doubles on its first call), and the stepped state
    equals that of a handle fed by the regular upload."""
    import torch

    kw = problem(64, 64, 4, seed=23)
    n = 64 * 64 * 4
    warm = FdmBackend(**problem(8, 4, 1, seed=2))
    assert _noalloc(gpu_lib, warm.handle, random_unit(8 * 4, 5)) == _abi.OK  # set-up of the device's array
    warm.close()
    be = FdmBackend(**kw)
    be.step(1e-14)  # two steps: the step graphs of both state buffers exist before the measurement
    be.step(1e-14)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for seed in (41, 42):
        assert _noalloc(gpu_lib, be.handle, random_unit(n, seed)) == _abi.OK
        be.step(1e-14)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    ref = FdmBackend(**kw)
    ref.step(1e-14)
    ref.step(1e-14)
    ref.upload(random_unit(n, 42))
    ref.step(1e-14)
    assert np.array_equal(ref.magnetization(), be.magnetization())
    be.close()
    ref.close()


def test_noalloc_upload_rejects_bad_input(gpu_lib):
    kw = problem(8, 4, 1, seed=2)
    be = FdmBackend(**kw)
    assert _noalloc(gpu_lib, be.handle, np.zeros((31, 3))) == _abi.ERR_INVALID
    big = problem(1024, 257, 1, seed=3, enable_demag=False)  # 263,168 cells > 262,144
    be_big = FdmBackend(**big)
    assert _noalloc(gpu_lib, be_big.handle, big["m0"]) == _abi.ERR_INVALID
    msg = gpu_lib.fullmag_fdm_backend_last_error(be_big.handle).decode()
    assert "allocation-free" in msg
    with pytest.raises(FdmError):
        be_big._check(_abi.ERR_INVALID, "noalloc")
