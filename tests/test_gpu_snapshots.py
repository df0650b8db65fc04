"""Asynchronous field and preview snapshots (native/backends/fdm/src/context.cu:1073-1745,
native/include/fullmag_fdm.h:397-473): begin captures the observable as it is at that
moment and returns before the copy to the host is done; wait blocks on that copy only,
may run on another thread and works after the backend is destroyed.  Previews are box
averages computed on the device with the same FP64 sums as a host loop."""
import ctypes as C
import threading

import numpy as np
import pytest

from fullmag_gb300 import _abi
from helpers import problem
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def _wait(lib, s, preview=False):
    data, nbytes, desc = C.c_void_p(), C.c_uint64(), _abi.SnapshotDesc()
    wait = lib.fullmag_fdm_preview_snapshot_wait if preview else lib.fullmag_fdm_field_snapshot_wait
    assert wait(s, C.byref(data), C.byref(nbytes), C.byref(desc)) == 0
    arr = np.ctypeslib.as_array((C.c_float * (nbytes.value // 4)).from_address(data.value)).copy()
    return arr, desc


def _box_preview(full, pnx, pny, pnz, z0, zs):
    """Restatement of the preview bins: x in [px nx/pnx, (px+1) nx/pnx) (at least one cell),
    same for y, z in [z0 + pz zs, z0 + (pz+1) zs), clamped; mean in float64."""
    nz, ny, nx, _ = full.shape
    out = np.zeros((pnz, pny, pnx, 3))
    for pz in range(pnz):
        z_lo = min(z0 + pz * zs, nz - 1)
        z_hi = min(max(z0 + (pz + 1) * zs, z_lo + 1), nz)
        for py in range(pny):
            y_lo, y_hi = py * ny // pny, (py + 1) * ny // pny
            y_hi = min(max(y_hi, y_lo + 1), ny)
            for px in range(pnx):
                x_lo, x_hi = px * nx // pnx, (px + 1) * nx // pnx
                x_hi = min(max(x_hi, x_lo + 1), nx)
                out[pz, py, px] = full[z_lo:z_hi, y_lo:y_hi, x_lo:x_hi].astype(np.float64).reshape(-1, 3).mean(axis=0)
    return out.reshape(-1, 3)


def test_snapshot_holds_the_state_at_begin(gpu_lib, oracle):
    kw = problem(12, 9, 4, seed=21)
    gpu, _ = make_pair(oracle, kw)
    lib = gpu.lib
    m0 = gpu.copy_field(_abi.OBSERVABLE_M)
    s = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_M)
    assert s
    for _ in range(3):
        gpu.step(5e-14)
    m3 = gpu.copy_field(_abi.OBSERVABLE_M)
    assert not np.array_equal(m0, m3)
    arr, desc = _wait(lib, s)
    lib.fullmag_fdm_field_snapshot_destroy(s)
    assert desc.cell_count == 12 * 9 * 4 and desc.component_count == 3 and desc.scalar_bytes == 4
    assert np.array_equal(arr.reshape(3, -1).T, m0.astype(np.float32))
    # a field snapshot after the steps evaluates the post-step field first
    s = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_H_EFF)
    arr, _ = _wait(lib, s)
    lib.fullmag_fdm_field_snapshot_destroy(s)
    assert np.array_equal(arr.reshape(3, -1).T, gpu.copy_field(_abi.OBSERVABLE_H_EFF).astype(np.float32))


@pytest.mark.parametrize("shape", [(6, 3, 2, 0, 2), (12, 9, 4, 0, 1), (5, 4, 1, 1, 3), (24, 18, 3, 1, 1), (1, 1, 1, 0, 4)])
def test_preview_matches_box_average(gpu_lib, oracle, shape):
    """Downsampled, identity, ragged bins, z origin and stride, previews larger than the
    grid (repeated cells) and a single whole-grid average."""
    pnx, pny, pnz, z0, zs = shape
    kw = problem(12, 9, 4, seed=22)
    gpu, _ = make_pair(oracle, kw)
    full = gpu.copy_field(_abi.OBSERVABLE_M).reshape(4, 9, 12, 3)
    want = _box_preview(full, pnx, pny, pnz, z0, zs)
    got = gpu.preview(_abi.OBSERVABLE_M, pnx, pny, pnz, z0, zs)
    assert np.allclose(got, want, rtol=0, atol=1e-14)
    s = gpu.lib.fullmag_fdm_backend_begin_preview_snapshot(gpu.handle, _abi.OBSERVABLE_M, pnx, pny, pnz, z0, zs)
    assert s
    arr, desc = _wait(gpu.lib, s, preview=True)
    gpu.lib.fullmag_fdm_preview_snapshot_destroy(s)
    assert desc.cell_count == pnx * pny * pnz
    assert np.array_equal(arr.reshape(-1, 3), got.astype(np.float32))


def test_snapshot_wait_on_another_thread_and_after_destroy(gpu_lib, oracle):
    kw = problem(16, 8, 2, seed=23)
    gpu, _ = make_pair(oracle, kw)
    lib = gpu.lib
    m0 = gpu.copy_field(_abi.OBSERVABLE_M).astype(np.float32)
    s1 = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_M)
    s2 = lib.fullmag_fdm_backend_begin_preview_snapshot(gpu.handle, _abi.OBSERVABLE_M, 4, 2, 1, 0, 2)
    pv = gpu.preview(_abi.OBSERVABLE_M, 4, 2, 1, 0, 2).astype(np.float32)
    out = {}

    def waiter():
        out["field"] = _wait(lib, s1)[0]

    t = threading.Thread(target=waiter)
    t.start()
    t.join(timeout=60)
    assert not t.is_alive()
    assert np.array_equal(out["field"].reshape(3, -1).T, m0)
    gpu.close()  # the preview snapshot outlives its backend
    arr, _ = _wait(lib, s2, preview=True)
    assert np.array_equal(arr.reshape(-1, 3), pv)
    lib.fullmag_fdm_field_snapshot_destroy(s1)
    lib.fullmag_fdm_preview_snapshot_destroy(s2)


def test_snapshot_of_host_synthesised_field_and_bad_origin(gpu_lib, oracle):
    kw = problem(8, 4, 2, seed=24)
    gpu, _ = make_pair(oracle, kw)
    lib = gpu.lib
    s = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_H_EXT)
    arr, _ = _wait(lib, s)
    lib.fullmag_fdm_field_snapshot_destroy(s)
    assert np.allclose(arr.reshape(3, -1).T, np.tile(kw["h_ext"], (64, 1)), rtol=1e-6)
    assert not lib.fullmag_fdm_backend_begin_preview_snapshot(gpu.handle, _abi.OBSERVABLE_M, 2, 2, 1, 2, 1)
