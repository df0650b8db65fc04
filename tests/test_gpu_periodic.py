"""Periodic boundaries on the GPU (fullmag_fdm_backend_create_periodic) against the FP64
oracle, which follows the reference CPU engine (crates/fullmag-engine/src/fdm_fft.rs:140-233,
614-717; fdm_fields.rs:109-160,356-445,1253-1340): H_eff and the energies at step 0 for
films and volumes periodic along one, two or three axes (unpadded transforms, the complex
image-sum kernel, wrapped exchange / DMI / Zhang-Li stencils), short trajectories, and the
error paths of the entry point."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmError, _abi
from helpers import problem, rel_l2

pytestmark = pytest.mark.gpu


def _pair(oracle, kw, periodic, images=None, integrator=_abi.INTEGRATOR_HEUN, mask=None):
    oint = {_abi.INTEGRATOR_HEUN: oracle.HEUN, _abi.INTEGRATOR_RK4: oracle.RK4}[integrator]
    orc = oracle.Problem(**kw, integrator=oint, active_mask=mask, periodic=periodic, image_counts=images)
    gpu = FdmBackend(**kw, integrator=integrator, active_mask=mask, periodic=periodic, image_counts=images)
    return gpu, orc


CASES = {
    # thin films: the 2-D y pass with the complex kernel
    "film_32x16x1_xy": (dict(nx=32, ny=16, nz=1, d=(4e-9, 4e-9, 2e-9)), (1, 1, 0), (3, 3, 0)),
    "film_24x12x1_x": (dict(nx=24, ny=12, nz=1, d=(3e-9, 4e-9, 2e-9)), (1, 0, 0), (4, 0, 0)),
    "film_16x16x1_xyz_default": (dict(nx=16, ny=16, nz=1, d=(4e-9, 4e-9, 2e-9)), (1, 1, 1), None),
    # volumes: y forward / general z convolution / y inverse
    "vol_16x8x4_x": (dict(nx=16, ny=8, nz=4), (1, 0, 0), (2, 0, 0)),
    "vol_12x10x6_yz": (dict(nx=12, ny=10, nz=6, d=(3e-9, 2e-9, 2.5e-9)), (0, 1, 1), (0, 2, 1)),
    "vol_8x6x5_xyz": (dict(nx=8, ny=6, nz=5), (1, 1, 1), (1, 1, 1)),
    "vol_20x9x3_y_odd": (dict(nx=20, ny=9, nz=3), (0, 1, 0), (0, 3, 0)),
    "vol_64x32x4_xy": (dict(nx=64, ny=32, nz=4), (1, 1, 0), (2, 2, 0)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_heff_and_energies_at_step0(gpu_lib, oracle, name):
    shape, periodic, images = CASES[name]
    kw = problem(shape["nx"], shape["ny"], shape["nz"], d=shape.get("d", (4e-9, 4e-9, 4e-9)), seed=71,
                 ku1=4e4, u_axis=(0.3, 0.2, 1.0))
    gpu, orc = _pair(oracle, kw, periodic, images)
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_DEMAG), ref["h_demag"]) < 1e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EX), ref["h_ex"]) < 1e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    for k, o in (("exchange_energy_joules", "e_exchange"), ("demag_energy_joules", "e_demag"),
                 ("total_energy_joules", "e_total")):
        assert abs(st[k] - ost[o]) <= 1e-5 * abs(ost[o]) + 1e-30, k


def test_four_cells_per_thread_path_wraps(gpu_lib, oracle, monkeypatch):
    # 4 rows of 256 cells per CTA: the row pass takes its float4 path, whose first and
    # last groups of a row read the wrapped neighbours
    monkeypatch.setenv("FULLMAG_FDM_TUNE", "4,8,8,8,4,0,0,0,0")
    kw = problem(256, 8, 2, seed=77)
    gpu, orc = _pair(oracle, kw, (1, 1, 1), (1, 1, 1))
    assert gpu.tuning()["rows_per_cta"] == 4
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EX), ref["h_ex"]) < 1e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["exchange_energy_joules"] - ost["e_exchange"]) <= 1e-5 * abs(ost["e_exchange"])


def test_masked_periodic_volume(gpu_lib, oracle):
    kw = problem(16, 12, 3, seed=72)
    mask = (np.random.default_rng(4).random(16 * 12 * 3) > 0.15).astype(np.uint8)
    gpu, orc = _pair(oracle, kw, (1, 1, 0), (2, 2, 0), mask=mask)
    ref = orc.fields(kw["m0"] * mask[:, None])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5


def test_dmi_and_zhang_li_wrap(gpu_lib, oracle):
    # central-difference DMI and the upwind Zhang-Li derivative take the wrapped neighbour
    kw = problem(24, 8, 2, seed=73, alpha=0.3, dmi_d_interfacial=2.5e-3, dmi_d_bulk=1e-3,
                 current_density=(-4e11, 2e11, 0.0), stt_degree=0.6, stt_beta=0.05)
    gpu, orc = _pair(oracle, kw, (1, 1, 0), (2, 2, 0), integrator=_abi.INTEGRATOR_RK4)
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    for _ in range(20):
        sg = gpu.step(5e-14)
        so = orc.step(5e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 2e-5
    assert abs(sg["dmi_energy_joules"] - so["e_dmi"]) <= 1e-4 * abs(so["e_dmi"])


@pytest.mark.parametrize("name", ["film_32x16x1_xy", "vol_12x10x6_yz"])
def test_rk4_trajectory(gpu_lib, oracle, name):
    shape, periodic, images = CASES[name]
    kw = problem(shape["nx"], shape["ny"], shape["nz"], d=shape.get("d", (4e-9, 4e-9, 4e-9)), seed=74, alpha=0.2)
    gpu, orc = _pair(oracle, kw, periodic, images, integrator=_abi.INTEGRATOR_RK4)
    for _ in range(40):
        sg = gpu.step(1e-13)
        so = orc.step(1e-13)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 5e-5
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"])


def test_fft_shape_is_unpadded_on_periodic_axes(gpu_lib):
    kw = problem(16, 12, 5, seed=75)
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN, periodic=(1, 0, 1), image_counts=(1, 0, 1))
    px, py, pz = gpu.fft_shape()
    assert (px, pz) == (16, 5) and py >= 2 * 12 - 1


def test_error_paths(gpu_lib, oracle):
    kw = problem(9, 8, 2, seed=76)
    with pytest.raises(FdmError, match="even"):
        FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN, periodic=(1, 0, 0))
    kw = problem(8, 8, 2, seed=76)
    sp = oracle.newell_spectra(8, 8, 2, kw["dx"], kw["dy"], kw["dz"])
    with pytest.raises(FdmError, match="no spectra"):
        FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN, periodic=(0, 1, 0), spectra=sp)
    with pytest.raises(FdmError, match="no spectra"):
        FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN, periodic=(0, 1, 0), spectra=sp,
                   precision=_abi.PRECISION_DOUBLE)
    with pytest.raises(FdmError, match="boundary correction"):
        FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN, periodic=(1, 0, 0), precision=_abi.PRECISION_DOUBLE,
                   boundary={"tier": _abi.BOUNDARY_VOLUME, "volume_fraction": np.ones(8 * 8 * 2),
                             "face": [np.ones(8 * 8 * 2)] * 6})
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, periodic=(0, 1, 0), image_counts=(0, 1, 0))
    with pytest.raises(FdmError, match="periodic"):
        gpu.adjoint_forward(1e-13, 4)


@pytest.mark.parametrize("shape,periodic,images", [
    ((24, 16, 1), (1, 1, 0), (3, 3, 0)),
    ((12, 10, 6), (0, 1, 1), (0, 2, 1)),
    ((9, 8, 3), (1, 0, 0), (2, 0, 0)),      # odd periodic x: the FP64 transforms take any length
    ((8, 6, 5), (1, 1, 1), (1, 1, 1)),
])
def test_double_precision_periodic(gpu_lib, oracle, shape, periodic, images):
    # the double-precision path against the FP64 oracle: both compute in FP64; the tensor is
    # built on the GPU, whose f/g evaluations (log1p, atan) differ from the host's by an
    # ulp that the 27-point second difference amplifies, so the bound is the one of the
    # GPU-built FP64 tensor elsewhere: 1e-9 relative L2
    nx, ny, nz = shape
    kw = problem(nx, ny, nz, seed=78, ku1=4e4, u_axis=(0.3, 0.2, 1.0))
    orc = oracle.Problem(**kw, integrator=oracle.RK4, periodic=periodic, image_counts=images)
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, periodic=periodic, image_counts=images,
                     precision=_abi.PRECISION_DOUBLE)
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_DEMAG), ref["h_demag"]) < 1e-9
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-9
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["exchange_energy_joules"] - ost["e_exchange"]) <= 1e-9 * abs(ost["e_exchange"])
    assert abs(st["demag_energy_joules"] - ost["e_demag"]) <= 1e-9 * abs(ost["e_demag"])
    for _ in range(20):
        gpu.step(1e-13)
        orc.step(1e-13)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-9
