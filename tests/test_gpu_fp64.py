"""The double-precision state path (plan precision FULLMAG_FDM_PRECISION_DOUBLE) against
the FP64 oracle, through the C ABI.  Both sides compute in FP64, so the bound is far
below the single-precision path's 1e-5: H_eff within 1e-10 relative L2 (the two FFTs and
summation orders differ), short trajectories within 1e-9 per component, energies within
1e-9 relative.  Also the boundary-correction tiers, which the reference runs on its FP64
path only (exchange_fp64.cu:162-231): T0 face links, T1 boundary distances, the
phi-weighted demag input and the sparse demag correction, on a sphere in a box."""
import ctypes as C

import numpy as np
import pytest

from boundary_geometry import sphere_geometry
from fullmag_gb300 import FdmBackend, _abi
from helpers import problem, rel_l2

pytestmark = pytest.mark.gpu

TOL_H = 1e-10

OINT = {_abi.INTEGRATOR_HEUN: "HEUN", _abi.INTEGRATOR_RK4: "RK4", _abi.INTEGRATOR_DP45: "DP45",
        _abi.INTEGRATOR_RK23: "RK23", _abi.INTEGRATOR_ABM3: "ABM3"}


def pair(oracle, kw, integrator=_abi.INTEGRATOR_RK4, spectra=True, mask=None, boundary=None, **gpu_extra):
    nx, ny, nz = kw["nx"], kw["ny"], kw["nz"]
    sp = None
    if spectra and kw.get("enable_demag", True):
        sp = oracle.newell_spectra(nx, ny, nz, kw["dx"], kw["dy"], kw["dz"], thin_film_2d=nz == 1)
    okw = {k: v for k, v in kw.items() if k != "adaptive_max_error"}
    orc = oracle.Problem(**okw, integrator=getattr(oracle, OINT[integrator]), active_mask=mask,
                         max_error=kw.get("adaptive_max_error", 1e-5) or 1e-5, boundary=boundary)
    gpu = FdmBackend(**kw, integrator=integrator, spectra=sp, active_mask=mask, precision=_abi.PRECISION_DOUBLE,
                     boundary=boundary, **gpu_extra)
    return gpu, orc


CASES = {
    "box_24x16x6": dict(nx=24, ny=16, nz=6),
    "odd_7x5x3": dict(nx=7, ny=5, nz=3, d=(3e-9, 2e-9, 2.5e-9)),
    "thin_40x12x1": dict(nx=40, ny=12, nz=1, d=(3.90625e-9, 3.90625e-9, 3e-9)),
    "line_9x1x1": dict(nx=9, ny=1, nz=1),
    "single_1x1x1": dict(nx=1, ny=1, nz=1),
}


@pytest.mark.parametrize("name", list(CASES))
def test_fp64_heff_at_step0(gpu_lib, oracle, name):
    c = dict(CASES[name])
    kw = problem(c.pop("nx"), c.pop("ny"), c.pop("nz"), seed=4, ku1=3e4, u_axis=(0.3, 0.2, 1.0), kc1=-2e4, **c)
    gpu, orc = pair(oracle, kw)
    f = orc.fields()
    for obs, key in ((_abi.OBSERVABLE_H_EFF, "h_eff"), (_abi.OBSERVABLE_H_DEMAG, "h_demag"), (_abi.OBSERVABLE_H_EX, "h_ex")):
        ref = f[key]
        if np.abs(ref).max() == 0.0:
            continue
        assert rel_l2(gpu.copy_field(obs), ref) < TOL_H, (name, key)
    st, so = gpu.stats(), orc.observe()
    for a, b in (("exchange_energy_joules", "e_exchange"), ("demag_energy_joules", "e_demag"),
                 ("external_energy_joules", "e_external"), ("anisotropy_energy_joules", "e_uniaxial"),
                 ("cubic_energy_joules", "e_cubic")):
        assert abs(st[a] - so[b]) <= 1e-10 * abs(so[b]) + 1e-40, (a, st[a], so[b])
    gpu.close()
    orc.close()


def test_fp64_mask_and_regions(gpu_lib, oracle):
    nx, ny, nz = 20, 12, 3
    n = nx * ny * nz
    mask = np.ones(n, dtype=np.uint8)
    mask[::5] = 0
    x = np.tile(np.arange(nx), ny * nz)
    reg = np.where(x < nx // 2, 1, 200).astype(np.uint32)
    lut = np.zeros((256, 256))
    lut[1, 1], lut[200, 200], lut[1, 200], lut[200, 1] = 1.3e-11, 0.9e-11, 0.4e-11, 0.4e-11
    kw = problem(nx, ny, nz, seed=6, region_mask=reg, exchange_lut=lut)
    gpu, orc = pair(oracle, kw, mask=mask)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"]) < TOL_H
    assert abs(gpu.stats()["exchange_energy_joules"] - orc.observe()["e_exchange"]) <= 1e-10 * abs(orc.observe()["e_exchange"])


@pytest.mark.parametrize("integrator,dt,steps", [(_abi.INTEGRATOR_HEUN, 5e-14, 40), (_abi.INTEGRATOR_RK4, 5e-14, 30),
                                                 (_abi.INTEGRATOR_ABM3, 5e-14, 30)])
def test_fp64_fixed_step_trajectory(gpu_lib, oracle, integrator, dt, steps):
    kw = problem(32, 16, 4, seed=0)
    gpu, orc = pair(oracle, kw, integrator=integrator)
    for _ in range(steps):
        sg = gpu.step(dt)
        so = orc.step(dt)
    assert sg["step"] == steps
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-9
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-9 * abs(so["e_total"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"]) < 1e-9


@pytest.mark.parametrize("integrator", [_abi.INTEGRATOR_DP45, _abi.INTEGRATOR_RK23])
def test_fp64_adaptive_trajectory(gpu_lib, oracle, integrator):
    kw = problem(48, 16, 1, d=(3.90625e-9, 3.90625e-9, 3e-9), seed=2, alpha=0.02, ku1=5e3, u_axis=(1, 0, 0),
                 b_mt=(-24.6, 4.3, 0.0), adaptive_max_error=1e-5)
    gpu, orc = pair(oracle, kw, integrator=integrator)
    dt_g = dt_o = 1e-13
    for _ in range(25):
        sg = gpu.step(dt_g)
        so = orc.step(dt_o)
        # FP64 on both sides: the controllers take the same steps
        assert sg["dt_seconds"] == pytest.approx(so["dt_used"], rel=1e-9)
        dt_g, dt_o = sg["suggested_next_dt"], so["suggested_next_dt"]
    assert sg["time_seconds"] == pytest.approx(so["time"], rel=1e-9)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-8
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-8 * abs(so["e_total"])


def test_fp64_gpu_newell_matches_oracle(gpu_lib, oracle):
    """The FP64 tensor built on the GPU (no spectra passed) against the oracle's."""
    kw = problem(48, 44, 6, d=(2e-9, 3e-9, 2.5e-9), seed=9, b_mt=None, enable_exchange=False)
    gpu, orc = pair(oracle, kw, spectra=False)
    assert gpu.fft_shape() == (96, 88, 12)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_DEMAG), orc.fields()["h_demag"]) < 1e-9


@pytest.mark.parametrize("tier", [_abi.BOUNDARY_VOLUME, _abi.BOUNDARY_FULL])
def test_fp64_boundary_tiers_on_a_sphere(gpu_lib, oracle, tier):
    nx, ny, nz, d = 20, 20, 12, (2e-9, 2e-9, 2e-9)
    geo = sphere_geometry(nx, ny, nz, d, radius=9e-9, corr_stencil=3, seed=1)
    geo["tier"] = tier
    kw = problem(nx, ny, nz, d=d, seed=12)
    gpu, orc = pair(oracle, kw, boundary=geo)
    f = orc.fields()
    inside = geo["volume_fraction"] > 0
    assert inside.sum() > 100 and (~inside).sum() > 100
    for obs, key in ((_abi.OBSERVABLE_H_EX, "h_ex"), (_abi.OBSERVABLE_H_DEMAG, "h_demag"), (_abi.OBSERVABLE_H_EFF, "h_eff")):
        assert rel_l2(gpu.copy_field(obs), f[key]) < TOL_H, key
    m = gpu.copy_field(_abi.OBSERVABLE_M)
    assert np.all(m[~inside] == 0.0)
    st, so = gpu.stats(), orc.observe()
    for a, b in (("exchange_energy_joules", "e_exchange"), ("demag_energy_joules", "e_demag"),
                 ("external_energy_joules", "e_external")):
        assert abs(st[a] - so[b]) <= 1e-10 * abs(so[b]), (a, st[a], so[b])
    for _ in range(10):
        sg = gpu.step(3e-14)
        so = orc.step(3e-14)
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < 1e-9
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-9 * abs(so["e_total"])


def test_fp64_matches_single_precision_within_its_tolerance(gpu_lib, oracle):
    kw = problem(32, 16, 4, seed=1)
    sp = oracle.newell_spectra(32, 16, 4, kw["dx"], kw["dy"], kw["dz"])
    g64 = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, spectra=sp, precision=_abi.PRECISION_DOUBLE)
    g32 = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, spectra=sp)
    assert rel_l2(g32.copy_field(_abi.OBSERVABLE_H_EFF), g64.copy_field(_abi.OBSERVABLE_H_EFF)) < 1e-5
    for _ in range(5):
        g64.step(5e-14)
        g32.step(5e-14)
    assert np.abs(g32.magnetization() - g64.magnetization()).max() < 1e-5


def test_fp64_upload_previews_snapshots_interrupt(gpu_lib, oracle):
    from helpers import random_unit
    nx, ny, nz = 12, 10, 4
    kw = problem(nx, ny, nz, seed=3)
    gpu, orc = pair(oracle, kw, integrator=_abi.INTEGRATOR_HEUN)
    m1 = random_unit(nx * ny * nz, 44)
    gpu.upload(m1)
    orc.set_m(m1)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"]) < TOL_H
    # previews: box averages of the FP64 field
    full = gpu.copy_field(_abi.OBSERVABLE_M).reshape(nz, ny, nx, 3)
    pv = gpu.preview(_abi.OBSERVABLE_M, 6, 5, 2, 0, 2)
    want = full.reshape(2, 2, 5, 2, 6, 2, 3).mean(axis=(1, 3, 5)).reshape(-1, 3)
    assert np.allclose(pv.reshape(-1, 3), want, rtol=0, atol=1e-15)
    # field snapshot: FP64, component-major, the state at begin
    lib = gpu_lib
    snap = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_M)
    assert snap
    gpu.step(5e-14)
    data, ln, desc = C.c_void_p(), C.c_uint64(), _abi.SnapshotDesc()
    assert lib.fullmag_fdm_field_snapshot_wait(snap, C.byref(data), C.byref(ln), C.byref(desc)) == _abi.OK
    assert desc.scalar_bytes == 8 and desc.scalar_type == 2 and ln.value == 8 * 3 * nx * ny * nz
    soa = np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_double)), shape=(3, nx * ny * nz)).copy()
    lib.fullmag_fdm_field_snapshot_destroy(snap)
    assert np.array_equal(soa.T, full.reshape(-1, 3))  # the state at begin, not after the step
    # an interrupt leaves the state as it was
    before = gpu.copy_field(_abi.OBSERVABLE_M)
    gpu.set_interrupt_poll(lambda: 1)
    with pytest.raises(Exception):
        gpu.step(5e-14)
    gpu.set_interrupt_poll(None)
    assert np.array_equal(gpu.copy_field(_abi.OBSERVABLE_M), before)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(before)["h_eff"]) < TOL_H


def test_fp64_rejects_what_it_does_not_model(gpu_lib, oracle):
    from fullmag_gb300 import FdmError
    kw = problem(8, 8, 2, seed=1, dmi_d_interfacial=1e-3)
    with pytest.raises(FdmError, match="double-precision"):
        FdmBackend(**kw, precision=_abi.PRECISION_DOUBLE)
