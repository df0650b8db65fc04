"""CUDA engine vs the FP64 oracle, through the C ABI (libfullmag_fdm.so).

Spectra are produced the way the reference runner produces them
(crates/fullmag-runner/src/native_fdm.rs:192-210: thin-film 2-D spectra when nz == 1).
Tolerances: H_eff per evaluation within 1e-5 relative L2 (the engine target), and
trajectories within the Tier B tolerances of native/backends/fdm/tests/tier_b_compare.cu
(m 1e-5 max-abs per component after short runs, energies 1e-4 relative) where FP32 allows.
"""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmError, FdmInterrupted, _abi
from helpers import problem, rel_l2

pytestmark = pytest.mark.gpu

HEFF_TOL = 1e-5


def make_pair(oracle, kw, integrator=_abi.INTEGRATOR_HEUN, thin=None, mask=None, spectra=True, **gpu_extra):
    nx, ny, nz = kw["nx"], kw["ny"], kw["nz"]
    if thin is None:
        thin = nz == 1
    sp = None
    if spectra and kw.get("enable_demag", True):
        sp = oracle.newell_spectra(nx, ny, nz, kw["dx"], kw["dy"], kw["dz"], thin_film_2d=thin)
    okw = dict(kw)
    oint = {_abi.INTEGRATOR_HEUN: oracle.HEUN, _abi.INTEGRATOR_RK4: oracle.RK4, _abi.INTEGRATOR_DP45: oracle.DP45,
            _abi.INTEGRATOR_RK23: oracle.RK23, _abi.INTEGRATOR_ABM3: oracle.ABM3}[integrator]
    for k in ("adaptive_max_error",):
        okw.pop(k, None)
    orc = oracle.Problem(**okw, integrator=oint, active_mask=mask,
                         max_error=kw.get("adaptive_max_error", 1e-5) or 1e-5)
    gpu = FdmBackend(**kw, integrator=integrator, spectra=sp, active_mask=mask, **gpu_extra)
    return gpu, orc


CASES = {
    "cfg1_64x32x4": dict(nx=64, ny=32, nz=4),
    "thin_64x16x1": dict(nx=64, ny=16, nz=1, d=(3.90625e-9, 3.90625e-9, 3e-9)),
    # py = 512: the thin-film pass's own 32 x 16 instance
    "thin_16x256x1": dict(nx=16, ny=256, nz=1, d=(3e-9, 2.5e-9, 2e-9)),
    "odd_7x5x3": dict(nx=7, ny=5, nz=3, d=(3e-9, 2e-9, 2.5e-9)),
    "line_9x1x1": dict(nx=9, ny=1, nz=1),
    "single_1x1x1": dict(nx=1, ny=1, nz=1),
    "slab_12x10x2": dict(nx=12, ny=10, nz=2, d=(2e-9, 2e-9, 2e-9)),
    # fused y+z pass on its pruned two-level path (py = 256, pz = 4; py = 128, pz = 8)
    "yzf_8x128x2": dict(nx=8, ny=128, nz=2, d=(4e-9, 4e-9, 4e-9)),
    "yzf_16x64x4": dict(nx=16, ny=64, nz=4, d=(4e-9, 4e-9, 4e-9)),
    # (y, z) planes too large for the fused y+z pass: y-forward / z-convolve / y-inverse,
    # the z pass on its pruned two-level path for pz = 16, 32, 64, 128 and on the
    # general path for pz = 24
    "zcols_4x120x8": dict(nx=4, ny=120, nz=8, d=(2e-9, 2e-9, 2e-9)),
    "zcols_4x64x16": dict(nx=4, ny=64, nz=16, d=(2e-9, 2e-9, 2e-9)),
    "zcols_8x32x32": dict(nx=8, ny=32, nz=32, d=(2e-9, 2e-9, 2e-9)),
    "zcols_8x16x64": dict(nx=8, ny=16, nz=64, d=(2e-9, 2e-9, 2e-9)),
    "zcols_4x84x12": dict(nx=4, ny=84, nz=12, d=(2e-9, 2e-9, 2e-9)),
}


@pytest.mark.parametrize("name", [k for k in CASES if k.startswith("zcols")])
def test_three_pass_columns_are_used(gpu_lib, oracle, name):
    c = dict(CASES[name])
    d = c.pop("d")
    kw = problem(c["nx"], c["ny"], c["nz"], d=d, seed=3)
    gpu = FdmBackend(**kw)
    gpu.set_kernel_timing(True)
    gpu.refresh()
    kt = gpu.kernel_times()
    assert kt["z_convolve"][1] >= 1 and kt["yz_convolve"][1] == 0, kt


@pytest.mark.parametrize("name", list(CASES))
def test_heff_at_step0(gpu_lib, oracle, name):
    c = dict(CASES[name])
    d = c.pop("d", (4e-9, 4e-9, 4e-9))
    kw = problem(c["nx"], c["ny"], c["nz"], d=d, seed=11)
    gpu, orc = make_pair(oracle, kw)
    ref = orc.fields(kw["m0"])
    m_gpu = gpu.copy_field(_abi.OBSERVABLE_M)
    assert np.abs(m_gpu - kw["m0"]).max() < 1e-7
    for obs, key in ((_abi.OBSERVABLE_H_EX, "h_ex"), (_abi.OBSERVABLE_H_DEMAG, "h_demag"),
                     (_abi.OBSERVABLE_H_EXT, "h_ext"), (_abi.OBSERVABLE_H_EFF, "h_eff")):
        got = gpu.copy_field(obs)
        if np.linalg.norm(ref[key]) > 0:
            assert rel_l2(got, ref[key]) < HEFF_TOL, (name, key, rel_l2(got, ref[key]))


def test_heff_roofline_kernel_shapes(gpu_lib, oracle, monkeypatch):
    """The kernel instances of the 256x256x64 roofline volume (x half-length 256 in the
    row pass, py = 512 y passes) on a 256x256x2 grid forced onto the three-pass column
    path, and the 256x64 film of the adjoint workload (thin-film py = 128)."""
    monkeypatch.setenv("FULLMAG_FDM_NO_FUSED_YZ", "1")
    for nx, ny, nz in ((256, 256, 2), (256, 64, 1)):
        kw = problem(nx, ny, nz, d=(2e-9, 2e-9, 2e-9), ms=1.4e6, a_ex=2.1e-11, alpha=0.01, seed=17, kc1=-4.8e4)
        gpu, orc = make_pair(oracle, kw)
        ref = orc.fields(kw["m0"])
        assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < HEFF_TOL, (nx, ny, nz)
        assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_DEMAG), ref["h_demag"]) < HEFF_TOL, (nx, ny, nz)
        if nz > 1:
            gpu.set_kernel_timing(True)
            gpu.refresh()
            assert gpu.kernel_times()["y_forward"][1] >= 1


def test_heff_3d_spectra_for_single_layer(gpu_lib, oracle):
    """nz == 1 with full 3-D spectra (pz = 2) takes the 3-D column path."""
    kw = problem(16, 12, 1, seed=12)
    gpu, orc = make_pair(oracle, kw, thin=False)
    assert gpu.fft_shape() == (32, 24, 2)
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < HEFF_TOL


def test_heff_with_mask_and_anisotropy(gpu_lib, oracle):
    kw = problem(20, 14, 3, seed=13, ku1=5e3, ku2=1e3, u_axis=(1.0, 0.5, 0.2), kc1=-4.8e4, kc2=1e4, kc3=0.0,
                 c1=(1, 0, 0), c2=(0, 1, 0))
    rng = np.random.default_rng(5)
    mask = (rng.random(20 * 14 * 3) > 0.15).astype(np.uint8)
    gpu, orc = make_pair(oracle, kw, mask=mask)
    m = kw["m0"] * mask[:, None]
    ref = orc.fields(m)
    for obs, key in ((_abi.OBSERVABLE_H_EX, "h_ex"), (_abi.OBSERVABLE_H_DEMAG, "h_demag"),
                     (_abi.OBSERVABLE_H_EFF, "h_eff")):
        got = gpu.copy_field(obs)
        assert rel_l2(got, ref[key]) < HEFF_TOL, key
        assert np.abs(got[mask == 0]).max() == 0.0


def test_stats_at_step0(gpu_lib, oracle):
    kw = problem(24, 16, 4, seed=14, ku1=5e3, u_axis=(1, 0, 0), kc1=-4.8e4)
    gpu, orc = make_pair(oracle, kw)
    st = gpu.stats()
    ref = orc.observe()
    assert st["step"] == 0 and st["time_seconds"] == 0.0
    pairs = (("exchange_energy_joules", "e_exchange"), ("demag_energy_joules", "e_demag"),
             ("external_energy_joules", "e_external"), ("anisotropy_energy_joules", "e_uniaxial"),
             ("cubic_energy_joules", "e_cubic"), ("total_energy_joules", "e_total"),
             ("max_effective_field_amplitude", "max_h_eff"), ("max_demag_field_amplitude", "max_h_demag"),
             ("max_rhs_amplitude", "max_rhs"))
    for a, b in pairs:
        assert abs(st[a] - ref[b]) <= 1e-5 * abs(ref[b]) + 1e-30, (a, st[a], ref[b])


@pytest.mark.parametrize("integrator,dt,steps", [(_abi.INTEGRATOR_HEUN, 5e-14, 100),
                                                 (_abi.INTEGRATOR_RK4, 5e-14, 50)])
def test_fixed_step_trajectory_cfg1(gpu_lib, oracle, integrator, dt, steps):
    kw = problem(64, 32, 4, seed=0)
    gpu, orc = make_pair(oracle, kw, integrator=integrator)
    for s in range(steps):
        sg = gpu.step(dt)
        so = orc.step(dt)
    assert sg["step"] == steps
    assert abs(sg["time_seconds"] - steps * dt) < 1e-25
    m_g, m_o = gpu.copy_field(_abi.OBSERVABLE_M), orc.get_m()
    assert np.abs(m_g - m_o).max() < 2e-5
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-4 * abs(so["e_total"])
    assert abs(sg["max_rhs_amplitude"] - so["max_rhs"]) <= 1e-4 * so["max_rhs"]
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields()["h_eff"]) < 1e-4


def test_cfg1_full_heun_run(gpu_lib, oracle):
    """The 64x32x4 Heun configuration over its full 2000 steps (dt 5e-14, through the
    graph-replayed step_many): m and the energies against the FP64 oracle every 100 steps."""
    kw = problem(64, 32, 4, seed=0)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_HEUN)
    worst_m = worst_e = 0.0
    for _ in range(20):
        sg = gpu.step_many(5e-14, 100)
        for _ in range(100):
            so = orc.step(5e-14)
        worst_m = max(worst_m, float(np.abs(gpu.magnetization() - orc.get_m()).max()))
        for a, b in (("exchange_energy_joules", "e_exchange"), ("demag_energy_joules", "e_demag"),
                     ("external_energy_joules", "e_external"), ("total_energy_joules", "e_total")):
            worst_e = max(worst_e, abs(sg[a] - so[b]) / abs(so[b]))
    assert sg["step"] == 2000
    # FP32 state over 2000 steps from random unit vectors: max |dm| reaches ~1.5e-4
    # (the short-run Tier B bound of 1e-5 holds over the first 100 steps, see above);
    # the energies stay within ~2e-6 relative
    assert worst_m < 5e-4 and worst_e < 1e-5, (worst_m, worst_e)


def test_dp45_trajectory_thin_film(gpu_lib, oracle):
    kw = problem(64, 16, 1, d=(3.90625e-9, 3.90625e-9, 3e-9), seed=2, alpha=0.02, ku1=5e3, u_axis=(1, 0, 0),
                 b_mt=(-24.6, 4.3, 0.0), adaptive_max_error=1e-5)
    gpu, orc = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_DP45)
    dt_g = dt_o = 1e-13
    t_g = t_o = 0.0
    for _ in range(20):
        sg = gpu.step(dt_g)
        so = orc.step(dt_o)
        dt_g, dt_o = sg["suggested_next_dt"], so["suggested_next_dt"]
        t_g, t_o = sg["time_seconds"], so["time"]
    assert abs(t_g - t_o) <= 1e-3 * t_o
    m_g, m_o = gpu.copy_field(_abi.OBSERVABLE_M), orc.get_m()
    assert np.abs(m_g - m_o).max() < 1e-3
    assert abs(sg["total_energy_joules"] - so["e_total"]) <= 1e-3 * abs(so["e_total"])


def test_norm_preserved_and_energy_decreases(gpu_lib, oracle):
    kw = problem(32, 32, 2, seed=9, alpha=1.0, b_mt=None)
    gpu, _ = make_pair(oracle, kw)
    e0 = gpu.stats()["total_energy_joules"]
    for _ in range(50):
        st = gpu.step(5e-14)
    m = gpu.copy_field(_abi.OBSERVABLE_M)
    assert np.abs(np.linalg.norm(m, axis=1) - 1).max() < 1e-5
    assert st["total_energy_joules"] < e0


def test_upload_refresh_roundtrip(gpu_lib, oracle):
    kw = problem(16, 8, 2, seed=15)
    gpu, orc = make_pair(oracle, kw)
    m1 = problem(16, 8, 2, seed=16)["m0"]
    gpu.upload(m1)
    gpu.refresh()
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - m1).max() < 1e-7
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(m1)["h_eff"]) < HEFF_TOL
    f32 = gpu.copy_field(_abi.OBSERVABLE_H_EFF, dtype=np.float32)
    assert np.array_equal(f32.astype(np.float64), gpu.copy_field(_abi.OBSERVABLE_H_EFF))


def test_invalid_inputs_are_rejected(gpu_lib, oracle):
    kw = problem(8, 8, 1, seed=1)
    bad = dict(kw)
    bad["m0"] = kw["m0"][:-1]
    with pytest.raises(FdmError):
        FdmBackend(**bad, spectra=oracle.newell_spectra(8, 8, 1, 4e-9, 4e-9, 4e-9, True))
    with pytest.raises(FdmError, match="demag_kernel_spectrum_len"):
        FdmBackend(**kw, spectra=np.zeros((6, 10)))
    gpu, _ = make_pair(oracle, kw)
    with pytest.raises(FdmError):
        gpu.step(-1.0)
    with pytest.raises(FdmError):
        gpu.upload(kw["m0"][:5])


def test_interrupt_restores_state(gpu_lib, oracle):
    kw = problem(16, 16, 2, seed=3)
    gpu, _ = make_pair(oracle, kw, integrator=_abi.INTEGRATOR_RK4)
    gpu.step(5e-14)
    m_before = gpu.copy_field(_abi.OBSERVABLE_M)
    calls = {"n": 0}

    def poll():
        calls["n"] += 1
        return calls["n"] >= 2

    gpu.set_interrupt_poll(poll)
    with pytest.raises(FdmInterrupted):
        gpu.step(5e-14)
    gpu.set_interrupt_poll(None)
    assert np.array_equal(gpu.copy_field(_abi.OBSERVABLE_M), m_before)
    st = gpu.stats()
    assert st["step"] == 1
    gpu.step(5e-14)
    assert gpu.stats()["step"] == 2


def test_preview_and_snapshots(gpu_lib, oracle):
    kw = problem(12, 9, 4, seed=4)
    gpu, _ = make_pair(oracle, kw)
    full = gpu.copy_field(_abi.OBSERVABLE_M).reshape(4, 9, 12, 3)
    pv = gpu.preview(_abi.OBSERVABLE_M, 6, 3, 2, 0, 2).reshape(2, 3, 6, 3)
    ref = full.reshape(2, 2, 3, 3, 6, 2, 3).mean(axis=(1, 3, 5))
    assert np.allclose(pv, ref, rtol=0, atol=1e-12)
    # identity preview equals the full copy
    assert np.allclose(gpu.preview(_abi.OBSERVABLE_M, 12, 9, 4), full.reshape(-1, 3))
    import ctypes as C
    lib = gpu.lib
    s = lib.fullmag_fdm_backend_begin_field_snapshot(gpu.handle, _abi.OBSERVABLE_M)
    assert s
    data, nbytes, desc = C.c_void_p(), C.c_uint64(), _abi.SnapshotDesc()
    assert lib.fullmag_fdm_field_snapshot_wait(s, C.byref(data), C.byref(nbytes), C.byref(desc)) == 0
    arr = np.ctypeslib.as_array((C.c_float * (nbytes.value // 4)).from_address(data.value)).copy()
    lib.fullmag_fdm_field_snapshot_destroy(s)
    assert desc.cell_count == 12 * 9 * 4 and desc.scalar_bytes == 4
    assert np.allclose(arr.reshape(3, -1).T, full.reshape(-1, 3), atol=1e-7)


def test_device_info(gpu_lib, oracle):
    gpu, _ = make_pair(oracle, problem(4, 4, 1, seed=1))
    info = gpu.device_info()
    assert info["cc"][0] >= 10
