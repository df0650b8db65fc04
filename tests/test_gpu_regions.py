"""Exchange with region ids and a 256 x 256 stiffness table on the GPU against the FP64
oracle (native/backends/fdm/src/exchange_fp32.cu:48-104, api.cpp:405-420,
reductions_fp64.cu:123-215): the H_EX and H_eff observables, the exchange energy, the
default table (A on the diagonal, regions decoupled) and trajectories."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, FdmError, _abi
from helpers import problem, rel_l2
from test_gpu_parity import make_pair

pytestmark = pytest.mark.gpu


def _regions(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    x = np.tile(np.arange(nx), ny * nz)
    reg = np.where(x < nx // 2, 0, 1).astype(np.uint32)
    reg[rng.random(reg.size) < 0.15] = 7
    lut = np.zeros((256, 256))
    lut[0, 0], lut[1, 1], lut[7, 7] = 1.3e-11, 0.7e-11, 2e-11
    lut[0, 1] = lut[1, 0] = 0.3e-11
    lut[1, 7] = lut[7, 1] = 0.5e-11
    return reg, lut


@pytest.mark.parametrize("with_table", [True, False])
@pytest.mark.parametrize("with_mask", [False, True])
def test_fields_and_exchange_energy(gpu_lib, oracle, with_table, with_mask):
    nx, ny, nz = 20, 12, 3
    reg, lut = _regions(nx, ny, nz, seed=5)
    kw = problem(nx, ny, nz, seed=101, region_mask=reg, exchange_lut=lut if with_table else None)
    mask = (np.random.default_rng(6).random(nx * ny * nz) > 0.15).astype(np.uint8) if with_mask else None
    gpu, orc = make_pair(oracle, kw, mask=mask)
    m = kw["m0"] if mask is None else kw["m0"] * mask[:, None]
    ref = orc.fields(m)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EX), ref["h_ex"]) < 1e-5
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["exchange_energy_joules"] - ost["e_exchange"]) <= 1e-5 * abs(ost["e_exchange"])
    assert abs(st["total_energy_joules"] - ost["e_total"]) <= 1e-5 * abs(ost["e_total"])


def test_default_table_decouples_regions(gpu_lib, oracle):
    # one region per half and no table: A on the diagonal, so the halves do not couple and
    # H_EX differs from the single-region field only in the two columns at the interface
    nx, ny, nz = 16, 8, 2
    x = np.tile(np.arange(nx), ny * nz)
    reg = np.where(x < nx // 2, 3, 4).astype(np.uint32)
    kw = problem(nx, ny, nz, seed=102, region_mask=reg)
    gpu, orc = make_pair(oracle, kw)
    h = gpu.copy_field(_abi.OBSERVABLE_H_EX)
    assert rel_l2(h, orc.fields(kw["m0"])["h_ex"]) < 1e-5
    hs = FdmBackend(**problem(nx, ny, nz, seed=102)).copy_field(_abi.OBSERVABLE_H_EX)
    interface = (x == nx // 2 - 1) | (x == nx // 2)
    assert rel_l2(h[~interface], hs[~interface]) < 1e-5
    assert np.abs(h[interface] - hs[interface]).max() > 1e-3 * np.abs(hs).max()


@pytest.mark.parametrize("integrator", [_abi.INTEGRATOR_RK4, _abi.INTEGRATOR_DP45])
def test_trajectory(gpu_lib, oracle, integrator):
    nx, ny, nz = 24, 12, 2
    reg, lut = _regions(nx, ny, nz, seed=7)
    kw = problem(nx, ny, nz, seed=103, alpha=0.1, region_mask=reg, exchange_lut=lut,
                 adaptive_max_error=1e-5 if integrator == _abi.INTEGRATOR_DP45 else 0.0)
    gpu, orc = make_pair(oracle, kw, integrator=integrator)
    dt = 5e-14
    for _ in range(20):
        sg = gpu.step(dt)
        so = orc.step(dt)
        if integrator == _abi.INTEGRATOR_DP45:
            # both take the oracle's suggestion, so the trajectories compare at equal times.
            # The suggestions themselves differ: on this random initial state dt |k| is about
            # 0.05, so the FP32 rounding of the stage derivatives (about 3e-9) is of the order
            # of the error estimate itself on the first step, and its fifth root moves the
            # suggestion by a few percent
            assert abs(sg["suggested_next_dt"] - so["suggested_next_dt"]) <= 0.1 * so["suggested_next_dt"]
            dt = so["suggested_next_dt"]
    # a rejected attempt retries at a size from each side's own error estimate
    assert abs(sg["time_seconds"] - so["time"]) <= 1e-6 * so["time"]
    tol = 2e-5 if integrator == _abi.INTEGRATOR_RK4 else 1e-4  # DP45 steps are about 4x longer
    assert np.abs(gpu.copy_field(_abi.OBSERVABLE_M) - orc.get_m()).max() < tol
    assert abs(sg["exchange_energy_joules"] - so["e_exchange"]) <= 1e-4 * abs(so["e_exchange"])


def test_bad_region_ids_are_rejected(gpu_lib):
    reg = np.zeros(8 * 4, dtype=np.uint32)
    reg[5] = 256
    with pytest.raises(FdmError):
        FdmBackend(**problem(8, 4, 1, seed=104, region_mask=reg))


def test_high_region_ids(gpu_lib, oracle):
    """Ids 128 and 255 (one byte per cell on the device: the values a signed or narrowed
    load would get wrong, and the largest table row offsets) with non-zero stiffness
    between them and with region 0, against the oracle."""
    nx, ny, nz = 18, 10, 2
    rng = np.random.default_rng(9)
    reg = rng.choice(np.array([0, 128, 255], dtype=np.uint32), size=nx * ny * nz)
    lut = np.zeros((256, 256))
    lut[0, 0], lut[128, 128], lut[255, 255] = 1.3e-11, 0.8e-11, 1.9e-11
    lut[128, 255] = lut[255, 128] = 0.6e-11
    lut[0, 255] = lut[255, 0] = 0.2e-11
    kw = problem(nx, ny, nz, seed=103, region_mask=reg, exchange_lut=lut)
    gpu, orc = make_pair(oracle, kw)
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EX), ref["h_ex"]) < 1e-5
    assert abs(gpu.stats()["exchange_energy_joules"] - orc.observe()["e_exchange"]) <= 1e-5 * abs(orc.observe()["e_exchange"])
