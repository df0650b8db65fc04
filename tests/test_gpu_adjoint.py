"""Reverse-mode RK4 gradients of the CUDA engine vs the FP64 oracle.

The engine's adjoint (fullmag_fdm_adjoint_forward / _backward) returns d loss / d field
map and d loss / d m0 for a fixed-step RK4 run.  Checks:
  * the applied field map enters H_eff exactly like the oracle's (step 0 parity);
  * directional derivatives g . dh and lambda0 . dm0 equal w . dm_T from the oracle's
    FP64 tangent-linear RK4 (exact for the discrete scheme; the tolerance covers FP32);
  * per-cell gradients through the torch.autograd.Function equal FP64 central finite
    differences of the oracle loss with a 1e-3 mT step;
  * the checkpoint interval does not change the gradient;
  * misuse is rejected with an error code.
"""
import numpy as np
import pytest
import torch

from fullmag_gb300 import FdmBackend, FdmError, _abi
from fullmag_gb300.adjoint import rk4_final_state
from helpers import MU0, problem, rel_l2

pytestmark = pytest.mark.gpu

DT = 5e-14


def film(nx, ny, seed, ku1=None, tilt=0.05):
    """In-plane film: m0 = +x with a small seeded tilt, (5, 0, 0) mT uniform field,
    alpha 0.05, and a seeded in-plane field map N(0, 2 mT) in A/m."""
    rng = np.random.default_rng(seed)
    n = nx * ny
    kw = problem(nx, ny, 1, alpha=0.05, b_mt=(5.0, 0.0, 0.0), seed=seed)
    m0 = np.tile([1.0, 0.0, 0.0], (n, 1)) + tilt * rng.normal(size=(n, 3))
    kw["m0"] = m0 / np.linalg.norm(m0, axis=1, keepdims=True)
    if ku1 is not None:
        kw.update(ku1=ku1, u_axis=(1.0, 0.0, 0.0))
    hmap = np.zeros((n, 3))
    hmap[:, :2] = rng.normal(0.0, 2e-3, size=(n, 2)) / MU0
    return kw, hmap


def pair(oracle, kw, hmap):
    sp = oracle.newell_spectra(kw["nx"], kw["ny"], kw["nz"], kw["dx"], kw["dy"], kw["dz"], thin_film_2d=True)
    gpu = FdmBackend(**kw, integrator=_abi.INTEGRATOR_RK4, spectra=sp)
    orc = oracle.Problem(**kw, integrator=oracle.RK4)
    gpu.set_field_map(hmap)
    orc.set_field_map(hmap)
    return gpu, orc


def test_field_map_heff(gpu_lib, oracle):
    kw, hmap = film(24, 12, seed=3, ku1=5e3)
    gpu, orc = pair(oracle, kw, hmap)
    gpu.refresh()
    ref = orc.fields(kw["m0"])
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), ref["h_eff"]) < 1e-5
    st, ost = gpu.stats(), orc.observe()
    assert abs(st["external_energy_joules"] - ost["e_external"]) <= 1e-4 * abs(ost["e_external"])
    gpu.set_field_map(None)
    gpu.refresh()
    orc.set_field_map(None)
    assert rel_l2(gpu.copy_field(_abi.OBSERVABLE_H_EFF), orc.fields(kw["m0"])["h_eff"]) < 1e-5


@pytest.mark.parametrize("ku1", [None, 5e3])
def test_gradient_vs_fp64_tangent(gpu_lib, oracle, ku1):
    nx, ny, steps = 32, 16, 160
    kw, hmap = film(nx, ny, seed=5, ku1=ku1)
    n = nx * ny
    gpu, orc = pair(oracle, kw, hmap)
    rng = np.random.default_rng(7)
    w = rng.normal(size=(n, 3))                       # loss L = sum w . m_T
    gpu.adjoint_forward(DT, steps)
    m_gpu = gpu.magnetization()
    grad, lam0 = gpu.adjoint_backward(w)
    for trial in range(3):
        dh = np.zeros((n, 3))
        dh[:, :2] = rng.normal(size=(n, 2)) * 1e3
        orc.set_m(kw["m0"])
        dm = orc.tangent_rk4(DT, steps, dh=dh)
        if trial == 0:
            assert np.abs(m_gpu - orc.get_m()).max() < 2e-5
        want = float(np.sum(w * dm))
        got = float(np.sum(grad * dh))
        assert abs(got - want) <= 1e-4 * abs(want), (trial, got, want)
    dm0 = rng.normal(size=(n, 3)) * 0.1
    orc.set_m(kw["m0"])
    dm = orc.tangent_rk4(DT, steps, dm0=dm0)
    want = float(np.sum(w * dm))
    got = float(np.sum(lam0 * dm0))
    assert abs(got - want) <= 1e-4 * abs(want), (got, want)


def test_torch_gradient_vs_central_fd(gpu_lib, oracle):
    """mean |m_T - m*|^2 through the autograd Function vs FP64 central differences
    (step 1e-3 mT) of the oracle loss at 64 random cells of the in-plane map."""
    nx, ny, steps = 24, 12, 120
    kw, hmap = film(nx, ny, seed=9)
    n = nx * ny
    gpu, orc = pair(oracle, kw, hmap)
    rng = np.random.default_rng(11)
    target = np.tile([1.0, 0.0, 0.0], (n, 1)) + 0.5 * rng.normal(size=(n, 3))
    target /= np.linalg.norm(target, axis=1, keepdims=True)
    b = torch.tensor(hmap[:, :2] * MU0, dtype=torch.float64, requires_grad=True)
    m0 = torch.tensor(kw["m0"], dtype=torch.float64)
    m_t = rk4_final_state(m0, b, gpu, DT, steps)
    loss = ((m_t - torch.tensor(target)) ** 2).mean()
    loss.backward()
    g = b.grad.numpy()

    def oracle_loss(bmap):
        h = np.zeros((n, 3))
        h[:, :2] = bmap / MU0
        orc.set_field_map(h)
        orc.set_m(kw["m0"])
        orc.tangent_rk4(DT, steps)  # advances the state; the tangent is not used here
        return float(np.mean((orc.get_m() - target) ** 2))

    assert abs(oracle_loss(hmap[:, :2] * MU0) - float(loss.detach())) < 1e-6
    step = 1e-6  # 1e-3 mT in tesla
    cells = rng.choice(n, size=64, replace=False)
    got, want = [], []
    for c in cells:
        for comp in range(2):
            bp = hmap[:, :2] * MU0
            bm = bp.copy()
            bp[c, comp] += step
            bm[c, comp] -= step
            want.append((oracle_loss(bp) - oracle_loss(bm)) / (2 * step))
            got.append(g[c, comp])
    got, want = np.array(got), np.array(want)
    # 1e-4 relative: in L2 over the 128 entries and per entry against the largest one
    assert rel_l2(got, want) < 1e-4, rel_l2(got, want)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()


def test_checkpoint_interval_invariance(gpu_lib, oracle):
    kw, hmap = film(16, 8, seed=13)
    n = 16 * 8
    gpu, _ = pair(oracle, kw, hmap)
    lam = np.random.default_rng(1).normal(size=(n, 3))
    grads = []
    for every in (0, 1, 7, 50):
        gpu.upload(kw["m0"])
        gpu.adjoint_forward(DT, 50, every)
        g, l0 = gpu.adjoint_backward(lam)
        grads.append((g, l0))
    for g, l0 in grads[1:]:
        assert np.allclose(g, grads[0][0], rtol=1e-6, atol=1e-12 * np.abs(grads[0][0]).max())
        assert np.allclose(l0, grads[0][1], rtol=1e-6, atol=1e-12 * np.abs(grads[0][1]).max())


def test_adjoint_misuse(gpu_lib, oracle):
    kw, hmap = film(8, 4, seed=1)
    gpu, _ = pair(oracle, kw, hmap)
    with pytest.raises(FdmError):
        gpu.adjoint_backward(np.zeros((32, 3)))   # no forward yet
    with pytest.raises(FdmError):
        gpu.adjoint_forward(DT, 0)
    gpu.adjoint_forward(DT, 4)
    with pytest.raises(FdmError):
        gpu.adjoint_backward(np.zeros((31, 3)))   # wrong length
    with pytest.raises(FdmError):
        gpu.set_field_map(np.zeros((31, 3)))
    heun = FdmBackend(**kw, integrator=_abi.INTEGRATOR_HEUN)
    with pytest.raises(FdmError):
        heun.adjoint_forward(DT, 4)


def test_config5_full_size_directional_derivative(gpu_lib, oracle):
    """The adjoint benchmark configuration at its own size (256x64x1 film of 4 nm cells,
    4000 RK4 steps of 5e-14 s, field map N(0, 2 mT), m0 = +x, the seeded target of eight
    Gaussian bumps, loss mean |m_T - m*|^2): the gradient through the autograd Function
    along one seeded field-map direction against the oracle's FP64 tangent-linear RK4
    of the same 4000 steps, within 1e-4 relative."""
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    import bench
    kw, bmap, target = bench.adjoint_problem()
    n = kw["nx"] * kw["ny"]
    steps = 4000
    gpu = FdmBackend(**kw)
    b = torch.tensor(bmap, dtype=torch.float64, requires_grad=True)
    m_t = rk4_final_state(torch.tensor(kw["m0"], dtype=torch.float64), b, gpu, DT, steps)
    loss = ((m_t - torch.tensor(target)) ** 2).mean()
    loss.backward()
    g = b.grad.numpy()  # d loss / d B (tesla)
    gpu.close()
    okw = {k: v for k, v in kw.items() if k != "integrator"}
    orc = oracle.Problem(**okw, integrator=oracle.RK4)
    hmap = np.zeros((n, 3))
    hmap[:, :2] = bmap / MU0
    orc.set_field_map(hmap)
    rng = np.random.default_rng(21)
    db = rng.normal(size=(n, 2)) * 1e-3  # direction in tesla
    dh = np.zeros((n, 3))
    dh[:, :2] = db / MU0
    dm = orc.tangent_rk4(DT, steps, dh=dh)
    m_o = orc.get_m()
    # d loss = (2/(3n)) sum (m_T - m*) . dm
    want = float(2.0 / (3 * n) * np.sum((m_o - target) * dm))
    got = float(np.sum(g * db))
    assert np.abs(m_t.detach().numpy() - m_o).max() < 5e-4  # FP32 state over 4000 steps
    assert abs(got - want) <= 1e-4 * abs(want), (got, want)
    orc.close()
