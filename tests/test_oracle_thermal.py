"""Brown thermal field of the oracle (crates/fullmag-engine/src/fdm_fields.rs:818-896,
fdm_problem.rs:24-35,92-94,244-273): Gaussian noise from a SplitMix64 counter keyed by
(seed, step counter, cell, stream), Box-Muller on four uniforms per cell, amplitude
sigma = sqrt(2 alpha kB T / (gamma (1 + alpha^2) mu0 Ms V dt)); one counter value per step,
so every evaluation inside a step sees the same noise.

The reference has no thermal test vectors; the field is checked against a restatement of
that Rust code written with Python integers, and by its statistics."""
import math

import numpy as np
import pytest

from helpers import problem

MASK64 = (1 << 64) - 1
MU0 = 1.2566370614359173e-6
KB = 1.380649e-23


def _mix(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def _uniform(seed, step, cell, stream):
    key = (seed + step * 0x9E3779B97F4A7C15 + cell * 0x517CC1B727220A95 + stream * 0x6C62272E07BB0142) & MASK64
    return ((_mix(key) >> 11) + 1.0) / (float(1 << 53) + 1.0)


def _noise(seed, step, cell, sigma):
    u1, u2, u3, u4 = (_uniform(seed, step, cell, s) for s in range(4))
    r1, r2 = math.sqrt(-2.0 * math.log(max(u1, 1e-300))), math.sqrt(-2.0 * math.log(max(u3, 1e-300)))
    return sigma * np.array([r1 * math.cos(2 * math.pi * u2), r1 * math.sin(2 * math.pi * u2),
                             r2 * math.cos(2 * math.pi * u4)])


def _sigma(kw, T, dt):
    g0 = kw["gamma"] * (1.0 + kw["alpha"] ** 2)
    return math.sqrt(2.0 * kw["alpha"] * KB * T / (g0 * MU0 * kw["ms"] * kw["dx"] * kw["dy"] * kw["dz"] * dt))


def _bare(nx, ny, nz, **extra):
    kw = problem(nx, ny, nz, seed=3, b_mt=None, alpha=0.1)
    kw.update(enable_demag=False, a_ex=0.0, gamma=2.211e5)
    kw.update(extra)
    return kw


def test_field_matches_the_restated_counter_rng(oracle):
    kw = _bare(7, 5, 2, temperature=300.0)
    pr = oracle.Problem(**kw)
    h = pr.fields(pr.get_m())["h_eff"]
    sig = _sigma(kw, 300.0, 1e-13)  # no step yet: the default thermal dt
    want = np.array([_noise(42, 0, i, sig) for i in range(7 * 5 * 2)])
    assert np.allclose(h, want, rtol=1e-12, atol=1e-12 * sig)
    # a Heun step of 2e-13 s advances the counter and sets the amplitude's dt
    pr.step(2e-13)
    h = pr.fields(pr.get_m())["h_eff"]
    want = np.array([_noise(42, 1, i, _sigma(kw, 300.0, 2e-13)) for i in range(70)])
    assert np.allclose(h, want, rtol=1e-12, atol=1e-12 * sig)
    # another seed gives another stream
    pr2 = oracle.Problem(**kw, thermal_seed=7)
    h2 = pr2.fields(pr2.get_m())["h_eff"]
    assert np.allclose(h2[3], _noise(7, 0, 3, sig), rtol=1e-12)


def test_statistics(oracle):
    nx, ny, nz = 64, 32, 4
    kw = _bare(nx, ny, nz, temperature=50.0)
    pr = oracle.Problem(**kw)
    h = pr.fields(pr.get_m())["h_eff"]
    sig = _sigma(kw, 50.0, 1e-13)
    z = (h / sig).reshape(-1)
    n = z.size
    assert abs(z.mean()) < 5.0 / math.sqrt(n)
    assert abs(z.std() - 1.0) < 0.02
    c = np.corrcoef(h.T)
    assert np.abs(c - np.eye(3)).max() < 0.03
    # fourth moment of a Gaussian (3, standard error sqrt(96 / n)), within five errors
    assert abs((z ** 4).mean() - 3.0) < 5.0 * math.sqrt(96.0 / n)


def test_noise_is_fixed_within_a_step_and_fresh_across_steps(oracle):
    kw = _bare(6, 4, 1, temperature=300.0)
    pr = oracle.Problem(**kw)
    a = pr.fields(pr.get_m())["h_eff"]
    b = pr.fields(pr.get_m())["h_eff"]
    assert np.array_equal(a, b)
    pr.step(1e-13)
    c = pr.fields(pr.get_m())["h_eff"]
    assert np.abs(np.corrcoef(a.reshape(-1), c.reshape(-1))[0, 1]) < 0.3


def test_masked_cells_get_no_noise(oracle):
    kw = _bare(8, 4, 1, temperature=300.0)
    mask = np.ones(32, dtype=np.uint8)
    mask[[1, 9, 30]] = 0
    pr = oracle.Problem(**kw, active_mask=mask)
    h = pr.fields(pr.get_m())["h_eff"]
    assert np.abs(h[mask == 0]).max() == 0.0
    assert np.abs(h[mask == 1]).min() > 0.0


@pytest.mark.parametrize("alpha", [0.0])
def test_no_damping_no_noise(oracle, alpha):
    kw = _bare(4, 4, 1, temperature=300.0)
    kw["alpha"] = alpha
    pr = oracle.Problem(**kw)
    assert np.abs(pr.fields(pr.get_m())["h_eff"]).max() == 0.0
