"""The cuFFT + unfused measurement baseline computes the same steps as the fused engine
(and hence the oracle): a baseline that diverged would make its timing meaningless."""
import numpy as np
import pytest

from fullmag_gb300 import FdmBackend, _abi
from fullmag_gb300.plain import PlainBaseline
from helpers import problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("integrator,extra", [(_abi.INTEGRATOR_RK4, dict(kc1=-4.8e4)),
                                              (_abi.INTEGRATOR_HEUN, dict(ku1=5e3, u_axis=(1.0, 0.0, 0.0)))])
def test_plain_matches_fused(gpu_lib, integrator, extra):
    kw = problem(32, 16, 4, d=(2e-9, 2e-9, 2e-9), ms=1.4e6, a_ex=2.1e-11, alpha=0.01, seed=4, **extra)
    fused = FdmBackend(**kw, integrator=integrator)
    plain = PlainBaseline(**kw, integrator=integrator)
    for _ in range(5):
        sf = fused.step(2e-14)
        sp = plain.step(2e-14)
    assert np.abs(fused.magnetization() - plain.magnetization()).max() < 1e-5
    for key in ("exchange_energy_joules", "demag_energy_joules", "external_energy_joules",
                "anisotropy_energy_joules", "cubic_energy_joules", "total_energy_joules"):
        a, b = sf[key], sp[key]
        assert abs(a - b) <= 1e-4 * max(abs(a), abs(b)) + 1e-30, (key, a, b)
    for key in ("max_effective_field_amplitude", "max_demag_field_amplitude", "max_rhs_amplitude"):
        assert abs(sf[key] - sp[key]) <= 1e-4 * abs(sf[key]), (key, sf[key], sp[key])
