"""The benchmark's workload definitions on CPU: every workload maps to plan keywords that
the oracle accepts, and the periodic film carries its boundary policy to both sides (the
oracle's sample problem gets the same periodic axes and image counts as the engine)."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


@pytest.mark.parametrize("name", sorted(bench.WORKLOADS))
def test_workload_plan_keywords(name):
    w = bench.WORKLOADS[name]
    kw, integ = bench.plan_kwargs(w)
    n = w["nx"] * w["ny"] * w["nz"]
    assert kw["m0"].shape == (n, 3)
    assert np.allclose(np.linalg.norm(kw["m0"], axis=1), 1.0)
    assert ("periodic" in kw) == ("periodic" in w)


def test_periodic_workload_reaches_the_oracle(oracle):
    w = dict(bench.WORKLOADS["film_256x256x1_periodic_rk4"])
    kw, _ = bench.plan_kwargs(w)
    assert tuple(kw["periodic"]) == (1, 1, 0) and tuple(kw["image_counts"]) == (10, 10, 0)
    # a small sample of the workload through the bench's own oracle constructor against an
    # explicitly periodic oracle problem of the same sample
    pr = bench.oracle_problem(oracle, dict(w, nx=16, ny=16, nz=1), 16, 16, 1)
    kws, _ = bench.plan_kwargs(dict(w, nx=16, ny=16, nz=1))
    ref = oracle.Problem(**{k: v for k, v in kws.items() if k not in ("periodic", "image_counts")},
                         integrator=oracle.RK4, periodic=(1, 1, 0), image_counts=(10, 10, 0))
    open_ = oracle.Problem(**{k: v for k, v in kws.items() if k not in ("periodic", "image_counts")},
                           integrator=oracle.RK4)
    h, hr, ho = pr.fields()["h_demag"], ref.fields()["h_demag"], open_.fields()["h_demag"]
    assert np.array_equal(h, hr)
    assert np.abs(h - ho).max() > 1e-3 * np.abs(ho).max()
