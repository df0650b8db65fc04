"""Pins the FP64 oracle's Newell tensor to the reference's own known answers
(crates/fullmag-fdm-demag/src/newell.rs:673-908, extracted into golden/newell_kat.json)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

KAT = json.loads((Path(__file__).parent / "golden" / "newell_kat.json").read_text())


def test_f_g_vanish_at_origin(oracle):
    assert oracle.newell_f(0.0, 0.0, 0.0) == 0.0
    assert oracle.newell_g(0.0, 0.0, 0.0) == 0.0


@pytest.mark.parametrize("d", [(1.0, 1.0, 1.0), (5e-9, 5e-9, 2e-9), (5e-9, 5e-9, 1e-9), (3e-9, 4e-9, 5e-9)])
def test_self_term_trace_is_one(oracle, d):
    k = oracle.newell_kernels(1, 1, 1, *d)
    assert abs(k[0, 0, 0, 0] + k[1, 0, 0, 0] + k[2, 0, 0, 0] - 1.0) < KAT["self_trace_tol"]


def test_cube_self_term_is_one_third(oracle):
    k = oracle.newell_kernels(1, 1, 1, 1.0, 1.0, 1.0)
    assert abs(k[0, 0, 0, 0] - 1.0 / 3.0) < KAT["cubic_self_third_tol"]


def test_offdiagonal_self_terms_vanish(oracle):
    k = oracle.newell_kernels(1, 1, 1, 3e-9, 4e-9, 5e-9)
    for c in (3, 4, 5):
        assert abs(k[c, 0, 0, 0]) < KAT["offdiag_self_zero_tol"]


def test_flat_cell_ordering(oracle):
    k = oracle.newell_kernels(1, 1, 1, 5e-9, 5e-9, 2e-9)
    assert k[2, 0, 0, 0] > k[0, 0, 0, 0]
    assert abs(k[0, 0, 0, 0] - k[1, 0, 0, 0]) < 1e-12
    k = oracle.newell_kernels(1, 1, 1, 5e-9, 5e-9, 1e-9)
    assert k[2, 0, 0, 0] > 0.5


def test_parity_of_placed_kernel(oracle):
    k = oracle.newell_kernels(4, 4, 4, 1.0, 1.0, 1.0)
    px = 8
    assert abs(k[0, 3, 2, 1] - k[0, 3, 2, px - 1]) < 1e-15   # xx even in x
    assert abs(k[3, 3, 2, 1] + k[3, 3, 2, px - 1]) < 1e-15   # xy odd in x


def test_nxy_known_answers(oracle):
    k = oracle.newell_kernels(10, 10, 1, 1.0, 1.0, 1.0)
    for tag, v in KAT["nxy_10x10x1_unit"].items():
        i, j, _ = (int(t) for t in tag.split(","))
        got = k[3, 0, j, i]
        assert abs(got - v["check"]) < v["tol"], tag
        assert abs(got - v["reference"]) <= 6e-9 * abs(v["reference"]), tag  # 9 printed digits
    assert abs(k[3, 0, 0, 1]) < 1e-15
    for i in range(1, 5):
        for j in range(1, 5):
            assert k[3, 0, j, i] < 0.0


def test_nxy_far_field_matches_dipole(oracle):
    k = oracle.newell_kernels(12, 12, 1, 1.0, 1.0, 1.0)
    x = y = 8.0
    asym = -3 * x * y / (4 * math.pi * (x * x + y * y) ** 2.5)
    assert abs(k[3, 0, 8, 8] - asym) / abs(asym) < KAT["asymptotic_rel_tol_8_8_0"]


def test_spectra_thin_film_equals_3d_plane(oracle):
    """The 2-D thin-film spectra equal both kz planes of the nz=1 3-D spectra (pz=2)."""
    s2 = oracle.newell_spectra(6, 5, 1, 4e-9, 3e-9, 2e-9, thin_film_2d=True)
    s3 = oracle.newell_spectra(6, 5, 1, 4e-9, 3e-9, 2e-9, thin_film_2d=False)
    P2 = s2.shape[1] // 2
    for c in range(6):
        a = s2[c].reshape(P2, 2)
        b = s3[c].reshape(2, P2, 2)
        assert np.abs(a - b[0]).max() < 1e-12 * (np.abs(a).max() + 1e-300) + 1e-25
        assert np.abs(a - b[1]).max() < 1e-12 * (np.abs(a).max() + 1e-300) + 1e-25


def test_spectra_are_real_and_octant_symmetric(oracle):
    s = oracle.newell_spectra(5, 4, 3, 2e-9, 2e-9, 2e-9)
    px, py, pz = 10, 8, 6
    sp = s.reshape(6, pz, py, px, 2)
    for c in range(6):
        assert np.abs(sp[c, ..., 1]).max() < 1e-9 * np.abs(sp[c, ..., 0]).max()
    # even/odd under ky -> py-ky
    for c, sign in ((0, 1), (1, 1), (2, 1), (3, -1), (4, 1), (5, -1)):
        a = sp[c, :, 1, :, 0]
        b = sp[c, :, py - 1, :, 0]
        assert np.allclose(a, sign * b, rtol=1e-9, atol=1e-12 * np.abs(sp[c]).max())
