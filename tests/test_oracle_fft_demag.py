"""The oracle's own FFT (stand-in for rustfft 6.4.1) and its FFT demag convolution,
checked against numpy.fft and against a direct O(N^2) real-space Newell sum."""
import numpy as np
import pytest

from helpers import random_unit


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 17, 34, 64, 100, 128, 251, 274, 502, 1024])
def test_fft1d_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(oracle.fft1d(x) - ref).max() / scale < 1e-14
    assert np.abs(oracle.fft1d(x, inverse=True) - np.fft.ifft(x) * n).max() / scale < 1e-14


def test_fft3d_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((6, 10, 12)) + 1j * rng.standard_normal((6, 10, 12))
    ref = np.fft.fftn(x)
    assert np.abs(oracle.fft3d(x) - ref).max() / np.abs(ref).max() < 1e-14


@pytest.mark.parametrize("shape", [(6, 5, 3), (7, 4, 1), (5, 5, 2), (1, 1, 1), (3, 1, 1), (9, 2, 1)])
def test_fft_demag_equals_direct_sum(oracle, shape):
    nx, ny, nz = shape
    n = nx * ny * nz
    rng = np.random.default_rng(n)
    mask = (rng.random(n) > 0.2).astype(np.uint8) if n > 3 else None
    pr = oracle.Problem(nx=nx, ny=ny, nz=nz, dx=4e-9, dy=3e-9, dz=2e-9, ms=8e5, a_ex=1.3e-11, alpha=0.5,
                        m0=random_unit(n, 7), active_mask=mask)
    hd = pr.fields()["h_demag"]
    ref = pr.demag_direct()
    assert np.abs(hd - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0)


def test_uniformly_magnetised_cube_field_is_minus_third_ms(oracle):
    pr = oracle.Problem(nx=1, ny=1, nz=1, dx=2e-9, dy=2e-9, dz=2e-9, ms=8e5, a_ex=0.0, alpha=0.5,
                        m0=np.array([[0.0, 0.0, 1.0]]), enable_exchange=False)
    hd = pr.fields()["h_demag"]
    assert abs(hd[0, 2] + 8e5 / 3.0) < 1e-6 * 8e5
