import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA engine; fails loudly when it cannot be built or no GPU is visible."""
    from fullmag_gb300 import build, load_library
    build.build()
    lib = load_library()
    assert lib.fullmag_fdm_is_available() == 1, "no CUDA device visible to libfullmag_fdm"
    return lib
