import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def lib():
    """The sm_103a library, built in-tree if missing (nvcc cross-compiles)."""
    from sph_fem_2d_cutting_gpu_gb300 import abi, build
    if not abi.LIB_PATH.exists():
        build.build()
    return abi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    return oracle.load()


def rel_err(a, b, scale=None):
    """Norm-wise error max|a-b| / max(max|b|, rms(b)) (field scale guards cancelling sums)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    s = max(float(np.max(np.abs(b))), float(np.sqrt(np.mean(b * b))), 1e-300)
    if scale is not None:
        s = max(s, scale)
    return float(np.max(np.abs(a - b))) / s


def assert_close(a, b, rtol, what="", scale=None):
    e = rel_err(a, b, scale)
    assert e <= rtol, f"{what}: relative error {e:.3e} > {rtol:.1e}"
