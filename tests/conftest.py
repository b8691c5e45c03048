import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "gapbs_ref.npz"
INT_MAX = 2**31 - 1


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a engine")


@pytest.fixture(scope="session", autouse=True)
def built_libs():
    """libgg.so and the oracle library, built in-tree if missing."""
    from easy_graphit_gb300 import build

    if not build.LIB.exists():
        build.build_lib()
    import oracle

    if not oracle.LIB.exists():
        oracle.build()
    yield


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def rel_l1(x, ref):
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(x - ref).sum() / max(np.abs(ref).sum(), 1e-300))
