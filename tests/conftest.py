import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "loglik_golden.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); runs the product kernels")


@pytest.fixture(scope="session")
def golden():
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the in-tree GPU library; fail loudly when it cannot be used."""
    from libkriging_gb300.build import build
    build()
    import libkriging_gb300 as lk
    lib = lk.load()
    name = lib.lkg_device_name()
    if not name:
        pytest.fail("no CUDA device visible to the GPU library")
    return lk


def rel_err(a, b):
    a = np.atleast_1d(np.asarray(a, dtype=float))
    b = np.atleast_1d(np.asarray(b, dtype=float))
    na, nb = np.linalg.norm(a), np.linalg.norm(b)
    if na == 0 and nb == 0:
        return 0.0
    return float(np.linalg.norm(a - b) / max(na, nb))
