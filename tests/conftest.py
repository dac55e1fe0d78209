import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build (incrementally) the product library and the CPU oracle once per session."""
    from vierkant_gb300.build import build
    import oracle
    build()
    oracle.build(ref=None)
    yield


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(GOLDEN / f"{name}.npz")
    return load


@pytest.fixture(scope="session")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vierkant_gb300.raytracing import Context
    c = Context(0)
    yield c
    c.close()
