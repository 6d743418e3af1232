"""Shared pytest configuration: the ``gpu`` marker, golden-fixture loaders and GPU gating."""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def kat():
    return dict(np.load(GOLDEN / "kat.npz"))


@pytest.fixture(scope="session")
def mc():
    path = GOLDEN / "mc.json"
    if not path.exists():
        pytest.skip("tests/golden/mc.json (the reference's own Monte-Carlo results) is not present")
    return json.loads(path.read_text())


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import dmipy_sim_gb300._lib as L
    L.load()
    return torch.device("cuda", 0)
